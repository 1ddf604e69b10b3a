/*
 * sandengine_gb300 C ABI: the Margolus 2x2 block grid update of sandengine on GB300.
 *
 * This is the drop-in boundary for the reference's simulation path.  A host binds these
 * functions (Rust extern "C", ctypes, ...) in place of:
 *   - sandengine-lang: parse_string / parse_path / create_glsl_from_parser
 *       (sandengine-lang/src/parser.rs:93-152, sandengine-lang/src/lib.rs:10-17)
 *   - sandengine-core::simulation::Simulation: new / run / params.frame / modifications
 *       (sandengine-core/src/simulation.rs:97-253)
 *
 * Conventions: every function returns an int status (SE_OK = 0); on failure
 * se_last_error() returns a message for the calling thread.  Nothing aborts or throws
 * across the boundary.  Handles are not thread-safe; distinct handles may be used from
 * distinct threads.  Cells are uint32 material ids (the reference stores the id in the .r
 * channel of an RGBA32F texel, operations.glsl:111-112); ids that name no material read
 * as NULL, as getMaterialFromID does (gen/materials.glsl:79-86).
 */
#ifndef SANDENGINE_GB300_H
#define SANDENGINE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The parse kinds mirror ParsingErr (sandengine-lang/src/parser.rs:42-73). */
enum se_status {
  SE_OK = 0,
  SE_ERR_INVALID_ARGUMENT = 1,
  SE_ERR_MISSING_FIELD = 2,   /* ParsingErr::MissingField */
  SE_ERR_INVALID_TYPE = 3,    /* ParsingErr::InvalidType */
  SE_ERR_NOT_FOUND = 4,       /* ParsingErr::NotFound */
  SE_ERR_NOT_RECOGNIZED = 5,  /* ParsingErr::NotRecognized */
  SE_ERR_YAML = 6,            /* serde_yaml rejected the text */
  SE_ERR_PANIC = 7,           /* the reference panics on this input (e.g. unknown parent type) */
  SE_ERR_GLSL = 8,            /* the generated shader would not compile (reference panics, simulation.rs:133-137) */
  SE_ERR_UNSUPPORTED = 9,     /* valid rule GLSL the CUDA back end does not translate */
  SE_ERR_COMPILE = 10,        /* NVRTC failed */
  SE_ERR_CUDA = 11,           /* a CUDA runtime call failed */
  SE_ERR_OUT_OF_MEMORY = 12,
  SE_ERR_BUFFER_TOO_SMALL = 13,
  SE_ERR_NOT_COMPILED = 14,   /* se_ruleset_compile has not succeeded yet */
  SE_ERR_BUDGET = 15,         /* serving: the request cannot fit the HBM budget */
  SE_ERR_TIMEOUT = 16,
  SE_ERR_CANCELLED = 17       /* serving: the request was withdrawn */
};

/* Modification shapes (sandengine-core/src/simulation.rs:41-42). */
#define SE_MODSHAPE_CIRCLE 0
#define SE_MODSHAPE_SQUARE 1
#define SE_MAX_MODIFICATIONS 256 /* simulation.rs:43 */

/* SimModification, repr(C), 32 bytes = the std140 UBO record (simulation.rs:45-56). */
typedef struct se_modification {
  int32_t position[2];
  int32_t mod_shape;
  int32_t mod_size;
  int32_t mod_matID;
  int32_t _pad4[3];
} se_modification;

typedef struct se_ruleset se_ruleset;
typedef struct se_world se_world;

/* Message of the last failed call on this thread ("" if none). */
const char* se_last_error(void);
/* Library version as 10000*major + 100*minor + patch. */
int se_version(void);

/* ---- rule language (replaces sandengine-lang; no GPU needed) ------------------------- */

/* parse_string (parser.rs:93-152): parses the YAML rule set and generates the CUDA rule
 * code.  Parse errors return SE_ERR_MISSING_FIELD / _INVALID_TYPE / _NOT_FOUND /
 * _NOT_RECOGNIZED / _YAML / _PANIC with the reference's message text in se_last_error().
 * Rule text whose GLSL would not compile (SE_ERR_GLSL) or that the CUDA back end does not
 * translate (SE_ERR_UNSUPPORTED) parses, and fails in se_ruleset_compile / se_world_create,
 * where the reference panics building its shader (simulation.rs:133-137). */
int se_ruleset_parse(const char* yaml_text, se_ruleset** out);
/* parse_path (sandengine-lang/src/lib.rs:10-13). */
int se_ruleset_parse_path(const char* path, se_ruleset** out);
/* create_glsl_from_parser (sandengine-lang/src/lib.rs:17-147), returned as text:
 * which = 0 -> gen/materials.glsl, 1 -> gen/rules.glsl, 2 -> generated CUDA rule code,
 * 3 -> the complete device source handed to NVRTC.
 * Writes at most cap bytes (NUL-terminated when room); *len gets the full length. */
int se_ruleset_text(const se_ruleset* rs, int which, char* buf, size_t cap, size_t* len);
/* Compiles the rule set's kernels for sm_103a with NVRTC (cached on disk under
 * $SE_CACHE_DIR or ~/.cache/sandengine_gb300).  Needs no GPU. */
int se_ruleset_compile(se_ruleset* rs);
/* CHECKED build (no counterpart in the reference; the sanitizer substitute): before the
 * rule set is first compiled, enable != 0 compiles its kernels with index checks on every
 * shared-memory, global and table access that could leave its buffer.  A failed check sets
 * a bit of the module's check word and skips the access (no trap).  Bits: 1 table index,
 * 2 shared-array index, 4 chunk-list capacity, 8 chunk window, 16 global index, 32 edit
 * index.  se_ruleset_check_word synchronizes the device and reads (and with reset != 0
 * clears) the word; it covers every world, batch and server of the rule set. */
int se_ruleset_set_checked(se_ruleset* rs, int enable);
int se_ruleset_check_word(se_ruleset* rs, unsigned int* word, int reset);
/* Number of materials (ids 0..n-1; EMPTY=0, NULL=1, WALL=2, then YAML order). */
int se_ruleset_num_materials(const se_ruleset* rs, int* n);
/* Material id by name (materials.rs ids), or SE_ERR_NOT_FOUND. */
int se_ruleset_material_id(const se_ruleset* rs, const char* name, int* id);
/* The block transition table this device built for the rule set (no counterpart in the
 * reference, whose shader evaluates the rules per block; this is introspection for
 * tests).  An entry holds the block's four output ids, 4 bits each, as top-left |
 * bottom-left << 4 | top-right << 8 | bottom-right << 12.  *entries gets the number of u16
 * entries and *static_words the 32-bit words of
 * the bitset of static keys (both 0 when the rules need the direct path); when `table` /
 * `bits` are not null, at most cap_entries / cap_words of them are copied from the device.
 * Loads the kernels on the current device first. */
int se_ruleset_table(se_ruleset* rs, uint16_t* table, size_t cap_entries, uint32_t* bits, size_t cap_words,
                     unsigned long long* entries, unsigned long long* static_words);
void se_ruleset_free(se_ruleset* rs);

/* ---- one world (replaces sandengine-core::simulation::Simulation) --------------------- */

/* Simulation::new (simulation.rs:128-192): an all-EMPTY width x height world with frame
 * counter 0 on the current CUDA device.  Compiles the rule set if needed.  Sides up to
 * 1048576 cells and at most 2^36 cells (SE_ERR_INVALID_ARGUMENT beyond). */
int se_world_create(se_ruleset* rs, int width, int height, se_world** out);
void se_world_destroy(se_world* w);

/* ---- colour and light (the other two outputs of the reference's setCell,
 * operations.glsl:99-169; Simulation::output_color / output_light, simulation.rs:110-114) ----
 * se_world_set_light(w, 1) keeps a light field (RGBA32F per cell, zero at first, as the
 * reference's textures are): every later se_world_step frame is followed by the light pass
 * (a cell's light is its new material's emission if it emits, the sky value on row 0,
 * else a blend of its 8 neighbours' previous light, masked by their old cells).  Light on
 * makes every frame a separate launch.  0 frees the field. */
int se_world_set_light(se_world* w, int enable);
/* The current light field to / from a host or device buffer of width * height * 4 floats. */
int se_world_get_light(se_world* w, float* rgba, size_t n_floats);
int se_world_set_light_field(se_world* w, const float* rgba, size_t n_floats);
/* output_color of the current grid (RGBA32F, width * height * 4 floats, host or device
 * buffer): the material colour, darkened by noise(pos) / 4 for every material but EMPTY.
 * The noise field is computed on the first call and kept. */
int se_world_render_color(se_world* w, float* rgba, size_t n_floats);
/* The same into the world's own device buffer, ordered on the world's stream (no
 * synchronization); *rgba stays valid until the next render or se_world_destroy. */
int se_world_render_color_device(se_world* w, float** rgba);

/* Headless composite of the current grid (shaders/fragment140.glsl:70-100, drawn by
 * renderer.rs:212-246 as a full-screen quad): one RGBA32F pixel per cell, rows top to
 * bottom.  The colour field's box-filter mip pyramid gives the three blurred-alpha
 * occlusion terms; the light field is used when kept (else zero light); bg_rgba is an
 * optional bg_w x bg_h RGBA32F background (host or device memory; NULL: transparent).
 * GL filtering is fixed to the spec's formulas in binary32: mirrored-repeat wrap,
 * nearest / bilinear taps, LINEAR_MIPMAP_NEAREST level choice. */
int se_world_composite(se_world* w, const float* bg_rgba, int bg_w, int bg_h, float* out_rgba, size_t n_floats);
/* The same into the world's own device buffer, stream-ordered; *out_rgba stays valid until
 * the next composite or se_world_destroy. */
int se_world_composite_device(se_world* w, const float* bg_rgba, int bg_w, int bg_h, float** out_rgba);

/* ---- row bands of one world (no counterpart in the reference, which runs one world on
 * one GPU) ------------------------------------------------------------------------------
 * A band world holds rows [row0, row0 + rows) of a width x world_height world plus up to
 * `halo` rows on either side (clipped to the world).  It steps like a world in world
 * coordinates (hash, block parity, WALL border, edit positions), but may advance at most
 * `halo` frames per se_world_step: after n frames its rows at least n rows inside the
 * buffer are exact (its own rows, when n <= halo), and the halo rows must be refreshed from
 * the neighbouring bands (se_world_copy_rows) before the next step.  se_world_set_grid /
 * get_grid / digest / histogram cover the whole buffer; snapshots refuse bands. */
int se_world_create_band(se_ruleset* rs, int width, int world_height, int row0, int rows, int halo,
                         se_world** out);
/* Buffer rows [*buffer_row0, *buffer_row0 + *buffer_rows) of a *world_height-row world;
 * *halo = -1 for a whole world. */
int se_world_band_info(const se_world* w, int* buffer_row0, int* buffer_rows, int* world_height, int* halo);
/* Copies world rows [row, row + nrows) (inside the buffer) of the current grid to `ptr`
 * (to_world = 0) or from `ptr` into the grid (to_world = 1).  `ptr` is host or device
 * memory (the copy direction is inferred from it); returns when the copy is done. */
int se_world_copy_rows(se_world* w, int row, int nrows, void* ptr, int to_world);
/* Work is issued on this stream (cudaStream_t; NULL = the world's own stream). */
int se_world_set_stream(se_world* w, void* cuda_stream);
int se_world_get_stream(se_world* w, void** cuda_stream);
/* Fusion depth: frames advanced per launch when no edit intervenes (1 = one launch per
 * frame, like the reference; 0 = chosen by the autotuner on the first multi-frame step). */
int se_world_set_steps_per_launch(se_world* w, int k);
/* Times every compiled tile shape and fusion depth on this world (`reps` launches each,
 * reading the current grid into the spare buffer, so the world's state is unchanged) and
 * keeps the fastest; *best_k gets the chosen frames per launch.  (No counterpart in the
 * reference, which dispatches one frame at a time.) */
int se_world_autotune(se_world* w, int reps, int* best_k);
/* Chooses the compiled tile variant for multi-frame launches (k >= 2) or for one-frame
 * launches (k = 1) directly: tile_w x tile_h output cells, up to k frames per launch.  An
 * override of the autotuner, for profiling one variant.  (No counterpart in the reference.) */
int se_world_set_tile(se_world* w, int tile_w, int tile_h, int k);
/* The variant the next multi-frame launch uses (0, 0, 0 before the autotuner has run when
 * it is to choose). */
int se_world_get_tile(const se_world* w, int* tile_w, int* tile_h, int* k);
/* Replace / read the grid (width*height uint32, row-major) from host memory.  Both
 * synchronize the world's stream. */
int se_world_set_grid(se_world* w, const uint32_t* cells, size_t count);
int se_world_get_grid(se_world* w, uint32_t* cells, size_t count);
/* Stream-ordered copies with pinned host memory that the caller keeps alive until the
 * stream reaches them. */
int se_world_set_grid_async(se_world* w, const uint32_t* cells, size_t count);
int se_world_get_grid_async(se_world* w, uint32_t* cells, size_t count);
/* Read-back that overlaps the world's next frames: the current grid is copied on the
 * device into one of two staging buffers (ordered on the world's stream), then to `cells`
 * (pinned host memory for full overlap; count = width * height) on a separate copy stream.
 * `cells` holds this grid once se_world_synchronize returns.  At most two such reads are
 * in flight; a third waits for the first.  (No counterpart in the reference.) */
int se_world_read_grid_overlapped(se_world* w, uint32_t* cells, size_t count);
/* The same read-back with each cell's material id packed into one byte on the device (a
 * quarter of the bytes over the host link; rule sets of at most 256 materials).  Ids that
 * name no material are reported as NULL (1), the value the next frame reads them as; after
 * any frame every cell already holds a material id, so the bytes then equal the grid. */
int se_world_read_grid_u8_overlapped(se_world* w, uint8_t* cells, size_t count);
/* Device pointer of the current grid (valid until the next step, which ping-pongs). */
int se_world_device_grid(se_world* w, uint32_t** device_cells);
/* Params.frame (simulation.rs:78): the counter before the next step (>= 0). */
int se_world_set_frame(se_world* w, int32_t frame);
int se_world_get_frame(const se_world* w, int32_t* frame);
/* Simulation::run repeated nframes times (simulation.rs:195-253): each frame does
 * frame += 1 and one Margolus step (frame 1 clears the grid, falling_sand.glsl:128-131).
 * `mods` (up to 256 used, the scan stops at the first mod_size == 0) apply to the first
 * of these frames only, as the reference clears its list after each run.  Asynchronous on
 * the world's stream. */
int se_world_step(se_world* w, int nframes, const se_modification* mods, int nmods);
/* Waits for the world's stream and for its overlapped read-backs. */
int se_world_synchronize(se_world* w);
/* Order-independent 64-bit digest of the current grid: sum over cells i of
 * splitmix64_finalize((i << 32) | cell[i]) mod 2^64.  Synchronizes the stream.
 * (No counterpart in the reference: a device-side check for full-size worlds.) */
int se_world_digest(se_world* w, uint64_t* digest);
/* counts[m] = number of cells holding value m, for m < nbins-1; counts[nbins-1] gets all
 * values >= nbins-1.  nbins in [1, 257].  Synchronizes the stream.  (No counterpart in the
 * reference: material-conservation checks.) */
int se_world_histogram(se_world* w, uint64_t* counts, int nbins);
/* The same material counts as se_world_histogram, for any grid already on the device
 * (`count` uint32 cells at `device_cells`), WITHOUT allocating: no cudaMalloc, cudaFree or
 * allocating library call.  It exists for callers that cannot allocate device memory at
 * the point they need the counts: a frame loop that sized all of its GPU memory up front
 * and may not allocate per frame, a serving process whose HBM budget is already fully
 * committed to resident worlds, or code running while another allocator (e.g. a framework's
 * caching allocator) holds the free memory.  The counters live in a static device array of
 * SE_NOALLOC_MAX_BINS (257) 64-bit words, 2,056 bytes, which every GPU that loads the
 * library keeps until the process exits; nbins above 257 is rejected with
 * SE_ERR_INVALID_ARGUMENT.  The first call on a device looks up the array's device address
 * (make that first call before any stream capture); after a device reset (a new context on
 * the device) the next call looks it up again.  Every call shares the array: it clears
 * the counters on `cuda_stream` (NULL = the legacy default stream), counts, copies nbins
 * counters to host_counts and synchronizes the stream before returning, so calls from one
 * thread never overlap, and no call may be made on a stream that is being captured into a
 * graph; calls from different threads or streams that overlap on the GPU race on the
 * counters.  (No counterpart in the reference.) */
#define SE_NOALLOC_MAX_BINS 257
int se_grid_histogram_noalloc(const uint32_t* device_cells, uint64_t count, int nbins, uint64_t* host_counts,
                              void* cuda_stream);
/* Opt-in timing of the Margolus tile kernel: with enable != 0, every tile launch is
 * bracketed by CUDA events on the world's stream.  se_world_read_timing synchronizes and
 * returns, since the last read, the summed kernel time, the number of launches, the cell
 * updates they performed (cells x frames) and the cells they read (one u32 read + one u32
 * write each: the launch's algorithmic bytes are 8 x cells).  (No counterpart in the
 * reference: roofline measurement.) */
int se_world_set_timing(se_world* w, int enable);
int se_world_read_timing(se_world* w, double* kernel_ms, long long* launches, long long* cell_frames,
                         long long* cells);
/* The summed kernel time and the number of the tile launches since the last read that
 * advanced exactly `frames` frames each (synchronizes; does not reset: se_world_read_timing
 * does).  The roofline of one fusion depth, e.g. the k = 8 launches of 60-frame steps. */
int se_world_peek_timing_frames(se_world* w, int frames, double* kernel_ms, long long* launches);
/* The same for the light pass (pass = 1; algorithmic bytes 40 x cells: old and new id, old
 * and new RGBA32F light), the colour pass (pass = 2; 24 x cells: id, noise, RGBA32F) and the
 * composite (pass = 3; 48 x cells: colour, light, output; its pyramid is not timed). */
int se_world_read_pass_timing(se_world* w, int pass, double* kernel_ms, long long* launches, long long* cells);

/* ---- many worlds (no counterpart in the reference, which runs one world) --------------- */

typedef struct se_batch se_batch;

/* n independent worlds of the given sizes, all EMPTY, frame 0, in one device arena.
 * Worlds whose grid (plus a WALL border) fits in one CTA's shared memory are advanced a
 * whole launch at a time on chip; the others by temporally blocked tile passes. */
int se_batch_create(se_ruleset* rs, int n, const int* widths, const int* heights, se_batch** out);
void se_batch_destroy(se_batch* b);
int se_batch_set_grid(se_batch* b, int world, const uint32_t* cells, size_t count);
int se_batch_get_grid(se_batch* b, int world, uint32_t* cells, size_t count);
int se_batch_set_frame(se_batch* b, int world, int32_t frame);
int se_batch_get_frame(const se_batch* b, int world, int32_t* frame);
/* Advances every world by nframes frames with one CUDA graph launch (captured on first use
 * for each nframes): the resident worlds and the tile passes run as concurrent branches
 * and the frame counters advance on the device.  Either all worlds or none may be at
 * frame 0 (whose next frame clears, falling_sand.glsl:128-131).  Asynchronous. */
int se_batch_step(se_batch* b, int nframes);
/* The same frames with one kernel launch per world per frame, as the reference dispatches
 * (the baseline the batched launch is measured against). */
int se_batch_step_plain(se_batch* b, int nframes);
/* Times every tile shape / fusion depth on the tiled worlds (state unchanged) and keeps
 * the fastest; *best_k = frames per tile pass. */
int se_batch_autotune(se_batch* b, int reps, int* best_k);
int se_batch_set_steps_per_launch(se_batch* b, int k);
/* Worlds whose whole-world CTA needs at most `bytes` of shared memory are advanced in
 * shared memory for all frames of a launch group; the others by tile passes (0: all by tile
 * passes).  The default is the device's opt-in maximum. */
int se_batch_set_resident_limit(se_batch* b, size_t bytes);
int se_batch_synchronize(se_batch* b);
int se_batch_get_stream(se_batch* b, void** cuda_stream);
int se_batch_info(const se_batch* b, int* resident_worlds, int* tiled_worlds, long long* cells,
                  int* steps_per_launch);

/* ---- serving (no counterpart in the reference) ---------------------------------------- */

typedef struct se_server se_server;

typedef struct se_server_stats {
  long long requests;          /* requests served by the last run */
  double p50_ms, p99_ms;       /* latency percentiles: completion on the GPU minus arrival */
  double mean_ms, max_ms;
  double wall_ms;              /* run start to the last completion */
  double cell_updates;         /* cells x frames advanced by the last run */
  long long iterations;        /* batched iterations (plain path: requests) */
  long long evictions, restores;
  long long peak_resident_bytes;
  double restore_ms;           /* mean host time to bring an evicted session back into HBM */
  double kernel_ms;            /* GPU time of the last run's iterations, each from its first launch
                                  to its end (iterations run in order on one stream, so the gaps
                                  between them are left out: kernel_ms / wall_ms is the share of the
                                  run the GPU spent serving) */
} se_server_stats;

/* A server whose sessions' grids (two u32 buffers each) share one HBM arena of
 * budget_bytes; sessions that do not fit are evicted to host memory, least recently used
 * first, and restored when a request needs them. */
int se_server_create(se_ruleset* rs, long long budget_bytes, se_server** out);
void se_server_destroy(se_server* s);
/* Frames a session may advance per batched iteration (a compiled fusion depth). */
int se_server_set_frames_per_iteration(se_server* s, int k);
/* A session with an initial grid (NULL = all EMPTY) and frame counter. */
int se_server_open_session(se_server* s, int width, int height, const uint32_t* cells, int32_t frame,
                           int* session);
int se_server_close_session(se_server* s, int session);
/* Queues "advance nframes frames, applying mods to the first" for a session.  Requests of
 * one session run in order.  Before se_server_run it arrives arrival_ms after the start of
 * that run; while the live loop runs (se_server_start) it arrives when it is submitted and
 * arrival_ms is ignored.  Safe to call from any thread while the live loop runs. */
int se_server_submit(se_server* s, int session, int nframes, const se_modification* mods, int nmods,
                     double arrival_ms, int* request);
/* Withdraws a submitted request that has not started: it is skipped, its session does not
 * advance for it, and waiting for it returns SE_ERR_CANCELLED.  Any thread. */
int se_server_cancel(se_server* s, int request);
/* Replay: serves every queued request in real time, admitting requests when their arrival
 * time has passed and memory allows, and returns when all are done.  plain = 0: continuous
 * batching (every active session advances in one launch per iteration; sessions join and
 * leave between iterations); plain = 1: one request at a time, one launch per frame (the
 * reference's dispatch). */
int se_server_run(se_server* s, int plain);
/* Live: starts the serving loop on a host thread of its own (plain as for se_server_run).
 * Requests submitted from any thread are admitted at the loop's next iteration, while
 * others are on the GPU, as sessions and HBM free up.  The reference's host likewise feeds
 * edits into its running event loop (sandengine-core/src/lib.rs:57-69).  se_server_stop
 * serves what was submitted, then ends the loop and returns its status. */
int se_server_start(se_server* s, int plain);
int se_server_stop(se_server* s);
/* Blocks until the request has completed on the GPU (timeout_ms < 0: no limit), then gives
 * its latency (completion minus submission).  SE_ERR_TIMEOUT when it has not completed in
 * time, SE_ERR_CANCELLED for a withdrawn request.  se_server_poll does not block: *done = 1
 * (and the latency) once completed, else 0.  Any thread. */
int se_server_wait(se_server* s, int request, double timeout_ms, double* latency_ms);
int se_server_poll(se_server* s, int request, int* done, double* latency_ms);
int se_server_stats_get(se_server* s, se_server_stats* out);
int se_server_request_latency(se_server* s, int request, double* latency_ms);
int se_server_get_grid(se_server* s, int session, uint32_t* cells, size_t count);
int se_server_get_frame(se_server* s, int session, int32_t* frame);

/* ---- world snapshots (the reference lists world saving/loading as a TODO, README.md:85-87) */
/* A snapshot file holds a world's whole state: its grid and frame counter, plus the size,
 * the number of materials and a fingerprint of the rule set it was saved with (loading
 * under a different rule set is refused).  Layout: 32-byte little-endian header ("SEW1",
 * header size, width, height, frame, materials, u64 rule-set fingerprint), then the cells. */
int se_snapshot_info(const char* path, int* width, int* height, int32_t* frame);
int se_world_save(se_world* w, const char* path);
/* The snapshot's size must equal the world's. */
int se_world_load(se_world* w, const char* path);
/* The same format for serving sessions (an evicted session is this record in host memory). */
int se_server_save_session(se_server* s, int session, const char* path);
int se_server_open_session_from(se_server* s, const char* path, int* session);

#ifdef __cplusplus
}
#endif

#endif /* SANDENGINE_GB300_H */
