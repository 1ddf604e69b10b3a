// Ahead-of-time sm_103a kernels that do not depend on a rule set: grid digests and
// material histograms, used to check full-size worlds on the device without copying
// them out (order-independent digest; per-material counts for conservation checks).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

// Counters for se_grid_histogram_noalloc, in the module's own static device memory so
// that entry point never allocates.  257 counters (2,056 bytes); every GPU that loads the
// library keeps this array until the process exits.  All calls share it.
#define SE_NOALLOC_MAX_BINS 257
static __device__ __align__(256) unsigned long long se_noalloc_hist[SE_NOALLOC_MAX_BINS];

namespace {

__device__ __forceinline__ unsigned long long se_mix64(unsigned long long z) {
  // splitmix64 finaliser
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// digest = sum over cells of mix64(index * 2^32 + value)  (mod 2^64)
__global__ void __launch_bounds__(256) se_digest_kernel(const uint32_t* __restrict__ g, unsigned long long n,
                                                        unsigned long long* __restrict__ out) {
  unsigned long long acc = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    acc += se_mix64((i << 32) | g[i]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ unsigned long long part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
    atomicAdd(out, s);
  }
}

// counts[min(value, nbins-1)] += 1
__global__ void __launch_bounds__(256) se_histogram_kernel(const uint32_t* __restrict__ g, unsigned long long n,
                                                           int nbins, unsigned long long* __restrict__ counts) {
  __shared__ unsigned int local[257];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) local[i] = 0;
  __syncthreads();
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t v = g[i];
    atomicAdd(&local[v < (uint32_t)nbins ? v : (uint32_t)(nbins - 1)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (local[i]) atomicAdd(&counts[i], (unsigned long long)local[i]);
}

// out[i] = g[i] < nmat ? g[i] : 1 (the material id as the next frame reads it, unknown ids
// NULL) as one byte; four cells per thread and step (16-byte load, 4-byte store), then the
// tail.  nmat <= 256.
__global__ void __launch_bounds__(256) se_pack_ids_kernel(const uint32_t* __restrict__ g, uint8_t* __restrict__ out,
                                                          unsigned long long n, uint32_t nmat) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  const unsigned long long n4 = n / 4;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(g) + i);
    const uint32_t a = v.x < nmat ? v.x : 1u, b = v.y < nmat ? v.y : 1u, c = v.z < nmat ? v.z : 1u,
                   d = v.w < nmat ? v.w : 1u;
    reinterpret_cast<uint32_t*>(out)[i] = __byte_perm(__byte_perm(a, b, 0x0040), __byte_perm(c, d, 0x0040), 0x5410);
  }
  for (unsigned long long i = 4 * n4 + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t v = g[i];
    out[i] = (uint8_t)(v < nmat ? v : 1u);
  }
}

}  // namespace

namespace se::rt {

cudaError_t pack_ids_u8(const uint32_t* g, uint8_t* out, unsigned long long n, uint32_t nmat, cudaStream_t s) {
  if (nmat < 1 || nmat > 256) return cudaErrorInvalidValue;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  se_pack_ids_kernel<<<sms * 8, 256, 0, s>>>(g, out, n, nmat);
  return cudaGetLastError();
}

cudaError_t grid_digest(const uint32_t* g, unsigned long long n, unsigned long long* d_out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  se_digest_kernel<<<sms * 8, 256, 0, s>>>(g, n, d_out);
  return cudaGetLastError();
}

cudaError_t grid_histogram(const uint32_t* g, unsigned long long n, int nbins, unsigned long long* d_counts,
                           cudaStream_t s) {
  if (nbins < 1 || nbins > 257) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(d_counts, 0, sizeof(unsigned long long) * (size_t)nbins, s);
  if (e != cudaSuccess) return e;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  se_histogram_kernel<<<sms * 4, 256, 0, s>>>(g, n, nbins, d_counts);
  return cudaGetLastError();
}

int noalloc_max_bins() { return SE_NOALLOC_MAX_BINS; }

namespace {
// The driver's id of the calling thread's current context (cuCtxGetCurrent, cuCtxGetId),
// reached through the runtime's entry-point query, so the library still needs no link to
// the driver library.  False when the driver does not offer them.
bool current_context_id(unsigned long long* id) {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  void* ctx = nullptr;
  return get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, id) == 0;
}
}  // namespace

// The histogram of grid_histogram, counted in se_noalloc_hist instead of caller- or
// library-allocated memory.  The host must not pass the array's name to a kernel (in host
// code it is a stand-in, not a device address), so its device address is looked up with
// the device current (set-up on the first call on a device) and cached per device, tagged
// with the id of the context it was looked up in: after a device reset (a new primary
// context) the next call looks it up again.  The counters are cleared on the stream
// before each use; the results are copied to host_counts and the stream is synchronized
// before returning.
cudaError_t histogram_noalloc(const uint32_t* g, unsigned long long n, int nbins, unsigned long long* host_counts,
                              cudaStream_t s) {
  constexpr int kMaxDevices = 64;
  struct Slot {
    unsigned long long* addr = nullptr;
    unsigned long long ctx_id = 0;
  };
  static Slot slots[kMaxDevices];
  static std::mutex mu;
  if (nbins < 1 || nbins > SE_NOALLOC_MAX_BINS) return cudaErrorInvalidValue;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  e = cudaSetDevice(dev);  // makes the device's primary context current on this thread
  if (e != cudaSuccess) return e;
  unsigned long long ctx = 0;
  const bool have_ctx = current_context_id(&ctx);
  unsigned long long* p = nullptr;
  {
    std::lock_guard<std::mutex> lock(mu);
    Slot& sl = slots[dev];
    if (!sl.addr || (have_ctx && sl.ctx_id != ctx)) {
      void* q = nullptr;
      e = cudaGetSymbolAddress(&q, se_noalloc_hist);
      if (e != cudaSuccess) return e;
      sl.addr = static_cast<unsigned long long*>(q);
      sl.ctx_id = have_ctx ? ctx : 0;
    }
    p = sl.addr;
  }
  e = cudaMemsetAsync(p, 0, sizeof(unsigned long long) * (size_t)nbins, s);
  if (e != cudaSuccess) return e;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  se_histogram_kernel<<<sms * 4, 256, 0, s>>>(g, n, nbins, p);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(host_counts, p, sizeof(unsigned long long) * (size_t)nbins, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

}  // namespace se::rt
