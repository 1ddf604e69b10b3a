"""ctypes binding of libsandengine_gb300.so (the C ABI in include/sandengine.h).

The library is built in-tree by ``python -m sandengine_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU or Python fallback for the simulation path.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsandengine_gb300.so")

# status codes (include/sandengine.h)
SE_OK = 0
STATUS_NAMES = {
    1: "InvalidArgument", 2: "MissingField", 3: "InvalidType", 4: "NotFound", 5: "NotRecognized",
    6: "Yaml", 7: "Panic", 8: "Glsl", 9: "Unsupported", 10: "Compile", 11: "Cuda", 12: "OutOfMemory",
    13: "BufferTooSmall", 14: "NotCompiled", 15: "Budget", 16: "Timeout", 17: "Cancelled",
}
PARSE_KINDS = {"MissingField", "InvalidType", "NotFound", "NotRecognized", "Yaml", "Panic", "Glsl",
               "Unsupported"}


class SandengineError(RuntimeError):
    """A failed C ABI call: ``code`` is the status, ``kind`` its name."""

    def __init__(self, code: int, message: str):
        self.code = code
        self.kind = STATUS_NAMES.get(code, str(code))
        super().__init__(f"[{self.kind}] {message}")


class ParseError(SandengineError):
    """Rule-language error; ``kind`` is the reference's ParsingErr kind
    (MissingField, InvalidType, NotFound, NotRecognized) or Yaml / Panic / Glsl /
    Unsupported."""


class SeModification(ctypes.Structure):
    """SimModification (sandengine-core/src/simulation.rs:45-56), 32 bytes."""
    _fields_ = [("position", ctypes.c_int32 * 2), ("mod_shape", ctypes.c_int32),
                ("mod_size", ctypes.c_int32), ("mod_matID", ctypes.c_int32),
                ("_pad4", ctypes.c_int32 * 3)]


assert ctypes.sizeof(SeModification) == 32

_P = ctypes.c_void_p
_I = ctypes.c_int
_SIGS = {
    "se_last_error": ([], ctypes.c_char_p),
    "se_version": ([], _I),
    "se_ruleset_parse": ([ctypes.c_char_p, ctypes.POINTER(_P)], _I),
    "se_ruleset_parse_path": ([ctypes.c_char_p, ctypes.POINTER(_P)], _I),
    "se_ruleset_text": ([_P, _I, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], _I),
    "se_ruleset_compile": ([_P], _I),
    "se_ruleset_num_materials": ([_P, ctypes.POINTER(_I)], _I),
    "se_ruleset_material_id": ([_P, ctypes.c_char_p, ctypes.POINTER(_I)], _I),
    "se_world_set_light": ([_P, _I], _I),
    "se_world_read_grid_overlapped": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_read_grid_u8_overlapped": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_read_pass_timing": ([_P, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                   ctypes.POINTER(ctypes.c_longlong)], _I),
    "se_world_get_light": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_set_light_field": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_render_color": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_render_color_device": ([_P, ctypes.POINTER(_P)], _I),
    "se_world_composite": ([_P, _P, _I, _I, _P, ctypes.c_size_t], _I),
    "se_world_composite_device": ([_P, _P, _I, _I, ctypes.POINTER(_P)], _I),
    "se_world_create_band": ([_P, _I, _I, _I, _I, _I, ctypes.POINTER(_P)], _I),
    "se_world_band_info": ([_P] + [ctypes.POINTER(_I)] * 4, _I),
    "se_world_copy_rows": ([_P, _I, _I, _P, _I], _I),
    "se_ruleset_set_checked": ([_P, _I], _I),
    "se_ruleset_check_word": ([_P, ctypes.POINTER(ctypes.c_uint), _I], _I),
    "se_ruleset_table": ([_P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_ulonglong),
                          ctypes.POINTER(ctypes.c_ulonglong)], _I),
    "se_ruleset_free": ([_P], None),
    "se_world_create": ([_P, _I, _I, ctypes.POINTER(_P)], _I),
    "se_world_destroy": ([_P], None),
    "se_world_set_stream": ([_P, _P], _I),
    "se_world_get_stream": ([_P, ctypes.POINTER(_P)], _I),
    "se_world_set_steps_per_launch": ([_P, _I], _I),
    "se_world_set_grid": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_get_grid": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_set_grid_async": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_get_grid_async": ([_P, _P, ctypes.c_size_t], _I),
    "se_world_device_grid": ([_P, ctypes.POINTER(_P)], _I),
    "se_world_set_frame": ([_P, ctypes.c_int32], _I),
    "se_world_get_frame": ([_P, ctypes.POINTER(ctypes.c_int32)], _I),
    "se_world_step": ([_P, _I, _P, _I], _I),
    "se_world_synchronize": ([_P], _I),
    "se_world_digest": ([_P, ctypes.POINTER(ctypes.c_uint64)], _I),
    "se_world_histogram": ([_P, _P, _I], _I),
    "se_world_set_timing": ([_P, _I], _I),
    "se_world_autotune": ([_P, _I, ctypes.POINTER(_I)], _I),
    "se_world_set_tile": ([_P, _I, _I, _I], _I),
    "se_world_get_tile": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "se_grid_histogram_noalloc": ([_P, ctypes.c_uint64, _I, _P, _P], _I),
    "se_batch_create": ([_P, _I, _P, _P, ctypes.POINTER(_P)], _I),
    "se_batch_destroy": ([_P], None),
    "se_batch_set_grid": ([_P, _I, _P, ctypes.c_size_t], _I),
    "se_batch_get_grid": ([_P, _I, _P, ctypes.c_size_t], _I),
    "se_batch_set_frame": ([_P, _I, ctypes.c_int32], _I),
    "se_batch_get_frame": ([_P, _I, ctypes.POINTER(ctypes.c_int32)], _I),
    "se_batch_step": ([_P, _I], _I),
    "se_batch_step_plain": ([_P, _I], _I),
    "se_batch_autotune": ([_P, _I, ctypes.POINTER(_I)], _I),
    "se_batch_set_steps_per_launch": ([_P, _I], _I),
    "se_batch_set_resident_limit": ([_P, ctypes.c_size_t], _I),
    "se_batch_synchronize": ([_P], _I),
    "se_batch_get_stream": ([_P, ctypes.POINTER(_P)], _I),
    "se_batch_info": ([_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_longlong),
                       ctypes.POINTER(_I)], _I),
    "se_server_create": ([_P, ctypes.c_longlong, ctypes.POINTER(_P)], _I),
    "se_server_destroy": ([_P], None),
    "se_server_set_frames_per_iteration": ([_P, _I], _I),
    "se_server_open_session": ([_P, _I, _I, _P, ctypes.c_int32, ctypes.POINTER(_I)], _I),
    "se_server_close_session": ([_P, _I], _I),
    "se_server_submit": ([_P, _I, _I, _P, _I, ctypes.c_double, ctypes.POINTER(_I)], _I),
    "se_server_run": ([_P, _I], _I),
    "se_server_start": ([_P, _I], _I),
    "se_server_stop": ([_P], _I),
    "se_server_wait": ([_P, _I, ctypes.c_double, ctypes.POINTER(ctypes.c_double)], _I),
    "se_server_poll": ([_P, _I, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double)], _I),
    "se_server_stats_get": ([_P, _P], _I),
    "se_server_cancel": ([_P, _I], _I),
    "se_server_request_latency": ([_P, _I, ctypes.POINTER(ctypes.c_double)], _I),
    "se_server_get_grid": ([_P, _I, _P, ctypes.c_size_t], _I),
    "se_server_get_frame": ([_P, _I, ctypes.POINTER(ctypes.c_int32)], _I),
    "se_snapshot_info": ([ctypes.c_char_p, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_int32)],
                         _I),
    "se_world_save": ([_P, ctypes.c_char_p], _I),
    "se_world_load": ([_P, ctypes.c_char_p], _I),
    "se_server_save_session": ([_P, _I, ctypes.c_char_p], _I),
    "se_server_open_session_from": ([_P, ctypes.c_char_p, ctypes.POINTER(_I)], _I),
    "se_world_peek_timing_frames": ([_P, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)],
                                    _I),
    "se_world_read_timing": ([_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                              ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)], _I),
}

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded library (raises ImportError when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m sandengine_gb300.build` "
                              f"(the simulation path has no fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc: int, parse: bool = False) -> None:
    if rc != SE_OK:
        msg = lib().se_last_error().decode(errors="replace")
        kind = STATUS_NAMES.get(rc, "")
        if parse or kind in PARSE_KINDS:
            raise ParseError(rc, msg)
        raise SandengineError(rc, msg)
