"""ctypes binding of libpuck_gb300.so (the C ABI declared in include/puck_gpu.h).

The library is built in-tree (``puck_gb300/_build``).  There is no CPU
fallback: if the shared object cannot be built or loaded, every entry point
raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

STATUS = {0: "OK", 1: "OOM", 2: "BAD_GRAMMAR", 3: "SENT_TOO_LONG", 4: "OOV", 5: "DEVICE_TIMEOUT",
          6: "INVALID_ARG", 7: "CUDA", 8: "INTERNAL", 9: "EMPTY"}


class PuckError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Options(ctypes.Structure):
    _fields_ = [("mem_bytes", ctypes.c_int64), ("device", ctypes.c_int32), ("profile", ctypes.c_int32),
                ("decode", ctypes.c_int32), ("max_length", ctypes.c_int32),
                ("max_batch_sentences", ctypes.c_int32), ("prune_threshold", ctypes.c_float),
                ("use_graphs", ctypes.c_int32), ("tensor_cores", ctypes.c_int32), ("server_lanes", ctypes.c_int32)]


class TreeNode(ctypes.Structure):
    _fields_ = [("top", ctypes.c_int32), ("bot", ctypes.c_int32), ("width", ctypes.c_int32),
                ("score", ctypes.c_float)]


class Stats(ctypes.Structure):
    _fields_ = [("ms_total", ctypes.c_double), ("ms_inside", ctypes.c_double), ("ms_outside", ctypes.c_double),
                ("ms_masks", ctypes.c_double), ("ms_decode", ctypes.c_double), ("ms_h2d", ctypes.c_double),
                ("ms_d2h", ctypes.c_double), ("cells", ctypes.c_int64), ("cells_pruned", ctypes.c_int64),
                ("batches", ctypes.c_int64), ("kernel_launches", ctypes.c_int64), ("binary_work", ctypes.c_int64),
                ("ms_device", ctypes.c_double), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("ticks", ctypes.c_int64), ("kernel_launches", ctypes.c_int64), ("resident", ctypes.c_int64),
                ("resident_peak", ctypes.c_int64), ("arena_cells", ctypes.c_int64),
                ("arena_cells_peak", ctypes.c_int64), ("ms_device", ctypes.c_double),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]


EXPORTS = ("puck_default_options", "puck_default_compile_options", "puck_compile_grammar", "puck_grammar_load", "puck_grammar_free", "puck_grammar_num_levels",
           "puck_grammar_level_info", "puck_grammar_word_id", "puck_grammar_word_id_at", "puck_parser_create", "puck_parser_destroy",
           "puck_parse", "puck_partitions", "puck_inside_outside", "puck_debug_copy", "puck_debug_num_cells", "puck_debug_flat_check",
           "puck_parser_stats", "puck_parser_pass_ms", "puck_parser_level_work", "puck_parser_autotune", "puck_parser_flat_from", "puck_parser_set_flat_from", "puck_parser_tensor_cores", "puck_mbr_decode_static",
           "puck_tc_selftest", "puck_server_create",
           "puck_server_destroy", "puck_server_now_ns", "puck_server_submit", "puck_server_poll",
           "puck_server_take", "puck_server_get_stats", "puck_server_pass_ms", "puck_server_lanes", "puck_last_error")

_lib = None
_lock = threading.Lock()


def load(build: bool = True) -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(f"libpuck_gb300.so missing at {path}; run puck_gb300.build.build()")
        L = ctypes.CDLL(path)
        P, I, I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        L.puck_default_options.argtypes = [ctypes.POINTER(Options)]
        L.puck_grammar_load.restype = P
        L.puck_grammar_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(I)]
        L.puck_grammar_free.argtypes = [P]
        L.puck_grammar_num_levels.argtypes = [P]
        L.puck_grammar_num_levels.restype = I
        L.puck_grammar_level_info.argtypes = [P, I, ctypes.POINTER(I)]
        L.puck_grammar_level_info.restype = I
        L.puck_grammar_word_id.argtypes = [P, ctypes.c_char_p]
        L.puck_grammar_word_id.restype = I
        L.puck_grammar_word_id_at.argtypes = [P, ctypes.c_char_p, I]
        L.puck_grammar_word_id_at.restype = I
        L.puck_parser_create.restype = P
        L.puck_parser_create.argtypes = [P, ctypes.POINTER(Options), ctypes.POINTER(I)]
        L.puck_parser_destroy.argtypes = [P]
        L.puck_parse.argtypes = [P, P, P, I, P, P]
        L.puck_parse.restype = I
        L.puck_partitions.argtypes = [P, P, P, I, P, P]
        L.puck_partitions.restype = I
        L.puck_inside_outside.argtypes = [P, P, P, I]
        L.puck_inside_outside.restype = I
        L.puck_debug_copy.argtypes = [P, I, I, P, ctypes.c_size_t]
        L.puck_debug_copy.restype = I
        L.puck_debug_num_cells.argtypes = [P]
        L.puck_debug_num_cells.restype = I64
        L.puck_parser_stats.argtypes = [P, ctypes.POINTER(Stats)]
        L.puck_parser_stats.restype = I
        L.puck_parser_pass_ms.argtypes = [P, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(I64)]
        L.puck_parser_pass_ms.restype = I
        L.puck_parser_level_work.argtypes = [P, I, ctypes.POINTER(I64)]
        L.puck_parser_level_work.restype = I
        L.puck_parser_autotune.argtypes = [P, P, P, I, P]
        L.puck_parser_autotune.restype = I
        L.puck_parser_tensor_cores.argtypes = [P, I, ctypes.c_char_p, ctypes.c_size_t]
        L.puck_parser_tensor_cores.restype = I
        L.puck_debug_flat_check.argtypes = [P, I, I, I, ctypes.POINTER(ctypes.c_int64)]
        L.puck_debug_flat_check.restype = I
        L.puck_parser_flat_from.argtypes = [P, I]
        L.puck_parser_flat_from.restype = I
        L.puck_parser_set_flat_from.argtypes = [P, I, I]
        L.puck_parser_set_flat_from.restype = I
        L.puck_tc_selftest.argtypes = [I, I, I, P, P, P]
        L.puck_tc_selftest.restype = I
        L.puck_server_create.restype = P
        L.puck_server_create.argtypes = [P, ctypes.POINTER(Options), ctypes.POINTER(I)]
        L.puck_server_destroy.argtypes = [P]
        L.puck_server_now_ns.argtypes = []
        L.puck_server_now_ns.restype = I64
        L.puck_server_submit.argtypes = [P, P, P, I, P, P]
        L.puck_server_submit.restype = I
        L.puck_server_poll.argtypes = [P, P, I, I]
        L.puck_server_poll.restype = I
        L.puck_server_take.argtypes = [P, I64, P, I, ctypes.POINTER(I), ctypes.POINTER(I64)]
        L.puck_server_take.restype = I
        L.puck_server_get_stats.argtypes = [P, ctypes.POINTER(ServerStats)]
        L.puck_server_get_stats.restype = I
        L.puck_server_pass_ms.argtypes = [P, I, ctypes.POINTER(ctypes.c_double)]
        L.puck_server_pass_ms.restype = I
        L.puck_server_lanes.argtypes = [P]
        L.puck_server_lanes.restype = I
        L.puck_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        L.puck_last_error.restype = ctypes.c_size_t
        L.puck_default_compile_options.argtypes = [P]
        L.puck_compile_grammar.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P]
        L.puck_compile_grammar.restype = I
        L.puck_mbr_decode_static.argtypes = [P, P, P, P, I, P, P]
        L.puck_mbr_decode_static.restype = I
        _lib = L
        return L


def last_error() -> str:
    L = load()
    buf = ctypes.create_string_buffer(4096)
    L.puck_last_error(buf, 4096)
    return buf.value.decode("utf-8", "replace")


def check(status: int) -> None:
    if status != 0:
        raise PuckError(status, last_error())
