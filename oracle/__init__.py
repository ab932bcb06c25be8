"""CPU oracle for the chart-parsing hot path -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_build/libpuck_oracle.so`` (a C++ restatement of the
reference's span loops, work queues and generated kernels, see
``puck_oracle.cc``) and drives it from compiled grammar levels.  Only the
test-suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this package, always as the checker / baseline and never as the product.

Parity status: UNPINNED -- the reference cannot run here and holds no golden
vectors for this path (see the header of ``puck_oracle.cc``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpuck_oracle.so")
SRC = os.path.join(HERE, "puck_oracle.cc")

JOB_IDS = ("in_NN", "in_NT", "in_TN", "in_TT", "out_L_NN", "out_R_NN", "out_L_NT", "out_R_NT",
           "out_L_TN", "out_R_TN", "out_L_TT", "out_R_TT")
UJOB_IDS = ("in_NU", "in_TU", "out_NU", "out_TU")
SEMI = {"viterbi": 0, "real": 1, "logsum": 2}

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
                               "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        I = ctypes.c_int
        L.po_level_new.restype = P
        L.po_level_new.argtypes = [I, I, I, I, I, I, I, P, P]
        L.po_level_set_job.argtypes = [P, I, I, P, P, P, P, I, P, I, P, P, P]
        L.po_level_set_ujob.argtypes = [P, I, I, P, P, P]
        L.po_level_set_lexicon.argtypes = [P, I, P, P, P]
        L.po_level_set_viterbi.argtypes = [P, I, P, I, P, P, P]
        L.po_level_free.argtypes = [P]
        L.po_run_new.restype = P
        L.po_run_new.argtypes = [I, P, I, P, P, I, I]
        L.po_run_set_final_masks.argtypes = [P, P, P, P]
        L.po_run.argtypes = [P, I]
        L.po_run.restype = I
        L.po_run_num_cells.argtypes = [P]
        L.po_run_num_cells.restype = ctypes.c_int64
        L.po_run_num_nodes.argtypes = [P]
        L.po_run_num_nodes.restype = ctypes.c_int64
        L.po_run_get_chart.argtypes = [P, I, I, P]
        L.po_run_get_chart.restype = I
        L.po_run_get_chart64.argtypes = [P, I, I, P]
        L.po_run_get_chart64.restype = I
        L.po_run_get_masks.argtypes = [P, I, P, P, P]
        L.po_run_get_masks.restype = I
        L.po_run_get_partition_scales.argtypes = [P, I, P]
        L.po_run_corner_drops.argtypes = [P, I]
        L.po_run_corner_drops.restype = ctypes.c_int64
        L.po_run_rule_apps.argtypes = [P, I, I]
        L.po_run_rule_apps.restype = ctypes.c_int64
        L.po_run_get_trees.argtypes = [P, P]
        L.po_run_get_partitions.argtypes = [P, P]
        L.po_run_get_mbr.argtypes = [P, P, P]
        L.po_run_free.argtypes = [P]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleLevel:
    """A grammar level copied into the oracle.

    Accepts a compiled level (``puck_gb300.grammar.CompiledLevel``) or the
    header + arrays of a ``grammar.grz`` level (``puck_gb300.grz.LevelInfo``
    read with ``load_arrays=True``); both go through the artifact's array
    layout, so the oracle reads exactly what the device library reads.
    """

    def __init__(self, level):
        from puck_gb300 import grz as _grz
        L = lib()
        if hasattr(level, "jobs"):
            arrays = _grz.level_arrays(level)
            hdr = dict(semiring=level.semiring, n_nt=level.n_nt, n_t=level.n_t, cell_size=level.cell_size,
                       mask_size=level.mask_size, n_coarse=level.n_coarse, root=level.root)
        else:
            arrays = level.arrays
            hdr = dict(semiring=level.semiring, n_nt=level.n_nt, n_t=level.n_t, cell_size=level.cell_size,
                       mask_size=level.mask_size, n_coarse=level.n_coarse, root=level.root)
        self.hdr = hdr
        self.cell_size = hdr["cell_size"]
        self.mask_size = hdr["mask_size"]
        keep = self._keep = []

        def arr(name, dt):
            a = np.ascontiguousarray(arrays[name], dtype=dt)
            keep.append(a)
            return a

        self.h = L.po_level_new(SEMI[hdr["semiring"]], hdr["n_nt"], hdr["n_t"], hdr["cell_size"],
                                hdr["mask_size"], hdr["n_coarse"], hdr["root"],
                                _p(arr("nt_coarse", np.int32)), _p(arr("t_coarse", np.int32)))
        for ji, name in enumerate(JOB_IDS):
            tgt = arr(f"{name}/tgt", np.int32)
            seg_bits = arr(f"{name}/seg_bits", np.int32)
            sub_seg = arr(f"{name}/sub_seg", np.int32)
            sub_off = arr(f"{name}/sub_off", np.int32)
            sub_rules = arr(f"{name}/sub_rules", np.int32)
            ia = arr(f"{name}/ia", np.int32)
            ib = arr(f"{name}/ib", np.int32)
            # the generator sorts each sub-segment by (parent, left, right)
            sorted_rules = sub_rules.copy()
            for k in range(sub_seg.shape[0]):
                r = sub_rules[sub_off[k]:sub_off[k + 1]]
                sorted_rules[sub_off[k]:sub_off[k + 1]] = r[np.lexsort((ib[r], ia[r], tgt[r]))]
            keep.append(sorted_rules)
            nseg = seg_bits.shape[0] // max(1, hdr["mask_size"])
            L.po_level_set_job(self.h, ji, tgt.shape[0], _p(tgt), _p(ia), _p(ib),
                               _p(arr(f"{name}/score", np.float32)), nseg, _p(seg_bits),
                               sub_seg.shape[0], _p(sub_seg), _p(sub_off), _p(sorted_rules))
        for ui, name in enumerate(UJOB_IDS):
            tgt = arr(f"{name}/tgt", np.int32)
            L.po_level_set_ujob(self.h, ui, tgt.shape[0], _p(tgt), _p(arr(f"{name}/osrc", np.int32)),
                                _p(arr(f"{name}/score", np.float32)))
        lex_off = arr("lex_off", np.int64)
        L.po_level_set_lexicon(self.h, lex_off.shape[0] - 1, _p(lex_off), _p(arr("lex_term", np.int32)),
                               _p(arr("lex_score", np.float32)))
        v_off = arr("v_off", np.int32)
        v_score = arr("v_score", np.float32)
        L.po_level_set_viterbi(self.h, v_off.shape[0], _p(v_off), v_score.shape[0],
                               _p(arr("v_left", np.int32)), _p(arr("v_right", np.int32)), _p(v_score))

    def __del__(self):
        try:
            lib().po_level_free(self.h)
        except Exception:
            pass


MODES = {"parse": 0, "partitions": 1, "inside_outside": 2}


class OracleRun:
    """One oracle invocation over a list of sentences (one batch)."""

    def __init__(self, levels: Sequence[OracleLevel], sentences: Sequence[np.ndarray], threads: int = 0,
                 precision: int = 32):
        L = lib()
        self.levels = list(levels)
        self.lengths = np.asarray([len(s) for s in sentences], np.int64)
        self.word_off = np.zeros(len(sentences) + 1, np.int64)
        np.cumsum(self.lengths, out=self.word_off[1:])
        self.words = np.concatenate([np.asarray(s, np.int32) for s in sentences]) if sentences \
            else np.zeros(0, np.int32)
        self.words = np.ascontiguousarray(self.words, np.int32)
        hs = (ctypes.c_void_p * len(levels))(*[l.h for l in levels])
        self._hs = hs
        if threads <= 0:
            threads = os.cpu_count() or 1
        self.precision = precision
        self.h = L.po_run_new(len(levels), ctypes.cast(hs, ctypes.c_void_p), len(sentences),
                              _p(self.word_off), _p(self.words), threads, precision)
        tri = self.lengths * (self.lengths + 1) // 2
        self.cell_off = np.zeros(len(sentences) + 1, np.int64)
        np.cumsum(2 * tri, out=self.cell_off[1:])

    def set_final_masks(self, masks, iscale, oscale):
        L = lib()
        self._ext = [np.ascontiguousarray(masks, np.int32), np.ascontiguousarray(iscale, np.float32),
                     np.ascontiguousarray(oscale, np.float32)]
        L.po_run_set_final_masks(self.h, *[_p(a) for a in self._ext])

    def run(self, mode: str = "parse") -> int:
        return lib().po_run(self.h, MODES[mode])

    @property
    def num_cells(self) -> int:
        return int(lib().po_run_num_cells(self.h))

    def chart(self, level: int, which: str = "inside") -> Optional[np.ndarray]:
        cs = self.levels[level].cell_size
        if self.precision == 64:
            out = np.empty((self.num_cells, cs), np.float64)
            rc = lib().po_run_get_chart64(self.h, level, 0 if which == "inside" else 1, _p(out))
        else:
            out = np.empty((self.num_cells, cs), np.float32)
            rc = lib().po_run_get_chart(self.h, level, 0 if which == "inside" else 1, _p(out))
        return None if rc else out

    def masks(self, level: int):
        ms = self.levels[level].mask_size
        m = np.empty((self.num_cells, ms), np.int32)
        i = np.empty(self.num_cells, np.float32)
        o = np.empty(self.num_cells, np.float32)
        rc = lib().po_run_get_masks(self.h, level, _p(m), _p(i), _p(o))
        return None if rc else (m, i, o)

    def partition_scales(self, level: int) -> np.ndarray:
        out = np.empty(len(self.lengths), np.float64)
        lib().po_run_get_partition_scales(self.h, level, _p(out))
        return out

    def corner_drops(self, level: int) -> int:
        return int(lib().po_run_corner_drops(self.h, level))

    def rule_apps(self, level: int, which: str = "inside") -> int:
        """(rule, split) applications of the reference's binary queues in
        one pass of one level: rows queued per rule block times its rules."""
        return int(lib().po_run_rule_apps(self.h, level, 0 if which == "inside" else 1))

    def trees(self) -> np.ndarray:
        n = int(lib().po_run_num_nodes(self.h))
        out = np.empty((n, 4), np.int32)
        lib().po_run_get_trees(self.h, _p(out))
        return out

    def partitions(self) -> np.ndarray:
        out = np.empty(len(self.lengths), np.float32)
        lib().po_run_get_partitions(self.h, _p(out))
        return out

    def mbr_cells(self):
        s = np.empty(self.num_cells, np.float32)
        y = np.empty(self.num_cells, np.int32)
        lib().po_run_get_mbr(self.h, _p(s), _p(y))
        return s, y

    def __del__(self):
        try:
            lib().po_run_free(self.h)
        except Exception:
            pass


def run(compiled_levels, sentences, mode="parse", threads=0, precision=32) -> OracleRun:
    levels = [OracleLevel(c) for c in compiled_levels]
    r = OracleRun(levels, sentences, threads=threads, precision=precision)
    rc = r.run(mode)
    if rc != 0:
        raise RuntimeError(f"oracle run failed with code {rc}")
    return r
