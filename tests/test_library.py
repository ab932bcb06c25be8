"""The C-ABI library: builds, loads, exports what include/puck_gpu.h declares,
and reads grammar artifacts on the host (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from puck_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    src = open(os.path.join(ROOT, "include", "puck_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(puck_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(names) >= set(_lib.EXPORTS)


def test_options_layout_and_defaults():
    """The ctypes mirror of puck_options has the C layout (40 bytes, no
    padding after tensor_cores) and the library's defaults."""
    L = _lib.load()
    assert ctypes.sizeof(_lib.Options) == 40
    assert _lib.Options.tensor_cores.offset == 36
    opt = _lib.Options()
    opt.tensor_cores = 7
    L.puck_default_options(ctypes.byref(opt))
    assert opt.tensor_cores == 0 and opt.use_graphs == 0 and abs(opt.prune_threshold + 9.0) < 1e-6


def test_tc_selftest_rejects_bad_shapes_without_a_device_call():
    L = _lib.load()
    z = np.zeros(128 * 32, np.uint16)
    d = np.zeros(128 * 32, np.float32)
    for k, n in ((24, 16), (16, 8), (0, 16), (272, 16), (16, 272)):
        assert L.puck_tc_selftest(0, k, n, z.ctypes.data, z.ctypes.data, d.ctypes.data) == 6


def test_grammar_load_and_queries_on_host():
    L = _lib.load()
    st = ctypes.c_int32(-1)
    g = L.puck_grammar_load(os.path.join(GOLDEN, "split_cascade_viterbi.grz").encode(), ctypes.byref(st))
    assert g and st.value == 0
    try:
        assert L.puck_grammar_num_levels(g) == 2
        info = (ctypes.c_int32 * 8)()
        assert L.puck_grammar_level_info(g, 1, info) == 0
        semiring, n_nt, n_t, cs, ms, nc, root, nw = list(info)
        assert semiring == 0 and cs % 32 == 0 and cs >= max(n_nt, n_t) and nw == 300
        assert L.puck_grammar_word_id(g, b"w17") == 17
        assert L.puck_grammar_word_id(g, b"no-such-word") == -1
        assert L.puck_grammar_level_info(g, 5, info) == 6
    finally:
        L.puck_grammar_free(g)


def test_bad_artifacts_fail_cleanly(tmp_path):
    L = _lib.load()
    st = ctypes.c_int32(0)
    assert not L.puck_grammar_load(str(tmp_path / "missing.grz").encode(), ctypes.byref(st))
    assert st.value == 2 and "cannot open" in _lib.last_error()
    p = tmp_path / "trunc.grz"
    data = open(os.path.join(GOLDEN, "tiny_pcfg_viterbi.grz"), "rb").read()
    p.write_bytes(data[: len(data) // 2])
    assert not L.puck_grammar_load(str(p).encode(), ctypes.byref(st))
    assert st.value == 2
    import zipfile
    q = tmp_path / "deflated.grz"
    with zipfile.ZipFile(q, "w", compression=zipfile.ZIP_DEFLATED) as z:
        z.writestr("parserNames", "parser-0")
        z.writestr("parser-0/header", "semiring viterbi\n")
    assert not L.puck_grammar_load(str(q).encode(), ctypes.byref(st))
    assert st.value == 2


def test_build_flags_target_sm103a():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
