"""The allocation-free MBR decode entry point (puck_mbr_decode_static).

Callers that cannot allocate device memory where they decode -- a host running
inside a device arena its own pool carved out, or a serving loop that keeps
the CUDA allocator off its request path -- use this entry point with buffers
they already own.  It must produce exactly the trees of puck_parse's MBR path
for the same per-cell marginals, on consecutive calls that reuse its fixed
scratch array, with the coarse level's scales (a Real fine level) and without
them (a LogSum fine level).

This file is collected last so that a run stopping at the first failure has
run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from helpers import split_levels, split_sentences, write_grz
from puck_gb300 import _lib
from puck_gb300.parser import CLParser, pack_sentences

pytestmark = pytest.mark.gpu


def _cells(lengths):
    off = np.zeros(len(lengths) + 1, np.int64)
    np.cumsum([n * (n + 1) for n in lengths], out=off[1:])
    return off


def _bind():
    L = _lib.load()
    L.puck_mbr_decode_static.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    L.puck_mbr_decode_static.restype = ctypes.c_int32
    return L


def _consecutive_calls(semiring, name):
    """puck_parse's MBR trees, then the same decode through the static entry
    point on two calls in a row: every sentence, then a later subset whose
    tables land where the first call left its own."""
    torch = pytest.importorskip("torch")
    levels = split_levels(semiring, "medium")
    sents = split_sentences(32, seed=12)
    P = CLParser(write_grz(levels, name), max_alloc_size=4 << 30, decode="mbr")
    words, offsets, lens = pack_sentences(sents)
    ref_nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    decode = P.debug_copy(1, "mbr")          # per cell {best marginal, coarse symbol bits}
    scaled = semiring == "real"
    iscale = P.debug_copy(0, "iscale") if scaled else None
    oscale = P.debug_copy(0, "oscale") if scaled else None
    L = _bind()
    cell_off = _cells([int(n) for n in lens])
    node_off = np.zeros(len(lens) + 1, np.int64)
    np.cumsum(2 * lens - 1, out=node_off[1:])
    stream = torch.cuda.current_stream()

    def call(first, last):
        c0, c1 = cell_off[first], cell_off[last]
        d = torch.from_numpy(np.ascontiguousarray(decode[c0:c1])).cuda()
        i = torch.from_numpy(np.ascontiguousarray(iscale[c0:c1])).cuda() if scaled else None
        o = torch.from_numpy(np.ascontiguousarray(oscale[c0:c1])).cuda() if scaled else None
        ln = np.ascontiguousarray(lens[first:last], np.int32)
        out = torch.full((int(node_off[last] - node_off[first]), 4), -7, dtype=torch.int32, device="cuda")
        rc = L.puck_mbr_decode_static(d.data_ptr(), i.data_ptr() if scaled else None,
                                      o.data_ptr() if scaled else None, ln.ctypes.data, len(ln),
                                      out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        return out.cpu().numpy()

    got_all = call(0, len(lens))
    got_sub = call(5, 17)
    assert np.array_equal(got_all, ref_nodes)
    assert np.array_equal(got_sub, ref_nodes[node_off[5]:node_off[17]])


def test_static_mbr_decode_matches_parse_on_consecutive_calls():
    """Real fine level: the decode rescales marginals by the coarse scales."""
    _consecutive_calls("real", "split_medium_real")


def test_static_mbr_decode_unscaled_matches_parse():
    """LogSum fine level: no scales (iscale = oscale = NULL)."""
    _consecutive_calls("logsum", "split_medium_logsum")


def test_static_mbr_decode_rejects_oversized_calls():
    torch = pytest.importorskip("torch")
    L = _bind()
    # more sentences than the fixed scratch holds: refused before anything is
    # read, whatever the pointers
    many = np.full(65537, 1, np.int32)
    fake = ctypes.c_void_p(16)
    rc = L.puck_mbr_decode_static(fake, None, None, many.ctypes.data, len(many), fake, None)
    assert rc == 6 and "sentences in one call" in _lib.last_error()
    # tables larger than the scratch (3 * 41^2 * 4000 floats): real buffers of
    # the full size, so that the call could not fault even if it were accepted
    ln = np.full(4000, 40, np.int32)
    d = torch.zeros((4000 * 40 * 41, 2), dtype=torch.float32, device="cuda")
    out = torch.zeros((4000 * 79, 4), dtype=torch.int32, device="cuda")
    rc = L.puck_mbr_decode_static(d.data_ptr(), None, None, ln.ctypes.data, len(ln), out.data_ptr(), None)
    assert rc == 6 and "split the call" in _lib.last_error()
    bad = np.array([3, 0, 5], np.int32)
    assert L.puck_mbr_decode_static(d.data_ptr(), None, None, bad.ctypes.data, 3, out.data_ptr(), None) == 6
    # a decode buffer that is not 8-byte aligned
    assert L.puck_mbr_decode_static(d.data_ptr() + 4, None, None, ln.ctypes.data, 1, out.data_ptr(), None) == 6
    assert "aligned" in _lib.last_error()
