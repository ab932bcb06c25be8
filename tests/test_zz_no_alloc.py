"""The allocation-free MBR decode entry point (puck_mbr_decode_static).

Callers that cannot allocate device memory where they decode -- a host running
inside a device arena its own pool carved out, a serving loop that keeps the
CUDA allocator off its request path, or work issued while another framework
captures the stream -- use this entry point with buffers they already own.  It
must produce exactly the trees of puck_parse's MBR path for the same per-cell
marginals, on consecutive calls that reuse its fixed scratch array.

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


def test_static_mbr_decode_matches_parse_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    levels = split_levels("real", "medium")
    sents = split_sentences(32, seed=12)
    P = CLParser(write_grz(levels, "split_medium_real"), max_alloc_size=4 << 30, decode="mbr")
    words, offsets, lens = pack_sentences(sents)
    ref_nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    decode = P.debug_copy(1, "mbr")          # per cell {best marginal, coarse symbol bits}
    iscale = P.debug_copy(0, "iscale")
    oscale = P.debug_copy(0, "oscale")
    L = _lib.load()
    L.puck_mbr_decode_static.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    L.puck_mbr_decode_static.restype = ctypes.c_int32
    cell_off = _cells([int(n) for n in lens])
    node_off = np.zeros(len(lens) + 1, np.int64)
    np.cumsum(2 * lens - 1, out=node_off[1:])
    stream = torch.cuda.current_stream()

    def call(first, last):
        c0, c1 = cell_off[first], cell_off[last]
        d = torch.from_numpy(np.ascontiguousarray(decode[c0:c1])).cuda()
        i = torch.from_numpy(np.ascontiguousarray(iscale[c0:c1])).cuda()
        o = torch.from_numpy(np.ascontiguousarray(oscale[c0:c1])).cuda()
        ln = np.ascontiguousarray(lens[first:last], np.int32)
        out = torch.full((int(node_off[last] - node_off[first]), 4), -7, dtype=torch.int32, device="cuda")
        rc = L.puck_mbr_decode_static(d.data_ptr(), i.data_ptr(), o.data_ptr(), ln.ctypes.data, len(ln),
                                      out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        return out.cpu().numpy()

    # two calls in a row through the same fixed scratch: all sentences, then a
    # later subset whose tables land where the first call left its own
    got_all = call(0, len(lens))
    got_sub = call(5, 17)
    assert np.array_equal(got_all, ref_nodes)
    assert np.array_equal(got_sub, ref_nodes[node_off[5]:node_off[17]])


def test_static_mbr_decode_rejects_oversized_calls():
    L = _lib.load()
    L.puck_mbr_decode_static.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    L.puck_mbr_decode_static.restype = ctypes.c_int32
    ln = np.full(4000, 40, np.int32)          # 3 * 41^2 * 4000 floats > the fixed capacity
    dummy = ctypes.c_void_p(16)               # never dereferenced: the size check fails first
    rc = L.puck_mbr_decode_static(dummy, None, None, ln.ctypes.data, len(ln), dummy, None)
    assert rc == 6 and "split the call" in _lib.last_error()
    bad = np.array([3, 0, 5], np.int32)
    assert L.puck_mbr_decode_static(dummy, None, None, bad.ctypes.data, 3, dummy, None) == 6
