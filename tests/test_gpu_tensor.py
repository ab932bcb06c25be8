"""The tcgen05 BF16 -> FP32 tile product (puck_tc_selftest) against a host
product of the same BF16 values.

BF16 x BF16 products are exact in FP32, so the only difference is the FP32
accumulation order over k; the tolerance is 1e-5 relative to the sum of
absolute terms.
"""
import ctypes

import numpy as np
import pytest

from puck_gb300 import _lib

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    """Round-to-nearest-even FP32 -> BF16 bit patterns."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("k,n", [(16, 16), (64, 32), (112, 16), (240, 48), (256, 256)])
def test_tc_tile_product_matches_host(k, n):
    L = _lib.load()
    rng = np.random.default_rng(k * 1000 + n)
    a = to_bf16_bits(rng.standard_normal((128, k)).astype(np.float32))
    b = to_bf16_bits((rng.random((n, k)) * np.exp(-3 * rng.random((n, k)))).astype(np.float32))
    d = np.zeros((128, n), np.float32)
    st = L.puck_tc_selftest(0, k, n, a.ctypes.data, b.ctypes.data, d.ctypes.data)
    assert st == 0, _lib.last_error()
    A, B = from_bf16_bits(a).astype(np.float64), from_bf16_bits(b).astype(np.float64)
    ref = A @ B.T
    scale = np.abs(A) @ np.abs(B).T
    err = np.abs(d - ref) / np.maximum(scale, 1e-30)
    assert err.max() < 1e-5, (err.max(), np.unravel_index(err.argmax(), err.shape))



# --- the sum-product inside pass on tensor cores ------------------------------
# BF16 operands (outer products and rule weights) with FP32 accumulation:
# each product carries two BF16 roundings (relative 2^-9 each).  The stated
# tolerances: log Z within LOGZ_RTOL_TC of the FP64 oracle (relative; the
# largest error seen over 500 bench sentences was 3.2e-4, median 6e-6), the
# inside chart within a median relative 4e-3 of the FP32 path, and MBR trees
# equal to the FP32 path's for at least 90% of sentences (the rest differ at
# near-ties).
LOGZ_RTOL_TC = 5e-4


def _fp64_logz(levels, sents):
    import oracle
    r32 = oracle.run(levels, sents, mode="partitions")
    masks, isc, osc = r32.masks(0)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sents, precision=64)
    r64.set_final_masks(masks, isc, osc)
    assert r64.run("partitions") == 0
    return r64.partitions().astype(np.float64), masks


@pytest.mark.parametrize("size,n,seed", [("medium", 40, 61), ("wide", 24, 62), ("c1", 16, 63)])
def test_tc_inside_logz_vs_fp64(size, n, seed):
    from helpers import split_levels, split_sentences, write_grz
    from puck_gb300.parser import CLParser, pack_sentences
    levels = split_levels("real", size)
    kw = dict(n_words=40000, mean=23, hi=40) if size == "c1" else (dict(n_words=400, mean=24, hi=40) if size == "wide" else {})
    sents = split_sentences(n, seed=seed, **kw)
    words, offsets, _ = pack_sentences(sents)
    path = write_grz(levels, f"split_{size}_real")
    T = CLParser(path, max_alloc_size=4 << 30, tensor_cores=True)
    on, why = T.tensor_cores(len(levels) - 1)
    assert on, why
    F = CLParser(path, max_alloc_size=4 << 30)
    assert F.tensor_cores(len(levels) - 1)[0] is False
    z, st = T.partitions_ids(words, offsets)
    assert (st == 0).all()
    zf, _ = F.partitions_ids(words, offsets)
    z64, masks = _fp64_logz(levels, sents)
    assert np.array_equal(T.debug_copy(0, "masks"), masks)
    rel = np.abs(z.astype(np.float64) - z64) / np.abs(z64)
    relf = np.abs(zf.astype(np.float64) - z64) / np.abs(z64)
    print(f"{size}: log Z rel err vs FP64: tensor cores max {rel.max():.2e} median {np.median(rel):.2e}; "
          f"FP32 max {relf.max():.2e}")
    assert rel.max() < LOGZ_RTOL_TC, rel.max()
    gi, fi = T.debug_copy(1, "inside"), F.debug_copy(1, "inside")
    nz = np.abs(fi) > 1e-30
    med = np.median(np.abs(gi - fi)[nz] / np.abs(fi)[nz])
    print(f"{size}: inside chart median rel diff vs FP32 {med:.2e}")
    assert med < 4e-3
    # exact zeros stay exact (pruned cells, gated targets, uncovered rows)
    assert np.array_equal(gi == 0, fi == 0)


def test_tc_mbr_trees_close_to_fp32_path():
    from helpers import split_levels, split_sentences, write_grz
    from puck_gb300.parser import CLParser, pack_sentences
    levels = split_levels("real", "medium")
    sents = split_sentences(48, seed=64)
    words, offsets, lens = pack_sentences(sents)
    path = write_grz(levels, "split_medium_real")
    nt, st = CLParser(path, max_alloc_size=4 << 30, tensor_cores=True).parse_ids(words, offsets)
    nf, _ = CLParser(path, max_alloc_size=4 << 30).parse_ids(words, offsets)
    assert (st == 0).all()
    same, o = 0, 0
    for L in lens:
        k = max(2 * L - 1, 0)
        same += np.array_equal(nt[o:o + k, :3], nf[o:o + k, :3])
        o += k
    assert same >= 0.9 * len(lens), (same, len(lens))


def test_tensor_cores_option_on_a_viterbi_level_keeps_the_fp32_path():
    """tensor_cores on a Viterbi cascade: the level reports why the form does
    not apply, and the parse is the oracle's, bit for bit."""
    import oracle
    from helpers import split_levels, split_sentences, write_grz
    from puck_gb300.parser import CLParser, pack_sentences
    levels = split_levels("viterbi", "small")
    sents = split_sentences(16, seed=65, n_words=300, mean=12, hi=30)
    words, offsets, _ = pack_sentences(sents)
    P = CLParser(write_grz(levels, "split_small"), max_alloc_size=2 << 30, tensor_cores=True)
    on, why = P.tensor_cores(len(levels) - 1)
    assert not on and "sum-product" in why
    on0, why0 = P.tensor_cores(0)  # only the parsing level is considered
    assert not on0 and "coarse level" in why0
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    assert np.array_equal(nodes, oracle.run(levels, sents, mode="parse").trees())
