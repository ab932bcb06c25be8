"""GPU parity on long sentences (41-100 words) and on the LogSum semiring.

Sentences longer than 64 words give a cell more than 64 allowed splits, so
the pair-factored kernels walk their liveness chunks more than once (64
splits per chunk): the second chunk starts at split 64 and rebuilds the
pair list.  The outside range jobs of the first cells of such a sentence
also span more than 64 splits.  Viterbi charts, masks and trees must be
bit-identical to the oracle; sum-product log partitions must lie within the
stated tolerance of the FP64 oracle.
"""
import numpy as np
import pytest

import oracle
from helpers import node_blocks, split_levels, write_grz
from puck_gb300.parser import CLParser, pack_sentences

pytestmark = pytest.mark.gpu

# log partition against FP64, relative: Real semiring (FP32 sums of scaled
# products) and LogSum (FP32 log-add-exp, one rounding of log1p(exp) per
# term, the reference's native_log/native_exp being no closer)
LOGZ_RTOL = 1e-4
LOGSUM_LOGZ_RTOL = 1e-4

LONG_LENGTHS = (41, 47, 55, 63, 64, 65, 66, 72, 80, 91, 100)


def bits(a):
    return np.ascontiguousarray(a).view(np.int32)


def long_sentences(n_words, seed, lengths=LONG_LENGTHS):
    rng = np.random.default_rng(seed)
    return [rng.integers(0, n_words, size=n).astype(np.int32) for n in lengths]


def gpu(levels, name, **kw):
    kw.setdefault("max_alloc_size", 4 << 30)
    return CLParser(write_grz(levels, name), **kw)


@pytest.mark.parametrize("size,n_words", [("medium", 500), ("deep", 300)])
def test_long_sentences_cascade_bit_exact(size, n_words):
    """Coarse inside/outside, masks, fine inside and trees for sentences of
    41-100 words; cells of the longest ones run more than one 64-split chunk."""
    levels = split_levels("viterbi", size)
    sents = long_sentences(n_words, seed=71)
    P = gpu(levels, f"split_{size}")
    words, offsets, _ = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all(), st
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
    assert np.array_equal(bits(P.debug_copy(0, "outside")), bits(r.chart(0, "outside")))
    m, _, _ = r.masks(0)
    assert np.array_equal(P.debug_copy(0, "masks"), m)
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(nodes, r.trees())
    assert r.corner_drops(1) == 0


def test_long_sentences_fine_outside_bit_exact():
    """insideOutside on 41-100 words: the fine level's pair-factored outside
    range jobs (L_NN over e+1..n, R_NN over 0..b-1) exceed 64 splits."""
    levels = split_levels("viterbi", "medium")
    sents = long_sentences(500, seed=72, lengths=(66, 83, 100))
    P = gpu(levels, "split_medium")
    words, offsets, _ = pack_sentences(sents)
    P.inside_outside_ids(words, offsets)
    r = oracle.run(levels, sents, mode="inside_outside")
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(bits(P.debug_copy(1, "outside")), bits(r.chart(1, "outside")))


def test_long_sentences_split_cells_match_one_by_one():
    """Each long sentence parsed alone (its long cells split over several
    CTAs) gives the node block it gets in the batch."""
    levels = split_levels("viterbi", "medium")
    sents = long_sentences(500, seed=73, lengths=(44, 70, 100))
    P = gpu(levels, "split_medium")
    words, offsets, lens = pack_sentences(sents)
    whole, _ = P.parse_ids(words, offsets)
    blocks = node_blocks(whole, lens)
    for i, s in enumerate(sents):
        w1, o1, _ = pack_sentences([s])
        alone, st = P.parse_ids(w1, o1)
        assert st[0] == 0 and np.array_equal(alone, blocks[i]), i


def test_long_sentences_real_logz_vs_fp64():
    levels = split_levels("real", "medium")
    sents = long_sentences(500, seed=74, lengths=(41, 66, 100))
    P = gpu(levels, "split_medium_real")
    words, offsets, _ = pack_sentences(sents)
    z, st = P.partitions_ids(words, offsets)
    assert (st == 0).all()
    r32 = oracle.run(levels, sents, mode="partitions")
    masks, isc, osc = r32.masks(0)
    assert np.array_equal(P.debug_copy(0, "masks"), masks)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sents, precision=64)
    r64.set_final_masks(masks, isc, osc)
    assert r64.run("partitions") == 0
    z64 = r64.partitions().astype(np.float64)
    rel = np.abs(z.astype(np.float64) - z64) / np.abs(z64)
    assert rel.max() < LOGZ_RTOL, rel.max()


def test_max_length_boundary():
    """A sentence of exactly max_length words parses; one word more is
    refused with PUCK_ERR_SENT_TOO_LONG and leaves its nodes zeroed."""
    levels = split_levels("viterbi", "small")
    sents = long_sentences(300, seed=75, lengths=(100, 101, 7))
    P = gpu(levels, "split_small")   # max_length defaults to 100
    words, offsets, lens = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert list(st) == [0, 3, 0]
    blocks = node_blocks(nodes, lens)
    assert not blocks[1].any()
    r = oracle.run(levels, [sents[0], sents[2]], mode="parse")
    ref = node_blocks(r.trees(), [100, 7])
    assert np.array_equal(blocks[0], ref[0]) and np.array_equal(blocks[2], ref[1])


def _logsum_case(sents, name):
    levels = split_levels("logsum", "medium")
    P = gpu(levels, name)
    words, offsets, _ = pack_sentences(sents)
    z, st = P.partitions_ids(words, offsets)
    assert (st == 0).all()
    r32 = oracle.run(levels, sents, mode="partitions")
    masks, isc, osc = r32.masks(0)
    assert np.array_equal(P.debug_copy(0, "masks"), masks)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sents, precision=64)
    r64.set_final_masks(masks, isc, osc)
    assert r64.run("partitions") == 0
    z64 = r64.partitions().astype(np.float64)
    assert np.all(np.isfinite(z))
    rel = np.abs(z.astype(np.float64) - z64) / np.abs(z64)
    assert rel.max() < LOGSUM_LOGZ_RTOL, rel.max()
    # the FP32 oracle and the GPU run the same log-add-exp per term, in other orders
    rel32 = np.abs(z.astype(np.float64) - r32.partitions().astype(np.float64)) / np.abs(z64)
    assert rel32.max() < LOGSUM_LOGZ_RTOL, rel32.max()
    return z


def test_logsum_semiring_logz_vs_fp64():
    """The LogSum fine level (RuleSemiring.scala:45-76, zero -1e6, log-add-exp
    sums; CompileGrammar --logsum) on the GPU's target-major path."""
    from helpers import split_sentences
    _logsum_case(split_sentences(32, seed=76), "split_medium_logsum")


def test_logsum_semiring_long_sentences_vs_fp64():
    _logsum_case(long_sentences(500, seed=77, lengths=(45, 70)), "split_medium_logsum")
