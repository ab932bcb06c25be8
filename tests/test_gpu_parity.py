"""GPU parity: the sm_103a library (through its C ABI) against the CPU oracle.

Viterbi charts, pruning masks and trees must be bit-identical to the oracle's
restatement of the reference.  Sum-product (Real semiring) results are not
bit-reproducible in the reference either (atomic accumulation order,
``native_exp``); they are compared against the FP64 oracle with the
tolerances stated below.
"""
import numpy as np
import pytest

import oracle
from helpers import (c0_sentences, node_blocks, small_pcfg_levels, split_levels, split_sentences,
                     tiny_pcfg_levels, write_grz)
from puck_gb300.parser import CLParser, pack_sentences

pytestmark = pytest.mark.gpu

# log-partition tolerance against FP64 (relative)
LOGZ_RTOL = 1e-4


def bits(a):
    return np.ascontiguousarray(a).view(np.int32)


def gpu(levels, name, **kw):
    kw.setdefault("max_alloc_size", 4 << 30)
    return CLParser(write_grz(levels, name), **kw)


def test_c0_inside_chart_and_trees_bit_exact():
    levels = small_pcfg_levels()
    sents = c0_sentences(64)
    P = gpu(levels, "c0")
    words, offsets, _ = pack_sentences(sents)
    nodes, status = P.parse_ids(words, offsets)
    assert (status == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
    assert np.array_equal(nodes, r.trees())
    assert r.corner_drops(0) == 0


def test_c0_outside_chart_bit_exact():
    levels = small_pcfg_levels()
    sents = c0_sentences(32, seed=2)
    P = gpu(levels, "c0")
    words, offsets, _ = pack_sentences(sents)
    P.inside_outside_ids(words, offsets)
    r = oracle.run(levels, sents, mode="inside_outside")
    assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
    assert np.array_equal(bits(P.debug_copy(0, "outside")), bits(r.chart(0, "outside")))


def test_c0_partitions_match():
    levels = small_pcfg_levels()
    sents = c0_sentences(48, seed=3)
    P = gpu(levels, "c0")
    words, offsets, _ = pack_sentences(sents)
    z, st = P.partitions_ids(words, offsets)
    r = oracle.run(levels, sents, mode="partitions")
    assert (st == 0).all()
    assert np.array_equal(bits(z), bits(r.partitions()))


@pytest.mark.parametrize("size", ["small", "medium"])
def test_cascade_masks_charts_trees_bit_exact(size):
    levels = split_levels("viterbi", size)
    nw = 300 if size == "small" else 500
    sents = split_sentences(48, seed=5, n_words=nw)
    P = gpu(levels, f"split_{size}")
    words, offsets, _ = pack_sentences(sents)
    nodes, status = P.parse_ids(words, offsets)
    assert (status == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
    assert np.array_equal(bits(P.debug_copy(0, "outside")), bits(r.chart(0, "outside")))
    m, _, _ = r.masks(0)
    assert np.array_equal(P.debug_copy(0, "masks"), m)
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(nodes, r.trees())
    # the masks really prune (otherwise the gating paths are untested)
    pops = np.unpackbits(m.view(np.uint8)).sum() / m.shape[0]
    assert pops < 0.8 * levels[0].n_coarse
    # cells_pruned counts the cells whose mask has no bit set
    st = P.stats()
    assert st["cells"] == m.shape[0]
    assert st["cells_pruned"] == int((~m.any(axis=1)).sum()) > 0


def test_wide_grammar_split_cells_bit_exact():
    """Hundreds of live coarse pairs per cell and few cells per span launch,
    so long cells run as several CTAs that must share one pair order."""
    levels = split_levels("viterbi", "wide")
    sents = split_sentences(24, seed=31, n_words=400, mean=24, hi=40)
    P = gpu(levels, "split_wide")
    words, offsets, _ = pack_sentences(sents)
    nodes, status = P.parse_ids(words, offsets)
    assert (status == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(nodes, r.trees())


def test_deep_refinements_bit_exact():
    """Coarse symbols with up to 17 refinements: tiles of every lane-grid
    shape of the flat-tile outer product, and pairs just over 16 members cut
    into a 16-member and a 1-member sub-tile."""
    levels = split_levels("viterbi", "deep")
    sents = split_sentences(24, seed=67, n_words=300, mean=16, hi=30)
    P = gpu(levels, "split_deep")
    words, offsets, _ = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(nodes, r.trees())


@pytest.mark.parametrize("lengths", ["short", "long"])
def test_big_tiles_sub_tiled_bit_exact(lengths):
    """25-33 refinements per coarse symbol: the fine inside pass runs the
    flat-tile form on 16 x 16 sub-tiles of each pair (16 + 16 + rest per
    side), with blocks of more than 32 targets cut into runs.  Short
    sentences, and 41-100 words (two 64-split liveness chunks)."""
    levels = split_levels("viterbi", "big")
    if lengths == "short":
        sents = split_sentences(32, seed=83, n_words=300, mean=14, hi=30)
    else:
        rng = np.random.default_rng(84)
        sents = [rng.integers(0, 300, size=n).astype(np.int32) for n in (41, 64, 65, 77, 100)]
    P = gpu(levels, "split_big")
    words, offsets, _ = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
    m, _, _ = r.masks(0)
    assert np.array_equal(P.debug_copy(0, "masks"), m)
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(nodes, r.trees())
    # the fine level really runs the flat-tile inside pass, from span 2
    assert P.flat_from(1) == 2


def test_bench_grammar_bit_exact():
    """The 1,091-symbol, 1.5M-rule bench grammar on 40 sentences up to 40
    words: split long cells, hundreds of live pairs, the batched inside form."""
    levels = split_levels("viterbi", "c1")
    sents = split_sentences(40, seed=2, n_words=40000, mean=23, hi=40)
    P = gpu(levels, "split_c1")
    words, offsets, _ = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(nodes, r.trees())


def test_wide_grammar_fine_outside_bit_exact():
    """insideOutside on a cascade: the fine level's pair-factored outside pass
    (its own rule layout) against the oracle, with split cells."""
    levels = split_levels("viterbi", "wide")
    sents = split_sentences(24, seed=33, n_words=400, mean=24, hi=40)
    P = gpu(levels, "split_wide")
    words, offsets, _ = pack_sentences(sents)
    P.inside_outside_ids(words, offsets)
    r = oracle.run(levels, sents, mode="inside_outside")
    assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
    assert np.array_equal(bits(P.debug_copy(1, "outside")), bits(r.chart(1, "outside")))


def test_wide_grammar_real_split_cells_vs_fp64():
    levels = split_levels("real", "wide")
    sents = split_sentences(24, seed=32, n_words=400, mean=24, hi=40)
    P = gpu(levels, "split_wide_real")
    words, offsets, _ = pack_sentences(sents)
    z, st = P.partitions_ids(words, offsets)
    assert (st == 0).all()
    r32 = oracle.run(levels, sents, mode="partitions")
    masks, isc, osc = r32.masks(0)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sents, precision=64)
    r64.set_final_masks(masks, isc, osc)
    assert r64.run("partitions") == 0
    z64 = r64.partitions().astype(np.float64)
    rel = np.abs(z.astype(np.float64) - z64) / np.abs(z64)
    assert rel.max() < LOGZ_RTOL, rel.max()
    # the inside chart agrees with the FP32 oracle to rounding
    gi, oi = P.debug_copy(1, "inside"), r32.chart(1, "inside")
    nz = np.abs(oi) > 1e-30
    assert np.median(np.abs(gi - oi)[nz] / np.abs(oi)[nz]) < 1e-5


def test_graph_capture_gives_identical_results():
    """use_graphs: span sequences captured and replayed as CUDA graphs, the
    second and third calls updating the kept graphs in place."""
    levels = split_levels("viterbi", "small")
    sents = split_sentences(40, seed=41, n_words=300, mean=12, hi=30)
    words, offsets, _ = pack_sentences(sents)
    ref, _ = gpu(levels, "split_small").parse_ids(words, offsets)
    G = gpu(levels, "split_small", use_graphs=True)
    for _ in range(3):
        nodes, st = G.parse_ids(words, offsets)
        assert (st == 0).all()
        assert np.array_equal(nodes, ref)
    # a batch with another shape re-captures
    w2, o2, _ = pack_sentences(sents[:17])
    n2, _ = G.parse_ids(w2, o2)
    r2, _ = gpu(levels, "split_small").parse_ids(w2, o2)
    assert np.array_equal(n2, r2)


@pytest.mark.parametrize("size", ["medium", "big"])
def test_flat_tile_span_bands_bit_exact(size):
    """Every span band of the flat-tile inside form, on both levels: the
    coarse level's groups of 16 coarse ids (target-major otherwise) and the
    fine level's 16 x 16 sub-tiles (the pair form otherwise), switched at
    span 2, 9, 17 or never.  Charts and trees stay bit-identical."""
    levels = split_levels("viterbi", size)
    sents = split_sentences(40, seed=47, n_words=300 if size == "big" else 500, mean=16, hi=30)
    words, offsets, _ = pack_sentences(sents)
    r = oracle.run(levels, sents, mode="parse")
    P = gpu(levels, f"split_{size}")
    for f0, f1 in ((0, 0), (2, 2), (9, 17), (17, 9), (2, 0), (0, 2)):
        P.set_flat_from(0, f0)
        P.set_flat_from(1, f1)
        assert (P.flat_from(0), P.flat_from(1)) == (f0, f1)
        nodes, st = P.parse_ids(words, offsets)
        assert (st == 0).all()
        assert np.array_equal(bits(P.debug_copy(0, "inside")), bits(r.chart(0, "inside")))
        assert np.array_equal(bits(P.debug_copy(1, "inside")), bits(r.chart(1, "inside")))
        assert np.array_equal(nodes, r.trees())


def test_autotune_keeps_results():
    """The autotuner may switch a level's gather form and the split waves;
    Viterbi results stay bit-identical."""
    levels = split_levels("viterbi", "medium")
    sents = split_sentences(48, seed=43)
    words, offsets, _ = pack_sentences(sents)
    P = gpu(levels, "split_medium")
    ref, _ = P.parse_ids(words, offsets)
    choice = P.autotune(words, offsets)
    assert len(choice["levels"]) == 2 and choice["waves"] in (1.0, 2.0, 4.0)
    assert all(f in (0, 2, 8, 16) for f in choice["flat_from"])
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all() and np.array_equal(nodes, ref)
    r = oracle.run(levels, sents, mode="parse")
    assert np.array_equal(nodes, r.trees())


def test_batching_does_not_change_results():
    levels = split_levels("viterbi", "medium")
    sents = split_sentences(40, seed=9)
    words, offsets, _ = pack_sentences(sents)
    whole, _ = gpu(levels, "split_medium").parse_ids(words, offsets)
    chunked, _ = gpu(levels, "split_medium", max_batch_sentences=7).parse_ids(words, offsets)
    assert np.array_equal(whole, chunked)
    lens = np.diff(offsets)
    blocks = node_blocks(whole, lens)
    one = gpu(levels, "split_medium")
    for i in (0, 5, 17):
        w1, o1, _ = pack_sentences([sents[i]])
        alone, _ = one.parse_ids(w1, o1)
        assert np.array_equal(alone, blocks[i])


def test_edge_cases_lengths_oov_too_long():
    levels = tiny_pcfg_levels()
    rng = np.random.default_rng(0)
    sents = [rng.integers(0, 120, size=n).astype(np.int32) for n in (1, 2, 3, 1, 7, 30, 12)]
    oov = [np.array([3, 4, 10_000, 5], np.int32)]
    empty = [np.zeros(0, np.int32)]
    allsents = sents + oov + empty
    P = gpu(levels, "tiny", max_length=20)
    words, offsets, lens = pack_sentences(allsents)
    nodes, status = P.parse_ids(words, offsets)
    assert status[5] == 3           # longer than max_length
    assert status[7] == 4           # out-of-vocabulary id
    assert status[8] == 9           # empty
    ok = [i for i in range(len(allsents)) if status[i] == 0]
    assert ok == [0, 1, 2, 3, 4, 6]
    r = oracle.run(levels, [allsents[i] for i in ok], mode="parse")
    blocks = node_blocks(nodes, lens)
    ref = node_blocks(r.trees(), [len(allsents[i]) for i in ok])
    for k, i in enumerate(ok):
        assert np.array_equal(blocks[i], ref[k])
    assert not blocks[5].any() and not blocks[7].any()
    res = P.parse([[int(w) for w in s] for s in allsents])
    assert [t.is_success for t in res] == [s == 0 for s in status]


def test_one_word_batch_quirk_matches_oracle():
    # a batch whose longest sentence has one word
    levels = tiny_pcfg_levels()
    sents = [np.array([i], np.int32) for i in (3, 8, 40)]
    P = gpu(levels, "tiny")
    words, offsets, _ = pack_sentences(sents)
    P.inside_outside_ids(words, offsets)
    r = oracle.run(levels, sents, mode="inside_outside")
    assert np.array_equal(bits(P.debug_copy(0, "outside")), bits(r.chart(0, "outside")))


def test_real_semiring_logz_vs_fp64():
    levels = split_levels("real", "medium")
    sents = split_sentences(40, seed=11)
    P = gpu(levels, "split_medium_real")
    words, offsets, _ = pack_sentences(sents)
    z, st = P.partitions_ids(words, offsets)
    assert (st == 0).all()
    r32 = oracle.run(levels, sents, mode="partitions")
    masks, isc, osc = r32.masks(0)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sents, precision=64)
    r64.set_final_masks(masks, isc, osc)
    assert r64.run("partitions") == 0
    z64 = r64.partitions().astype(np.float64)
    assert np.all(np.isfinite(z))
    rel = np.abs(z.astype(np.float64) - z64) / np.abs(z64)
    assert rel.max() < LOGZ_RTOL, rel.max()
    # GPU masks identical to the oracle's
    assert np.array_equal(P.debug_copy(0, "masks"), masks)


def test_real_semiring_mbr_trees_match_oracle():
    levels = split_levels("real", "medium")
    sents = split_sentences(32, seed=12)
    P = gpu(levels, "split_medium_real")
    words, offsets, lens = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    r = oracle.run(levels, sents, mode="parse")
    ref = r.trees()
    # symbols and shape must agree; scores are float sums in different orders
    assert np.array_equal(nodes[:, :3], ref[:, :3])
    gs = nodes[:, 3].view(np.float32).astype(np.float64)
    rs = ref[:, 3].view(np.float32).astype(np.float64)
    assert np.allclose(gs, rs, rtol=1e-4, atol=1e-5)


def _golden():
    import os
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    return d, sorted(f[:-4] for f in os.listdir(d) if f.endswith(".npz"))


@pytest.mark.parametrize("case", _golden()[1])
def test_gpu_matches_golden_fixture(case):
    import os
    d = _golden()[0]
    data = np.load(os.path.join(d, case + ".npz"))
    P = CLParser(os.path.join(d, case + ".grz"), max_alloc_size=1 << 30)
    words, offsets = data["words"], data["offsets"]
    mode = str(data["mode"])
    if mode == "parse":
        nodes, st = P.parse_ids(words, offsets)
        assert (st == 0).all()
        assert np.array_equal(nodes, data["trees"])
    else:
        z, st = P.partitions_ids(words, offsets)
        assert (st == 0).all()
        if "real" in case:
            assert np.allclose(z, data["partitions"], rtol=LOGZ_RTOL)
        else:
            assert np.array_equal(bits(z), bits(data["partitions"]))
    if "masks" in data:
        assert np.array_equal(P.debug_copy(0, "masks"), data["masks"])


def test_compile_then_parse_through_the_c_abi(tmp_path):
    """CompileGrammar and CLParser both through the C ABI: text grammars ->
    puck_compile_grammar -> puck_grammar_load / puck_parse, trees
    bit-identical to the oracle's parse of the same archive."""
    import ctypes
    from helpers import write_text_grammar
    from puck_gb300 import _lib, grz
    c = write_text_grammar(str(tmp_path), "coarse", 1, seed=5)
    f = write_text_grammar(str(tmp_path), "fine", 4, seed=6)
    out = str(tmp_path / "abi.grz")
    L = _lib.load()
    L.puck_compile_grammar.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p]
    assert L.puck_compile_grammar(f"{c}:{f}".encode(), out.encode(), None) == 0, _lib.last_error()
    P = CLParser(out, max_alloc_size=1 << 30)
    text = ["the dog sees a cat", "a cat chases the dog", "the cat sees the dog"]
    sents = [np.array(P.word_ids(t.split()), np.int32) for t in text]
    assert all((s >= 0).all() for s in sents)
    words, offsets, _ = pack_sentences(sents)
    nodes, st = P.parse_ids(words, offsets)
    assert (st == 0).all()
    r = oracle.run(grz.read_sequence(out, load_arrays=True), sents, mode="parse")
    assert np.array_equal(nodes, r.trees())
    assert P.parse([t.split() for t in text])[0].is_success
