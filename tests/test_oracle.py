"""The CPU oracle: hand-derived known answers, golden fixtures, self-consistency."""
import os

import numpy as np
import pytest

import oracle
from helpers import c0_sentences, small_pcfg_levels, split_levels, split_sentences
from puck_gb300 import grammar, grz
from test_grammar import _hand_grammar

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def f32bits(x):
    return int(np.float32(x).view(np.int32))


def test_chart_index_matches_formula():
    # ParseChart.chartIndex for n = 4: span-major, then begin
    n = 4
    want = {(0, 1): 0, (1, 2): 1, (2, 3): 2, (3, 4): 3, (0, 2): 4, (1, 3): 5, (2, 4): 6,
            (0, 3): 7, (1, 4): 8, (0, 4): 9}
    def ci(b, e, n):
        sp = abs(e - b) - 1
        return min(b, e) + sp * n - sp * (sp - 1) // 2
    for (b, e), v in want.items():
        assert ci(b, e, n) == v


def test_hand_grammar_viterbi_known_answer():
    """Two words; S is reachable by NT (A T2) and TT (T1 T2) with the same
    score -1.1875.  The backtrace scans NT before TT with '>=', so TT wins."""
    cl = grammar.compile_level(_hand_grammar())
    r = oracle.run([cl], [np.array([0, 1], np.int32)], mode="parse")
    ins = r.chart(0, "inside")
    n = 2
    bot02 = 2          # chartIndex(0,2,2)
    top = 3            # top half starts after 3 bot cells
    assert ins[0, 0] == np.float32(-0.125)                    # bot(0,1)[T1]
    assert ins[1, 1] == np.float32(-0.0625)                   # bot(1,2)[T2]
    assert ins[top + 0, 2] == np.float32(-0.875)              # top(0,1)[A] via A -> T1
    assert ins[bot02, 1] == np.float32(-1.1875)               # bot(0,2)[S]
    assert ins[top + bot02, 0] == np.float32(-1.6875)         # top(0,2)[ROOT]
    t = r.trees()
    assert t.tolist() == [[0, 1, 2, f32bits(-1.1875)],
                          [-1, 0, 1, f32bits(-0.125)],
                          [-1, 1, 1, f32bits(-0.0625)]]
    p = oracle.run([cl], [np.array([0, 1], np.int32)], mode="partitions").partitions()
    assert p[0] == np.float32(-1.6875)


def test_hand_grammar_outside_and_masks():
    cl = grammar.compile_level(_hand_grammar())
    r = oracle.run([cl], [np.array([0, 1], np.int32)], mode="inside_outside")
    out = r.chart(0, "outside")
    top = 3
    assert out[top + 2, 0] == 0.0                              # outside root = one
    assert out[2, 1] == np.float32(-0.5)                        # bot(0,2)[S] via ROOT -> S
    # bot(0,1)[T1]: TT_L gives (-0.5 + -1.0) + -0.0625 ... max with A -> T1 route
    # through top(0,1)[A]: outside A = (-0.5 + -0.0625) + -0.25 = -0.8125, then -0.75
    assert out[top + 0, 2] == np.float32(-0.8125)
    assert out[0, 0] == max(np.float32(-1.5625), np.float32(-1.5625))
    ins = r.chart(0, "inside")
    # every symbol on the best tree has inside + outside equal to the root score
    root = ins[top + 2, 0]
    assert ins[2, 1] + out[2, 1] == root


def test_viterbi_max_marginal_consistency_c0():
    levels = small_pcfg_levels()
    sents = c0_sentences(12, seed=21)
    r = oracle.run(levels, sents, mode="inside_outside")
    ins, out = r.chart(0, "inside"), r.chart(0, "outside")
    cl = levels[0]
    for s in range(len(sents)):
        c0, c1 = r.cell_off[s], r.cell_off[s + 1]
        root = ins[c1 - 1, cl.root]
        v = (ins[c0:c1, :cl.num_syms].astype(np.float64) + out[c0:c1, :cl.num_syms])
        # max over symbols of in+out never exceeds the best parse (up to rounding)
        assert np.all(v.max(1) <= root + 1e-4)
        # the root cell attains it exactly
        assert np.isclose(v[-1].max(), root, atol=1e-4)


def test_fp64_oracle_close_to_fp32_real():
    levels = split_levels("real", "small")
    sents = split_sentences(10, seed=3, n_words=300)
    r32 = oracle.run(levels, sents, mode="partitions")
    m, i, o = r32.masks(0)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in levels], sents, precision=64)
    r64.set_final_masks(m, i, o)
    assert r64.run("partitions") == 0
    z32, z64 = r32.partitions().astype(np.float64), r64.partitions().astype(np.float64)
    assert np.all(np.abs(z32 - z64) / np.abs(z64) < 1e-4)


def _golden_cases():
    if not os.path.isdir(GOLDEN):
        return []
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


@pytest.mark.parametrize("case", _golden_cases())
def test_oracle_matches_golden_fixture(case):
    data = np.load(os.path.join(GOLDEN, case + ".npz"))
    levels = grz.read_sequence(os.path.join(GOLDEN, case + ".grz"), load_arrays=True)
    off = data["offsets"]
    words = data["words"]
    sents = [words[off[i]:off[i + 1]] for i in range(len(off) - 1)]
    mode = str(data["mode"])
    r = oracle.run(levels, sents, mode=mode)
    if mode == "parse":
        assert np.array_equal(r.trees(), data["trees"])
    else:
        assert np.array_equal(r.partitions().view(np.int32), data["partitions"].view(np.int32))
    if "masks" in data:
        assert np.array_equal(r.masks(0)[0], data["masks"])
