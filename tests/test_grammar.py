"""Compile-time derivation: symbol classes, buckets, clusterer, tables, artifact."""
import os
import tempfile

import numpy as np
import pytest

from puck_gb300 import grammar, grz, synth
from puck_gb300.grammar import Grammar


def test_java_hashmap_iteration_order():
    # 4 keys -> 16 buckets; 17 and 1 share bucket 1 in insertion order
    assert grammar._java_hashmap_order([20, 3, 17, 1]) == [17, 1, 3, 20]
    # 13 keys -> 32 buckets (resize at size > 12)
    keys = [40, 8, 1, 2, 3, 4, 5, 6, 7, 9, 10, 11, 12]
    assert grammar._java_hashmap_order(keys) == [1, 2, 3, 4, 5, 6, 7, 40, 8, 9, 10, 11, 12]


def test_coarse_parent_segments_and_subsegments():
    # coarse parent 5 has 350 rules, 2 has 100, 9 has 20 (interleaved)
    pc = np.array([5] * 350 + [2] * 100 + [9] * 20)
    rng = np.random.default_rng(0)
    pc = pc[rng.permutation(pc.shape[0])]
    segs = grammar.coarse_parent_segments(pc, mask_size=1)
    assert len(segs) == 2
    big, rest = segs
    assert int(big.bits[0]) == 1 << 5
    assert int(rest.bits[0]) == (1 << 2) | (1 << 9)
    sizes = [len(s) for s in big.subsegments]
    assert sizes == [44] * 6 + [43] * 2                  # floor(350/8)=43, 6 left over
    assert np.array_equal(np.concatenate([s[:43] for s in big.subsegments]),
                          np.nonzero(pc == 5)[0][:8 * 43])  # rule order kept
    assert sum(len(s) for s in rest.subsegments) == 120
    # merged list = the 100-rule parent then the 20-rule one (size order),
    # cut into 8 x 15 rules
    assert set(pc[rest.subsegments[0]]) == {2} and set(pc[rest.subsegments[5]]) == {2}
    assert set(pc[rest.subsegments[6]]) == {2, 9} and set(pc[rest.subsegments[7]]) == {9}


def test_small_segment_fewer_than_eight_rules():
    segs = grammar.coarse_parent_segments(np.array([1, 1, 3]), mask_size=1)
    assert len(segs) == 1
    assert [len(s) for s in segs[0].subsegments] == [1, 1, 1]   # empty sub-segments dropped


def _hand_grammar():
    # labels: 0 ROOT, 1 S, 2 A, 3 T1, 4 T2
    labels = ["ROOT", "S", "A", "T1", "T2"]
    g = Grammar(
        labels=labels, coarse=np.arange(5, dtype=np.int32), coarse_names=list(labels), root=0,
        bin_rules=np.array([[1, 3, 4], [1, 2, 4], [2, 3, 3]], np.int32),
        bin_score=np.array([-1.0, -0.25, -2.0], np.float32),
        un_rules=np.array([[0, 1], [2, 3], [0, 0], [1, 1], [2, 2]], np.int32),
        un_score=np.array([-0.5, -0.75, 0.0, 0.0, 0.0], np.float32),
        words=["a", "b"], lex_offsets=np.array([0, 1, 2], np.int64),
        lex_label=np.array([3, 4], np.int32), lex_score=np.array([-0.125, -0.0625], np.float32))
    return g


def test_rule_structure_classes_and_buckets():
    cl = grammar.compile_level(_hand_grammar())
    # nonterminals: parents of binaries / non-identity unaries
    assert list(cl.nt_labels) == [0, 1, 2]
    assert list(cl.t_labels) == [3, 4]
    assert cl.cell_size == 32 and cl.mask_size == 1
    assert cl.bucket_rules[grammar.TT].tolist() == [[1, 0, 1], [2, 0, 0]]
    assert cl.bucket_rules[grammar.NT].tolist() == [[1, 2, 1]]
    assert cl.nu_rules.tolist() == [[0, 1], [0, 0], [1, 1], [2, 2]]
    assert cl.tu_rules.tolist() == [[2, 0]]
    v = cl.viterbi
    assert v["offsets"].shape[0] == 6 * 3 + 1
    # TT group (index 3): parent S (1) has one rule, parent A (2) one rule
    tt = v["offsets"][9:13]
    assert list(np.diff(tt)) == [0, 1, 1]


def test_outside_rotations():
    cl = grammar.compile_level(_hand_grammar())
    j = cl.jobs["out_L_NT"]                          # (S -> A T2) rotated: target A
    assert j["tgt"].tolist() == [2] and j["ia"].tolist() == [1] and j["ib"].tolist() == [1]
    j = cl.jobs["out_R_NT"]                          # target T2, a = A, b = S
    assert j["tgt"].tolist() == [1] and j["ia"].tolist() == [2] and j["ib"].tolist() == [1]


def test_artifact_round_trip():
    levels = [grammar.compile_level(_hand_grammar())]
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "g.grz")
        grz.write_sequence(p, levels)
        back = grz.read_sequence(p, load_arrays=True)
        assert len(back) == 1
        b = back[0]
        assert (b.n_nt, b.n_t, b.cell_size, b.root) == (3, 2, 32, 0)
        assert b.words == ["a", "b"]
        ref = grz.level_arrays(levels[0])
        for k, a in ref.items():
            assert np.array_equal(b.arrays[k], a), k


def test_reference_archive_is_refused():
    import zipfile
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "ref.grz")
        with zipfile.ZipFile(p, "w") as z:
            z.writestr("parserNames", "parser-0")
            z.writestr("parser-0/grammar", b"\xac\xed\x00\x05")      # a Java serialisation stream
            z.writestr("parser-0/insideNT/0/kernels.program", b"opaque")
        with pytest.raises(ValueError):
            grz.read_sequence(p)


def test_projection_is_a_distribution():
    c, f = synth.split_grammar(seed=3, n_coarse_nt=8, n_coarse_pt=6, max_split=4, mean_split=3.0,
                               n_coarse_rules=60, target_fine_rules=3000, n_coarse_unaries=12, n_words=300)
    nonid = c.un_rules[:, 0] != c.un_rules[:, 1]
    parents = np.concatenate([c.bin_rules[:, 0], c.un_rules[nonid, 0]])
    p = np.exp(np.concatenate([c.bin_score, c.un_score[nonid]]).astype(np.float64))
    tot = np.bincount(parents, weights=p)
    assert np.allclose(tot[np.unique(parents)], 1.0, atol=1e-5)
    assert np.all(f.bin_score < 0)                       # every binary weight strictly below log 1
