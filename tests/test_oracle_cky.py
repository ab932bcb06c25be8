"""An independent CKY, written from the grammar's definition alone, pins the
oracle's inside pass.

The oracle restates the reference's queue-and-segment machinery
(BinaryUpdateManager / SimpleGenRuleMultiply); this file restates none of it.
It fills each cell straight from the rule lists of a compiled level:

* bottom cell of span 1: the word's lexicon entries (terminal index space);
* top cell of span 1: terminal unaries over the bottom cell;
* bottom cell of span >= 2: every binary rule over every split, children in
  the top half for nonterminals and in the span-1 bottom half for terminals
  (buckets NN, NT, TN, TT of RuleStructure.scala);
* top cell of span >= 2: nonterminal unaries over the bottom cell, a fresh
  row holding only the rules' parents.

Viterbi charts must agree bit for bit (max is exact and each candidate is
``(left + right) + rule`` in float32, the order the device kernels use).
Sum-product is checked through log Z against a float64 log-space CKY.
"""
import numpy as np
import pytest

import oracle
from helpers import small_pcfg_levels, tiny_pcfg_levels
from puck_gb300 import grammar, synth

NEG = np.float32(-np.inf)


def _chart_index(b, e, n):
    sp = e - b - 1
    return b + sp * n - sp * (sp - 1) // 2


def _viterbi_cky(cl, words):
    n, cs = len(words), cl.cell_size
    bot = np.full((n + 1, n + 1, cs), NEG, np.float32)
    top = np.full((n + 1, n + 1, cs), NEG, np.float32)
    nu_p, nu_c = cl.nu_rules[:, 0], cl.nu_rules[:, 1]
    tu_p, tu_c = cl.tu_rules[:, 0], cl.tu_rules[:, 1]

    def unary(dst, src, p, c, w):
        dst[:] = NEG
        np.maximum.at(dst, p, (src[c] + w).astype(np.float32))

    for i, w in enumerate(words):
        lo, hi = cl.lex_offsets[w], cl.lex_offsets[w + 1]
        bot[i, i + 1, cl.lex_term[lo:hi]] = cl.lex_score[lo:hi]
        unary(top[i, i + 1], bot[i, i + 1], tu_p, tu_c, cl.tu_scores)

    def binary(dst, left, right, bucket):
        r, w = cl.bucket_rules[bucket], cl.bucket_scores[bucket]
        if r.shape[0]:
            np.maximum.at(dst, r[:, 0], ((left[r[:, 1]] + right[r[:, 2]]) + w).astype(np.float32))

    for span in range(2, n + 1):
        for b in range(n - span + 1):
            e = b + span
            cell = bot[b, e]
            if span == 2:
                binary(cell, bot[b, b + 1], bot[b + 1, e], grammar.TT)
            binary(cell, top[b, e - 1], bot[e - 1, e], grammar.NT)
            binary(cell, bot[b, b + 1], top[b + 1, e], grammar.TN)
            for k in range(b + 1, e):
                binary(cell, top[b, k], top[k, e], grammar.NN)
            unary(top[b, e], cell, nu_p, nu_c, cl.nu_scores)
    return bot, top


def _logsum_cky(cl, words):
    """log Z in float64 log space over the same cell recursion."""
    n, cs = len(words), cl.cell_size
    ninf = -np.inf
    bot = np.full((n + 1, n + 1, cs), ninf)
    top = np.full((n + 1, n + 1, cs), ninf)
    lw = [np.log(s.astype(np.float64)) for s in cl.bucket_scores]
    lnu = np.log(cl.nu_scores.astype(np.float64))
    ltu = np.log(cl.tu_scores.astype(np.float64))

    def unary(dst, src, rules, w):
        dst[:] = ninf
        np.logaddexp.at(dst, rules[:, 0], src[rules[:, 1]] + w)

    for i, w in enumerate(words):
        lo, hi = cl.lex_offsets[w], cl.lex_offsets[w + 1]
        bot[i, i + 1, cl.lex_term[lo:hi]] = cl.lex_score[lo:hi].astype(np.float64)
        unary(top[i, i + 1], bot[i, i + 1], cl.tu_rules, ltu)

    def binary(dst, left, right, bucket):
        r = cl.bucket_rules[bucket]
        if r.shape[0]:
            np.logaddexp.at(dst, r[:, 0], left[r[:, 1]] + right[r[:, 2]] + lw[bucket])

    for span in range(2, n + 1):
        for b in range(n - span + 1):
            e = b + span
            cell = bot[b, e]
            if span == 2:
                binary(cell, bot[b, b + 1], bot[b + 1, e], grammar.TT)
            binary(cell, top[b, e - 1], bot[e - 1, e], grammar.NT)
            binary(cell, bot[b, b + 1], top[b + 1, e], grammar.TN)
            for k in range(b + 1, e):
                binary(cell, top[b, k], top[k, e], grammar.NN)
            unary(top[b, e], cell, cl.nu_rules, lnu)
    return top[0, n, cl.root]


def _sentences(cl, n, seed, lo=1, hi=9):
    return synth.uniform_sentences(seed, n, lo, hi, len(cl.lex_offsets) - 1)


@pytest.mark.parametrize("make", [tiny_pcfg_levels, small_pcfg_levels], ids=["tiny", "small"])
def test_viterbi_inside_chart_equals_independent_cky(make):
    cl = make()[0]
    sents = _sentences(cl, 8, seed=31, hi=9 if make is tiny_pcfg_levels else 7)
    r = oracle.run([cl], sents, mode="inside_outside")
    ins = r.chart(0, "inside")
    checked, finite_roots = 0, 0
    for s, words in enumerate(sents):
        n = len(words)
        bot, top = _viterbi_cky(cl, words)
        finite_roots += bool(np.isfinite(top[0, n, cl.root]))
        base, tri = r.cell_off[s], n * (n + 1) // 2
        for b in range(n):
            for e in range(b + 1, n + 1):
                ci = _chart_index(b, e, n)
                got_bot = ins[base + ci].view(np.int32)
                got_top = ins[base + tri + ci].view(np.int32)
                assert np.array_equal(got_bot, bot[b, e].view(np.int32)), (s, b, e, "bot")
                assert np.array_equal(got_top, top[b, e].view(np.int32)), (s, b, e, "top")
                checked += 1
    # one-word sentences have no root (it is reached through binaries only):
    # the oracle must agree on that -inf too; the rest parse
    assert checked > 0 and finite_roots >= len(sents) // 2


def test_viterbi_root_scores_equal_independent_cky():
    cl = tiny_pcfg_levels()[0]
    sents = _sentences(cl, 12, seed=32, lo=3, hi=12)
    p = oracle.run([cl], sents, mode="partitions").partitions()
    for s, words in enumerate(sents):
        _, top = _viterbi_cky(cl, words)
        assert p[s].view(np.int32) == top[0, len(words), cl.root].view(np.int32)


def test_sum_product_log_z_equals_independent_cky():
    """Tolerances: the float64 oracle's scaled root cell, unscaled with its
    per-sentence lexicon scales, differs from the float64 CKY only by
    summation order (relative 1e-10); the float32 partition carries float32
    rounding of every product and sum (relative 1e-5)."""
    cl = tiny_pcfg_levels("real")[0]
    sents = _sentences(cl, 10, seed=33, lo=2, hi=10)
    r64 = oracle.OracleRun([oracle.OracleLevel(cl)], sents, precision=64)
    assert r64.run("partitions") == 0
    ins64 = r64.chart(0, "inside")
    scales = r64.partition_scales(0)
    z32 = oracle.run([cl], sents, mode="partitions").partitions().astype(np.float64)
    for s, words in enumerate(sents):
        n = len(words)
        want = _logsum_cky(cl, words)
        assert np.isfinite(want)
        root = r64.cell_off[s] + n * (n + 1) // 2 + _chart_index(0, n, n)
        got64 = np.log(ins64[root, cl.root]) + scales[s]
        assert abs(got64 - want) <= 1e-10 * max(1.0, abs(want)), (s, got64, want)
        assert abs(z32[s] - want) <= 1e-5 * max(1.0, abs(want)), (s, z32[s], want)
