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

The cascade is restated the same way: the coarse level's outside pass
scattered from each parent cell to its children (the oracle gathers per
child), the pruning masks from ``inside + outside >= root - 9``
(CLParser.scala computeMasks), and the fine level's inside pass under those
masks with the reference's gating: a rule runs at a parent cell when the
cell's mask meets the coarse bits of the rule's segment
(CoarseParentSymbolGrammarClusterer: one segment per large coarse parent,
one for the rest), and a split only when both child cells hold a live bit.
"""
import numpy as np
import pytest

import oracle
from helpers import node_blocks, small_pcfg_levels, split_levels, split_sentences, tiny_pcfg_levels
from puck_gb300 import grammar, synth

NEG = np.float32(-np.inf)


def _chart_index(b, e, n):
    sp = e - b - 1
    return b + sp * n - sp * (sp - 1) // 2


class _Semiring:
    """Max in float32 (Viterbi, bit-exact with the oracle) or log-add in
    float64 (sum-product, log space).  Rule weights are taken in log space:
    a Real level's linear float32 weights are logged in float64."""

    def __init__(self, dtype, acc, linear_weights):
        self.dtype, self.acc, self.linear = dtype, acc, linear_weights

    def w(self, x):
        x = np.asarray(x)
        return np.log(x.astype(np.float64)) if self.linear else x.astype(self.dtype)


VIT = _Semiring(np.float32, np.maximum, False)


def _log(cl):
    return _Semiring(np.float64, np.logaddexp, cl.semiring == "real")


_BUCKET_NAME = {grammar.NN: "NN", grammar.NT: "NT", grammar.TN: "TN", grammar.TT: "TT"}


def _live(m, b, e):
    return m is None or bool(np.any(m[b, e]))


def _gate(cl, job, syms, m, merged=False):
    """Rows whose target symbol's segment meets the cell mask ``m``.  A
    merged level (a middle level of a cascade) runs every rule as one block,
    gated by segment 0's bits (CLParser.scala:783-785)."""
    j = cl.jobs[job]
    if merged:
        hit = j["seg_bits"].shape[0] > 0 and bool(np.any(j["seg_bits"][0] & m))
        return np.full(len(syms), hit)
    return np.any(j["seg_bits"][j["tgt_seg"][syms]] & m, axis=1)


def _inside(cl, words, sr, mbot=None, mtop=None, apps=None, merged=False):
    """Inside pass.  ``mbot``/``mtop`` (int32[n+1, n+1, mask_size]) are the
    coarse level's masks; None runs unpruned.  ``apps`` (a one-item list)
    accumulates the (rule, split) applications made."""
    n, cs = len(words), cl.cell_size
    zero = sr.dtype(-np.inf)
    bot = np.full((n + 1, n + 1, cs), zero, sr.dtype)
    top = np.full((n + 1, n + 1, cs), zero, sr.dtype)
    wb = [sr.w(x) for x in cl.bucket_scores]
    wnu, wtu = sr.w(cl.nu_scores), sr.w(cl.tu_scores)

    def unary(dst, src, rules, w):
        dst[:] = zero
        sr.acc.at(dst, rules[:, 0], (src[rules[:, 1]] + w).astype(sr.dtype))

    for i, w in enumerate(words):
        lo, hi = cl.lex_offsets[w], cl.lex_offsets[w + 1]
        bot[i, i + 1, cl.lex_term[lo:hi]] = cl.lex_score[lo:hi]
        if _live(mtop, i, i + 1):
            unary(top[i, i + 1], bot[i, i + 1], cl.tu_rules, wtu)

    def binary(dst, left, right, bucket, b, e, lcell, rcell):
        r, w = cl.bucket_rules[bucket], wb[bucket]
        if not r.shape[0] or not (_live(*lcell) and _live(*rcell)):
            return
        if mbot is not None:
            keep = _gate(cl, "in_" + _BUCKET_NAME[bucket], r[:, 0], mbot[b, e], merged)
            r, w = r[keep], w[keep]
        if apps is not None:
            apps[0] += r.shape[0]
        sr.acc.at(dst, r[:, 0], ((left[r[:, 1]] + right[r[:, 2]]) + w).astype(sr.dtype))

    for span in range(2, n + 1):
        for b in range(n - span + 1):
            e = b + span
            cell = bot[b, e]
            if span == 2:
                binary(cell, bot[b, b + 1], bot[b + 1, e], grammar.TT, b, e,
                       (mbot, b, b + 1), (mbot, b + 1, e))
            binary(cell, top[b, e - 1], bot[e - 1, e], grammar.NT, b, e,
                   (mtop, b, e - 1), (mbot, e - 1, e))
            binary(cell, bot[b, b + 1], top[b + 1, e], grammar.TN, b, e,
                   (mbot, b, b + 1), (mtop, b + 1, e))
            for k in range(b + 1, e):
                binary(cell, top[b, k], top[k, e], grammar.NN, b, e, (mtop, b, k), (mtop, k, e))
            if _live(mtop, b, e):
                unary(top[b, e], cell, cl.nu_rules, wnu)
    return bot, top


def _outside(cl, words, ibot, itop, sr, mbot=None, mtop=None, merged=False):
    """Outside pass, scattered from each parent cell to its children (spans
    in decreasing order, so a child's parents are all done first).  Under
    masks a parent's share reaches a child when the parent's bottom cell and
    the sibling's cell hold a live bit and the child's cell mask meets the
    segment of the child's symbol in the rotated job (out_L_* / out_R_*);
    unaries run from live top cells only."""
    n, cs = len(words), cl.cell_size
    zero = sr.dtype(-np.inf)
    obot = np.full((n + 1, n + 1, cs), zero, sr.dtype)
    otop = np.full((n + 1, n + 1, cs), zero, sr.dtype)
    term = np.full((n + 1, cs), zero, sr.dtype)   # terminal cells' binary share
    otop[0, n, cl.root] = 0.0
    wb = [sr.w(x) for x in cl.bucket_scores]
    wnu, wtu = sr.w(cl.nu_scores), sr.w(cl.tu_scores)

    def unary(dst, src, rules, w):
        dst[:] = zero
        sr.acc.at(dst, rules[:, 1], (src[rules[:, 0]] + w).astype(sr.dtype))

    def push(dst, child_cell, parent, sib, sib_cell, bucket, child):
        r, w = cl.bucket_rules[bucket], wb[bucket]
        if not r.shape[0] or not _live(*sib_cell):
            return
        if child_cell[0] is not None:
            m, cb, ce = child_cell
            keep = _gate(cl, "out_%s_%s" % ("L" if child == 1 else "R", _BUCKET_NAME[bucket]),
                         r[:, child], m[cb, ce], merged)
            r, w = r[keep], w[keep]
        other = 2 if child == 1 else 1
        sr.acc.at(dst, r[:, child], ((parent[r[:, 0]] + sib[r[:, other]]) + w).astype(sr.dtype))

    for span in range(n, 1, -1):
        for b in range(n - span + 1):
            e = b + span
            if _live(mtop, b, e):
                unary(obot[b, e], otop[b, e], cl.nu_rules, wnu)
            if not _live(mbot, b, e):
                continue
            P = obot[b, e]
            if span == 2:
                push(term[b], (mbot, b, b + 1), P, ibot[b + 1, e], (mbot, b + 1, e), grammar.TT, 1)
                push(term[b + 1], (mbot, b + 1, e), P, ibot[b, b + 1], (mbot, b, b + 1), grammar.TT, 2)
            push(otop[b, e - 1], (mtop, b, e - 1), P, ibot[e - 1, e], (mbot, e - 1, e), grammar.NT, 1)
            push(term[e - 1], (mbot, e - 1, e), P, itop[b, e - 1], (mtop, b, e - 1), grammar.NT, 2)
            push(term[b], (mbot, b, b + 1), P, itop[b + 1, e], (mtop, b + 1, e), grammar.TN, 1)
            push(otop[b + 1, e], (mtop, b + 1, e), P, ibot[b, b + 1], (mbot, b, b + 1), grammar.TN, 2)
            for k in range(b + 1, e):
                push(otop[b, k], (mtop, b, k), P, itop[k, e], (mtop, k, e), grammar.NN, 1)
                push(otop[k, e], (mtop, k, e), P, itop[b, k], (mtop, b, k), grammar.NN, 2)
    for i in range(n):
        if _live(mtop, i, i + 1):
            unary(obot[i, i + 1], otop[i, i + 1], cl.tu_rules, wtu)
        obot[i, i + 1] = sr.acc(obot[i, i + 1], term[i])
    return obot, otop


def _viterbi_cky(cl, words, mbot=None, mtop=None):
    return _inside(cl, words, VIT, mbot, mtop)


def _viterbi_outside(cl, words, ibot, itop):
    return _outside(cl, words, ibot, itop, VIT)


def _masks(cl, words, ibot, itop, obot, otop, thresh=-9.0):
    """A coarse bit is live in a cell when some symbol projecting onto it has
    inside + outside >= root + thresh (float32); span-1 bottom cells hold
    terminals, every other cell nonterminals."""
    n = len(words)
    mb = np.zeros((n + 1, n + 1, cl.mask_size), np.int64)
    mt = np.zeros_like(mb)
    cutoff = np.float32(itop[0, n, cl.root] + np.float32(thresh))
    ns = max(cl.n_nt, cl.n_t)
    for b in range(n):
        for e in range(b + 1, n + 1):
            for m, ins, out, is_t in ((mb, ibot, obot, e == b + 1), (mt, itop, otop, False)):
                score = (ins[b, e, :ns] + out[b, e, :ns]).astype(np.float32)
                syms = np.nonzero(score >= cutoff)[0]
                if is_t:
                    field = np.where(syms < cl.n_t, cl.t_coarse[np.minimum(syms, cl.n_t - 1)], 0)
                else:
                    field = np.where(syms < cl.n_nt, cl.nt_coarse[np.minimum(syms, cl.n_nt - 1)], 0)
                for f in field:
                    m[b, e, f // 32] |= 1 << (f % 32)
    to32 = lambda m: (m & 0xFFFFFFFF).astype(np.uint32).view(np.int32)
    return to32(mb), to32(mt)


def _logsum_cky(cl, words):
    """log Z in float64 log space over the same cell recursion."""
    _, top = _inside(cl, words, _log(cl))
    return top[0, len(words), cl.root]


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


def _cells(r, s, n):
    """(b, e, chart row of bot(b, e), chart row of top(b, e)) for sentence s."""
    base, tri = r.cell_off[s], n * (n + 1) // 2
    for b in range(n):
        for e in range(b + 1, n + 1):
            ci = _chart_index(b, e, n)
            yield b, e, base + ci, base + tri + ci


def test_cascade_outside_masks_and_pruned_inside_equal_independent_cky():
    coarse, fine = split_levels("viterbi", "medium")
    sents = split_sentences(6, seed=34, n_words=500, mean=8, hi=12)
    sents[1] = sents[1][:1]                       # one word: the root is -inf
    r = oracle.run([coarse, fine], sents, mode="parse")
    cin, cout = r.chart(0, "inside"), r.chart(0, "outside")
    masks = r.masks(0)[0]
    fin = r.chart(1, "inside")
    as_bits = lambda a: a.view(np.int32)
    live_cells = total_cells = pruned_rules = 0
    for s, words in enumerate(sents):
        n = len(words)
        ibot, itop = _viterbi_cky(coarse, words)
        obot, otop = _viterbi_outside(coarse, words, ibot, itop)
        mbot, mtop = _masks(coarse, words, ibot, itop, obot, otop)
        fbot, ftop = _viterbi_cky(fine, words, mbot, mtop)
        for b, e, rb, rt in _cells(r, s, n):
            where = (s, b, e)
            assert np.array_equal(as_bits(cin[rb]), as_bits(ibot[b, e])), where
            assert np.array_equal(as_bits(cin[rt]), as_bits(itop[b, e])), where
            assert np.array_equal(as_bits(cout[rb]), as_bits(obot[b, e])), where
            assert np.array_equal(as_bits(cout[rt]), as_bits(otop[b, e])), where
            assert np.array_equal(masks[rb], mbot[b, e]) and np.array_equal(masks[rt], mtop[b, e]), where
            assert np.array_equal(as_bits(fin[rb]), as_bits(fbot[b, e])), where
            assert np.array_equal(as_bits(fin[rt]), as_bits(ftop[b, e])), where
            live_cells += bool(np.any(mtop[b, e]))
            total_cells += 1
        if n > 1:
            full_bot, _ = _viterbi_cky(fine, words)
            pruned_rules += int(np.sum(np.isfinite(full_bot) & ~np.isfinite(fbot)))
    # the masks prune: some cells die entirely and some fine entries are cut
    assert 0 < live_cells < total_cells and pruned_rules > 0


def _check_tree(cl, words, bot, top, nodes):
    """Re-scores a preorder node block {top or -1, bot, width, score bits}
    against an inside chart: every rule exists, every leaf is a lexicon entry
    of its word, and every choice attains the maximum of the backtrace's
    candidates, ``(rule + left) + right`` and ``rule + child`` in float32
    (CLParser.scala extractParses; ties are not told apart here)."""
    f32 = np.float32
    n = len(words)
    assert nodes.shape == (max(2 * n - 1, 0), 4)

    def unary_best(parent, child_cell, rules, scores, chosen):
        sel = rules[:, 0] == parent
        assert np.any(sel & (rules[:, 1] == chosen)), ("no unary", parent, chosen)
        cand = (scores[sel] + child_cell[rules[sel, 1]]).astype(f32)
        got = (scores[sel & (rules[:, 1] == chosen)][0] + child_cell[chosen]).astype(f32)
        assert got == cand.max(), ("unary not best", parent, chosen)

    def walk(p, b):
        t, sym, width = (int(x) for x in nodes[p, :3])
        e = b + width
        if t != -1:
            if width == 1:
                unary_best(t, bot[b, e], cl.tu_rules, cl.tu_scores, sym)
            else:
                unary_best(t, bot[b, e], cl.nu_rules, cl.nu_scores, sym)
        if width == 1:
            lo, hi = cl.lex_offsets[words[b]], cl.lex_offsets[words[b] + 1]
            assert sym in set(cl.lex_term[lo:hi].tolist()), ("not a tag of the word", b, sym)
            assert nodes[p, 3] == bot[b, e, sym].view(np.int32)
            return p + 1
        lp, rp = p + 1, p + 2 * int(nodes[p + 1, 2])
        k = b + int(nodes[lp, 2])
        assert int(nodes[rp, 2]) == e - k

        def child(q, cb, ce):
            ct = int(nodes[q, 0])
            return (False, int(nodes[q, 1]), bot[cb, ce]) if ct == -1 else (True, ct, top[cb, ce])

        l_nt, a, lcell = child(lp, b, k)
        r_nt, c, rcell = child(rp, k, e)
        bucket = {(True, True): grammar.NN, (True, False): grammar.NT,
                  (False, True): grammar.TN, (False, False): grammar.TT}[(l_nt, r_nt)]
        rules, w = cl.bucket_rules[bucket], cl.bucket_scores[bucket]
        hit = (rules[:, 0] == sym) & (rules[:, 1] == a) & (rules[:, 2] == c)
        assert np.count_nonzero(hit) == 1, ("no binary rule", sym, a, c)
        got = f32(f32(w[hit][0] + lcell[a]) + rcell[c])
        assert nodes[p, 3] == got.view(np.int32)
        best = f32(-np.inf)
        splits = [(grammar.NT, top[b, e - 1], bot[e - 1, e]), (grammar.TN, bot[b, b + 1], top[b + 1, e])]
        if width == 2:
            splits.append((grammar.TT, bot[b, b + 1], bot[b + 1, e]))
        splits += [(grammar.NN, top[b, j], top[j, e]) for j in range(b + 1, e)]
        for bk, lc, rc in splits:
            r, ww = cl.bucket_rules[bk], cl.bucket_scores[bk]
            sel = r[:, 0] == sym
            if np.any(sel):
                best = max(best, ((ww[sel] + lc[r[sel, 1]]).astype(f32) + rc[r[sel, 2]]).astype(f32).max())
        assert got == best, ("binary not best", b, e, sym)
        q = walk(lp, b)
        assert q == rp
        return walk(rp, k)

    assert int(nodes[0, 0]) == cl.root and int(nodes[0, 2]) == n
    assert walk(0, 0) == nodes.shape[0]


def test_viterbi_trees_are_argmax_derivations():
    cl = tiny_pcfg_levels()[0]
    sents = [s for s in _sentences(cl, 16, seed=35, lo=2, hi=12)]
    r = oracle.run([cl], sents, mode="parse")
    checked = 0
    for s, nodes in enumerate(node_blocks(r.trees(), [len(x) for x in sents])):
        bot, top = _viterbi_cky(cl, sents[s])
        if not np.isfinite(top[0, len(sents[s]), cl.root]):
            continue
        _check_tree(cl, sents[s], bot, top, nodes)
        checked += 1
        # negative controls on a copy: a score one ulp off, a wrong symbol
        for row, col, delta in ((0, 3, 1), (1, 1, 1)):
            bad = nodes.copy()
            bad[row, col] += delta
            with pytest.raises(AssertionError):
                _check_tree(cl, sents[s], bot, top, bad)
    assert checked >= len(sents) // 2


def test_cascade_trees_are_argmax_derivations_of_the_pruned_chart():
    coarse, fine = split_levels("viterbi", "medium")
    sents = split_sentences(5, seed=36, n_words=500, mean=9, hi=14)
    r = oracle.run([coarse, fine], sents, mode="parse")
    blocks = node_blocks(r.trees(), [len(x) for x in sents])
    for s, words in enumerate(sents):
        ibot, itop = _viterbi_cky(coarse, words)
        obot, otop = _viterbi_outside(coarse, words, ibot, itop)
        mbot, mtop = _masks(coarse, words, ibot, itop, obot, otop)
        fbot, ftop = _viterbi_cky(fine, words, mbot, mtop)
        assert np.isfinite(ftop[0, len(words), fine.root])
        _check_tree(fine, words, fbot, ftop, blocks[s])


def _coarse_marginals(cl, ins, out, log_z, is_terminal_cell):
    """Posterior mass of each coarse symbol in one cell half (float64)."""
    nk, proj = (cl.n_t, cl.t_coarse) if is_terminal_cell else (cl.n_nt, cl.nt_coarse)
    m = np.zeros(cl.n_coarse)
    np.add.at(m, proj[:nk], np.exp(ins[:nk] + out[:nk] - log_z))
    return m


def test_sum_product_cascade_marginals_equal_independent_cky():
    """The FP64 oracle's MBR cell scores are posterior coarse marginals in
    scaled space: ``score * exp(iscale + oscale - iscale[root cell])`` must
    equal the best coarse marginal of a float64 log-space inside/outside
    under the same masks (relative 1e-6: the score is returned in float32),
    and its symbol must be the argmax wherever the top two differ by more
    than 1e-5 relative.  The lexicon's per-word normalisers cancel between
    inside * outside and the root."""
    coarse, fine = split_levels("real", "medium")
    sents = split_sentences(5, seed=37, n_words=500, mean=8, hi=12)
    r32 = oracle.run([coarse, fine], sents, mode="parse")
    m, isc, osc = r32.masks(0)
    r64 = oracle.OracleRun([oracle.OracleLevel(l) for l in (coarse, fine)], sents, precision=64)
    r64.set_final_masks(m, isc, osc)
    assert r64.run("parse") == 0
    score, sym = r64.mbr_cells()
    lg = _log(fine)
    cells = decided = 0
    for s, words in enumerate(sents):
        n = len(words)
        ibot, itop = _viterbi_cky(coarse, words)
        obot, otop = _viterbi_outside(coarse, words, ibot, itop)
        mbot, mtop = _masks(coarse, words, ibot, itop, obot, otop)
        fb, ft = _inside(fine, words, lg, mbot, mtop)
        ob, ot = _outside(fine, words, fb, ft, lg, mbot, mtop)
        log_z = ft[0, n, fine.root]
        assert np.isfinite(log_z)
        root_row = r32.cell_off[s] + n * (n + 1) // 2 + _chart_index(0, n, n)
        for b, e, rb, rt in _cells(r32, s, n):
            assert np.array_equal(m[rb], mbot[b, e]) and np.array_equal(m[rt], mtop[b, e])
            for row, ins, out, term in ((rb, fb[b, e], ob[b, e], e == b + 1), (rt, ft[b, e], ot[b, e], False)):
                marg = _coarse_marginals(fine, ins, out, log_z, term)
                got = float(score[row]) * np.exp(float(isc[row]) + float(osc[row]) - float(isc[root_row]))
                assert abs(got - marg.max()) <= 1e-6 * marg.max() + 1e-12, (s, b, e, got, marg.max())
                two = np.sort(marg)[-2:]
                if two[1] - two[0] > 1e-5 * two[1]:
                    assert sym[row] == int(np.argmax(marg)), (s, b, e)
                    decided += 1
                cells += 1
        # the root cell's top half holds the whole mass on the root's symbol
        assert np.isclose(_coarse_marginals(fine, ft[0, n], ot[0, n], log_z, False).max(), 1.0)
    assert decided > cells // 2


def test_logsum_log_z_equals_independent_cky():
    """LogSum (RuleSemiring.scala LogSumRuleSemiring: log-add with zero
    -1e6) computes log Z directly in float32: within 1e-5 relative of the
    float64 log-space CKY, on the unpruned tiny grammar."""
    cl = tiny_pcfg_levels("logsum")[0]
    sents = _sentences(cl, 10, seed=38, lo=2, hi=10)
    z = oracle.run([cl], sents, mode="partitions").partitions().astype(np.float64)
    for s, words in enumerate(sents):
        want = _logsum_cky(cl, words)
        assert np.isfinite(want)
        assert abs(z[s] - want) <= 1e-5 * max(1.0, abs(want)), (s, z[s], want)


def _mbr_tree(n, cell_score, cell_sym, bot_row, top_row, iscale, oscale):
    """extractMBRParses (CLParser.scala:589-686) restated in float32 from the
    per-cell best marginals: unscale each half by
    exp((iscale + oscale) - iscale[root]), NaN -> 0, clamp at 1; a cell takes
    its unary when it spans two words or more or its top score passes 0.4;
    the best split wins by strict '>' starting from 0 and the first split."""
    f32 = np.float32
    root_row = top_row(0, n)
    best, split, uu = {}, {}, {}
    for span in range(1, n + 1):
        for b in range(n - span + 1):
            e = b + span
            halves = []
            for row in (top_row(b, e), bot_row(b, e)):
                at = f32(f32(iscale[row] + oscale[row]) - iscale[root_row])
                v = f32(cell_score[row] * f32(np.exp(np.float64(at))))
                v = f32(0.0) if np.isnan(v) else v
                halves.append(min(v, f32(1.0)))
            top, bot = halves
            uu[b, e] = (b + 1 < e) or top > f32(0.4)
            best[b, e] = f32(top + bot) if uu[b, e] else bot
            if span > 1:
                bs, bss = b + 1, f32(0.0)
                for k in range(b + 1, e):
                    sc = f32(best[b, k] + best[k, e])
                    if sc > bss:
                        bs, bss = k, sc
                split[b, e] = bs
                best[b, e] = f32(best[b, e] + bss)
    out = []

    def emit(b, e):
        out.append([int(cell_sym[top_row(b, e)]) if uu[b, e] else -1, int(cell_sym[bot_row(b, e)]),
                    e - b, int(best[b, e].view(np.int32))])
        if e - b > 1:
            emit(b, split[b, e])
            emit(split[b, e], e)

    emit(0, n)
    return np.array(out, np.int32)


def test_mbr_trees_equal_restated_extraction():
    coarse, fine = split_levels("real", "medium")
    sents = split_sentences(8, seed=39, n_words=500, mean=10, hi=16)
    sents[2] = sents[2][:1]
    r = oracle.run([coarse, fine], sents, mode="parse")
    _, isc, osc = r.masks(0)
    score, sym = r.mbr_cells()
    blocks = node_blocks(r.trees(), [len(x) for x in sents])
    unary_spans = 0
    for s, words in enumerate(sents):
        n = len(words)
        base, tri = r.cell_off[s], n * (n + 1) // 2
        want = _mbr_tree(n, score, sym, lambda b, e: base + _chart_index(b, e, n),
                         lambda b, e: base + tri + _chart_index(b, e, n), isc, osc)
        assert np.array_equal(blocks[s], want), s
        unary_spans += int(np.sum((want[:, 2] == 1) & (want[:, 0] != -1)))
    # some one-word spans pass the 0.4 threshold and take their unary
    assert unary_spans > 0


def test_rule_application_counts():
    """The oracle's count of (rule, split) applications, the reference's
    work measure ("CKY rule-apps"): unpruned, a closed form over the split
    ranges of each bucket; pruned, the independent CKY's own count."""
    cl = tiny_pcfg_levels()[0]
    sents = _sentences(cl, 6, seed=40, lo=1, hi=9)
    r = oracle.run([cl], sents, mode="inside_outside")
    nr = {k: cl.bucket_rules[k].shape[0] for k in (grammar.NN, grammar.NT, grammar.TN, grammar.TT)}
    want_in = want_out = 0
    for words in sents:
        n = len(words)
        for span in range(2, n + 1):
            cells = n - span + 1
            want_in += cells * (nr[grammar.NN] * (span - 1) + nr[grammar.NT] + nr[grammar.TN]
                                + (nr[grammar.TT] if span == 2 else 0))
        for b in range(n):
            for e in range(b + 1, n + 1):
                right, left = n - e, b          # parents ending after e / starting before b
                # the cell as a nonterminal child (top half)
                want_out += nr[grammar.NN] * (right + left) + nr[grammar.NT] * (e < n) + nr[grammar.TN] * (b > 0)
                if e == b + 1:                  # as a terminal child (bottom half)
                    want_out += nr[grammar.TT] * ((e < n) + (b > 0)) + nr[grammar.NT] * left + nr[grammar.TN] * right
    assert r.rule_apps(0, "inside") == want_in
    assert r.rule_apps(0, "outside") == want_out

    coarse, fine = split_levels("viterbi", "medium")
    sents = split_sentences(4, seed=41, n_words=500, mean=8, hi=12)
    r = oracle.run([coarse, fine], sents, mode="parse")
    apps, full = [0], [0]
    for words in sents:
        ibot, itop = _viterbi_cky(coarse, words)
        obot, otop = _viterbi_outside(coarse, words, ibot, itop)
        mbot, mtop = _masks(coarse, words, ibot, itop, obot, otop)
        _inside(fine, words, VIT, mbot, mtop, apps)
        _inside(fine, words, VIT, None, None, full)
    assert r.rule_apps(1, "inside") == apps[0] < full[0]


def test_bench_cpu_baseline_reports_reference_work():
    """bench.py's CPU-baseline leg and its rule-application report, run on a
    small cascade exactly as the bench calls them (host only)."""
    import json
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    levels = split_levels("viterbi", "medium")
    sents = split_sentences(8, seed=42, n_words=500, mean=8, hi=12)
    base, r = bench.cpu_baseline(levels, sents, 6)
    assert base["kind"] == "port" and base["value"] > 0
    rep = bench.reference_work(r, 1000.0)
    assert rep["rule_apps_per_sentence"] == round(r.rule_apps(1, "inside") / 6) > 0
    assert abs(rep["rule_apps_per_s"] / (r.rule_apps(1, "inside") / 6 * 1000.0) - 1) < 1e-3
    json.dumps(rep)


class _ArtifactLevel:
    """The attributes the independent CKY reads, taken from one level of a
    compiled ``.grz`` artifact (rule-order job tables, lexicon, coarse maps)."""

    def __init__(self, info):
        a = info.arrays
        for k in ("semiring", "n_nt", "n_t", "cell_size", "mask_size", "n_coarse", "root"):
            setattr(self, k, getattr(info, k))
        names = [_BUCKET_NAME[b] for b in (grammar.NN, grammar.NT, grammar.TN, grammar.TT)]
        self.bucket_rules = [np.stack([a[f"in_{n}/tgt"], a[f"in_{n}/ia"], a[f"in_{n}/ib"]], 1) for n in names]
        self.bucket_scores = [a[f"in_{n}/score"] for n in names]
        self.nu_rules = np.stack([a["in_NU/tgt"], a["in_NU/osrc"]], 1)
        self.nu_scores = a["in_NU/score"]
        self.tu_rules = np.stack([a["in_TU/tgt"], a["in_TU/osrc"]], 1)
        self.tu_scores = a["in_TU/score"]
        self.lex_offsets, self.lex_term, self.lex_score = a["lex_off"], a["lex_term"], a["lex_score"]
        self.nt_coarse, self.t_coarse = a["nt_coarse"], a["t_coarse"]
        self.jobs = {}
        for j in grammar.JOBS:
            self.jobs[j[0]] = {"seg_bits": a[f"{j[0]}/seg_bits"].reshape(-1, self.mask_size),
                               "tgt_seg": a[f"{j[0]}/tgt_seg"]}


def _golden_cases():
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    return sorted(f[:-4] for f in os.listdir(here) if f.endswith(".npz"))


@pytest.mark.parametrize("case", _golden_cases())
def test_golden_fixture_equals_independent_cky(case):
    """Every committed fixture, read back from its ``.grz`` artifact (the
    wsj_0 -> wsj_1 one holds the reference's own Berkeley grammars, every
    rule kept).  Cascades: the coarse masks are the independent CKY's bit
    for bit.  Viterbi parses: each tree is an argmax derivation of the
    independent (pruned) fine chart.  Partitions: Viterbi root scores bit
    for bit; sum-product log Z within 1e-5 relative of the float64 CKY."""
    import os
    from puck_gb300 import grz
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    levels = [_ArtifactLevel(l) for l in grz.read_sequence(os.path.join(here, case + ".grz"), load_arrays=True)]
    data = np.load(os.path.join(here, case + ".npz"))
    off, words, mode = data["offsets"], data["words"], str(data["mode"])
    sents = [words[off[i]:off[i + 1]] for i in range(len(off) - 1)]
    fine = levels[-1]
    blocks = node_blocks(data["trees"], [len(x) for x in sents]) if mode == "parse" else None
    base = 0
    for s, w in enumerate(sents):
        n = len(w)
        tri = n * (n + 1) // 2
        mbot = mtop = None
        if len(levels) > 1:
            coarse = levels[0]
            ibot, itop = _viterbi_cky(coarse, w)
            obot, otop = _viterbi_outside(coarse, w, ibot, itop)
            mbot, mtop = _masks(coarse, w, ibot, itop, obot, otop)
            if "masks" in data:
                for b in range(n):
                    for e in range(b + 1, n + 1):
                        ci = _chart_index(b, e, n)
                        assert np.array_equal(data["masks"][base + ci], mbot[b, e]), (s, b, e)
                        assert np.array_equal(data["masks"][base + tri + ci], mtop[b, e]), (s, b, e)
        base += 2 * tri
        if fine.semiring == "viterbi":
            fbot, ftop = _inside(fine, w, VIT, mbot, mtop)
            if mode == "parse":
                if np.isfinite(ftop[0, n, fine.root]):
                    _check_tree(fine, w, fbot, ftop, blocks[s])
                else:
                    # no parse: one word whose tags no root unary reaches.
                    # The backtrace's unary scan starts from -30000 and keeps
                    # symbol 0, and the leaf reports that terminal's score.
                    assert n == 1, s
                    assert blocks[s].tolist() == [[fine.root, 0, 1, int(fbot[0, 1, 0].view(np.int32))]], s
            else:
                assert data["partitions"][s].view(np.int32) == ftop[0, n, fine.root].view(np.int32), s
        else:
            _, ftop = _inside(fine, w, _log(fine), mbot, mtop)
            want = ftop[0, n, fine.root]
            got = float(data["partitions"][s])
            assert abs(got - want) <= 1e-5 * max(1.0, abs(want)), (s, got, want)


def test_pruned_fine_outside_chart_equals_independent_cky():
    """The fine level's Viterbi outside pass under the coarse masks (the
    chart the GPU tests compare bit for bit): the independent scatter form
    with the rotated jobs' gating gives the oracle's chart bit for bit."""
    coarse, fine = split_levels("viterbi", "medium")
    sents = split_sentences(5, seed=43, n_words=500, mean=9, hi=13)
    r = oracle.run([coarse, fine], sents, mode="inside_outside")
    fin, fout = r.chart(1, "inside"), r.chart(1, "outside")
    bits = lambda a: a.view(np.int32)
    live = 0
    for s, words in enumerate(sents):
        n = len(words)
        ibot, itop = _viterbi_cky(coarse, words)
        obot, otop = _viterbi_outside(coarse, words, ibot, itop)
        mbot, mtop = _masks(coarse, words, ibot, itop, obot, otop)
        fb, ft = _inside(fine, words, VIT, mbot, mtop)
        ob, ot = _outside(fine, words, fb, ft, VIT, mbot, mtop)
        for b, e, rb, rt in _cells(r, s, n):
            assert np.array_equal(bits(fin[rb]), bits(fb[b, e])) and np.array_equal(bits(fin[rt]), bits(ft[b, e]))
            assert np.array_equal(bits(fout[rb]), bits(ob[b, e])), (s, b, e, "bot")
            assert np.array_equal(bits(fout[rt]), bits(ot[b, e])), (s, b, e, "top")
            live += int(np.isfinite(ot[b, e]).sum())
    assert live > 0


def test_three_level_cascade_with_a_merged_middle_level():
    """coarse -> fine -> fine (a self-cascade, as the reference's own
    CLParserTest builds): the middle level runs merged blocks under the
    coarse masks and makes the masks of the last.  Its inside and outside
    charts, both mask sets and the last level's charts and trees equal the
    independent CKY's."""
    coarse, fine = split_levels("viterbi", "medium")
    sents = split_sentences(4, seed=44, n_words=500, mean=8, hi=11)
    r = oracle.run([coarse, fine, fine], sents, mode="parse")
    bits = lambda a: a.view(np.int32)
    c1_in, c1_out, m0, m1 = r.chart(1, "inside"), r.chart(1, "outside"), r.masks(0)[0], r.masks(1)[0]
    c2_in = r.chart(2, "inside")
    blocks = node_blocks(r.trees(), [len(x) for x in sents])
    skipped = 0
    for s, words in enumerate(sents):
        n = len(words)
        ib, it = _viterbi_cky(coarse, words)
        ob, ot = _viterbi_outside(coarse, words, ib, it)
        mb0, mt0 = _masks(coarse, words, ib, it, ob, ot)
        fb1, ft1 = _inside(fine, words, VIT, mb0, mt0, merged=True)
        ob1, ot1 = _outside(fine, words, fb1, ft1, VIT, mb0, mt0, merged=True)
        mb1, mt1 = _masks(fine, words, fb1, ft1, ob1, ot1)
        fb2, ft2 = _inside(fine, words, VIT, mb1, mt1)
        for b, e, rb, rt in _cells(r, s, n):
            where = (s, b, e)
            assert np.array_equal(m0[rb], mb0[b, e]) and np.array_equal(m0[rt], mt0[b, e]), where
            assert np.array_equal(bits(c1_in[rb]), bits(fb1[b, e])) and np.array_equal(bits(c1_in[rt]), bits(ft1[b, e])), where
            assert np.array_equal(bits(c1_out[rb]), bits(ob1[b, e])) and np.array_equal(bits(c1_out[rt]), bits(ot1[b, e])), where
            assert np.array_equal(m1[rb], mb1[b, e]) and np.array_equal(m1[rt], mt1[b, e]), where
            assert np.array_equal(bits(c2_in[rb]), bits(fb2[b, e])) and np.array_equal(bits(c2_in[rt]), bits(ft2[b, e])), where
            skipped += int(np.any(mb0[b, e]) and not np.any(fine.jobs["in_NN"]["seg_bits"][0] & mb0[b, e]))
        if np.isfinite(ft2[0, n, fine.root]):
            _check_tree(fine, words, fb2, ft2, blocks[s])
    # some live cells miss segment 0's bits: the merged gate is exercised
    assert skipped > 0


def test_bench_e2e_roofline_arithmetic():
    """bench.py's end-to-end fraction from a parser's per-level work: 2 ops
    per unit over all levels, at the peak, over the mean device time; a
    failing parser call gives an 'unavailable' entry instead of an error."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    class FakeParser:
        def level_work(self, level):
            return ((1e12, 0), (3e12, 0))[level]

    rep = bench.e2e_roofline(FakeParser(), 2, [2000.0, 2000.0], 40.0)
    assert rep["ops_per_step"] == 8e12 and rep["frac"] == round(8e12 / 40e12 / 2.0, 4)

    class Broken:
        def level_work(self, level):
            raise RuntimeError("no device")

    assert "unavailable" in bench.e2e_roofline(Broken(), 2, [1.0], 40.0)
