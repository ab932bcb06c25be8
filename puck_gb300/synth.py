"""Seeded synthetic grammars and sentences for the parser workloads.

The Berkeley treebank grammars and the WSJ sentences the reference was
benchmarked on are not available, so every workload uses generated grammars
with the shapes of the published setups:

* ``small_pcfg`` -- a plain PCFG: 64 nonterminals + 32 preterminals, 20,000
  distinct binaries sampled uniformly without replacement, 200 acyclic unaries,
  per-parent Gamma(0.5) weights, 5,000 words with 1-8 preterminals scored by
  Dirichlet(0.5); 512 sentences of length U[5,20] with Zipf(1.1) word ids.
* ``split_grammar`` -- a latent-annotation ("split") grammar: coarse symbols
  split into 1-16 subsymbols (fine label id = coarse id << 4 | sub), binaries
  grown from coarse rules into split-correlated blocks of fine rules with
  Gamma(0.3) weights, unary depth 1, a Zipf(1.1) vocabulary.  Its coarse level
  is the projection of the fine grammar (fine probabilities summed over child
  subsymbols and averaged over parent subsymbols, in log space).
* ``lognormal_lengths`` -- sentence lengths from a lognormal with the stated
  mean (sigma 0.5), rounded and clipped.

All generators are deterministic for a given seed on one machine.  Scores are
float32 log-probabilities.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from .grammar import Grammar


def _normalise_per_parent(parents: np.ndarray, raw: np.ndarray) -> np.ndarray:
    tot = np.bincount(parents, weights=raw)
    p = raw / tot[parents]
    return np.log(np.maximum(p, 1e-300)).astype(np.float32)


def _zipf_sampler(rng: np.random.Generator, n: int, a: float):
    w = np.arange(1, n + 1, dtype=np.float64) ** (-a)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]

    def sample(size):
        return np.minimum(np.searchsorted(cdf, rng.random(size), side="right"), n - 1).astype(np.int32)
    return sample


def _lexicon(rng, n_words, tag_labels, min_tags, max_tags, tag_weights=None, refinements=None):
    """Per word: 1-8 candidate tags with Dirichlet(0.5) scores.  With
    ``refinements`` (coarse tag -> fine labels) each candidate coarse tag's
    mass is spread over its subsymbols by a Dirichlet(1.0)."""
    offsets = [0]
    labels: List[np.ndarray] = []
    scores: List[np.ndarray] = []
    n_tags = len(tag_labels)
    for _ in range(n_words):
        k = int(rng.integers(min_tags, max_tags + 1))
        k = min(k, n_tags)
        tags = rng.choice(n_tags, size=k, replace=False, p=tag_weights)
        probs = np.maximum(rng.dirichlet(np.full(k, 0.5)), 1e-30)
        if refinements is None:
            labels.append(np.asarray(tag_labels, np.int32)[tags])
            scores.append(np.log(probs))
        else:
            for t, p in zip(tags, probs):
                fine = refinements[tag_labels[t]]
                q = np.maximum(rng.dirichlet(np.ones(len(fine))), 1e-30)
                labels.append(np.asarray(fine, np.int32))
                scores.append(np.log(p * q))
        offsets.append(offsets[-1] + (k if refinements is None else
                                      sum(len(refinements[tag_labels[t]]) for t in tags)))
    return (np.asarray(offsets, np.int64), np.concatenate(labels).astype(np.int32),
            np.concatenate(scores).astype(np.float32))


def small_pcfg(seed: int = 0, n_nt: int = 64, n_pt: int = 32, n_binary: int = 20000,
               n_unary: int = 200, n_words: int = 5000) -> Grammar:
    rng = np.random.default_rng(seed)
    n = n_nt + n_pt
    labels = [f"N{i}" for i in range(n_nt)] + [f"P{i}" for i in range(n_pt)]
    total = n_nt * n * n
    n_binary = min(n_binary, total)
    flat = rng.choice(total, size=n_binary, replace=False)
    parent = (flat // (n * n)).astype(np.int32)
    left = ((flat // n) % n).astype(np.int32)
    right = (flat % n).astype(np.int32)
    # acyclic unaries: A -> B with B a later nonterminal or any preterminal
    un = set()
    while len(un) < n_unary:
        a = int(rng.integers(0, n_nt))
        b = int(rng.integers(a + 1, n))
        un.add((a, b))
    un = np.asarray(sorted(un), np.int32).reshape(-1, 2)
    raw_b = rng.gamma(0.5, size=n_binary)
    raw_u = rng.gamma(0.5, size=un.shape[0])
    logp = _normalise_per_parent(np.concatenate([parent, un[:, 0]]), np.concatenate([raw_b, raw_u]))
    ident = np.stack([np.arange(n_nt), np.arange(n_nt)], axis=1).astype(np.int32)
    lex_offsets, lex_label, lex_score = _lexicon(rng, n_words, list(range(n_nt, n)), 1, 8)
    # make sure every preterminal can appear (it must be on some right-hand side)
    g = Grammar(
        labels=labels, coarse=np.arange(n, dtype=np.int32), coarse_names=list(labels), root=0,
        bin_rules=np.stack([parent, left, right], axis=1).astype(np.int32),
        bin_score=logp[:n_binary],
        un_rules=np.concatenate([un, ident]).astype(np.int32),
        un_score=np.concatenate([logp[n_binary:], np.zeros(n_nt, np.float32)]).astype(np.float32),
        words=[f"w{i}" for i in range(n_words)],
        lex_offsets=lex_offsets, lex_label=lex_label, lex_score=lex_score, name="small_pcfg")
    g.validate()
    return g


def uniform_sentences(seed: int, n_sent: int, min_len: int, max_len: int, n_words: int,
                      zipf_a: float = 1.1) -> List[np.ndarray]:
    rng = np.random.default_rng(seed)
    sample = _zipf_sampler(rng, n_words, zipf_a)
    lens = rng.integers(min_len, max_len + 1, size=n_sent)
    return [sample(int(l)) for l in lens]


def lognormal_lengths(rng: np.random.Generator, n: int, mean: float, lo: int, hi: int,
                      sigma: float = 0.5) -> np.ndarray:
    mu = math.log(mean) - sigma * sigma / 2
    x = np.rint(rng.lognormal(mu, sigma, size=n)).astype(np.int64)
    return np.clip(x, lo, hi)


def lognormal_sentences(seed: int, n_sent: int, mean: float, lo: int, hi: int, n_words: int,
                        zipf_a: float = 1.1) -> List[np.ndarray]:
    rng = np.random.default_rng(seed)
    sample = _zipf_sampler(rng, n_words, zipf_a)
    lens = lognormal_lengths(rng, n_sent, mean, lo, hi)
    return [sample(int(l)) for l in lens]


def split_grammar(seed: int = 1, n_coarse_nt: int = 53, n_coarse_pt: int = 45,
                  max_split: int = 16, mean_split: float = 11.3, n_coarse_rules: int = 3800,
                  target_fine_rules: int = 1_500_000, n_coarse_unaries: int = 300,
                  n_words: int = 40000, gamma_shape: float = 0.3) -> Tuple[Grammar, Grammar]:
    """Returns ``(coarse, fine)``: a split grammar and its coarse projection.

    Coarse label 0 is ROOT (one subsymbol, unary-only), labels
    ``1..n_coarse_nt-1`` are phrasal categories, the rest preterminals.
    """
    rng = np.random.default_rng(seed)
    nc = n_coarse_nt + n_coarse_pt
    coarse_names = ["ROOT"] + [f"X{i}" for i in range(1, n_coarse_nt)] + [f"T{i}" for i in range(n_coarse_pt)]
    # subsymbol counts: 1..max_split with the requested mean
    p = min(max((max_split - mean_split) / max(max_split - 1, 1), 0.0), 1.0)
    splits = max_split - rng.binomial(max_split - 1, p, size=nc)
    splits[0] = 1
    sb = max(1, int(math.ceil(math.log2(max_split))))
    fine_of = [np.arange(splits[c]) + (c << sb) for c in range(nc)]   # fine label ids
    n_labels = nc << sb
    labels = [f"{coarse_names[i >> sb]}_{i & ((1 << sb) - 1)}" for i in range(n_labels)]
    coarse = (np.arange(n_labels) >> sb).astype(np.int32)
    nts = np.arange(1, n_coarse_nt)
    pts = np.arange(n_coarse_nt, nc)
    child_pool = np.concatenate([nts, pts])
    # category popularity (Zipf) for children and parents
    pop = 1.0 / np.arange(1, child_pool.shape[0] + 1) ** 0.8
    pop = pop[rng.permutation(pop.shape[0])]
    pop /= pop.sum()
    # coarse binary rules: every phrasal parent gets a share (at least 8)
    share = rng.gamma(1.0, size=nts.shape[0]) + 0.3
    per_parent = np.maximum(8, np.rint(share / share.sum() * n_coarse_rules)).astype(np.int64)
    crules = []
    for X, k in zip(nts, per_parent):
        seen = set()
        tries = 0
        while len(seen) < k and tries < 50 * k:
            Y = int(rng.choice(child_pool, p=pop))
            Z = int(rng.choice(child_pool, p=pop))
            seen.add((Y, Z))
            tries += 1
        crules.extend((int(X), Y, Z) for Y, Z in sorted(seen))
    crules = np.asarray(crules, np.int64)
    # block sizes and split-correlated densities
    a = splits[crules[:, 0]]; b = splits[crules[:, 1]]; c = splits[crules[:, 2]]
    full = (a * b * c).astype(np.float64)
    raw = rng.gamma(0.6, size=crules.shape[0]) * (1.0 + 4.0 * pop[np.searchsorted(child_pool, crules[:, 1])]
                                                   * child_pool.shape[0])
    lo_s, hi_s = 1e-6, 1e6
    for _ in range(100):
        s = math.sqrt(lo_s * hi_s)
        m = np.minimum(full, np.maximum(1.0, np.rint(full * np.minimum(1.0, s * raw))))
        if m.sum() > target_fine_rules:
            hi_s = s
        else:
            lo_s = s
    m = np.minimum(full, np.maximum(1.0, np.rint(full * np.minimum(1.0, lo_s * raw)))).astype(np.int64)
    fp, fl, fr = [], [], []
    for r in range(crules.shape[0]):
        A, B, C = crules[r]
        ai, bi, ci = splits[A], splits[B], splits[C]
        n_full = ai * bi * ci
        if m[r] >= n_full:
            pick = np.arange(n_full)
        else:
            ii, jj, kk = np.meshgrid(np.arange(ai) / max(ai - 1, 1), np.arange(bi) / max(bi - 1, 1),
                                     np.arange(ci) / max(ci - 1, 1), indexing="ij")
            wgt = np.exp(-2.0 * ((ii - jj) ** 2 + (ii - kk) ** 2)).ravel()
            pick = rng.choice(n_full, size=int(m[r]), replace=False, p=wgt / wgt.sum())
        i, rem = np.divmod(pick, bi * ci)
        j, k = np.divmod(rem, ci)
        fp.append(fine_of[A][i]); fl.append(fine_of[B][j]); fr.append(fine_of[C][k])
    fp = np.concatenate(fp).astype(np.int32); fl = np.concatenate(fl).astype(np.int32)
    fr = np.concatenate(fr).astype(np.int32)
    # coarse unaries: ROOT -> a few phrasal categories, others X -> Y (Y != X)
    cu = set()
    for Y in rng.choice(nts, size=min(6, nts.shape[0]), replace=False):
        cu.add((0, int(Y)))
    while len(cu) < n_coarse_unaries:
        X = int(rng.choice(nts))
        Y = int(rng.choice(child_pool, p=pop))
        if Y != X:
            cu.add((X, Y))
    cu = np.asarray(sorted(cu), np.int64)
    up, uc = [], []
    for X, Y in cu:
        ai, bi = splits[X], splits[Y]
        if X == 0:
            pick = np.arange(ai * bi)
        else:
            n_full = ai * bi
            k = max(1, int(round(n_full * rng.uniform(0.3, 1.0))))
            pick = rng.choice(n_full, size=k, replace=False)
        i, j = np.divmod(pick, bi)
        up.append(fine_of[X][i]); uc.append(fine_of[Y][j])
    up = np.concatenate(up).astype(np.int32); uc = np.concatenate(uc).astype(np.int32)
    # weights: Gamma(shape) per fine rule, normalised per fine parent
    raw_b = rng.gamma(gamma_shape, size=fp.shape[0])
    raw_u = rng.gamma(gamma_shape, size=up.shape[0])
    raw_all = np.maximum(np.concatenate([raw_b, raw_u]), 1e-30)
    parents_all = np.concatenate([fp, up])
    tot = np.bincount(parents_all, weights=raw_all, minlength=n_labels)
    prob = raw_all / tot[parents_all]
    logp = np.log(np.maximum(prob, 1e-300)).astype(np.float32)
    fine_nt = np.concatenate([fine_of[x] for x in range(n_coarse_nt)]).astype(np.int32)
    ident = np.stack([fine_nt, fine_nt], axis=1)
    # lexicon over fine preterminals
    refinements = {int(t): fine_of[t] for t in pts}
    pt_pop = 1.0 / np.arange(1, pts.shape[0] + 1) ** 1.0
    pt_pop = pt_pop[rng.permutation(pts.shape[0])]
    pt_pop /= pt_pop.sum()
    lex_offsets, lex_label, lex_score = _lexicon(rng, n_words, [int(t) for t in pts], 1, 8,
                                                 tag_weights=pt_pop, refinements=refinements)
    words = [f"w{i}" for i in range(n_words)]
    fine = Grammar(
        labels=labels, coarse=coarse, coarse_names=coarse_names, root=int(fine_of[0][0]),
        bin_rules=np.stack([fp, fl, fr], axis=1), bin_score=logp[:fp.shape[0]],
        un_rules=np.concatenate([np.stack([up, uc], axis=1), ident]).astype(np.int32),
        un_score=np.concatenate([logp[fp.shape[0]:], np.zeros(ident.shape[0], np.float32)]).astype(np.float32),
        words=words, lex_offsets=lex_offsets, lex_label=lex_label, lex_score=lex_score,
        name="split_fine")
    fine.validate()
    coarse_g = project_grammar(fine, n_parent_refinements=splits)
    return coarse_g, fine


def project_grammar(fine: Grammar, n_parent_refinements: np.ndarray) -> Grammar:
    """Coarse projection of a split grammar: a coarse rule's probability is the
    sum of its fine rules' probabilities over child subsymbols, averaged over
    parent subsymbols (computed in float64 log space, stored as float32)."""
    cn = fine.coarse_names
    nc = len(cn)
    co = fine.coarse
    npr = np.asarray(n_parent_refinements, dtype=np.float64)

    def agg(keys, logp, parents_c):
        uniq, inv = np.unique(keys, axis=0, return_inverse=True)
        inv = inv.ravel()
        mx = np.full(uniq.shape[0], -np.inf)
        np.maximum.at(mx, inv, logp)
        s = np.zeros(uniq.shape[0])
        np.add.at(s, inv, np.exp(logp - mx[inv]))
        out = mx + np.log(s) - np.log(npr[uniq[:, 0]])
        return uniq, out

    bk = np.stack([co[fine.bin_rules[:, 0]], co[fine.bin_rules[:, 1]], co[fine.bin_rules[:, 2]]], axis=1)
    bu, bs = agg(bk, fine.bin_score.astype(np.float64), None)
    nonid = fine.un_rules[:, 0] != fine.un_rules[:, 1]
    uk = np.stack([co[fine.un_rules[nonid, 0]], co[fine.un_rules[nonid, 1]]], axis=1)
    uu, us = agg(uk, fine.un_score[nonid].astype(np.float64), None)
    coarse_nt = np.unique(bu[:, 0]).tolist()
    coarse_nt = sorted(set(coarse_nt) | set(uu[:, 0].tolist()))
    ident = np.stack([np.asarray(coarse_nt), np.asarray(coarse_nt)], axis=1)
    # lexicon: log-sum-exp over subsymbols of the same coarse tag
    word_of = np.repeat(np.arange(len(fine.words)), np.diff(fine.lex_offsets))
    lk = np.stack([word_of, co[fine.lex_label]], axis=1)
    uniq, inv = np.unique(lk, axis=0, return_inverse=True)
    inv = inv.ravel()
    ls = fine.lex_score.astype(np.float64)
    mx = np.full(uniq.shape[0], -np.inf)
    np.maximum.at(mx, inv, ls)
    s = np.zeros(uniq.shape[0])
    np.add.at(s, inv, np.exp(ls - mx[inv]))
    lscore = (mx + np.log(s)).astype(np.float32)
    lex_offsets = np.zeros(len(fine.words) + 1, np.int64)
    np.cumsum(np.bincount(uniq[:, 0], minlength=len(fine.words)), out=lex_offsets[1:])
    g = Grammar(
        labels=list(cn), coarse=np.arange(nc, dtype=np.int32), coarse_names=list(cn),
        root=int(co[fine.root]),
        bin_rules=bu.astype(np.int32), bin_score=bs.astype(np.float32),
        un_rules=np.concatenate([uu, ident]).astype(np.int32),
        un_score=np.concatenate([us, np.zeros(ident.shape[0])]).astype(np.float32),
        words=list(fine.words), lex_offsets=lex_offsets, lex_label=uniq[:, 1].astype(np.int32),
        lex_score=lscore, name="split_coarse")
    g.validate()
    return g
