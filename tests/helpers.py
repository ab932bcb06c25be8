"""Grammar and sentence builders shared by the tests (seeded, cached per process)."""
from __future__ import annotations

import functools
import os
import tempfile

import numpy as np

from puck_gb300 import grammar, grz, synth

_TMP = tempfile.mkdtemp(prefix="puck_tests_")


@functools.lru_cache(maxsize=None)
def small_pcfg_levels(semiring="viterbi"):
    """The plain 64+32-symbol PCFG, single level."""
    g = synth.small_pcfg(0)
    return (grammar.compile_level(g, semiring),)


@functools.lru_cache(maxsize=None)
def tiny_pcfg_levels(semiring="viterbi"):
    g = synth.small_pcfg(7, n_nt=12, n_pt=6, n_binary=500, n_unary=10, n_words=120)
    return (grammar.compile_level(g, semiring),)


@functools.lru_cache(maxsize=None)
def split_levels(fine_semiring="viterbi", size="medium"):
    """Coarse (Viterbi) + fine split grammar cascade."""
    if size == "c1":
        # the bench grammar: 98 coarse / 1,091 fine symbols, 1.5M binaries
        c, f = synth.split_grammar(seed=1)
    elif size == "wide":
        # many coarse pairs per job (hundreds of live pairs per cell), small splits
        c, f = synth.split_grammar(seed=6, n_coarse_nt=30, n_coarse_pt=20, max_split=4, mean_split=3.0,
                                   n_coarse_rules=1500, target_fine_rules=40000, n_coarse_unaries=40, n_words=400)
    elif size == "deep":
        # coarse symbols with up to 30 refinements: outer-product tiles on
        # each path of the fine kernel (<= 16 members, <= 32, and larger tiles)
        c, f = synth.split_grammar(seed=11, n_coarse_nt=8, n_coarse_pt=6, max_split=30, mean_split=13.0,
                                   n_coarse_rules=70, target_fine_rules=30000, n_coarse_unaries=12, n_words=300)
    elif size == "big":
        # 25-33 refinements per coarse symbol: the flat-tile inside pass cuts
        # each pair into 16 + 16 + rest sub-tiles and blocks of more than 32
        # targets into runs of 32
        c, f = synth.split_grammar(seed=12, n_coarse_nt=5, n_coarse_pt=4, max_split=40, mean_split=30.0,
                                   n_coarse_rules=60, target_fine_rules=60000, n_coarse_unaries=10, n_words=300)
    elif size == "medium":
        c, f = synth.split_grammar(seed=4, n_coarse_nt=10, n_coarse_pt=8, max_split=8, mean_split=6.0,
                                   n_coarse_rules=120, target_fine_rules=20000, n_coarse_unaries=20, n_words=500)
    else:
        c, f = synth.split_grammar(seed=3, n_coarse_nt=8, n_coarse_pt=6, max_split=4, mean_split=3.0,
                                   n_coarse_rules=60, target_fine_rules=3000, n_coarse_unaries=12, n_words=300)
    return (grammar.compile_level(c, "viterbi"), grammar.compile_level(f, fine_semiring))


def write_grz(levels, name):
    path = os.path.join(_TMP, name + ".grz")
    if not os.path.exists(path):
        grz.write_sequence(path, levels)
    return path


def c0_sentences(n=64, seed=1):
    return synth.uniform_sentences(seed, n, 5, 20, 5000)


def split_sentences(n=48, seed=5, n_words=500, mean=14, hi=30):
    return synth.lognormal_sentences(seed, n, mean, 1, hi, n_words)


def node_blocks(nodes, lengths):
    out, start = [], 0
    for n in lengths:
        k = max(2 * int(n) - 1, 0)
        out.append(nodes[start:start + k])
        start += k
    return out


def write_text_grammar(directory, name, splits, seed=0):
    """A small Berkeley-format text grammar (``<name>.numstates``, ``.binary``,
    ``.unary``, ``.lexicon``) with ``splits`` substates per label: ROOT -> S,
    S -> NP VP, NP -> DT NN, VP -> VB NP, six words.  Returns the prefix."""
    rng = np.random.default_rng(seed)
    labels = {"ROOT": 1, "S": splits, "NP": splits, "VP": splits, "DT": splits, "NN": splits, "VB": splits}
    prefix = os.path.join(directory, name)
    with open(prefix + ".numstates", "w") as f:
        for lab, k in labels.items():
            f.write(f"{lab}\t{k}\n")
    with open(prefix + ".binary", "w") as f:
        for p, l, r in (("S", "NP", "VP"), ("NP", "DT", "NN"), ("VP", "VB", "NP")):
            for i in range(labels[p]):
                w = rng.dirichlet(np.ones(labels[l] * labels[r]))
                for j in range(labels[l]):
                    for k in range(labels[r]):
                        f.write(f"{p}_{i} {l}_{j} {r}_{k} {w[j * labels[r] + k]:.6g}\n")
    with open(prefix + ".unary", "w") as f:
        w = rng.dirichlet(np.ones(labels["S"]))
        for j in range(labels["S"]):
            f.write(f"ROOT_0 S_{j} {w[j]:.6g}\n")
    with open(prefix + ".lexicon", "w") as f:
        for tag, words in (("DT", ("the", "a")), ("NN", ("dog", "cat")), ("VB", ("sees", "chases"))):
            for wd in words:
                probs = ", ".join(f"{x:.6g}" for x in rng.uniform(0.05, 0.5, size=labels[tag]))
                f.write(f"{tag} {wd} [{probs}]\n")
    return prefix
