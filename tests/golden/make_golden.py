"""Regenerates the golden fixtures in this directory.

Each case is a compiled grammar artifact (``<case>.grz``) plus ``<case>.npz``
holding the sentences (word ids, CSR offsets), the mode and the oracle's
outputs for them: Viterbi trees (preorder ``{top, bot, width, score bits}``
nodes), log partitions and the coarse level's pruning masks.  The grammar is
stored, not regenerated, so the fixtures do not depend on the random number
generator of the machine that reads them.

The expected outputs come from the CPU oracle (``oracle/``), the restatement
of the reference's algorithm; the reference itself cannot run here, so these
vectors pin regressions and cross-machine agreement, not reference parity.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from puck_gb300 import grammar, grz, synth  # noqa: E402


def save(case, levels, sents, mode):
    grz.write_sequence(os.path.join(HERE, case + ".grz"), levels)
    r = oracle.run(levels, sents, mode=mode)
    off = np.zeros(len(sents) + 1, np.int64)
    np.cumsum([len(s) for s in sents], out=off[1:])
    words = np.concatenate(sents).astype(np.int32)
    out = dict(words=words, offsets=off, mode=np.array(mode))
    if mode == "parse":
        out["trees"] = r.trees()
    else:
        out["partitions"] = r.partitions()
    if len(levels) > 1:
        out["masks"] = r.masks(0)[0]
    np.savez_compressed(os.path.join(HERE, case + ".npz"), **out)
    print(case, {k: v.shape for k, v in out.items()})


def main():
    g = synth.small_pcfg(7, n_nt=12, n_pt=6, n_binary=500, n_unary=10, n_words=120)
    tiny = [grammar.compile_level(g)]
    sents = [s % 120 for s in synth.uniform_sentences(31, 24, 1, 14, 120)]
    save("tiny_pcfg_viterbi", tiny, sents, "parse")
    save("tiny_pcfg_partitions", tiny, sents, "partitions")

    c, f = synth.split_grammar(seed=3, n_coarse_nt=8, n_coarse_pt=6, max_split=4, mean_split=3.0,
                               n_coarse_rules=60, target_fine_rules=3000, n_coarse_unaries=12, n_words=300)
    sents = synth.lognormal_sentences(17, 24, 12, 1, 25, 300)
    save("split_cascade_viterbi", [grammar.compile_level(c), grammar.compile_level(f)], sents, "parse")
    save("split_cascade_real_partitions", [grammar.compile_level(c), grammar.compile_level(f, "real")],
         sents, "partitions")


if __name__ == "__main__":
    main()
