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

    python tests/golden/make_golden.py [case ...]

The ``wsj01_cascade_viterbi`` case is built from the reference's own
Berkeley text grammars ``wsj_0`` and ``wsj_1`` (dlwh/puck ``textGrammars/``,
read by ``puck_gb300.berkeley``) when they are present: the directory named
by ``PUCK_TEXT_GRAMMARS``, else ``/root/reference/textGrammars``.  Every binary and unary rule of both
levels is kept; the lexicon is restricted to the words of the fixture's
sentences so that the stored archive stays small.  Without the text grammars
that case is left as committed.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from puck_gb300 import berkeley, grammar, grz, synth  # noqa: E402

TEXT_GRAMMARS = os.environ.get("PUCK_TEXT_GRAMMARS", "/root/reference/textGrammars")

# Sentences written for this fixture (tokenised like the treebank: punctuation
# split off), lengths 3-46.
WSJ_SENTENCES = [
    "The company said it expects revenue to rise .",
    "He sold shares of the stock .",
    "Prices fell .",
    "The board approved the plan on Tuesday .",
    "Analysts said the market will remain weak for several months .",
    "The bank , which is based in New York , reported a loss in the third quarter .",
    "Investors bought bonds and sold stocks as interest rates declined .",
    "She said that the new rules would not affect the company 's earnings .",
    "Sales of new cars rose 5 % last year , according to the report .",
    "The government plans to cut spending and raise taxes next year .",
    "Officials expect the economy to grow slowly .",
    "The chairman of the firm declined to comment on the proposed merger .",
    "Many traders were worried about the dollar .",
    "It was the largest drop since October .",
    "The agency will review the contract and make a decision by the end of the month .",
    "Shares of the computer maker closed at $ 30 , up 2 cents , in heavy trading on the exchange "
    "as investors bet that the company would report strong profits .",
    "The president said the country needs a stronger economy and more jobs , but he did not say "
    "how the government would pay for the new programs that he proposed last week in a speech .",
    "Yesterday the stock market fell sharply .",
    "The firm has about 2,000 employees .",
    "Japanese banks have been buying American companies .",
]


def restrict_vocabulary(gs, words):
    """The cascade with its shared vocabulary cut to ``words`` (sorted): the
    lexicon entries of every other word are dropped, rules are unchanged."""
    vocab = sorted(set(words))
    out = []
    for g in gs:
        idx = {w: i for i, w in enumerate(g.words)}
        labels, scores, offsets = [], [], [0]
        for w in vocab:
            i = idx[w]
            a, b = int(g.lex_offsets[i]), int(g.lex_offsets[i + 1])
            labels.append(g.lex_label[a:b])
            scores.append(g.lex_score[a:b])
            offsets.append(offsets[-1] + (b - a))
        h = grammar.Grammar(labels=g.labels, coarse=g.coarse, coarse_names=g.coarse_names, root=g.root,
                            bin_rules=g.bin_rules, bin_score=g.bin_score, un_rules=g.un_rules,
                            un_score=g.un_score, words=vocab, lex_offsets=np.asarray(offsets, np.int64),
                            lex_label=np.concatenate(labels).astype(np.int32),
                            lex_score=np.concatenate(scores).astype(np.float32), name=g.name)
        h.validate()
        out.append(h)
    return out


def wsj_case():
    prefixes = [os.path.join(TEXT_GRAMMARS, p) for p in ("wsj_0.gr", "wsj_1.gr")]
    if not os.path.exists(prefixes[1] + ".binary"):
        print("wsj01_cascade_viterbi: text grammars absent, left as committed")
        return
    toks = [s.split() for s in WSJ_SENTENCES]
    gs = restrict_vocabulary(berkeley.read_cascade(prefixes), [w for t in toks for w in t])
    wid = {w: i for i, w in enumerate(gs[1].words)}
    sents = [np.array([wid[w] for w in t], np.int32) for t in toks]
    levels = [grammar.compile_level(gs[0], "viterbi"), grammar.compile_level(gs[1], "viterbi")]
    save("wsj01_cascade_viterbi", levels, sents, "parse")


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


def main(only=()):
    if only:
        for case in only:
            {"wsj01_cascade_viterbi": wsj_case}[case]()
        return
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
    wsj_case()


if __name__ == "__main__":
    main(sys.argv[1:])
