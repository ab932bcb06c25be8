"""Reader for Berkeley-parser text grammars (``<prefix>.numstates``,
``.binary``, ``.unary``, ``.lexicon``), the input of the reference's
CompileGrammar (``--textGrammarPrefix a:b``, src/main/scala/puck/parser/
CompileGrammar.scala:56, which hands each prefix to epic's
``SimpleGrammar.parseBerkeleyText(prefix, -12, CloseUnaries.None)``).

epic is not part of the reference sources, so this restates the published
file format, and parity with epic's reader is unpinned:

* ``numstates``: ``LABEL<tab>k`` -- the label has substates ``LABEL_0 ..
  LABEL_{k-1}``; LABEL is the coarse label the substates project onto.
* ``binary``: ``P_i L_j R_k prob``; ``unary``: ``P_i C_j prob``.
* ``lexicon``: ``TAG word [p_0, ..., p_{k-1}]`` -- one probability per
  substate of TAG.

Scores are natural logs of the probabilities; rules and lexicon entries whose
log score is below ``threshold`` (epic's -12) are dropped.  Every
nonterminal substate gets an identity unary ``X_i -> X_i`` with score 0 when
the file has none, because the unary layer replaces the whole top cell (the
reference's unary bucket includes identities, RuleStructure.scala:86-97).
The lexicon's unknown-word classes (``UNK-INITC-s``, ``UNK-LC``, ...) are
ordinary words of the vocabulary.  The library maps a word missing from the
vocabulary to its class by its spelling and position
(``puck_grammar_word_id_at``); epic's own lexicon model, which the reference
uses, is not present, so that mapping is not checked against it.  A word
with no class in the lexicon is out of vocabulary.

A cascade (``a:b``) shares one coarse label set (the union of the levels'
numstates labels, first level first) and one vocabulary (the union of the
levels' lexicon words, sorted), so that masks and word ids mean the same at
every level.
"""
from __future__ import annotations

import math
import re
from typing import Dict, List, Sequence, Tuple

import numpy as np

from .grammar import Grammar

_LEX = re.compile(r"^(\S+)\s+(\S+)\s+\[(.*)\]\s*$")


def _read_numstates(path: str) -> List[Tuple[str, int]]:
    out = []
    with open(path, encoding="utf-8") as f:
        for line in f:
            parts = line.split()
            if len(parts) == 2:
                out.append((parts[0], int(parts[1])))
    return out


def _split_label(name: str) -> Tuple[str, int]:
    base, _, k = name.rpartition("_")
    if not base or not k.isdigit():
        raise ValueError(f"label {name!r} is not LABEL_substate")
    return base, int(k)


class _Reader:
    def __init__(self, prefix: str, threshold: float):
        self.prefix = prefix
        self.threshold = threshold
        self.numstates = _read_numstates(prefix + ".numstates")
        self.binary: List[Tuple[str, str, str, float]] = []
        self.unary: List[Tuple[str, str, float]] = []
        self.lexicon: List[Tuple[str, str, List[float]]] = []
        with open(prefix + ".binary", encoding="utf-8") as f:
            for line in f:
                p = line.split()
                if len(p) == 4:
                    self.binary.append((p[0], p[1], p[2], float(p[3])))
        with open(prefix + ".unary", encoding="utf-8") as f:
            for line in f:
                p = line.split()
                if len(p) == 3:
                    self.unary.append((p[0], p[1], float(p[2])))
        with open(prefix + ".lexicon", encoding="utf-8") as f:
            for line in f:
                m = _LEX.match(line.rstrip("\n"))
                if m:
                    probs = [float(x) for x in m.group(3).split(",") if x.strip()]
                    self.lexicon.append((m.group(1), m.group(2), probs))

    def keep(self, prob: float) -> bool:
        return prob > 0.0 and math.log(prob) >= self.threshold


def read_cascade(prefixes: Sequence[str], threshold: float = -12.0) -> List[Grammar]:
    """One Grammar per prefix, coarse level first."""
    readers = [_Reader(p, threshold) for p in prefixes]
    coarse_names: List[str] = []
    seen = set()
    for r in readers:
        for name, _ in r.numstates:
            if name not in seen:
                seen.add(name)
                coarse_names.append(name)
    coarse_id = {n: i for i, n in enumerate(coarse_names)}
    vocab = sorted({w for r in readers for _, w, _ in r.lexicon})
    word_id = {w: i for i, w in enumerate(vocab)}
    return [_grammar(r, coarse_names, coarse_id, vocab, word_id) for r in readers]


def _grammar(r: _Reader, coarse_names: List[str], coarse_id: Dict[str, int], vocab: List[str],
             word_id: Dict[str, int]) -> Grammar:
    labels: List[str] = []
    coarse: List[int] = []
    lid: Dict[str, int] = {}
    for name, k in r.numstates:
        for i in range(k):
            lid[f"{name}_{i}"] = len(labels)
            labels.append(f"{name}_{i}")
            coarse.append(coarse_id[name])

    def label(name: str) -> int:
        if name not in lid:
            base, _ = _split_label(name)
            if base not in coarse_id:
                raise ValueError(f"{r.prefix}: label {name!r} has no numstates entry")
            lid[name] = len(labels)
            labels.append(name)
            coarse.append(coarse_id[base])
        return lid[name]

    bins = [(label(p), label(a), label(b), math.log(pr)) for p, a, b, pr in r.binary if r.keep(pr)]
    uns = [(label(p), label(c), math.log(pr)) for p, c, pr in r.unary if r.keep(pr)]
    nts = {b[0] for b in bins} | {u[0] for u in uns if u[0] != u[1]}
    have_ident = {u[0] for u in uns if u[0] == u[1]}
    uns += [(x, x, 0.0) for x in sorted(nts - have_ident)]
    entries: List[Tuple[int, int, float]] = []
    for tag, word, probs in r.lexicon:
        for i, pr in enumerate(probs):
            if r.keep(pr):
                entries.append((word_id[word], label(f"{tag}_{i}"), math.log(pr)))
    entries.sort(key=lambda e: (e[0], e[1]))
    lex_offsets = np.zeros(len(vocab) + 1, np.int64)
    if entries:
        np.cumsum(np.bincount([e[0] for e in entries], minlength=len(vocab)), out=lex_offsets[1:])
    root = lid.get("ROOT_0")
    if root is None:
        raise ValueError(f"{r.prefix}: no ROOT_0 label")
    g = Grammar(
        labels=labels,
        coarse=np.asarray(coarse, np.int32),
        coarse_names=list(coarse_names),
        root=root,
        bin_rules=np.asarray([b[:3] for b in bins], np.int32).reshape(-1, 3),
        bin_score=np.asarray([b[3] for b in bins], np.float32),
        un_rules=np.asarray([u[:2] for u in uns], np.int32).reshape(-1, 2),
        un_score=np.asarray([u[2] for u in uns], np.float32),
        words=list(vocab),
        lex_offsets=lex_offsets,
        lex_label=np.asarray([e[1] for e in entries], np.int32),
        lex_score=np.asarray([e[2] for e in entries], np.float32),
        name=r.prefix.rsplit("/", 1)[-1],
    )
    g.validate()
    return g
