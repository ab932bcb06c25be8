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

``reproject`` (CompileGrammar ``--reproject``; CLParser.reprojectGrammar and
readHierarchy, CLParser.scala:1153-1209) keeps the first and the last level
and makes the first level's substates the coarse label set: the first level
projects onto itself, and each substate of the last level onto its ancestor
at the first level's split depth, read from the last level's ``.hierarchy``
file.  The two levels' depths are the last run of digits in their prefixes
(``wsj_1.gr`` is depth 1).
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


# -- split hierarchies (readHierarchy) ---------------------------------------

class _Node:
    __slots__ = ("label", "kids", "start", "end")

    def __init__(self, label: str):
        self.label, self.kids, self.start, self.end = label, [], 0, 0

    def left_height(self) -> int:
        return 0 if not self.kids else 1 + self.kids[0].left_height()

    def preorder(self):
        yield self
        for k in self.kids:
            yield from k.preorder()


def _parse_bracketed(text: str):
    """A bracketed split tree: ``(label child ...)``, a child being a subtree
    or a bare leaf token.  Returns the root and the leaf tokens in order; a
    node's [start, end) covers its leaves."""
    toks = re.findall(r"\(|\)|[^\s()]+", text)
    leaves: List[str] = []
    pos = 0

    def node() -> _Node:
        nonlocal pos
        if toks[pos] != "(":
            raise ValueError("hierarchy: expected '('")
        n = _Node(toks[pos + 1])
        pos += 2
        n.start = len(leaves)
        while toks[pos] != ")":
            if toks[pos] == "(":
                n.kids.append(node())
            else:
                leaves.append(toks[pos])
                pos += 1
        pos += 1
        n.end = len(leaves)
        return n

    root = node()
    if pos != len(toks):
        raise ValueError("hierarchy: trailing tokens")
    return root, leaves


def _depth(prefix: str) -> int:
    """The split depth of a grammar: the last run of digits in its name."""
    m = re.match(r"^.*(?:^|[^0-9])([0-9]+)([^0-9]*)$", prefix)
    if not m:
        raise ValueError(f"no split depth in {prefix!r}")
    return int(m.group(1))


def read_hierarchy(fine_prefix: str, coarse_prefix: str) -> Dict[str, List[str]]:
    """Coarse substate -> the fine substates below it, from
    ``<fine_prefix>.hierarchy`` (one ``SYM (tree)`` line per label)."""
    fine, coarse = _depth(fine_prefix), _depth(coarse_prefix)
    out: Dict[str, List[str]] = {}
    with open(fine_prefix + ".hierarchy", encoding="utf-8") as f:
        for line in f:
            parts = line.strip().split(None, 1)
            if len(parts) != 2:
                continue
            sym, (root, leaves) = parts[0], _parse_bracketed(parts[1])
            total = root.left_height()
            for sub in root.preorder():
                if sub.left_height() != total - coarse:
                    continue
                if fine - 1 == total:
                    fines = [f"{sym}_{leaves[i]}" for i in range(sub.start, sub.end)]
                else:
                    fines = [f"{sym}_{n.label}" for n in sub.preorder() if n.left_height() == total - fine]
                out[f"{sym}_{sub.label}"] = fines
    return out


def read_cascade(prefixes: Sequence[str], threshold: float = -12.0, reproject: bool = False) -> List[Grammar]:
    """One Grammar per prefix, coarse level first.  With ``reproject`` and
    more than one prefix: the first and last levels, projected onto the
    first level's substates."""
    if reproject and len(prefixes) > 1:
        return _reprojected(prefixes[0], prefixes[-1], threshold)
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

    def by_base(r):
        def project(name: str) -> int:
            base, _ = _split_label(name)
            if base not in coarse_id:
                raise ValueError(f"{r.prefix}: label {name!r} has no numstates entry")
            return coarse_id[base]
        return project

    return [_grammar(r, coarse_names, by_base(r), vocab, word_id) for r in readers]


def _reprojected(coarse_prefix: str, fine_prefix: str, threshold: float) -> List[Grammar]:
    rc, rf = _Reader(coarse_prefix, threshold), _Reader(fine_prefix, threshold)
    coarse_names = [f"{name}_{i}" for name, k in rc.numstates for i in range(k)]
    coarse_id = {n: i for i, n in enumerate(coarse_names)}
    up = {f: c for c, fs in read_hierarchy(fine_prefix, coarse_prefix).items() for f in fs}
    vocab = sorted({w for r in (rc, rf) for _, w, _ in r.lexicon})
    word_id = {w: i for i, w in enumerate(vocab)}

    def itself(name: str) -> int:
        if name not in coarse_id:
            raise ValueError(f"{coarse_prefix}: label {name!r} has no numstates entry")
        return coarse_id[name]

    def through_hierarchy(name: str) -> int:
        c = name if name == "ROOT_0" else up.get(name)   # the root projects onto itself
        if c is None or c not in coarse_id:
            raise ValueError(f"{fine_prefix}: substate {name!r} has no ancestor among {coarse_prefix}'s")
        return coarse_id[c]

    return [_grammar(rc, coarse_names, itself, vocab, word_id),
            _grammar(rf, coarse_names, through_hierarchy, vocab, word_id)]


def _grammar(r: _Reader, coarse_names: List[str], project, vocab: List[str],
             word_id: Dict[str, int]) -> Grammar:
    """``project(substate name) -> coarse id``."""
    labels: List[str] = []
    coarse: List[int] = []
    lid: Dict[str, int] = {}
    for name, k in r.numstates:
        for i in range(k):
            lid[f"{name}_{i}"] = len(labels)
            labels.append(f"{name}_{i}")
            coarse.append(project(f"{name}_{i}"))

    def label(name: str) -> int:
        if name not in lid:
            _split_label(name)
            lid[name] = len(labels)
            labels.append(name)
            coarse.append(project(name))
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
