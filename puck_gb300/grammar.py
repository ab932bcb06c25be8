"""Grammar model and compile-time derivation for Puck's chart-parsing hot path.

A :class:`Grammar` is one level of a coarse-to-fine cascade (the role of epic's
``SimpleGrammar`` plus its refinements in the reference).  :func:`compile_level`
derives everything the device passes need, restating the reference's
compile-time logic (paths are relative to the dlwh/puck project):

* symbol indexing and rule buckets -- ``RuleStructure``
  (src/main/scala/puck/parser/RuleStructure.scala:50-100): a symbol is a
  *nonterminal* iff it is the parent of a binary rule or of a non-identity
  unary; every other symbol that occurs on a right-hand side is a *terminal*
  (preterminal).  Binaries split into NN / NT (right child terminal) /
  TN (left child terminal) / TT; unaries into N-child (identity rules
  included) and T-child, dropping rules whose parent is a terminal.
* rule segments (the reference's "kernels") -- the CoarseParent clusterer
  (src/main/java/puck/parser/gen/CoarseParentSymbolGrammarClusterer.java:38-150)
  with ``MIN_SINGLE_COARSE_PARENT_GROUP_SIZE = 300`` and ``NUM_SM = 8``
  sub-segments.  A segment's coarse-parent bitset gates it per chart cell
  (src/main/scala/puck/parser/CLParser.scala:845-855).
* outside rule rotations -- src/main/scala/puck/parser/gen/CLOutside.scala:61-71 (rotations), 73-112 (the rotated jobs).
* Viterbi backtrace tables -- src/main/scala/puck/parser/gen/CLViterbi.scala:274-353,610-628.

Symbol order: the reference orders symbols by the bundled ``symbols_dump``
resource and falls back to set-iteration order for unknown names.  Grammars
built here (synthetic or read from text) fix the order explicitly: symbols are
indexed in increasing label order, which is the stand-in for that resource.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

NN, NT, TN, TT = 0, 1, 2, 3
BUCKET_NAMES = ("NN", "NT", "TN", "TT")

SEMIRINGS = {"viterbi": 0, "real": 1, "logsum": 2}

# Zero / one of each semiring (src/main/scala/puck/parser/RuleSemiring.scala:22-98).
SEMIRING_ZERO = {"viterbi": -math.inf, "real": 0.0, "logsum": -1000000.0}
SEMIRING_ONE = {"viterbi": 0.0, "real": 1.0, "logsum": 0.0}

MIN_SINGLE_COARSE_PARENT_GROUP_SIZE = 300
NUM_SUBSEGMENTS = 8

# Inside jobs: (bucket) -> target is the parent.  Outside jobs rotate a
# bucket's rules so that the updated child becomes the "parent"
# (CLOutside.scala:61-67).  Each job records the index space of its target
# and of the two operands that are added before the rule score:
# value = (A[ia] + B[ib]) + w.
#                 name     bucket rotate  tgt_is_t a_is_t b_is_t
JOBS = (
    ("in_NN", NN, None, False, False, False),
    ("in_NT", NT, None, False, False, True),
    ("in_TN", TN, None, False, True, False),
    ("in_TT", TT, None, False, True, True),
    ("out_L_NN", NN, "L", False, False, False),
    ("out_R_NN", NN, "R", False, False, False),
    ("out_L_NT", NT, "L", False, False, True),
    ("out_R_NT", NT, "R", True, False, False),
    ("out_L_TN", TN, "L", True, False, False),
    ("out_R_TN", TN, "R", False, True, False),
    ("out_L_TT", TT, "L", True, False, True),
    ("out_R_TT", TT, "R", True, True, False),
)
JOB_INDEX = {j[0]: i for i, j in enumerate(JOBS)}

# Unary jobs: target index space is_t, operand is_t.
UNARY_JOBS = (
    ("in_NU", False, False),   # top[A] from bot[B], B nonterminal (identity included)
    ("in_TU", False, True),    # top[A] from bot[T] at span 1
    ("out_NU", False, False),  # outside bot[B] from outside top[A]
    ("out_TU", True, False),   # outside bot[T] from outside top[A] at span 1
)


def round_up(n: int, m: int) -> int:
    return (n + m - 1) // m * m


@dataclasses.dataclass
class Grammar:
    """One cascade level, over fine labels that project onto coarse labels."""

    labels: List[str]
    coarse: np.ndarray            # int32[n_labels] -> coarse label id
    coarse_names: List[str]
    root: int                     # label id of the root symbol
    bin_rules: np.ndarray         # int32[nb, 3] (parent, left, right) label ids, rule-id order
    bin_score: np.ndarray         # float32[nb] log-probabilities
    un_rules: np.ndarray          # int32[nu, 2] (parent, child) label ids (identity rules included)
    un_score: np.ndarray          # float32[nu]
    words: List[str]
    lex_offsets: np.ndarray       # int64[V+1] CSR over word ids
    lex_label: np.ndarray         # int32[nnz] label id of an allowed preterminal
    lex_score: np.ndarray         # float32[nnz] log score
    name: str = "grammar"

    def validate(self) -> None:
        nl = len(self.labels)
        assert self.coarse.shape == (nl,)
        assert self.bin_rules.ndim == 2 and self.bin_rules.shape[1] == 3
        assert self.un_rules.ndim == 2 and self.un_rules.shape[1] == 2
        assert self.bin_score.shape == (self.bin_rules.shape[0],)
        assert self.un_score.shape == (self.un_rules.shape[0],)
        assert self.lex_offsets.shape == (len(self.words) + 1,)
        assert int(self.lex_offsets[-1]) == self.lex_label.shape[0] == self.lex_score.shape[0]
        for arr in (self.bin_rules, self.un_rules, self.lex_label):
            if arr.size:
                assert arr.min() >= 0 and arr.max() < nl
        assert 0 <= self.root < nl


@dataclasses.dataclass
class Segment:
    bits: np.ndarray                 # int32[mask_size] coarse-parent bitset
    subsegments: List[np.ndarray]    # rule positions (into the job's rule list), generator order


@dataclasses.dataclass
class CompiledLevel:
    """Derived tables for one level (what ``CLParserData.make`` builds)."""

    grammar: Grammar
    semiring: str
    nt_labels: np.ndarray            # int32[n_nt] label id of each nonterminal index
    t_labels: np.ndarray             # int32[n_t]
    label_nt: np.ndarray             # int32[n_labels] -> nt index or -1
    label_t: np.ndarray              # int32[n_labels] -> t index or -1
    root: int                        # nonterminal index of the root
    n_coarse: int
    cell_size: int
    mask_size: int
    nt_coarse: np.ndarray            # int32[n_nt]
    t_coarse: np.ndarray             # int32[n_t]
    bucket_rules: List[np.ndarray]   # per bucket: int32[n, 3] (parent, left, right) gpu ids, rule-id order
    bucket_scores: List[np.ndarray]  # per bucket: float32[n] (semiring space)
    bucket_ids: List[np.ndarray]     # per bucket: rule ids
    nu_rules: np.ndarray             # int32[n, 2] (parent nt, child nt) -- ntUnaries
    nu_scores: np.ndarray
    tu_rules: np.ndarray             # int32[n, 2] (parent nt, child t) -- tUnaries
    tu_scores: np.ndarray
    lex_offsets: np.ndarray
    lex_term: np.ndarray             # int32 terminal index
    lex_score: np.ndarray            # float32 log space (semiring applied on device)
    jobs: Dict[str, dict]            # per job: rules (rotated), segments, CSR tables
    unary_jobs: Dict[str, dict]
    viterbi: dict                    # backtrace tables
    members: dict                    # coarse -> fine member lists (NT and T spaces)

    @property
    def n_nt(self) -> int:
        return int(self.nt_labels.shape[0])

    @property
    def n_t(self) -> int:
        return int(self.t_labels.shape[0])

    @property
    def num_syms(self) -> int:
        return max(self.n_nt, self.n_t)


def from_log_space(semiring: str, scores: np.ndarray) -> np.ndarray:
    """``RuleSemiring.fromLogSpace`` (RuleSemiring.scala:30,53,86): identity for
    Viterbi/LogSum, ``math.exp(float).toFloat`` for Real."""
    scores = np.asarray(scores, dtype=np.float32)
    if semiring == "real":
        return np.exp(scores.astype(np.float64)).astype(np.float32)
    return scores.copy()


def _java_hashmap_order(keys_in_insertion_order: Sequence[int]) -> List[int]:
    """Iteration order of a ``java.util.HashMap<Integer, ...>`` filled in the
    given insertion order (keys distinct, small non-negative ints).  The table
    starts at 16 buckets and doubles while size > 0.75 * capacity; iteration
    walks buckets ``key & (cap - 1)`` in order, and within a bucket keeps
    insertion order (resizes split buckets without reordering)."""
    n = len(keys_in_insertion_order)
    cap = 16
    while n > cap * 3 // 4:
        cap *= 2
    pos = {k: i for i, k in enumerate(keys_in_insertion_order)}
    return sorted(keys_in_insertion_order, key=lambda k: ((k ^ (k >> 16)) & (cap - 1), pos[k]))


def coarse_parent_segments(parent_coarse: np.ndarray, mask_size: int) -> List[Segment]:
    """``CoarseParentSymbolGrammarClusterer.segmentBinaries`` over a job's rule
    list (positions 0..n-1 in rule order).  One segment per coarse parent with
    at least 300 rules (largest first), then one segment holding every
    remaining rule; each segment is cut into 8 equal sub-segments
    (``equalSizeSubsegmentBinaries``) and empty ones are dropped."""
    n = int(parent_coarse.shape[0])
    if n == 0:
        return []
    pc = np.asarray(parent_coarse, dtype=np.int64)
    keys, first = np.unique(pc, return_index=True)
    insertion = [int(k) for k in keys[np.argsort(first, kind="stable")]]
    pos_sorted = np.argsort(pc, kind="stable")           # rule positions grouped by coarse, rule order kept
    bounds = np.searchsorted(pc[pos_sorted], keys)
    by_parent = {int(k): pos_sorted[bounds[i]:(bounds[i + 1] if i + 1 < len(keys) else n)]
                 for i, k in enumerate(keys)}
    lists = [by_parent[c] for c in _java_hashmap_order(insertion)]
    lists.sort(key=lambda l: -len(l))  # stable, like Collections.sort
    segments: List[Segment] = []
    while lists:
        seg = lists.pop(0)
        if len(seg) < MIN_SINGLE_COARSE_PARENT_GROUP_SIZE:
            seg = np.concatenate([seg] + lists)
            lists = []
        subs = [s for s in _equal_size_subsegments(seg, NUM_SUBSEGMENTS) if s.size]
        if subs:
            bits = np.zeros(mask_size, dtype=np.int64)
            for c in np.unique(pc[seg]):
                bits[int(c) // 32] |= (1 << (int(c) % 32))
            bits = bits.astype(np.uint32).view(np.int32)
            segments.append(Segment(bits=bits, subsegments=subs))
    return segments


def _equal_size_subsegments(rules: np.ndarray, k: int) -> List[np.ndarray]:
    """``equalSizeSubsegmentBinaries``: ``floor(n/k)`` rules to each of the k
    sub-segments in list order, then the remainder one by one from the first."""
    n = int(rules.shape[0])
    per = n // k
    rest = rules[k * per:]
    return [np.concatenate([rules[i * per:(i + 1) * per], rest[i:i + 1]]).astype(np.int64)
            for i in range(k)]


def _csr(targets: np.ndarray, n_targets: int, order: np.ndarray) -> np.ndarray:
    counts = np.bincount(targets[order], minlength=n_targets) if order.size else np.zeros(n_targets, np.int64)
    rowptr = np.zeros(n_targets + 1, dtype=np.int32)
    np.cumsum(counts, out=rowptr[1:])
    return rowptr


def compile_level(g: Grammar, semiring: str = "viterbi") -> CompiledLevel:
    g.validate()
    assert semiring in SEMIRINGS
    nl = len(g.labels)
    bp, bl, br = g.bin_rules[:, 0], g.bin_rules[:, 1], g.bin_rules[:, 2]
    up, uc = g.un_rules[:, 0], g.un_rules[:, 1]

    # RuleStructure.scala:53-65: nonterminals are parents of binaries and of
    # non-identity unaries; everything else on a right-hand side is terminal.
    is_nt = np.zeros(nl, dtype=bool)
    is_nt[bp] = True
    nonid = up != uc
    is_nt[up[nonid]] = True
    used = is_nt.copy()
    used[bl] = True
    used[br] = True
    used[uc[nonid]] = True
    syms = np.nonzero(used)[0]
    nt_labels = syms[is_nt[syms]].astype(np.int32)
    t_labels = syms[~is_nt[syms]].astype(np.int32)
    label_nt = np.full(nl, -1, dtype=np.int32)
    label_t = np.full(nl, -1, dtype=np.int32)
    label_nt[nt_labels] = np.arange(nt_labels.shape[0], dtype=np.int32)
    label_t[t_labels] = np.arange(t_labels.shape[0], dtype=np.int32)
    assert label_nt[g.root] >= 0, "root must be a nonterminal"

    n_nt, n_t = nt_labels.shape[0], t_labels.shape[0]
    n_coarse = len(g.coarse_names)
    cell_size = round_up(max(n_nt, n_t), 32)
    mask_size = round_up(n_coarse, 32) // 32
    nt_coarse = g.coarse[nt_labels].astype(np.int32)
    t_coarse = g.coarse[t_labels].astype(np.int32)

    def gpu(lbl):
        return np.where(label_nt[lbl] >= 0, label_nt[lbl], label_t[lbl]).astype(np.int32)

    bscore = from_log_space(semiring, g.bin_score)
    uscore = from_log_space(semiring, g.un_score)

    lt, rt = ~is_nt[bl], ~is_nt[br]
    bucket_of = np.where(~lt & ~rt, NN, np.where(~lt & rt, NT, np.where(lt & ~rt, TN, TT)))
    bucket_rules, bucket_scores, bucket_ids = [], [], []
    for b in range(4):
        ids = np.nonzero(bucket_of == b)[0]
        rules = np.stack([label_nt[bp[ids]], gpu(bl[ids]), gpu(br[ids])], axis=1).astype(np.int32) \
            if ids.size else np.zeros((0, 3), np.int32)
        bucket_rules.append(rules)
        bucket_scores.append(bscore[ids].astype(np.float32))
        bucket_ids.append(ids.astype(np.int64))

    # RuleStructure.scala:94-96: drop unaries with a terminal parent; split by child.
    keep = is_nt[up]
    nu_ids = np.nonzero(keep & is_nt[uc])[0]
    tu_ids = np.nonzero(keep & ~is_nt[uc])[0]
    nu_rules = np.stack([label_nt[up[nu_ids]], label_nt[uc[nu_ids]]], axis=1).astype(np.int32) \
        if nu_ids.size else np.zeros((0, 2), np.int32)
    tu_rules = np.stack([label_nt[up[tu_ids]], label_t[uc[tu_ids]]], axis=1).astype(np.int32) \
        if tu_ids.size else np.zeros((0, 2), np.int32)
    nu_scores = uscore[nu_ids].astype(np.float32)
    tu_scores = uscore[tu_ids].astype(np.float32)

    # Lexicon: word -> (terminal index, log score).  Entries whose label is not
    # a terminal of this level are dropped (they could never be scored).
    lex_t = label_t[g.lex_label]
    keep_lex = lex_t >= 0
    word_of = np.repeat(np.arange(len(g.words)), np.diff(g.lex_offsets))
    lex_offsets = np.zeros(len(g.words) + 1, dtype=np.int64)
    np.cumsum(np.bincount(word_of[keep_lex], minlength=len(g.words)), out=lex_offsets[1:])
    lex_term = lex_t[keep_lex].astype(np.int32)
    lex_score = g.lex_score[keep_lex].astype(np.float32)

    coarse_nt = nt_coarse
    coarse_t = t_coarse

    nt_mem_off, nt_mem, nt_local = _coarse_members(coarse_nt, n_coarse)
    t_mem_off, t_mem, t_local = _coarse_members(coarse_t, n_coarse)
    members = dict(nt_mem_off=nt_mem_off, nt_mem=nt_mem, t_mem_off=t_mem_off, t_mem=t_mem)
    jobs: Dict[str, dict] = {}
    for name, bucket, rot, tgt_is_t, a_is_t, b_is_t in JOBS:
        rules = bucket_rules[bucket]
        scores = bucket_scores[bucket]
        if rot is None:
            tgt, ia, ib = rules[:, 0], rules[:, 1], rules[:, 2]
        elif rot == "L":   # BinaryRule(left, parent, right)
            tgt, ia, ib = rules[:, 1], rules[:, 0], rules[:, 2]
        else:              # BinaryRule(right, left, parent)
            tgt, ia, ib = rules[:, 2], rules[:, 1], rules[:, 0]
        tc = (coarse_t if tgt_is_t else coarse_nt)[tgt] if tgt.size else np.zeros(0, np.int32)
        ac = (coarse_t if a_is_t else coarse_nt)[ia] if ia.size else np.zeros(0, np.int32)
        bc = (coarse_t if b_is_t else coarse_nt)[ib] if ib.size else np.zeros(0, np.int32)
        segments = coarse_parent_segments(tc, mask_size)
        n_tgt = n_t if tgt_is_t else n_nt
        tgt_seg = np.full(n_tgt, -1, dtype=np.int32)
        rule_seg = np.zeros(tgt.shape[0], dtype=np.int32)
        for si, seg in enumerate(segments):
            for sub in seg.subsegments:
                rule_seg[sub] = si
        if tgt.size:
            tgt_seg[tgt] = rule_seg
            # every rule of one target shares a segment
            assert np.all(tgt_seg[tgt] == rule_seg)
        # CSR over targets; within a target, rules ordered by (coarse a,
        # coarse b, a, b) so that dense coarse blocks are contiguous runs.
        order = np.lexsort((ib, ia, bc, ac, tgt)) if tgt.size else np.zeros(0, np.int64)
        rowptr = _csr(tgt, n_tgt, order)
        seg_bits = np.stack([s.bits for s in segments]).astype(np.int32) if segments \
            else np.zeros((0, mask_size), np.int32)
        a_loc = t_local if a_is_t else nt_local
        b_loc = t_local if b_is_t else nt_local
        blocks = _pair_tables(tgt, ia, ib, scores, ac, bc, rule_seg, a_loc, b_loc, seg_bits, mask_size)
        jobs[name] = dict(
            bucket=bucket, rot=rot, tgt_is_t=tgt_is_t, a_is_t=a_is_t, b_is_t=b_is_t,
            tgt=tgt.astype(np.int32), ia=ia.astype(np.int32), ib=ib.astype(np.int32),
            score=scores.astype(np.float32), tgt_coarse=tc.astype(np.int32),
            segments=segments, seg_bits=seg_bits, tgt_seg=tgt_seg,
            rowptr=rowptr, csr_a=ia[order].astype(np.int32), csr_b=ib[order].astype(np.int32),
            csr_w=scores[order].astype(np.float32),
            csr_ac=ac[order].astype(np.int32), csr_bc=bc[order].astype(np.int32),
            **blocks,
        )

    unary_jobs: Dict[str, dict] = {}
    for name, tgt_is_t, c_is_t in UNARY_JOBS:
        if name == "in_NU":
            tgt, src, w = nu_rules[:, 0], nu_rules[:, 1], nu_scores
        elif name == "in_TU":
            tgt, src, w = tu_rules[:, 0], tu_rules[:, 1], tu_scores
        elif name == "out_NU":
            tgt, src, w = nu_rules[:, 1], nu_rules[:, 0], nu_scores
        else:
            tgt, src, w = tu_rules[:, 1], tu_rules[:, 0], tu_scores
        n_tgt = n_t if tgt_is_t else n_nt
        order = np.argsort(tgt, kind="stable") if tgt.size else np.zeros(0, np.int64)
        unary_jobs[name] = dict(
            tgt=tgt.astype(np.int32), src=src.astype(np.int32), score=w.astype(np.float32),
            rowptr=_csr(tgt, n_tgt, order), csr_src=src[order].astype(np.int32),
            csr_w=w[order].astype(np.float32))

    viterbi = _viterbi_tables(n_nt, bucket_rules, bucket_scores, nu_rules, nu_scores, tu_rules, tu_scores)

    return CompiledLevel(
        grammar=g, semiring=semiring, nt_labels=nt_labels, t_labels=t_labels,
        label_nt=label_nt, label_t=label_t, root=int(label_nt[g.root]),
        n_coarse=n_coarse, cell_size=cell_size, mask_size=mask_size,
        nt_coarse=nt_coarse, t_coarse=t_coarse,
        bucket_rules=bucket_rules, bucket_scores=bucket_scores, bucket_ids=bucket_ids,
        nu_rules=nu_rules, nu_scores=nu_scores, tu_rules=tu_rules, tu_scores=tu_scores,
        lex_offsets=lex_offsets, lex_term=lex_term, lex_score=lex_score,
        jobs=jobs, unary_jobs=unary_jobs, viterbi=viterbi, members=members)


PAIR_MIN_MEAN = 16      # the pair-factored layout pays off when coarse blocks hold this many rules


def _coarse_members(coarse_of: np.ndarray, n_coarse: int):
    """CSR from coarse symbol to its fine symbols (ascending) in one index space."""
    order = np.argsort(coarse_of, kind="stable")
    off = np.zeros(n_coarse + 1, np.int32)
    np.cumsum(np.bincount(coarse_of, minlength=n_coarse), out=off[1:])
    local = np.empty(coarse_of.shape[0], np.int32)
    local[order] = np.arange(coarse_of.shape[0]) - off[coarse_of[order]]
    return off, order.astype(np.int32), local


def _pair_tables(tgt, ia, ib, w, ac, bc, rule_seg, a_local, b_local, seg_bits, mask_size) -> dict:
    """Pair-factored layout for the device gather.

    Rules are grouped by the coarse projection (ca, cb) of their two operands
    ("pairs"), then by segment ("blocks"), then by target.  For one chart cell
    the device computes, per live pair, the max-plus outer product
    M[j][k] = max_s A_s[Y_j] + B_s[Z_k] over the pair's live splits once and
    applies every rule of the pair as M[j][k] + w; a pair is skipped when no
    staged split has a live Y on the left and a live Z on the right, which is
    exact (every skipped term is the semiring zero).  ``pair_gate`` ORs the
    segment bits of a pair's blocks so that pruned pairs are dropped before
    any block is visited.  Rules are packed as ``j | k << 8 | target << 16``
    with j, k the operands' positions among their coarse symbol's members.
    """
    n = tgt.shape[0]
    if n == 0:
        z = np.zeros(0, np.int32)
        return dict(pair_mode=0, pair_key=z, pair_gate=z, pair_blk=np.zeros(1, np.int32), blk_seg=z,
                    blk_ptr=np.zeros(1, np.int32), pair_rule=z, pair_w=np.zeros(0, np.float32))
    pkey = (bc.astype(np.int64) << 8) | ac.astype(np.int64)
    order = np.lexsort((b_local[ib], a_local[ia], tgt, rule_seg, pkey))
    pk, sg = pkey[order], rule_seg[order]
    pstart = np.flatnonzero(np.r_[True, pk[1:] != pk[:-1]])
    bstart = np.flatnonzero(np.r_[True, (pk[1:] != pk[:-1]) | (sg[1:] != sg[:-1])])
    npair, nblk = pstart.shape[0], bstart.shape[0]
    pair_blk = np.searchsorted(bstart, np.r_[pstart, n]).astype(np.int32)
    blk_seg = sg[bstart].astype(np.int32)
    gate = np.zeros((npair, mask_size), np.int64)
    pair_of_blk = np.repeat(np.arange(npair), np.diff(pair_blk))
    np.bitwise_or.at(gate, pair_of_blk, seg_bits[blk_seg].astype(np.uint32).astype(np.int64))
    packed = (a_local[ia[order]].astype(np.int64) | (b_local[ib[order]].astype(np.int64) << 8)
              | (tgt[order].astype(np.int64) << 16))
    mode = 2 if n / nblk >= PAIR_MIN_MEAN else 0
    return dict(pair_mode=mode, pair_key=pk[pstart].astype(np.int32),
                pair_gate=gate.astype(np.uint32).view(np.int32).reshape(-1).astype(np.int32),
                pair_blk=pair_blk, blk_seg=blk_seg, blk_ptr=np.r_[bstart, n].astype(np.int32),
                pair_rule=packed.astype(np.uint32).view(np.int32).astype(np.int32),
                pair_w=w[order].astype(np.float32))


def _viterbi_tables(n_nt, bucket_rules, bucket_scores, nu_rules, nu_scores, tu_rules, tu_scores) -> dict:
    """``CLViterbi.make`` (CLViterbi.scala:285-309,610-628): six rule groups
    (NN, NT, TN, TT, U, UT), each stable-sorted by parent, concatenated, with
    one CSR offset array of size ``6 * n_nt + 1``."""
    groups = []
    for b in (NN, NT, TN, TT):
        r, s = bucket_rules[b], bucket_scores[b]
        groups.append((r[:, 0], r[:, 1], r[:, 2], s))
    groups.append((nu_rules[:, 0], nu_rules[:, 1], np.zeros(nu_rules.shape[0], np.int32), nu_scores))
    groups.append((tu_rules[:, 0], tu_rules[:, 1], np.zeros(tu_rules.shape[0], np.int32), tu_scores))
    offsets = [np.zeros(1, np.int64)]
    left, right, score = [], [], []
    start = 0
    for p, l, r, s in groups:
        order = np.argsort(p, kind="stable")
        ps = p[order]
        ends = np.searchsorted(ps, np.arange(n_nt), side="right") + start
        offsets.append(ends.astype(np.int64))
        left.append(l[order]); right.append(r[order]); score.append(s[order])
        start += p.shape[0]
    return dict(
        offsets=np.concatenate(offsets).astype(np.int32),
        left=np.concatenate(left).astype(np.int32),
        right=np.concatenate(right).astype(np.int32),
        score=np.concatenate(score).astype(np.float32),
        group_offsets=np.arange(6, dtype=np.int32) * n_nt,
    )
