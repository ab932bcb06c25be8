"""Python mirror of the reference's parser API over the C ABI.

``CLParser`` keeps the names, argument meaning and error behaviour of
dlwh/puck's ``puck.parser.CLParser`` (src/main/scala/puck/parser/CLParser.scala:46-89):
``parse`` returns one ``Success(tree)`` / ``Failure(error)`` per sentence,
``partitions`` the per-sentence log partition, ``inside_outside`` runs the
passes without extraction, ``release`` frees the device state.  The work runs
in libpuck_gb300.so; this module only converts words to ids and preorder
nodes to trees.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import List, Optional, Sequence, Union

import numpy as np

from . import _lib, grz


@dataclasses.dataclass
class Tree:
    label: str
    children: List["Tree"]
    begin: int
    end: int

    def render(self, words: Sequence[str]) -> str:
        """One-line bracketed form, words at the leaves."""
        if not self.children:
            return f"({self.label} {words[self.begin]})"
        return "(" + self.label + " " + " ".join(c.render(words) for c in self.children) + ")"

    def preterminal_labels(self) -> List[str]:
        if not self.children:
            return [self.label]
        out: List[str] = []
        for c in self.children:
            out.extend(c.preterminal_labels())
        return out


@dataclasses.dataclass
class Success:
    tree: Tree

    def get(self) -> Tree:
        return self.tree

    @property
    def is_success(self) -> bool:
        return True


@dataclasses.dataclass
class Failure:
    error: str

    def get(self) -> Tree:
        raise RuntimeError(self.error)

    @property
    def is_success(self) -> bool:
        return False


Try = Union[Success, Failure]


def debinarize(t: Tree) -> Tree:
    """Splice out intermediate ``@`` nodes and identity unaries."""
    kids: List[Tree] = []
    for c in t.children:
        c = debinarize(c)
        if c.label.startswith("@") and c.children:
            kids.extend(c.children)
        else:
            kids.append(c)
    if len(kids) == 1 and kids[0].label == t.label and kids[0].children:
        return kids[0]
    return Tree(t.label, kids, t.begin, t.end)


class CLParserData:
    """One cascade level of a compiled ``grammar.grz`` (names and projections)."""

    def __init__(self, info: grz.LevelInfo):
        self.info = info
        self.nt_coarse = info.arrays.get("nt_coarse")
        self.t_coarse = info.arrays.get("t_coarse")

    @property
    def is_viterbi(self) -> bool:
        return self.info.is_viterbi

    @staticmethod
    def read_sequence(path: str) -> List["CLParserData"]:
        levels = grz.read_sequence(path, load_arrays=False)
        import zipfile
        with zipfile.ZipFile(path) as z:
            for i, lv in enumerate(levels):
                for k in ("nt_coarse", "t_coarse"):
                    lv.arrays[k] = grz._parse_arr(z.read(f"parser-{i}/arrays/{k}"))
        return [CLParserData(l) for l in levels]

    @staticmethod
    def write_sequence(path: str, compiled_levels) -> None:
        grz.write_sequence(path, compiled_levels)

    # the reference's names (CLParser.scala:1302-1317; CLParserData.isViterbi)
    readSequence = read_sequence
    writeSequence = write_sequence
    isViterbi = is_viterbi

    def nt_label(self, i: int) -> str:
        return self.info.coarse_names[int(self.nt_coarse[i])]

    def t_label(self, i: int) -> str:
        return self.info.coarse_names[int(self.t_coarse[i])]


def nodes_to_viterbi_tree(nodes: np.ndarray, data: CLParserData) -> Tree:
    """``extractParses`` (CLParser.scala:529-585): rebuild the binarized tree
    from preorder ``{top, bot, width}`` nodes, projecting symbols to coarse labels."""
    pos = [0]

    def rec(p: int) -> Tree:
        top, bot, width = int(nodes[p, 0]), int(nodes[p, 1]), int(nodes[p, 2])
        if width == 1:
            pos[0] += 1
            if not (0 <= bot < data.info.n_t):
                raise ValueError(f"terminal index {bot} out of range")
            part = Tree(data.t_label(bot), [], pos[0] - 1, pos[0])
        else:
            if not (0 <= bot < data.info.n_nt):
                raise ValueError(f"nonterminal index {bot} out of range")
            lc = rec(p + 1)
            if pos[0] != lc.end:
                raise ValueError("malformed tree")
            rc = rec(p + 2 * (lc.end - lc.begin))
            if pos[0] != rc.end:
                raise ValueError("malformed tree")
            part = Tree(data.nt_label(bot), [lc, rc], lc.begin, rc.end)
        if top == -1:
            return part
        if not (0 <= top < data.info.n_nt):
            raise ValueError(f"nonterminal index {top} out of range")
        return Tree(data.nt_label(top), [part], part.begin, part.end)

    return rec(0)


def nodes_to_mbr_tree(nodes: np.ndarray, data: CLParserData) -> Tree:
    """``extractMBRParses`` extraction (CLParser.scala:660-683): coarse labels."""
    names = data.info.coarse_names
    pos = [0]

    def rec(p: int) -> Tree:
        top, bot, width = int(nodes[p, 0]), int(nodes[p, 1]), int(nodes[p, 2])
        if width == 1:
            pos[0] += 1
            part = Tree(names[bot], [], pos[0] - 1, pos[0])
        else:
            lc = rec(p + 1)
            rc = rec(p + 2 * (lc.end - lc.begin))
            part = Tree(names[bot], [lc, rc], lc.begin, rc.end)
        if top == -1:
            return part
        return Tree(names[top], [part], part.begin, part.end)

    return rec(0)


def pack_sentences(sentences: Sequence[Sequence[int]]):
    lens = np.fromiter((len(s) for s in sentences), dtype=np.int64, count=len(sentences))
    offsets = np.zeros(len(sentences) + 1, np.int64)
    np.cumsum(lens, out=offsets[1:])
    words = np.concatenate([np.asarray(s, np.int32) for s in sentences]) if len(sentences) else np.zeros(0, np.int32)
    return np.ascontiguousarray(words, np.int32), offsets, lens


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class CLParser:
    """GPU parser over a compiled grammar cascade (coarse levels first)."""

    DECODE = {"auto": 0, "viterbi": 1, "mbr": 2}

    def __init__(self, grammar_path: str, max_alloc_size: int = 1 << 30, profile: bool = False,
                 device: int = 0, decode: str = "auto", max_length: int = 100,
                 prune_threshold: float = -9.0, max_batch_sentences: int = 0, use_graphs: bool = False,
                 tensor_cores: bool = False):
        L = _lib.load()
        st = ctypes.c_int32(0)
        self._g = L.puck_grammar_load(grammar_path.encode(), ctypes.byref(st))
        if not self._g:
            raise _lib.PuckError(st.value, _lib.last_error())
        self.data = CLParserData.read_sequence(grammar_path)
        opt = _lib.Options()
        L.puck_default_options(ctypes.byref(opt))
        opt.mem_bytes = int(max_alloc_size)
        opt.device = device
        opt.profile = 1 if profile else 0
        opt.decode = self.DECODE[decode]
        opt.max_length = max_length
        opt.prune_threshold = prune_threshold
        opt.max_batch_sentences = max_batch_sentences
        opt.use_graphs = 1 if use_graphs else 0
        opt.tensor_cores = 1 if tensor_cores else 0
        self.max_length = max_length
        self._p = L.puck_parser_create(self._g, ctypes.byref(opt), ctypes.byref(st))
        if not self._p:
            err = _lib.last_error()
            L.puck_grammar_free(self._g)
            self._g = None
            raise _lib.PuckError(st.value, err)
        self._L = L
        self.decode = decode

    # -- word handling ----------------------------------------------------
    def word_ids(self, sentence: Sequence[Union[str, int]]) -> List[int]:
        # a word missing from the lexicon takes its unknown-word class where
        # the lexicon has one (puck_grammar_word_id_at)
        out = []
        for i, w in enumerate(sentence):
            if isinstance(w, (int, np.integer)):
                out.append(int(w))
            else:
                out.append(self._L.puck_grammar_word_id_at(self._g, str(w).encode(), i))
        return out

    @property
    def is_viterbi(self) -> bool:
        return self.data[-1].is_viterbi

    # -- raw id-level calls (the C ABI) -----------------------------------
    def parse_ids(self, words: np.ndarray, offsets: np.ndarray):
        n = len(offsets) - 1
        lens = np.diff(offsets)
        total = int(np.maximum(2 * lens - 1, 0).sum())
        nodes = np.zeros((total, 4), np.int32)
        status = np.zeros(n, np.int32)
        _lib.check(self._L.puck_parse(self._p, _ptr(words), _ptr(offsets), n, _ptr(nodes), _ptr(status)))
        return nodes, status

    def partitions_ids(self, words: np.ndarray, offsets: np.ndarray):
        n = len(offsets) - 1
        out = np.zeros(n, np.float32)
        status = np.zeros(n, np.int32)
        _lib.check(self._L.puck_partitions(self._p, _ptr(words), _ptr(offsets), n, _ptr(out), _ptr(status)))
        return out, status

    def inside_outside_ids(self, words: np.ndarray, offsets: np.ndarray) -> None:
        n = len(offsets) - 1
        _lib.check(self._L.puck_inside_outside(self._p, _ptr(words), _ptr(offsets), n))

    # -- reference-shaped API ---------------------------------------------
    def parse(self, sentences: Sequence[Sequence[Union[str, int]]]) -> List[Try]:
        ids = [self.word_ids(s) for s in sentences]
        words, offsets, lens = pack_sentences(ids)
        nodes, status = self.parse_ids(words, offsets)
        nodes = nodes.view(np.int32)
        out: List[Try] = []
        start = 0
        fine = self.data[-1]
        mbr = not (self.decode == "viterbi" or (self.decode == "auto" and fine.is_viterbi))
        for i, n in enumerate(lens):
            k = max(2 * int(n) - 1, 0)
            if status[i] != 0:
                out.append(Failure(_lib.STATUS.get(int(status[i]), str(status[i]))))
            else:
                try:
                    blk = nodes[start:start + k]
                    t = nodes_to_mbr_tree(blk, fine) if mbr else nodes_to_viterbi_tree(blk, fine)
                    out.append(Success(t))
                except Exception as ex:  # the reference maps extraction errors to Failure
                    out.append(Failure(str(ex)))
            start += k
        return out

    def partitions(self, sentences: Sequence[Sequence[Union[str, int]]]) -> List[float]:
        ids = [self.word_ids(s) for s in sentences]
        words, offsets, _ = pack_sentences(ids)
        z, _ = self.partitions_ids(words, offsets)
        return [float(v) for v in z]

    def inside_outside(self, sentences: Sequence[Sequence[Union[str, int]]]) -> None:
        ids = [self.word_ids(s) for s in sentences]
        words, offsets, _ = pack_sentences(ids)
        self.inside_outside_ids(words, offsets)

    # the reference's names (CLParser.scala:60,71)
    insideOutside = inside_outside
    isViterbi = is_viterbi

    # -- device state of the last call (single batch only) ----------------
    def debug_num_cells(self) -> int:
        return int(self._L.puck_debug_num_cells(self._p))

    def debug_copy(self, level: int, which: str) -> np.ndarray:
        kinds = {"inside": 0, "outside": 1, "masks": 2, "iscale": 3, "oscale": 4, "mbr": 5}
        nc = self.debug_num_cells()
        info = self.data[level].info
        if which in ("inside", "outside"):
            out = np.empty((nc, info.cell_size), np.float32)
        elif which == "masks":
            out = np.empty((nc, info.mask_size), np.int32)
        elif which == "mbr":
            out = np.empty((nc, 2), np.float32)
        else:
            out = np.empty(nc, np.float32)
        _lib.check(self._L.puck_debug_copy(self._p, level, kinds[which], _ptr(out), out.nbytes))
        return out

    def stats(self) -> dict:
        s = _lib.Stats()
        _lib.check(self._L.puck_parser_stats(self._p, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def pass_ms(self, level: int):
        """Per-level [inside, outside, masks, decode] CUDA-event ms and launch
        counts of the last call."""
        ms = (ctypes.c_double * 4)()
        n = (ctypes.c_int64 * 4)()
        _lib.check(self._L.puck_parser_pass_ms(self._p, level, ms, n))
        return list(ms), list(n)

    def autotune(self, words: np.ndarray, offsets: np.ndarray) -> dict:
        """Runs the library's autotuner on a sample (word ids + offsets) and
        returns the gather form per level, the span band of the flat-tile
        inside form per level and the split waves."""
        nl = len(self.data)
        out = np.zeros(nl + 1, np.int32)
        _lib.check(self._L.puck_parser_autotune(self._p, _ptr(words), _ptr(offsets), len(offsets) - 1, _ptr(out)))
        names = {0: "target-major", 2: "pair-factored"}
        return {"levels": [names.get(int(m), str(int(m))) for m in out[:nl]],
                "flat_from": [self.flat_from(l) for l in range(nl)], "waves": int(out[nl]) / 100.0}

    def set_flat_from(self, level: int, span: int) -> None:
        """Pins the first span whose inside launch of `level` runs the
        flat-tile form (0: none)."""
        _lib.check(self._L.puck_parser_set_flat_from(self._p, level, span))

    def flat_from(self, level: int) -> int:
        """First span whose inside launch of `level` runs the flat-tile form
        (0: none)."""
        r = self._L.puck_parser_flat_from(self._p, level)
        if r < 0:
            raise ValueError(f"bad level {level}")
        return r

    def tensor_cores(self, level: int):
        """(True, "") if the level's inside binary sums run on tensor cores,
        else (False, reason)."""
        buf = ctypes.create_string_buffer(256)
        r = self._L.puck_parser_tensor_cores(self._p, level, buf, 256)
        if r < 0:
            raise ValueError(f"bad level {level}")
        return r == 1, buf.value.decode()

    def level_work(self, level: int):
        """(binary work units, +0.0 partials) of one level in the last call."""
        out = (ctypes.c_int64 * 2)()
        _lib.check(self._L.puck_parser_level_work(self._p, level, out))
        return int(out[0]), int(out[1])

    def release(self) -> None:
        if getattr(self, "_p", None):
            self._L.puck_parser_destroy(self._p)
            self._p = None
        if getattr(self, "_g", None):
            self._L.puck_grammar_free(self._g)
            self._g = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass
