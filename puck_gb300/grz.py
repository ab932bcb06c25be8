"""The compiled grammar artifact, ``grammar.grz``.

Like the reference (``CLParserData.writeSequence``,
src/main/scala/puck/parser/CLParser.scala:1302-1317) the artifact is a zip
holding a ``parserNames`` entry (one ``parser-<i>`` per cascade level, coarse
first) and one directory per level.  The payloads are this library's own:
a ``header`` of ``key value`` lines, typed little-endian arrays (16-byte
header: magic ``PKA1``, dtype tag, int64 count) and newline-separated name
lists.  Entries are stored uncompressed so the C++ loader can read them
without a zlib dependency.

Reference-produced archives hold Java-serialised objects and OpenCL program
binaries (``*.program``).  Those are never decoded: :func:`read_sequence`
refuses an archive without this library's ``header`` entries, and skips any
``.program`` entry it meets.
"""
from __future__ import annotations

import io
import struct
import zipfile
from typing import Dict, List, Sequence

import numpy as np

from .grammar import JOBS, UNARY_JOBS, CompiledLevel

MAGIC = b"PKA1"
DTYPES = {np.dtype(np.int32): b"i4  ", np.dtype(np.float32): b"f4  ", np.dtype(np.int64): b"i8  "}
RDTYPES = {v: k for k, v in DTYPES.items()}
FORMAT_VERSION = 1


def _arr_bytes(a: np.ndarray) -> bytes:
    a = np.ascontiguousarray(a)
    if a.dtype not in DTYPES:
        raise TypeError(f"unsupported dtype {a.dtype}")
    return MAGIC + DTYPES[a.dtype] + struct.pack("<q", a.size) + a.astype(a.dtype.newbyteorder("<")).tobytes()


def _parse_arr(b: bytes) -> np.ndarray:
    if b[:4] != MAGIC:
        raise ValueError("bad array entry")
    dt = RDTYPES[b[4:8]]
    (n,) = struct.unpack("<q", b[8:16])
    return np.frombuffer(b[16:16 + n * dt.itemsize], dtype=dt.newbyteorder("<")).astype(dt).copy()


def level_arrays(cl: CompiledLevel) -> Dict[str, np.ndarray]:
    """Every array a level needs on the device (and for the oracle)."""
    out: Dict[str, np.ndarray] = {
        "nt_coarse": cl.nt_coarse, "t_coarse": cl.t_coarse,
        "nt_labels": cl.nt_labels, "t_labels": cl.t_labels,
        "lex_off": cl.lex_offsets.astype(np.int64), "lex_term": cl.lex_term, "lex_score": cl.lex_score,
        "v_off": cl.viterbi["offsets"], "v_left": cl.viterbi["left"],
        "v_right": cl.viterbi["right"], "v_score": cl.viterbi["score"],
        **cl.members,
    }
    for name, *_ in JOBS:
        j = cl.jobs[name]
        packed = (j["csr_a"].astype(np.int64) | (j["csr_b"].astype(np.int64) << 16)).astype(np.int32)
        out[f"{name}/rowptr"] = j["rowptr"]
        out[f"{name}/ab"] = packed
        out[f"{name}/w"] = j["csr_w"]
        out[f"{name}/ac"] = j["csr_ac"]
        out[f"{name}/bc"] = j["csr_bc"]
        out[f"{name}/tgt_seg"] = j["tgt_seg"]
        out[f"{name}/seg_bits"] = j["seg_bits"].reshape(-1)
        out[f"{name}/pair_mode"] = np.asarray([j["pair_mode"]], np.int32)
        for k in ("pair_key", "pair_gate", "pair_blk", "blk_seg", "blk_ptr", "pair_rule", "pair_w"):
            out[f"{name}/{k}"] = j[k]
        # rule-order form and sub-segments (the oracle's view)
        out[f"{name}/tgt"] = j["tgt"]
        out[f"{name}/ia"] = j["ia"]
        out[f"{name}/ib"] = j["ib"]
        out[f"{name}/score"] = j["score"]
        sub_seg, sub_off, sub_rules = [], [0], []
        for si, seg in enumerate(j["segments"]):
            for sub in seg.subsegments:
                sub_seg.append(si)
                sub_off.append(sub_off[-1] + len(sub))
                sub_rules.append(np.asarray(sub, np.int32))
        out[f"{name}/sub_seg"] = np.asarray(sub_seg, np.int32)
        out[f"{name}/sub_off"] = np.asarray(sub_off, np.int32)
        out[f"{name}/sub_rules"] = np.concatenate(sub_rules).astype(np.int32) if sub_rules else np.zeros(0, np.int32)
    for name, *_ in UNARY_JOBS:
        u = cl.unary_jobs[name]
        out[f"{name}/rowptr"] = u["rowptr"]
        out[f"{name}/src"] = u["csr_src"]
        out[f"{name}/w"] = u["csr_w"]
        out[f"{name}/tgt"] = u["tgt"]
        out[f"{name}/osrc"] = u["src"]
        out[f"{name}/score"] = u["score"]
    return {k: np.ascontiguousarray(v) for k, v in out.items()}


def _entry(z: zipfile.ZipFile, name: str, data: bytes) -> None:
    info = zipfile.ZipInfo(name, date_time=(1980, 1, 1, 0, 0, 0))   # fixed: same grammar, same bytes
    info.compress_type = zipfile.ZIP_STORED
    z.writestr(info, data)


def write_sequence(path: str, levels: Sequence[CompiledLevel]) -> None:
    names = [f"parser-{i}" for i in range(len(levels))]
    with zipfile.ZipFile(path, "w", compression=zipfile.ZIP_STORED) as z:
        _entry(z, "parserNames", "\n".join(names).encode("utf-8"))
        for name, cl in zip(names, levels):
            g = cl.grammar
            hdr = {
                "format": FORMAT_VERSION, "semiring": cl.semiring, "n_nt": cl.n_nt, "n_t": cl.n_t,
                "cell_size": cl.cell_size, "mask_size": cl.mask_size, "n_coarse": cl.n_coarse,
                "root": cl.root, "n_words": len(g.words), "name": g.name,
            }
            _entry(z, f"{name}/header", "".join(f"{k} {v}\n" for k, v in hdr.items()).encode("utf-8"))
            for k, a in level_arrays(cl).items():
                _entry(z, f"{name}/arrays/{k}", _arr_bytes(a))
            _entry(z, f"{name}/nt_names.txt", "\n".join(g.labels[i] for i in cl.nt_labels).encode("utf-8"))
            _entry(z, f"{name}/t_names.txt", "\n".join(g.labels[i] for i in cl.t_labels).encode("utf-8"))
            _entry(z, f"{name}/coarse_names.txt", "\n".join(g.coarse_names).encode("utf-8"))
            _entry(z, f"{name}/words.txt", "\n".join(g.words).encode("utf-8"))


class LevelInfo:
    """What the host side needs from one level of an artifact (names, sizes)."""

    def __init__(self, header: Dict[str, str], nt_names, t_names, coarse_names, words, arrays):
        self.header = header
        self.semiring = header["semiring"]
        self.n_nt = int(header["n_nt"])
        self.n_t = int(header["n_t"])
        self.cell_size = int(header["cell_size"])
        self.mask_size = int(header["mask_size"])
        self.n_coarse = int(header["n_coarse"])
        self.root = int(header["root"])
        self.nt_names = nt_names
        self.t_names = t_names
        self.coarse_names = coarse_names
        self.words = words
        self.word_index = {w: i for i, w in enumerate(words)}
        self.arrays = arrays

    @property
    def is_viterbi(self) -> bool:
        return self.semiring == "viterbi"


def read_sequence(path: str, load_arrays: bool = False) -> List[LevelInfo]:
    out = []
    with zipfile.ZipFile(path, "r") as z:
        entries = set(z.namelist())
        names = [l.strip() for l in z.read("parserNames").decode("utf-8").splitlines() if l.strip()]
        for n in names:
            if f"{n}/header" not in entries:
                raise ValueError(f"{path}: level {n} has no header entry (not a puck_gb300 artifact; "
                                 "reference archives with serialised objects are not decoded)")
            header = dict(l.split(" ", 1) for l in z.read(f"{n}/header").decode("utf-8").splitlines() if l)
            txt = lambda e: [l for l in z.read(f"{n}/{e}").decode("utf-8").split("\n")] \
                if z.read(f"{n}/{e}") else []
            arrays = {}
            if load_arrays:
                for e in entries:
                    if e.startswith(f"{n}/arrays/") and not e.endswith(".program"):
                        arrays[e[len(f"{n}/arrays/"):]] = _parse_arr(z.read(e))
            out.append(LevelInfo(header, txt("nt_names.txt"), txt("t_names.txt"), txt("coarse_names.txt"),
                                 txt("words.txt"), arrays))
    return out
