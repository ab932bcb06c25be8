"""Continuous-batching parse server over the C ABI (puck_server_* in
include/puck_gpu.h).

Mirrors the contract of the reference's batching front,
BatchFunctionAnnotatorService (dlwh/puck,
src/main/scala/puck/AnnotatorService.scala:29-78): ``submit`` returns one
future per sentence, completed with ``Success(tree)`` or ``Failure(msg)``,
and ``parse`` returns results in input order.  Unlike the reference there is
no flush interval or batch size: the library's request loop admits sentences
as chart memory frees up and batches them continuously on the GPU.
"""
from __future__ import annotations

import ctypes
import threading
import time
from concurrent.futures import Future
from typing import Dict, List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _lib
from .parser import (CLParserData, Failure, Success, nodes_to_mbr_tree, nodes_to_viterbi_tree,
                     pack_sentences)


def now_ns() -> int:
    """The server's clock (monotonic ns), for arrival times."""
    return int(_lib.load().puck_server_now_ns())


class CLServer:
    DECODE = {"auto": 0, "viterbi": 1, "mbr": 2}

    def __init__(self, grammar_path: str, max_alloc_size: int = 1 << 30, device: int = 0,
                 decode: str = "auto", max_length: int = 100, prune_threshold: float = -9.0,
                 max_resident: int = 0, collect: bool = True, profile: bool = False, lanes: int = 0):
        """collect=True starts a thread that takes finished requests and
        completes their futures; with collect=False the caller drives
        ``poll``/``take`` itself.  lanes: independent request loops (0: the
        library's default)."""
        L = _lib.load()
        self._L = L
        st = ctypes.c_int32(0)
        self._g = L.puck_grammar_load(grammar_path.encode(), ctypes.byref(st))
        if not self._g:
            raise _lib.PuckError(st.value, _lib.last_error())
        self.data = CLParserData.read_sequence(grammar_path)
        opt = _lib.Options()
        L.puck_default_options(ctypes.byref(opt))
        opt.mem_bytes = int(max_alloc_size)
        opt.device = device
        opt.decode = self.DECODE[decode]
        opt.max_length = max_length
        opt.prune_threshold = prune_threshold
        opt.max_batch_sentences = max_resident
        opt.profile = 1 if profile else 0
        opt.server_lanes = lanes
        self._s = L.puck_server_create(self._g, ctypes.byref(opt), ctypes.byref(st))
        if not self._s:
            err = _lib.last_error()
            L.puck_grammar_free(self._g)
            self._g = None
            raise _lib.PuckError(st.value, err)
        fine = self.data[-1]
        self.mbr = not (decode == "viterbi" or (decode == "auto" and fine.is_viterbi))
        self._futures: Dict[int, Tuple[Future, int]] = {}
        self._lock = threading.Lock()
        self._stop = threading.Event()
        self._collector: Optional[threading.Thread] = None
        if collect:
            self._collector = threading.Thread(target=self._collect, daemon=True)
            self._collector.start()

    # -- raw calls ------------------------------------------------------------
    def submit_ids(self, words: np.ndarray, offsets: np.ndarray,
                   arrival_ns: Optional[np.ndarray] = None) -> np.ndarray:
        n = len(offsets) - 1
        ids = np.zeros(n, np.int64)
        arr = None if arrival_ns is None else np.ascontiguousarray(arrival_ns, np.int64)
        _lib.check(self._L.puck_server_submit(self._s, words.ctypes.data, offsets.ctypes.data, n,
                                              None if arr is None else arr.ctypes.data, ids.ctypes.data))
        return ids

    def poll(self, max_ids: int = 4096, wait_ms: int = 10) -> np.ndarray:
        ids = np.zeros(max_ids, np.int64)
        k = self._L.puck_server_poll(self._s, ids.ctypes.data, max_ids, wait_ms)
        return ids[:k]

    def take(self, rid: int, n: int) -> Tuple[np.ndarray, int, int]:
        """(nodes[2n-1, 4] int32 view, status, latency ns) of a finished request."""
        nodes = np.zeros((max(2 * n - 1, 1), 4), np.int32)
        st = ctypes.c_int32(0)
        lat = ctypes.c_int64(0)
        _lib.check(self._L.puck_server_take(self._s, int(rid), nodes.ctypes.data, nodes.shape[0],
                                            ctypes.byref(st), ctypes.byref(lat)))
        return nodes[:max(2 * n - 1, 0)], int(st.value), int(lat.value)

    def lanes(self) -> int:
        """Lanes (independent request loops) the server runs."""
        return int(self._L.puck_server_lanes(self._s))

    def stats(self) -> dict:
        s = _lib.ServerStats()
        _lib.check(self._L.puck_server_get_stats(self._s, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def pass_ms(self, level: int) -> List[float]:
        """[lexicon, inside, outside, masks, decode] CUDA-event ms of one level
        summed over ticks (needs profile=True)."""
        out = (ctypes.c_double * 5)()
        _lib.check(self._L.puck_server_pass_ms(self._s, level, out))
        return list(out)

    # -- future-based API -------------------------------------------------------
    def _word_ids(self, sentence: Sequence[Union[str, int]]) -> List[int]:
        # a word missing from the lexicon takes its unknown-word class where
        # the lexicon has one (puck_grammar_word_id_at)
        out = []
        for i, w in enumerate(sentence):
            if isinstance(w, (int, np.integer)):
                out.append(int(w))
            else:
                out.append(self._L.puck_grammar_word_id_at(self._g, str(w).encode(), i))
        return out

    def submit_many(self, sentences: Sequence[Sequence[Union[str, int]]]) -> List[Future]:
        ids = [self._word_ids(s) for s in sentences]
        words, offsets, lens = pack_sentences(ids)
        futs = [Future() for _ in sentences]
        with self._lock:  # register before the collector can see the ids
            rids = self.submit_ids(words, offsets)
            for f, rid, n in zip(futs, rids, lens):
                self._futures[int(rid)] = (f, int(n))
        return futs

    def submit(self, sentence: Sequence[Union[str, int]]) -> Future:
        return self.submit_many([sentence])[0]

    def parse(self, sentences: Sequence[Sequence[Union[str, int]]], timeout: Optional[float] = None) -> list:
        """Results in input order (the reference service's ordered output)."""
        return [f.result(timeout) for f in self.submit_many(sentences)]

    def _result(self, nodes: np.ndarray, status: int):
        if status != 0:
            return Failure(_lib.STATUS.get(status, str(status)))
        fine = self.data[-1]
        try:
            t = nodes_to_mbr_tree(nodes, fine) if self.mbr else nodes_to_viterbi_tree(nodes, fine)
            return Success(t)
        except Exception as ex:  # the reference maps extraction errors to Failure
            return Failure(str(ex))

    def _collect(self) -> None:
        while not self._stop.is_set():
            ids = self.poll(4096, 20)
            for rid in ids:
                with self._lock:
                    f, n = self._futures.pop(int(rid))
                nodes, status, lat = self.take(int(rid), n)
                res = self._result(nodes, status)
                res.latency_ns = lat
                f.set_result(res)

    def close(self) -> None:
        """Waits for every submitted sentence, then stops the server."""
        if getattr(self, "_s", None):
            if self._collector is not None:
                while True:
                    with self._lock:
                        left = len(self._futures)
                    if not left:
                        break
                    time.sleep(0.005)
                self._stop.set()
                self._collector.join()
            self._L.puck_server_destroy(self._s)
            self._s = None
        if getattr(self, "_g", None):
            self._L.puck_grammar_free(self._g)
            self._g = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
