"""Continuous-batching server (puck_server_*): each result is the same alone
and in the mix, and equal to the oracle's parse.

Viterbi trees are compared bit for bit.  MBR trees come from float sums
accumulated in a data-dependent order; their symbols and shapes must agree
and their scores agree within the stated tolerance.
"""
import time

import numpy as np
import pytest

import oracle
from helpers import node_blocks, split_levels, split_sentences, write_grz
from puck_gb300.parser import CLParser, pack_sentences
from puck_gb300.server import CLServer, now_ns

pytestmark = pytest.mark.gpu

MBR_SCORE_RTOL = 1e-4


def _serve_alone(S, sents):
    out = []
    for s in sents:
        w, o, lens = pack_sentences([s])
        rid = S.submit_ids(w, o)[0]
        deadline = time.time() + 60
        while True:
            assert time.time() < deadline
            ids = S.poll(16, 50)
            if len(ids):
                assert ids[0] == rid
                nodes, st, _ = S.take(int(rid), int(lens[0]))
                assert st == 0
                out.append(nodes.copy())
                break
    return out


def _serve_mix(S, sents, gap_s=0.0005, chunk=3):
    """Submits in small groups with pauses, so sentences arrive while others
    are on the GPU; returns node blocks in input order."""
    ids, lens = [], []
    for k in range(0, len(sents), chunk):
        w, o, ln = pack_sentences(sents[k:k + chunk])
        ids.extend(int(x) for x in S.submit_ids(w, o))
        lens.extend(int(x) for x in ln)
        time.sleep(gap_s)
    want = dict(zip(ids, lens))
    got = {}
    deadline = time.time() + 120
    while len(got) < len(ids) and time.time() < deadline:
        for rid in S.poll(4096, 50):
            nodes, st, lat = S.take(int(rid), want[int(rid)])
            assert st == 0
            assert lat > 0
            got[int(rid)] = nodes.copy()
    assert len(got) == len(ids)
    return [got[i] for i in ids]


def test_server_viterbi_same_alone_and_in_mix_and_oracle():
    levels = split_levels("viterbi", "medium")
    path = write_grz(levels, "split_medium")
    sents = split_sentences(60, seed=21, mean=14, hi=30)
    sents[7] = sents[7][:1]  # a one-word sentence among longer ones
    r = oracle.run(levels, sents, mode="parse")
    ref = node_blocks(r.trees(), [len(s) for s in sents])
    S = CLServer(path, max_alloc_size=2 << 30, collect=False)
    try:
        alone = _serve_alone(S, sents[:12])
        mixed = _serve_mix(S, sents)
        st = S.stats()
    finally:
        S.close()
    for i in range(12):
        assert np.array_equal(alone[i], mixed[i]), i
    for i, blk in enumerate(mixed):
        assert np.array_equal(blk, ref[i]), i
    assert st["completed"] == 72 and st["failed"] == 0
    assert st["resident_peak"] > 1  # sentences shared the GPU


@pytest.mark.parametrize("lanes", [1, 3])
def test_server_lanes_match_oracle(lanes):
    """One lane, or three independent request loops sharing the GPU: every
    served tree equals the oracle's whatever lane it ran in."""
    levels = split_levels("viterbi", "medium")
    path = write_grz(levels, "split_medium")
    sents = split_sentences(45, seed=29, mean=16, hi=40)
    r = oracle.run(levels, sents, mode="parse")
    ref = node_blocks(r.trees(), [len(s) for s in sents])
    S = CLServer(path, max_alloc_size=2 << 30, collect=False, lanes=lanes)
    try:
        assert S.lanes() == lanes
        served = _serve_mix(S, sents, gap_s=0.0005, chunk=5)
        st = S.stats()
    finally:
        S.close()
    for i, blk in enumerate(served):
        assert np.array_equal(blk, ref[i]), i
    assert st["completed"] == len(sents) and st["failed"] == 0


def test_server_lengths_to_60_match_oracle_and_batch():
    """The serving lengths (lognormal mean 23 clipped 1-60) with several
    sentences of 41-60 words: each served tree equals the oracle's and the
    batch parse's, in a mix with short sentences."""
    levels = split_levels("viterbi", "medium")
    path = write_grz(levels, "split_medium")
    sents = split_sentences(36, seed=27, n_words=500, mean=23, hi=60)
    rng = np.random.default_rng(27)
    for i, n in zip((3, 11, 19, 30), (45, 52, 58, 60)):
        sents[i] = rng.integers(0, 500, size=n).astype(np.int32)
    assert max(len(s) for s in sents) == 60
    r = oracle.run(levels, sents, mode="parse")
    ref = node_blocks(r.trees(), [len(s) for s in sents])
    P = CLParser(path, max_alloc_size=2 << 30)
    w, o, lens = pack_sentences(sents)
    nodes, st = P.parse_ids(w, o)
    assert (st == 0).all()
    batch = node_blocks(nodes, lens)
    S = CLServer(path, max_alloc_size=2 << 30, collect=False)
    try:
        served = _serve_mix(S, sents, gap_s=0.001, chunk=4)
    finally:
        S.close()
    for i in range(len(sents)):
        assert np.array_equal(served[i], ref[i]), i
        assert np.array_equal(batch[i], ref[i]), i


def test_server_matches_batch_parse():
    levels = split_levels("viterbi", "small")
    path = write_grz(levels, "split_small")
    sents = split_sentences(80, seed=22, n_words=300, mean=12, hi=40)
    P = CLParser(path, max_alloc_size=1 << 30)
    w, o, lens = pack_sentences(sents)
    nodes, st = P.parse_ids(w, o)
    assert (st == 0).all()
    batch = node_blocks(nodes, lens)
    S = CLServer(path, max_alloc_size=1 << 30, collect=False, max_resident=16)
    try:
        served = _serve_mix(S, sents, gap_s=0.0, chunk=80)  # all at once, 16 resident at a time
        st = S.stats()
    finally:
        S.close()
    for i in range(len(sents)):
        assert np.array_equal(served[i], batch[i]), i
    assert st["resident_peak"] <= 16


def test_server_small_arena_admits_as_memory_frees():
    levels = split_levels("viterbi", "small")
    path = write_grz(levels, "split_small")
    sents = split_sentences(40, seed=23, n_words=300, mean=20, hi=40)
    r = oracle.run(levels, sents, mode="parse")
    ref = node_blocks(r.trees(), [len(s) for s in sents])
    # an arena a few sentences large: most requests wait for cells to free up
    S = CLServer(path, max_alloc_size=2 << 20, collect=False, max_length=40, max_resident=64)
    try:
        served = _serve_mix(S, sents, gap_s=0.0, chunk=40)
        st = S.stats()
    finally:
        S.close()
    for i in range(len(sents)):
        assert np.array_equal(served[i], ref[i]), i
    assert st["resident_peak"] < len(sents)


def test_server_mbr_same_alone_and_in_mix():
    levels = split_levels("real", "medium")
    path = write_grz(levels, "split_medium_real")
    sents = split_sentences(30, seed=24)
    r = oracle.run(levels, sents, mode="parse")
    ref = node_blocks(r.trees(), [len(s) for s in sents])
    S = CLServer(path, max_alloc_size=2 << 30, collect=False)
    try:
        alone = _serve_alone(S, sents[:6])
        mixed = _serve_mix(S, sents)
    finally:
        S.close()
    for i in range(len(sents)):
        a = mixed[i]
        assert np.array_equal(a[:, :3], ref[i][:, :3]), i
        assert np.allclose(a[:, 3].view(np.float32), ref[i][:, 3].view(np.float32), rtol=MBR_SCORE_RTOL,
                           atol=1e-5), i
        if i < 6:
            assert np.array_equal(alone[i][:, :3], a[:, :3])
            assert np.allclose(alone[i][:, 3].view(np.float32), a[:, 3].view(np.float32),
                               rtol=MBR_SCORE_RTOL, atol=1e-5)


def test_server_failures_and_futures():
    levels = split_levels("viterbi", "small")
    path = write_grz(levels, "split_small")
    good = split_sentences(5, seed=25, n_words=300, mean=8, hi=20)
    with CLServer(path, max_alloc_size=1 << 30, max_length=20) as S:
        futs = S.submit_many([good[0], [], list(range(25)), [good[1][0], 10 ** 6], good[2]])
        res = [f.result(60) for f in futs]
    assert res[0].is_success and res[4].is_success
    assert [r.error for r in res[1:4]] == ["EMPTY", "SENT_TOO_LONG", "OOV"]
    assert res[0].latency_ns > 0


def test_server_arrival_time_counts_latency():
    levels = split_levels("viterbi", "small")
    path = write_grz(levels, "split_small")
    s = split_sentences(1, seed=26, n_words=300, mean=8, hi=20)
    S = CLServer(path, max_alloc_size=1 << 30, collect=False)
    try:
        w, o, lens = pack_sentences(s)
        t0 = now_ns() - 5_000_000_000  # arrived 5 s ago
        rid = S.submit_ids(w, o, np.array([t0], np.int64))[0]
        deadline = time.time() + 60
        while not len(S.poll(4, 50)):
            assert time.time() < deadline
        _, st, lat = S.take(int(rid), int(lens[0]))
    finally:
        S.close()
    assert st == 0 and lat >= 5_000_000_000
