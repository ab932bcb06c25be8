"""Host-side check of the flat-tile and pair-major tables (no GPU).

The library builds, per job, sub-tiles of at most 16 x 16 members, blocks
of at most 32 targets and bank-scheduled four-rule records; on the coarse
level it builds the same layout over groups of 16 coarse ids.
puck_debug_flat_check builds them as a parser would and rebuilds every rule
they hold: the rules must equal the job's target-major rule table exactly
(target, operands and weight bits), with every tile entry inside its tile.
"""
import ctypes

import pytest

from helpers import small_pcfg_levels, split_levels, write_grz
from puck_gb300 import _lib

JOBS = range(12)  # in_NN .. in_TT, then the eight outside jobs


def _grammar(levels, name):
    L = _lib.load()
    st = ctypes.c_int32(0)
    g = L.puck_grammar_load(write_grz(levels, name).encode(), ctypes.byref(st))
    assert g, _lib.last_error()
    return L, g


@pytest.mark.parametrize("size,semiring", [("big", "viterbi"), ("deep", "viterbi"), ("wide", "viterbi"),
                                           ("medium", "real"), ("big", "real")])
def test_fine_level_flat_tables_hold_every_rule_once(size, semiring):
    """25-33 refinements (sub-tiles of 16 + 16 + rest, blocks cut into runs
    of 32 targets), up to 17, and many small pairs; Viterbi (padding -inf)
    and sum-product (padding 0) weights; inside and outside jobs."""
    levels = split_levels(semiring, size)
    L, g = _grammar(levels, f"split_{size}" + ("_real" if semiring == "real" else ""))
    try:
        out = (ctypes.c_int64 * 4)()
        subtiles = 0
        for job in JOBS:
            rc = L.puck_debug_flat_check(g, 1, job, 0, out)
            assert rc == 0, (job, rc)
            subtiles += out[1]
        if size == "big":
            assert subtiles > sum(len(levels[1].jobs[n]["pair_key"]) for n in levels[1].jobs
                                  if "pair_key" in levels[1].jobs[n])  # pairs were cut
    finally:
        L.puck_grammar_free(g)


def test_bench_grammar_flat_tables_hold_every_rule_once():
    """The 1,091-symbol, 1.5M-rule bench grammar: all twelve jobs of its
    fine level."""
    levels = split_levels("viterbi", "c1")
    L, g = _grammar(levels, "split_c1")
    try:
        out = (ctypes.c_int64 * 4)()
        rules = 0
        for job in range(4):
            assert L.puck_debug_flat_check(g, 1, job, 0, out) == 0, job
            rules += out[0]
        assert rules == sum(levels[1].bucket_rules[b].shape[0] for b in range(4))
        for job in range(4, 12):
            assert L.puck_debug_flat_check(g, 1, job, 0, out) == 0, job
    finally:
        L.puck_grammar_free(g)


@pytest.mark.parametrize("size", ["medium", "big"])
def test_coarse_level_group_tables_hold_every_rule_once(size):
    """The coarse level (one symbol per coarse id) as pairs of groups of 16
    coarse ids, inside jobs."""
    levels = split_levels("viterbi", size)
    L, g = _grammar(levels, f"split_{size}")
    try:
        out = (ctypes.c_int64 * 4)()
        for job in range(4):
            rc = L.puck_debug_flat_check(g, 0, job, 1, out)
            assert rc == 0, (job, rc)
            assert out[0] == levels[0].jobs[["in_NN", "in_NT", "in_TN", "in_TT"][job]]["tgt"].shape[0]
    finally:
        L.puck_grammar_free(g)


@pytest.mark.parametrize("size", ["medium", "c1"])
def test_coarse_level_pair_major_tables_hold_every_rule_once(size):
    """The coarse level's pair-major tables (every job: each distinct child
    pair once, with all of its rules)."""
    levels = split_levels("viterbi", size)
    L, g = _grammar(levels, f"split_{size}")
    try:
        out = (ctypes.c_int64 * 4)()
        for job in JOBS:
            assert L.puck_debug_flat_check(g, 0, job, 2, out) == 0, job
            assert 0 < out[1] <= out[0]
    finally:
        L.puck_grammar_free(g)


def test_pair_major_tables_skip_dense_targets():
    """A job whose targets average more than 48 rules keeps the target-major
    scan: the 64 + 32-symbol plain grammar's NN job (137 per target)."""
    levels = small_pcfg_levels()
    L, g = _grammar(levels, "small_pcfg")
    try:
        out = (ctypes.c_int64 * 4)()
        assert L.puck_debug_flat_check(g, 0, 0, 2, out) == -1   # in_NN
        assert L.puck_debug_flat_check(g, 0, 3, 2, out) == 0    # in_TT, 34 per target
    finally:
        L.puck_grammar_free(g)


def test_flat_check_rejects_bad_arguments():
    levels = split_levels("viterbi", "small")
    L, g = _grammar(levels, "split_small")
    try:
        out = (ctypes.c_int64 * 4)()
        assert L.puck_debug_flat_check(g, 2, 0, 0, out) == -3   # no such level
        assert L.puck_debug_flat_check(g, 1, 12, 0, out) == -3  # no such job
        assert L.puck_debug_flat_check(g, 0, 5, 1, out) == -3   # groups: inside jobs only
        assert L.puck_debug_flat_check(g, 0, 0, 3, out) == -3   # no such form
    finally:
        L.puck_grammar_free(g)


def test_flat_tables_need_contiguous_members(tmp_path):
    """A reprojected cascade whose hierarchy interleaves the fine substates
    (0 and 2 under one coarse substate, 1 and 3 under the other) gives
    coarse symbols whose members are not contiguous in symbol order.  The
    flat-tile layout, which addresses a tile's members as one index range,
    is declined for them (the level keeps the whole-pair form, which reads
    members through the member lists); the same cascade with a contiguous
    hierarchy gets it for all twelve jobs, every rule held once."""
    from test_cli import _hierarchy_pair
    from puck_gb300 import berkeley, grammar
    for interleaved in (True, False):
        c, f = _hierarchy_pair(tmp_path, interleaved)
        gc, gf = berkeley.read_cascade([c, f], reproject=True)
        members = [[gf.labels[i] for i in range(len(gf.labels)) if gf.coarse[i] == k]
                   for k in range(len(gc.labels))]
        assert (["NP_0", "NP_2"] if interleaved else ["NP_0", "NP_1"]) in members
        levels = (grammar.compile_level(gc), grammar.compile_level(gf))
        L, g = _grammar(levels, f"reprojected_{'interleaved' if interleaved else 'contiguous'}")
        try:
            out = (ctypes.c_int64 * 4)()
            codes = [L.puck_debug_flat_check(g, 1, job, 0, out) for job in JOBS]
        finally:
            L.puck_grammar_free(g)
        if interleaved:
            assert codes[0] == -1 and all(rc in (-1, 0) for rc in codes), codes
        else:
            assert codes == [0] * len(JOBS), codes
