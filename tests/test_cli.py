"""The command-line front ends (compile_grammar, run_parser) and the
Berkeley text-grammar reader.

The reader is checked on the reference's own text grammars when they are
present on this machine; its parity with epic's reader is unpinned.
"""
import io
import os
import subprocess
import sys
from concurrent.futures import Future

import numpy as np
import pytest

import oracle
from puck_gb300 import berkeley, compile_grammar, grammar, grz, run_parser
from puck_gb300.parser import CLParserData, Failure, Success, Tree, nodes_to_viterbi_tree

# the reference's Berkeley text grammars (dlwh/puck textGrammars/), when a copy is named
TEXT = os.environ.get("PUCK_TEXT_GRAMMARS", "")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parse_mem_matches_reference_suffixes():
    assert run_parser.parse_mem("3g") == 3 << 30
    assert run_parser.parse_mem("512m") == 512 << 20
    assert run_parser.parse_mem("100") == 100
    with pytest.raises(Exception):
        run_parser.parse_mem("lots")


def test_fine_semiring_flags():
    assert compile_grammar.fine_semiring(True, False) == "viterbi"
    assert compile_grammar.fine_semiring(True, True) == "viterbi"
    assert compile_grammar.fine_semiring(False, True) == "logsum"
    assert compile_grammar.fine_semiring(False, False) == "real"


def test_compile_grammar_synthetic_writes_a_loadable_archive(tmp_path):
    out = str(tmp_path / "g.grz")
    assert compile_grammar.main(["--synthetic", "pcfg", "--seed", "0", "--grammar", out, "--viterbi", "false"]) == 0
    levels = grz.read_sequence(out)
    assert len(levels) == 1 and not levels[0].is_viterbi


def _hierarchy_pair(tmp_path, interleaved=True):
    """tg_1 (2 substates per label) and tg_2 (4), with tg_2's hierarchy
    putting substates 0 and 2 under tg_1's 0, and 1 and 3 under its 1 (or,
    not interleaved, 0 and 1 under 0, and 2 and 3 under 1)."""
    from helpers import write_text_grammar
    d = tmp_path / ("interleaved" if interleaved else "contiguous")
    d.mkdir(exist_ok=True)
    c = write_text_grammar(str(d), "tg_1", 2, seed=5)
    f = write_text_grammar(str(d), "tg_2", 4, seed=6)
    tree = "(0 (0 (0 0) (2 2)) (1 (1 1) (3 3)))" if interleaved else "(0 (0 (0 0) (1 1)) (1 (2 2) (3 3)))"
    with open(f + ".hierarchy", "w") as h:
        for lab in ("S", "NP", "VP", "DT", "NN", "VB"):
            h.write(f"{lab}\t{tree}\n")
    return c, f


def test_reproject_maps_fine_substates_through_the_hierarchy(tmp_path):
    c, f = _hierarchy_pair(tmp_path)
    assert berkeley.read_hierarchy(f, c)["NP_0"] == ["NP_0", "NP_2"]
    gc, gf = berkeley.read_cascade([c, f], reproject=True)
    names = gc.coarse_names
    assert names == gc.labels                        # the coarse level projects onto itself
    assert [names[gc.coarse[i]] for i in range(len(gc.labels))] == gc.labels
    proj = {gf.labels[i]: names[gf.coarse[i]] for i in range(len(gf.labels))}
    assert proj["VP_2"] == "VP_0" and proj["VP_3"] == "VP_1" and proj["ROOT_0"] == "ROOT_0"
    levels = [grammar.compile_level(gc), grammar.compile_level(gf)]
    wid = {w: i for i, w in enumerate(gf.words)}
    sent = np.array([wid[w] for w in "the dog sees a cat".split()], np.int32)
    r = oracle.run(levels, [sent], mode="parse")
    assert np.isfinite(r.trees()[0, 3:4].view(np.float32)[0])
    # the command line: a written archive; --reproject with --synthetic is refused
    out = str(tmp_path / "r.grz")
    assert compile_grammar.main(["--textGrammarPrefix", f"{c}:{f}", "--grammar", out, "--reproject"]) == 0
    assert [lv.n_coarse for lv in grz.read_sequence(out)] == [len(gc.labels)] * 2
    assert compile_grammar.main(["--synthetic", "pcfg", "--grammar", str(tmp_path / "g.grz"),
                                 "--reproject"]) == 2


def test_read_hierarchy_leaf_level(tmp_path):
    """A fine level one below the tree's height takes the tree's leaves."""
    p = str(tmp_path / "h_3")
    for name in ("h_3", "h_2"):
        with open(str(tmp_path / name) + ".hierarchy", "w") as h:
            h.write("X\t(0 (0 (0 0 1) (1 2)) (1 (2 3 4)))\n")
    assert berkeley.read_hierarchy(p, str(tmp_path / "h_1")) == {"X_0": ["X_0", "X_1", "X_2"], "X_1": ["X_3", "X_4"]}
    assert berkeley.read_hierarchy(str(tmp_path / "h_2"), str(tmp_path / "h_0")) == {
        "X_0": ["X_0", "X_1", "X_2"]}


@pytest.mark.skipif(not os.path.exists(TEXT + "/wsj_1.gr.binary"), reason="reference text grammars absent")
def test_reproject_of_wsj_0_1_equals_the_base_label_projection():
    """wsj_0 has one substate per label, so projecting wsj_1 onto wsj_0's
    substates through the hierarchy is the base-label projection renamed:
    same masks and trees."""
    plain = berkeley.read_cascade([TEXT + "/wsj_0.gr", TEXT + "/wsj_1.gr"])
    rep = berkeley.read_cascade([TEXT + "/wsj_0.gr", TEXT + "/wsj_1.gr"], reproject=True)
    base = lambda n: n.rsplit("_", 1)[0]
    for a, b in zip(plain, rep):
        assert a.labels == b.labels
        assert [a.coarse_names[x] for x in a.coarse] == [base(b.coarse_names[x]) for x in b.coarse]
    wid = {w: i for i, w in enumerate(plain[1].words)}
    sents = [np.array([wid[w] for w in s.split()], np.int32)
             for s in ("The company said it expects revenue to rise .", "He sold shares of the stock .")]
    runs = [oracle.run([grammar.compile_level(g, "viterbi") for g in gs], sents, mode="parse") for gs in (plain, rep)]
    assert np.array_equal(runs[0].trees(), runs[1].trees())
    assert np.array_equal(runs[0].masks(0)[0], runs[1].masks(0)[0])


class _FakeServer:
    """Completes every sentence with a one-node-per-word flat tree, or with a
    failure for sentences containing 'BAD'."""

    def submit(self, words):
        f = Future()
        if "BAD" in words:
            f.set_result(Failure("OOV"))
        else:
            kids = [Tree("T", [], i, i + 1) for i in range(len(words))]
            f.set_result(Success(Tree("ROOT", kids, 0, len(words))))
        return f


def test_run_parser_stream_order_and_failure_policy():
    src = io.StringIO("a b c\n\n  \nx BAD y\n" + " ".join(["w"] * 7) + "\nd e\n")
    sink = io.StringIO()
    n = run_parser.parse_stream(_FakeServer(), src, sink, max_length=7, window=2)
    assert n == 4  # blank lines are skipped
    lines = sink.getvalue().splitlines()
    assert lines == ["(ROOT (T a) (T b) (T c))", "(())", "(())", "(ROOT (T d) (T e))"]


@pytest.mark.skipif(not os.path.exists(TEXT + "/wsj_1.gr.binary"), reason="reference text grammars absent")
def test_berkeley_reader_on_reference_grammars():
    g0, g1 = berkeley.read_cascade([TEXT + "/wsj_0.gr", TEXT + "/wsj_1.gr"])
    assert g0.coarse_names == g1.coarse_names and g0.words == g1.words
    # every substate of wsj_1 projects onto its base label
    for lab, c in zip(g1.labels, g1.coarse):
        assert lab.rsplit("_", 1)[0] == g1.coarse_names[c]
    # identity unaries exist for every nonterminal
    l1 = grammar.compile_level(g1, "viterbi")
    ident = {(int(p), int(c)) for p, c in g1.un_rules if p == c}
    assert all((int(x), int(x)) in ident for x in l1.nt_labels)
    # the lexicon keeps one entry per substate with a positive probability
    assert g1.lex_label.shape[0] > g0.lex_label.shape[0]
    assert np.all(g1.lex_score <= 0)


@pytest.mark.skipif(not os.path.exists(TEXT + "/wsj_1.gr.binary"), reason="reference text grammars absent")
def test_berkeley_cascade_parses_english_on_the_oracle(tmp_path):
    gs = berkeley.read_cascade([TEXT + "/wsj_0.gr", TEXT + "/wsj_1.gr"])
    levels = [grammar.compile_level(gs[0], "viterbi"), grammar.compile_level(gs[1], "viterbi")]
    wid = {w: i for i, w in enumerate(gs[1].words)}
    text = ["The company said it expects revenue to rise .", "He sold shares of the stock ."]
    sents = [np.array([wid[w] for w in s.split()], np.int32) for s in text]
    r = oracle.run(levels, sents, mode="parse")
    nodes = r.trees()
    path = str(tmp_path / "wsj.grz")
    grz.write_sequence(path, levels)
    data = CLParserData.read_sequence(path)[-1]
    first = nodes_to_viterbi_tree(nodes[:2 * len(sents[0]) - 1], data)
    assert first.label == "ROOT"
    assert np.isfinite(nodes[0, 3].view(np.float32))
    assert first.preterminal_labels()[-1] == "."


def test_wsj_fixture_trees_are_english_parses():
    """The committed wsj_0 -> wsj_1 fixture (compiled from the reference's
    text grammars by tests/golden/make_golden.py): its stored trees decode
    to ROOT trees whose last preterminal is the sentence-final '.'."""
    d = os.path.join(ROOT, "tests", "golden")
    data = np.load(os.path.join(d, "wsj01_cascade_viterbi.npz"))
    lv = CLParserData.read_sequence(os.path.join(d, "wsj01_cascade_viterbi.grz"))[-1]
    off, trees = data["offsets"], data["trees"]
    start = 0
    for i in range(len(off) - 1):
        n = int(off[i + 1] - off[i])
        t = nodes_to_viterbi_tree(trees[start:start + 2 * n - 1], lv)
        start += 2 * n - 1
        assert t.label == "ROOT" and t.end == n
        assert t.preterminal_labels()[-1] == "."


def _module(mod, *args, **kw):
    return subprocess.run([sys.executable, "-m", mod, *args], cwd=ROOT, capture_output=True, text=True,
                          timeout=600, **kw)


def test_cli_help_runs():
    for mod in ("puck_gb300.run_parser", "puck_gb300.compile_grammar"):
        r = _module(mod, "--help")
        assert r.returncode == 0 and "--grammar" in r.stdout


@pytest.mark.gpu
def test_run_parser_end_to_end_matches_oracle(tmp_path):
    from puck_gb300 import synth
    out = str(tmp_path / "g.grz")
    assert compile_grammar.main(["--synthetic", "pcfg", "--seed", "0", "--grammar", out]) == 0
    g = synth.small_pcfg(0)
    sents = synth.uniform_sentences(5, 12, 5, 20, 5000)
    text = [" ".join(g.words[i] for i in s) for s in sents]
    text[3] = text[3] + " not_a_word"
    inp = tmp_path / "in.txt"
    inp.write_text("\n".join(text) + "\n")
    r = _module("puck_gb300.run_parser", "--grammar", out, "--maxLength", "19", "--mem", "2g",
                "--sentences", "newline", "--tokens", "whitespace", str(inp))
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "in.txt.parsed").read_text().splitlines()
    assert len(lines) == len(text)
    levels = [grammar.compile_level(g, "viterbi")]
    data = CLParserData.read_sequence(out)[-1]
    from puck_gb300.parser import debinarize
    for i, s in enumerate(sents):
        words = text[i].split()
        if i == 3 or len(words) >= 19:
            assert lines[i] == "(())"
            continue
        ref = oracle.run(levels, [s], mode="parse").trees()
        assert lines[i] == debinarize(nodes_to_viterbi_tree(ref, data)).render(words)


@pytest.mark.skipif(not os.path.exists(TEXT + "/wsj_1.gr.binary"), reason="reference text grammars absent")
def test_treebank_tokens_of_running_text_are_in_the_wsj_vocabulary():
    """run_parser's default front end (rule-based segmenter, treebank
    tokenizer) turns running English into the lexicon's own token forms;
    whitespace tokens of the same text mostly miss it."""
    from puck_gb300.preprocess import segment, treebank_tokens
    gs = berkeley.read_cascade([TEXT + "/wsj_0.gr", TEXT + "/wsj_1.gr"])
    vocab = set(gs[1].words)
    text = ("The company said it expects revenue to rise 5% next year, but analysts weren't convinced. "
            '"We can\'t predict the market," Mr. Jones said (in an interview). Shares of the U.S. unit '
            "fell $1.25 to $30. It's the firm's third quarterly loss -- and investors' patience is thin...")
    sents = segment(text)
    assert len(sents) == 4
    toks = [t for s in sents for t in treebank_tokens(s)]
    assert [t for t in toks if t not in vocab] == []
    assert sum(t not in vocab for s in sents for t in s.split()) >= 10


def test_run_parser_takes_the_reference_params():
    """Every RunParser.Params field (RunParser.scala:34-43) parses, with the
    reference's defaults; numToParse and maxParseLength are accepted and, as
    in the reference's main, unused."""
    a = run_parser.parse_args([])
    assert (a.device, a.sentences, a.tokens, a.profile, a.numToParse, a.grammar, a.maxParseLength, a.mem,
            a.maxLength, a.outputSuffix) == ("nvidia", "trained", "default", False, 1000, "grammar.grz", 10000,
                                             3 << 30, 50, ".parsed")
    a = run_parser.parse_args(["--device", "1", "--sentences", "newline", "--tokens", "whitespace", "--profile",
                               "true", "--numToParse", "5", "--grammar", "g.grz", "--maxParseLength", "40",
                               "--mem", "2g", "--maxLength", "30", "--outputSuffix", ".out", "a.txt", "b.txt"])
    assert a.files == ["a.txt", "b.txt"] and a.device == "1" and a.profile is True and a.mem == 2 << 30
    assert a.maxLength == 30 and a.outputSuffix == ".out" and a.numToParse == 5
