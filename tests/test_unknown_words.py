"""Unknown words take the unknown-word class of the Berkeley parser's English
lexicons (puck_grammar_word_id_at), backing off to shorter classes and to
"UNK" when the lexicon lacks the full class.  Host only: no GPU."""
import ctypes

import pytest

from helpers import write_text_grammar
from puck_gb300 import _lib, compile_grammar

CLASSES = ("UNK", "UNK-LC", "UNK-LC-s", "UNK-LC-ing", "UNK-INITC", "UNK-INITC-KNOWNLC", "UNK-CAPS",
           "UNK-CAPS-NUM", "UNK-NUM", "UNK-LC-DASH", "UNK-INITC-s")


@pytest.fixture(scope="module")
def grammar(tmp_path_factory):
    d = tmp_path_factory.mktemp("unk")
    c = write_text_grammar(str(d), "coarse", 1, seed=1)
    f = write_text_grammar(str(d), "fine", 2, seed=2)
    for prefix, k in ((c, 1), (f, 2)):
        with open(prefix + ".lexicon", "a") as out:
            for cls in CLASSES:
                out.write(f"NN {cls} [{', '.join(['0.01'] * k)}]\n")
    path = str(d / "unk.grz")
    assert compile_grammar.main(["--textGrammarPrefix", f"{c}:{f}", "--grammar", path]) == 0
    L = _lib.load()
    st = ctypes.c_int32(0)
    g = L.puck_grammar_load(path.encode(), ctypes.byref(st))
    assert g, _lib.last_error()
    yield L, g
    L.puck_grammar_free(g)


def _cls(L, g, word, pos):
    i = L.puck_grammar_word_id_at(g, word.encode(), pos)
    names = {L.puck_grammar_word_id(g, c.encode()): c for c in CLASSES}
    return names.get(i, i)


@pytest.mark.parametrize("word,pos,want", [
    ("dog", 3, None),                       # known: its own id
    ("cats", 2, "UNK-LC-s"),                # lowercase, final s
    ("running", 1, "UNK-LC-ing"),           # lowercase, -ing (five letters or more)
    ("glass", 1, "UNK-LC"),                 # final s after s: no -s class
    ("Dog", 0, "UNK-INITC-KNOWNLC"),        # sentence-initial capital, "dog" is known
    ("Zebras", 0, "UNK-INITC-s"),           # sentence-initial capital, final s
    ("Zebra", 0, "UNK-INITC"),
    ("Zebra", 4, "UNK-CAPS"),               # a capital elsewhere in the sentence
    ("B52", 2, "UNK-CAPS-NUM"),
    ("1984", 1, "UNK-NUM"),
    ("well-known", 1, "UNK-LC-DASH"),
    ("quickly", 1, "UNK-LC"),               # UNK-LC-ly is not in this lexicon: back off to UNK-LC
    ("!?", 1, "UNK"),                       # no class feature at all
])
def test_unknown_word_classes(grammar, word, pos, want):
    L, g = grammar
    got = _cls(L, g, word, pos)
    if want is None:
        assert got == L.puck_grammar_word_id(g, word.encode()) >= 0
    else:
        assert got == want


def test_no_class_without_unk_entries(tmp_path):
    """A lexicon without unknown-word classes leaves an unknown word at -1
    (the sentence then fails with the OOV status)."""
    c = write_text_grammar(str(tmp_path), "coarse", 1, seed=1)
    f = write_text_grammar(str(tmp_path), "fine", 2, seed=2)
    path = str(tmp_path / "plain.grz")
    assert compile_grammar.main(["--textGrammarPrefix", f"{c}:{f}", "--grammar", path]) == 0
    L = _lib.load()
    st = ctypes.c_int32(0)
    g = L.puck_grammar_load(path.encode(), ctypes.byref(st))
    try:
        assert L.puck_grammar_word_id_at(g, b"zebras", 1) == -1
        assert L.puck_grammar_word_id_at(g, b"dog", 1) == L.puck_grammar_word_id(g, b"dog") >= 0
        assert L.puck_grammar_word_id_at(g, b"", 0) == -1
    finally:
        L.puck_grammar_free(g)
