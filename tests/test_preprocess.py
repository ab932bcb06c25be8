"""Sentence segmentation and tokenization in front of run_parser
(RunParser.scala:63-77's --sentences / --tokens choices).  Host only."""
import io

import pytest

from puck_gb300 import preprocess, run_parser
from puck_gb300.preprocess import segment, treebank_tokens
from test_cli import _FakeServer


@pytest.mark.parametrize("text,want", [
    ("The company said it expects revenue to rise.",
     "The company said it expects revenue to rise ."),
    ('He said, "I can\'t do it."', "He said , `` I ca n't do it . ''"),
    ("They won't go; we're staying (for now).",
     "They wo n't go ; we 're staying -LRB- for now -RRB- ."),
    ("The U.S. economy grew 3.5% in 1,000 days.", "The U.S. economy grew 3.5 % in 1,000 days ."),
    ("It cost $5.20 at Smith & Co.", "It cost $ 5.20 at Smith & Co. ."),
    ("Investors' shares rose -- sharply...", "Investors ' shares rose -- sharply ..."),
    ("I cannot believe you're gonna do that!", "I can not believe you 're gon na do that !"),
    ("Mr. Smith visited the U.S.", "Mr. Smith visited the U.S. ."),
    ("“Smart quotes” and ‘single’ ones don’t break.",
     "`` Smart quotes '' and ` single ' ones do n't break ."),
    ("She asked: is it 3:30?", "She asked : is it 3:30 ?"),
    ("'Tis the season, isn't it?", "'T is the season , is n't it ?"),
    ("The firm filed [again] {today}.", "The firm filed -LSB- again -RSB- -LCB- today -RCB- ."),
    ("AT&T and e-mail stay whole.", "AT&T and e-mail stay whole ."),
    ("A list: a, b, c.", "A list : a , b , c ."),
    ("It was signed by John F.", "It was signed by John F. ."),
    ("She said 'no'.", "She said ` no ' ."),
    ("word", "word"),
])
def test_treebank_tokens(text, want):
    assert treebank_tokens(text) == want.split()


def test_treebank_tokens_are_in_the_berkeley_lexicon_forms():
    # the forms the Berkeley English lexicons list for quotes, brackets and clitics
    toks = set(treebank_tokens('"Don\'t (ever) say {that} [again]," he\'d said.'))
    assert {"``", "''", "-LRB-", "-RRB-", "-LCB-", "-RCB-", "-LSB-", "-RSB-", "n't", "'d"} <= toks


def test_segment():
    text = ("Mr. Smith went to Washington. He met J. Doe at the U.S. Capitol. "
            '"Is it done?" she asked. Yes! The end... Prices rose 5. Then they fell.')
    assert segment(text) == ["Mr. Smith went to Washington.", "He met J. Doe at the U.S. Capitol.",
                             '"Is it done?" she asked.', "Yes!", "The end...", "Prices rose 5.",
                             "Then they fell."]
    # a stop followed by a lowercase word does not end the sentence
    assert segment("It rose 5 p.c. overall. done") == ["It rose 5 p.c. overall. done"]
    assert segment("") == []


def test_rule_sentences_do_not_cross_blank_lines():
    src = io.StringIO("First line of a\nsentence. Second one\n\nthird paragraph without a stop\n")
    assert list(preprocess.rule_sentences(src)) == ["First line of a sentence.", "Second one",
                                                    "third paragraph without a stop"]


def test_rule_sentences_stream():
    """A sentence is yielded as soon as the line after its end has been
    read, not at the end of the input."""
    read = []

    def lines():
        for i, line in enumerate(["One sentence here. Another one", "starts here. And a", "third.", ""]):
            read.append(i)
            yield line + "\n"

    it = preprocess.rule_sentences(lines())
    assert next(it) == "One sentence here." and read == [0]
    assert next(it) == "Another one starts here." and read == [0, 1]
    assert list(it) == ["And a third."]
    # the streamed split equals splitting the whole paragraph at once
    text = ("Mr. Smith went to Washington. He met J. Doe at the U.S. Capitol. "
            '"Is it done?" she asked. Yes! The end... Prices rose 5. Then they fell.')
    words = text.split()
    chunks = [" ".join(words[i:i + 3]) + "\n" for i in range(0, len(words), 3)]
    assert list(preprocess.rule_sentences(io.StringIO("".join(chunks)))) == segment(text)


def test_flag_values_follow_the_reference():
    assert preprocess.sentence_segmenter("newline") is preprocess.newline_sentences
    for v in ("java", "trained", "default", "TRAINED"):
        assert preprocess.sentence_segmenter(v) is preprocess.rule_sentences
    for v in ("none", "whitespace"):
        assert preprocess.tokenizer(v) is preprocess.whitespace_tokens
    for v in ("default", "treebank"):
        assert preprocess.tokenizer(v) is preprocess.treebank_tokens
    with pytest.raises(ValueError):
        preprocess.tokenizer("moses")
    with pytest.raises(ValueError):
        preprocess.sentence_segmenter("punkt")


def test_run_parser_defaults_segment_and_tokenize_running_text():
    src = io.StringIO('He said, "No." Then he left.\n\nBAD luck follows.\n')
    sink = io.StringIO()
    n = run_parser.parse_stream(_FakeServer(), src, sink, max_length=50,
                                segment=preprocess.rule_sentences, tokenize=preprocess.treebank_tokens)
    assert n == 3
    assert sink.getvalue().splitlines() == [
        "(ROOT (T He) (T said) (T ,) (T ``) (T No) (T .) (T ''))",
        "(ROOT (T Then) (T he) (T left) (T .))",
        "(())",
    ]


def test_run_parser_rejects_unknown_flag_values(capsys):
    with pytest.raises(SystemExit):
        run_parser.main(["--tokens", "moses"])
    assert "unknown tokenizer" in capsys.readouterr().err
