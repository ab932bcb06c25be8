"""Sentence segmentation and tokenization in front of the parser -- the
input side of the reference's RunParser (RunParser.scala:63-77, which picks
epic's segmenters and tokenizers by ``--sentences`` and ``--tokens``).

* ``newline`` sentences (puck.preprocess.NewLineSentenceSegmenter): one
  sentence per non-blank line.
* ``java`` / ``trained`` / ``default`` sentences: a rule-based segmenter.
  The reference's choices are java.text.BreakIterator and epic's trained
  model (MLSentenceSegmenter), neither of which exists here; this one splits
  after ``.``, ``?`` or ``!`` (plus closing quotes and brackets) when the
  next word starts a sentence, and not after titles, single initials or
  dotted abbreviations.  Sentences never cross a blank line.
* ``whitespace`` / ``none`` tokens: split on whitespace.
* ``treebank`` / ``default`` tokens: the Penn Treebank conventions that the
  Berkeley grammars' lexicons are written in (double quotes as two
  backquotes or two apostrophes, ``-LRB-`` style brackets, ``n't`` and ``'s`` clitics split off,
  ``ca n't``, ``gon na``, a sentence-final period split off -- repeated after
  an abbreviation, as in ``U.S. .``).  epic's TreebankTokenizer, the
  reference's, is a generated lexer that is not in the tree, so agreement
  with it is not pinned.
"""
from __future__ import annotations

import re
from typing import Callable, Iterable, Iterator, List, TextIO

# -- sentences ---------------------------------------------------------------

# words after which a period never ends a sentence
_TITLES = frozenset("mr mrs ms dr prof gen sen rep gov st lt col sgt capt messrs mt ft rev hon".split())
# shortened words that keep their period inside a sentence and, at its end,
# are followed by a separate "." token
_ABBREV = _TITLES | frozenset(
    "inc corp co ltd jr sr bros vs etc jan feb mar apr jun jul aug sep sept oct nov dec "
    "calif conn fla ill mass mich minn n.j n.y pa tenn tex va wash wis ariz colo".split())

_BOUNDARY = re.compile(r"[.?!]+[\"'”’)\]}]*(?=\s)")
_OPENERS = "\"'“‘([{`"


def _ends_sentence(text: str, end: int) -> bool:
    """Whether the terminal punctuation ending at ``end`` closes a sentence."""
    rest = text[end:].lstrip()
    if not rest:
        return True
    nxt = rest[0]
    if not (nxt.isupper() or nxt.isdigit() or nxt in _OPENERS):
        return False
    start = text.rfind(" ", 0, end) + 1
    word = text[start:end].lstrip(_OPENERS)
    core = word.rstrip("\"'”’)]}")
    if not core.endswith(".") or core.endswith(".."):
        return True                                  # ? ! or an ellipsis
    stem = core[:-1]
    if stem.lower() in _TITLES:
        return False
    if len(stem) == 1 and stem.isupper():           # an initial: "J. Smith"
        return False
    if "." in stem:                                 # a dotted abbreviation: "U.S."
        return False
    return True


def segment(text: str) -> List[str]:
    """Splits one paragraph of running text into sentences."""
    text = " ".join(text.split())
    out, start = [], 0
    for m in _BOUNDARY.finditer(text):
        if _ends_sentence(text, m.end()):
            piece = text[start:m.end()].strip()
            if piece:
                out.append(piece)
            start = m.end()
    tail = text[start:].strip()
    if tail:
        out.append(tail)
    return out


def newline_sentences(src: TextIO) -> Iterator[str]:
    """One sentence per non-blank line (RunParser.scala:92 drops blank ones)."""
    for line in src:
        if line.strip():
            yield line.rstrip("\n")


def rule_sentences(src: TextIO) -> Iterator[str]:
    """Running text split by :func:`segment`, streamed: a boundary depends
    only on the words around it, so every sentence but the last of the text
    read so far is final and is yielded at once; the unfinished rest waits
    for more lines.  A blank line ends a paragraph, and no sentence crosses
    it."""
    buf = ""
    for line in src:
        text = line.strip()
        if not text:
            if buf:
                yield from segment(buf)
            buf = ""
            continue
        buf = f"{buf} {text}" if buf else text
        parts = segment(buf)
        if len(parts) > 1:
            yield from parts[:-1]
            buf = parts[-1]
    if buf:
        yield from segment(buf)


# -- tokens ------------------------------------------------------------------

def whitespace_tokens(sentence: str) -> List[str]:
    return sentence.split()


_BRACKETS = {"(": "-LRB-", ")": "-RRB-", "[": "-LSB-", "]": "-RSB-", "{": "-LCB-", "}": "-RCB-"}
# whole words the Treebank writes as two tokens
_SPLIT_WORDS = {"cannot": (3,), "gonna": (3,), "gotta": (3,), "wanna": (3,), "gimme": (3,),
                "lemme": (3,), "'tis": (2,), "'twas": (2,), "d'ye": (2,), "more'n": (4,)}
_CLITIC = re.compile(r"(?i)^(.+?)('s|'m|'d|'re|'ve|'ll)$")
_PREFIX = "([{<$#`"
_SUFFIX = ",;:?!)]}>%"


def _clitics(core: str) -> List[str]:
    low = core.lower()
    if low in _SPLIT_WORDS:
        (k,) = _SPLIT_WORDS[low]
        return [core[:k], core[k:]]
    if len(core) > 3 and low.endswith("n't"):
        return [core[:-3], core[-3:]]
    m = _CLITIC.match(core)
    if m:
        return [m.group(1), m.group(2)]
    return [core]


def _chunk(c: str) -> List[str]:
    """One whitespace-separated chunk: peel leading and trailing punctuation,
    then split clitics off the remaining word."""
    head: List[str] = []
    tail: List[str] = []
    while c:
        if c.startswith("``"):
            head.append("``")
            c = c[2:]
        elif c[0] in _PREFIX:
            head.append(c[0])
            c = c[1:]
        elif c[0] == "'" and len(c) > 1 and c[1].isalpha() and not _CLITIC.match("x" + c) \
                and c.lower() not in _SPLIT_WORDS:
            head.append("`")                        # an opening single quote
            c = c[1:]
        else:
            break
    while c:
        if c.endswith("''"):
            tail.append("''")
            c = c[:-2]
        elif c[-1] in _SUFFIX:
            tail.append(c[-1])
            c = c[:-1]
        elif c[-1] == "." and len(c) > 1 and c[-2] in ")]}>'":
            tail.append(".")                        # a stop after a closer: "(now)."
            c = c[:-1]
        elif c[-1] == "'" and len(c) > 1:           # a closing quote or a plural possessive
            tail.append("'")
            c = c[:-1]
        else:
            break
    mid = _clitics(c) if c else []
    return head + mid + tail[::-1]


def _final_period(tokens: List[str]) -> List[str]:
    """Splits the sentence-final period off the last word (before any
    closing quotes or brackets); after an abbreviation the word keeps its
    period and a separate "." follows."""
    closing = {"''", "'", ")", "]", "}", ">"}
    i = len(tokens) - 1
    while i >= 0 and tokens[i] in closing:
        i -= 1
    if i < 0:
        return tokens
    w = tokens[i]
    if len(w) < 2 or not w.endswith(".") or w.endswith(".."):
        return tokens
    stem = w[:-1]
    keep = stem.lower() in _ABBREV or "." in stem or (len(stem) == 1 and stem.isupper())
    return tokens[:i] + ([w, "."] if keep else [stem, "."]) + tokens[i + 1:]


def treebank_tokens(sentence: str) -> List[str]:
    s = (sentence.replace("“", " `` ").replace("”", " '' ")
         .replace("‘", " ` ").replace("’", "'"))
    # a double quote at the start or after a space or an opening bracket opens
    s = re.sub(r'(^|(?<=[\s(\[{<]))"', " `` ", s)
    s = s.replace('"', " '' ")
    s = s.replace("...", " ... ").replace("--", " -- ")
    out: List[str] = []
    for c in s.split():
        out.extend(t for t in _chunk(c) if t)
    out = _final_period(out)
    return [_BRACKETS.get(t, t) for t in out]


# -- the flags ---------------------------------------------------------------

def sentence_segmenter(name: str) -> Callable[[TextIO], Iterable[str]]:
    """``--sentences``: the reference's names (RunParser.scala:63-69)."""
    n = name.lower()
    if n == "newline":
        return newline_sentences
    if n in ("java", "default", "trained"):
        return rule_sentences
    raise ValueError(f"unknown sentence segmenter {name!r} (newline, java, trained, default)")


def tokenizer(name: str) -> Callable[[str], List[str]]:
    """``--tokens``: the reference's names (RunParser.scala:72-75)."""
    n = name.lower()
    if n in ("none", "whitespace"):
        return whitespace_tokens
    if n in ("default", "treebank"):
        return treebank_tokens
    raise ValueError(f"unknown tokenizer {name!r} (whitespace, none, treebank, default)")
