"""``python -m puck_gb300.run_parser`` -- the reference's RunParser
(src/main/scala/puck/parser/RunParser.scala:34-118) on this library.

Flags keep the reference's names and meaning: ``--grammar`` (grammar.grz),
``--maxLength`` (sentences with at least this many tokens print ``(())``,
the reference's strict ``<`` test), ``--mem`` (device memory, ``3g`` style),
``--profile``, ``--device`` (a CUDA ordinal here; a non-numeric value picks
device 0), ``--sentences``, ``--tokens`` and ``--outputSuffix``.  Input files
are parsed to ``<file><outputSuffix>``; with no files, stdin goes to stdout.
One tree per line, in input order, debinarized and rendered with coarse
labels; a sentence that fails prints ``(())`` (RunParser.scala:100-107).

Like the reference, sentences stream through a batching service -- here the
library's continuous-batching server -- and results are written in order.
``--sentences`` and ``--tokens`` take the reference's values and defaults
(``trained`` and ``default``: running text is split into sentences and
tokenized the Penn Treebank way); see :mod:`puck_gb300.preprocess` for what
stands in for epic's segmenters and tokenizer.
"""
from __future__ import annotations

import argparse
import collections
import re
import sys
import time
from typing import Callable, Iterable, List, Optional, TextIO

from . import preprocess
from .parser import debinarize
from .server import CLServer

FAIL = "(())"


def parse_mem(s: str) -> int:
    """CLParser.parseMemString: ``<number>[k|m|g]`` bytes."""
    m = re.fullmatch(r"\s*([0-9.]+)\s*([kKmMgG]?)[bB]?\s*", s)
    if not m:
        raise argparse.ArgumentTypeError(f"bad memory size {s!r}")
    mult = {"": 1, "k": 1 << 10, "m": 1 << 20, "g": 1 << 30}[m.group(2).lower()]
    return int(float(m.group(1)) * mult)


def _bool(v: str) -> bool:
    return v.lower() in ("true", "1", "yes")


def parse_stream(server: CLServer, src: TextIO, sink: TextIO, max_length: int, window: int = 4096,
                 segment: Callable[[TextIO], Iterable[str]] = preprocess.newline_sentences,
                 tokenize: Callable[[str], List[str]] = preprocess.whitespace_tokens) -> int:
    """Submits sentences as they are read and writes results in input order;
    at most ``window`` results are outstanding.  Returns the count."""
    pending = collections.deque()
    n = 0

    def emit(item):
        words, fut = item
        if fut is None:
            sink.write(FAIL + "\n")
            return
        res = fut.result()
        if not res.is_success:
            sink.write(FAIL + "\n")
        else:
            sink.write(debinarize(res.get()).render(words) + "\n")

    for sent in segment(src):
        words = tokenize(sent)
        if not words:
            continue
        n += 1
        fut = server.submit(words) if len(words) < max_length else None
        pending.append((words, fut))
        while len(pending) > window or (pending and (pending[0][1] is None or pending[0][1].done())):
            emit(pending.popleft())
    while pending:
        emit(pending.popleft())
    sink.flush()
    return n


def parse_args(argv: Optional[List[str]] = None) -> argparse.Namespace:
    """RunParser.Params (RunParser.scala:34-43), same names and defaults."""
    ap = argparse.ArgumentParser(prog="run_parser", description=__doc__.split("\n")[0])
    ap.add_argument("files", nargs="*")
    ap.add_argument("--grammar", default="grammar.grz")
    ap.add_argument("--maxLength", type=int, default=50)
    ap.add_argument("--mem", type=parse_mem, default=parse_mem("3g"))
    ap.add_argument("--profile", type=_bool, nargs="?", const=True, default=False)
    ap.add_argument("--device", default="nvidia")
    ap.add_argument("--sentences", default="trained")
    ap.add_argument("--tokens", default="default")
    ap.add_argument("--outputSuffix", default=".parsed")
    # declared by the reference's Params but read by neither RunParser.main
    # nor anything it calls: accepted so that its command lines run here
    ap.add_argument("--numToParse", type=int, default=1000)
    ap.add_argument("--maxParseLength", type=int, default=10000)
    a = ap.parse_args(argv)
    try:
        preprocess.sentence_segmenter(a.sentences)
        preprocess.tokenizer(a.tokens)
    except ValueError as exc:
        ap.error(str(exc))
    return a


def main(argv: Optional[List[str]] = None) -> int:
    a = parse_args(argv)
    segment = preprocess.sentence_segmenter(a.sentences)
    tokenize = preprocess.tokenizer(a.tokens)
    device = int(a.device) if a.device.isdigit() else 0
    # sentences with maxLength tokens or more never reach the parser
    server = CLServer(a.grammar, max_alloc_size=a.mem, device=device, max_length=min(max(a.maxLength - 1, 1), 256),
                      profile=a.profile)
    t0 = time.time()
    total = 0
    try:
        if not a.files:
            total += parse_stream(server, sys.stdin, sys.stdout, a.maxLength,
                                  segment=segment, tokenize=tokenize)
        for f in a.files:
            with open(f, encoding="utf-8") as src, open(f + a.outputSuffix, "w", encoding="utf-8") as sink:
                total += parse_stream(server, src, sink, a.maxLength, segment=segment, tokenize=tokenize)
    finally:
        server.close()
    wall = time.time() - t0
    print(f"Parsing took {wall:.3f}s seconds. {total / max(wall, 1e-9):.3f} sentences per second.", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
