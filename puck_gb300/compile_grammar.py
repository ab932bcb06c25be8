"""``python -m puck_gb300.compile_grammar`` -- the reference's CompileGrammar
(src/main/scala/puck/parser/CompileGrammar.scala:20-72) for this library.

Same flags and meaning: ``--textGrammarPrefix a:b`` (Berkeley text grammars,
coarse first), ``--grammar out.grz``, ``--viterbi`` (default true; the fine
level's semiring), ``--logsum`` (used when ``--viterbi false``; otherwise the
Real semiring).  Coarse levels are always Viterbi.  ``--device`` is accepted
and ignored (the tables are built on the host).  ``--reproject`` keeps the
first and last levels and projects the last onto the first's substates
through the last level's ``.hierarchy`` file (berkeley.read_cascade).

Extra flag for the synthetic workloads: ``--synthetic split|pcfg`` with
``--seed`` builds the seeded split-grammar cascade or the plain PCFG instead
of reading text files.
"""
from __future__ import annotations

import argparse
import sys
from typing import List, Optional

from . import berkeley, grammar, grz, synth


def _bool(v: str) -> bool:
    if v.lower() in ("true", "1", "yes"):
        return True
    if v.lower() in ("false", "0", "no"):
        return False
    raise argparse.ArgumentTypeError(f"expected true or false, got {v!r}")


def fine_semiring(viterbi: bool, logsum: bool) -> str:
    """CompileGrammar.scala:45-51."""
    if viterbi:
        return "viterbi"
    return "logsum" if logsum else "real"


def main(argv: Optional[List[str]] = None) -> int:
    ap = argparse.ArgumentParser(prog="compile_grammar", description=__doc__.split("\n")[0])
    ap.add_argument("--textGrammarPrefix", help="colon-separated Berkeley grammar prefixes, coarse first")
    ap.add_argument("--grammar", default="grammar.grz", help="output archive")
    ap.add_argument("--viterbi", type=_bool, nargs="?", const=True, default=True)
    ap.add_argument("--logsum", type=_bool, nargs="?", const=True, default=False)
    ap.add_argument("--reproject", type=_bool, nargs="?", const=True, default=False)
    ap.add_argument("--device", default="nvidia")
    ap.add_argument("--threshold", type=float, default=-12.0, help="drop rules with log score below this")
    ap.add_argument("--synthetic", choices=["split", "pcfg"])
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args(argv)
    sem = fine_semiring(a.viterbi, a.logsum)
    if a.reproject and a.synthetic:
        print("compile_grammar: --reproject needs --textGrammarPrefix", file=sys.stderr)
        return 2
    if a.synthetic == "split":
        c, f = synth.split_grammar(seed=a.seed)
        grammars = [c, f]
    elif a.synthetic == "pcfg":
        grammars = [synth.small_pcfg(a.seed)]
    elif a.textGrammarPrefix:
        grammars = berkeley.read_cascade(a.textGrammarPrefix.split(":"), a.threshold, reproject=a.reproject)
    else:
        ap.error("give --textGrammarPrefix or --synthetic")
    levels = [grammar.compile_level(g, "viterbi") for g in grammars[:-1]]
    levels.append(grammar.compile_level(grammars[-1], sem))
    grz.write_sequence(a.grammar, levels)
    print(f"wrote {a.grammar}: {len(levels)} level(s), fine semiring {sem}", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
