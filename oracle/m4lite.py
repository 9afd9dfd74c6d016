#!/usr/bin/env python3
"""Stand-in for the `m4` preprocessor that the reference's case reader shells
out to (sppde/sppde_parser.c:177-210), for running the reference here as a CPU
oracle (TEST INFRASTRUCTURE ONLY).

Covers the subset SW2 case files use: `define(NAME,VALUE)`, `include(FILE)`,
identifier replacement with rescanning, and `#` comments copied verbatim.
Usage (as the reference calls it): m4lite.py FILE  -> expanded text on stdout.
"""
import os
import re
import sys

_WORD = re.compile(r"[A-Za-z_][A-Za-z0-9_]*")


def _args(text, pos):
    """Parse a parenthesised, comma-separated argument list starting at text[pos] == '('."""
    depth, cur, out, i = 0, [], [], pos
    while i < len(text):
        c = text[i]
        if c == "(":
            depth += 1
            if depth > 1:
                cur.append(c)
        elif c == ")":
            depth -= 1
            if depth == 0:
                out.append("".join(cur))
                return [a.lstrip() for a in out], i + 1
            cur.append(c)
        elif c == "," and depth == 1:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(c)
        i += 1
    raise SystemExit("m4lite: unterminated argument list")


def expand(text, macros, base, depth=0):
    if depth > 50:
        raise SystemExit("m4lite: recursion too deep")
    out, i = [], 0
    while i < len(text):
        c = text[i]
        if c == "#":
            j = text.find("\n", i)
            j = len(text) if j < 0 else j
            out.append(text[i:j])
            i = j
            continue
        m = _WORD.match(text, i)
        if m and (i == 0 or not (text[i - 1].isalnum() or text[i - 1] == "_")):
            w = m.group(0)
            j = m.end()
            if w in ("define", "include") and j < len(text) and text[j] == "(":
                args, j = _args(text, j)
                if w == "define":
                    macros[args[0].strip()] = args[1] if len(args) > 1 else ""
                else:
                    path = os.path.join(base, args[0].strip())
                    with open(path) as fh:
                        out.append(expand(fh.read(), macros, os.path.dirname(path), depth + 1))
                i = j
                continue
            if w in macros:
                out.append(expand(macros[w], macros, base, depth + 1))
            else:
                out.append(w)
            i = j
            continue
        out.append(c)
        i += 1
    return "".join(out)


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: m4lite.py FILE")
    path = sys.argv[1]
    with open(path) as fh:
        sys.stdout.write(expand(fh.read(), {}, os.path.dirname(path) or "."))


if __name__ == "__main__":
    main()
