"""Prints one brace-balanced block of a reference source file, unchanged.

Used by oracle/Makefile (target `ref`) to compile one piece of the reference's own
code with stand-in types: the first line containing START after the first line
containing ANCHOR, through the line that closes its braces.
usage: python3 extract_block.py FILE ANCHOR START
"""
import sys


def main():
    path, anchor, start = sys.argv[1:4]
    lines = open(path, encoding="utf-8", errors="replace").read().split("\n")
    a = next(i for i, s in enumerate(lines) if anchor in s)
    b = next(i for i in range(a, len(lines)) if start in lines[i])
    depth, out = 0, []
    for s in lines[b:]:
        out.append(s)
        depth += s.count("{") - s.count("}")
        if depth == 0 and "{" in "".join(out):
            break
    sys.stdout.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
