"""Prints one brace-balanced block of a reference source file, unchanged.

Used by oracle/Makefile (target `ref`) to compile one piece of the reference's own
code with stand-in types: the first line containing START at or after the N-th
line containing ANCHOR (N = 1 by default), through the line that closes its braces.
usage: python3 extract_block.py FILE ANCHOR START [N]
"""
import sys


def main():
    path, anchor, start = sys.argv[1:4]
    nth = int(sys.argv[4]) if len(sys.argv) > 4 else 1
    lines = open(path, encoding="utf-8", errors="replace").read().split("\n")
    a = [i for i, s in enumerate(lines) if anchor in s][nth - 1]
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
