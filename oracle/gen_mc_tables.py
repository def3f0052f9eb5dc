"""Generate the packed marching-cubes triangle table used by the CUDA library and the oracle.

Marching-cubes case and triangle counts must be bit-exact with the reference, so the
triangulation per cube case has to be the one the reference uses (the classic
Lorensen-Cline / Bourke table, reference: src/MarchingCubes.cpp:35 and
src/MarchingCubes.cu:28).  This script reads that table from the reference source
tree and writes it in a packed form of our own: one 64-bit word per cube case, four
bits per edge index, low nibble first, terminated by 0xF.  The edge table (which
edges a case cuts) is not copied: both consumers derive it from the corner
numbering at start-up, and ``tests/test_mc_tables.py`` checks it against the
reference's edgeTable when the reference tree is available.

Usage (in a checkout that has the reference at REF):
    python oracle/gen_mc_tables.py REF
It rewrites ``volumefusion_gb300/csrc/mc_tables.inc`` and ``oracle/mc_tables.inc``.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def parse_tri_table(ref_root):
    src = open(os.path.join(ref_root, "src", "MarchingCubes.cpp")).read()
    start = src.index("int triTable[256][16]")
    body = src[src.index("{", start):]
    rows = re.findall(r"\{([-0-9,\s]+)\}", body)[:256]
    table = []
    for row in rows:
        vals = [int(v) for v in row.replace("\n", " ").split(",") if v.strip()]
        assert len(vals) == 16, row
        table.append(vals)
    assert len(table) == 256
    return table


def pack(table):
    words = []
    for vals in table:
        w = 0
        n = 0
        for v in vals:
            if v < 0:
                break
            w |= (v & 0xF) << (4 * n)
            n += 1
        assert n % 3 == 0 and n <= 15
        w |= 0xF << (4 * n)
        words.append(w)
    return words


def write(words, path, comment):
    lines = [
        "// Packed marching-cubes triangle table: one word per cube case, 4 bits per edge",
        "// index (low nibble first), 0xF terminates the list.  " + comment,
        "// Generated by oracle/gen_mc_tables.py; do not edit by hand.",
    ]
    for i in range(0, 256, 4):
        lines.append("    " + ", ".join("0x%016xull" % w for w in words[i:i + 4]) + ",")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VF_REFERENCE", "")
    if not ref:
        sys.exit("usage: gen_mc_tables.py <reference tree>  (or set VF_REFERENCE)")
    words = pack(parse_tri_table(ref))
    write(words, os.path.join(ROOT, "volumefusion_gb300", "csrc", "mc_tables.inc"),
          "Triangulation per case equals the reference's (src/MarchingCubes.cpp:35).")
    write(words, os.path.join(HERE, "mc_tables.inc"),
          "Oracle copy; must equal volumefusion_gb300/csrc/mc_tables.inc.")


if __name__ == "__main__":
    main()
