"""Generate mc_cases.inc: Bourke's marching-cubes triangle table, packed.

The triangle table of Paul Bourke's "Polygonising a scalar field"
(http://paulbourke.net/geometry/polygonise/, public domain) decides which
triangles each of the 256 cube cases emits.  Mesh topology can only match the
reference's (meshing/mc_tables.h:54-311 holds the same public table) if the
table is identical, so this script reads a C array in Bourke's layout
(int [256][16], edge triples terminated by -1) and packs every case into one
uint64: bits 0-3 hold the triangle count, bits 4+4k hold the k-th edge index.

Usage:  python gen_mc_cases.py <path to a header holding the table>

The corner numbering is Bourke's: corner i of the cube at voxel v sits at
v + kCorner[i] with kCorner = (0,1,1) (1,1,1) (1,1,0) (0,1,0) (0,0,1) (1,0,1)
(1,0,0) (0,0,0); the edge table is derived from it in code, not stored.
"""
import os
import re
import sys


def parse(path):
    src = open(path).read()
    i = src.index("[256][16]")
    body = src[i:src.index("};", i)]
    rows = re.findall(r"\{([^{}]*)\}", body)
    table = [[int(x) for x in r.split(",") if x.strip()] for r in rows]
    if len(table) != 256 or any(len(r) != 16 for r in table):
        raise SystemExit("unexpected table shape")
    return table


def pack(row):
    edges = []
    for k in range(0, 15, 3):
        if row[k] < 0:
            break
        edges += row[k:k + 3]
    word = len(edges) // 3
    for k, e in enumerate(edges):
        word |= (e & 0xF) << (4 + 4 * k)
    return word


def main():
    table = parse(sys.argv[1])
    words = [pack(r) for r in table]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mc_cases.inc")
    with open(out, "w") as f:
        f.write("// Generated by gen_mc_cases.py -- Bourke's public marching-cubes triangle\n")
        f.write("// table (paulbourke.net/geometry/polygonise), one uint64 per cube case:\n")
        f.write("// bits 0-3 = triangle count, bits 4+4k = k-th edge of the triangle list.\n")
        f.write("MH_MC_TABLE_QUALIFIER uint64_t kMcCases[256] = {\n")
        for i in range(0, 256, 4):
            f.write("  " + ", ".join("0x%016xull" % w for w in words[i:i + 4]) + ",\n")
        f.write("};\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
