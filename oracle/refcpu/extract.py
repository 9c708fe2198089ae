"""TEST INFRASTRUCTURE: pull the reference's device functions out of its .cu
files for the CPU build of the reference (oracle/refcpu).

The reference's .cu files mix kernels with host wrappers that use the <<<>>>
launch syntax and engine headers (OpenCV, glog, GL), which a host compiler
cannot take.  This script copies only the top-level ``__global__`` and
``__device__`` functions, verbatim and with #line directives, from the
reference tree into a generated file under oracle/_ref/ (git-ignored, never
committed), which refcpu.cpp includes.

Usage: python extract.py <reference root> <output file>
"""
import os
import re
import sys

# (file, functions to skip)
SOURCES = [
    ("src/mapping/allocate.cu", ()),
    ("src/core/collect_block_array.cu", ()),
    ("src/mapping/update_simple.cu", ()),
    ("src/mapping/update_bayesian.cu", ("BuildSensorDataEquationKernel",)),
    ("src/meshing/marching_cubes.cu", ()),
    ("src/visualization/ray_caster.cu", ()),
    ("src/mapping/recycle.cu", ()),
    ("src/optimize/primal_dual.cu", ()),
    ("src/localizing/point_to_psdf.cu", ()),
    ("src/visualization/compress_mesh.cu", ()),
]


def functions(text):
    """Yield (name, start, end) of top-level __global__/__device__ functions."""
    for m in re.finditer(r"^(__global__|__device__)\b", text, re.M):
        start = m.start()
        # a template header on the line before belongs to the function
        prev = text.rfind("\n", 0, max(start - 1, 0))
        if text[prev + 1:start].lstrip().startswith("template"):
            start = prev + 1
        brace = text.find("{", start)
        semi = text.find(";", start)
        if brace < 0 or (0 <= semi < brace):
            continue
        header = text[start:brace]
        name = re.findall(r"(\w+)\s*\(", header)
        if not name:
            continue
        depth, i = 0, brace
        while i < len(text):
            c = text[i]
            if text.startswith("//", i):          # braces in comments and literals do not count
                i = text.find("\n", i)
                continue
            if text.startswith("/*", i):
                i = text.find("*/", i) + 2
                continue
            if c in "\"'":
                j = i + 1
                while text[j] != c:
                    j += 2 if text[j] == "\\" else 1
                i = j + 1
                continue
            if c == "{":
                depth += 1
            elif c == "}":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        yield name[0], start, i + 1


def main():
    root, out = sys.argv[1], sys.argv[2]
    os.makedirs(os.path.dirname(out), exist_ok=True)
    chunks = ["// generated by oracle/refcpu/extract.py from the reference tree; not for commit\n"]
    names = []
    for rel, skip in SOURCES:
        path = os.path.join(root, rel)
        text = open(path).read()
        for name, a, b in functions(text):
            if name in skip:
                continue
            line = text.count("\n", 0, a) + 1
            chunks.append(f'#line {line} "{path}"\n' + text[a:b] + "\n")
            names.append(name)
    with open(out, "w") as f:
        f.write("".join(chunks))
    print(" ".join(names))


if __name__ == "__main__":
    main()
