"""Extracts the reference's published known answers into reference_kat.json.

Reads two text files of the fdcl-gwu/FFTSO3 project (given its root as the
first argument):
  * README.md -- the printed output of example/example0.cpp: the real SO(3)
    forward transform of f(R) = tr R at l_max = 2, and f(I) (README.md:121-173);
  * bin/example4.txt -- the round-trip errors sum_l ||F - forward(inverse(F))||
    of example/example4.cpp for uniform random F at l_max = 7, 15, 31, 63
    (bin/example4.txt:1-5).
Run:  python tests/golden/make_golden.py /path/to/FFTSO3
"""
import json
import os
import re
import sys


def main(ref_root: str) -> None:
    readme = open(os.path.join(ref_root, "README.md")).read()
    start = readme.index("```\nFourier parameter F =", readme.index("bin/example0")) + 4
    block = readme[start:readme.index("```", start)]
    blocks = {}
    for m in re.finditer(r"l=(\d+)\n((?:[ \t]*[-0-9.e+ \t]+\n)+)", block):
        l = int(m.group(1))
        rows = [[float(x) for x in line.split()] for line in m.group(2).strip().splitlines()]
        blocks[l] = rows
    f_identity = float(re.search(r"f = ([-0-9.e+]+)", block).group(1))
    ex4 = open(os.path.join(ref_root, "bin", "example4.txt")).read()
    rt = {int(a): float(b) for a, b in re.findall(r"l_max = (\d+), error = ([-0-9.e+]+)", ex4)}
    out = {
        "source": {"example0": "README.md:121-173", "example4": "bin/example4.txt:1-5"},
        "example0_trace_real_forward_l_max_2": {str(l): rows for l, rows in sorted(blocks.items())},
        "example0_f_at_identity": f_identity,
        "example4_real_roundtrip_error": {str(k): v for k, v in sorted(rt.items())},
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kat.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else ".")
