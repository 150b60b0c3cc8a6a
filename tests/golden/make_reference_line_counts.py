"""Write tests/golden/reference_line_counts.json: the line count of every
source file of the reference tree (rodosti/Taylor-Couette-AFiD), so that
tests/test_citations.py can check `File.F90:line` citations on machines
without the reference checkout.

Usage: python tests/golden/make_reference_line_counts.py [REFERENCE_DIR]
(default /root/reference).
"""
import json
import os
import sys

SUFFIXES = (".F90", ".f90", ".in", ".dat", ".sh", ".sbatch")


def line_counts(ref_dir):
    out = {}
    for name in sorted(os.listdir(ref_dir)):
        path = os.path.join(ref_dir, name)
        if os.path.isfile(path) and (name.endswith(SUFFIXES) or name == "Makefile"):
            with open(path, errors="replace") as f:
                out[name] = sum(1 for _ in f)
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_line_counts.json")
    with open(dst, "w") as f:
        json.dump(line_counts(ref), f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", dst)
