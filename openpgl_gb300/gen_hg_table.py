"""Writes csrc/hg_table.h: the 128 three-lobe von Mises-Fisher fits of the
single-lobe Henyey-Greenstein phase function that Open PGL's volume sampling
distribution multiplies with (directional/vmm/VMMPhaseFunctions.cpp, the table
filled by VMMSingleLobeHenyeyGreensteinOracle::init; entry i covers mean
cosines |g| in [i, i + 1) * 0.99 / 128).  The table is fitted data the
reference's products depend on, so its values are kept as they are: this
script reads the reference source (given on the command line), converts every
decimal literal to the float32 a C++ compiler makes of it (correctly rounded
from the exact decimal value) and emits the values as hexadecimal float
literals in this repository's own layout.  Run once; the header is committed.

usage: python openpgl_gb300/gen_hg_table.py <path of VMMPhaseFunctions.cpp>
"""

import os
import re
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("weights", "meanCosines", "kappas", "normalizations")


def to_f32(literal):
    """float32 nearest to the exact decimal value (ties to even)."""
    x = Fraction(literal.rstrip("fF"))
    if x == 0:
        return np.float32(0.0)
    sign = -1 if x < 0 else 1
    x = abs(x)
    lo = np.float32(float(x))  # within one ulp of the answer
    cands = [np.nextafter(lo, np.float32(0)), lo, np.nextafter(lo, np.float32(np.inf))]
    best = min(cands, key=lambda c: (abs(Fraction(float(c)) - x), int(np.float32(c).view(np.uint32)) & 1))
    return np.float32(sign * float(best))


def main(path):
    text = open(path).read()
    reps = {}
    for m in re.finditer(r"representations\[(\d+)\]\.(\w+)(?:\[(\d+)\])?\s*=\s*([^;]+);", text):
        i, field, j, value = int(m.group(1)), m.group(2), m.group(3), m.group(4).strip()
        reps.setdefault(i, {})[(field, None if j is None else int(j))] = value
    assert sorted(reps) == list(range(128)), "expected 128 entries"
    lines = []
    for i in range(128):
        r = reps[i]
        assert int(r[("K", None)]) == 3, "every entry has three lobes"
        lobes = []
        for j in range(3):
            vals = [to_f32(r[(f, j)]) for f in FIELDS]
            lobes.append("{" + ", ".join(float(v).hex() + "f" for v in vals) + "}")
        lines.append("    {" + ", ".join(lobes) + "},")
    out = os.path.join(HERE, "csrc", "hg_table.h")
    with open(out, "w") as f:
        f.write("// Generated by openpgl_gb300/gen_hg_table.py: three-lobe vMF fits of the single-lobe\n"
                "// Henyey-Greenstein phase function (directional/vmm/VMMPhaseFunctions.cpp, the table of\n"
                "// VMMSingleLobeHenyeyGreensteinOracle::init), entry i for mean cosines |g| in\n"
                "// [i, i + 1) * 0.99 / 128.  Per lobe: weight, mean cosine, kappa, normalisation.\n"
                "#pragma once\n\n"
                "namespace pgl {\n\n"
                "struct HgLobeFit {\n  float weight, meanCosine, kappa, normalization;\n};\n"
                "constexpr int kHgFits = 128;\nconstexpr int kHgLobes = 3;\n"
                "constexpr float kHgMinMeanCosine = 0.0f, kHgMaxMeanCosine = 0.99f;\n\n"
                "constexpr HgLobeFit kHgTable[kHgFits][kHgLobes] = {\n")
        f.write("\n".join(lines) + "\n};\n\n}  // namespace pgl\n")
    print(out)


if __name__ == "__main__":
    main(sys.argv[1])
