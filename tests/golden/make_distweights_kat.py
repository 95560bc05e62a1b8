"""Writes distweights_kat.json: the known-answer cases of the reference test
suite for ``distweights`` (MaxwellFDFD.jl test/source.jl:5-121).

Each case is restated from that file: the deliberately non-uniform 1D grid
(test/source.jl:6-15), the query point ``c``, the grid type, the boundary
(Bloch or symmetry) and the expected ``(ind, wt)`` written exactly as the
test's formulas compute them (1-based indices, as in Julia), or ``throws``
for the cases the test expects an ArgumentError.  The random N = 1 case
(test/source.jl:106-120) is a property test and lives in the test module.

Run:  python tests/golden/make_distweights_kat.py
"""
import json
import os

import numpy as np


def main():
    dlg = np.arange(2, 23, 2, dtype=float)                    # ∆lg = 2:2:22
    lq = np.cumsum(np.concatenate([[-1.0], dlg]))             # l′
    lprim_g = 0.5 * (lq[:-1] + lq[1:])                        # movingavg(l′)
    ldual_g = lq[:-1]
    domain = [float(lprim_g[0]), float(lprim_g[-1])]
    lprim, dlprim = lprim_g[:-1], np.diff(ldual_g)
    ldual, dldual = ldual_g[1:], np.diff(lprim_g)

    P, D = "PRIM", "DUAL"
    cases = []

    def add(c, gt, bloch, ind=None, wt=None, throws=False, line=None):
        cases.append({"c": float(c), "gt": gt, "isbloch": bool(bloch),
                      "ind": ind, "wt": None if wt is None else [float(x) for x in wt],
                      "throws": throws, "ref_line": line})

    dp, dd = dlprim, dldual
    # primal grid points [0,3,8,15,24,35,48,63,80,99 (,120)]
    add(8, P, True, [3, 3], [1 / dp[2], 0], line=19)
    add(8, P, False, [3, 3], [1 / dp[2], 0], line=20)
    r = (11 - 8) / (15 - 8)
    add(11, P, True, [3, 4], [1 / dp[2] * (1 - r), 1 / dp[3] * r], line=24)
    add(11, P, False, [3, 4], [1 / dp[2] * (1 - r), 1 / dp[3] * r], line=25)
    add(3, P, True, [2, 2], [1 / dp[1], 0], line=28)
    add(3, P, False, [2, 2], [1 / dp[1], 0], line=29)
    r = (3 - 1) / (3 - 0)
    add(1, P, True, [1, 2], [1 / dp[0] * r, 1 / dp[1] * (1 - r)], line=33)
    add(1, P, False, [2, 2], [1 / dp[1] * (1 - r), 0], line=34)
    add(0, P, True, [1, 1], [1 / dp[0], 0], line=37)
    add(0, P, False, [2, 2], [0, 0], line=38)
    add(-0.5, P, True, throws=True, line=41)
    add(-0.5, P, False, throws=True, line=42)
    add(-1, P, True, throws=True, line=45)
    add(-1, P, False, throws=True, line=46)
    add(99, P, True, [10, 10], [1 / dp[9], 0], line=49)
    add(99, P, False, [10, 10], [1 / dp[9], 0], line=50)
    r = (105 - 99) / (120 - 99)
    add(105, P, True, [10, 1], [1 / dp[9] * (1 - r), 1 / dp[0] * r], line=54)
    add(105, P, False, [10, 10], [1 / dp[9] * (1 - r), 0], line=55)
    r = (120 - 99) / (120 - 99)
    add(120, P, True, [10, 1], [1 / dp[9] * (1 - r), 1 / dp[0] * r], line=59)
    add(120, P, False, [10, 10], [1 / dp[9] * (1 - r), 0], line=60)
    # dual grid points [(-1,) 1,5,11,19,29,41,55,71,89,109]
    add(11, D, True, [3, 3], [1 / dd[2], 0], line=66)
    add(11, D, False, [3, 3], [1 / dd[2], 0], line=67)
    r = (15 - 11) / (19 - 11)
    add(15, D, True, [3, 4], [1 / dd[2] * (1 - r), 1 / dd[3] * r], line=71)
    add(15, D, False, [3, 4], [1 / dd[2] * (1 - r), 1 / dd[3] * r], line=72)
    add(1, D, True, [1, 1], [1 / dd[0], 0], line=75)
    add(1, D, False, [1, 1], [1 / dd[0], 0], line=76)
    r = (1 - 0.5) / ((1 - 0) + (120 - 109))
    add(0.5, D, True, [1, 10], [1 / dd[0] * (1 - r), 1 / dd[9] * r], line=80)
    add(0.5, D, False, [1, 1], [1 / dd[0], 0], line=81)
    r = (1 - 0) / ((1 - 0) + (120 - 109))
    add(0, D, True, [1, 10], [1 / dd[0] * (1 - r), 1 / dd[9] * r], line=85)
    add(0, D, False, [1, 1], [1 / dd[0], 0], line=86)
    add(-0.5, D, True, throws=True, line=89)
    add(-0.5, D, False, throws=True, line=90)
    add(109, D, True, [10, 10], [1 / dd[9], 0], line=93)
    add(109, D, False, [10, 10], [1 / dd[9], 0], line=94)
    r = (115 - 109) / ((120 - 109) + (1 - 0))
    add(115, D, True, [10, 1], [1 / dd[9] * (1 - r), 1 / dd[0] * r], line=98)
    add(115, D, False, [10, 10], [1 / dd[9], 0], line=99)
    r = (120 - 109) / ((120 - 109) + (1 - 0))
    add(120, D, True, [10, 1], [1 / dd[9] * (1 - r), 1 / dd[0] * r], line=103)
    add(120, D, False, [10, 10], [1 / dd[9], 0], line=104)

    out = {
        "source": "MaxwellFDFD.jl test/source.jl:5-121 (distweights testset); ref_line is the "
                  "line of the @test in test/source.jl",
        "domain": domain,
        "PRIM": {"l": lprim.tolist(), "dl": dlprim.tolist()},
        "DUAL": {"l": ldual.tolist(), "dl": dldual.tolist()},
        "cases": cases,
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "distweights_kat.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(cases)} cases to {path}")


if __name__ == "__main__":
    main()
