"""Generate tests/golden/*.json from the reference's own unit tests.

Reads, as text, the known-answer data the reference's tests pin the banded
solve path with, and writes it as JSON fixtures:

  bsmbsm_kat.json    tests/test_bsmbsm.cpp
                       q / qinv for S=5, n=9 (Octave-derived expectations,
                       :48-152); collocation bands M, D1, D2 of order-6
                       B-splines on breakpoints {0,1/4,3/4,1,5/4,2}, right
                       hand side BR and the 30-digit solution XR of the
                       S=3 BSMBSM operator (Mathematica, :700-800).
  bsplineop_kat.json tests/test_bsplineop.cpp
                       transposed mass band of order-3 B-splines on
                       {0,1,2,3} and its complex apply (:465-540).
  bsplineop_luz_kat.json tests/test_bsplineop.cpp
                       the complex operator (2-3i) D0 + (7-5i) D1 +
                       (999-999i) D2 of order-2 B-splines on {0,1,2,3}:
                       its solves against the unit basis vectors and two
                       right-hand sides, contiguous and with incb 2
                       (:340-462, Octave rationals).

Rational entries such as 1024.0/3125.0 are evaluated exactly with
fractions.Fraction and rounded once to double.  Run from the repository root:
    python tests/golden/make_golden.py [reference_checkout]
"""
from __future__ import annotations

import json
import os
import re
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))


def _num(tok: str) -> float:
    tok = tok.strip().replace(" ", "")
    if not tok:
        raise ValueError("empty token")
    if "/" in tok:
        a, b = tok.split("/")
        return float(Fraction(a.rstrip(".")) / Fraction(b.rstrip(".")))
    return float(Fraction(tok.rstrip(".")) if tok[-1] == "." else tok)


def _array(src: str, name: str) -> list[float]:
    m = re.search(r"static const double\s+" + re.escape(name) +
                  r"\[\]\s*=\s*\{(.*?)\};", src, re.S)
    if not m:
        raise KeyError(name)
    body = re.sub(r"//[^\n]*", "", m.group(1))
    return [_num(t) for t in body.split(",") if t.strip()]


def _checks(src: str, case: str, fn: str) -> list[list[int]]:
    m = re.search(r"BOOST_AUTO_TEST_CASE\(\s*" + case + r"\s*\)(.*?)\n\}", src,
                  re.S)
    pairs = re.findall(r"BOOST_CHECK_EQUAL\(\s*(\d+),\s*" + fn +
                       r"\(S, n,\s*(\d+)\)\)", m.group(1))
    return [[int(i), int(v)] for v, i in pairs]


def bsmbsm_kat(ref: str) -> dict:
    src = open(os.path.join(ref, "tests", "test_bsmbsm.cpp")).read()
    out = {"source": "tests/test_bsmbsm.cpp",
           "q_S5n9": _checks(src, "q_S5n9", "suzerain_bsmbsm_q"),
           "qinv_S5n9": _checks(src, "qinv_S5n9", "suzerain_bsmbsm_qinv"),
           "S": 3, "n": 10, "kl": 4, "ku": 4,
           "breakpoints": [0, 0.25, 0.75, 1.0, 1.25, 2.0], "k": 6,
           "tolerance_eps_multiple": 1.8e4}
    for nm in ("M", "D1", "D2", "BR", "XR"):
        out[nm] = _array(src, nm)
    # The operator: op = [[M, D1/5, 0], [D2/7, 2M, D2/14], [0, D1/10, 4M]]
    out["blocks"] = [[["M", 1.0], ["D1", 0.2], None],
                     [["D2", 1 / 7], ["M", 2.0], ["D2", 1 / 14]],
                     [None, ["D1", 0.1], ["M", 4.0]]]
    return out


def bsplineop_kat(ref: str) -> dict:
    src = open(os.path.join(ref, "tests", "test_bsplineop.cpp")).read()
    sect = src[src.index("BOOST_AUTO_TEST_CASE( collocation_piecewise_quadratic)"):]
    m = re.search(r"good_D_T0\[\]\s*=\s*\{(.*?)\};", sect, re.S)
    body = re.sub(r"/\*.*?\*/", "", m.group(1))
    band = [_num(t) for t in body.split(",") if t.strip()]
    return {"source": "tests/test_bsplineop.cpp",
            "k": 3, "breakpoints": [0.0, 1.0, 2.0, 3.0], "n": 5,
            "kl": 1, "ku": 1, "ld": 3,
            "mass_D_T0_band": band,
            "apply_complex_x": [[1, 2], [3, 4], [5, 6], [7, 8], [9, 10]],
            "apply_complex_good": [[1., 2.], [2.75, 3.75], [5., 6.],
                                   [7.25, 8.25], [9., 10.]]}


def _pairs(sect: str, name: str) -> list[list[float]]:
    m = re.search(re.escape(name) + r"\[\]\[2\]\s*=\s*\{(.*?)\};", sect, re.S)
    if not m:
        raise KeyError(name)
    body = re.sub(r"//[^\n]*", "", m.group(1))
    return [[_num(a), _num(b)] for a, b in re.findall(r"\{([^,{}]+),([^,{}]+)\}", body)]


def bsplineop_luz_kat(ref: str) -> dict:
    src = open(os.path.join(ref, "tests", "test_bsplineop.cpp")).read()
    case = src[src.index("BOOST_AUTO_TEST_CASE( collocation_piecewise_linear )"):
               src.index("BOOST_AUTO_TEST_CASE( collocation_piecewise_quadratic)")]
    marks = ['BOOST_TEST_MESSAGE("suzerain_bspline_luz_form")',
             'BOOST_TEST_MESSAGE("suzerain_bspline_luz_solve contiguous")',
             'BOOST_TEST_MESSAGE("suzerain_bspline_luz_solve noncontiguous")']
    sects = [case[case.index(marks[i]):case.index(marks[i + 1]) if i + 1 < 3 else len(case)]
             for i in range(3)]
    solves = []
    for sect, nrhs, incb in zip(sects, (8, 2, 2), (1, 1, 2)):
        solves.append({"nrhs": nrhs, "incb": incb, "b": _pairs(sect, "b"),
                       "b_good": _pairs(sect, "b_good"), "tolerance": 1e-5})
    return {"source": "tests/test_bsplineop.cpp",
            "k": 2, "breakpoints": [0.0, 1.0, 2.0, 3.0], "nderiv": 2, "n": 4,
            "coefficients": _pairs(sects[0], "coeff"), "solves": solves}


def main(ref: str) -> None:
    for name, fn in (("bsmbsm_kat.json", bsmbsm_kat),
                     ("bsplineop_kat.json", bsplineop_kat),
                     ("bsplineop_luz_kat.json", bsplineop_luz_kat)):
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(fn(ref), f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    # the reference checkout: argument, else SUZERAIN_REFERENCE_DIR, else the
    # oracle build recipe's default
    ROOT = os.path.dirname(os.path.dirname(HERE))
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    ref = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    if not ref:
        sys.exit("no reference checkout: pass its path or set SUZERAIN_REFERENCE_DIR")
    main(ref)
