"""Generate tests/golden/rholut_imexop.npz from the reference's own
suzerain/rholut_imexop.c (the oracle's reference build, oracle/_ref).

Cases follow the geometry and scenario of the reference's consistency test
(tests/test_rholut_imexop.cpp:86-130: order-6 B-splines on breakpoints
0, 0.5, 1.5, 2.25, 2.5, 3.0, 3.35; Re 3000, Pr 0.7, Ma 1.5, alpha 3,
gamma 1.4; phi = sqrt(2)/11 + i log2(e)/13) with every reference profile
nonzero (seeded U(0.5, 1.5)):

  A  km = 7e, kn = 3 pi, equations E, u, v, w, rho;
  B  km = 1, kn = 3 pi, with the non-reflecting matrices a, b, c;
  C  the zero-zero forms (packc00, packf00, accumulate00) with c;
  D  km = 0.5, kn = -2, equations in reversed positions;
  E  km = 2, kn = 1, density omitted.

Each case stores the packc band, the packf band (rows KL..), and
y = (M + phi L) x + beta y0 from accumulate for seeded x, y0.

Run from the repository root after the oracle's reference build:
    python tests/golden/make_rholut_golden.py
"""
import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

BREAKPTS = [0.0, 0.5, 1.5, 2.25, 2.5, 3.0, 3.35]
K = 6
SCENARIO = dict(Re=3000.0, Pr=0.7, Ma=1.5, alpha=3.0, gamma=1.4)
PHI = complex(math.sqrt(2) / 11, math.log2(math.e) / 13)
CASES = {
    "A": dict(km=7 * math.e, kn=3 * math.pi, order=(0, 1, 2, 3, 4), nrbc=""),
    "B": dict(km=1.0, kn=3 * math.pi, order=(0, 1, 2, 3, 4), nrbc="abc"),
    "C": dict(km=0.0, kn=0.0, order=(0, 1, 2, 3, 4), nrbc="c", zero_zero=True),
    "D": dict(km=0.5, kn=-2.0, order=(4, 3, 2, 1, 0), nrbc=""),
    "E": dict(km=2.0, kn=1.0, order=(0, 1, 2, 3, -1), nrbc=""),
}


class _Z(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def _z(v):
    v = complex(v)
    return _Z(v.real, v.imag)


def inputs(seed=20240611):
    """Profiles, NRBC matrices, x and y0 of every case (seeded)."""
    from suzerain_gb300 import rholut
    rng = np.random.default_rng(seed)
    n = len(BREAKPTS) + K - 2
    prof = {nm: rng.uniform(0.5, 1.5, n) for nm in rholut.PROFILES}
    mats = {m: rng.uniform(-1, 1, 25) for m in "abc"}
    xs = {c: (rng.normal(size=5 * n) + 1j * rng.normal(size=5 * n)) for c in CASES}
    y0 = {c: (rng.normal(size=5 * n) + 1j * rng.normal(size=5 * n)) for c in CASES}
    return n, prof, mats, xs, y0


def generate(ref_lib, synth_lib):
    from suzerain_gb300 import _native as nat, rholut
    R = ref_lib
    G = synth_lib
    G.sgb_bsplineop_alloc_breakpoints.restype = C.POINTER(nat.BsplineopWorkspace)
    G.sgb_bsplineop_alloc_breakpoints.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int]
    G.suzerain_bsplineop_free.argtypes = [C.POINTER(nat.BsplineopWorkspace)]
    P, D, I, W = C.c_void_p, C.c_double, C.c_int, C.POINTER(nat.BsplineopWorkspace)
    R.suzerain_rholut_imexop_packc.argtypes = [_Z, D, D, P, P, P, W] + [I] * 5 + [P] * 6
    R.suzerain_rholut_imexop_packf.argtypes = [_Z, D, D, P, P, P, W] + [I] * 5 + [P] * 6
    R.suzerain_rholut_imexop_packc00.argtypes = [_Z, P, P, P, W] + [I] * 5 + [P] * 4
    R.suzerain_rholut_imexop_packf00.argtypes = [_Z, P, P, P, W] + [I] * 5 + [P] * 4
    R.suzerain_rholut_imexop_accumulate.argtypes = [_Z, D, D, P, P, P, W] + [P] * 5 + [_Z] \
        + [P] * 5 + [P] * 3
    R.suzerain_rholut_imexop_accumulate00.argtypes = [_Z, P, P, P, W] + [P] * 5 + [_Z] \
        + [P] * 5 + [P]
    for f in ("packc", "packf", "packc00", "packf00", "accumulate", "accumulate00"):
        getattr(R, "suzerain_rholut_imexop_" + f).restype = None
    bp = np.array(BREAKPTS)
    w = G.sgb_bsplineop_alloc_breakpoints(K, len(bp), bp.ctypes.data, 2)
    n, prof, mats, xs, y0 = inputs()
    assert w.contents.n == n
    s = rholut.Scenario(**SCENARIO)
    r, ld, keep = rholut.ref_structs(prof, n)
    out = {"breakpts": bp, "k": K, "n": n, "phi": PHI,
           **{f"prof_{nm}": v for nm, v in prof.items()}, **{f"nrbc_{m}": v for m, v in mats.items()}}
    beta = complex(0.3, -0.2)
    out["beta"] = beta
    for name, cs in CASES.items():
        abc = [mats[m].ctypes.data if m in cs["nrbc"] else None for m in "abc"]
        order = cs["order"]
        S = sum(o >= 0 for o in order)
        A = nat.Bsmbsm()
        kl, ku = w.contents.max_kl, w.contents.max_ku
        KL, KU = S * (kl + 1) - 1, S * (ku + 1) - 1
        LD, N = KL + KU + 1, S * n
        buf = np.zeros(max(75, n * (kl + 1 + ku)), complex)
        packc = np.full(LD * N, np.nan, complex)
        packf = np.full((LD + KL) * N, np.nan, complex)
        if cs.get("zero_zero"):
            for fn, dst in (("suzerain_rholut_imexop_packc00", packc),
                            ("suzerain_rholut_imexop_packf00", packf)):
                getattr(R, fn)(_z(PHI), C.byref(s), C.byref(r), C.byref(ld), w, *order,
                               buf.ctypes.data, C.byref(A), dst.ctypes.data, abc[2])
        else:
            for fn, dst in (("suzerain_rholut_imexop_packc", packc),
                            ("suzerain_rholut_imexop_packf", packf)):
                getattr(R, fn)(_z(PHI), C.c_double(cs["km"]), C.c_double(cs["kn"]), C.byref(s),
                               C.byref(r), C.byref(ld), w, *order, buf.ctypes.data, C.byref(A),
                               dst.ctypes.data, *abc)
        assert (A.S, A.N, A.KL, A.KU, A.LD) == (S, N, KL, KU, LD)
        # accumulate: per-equation vectors (E, u, v, w, rho) of length n
        x = xs[name].copy()
        y = y0[name].copy()
        ins = [x[e * n:(e + 1) * n].ctypes.data if order[e] >= 0 else None for e in range(5)]
        outs = [y[e * n:(e + 1) * n].ctypes.data if order[e] >= 0 else None for e in range(5)]
        if cs.get("zero_zero"):
            R.suzerain_rholut_imexop_accumulate00(_z(PHI), C.byref(s), C.byref(r), C.byref(ld), w,
                                                  *ins, _z(beta), *outs, abc[2])
        else:
            R.suzerain_rholut_imexop_accumulate(_z(PHI), C.c_double(cs["km"]),
                                                C.c_double(cs["kn"]), C.byref(s), C.byref(r),
                                                C.byref(ld), w, *ins, _z(beta), *outs, *abc)
        out[f"{name}_packc"] = packc.reshape(N, LD)
        out[f"{name}_packf"] = packf.reshape(N, LD + KL)[:, KL:]
        out[f"{name}_x"] = xs[name]
        out[f"{name}_y0"] = y0[name]
        out[f"{name}_y"] = y
    G.suzerain_bsplineop_free(w)
    return out


def main():
    from oracle import oracle as O
    O.build()
    if not os.path.exists(O.REF_PATH):
        sys.exit("the oracle's reference build is missing (no reference checkout)")
    out = generate(C.CDLL(O.REF_PATH), C.CDLL(O.SYNTH_PATH))
    np.savez_compressed(os.path.join(HERE, "rholut_imexop.npz"), **out)
    print("wrote rholut_imexop.npz")


if __name__ == "__main__":
    main()
