"""Shape tuner of the blocked band LU, keyed (precision, N, KL, KU).

The blocked factor kernels take a panel width nb (4, 8, 16), a number of
warps per system nw (1, 2, 4, and 3 for the complex64 bandwidth-specialized
geometries) and a form (phased, or lookahead with nw < 0 in the shape
table).  Which one is fastest depends on the geometry, the
precision and the row source (a packed band in HBM, or the synthetic operator
assembled on the fly), so the choice is measured, not guessed: every
candidate is timed with CUDA events on the device and the fastest is recorded
with ``sgb_gbtrf_set_shape`` for every later factorization of that geometry
in the process (the plan and the refinement driver included).

``tune_plan`` times the plan's own substep (model rows; complex64 factor of
method 'M', complex128 factor of method 'Z'); ``tune_packed`` times
``sgb_gbtrf_batched_ex`` on a synthetic diagonally dominant packed band.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat

CANDIDATES = [(4, 1), (4, 2), (4, 3), (4, 4), (8, 1), (8, 2), (8, 4), (16, 2), (16, 4),
              (4, -2), (4, -4), (8, -2), (8, -4)]


def _supported(L, prec: bytes, N: int, KL: int, KU: int, nb: int, nw: int) -> bool:
    # set_shape validates; restore the previous entry afterwards
    b0, w0 = C.c_int(), C.c_int()
    L.sgb_gbtrf_get_shape(prec, N, KL, KU, C.byref(b0), C.byref(w0))
    ok = L.sgb_gbtrf_set_shape(prec, N, KL, KU, nb, nw) == 0
    L.sgb_gbtrf_set_shape(prec, N, KL, KU, b0.value, w0.value)
    return ok


def get_shape(prec: str, N: int, KL: int, KU: int) -> tuple[int, int]:
    L = nat.load()
    nb, nw = C.c_int(), C.c_int()
    L.sgb_gbtrf_get_shape(prec.encode(), N, KL, KU, C.byref(nb), C.byref(nw))
    return nb.value, nw.value


def set_shape(prec: str, N: int, KL: int, KU: int, nb: int, nw: int) -> None:
    L = nat.load()
    nat.check(L.sgb_gbtrf_set_shape(prec.encode(), N, KL, KU, nb, nw), "sgb_gbtrf_set_shape")


def tune_plan(plan, phi_exp: float, phi_imp: float, u_in, u_out, spec=None,
              precs: str = "C", candidates=CANDIDATES, reps: int = 2) -> dict:
    """Time the plan's factor phase for every candidate shape and keep the
    fastest per precision ('C': method 'M', 'Z': method 'Z').  u_in/u_out are
    device buffers of the plan's size (their contents are overwritten).
    Returns {prec: {(nb, nw): ms, ..., "best": (nb, nw)}}."""
    import torch
    L = nat.load()
    N, KL, KU = plan.N, plan.KL, plan.KU
    out = {}
    for prec in precs:
        method, phase = ("M", "factor_c64") if prec == "C" else ("Z", "factor_c128")
        res = {}
        for nb, nw in candidates:
            if not _supported(L, prec.encode(), N, KL, KU, nb, nw):
                continue
            set_shape(prec, N, KL, KU, nb, nw)
            plan.substep(method, phi_exp, phi_imp, u_in, u_out, spec)   # warm-up
            torch.cuda.synchronize()
            plan.set_timing(True)
            for _ in range(reps):
                plan.substep(method, phi_exp, phi_imp, u_in, u_out, spec)
            torch.cuda.synchronize()
            t = plan.timings()
            plan.set_timing(False)
            res[(nb, nw)] = t[phase][0] / t[phase][1]
        best = min(res, key=res.get)
        set_shape(prec, N, KL, KU, *best)
        res["best"] = best
        out[prec] = res
    return out


def tune_packed(prec: str, N: int, KL: int, KU: int, nsys: int = 2048,
                candidates=CANDIDATES, reps: int = 3, seed: int = 0) -> dict:
    """Time sgb_gbtrf_batched_ex on a diagonally dominant random packed band
    of nsys systems and keep the fastest shape.  Returns {(nb, nw): ms,
    "best": (nb, nw)}."""
    import torch
    L = nat.load()
    ld = KL + KU + 1
    g = torch.Generator(device="cuda").manual_seed(seed)
    ab = torch.complex(torch.randn(nsys, N, ld, device="cuda", dtype=torch.float64, generator=g),
                       torch.randn(nsys, N, ld, device="cuda", dtype=torch.float64, generator=g))
    ab[:, :, KU] += 4.0 * (KL + KU + 1)
    ab = ab.contiguous()
    fe = L.sgb_factor_elems(N, KL, KU)
    dt = torch.complex128 if prec == "Z" else torch.complex64
    fac = torch.empty(nsys * fe, dtype=dt, device="cuda")
    ipiv = torch.empty(nsys * N, dtype=torch.int32, device="cuda")
    info = torch.empty(nsys, dtype=torch.int32, device="cuda")
    res = {}
    for nb, nw in candidates:
        variant, w = (2, -nw) if nw < 0 else (0, nw)
        args = (prec.encode(), nsys, N, KL, KU, ab.data_ptr(), ld, ld * N, fac.data_ptr(),
                ipiv.data_ptr(), info.data_ptr(), variant, nb, w, 0)
        if L.sgb_gbtrf_batched_ex(*args) != 0:
            continue
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            L.sgb_gbtrf_batched_ex(*args)
        e1.record()
        torch.cuda.synchronize()
        res[(nb, nw)] = e0.elapsed_time(e1) / reps
    best = min(res, key=res.get)
    set_shape(prec, N, KL, KU, *best)
    res["best"] = best
    return res
