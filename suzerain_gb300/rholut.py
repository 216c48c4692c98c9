"""The production implicit operator (Python face of sgb_rholut_* and the
suzerain_rholut_imexop_* drop-ins).

An Operator holds, on the device, the collocation bands of a B-spline
workspace, the 26 wall-normal reference profiles of the linearisation, the
scenario constants and the optional non-reflecting boundary matrices; pack()
writes P (M + phi L)^T P^T for many wavenumber pairs as packed bands and
accumulate() applies y <- (M + phi L) x + beta y, both batched over the
pairs (suzerain/rholut_imexop.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as nat

PROFILES = ("ux", "uy", "uz", "u2", "uxux", "uxuy", "uxuz", "uyuy", "uyuz", "uzuz",
            "nu", "nuux", "nuuy", "nuuz", "nuu2", "nuuxux", "nuuxuy", "nuuxuz", "nuuyuy",
            "nuuyuz", "nuuzuz", "ex_gradrho", "ey_gradrho", "ez_gradrho", "e_divm",
            "e_deltarho")


class Scenario(C.Structure):
    _fields_ = [("Re", C.c_double), ("Pr", C.c_double), ("Ma", C.c_double),
                ("alpha", C.c_double), ("gamma", C.c_double)]


class Ref(C.Structure):
    _fields_ = [(nm, C.c_void_p) for nm in PROFILES]


class RefLd(C.Structure):
    _fields_ = [(nm, C.c_int) for nm in PROFILES]


def ref_structs(profiles: dict, n: int):
    """(Ref, RefLd, keep-alive list) for profile arrays of length n (missing
    names are zero profiles)."""
    keep = []
    r, ld = Ref(), RefLd()
    for nm in PROFILES:
        a = np.ascontiguousarray(profiles.get(nm, np.zeros(n)), dtype=np.float64)
        assert a.shape == (n,)
        keep.append(a)
        setattr(r, nm, a.ctypes.data)
        setattr(ld, nm, 1)
    return r, ld, keep


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


def _mat(m):
    return None if m is None else np.ascontiguousarray(m, dtype=np.float64).reshape(25)


class Operator:
    def __init__(self, scenario: dict, profiles: dict, workspace, order=(0, 1, 2, 3, 4),
                 a=None, b=None, c=None):
        """workspace: a pointer to a suzerain_bsplineop_workspace (nderiv >= 2),
        e.g. from sgb_bsplineop_alloc_breakpoints; profiles: {name: array of
        length n}; order: positions of E, u, v, w, rho (negative omits)."""
        self.L = nat.load()
        self.s = Scenario(**scenario)
        n = workspace.contents.n
        self.r, self.ld, self._keep = ref_structs(profiles, n)
        self._abc = [_mat(m) for m in (a, b, c)]
        self.order = (C.c_int * 5)(*order)
        h = self.L.sgb_rholut_create(C.byref(self.s), C.byref(self.r), C.byref(self.ld),
                                     workspace, self.order,
                                     *[None if m is None else m.ctypes.data for m in self._abc])
        if not h:
            raise RuntimeError(f"sgb_rholut_create failed: {nat.last_error()}")
        self.handle = h
        g = nat.Bsmbsm()
        nat.check(self.L.sgb_rholut_geometry(h, C.byref(g)), "sgb_rholut_geometry")
        self.geometry = g

    def close(self):
        if getattr(self, "handle", None):
            self.L.sgb_rholut_destroy(self.handle)
            self.handle = None

    __del__ = close

    def pack(self, phi: complex, km, kn, ab, packf: bool = False, stream=0) -> None:
        """P (M + phi L)^T P^T of every pair (km, kn: device float64 arrays)
        into ab (device, nsys x ldab x N complex128): packc (ldab = LD) or
        packf (ldab = LD + KL, band from row KL)."""
        g = self.geometry
        ldab, off = (g.LD + g.KL, g.KL) if packf else (g.LD, 0)
        nsys = int(km.shape[0])
        phi = complex(phi)
        nat.check(self.L.sgb_rholut_pack_batched(self.handle, phi.real, phi.imag, nsys, _ptr(km),
                                                 _ptr(kn), _ptr(ab), ldab, ldab * g.N, off,
                                                 _ptr(stream)), "sgb_rholut_pack_batched")

    def accumulate(self, phi: complex, km, kn, x, beta: complex, y, stream=0) -> None:
        """y <- (M + phi L) x + beta y per pair; x, y device (nsys x S n,
        equation position major)."""
        g = self.geometry
        nsys = int(km.shape[0])
        phi, beta = complex(phi), complex(beta)
        nat.check(self.L.sgb_rholut_accumulate_batched(self.handle, phi.real, phi.imag, nsys,
                                                       _ptr(km), _ptr(kn), _ptr(x), g.N,
                                                       beta.real, beta.imag, _ptr(y), g.N,
                                                       _ptr(stream)),
                  "sgb_rholut_accumulate_batched")
