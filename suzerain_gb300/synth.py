"""Seeded synthetic benchmark inputs (host side), over the C-ABI generator.

A case is a B-spline collocation basis (k, Ny, tanh stretching) plus the
S x S coefficients of the block operator defined in csrc/sgb_model.h; a batch
adds the Fourier wavenumber pairs of an (Nx, Nz) grid and one right-hand side
per pair.  The five benchmark configurations are named in CONFIGS.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat

SEED_BASE = 0x5A2E0000
DIRICHLET_MOMENTUM = 0b01110   # momentum equations 1..3 only (near-singular stress case)
DIRICHLET_ALL = 0xFFFFFFFF     # every equation (any S) gets its two wall rows


@dataclass
class SynthCase:
    S: int
    Ny: int
    k: int
    htdelta: float = 2.0
    left: float = 0.0
    right: float = 2.0
    offscale: float = 0.1
    complex_coupling: bool = False
    seed: int = SEED_BASE
    dirichlet_mask: int = DIRICHLET_ALL
    kl: int = 0
    ku: int = 0
    M: np.ndarray = field(default=None, repr=False)
    D1: np.ndarray = field(default=None, repr=False)
    D2: np.ndarray = field(default=None, repr=False)
    a: np.ndarray = field(default=None, repr=False)
    b: np.ndarray = field(default=None, repr=False)
    c: np.ndarray = field(default=None, repr=False)
    g: np.ndarray = field(default=None, repr=False)

    @property
    def n(self) -> int:
        return self.Ny

    @property
    def ld(self) -> int:
        return self.kl + 1 + self.ku

    @property
    def N(self) -> int:
        return self.S * self.Ny

    @property
    def KL(self) -> int:
        return self.S * (self.kl + 1) - 1

    @property
    def KU(self) -> int:
        return self.S * (self.ku + 1) - 1

    @property
    def LD(self) -> int:
        return self.KL + 1 + self.KU

    def ctypes_case(self) -> nat.Case:
        """sgb_case with HOST pointers into this object's arrays."""
        def p(a):
            return a.ctypes.data
        cs = nat.Case(self.S, self.n, self.kl, self.ku, self.ld, p(self.M),
                      p(self.D1), p(self.D2), p(self.a), p(self.b), p(self.c),
                      p(self.g), self.dirichlet_mask, 0)
        cs._keep = self   # keep arrays alive with the struct
        return cs


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc})")


def make_case(S=5, Ny=48, k=8, htdelta=2.0, left=0.0, right=2.0,
              offscale=0.1, complex_coupling=False, seed=SEED_BASE,
              dirichlet_mask=DIRICHLET_ALL) -> SynthCase:
    L = nat.generator()
    kl, ku = C.c_int(0), C.c_int(0)
    rc = L.sgb_synth_case(S, Ny, k, htdelta, left, right, offscale,
                          int(complex_coupling), seed, dirichlet_mask,
                          C.byref(kl), C.byref(ku), None, None, None, None,
                          None, None, None)
    _check(rc, "sgb_synth_case(query)")
    ld = kl.value + 1 + ku.value
    arrs = {nm: np.zeros(ld * Ny) for nm in ("M", "D1", "D2")}
    co = {nm: np.zeros(S * S) for nm in ("a", "b", "c", "g")}
    rc = L.sgb_synth_case(S, Ny, k, htdelta, left, right, offscale,
                          int(complex_coupling), seed, dirichlet_mask,
                          C.byref(kl), C.byref(ku), arrs["M"].ctypes.data,
                          arrs["D1"].ctypes.data, arrs["D2"].ctypes.data,
                          co["a"].ctypes.data, co["b"].ctypes.data,
                          co["c"].ctypes.data, co["g"].ctypes.data)
    _check(rc, "sgb_synth_case")
    return SynthCase(S=S, Ny=Ny, k=k, htdelta=htdelta, left=left, right=right,
                     offscale=offscale, complex_coupling=complex_coupling,
                     seed=seed, dirichlet_mask=dirichlet_mask, kl=kl.value,
                     ku=ku.value, **arrs, **co)


def wavenumbers(Nx: int, Nz: int, Lx: float, Lz: float):
    """(kx, kz) of every retained R2C mode pair, m fastest."""
    L = nat.generator()
    nsys = (Nx // 2 + 1) * Nz
    kx, kz = np.zeros(nsys), np.zeros(nsys)
    _check(L.sgb_synth_wavenumbers(Nx, Nz, Lx, Lz, kx.ctypes.data,
                                   kz.ctypes.data), "sgb_synth_wavenumbers")
    return kx, kz


def rhs(seed: int, nsys: int, N: int) -> np.ndarray:
    """(nsys, N) complex128 with independent N(0,1) parts, natural order."""
    L = nat.generator()
    u = np.zeros((nsys, N), dtype=np.complex128)
    _check(L.sgb_synth_rhs(seed, nsys, N, u.ctypes.data), "sgb_synth_rhs")
    return u


def zero_dirichlet_rows(case: SynthCase, u: np.ndarray) -> np.ndarray:
    """Zero the wall rows (natural order e*n + p) of every right-hand side."""
    for e in range(case.S):
        if (case.dirichlet_mask >> e) & 1:
            u[..., e * case.n] = 0
            u[..., e * case.n + case.n - 1] = 0
    return u


@dataclass
class Config:
    name: str
    S: int
    Ny: int
    k: int
    Nx: int
    Nz: int
    Lx: float
    Lz: float
    phi: float
    offscale: float = 0.1
    seed: int = SEED_BASE
    dirichlet_mask: int = DIRICHLET_ALL
    # zcgbsvx tolerance scale: stop when ||r||_2 <= tolsc sqrt(N) eps ||A||_F
    # ||x||_2 (suzerain/blas_et_al/dsgbsvx.def:160-163); chosen per operator
    # so that the normwise backward error of every system is <= 1e-12
    tolsc: float = 145.0

    @property
    def nsys(self) -> int:
        return (self.Nx // 2 + 1) * self.Nz

    def case(self, complex_coupling=False) -> SynthCase:
        return make_case(S=self.S, Ny=self.Ny, k=self.k, offscale=self.offscale,
                         complex_coupling=complex_coupling, seed=self.seed,
                         dirichlet_mask=self.dirichlet_mask)

    def batch(self, complex_coupling=False):
        cs = self.case(complex_coupling)
        kx, kz = wavenumbers(self.Nx, self.Nz, self.Lx, self.Lz)
        u = rhs(self.seed + 1, self.nsys, cs.N)
        return cs, kx, kz, u


FOURPI = 4 * math.pi
CONFIGS = {
    0: Config("plain-fp64-cpu-runnable", 5, 48, 8, 24, 24, FOURPI, FOURPI / 3,
              1e-3, seed=SEED_BASE + 0),
    1: Config("plain-fp64-production", 5, 192, 8, 256, 192, FOURPI,
              FOURPI / 3, 1e-3, seed=SEED_BASE + 1),
    2: Config("mixed-production", 5, 192, 8, 256, 192, FOURPI, FOURPI / 3,
              1e-3, seed=SEED_BASE + 2),
    # 145 sqrt(N) eps ~ 1e-12 leaves backward errors up to ~6e-12 on these two
    "2stiff": Config("mixed-stiff", 5, 192, 8, 256, 192, FOURPI, FOURPI / 3,
                     5e-2, offscale=0.5, seed=SEED_BASE + 2, tolsc=20.0),
    # the configuration text's wall rows (momentum equations 1..3 only)
    "2literal": Config("mixed-literal-walls", 5, 192, 8, 256, 192, FOURPI, FOURPI / 3,
                       1e-3, seed=SEED_BASE + 2, dirichlet_mask=DIRICHLET_MOMENTUM,
                       tolsc=20.0),
}


def describe_operator(cfg: Config) -> str:
    """One line naming the operator a configuration solves: wall rows, the
    sign of the implicit scale, phi dt and the off-diagonal scale."""
    if cfg.dirichlet_mask == DIRICHLET_ALL:
        walls = "wall rows on every equation"
    else:
        eqs = [e for e in range(cfg.S) if (cfg.dirichlet_mask >> e) & 1]
        walls = "wall rows on equations " + ",".join(map(str, eqs))
    return (f"(M - phi dt L) x = (M + dt alpha_0 L) u, L = a D1 + b D2 - c k^2 M, "
            f"phi dt = {cfg.phi:g}, off-diagonal scale {cfg.offscale:g}, {walls}, "
            f"zcgbsvx tolsc {cfg.tolsc:g}")

# SMR91 coefficients (suzerain/lowstorage.hpp:1242-1305), numerators / 480.
SMR91_ALPHA = (29 / 96, -3 / 40, 1 / 6)
SMR91_BETA = (37 / 160, 5 / 24, 1 / 6)
SMR91_GAMMA = (8 / 15, 5 / 12, 3 / 4)


def smr91_phis(dt_beta: float, substep: int = 0, explicit: bool = True):
    """(phi_explicit, phi_implicit) of SMR91 substep `substep` whose implicit
    scale dt*beta_i is dt_beta (the configurations' phi*dt).

    The substep solves (M - dt beta_i L) u' = (M + dt alpha_i L) u + ...
    (suzerain/lowstorage.hpp:1403-1436), so the block operator M + phi L of
    the model is assembled with phi_implicit = -dt beta_i and applied with
    phi_explicit = dt alpha_i.  L = a D1 + b D2 - c k^2 M is dissipative
    (b, c > 0), which makes M - dt beta L the well-posed implicit operator.
    explicit=False returns phi_explicit = 0 (solve-only step)."""
    dt = dt_beta / SMR91_BETA[substep]
    return (dt * SMR91_ALPHA[substep] if explicit else 0.0), -dt_beta


# Configuration 3: 64 independent cases of uneven size.  Ny uniform on
# {32, 48, ..., 256}, spline order k on {6, 8}, S on {5, 7} (S = 7: the perfect
# gas plus two species with the same block generator), (Nx, Nz) on
# {(32, 32), (64, 48), (128, 96)}, all drawn from one seeded generator.
CONFIG3_NY = tuple(range(32, 257, 16))
CONFIG3_GRIDS = ((32, 32), (64, 48), (128, 96))


def config3_cases(ncases: int = 64, seed: int = SEED_BASE + 3) -> list[Config]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(ncases):
        Ny = int(rng.choice(CONFIG3_NY))
        k = int(rng.choice((6, 8)))
        S = int(rng.choice((5, 7)))
        Nx, Nz = CONFIG3_GRIDS[int(rng.integers(len(CONFIG3_GRIDS)))]
        out.append(Config(f"config3-case{i}", S, Ny, k, Nx, Nz, FOURPI, FOURPI / 3, 1e-3,
                          seed=seed * 1000 + i))
    return out
