"""GPU parity of the production implicit operator (suzerain/rholut_imexop):
packc/packf assembly and accumulate, batched and through the drop-ins,
against the reference's own rholut_imexop.c (golden vectors made by
tests/golden/make_rholut_golden.py from the oracle's reference build), and
the reference's consistency property (M + phi L)^-1 (M + phi L) = I
(tests/test_rholut_imexop.cpp:86-300) with the GPU's accumulate, pack and
zgbsvx, over the reference test's parameter sets.

Bars: every in-matrix band entry and accumulate output within 1e-13 of the
reference relative to the largest magnitude; the identity recovered within
eps / rcond (the reference's own bar); at production size (k = 8, Ny = 192)
the packed operator solved by the mixed-precision batched path meets a
normwise backward error <= 1e-12 against the GPU accumulate."""
import ctypes as C
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "rholut_imexop.npz")
SCENARIO = dict(Re=3000.0, Pr=0.7, Ma=1.5, alpha=3.0, gamma=1.4)
CASES = {
    "A": dict(km=7 * math.e, kn=3 * math.pi, order=(0, 1, 2, 3, 4), nrbc=""),
    "B": dict(km=1.0, kn=3 * math.pi, order=(0, 1, 2, 3, 4), nrbc="abc"),
    "C": dict(km=0.0, kn=0.0, order=(0, 1, 2, 3, 4), nrbc="c", zero_zero=True),
    "D": dict(km=0.5, kn=-2.0, order=(4, 3, 2, 1, 0), nrbc=""),
    "E": dict(km=2.0, kn=1.0, order=(0, 1, 2, 3, -1), nrbc=""),
}


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


@pytest.fixture(scope="module")
def lib(native, torch_cuda):
    assert native.sgb_device_ok() == 0, native.sgb_last_error().decode()
    return native


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def workspace(lib, breakpts, k):
    bp = np.ascontiguousarray(breakpts, dtype=np.float64)
    w = lib.sgb_bsplineop_alloc_breakpoints(int(k), len(bp), bp.ctypes.data, 2)
    assert w, "workspace"
    return w


def profiles_of(gold):
    from suzerain_gb300 import rholut
    return {nm: gold[f"prof_{nm}"] for nm in rholut.PROFILES}


def in_matrix_mask(N, KL, KU, off=0, ldab=None):
    """(N, ldab) mask of band positions inside the matrix."""
    ldab = ldab or KL + KU + 1
    i = np.arange(ldab)[None, :]
    c = np.arange(N)[:, None]
    r = c + i - off - KU
    return (i >= off) & (i <= off + KL + KU) & (r >= 0) & (r < N)


def close(got, want, tol=1e-13):
    scale = np.max(np.abs(want))
    err = np.max(np.abs(got - want))
    assert err <= tol * scale, (err, scale)


def nat_from_eq(v, order, n):
    """Equation-major (E, u, v, w, rho) vector -> position-major (present only)."""
    S = sum(o >= 0 for o in order)
    out = np.zeros(S * n, complex)
    for e, o in enumerate(order):
        if o >= 0:
            out[o * n:(o + 1) * n] = v[e * n:(e + 1) * n]
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_batched_pack_and_accumulate_match_reference(lib, torch_cuda, gold, name):
    torch = torch_cuda
    from suzerain_gb300 import rholut
    cs = CASES[name]
    w = workspace(lib, gold["breakpts"], int(gold["k"]))
    n = int(gold["n"])
    mats = {m: (gold[f"nrbc_{m}"] if m in cs["nrbc"] else None) for m in "abc"}
    op = rholut.Operator(SCENARIO, profiles_of(gold), w, cs["order"], **mats)
    g = op.geometry
    N, KL, KU, LD = g.N, g.KL, g.KU, g.LD
    nsys = 3                                     # the same pair thrice: batching
    km = torch.full((nsys,), cs["km"], dtype=torch.float64, device="cuda")
    kn = torch.full((nsys,), cs["kn"], dtype=torch.float64, device="cuda")
    phi = complex(gold["phi"])
    for packf, key, ldab, off in ((False, "packc", LD, 0), (True, "packf", LD + KL, KL)):
        ab = torch.full((nsys, N * ldab), complex(7, 7), dtype=torch.complex128, device="cuda")
        op.pack(phi, km, kn, ab, packf=packf)
        torch.cuda.synchronize()
        got = ab.cpu().numpy().reshape(nsys, N, ldab)
        mask = in_matrix_mask(N, KL, KU)
        want = gold[f"{name}_{key}"]
        for s in range(nsys):
            band = got[s][:, off:off + LD]
            close(band[mask], want[mask])
            if packf:                            # rows above the band untouched
                assert (got[s][:, :off] == complex(7, 7)).all()
    x = torch.from_numpy(np.tile(nat_from_eq(gold[f"{name}_x"], cs["order"], n), (nsys, 1))).cuda()
    y = torch.from_numpy(np.tile(nat_from_eq(gold[f"{name}_y0"], cs["order"], n), (nsys, 1))).cuda()
    op.accumulate(phi, km, kn, x, complex(gold["beta"]), y)
    torch.cuda.synchronize()
    want = nat_from_eq(gold[f"{name}_y"], cs["order"], n)
    for s in range(nsys):
        close(y.cpu().numpy()[s], want)
    op.close()
    lib.suzerain_bsplineop_free(w)


@pytest.mark.parametrize("name", list(CASES))
def test_dropins_match_reference(lib, gold, name):
    """suzerain_rholut_imexop_{packc,packf,accumulate}[00] with host buffers."""
    from suzerain_gb300 import _native as nat, rholut
    cs = CASES[name]
    w = workspace(lib, gold["breakpts"], int(gold["k"]))
    n = int(gold["n"])
    s = rholut.Scenario(**SCENARIO)
    r, ld, keep = rholut.ref_structs(profiles_of(gold), n)
    abc = [gold[f"nrbc_{m}"].ctypes.data if m in cs["nrbc"] else None for m in "abc"]
    phi = nat.zc(complex(gold["phi"]))
    order = cs["order"]
    S = sum(o >= 0 for o in order)
    kl, ku = w.contents.max_kl, w.contents.max_ku
    KL, KU = S * (kl + 1) - 1, S * (ku + 1) - 1
    LD, N = KL + KU + 1, S * n
    buf = np.zeros(max(75, n * (kl + 1 + ku)), complex)
    A = nat.Bsmbsm()
    packc = np.zeros(LD * N, complex)
    packf = np.full((LD + KL) * N, complex(3, 3))
    if cs.get("zero_zero"):
        lib.suzerain_rholut_imexop_packc00(phi, C.byref(s), C.byref(r), C.byref(ld), w, *order,
                                           buf.ctypes.data, C.byref(A), packc.ctypes.data, abc[2])
        lib.suzerain_rholut_imexop_packf00(phi, C.byref(s), C.byref(r), C.byref(ld), w, *order,
                                           buf.ctypes.data, C.byref(A), packf.ctypes.data, abc[2])
    else:
        for fn, dst in ((lib.suzerain_rholut_imexop_packc, packc),
                        (lib.suzerain_rholut_imexop_packf, packf)):
            fn(phi, cs["km"], cs["kn"], C.byref(s), C.byref(r), C.byref(ld), w, *order,
               buf.ctypes.data, C.byref(A), dst.ctypes.data, *abc)
    assert (A.S, A.N, A.KL, A.KU, A.LD) == (S, N, KL, KU, LD), nat.last_error()
    mask = in_matrix_mask(N, KL, KU)
    close(packc.reshape(N, LD)[mask], gold[f"{name}_packc"][mask])
    pf = packf.reshape(N, LD + KL)
    close(pf[:, KL:][mask], gold[f"{name}_packf"][mask])
    assert (pf[:, :KL] == complex(3, 3)).all()
    x = gold[f"{name}_x"].copy()
    y = gold[f"{name}_y0"].copy()
    ins = [x[e * n:(e + 1) * n].ctypes.data if order[e] >= 0 else None for e in range(5)]
    outs = [y[e * n:(e + 1) * n].ctypes.data if order[e] >= 0 else None for e in range(5)]
    beta = nat.zc(complex(gold["beta"]))
    if cs.get("zero_zero"):
        lib.suzerain_rholut_imexop_accumulate00(phi, C.byref(s), C.byref(r), C.byref(ld), w,
                                                *ins, beta, *outs, abc[2])
    else:
        lib.suzerain_rholut_imexop_accumulate(phi, cs["km"], cs["kn"], C.byref(s), C.byref(r),
                                              C.byref(ld), w, *ins, beta, *outs, *abc)
    close(y, gold[f"{name}_y"])
    lib.suzerain_bsplineop_free(w)


# The reference test's parameter sets: one nonzero profile at a time (refndx,
# -1 for none) over six wavenumber pairs, then each entry of a, b or c alone.
WAVENUMBERS = [(0, 0), (0, 3 * math.pi), (7 * math.e, 0), (1, 3 * math.pi), (7 * math.e, 1),
               (7 * math.e, 3 * math.pi)]
PARAMS = ([(km, kn, ref, -1, -1, -1) for km, kn in WAVENUMBERS for ref in range(-1, 26)]
          + [(7 * math.e, 3 * math.pi, -1, i, -1, -1) for i in range(26)]
          + [(7 * math.e, 3 * math.pi, -1, -1, i, -1) for i in range(26)]
          + [(7 * math.e, 3 * math.pi, -1, -1, -1, i) for i in range(26)])


def test_apply_then_solve_is_identity(lib, torch_cuda):
    """tests/test_rholut_imexop.cpp:86-300 on the GPU: B2 = (M + phi L) I by
    accumulate, B1 = P B2, PAP^T by packc, X = zgbsvx('E', 'T') of B1,
    P^T X = I within eps / rcond, for all of the reference's 240 parameter
    sets."""
    torch = torch_cuda
    from suzerain_gb300 import rholut
    w = workspace(lib, [0.0, 0.5, 1.5, 2.25, 2.5, 3.0, 3.35], 6)
    n = w.contents.n
    S, N = 5, 5 * n
    phi = complex(math.sqrt(2) / 11, math.log2(math.e) / 13)
    q = np.array([lib.suzerain_bsmbsm_q(S, n, i) for i in range(N)])
    eps = np.finfo(float).eps
    worst = 0.0
    for km, kn, refndx, andx, bndx, cndx in PARAMS:
        prof = {nm: (np.ones(n) if i == refndx else np.zeros(n))
                for i, nm in enumerate(rholut.PROFILES)}

        def mat(ix):
            if ix < 0:
                return None
            m = np.zeros(25)
            if ix > 0:
                m[ix - 1] = 1
            return m
        op = rholut.Operator(SCENARIO, prof, w, a=mat(andx), b=mat(bndx), c=mat(cndx))
        g = op.geometry
        kmd = torch.full((N,), km, dtype=torch.float64, device="cuda")
        knd = torch.full((N,), kn, dtype=torch.float64, device="cuda")
        eye = torch.eye(N, dtype=torch.complex128, device="cuda")   # columns as systems
        B2 = torch.zeros_like(eye)
        op.accumulate(phi, kmd, knd, eye, 0, B2)
        papt = torch.empty((1, N * g.LD), dtype=torch.complex128, device="cuda")
        op.pack(phi, kmd[:1], knd[:1], papt)
        torch.cuda.synchronize()
        B1 = B2.cpu().numpy()[:, q].T.copy(order="F")          # column j = P B2[j]
        ab = papt.cpu().numpy().reshape(-1).copy()
        X = np.zeros((N, N), complex, order="F")
        afb = np.zeros((g.LD + g.KL) * N, complex)
        ipiv = np.zeros(N, np.int32)
        eq = C.create_string_buffer(b"N", 1)
        rr, cc = np.zeros(N), np.zeros(N)
        rcond = C.c_double(0)
        ferr, berr = np.zeros(N), np.zeros(N)
        work, rwork = np.zeros(2 * N, complex), np.zeros(N)
        info = lib.suzerain_lapack_zgbsvx(b"E", b"T", N, g.KL, g.KU, N, ab.ctypes.data, g.LD,
                                          afb.ctypes.data, g.LD + g.KL, ipiv.ctypes.data,
                                          C.addressof(eq), rr.ctypes.data, cc.ctypes.data,
                                          B1.ctypes.data, N, X.ctypes.data, N,
                                          C.addressof(rcond), ferr.ctypes.data, berr.ctypes.data,
                                          work.ctypes.data, rwork.ctypes.data)
        assert info == 0, (km, kn, refndx, andx, bndx, cndx, info)
        back = np.empty_like(X)
        back[q, :] = X                                         # P^T per column
        dev = np.max(np.abs(back - np.eye(N)))
        assert dev <= eps / rcond.value, (km, kn, refndx, andx, bndx, cndx, dev, rcond.value)
        worst = max(worst, dev * rcond.value / eps)
        op.close()
    lib.suzerain_bsplineop_free(w)


def test_production_size_mixed_solve_of_packed_operator(lib, torch_cuda):
    """k = 8 B-splines on Ny = 192 stretched breakpoints (N = 960), smooth
    reference profiles, 64 wavenumber pairs: the packed transpose solved by
    the batched mixed-precision path (trans 'T') meets a normwise backward
    error <= 1e-12 against the GPU's own accumulate of the operator."""
    torch = torch_cuda
    from suzerain_gb300 import _native as nat, rholut
    Ny, k = 192, 8
    nbreak = Ny - k + 2
    x01 = np.linspace(0, 1, nbreak)
    bp = np.array([2 * lib.suzerain_htstretch2(2.0, 1.0, float(t)) for t in x01])
    w = workspace(lib, bp, k)
    n = w.contents.n
    assert n == Ny
    y = np.linspace(0, 2, n)
    prof = {nm: 0.2 * (1 + 0.3 * np.sin((i + 1) * y)) for i, nm in enumerate(rholut.PROFILES)}
    prof["nu"] = 1 + 0.1 * np.cos(y)
    op = rholut.Operator(SCENARIO, prof, w)
    g = op.geometry
    nsys = 64
    rng = np.random.default_rng(3)
    km = torch.from_numpy(rng.uniform(0, 20, nsys)).cuda()
    kn = torch.from_numpy(rng.uniform(-20, 20, nsys)).cuda()
    phi = complex(-1e-3, 0)
    ab = torch.empty((nsys, g.N * g.LD), dtype=torch.complex128, device="cuda")
    op.pack(phi, km, kn, ab)
    xt = torch.from_numpy(rng.normal(size=(nsys, g.N)) + 1j * rng.normal(size=(nsys, g.N))).cuda()
    yt = torch.zeros_like(xt)
    op.accumulate(phi, km, kn, xt, 0, yt)                    # y = A x, natural order
    qv = torch.tensor([lib.suzerain_bsmbsm_q(5, n, i) for i in range(g.N)], device="cuda")
    b = yt[:, qv].contiguous()                               # P y
    xs = torch.zeros_like(b)
    spec = nat.RefineSpec(5, 25, 5, 1.0)
    rep = {kk: torch.zeros(nsys, dtype=t, device="cuda") for kk, t in
           (("info", torch.int32), ("siter", torch.int32), ("diter", torch.int32),
            ("res", torch.float64), ("tolsc", torch.float64), ("fact", torch.uint8))}
    R = nat.RefineReport(*(rep[kk].data_ptr() for kk in ("info", "siter", "diter", "res",
                                                         "tolsc", "fact")))
    rc = lib.sgb_zcgbsvx_batched(nsys, g.N, g.KL, g.KU, b"T", ab.data_ptr(), g.LD, g.LD * g.N,
                                 b.data_ptr(), xs.data_ptr(), C.byref(spec), C.byref(R), 0)
    assert rc == 0, nat.last_error()
    torch.cuda.synchronize()
    assert (rep["info"].cpu().numpy() == 0).all()
    xr = torch.empty_like(xs)
    xr[:, qv] = xs                                           # P^T w
    yr = torch.zeros_like(xr)
    op.accumulate(phi, km, kn, xr, 0, yr)
    torch.cuda.synchronize()
    # ||A||_inf from the packed band (row sums of A = column sums of A^T)
    band = ab.cpu().numpy().reshape(nsys, g.N, g.LD)
    mask = in_matrix_mask(g.N, g.KL, g.KU)
    anorm = np.array([np.sum(np.abs(band[s]) * mask, axis=1).max() for s in range(nsys)])
    r = (yt - yr).abs().amax(dim=1).cpu().numpy()
    berr = r / (anorm * xr.abs().amax(dim=1).cpu().numpy() + yt.abs().amax(dim=1).cpu().numpy())
    assert berr.max() <= 1e-12, berr.max()
    op.close()
    lib.suzerain_bsplineop_free(w)
