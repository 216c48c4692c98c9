"""GPU parity: the CUDA path through the C-ABI against the oracle.

Bars: integer results (pivots, info) bit-exact; complex128 solutions within
1e-11 relative of the oracle and normwise backward error <= 1e-13; mixed
precision results with backward error <= 1e-12 and the reference's
convergence decisions."""
import ctypes as C
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


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


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rand_band(rng, n, kl, ku, extra=0, dtype=np.complex128):
    ld = extra + kl + ku + 1
    ab = np.zeros(ld * n, dtype=dtype)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[extra + ku + i - j + j * ld] = complex(rng.normal(), rng.normal())
    return ab, ld


GEOMS = [(40, 3, 5), (240, 34, 34), (13, 12, 0), (7, 0, 3), (97, 48, 48),
         (64, 31, 2), (50, 33, 40), (1, 0, 0), (200, 24, 24)]


@pytest.mark.parametrize("n,kl,ku", GEOMS)
def test_gbtrf_batched_fp64_matches_zgbtf2(lib, oracle, torch_cuda, n, kl, ku):
    torch = torch_cuda
    rng = np.random.default_rng(100 + n + kl)
    nsys = 5
    bands = [rand_band(rng, n, kl, ku)[0] for _ in range(nsys)]
    ld = kl + ku + 1
    ab = dev(torch, np.stack(bands))
    fe = lib.sgb_factor_elems(n, kl, ku)
    fac = torch.zeros(nsys * fe, dtype=torch.complex128, device="cuda")
    ipiv = torch.zeros(nsys * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
    assert lib.sgb_gbtrf_batched(b"Z", nsys, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                 fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0) == 0
    ldab = 2 * kl + ku + 1
    lap = torch.zeros(nsys * ldab * n, dtype=torch.complex128, device="cuda")
    assert lib.sgb_factor_to_lapack(b"Z", nsys, n, kl, ku, fac.data_ptr(), lap.data_ptr(), 0) == 0
    torch.cuda.synchronize()
    lap = lap.cpu().numpy().reshape(nsys, -1)
    ipiv = ipiv.cpu().numpy().reshape(nsys, n)
    for s in range(nsys):
        full = np.zeros(ldab * n, dtype=np.complex128)
        for j in range(n):
            full[kl + j * ldab: kl + j * ldab + ld] = bands[s][j * ld:(j + 1) * ld]
        oinfo, opiv = oracle.zgbtrf(full, n, kl, ku, ldab)
        assert info[s].item() == oinfo
        assert np.array_equal(ipiv[s], opiv)
        scale = max(1.0, np.abs(full).max())
        assert np.max(np.abs(lap[s] - full)) <= 1e-12 * scale


@pytest.mark.parametrize("n,kl,ku", GEOMS)
@pytest.mark.parametrize("prec", ["Z", "C"])
def test_blocked_factor_equals_unblocked(lib, torch_cuda, n, kl, ku, prec):
    """The blocked kernels (phased and lookahead) defer the rank-1 updates
    into GEMMs but apply the same multiply-adds in the same order: factors
    are bit-identical to the unblocked kernel's."""
    torch = torch_cuda
    rng = np.random.default_rng(300 + n + kl)
    nsys = 5
    bands = [rand_band(rng, n, kl, ku)[0] for _ in range(nsys)]
    # make pivoting frequent: scale random rows up
    for b_ in bands:
        for j in range(n):
            if rng.random() < 0.3:
                for i in range(max(0, j - ku), min(n, j + kl + 1)):
                    b_[ku + i - j + j * (kl + ku + 1)] *= 8.0
    ld = kl + ku + 1
    ab = dev(torch, np.stack(bands))
    fe = lib.sgb_factor_elems(n, kl, ku)
    dt = torch.complex128 if prec == "Z" else torch.complex64
    outs = []
    shapes = [(1, 8, 1)] + [(0, nb, nw) for nb in (4, 8, 16) for nw in (1, 2, 4)
                            if kl <= {1: 52, 2: 56, 4: 64}[nw]] \
        + [(2, nb, nw) for nb in (4, 8, 16) for nw in (2, 4) if kl <= {2: 56, 4: 64}[nw]]
    for variant, nb, nw in shapes:
        fac = torch.full((nsys * fe,), float("nan"), dtype=dt, device="cuda")
        ipiv = torch.zeros(nsys * n, dtype=torch.int32, device="cuda")
        info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
        assert lib.sgb_gbtrf_batched_ex(prec.encode(), nsys, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                        fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), variant,
                                        nb, nw, 0) == 0, lib.sgb_last_error().decode()
        torch.cuda.synchronize()
        outs.append((fac.cpu().numpy(), ipiv.cpu().numpy(), info.cpu().numpy()))
    fv = np.float32 if prec == "C" else np.float64
    for (variant, nb, nw), (fac, ipiv, info) in zip(shapes[1:], outs[1:]):
        assert np.array_equal(ipiv, outs[0][1]) and np.array_equal(info, outs[0][2]), (nb, nw)
        assert np.array_equal(fac.view(fv), outs[0][0].view(fv)), (nb, nw)


def test_specialized_factor_matches_generic(lib, torch_cuda):
    """The complex64 factor's compile-time bandwidth instances (KL = KU = 24,
    34, 48, N a multiple of 4; two warps, and three for KL <= 34) give the
    generic instance's bits: factors, pivots and info of packed bands with
    frequent pivoting, and the mixed substeps of plans whose operators
    assemble in the kernel (fused forward elimination), per case with two
    and three warps and as one ragged batch."""
    torch = torch_cuda
    from suzerain_gb300 import multicase, plan as P, synth
    rng = np.random.default_rng(77)
    nsys = 6
    try:
        for n, kl in ((240, 24), (480, 34), (192, 48), (97, 34)):
            ku = kl
            bands = [rand_band(rng, n, kl, ku)[0] for _ in range(nsys)]
            for b_ in bands:
                for j in range(n):
                    if rng.random() < 0.3:
                        for i in range(max(0, j - ku), min(n, j + kl + 1)):
                            b_[ku + i - j + j * (kl + ku + 1)] *= 8.0
            ld = kl + ku + 1
            ab = dev(torch, np.stack(bands))
            fe = lib.sgb_factor_elems(n, kl, ku)
            outs = []
            three = kl <= 34 and n % 4 == 0
            for on, nw in ((0, 2), (1, 2)) + (((1, 3),) if three else ()):
                assert lib.sgb_gbtrf_set_specialized(on) == 0
                fac = torch.full((nsys * fe,), float("nan"), dtype=torch.complex64, device="cuda")
                ipiv = torch.zeros(nsys * n, dtype=torch.int32, device="cuda")
                info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
                assert lib.sgb_gbtrf_batched_ex(b"C", nsys, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                                fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0,
                                                4, nw, 0) == 0, lib.sgb_last_error().decode()
                torch.cuda.synchronize()
                outs.append((fac.cpu().numpy().view(np.float32), ipiv.cpu().numpy(),
                             info.cpu().numpy()))
            assert (lib.sgb_gbtrf_batched_ex(b"C", nsys, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                             fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0,
                                             4, 3, 0) == 0) == three
            for o in outs[1:]:
                for x, y in zip(outs[0], o):
                    assert np.array_equal(x, y), (n, kl)
        # plans (model assembly + fused forward elimination), KL = 24, 48, 34
        cfgs = [synth.Config("a", 5, 48, 6, 8, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=11),
                synth.Config("b", 7, 64, 8, 8, 6, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=12),
                synth.Config("c", 5, 96, 8, 16, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=13)]
        spec = P.RefineSpec(aiter=5, siter=3, diter=5, tolsc=145.0)
        from suzerain_gb300 import tune as T
        res = {}
        for on, ragged, nw in ((0, False, 0), (1, False, 0), (1, True, 0), (1, False, 3)):
            assert lib.sgb_gbtrf_set_specialized(on) == 0
            mc = multicase.MultiCase(cfgs, nstreams=2, ragged=ragged)
            if nw:
                for cs in mc.cases:
                    if cs.KL <= 34:
                        T.set_shape("C", cs.N, cs.KL, cs.KU, 4, nw)
            mc.capture("M", spec)
            mc.reset()
            mc.replay()
            torch.cuda.synchronize()
            res[(on, ragged, nw)] = [mc.result(i).cpu().numpy() for i in range(len(cfgs))]
            mc.close()
            if nw:
                for cs in mc.cases:
                    if cs.KL <= 34:
                        T.set_shape("C", cs.N, cs.KL, cs.KU, 4, 2)
        assert sorted(c.KL for c in mc.cases) == [24, 34, 48]
        for key, r in res.items():
            for i in range(len(cfgs)):
                assert np.array_equal(r[i], res[(0, False, 0)][i]), (key, i)
    finally:
        lib.sgb_gbtrf_set_specialized(1)


@pytest.mark.parametrize("n,kl,ku", [(40, 3, 5), (240, 34, 34), (97, 48, 48)])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("prec", ["Z", "C"])
def test_gbtrs_batched(lib, oracle, torch_cuda, n, kl, ku, trans, prec):
    torch = torch_cuda
    rng = np.random.default_rng(7 + n)
    nsys = 4
    ld = kl + ku + 1
    bands = [rand_band(rng, n, kl, ku)[0] for _ in range(nsys)]
    b = rng.normal(size=(nsys, n)) + 1j * rng.normal(size=(nsys, n))
    ab = dev(torch, np.stack(bands))
    fe = lib.sgb_factor_elems(n, kl, ku)
    fdt = torch.complex128 if prec == "Z" else torch.complex64
    fac = torch.zeros(nsys * fe, dtype=fdt, device="cuda")
    ipiv = torch.zeros(nsys * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
    assert lib.sgb_gbtrf_batched(prec.encode(), nsys, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                 fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0) == 0
    db = dev(torch, b)
    x = torch.zeros_like(db)
    assert lib.sgb_gbtrs_batched(prec.encode(), trans.encode(), nsys, n, kl, ku, fac.data_ptr(),
                                 ipiv.data_ptr(), db.data_ptr(), x.data_ptr(), 0) == 0
    torch.cuda.synchronize()
    x = x.cpu().numpy()
    for s in range(nsys):
        A = oracle.band_to_dense(bands[s], n, kl, ku, ld)
        op = A if trans == "N" else (A.T if trans == "T" else A.conj().T)
        berr = np.max(np.abs(op @ x[s] - b[s])) / (np.abs(op).sum(1).max() * np.abs(x[s]).max() + np.abs(b[s]).max())
        assert berr <= (1e-14 if prec == "Z" else 1e-5), berr


@pytest.mark.parametrize("n,kl,ku", [(40, 3, 5), (240, 34, 34), (97, 48, 48)])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("prec", ["Z", "C"])
def test_gbtrs_shared_factor_many_rhs(lib, oracle, torch_cuda, n, kl, ku, trans, prec):
    """One factor, nrhs right-hand sides with padded leading dimensions:
    bit-identical to the batched solve over copies of the factor (the same
    kernels, with and without the quad-lane scratch), padding untouched, and
    every column a backward-stable solution of the dense system."""
    torch = torch_cuda
    rng = np.random.default_rng(23 + n + kl)
    nrhs, ldb = 37, n + 3
    band, ld = rand_band(rng, n, kl, ku)
    fe = lib.sgb_factor_elems(n, kl, ku)
    fdt = torch.complex128 if prec == "Z" else torch.complex64
    fac = torch.zeros(fe, dtype=fdt, device="cuda")
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    ab = dev(torch, band)
    assert lib.sgb_gbtrf_batched(prec.encode(), 1, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                 fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0) == 0
    B = rng.normal(size=(nrhs, ldb)) + 1j * rng.normal(size=(nrhs, ldb))
    db = dev(torch, B)
    facr, ipr = fac.repeat(nrhs), ipiv.repeat(nrhs)
    bb = db[:, :n].contiguous()
    A = oracle.band_to_dense(band, n, kl, ku, ld)
    op = A if trans == "N" else (A.T if trans == "T" else A.conj().T)
    for ws in (False, True):
        x = torch.full((nrhs, ldb), float("nan"), dtype=torch.complex128, device="cuda")
        yw = torch.zeros(nrhs * n, dtype=fdt, device="cuda") if ws else None
        rc = lib.sgb_gbtrs_shared(prec.encode(), trans.encode(), nrhs, n, kl, ku, fac.data_ptr(),
                                  ipiv.data_ptr(), db.data_ptr(), ldb, x.data_ptr(), ldb,
                                  yw.data_ptr() if ws else None, 0)
        assert rc == 0, lib.sgb_last_error().decode()
        xr = torch.zeros_like(bb)
        if ws:
            ywr = torch.zeros(nrhs * n, dtype=fdt, device="cuda")
            rc = lib.sgb_gbtrs_batched_ws(prec.encode(), trans.encode(), nrhs, n, kl, ku,
                                          facr.data_ptr(), ipr.data_ptr(), bb.data_ptr(),
                                          xr.data_ptr(), ywr.data_ptr(), 0)
        else:
            rc = lib.sgb_gbtrs_batched(prec.encode(), trans.encode(), nrhs, n, kl, ku,
                                       facr.data_ptr(), ipr.data_ptr(), bb.data_ptr(),
                                       xr.data_ptr(), 0)
        assert rc == 0, lib.sgb_last_error().decode()
        torch.cuda.synchronize()
        xh, xrh = x.cpu().numpy(), xr.cpu().numpy()
        assert np.array_equal(xh[:, :n].view(np.float64), xrh.view(np.float64)), ws
        assert np.isnan(xh[:, n:].real).all() and (xh[:, n:].imag == 0).all()   # fill untouched
        for r in range(nrhs):
            berr = np.max(np.abs(op @ xh[r, :n] - B[r, :n])) / (
                np.abs(op).sum(1).max() * np.abs(xh[r, :n]).max() + np.abs(B[r, :n]).max())
            assert berr <= (1e-14 if prec == "Z" else 1e-5), (ws, r, berr)


@pytest.mark.parametrize("n,kl,ku", [(1, 0, 0), (7, 0, 3), (13, 12, 0), (40, 3, 5),
                                     (240, 34, 34), (97, 48, 48), (50, 33, 40)])
@pytest.mark.parametrize("prec", ["Z", "C"])
def test_gbtrs_quad_path(lib, oracle, torch_cuda, n, kl, ku, prec):
    """The four-lanes-per-system solve (enabled by caller scratch) against the
    one-warp solve and the dense backward error, with a batch that leaves the
    last warp's eight-system group partly empty; b and x alias."""
    torch = torch_cuda
    rng = np.random.default_rng(11 + n + kl)
    nsys = 13
    ld = kl + ku + 1
    bands = [rand_band(rng, n, kl, ku)[0] for _ in range(nsys)]
    b = rng.normal(size=(nsys, n)) + 1j * rng.normal(size=(nsys, n))
    ab = dev(torch, np.stack(bands))
    fe = lib.sgb_factor_elems(n, kl, ku)
    fdt = torch.complex128 if prec == "Z" else torch.complex64
    fac = torch.zeros(nsys * fe, dtype=fdt, device="cuda")
    ipiv = torch.zeros(nsys * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
    assert lib.sgb_gbtrf_batched(prec.encode(), nsys, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                 fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0) == 0
    x1 = dev(torch, b)
    assert lib.sgb_gbtrs_batched(prec.encode(), b"N", nsys, n, kl, ku, fac.data_ptr(),
                                 ipiv.data_ptr(), x1.data_ptr(), x1.data_ptr(), 0) == 0
    x2 = dev(torch, b)
    yw = torch.full((nsys * n,), float("nan"), dtype=fdt, device="cuda")
    assert lib.sgb_gbtrs_batched_ws(prec.encode(), b"N", nsys, n, kl, ku, fac.data_ptr(),
                                    ipiv.data_ptr(), x2.data_ptr(), x2.data_ptr(),
                                    yw.data_ptr(), 0) == 0, lib.sgb_last_error().decode()
    torch.cuda.synchronize()
    x1, x2 = x1.cpu().numpy(), x2.cpu().numpy()
    for s in range(nsys):
        A = oracle.band_to_dense(bands[s], n, kl, ku, ld)
        scale = np.abs(A).sum(1).max() * np.abs(x2[s]).max() + np.abs(b[s]).max()
        berr = np.max(np.abs(A @ x2[s] - b[s])) / scale
        assert berr <= (1e-14 if prec == "Z" else 1e-5), (s, berr)
        # the same factor and the same forward sweep: only the dot products'
        # summation order differs from the one-warp solve
        d = np.max(np.abs(x2[s] - x1[s])) / np.abs(x1[s]).max()
        assert d <= (1e-9 if prec == "Z" else 1e-2), (s, d)


@pytest.mark.parametrize("n,kl,ku", [(7, 0, 3), (240, 34, 34), (97, 48, 48)])
def test_gbtrs_quad_depth_does_not_change_results(lib, torch_cuda, n, kl, ku):
    """Every prefetch depth of the quad solves gives the same bits."""
    torch = torch_cuda
    rng = np.random.default_rng(5 + n)
    nsys, ld = 21, kl + ku + 1
    bands = [rand_band(rng, n, kl, ku)[0] for _ in range(nsys)]
    b = rng.normal(size=(nsys, n)) + 1j * rng.normal(size=(nsys, n))
    ab = dev(torch, np.stack(bands))
    fe = lib.sgb_factor_elems(n, kl, ku)
    assert lib.sgb_gbtrs_set_quad_depth(3, 0) == -1
    try:
        for prec, fdt in (("Z", torch.complex128), ("C", torch.complex64)):
            fac = torch.zeros(nsys * fe, dtype=fdt, device="cuda")
            ipiv = torch.zeros(nsys * n, dtype=torch.int32, device="cuda")
            info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
            assert lib.sgb_gbtrf_batched(prec.encode(), nsys, n, kl, ku, ab.data_ptr(), ld,
                                         ld * n, fac.data_ptr(), ipiv.data_ptr(),
                                         info.data_ptr(), 0) == 0
            outs = []
            for f, bk in [(2, 2), (8, 4), (4, 8), (16, 16)]:
                assert lib.sgb_gbtrs_set_quad_depth(f, bk) == 0
                x = dev(torch, b)
                yw = torch.zeros(nsys * n, dtype=fdt, device="cuda")
                assert lib.sgb_gbtrs_batched_ws(prec.encode(), b"N", nsys, n, kl, ku,
                                                fac.data_ptr(), ipiv.data_ptr(), x.data_ptr(),
                                                x.data_ptr(), yw.data_ptr(), 0) == 0
                torch.cuda.synchronize()
                outs.append(x.cpu().numpy())
            for o in outs[1:]:
                assert np.array_equal(o, outs[0]), prec
    finally:
        lib.sgb_gbtrs_set_quad_depth(2, 2)


def test_singular_and_nan_systems(lib, oracle, torch_cuda):
    torch = torch_cuda
    n, kl, ku = 30, 2, 3
    ld = kl + ku + 1
    rng = np.random.default_rng(11)
    bands = [rand_band(rng, n, kl, ku)[0] for _ in range(3)]
    j = 17
    for i in range(max(0, j - ku), min(n, j + kl + 1)):
        bands[1][ku + i - j + j * ld] = 0          # system 1: zero column 17
    ab = dev(torch, np.stack(bands))
    fe = lib.sgb_factor_elems(n, kl, ku)
    fac = torch.zeros(3 * fe, dtype=torch.complex128, device="cuda")
    ipiv = torch.zeros(3 * n, dtype=torch.int32, device="cuda")
    info = torch.zeros(3, dtype=torch.int32, device="cuda")
    assert lib.sgb_gbtrf_batched(b"Z", 3, n, kl, ku, ab.data_ptr(), ld, ld * n,
                                 fac.data_ptr(), ipiv.data_ptr(), info.data_ptr(), 0) == 0
    torch.cuda.synchronize()
    assert info.cpu().tolist() == [0, j + 1, 0]


def _zcgbsvx_batch(lib, torch, bands, b, n, kl, ku, spec, trans="N"):
    nsys = len(bands)
    ld = kl + ku + 1
    ab = dev(torch, np.stack(bands))
    db = dev(torch, b)
    x = torch.zeros_like(db)
    rep = {k: torch.zeros(nsys, dtype=t, device="cuda") for k, t in
           (("info", torch.int32), ("siter", torch.int32), ("diter", torch.int32),
            ("res", torch.float64), ("tolsc", torch.float64), ("fact", torch.uint8))}
    from suzerain_gb300 import _native as nat
    R = nat.RefineReport(*(rep[k].data_ptr() for k in ("info", "siter", "diter", "res", "tolsc", "fact")))
    S = nat.RefineSpec(*spec)
    assert lib.sgb_zcgbsvx_batched(nsys, n, kl, ku, trans.encode(), ab.data_ptr(), ld, ld * n,
                                   db.data_ptr(), x.data_ptr(), C.byref(S), C.byref(R), 0) == 0, \
        lib.sgb_last_error().decode()
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in rep.items()}
    out["x"] = x.cpu().numpy()
    return out


@pytest.mark.parametrize("n,kl,ku", [(60, 5, 4), (240, 34, 34)])
def test_zcgbsvx_batched_matches_oracle(lib, oracle, torch_cuda, n, kl, ku):
    torch = torch_cuda
    rng = np.random.default_rng(21)
    nsys = 6
    bands = []
    for s in range(nsys):
        ab, ld = rand_band(rng, n, kl, ku)
        # diagonally weighted so complex64 refinement converges
        for j in range(n):
            ab[ku + j * ld] += 4 * (kl + ku + 1)
        bands.append(ab)
    b = rng.normal(size=(nsys, n)) + 1j * rng.normal(size=(nsys, n))
    spec = (5, 25, 5, 1.0)
    g = _zcgbsvx_batch(lib, torch, bands, b, n, kl, ku, spec)
    for s in range(nsys):
        o = oracle.zcgbsvx(bands[s], n, kl, ku, b[s], aiter=5, siter=25, diter=5, tolsc=1.0)
        assert g["info"][s] == o["info"] == 0
        assert chr(g["fact"][s]) == o["fact"] == "S"
        assert abs(int(g["siter"][s]) - o["siter"]) <= 1
        assert g["tolsc"][s] <= 1.0
        A = oracle.band_to_dense(bands[s], n, kl, ku, kl + ku + 1)
        xref = np.linalg.solve(A, b[s])
        assert np.max(np.abs(g["x"][s] - xref)) <= 1e-11 * np.max(np.abs(xref))


def test_zcgbsvx_batched_fallback_to_double(lib, oracle, torch_cuda):
    """An ill-conditioned (Lotkin) system stalls in complex64 and must finish
    on the complex128 factor, matching the oracle's fact/diter decisions."""
    torch = torch_cuda
    n = 10
    A = np.array([[1.0 if i == 0 else 1.0 / (i + j + 1) for j in range(n)] for i in range(n)]) * (1 + 0.5j)
    kl = ku = n - 1
    ld = kl + ku + 1
    ab = np.zeros(ld * n, dtype=np.complex128)
    for j in range(n):
        for i in range(n):
            ab[ku + i - j + j * ld] = A[i, j]
    xt = np.ones(n, dtype=np.complex128)
    b = (A @ xt)[None, :]
    good = np.zeros(ld * n, dtype=np.complex128)
    for j in range(n):
        good[ku + j * ld] = 2.0 + 0.1 * j
    bg = (np.ones(n) * 3.0 + 0j)[None, :]
    g = _zcgbsvx_batch(lib, torch, [ab, good], np.vstack([b, bg]), n, kl, ku, (5, 25, 10, 1.0))
    o = oracle.zcgbsvx(ab, n, kl, ku, b[0], aiter=5, siter=25, diter=10, tolsc=1.0)
    assert chr(g["fact"][0]) == o["fact"] == "D"
    # cond(Lotkin_10) ~ 1e13: FMA rounding can move res across tol by one step
    assert abs(int(g["diter"][0]) - o["diter"]) <= 1
    assert g["tolsc"][0] <= 1.0 and g["info"][0] == 0
    assert np.linalg.norm(A @ g["x"][0] - b[0]) <= 10 * g["res"][0] + 1e-30
    assert chr(g["fact"][1]) == "S" and g["info"][1] == 0


# ---------------------------------------------------------------------------
# Synthetic substep through the plan
# ---------------------------------------------------------------------------
def config0(complex_coupling=False):
    from suzerain_gb300 import synth
    c = synth.CONFIGS[0]
    cs, kx, kz, u = c.batch(complex_coupling)
    synth.zero_dirichlet_rows(cs, u)
    return c, cs, kx, kz, u


def forward_tolerance(oracle, cs, kx, kz, phi_imp, eps=2.220446049250313e-16):
    """Per-system bound on the forward difference of two backward-stable
    solvers: max(1e-11, 8 kappa_inf(A) eps).  The synthetic operators are
    ill-conditioned (kappa ~ 1e7), so the reference's own LAPACK builds
    differ from each other by ~1e-9 on them; well-conditioned systems keep
    the 1e-11 bar (test_gbtrf_*, test_zcgbsvx_batched_matches_oracle)."""
    tol = np.empty(len(kx))
    for s in range(len(kx)):
        A = oracle.band_to_dense(oracle.assemble_case(cs, phi_imp, kx[s], kz[s]), cs.N,
                                 cs.KL, cs.KU, cs.LD)
        tol[s] = max(1e-11, 8 * np.linalg.cond(A, np.inf) * eps)
    return tol


@pytest.mark.parametrize("complex_coupling", [False, True])
@pytest.mark.parametrize("explicit", [False, True])
def test_plan_plain_fp64_matches_oracle(lib, oracle, torch_cuda, complex_coupling, explicit):
    torch = torch_cuda
    from suzerain_gb300 import plan as P, synth
    c, cs, kx, kz, u = config0(complex_coupling)
    phi_e, phi_i = synth.smr91_phis(c.phi, explicit=explicit)
    pl = P.Plan(cs, kx, kz)
    du = dev(torch, u)
    out = torch.zeros_like(du)
    pl.substep("Z", phi_e, phi_i, du, out)
    torch.cuda.synchronize()
    x = out.cpu().numpy()
    rep = pl.report()
    berr = pl.backward_error()
    o = oracle.batch_solve(cs, kx, kz, u, phi_exp=phi_e, phi_imp=phi_i, nthreads=8)
    assert (rep["info"] == o["info"]).all() and (o["info"] == 0).all()
    assert berr.max() <= 1e-13, berr.max()
    rel = np.max(np.abs(x - o["x"]), axis=1) / np.max(np.abs(o["x"]), axis=1)
    tol = forward_tolerance(oracle, cs, kx, kz, phi_i)
    assert (rel <= tol).all(), (rel / tol).max()


@pytest.mark.parametrize("complex_coupling", [False, True])
def test_plan_mixed_matches_oracle(lib, oracle, torch_cuda, complex_coupling):
    torch = torch_cuda
    from suzerain_gb300 import plan as P, synth
    c, cs, kx, kz, u = config0(complex_coupling)
    phi_e, phi_i = synth.smr91_phis(c.phi)
    pl = P.Plan(cs, kx, kz)
    du = dev(torch, u)
    out = torch.zeros_like(du)
    spec = P.RefineSpec(aiter=5, siter=25, diter=5, tolsc=145.0)
    pl.substep("M", phi_e, phi_i, du, out, spec)
    torch.cuda.synchronize()
    x = out.cpu().numpy()
    rep = pl.report()
    berr = pl.backward_error()
    o = oracle.batch_solve(cs, kx, kz, u, phi_exp=phi_e, phi_imp=phi_i, nthreads=8)
    om = oracle.batch_solve(cs, kx, kz, u, phi_exp=phi_e, phi_imp=phi_i, mixed=True,
                            tolsc=145.0, nthreads=8)
    assert (rep["info"] == 0).all()
    assert berr.max() <= 1e-12, berr.max()
    assert (rep["tolsc"] <= 1.0).all()
    rel = np.max(np.abs(x - o["x"]), axis=1) / np.max(np.abs(o["x"]), axis=1)
    tol = forward_tolerance(oracle, cs, kx, kz, phi_i)
    assert (rel <= 10 * tol).all(), (rel / tol).max()
    # the same convergence decisions as the reference algorithm, per system
    assert set(rep["fact"]) <= {"S", "D"}
    agree = np.mean(np.abs(rep["siter"] - om["siter"]) <= 1)
    assert agree >= 0.95, agree


def test_plan_mixed_fallback_at_scale(lib, oracle, torch_cuda):
    """Walls on the momentum equations only leave two second-order equations
    without boundary rows (kappa up to 1e8 at Ny=48): complex64 refinement
    stalls for many systems, which must finish on complex128 factors.  Few
    fallback slots force several chunks."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P, synth
    c = synth.Config(**{**synth.CONFIGS[0].__dict__, "dirichlet_mask": synth.DIRICHLET_MOMENTUM})
    cs, kx, kz, u = c.batch()
    synth.zero_dirichlet_rows(cs, u)
    phi_e, phi_i = synth.smr91_phis(c.phi)
    pl = P.Plan(cs, kx, kz, max_double_slots=17)
    out = torch.zeros(u.shape, dtype=torch.complex128, device="cuda")
    pl.substep("M", phi_e, phi_i, dev(torch, u), out, P.RefineSpec(aiter=5, siter=25, diter=5, tolsc=145.0))
    torch.cuda.synchronize()
    rep = pl.report()
    berr = pl.backward_error()
    om = oracle.batch_solve(cs, kx, kz, u, phi_exp=phi_e, phi_imp=phi_i, mixed=True, tolsc=145.0,
                            nthreads=8)
    nd = sum(1 for f in rep["fact"] if f == "D")
    nd_o = sum(1 for f in om["fact"] if f == "D")
    assert nd >= 17 and abs(nd - nd_o) <= 0.1 * len(kx), (nd, nd_o)
    assert (rep["info"] == 0).all()
    assert berr.max() <= 1e-12, berr.max()


def test_plan_result_independent_of_batch(lib, torch_cuda):
    """A system's result does not depend on which other systems share the batch."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P
    c, cs, kx, kz, u = config0()
    full = P.Plan(cs, kx, kz)
    sub_idx = np.array([3, 77, 200, 311])
    part = P.Plan(cs, kx[sub_idx], kz[sub_idx])
    for method in ("Z", "M"):
        a = torch.zeros(u.shape, dtype=torch.complex128, device="cuda")
        b = torch.zeros((len(sub_idx), u.shape[1]), dtype=torch.complex128, device="cuda")
        full.substep(method, 0.0, -c.phi, dev(torch, u), a, P.RefineSpec(tolsc=145.0))
        part.substep(method, 0.0, -c.phi, dev(torch, u[sub_idx]), b, P.RefineSpec(tolsc=145.0))
        torch.cuda.synchronize()
        assert np.array_equal(a.cpu().numpy()[sub_idx], b.cpu().numpy())


def test_plan_result_independent_of_factor_shape(lib, torch_cuda):
    """The plan assembles its bands inside the factor kernel; every blocked
    shape (panel width, warps per system) and the unblocked kernel give the
    same bits, in complex128 and through the complex64 refinement."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P
    c, cs, kx, kz, u = config0()
    sel = np.arange(0, len(kx), 7)
    kx, kz, u = kx[sel], kz[sel], u[sel]
    N, KL, KU = cs.N, cs.KL, cs.KU
    saved = {}
    for prec in (b"Z", b"C"):
        nb, nw = C.c_int(), C.c_int()
        lib.sgb_gbtrf_get_shape(prec, N, KL, KU, C.byref(nb), C.byref(nw))
        saved[prec] = (nb.value, nw.value)
    results = []
    try:
        for nb, nw in [(4, 1), (8, 2), (16, 4), (8, 1), (4, 4), (16, 2)]:
            for prec in (b"Z", b"C"):
                assert lib.sgb_gbtrf_set_shape(prec, N, KL, KU, nb, nw) == 0
            pl = P.Plan(cs, kx, kz)
            row = []
            for method in ("Z", "M"):
                a = torch.zeros(u.shape, dtype=torch.complex128, device="cuda")
                pl.substep(method, 0.0, -c.phi, dev(torch, u), a, P.RefineSpec(tolsc=145.0))
                torch.cuda.synchronize()
                row.append(a.cpu().numpy())
            results.append(row)
    finally:
        for prec, (nb, nw) in saved.items():
            lib.sgb_gbtrf_set_shape(prec, N, KL, KU, nb, nw)
    for row in results[1:]:
        for m in range(2):
            assert np.array_equal(row[m], results[0][m])


@pytest.mark.parametrize("config", [0, 2])
def test_quad_solve_bulk_copies_match_cp_async(lib, torch_cuda, config):
    """The backward quad solve fetching records of 2, 4 or 8 factor rows by
    one bulk copy (TMA) per system gives the bits of the one-row 16-byte
    cp.async form, for both methods and both precisions' factors
    (configuration 0's geometry and a 512-system sample of configuration 2),
    and records no wait time-out."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P, synth
    if config == 0:
        c, cs, kx, kz, u = config0()
    else:
        c = synth.CONFIGS[2]
        cs, kx, kz, u = c.batch()
        kx, kz, u = kx[:512], kz[:512], u[:512]
    assert lib.sgb_async_faults() == 0
    out = {}
    try:
        for bulk in (1, 2, 4, 8):
            assert lib.sgb_gbtrs_set_quad_bulk(bulk) == 0
            pl = P.Plan(cs, kx, kz)
            for method in ("Z", "M"):
                a = torch.zeros(u.shape, dtype=torch.complex128, device="cuda")
                pl.substep(method, 0.0, -c.phi, dev(torch, u), a, P.RefineSpec(tolsc=145.0))
                b = torch.zeros_like(a)
                pl.substep_capturable(method, 0.0, -c.phi, dev(torch, u), b, P.RefineSpec(tolsc=145.0))
                torch.cuda.synchronize()
                out[(bulk, method)] = (a.cpu().numpy(), b.cpu().numpy())
            pl.close()
    finally:
        lib.sgb_gbtrs_set_quad_bulk(2)
    assert lib.sgb_async_faults() == 0
    for bulk in (2, 4, 8):
        for method in ("Z", "M"):
            for i in range(2):
                assert np.array_equal(out[(bulk, method)][i], out[(1, method)][i]), (bulk, method)
    assert lib.sgb_gbtrs_set_quad_bulk(3) != 0


def test_plan_memory_reuse_waits_for_issued_work(lib, torch_cuda):
    """Plans take device memory from a pool that keeps freed blocks.  A plan
    destroyed right after issuing a substep on a side stream must not hand
    its blocks to the next plan before that substep completes: the results
    equal a synchronised run, and the next plan (same sizes, so it reuses
    the blocks) computes its own correctly."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P
    c, cs, kx, kz, u = config0()
    spec = P.RefineSpec(tolsc=145.0)
    du = dev(torch, u)
    ref = torch.zeros_like(du)
    pl = P.Plan(cs, kx, kz)
    pl.prepare("M")
    pl.substep_capturable("M", 0.0, -c.phi, du, ref, spec)
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    pl.close()
    side = torch.cuda.Stream()
    outs = []
    for rep in range(3):
        out = torch.zeros_like(du)
        pl = P.Plan(cs, kx, kz)
        pl.prepare("M")
        with torch.cuda.stream(side):
            pl.substep_capturable("M", 0.0, -c.phi, du, out, spec, stream=side.cuda_stream)
        pl.close()                      # no synchronisation before the destroy
        outs.append(out)
    torch.cuda.synchronize()
    for out in outs:
        assert np.array_equal(out.cpu().numpy(), want)
    assert lib.sgb_plan_pool_trim(0) == 0


def test_batch_plan_parts_match_one_plan(lib, torch_cuda):
    """A batch split into resident plans on their own streams gives the same
    bits as one plan over the batch (capturable substeps both)."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P
    c, cs, kx, kz, u = config0()
    spec = P.RefineSpec(aiter=5, siter=25, diter=5, tolsc=145.0)
    du = dev(torch, u)
    one = P.Plan(cs, kx, kz, max_double_slots=64)
    one.prepare("M")
    want = torch.zeros_like(du)
    one.substep_capturable("M", 0.0, -c.phi, du, want, spec)
    torch.cuda.synchronize()
    one.close()
    bp = P.BatchPlan(cs, kx, kz, parts=3, max_double_slots=66)
    got = torch.zeros_like(du)
    bp.substep("M", 0.0, -c.phi, du, got, spec)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), want.cpu().numpy())
    assert bp.unserved() == 0
    rep = bp.report()
    assert (rep["info"] == 0).all() and len(rep["fact"]) == len(kx)
    assert bp.backward_error().max() <= 1e-12
    bp.close()


def test_plan_host_entry_matches_device_entry(lib, torch_cuda):
    torch = torch_cuda
    from suzerain_gb300 import plan as P
    c, cs, kx, kz, u = config0()
    pl = P.Plan(cs, kx, kz)
    a = torch.zeros(u.shape, dtype=torch.complex128, device="cuda")
    pl.substep("M", 0.0, -c.phi, dev(torch, u), a, P.RefineSpec(tolsc=145.0))
    torch.cuda.synchronize()
    h = np.zeros_like(u)
    pl.substep_host("M", 0.0, -c.phi, u, h, P.RefineSpec(tolsc=145.0))
    assert np.array_equal(a.cpu().numpy(), h)


# ---------------------------------------------------------------------------
# Drop-in entry points
# ---------------------------------------------------------------------------
def test_dropin_kat_solve(lib, oracle):
    """tests/test_bsmbsm.cpp:801-872 through the GPU drop-ins: zdpackf/zpackf,
    zaPxpby, zgbsv, unpermute."""
    from suzerain_gb300 import _native as nat
    d = json.load(open(os.path.join(GOLD, "bsmbsm_kat.json")))
    A = lib.suzerain_bsmbsm_construct(d["S"], d["n"], d["kl"], d["ku"])
    papt = np.full((A.LD + A.KL) * A.N, np.nan, dtype=np.complex128)
    for ih, row in enumerate(d["blocks"]):
        for jh, blk in enumerate(row):
            if blk is None:
                rc = lib.suzerain_bsmbsm_zpackf(C.byref(A), ih, jh, nat.zc(0), None, papt.ctypes.data)
            else:
                b = np.array(d[blk[0]]) * blk[1]
                rc = lib.suzerain_bsmbsm_zdpackf(C.byref(A), ih, jh, nat.zc(1), b.ctypes.data, papt.ctypes.data)
            assert rc == 0, lib.sgb_last_error().decode()
    br = np.array(d["BR"], dtype=np.complex128)
    pb = np.zeros(A.N, dtype=np.complex128)
    assert lib.suzerain_bsmbsm_zaPxpby(b"N", A.S, A.n, nat.zc(1), br.ctypes.data, 1, nat.zc(0), pb.ctypes.data, 1) == 0
    ipiv = np.zeros(A.N, np.int32)
    fact = C.create_string_buffer(b"N", 1)
    assert lib.suzerain_lapackext_zgbsv(C.addressof(fact), b"N", A.N, A.KL, A.KU, 1, papt.ctypes.data,
                                        A.LD + A.KL, ipiv.ctypes.data, pb.ctypes.data, A.N) == 0
    assert fact.raw == b"F"
    x = np.zeros(A.N, dtype=np.complex128)
    assert lib.suzerain_bsmbsm_zaPxpby(b"T", A.S, A.n, nat.zc(1), pb.ctypes.data, 1, nat.zc(0), x.ctypes.data, 1) == 0
    xr = np.array(d["XR"])
    tol = np.finfo(float).eps * d["tolerance_eps_multiple"]
    assert np.allclose(x.real, xr, rtol=tol, atol=tol * np.abs(xr).max())


def test_dropin_pack_and_aPxpby_match_oracle(lib, oracle):
    from suzerain_gb300 import _native as nat
    rng = np.random.default_rng(5)
    for (S, n, kl, ku) in [(1, 10, 2, 3), (3, 17, 4, 3), (5, 12, 6, 6)]:
        g = oracle.bsmbsm(S, n, kl, ku)
        b = rng.normal(size=g["ld"] * n) + 1j * rng.normal(size=g["ld"] * n)
        p1 = np.full(g["LD"] * g["N"], np.nan, dtype=np.complex128)
        p2 = p1.copy()
        for ih in range(S):
            for jh in range(S):
                al = complex(ih + 2, jh - 1)
                assert lib.suzerain_bsmbsm_zpack(S, n, ih, jh, kl, ku, nat.zc(al), b.ctypes.data, g["ld"],
                                                 g["KL"], g["KU"], p1.ctypes.data, g["LD"]) == 0
                oracle.lib().orc_zpack(S, n, ih, jh, kl, ku, oracle._z(al), b.ctypes.data, g["ld"],
                                       g["KL"], g["KU"], p2.ctypes.data, g["LD"])
        assert np.array_equal(np.isnan(p1), np.isnan(p2))
        m = ~np.isnan(p1)
        assert np.allclose(p1[m], p2[m], rtol=4e-16, atol=0)
        for trans in "NT":
            for incx, incy in ((1, 1), (-2, 3), (2, -1)):
                N = S * n
                x = rng.normal(size=N * abs(incx)) + 1j * rng.normal(size=N * abs(incx))
                y = rng.normal(size=N * abs(incy)) + 1j * rng.normal(size=N * abs(incy))
                y1, y2 = y.copy(), y.copy()
                assert lib.suzerain_bsmbsm_zaPxpby(trans.encode(), S, n, nat.zc(3 - 1j), x.ctypes.data, incx,
                                                   nat.zc(0.5j), y1.ctypes.data, incy) == 0
                oracle.zaPxpby(trans, S, n, 3 - 1j, x, incx, 0.5j, y2, incy)
                assert np.allclose(y1, y2, rtol=4 * np.finfo(float).eps, atol=1e-14)
    # argument checks in the reference's order: S, n, aliasing, then trans
    xa, ya = np.zeros(4, complex), np.zeros(4, complex)
    assert lib.suzerain_bsmbsm_zaPxpby(b"X", 2, 2, nat.zc(1), xa.ctypes.data, 1, nat.zc(0), ya.ctypes.data, 1) == 1
    assert lib.suzerain_bsmbsm_zaPxpby(b"N", 2, 2, nat.zc(1), xa.ctypes.data, 1, nat.zc(0), xa.ctypes.data, 1) == 58
    assert lib.suzerain_bsmbsm_zaPxpby(b"N", -1, 2, nat.zc(1), xa.ctypes.data, 1, nat.zc(0), ya.ctypes.data, 1) == 2


def test_dropin_zcgbsvx_lotkin(lib, oracle):
    from suzerain_gb300 import _native as nat
    for n in (4, 8, 12):
        A = np.array([[1.0 if i == 0 else 1.0 / (i + j + 1) for j in range(n)] for i in range(n)]) * (1 - 0.25j)
        kl = ku = n - 1
        ld = kl + ku + 1
        ab = np.zeros(ld * n, dtype=np.complex128)
        for j in range(n):
            for i in range(n):
                ab[ku + i - j + j * ld] = A[i, j]
        b = A @ np.ones(n)
        o = oracle.zcgbsvx(ab, n, kl, ku, b, aiter=5, siter=25, diter=10, tolsc=1.0)
        fact = C.create_string_buffer(b"N", 1)
        apprx, afrob = C.c_int(0), C.c_double(-1)
        afb = np.zeros((2 * kl + ku + 1) * n, dtype=np.complex128)
        ipiv = np.zeros(n, np.int32)
        x = np.zeros(n, dtype=np.complex128)
        r = np.zeros(n, dtype=np.complex128)
        si, di, ts, res = C.c_int(25), C.c_int(10), C.c_double(1.0), C.c_double(0)
        info = lib.suzerain_lapackext_zcgbsvx(C.addressof(fact), C.addressof(apprx), 5, b"N", n, kl, ku,
                                              ab.ctypes.data, C.addressof(afrob), afb.ctypes.data,
                                              ipiv.ctypes.data, b.ctypes.data, x.ctypes.data,
                                              C.addressof(si), C.addressof(di), C.addressof(ts),
                                              r.ctypes.data, C.addressof(res))
        assert info == o["info"] == 0
        assert fact.raw.decode() == o["fact"]
        assert ts.value <= 1.0
        assert np.linalg.norm(A @ x - b) <= 10 * res.value + 1e-30
        assert np.allclose(r, b - A @ x, rtol=0, atol=1e-12 * np.abs(b).max())
        assert abs(afrob.value - o["afrob"]) <= 1e-12 * o["afrob"]


def test_dropin_gbtrf_gbtrs_lapack_layout(lib, oracle):
    n, kl, ku = 50, 6, 4
    rng = np.random.default_rng(9)
    ldab = 2 * kl + ku + 1
    ab = np.zeros(ldab * n, dtype=np.complex128)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[kl + ku + i - j + j * ldab] = complex(rng.normal(), rng.normal())
    a1, a2 = ab.copy(), ab.copy()
    p1 = np.zeros(n, np.int32)
    assert lib.suzerain_lapack_zgbtrf(n, n, kl, ku, a1.ctypes.data, ldab, p1.ctypes.data) == 0
    info, p2 = oracle.zgbtrf(a2, n, kl, ku, ldab)
    assert np.array_equal(p1, p2)
    assert np.max(np.abs(a1 - a2)) <= 1e-12 * np.abs(a2).max()
    for tr in "NTC":
        b = rng.normal(size=(n, 2)) + 1j * rng.normal(size=(n, 2))
        x1 = np.asfortranarray(b.copy())
        assert lib.suzerain_lapack_zgbtrs(tr.encode(), n, kl, ku, 2, a1.ctypes.data, ldab, p1.ctypes.data,
                                          x1.ctypes.data, n) == 0
        x2 = b.copy()
        oracle.zgbtrs(tr, a2, n, kl, ku, ldab, p2, x2)
        assert np.allclose(x1, x2, rtol=1e-11, atol=1e-12)


def test_dropin_gbmv_and_diffwave(lib, oracle):
    from suzerain_gb300 import _native as nat
    rng = np.random.default_rng(13)
    for tr in "NTC":
        m, n, kl, ku = 30, 30, 3, 5
        lda = kl + ku + 2
        a = rng.normal(size=lda * n) + 1j * rng.normal(size=lda * n)
        x = rng.normal(size=n) + 1j * rng.normal(size=n)
        y = rng.normal(size=m) + 1j * rng.normal(size=m)
        y1, y2 = y.copy(), y.copy()
        assert lib.suzerain_blas_zgbmv(tr.encode(), m, n, kl, ku, nat.zc(2 - 1j), a.ctypes.data, lda,
                                       x.ctypes.data, 1, nat.zc(0.5), y1.ctypes.data, 1) == 0
        oracle.zgbmv(tr, m, n, kl, ku, 2 - 1j, a, lda, x, 0.5, y2)
        assert np.allclose(y1, y2, rtol=1e-13, atol=1e-13)
    # diffwave: x <- alpha (i kx)^dx (i kz)^dz x on (Ny, Nx, Nz), dealiased
    Ny, Nx, Nz, dNx, dNz = 4, 8, 6, 12, 9
    Lx, Lz = 4.0, 3.0
    for dx, dz in ((0, 0), (1, 0), (0, 2), (1, 1)):
        f = rng.normal(size=(dNz, dNx, Ny)) + 1j * rng.normal(size=(dNz, dNx, Ny))
        g = f.copy()
        assert lib.suzerain_diffwave_apply(dx, dz, nat.zc(1.5 - 0.5j), g.ctypes.data, Lx, Lz, Ny, Nx, dNx,
                                           0, dNx, Nz, dNz, 0, dNz) == 0
        def keep_diff(N, dN, i):
            return i if i < (N + 1) // 2 else (-dN + i if i >= dN - (N - 1) // 2 else 0)
        def wabs(N, i):
            return i if i < N // 2 + 1 else N - i
        exp = np.zeros_like(f)
        for nz in range(dNz):
            for mx in range(dNx):
                nf = keep_diff(Nz, dNz, nz) if dz else None
                mf = keep_diff(Nx, dNx, mx) if dx else None
                nk = nf != 0 if dz else wabs(dNz, nz) <= (Nz - 1) // 2
                mk = mf != 0 if dx else wabs(dNx, mx) <= (Nx - 1) // 2
                if nk and mk:
                    sc = (1.5 - 0.5j) * (1j * 2 * np.pi / Lz * (nf or 0)) ** dz * (1j * 2 * np.pi / Lx * (mf or 0)) ** dx
                    exp[nz, mx] = f[nz, mx] * sc
        assert np.allclose(g, exp, rtol=1e-14, atol=1e-13)
        # accumulate: y <- alpha D x + beta y, y <- beta y where D zeroes the
        # mode; on a sub-block of modes (dkbx..dkex, dkbz..dkez)
        bx, ex, bz, ez = 1, dNx - 2, 2, dNz
        xs = np.ascontiguousarray(f[bz:ez, bx:ex])
        y0 = rng.normal(size=xs.shape) + 1j * rng.normal(size=xs.shape)
        y1 = y0.copy()
        assert lib.suzerain_diffwave_accumulate(dx, dz, nat.zc(1.5 - 0.5j), xs.ctypes.data,
                                                nat.zc(0.25 + 2j), y1.ctypes.data, Lx, Lz, Ny,
                                                Nx, dNx, bx, ex, Nz, dNz, bz, ez) == 0
        keep = (exp[bz:ez, bx:ex] != 0).any(axis=2)
        want = np.where(keep[..., None], exp[bz:ez, bx:ex], 0) + (0.25 + 2j) * y0
        assert np.allclose(y1, want, rtol=1e-14, atol=1e-13)
        assert lib.suzerain_diffwave_accumulate(dx, dz, nat.zc(1.0), y1.ctypes.data, nat.zc(1.0),
                                                y1.ctypes.data, Lx, Lz, Ny, Nx, dNx, bx, ex,
                                                Nz, dNz, bz, ez) == -1   # x, y alias


def _strided(v, inc):
    s = np.zeros((len(v) - 1) * abs(inc) + 1, dtype=v.dtype)
    s[::abs(inc)] = v if inc > 0 else v[::-1]
    return s


def _logical(s, n, inc):
    v = s[::abs(inc)][:n]
    return v if inc > 0 else v[::-1]


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("xreal", [False, True])
def test_dropin_blasext_gbdmv(lib, k, xreal):
    """y <- (sum alpha_t D_t) op(A) x + beta y against a dense evaluation, over
    trans N/T/C, strides of both signs, diagonal strides 0..3; beta = 0 clears
    NaN in y, all-zero alphas leave beta y; argument errors at the reference's
    positions (suzerain/blas_et_al/gbd*mv.def)."""
    from suzerain_gb300 import _native as nat
    name = {1: "zgbdmv", 2: "zgbddmv", 3: "zgbdddmv", 4: "zgbddddmv", 5: "zgbdddddmv"}[k]
    f = getattr(lib, f"suzerain_blasext_{name}_{'d_d' if xreal else 'd_z'}")
    rng = np.random.default_rng(31 + k + 7 * xreal)
    n, kl, ku = 37, 4, 3
    lda = kl + ku + 2
    a = rng.normal(size=lda * n)
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            A[i, j] = a[ku + i - j + j * lda]
    ldd = [1, 0, 2, 1, 3][:k]
    ds = [rng.normal(size=(n - 1) * l + 1) for l in ldd]

    def call(trans, alphas, x, incx, beta, y, incy, lda_=lda, ldd_=ldd):
        args = [trans.encode(), n, kl, ku]
        for al, d, l in zip(alphas, ds, ldd_):
            args += [nat.zc(al), d.ctypes.data, l]
        return f(*args, a.ctypes.data, lda_, x.ctypes.data, incx, nat.zc(beta), y.ctypes.data, incy)

    for trans, incx, incy in (("N", 1, 1), ("T", 2, -1), ("C", -1, 3), ("n", -2, 2)):
        alphas = [complex(rng.normal(), rng.normal()) for _ in range(k)]
        beta = 0.5 - 0.25j
        xl = rng.normal(size=n) if xreal else rng.normal(size=n) + 1j * rng.normal(size=n)
        yl = rng.normal(size=n) + 1j * rng.normal(size=n)
        xs, ys = _strided(xl, incx), _strided(yl, incy)
        if abs(incy) > 1:
            ys[np.arange(len(ys)) % abs(incy) != 0] = 7 + 7j    # gaps stay untouched
        ys0 = ys.copy()
        c = sum(al * d[np.arange(n) * l] for al, d, l in zip(alphas, ds, ldd))
        op = A if trans.upper() == "N" else A.T
        want = beta * yl + c * (op @ xl)
        assert call(trans, alphas, xs, incx, beta, ys, incy) == 0
        assert np.allclose(_logical(ys, n, incy), want, rtol=1e-13, atol=1e-13), trans
        gap = np.arange(len(ys)) % abs(incy) != 0
        assert np.array_equal(ys[gap], ys0[gap])
    xs = rng.normal(size=n) if xreal else rng.normal(size=n) + 1j * rng.normal(size=n)
    y = np.full(n, np.nan + 0j)
    assert call("N", [1.0] * k, xs, 1, 0.0, y, 1) == 0                 # beta = 0 clears y
    c = sum(d[np.arange(n) * l] for d, l in zip(ds, ldd))
    assert np.allclose(y, c * (A @ xs), rtol=1e-13, atol=1e-13)
    y0 = rng.normal(size=n) + 1j * rng.normal(size=n)
    y = y0.copy()
    xn = np.full(n, np.nan) if xreal else np.full(n, np.nan + 0j)
    assert call("T", [0.0] * k, xn, 1, 2.0, y, 1) == 0                  # alphas zero: beta y
    assert np.array_equal(y, 2.0 * y0)
    y = y0.copy()
    assert call("X", [1.0] * k, xs, 1, 1.0, y, 1) == 1
    assert call("N", [1.0] * k, xs, 1, 1.0, y, 1, ldd_=[-1] + ldd[1:]) == 7
    if k > 1:
        assert call("N", [1.0] * k, xs, 1, 1.0, y, 1, ldd_=ldd[:-1] + [-1]) == 7 + 3 * (k - 1)
    assert call("N", [1.0] * k, xs, 1, 1.0, y, 1, lda_=kl + ku) == 3 * k + 6
    assert call("N", [1.0] * k, xs, 0, 1.0, y, 1) == 3 * k + 8
    assert call("N", [1.0] * k, xs, 1, 1.0, y, 0) == (13 if k == 1 else 3 * k + 11)
    assert np.array_equal(y, y0)


def test_dropin_bsplineop_accumulate_golden(lib):
    from suzerain_gb300 import _native as nat
    d = json.load(open(os.path.join(GOLD, "bsplineop_kat.json")))
    bp = np.array(d["breakpoints"])
    w = lib.sgb_bsplineop_alloc_breakpoints(d["k"], len(bp), bp.ctypes.data, 1)
    try:
        x = np.array([complex(a, b) for a, b in d["apply_complex_x"]])
        y = np.zeros_like(x)
        assert lib.suzerain_bsplineop_accumulate_complex(0, 1, nat.zc(1), x.ctypes.data, 1, len(x),
                                                         nat.zc(0), y.ctypes.data, 1, len(x), w) == 0
        good = np.array([complex(a, b) for a, b in d["apply_complex_good"]])
        assert np.allclose(y, good, rtol=0, atol=1e-14)
    finally:
        lib.suzerain_bsplineop_free(w)


def test_tuner_records_a_supported_shape(lib, torch_cuda):
    """tune_packed times every candidate and records the fastest; the
    recorded shape is then what the batched factor uses by default."""
    from suzerain_gb300 import tune
    n, kl, ku = 120, 9, 9
    saved = tune.get_shape("C", n, kl, ku)
    try:
        res = tune.tune_packed("C", n, kl, ku, nsys=64, reps=1)
        best = res["best"]
        assert best in res and all(v > 0 for k, v in res.items() if k != "best")
        assert tune.get_shape("C", n, kl, ku) == best
    finally:
        tune.set_shape("C", n, kl, ku, *saved)


def _three_substeps(plan_fn, phis, du, spec):
    """SMR91 substeps 0, 1, 2 in sequence through plan_fn(phi_e, phi_i, u_in, u_out)."""
    import torch
    a = du
    outs = []
    for phi_e, phi_i in phis:
        b = torch.empty_like(a)
        plan_fn(phi_e, phi_i, a, b)
        outs.append(b)
        a = b
    return outs


def test_plan_three_substeps_in_a_cuda_graph(lib, torch_cuda):
    """Three SMR91 substeps recorded into one CUDA graph give the same bits
    as the ordinary host-driven substeps (the device-counted refinement
    makes the same decisions)."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P, synth
    c, cs, kx, kz, u = config0()
    spec = P.RefineSpec(aiter=5, siter=25, diter=5, tolsc=145.0)
    dt_beta = c.phi
    phis = [synth.smr91_phis(dt_beta * synth.SMR91_BETA[i] / synth.SMR91_BETA[0], substep=i)
            for i in range(3)]
    pl = P.Plan(cs, kx, kz)
    du = dev(torch, u)
    ref = _three_substeps(lambda pe, pi, a, b: pl.substep("M", pe, pi, a, b, spec), phis, du, spec)
    torch.cuda.synchronize()
    ref = [r.cpu().numpy() for r in ref]
    # capture
    static_in = du.clone()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        pl.substep("M", phis[0][0], phis[0][1], static_in, torch.empty_like(du), spec, stream=s.cuda_stream)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    bufs = [torch.empty_like(du) for _ in range(3)]
    with torch.cuda.graph(g):
        st = torch.cuda.current_stream().cuda_stream
        a = static_in
        for (pe, pi), b in zip(phis, bufs):
            pl.substep_capturable("M", pe, pi, a, b, spec, stream=st)
            a = b
    static_in.copy_(du)
    g.replay()
    torch.cuda.synchronize()
    for k in range(3):
        assert np.array_equal(bufs[k].cpu().numpy(), ref[k]), k
    assert pl.unserved() == 0
    # a second replay from the same input reproduces the result
    g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(bufs[2].cpu().numpy(), ref[2])


@pytest.mark.parametrize("siter", [3, 25])
def test_plan_capturable_fallback_matches_host_driven(lib, oracle, torch_cuda, siter):
    """The stress mask (walls on momentum only) makes complex64 refinement
    slow (up to ~10 solves) and sends many systems to the complex128
    fallback: the capturable form, with enough fallback slots, runs the same
    decisions as the host-driven one (the reference's siter + 1 and
    diter + 2 bounds), so fact, siter and the solution are identical."""
    torch = torch_cuda
    from suzerain_gb300 import plan as P, synth
    c = synth.Config(**{**synth.CONFIGS[0].__dict__, "dirichlet_mask": synth.DIRICHLET_MOMENTUM})
    cs, kx, kz, u = c.batch()
    synth.zero_dirichlet_rows(cs, u)
    phi_e, phi_i = synth.smr91_phis(c.phi)
    spec = P.RefineSpec(aiter=5, siter=siter, diter=5, tolsc=145.0)
    pl = P.Plan(cs, kx, kz, max_double_slots=len(kx))
    du = dev(torch, u)
    a = torch.zeros_like(du)
    b = torch.zeros_like(du)
    pl.substep("M", phi_e, phi_i, du, a, spec)
    rep_a = pl.report()
    pl.substep_capturable("M", phi_e, phi_i, du, b, spec)
    torch.cuda.synchronize()
    rep_b = pl.report()
    assert pl.unserved() == 0
    assert list(rep_a["fact"]) == list(rep_b["fact"])
    assert np.array_equal(rep_a["siter"], rep_b["siter"])
    assert np.array_equal(rep_a["diter"], rep_b["diter"])
    assert np.array_equal(a.cpu().numpy(), b.cpu().numpy())
    assert pl.backward_error().max() <= 1e-12
    if siter == 25:
        assert rep_a["siter"].max() > 4      # beyond the old four-solve cap


def test_multicase_graph_matches_eager(lib, torch_cuda):
    """Cases of uneven S, Ny, k and grid, spread over streams and recorded
    into one CUDA graph per step, give the same bits as the host-driven step;
    each case's result does not depend on the other cases."""
    torch = torch_cuda
    from suzerain_gb300 import multicase, plan as P, synth
    cfgs = [synth.Config("a", 5, 48, 6, 8, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=11),
            synth.Config("b", 7, 64, 8, 8, 6, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=12),
            synth.Config("c", 5, 96, 8, 16, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=13)]
    # graph and host-driven runs make the same decisions (siter + 1 complex64
    # correction solves at most in both), so they agree bit for bit
    spec = P.RefineSpec(aiter=5, siter=3, diter=5, tolsc=145.0)
    mc = multicase.MultiCase(cfgs, nstreams=2)
    mc.step_eager("M", spec)
    torch.cuda.synchronize()
    eager = [mc.result(i).cpu().numpy() for i in range(len(cfgs))]
    assert mc.backward_error().max() <= 1e-12
    mc.capture("M", spec)
    mc.reset()
    mc.replay()
    torch.cuda.synchronize()
    for i in range(len(cfgs)):
        assert np.array_equal(mc.result(i).cpu().numpy(), eager[i]), i
    assert mc.unserved() == 0
    # the same case alone
    solo = multicase.MultiCase(cfgs[1:2], nstreams=1)
    solo.step_eager("M", spec)
    torch.cuda.synchronize()
    assert np.array_equal(solo.result(0).cpu().numpy(), eager[1])
    # the production spec (siter = 25) meets the backward error bar
    mc2 = multicase.MultiCase(cfgs, nstreams=2)
    mc2.capture("M", P.RefineSpec(aiter=5, siter=25, diter=5, tolsc=145.0))
    mc2.replay()
    torch.cuda.synchronize()
    assert mc2.backward_error().max() <= 1e-12 and mc2.unserved() == 0


def test_ragged_factor_matches_per_case(lib, torch_cuda):
    """One complex64 factor launch per kernel kind over every case of a
    substep (KL = 24: specialized; 39: generic two warps; 48 and 55: generic
    four warps with three and four rows per thread) gives the per-case
    step's bits, replayed from a CUDA graph and issued directly."""
    torch = torch_cuda
    from suzerain_gb300 import multicase, plan as P, synth
    cfgs = [synth.Config("a", 5, 48, 6, 8, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=11),
            synth.Config("b", 7, 64, 8, 8, 6, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=12),
            synth.Config("c", 5, 96, 9, 16, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=13),
            synth.Config("d", 7, 40, 9, 8, 6, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=14)]
    spec = P.RefineSpec(aiter=5, siter=3, diter=5, tolsc=145.0)
    ref = multicase.MultiCase(cfgs, nstreams=2)
    ref.capture("M", spec)
    ref.reset()
    ref.replay()
    torch.cuda.synchronize()
    want = [ref.result(i).cpu().numpy() for i in range(len(cfgs))]
    kls = sorted(cs.KL for cs in ref.cases)
    assert kls == [24, 39, 48, 55], kls
    rg = multicase.MultiCase(cfgs, nstreams=2, ragged=True)
    rg.capture("M", spec)
    rg.reset()
    rg.replay()
    torch.cuda.synchronize()
    for i in range(len(cfgs)):
        assert np.array_equal(rg.result(i).cpu().numpy(), want[i]), i
    assert rg.unserved() == 0 and rg.backward_error().max() <= 1e-12
    # issued directly, without the graph
    rg.reset()
    rg.step_capturable("M", spec)
    torch.cuda.synchronize()
    for i in range(len(cfgs)):
        assert np.array_equal(rg.result(i).cpu().numpy(), want[i]), i
    rg.close()
    # the creation checks: a plan without its mixed workspace
    bare = P.Plan(*cfgs[0].batch()[:3])
    with pytest.raises(RuntimeError, match="sgb_ragged_create"):
        P.RaggedFactor([bare], [1e-3], spec)
    bare.close()


def test_serving_result_same_alone_and_in_the_mix(lib, torch_cuda):
    """Continuous batching: requests that arrive while others run are
    admitted under the memory budget and overlap on the device; each
    request's final state is the same bits alone and in the mix."""
    torch = torch_cuda
    from suzerain_gb300 import serve, synth, plan as P
    pool = [synth.Config("s0", 5, 48, 6, 8, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=21),
            synth.Config("s1", 7, 32, 8, 8, 6, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=22),
            synth.Config("s2", 5, 64, 8, 16, 8, synth.FOURPI, synth.FOURPI / 3, 1e-3, seed=23)]
    trace = serve.poisson_trace(8, rate=200.0, seed=5, configs=pool, life=(3, 6))
    srv = serve.Server(budget_bytes=2e9, nstreams=4, keep_results=True)
    stats = srv.run(trace)
    assert stats["substeps"] == sum(r.nsubsteps for r in trace)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for r in trace[:3]:
        alone = serve.Server(budget_bytes=2e9, nstreams=1, keep_results=True)
        alone.run([serve.Request(r.rid, r.config, r.nsubsteps, 0.0)])
        assert np.array_equal(alone.results[r.rid], srv.results[r.rid]), r.rid
    # a budget that fits one case at a time still serves everything
    one = P.Plan.estimate_bytes(pool[2].case(), pool[2].nsys, 128, "M") + 2 * pool[2].nsys * 320 * 16
    tight = serve.Server(budget_bytes=one * 1.01, nstreams=2)
    st2 = tight.run(serve.poisson_trace(4, rate=500.0, seed=6, configs=pool, life=(3, 3)))
    assert st2["substeps"] == 12 and st2["peak_resident_cases"] >= 1


def test_cpp_solver_shim_runs(lib, tmp_path):
    """The header-only C++ bsmbsm_solver counterpart, linked against the
    library, packs S x S banded blocks, solves with the zgbsv and zcgbsvx
    specifications on the GPU and meets A x = b (dense check)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "suzerain_gb300", "_lib")
    exe = str(tmp_path / "shim")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(root, "include"),
                        os.path.join(root, "tests", "solver_shim_check.cpp"), "-L", libdir,
                        "-lsuzerain_gb300", "-Wl,-rpath," + libdir, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_dropin_zcgbsvx_factor_reuse_sequence(lib, oracle):
    """suzerain_lapackext_zcgbsvx with the caller's factor (fact 'S'/'D',
    apprx): over a series of perturbed bands the GPU drop-in makes the same
    decisions as the oracle (pinned to the reference build), call for call:
    reuse of the approximate factor, the restart with a fresh factor when
    refinement with it stalls, refinement with a supplied complex128 factor."""
    got = oracle.reuse_sequence(lib.suzerain_lapackext_zcgbsvx)
    want = oracle.reuse_sequence(oracle.lib().orc_zcgbsvx)
    for k, (g, w) in enumerate(zip(got, want)):
        for key in ("info", "fact", "apprx", "siter", "diter"):
            assert g[key] == w[key], (k, key, g[key], w[key])
        assert np.max(np.abs(g["x"] - w["x"])) <= 1e-11 * np.max(np.abs(w["x"])), k
