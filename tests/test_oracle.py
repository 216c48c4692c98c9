"""Pin the oracle: restated algorithm vs the reference's golden vectors and,
where it was built here, the reference's own compiled C (oracle/_ref).

Mirrors tests/test_bsmbsm.cpp (q/qinv KATs, aPxpby grid, pack NaN poisoning,
the Mathematica solve KAT) and tests/test_lapackext.c (Lotkin matrices, run
here against the complex zcgbsvx as well)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def kat():
    with open(os.path.join(GOLD, "bsmbsm_kat.json")) as f:
        return json.load(f)


def test_q_qinv_golden(oracle):
    d = kat()
    for i, v in d["q_S5n9"]:
        assert oracle.q(5, 9, i) == v
    for i, v in d["qinv_S5n9"]:
        assert oracle.qinv(5, 9, i) == v
    for S in range(1, 5):
        for n in range(1, 10):
            for i in range(S * n):
                assert oracle.qinv(S, n, oracle.q(S, n, i)) == i


def _kat_papt(oracle, d, complex_op):
    """Pack the S=3 KAT operator with packf (LD+KL rows), NaN-poisoned."""
    g = oracle.bsmbsm(d["S"], d["n"], d["kl"], d["ku"])
    rows = g["LD"] + g["KL"]
    papt = np.full(rows * g["N"], np.nan, dtype=np.complex128)
    L = oracle.lib()
    scale = 1j if complex_op else 1.0
    for ih, row in enumerate(d["blocks"]):
        for jh, blk in enumerate(row):
            if blk is None:
                rc = L.orc_zpack(d["S"], d["n"], ih, jh, d["kl"], d["ku"],
                                 oracle._z(0), None, g["ld"], g["KL"], g["KU"],
                                 papt[g["KL"]:].ctypes.data, rows)
            else:
                b = np.array(d[blk[0]], dtype=np.complex128) * blk[1]
                rc = L.orc_zpack(d["S"], d["n"], ih, jh, d["kl"], d["ku"],
                                 oracle._z(scale), b.ctypes.data, g["ld"],
                                 g["KL"], g["KU"], papt[g["KL"]:].ctypes.data,
                                 rows)
            assert rc == 0
    return g, papt


@pytest.mark.parametrize("complex_op", [False, True])
def test_solve_kat(oracle, complex_op):
    """tests/test_bsmbsm.cpp:801-966: pack, zgbsv, unpermute == XR."""
    d = kat()
    g, papt = _kat_papt(oracle, d, complex_op)
    # no NaN left inside the band
    A = oracle.band_to_dense(papt, g["N"], g["KL"], g["KU"], g["LD"] + g["KL"],
                             off=g["KL"])
    assert not np.isnan(A).any()
    br = np.array(d["BR"], dtype=np.complex128)
    pb = np.zeros(g["N"], dtype=np.complex128)
    rhs = br * (1j if complex_op else 1.0)   # i*op x = i*BR
    assert oracle.zaPxpby("N", g["S"], g["n"], 1, rhs, 1, 0, pb, 1) == 0
    info, ipiv = oracle.zgbtrf(papt, g["N"], g["KL"], g["KU"],
                               g["LD"] + g["KL"])
    assert info == 0
    oracle.zgbtrs("N", papt, g["N"], g["KL"], g["KU"], g["LD"] + g["KL"], ipiv,
                  pb)
    x = np.zeros(g["N"], dtype=np.complex128)
    assert oracle.zaPxpby("T", g["S"], g["n"], 1, pb, 1, 0, x, 1) == 0
    xr = np.array(d["XR"])
    tol = np.finfo(float).eps * d["tolerance_eps_multiple"]
    assert np.allclose(x.real, xr, rtol=tol, atol=tol * np.abs(xr).max())
    assert np.abs(x.imag).max() <= tol * np.abs(xr).max()


def _rand_band(rng, n, kl, ku, extra_rows):
    ldab = extra_rows + kl + ku + 1
    ab = np.zeros(ldab * n, dtype=np.complex128)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[extra_rows + ku + i - j + j * ldab] = complex(rng.normal(), rng.normal())
    return ab, ldab


@pytest.mark.parametrize("n,kl,ku", [(40, 3, 5), (240, 34, 34), (13, 12, 0),
                                     (7, 0, 3), (60, 48, 48), (1, 0, 0)])
def test_gbtrf_matches_reference_lapack(oracle, n, kl, ku):
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build absent (no reference checkout here)")
    rng = np.random.default_rng(n * 1000 + kl)
    ab, ldab = _rand_band(rng, n, kl, ku, kl)
    a1, a2 = ab.copy(), ab.copy()
    info1, p1 = oracle.zgbtrf(a1, n, kl, ku, ldab)
    p2 = np.zeros(n, np.int32)
    info2 = R.suzerain_lapack_zgbtrf(n, n, kl, ku, a2.ctypes.data, ldab,
                                     p2.ctypes.data)
    assert info1 == info2 == 0
    assert np.array_equal(p1, p2)
    assert np.max(np.abs(a1 - a2)) <= 1e-12 * max(1, np.max(np.abs(a2)))
    A = oracle.band_to_dense(ab, n, kl, ku, ldab, off=kl)
    for tr, op in (("N", A), ("T", A.T), ("C", A.conj().T)):
        b = rng.normal(size=n) + 1j * rng.normal(size=n)
        x1, x2 = b.copy(), b.copy()
        oracle.zgbtrs(tr, a1, n, kl, ku, ldab, p1, x1)
        R.suzerain_lapack_zgbtrs(tr.encode(), n, kl, ku, 1, a2.ctypes.data,
                                 ldab, p2.ctypes.data, x2.ctypes.data, n)
        assert np.max(np.abs(x1 - x2)) <= 1e-11 * np.max(np.abs(x2))
        assert np.max(np.abs(op @ x1 - b)) <= 1e-11 * np.max(np.abs(b)) * n


def test_zero_pivot_info(oracle):
    n, kl, ku = 6, 1, 1
    ab, ldab = _rand_band(np.random.default_rng(3), n, kl, ku, kl)
    for i in range(max(0, 3 - ku), min(n, 3 + kl + 1)):
        ab[kl + ku + i - 3 + 3 * ldab] = 0   # column 3 identically zero
    info, _ = oracle.zgbtrf(ab.copy(), n, kl, ku, ldab)
    assert info == 4
    R = oracle.ref()
    if R is not None:
        p = np.zeros(n, np.int32)
        assert R.suzerain_lapack_zgbtrf(n, n, kl, ku, ab.copy().ctypes.data,
                                        ldab, p.ctypes.data) == 4


def test_pack_matches_reference(oracle):
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build absent")
    L = oracle.lib()
    for (S, n, kl, ku) in [(1, 10, 2, 3), (2, 2, 0, 0), (3, 17, 4, 3), (5, 12, 6, 6)]:
        g = oracle.bsmbsm(S, n, kl, ku)
        rng = np.random.default_rng(S * n)
        b = rng.normal(size=g["ld"] * n) + 1j * rng.normal(size=g["ld"] * n)
        p1 = np.full(g["LD"] * g["N"], np.nan, dtype=np.complex128)
        p2 = p1.copy()
        for ih in range(S):
            for jh in range(S):
                al = oracle._z(complex(ih + 2, jh - 1))
                assert L.orc_zpack(S, n, ih, jh, kl, ku, al, b.ctypes.data,
                                   g["ld"], g["KL"], g["KU"], p1.ctypes.data,
                                   g["LD"]) == 0
                assert R.suzerain_bsmbsm_zpack(S, n, ih, jh, kl, ku, al,
                                               b.ctypes.data, g["ld"], g["KL"],
                                               g["KU"], p2.ctypes.data,
                                               g["LD"]) == 0
        assert np.array_equal(np.isnan(p1), np.isnan(p2))
        m = ~np.isnan(p1)
        assert np.array_equal(p1[m], p2[m])
        # every in-band position of P A P^T was written
        A = oracle.band_to_dense(p1, g["N"], g["KL"], g["KU"], g["LD"])
        assert not np.isnan(A).any()


@pytest.mark.parametrize("trans", ["N", "T"])
def test_aPxpby_grid(oracle, trans):
    """tests/test_bsmbsm.cpp:352-474 complex grid, against the reference."""
    R = oracle.ref()
    for S in (1, 2, 5):
        for n in (1, 7, 10):
            N = S * n
            for alpha in (1, 3, complex(-2, 2)):
                for incx in (1, 2, -1, -2):
                    for beta in (0, 1, -3, complex(4, -2)):
                        for incy in (1, 3, -1, -3):
                            x = np.cumsum(np.full(N * abs(incx), 2 * alpha + 1, dtype=np.complex128))
                            y = np.cumsum(np.full(N * abs(incy), alpha - 7 + 1j, dtype=np.complex128))
                            y1 = y.copy()
                            assert oracle.zaPxpby(trans, S, n, alpha, x, incx,
                                                  beta, y1, incy) == 0
                            # permute + axpby by hand
                            xs = x[::abs(incx)][:N]
                            if incx < 0:
                                xs = xs[::-1]
                            Sq, nq = (S, n) if trans == "N" else (n, S)
                            px = np.array([xs[(i % Sq) * nq + i // Sq] for i in range(N)])
                            y2 = y.copy()
                            ys = y2[::abs(incy)][:N].copy()
                            if incy < 0:
                                ys = ys[::-1]
                            ys = alpha * px + beta * ys
                            if incy < 0:
                                ys = ys[::-1]
                            y2[::abs(incy)][:N] = ys
                            tol = 4 * np.finfo(float).eps
                            assert np.allclose(y1, y2, rtol=tol, atol=tol * np.abs(y2).max())
                            if R is not None and incx > 0 and incy > 0:
                                y3 = y.copy()
                                R.suzerain_bsmbsm_zaPxpby(trans.encode(), S, n, oracle._z(alpha),
                                                          x.ctypes.data, incx, oracle._z(beta),
                                                          y3.ctypes.data, incy)
                                assert np.allclose(y1, y3, rtol=tol, atol=tol * np.abs(y3).max())


def lotkin(n):
    """Lotkin (1955) matrix as a dense band (tests/test_lapackext.c:41-72)."""
    A = np.array([[1.0 if i == 0 else 1.0 / (i + j + 1) for j in range(n)]
                  for i in range(n)])
    return A


def dense_to_band(A, kl, ku):
    n = A.shape[0]
    ldab = kl + ku + 1
    ab = np.zeros(ldab * n, dtype=np.complex128)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[ku + i - j + j * ldab] = A[i, j]
    return ab


@pytest.mark.parametrize("n", [2, 5, 8, 12])
def test_zcgbsvx_lotkin(oracle, n):
    """Complex Lotkin systems: the reference only pins dsgbsvx this way."""
    A = lotkin(n) * (1 + 0.5j)
    x_true = np.ones(n, dtype=np.complex128)
    b = A @ x_true
    ab = dense_to_band(A, n - 1, n - 1)
    out = oracle.zcgbsvx(ab, n, n - 1, n - 1, b, aiter=5, siter=25, diter=10,
                         tolsc=1.0)
    assert out["info"] == 0
    assert out["tolsc"] <= 1.0
    ores = np.linalg.norm(A @ out["x"] - b)
    assert ores <= 10 * out["res"] + 1e-30
    R = oracle.ref()
    if R is not None:
        kl = ku = n - 1
        fact = C.create_string_buffer(b"N", 1)
        apprx, afrob = C.c_int(0), C.c_double(-1)
        afb = np.zeros((2 * kl + ku + 1) * n, dtype=np.complex128)
        ipiv = np.zeros(n, np.int32)
        x = np.zeros(n, dtype=np.complex128)
        r = np.zeros(n, dtype=np.complex128)
        si, di, ts, res = C.c_int(25), C.c_int(10), C.c_double(1.0), C.c_double(0)
        bb = b.copy()
        info = R.suzerain_lapackext_zcgbsvx(C.addressof(fact), C.addressof(apprx), 5,
                                            b"N", n, kl, ku, ab.ctypes.data,
                                            C.addressof(afrob), afb.ctypes.data,
                                            ipiv.ctypes.data, bb.ctypes.data,
                                            x.ctypes.data, C.addressof(si),
                                            C.addressof(di), C.addressof(ts),
                                            r.ctypes.data, C.addressof(res))
        assert info == 0
        assert fact.raw.decode() == out["fact"]
        assert si.value == out["siter"] and di.value == out["diter"]
        assert np.max(np.abs(x - out["x"])) <= 1e-6 * np.max(np.abs(x))


def test_gbmv_matches_reference(oracle):
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build absent")
    rng = np.random.default_rng(7)
    for tr in "NTC":
        for (m, n, kl, ku) in [(30, 30, 3, 5), (20, 25, 2, 7)]:
            lda = kl + ku + 2
            a = rng.normal(size=lda * n) + 1j * rng.normal(size=lda * n)
            lx = n if tr == "N" else m
            ly = m if tr == "N" else n
            x = rng.normal(size=lx) + 1j * rng.normal(size=lx)
            y = rng.normal(size=ly) + 1j * rng.normal(size=ly)
            y1, y2 = y.copy(), y.copy()
            oracle.zgbmv(tr, m, n, kl, ku, 2 - 1j, a, lda, x, 0.5, y1)
            R.suzerain_blas_zgbmv(tr.encode(), m, n, kl, ku, oracle._z(2 - 1j),
                                  a.ctypes.data, lda, x.ctypes.data, 1,
                                  oracle._z(0.5), y2.ctypes.data, 1)
            assert np.allclose(y1, y2, rtol=1e-13, atol=1e-13)


def _strided(v, inc):
    s = np.zeros((len(v) - 1) * abs(inc) + 1, dtype=v.dtype)
    s[::abs(inc)] = v if inc > 0 else v[::-1]
    return s


def _logical(s, n, inc):
    v = s[::abs(inc)][:n]
    return v if inc > 0 else v[::-1]


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("xreal", [False, True])
def test_gbdmv_matches_reference(oracle, k, xreal):
    """The oracle's diagonally scaled band matvec (the formula the GPU drop-in
    tests check against) equals the reference's own gbd*mv.def code over
    trans N/T/C, strides of both signs, diagonal strides 0..3, beta = 0 and
    all-zero alphas; the reference's argument-error positions (which the
    drop-ins return) are those the GPU tests expect."""
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build absent")
    f = getattr(R, f"oracle_ref_gbd{k}mv_{'ddz' if xreal else 'dzz'}")
    rng = np.random.default_rng(41 + k + 5 * xreal)
    n, kl, ku = 37, 4, 3
    lda = kl + ku + 2
    a = rng.normal(size=lda * n)
    ldd = [1, 0, 2, 1, 3][:k]
    ds = [rng.normal(size=(n - 1) * l + 1) for l in ldd]

    def call(trans, alphas, xs, incx, beta, ys, incy, lda_=lda, ldd_=ldd):
        args = [trans.encode(), n, kl, ku]
        for al, d, l in zip(alphas, ds, ldd_):
            args += [oracle._z(al), d.ctypes.data, l]
        return f(*args, a.ctypes.data, lda_, xs.ctypes.data, incx, oracle._z(beta),
                 ys.ctypes.data, incy)

    cases = [("N", 1, 1, 0.5 - 0.25j), ("T", 2, -1, 1.0), ("C", -1, 3, 0.0), ("n", -2, 2, 2j)]
    for trans, incx, incy, beta in cases:
        alphas = [complex(rng.normal(), rng.normal()) for _ in range(k)]
        xl = rng.normal(size=n) if xreal else rng.normal(size=n) + 1j * rng.normal(size=n)
        yl = rng.normal(size=n) + 1j * rng.normal(size=n)
        xs, ys = _strided(xl, incx), _strided(yl, incy)
        assert call(trans, alphas, xs, incx, beta, ys, incy) == 0
        want = oracle.gbdmv(trans, n, kl, ku, alphas, ds, ldd, a, lda, xl, beta, yl)
        assert np.allclose(_logical(ys, n, incy), want, rtol=1e-13, atol=1e-13), trans
    y0 = rng.normal(size=n) + 1j * rng.normal(size=n)
    xn = np.full(n, np.nan) if xreal else np.full(n, np.nan + 0j)
    y = y0.copy()
    assert call("T", [0.0] * k, xn, 1, 2.0, y, 1) == 0
    assert np.array_equal(y, oracle.gbdmv("T", n, kl, ku, [0.0] * k, ds, ldd, a, lda, xn, 2.0, y0))
    xs = rng.normal(size=n) + (0 if xreal else 1j * rng.normal(size=n))
    assert call("X", [1.0] * k, xs, 1, 1.0, y, 1) == 1
    assert call("N", [1.0] * k, xs, 1, 1.0, y, 1, ldd_=[-1] + ldd[1:]) == 7
    if k > 1:
        assert call("N", [1.0] * k, xs, 1, 1.0, y, 1, ldd_=ldd[:-1] + [-1]) == 7 + 3 * (k - 1)
    assert call("N", [1.0] * k, xs, 1, 1.0, y, 1, lda_=kl + ku) == 3 * k + 6
    assert call("N", [1.0] * k, xs, 0, 1.0, y, 1) == 3 * k + 8
    assert call("N", [1.0] * k, xs, 1, 1.0, y, 0) == (13 if k == 1 else 3 * k + 11)


@pytest.mark.parametrize("Nx,dNx,Nz,dNz", [(8, 12, 6, 9), (7, 7, 6, 6), (16, 24, 11, 17)])
def test_diffwave_matches_reference(oracle, Nx, dNx, Nz, dNz):
    """The oracle's Fourier derivative (the formula of the GPU diffwave tests)
    equals the reference's own suzerain/diffwave.c for apply and accumulate,
    derivative orders 0..3, whole and partial blocks of modes, dealiased and
    undealiased grids, odd and even N."""
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build absent")
    rng = np.random.default_rng(Nx * 100 + Nz)
    Ny, Lx, Lz = 5, 4.0, 3.0
    al, be = 1.5 - 0.5j, 0.25 + 2j
    for dkbx, dkex, dkbz, dkez in ((0, dNx, 0, dNz), (1, dNx - 2, 2, dNz)):
        shape = (dkez - dkbz, dkex - dkbx, Ny)
        for dx, dz in ((0, 0), (1, 0), (0, 2), (1, 1), (3, 2)):
            args = (Lx, Lz, Nx, dNx, dkbx, dkex, Nz, dNz, dkbz, dkez)
            x = rng.normal(size=shape) + 1j * rng.normal(size=shape)
            g = x.copy()
            R.suzerain_diffwave_apply(dx, dz, oracle._z(al), g.ctypes.data, Lx, Lz, Ny, Nx,
                                      dNx, dkbx, dkex, Nz, dNz, dkbz, dkez)
            want = oracle.diffwave_apply(dx, dz, al, x, *args)
            assert np.allclose(g, want, rtol=1e-14, atol=1e-13), (dx, dz)
            assert np.array_equal(g == 0, want == 0)
            y0 = rng.normal(size=shape) + 1j * rng.normal(size=shape)
            y = y0.copy()
            R.suzerain_diffwave_accumulate(dx, dz, oracle._z(al), x.ctypes.data, oracle._z(be),
                                           y.ctypes.data, Lx, Lz, Ny, Nx, dNx, dkbx, dkex, Nz,
                                           dNz, dkbz, dkez)
            want = oracle.diffwave_accumulate(dx, dz, al, x, be, y0, *args)
            assert np.allclose(y, want, rtol=1e-14, atol=1e-13), (dx, dz)


# --------------------------------------------------------------------------
# zgbsvx: the restatement against LAPACK's own zgbsvx (SciPy's OpenBLAS, the
# routine suzerain_lapack_zgbsvx forwards to)
# --------------------------------------------------------------------------
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("fact", ["N", "E"])
@pytest.mark.parametrize("scaled", [False, True])
def test_zgbsvx_matches_lapack(oracle, trans, fact, scaled):
    from gbsvx_cases import GEOMS, assert_close, band, rhs
    if oracle.openblas_path() is None:
        pytest.skip("SciPy's OpenBLAS not found")
    for k, (n, kl, ku) in enumerate(GEOMS):
        ab, _ = band(n, kl, ku, seed=100 + k, scaled=scaled)
        b = rhs(n, 2, seed=100 + k)
        got = oracle.zgbsvx(ab, n, kl, ku, b, trans=trans, fact=fact)
        want = oracle.zgbsvx(ab, n, kl, ku, b, trans=trans, fact=fact, openblas=True)
        if want is None:
            pytest.skip("scipy_zgbsvx_ not exported")
        assert_close(got, want, n, kl, ku, f"{n},{kl},{ku},{trans},{fact}")
        np.testing.assert_array_equal(got["ipiv"], want["ipiv"])


def test_zgbsvx_fact_f_and_singular(oracle):
    """fact 'F' reuses an earlier call's factor and scalings; a zero column
    stops at the factor with info = its index, rcond = 0, x untouched."""
    from gbsvx_cases import assert_close, band, rhs
    if oracle.openblas_path() is None:
        pytest.skip("SciPy's OpenBLAS not found")
    n, kl, ku = 40, 5, 4
    ab, _ = band(n, kl, ku, seed=7, scaled=True)
    b = rhs(n, 1, seed=7)
    first = oracle.zgbsvx(ab, n, kl, ku, b, fact="E")
    assert first["equed"] == "B"
    kw = dict(fact="F", afb=first["afb"], ipiv=first["ipiv"], equed=first["equed"],
              r=first["r"], c=first["c"])
    b2 = rhs(n, 3, seed=8)
    for trans in "NTC":
        got = oracle.zgbsvx(first["ab"], n, kl, ku, b2, trans=trans, **kw)
        want = oracle.zgbsvx(first["ab"], n, kl, ku, b2, trans=trans, openblas=True, **kw)
        if want is None:
            pytest.skip("scipy_zgbsvx_ not exported")
        assert_close(got, want, n, kl, ku, "F" + trans)
    ab, _ = band(10, 2, 2, seed=9, singular_col=4)
    got = oracle.zgbsvx(ab, 10, 2, 2, rhs(10, 1, 9), fact="N")
    want = oracle.zgbsvx(ab, 10, 2, 2, rhs(10, 1, 9), fact="N", openblas=True)
    assert got["info"] == want["info"] == 5
    assert_close(got, want, 10, 2, 2, "singular")
    assert not got["x"].any()


def test_inorder_wavenumber_matches_reference(oracle, native):
    """The library's suzerain_inorder_wavenumber equals the reference's own
    (suzerain/inorder.h:92-96, extern definition in suzerain/inorder.c) for
    every index of even and odd N."""
    R = oracle.ref()
    if R is None:
        pytest.skip("reference build absent")
    R.suzerain_inorder_wavenumber.argtypes = [C.c_int, C.c_int]
    R.suzerain_inorder_wavenumber.restype = C.c_int
    for N in (1, 2, 3, 8, 13, 24, 192, 257):
        for i in range(N):
            assert native.suzerain_inorder_wavenumber(N, i) == R.suzerain_inorder_wavenumber(N, i)


def test_rholut_golden_reproduces_from_reference_build(oracle):
    """tests/golden/rholut_imexop.npz (the reference vectors of the GPU
    production-operator tests) is what the reference's own
    suzerain/rholut_imexop.c computes on its inputs, value for value."""
    import sys
    R = oracle.ref()
    if R is None:
        pytest.skip("no reference build here")
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_rholut_golden as M
    fresh = M.generate(C.CDLL(oracle.REF_PATH), C.CDLL(oracle.SYNTH_PATH))
    kept = np.load(os.path.join(os.path.dirname(__file__), "golden", "rholut_imexop.npz"))
    assert set(fresh) == set(kept.files)
    for k in kept.files:
        np.testing.assert_array_equal(np.asarray(fresh[k]), kept[k], err_msg=k)


def test_rholut_reference_pack_and_accumulate_agree(oracle):
    """The property the GPU tests rely on, checked on the reference itself:
    its packc band, applied as (P^T PATPT P)^T, equals its accumulate
    (suzerain/rholut_imexop.c:43-49 keeps the two in step)."""
    kept = np.load(os.path.join(os.path.dirname(__file__), "golden", "rholut_imexop.npz"))
    n = int(kept["n"])
    for name, order in (("A", (0, 1, 2, 3, 4)), ("B", (0, 1, 2, 3, 4)), ("C", (0, 1, 2, 3, 4)),
                        ("D", (4, 3, 2, 1, 0)), ("E", (0, 1, 2, 3, -1))):
        S = sum(o >= 0 for o in order)
        band = kept[f"{name}_packc"]                  # (N, LD): column C, band row
        N, LD = band.shape
        KU = (LD - 1) // 2
        AT = np.zeros((N, N), complex)
        for c in range(N):
            for i in range(LD):
                r = c + i - KU
                if 0 <= r < N:
                    AT[r, c] = band[c, i]
        # natural (position-major) order <-> permuted: global index p S + pos
        perm = np.array([(i % S) * n + i // S for i in range(N)])
        def to_nat(v):
            out = np.zeros(S * n, complex)
            for e, o in enumerate(order):
                if o >= 0:
                    out[o * n:(o + 1) * n] = v[e * n:(e + 1) * n]
            return out
        x, y0, y = (to_nat(kept[f"{name}_{k}"]) for k in ("x", "y0", "y"))
        A_nat = np.empty_like(AT)
        A_nat[np.ix_(perm, perm)] = AT.T                 # A = P^T (PATPT)^T P
        want = A_nat @ x + complex(kept["beta"]) * y0
        assert np.max(np.abs(want - y)) <= 1e-12 * np.max(np.abs(y)), name


DIAG_NAMES = {1: "zgb_diag_scale_acc_d", 2: "zgb_ddiag_scale_acc_d", 3: "zgb_dddiag_scale_acc_d",
              4: "zgb_ddddiag_scale_acc_d", 5: "zgb_dddddiag_scale_acc_d"}


def ref_diag_scale_acc(R, K, side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta, b, incb,
                       ldb):
    """The reference's own suzerain_blasext_zgb_<K>diag_scale_acc_d on copies."""
    from oracle import oracle
    f = getattr(R, "suzerain_blasext_" + DIAG_NAMES[K])
    Z, P, I = oracle._Z, C.c_void_p, C.c_int
    f.argtypes = [C.c_char, I, I, I, I] + [Z, P, I] * K + [P, I, I, Z, P, I, I]
    f.restype = I
    bb = np.array(b, dtype=np.complex128, copy=True)
    args = []
    for al, d, l in zip(alphas, ds, ldds):
        args += [oracle._z(al), d.ctypes.data if d is not None else None, l]
    rc = f(side.encode(), m, n, kl, ku, *args, a.ctypes.data, inca, lda, oracle._z(beta),
           bb.ctypes.data, incb, ldb)
    return rc, bb


@pytest.mark.parametrize("K", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("side", ["R", "L"])
@pytest.mark.parametrize("beta", [1.0, 0.0, 0.5 - 0.25j])
def test_diag_scale_acc_restatement_matches_reference(oracle, K, side, beta):
    """oracle.gb_diag_scale_acc equals the reference's blasext routines
    (rectangular band, row strides, a constant diagonal)."""
    R = oracle.ref()
    if R is None:
        pytest.skip("no reference build here")
    rng = np.random.default_rng(K * 10 + (side == "L"))
    # a rectangular band for side 'R'; the reference walks side 'L' over
    # rows 0..n-1 and columns 0..m-1, which only a square band keeps inside
    # its storage
    m, n, kl, ku, inca, incb = (9, 7, 2, 3, 1, 1) if side == "R" else (8, 8, 2, 3, 1, 1)
    lda, ldb = kl + ku + 2, kl + ku + 3
    a = rng.normal(size=lda * n + 4)
    b = rng.normal(size=ldb * n + 4) + 1j * rng.normal(size=ldb * n + 4)
    alphas = [complex(rng.normal(), rng.normal()) for _ in range(K)]
    ds = [rng.normal(size=3 * max(m, n)) for _ in range(K)]
    ldds = [1, 2, 0, 3, 1][:K]
    rc, want = ref_diag_scale_acc(R, K, side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta,
                                  b, incb, ldb)
    assert rc == 0
    got = oracle.gb_diag_scale_acc(side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta, b,
                                   incb, ldb)
    np.testing.assert_allclose(got, want, rtol=1e-15, atol=1e-15)


def test_diag_scale_acc_error_positions_of_reference(oracle):
    """The argument positions the reference returns, which the GPU drop-ins
    reproduce (tests/test_gpu_blasext.py): kl 4, ku 5, ldd_k 8 + 3k,
    inca 7 + 3K, lda 8 + 3K, incb 11 + 3K, ldb (lda for K >= 2) 12 + 3K,
    side 1."""
    R = oracle.ref()
    if R is None:
        pytest.skip("no reference build here")
    a = np.zeros(64)
    b = np.zeros(64, complex)
    d = np.zeros(16)
    for K in range(1, 6):
        base = dict(side="R", m=4, n=4, kl=1, ku=1, alphas=[1] * K, ds=[d] * K, ldds=[1] * K,
                    inca=1, lda=3, beta=1, incb=1, ldb=3)

        def rc(**over):
            kw = {**base, **over}
            return ref_diag_scale_acc(R, K, kw["side"], kw["m"], kw["n"], kw["kl"], kw["ku"],
                                      kw["alphas"], kw["ds"], kw["ldds"], a, kw["inca"],
                                      kw["lda"], kw["beta"], b, kw["incb"], kw["ldb"])[0]
        assert rc(kl=-1) == 4 and rc(ku=-1) == 5
        for k in range(K):
            assert rc(ldds=[1] * k + [-1] + [1] * (K - k - 1)) == 8 + 3 * k
        assert rc(inca=0) == 7 + 3 * K and rc(lda=2) == 8 + 3 * K
        assert rc(incb=0) == 11 + 3 * K
        assert rc(ldb=2) == (12 + 3 * K if K == 1 else 0)
        assert rc(side="X") == 1


def test_zcgbsvx_factor_reuse_sequence_matches_reference(oracle):
    """Factor reuse (fact 'S'/'D' supplied, apprx set) over a series of
    perturbed bands: the restatement makes the reference's decisions call
    for call, including the restart with a fresh factor when refinement with
    the approximate one stalls (suzerain/blas_et_al/dsgbsvx.def:214-227)."""
    R = oracle.ref()
    if R is None:
        pytest.skip("no reference build here")
    got = oracle.reuse_sequence(oracle.lib().orc_zcgbsvx)
    want = oracle.reuse_sequence(R.suzerain_lapackext_zcgbsvx)
    for k, (g, w) in enumerate(zip(got, want)):
        for key in ("info", "fact", "apprx", "siter", "diter"):
            assert g[key] == w[key], (k, key, g[key], w[key])
        assert np.max(np.abs(g["x"] - w["x"])) <= 1e-12 * np.max(np.abs(w["x"])), k
    # the sequence exercises reuse, the stall restart and a supplied factor
    assert [g["apprx"] for g in got[:4]] == [0, 1, 1, 0]
    assert got[1]["siter"] > got[0]["siter"] and got[3]["fact"] == "S"
    assert got[5]["fact"] == "D" and got[5]["diter"] > 0
