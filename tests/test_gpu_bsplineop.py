"""GPU drop-ins of the B-spline operator API (suzerain/bsplineop.c) against
the oracle's numpy restatement and the reference's own known answers:

  * apply, accumulate, apply_complex and accumulate_complex against dense
    products with the workspace's operators, several derivatives, right-hand
    sides and increments; argument errors return SUZERAIN_EINVAL (4);
  * the complex operator of tests/test_bsplineop.cpp:340-462 (order-2
    B-splines on {0,1,2,3}, (2-3i) D0 + (7-5i) D1 + (999-999i) D2): its
    solves against the unit basis and two right-hand sides, contiguous and
    with incb 2, within the reference test's 1e-5 of its Octave rationals;
  * lu / luz on order-6 and order-8 bases: the factor (pivots equal, entries
    within 1e-9 of the largest) against LAPACK's gbtrf (SciPy), solves within
    64 kappa_inf eps of dense solves, opnorm equal to the dense infinity norm,
    rcond within a factor 2 of LAPACK's gbcon;
  * the reference's opaccumulate consistency suites (:1613-1800): every way of
    reaching the mass matrix factors to the same band within the reference's
    tolerances;
  * the usage checks (factor twice, accumulate into a factor, solve or rcond
    before the factor, opnorm after it);
  * the zgbcon and dgbnorm1 drop-ins against SciPy's zgbcon and numpy."""
import ctypes as C
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
EPS = np.finfo(float).eps


@pytest.fixture(scope="module")
def lib(native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    assert native.sgb_device_ok() == 0, native.sgb_last_error().decode()
    return native


def workspace(lib, k, breakpoints, nderiv):
    bp = np.ascontiguousarray(breakpoints, dtype=float)
    w = lib.sgb_bsplineop_alloc_breakpoints(k, len(bp), bp.ctypes.data, nderiv)
    assert w, lib.sgb_last_error().decode()
    return w


BASES = {
    "k6": (6, np.linspace(0.0, 2.0, 15) ** 1.3),
    "k8": (8, np.concatenate([[0.0], np.sort(np.random.default_rng(5).uniform(0, 3, 11)), [3.0]])),
}


@pytest.mark.parametrize("basis", list(BASES))
@pytest.mark.parametrize("nderiv", [0, 1, 2])
def test_apply_and_accumulate_match_dense(lib, oracle, basis, nderiv):
    from suzerain_gb300 import _native as nat
    k, bp = BASES[basis]
    w = workspace(lib, k, bp, 2)
    try:
        n = w.contents.n
        DT = oracle.bsplineop_transposes(w)[nderiv]
        rng = np.random.default_rng(40 + nderiv + k)
        nrhs, inc = 3, 2
        ld = n * inc + 3
        # real apply, strided columns
        x = rng.normal(size=ld * nrhs)
        want = x.copy()
        for c in range(nrhs):
            want[c * ld:c * ld + n * inc:inc] = oracle.bsplineop_accumulate(
                DT, 1.5, x[c * ld:c * ld + n * inc:inc], 0, None)
        got = x.copy()
        assert lib.suzerain_bsplineop_apply(nderiv, nrhs, 1.5, got.ctypes.data, inc, ld, w) == 0
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13 * np.abs(want).max())
        # real accumulate, beta 0.25
        y = rng.normal(size=ld * nrhs)
        wy = y.copy()
        for c in range(nrhs):
            s = slice(c * ld, c * ld + n * inc, inc)
            wy[s] = oracle.bsplineop_accumulate(DT, -0.5, x[s], 0.25, y[s])
        gy = y.copy()
        assert lib.suzerain_bsplineop_accumulate(nderiv, nrhs, -0.5, x.ctypes.data, inc, ld, 0.25,
                                                 gy.ctypes.data, inc, ld, w) == 0
        np.testing.assert_allclose(gy, wy, rtol=1e-13, atol=1e-13 * np.abs(wy).max())
        # complex apply (real alpha) and complex accumulate
        z = rng.normal(size=n * nrhs) + 1j * rng.normal(size=n * nrhs)
        wz = np.concatenate([oracle.bsplineop_accumulate(DT, 2.0, z[c * n:(c + 1) * n], 0, None)
                             for c in range(nrhs)])
        gz = z.copy()
        assert lib.suzerain_bsplineop_apply_complex(nderiv, nrhs, 2.0, gz.ctypes.data, 1, n, w) == 0
        np.testing.assert_allclose(gz, wz, rtol=1e-13, atol=1e-13 * np.abs(wz).max())
        yz = rng.normal(size=n * nrhs) + 1j * rng.normal(size=n * nrhs)
        wyz = np.concatenate([oracle.bsplineop_accumulate(DT, 1 - 2j, z[c * n:(c + 1) * n], 0.5j,
                                                          yz[c * n:(c + 1) * n])
                              for c in range(nrhs)])
        gyz = yz.copy()
        assert lib.suzerain_bsplineop_accumulate_complex(nderiv, nrhs, nat.zc(1 - 2j), z.ctypes.data, 1,
                                                         n, nat.zc(0.5j), gyz.ctypes.data, 1, n, w) == 0
        np.testing.assert_allclose(gyz, wyz, rtol=1e-13, atol=1e-13 * np.abs(wyz).max())
    finally:
        lib.suzerain_bsplineop_free(w)


def test_operator_argument_errors(lib):
    k, bp = BASES["k6"]
    w = workspace(lib, k, bp, 1)
    try:
        n = w.contents.n
        x = np.ones(2 * n)
        y = np.ones(2 * n)
        assert lib.suzerain_bsplineop_apply(2, 1, 1.0, x.ctypes.data, 1, n, w) == 4      # nderiv
        assert lib.suzerain_bsplineop_apply(-1, 1, 1.0, x.ctypes.data, 1, n, w) == 4
        assert lib.suzerain_bsplineop_apply(0, 2, 1.0, x.ctypes.data, 1, n - 1, w) == 4  # ldx
        assert lib.suzerain_bsplineop_accumulate(0, 1, 1.0, x.ctypes.data, 1, n, 0.0, x.ctypes.data,
                                                 1, n, w) == 4                          # x == y
        assert lib.suzerain_bsplineop_accumulate(0, 2, 1.0, x.ctypes.data, 1, n, 0.0, y.ctypes.data,
                                                 1, n - 1, w) == 4                      # ldy
        assert np.all(x == 1) and np.all(y == 1)
    finally:
        lib.suzerain_bsplineop_free(w)


def luz_view(luz):
    ws = luz.contents
    return np.ctypeslib.as_array(ws.A_T, shape=(ws.ld * ws.n * 2,)).view(np.complex128)


def lu_view(lu):
    ws = lu.contents
    return np.ctypeslib.as_array(ws.A_T, shape=(ws.ld * ws.n,))


def test_luz_known_answers(lib):
    """tests/test_bsplineop.cpp:340-462: opnorm > 0, 0 < rcond <= 1, and the
    solves equal the reference's known answers within its 1e-5."""
    d = json.load(open(os.path.join(GOLD, "bsplineop_luz_kat.json")))
    w = workspace(lib, d["k"], d["breakpoints"], d["nderiv"])
    luz = lib.suzerain_bsplineop_luz_alloc(w)
    try:
        assert luz.contents.n == d["n"]
        coef = np.array([complex(a, b) for a, b in d["coefficients"]])
        assert lib.suzerain_bsplineop_luz_opform(len(coef), coef.ctypes.data, w, luz) == 0
        norm, rcond = C.c_double(-123), C.c_double(-456)
        assert lib.suzerain_bsplineop_luz_opnorm(luz, C.byref(norm)) == 0
        assert norm.value > 0
        assert lib.suzerain_bsplineop_luz_factor(luz) == 0
        assert lib.suzerain_bsplineop_luz_rcond(norm.value, C.byref(rcond), luz) == 0
        assert 0 < rcond.value <= 1
        for sv in d["solves"]:
            b = np.array([complex(a, c) for a, c in sv["b"]])
            good = np.array([complex(a, c) for a, c in sv["b_good"]])
            ldb = len(b) // sv["nrhs"]
            assert lib.suzerain_bsplineop_luz_solve(sv["nrhs"], b.ctypes.data, sv["incb"], ldb, luz) == 0
            np.testing.assert_allclose(b.real, good.real, rtol=0, atol=sv["tolerance"])
            np.testing.assert_allclose(b.imag, good.imag, rtol=0, atol=sv["tolerance"])
    finally:
        lib.suzerain_bsplineop_luz_free(luz)
        lib.suzerain_bsplineop_free(w)


@pytest.mark.parametrize("basis", list(BASES))
@pytest.mark.parametrize("kind", ["lu", "luz"])
def test_operator_workspace_matches_lapack(lib, oracle, basis, kind):
    import scipy.linalg as sl
    from scipy.linalg import lapack
    from suzerain_gb300 import _native as nat
    k, bp = BASES[basis]
    w = workspace(lib, k, bp, 2)
    cplx = kind == "luz"
    alloc = getattr(lib, f"suzerain_bsplineop_{kind}_alloc")
    free = getattr(lib, f"suzerain_bsplineop_{kind}_free")
    fn = lambda name: getattr(lib, f"suzerain_bsplineop_{kind}_{name}")
    luw = alloc(w)
    try:
        ws = luw.contents
        n, kl, ku, ld = ws.n, ws.kl, ws.ku, ws.ld
        assert ld == 2 * kl + ku + 1 and ws.ipiv[0] == -1
        DTs = oracle.bsplineop_transposes(w)
        coef = np.array([1.0 + 0.5j, -0.25 + 0.1j, 0.01 - 0.02j]) if cplx else np.array([1.0, -0.25, 0.01])
        assert fn("opform")(3, coef.ctypes.data, w, luw) == 0
        assert ws.ipiv[0] == -2                                  # one accumulation
        AT = oracle.bsplineop_operator(DTs, coef)
        view = luz_view(luw) if cplx else lu_view(luw)
        band = oracle.band_of(AT, kl, ku, ld, off=kl)
        np.testing.assert_allclose(view, band, rtol=0, atol=1e-14 * np.abs(band).max())
        # opnorm: infinity norm of A = 1-norm of A^T
        norm = C.c_double()
        assert fn("opnorm")(luw, C.byref(norm)) == 0
        assert norm.value == pytest.approx(np.abs(AT).sum(axis=0).max(), rel=1e-14)
        # factor against LAPACK gbtrf on the same band
        assert fn("factor")(luw) == 0
        trf = lapack.zgbtrf if cplx else lapack.dgbtrf
        lab, lpiv, linfo = trf(band.reshape(n, ld).T.copy(), kl, ku)
        assert linfo == 0
        piv = np.ctypeslib.as_array(ws.ipiv, shape=(n,)).copy()
        assert np.array_equal(piv, lpiv + 1)
        # entries agree to the rounding of the pivots' reciprocals, grown
        # through the elimination
        fac = (luz_view(luw) if cplx else lu_view(luw)).reshape(n, ld).T
        np.testing.assert_allclose(fac, lab, rtol=0, atol=1e-9 * np.abs(lab).max())
        # rcond against LAPACK gbcon (both estimates of ||A^-T||_1)
        rcond = C.c_double()
        assert fn("rcond")(norm.value, C.byref(rcond), luw) == 0
        con = lapack.zgbcon if cplx else lapack.dgbcon
        lr, cinfo = con(kl, ku, lab, lpiv, norm.value, norm="1")
        assert cinfo == 0
        assert lr / 2 <= rcond.value <= lr * 2, (rcond.value, lr)
        # solves A x = b (transposed solve with the factor of A^T), strided
        rng = np.random.default_rng(9)
        nrhs, inc = 3, 2
        ldb = n * inc + 1
        B = rng.normal(size=ldb * nrhs) + (1j * rng.normal(size=ldb * nrhs) if cplx else 0)
        want = B.copy()
        A = AT.T
        for c in range(nrhs):
            s = slice(c * ldb, c * ldb + n * inc, inc)
            want[s] = sl.solve(A, B[s])
        got = B.copy()
        assert fn("solve")(nrhs, got.ctypes.data, inc, ldb, luw) == 0
        # two backward-stable solvers: normwise within 64 kappa_inf eps
        kap = np.linalg.cond(A, np.inf)
        for c in range(nrhs):
            s = slice(c * ldb, c * ldb + n * inc, inc)
            err = np.abs(got[s] - want[s]).max() / np.abs(want[s]).max()
            assert err <= 64 * kap * EPS, (err, kap)
        gap = np.ones(len(B), bool)
        for c in range(nrhs):
            gap[c * ldb:c * ldb + n * inc:inc] = False
        assert np.array_equal(got[gap], B[gap])                  # untouched between strides
        # usage checks
        assert fn("factor")(luw) == 4                           # already factored
        assert fn("opnorm")(luw, C.byref(norm)) == 4             # norm of a factor
        one = np.array([1.0 + 0j]) if cplx else np.array([1.0])
        scale = nat.zc(1.0) if cplx else 1.0
        assert fn("opaccumulate")(1, one.ctypes.data, w, scale, luw) == 4   # into a factor
        assert fn("opaccumulate")(4, coef.ctypes.data, w, nat.zc(0) if cplx else 0.0, luw) == 4
        assert fn("opaccumulate")(-1, coef.ctypes.data, w, nat.zc(0) if cplx else 0.0, luw) == 4
        assert fn("opform_mass")(w, luw) == 0                    # scale 0: allowed again
        assert fn("solve")(1, got.ctypes.data, 1, n, luw) == 4   # not factored
        assert fn("rcond")(1.0, C.byref(rcond), luw) == 4
    finally:
        free(luw)
        lib.suzerain_bsplineop_free(w)


MASS_BREAKPOINTS = [0.0, 0.5, 1.0, 3.0, 3.3, 7.0, 12.0, 12.5, 14.0, 15.0]


@pytest.mark.parametrize("kind", ["lu", "luz"])
def test_opaccumulate_consistency(lib, kind):
    """tests/test_bsplineop.cpp:1600-1810: form_mass, form, opaccumulate
    with scale 0, two halves, a scaled half, and repeated combinations all
    factor to the mass matrix's factor (order-7 basis, nderiv 2)."""
    from suzerain_gb300 import _native as nat
    cplx = kind == "luz"
    w = workspace(lib, 7, MASS_BREAKPOINTS, 2)
    alloc = getattr(lib, f"suzerain_bsplineop_{kind}_alloc")
    free = getattr(lib, f"suzerain_bsplineop_{kind}_free")
    fn = lambda name: getattr(lib, f"suzerain_bsplineop_{kind}_{name}")
    view = luz_view if cplx else lu_view
    dt = np.complex128 if cplx else np.float64
    sc = (lambda v: nat.zc(v)) if cplx else float
    arr = lambda *v: np.array(v, dtype=dt)
    ref = alloc(w)
    assert fn("factor_mass")(w, ref) == 0
    good = view(ref).copy()
    free(ref)

    def check(steps, tol):
        t = alloc(w)
        try:
            for coefs, scale in steps:
                c = arr(*coefs) if coefs else arr(0)
                assert fn("opaccumulate")(len(coefs), c.ctypes.data, w, sc(scale), t) == 0
            assert fn("factor")(t) == 0
            np.testing.assert_allclose(view(t), good, rtol=0, atol=tol * np.abs(good).max())
        finally:
            free(t)

    t = alloc(w)
    assert fn("opform_mass")(w, t) == 0 and fn("factor")(t) == 0
    assert np.allclose(view(t), good, rtol=0, atol=1000 * EPS * np.abs(good).max())
    free(t)
    one = arr(1.0)
    t = alloc(w)
    assert fn("opform")(1, one.ctypes.data, w, t) == 0 and fn("factor")(t) == 0
    assert np.allclose(view(t), good, rtol=0, atol=1000 * EPS * np.abs(good).max())
    free(t)
    check([((1.0,), 0.0)], 1000 * EPS)
    check([((0.5,), 0.0), ((0.5,), 1.0)], 1000 * EPS)
    if cplx:
        check([((0.08 + 0.04j,), 0.0), ((), 10.0 - 5.0j)], 1000 * EPS)
        check([((5, 6, 4), 1.0), ((0, -2, 14), 0.0), ((2, 0, 0), 1.0), ((0, 1, -7), 0.5),
               ((0, -2j, 14j), 0.0), ((2, 0, 0), 1.0), ((0, 1j, -7j), 0.5)], 1e6 * EPS)
    else:
        check([((0.5,), 0.0), ((), 2.0)], 1000 * EPS)
        check([((5, 6, 4), 1.0), ((0, -2, 14), 0.0), ((2, 0, 0), 1.0), ((0, 1, -7), 0.5),
               ((0, 4, -8), 0.0), ((2, 0, 0), 1.0), ((0, -2, 4), 0.5)], 2.5e6 * EPS)
    lib.suzerain_bsplineop_free(w)


@pytest.mark.parametrize("norm", ["1", "I"])
def test_zgbcon_dropin_matches_lapack(lib, norm):
    from scipy.linalg import lapack
    rng = np.random.default_rng(31 if norm == "1" else 32)
    n, kl, ku = 60, 4, 3
    ld = 2 * kl + ku + 1
    ab = np.zeros((ld, n), np.complex128)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[kl + ku + i - j, j] = complex(rng.normal(), rng.normal())
        ab[kl + ku, j] += 2.0
    A = np.zeros((n, n), np.complex128)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            A[i, j] = ab[kl + ku + i - j, j]
    anorm = np.abs(A).sum(axis=0).max() if norm == "1" else np.abs(A).sum(axis=1).max()
    lab, piv, info = lapack.zgbtrf(ab.copy(), kl, ku)
    assert info == 0
    want, cinfo = lapack.zgbcon(kl, ku, lab, piv, anorm, norm=norm)
    assert cinfo == 0
    fab = np.ascontiguousarray(lab.T).reshape(-1)
    ipiv = (piv + 1).astype(np.int32)
    rc = C.c_double()
    assert lib.suzerain_lapack_zgbcon(norm.encode(), n, kl, ku, fab.ctypes.data, ld, ipiv.ctypes.data,
                                      anorm, C.byref(rc), None, None) == 0
    assert rc.value == pytest.approx(want, rel=1e-10)
    assert lib.suzerain_lapack_zgbcon(b"X", n, kl, ku, fab.ctypes.data, ld, ipiv.ctypes.data, anorm,
                                      C.byref(rc), None, None) == -1
    assert lib.suzerain_lapack_zgbcon(norm.encode(), n, kl, ku, fab.ctypes.data, ld - 1,
                                      ipiv.ctypes.data, anorm, C.byref(rc), None, None) == -6


def test_dgbnorm1_dropin(lib):
    rng = np.random.default_rng(44)
    m = n = 40
    kl, ku, lda = 3, 5, 10
    a = rng.normal(size=lda * n)
    want = max(np.abs(a[j * lda + max(0, ku - j):j * lda + ku + min(kl + 1, m - j)]).sum()
               for j in range(n))
    got = C.c_double()
    assert lib.suzerain_blasext_dgbnorm1(m, n, kl, ku, a.ctypes.data, lda, C.byref(got)) == 0
    assert got.value == pytest.approx(want, rel=1e-15)
    assert lib.suzerain_blasext_dgbnorm1(m, n, kl, ku, a.ctypes.data, kl + ku, C.byref(got)) == -6
