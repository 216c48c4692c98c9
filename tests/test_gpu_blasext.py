"""GPU drop-ins of the band assembly helpers (suzerain/blas_et_al/blasext.c,
blas.c) against the oracle's numpy restatement, which tests/test_oracle.py
pins to the reference's own blasext.c: diagonally scaled accumulation with
one to five diagonals on both sides and three kinds of beta, the
accumulation zgb_acc_d, the reference's argument-error positions, in-place
demote/promote and the band 1-norm.  Bars: results within 1e-15 relative;
error positions and integer outputs identical."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = {1: "zgb_diag_scale_acc_d", 2: "zgb_ddiag_scale_acc_d", 3: "zgb_dddiag_scale_acc_d",
         4: "zgb_ddddiag_scale_acc_d", 5: "zgb_dddddiag_scale_acc_d"}


@pytest.fixture(scope="module")
def lib(native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    assert native.sgb_device_ok() == 0, native.sgb_last_error().decode()
    return native


def call(lib, K, side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta, b, incb, ldb):
    from suzerain_gb300 import _native as nat
    f = getattr(lib, "suzerain_blasext_" + NAMES[K])
    bb = np.array(b, dtype=np.complex128, copy=True)
    args = []
    for al, d, l in zip(alphas, ds, ldds):
        args += [nat.zc(al), d.ctypes.data, l]
    rc = f(side.encode(), m, n, kl, ku, *args, a.ctypes.data, inca, lda, nat.zc(beta),
           bb.ctypes.data, incb, ldb)
    return rc, bb


@pytest.mark.parametrize("K", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("side", ["R", "L"])
@pytest.mark.parametrize("beta", [1.0, 0.0, 0.5 - 0.25j])
def test_diag_scale_acc_matches_oracle(lib, oracle, K, side, beta):
    rng = np.random.default_rng(100 + K * 10 + (side == "L"))
    m, n, kl, ku = (9, 7, 2, 3) if side == "R" else (8, 8, 2, 3)
    inca, incb = (1, 1) if K % 2 else (2, 3)        # strided bands too
    lda, ldb = (kl + ku + 1) * inca + 1, (kl + ku + 1) * incb + 2
    cols = n if side == "R" else m
    a = rng.normal(size=lda * cols + 8)
    b = rng.normal(size=ldb * cols + 8) + 1j * rng.normal(size=ldb * cols + 8)
    alphas = [complex(rng.normal(), rng.normal()) for _ in range(K)]
    ds = [rng.normal(size=3 * max(m, n)) for _ in range(K)]
    ldds = [1, 2, 0, 3, 1][:K]
    rc, got = call(lib, K, side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta, b, incb, ldb)
    assert rc == 0, lib.sgb_last_error().decode()
    want = oracle.gb_diag_scale_acc(side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta, b,
                                    incb, ldb)
    np.testing.assert_allclose(got, want, rtol=1e-15, atol=1e-15)


def test_diag_scale_acc_error_positions(lib):
    """The reference's positions (test_diag_scale_acc_error_positions_of_reference)."""
    a = np.zeros(64)
    b = np.zeros(64, complex)
    d = np.zeros(16)
    for K in range(1, 6):
        base = dict(side="R", m=4, n=4, kl=1, ku=1, alphas=[1] * K, ds=[d] * K, ldds=[1] * K,
                    inca=1, lda=3, beta=1, incb=1, ldb=3)

        def rc(**over):
            kw = {**base, **over}
            return call(lib, K, kw["side"], kw["m"], kw["n"], kw["kl"], kw["ku"], kw["alphas"],
                        kw["ds"], kw["ldds"], a, kw["inca"], kw["lda"], kw["beta"], b,
                        kw["incb"], kw["ldb"])[0]
        assert rc(kl=-1) == 4 and rc(ku=-1) == 5
        for k in range(K):
            assert rc(ldds=[1] * k + [-1] + [1] * (K - k - 1)) == 8 + 3 * k
        assert rc(inca=0) == 7 + 3 * K and rc(lda=2) == 8 + 3 * K
        assert rc(incb=0) == 11 + 3 * K
        assert rc(ldb=2) == (12 + 3 * K if K == 1 else 0)
        assert rc(side="X") == 1


def test_zgb_acc_d_matches_oracle(lib, oracle):
    from suzerain_gb300 import _native as nat
    rng = np.random.default_rng(5)
    m, n, kl, ku = 11, 11, 3, 2
    lda, ldb = kl + ku + 1, kl + ku + 2
    a = rng.normal(size=lda * n)
    b = rng.normal(size=ldb * n) + 1j * rng.normal(size=ldb * n)
    for alpha, beta in ((1.0, 0.3 + 0.1j), (0.5j, 1.0), (2.0, 0.0)):
        got = b.copy()
        assert lib.suzerain_blas_zgb_acc_d(m, n, kl, ku, nat.zc(alpha), a.ctypes.data, lda,
                                           nat.zc(beta), got.ctypes.data, ldb) == 0
        want = oracle.gb_diag_scale_acc("R", m, n, kl, ku, [alpha], [np.ones(1)], [0], a, 1, lda,
                                        beta, b, 1, ldb)
        np.testing.assert_allclose(got, want, rtol=1e-15, atol=1e-15)


def test_demote_promote_round_trip(lib):
    rng = np.random.default_rng(9)
    n = 1000
    z = rng.normal(size=n) + 1j * rng.normal(size=n)
    buf = z.copy()
    assert lib.suzerain_blasext_zdemote(n, buf.ctypes.data) == 0
    c64 = np.frombuffer(buf.tobytes()[:n * 8], dtype=np.complex64)
    np.testing.assert_array_equal(c64, z.astype(np.complex64))
    assert lib.suzerain_blasext_zpromote(n, buf.ctypes.data) == 0
    np.testing.assert_array_equal(buf, z.astype(np.complex64).astype(np.complex128))
    r = rng.normal(size=n)
    rb = r.copy()
    assert lib.suzerain_blasext_ddemote(n, rb.ctypes.data) == 0
    assert lib.suzerain_blasext_dpromote(n, rb.ctypes.data) == 0
    np.testing.assert_array_equal(rb, r.astype(np.float32).astype(np.float64))
    assert lib.suzerain_blasext_zdemote(-1, buf.ctypes.data) == -1
    assert lib.suzerain_blasext_zpromote(3, None) == -2


def test_gbnorm1_matches_oracle(lib, oracle):
    rng = np.random.default_rng(13)
    for m, n, kl, ku in ((12, 12, 3, 4), (15, 10, 2, 5), (8, 13, 4, 1)):
        lda = kl + ku + 2
        a = rng.normal(size=lda * n) + 1j * rng.normal(size=lda * n)
        out = C.c_double(-1)
        assert lib.suzerain_blasext_zgbnorm1(m, n, kl, ku, a.ctypes.data, lda,
                                             C.byref(out)) == 0
        assert abs(out.value - oracle.gbnorm1(m, n, kl, ku, a, lda)) <= 1e-14 * out.value
    assert lib.suzerain_blasext_zgbnorm1(4, 4, 1, 1, None, 3, C.byref(out)) == -5
