"""GPU parity of the zgbsvx expert driver (batched C entry point and the
suzerain_lapack_zgbsvx drop-in) against the oracle's restatement, which
tests/test_oracle.py pins to LAPACK's own zgbsvx.  Bars in gbsvx_cases:
info, equed, r, c, the scaled band and right-hand side identical; x, rcond,
ferr, berr, rpvgrw within the stated tolerances; pivots identical."""
import ctypes as C

import numpy as np
import pytest

from gbsvx_cases import GEOMS, assert_close, band, rhs

pytestmark = pytest.mark.gpu


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


def _systems(n, kl, ku, nsys, base):
    """nsys bands: plain and scaled alternate; the last one has a zero
    column when n > 4."""
    out = []
    for s in range(nsys):
        sing = n // 2 if (s == nsys - 1 and n > 4) else None
        out.append(band(n, kl, ku, seed=base + s, scaled=bool(s % 2), singular_col=sing)[0])
    return out


def _run_batched(lib, torch, fact, trans, n, kl, ku, bands, b, afb=None, ipiv=None,
                 equed=None, r=None, c=None):
    nsys, ld, ldf = len(bands), kl + ku + 1, 2 * kl + ku + 1
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()
    d_ab = t(np.stack(bands), np.complex128)
    d_afb = t(afb if afb is not None else np.zeros((nsys, ldf * n)), np.complex128)
    d_piv = t(ipiv if ipiv is not None else np.zeros((nsys, n)), np.int32)
    d_eq = t(np.frombuffer((equed or "N" * nsys).encode(), np.uint8).copy(), np.uint8)
    d_r = t(r if r is not None else np.zeros((nsys, n)), np.float64)
    d_c = t(c if c is not None else np.zeros((nsys, n)), np.float64)
    d_b = t(b, np.complex128)
    d_x = torch.zeros(nsys, n, dtype=torch.complex128, device="cuda")
    scal = torch.zeros(4, nsys, dtype=torch.float64, device="cuda")
    info = torch.zeros(nsys, dtype=torch.int32, device="cuda")
    p = lambda x: x.data_ptr()
    rc = lib.sgb_zgbsvx_batched(fact.encode(), trans.encode(), nsys, n, kl, ku, p(d_ab), ld,
                                ld * n, p(d_afb), ldf, ldf * n, p(d_piv), p(d_eq), p(d_r),
                                p(d_c), p(d_b), p(d_x), p(scal[0]), p(scal[1]), p(scal[2]),
                                p(scal[3]), p(info), None)
    assert rc == 0, lib.sgb_last_error().decode()
    torch.cuda.synchronize()
    h = lambda x: x.cpu().numpy()
    sc = h(scal)
    eqs = bytes(h(d_eq)).decode()
    return [dict(info=int(h(info)[s]), equed=eqs[s], r=h(d_r)[s], c=h(d_c)[s], ab=h(d_ab)[s],
                 b=h(d_b)[s], x=h(d_x)[s], rcond=sc[0, s], ferr=sc[1, s:s + 1],
                 berr=sc[2, s:s + 1], rpvgrw=sc[3, s], afb=h(d_afb)[s], ipiv=h(d_piv)[s])
            for s in range(nsys)]


@pytest.mark.parametrize("n,kl,ku", GEOMS)
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("fact", ["N", "E"])
def test_zgbsvx_batched_matches_oracle(lib, oracle, torch_cuda, n, kl, ku, trans, fact):
    nsys = 6
    bands = _systems(n, kl, ku, nsys, base=1000 * n + 10 * kl + ku)
    b = np.stack([rhs(n, 1, 500 + s)[:, 0] for s in range(nsys)])
    got = _run_batched(lib, torch_cuda, fact, trans, n, kl, ku, bands, b)
    for s in range(nsys):
        want = oracle.zgbsvx(bands[s], n, kl, ku, b[s], trans=trans, fact=fact)
        what = f"system {s} ({n},{kl},{ku}) {fact}{trans}"
        assert_close(got[s], want, n, kl, ku, what)
        np.testing.assert_array_equal(got[s]["ipiv"], want["ipiv"], err_msg=what)
        scale = max(1.0, np.abs(want["afb"]).max())
        assert np.abs(got[s]["afb"] - want["afb"]).max() <= 1e-12 * scale, what
        if want["info"] not in (0, n + 1):
            assert not got[s]["x"].any(), what     # x untouched


@pytest.mark.parametrize("trans", ["N", "T", "C"])
def test_zgbsvx_batched_fact_f(lib, oracle, torch_cuda, trans):
    """fact 'F': factor, pivots, equed, r, c of an earlier 'E' call."""
    n, kl, ku, nsys = 60, 19, 19, 4
    bands = [band(n, kl, ku, seed=77 + s, scaled=True)[0] for s in range(nsys)]
    b = np.stack([rhs(n, 1, 900 + s)[:, 0] for s in range(nsys)])
    first = _run_batched(lib, torch_cuda, "E", "N", n, kl, ku, bands, b)
    b2 = np.stack([rhs(n, 1, 950 + s)[:, 0] for s in range(nsys)])
    got = _run_batched(lib, torch_cuda, "F", trans, n, kl, ku, [f["ab"] for f in first], b2,
                       afb=np.stack([f["afb"] for f in first]),
                       ipiv=np.stack([f["ipiv"] for f in first]),
                       equed="".join(f["equed"] for f in first),
                       r=np.stack([f["r"] for f in first]), c=np.stack([f["c"] for f in first]))
    for s in range(nsys):
        f = first[s]
        want = oracle.zgbsvx(f["ab"], n, kl, ku, b2[s], trans=trans, fact="F", afb=f["afb"],
                             ipiv=f["ipiv"], equed=f["equed"], r=f["r"], c=f["c"])
        assert_close(got[s], want, n, kl, ku, f"F{trans} system {s}")


def test_dropin_zgbsvx(lib, oracle):
    """suzerain_lapack_zgbsvx with host buffers, several right-hand sides,
    padded leading dimensions; 'E' then 'F' as bsmbsm_solver_zgbsvx calls it."""
    n, kl, ku, nrhs = 60, 19, 19, 3
    ld, ldab, ldafb, ldb = kl + ku + 1, kl + ku + 3, 2 * kl + ku + 2, n + 5
    ab0, _ = band(n, kl, ku, seed=31, scaled=True)
    ab = np.zeros((n, ldab), complex)
    ab[:, :ld] = ab0.reshape(n, ld)
    ab = ab.reshape(-1)
    b0 = rhs(n, nrhs, 31)
    b = np.zeros((nrhs, ldb), complex)
    b[:, :n] = b0.T
    b = b.reshape(-1)
    x = np.zeros(nrhs * ldb, complex)
    afb = np.zeros(ldafb * n, complex)
    ipiv = np.zeros(n, np.int32)
    eq = C.create_string_buffer(b"N", 1)
    r, c = np.zeros(n), np.zeros(n)
    rcond = C.c_double(0)
    ferr, berr = np.zeros(nrhs), np.zeros(nrhs)
    work, rwork = np.zeros(2 * n, complex), np.zeros(n)

    def call(fact, trans):
        return lib.suzerain_lapack_zgbsvx(fact, trans, n, kl, ku, nrhs, ab.ctypes.data, ldab,
                                          afb.ctypes.data, ldafb, ipiv.ctypes.data,
                                          C.addressof(eq), r.ctypes.data, c.ctypes.data,
                                          b.ctypes.data, ldb, x.ctypes.data, ldb,
                                          C.addressof(rcond), ferr.ctypes.data,
                                          berr.ctypes.data, work.ctypes.data, rwork.ctypes.data)

    def view():
        return dict(ab=ab.reshape(n, ldab)[:, :ld].reshape(-1).copy(),
                    b=b.reshape(nrhs, ldb)[:, :n].T.copy(), x=x.reshape(nrhs, ldb)[:, :n].T.copy(),
                    afb=afb.reshape(n, ldafb)[:, :2 * kl + ku + 1].reshape(-1).copy(),
                    ipiv=ipiv.copy(), equed=eq.raw.decode(), r=r.copy(), c=c.copy(),
                    rcond=rcond.value, ferr=ferr.copy(), berr=berr.copy(), rpvgrw=rwork[0])

    info = call(b"E", b"N")
    got = dict(info=info, **view())
    want = oracle.zgbsvx(ab0, n, kl, ku, b0, trans="N", fact="E")
    assert_close(got, want, n, kl, ku, "E")
    np.testing.assert_array_equal(got["ipiv"], want["ipiv"])
    # second solve with the factor: fact 'F', transposed, new right-hand sides
    b1 = rhs(n, nrhs, 32)
    b.reshape(nrhs, ldb)[:, :n] = b1.T
    info = call(b"F", b"C")
    got = dict(info=info, **view())
    want = oracle.zgbsvx(want["ab"], n, kl, ku, b1, trans="C", fact="F", afb=want["afb"],
                         ipiv=want["ipiv"], equed=want["equed"], r=want["r"], c=want["c"])
    assert_close(got, want, n, kl, ku, "F")
    # argument errors follow zgbsvx's numbering
    assert lib.suzerain_lapack_zgbsvx(b"X", b"N", n, kl, ku, 1, ab.ctypes.data, ldab,
                                      afb.ctypes.data, ldafb, ipiv.ctypes.data, C.addressof(eq),
                                      r.ctypes.data, c.ctypes.data, b.ctypes.data, ldb,
                                      x.ctypes.data, ldb, C.addressof(rcond), ferr.ctypes.data,
                                      berr.ctypes.data, None, None) == -1
    assert lib.suzerain_lapack_zgbsvx(b"N", b"N", n, kl, ku, 1, ab.ctypes.data, kl + ku,
                                      afb.ctypes.data, ldafb, ipiv.ctypes.data, C.addressof(eq),
                                      r.ctypes.data, c.ctypes.data, b.ctypes.data, ldb,
                                      x.ctypes.data, ldb, C.addressof(rcond), ferr.ctypes.data,
                                      berr.ctypes.data, None, None) == -8
