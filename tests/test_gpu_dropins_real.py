"""GPU checks of the single-precision and real drop-ins: s/c/cs pack (and
their packc/packf forms) against the d/z/zd ones with exactly representable
scalings, and the real solvers (sgbsv, dgbsv, dsgbsvx) against the complex
ones on the same band with zero imaginary parts, which must agree bit for
bit (the complex kernels keep zero imaginary parts zero)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(native):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    assert native.sgb_device_ok() == 0, native.sgb_last_error().decode()
    return native


def _blocks(S, n, kl, ku, seed):
    rng = np.random.default_rng(seed)
    ld = kl + ku + 1
    return rng.standard_normal((S, S, n * ld)), rng.standard_normal((S, S, n * ld))


@pytest.mark.parametrize("form", ["pack", "packc", "packf"])
def test_single_precision_pack(lib, form):
    from suzerain_gb300 import _native as nat
    S, n, kl, ku = 3, 11, 2, 1
    g = lib.suzerain_bsmbsm_construct(S, n, kl, ku)
    ld, N, KL, KU = g.ld, g.N, g.KL, g.KU
    rows = g.LD + (KL if form == "packf" else 0)
    re, im = _blocks(S, n, kl, ku, 5)
    out = {}
    for kind in ("s", "d", "c", "z", "cs", "zd"):
        cplx = kind in ("c", "z", "cs", "zd")
        single = kind in ("s", "c", "cs")
        tgt = np.full(rows * N, np.nan, dtype=(np.complex64 if single else np.complex128)
                      if cplx else (np.float32 if single else np.float64))
        for i in range(S):
            for j in range(S):
                src = re[i, j] + (1j * im[i, j] if kind in ("c", "z") else 0)
                src = src.astype({"s": np.float32, "d": np.float64, "c": np.complex64,
                                  "z": np.complex128, "cs": np.float32, "zd": np.float64}[kind])
                a = 0.5
                alpha = (C.c_float(a) if kind == "s" else a if kind == "d"
                         else nat.cc(complex(a, 0)) if kind in ("c", "cs") else nat.zc(complex(a, 0)))
                f = getattr(lib, f"suzerain_bsmbsm_{kind}{form}")
                if form == "pack":
                    rc = f(S, n, i, j, kl, ku, alpha, src.ctypes.data, ld, KL, KU,
                           tgt.ctypes.data, rows)
                else:
                    rc = f(C.byref(g), i, j, alpha, src.ctypes.data, tgt.ctypes.data)
                assert rc == 0, (kind, rc)
        out[kind] = tgt
    for lo, hi in (("s", "d"), ("c", "z"), ("cs", "zd")):
        a, b = out[lo], out[hi]
        assert np.array_equal(np.isnan(a), np.isnan(b)), lo
        m = ~np.isnan(b)
        assert np.array_equal(a[m], b[m].astype(a.dtype)), lo


def _band(n, kl, ku, seed, dtype):
    rng = np.random.default_rng(seed)
    ldab = 2 * kl + ku + 1
    ab = np.zeros(ldab * n, dtype=dtype)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[kl + ku + i - j + j * ldab] = rng.standard_normal() + (4.0 if i == j else 0.0)
    return ab


@pytest.mark.parametrize("real,cplx,rt,ct", [("d", "z", np.float64, np.complex128),
                                             ("s", "c", np.float32, np.complex64)])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_real_gbsv_equals_complex(lib, real, cplx, rt, ct, trans):
    n, kl, ku, nrhs = 45, 4, 3, 2
    ab = _band(n, kl, ku, 11, rt)
    b = np.random.default_rng(12).standard_normal(n * nrhs).astype(rt)
    abz, bz = ab.astype(ct), b.astype(ct)
    pr, pz = np.zeros(n, np.int32), np.zeros(n, np.int32)
    fr, fz = C.create_string_buffer(b"N", 1), C.create_string_buffer(b"N", 1)
    ldab = 2 * kl + ku + 1
    assert getattr(lib, f"suzerain_lapackext_{real}gbsv")(
        C.addressof(fr), trans.encode(), n, kl, ku, nrhs, ab.ctypes.data, ldab,
        pr.ctypes.data, b.ctypes.data, n) == 0
    assert getattr(lib, f"suzerain_lapackext_{cplx}gbsv")(
        C.addressof(fz), trans.encode(), n, kl, ku, nrhs, abz.ctypes.data, ldab,
        pz.ctypes.data, bz.ctypes.data, n) == 0
    assert fr.raw == fz.raw == b"F"
    assert np.array_equal(pr, pz)
    assert np.array_equal(b, bz.real) and not bz.imag.any()
    assert np.array_equal(ab, abz.real)


def test_dsgbsvx_equals_zcgbsvx(lib):
    n, kl, ku = 60, 5, 5
    ldab = kl + ku + 1
    full = _band(n, kl, ku, 21, np.float64)
    ab = np.zeros(ldab * n)
    for j in range(n):
        ab[j * ldab:(j + 1) * ldab] = full[kl + j * (2 * kl + ku + 1): kl + j * (2 * kl + ku + 1) + ldab]
    b = np.random.default_rng(22).standard_normal(n)
    outs = []
    for real in (True, False):
        dt = np.float64 if real else np.complex128
        a_, b_ = ab.astype(dt), b.astype(dt)
        x, r = np.zeros(n, dt), np.zeros(n, dt)
        afb = np.zeros((2 * kl + ku + 1) * n, dt)
        ipiv = np.zeros(n, np.int32)
        fact = C.create_string_buffer(b"N", 1)
        apprx, afrob = C.c_int(0), C.c_double(-1)
        si, di, ts, res = C.c_int(25), C.c_int(5), C.c_double(1.0), C.c_double(0)
        f = lib.suzerain_lapackext_dsgbsvx if real else lib.suzerain_lapackext_zcgbsvx
        info = f(C.addressof(fact), C.addressof(apprx), 5, b"N", n, kl, ku, a_.ctypes.data,
                 C.addressof(afrob), afb.ctypes.data, ipiv.ctypes.data, b_.ctypes.data,
                 x.ctypes.data, C.addressof(si), C.addressof(di), C.addressof(ts),
                 r.ctypes.data, C.addressof(res))
        outs.append(dict(info=info, fact=fact.raw, x=x, r=r, ipiv=ipiv, si=si.value,
                         di=di.value, res=res.value, afb=afb))
    d, z = outs
    assert d["info"] == z["info"] == 0
    assert d["fact"] == z["fact"] and d["si"] == z["si"] and d["di"] == z["di"]
    assert np.array_equal(d["x"], z["x"].real) and not z["x"].imag.any()
    assert np.array_equal(d["r"], z["r"].real)
    assert np.array_equal(d["ipiv"], z["ipiv"])
    assert d["res"] == z["res"]
    if d["fact"] == b"S":   # float32 factor at the start of afb
        f32 = d["afb"].view(np.float32)[:(2 * kl + ku + 1) * n]
        c64 = z["afb"].view(np.complex64)[:(2 * kl + ku + 1) * n]
        assert np.array_equal(f32, c64.real)
