"""The allocation-free mixed-precision solve, for hosts that cannot let a
library call cudaMalloc (an application that reserves all device memory in
its own arena, or a time-stepping loop that must stay out of the driver's
allocator).  sgb_zcgbsvx_batched_static must give the results of
sgb_zcgbsvx_batched, call after call, from its fixed static scratch array.

Collected last (file name) so a run that stops at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _band_batch(rng, nsys, n, kl, ku):
    ld = kl + ku + 1
    ab = np.zeros((nsys, ld * n), dtype=np.complex128)
    for s in range(nsys):
        for j in range(n):
            for i in range(max(0, j - ku), min(n, j + kl + 1)):
                ab[s, ku + i - j + j * ld] = complex(rng.normal(), rng.normal())
            ab[s, ku + j * ld] += 4 * ld          # keeps complex64 refinement converging
    return ab, ld


def _solve(native, entry, torch, ab, b, n, kl, ku, ld, spec=(5, 25, 5, 1.0)):
    from suzerain_gb300 import _native as nat
    nsys = b.shape[0]
    dab = torch.from_numpy(ab).cuda()
    db = torch.from_numpy(b).cuda()
    x = torch.zeros_like(db)
    rep = {k: torch.zeros(nsys, dtype=t, device="cuda") for k, t in
           (("info", torch.int32), ("siter", torch.int32), ("diter", torch.int32),
            ("res", torch.float64), ("tolsc", torch.float64), ("fact", torch.uint8))}
    R = nat.RefineReport(*(rep[k].data_ptr() for k in ("info", "siter", "diter", "res", "tolsc", "fact")))
    S = nat.RefineSpec(*spec)
    rc = getattr(native, entry)(nsys, n, kl, ku, b"N", dab.data_ptr(), ld, ld * n, db.data_ptr(),
                                x.data_ptr(), C.byref(S), C.byref(R), 0)
    assert rc == 0, native.sgb_last_error().decode()
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in rep.items()}
    out["x"] = x.cpu().numpy()
    return out


def test_static_entry_matches_allocating_entry_twice(native):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    assert native.sgb_device_ok() == 0, native.sgb_last_error().decode()
    rng = np.random.default_rng(2024)
    nsys, n, kl, ku = 6, 240, 34, 34
    ab, ld = _band_batch(rng, nsys, n, kl, ku)
    for call in range(2):               # two calls in a row share the static array
        b = rng.normal(size=(nsys, n)) + 1j * rng.normal(size=(nsys, n))
        ref = _solve(native, "sgb_zcgbsvx_batched", torch, ab, b, n, kl, ku, ld)
        got = _solve(native, "sgb_zcgbsvx_batched_static", torch, ab, b, n, kl, ku, ld)
        rel = np.max(np.abs(got["x"] - ref["x"])) / np.max(np.abs(ref["x"]))
        assert rel <= 1e-11, (call, rel)
        for k in ("info", "siter", "diter", "fact"):
            assert np.array_equal(got[k], ref[k]), (call, k)
        assert (got["tolsc"] <= 1.0).all()


def test_static_entry_complex128_fallback_matches(native):
    """siter = 0 sends every system to the complex128 fallback, which the
    static scratch serves four systems at a time: the results, two calls in
    a row, are the allocating entry's."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    rng = np.random.default_rng(7)
    nsys, n, kl, ku = 9, 240, 34, 34
    ab, ld = _band_batch(rng, nsys, n, kl, ku)
    for call in range(2):
        b = rng.normal(size=(nsys, n)) + 1j * rng.normal(size=(nsys, n))
        ref = _solve(native, "sgb_zcgbsvx_batched", torch, ab, b, n, kl, ku, ld, (5, 0, 5, 1.0))
        got = _solve(native, "sgb_zcgbsvx_batched_static", torch, ab, b, n, kl, ku, ld,
                     (5, 0, 5, 1.0))
        assert bytes(got["fact"]) == b"D" * nsys, (call, bytes(got["fact"]))
        rel = np.max(np.abs(got["x"] - ref["x"])) / np.max(np.abs(ref["x"]))
        assert rel <= 1e-11, (call, rel)
        for k in ("info", "siter", "diter", "fact"):
            assert np.array_equal(got[k], ref[k]), (call, k)


def test_static_entry_argument_codes_match(native):
    """Both entries return the same negative codes for bad arguments."""
    from suzerain_gb300 import _native as nat
    good = nat.RefineSpec(5, 25, 5, 1.0)
    cases = [(6, 240, 34, 34, b"X", 69, good),                      # trans: -4
             (6, 240, 70, 34, b"N", 105, good),                     # geometry: -5
             (6, 240, 34, 34, b"N", 60, good),                      # ldab: -5
             (6, 240, 34, 34, b"N", 69, nat.RefineSpec(5, 25, 5, -1.0)),   # tolsc: -16
             (6, 240, 34, 34, b"N", 69, nat.RefineSpec(5, -1, -1, 1.0))]   # -99
    want = [-4, -5, -5, -16, -99]
    for (nsys, n, kl, ku, tr, ld, sp), w in zip(cases, want):
        a = native.sgb_zcgbsvx_batched(nsys, n, kl, ku, tr, None, ld, ld * n, None, None,
                                       C.byref(sp), None, 0)
        b = native.sgb_zcgbsvx_batched_static(nsys, n, kl, ku, tr, None, ld, ld * n, None,
                                              None, C.byref(sp), None, 0)
        assert a == b == w, (a, b, w)


def test_static_entry_rejects_oversized_problem(native):
    torch = pytest.importorskip("torch")
    from suzerain_gb300 import _native as nat
    nsys, n, kl, ku = 75, 960, 34, 34      # 67.7 MB of scratch > 64 MiB
    ld = kl + ku + 1
    S = nat.RefineSpec(5, 25, 5, 1.0)
    rc = native.sgb_zcgbsvx_batched_static(nsys, n, kl, ku, b"N", None, ld, ld * n, None, None,
                                           C.byref(S), None, 0)
    assert rc != 0
    msg = native.sgb_last_error().decode()
    assert "static workspace holds" in msg and "need" in msg
