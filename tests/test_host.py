"""Host-side product code (no GPU): the library loads and exports every
declared symbol; B-spline collocation operators match the reference's golden
bands and SciPy; the synthetic generator is deterministic with the expected
geometry."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b((?:suzerain|sgb)_[A-Za-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(native):
    missing = [n for n in declared_symbols() if not hasattr(native, n)]
    assert not missing, missing
    assert len(declared_symbols()) > 40


def declared_signatures():
    """name -> number of parameters, from the function declarations of the
    public headers (comments removed, one declaration per ';')."""
    out = {}
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b((?:suzerain|sgb)_[A-Za-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_bindings_match_declared_parameter_counts():
    """Every ctypes binding of the package passes as many arguments as the C
    declaration takes (a missing argument would shift every later one)."""
    from suzerain_gb300 import _native as nat
    sigs = declared_signatures()
    assert len(sigs) > 60
    bad = {name: (len(args), sigs[name]) for name, (_, args) in nat._SIGS.items()
           if name in sigs and len(args) != sigs[name]}
    assert not bad, bad
    unbound = [n for n in nat._SIGS if n not in sigs]
    assert not unbound, unbound


def test_construct_q_qinv(native):
    g = native.suzerain_bsmbsm_construct(5, 192, 6, 6)
    assert (g.S, g.n, g.N, g.KL, g.KU, g.LD) == (5, 192, 960, 34, 34, 69)
    d = json.load(open(os.path.join(GOLD, "bsmbsm_kat.json")))
    for i, v in d["q_S5n9"]:
        assert native.suzerain_bsmbsm_q(5, 9, i) == v
    for i, v in d["qinv_S5n9"]:
        assert native.suzerain_bsmbsm_qinv(5, 9, i) == v


def collocation(native, k, bp, nderiv):
    bp = np.ascontiguousarray(bp, dtype=np.float64)
    n, kl, ku = C.c_int(), C.c_int(), C.c_int()
    assert native.sgb_bspline_collocation_bands(k, len(bp), bp.ctypes.data, nderiv,
                                                C.byref(n), C.byref(kl), C.byref(ku),
                                                None, None) == 0
    ld = kl.value + 1 + ku.value
    bands = np.zeros((nderiv + 1) * ld * n.value)
    xi = np.zeros(n.value)
    assert native.sgb_bspline_collocation_bands(k, len(bp), bp.ctypes.data, nderiv,
                                                C.byref(n), C.byref(kl), C.byref(ku),
                                                bands.ctypes.data, xi.ctypes.data) == 0
    return n.value, kl.value, ku.value, bands.reshape(nderiv + 1, n.value, ld), xi


def test_collocation_matches_mathematica_golden(native):
    """k=6 bands of tests/test_bsmbsm.cpp:700-800 (ld 9, kl=ku=4)."""
    d = json.load(open(os.path.join(GOLD, "bsmbsm_kat.json")))
    n, kl, ku, bands, _ = collocation(native, d["k"], d["breakpoints"], 2)
    assert (n, kl, ku) == (10, 4, 4)
    for m, nm in enumerate(("M", "D1", "D2")):
        gold = np.array(d[nm]).reshape(n, 9)
        scale = np.abs(gold).max()
        assert np.allclose(bands[m], gold, rtol=0, atol=1e-13 * scale), nm


def test_bsplineop_workspace_golden_k3(native):
    """tests/test_bsplineop.cpp:465-540: transposed k=3 mass band."""
    d = json.load(open(os.path.join(GOLD, "bsplineop_kat.json")))
    bp = np.array(d["breakpoints"])
    w = native.sgb_bsplineop_alloc_breakpoints(d["k"], len(bp), bp.ctypes.data, 1)
    try:
        ws = w.contents
        assert ws.n == d["n"] and ws.kl[0] == d["kl"] and ws.ku[0] == d["ku"]
        band = np.ctypeslib.as_array(ws.D_T[0], shape=(ws.ld * ws.n,))
        gold = np.array(d["mass_D_T0_band"]).reshape(ws.n, d["ld"])
        got = band.reshape(ws.n, ws.ld)
        # compare the in-band entries (row offsets ku+i-j of each column)
        for j in range(ws.n):
            for i in range(max(0, j - d["ku"]), min(ws.n, j + d["kl"] + 1)):
                assert abs(got[j, ws.ku[0] + i - j] - gold[j, d["ku"] + i - j]) <= 1e3 * np.finfo(float).eps
    finally:
        native.suzerain_bsplineop_free(w)


def test_bsplineop_luz_golden_dense(native, oracle):
    """tests/test_bsplineop.cpp:340-462 restated densely on the host: the
    operator (2-3i) D0 + (7-5i) D1 + (999-999i) D2 of the order-2 basis on
    {0,1,2,3}, from this library's collocation bands, solves the reference's
    right-hand sides to its Octave rationals within its 1e-5 (pins the
    fixture the GPU luz test uses and the oracle's operator restatement)."""
    d = json.load(open(os.path.join(GOLD, "bsplineop_luz_kat.json")))
    bp = np.array(d["breakpoints"])
    w = native.sgb_bsplineop_alloc_breakpoints(d["k"], len(bp), bp.ctypes.data, d["nderiv"])
    try:
        coef = [complex(a, b) for a, b in d["coefficients"]]
        A = oracle.bsplineop_operator(oracle.bsplineop_transposes(w), coef).T
        n = d["n"]
        assert A.shape == (n, n)
        for sv in d["solves"]:
            b = np.array([complex(a, c) for a, c in sv["b"]])
            good = np.array([complex(a, c) for a, c in sv["b_good"]])
            ldb, inc = len(b) // sv["nrhs"], sv["incb"]
            x = b.copy()
            for c in range(sv["nrhs"]):
                s = slice(c * ldb, c * ldb + n * inc, inc)
                x[s] = np.linalg.solve(A, b[s])
            assert np.abs(x - good).max() <= sv["tolerance"]
    finally:
        native.suzerain_bsplineop_free(w)


@pytest.mark.parametrize("Ny,k", [(48, 8), (192, 8), (32, 6), (256, 6)])
def test_collocation_matches_scipy(native, Ny, k):
    interp = pytest.importorskip("scipy.interpolate")
    from suzerain_gb300 import synth
    nbreak = Ny - k + 2
    bp = np.array([2 * native.suzerain_htstretch2(2.0, 1.0, i / (nbreak - 1))
                   for i in range(nbreak)])
    bp[0], bp[-1] = 0.0, 2.0
    n, kl, ku, bands, xi = collocation(native, k, bp, 2)
    assert n == Ny
    assert kl == ku == k - 2
    t = np.concatenate([[bp[0]] * (k - 1), bp, [bp[-1]] * (k - 1)])
    assert np.allclose(xi, [t[i + 1:i + k].mean() for i in range(n)], rtol=0, atol=1e-14)
    ld = kl + 1 + ku
    for m in range(3):
        dense = np.zeros((n, n))
        for j in range(n):
            c = np.zeros(n); c[j] = 1
            sp = interp.BSpline(t, c, k - 1, extrapolate=False)
            vals = sp.derivative(m)(xi) if m else sp(xi)
            dense[:, j] = np.nan_to_num(vals)
        # scipy's right endpoint is open; take the last point from the left
        for j in range(n):
            c = np.zeros(n); c[j] = 1
            sp = interp.BSpline(t, c, k - 1, extrapolate=True)
            dense[-1, j] = (sp.derivative(m) if m else sp)(xi[-1] - 0.0)
        mine = np.zeros((n, n))
        for j in range(n):
            for i in range(max(0, j - ku), min(n, j + kl + 1)):
                mine[i, j] = bands[m, j, ku + i - j]
        scale = np.abs(dense).max()
        assert np.allclose(mine, dense, rtol=0, atol=1e-10 * scale), m
    # the synthetic generator uses exactly these bands
    cs = synth.make_case(S=5, Ny=Ny, k=k)
    assert (cs.kl, cs.ku) == (kl, ku)
    assert np.array_equal(cs.M.reshape(n, ld), bands[0])


def test_synth_deterministic_and_config_geometry(native):
    from suzerain_gb300 import synth
    c0 = synth.CONFIGS[0]
    cs, kx, kz, u = c0.batch()
    cs2, kx2, kz2, u2 = c0.batch()
    assert c0.nsys == 312 and len(kx) == 312 and u.shape == (312, 240)
    assert np.array_equal(u, u2) and np.array_equal(cs.a, cs2.a)
    assert (cs.KL, cs.KU, cs.LD) == (34, 34, 69)
    # wavenumbers: kx = 0.5 m, kz = 1.5 * inorder(24, iz)
    assert np.allclose(kx[:13], 0.5 * np.arange(13))
    assert np.isclose(kz[13 * 13], 1.5 * -11)
    assert abs(u.real.mean()) < 0.05 and abs(u.real.std() - 1) < 0.05
    diag = np.diag(cs.a.reshape(5, 5))
    assert ((diag >= 0.5) & (diag < 1.5)).all()
    off = cs.a.reshape(5, 5)[~np.eye(5, dtype=bool)]
    assert (np.abs(off) <= 0.1).all()
    assert native.suzerain_inorder_wavenumber(24, 13) == -11


def test_solver_spec_grammar_matches_reference_cases(native):
    """The cases of the reference's tests/test_specification_zgbsv.cpp."""
    from suzerain_gb300.plan import SolverSpec, RefineSpec
    d = SolverSpec()
    assert str(d) != "UNKNOWN" and d.method == "zcgbsvx"
    assert (d.aiter, d.siter, d.diter, d.tolsc, d.reuse) == (1, -1, 5, 0.0, False)
    e = SolverSpec(" ")
    assert str(e) not in ("", "UNKNOWN") and e == d
    z = SolverSpec("zgbsv")
    assert z.method == "zgbsv" and str(z) == "zgbsv" and z.in_place()
    x = SolverSpec("zgbsvx")
    assert x.method == "zgbsvx" and str(x) == "zgbsvx,equil=false"
    X = SolverSpec("ZGBSVX,EQUIL=TRUE")
    assert X.method == "zgbsvx" and str(X) == "zgbsvx,equil=true"
    c = SolverSpec("zcgbsvx")
    assert c.method == "zcgbsvx" and str(c) != "zcgbsvx"
    text = "zcgbsvx,reuse=true,aiter=2,siter=3,diter=4,tolsc=5"
    r = SolverSpec(text)
    assert (r.reuse, r.aiter, r.siter, r.diter, r.tolsc) == (True, 2, 3, 4, 5.0)
    assert str(r) == text
    a = SolverSpec("zcgbsvx , reuse = true\t\n,\t\nAITER=\t \t2")
    b = SolverSpec("zcgbsvx,reuse=true,aiter=2")
    cc = SolverSpec("zcgbsvx,aiter=2,reuse=true")
    assert a == b and b == cc and a == cc
    for bad in ("zgbsvq", "zcgbsvx,aiter=2,aiter=3", "zcgbsvx,reuse=maybe", "zgbsv,equil=true",
                "zcgbsvx,tolsc=", "lu"):
        with pytest.raises(ValueError, match="invalid beginning with"):
            SolverSpec(bad)
    rs = RefineSpec.from_string("zcgbsvx,aiter=5,siter=25,diter=5,tolsc=145")
    assert (rs.aiter, rs.siter, rs.diter, rs.tolsc) == (5, 25, 5, 145.0)


def test_cpp_solver_shim_compiles(tmp_path):
    """The header-only C++ solver shim compiles against the C ABI header
    (C++17, warnings as errors)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(root, "include"),
                        os.path.join(root, "tests", "solver_shim_check.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_bsmbsm_permutation_layout(native):
    """suzerain_bsmbsm_permutation: gsl_permutation layout holding q."""
    p = native.suzerain_bsmbsm_permutation(5, 12)
    assert p
    assert p.contents.size == 60
    assert [p.contents.data[i] for i in range(60)] == \
        [native.suzerain_bsmbsm_q(5, 12, i) for i in range(60)]
    native.sgb_permutation_free(p)
    assert not native.suzerain_bsmbsm_permutation(0, 12)


def test_ragged_and_stage_entries_check_arguments(native):
    """The ragged-batch and staged-substep entries reject bad arguments
    before touching the device (host logic, no GPU): null plans and batches,
    empty batches, stages other than 1 and 2, methods other than 'M'."""
    L = native
    assert L.sgb_ragged_create(None, 0, None, None) is None
    assert "sgb_ragged_create" in L.sgb_last_error().decode()
    assert L.sgb_ragged_create(None, 2, None, None) is None
    assert L.sgb_ragged_factor(None, None) != 0
    assert "sgb_ragged_factor" in L.sgb_last_error().decode()
    L.sgb_ragged_destroy(None)                      # no-op
    from suzerain_gb300 import _native as nat
    buf = np.zeros(4, dtype=np.complex128)
    p = buf.ctypes.data
    spec = nat.RefineSpec(5, 25, 5, 145.0)
    for stage, method in ((1, b"M"), (3, b"M"), (1, b"Z")):
        assert L.sgb_plan_substep_stage(None, stage, method, 0.0, 1e-3, p, p, C.byref(spec), None) != 0
        assert "sgb_plan_substep_stage" in L.sgb_last_error().decode()


def test_specialized_switch_and_wide_band_defaults(native):
    """Default factor shapes follow the compile-time-bandwidth instances:
    three warps for a packed complex64 band at KL = KU = 34 with them, two
    without (sgb_gbtrf_set_specialized(0)), four beyond KL = 40; complex128
    keeps one warp up to KL = 52 (host logic, no GPU)."""
    from suzerain_gb300 import tune
    L = native
    try:
        assert L.sgb_gbtrf_set_specialized(0) == 0
        assert tune.get_shape("C", 1920, 34, 34) == (4, 2)
        assert L.sgb_gbtrf_set_shape(b"C", 1920, 34, 34, 4, 3) != 0   # no three-warp shape off
        assert L.sgb_gbtrf_set_specialized(1) == 0
        assert tune.get_shape("C", 1920, 34, 34) == (4, 3)
        assert tune.get_shape("C", 1920, 24, 24) == (4, 3)
        assert tune.get_shape("C", 1344, 48, 48) == (4, 4)
        assert tune.get_shape("C", 1346, 41, 41) == (4, 4)
        assert tune.get_shape("C", 1344, 40, 40) == (4, 2)
        assert tune.get_shape("Z", 1344, 48, 48) == (4, 1)
    finally:
        L.sgb_gbtrf_set_specialized(1)


def test_factor_shape_table(native):
    """The process-wide shape table of the blocked factor (host logic, no
    GPU): built-in defaults per precision, recorded shapes per (precision,
    N, KL, KU), the supported-shape rule (nb 4/8/16, nw 1/2/4, KL within the
    per-warp-count bound, lookahead as nw < 0), and the tuner's probe leaves
    the table as it found it."""
    from suzerain_gb300 import tune

    def get(prec, N, KL, KU):
        return tune.get_shape(prec, N, KL, KU)

    N, KL, KU = 960, 34, 34
    # measured defaults at this geometry (packed band; the complex64 instance
    # with the bandwidths fixed at compile time has a three-warp shape)
    assert get("C", N, KL, KU) == (4, 3)
    assert get("Z", N, KL, KU) == (4, 1)
    assert get("C", 962, KL, KU) == (4, 2)        # N not a multiple of 4: generic
    L = native
    assert L.sgb_gbtrf_set_shape(b"Z", N, KL, KU, 4, 3) != 0    # nw 3: complex64 only
    assert L.sgb_gbtrf_set_shape(b"C", 962, KL, KU, 4, 3) != 0
    assert L.sgb_gbtrf_set_shape(b"C", N, KL, KU, 8, 3) != 0
    assert get("C", 500, 60, 60)[1] == 4          # KL > 56 needs four warps
    geo = (731, 21, 17)                           # a geometry no other test records
    for nb, nw in ((8, 4), (16, 2), (4, -2), (8, -4), (4, 1)):
        tune.set_shape("C", *geo, nb, nw)
        assert get("C", *geo) == (nb, nw)
    assert get("Z", *geo) == (4, 1)               # keyed by precision
    for bad in ((3, 2), (8, 3), (4, 3), (4, -1), (4, -3), (32, 2), (4, 0)):
        assert L.sgb_gbtrf_set_shape(b"C", *geo, *bad) != 0, bad
    assert L.sgb_gbtrf_set_shape(b"X", *geo, 4, 2) != 0
    assert get("C", *geo) == (4, 1)               # rejected calls change nothing
    for nw, kmax in ((1, 52), (2, 56), (4, 63)):   # KL + 1 <= 64 overall
        assert L.sgb_gbtrf_set_shape(b"Z", 400, kmax, 10, 4, nw) == 0
        assert L.sgb_gbtrf_set_shape(b"Z", 400, kmax + 1, 10, 4, nw) != 0
    before = get("C", *geo)
    assert tune._supported(L, b"C", *geo, 16, 4) is True
    assert tune._supported(L, b"C", *geo, 3, 4) is False
    assert get("C", *geo) == before


def test_configuration_geometries():
    """Configurations 1/2 (and the stiff variant) are 129 x 192 = 24,768
    systems of N = 960; configuration 3 draws 64 cases from the stated sets
    (Ny in {32, 48, ..., 256}, k in {6, 8}, S in {5, 7}, (Nx, Nz) in
    {(32, 32), (64, 48), (128, 96)}), deterministically: 172,160 systems over
    44 (S, Ny, k) geometries, each case contributing (Nx/2 + 1) Nz systems."""
    from suzerain_gb300 import synth
    for key in (1, 2, "2stiff"):
        c = synth.CONFIGS[key]
        assert (c.S, c.Ny, c.k, c.nsys) == (5, 192, 8, 24768)
    assert synth.CONFIGS["2stiff"].phi == 5e-2
    cases = synth.config3_cases()
    again = synth.config3_cases()
    assert [(c.S, c.Ny, c.k, c.Nx, c.Nz) for c in cases] == \
        [(c.S, c.Ny, c.k, c.Nx, c.Nz) for c in again]
    assert len(cases) == 64
    assert sum(c.nsys for c in cases) == 172160
    assert len({(c.S, c.Ny, c.k) for c in cases}) == 44
    for c in cases:
        assert c.Ny in range(32, 257, 16) and c.k in (6, 8) and c.S in (5, 7)
        assert (c.Nx, c.Nz) in ((32, 32), (64, 48), (128, 96))
        assert c.nsys == (c.Nx // 2 + 1) * c.Nz


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "suzerain_gb300.h"

int main(void)
{
    suzerain_bsmbsm A = suzerain_bsmbsm_construct(5, 192, 6, 6);
    sgb_solver_spec s;
    char err[256], buf[256];
    int nb = 0, nw = 0;
    double xv[20] = {0}, yv[20] = {0};
    printf("geom %d %d %d %d\n", A.N, A.KL, A.KU, A.LD);
    printf("q %d %d\n", suzerain_bsmbsm_q(5, 192, 7), suzerain_bsmbsm_qinv(5, 192, 193));
    printf("wn %d %d\n", suzerain_inorder_wavenumber(24, 13), suzerain_inorder_wavenumber(24, 12));
    if (sgb_solver_spec_parse("zcgbsvx,aiter=5,siter=25,diter=5,tolsc=145", &s, err, sizeof err))
        return 1;
    sgb_solver_spec_format(&s, buf, sizeof buf);
    printf("spec %s\n", buf);
    printf("bad %d\n", sgb_solver_spec_parse("zcgbsvx,bogus=1", &s, err, sizeof err));
    sgb_gbtrf_get_shape('C', 960, 34, 34, &nb, &nw);
    printf("shape %d %d\n", nb, nw);
    printf("args %d %d %d\n", suzerain_bsmbsm_daPxpby('X', 5, 4, 1.0, xv, 1, 0.0, yv, 1),
           suzerain_bsmbsm_daPxpby('N', 5, 4, 1.0, xv, 1, 0.0, xv, 1),
           suzerain_bsmbsm_zpack(5, 4, 5, 0, 1, 1, 1.0 + 0.5 * I, 0, 3, 9, 9, 0, 19));
    return 0;
}
"""


def test_c99_caller_links_and_calls_the_library(native, tmp_path):
    """A C99 translation unit includes the public header, links the library
    by its C names and calls host-side entry points (geometry, q, wavenumbers,
    the specification grammar, the shape table, argument errors): the
    boundary is a C ABI that the reference's C code can call unchanged."""
    import shutil
    import subprocess
    from suzerain_gb300 import build as B
    if not shutil.which("gcc"):
        pytest.skip("gcc absent")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(B.LIB)
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
           "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-l:" + os.path.basename(B.LIB), "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert out["geom"] == "960 34 34 69"
    assert out["q"] == f"{(7 % 5) * 192 + 7 // 5} {(193 % 192) * 5 + 193 // 192}"
    assert out["wn"] == "-11 12"
    assert out["spec"] == "zcgbsvx,reuse=false,aiter=5,siter=25,diter=5,tolsc=145"
    assert out["bad"] == "-1"
    assert out["shape"] == "4 3"            # packed-band default at this geometry
    assert out["args"] == "1 58 3"          # suzerain/bsmbsm_aPxpby_real.def:47-56, bsmbsm_pack.def:43-64


def test_reference_arm_prints_one_contract_line(native, oracle):
    """bench.py --impl reference (the reference algorithm on the host cores)
    prints one JSON line with the contract's keys, on a small sample."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--ref-sample", "32"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "systems/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1
    for k in ("metric", "n_gpus", "warmup", "ms_per_step", "scaling", "dtype", "data", "config"):
        assert k in d, k
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_plan_memory_estimate(native):
    """sgb_plan_estimate_bytes (host-only; serving admits cases with it) is
    linear in the number of systems, covers both methods when asked for
    both, and bounds the device memory that plans of the benchmark geometry
    actually held on a GB300 from above, by less than 1 KB per plan
    (allocations round up to 256 bytes): 2,144,368,304 bytes for one
    2,048-system plan with 256 complex128 slots, 24,270,595,776 bytes for
    four 6,192-system plans with 512 slots each (method 'M')."""
    from suzerain_gb300 import plan as P, synth
    cs = synth.CONFIGS[2].batch()[0]
    est = P.Plan.estimate_bytes
    for m in ("M", "Z"):
        d1 = est(cs, 2000, 100, m) - est(cs, 1000, 100, m)
        d2 = est(cs, 3000, 100, m) - est(cs, 2000, 100, m)
        assert d1 > 0 and abs(d1 - d2) <= 4096
    assert est(cs, 1000, 1000, "M") > est(cs, 1000, 100, "M")     # complex128 slots
    assert est(cs, 1000, 100, "Z") > est(cs, 1000, 100, "M")      # complex64 factors
    fac_c64 = 8 * native.sgb_factor_elems(cs.N, cs.KL, cs.KU)
    assert est(cs, 1000, 1, "M") > 1000 * fac_c64
    one = est(cs, 2048, 256, "M")
    assert 2_144_368_304 <= one <= 2_144_368_304 + 1024
    four = 4 * est(cs, 6192, 512, "M")
    assert 24_270_595_776 <= four <= 24_270_595_776 + 4 * 1024


def test_htstretch2_matches_reference_formula(native):
    """suzerain_htstretch2(delta, L, x) = (1 + tanh(delta (x/L - 1/2)) /
    tanh(delta/2)) / 2, and x/L for delta = 0 (suzerain/htstretch.c:112-125):
    the stretching of the breakpoints toward both walls."""
    import math
    for delta in (0.0, 0.5, 2.0, 7.0):
        for L in (1.0, 2.0):
            for x in np.linspace(0.0, L, 11):
                got = native.suzerain_htstretch2(delta, L, float(x))
                want = x / L if delta == 0 else \
                    0.5 * (1 + math.tanh(delta * (x / L - 0.5)) / math.tanh(delta / 2.0))
                assert abs(got - want) <= 2e-16 * max(1.0, abs(want)), (delta, L, x)
    assert native.suzerain_htstretch2(2.0, 1.0, 0.0) == 0.0
    assert native.suzerain_htstretch2(2.0, 1.0, 1.0) == 1.0
