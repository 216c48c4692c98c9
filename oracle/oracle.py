"""ORACLE — test infrastructure, not product code.

ctypes access to
  * oracle/_lib/liboracle.so   the C restatement of the reference's banded
                               solve path (oracle/oracle.c), and
  * oracle/_ref/libsuzref.so   the reference's own C sources of that path
                               compiled against SciPy's OpenBLAS
                               (oracle/ref/Makefile), present only where the
                               reference checkout was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, always as the checker.  Nothing in suzerain_gb300/ uses it.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsuzref.so")
# the seeded input generator alone (host C++, no CUDA): lets a CPU-only
# process make the benchmark inputs without loading the GPU library
SYNTH_PATH = os.path.join(HERE, "_lib", "libsynth.so")

_i = C.c_int
_d = C.c_double
_p = C.c_void_p
_cp = C.c_char_p


class _Z(C.Structure):
    """C99 double complex passed by value."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def _z(v) -> _Z:
    v = complex(v)
    return _Z(v.real, v.imag)


def reference_dir() -> str | None:
    """The reference checkout the reference build reads: the environment
    variable SUZERAIN_REFERENCE_DIR, else the default of the build recipe
    (oracle/ref/Makefile); None when that directory is absent."""
    d = os.environ.get("SUZERAIN_REFERENCE_DIR")
    if not d:
        r = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "print-ref"],
                           capture_output=True, text=True)
        d = r.stdout.strip() if r.returncode == 0 else ""
    return d if d and os.path.isdir(os.path.join(d, "suzerain")) else None


def build(quiet: bool = True) -> None:
    """Compile oracle.c and the host-only generator (always) and the
    reference build (when the reference checkout is present)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE], check=True, stdout=out, stderr=out)
    ref = reference_dir()
    if ref:
        subprocess.run(["make", "-C", HERE, "ref", f"REF={ref}"], check=True, stdout=out,
                       stderr=out)


def openblas_path() -> str | None:
    """SciPy's bundled OpenBLAS, located by glob (x86 here, aarch64 on Grace)."""
    try:
        import scipy
    except ImportError:  # pragma: no cover
        return None
    pats = [os.path.join(os.path.dirname(scipy.__file__) + ".libs",
                         "libscipy_openblas*.so"),
            os.path.join(os.path.dirname(scipy.__file__), ".dylibs",
                         "libscipy_openblas*")]
    for pat in pats:
        hits = sorted(glob.glob(pat))
        if hits:
            return hits[0]
    return None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_q.argtypes = [_i, _i, _i]
        L.orc_qinv.argtypes = [_i, _i, _i]
        L.orc_zaPxpby.argtypes = [C.c_char, _i, _i, _Z, _p, _i, _Z, _p, _i]
        L.orc_zpack.argtypes = [_i] * 6 + [_Z, _p, _i, _i, _i, _p, _i]
        L.orc_zdpack.argtypes = [_i] * 6 + [_Z, _p, _i, _i, _i, _p, _i]
        for f in ("orc_builtin_zgbtrf", "orc_builtin_cgbtrf", "orc_zgbtrf",
                  "orc_cgbtrf"):
            getattr(L, f).argtypes = [_i, _i, _i, _p, _i, _p]
        for f in ("orc_builtin_zgbtrs", "orc_builtin_cgbtrs", "orc_zgbtrs",
                  "orc_cgbtrs"):
            getattr(L, f).argtypes = [C.c_char, _i, _i, _i, _i, _p, _i, _p,
                                      _p, _i]
        L.orc_zgbmv.argtypes = [C.c_char, _i, _i, _i, _i, _Z, _p, _i, _p, _i,
                                _Z, _p, _i]
        L.orc_dznrm2.argtypes = [_i, _p]
        L.orc_dznrm2.restype = _d
        L.orc_zlangb_fro.argtypes = [_i, _i, _i, _p, _i]
        L.orc_zlangb_fro.restype = _d
        L.orc_zcgbsvx.argtypes = [_p, _p, _i, C.c_char, _i, _i, _i, _p, _p,
                                  _p, _p, _p, _p, _p, _p, _p, _p, _p]
        L.orc_use_openblas.argtypes = [_cp]
        gbsvx_args = [C.c_char, C.c_char, _i, _i, _i, _i, _p, _i, _p, _i, _p,
                      _p, _p, _p, _p, _i, _p, _i, _p, _p, _p, _p]
        L.orc_zgbsvx.argtypes = gbsvx_args
        L.orc_openblas_zgbsvx.argtypes = [_cp] + gbsvx_args
        L.orc_assemble_packed.argtypes = [_i, _i, _i, _i, _p, _p, _p, _i, _p,
                                          _p, _p, _p, _p, _i, _i]
        L.orc_block_coefs.argtypes = [_i, _p, _p, _p, _p, _d, _d, _d, _p, _p,
                                      _p]
        L.orc_batch_solve.argtypes = (
            [_i, _i, _i, _i, _i, C.c_char, _p, _p, _p, _i, _p, _p, _p, _p, _p,
             _p, _p, _d, _d, _p, _p, _p, _i, _i, _i, _i, _d, _p, _p, _p, _p,
             _p, _p, _i])
        L.orc_batch_solve.restype = _d
        _lib = L
    return _lib


def ref():
    """The reference's own compiled C, or None when it was not built here."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            return None
        L = C.CDLL(REF_PATH)
        L.suzerain_bsmbsm_zaPxpby.argtypes = [C.c_char, _i, _i, _Z, _p, _i,
                                              _Z, _p, _i]
        L.suzerain_bsmbsm_zpack.argtypes = [_i] * 6 + [_Z, _p, _i, _i, _i, _p,
                                                       _i]
        L.suzerain_bsmbsm_zdpack.argtypes = [_i] * 6 + [_Z, _p, _i, _i, _i,
                                                        _p, _i]
        L.suzerain_bsmbsm_dpack.argtypes = [_i] * 6 + [_d, _p, _i, _i, _i, _p,
                                                       _i]
        L.suzerain_lapack_zgbtrf.argtypes = [_i, _i, _i, _i, _p, _i, _p]
        L.suzerain_lapack_cgbtrf.argtypes = [_i, _i, _i, _i, _p, _i, _p]
        L.suzerain_lapack_zgbtrs.argtypes = [C.c_char, _i, _i, _i, _i, _p, _i,
                                             _p, _p, _i]
        L.suzerain_lapackext_zgbsv.argtypes = [_p, C.c_char, _i, _i, _i, _i,
                                               _p, _i, _p, _p, _i]
        L.suzerain_lapackext_zcgbsvx.argtypes = [_p, _p, _i, C.c_char, _i, _i,
                                                 _i, _p, _p, _p, _p, _p, _p,
                                                 _p, _p, _p, _p, _p]
        L.suzerain_blas_zgbmv.argtypes = [C.c_char, _i, _i, _i, _i, _Z, _p,
                                          _i, _p, _i, _Z, _p, _i]
        for k in range(1, 6):
            for sfx in ("dzz", "ddz"):
                f = getattr(L, f"oracle_ref_gbd{k}mv_{sfx}")
                f.argtypes = [C.c_char, _i, _i, _i] + [_Z, _p, _i] * k + [_p, _i, _p, _i,
                                                                          _Z, _p, _i]
                f.restype = _i
        dw = [_i, _i, _Z, _p, _d, _d, _i, _i, _i, _i, _i, _i, _i, _i, _i]
        L.suzerain_diffwave_apply.argtypes = dw
        L.suzerain_diffwave_apply.restype = None
        L.suzerain_diffwave_accumulate.argtypes = dw[:4] + [_Z, _p] + dw[4:]
        L.suzerain_diffwave_accumulate.restype = None
        L.oracle_ref_single_thread()
        _ref = L
    return _ref


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# --------------------------------------------------------------------------
# Pythonic helpers over the restatement
# --------------------------------------------------------------------------
def bsmbsm(S: int, n: int, kl: int, ku: int) -> dict:
    """Geometry of suzerain_bsmbsm_construct (suzerain/bsmbsm.h:130-149)."""
    KL = S * (kl + 1) - 1
    KU = S * (ku + 1) - 1
    return dict(S=S, n=n, kl=kl, ku=ku, ld=kl + 1 + ku, N=S * n, KL=KL, KU=KU,
                LD=KL + 1 + KU)


def q(S, n, i):
    return lib().orc_q(S, n, i)


def qinv(S, n, i):
    return lib().orc_qinv(S, n, i)


def zaPxpby(trans, S, n, alpha, x, incx, beta, y, incy) -> int:
    return lib().orc_zaPxpby(trans.encode(), S, n, _z(alpha), _ptr(x), incx,
                             _z(beta), _ptr(y), incy)


def zgbtrf(ab: np.ndarray, n, kl, ku, ldab, builtin=True):
    """In-place band LU; returns (info, ipiv 1-based)."""
    ipiv = np.zeros(n, dtype=np.int32)
    f = lib().orc_builtin_zgbtrf if builtin else lib().orc_zgbtrf
    info = f(n, kl, ku, _ptr(ab), ldab, _ptr(ipiv))
    return info, ipiv


def cgbtrf(ab: np.ndarray, n, kl, ku, ldab, builtin=True):
    ipiv = np.zeros(n, dtype=np.int32)
    f = lib().orc_builtin_cgbtrf if builtin else lib().orc_cgbtrf
    info = f(n, kl, ku, _ptr(ab), ldab, _ptr(ipiv))
    return info, ipiv


def zgbtrs(trans, ab, n, kl, ku, ldab, ipiv, b, builtin=True) -> int:
    nrhs = 1 if b.ndim == 1 else b.shape[1]
    f = lib().orc_builtin_zgbtrs if builtin else lib().orc_zgbtrs
    bb = np.asfortranarray(b)
    info = f(trans.encode(), n, kl, ku, nrhs, _ptr(ab), ldab, _ptr(ipiv),
             _ptr(bb), n)
    b[...] = bb
    return info


def cgbtrs(trans, ab, n, kl, ku, ldab, ipiv, b, builtin=True) -> int:
    nrhs = 1 if b.ndim == 1 else b.shape[1]
    f = lib().orc_builtin_cgbtrs if builtin else lib().orc_cgbtrs
    bb = np.asfortranarray(b)
    info = f(trans.encode(), n, kl, ku, nrhs, _ptr(ab), ldab, _ptr(ipiv),
             _ptr(bb), n)
    b[...] = bb
    return info


def zgbmv(trans, m, n, kl, ku, alpha, a, lda, x, beta, y) -> int:
    return lib().orc_zgbmv(trans.encode(), m, n, kl, ku, _z(alpha), _ptr(a),
                           lda, _ptr(x), 1, _z(beta), _ptr(y), 1)


def zcgbsvx(ab, n, kl, ku, b, trans="N", aiter=5, siter=25, diter=5,
            tolsc=1.0):
    """Restated suzerain_lapackext_zcgbsvx with fact='N'.  Returns dict."""
    ldafb = 2 * kl + ku + 1
    fact = C.create_string_buffer(b"N", 1)
    apprx = C.c_int(0)
    afrob = C.c_double(-1)
    afb = np.zeros(ldafb * n, dtype=np.complex128)
    ipiv = np.zeros(n, dtype=np.int32)
    x = np.zeros(n, dtype=np.complex128)
    r = np.zeros(n, dtype=np.complex128)
    si, di = C.c_int(siter), C.c_int(diter)
    ts, res = C.c_double(tolsc), C.c_double(0)
    bb = np.ascontiguousarray(b, dtype=np.complex128)
    info = lib().orc_zcgbsvx(C.addressof(fact), C.addressof(apprx), aiter,
                             trans.encode(), n, kl, ku, _ptr(ab),
                             C.addressof(afrob), _ptr(afb), _ptr(ipiv),
                             _ptr(bb), _ptr(x), C.addressof(si),
                             C.addressof(di), C.addressof(ts), _ptr(r),
                             C.addressof(res))
    return dict(info=info, fact=fact.raw.decode(), x=x, r=r, siter=si.value,
                diter=di.value, tolsc=ts.value, res=res.value,
                afrob=afrob.value)


def zgbsvx(ab, n, kl, ku, b, trans="N", fact="E", afb=None, ipiv=None,
           equed="N", r=None, c=None, ldab=None, openblas=False):
    """Restated LAPACK zgbsvx (or, with openblas=True, SciPy's OpenBLAS
    zgbsvx itself) on copies of the inputs.  ab: band with rows 0..kl+ku
    (ldab rows, column-major flat); b: n x nrhs (or n).  For fact 'F' pass
    the afb (ldafb = 2kl+ku+1), ipiv, equed, r, c of an earlier call.
    Returns a dict with every output."""
    ldab = ldab or kl + ku + 1
    ldafb = 2 * kl + ku + 1
    ab = np.array(ab, dtype=np.complex128).reshape(-1).copy()
    bb = np.array(b, dtype=np.complex128)
    nrhs = 1 if bb.ndim == 1 else bb.shape[1]
    bb = np.asfortranarray(bb.reshape(n, nrhs)).copy(order="F")
    x = np.zeros((n, nrhs), dtype=np.complex128, order="F")
    afb = (np.zeros(ldafb * n, dtype=np.complex128) if afb is None
           else np.array(afb, dtype=np.complex128).reshape(-1).copy())
    ipiv = (np.zeros(n, dtype=np.int32) if ipiv is None
            else np.array(ipiv, dtype=np.int32).copy())
    r = np.zeros(n) if r is None else np.array(r, dtype=np.float64).copy()
    c = np.zeros(n) if c is None else np.array(c, dtype=np.float64).copy()
    eq = C.create_string_buffer(equed.encode(), 1)
    rcond, rpv = C.c_double(0), C.c_double(0)
    ferr = np.zeros(nrhs)
    berr = np.zeros(nrhs)
    args = [fact.encode(), trans.encode(), n, kl, ku, nrhs, _ptr(ab), ldab,
            _ptr(afb), ldafb, _ptr(ipiv), C.addressof(eq), _ptr(r), _ptr(c),
            _ptr(bb), n, _ptr(x), n, C.addressof(rcond), _ptr(ferr),
            _ptr(berr), C.addressof(rpv)]
    if openblas:
        path = openblas_path()
        info = lib().orc_openblas_zgbsvx(path.encode() if path else None,
                                         *args)
        if info == -1000:
            return None
    else:
        info = lib().orc_zgbsvx(*args)
    return dict(info=info, x=x, ab=ab, afb=afb, ipiv=ipiv,
                equed=eq.raw.decode(), r=r, c=c, b=bb, rcond=rcond.value,
                ferr=ferr, berr=berr, rpvgrw=rpv.value)


def assemble_packed(S, n, kl, ku, M, D1, D2, ld, cM, cD1, cD2, dirichlet,
                    layout="packc"):
    """Packed P A P^T (complex128, column-major band) of one synthetic system.

    layout 'packc': LD rows; 'packf': LD + KL rows with A at row offset KL.
    """
    g = bsmbsm(S, n, kl, ku)
    rows = g["LD"] if layout == "packc" else g["LD"] + g["KL"]
    off = 0 if layout == "packc" else g["KL"]
    papt = np.full(rows * g["N"], np.nan, dtype=np.complex128)
    dm = np.ascontiguousarray(dirichlet, dtype=np.int32)
    lib().orc_assemble_packed(S, n, kl, ku, _ptr(M), _ptr(D1), _ptr(D2), ld,
                              _ptr(np.ascontiguousarray(cM, np.complex128)),
                              _ptr(np.ascontiguousarray(cD1, np.complex128)),
                              _ptr(np.ascontiguousarray(cD2, np.complex128)),
                              _ptr(dm), _ptr(papt), rows, off)
    return papt


def block_coefs(case, phi, kx, kz):
    """(cM, cD1, cD2), each (S, S) complex128, of one wavenumber pair."""
    S = case.S
    out = np.zeros((3, S, S), dtype=np.complex128)
    lib().orc_block_coefs(S, _ptr(case.a), _ptr(case.b), _ptr(case.c),
                          _ptr(case.g), float(phi), float(kx), float(kz),
                          _ptr(out[0]), _ptr(out[1]), _ptr(out[2]))
    return out[0], out[1], out[2]


def dirichlet_flags(case) -> np.ndarray:
    return np.array([(case.dirichlet_mask >> e) & 1 for e in range(case.S)],
                    dtype=np.int32)


def batch_solve(case, kx, kz, u, phi_exp=0.0, phi_imp=1e-3, trans="N",
                mixed=False, aiter=5, siter=25, diter=5, tolsc=1.0,
                nthreads=1, openblas=False):
    """One synthetic substep for every system on host threads.

    case: a suzerain_gb300.synth.SynthCase (bands + coefficients).  u: (nsys,
    N) complex128 natural-order input; with phi_exp != 0 the right-hand side
    is the explicit operator applied to u (wall rows zeroed), else u itself.
    Returns dict with x (natural order), info, wall seconds and, for the mixed
    path, per-system siter/diter/res/tolsc/fact and latencies.
    """
    L = lib()
    if openblas:
        path = openblas_path()
        if path is None or L.orc_use_openblas(path.encode()) != 0:
            raise RuntimeError("SciPy OpenBLAS not loadable for the oracle")
    else:
        L.orc_use_openblas(None)
    u = np.ascontiguousarray(u, dtype=np.complex128)
    nsys, N = u.shape
    kx = np.ascontiguousarray(kx, dtype=np.float64)
    kz = np.ascontiguousarray(kz, dtype=np.float64)
    x = np.zeros_like(u)
    info = np.zeros(nsys, dtype=np.int32)
    so = np.zeros(nsys, dtype=np.int32)
    do = np.zeros(nsys, dtype=np.int32)
    ro = np.zeros(nsys)
    to = np.zeros(nsys)
    fo = np.zeros(nsys, dtype=np.uint8)
    lat = np.zeros(nsys)
    dm = dirichlet_flags(case)
    wall = L.orc_batch_solve(nsys, case.S, case.n, case.kl, case.ku,
                             trans.encode(), _ptr(case.M), _ptr(case.D1),
                             _ptr(case.D2), case.ld, _ptr(case.a),
                             _ptr(case.b), _ptr(case.c), _ptr(case.g),
                             _ptr(dm), _ptr(kx), _ptr(kz), float(phi_exp),
                             float(phi_imp), _ptr(u), _ptr(x), _ptr(info),
                             int(mixed), aiter, siter, diter, float(tolsc),
                             _ptr(so), _ptr(do), _ptr(ro), _ptr(to), _ptr(fo),
                             _ptr(lat), int(nthreads))
    if openblas:
        L.orc_use_openblas(None)
    return dict(x=x, info=info, wall=wall, siter=so, diter=do, res=ro,
                tolsc=to, fact=fo.tobytes().decode(errors="replace"),
                latency=lat)


def assemble_case(case, phi, kx, kz, layout="packc"):
    """Packed P A P^T of one system of a synthetic case."""
    cM, cD1, cD2 = block_coefs(case, phi, kx, kz)
    return assemble_packed(case.S, case.n, case.kl, case.ku, case.M, case.D1,
                           case.D2, case.ld, cM, cD1, cD2,
                           dirichlet_flags(case), layout=layout)


# --------------------------------------------------------------------------
# Dense helpers for checks (small sizes only)
# --------------------------------------------------------------------------
def gbdmv(trans, n, kl, ku, alphas, ds, ldds, a, lda, x, beta, y) -> np.ndarray:
    """y <- (sum_t alpha_t D_t) op(A) x + beta y on logical (unit-stride)
    vectors, D_t[i] = ds[t][i*ldds[t]], A the real n x n band in BLAS storage,
    op(A) = A for 'N' and A^T for 'T' and 'C' (A is real); beta = 0 ignores
    y, and all-zero alphas leave beta y.  The operator of
    suzerain/blas_et_al/gbdmv.def ... gbdddddmv.def
    (suzerain/blas_et_al/gbddmv.def:131-190 for two diagonals)."""
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            A[i, j] = a[ku + i - j + j * lda]
    base = np.zeros(n, complex) if beta == 0 else beta * np.asarray(y, complex)
    if all(al == 0 for al in alphas):
        return base
    c = sum(al * d[np.arange(n) * l] for al, d, l in zip(alphas, ds, ldds))
    op = A if trans.upper() == "N" else A.T
    return base + c * (op @ x)


def diffwave_factors(dxcnt, dzcnt, alpha, Lx, Lz, Nx, dNx, dkbx, dkex, Nz, dNz,
                     dkbz, dkez) -> np.ndarray:
    """Per-mode factor alpha (i 2 pi m / Lx)^dxcnt (i 2 pi n / Lz)^dzcnt of the
    in-order modes dkbz..dkez-1 (rows) x dkbx..dkex-1 (columns), 0 where the
    mode is dropped: a differentiated direction keeps the wavenumbers that
    suzerain_inorder_wavenumber_diff maps to nonzero, an undifferentiated one
    those with |k| <= (N-1)/2 (suzerain/diffwave.c:66-131,
    suzerain/inorder.h:92-96, :112-116, :145-149, :282-296)."""
    def wabs(N, i):
        return i if i < N // 2 + 1 else N - i

    def wdiff(N, dN, i):
        return i if i < (N + 1) // 2 else (-dN + i if i >= dN - (N - 1) // 2 else 0)

    f = np.zeros((dkez - dkbz, dkex - dkbx), complex)
    for n in range(dkbz, dkez):
        nf = wdiff(Nz, dNz, n) if dzcnt else 0
        if not (nf != 0 if dzcnt else wabs(dNz, n) <= (Nz - 1) // 2):
            continue
        for m in range(dkbx, dkex):
            mf = wdiff(Nx, dNx, m) if dxcnt else 0
            if mf != 0 if dxcnt else wabs(dNx, m) <= (Nx - 1) // 2:
                f[n - dkbz, m - dkbx] = (alpha * (1j * 2 * np.pi / Lz * nf) ** dzcnt
                                         * (1j * 2 * np.pi / Lx * mf) ** dxcnt)
    return f


def diffwave_apply(dxcnt, dzcnt, alpha, x, Lx, Lz, Nx, dNx, dkbx, dkex, Nz, dNz,
                   dkbz, dkez) -> np.ndarray:
    """x (Z, X, Y in C order: Y fastest) scaled mode by mode."""
    f = diffwave_factors(dxcnt, dzcnt, alpha, Lx, Lz, Nx, dNx, dkbx, dkex, Nz, dNz, dkbz, dkez)
    return np.where(f[..., None] != 0, x * f[..., None], 0)


def diffwave_accumulate(dxcnt, dzcnt, alpha, x, beta, y, Lx, Lz, Nx, dNx, dkbx, dkex,
                        Nz, dNz, dkbz, dkez) -> np.ndarray:
    """alpha D x + beta y, beta y on dropped modes (suzerain/diffwave.c:132-198)."""
    return diffwave_apply(dxcnt, dzcnt, alpha, x, Lx, Lz, Nx, dNx, dkbx, dkex, Nz, dNz,
                          dkbz, dkez) + beta * y


def band_to_dense(ab, n, kl, ku, ldab, off=0):
    """Dense A from column-major band storage with A(i,j) at
    ab[off + ku + i - j + j*ldab]."""
    A = np.zeros((n, n), dtype=ab.dtype)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            A[i, j] = ab[off + ku + i - j + j * ldab]
    return A


def rel_resid(A_apply, x, b):
    """Normwise backward error ||b-Ax||inf / (||A||inf ||x||inf + ||b||inf)
    where A_apply = (callable y=A@x, ||A||inf)."""
    apply, anorm = A_apply
    r = b - apply(x)
    return np.max(np.abs(r)) / (anorm * np.max(np.abs(x)) + np.max(np.abs(b)))


# --------------------------------------------------------------------------
# Band assembly helpers of blas_et_al (numpy restatements, pinned against the
# reference build in tests/test_oracle.py)
# --------------------------------------------------------------------------
def gb_diag_scale_acc(side, m, n, kl, ku, alphas, ds, ldds, a, inca, lda, beta, b, incb, ldb):
    """B <- A (sum_k alpha_k D_k) + beta B ('R') or (sum_k alpha_k D_k) A +
    beta B ('L') on flat band storage, element (i, j) at (ku+i-j) inc + j ld
    (suzerain/blas_et_al/blasext.c:2070-2500).  Returns the new b."""
    b = np.array(b, dtype=np.complex128, copy=True)
    beta = complex(beta)
    if all(complex(al) == 0 for al in alphas) and beta == 1 or m <= 0 or n <= 0:
        return b
    # side 'L' walks rows 0..n-1 and columns 0..m-1 (the reference recasts a
    # left scaling as a traversal by rows without exchanging m and n)
    rows, cols = (n, m) if side.upper() == "L" else (m, n)
    for j in range(cols):
        for i in range(max(0, j - ku), min(rows, j + kl + 1)):
            s = i if side.upper() == "L" else j
            tmp = sum(complex(al) * d[s * l] for al, d, l in zip(alphas, ds, ldds))
            av = a[(ku + i - j) * inca + j * lda]
            ib = (ku + i - j) * incb + j * ldb
            if beta == 1:
                b[ib] += tmp * av
            elif beta == 0:
                b[ib] = tmp * av
            else:
                b[ib] = b[ib] * beta + tmp * av
    return b


def gbnorm1(m, n, kl, ku, a, lda):
    """Maximum column sum of |a_ij| of a complex band (blasext.c:2741-2778)."""
    best = 0.0
    for j in range(n):
        lo, hi = max(0, ku - j), ku + min(kl + 1, m - j)
        best = max(best, float(np.sum(np.abs(a[j * lda + lo:j * lda + hi]))))
    return best


def zcgbsvx_call(fn, ab, n, kl, ku, b, state, trans="N", aiter=5, siter=25, diter=5,
                 tolsc=1.0):
    """One call of any zcgbsvx implementation with the reference's 18
    arguments (this restatement's orc_zcgbsvx, the reference build's
    suzerain_lapackext_zcgbsvx, or a drop-in of it), carrying the caller's
    state across calls the way bsmbsm_solver_zcgbsvx does
    (suzerain/bsmbsm_solver.cpp:377-414): state holds fact, apprx, afb and
    ipiv and is updated in place.  Returns the call's outputs."""
    ldafb = 2 * kl + ku + 1
    if "afb" not in state:
        state.update(fact="N", apprx=0, afb=np.zeros(ldafb * n, np.complex128),
                     ipiv=np.zeros(n, np.int32))
    fact = C.create_string_buffer(state["fact"].encode(), 1)
    apprx = C.c_int(int(state["apprx"]))
    afrob = C.c_double(-1)
    x = np.zeros(n, np.complex128)
    r = np.zeros(n, np.complex128)
    si, di = C.c_int(siter), C.c_int(diter)
    ts, res = C.c_double(tolsc), C.c_double(0)
    abc = np.ascontiguousarray(ab, dtype=np.complex128).copy()
    bb = np.ascontiguousarray(b, dtype=np.complex128).copy()
    info = fn(C.addressof(fact), C.addressof(apprx), C.c_int(aiter), C.c_char(trans.encode()),
              C.c_int(n), C.c_int(kl), C.c_int(ku), C.c_void_p(abc.ctypes.data),
              C.addressof(afrob), C.c_void_p(state["afb"].ctypes.data),
              C.c_void_p(state["ipiv"].ctypes.data), C.c_void_p(bb.ctypes.data),
              C.c_void_p(x.ctypes.data), C.addressof(si), C.addressof(di), C.addressof(ts),
              C.c_void_p(r.ctypes.data), C.addressof(res))
    state["fact"] = fact.raw.decode()
    state["apprx"] = apprx.value
    return dict(info=info, fact=state["fact"], apprx=apprx.value, siter=si.value,
                diter=di.value, tolsc=ts.value, res=res.value, x=x)


def reuse_sequence(fn, n=120, kl=7, ku=5, seed=77):
    """A series of slightly (then strongly) changed bands solved with the
    factor of the first reused as an approximate factor, as a solver with
    the reuse=true specification does: call 0 factors (fact 'N'), calls 1-2
    reuse it for perturbed bands (apprx set), call 3 perturbs enough that
    refinement stalls and the approximate factor is replaced, call 4
    supplies the complex128 factor of a call that ran with siter < 0
    (fact 'D').  Returns the per-call outputs."""
    rng = np.random.default_rng(seed)
    ld = kl + ku + 1
    base = np.zeros(ld * n, np.complex128)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            base[ku + i - j + j * ld] = complex(rng.normal(), rng.normal())
        base[ku + j * ld] += 3 * ld
    noise = rng.normal(size=ld * n) + 1j * rng.normal(size=ld * n)
    mask = base != 0
    bands = [base, base + 1e-3 * noise * mask, base + 3e-3 * noise * mask,
             base + 0.6 * ld * noise * mask]
    rhs = [rng.normal(size=n) + 1j * rng.normal(size=n) for _ in range(5)]
    state = {}
    out = []
    for k, (band, b) in enumerate(zip(bands, rhs)):
        if k > 0:
            state["apprx"] = 1                    # the factor is of an earlier band
        out.append(zcgbsvx_call(fn, band, n, kl, ku, b, state, aiter=3, siter=25, diter=5,
                                tolsc=1.0))
    # fact 'D': factor in complex128 (siter < 0), then reuse that factor
    dstate = {}
    out.append(zcgbsvx_call(fn, bands[1], n, kl, ku, rhs[4], dstate, siter=-1, diter=5))
    dstate["apprx"] = 1
    out.append(zcgbsvx_call(fn, bands[2], n, kl, ku, rhs[4], dstate, siter=-1, diter=5))
    return out


# ---- B-spline operators and their workspaces (suzerain/bsplineop.c) -------

def bsplineop_transposes(w) -> list[np.ndarray]:
    """Dense D_m^T, m = 0..nderiv, from a workspace's transposed bands (the
    layout of suzerain/bsplineop.h:125-180: (i, j) of D_m^T at
    D_T[m][ku[m] + i - j + j ld])."""
    ws = w.contents
    n, ld = ws.n, ws.ld
    out = []
    for m in range(ws.nderiv + 1):
        kl, ku = ws.kl[m], ws.ku[m]
        t = np.zeros((n, n))
        for j in range(n):
            for i in range(max(0, j - ku), min(n, j + kl + 1)):
                t[i, j] = ws.D_T[m][ku + i - j + j * ld]
        out.append(t)
    return out


def bsplineop_accumulate(DT: np.ndarray, alpha, x, beta, y):
    """y <- alpha D x + beta y with D = DT^T ('T' band product of the stored
    transpose, suzerain/bsplineop.c:222-298); beta 0 ignores y."""
    ax = alpha * (DT.T @ x)
    return ax if beta == 0 else beta * y + ax


def bsplineop_operator(DTs: list[np.ndarray], coefficients, scale=0.0, prior=None):
    """The transpose A^T of the operator an opaccumulate call leaves:
    sum_k c_k D_k^T plus scale times the prior transpose
    (suzerain/bsplineop.c:976-1040, 1325-1380)."""
    acc = sum(c * t for c, t in zip(coefficients, DTs))
    if prior is not None and scale != 0:
        acc = acc + scale * prior
    return acc


def band_of(A: np.ndarray, kl: int, ku: int, ld: int, off: int = 0) -> np.ndarray:
    """The (kl, ku) band of a dense matrix in LAPACK storage with leading
    dimension ld, starting at row off (gbtrf storage: off = kl)."""
    n = A.shape[1]
    ab = np.zeros((n, ld), dtype=A.dtype)
    for j in range(n):
        for i in range(max(0, j - ku), min(A.shape[0], j + kl + 1)):
            ab[j, off + ku + i - j] = A[i, j]
    return ab.reshape(-1)
