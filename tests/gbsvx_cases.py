"""Seeded band systems for the zgbsvx parity tests: random complex bands
(diagonally weighted), optionally with rows and columns scaled over many
decades so that equilibration engages, a structurally singular case, and
the comparison rules shared by the oracle pin and the GPU parity tests."""
import numpy as np

# (n, kl, ku): scalar, small, the reference's kl/ku edge cases, and a BSMBSM
# geometry (S = 5, n = 12, kl = ku = 3 gives N = 60, KL = KU = 19)
GEOMS = [(1, 0, 0), (7, 2, 3), (40, 5, 4), (33, 0, 5), (25, 6, 0), (60, 19, 19)]


def band(n, kl, ku, seed, scaled=False, singular_col=None):
    """Returns (ab, A): ab the (kl+ku+1) x n band flattened column-major."""
    rng = np.random.default_rng(seed)
    A = np.zeros((n, n), complex)
    for i in range(n):
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            A[i, j] = rng.standard_normal() + 1j * rng.standard_normal()
        A[i, i] += 2.0 * (kl + ku + 1)
    if scaled:
        A = (10.0 ** rng.uniform(-6, 6, n))[:, None] * A
        A = A * (10.0 ** rng.uniform(-3, 3, n))[None, :]
    if singular_col is not None:
        A[:, singular_col] = 0
    ab = np.zeros((kl + ku + 1, n), complex)
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[ku + i - j, j] = A[i, j]
    return ab.reshape(-1, order="F"), A


def rhs(n, nrhs, seed):
    rng = np.random.default_rng(seed + 7919)
    return rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))


# Tolerances of the floating-point outputs (the integer and scaling outputs
# -- info, equed, r, c, the scaled band and right-hand side, ipiv -- must be
# identical):
#   x       normwise, relative to ||x|| max, within 64 eps * max(1, 1/rcond)
#   rcond   relative 1e-8 (the estimator takes the same path; its sums differ
#           in rounding only)
#   ferr    within a factor of 2 (a bound made of rounding-level residuals)
#   berr    both at most nz * eps, nz = min(kl+ku+2, n+1)
#   rpvgrw  relative 1e-12
EPS = 2.0 ** -53


def assert_close(got, want, n, kl, ku, what=""):
    assert got["info"] == want["info"], (what, got["info"], want["info"])
    assert got["equed"] == want["equed"], (what, got["equed"], want["equed"])
    if want["equed"] in "RB":
        np.testing.assert_array_equal(got["r"], want["r"], err_msg=what)
    if want["equed"] in "CB":
        np.testing.assert_array_equal(got["c"], want["c"], err_msg=what)
    np.testing.assert_array_equal(got["ab"], want["ab"], err_msg=what)
    np.testing.assert_array_equal(np.asarray(got["b"]).reshape(n, -1),
                                  np.asarray(want["b"]).reshape(n, -1), err_msg=what)
    assert abs(got["rpvgrw"] - want["rpvgrw"]) <= 1e-12 * want["rpvgrw"], what
    solved = want["info"] == 0 or want["info"] == n + 1
    if not solved:
        assert got["rcond"] == 0 and want["rcond"] == 0, what
        return
    assert abs(got["rcond"] - want["rcond"]) <= 1e-8 * want["rcond"], \
        (what, got["rcond"], want["rcond"])
    x, xw = np.asarray(got["x"]).reshape(n, -1), np.asarray(want["x"]).reshape(n, -1)
    tol = 64 * EPS * max(1.0, 1.0 / want["rcond"])
    for j in range(xw.shape[1]):
        err = np.abs(x[:, j] - xw[:, j]).max() / np.abs(xw[:, j]).max()
        assert err <= tol, (what, j, err, tol)
    nz = min(kl + ku + 2, n + 1)
    fe, fw = np.asarray(got["ferr"]), np.asarray(want["ferr"])
    assert np.all(fe <= 2 * fw) and np.all(fw <= 2 * fe), (what, fe, fw)
    assert np.all(np.asarray(got["berr"]) <= nz * EPS), (what, got["berr"])
    assert np.all(np.asarray(want["berr"]) <= nz * EPS), (what, want["berr"])
