"""ROCK2 against its definition, independently of the tabulated recurrence.

The kernels and the oracle both run the stage recurrence with the tabulated
(mu, nu, kappa) of csrc/rock2_table.h.  Here the step is computed a second
way, from the published construction of the method (Abdulle & Medovikov
2001) only:

  R_s(z) = w(z) P_{s-2}(x) / P_{s-2}(1),  x = 1 + 2 z / l_s,

with w(z) = 1 + 2 sigma z + tau z^2 and P_n the polynomial orthogonal on
[-1, 1] with respect to w(x)^2 / sqrt(1 - x^2).  P_n is found by solving its
orthogonality conditions in the Chebyshev basis (Gauss-Chebyshev
quadrature, exact for these polynomial integrands) in 40-digit arithmetic,
not with the generator's Stieltjes recurrence; the table supplies only l_s, sigma and tau, which the
order-condition test in test_host.py pins.  R_s(h A_z) u is then evaluated
by an eigendecomposition of the column's z-operator A_z (symmetrised with
the diagonal that makes the tridiagonal A_z symmetric), and compared with
the oracle's stage loop (ogw_rock2_step, the recurrence the GPU kernels
run and are checked against).  An error in any tabulated recurrence
coefficient changes R_s and fails this test."""
import numpy as np
import pytest

from geothermalwells_gb300 import rock2
from geothermalwells_gb300 import workloads as W
import oracle as O


mpmath = pytest.importorskip("mpmath")
MP = mpmath.mp.clone() if hasattr(mpmath.mp, "clone") else mpmath.mp
DPS = 40   # digits: the orthogonality system has condition ~1e5 at s = 40


def cheb_orthogonal_poly(n, a, b):
    """Chebyshev coefficients c_0..c_n (c_n = 1), in 40-digit arithmetic, of
    the polynomial orthogonal to T_0..T_{n-1} w.r.t.
    ((x-a)^2+b^2)^2/sqrt(1-x^2): the Gram system of its orthogonality
    conditions on M Gauss-Chebyshev nodes (exact for degree < 2M)."""
    with mpmath.workdps(DPS):
        a, b = mpmath.mpf(a), mpmath.mpf(b)
        M = n + 16
        xs = [mpmath.cos((2 * m - 1) * mpmath.pi / (2 * M)) for m in range(1, M + 1)]
        T = [[mpmath.cos(k * mpmath.acos(x)) for k in range(n + 1)] for x in xs]
        W2 = [((x - a) ** 2 + b ** 2) ** 2 for x in xs]
        G = mpmath.matrix(n, n)
        rhs = mpmath.matrix(n, 1)
        for j in range(n):
            for k in range(j, n):
                v = mpmath.fsum(W2[m] * T[m][j] * T[m][k] for m in range(M))
                G[j, k] = G[k, j] = v
            rhs[j] = -mpmath.fsum(W2[m] * T[m][j] * T[m][n] for m in range(M))
        c = mpmath.lu_solve(G, rhs)
        return [c[k] for k in range(n)] + [mpmath.mpf(1)]


def chebval_mp(x, c):
    """Clenshaw sum of the Chebyshev series c at x (mpmath)."""
    b1 = b2 = mpmath.mpf(0)
    for ck in reversed(c[1:]):
        b1, b2 = 2 * x * b1 - b2 + ck, b1
    return x * b1 - b2 + c[0]


def R_direct(s, z):
    """R_s(z) from (l_s, sigma, tau) and the orthogonality conditions."""
    l = rock2.stability_interval(s)
    _, _, _, sigma, tau = rock2.coefficients(s)
    zs = np.atleast_1d(np.asarray(z, dtype=float))
    n = s - 2
    out = np.empty(zs.shape)
    with mpmath.workdps(DPS):
        l_, sg, ta = mpmath.mpf(l), mpmath.mpf(sigma), mpmath.mpf(tau)
        # w in the x variable: ((x-a)^2+b^2)/w1 with w1 = 4/(l^2 tau), 1-a = sigma l w1/2
        w1 = 4 / (l_ * l_ * ta)
        one_minus_a = sg * l_ * w1 / 2
        c = cheb_orthogonal_poly(n, 1 - one_minus_a, mpmath.sqrt(w1 - one_minus_a ** 2)) if n > 0 else None
        p1 = chebval_mp(mpmath.mpf(1), c) if n > 0 else None
        for q, zq in enumerate(zs):
            zm = mpmath.mpf(float(zq))
            w = 1 + 2 * sg * zm + ta * zm * zm
            out[q] = float(w if n == 0 else w * chebval_mp(1 + 2 * zm / l_, c) / p1)
    return out if np.ndim(z) else float(out[0])


def column_operator(orc, w, j, i):
    """A_z of column (j, i) as a dense nz x nz matrix, from the oracle's
    rhs_diffusion_z applied to unit vectors (every column holds e_k)."""
    nz = len(w["gridz"])
    shape = w["T0"].shape
    A = np.zeros((nz, nz))
    for k in range(nz):
        phi = np.zeros(shape, order="F")
        phi[k, :, :] = 1.0
        d = np.zeros(shape, order="F")
        orc.rhs_diffusion_z(d, phi)
        A[:, k] = d[:, j, i]
    return A


def apply_R(A, s, h, u):
    """R_s(h A) u by the symmetrised eigendecomposition of tridiagonal A."""
    n = A.shape[0]
    assert np.all(np.abs(np.triu(A, 2)) == 0) and np.all(np.abs(np.tril(A, -2)) == 0)
    up, lo = np.diag(A, 1), np.diag(A, -1)
    assert np.all(up * lo > 0)
    d = np.ones(n)
    for k in range(n - 1):
        d[k + 1] = d[k] * np.sqrt(up[k] / lo[k])      # D A D^-1 symmetric
    B = (d[:, None] * A) / d[None, :]
    B = 0.5 * (B + B.T)
    lam, V = np.linalg.eigh(B)
    r = R_direct(s, h * lam)
    return (V @ (r * (V.T @ (d * u)))) / d, lam


@pytest.fixture(scope="module")
def case():
    w = W.small_case(n_layers=3, nz_cells=40)
    orc = O.Oracle(w["gridx"], w["gridy"], w["gridz"], w["boreholes"], w["materials"],
                   w["inlet_model"])
    yield w, orc
    orc.close()


def test_direct_polynomial_matches_order_conditions():
    for s in (3, 10, 40):
        z = np.array([-1e-3, 1e-3])
        R = R_direct(s, z)
        # R(z) = 1 + z + z^2/2 + O(z^3)
        assert np.allclose(R, 1 + z + z * z / 2, rtol=0, atol=1e-9)
        assert abs(R_direct(s, 0.0) - 1.0) < 1e-13


@pytest.mark.parametrize("s", [3, 10, 40])
@pytest.mark.parametrize("frac", [0.7, 0.95])
@pytest.mark.parametrize("where", ["pipe", "rock"])
def test_oracle_rock2_step_is_R_s(s, frac, where, case):
    """One oracle ROCK2 step equals R_s(h A_z) u on a column through the pipe
    (water, steel, grout and rock levels) and a column of plain layered rock,
    with h rho(A_z) at 0.7 and 0.95 of the stability interval l_s."""
    w, orc = case
    shape = w["T0"].shape
    ny, nx = shape[1], shape[2]
    if where == "pipe":
        i = int(np.argmin(np.abs(w["gridx"] - w["boreholes"][0].xc)))
        j = int(np.argmin(np.abs(w["gridy"] - w["boreholes"][0].yc)))
    else:
        i, j = 0, 0
    A = column_operator(orc, w, j, i)
    lam_max = np.max(np.abs(np.linalg.eigvals(A)))
    h = frac * rock2.stability_interval(s) / lam_max
    rng = np.random.default_rng(11 + s)
    u = np.asfortranarray(rng.uniform(-5.0, 5.0, shape))
    want, lam = apply_R(A, s, h, u[:, j, i].copy())
    assert np.isclose(np.max(np.abs(lam)), lam_max, rtol=1e-9)
    got = u.copy(order="F")
    orc.rock2_step(got, h, s, rock2.coefficients(s))
    err = np.max(np.abs(got[:, j, i] - want)) / np.max(np.abs(u[:, j, i]))
    # the oracle's s-stage recurrence runs in double: its own rounding grows
    # with the stage count (2.7e-12 measured at s = 40); a wrong digit in any
    # tabulated coefficient moves R_s by far more
    assert err < (1e-12 if s <= 10 else 1e-11), err


@pytest.mark.parametrize("which", ["mu", "nu", "kappa"])
def test_a_wrong_coefficient_is_caught(which, case):
    """The comparison detects a relative error of 1e-8 in one tabulated
    recurrence coefficient (planted in the coefficients the oracle gets)."""
    w, orc = case
    s = 10
    shape = w["T0"].shape
    A = column_operator(orc, w, 0, 0)
    h = 0.7 * rock2.stability_interval(s) / np.max(np.abs(np.linalg.eigvals(A)))
    u = np.asfortranarray(np.random.default_rng(5).uniform(-5.0, 5.0, shape))
    want, _ = apply_R(A, s, h, u[:, 0, 0].copy())
    mu, nu, kappa, sigma, tau = rock2.coefficients(s)
    bad = {"mu": mu.copy(), "nu": nu.copy(), "kappa": kappa.copy()}
    bad[which][3] *= 1.0 + 1e-8
    got = u.copy(order="F")
    orc.rock2_step(got, h, s, (bad["mu"], bad["nu"], bad["kappa"], sigma, tau))
    err = np.max(np.abs(got[:, 0, 0] - want)) / np.max(np.abs(u[:, 0, 0]))
    assert err > 1e-11, err
