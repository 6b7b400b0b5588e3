"""The mixed path's Chebyshev polynomial preconditioner, restated in numpy on the oracle's viscosity matrix (CPU).

cg_mixed_sr_kernel preconditions the CG_nomass solve with M^-1 = P_d(D^-1 V) D^-1, where 1 - lambda P_d(lambda)
is the Chebyshev polynomial of degree d + 1 on [lambda_max / r_d, lambda_max] (r_2 = 30, r_d = 120 for d >= 4)
scaled to 1 at 0, applied as d steps of the Chebyshev iteration for V z = r from z = 0. lambda_max comes from the
Lanczos matrix of a Jacobi-PCG solve (step lengths alpha_i, direction coefficients beta_i). These tests check the algorithm itself on a Kuhn cube's
matrix from the oracle (the reference's NoMass viscosity matrix, rigid modes shifted as the mixed path does):
the Lanczos estimate, positive definiteness for even degrees whatever the estimate, the scale 1 / P_d(0) of the
rigid-mode shift while the polynomial applies, and the iteration counts.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import pyoracle as po
from gen_golden import case_mesh, sheared

def ratio(degree):
    """The interval's width: the kernel's cheb_ratio."""
    return 120.0 if degree > 2 else 30.0


def shifted_system(n=8, seed=21):
    """V (vertex rows), the projected right-hand side, the shifted operator V + s D Z G^-1 Z^T D as a function of
    the shift's scale s, and the rigid modes Z."""
    m = case_mesh(n, seed)
    o = po.OracleBlob(m, solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=0, threads=1)
    o.set_pos(sheared(m, 0.02))
    x0 = o.pos()[:m.n_linear]  # the positions the step's matrix is assembled at: V Z = 0 there
    o.step(1)
    c = o.csr()
    nv = m.n_linear
    rows = np.repeat(np.arange(len(c["key"]) - 1), np.diff(c["key"]))
    V = sp.csr_matrix((c["val"], (rows, c["col"])), shape=(3 * m.n_nodes, 3 * m.n_nodes))[:3 * nv][:, :3 * nv]
    V = V.tocsr()
    f = o.rhs()[:nv].ravel()
    d = x0 - x0.mean(0)
    Z = np.zeros((3 * nv, 6))
    for k in range(3):
        Z[k::3, k] = 1.0
    Z[1::3, 3], Z[2::3, 3] = -d[:, 2], d[:, 1]
    Z[0::3, 4], Z[2::3, 4] = d[:, 2], -d[:, 0]
    Z[0::3, 5], Z[1::3, 5] = -d[:, 1], d[:, 0]
    D = V.diagonal()
    DZ = D[:, None] * Z
    Gi = np.linalg.inv(Z.T @ DZ)
    f = f - DZ @ (Gi @ (Z.T @ f))
    return V, D, f, lambda s: (lambda x: V @ x + s * (DZ @ (Gi @ (DZ.T @ x)))), Z


def chebyshev(V, D, lmax, degree):
    """z = P_d(D^-1 V) D^-1 r by the kernel's recurrence: y0 = D^-1 r / theta, res = D^-1 r - D^-1 V y0, then
    dd = c1 dd + c2 res, z += dd, res -= D^-1 V dd."""
    a, b = lmax / ratio(degree), lmax
    theta, delta = (b + a) / 2, (b - a) / 2
    sigma = theta / delta
    rho = [1 / sigma]
    for _ in range(degree):
        rho.append(1 / (2 * sigma - rho[-1]))

    def apply(r):
        s = r / D
        z = s / theta
        dd = z.copy()
        res = s - (V @ z) / D
        for j in range(degree):
            dd = rho[j + 1] * rho[j] * dd + 2 * rho[j + 1] / delta * res
            z = z + dd
            if j + 1 < degree:
                res = res - (V @ dd) / D
        return z

    return apply


def p_at_zero(lmax, degree):
    """P_d(0) by the kernel's recurrence at lambda = 0, where the residual stays D^-1 r."""
    a, b = lmax / ratio(degree), lmax
    theta, delta = (b + a) / 2, (b - a) / 2
    sigma = theta / delta
    rho, p0 = 1 / sigma, 1 / theta
    d0 = p0
    for _ in range(degree):
        rn = 1 / (2 * sigma - rho)
        d0 = rn * rho * d0 + 2 * rn / delta
        p0 += d0
        rho = rn
    return p0


def pcg(A, f, Minv, eps2=1e-20, imax=5000):
    """Preconditioned CG stopping on |r|^2 < eps2 |f|^2; returns (iterations, step lengths, coefficients)."""
    x = np.zeros_like(f)
    r = f.copy()
    z = Minv(r)
    p = z.copy()
    g = r @ z
    f2 = f @ f
    al, be = [], [0.0]
    for it in range(imax):
        q = A(p)
        a = g / (p @ q)
        al.append(a)
        x += a * p
        r -= a * q
        if r @ r < eps2 * f2:
            return it + 1, al, be
        z = Minv(r)
        gn = r @ z
        be.append(gn / g)
        p = z + (gn / g) * p
        g = gn
    return imax, al, be


def lanczos_max(al, be, n=64):
    n = min(n, len(al))
    T = np.zeros((n, n))
    for i in range(n):
        T[i, i] = 1 / al[i] + (be[i] / al[i - 1] if i > 0 else 0.0)
        if i + 1 < n:
            T[i, i + 1] = T[i + 1, i] = np.sqrt(be[i + 1]) / al[i]
    return float(np.linalg.eigvalsh(T).max())


@pytest.fixture(scope="module")
def system(oracle_built):
    return shifted_system()


def test_lanczos_estimate_of_lambda_max(system):
    V, D, f, A, _ = system
    _, al, be = pcg(A(1.0), f, lambda r: r / D)
    est = lanczos_max(al, be)
    # the largest eigenvalue of D^-1 V (symmetrically scaled), by a dense solve
    Ds = 1 / np.sqrt(D)
    true = float(np.linalg.eigvalsh((sp.diags(Ds) @ V @ sp.diags(Ds)).toarray()).max())
    assert 0.98 * true <= est <= 1.0001 * true


@pytest.mark.parametrize("scale", [0.5, 1.05, 3.0])
def test_even_degrees_stay_positive_definite(system, scale):
    """M^-1 is symmetric positive definite for even degrees even when lambda_max is under- or overestimated."""
    V, D, _, _, _ = system
    Ds = 1 / np.sqrt(D)
    lam = np.linalg.eigvalsh((sp.diags(Ds) @ V @ sp.diags(Ds)).toarray())
    lmax = float(lam.max()) * scale
    for degree in (2, 4, 6, 8):
        M = chebyshev(V, D, lmax, degree)
        Mi = np.column_stack([M(e) for e in np.eye(V.shape[0])[:, :60].T])[:60]
        assert np.allclose(Mi, Mi.T, rtol=1e-9, atol=1e-12 * np.abs(Mi).max())
        # the preconditioner's eigenvalues are P_d(lambda) D^-1: P_d > 0 on the whole spectrum of D^-1 V
        a, b = lmax / ratio(degree), lmax
        x = (b + a - 2 * lam) / (b - a)
        T = np.polynomial.chebyshev.chebval(x, [0] * (degree + 1) + [1])
        T0 = np.polynomial.chebyshev.chebval((b + a) / (b - a), [0] * (degree + 1) + [1])
        P = np.where(lam > 1e-12 * b, (1 - T / T0) / np.maximum(lam, 1e-300), 1.0)
        assert (P > 0).all(), (degree, scale, P.min())


@pytest.mark.parametrize("degree", [2, 4, 6, 8])
def test_p_at_zero(degree):
    """The recurrence's P_d(0) is -R'(0) of the residual polynomial R(lambda) = T_{d+1}(x(lambda)) / T_{d+1}(x(0)),
    x(lambda) = (b + a - 2 lambda) / (b - a)."""
    lmax = 2.5
    a, b = lmax / ratio(degree), lmax
    c = [0] * (degree + 1) + [1]
    x0 = (b + a) / (b - a)
    dT = np.polynomial.chebyshev.chebval(x0, np.polynomial.chebyshev.chebder(c))
    expect = 2 / (b - a) * dT / np.polynomial.chebyshev.chebval(x0, c)
    assert abs(p_at_zero(lmax, degree) - expect) <= 1e-12 * expect


def test_scaled_shift_puts_rigid_modes_at_one(system):
    """M^-1 = P_d(D^-1 V) D^-1 maps D Z c to P_d(0) Z c; with the shift scaled by 1 / P_d(0), M^-1 V~ keeps the
    rigid modes at eigenvalue 1 (unscaled they sit at P_d(0), far outside the cluster near 1)."""
    V, D, f, A, Z = system
    Ds = 1 / np.sqrt(D)
    lmax = 1.05 * float(np.linalg.eigvalsh((sp.diags(Ds) @ V @ sp.diags(Ds)).toarray()).max())
    c = np.random.default_rng(3).standard_normal(6)
    for degree in (2, 4, 8):
        M, p0 = chebyshev(V, D, lmax, degree), p_at_zero(lmax, degree)
        v = Z @ c
        assert np.allclose(M(A(1.0)(v)), p0 * v, rtol=1e-6, atol=1e-9 * p0 * np.abs(v).max())
        assert np.allclose(M(A(1.0 / p0)(v)), v, rtol=1e-6, atol=1e-9 * np.abs(v).max())
        assert p0 > 5


def test_chebyshev_cuts_iterations(system):
    V, D, f, A, _ = system
    it_j, al, be = pcg(A(1.0), f, lambda r: r / D)
    lmax = 1.05 * lanczos_max(al, be)
    its, its_unscaled = {}, {}
    for degree in (2, 4, 6, 8):
        M, p0 = chebyshev(V, D, lmax, degree), p_at_zero(lmax, degree)
        its[degree] = pcg(A(1.0 / p0), f, M)[0]
        its_unscaled[degree] = pcg(A(1.0), f, M)[0]
    print("Jacobi", it_j, "Chebyshev (shift scaled by 1/P(0))", its, "unscaled", its_unscaled)
    assert its[2] <= 0.4 * it_j and its[4] <= 0.25 * it_j and its[6] <= 0.2 * it_j and its[8] <= 0.15 * it_j
    assert all(its[d] <= its_unscaled[d] for d in its)
