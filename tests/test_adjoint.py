"""Adjoint of a window of CG_nomass steps against central finite differences of the oracle.

The oracle (the C restatement, pinned bit-exact to the reference build) runs the
same window at perturbed parameters; its FP64 trajectories match the GPU FP64
path to CG rounding, so the finite differences of L = sum |x_K - target|^2 are
the reference's derivative. Relative steps of 1e-4 keep the truncation error
(~1e-8) and the CG's own noise (tolerance 1e-10 over the step, ~1e-6) below
the tolerance.

Tolerances (relative, over the sampled components as a vector norm): 1e-4 for the FP64 and the mixed adjoint,
the bound the gradients are specified to. Besides the 3^3-cell cases, the benchmark's differentiated window is
checked at its own mesh size (20^3 cells, 48,000 tets, lognormal per-element moduli) on a shortened window of
20 steps, with the oracle on all host threads (at kT = 0 its threads change only the CG's summation order), a
relative step of 1e-3 and a CG tolerance of 1e-12.
"""
import os
import copy

import numpy as np
import pytest

import pyoracle as po
from ffea_ci_demo_gb300 import lib
from ffea_ci_demo_gb300.mesh import kuhn_cube
from gen_golden import case_mesh, sheared

pytestmark = pytest.mark.gpu

MESO = lib.MESO_LENGTH


def loss_and_grad(x, target):
    d = x - target
    return float((d * d).sum()), 2.0 * d


def oracle_loss(mesh, x0, target, steps, kw, threads=1):
    o = po.OracleBlob(mesh, threads=threads, **kw)
    o.set_pos(x0)
    assert o.step(steps) == 0
    return loss_and_grad(o.pos(), target)[0]


def run_case(mesh, steps, every, precision, kw, samples, seed=5, threads=1, rel_step=1e-4):
    rng = np.random.default_rng(seed)
    x0 = sheared(mesh, 0.02)
    target = x0 + rng.normal(0.0, 0.05, size=x0.shape)
    b = lib.Blob(mesh, solver="CG_nomass", precision=precision, **kw)
    b.set_state(pos=x0)
    adj = lib.Adjoint(b, steps, every)
    assert adj.forward() == steps
    xK = b.pos()
    L, dl = loss_and_grad(xK, target)
    g = lib.meso_to_si_gradients(adj.backward(dl))
    # the blob stays at the end of the window
    assert np.array_equal(b.pos(), xK)
    cols = {"shear_visc": 1, "bulk_visc": 2, "shear_mod": 3, "bulk_mod": 4}
    got, fd = [], []
    for name, e in samples:
        c = cols[name]
        h = rel_step * mesh.material[e, c]
        vals = []
        for sgn in (1, -1):
            m = copy.deepcopy(mesh)
            m.material[e, c] += sgn * h
            vals.append(oracle_loss(m, x0, target, steps, kw, threads))
        fd.append((vals[0] - vals[1]) / (2 * h))
        got.append(g[name][e])
    got, fd = np.array(got), np.array(fd)
    err = np.linalg.norm(got - fd) / np.linalg.norm(fd)
    return err, got, fd


SAMPLES = [("shear_mod", 0), ("shear_mod", 77), ("bulk_mod", 5), ("bulk_mod", 100), ("shear_visc", 3),
           ("shear_visc", 140), ("bulk_visc", 9), ("bulk_visc", 120)]


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-4), ("mixed", 1e-4)])
def test_adjoint_matches_finite_differences_kT0(gpu, oracle_built, precision, tol):
    m = case_mesh(3, 7)
    m.material[:, 3] *= np.random.default_rng(1).lognormal(0.0, 0.3, m.n_elem)
    m.material[:, 4] = 3.9 * m.material[:, 3]
    kw = dict(dt=1e-12, kT=0.0, calc_noise=0, epsilon=1e-10)
    err, got, fd = run_case(m, 12, 5, precision, kw, SAMPLES)
    print(precision, "kT=0 relative error", err, got, fd)
    assert err < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_benchmark_window_size(gpu, oracle_built, precision):
    """The differentiated window's mesh (20^3 cells, lognormal moduli), 20 steps with checkpoints every 5. One
    element's modulus moves the loss by ~1e-11 of itself, so the differences take a relative step of 1e-3 and both
    the oracle's and the GPU's CG solve to |r|/|f| < 1e-12, which keeps the solves' own error below the
    differences' (at 1e-10 it is ~7e-5 of the gradient)."""
    m = kuhn_cube(20, side=100.0, seed=12345)
    rng = np.random.default_rng(2025)
    m.material[:, 3] = rng.lognormal(np.log(5e8), 0.3, m.n_elem)
    m.material[:, 4] = rng.lognormal(np.log(5e8), 0.3, m.n_elem)
    kw = dict(dt=1e-12, kT=0.0, calc_noise=0, epsilon=1e-12)
    samples = [("shear_mod", 17), ("shear_mod", 23456), ("bulk_mod", 401), ("bulk_mod", 40000),
               ("shear_visc", 999), ("shear_visc", 31000), ("bulk_visc", 5), ("bulk_visc", 47000)]
    err, got, fd = run_case(m, 20, 5, precision, kw, samples, threads=os.cpu_count() or 1, rel_step=1e-3)
    print(precision, "20^3 window relative error", err, got, fd)
    assert err < 1e-4


def test_adjoint_with_frozen_noise(gpu, oracle_built):
    """kT > 0: the noise terms' derivatives (sqrt A, sqrt B scaling) with the same draws replayed."""
    m = case_mesh(3, 7)
    kw = dict(dt=1e-12, kT=4.11e-21, calc_noise=1, epsilon=1e-10)
    err, got, fd = run_case(m, 8, 3, "fp64", kw, SAMPLES)
    print("kT>0 relative error", err, got, fd)
    assert err < 1e-4


def test_adjoint_with_pinned_nodes(gpu, oracle_built):
    """One pinned vertex: the rigid modes are the rotations about it (the constraint terms move)."""
    m = case_mesh(3, 7, [0])
    kw = dict(dt=1e-12, kT=0.0, calc_noise=0, epsilon=1e-10)
    err, got, fd = run_case(m, 10, 4, "fp64", kw, SAMPLES)
    print("pinned relative error", err)
    assert err < 1e-4


def test_adjoint_initial_position_gradient(gpu, oracle_built):
    m = case_mesh(3, 7)
    kw = dict(dt=1e-12, kT=0.0, calc_noise=0, epsilon=1e-10)
    rng = np.random.default_rng(3)
    x0 = sheared(m, 0.02)
    target = x0 + rng.normal(0.0, 0.05, size=x0.shape)
    b = lib.Blob(m, solver="CG_nomass", precision="fp64", **kw)
    b.set_state(pos=x0)
    adj = lib.Adjoint(b, 6, 4)
    adj.forward()
    g = adj.backward(loss_and_grad(b.pos(), target)[1])["x0"]
    got, fd = [], []
    for node, c in ((20, 0), (21, 2), (42, 1), (10, 1)):  # vertex nodes (the first (n+1)^3 nodes)
        h = 1e-6 * np.abs(x0).max()
        vals = []
        for sgn in (1, -1):
            xp = x0.copy()
            xp[node, c] += sgn * h
            o = po.OracleBlob(m, threads=1, **kw)
            o.set_pos(xp)
            assert o.step(6) == 0
            vals.append(loss_and_grad(o.pos(), target)[0])
        fd.append((vals[0] - vals[1]) / (2 * h))
        got.append(g[node, c])
    err = np.linalg.norm(np.array(got) - np.array(fd)) / np.linalg.norm(fd)
    print("x0 gradient relative error", err, got, fd)
    assert err < 1e-4


def test_autograd_function(gpu):
    torch = pytest.importorskip("torch")
    from ffea_ci_demo_gb300.autograd import window

    m = case_mesh(2, 11)
    mat = torch.tensor(m.material, dtype=torch.float64, requires_grad=True)
    x0 = torch.tensor(sheared(m, 0.02), dtype=torch.float64, requires_grad=True)
    xk = window(m, mat, x0, 4, 2, dt=1e-12, kT=0.0, calc_noise=0)
    loss = (xk ** 2).sum()
    loss.backward()
    assert mat.grad is not None and x0.grad is not None
    assert torch.isfinite(mat.grad).all() and mat.grad[:, 3].abs().sum() > 0
    assert float(mat.grad[:, 0].abs().sum()) == 0.0  # density does not enter a massless step


def test_autograd_frees_device_memory(gpu, device_free_bytes):
    """The window's blob and checkpoints (its matrix sources alone take 6 MB on this 12^3-cell cube) are freed by
    a forward that needs no gradient (no_grad, or inputs without requires_grad), by the backward pass, and when a
    graph whose backward never ran is dropped: three windows of each kind leave the device's free memory within
    4 MB (the driver's allocation granularity) of where it was."""
    import gc

    torch = pytest.importorskip("torch")
    from ffea_ci_demo_gb300.autograd import window

    m = case_mesh(12, 11)
    kw = dict(dt=1e-12, kT=0.0, calc_noise=0)
    slack = 4 << 20

    def run(grad: bool):
        mat = torch.tensor(m.material, dtype=torch.float64, requires_grad=grad)
        x0 = torch.tensor(sheared(m, 0.02), dtype=torch.float64, requires_grad=grad)
        return window(m, mat, x0, 6, 3, **kw)

    run(True).sum().backward()  # loads the kernels once
    gc.collect()
    base = device_free_bytes()
    for _ in range(3):
        with torch.no_grad():
            run(True)
    assert device_free_bytes() >= base - slack, "a no_grad forward kept device memory"
    for _ in range(3):
        run(False)
    assert device_free_bytes() >= base - slack, "a forward without differentiable inputs kept device memory"
    for _ in range(3):
        run(True).sum().backward()
    gc.collect()
    assert device_free_bytes() >= base - slack, "backward left device memory behind"
    for _ in range(3):
        xk = run(True)
        del xk
    gc.collect()
    assert device_free_bytes() >= base - slack, "dropping the graph left device memory behind"
