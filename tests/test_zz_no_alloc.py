"""ffea_gpu_blob_solve_static: the Jacobi-PCG solve with its work arrays in the
library's static device scratch (no allocation per call), through the C ABI.

The reference entry point it is checked against is the regular step
(ffea_gpu_blob_step): after one step the blob holds the force vector it solved
(ffea_gpu_blob_get_rhs) and the matrix it solved with, and the solution sits in
the velocities (CG_nomass: v = x; CG from rest: v = x dt, src/Blob.cpp:3249-3279).
Solving the same force again with the static-scratch entry point must give the
same solution: the same kernel runs with the same grid and the same opening
sums, so the tolerance (1e-12 of the largest component) only covers the
velocity's dt scaling on the CG solver. Two calls in a row check that the
scratch left by one call does not leak into the next.
"""
import ctypes as C

import numpy as np
import pytest

from ffea_ci_demo_gb300 import lib
from gen_golden import case_mesh, sheared

pytestmark = pytest.mark.gpu


def solve_static(L, blob, rhs, out=None):
    x = np.full_like(rhs, np.nan) if out is None else out
    it = C.c_int(-1)
    rc = L.ffea_gpu_blob_solve_static(blob._h, rhs.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p),
                                      C.byref(it))
    return rc, x, it.value


@pytest.mark.parametrize("solver,dt", [("CG_nomass", 1e-12), ("CG", 1e-14)])
def test_static_solve_matches_step(gpu, solver, dt):
    L = lib.load()
    m = case_mesh(6, 12345)
    b = lib.Blob(m, solver=solver, dt=dt, kT=4.11e-21, calc_noise=1)
    b.set_state(pos=sheared(m, 0.02))
    b.update(1)
    f = b.rhs()
    dt_meso = lib.make_params(solver=solver, dt=dt).dt
    ref = b.vel() if solver == "CG_nomass" else b.vel() / dt_meso
    iters = b.cg_iterations()[0]
    scale = np.abs(ref).max()
    assert scale > 0
    first = None
    for call in range(2):
        rc, x, it = solve_static(L, b, f)
        assert rc == lib.OK, lib.last_error()
        assert it == iters, (call, it, iters)
        err = np.abs(x - ref).max() / scale
        print(f"{solver} call {call}: {it} iterations, max error {err:.3e} of max |x|")
        assert err <= 1e-12, (call, err)
        if first is None:
            first = x.copy()
        else:
            assert np.array_equal(x, first)
    # in place (rhs and x the same array), as the reference's solve(std::vector<arr3>&)
    g = f.copy()
    rc, x, _ = solve_static(L, b, g, out=g)
    assert rc == lib.OK and np.array_equal(x, first)


def test_static_solve_rejects_what_does_not_fit(gpu):
    L = lib.load()
    m = case_mesh(2, 11)
    bm = lib.Blob(m, solver="CG_nomass", precision="mixed", kT=0.0, calc_noise=0)
    rc, _, _ = solve_static(L, bm, np.zeros((m.n_nodes, 3)))
    assert rc == lib.EINPUT and "FP64" in lib.last_error()
    bl = lib.Blob(m, solver="masslumped", kT=0.0, calc_noise=0)
    rc, _, _ = solve_static(L, bl, np.zeros((m.n_nodes, 3)))
    assert rc == lib.EINPUT
    big = case_mesh(32, 1)  # 33^3 = 35,937 vertex nodes > 32,768
    bb = lib.Blob(big, solver="CG_nomass", kT=0.0, calc_noise=0)
    rc, _, _ = solve_static(L, bb, np.zeros((big.n_nodes, 3)))
    assert rc == lib.EINPUT and "static scratch limit" in lib.last_error()
