"""ffea_gpu_blob_solve_static: the Jacobi-PCG solve with its work arrays in the
library's static device scratch (no allocation per call), through the C ABI.

Callers that cannot allocate device memory when they solve (a host code whose
memory pool already holds the GPU, or an integrator inside a fixed-memory loop)
use this entry point. It is checked against the regular step
(ffea_gpu_blob_step): after one step the blob holds the force vector it solved
(ffea_gpu_blob_get_rhs) and the matrix it solved with, and the solution sits in
the velocities (CG_nomass: v = x; CG from rest: v = x dt, src/Blob.cpp:3249-3279).
Solving the same force again with the static-scratch entry point must give the
same solution to rounding: the step of this 343-node blob runs the owned-rows
CG kernel, whose sums run in another order than the grid-strided kernel of
the static solve, so the iteration counts may differ by one and the solutions
agree to 1e-10 of the largest component, far inside the CG tolerance. Two
calls in a row check that the scratch left by one call does not leak into the
next, and the device's free memory (cudaMemGetInfo) must not change across
any of the calls, the first included.
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
def test_static_solve_matches_step(gpu, device_free_bytes, solver, dt):
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
    x = np.full_like(f, np.nan)
    for call in range(3):
        before = device_free_bytes()
        rc, x, it = solve_static(L, b, f, out=x)
        assert device_free_bytes() == before, f"call {call} changed the device's free memory"
        assert rc == lib.OK, lib.last_error()
        assert abs(it - iters) <= 1, (call, it, iters)
        err = np.abs(x - ref).max() / scale
        print(f"{solver} call {call}: {it} iterations (step: {iters}), max error {err:.3e} of max |x|")
        assert err <= 1e-10, (call, err)
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
