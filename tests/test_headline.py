"""The benchmark's headline configuration checked where its accuracy targets are stated.

Workload: the 40^3-cell Kuhn cube of side 200 nm (384,000 tets, 68,921 vertex nodes), the construction
the benchmark times, with CG_nomass at epsilon 1e-10, dt = 1e-12 s, run at kT = 0 from a seeded 2% shear
(no noise, so every path follows the same deterministic trajectory).

* FP64 GPU path against the oracle (the C restatement pinned bit-exact to the reference build), run on all
  host threads: at kT = 0 OpenMP changes only the order of the CG's dot products. The first step's assembled
  right-hand side is bit-exact; after 3 steps the positions agree within 1e-8 of the displacement (both CGs
  stop at |r|^2/|f|^2 < 1e-20 and sum in different orders).
* Mixed path with the arithmetic the benchmark times (single-reduction CG kernel, Chebyshev preconditioner
  of the default degree after the first two solves) against the FP64 GPU path after 1000 steps: the stated bound,
  max |x_mixed - x_fp64| <= 1e-5 * max |x_fp64 - x_0|.

Reference: NoMassCGSolver::solve (src/NoMassCGSolver.cpp:156-188), Blob::update_internal_forces and
update_positions (src/Blob.cpp:400-508).
"""
import os

import numpy as np
import pytest

import pyoracle as po
from ffea_ci_demo_gb300 import lib
from ffea_ci_demo_gb300.mesh import apply_shear, kuhn_cube

pytestmark = pytest.mark.gpu

CELLS, SIDE = 40, 200.0
KW = dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0, epsilon=1e-10, max_iterations_cg=10000)


@pytest.fixture(scope="module")
def headline():
    m = kuhn_cube(CELLS, side=SIDE, seed=12345)
    x0 = apply_shear(m, 0.02, seed=3) * (m.scale / lib.MESO_LENGTH)
    return m, x0


def disp_err(x, ref, x0):
    return float(np.abs(x - ref).max() / np.abs(ref - x0).max())


def test_headline_fp64_matches_oracle(gpu, oracle_built, headline):
    m, x0 = headline
    threads = os.cpu_count() or 1
    o = po.OracleBlob(m, threads=threads, **KW)
    o.set_pos(x0)
    b = lib.Blob(m, precision="fp64", **KW)
    b.set_state(pos=x0)
    assert b.cg_kernel() == "cg_own_kernel"
    assert o.step(1) == 0
    b.update(1)
    assert np.array_equal(b.rhs(), o.rhs()), "assembled force of the 40^3 cube differs from the oracle"
    assert o.step(2) == 0
    b.update(2)
    err = disp_err(b.pos(), o.pos(), x0)
    print(f"40^3 FP64 GPU vs oracle ({threads} threads) after 3 steps: {err:.3e} of the displacement; "
          f"CG iterations GPU {b.cg_iterations()[1]}, oracle {o.total_cg_iters()}")
    assert err < 1e-8


def test_headline_mixed_1000_steps_within_bound(gpu, headline):
    m, x0 = headline
    res = {}
    for prec in ("fp64", "mixed"):
        b = lib.Blob(m, precision=prec, **KW)
        b.set_state(pos=x0)
        b.update(2)
        if prec == "mixed":
            # the benchmark's arithmetic: single-reduction kernel with the default polynomial
            assert b.cg_kernel() == "cg_mixed_sr_kernel"
            assert b.cg_preconditioner()[0] == lib.CG_POLY_DEFAULT
        b.update(998)
        res[prec] = (b.pos(), b.cg_iterations()[1])
        b.close()
    err = disp_err(res["mixed"][0], res["fp64"][0], x0)
    print(f"40^3 mixed vs FP64 after 1000 kT=0 steps: {err:.3e} of the max displacement "
          f"(CG iterations: mixed {res['mixed'][1]}, FP64 {res['fp64'][1]})")
    assert err <= 1e-5
