"""GPU parity: the CUDA path through the C ABI against the reference.

Reference results come from tests/golden/*.npz (produced by the reference's
own compiled classes) and from the oracle (oracle/orc_*.c, pinned bit-exact
to those goldens by tests/test_oracle.py), run on the same seeded inputs.

Tolerances:
* integer structure (pattern, connectivity, RNG states): bit-exact.
* FP64 path, per-element forces / volumes / assembled matrix values /
  right-hand side: bit-exact (same expression order, no FMA).
* FP64 path, trajectories through the CG: the CG's cross-node dot products
  are reduced in a different order than the reference's sequential loop, so
  positions agree to rounding: max |x_gpu - x_ref| <= 1e-8 * max |x_ref - x_0|.
* mass-lumped FP64 trajectories (no reductions at all): bit-exact.
* mixed path, kT = 0: max |x_mixed - x_ref| <= 1e-5 * max |x_ref - x_0| after 1000 steps.
"""
import os
import tempfile

import numpy as np
import pytest

import pyoracle as po
from ffea_ci_demo_gb300 import lib
from ffea_ci_demo_gb300.mesh import write_structure
from gen_golden import case_mesh, sheared

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def gpu_blob(m, strain, **kw):
    b = lib.Blob(m, **kw)
    b.set_state(pos=sheared(m, strain))
    return b


def disp_err(x, ref, x0):
    return float(np.abs(x - ref).max() / np.abs(ref - x0).max())


def test_pattern_and_connectivity_bit_exact(gpu):
    g = load("cube2_nomass_kT0")
    b = gpu_blob(case_mesh(2, 11), 0.02, solver="CG_nomass", kT=0.0, calc_noise=0)
    pat = b.pattern(values=False)
    for k in ("key", "col", "nsrc"):
        assert np.array_equal(pat[k], g["csr_" + k]), k
    c = b.connectivity()
    assert np.array_equal(c["ptr"], g["contrib_ptr"]) and np.array_equal(c["elem_slot"], g["contrib_es"])
    # pinned vertex + pinned midpoint + Stokes drag sources on the diagonal
    g3 = load("cube3_nomass_pin_stokes")
    b3 = gpu_blob(case_mesh(3, 7, [0, 1, 5, 66]), 0.02, solver="CG_nomass", kT=0.0, calc_noise=0, calc_stokes=1)
    pat3 = b3.pattern(values=False)
    for k in ("key", "col", "nsrc"):
        assert np.array_equal(pat3[k], g3["csr_" + k]), k


@pytest.mark.parametrize("name,kw", [
    ("cube2_nomass_kT0", dict(kT=0.0, calc_noise=0)),
    ("cube2_nomass_noise", dict(kT=4.11e-21, calc_noise=1)),
])
def test_fp64_step_bit_exact(gpu, name, kw):
    g = load(name)
    m = case_mesh(2, 11)
    b = gpu_blob(m, 0.02, solver="CG_nomass", dt=1e-12, **kw)
    b.update(1)
    e = b.elements(visc=True)
    assert np.array_equal(e["node_force"], g["step1_node_force"])
    assert np.array_equal(e["vol"], g["step1_vol"])
    assert np.array_equal(e["visc"], g["step1_visc"])
    assert np.array_equal(b.rhs(), g["step1_rhs"])
    assert np.array_equal(b.pattern()["val"], g["step1_csr_val"])
    x0 = sheared(m, 0.02)
    assert disp_err(b.pos(), g["step1_pos"], x0) < 1e-10
    steps = int(g["steps"])
    b.update(steps - 1)
    assert disp_err(b.pos(), g["final_pos"], x0) < 1e-8
    assert np.array_equal(b.rng_state(), g["final_rng"])


@pytest.mark.parametrize("name,strain,kw", [
    ("cube6_masslumped_kT0_1000", 0.02, dict(solver="masslumped", dt=1e-14, kT=0.0, calc_noise=0)),
    ("cube6_masslumped_noise_1000", 0.0, dict(solver="masslumped", dt=1e-14, kT=4.11e-21, calc_noise=1)),
])
def test_masslumped_1000_steps_bit_exact(gpu, name, strain, kw):
    g = load(name)
    m = case_mesh(6, 12345)
    b = gpu_blob(m, strain, **kw)
    b.update(1)
    assert np.array_equal(b.rhs(), g["step1_rhs"])
    b.update(int(g["steps"]) - 1)
    assert np.array_equal(b.pos(), g["final_pos"])
    assert np.array_equal(b.vel(), g["final_vel"])
    assert np.array_equal(b.rng_state(), g["final_rng"])
    np.testing.assert_allclose(b.measure(), g["final_energy"], rtol=1e-12)


@pytest.mark.parametrize("name,strain,kw,tol", [
    ("cube6_nomass_kT0_1000", 0.02, dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0), 1e-8),
    ("cube6_nomass_noise_100", 0.0, dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1), 1e-8),
    ("cube6_CG_kT0_1000", 0.02, dict(solver="CG", dt=1e-14, kT=0.0, calc_noise=0), 1e-8),
    ("cube6_CG_noise_1000", 0.0, dict(solver="CG", dt=1e-14, kT=4.11e-21, calc_noise=1), 1e-8),
])
def test_fp64_trajectories_match_reference(gpu, name, strain, kw, tol):
    g = load(name)
    m = case_mesh(6, 12345)
    b = gpu_blob(m, strain, **kw)
    b.update(1)
    assert np.array_equal(b.rhs(), g["step1_rhs"])
    b.update(int(g["steps"]) - 1)
    x0 = sheared(m, strain)
    assert disp_err(b.pos(), g["final_pos"], x0) < tol
    assert np.array_equal(b.rng_state(), g["final_rng"])
    # strain energy sums G (F:F - 3) over elements: near rest it cancels to ~1e-10, so compare with a
    # floor at the rounding level of the sum (~1e-16 x 3 G vol0 x 1296 elements)
    np.testing.assert_allclose(b.measure(), g["final_energy"], rtol=1e-6, atol=2e-11)


def test_mixed_precision_kT0_error_bound(gpu):
    """Mixed path after 1000 kT=0 steps within 1e-5 of the reference displacement."""
    g = load("cube6_nomass_kT0_1000")
    m = case_mesh(6, 12345)
    b = gpu_blob(m, 0.02, solver="CG_nomass", precision="mixed", dt=1e-12, kT=0.0, calc_noise=0)
    b.update(1000)
    err = disp_err(b.pos(), g["final_pos"], sheared(m, 0.02))
    print("mixed kT=0 1000-step displacement error", err)
    assert err < 1e-5


@pytest.mark.parametrize("kw", [
    dict(kT=4.11e-21, calc_noise=1),
    dict(kT=0.0, calc_noise=0, calc_stokes=1),
])
def test_mixed_precision_iterations_and_error(gpu, kw):
    """Mixed CG (FP32 matrix, deflated rigid modes) with the reference's Jacobi preconditioner needs the FP64
    path's iteration count."""
    m = case_mesh(8, 21)
    out = {}
    for prec in ("fp64", "mixed"):
        b = gpu_blob(m, 0.02, solver="CG_nomass", precision=prec, dt=1e-12, cg_poly=-1, **kw)
        its = []
        for _ in range(5):
            b.update(1)
            its.append(b.cg_iterations()[0])
        out[prec] = (its, b.pos())
    assert all(abs(a - b) <= 2 for a, b in zip(out["fp64"][0], out["mixed"][0])), out
    assert disp_err(out["mixed"][1], out["fp64"][1], sheared(m, 0.02)) < 1e-5


@pytest.mark.parametrize("poly", [2, 4, 6, 8])
def test_chebyshev_preconditioner(gpu, poly):
    """Mixed CG_nomass with a Chebyshev polynomial preconditioner (degree 2, 4, 6 or 8 in D^-1 V). The blob's
    first solve is Jacobi's and estimates lambda_max of D^-1 V; the second is the polynomial's trial, kept when it
    saves work. With thermal noise on a 12^3-cell cube (about 180 Jacobi iterations a step) it is kept and needs
    at most 0.45x (degree 2), 0.35x (4), 0.3x (6) or 0.25x (8) of the iterations; with a Stokes drag (about 26
    Jacobi iterations) the trial saves nothing worth its cost and Jacobi is kept. The trajectory stays within 1e-5
    of the FP64 path's displacement, and the blob is reproducible run to run."""
    m = case_mesh(12, 21)  # 2,197 vertex nodes: nine CG blocks exchanging with their neighbours
    for kw, kept in ((dict(kT=4.11e-21, calc_noise=1), True), (dict(kT=0.0, calc_noise=0, calc_stokes=1), False)):
        its, pos = {}, {}
        for name, prec, cg_poly in (("fp64", "fp64", 0), ("jacobi", "mixed", -1), ("cheb", "mixed", poly),
                                    ("cheb2", "mixed", poly)):
            b = gpu_blob(m, 0.02, solver="CG_nomass", precision=prec, dt=1e-12, cg_poly=cg_poly, **kw)
            its[name] = []
            for step in range(8):
                b.update(1)
                its[name].append(b.cg_iterations()[0])
                if name == "cheb" and step == 0:
                    deg, lm = b.cg_preconditioner()
                    assert deg == poly and 1.5 < lm < 4.0, (deg, lm)  # lambda_max(D^-1 V) of a Kuhn mesh ~2.4
            pos[name] = b.pos()
            if prec == "mixed":
                assert b.cg_preconditioner()[0] == (poly if cg_poly > 0 and kept else 0)
        print(poly, kw, its)
        assert its["cheb"][0] == its["jacobi"][0]
        if kept:
            bound = {2: 0.45, 4: 0.35, 6: 0.3, 8: 0.25}[poly]
            assert all(c <= bound * j for c, j in zip(its["cheb"][1:], its["jacobi"][1:])), its
        else:
            assert its["cheb"][1] <= its["jacobi"][1]
            assert all(abs(c - j) <= 1 for c, j in zip(its["cheb"][2:], its["jacobi"][2:])), its
        x0 = sheared(m, 0.02)
        assert disp_err(pos["cheb"], pos["fp64"], x0) < 1e-5
        assert disp_err(pos["jacobi"], pos["fp64"], x0) < 1e-5
        assert its["cheb2"] == its["cheb"] and np.array_equal(pos["cheb2"], pos["cheb"])


def test_matrix_cache_is_bit_identical(gpu):
    """The single-reduction CG's shared-memory copy of each owned row's first blocks changes where the matrix is
    read from, not the arithmetic: a blob without it (cg_smem_blocks = -1) and blobs with it capped at two blocks
    per row or at what fits (0) step to the same bits."""
    m = case_mesh(12, 21)
    out = []
    for cache in (0, -1, 2):
        b = gpu_blob(m, 0.02, solver="CG_nomass", precision="mixed", dt=1e-12, kT=4.11e-21, calc_noise=1,
                     cg_smem_blocks=cache)
        b.update(6)
        out.append((b.pos(), b.cg_iterations()[1]))
    for x, it in out[1:]:
        assert it == out[0][1] and np.array_equal(x, out[0][0])


def test_mixed_precision_pinned_nodes(gpu):
    """With pinned vertices the deflated modes are the rigid motions that keep them at rest."""
    for pins in ([0], [0, 1], [0, 1, 5]):
        m = case_mesh(4, 3, pins)
        res = {}
        for prec in ("fp64", "mixed"):
            b = gpu_blob(m, 0.02, solver="CG_nomass", precision=prec, kT=0.0, calc_noise=0)
            b.update(20)
            res[prec] = b.pos()
        assert disp_err(res["mixed"], res["fp64"], sheared(m, 0.02)) < 1e-5, pins


def test_pinned_nodes_and_stokes_drag_match_oracle(gpu, oracle_built):
    m = case_mesh(3, 7, [0, 1, 5, 66])
    kw = dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0, calc_stokes=1)
    o = po.OracleBlob(m, threads=1, **kw)
    o.set_pos(sheared(m, 0.02))
    b = gpu_blob(m, 0.02, **kw)
    assert o.step(1) == 0
    b.update(1)
    assert np.array_equal(b.rhs(), o.rhs())
    assert np.array_equal(b.pattern()["val"], o.csr()["val"])
    assert o.step(9) == 0
    b.update(9)
    assert disp_err(b.pos(), o.pos(), sheared(m, 0.02)) < 1e-8
    p = b.pos()
    assert np.array_equal(p[[0, 1, 5]], sheared(m, 0.02)[[0, 1, 5]])  # pinned vertices never move


def test_structure_files_load_like_arrays(gpu):
    m = case_mesh(2, 11)
    with tempfile.TemporaryDirectory() as d:
        paths = write_structure(m, d, "cube2")
        bf = lib.Blob.from_files(paths["node"], paths["top"], paths["mat"], paths["stokes"], paths["pin"], m.scale,
                                 solver="CG_nomass", dt=1e-12, kT=4.11e-21, epsilon=1e-10, calc_noise=1,
                                 calc_stokes=0, max_iterations_cg=10000)
    ba = lib.Blob(m, solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1)
    bf.update(5)
    ba.update(5)
    assert np.array_equal(bf.pos(), ba.pos())


def test_deterministic_rerun(gpu):
    m = case_mesh(4, 5)
    out = []
    for _ in range(2):
        b = gpu_blob(m, 0.01, solver="CG_nomass", kT=4.11e-21, calc_noise=1)
        b.update(10)
        out.append(b.pos())
    assert np.array_equal(out[0], out[1])


def test_inversion_is_reported(gpu):
    m = case_mesh(2, 11)
    p = sheared(m, 0.0)
    t = m.tets[0]
    p[t[3]] = p[t[0]] - (p[t[3]] - p[t[0]])
    b = lib.Blob(m, solver="CG_nomass", kT=0.0, calc_noise=0)
    b.set_state(pos=p)
    rc, done = b.try_update(3)
    assert rc == lib.EINVERTED and done == 0


def test_cg_max_iterations_is_reported(gpu):
    m = case_mesh(2, 11)
    b = gpu_blob(m, 0.02, solver="CG_nomass", kT=0.0, calc_noise=0, max_iterations_cg=2)
    rc, done = b.try_update(1)
    assert rc == lib.ECGMAXIT and done == 0
    with pytest.raises(lib.FFEAError):
        b.update(1)


def test_larger_cube_fp64_matches_oracle(gpu, oracle_built):
    """A 10^3-cell cube (6000 tets): one step bit-exact forces, 5 steps to CG rounding."""
    m = case_mesh(10, 99)
    kw = dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1)
    o = po.OracleBlob(m, threads=1, **kw)
    o.set_pos(sheared(m, 0.01))
    b = gpu_blob(m, 0.01, **kw)
    assert o.step(1) == 0
    b.update(1)
    assert np.array_equal(b.rhs(), o.rhs())
    assert o.step(4) == 0
    b.update(4)
    assert disp_err(b.pos(), o.pos(), sheared(m, 0.01)) < 1e-8
    assert np.array_equal(b.rng_state(), o.rng_state())


@pytest.mark.parametrize("name,kw,exact", [
    ("cube3_nomass_pin_stokes", dict(solver="CG_nomass", dt=1e-12), False),
    ("cube3_lumped_pin_stokes", dict(solver="masslumped", dt=1e-14), True),
    ("cube3_cg_pin_stokes", dict(solver="CG", dt=1e-14), False),
])
def test_stokes_noise_matches_reference(gpu, name, kw, exact):
    """Stokes drag with noise: 3 draws per node (midpoints included) after the elements' draws, midpoint
    forces moved to their edge ends by the reference's element-order linearisation, pins zeroed."""
    g = load(name)
    m = case_mesh(3, 7, [0, 1, 5, 66])
    b = gpu_blob(m, 0.02, kT=4.11e-21, calc_noise=1, calc_stokes=1, **kw)
    b.update(1)
    assert np.array_equal(b.rhs(), g["step1_rhs"])
    b.update(int(g["steps"]) - 1)
    assert np.array_equal(b.rng_state(), g["final_rng"])
    if exact:
        assert np.array_equal(b.pos(), g["final_pos"]) and np.array_equal(b.vel(), g["final_vel"])
    else:
        assert disp_err(b.pos(), g["final_pos"], sheared(m, 0.02)) < 1e-8


def test_stokes_noise_mixed_precision(gpu):
    m = case_mesh(4, 3, [0, 2])
    out = {}
    for prec in ("fp64", "mixed"):
        b = gpu_blob(m, 0.02, solver="CG_nomass", precision=prec, kT=4.11e-21, calc_noise=1, calc_stokes=1)
        b.update(20)
        out[prec] = b.pos()
    assert disp_err(out["mixed"], out["fp64"], sheared(m, 0.02)) < 1e-5
