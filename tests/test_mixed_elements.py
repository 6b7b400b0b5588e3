"""The mixed path's element phase (element_mixed_kernel) on the GPU, through the C ABI.

* Near-degenerate elements: one tetrahedron compressed to 3 % and to 6 % of its rest volume, either side of
  the 5 % threshold below which the kernel takes its FP64 Jacobian branch: the mixed right-hand side equals
  the FP64 path's (the reference's arithmetic, bit-exact against it) within 1e-5 of its largest component, and
  so does an element at 60 % of its volume.
* Inversion is reported by every solver of the mixed path, as by the FP64 path.
* The inertial solvers (mass-lumped and consistent mass) after 1000 kT = 0 steps from a 2 % shear against the
  reference's own trajectories (goldens): within 1e-5 of the displacement, the stated bound of the mixed path.
* With noise, the mixed path draws the reference's numbers. At rest the elastic stress vanishes, so one step's
  right-hand side is the thermal stress alone, a linear function of each element's 7 draws: mixed and FP64
  (bit-exact against the reference) agree within 1e-5 of the largest component, which no single wrong draw
  would. The stream state stays bit-exact, and over 100 mass-lumped steps the positions stay within 1e-4 of
  the RMS displacement of the FP64 path's (the same draws, each rounded to FP32).
"""
import os

import numpy as np
import pytest

from ffea_ci_demo_gb300 import lib
from ffea_ci_demo_gb300.mesh import Mesh
from gen_golden import case_mesh, sheared

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def one_tet() -> Mesh:
    """A single 10-node tetrahedron (vertices then the six edge midpoints), benchmark material, file units nm."""
    v = np.array([[0.0, 0.0, 0.0], [4.0, 0.3, 0.2], [0.5, 4.2, -0.1], [0.3, 0.4, 3.9]])
    mids = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    pos = np.vstack([v] + [0.5 * (v[a] + v[b])[None] for a, b in mids])
    mat = np.array([[1500.0, 1e-3, 1e-3, 5.7e8, 2.2e9, 1.0]])
    return Mesh(pos=pos, tets=np.arange(10, dtype=np.int32)[None], material=mat, stokes_radius=np.full(10, 0.5),
                n_linear=4)


def compressed(m: Mesh, frac: float) -> np.ndarray:
    """Positions (meso units) with vertex 3 moved toward the opposite face so the volume is `frac` of rest."""
    p = m.pos.copy()
    n = np.cross(p[1] - p[0], p[2] - p[0])
    n /= np.linalg.norm(n)
    h = np.dot(p[3] - p[0], n)
    p[3] -= (1.0 - frac) * h * n
    for k, (a, b) in enumerate([(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]):
        p[4 + k] = 0.5 * (p[a] + p[b])
    return p * (m.scale / lib.MESO_LENGTH)


@pytest.mark.parametrize("frac", [0.03, 0.06, 0.6])
def test_near_degenerate_element_forces(gpu, frac):
    m = one_tet()
    p = compressed(m, frac)
    rhs = {}
    for prec in ("fp64", "mixed"):
        b = lib.Blob(m, solver="masslumped", precision=prec, dt=1e-14, kT=0.0, calc_noise=0)
        b.set_state(pos=p)
        b.update(1)
        rhs[prec] = b.rhs()
    scale = np.abs(rhs["fp64"]).max()
    err = np.abs(rhs["mixed"] - rhs["fp64"]).max() / scale
    print(f"volume {frac:.0%} of rest: mixed vs FP64 right-hand side {err:.2e} of the largest")
    assert scale > 0 and err <= 1e-5


@pytest.mark.parametrize("solver", ["CG_nomass", "CG", "masslumped"])
def test_inversion_is_reported_mixed(gpu, solver):
    m = case_mesh(2, 11)
    p = sheared(m, 0.0)
    t = m.tets[0]
    p[t[3]] = p[t[0]] - (p[t[3]] - p[t[0]])
    b = lib.Blob(m, solver=solver, precision="mixed", dt=1e-14, kT=0.0, calc_noise=0)
    b.set_state(pos=p)
    rc, done = b.try_update(3)
    assert rc == lib.EINVERTED and done == 0


@pytest.mark.parametrize("name,solver", [("cube6_masslumped_kT0_1000", "masslumped"), ("cube6_CG_kT0_1000", "CG")])
def test_mixed_inertial_solvers_within_bound(gpu, name, solver):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    m = case_mesh(6, 12345)
    x0 = sheared(m, 0.02)
    b = lib.Blob(m, solver=solver, precision="mixed", dt=1e-14, kT=0.0, calc_noise=0)
    b.set_state(pos=x0)
    b.update(int(g["steps"]))
    err = float(np.abs(b.pos() - g["final_pos"]).max() / np.abs(g["final_pos"] - x0).max())
    print(f"{solver} mixed after {int(g['steps'])} kT=0 steps: {err:.2e} of the reference displacement")
    assert err <= 1e-5


def test_mixed_noise_follows_fp64_draws(gpu):
    m = case_mesh(6, 12345)
    out = {}
    for prec in ("fp64", "mixed"):
        b = lib.Blob(m, solver="masslumped", precision=prec, dt=1e-14, kT=4.11e-21, calc_noise=1)
        x0 = b.pos()
        b.update(100)
        out[prec] = (b.pos(), b.rng_state())
    assert np.array_equal(out["mixed"][1], out["fp64"][1])
    d = out["fp64"][0] - x0
    rms = float(np.sqrt(np.mean((out["mixed"][0] - out["fp64"][0]) ** 2)) / np.sqrt(np.mean(d ** 2)))
    print(f"mass-lumped with noise, 100 steps: mixed vs FP64 {rms:.2e} of the RMS displacement")
    assert rms <= 1e-4


@pytest.mark.parametrize("n", [3, 7])
def test_mixed_noise_draws_at_rest(gpu, n):
    m = case_mesh(n, 21)
    rhs = {}
    for prec in ("fp64", "mixed"):
        b = lib.Blob(m, solver="masslumped", precision=prec, dt=1e-14, kT=4.11e-21, calc_noise=1)
        b.update(1)
        rhs[prec] = (b.rhs(), b.rng_state())
    scale = np.abs(rhs["fp64"][0]).max()
    err = np.abs(rhs["mixed"][0] - rhs["fp64"][0]).max() / scale
    print(f"{m.n_elem} elements at rest with noise: mixed vs FP64 right-hand side {err:.2e} of the largest")
    assert scale > 0 and err <= 1e-5
    assert np.array_equal(rhs["mixed"][1], rhs["fp64"][1])


def test_masslumped_continuation_steps_match_single_steps(gpu):
    """A multi-step call of the mixed mass-lumped solver forms each later step's FP32 node state in the previous
    step's gather (no separate node pass); the trajectory is bit-identical to steps taken one call at a time."""
    m = case_mesh(5, 3)
    out = []
    for chunks in ([12], [1] * 12, [5, 7]):
        b = lib.Blob(m, solver="masslumped", precision="mixed", dt=1e-14, kT=4.11e-21, calc_noise=1)
        b.set_state(pos=sheared(m, 0.02))
        for n in chunks:
            b.update(n)
        out.append((b.pos(), b.vel(), b.rng_state()))
    for p, v, r in out[1:]:
        assert np.array_equal(p, out[0][0]) and np.array_equal(v, out[0][1]) and np.array_equal(r, out[0][2])


def test_masslumped_state_set_between_calls_is_seen(gpu):
    """State set between two calls (positions, velocities, stream) reaches the next call's first step whichever
    stream buffer is current (an odd number of steps leaves the second one current): the blob then steps as a fresh
    blob given that state does, bit for bit."""
    m = case_mesh(5, 3)
    kw = dict(solver="masslumped", precision="mixed", dt=1e-14, kT=4.11e-21, calc_noise=1)
    for first in (1, 2):
        b = lib.Blob(m, **kw)
        b.set_state(pos=sheared(m, 0.02))
        b.update(first)
        x1, v1 = sheared(m, 0.03, seed=9), 0.5 * b.vel()
        s1 = b.rng_state()
        s1[0] = (int(s1[0]) + 1) % 4294967087
        b.set_state(pos=x1, vel=v1)
        b.set_rng_state(s1)
        b.update(4)
        f = lib.Blob(m, rng_state=s1, **kw)
        f.set_state(pos=x1, vel=v1)
        f.update(4)
        assert np.array_equal(b.pos(), f.pos()) and np.array_equal(b.vel(), f.vel()), first
        assert np.array_equal(b.rng_state(), f.rng_state()), first


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nomass_state_set_between_calls_is_seen(gpu, precision):
    """CG_nomass: positions set between two calls move the rigid modes' centre, which the step's gather and CG take
    as launch arguments; the blob's step graph is re-captured with them and updated in place. The next steps then
    match, bit for bit, a fresh blob given the same positions and stream (Jacobi preconditioner on both, so that
    neither carries a polynomial estimate from earlier solves). 2,197 vertex rows: the multi-block CG kernels."""
    m = case_mesh(12, 21)
    kw = dict(solver="CG_nomass", precision=precision, dt=1e-12, kT=4.11e-21, calc_noise=1, cg_poly=-1)
    b = lib.Blob(m, **kw)
    b.set_state(pos=sheared(m, 0.02))
    b.update(2)
    x1 = sheared(m, 0.03, seed=9)
    s1 = b.rng_state()
    b.set_state(pos=x1)
    b.update(3)
    f = lib.Blob(m, rng_state=s1, **kw)
    f.set_state(pos=x1)
    f.update(3)
    assert b.cg_kernel() == f.cg_kernel()
    assert np.array_equal(b.pos(), f.pos()), precision
    assert np.array_equal(b.rng_state(), f.rng_state()), precision
    assert b.cg_iterations()[0] == f.cg_iterations()[0]
