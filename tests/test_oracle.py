"""The oracle (C restatement, oracle/orc_*.c) pinned against the reference.

Golden vectors in tests/golden/*.npz come from the reference's own compiled
classes (tests/golden/gen_golden.py). The oracle is compiled with
-ffp-contract=off and run single-threaded, so it must reproduce them bit for
bit: RNG draws and states, sparsity pattern, connectivity, per-element
forces and viscosity matrices, assembled right-hand sides and trajectories.
"""
import os

import numpy as np
import pytest

import pyoracle as po
from gen_golden import case_mesh, ctf_case, digest, file_digest, sheared

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def test_rngstream_known_answer(oracle_built):
    """tests/consistency/rngstream/testRngStream.cpp:129 expects 39.697547445251."""
    po.OracleRng.set_package_seed([12345] * 6)
    s = po.rngstream_known_answer(po.OracleRng, po.OracleRng.set_package_seed)
    assert "%.14g" % s == "39.697547445251"
    assert s == float(load("rng")["known_answer"])


def test_rng_golden(oracle_built):
    g0 = load("rng")
    po.OracleRng.set_package_seed([12345] * 6)
    g = po.OracleRng()
    assert np.array_equal([g.rand_u01() for _ in range(256)], g0["draws"])
    g.reset_start_stream()
    for k in range(4):
        assert np.array_equal([g.rand_u01() for _ in range(16)], g0["substreams"][k])
        g.reset_next_substream()
    g.reset_start_stream()
    g.advance_state(5, 3)
    assert np.array_equal(g.get_state(), g0["adv_5_3"])
    g.advance_state(-127, 0)
    assert np.array_equal(g.get_state(), g0["adv_m127_0"])
    g.reset_start_stream()
    g.advance_state(0, 7 * 1296)
    assert np.array_equal(g.get_state(), g0["adv_0_9072"])
    g2 = po.OracleRng()
    assert np.array_equal([g2.rand_u01() for _ in range(16)], g0["stream2"])


CASES = {
    "cube2_nomass_kT0": (lambda: case_mesh(2, 11), 0.02, dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0)),
    "cube2_nomass_noise": (lambda: case_mesh(2, 11), 0.02,
                           dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1)),
    "cube3_nomass_pin_stokes": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                                dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    "cube3_lumped_pin_stokes": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                                dict(solver="masslumped", dt=1e-14, kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    "cube3_cg_pin_stokes": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                            dict(solver="CG", dt=1e-14, kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    "cube3_nomass_ctf": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                         dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    "cube3_lumped_ctf": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                         dict(solver="masslumped", dt=1e-14, kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    "cube3_cg_ctf": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                     dict(solver="CG", dt=1e-14, kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    "cube3_nomass_ctf_kT0": (lambda: case_mesh(3, 7, [0, 1, 5, 66]), 0.02,
                             dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0, calc_stokes=1)),
    "cube6_masslumped_kT0_1000": (lambda: case_mesh(6, 12345), 0.02,
                                  dict(solver="masslumped", dt=1e-14, kT=0.0, calc_noise=0)),
    "cube6_masslumped_noise_1000": (lambda: case_mesh(6, 12345), 0.0,
                                    dict(solver="masslumped", dt=1e-14, kT=4.11e-21, calc_noise=1)),
    "cube6_CG_kT0_1000": (lambda: case_mesh(6, 12345), 0.02, dict(solver="CG", dt=1e-14, kT=0.0, calc_noise=0)),
    "cube6_CG_noise_1000": (lambda: case_mesh(6, 12345), 0.0,
                            dict(solver="CG", dt=1e-14, kT=4.11e-21, calc_noise=1)),
    "cube6_nomass_kT0_1000": (lambda: case_mesh(6, 12345), 0.02,
                              dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0)),
    "cube6_nomass_noise_100": (lambda: case_mesh(6, 12345), 0.0,
                               dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden(oracle_built, name, tmp_path):
    make, strain, kw = CASES[name]
    g = load(name)
    m = make()
    b = po.OracleBlob(m, threads=1, **kw)
    b.set_pos(sheared(m, strain))
    if "ctf_sha256" in g:  # constant forces: the same files the reference was given
        ctf = ctf_case(m, str(tmp_path))
        assert file_digest(*ctf) == str(g["ctf_sha256"])
        b.set_ctforces(po.read_ctforces(ctf[0], 0, m.n_nodes), po.read_surface(ctf[1]))
    solver = kw["solver"]
    c = b.contrib()
    if "contrib_ptr" in g:
        assert np.array_equal(c["ptr"], g["contrib_ptr"]) and np.array_equal(c["elem_slot"], g["contrib_es"])
        rest = b.rest()
        assert np.array_equal(rest["jinv0"], g["jinv0"]) and np.array_equal(rest["mat"], g["mat"])
    else:
        assert digest(c["ptr"], c["elem_slot"]) == str(g["contrib_sha256"])
    if solver == "CG_nomass":
        csr = b.csr()
        if "csr_key" in g:
            for k in ("key", "col", "nsrc"):
                assert np.array_equal(csr[k], g["csr_" + k]), k
        else:
            assert digest(csr["key"], csr["col"], csr["nsrc"]) == str(g["csr_sha256"])
    elif solver == "CG":
        mc = b.mass_csr()
        if "mass_key" in g:
            for k in ("key", "col", "val"):
                assert np.array_equal(mc[k], g["mass_" + k]), k
        else:
            assert digest(mc["key"], mc["col"], mc["val"]) == str(g["mass_sha256"])
    elif "inv_mass" in g:
        assert np.array_equal(b.inv_mass(), g["inv_mass"])
    assert b.step(1) == 0
    e = b.elem()
    assert np.array_equal(e["vol"], g["step1_vol"])
    assert np.array_equal(b.rhs(), g["step1_rhs"])
    if "step1_node_force" in g:
        assert np.array_equal(e["node_force"], g["step1_node_force"])
        assert np.array_equal(e["stress_mag"], g["step1_stress_mag"])
        assert np.array_equal(b.pos(), g["step1_pos"]) and np.array_equal(b.vel(), g["step1_vel"])
    if "step1_visc" in g:
        assert np.array_equal(e["visc"], g["step1_visc"]) and np.array_equal(e["dpsi"], g["step1_dpsi"])
    if "step1_csr_val" in g:
        assert np.array_equal(b.csr()["val"], g["step1_csr_val"])
    steps = int(g["steps"])
    if steps > 1:
        assert b.step(steps - 1) == 0
    assert np.array_equal(b.pos(), g["final_pos"])
    assert np.array_equal(b.vel(), g["final_vel"])
    assert np.array_equal(b.rng_state(), g["final_rng"])
    np.testing.assert_allclose(b.measure(), g["final_energy"], rtol=1e-13, atol=0)


def test_oracle_threads_agree_at_kT0(oracle_built):
    """OpenMP threads change only reduction order: kT=0 trajectories agree to rounding."""
    m = case_mesh(3, 7)
    kw = dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0)
    a = po.OracleBlob(m, threads=1, **kw)
    b = po.OracleBlob(m, threads=4, **kw)
    p = sheared(m, 0.02)
    a.set_pos(p)
    b.set_pos(p)
    assert a.step(20) == 0 and b.step(20) == 0
    d0 = a.pos() - p
    np.testing.assert_allclose(b.pos() - p, d0, rtol=0, atol=1e-9 * np.abs(d0).max())


def test_oracle_reports_inversion(oracle_built):
    """An element flipped inside-out between steps is counted and reported (src/Blob.cpp:484-490)."""
    m = case_mesh(2, 11)
    b = po.OracleBlob(m, solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0, threads=1)
    p = sheared(m, 0.0)
    t = m.tets[0]
    p[t[3]] = p[t[0]] - (p[t[3]] - p[t[0]])  # reflect vertex 3 through vertex 0
    b.set_pos(p)
    assert b.step(1) == 1  # ORC_EINVERTED


def test_oracle_reports_cg_max_iterations(oracle_built):
    m = case_mesh(2, 11)
    b = po.OracleBlob(m, solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0, threads=1, max_iterations_cg=2)
    b.set_pos(sheared(m, 0.02))
    assert b.step(1) == 2  # ORC_ECGMAXIT


@pytest.mark.skipif(not os.path.exists(po.REF_LIB), reason="the reference's own build exists only where its sources are")
@pytest.mark.parametrize("solver,dt,kw", [
    ("CG_nomass", 1e-12, dict(kT=4.11e-21, calc_noise=1)),
    ("masslumped", 1e-14, dict(kT=4.11e-21, calc_noise=1, calc_stokes=1)),
    ("CG", 1e-14, dict(kT=0.0, calc_noise=0)),
])
def test_oracle_matches_reference_blob(oracle_built, solver, dt, kw):
    """Where the reference's sources are, its own Blob (Blob::config/init from structure files, World::run's step;
    oracle/_ref) and the C restatement step a fresh seeded cube to the same bits: positions, velocities, the
    last right-hand side and the stream state."""
    m = case_mesh(2, 31, [3])
    p = sheared(m, 0.02)
    r = po.RefBlob(m, solver=solver, dt=dt, threads=1, **kw)
    o = po.OracleBlob(m, solver=solver, dt=dt, threads=1, **kw)
    r.set_pos(p)
    o.set_pos(p)
    assert r.step(15) == 0 and o.step(15) == 0
    for get in ("pos", "vel", "rhs"):
        assert np.array_equal(getattr(r, get)(), getattr(o, get)()), get
    assert np.array_equal(r.rng_state(), o.rng_state())
