"""Constant forces (Blob::load_ctforces / apply_ctforces, src/Blob.cpp:1676-1741, 2478-2805) on the GPU.

* Against the reference: tests/golden/cube3_*_ctf*.npz come from the reference's own Face and element
  classes and its intersectingPointToLine, driven through the reference's apply_ctforces order
  (oracle/ref_driver.cpp), on a Kuhn cube with pins, Stokes drag and noise, linear forces on a vertex
  (twice), a midpoint and every node, rotational forces ("pf" and "pt", on vertices, a midpoint and every
  node), and two overlapping sets of surface faces. Tolerances as the other FP64 parity tests: right-hand side and
  RNG state bit-exact; positions bit-exact for the mass-lumped solver, else within 1e-8 of the
  displacement (CG reductions in another order).
* Mixed precision against FP64 on the same inputs: within 1e-5 of the displacement.
* The .ffea front-end with <interactions><ctforces> and the conformation's surface file steps exactly
  as a blob given the same files through the C ABI.
* Physics, after the reference's tests/physics/E_cyl_160_fine (a rod clamped at one end and pulled at
  the other by a surface force; Young's modulus from the extension): a synthetic square bar with the
  same material, force and run length. Its extension must match the linear-elastic finite-element
  solution of the same mesh within 1%, and Young's modulus within the clamping error of a Poisson
  ratio 0.4 bar (4%).
"""
import os

import numpy as np
import pytest

from ffea_ci_demo_gb300 import lib
from ffea_ci_demo_gb300.mesh import (faces_on_plane, kuhn_box, surface_faces, write_ctforces, write_script,
                                     write_structure, write_surface)
from gen_golden import case_mesh, ctf_case, file_digest, sheared
from fe import linear_fe_extension
from test_world import seeds_from

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def disp_err(x, ref, x0):
    return float(np.abs(x - ref).max() / np.abs(ref - x0).max())


def ctf_blob(m, ctf, precision="fp64", **kw):
    b = lib.Blob(m, precision=precision, **kw)
    b.load_ctforces(*ctf)
    b.set_state(pos=sheared(m, 0.02))
    return b


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw,exact", [
    ("cube3_nomass_ctf", dict(solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1), False),
    ("cube3_lumped_ctf", dict(solver="masslumped", dt=1e-14, kT=4.11e-21, calc_noise=1), True),
    ("cube3_cg_ctf", dict(solver="CG", dt=1e-14, kT=4.11e-21, calc_noise=1), False),
    ("cube3_nomass_ctf_kT0", dict(solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0), False),
])
def test_constant_forces_match_reference(gpu, tmp_path, name, kw, exact):
    g = load(name)
    m = case_mesh(3, 7, [0, 1, 5, 66])
    ctf = ctf_case(m, str(tmp_path))
    assert file_digest(*ctf) == str(g["ctf_sha256"])
    b = ctf_blob(m, ctf, calc_stokes=1, **kw)
    b.update(1)
    assert np.array_equal(b.rhs(), g["step1_rhs"])
    b.update(int(g["steps"]) - 1)
    assert np.array_equal(b.rng_state(), g["final_rng"])
    if exact:
        assert np.array_equal(b.pos(), g["final_pos"]) and np.array_equal(b.vel(), g["final_vel"])
    else:
        assert disp_err(b.pos(), g["final_pos"], sheared(m, 0.02)) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("solver,dt", [("CG_nomass", 1e-12), ("masslumped", 1e-14)])
def test_constant_forces_mixed_precision(gpu, tmp_path, solver, dt):
    m = case_mesh(3, 7, [0, 1, 5, 66])
    ctf = ctf_case(m, str(tmp_path))
    out = {}
    for prec in ("fp64", "mixed"):
        b = ctf_blob(m, ctf, precision=prec, solver=solver, dt=dt, kT=0.0, calc_noise=0, calc_stokes=1)
        b.update(20)
        out[prec] = b.pos()
    assert disp_err(out["mixed"], out["fp64"], sheared(m, 0.02)) < 1e-5


@pytest.mark.gpu
def test_constant_force_input_errors(gpu, tmp_path):
    m = case_mesh(2, 11)
    faces = surface_faces(m)
    surf = os.path.join(str(tmp_path), "c.surf")
    write_surface(surf, faces)
    b = lib.Blob(m, solver="CG_nomass", calc_stokes=1)
    path = os.path.join(str(tmp_path), "c.ctforces")

    def expect(ok, surf_file=surf, blob_index=0, **files):
        write_ctforces(path, **files)
        if ok:
            b.load_ctforces(path, surf_file, blob_index)
        else:
            with pytest.raises(lib.FFEAError):
                b.load_ctforces(path, surf_file, blob_index)

    expect(True, linear=[(1e-12, (1.0, 0.0, 0.0), 0, 0, 3)])
    expect(False, linear=[(1e-12, (0.0, 0.0, 0.0), 0, 0, 3)])            # zero direction
    expect(False, linear=[(1e-12, (1.0, 0.0, 0.0), 0, 0, m.n_nodes)])    # node out of range
    expect(True, linear=[(1e-12, (1.0, 0.0, 0.0), 1, 0, m.n_nodes)])     # another blob's force is skipped
    write_ctforces(path, surface=[(1e-11, (0.0, 0.0, 1.0), 0, 0, [0, 1])])
    with pytest.raises(lib.FFEAError):
        b.load_ctforces(path, None, 0)                                   # surface forces need the surface
    expect(False, surface=[(1e-11, (0.0, 0.0, 1.0), 0, 0, [faces.shape[0]])])  # face out of range
    expect(True, surface=[(1e-11, (0.0, 0.0, 1.0), 0, 0, [0, 1])])
    expect(True, rotational=[(1e-12, "pt", (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0, 0, 5)])
    expect(False, rotational=[(1e-12, "nt", (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0, 0, 5)])  # axis between nodes
    expect(False, rotational=[(1e-12, "px", (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0, 0, 5)])  # neither f nor t
    expect(False, rotational=[(1e-12, "pf", (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0, 0, 5)])  # zero axis
    with open(path, "w") as f:  # header count disagrees with the lines
        f.write("ffea ctforces file\nnum_ctforces 2\nnum_linear_forces 1\nlinear forces:\n1e-12 1 0 0 0 0 3\n")
    with pytest.raises(lib.FFEAError):
        b.load_ctforces(path, None, 0)


@pytest.mark.gpu
def test_script_with_constant_forces_matches_blob(gpu, tmp_path):
    """calc_ctforces = 1 with <interactions><ctforces> and the conformation's surface file: the World
    loads each blob's forces (Blob::init) and steps exactly as a blob given the same files."""
    m = case_mesh(3, 7, [0, 1, 5, 66])
    d = str(tmp_path)
    ctf, surf = ctf_case(m, d)
    paths = write_structure(m, d, "w")
    script = os.path.join(d, "w.ffea")
    write_script(script, paths, num_steps=10, check=5, rng_seed=31, dt=1e-12, calc_noise=1, calc_stokes=1,
                 ctforces=ctf, surface=surf)
    w = lib.World(script)
    x0 = w.blob(0).pos()
    w.run()
    b = lib.Blob(m, solver="CG_nomass", rng_state=seeds_from(31), dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=1)
    b.load_ctforces(ctf, surf, 0)
    b.set_state(pos=x0)
    b.update(11)
    assert np.array_equal(w.blob(0).pos(), b.pos())
    # without the surface file the surface forces cannot be placed
    txt = open(script).read()
    with open(script, "w") as f:
        f.write("\n".join(ln for ln in txt.split("\n") if "<surface =" not in ln))
    with pytest.raises(lib.FFEAError):
        lib.World(script)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bar_youngs_modulus(gpu, tmp_path, precision):
    """A 16 x 16 x 160 nm bar of the reference's rod material (G = 214.3 MPa, K = 1 GPa: E = 600 MPa,
    Poisson ratio 0.4), clamped at z = 0 and pulled along z by 1e-11 N spread over its z = 160 nm face,
    run as the reference's Young's-modulus test is (CG_nomass, dt 1e-13 s, 300 steps, CG tolerance 1e-2,
    no noise, no Stokes drag) through the .ffea front-end."""
    G, K, F = 214285714.3, 1e9, 1e-11
    E = 9 * K * G / (3 * K + G)
    n, nz, h = 4, 40, 4.0
    m = kuhn_box(n, n, nz, h, shear_mod=G, bulk_mod=K)
    L, A = nz * h * 1e-9, (n * h * 1e-9) ** 2
    m.pinned = np.nonzero(np.abs(m.pos[:, 2]) < 1e-9)[0].astype(np.int32)
    faces = surface_faces(m)
    d = str(tmp_path)
    surf, ctf = os.path.join(d, "bar.surf"), os.path.join(d, "bar.ctforces")
    write_surface(surf, faces)
    write_ctforces(ctf, surface=[(F, (0.0, 0.0, 1.0), 0, 0, faces_on_plane(m, faces, 2, nz * h))])
    paths = write_structure(m, d, "bar")
    script = os.path.join(d, "bar.ffea")
    write_script(script, paths, num_steps=300, check=100, dt=1e-13, kT=4.11e-21, epsilon=1e-2,
                 max_iterations_cg=1000, calc_noise=0, calc_stokes=0, ctforces=ctf, surface=surf)
    w = lib.World(script, precision=precision)
    x0 = w.blob(0).pos()
    w.run()
    end = np.nonzero(np.abs(m.pos[:, 2] - nz * h) < 1e-9)[0]
    dl = float((w.blob(0).pos()[end, 2] - x0[end, 2]).mean()) * lib.MESO_LENGTH
    # the same nodal forces in a static linear-elastic solve of the same mesh
    b = lib.Blob(m, solver="CG_nomass", dt=1e-13, kT=4.11e-21, calc_noise=0, epsilon=1e-2)
    b.load_ctforces(ctf, surf, 0)
    b.update(1)
    f_ext = b.rhs() * 2.4364705882352941e-11  # meso force -> N (mesoDimensions::force)
    assert abs(f_ext[:, 2].sum() / F - 1) < 1e-9 and abs(f_ext[:, :2]).sum() < 1e-9 * F
    u = linear_fe_extension(m, f_ext, m.pinned, G, K)
    dl_fe = float(u[end[end < m.n_linear], 2].mean())
    e_c = F * L / (A * dl)
    print(f"{precision}: extension {dl:.6e} m, static FE {dl_fe:.6e} m, E_c/E = {e_c / E:.4f} "
          f"(static FE {F * L / (A * dl_fe) / E:.4f})")
    assert abs(dl / dl_fe - 1) < 0.01
    assert abs(e_c / E - 1) < 0.02
