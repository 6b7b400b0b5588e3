"""Generate the golden vectors in this directory from the reference's own code.

Run in a container that has the reference sources (default /root/reference):

    make -C oracle ref
    OMP_NUM_THREADS=1 python tests/golden/gen_golden.py

It drives oracle/_ref/libffea_ref.so (the reference's own Blob with its
solvers, compiled from its sources by oracle/Makefile) through
oracle/pyoracle.py and writes small .npz files. OMP_NUM_THREADS=1 is required: the reference's
NoMass CG reductions and noise streams are only reproducible single-threaded,
which is also how the reference's own physics tests run them.

Inputs are seeded synthetic Kuhn cubes (ffea_ci_demo_gb300.mesh), so the
fixtures hold only outputs plus the seeds and sizes needed to rebuild inputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from ffea_ci_demo_gb300.mesh import (apply_shear, faces_on_plane, kuhn_cube, surface_faces,  # noqa: E402
                                     write_ctforces, write_surface)

MESO_LENGTH = 1.7e-10


def case_mesh(n, seed, pinned=None):
    m = kuhn_cube(n, side=20.0, seed=seed)
    if pinned is not None:
        m.pinned = np.asarray(pinned, np.int32)
    return m


def sheared(m, strain=0.02, seed=3):
    return apply_shear(m, strain, seed=seed) * (m.scale / MESO_LENGTH)


def gen_rng():
    po.RefRng.set_package_seed([12345] * 6)
    g = po.RefRng()
    draws = np.array([g.rand_u01() for _ in range(256)])
    g.reset_start_stream()
    sub = []
    for _ in range(4):
        sub.append([g.rand_u01() for _ in range(16)])
        g.reset_next_substream()
    states = {}
    g.reset_start_stream()
    g.advance_state(5, 3)
    states["adv_5_3"] = g.get_state()
    g.advance_state(-127, 0)
    states["adv_m127_0"] = g.get_state()
    g.reset_start_stream()
    g.advance_state(0, 7 * 1296)
    states["adv_0_9072"] = g.get_state()
    g2 = po.RefRng()  # second stream of the package (A^(2^127) later)
    stream2 = np.array([g2.rand_u01() for _ in range(16)])
    po.RefRng.set_package_seed([12345] * 6)
    known = po.rngstream_known_answer(po.RefRng, po.RefRng.set_package_seed)
    np.savez_compressed(os.path.join(HERE, "rng.npz"), draws=draws, substreams=np.array(sub), stream2=stream2,
                        known_answer=known, **{k: v for k, v in states.items()})


def ctf_case(m, directory, name="ctf"):
    """Constant-force inputs for a Kuhn cube of side 20 (file units, scale 1e-9 m): linear forces on a vertex
    (twice), on a midpoint and on every node; rotational forces about the cube's vertical axis ("pf" on a
    vertex and on every node, "pt" on the same vertex) and about an oblique axis ("pt" on a midpoint); two sets
    of surface faces, the top face z = 20 and half of the x = 0 face together with three top faces (so three
    faces carry both sets). Writes ``name``.ctforces and ``name``.surf into ``directory`` and returns their
    paths."""
    faces = surface_faces(m)
    top = faces_on_plane(m, faces, 2, 20.0)
    side = faces_on_plane(m, faces, 0, 0.0)
    ctf = os.path.join(directory, name + ".ctforces")
    surf = os.path.join(directory, name + ".surf")
    write_surface(surf, faces)
    write_ctforces(ctf, linear=[(2e-12, (1.0, 2.0, 3.0), 0, 0, 9), (5e-12, (0.0, 0.0, -1.0), 0, 0, m.n_linear + 7),
                                (3e-13, (1.0, 0.0, 0.0), 0, 0, "all"), (1e-12, (-1.0, 0.5, 0.0), 0, 0, 9),
                                (4e-12, (0.0, 1.0, 0.0), 1, 0, 3)],
                   rotational=[(3e-14, "pf", (1e-8, 1e-8, 0.0), (0.0, 0.0, 2.0), 0, 0, 22),
                               (1e-12, "pt", (0.0, 0.0, 0.0), (1.0, 1.0, 0.0), 0, 0, m.n_linear + 11),
                               (2e-14, "pf", (1e-8, 1e-8, 0.0), (0.0, 0.0, 1.0), 0, 0, "all"),
                               (5e-13, "pt", (1e-8, 1e-8, 0.0), (0.0, 0.0, 1.0), 0, 0, 22),
                               (1e-12, "pt", (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 1, 0, 5)],
                   surface=[(2e-11, (0.0, 0.0, 1.0), 0, 0, top),
                            (1e-11, (0.3, -1.0, 0.2), 0, 0, np.concatenate([side[: len(side) // 2], top[:3]])),
                            (1e-11, (1.0, 0.0, 0.0), 1, 0, top)])
    return ctf, surf


def file_digest(*paths):
    import hashlib
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def digest(*arrays):
    """sha256 of the arrays' bytes: pins large integer structures without storing them."""
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def dump_blob(name, m, pos0, steps, full=True, ctf=None, **kw):
    b = po.RefBlob(m, ctforces=ctf, **kw)
    b.set_pos(pos0)
    out = {"n": m.n_nodes, "T": m.n_elem, "steps": steps}
    if ctf is not None:
        out["ctf_sha256"] = file_digest(*ctf)
    rest = b.rest()
    out["jinv0"] = rest["jinv0"]
    out["mat"] = rest["mat"]
    c = b.contrib()
    out["contrib_ptr"], out["contrib_es"] = c["ptr"], c["elem_slot"]
    solver = kw.get("solver", "CG_nomass")
    if solver == "CG_nomass":
        csr = b.csr()
        out["csr_key"], out["csr_col"], out["csr_nsrc"] = csr["key"], csr["col"], csr["nsrc"]
    elif solver == "CG":
        mc = b.mass_csr()
        out["mass_key"], out["mass_col"], out["mass_val"] = mc["key"], mc["col"], mc["val"]
    else:
        out["inv_mass"] = b.inv_mass()
    assert b.step(1) == 0
    e = b.elem()
    out["step1_node_force"] = e["node_force"]
    out["step1_vol"] = e["vol"]
    out["step1_stress_mag"] = e["stress_mag"]
    if m.n_elem <= 64:
        out["step1_visc"] = e["visc"]
        out["step1_dpsi"] = e["dpsi"]
    out["step1_rhs"] = b.rhs()
    out["step1_pos"] = b.pos()
    out["step1_vel"] = b.vel()
    if solver == "CG_nomass":
        out["step1_csr_val"] = b.csr()["val"]
    if steps > 1:
        assert b.step(steps - 1) == 0
    out["final_pos"] = b.pos()
    out["final_vel"] = b.vel()
    out["final_rng"] = b.rng_state()
    out["final_energy"] = np.array(b.measure())
    if not full:
        keep = ("n", "T", "steps", "step1_rhs", "step1_vol", "final_pos", "final_vel", "final_rng", "final_energy")
        big = {k: v for k, v in out.items() if k not in keep}
        out = {k: out[k] for k in keep}
        out["contrib_sha256"] = digest(big["contrib_ptr"], big["contrib_es"])
        if "csr_key" in big:
            out["csr_sha256"] = digest(big["csr_key"], big["csr_col"], big["csr_nsrc"])
        if "mass_key" in big:
            out["mass_sha256"] = digest(big["mass_key"], big["mass_col"], big["mass_val"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, {k: getattr(v, "shape", v) for k, v in out.items() if k.startswith("final")})


def main():
    if os.environ.get("OMP_NUM_THREADS") != "1":
        raise SystemExit("set OMP_NUM_THREADS=1 (reference reductions are thread-count dependent)")
    gen_rng()
    # small cube, every per-element quantity kept
    m2 = case_mesh(2, seed=11)
    dump_blob("cube2_nomass_kT0", m2, sheared(m2), 20, solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0)
    dump_blob("cube2_nomass_noise", m2, sheared(m2), 20, solver="CG_nomass", dt=1e-12, kT=4.11e-21, calc_noise=1)
    # pinned nodes (vertex + midpoint) and Stokes drag/noise
    m3 = case_mesh(3, seed=7, pinned=[0, 1, 5, 64 + 2])
    dump_blob("cube3_nomass_pin_stokes", m3, sheared(m3), 10, solver="CG_nomass", dt=1e-12, kT=4.11e-21,
              calc_noise=1, calc_stokes=1)
    dump_blob("cube3_lumped_pin_stokes", m3, sheared(m3), 10, solver="masslumped", dt=1e-14, kT=4.11e-21,
              calc_noise=1, calc_stokes=1)
    dump_blob("cube3_cg_pin_stokes", m3, sheared(m3), 10, solver="CG", dt=1e-14, kT=4.11e-21,
              calc_noise=1, calc_stokes=1)
    # constant linear and surface forces (with the pins, drag and noise of the previous cases)
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        ctf = ctf_case(m3, d)
        common = dict(kT=4.11e-21, calc_noise=1, calc_stokes=1, ctf=ctf)
        dump_blob("cube3_nomass_ctf", m3, sheared(m3), 10, solver="CG_nomass", dt=1e-12, **common)
        dump_blob("cube3_lumped_ctf", m3, sheared(m3), 10, solver="masslumped", dt=1e-14, **common)
        dump_blob("cube3_cg_ctf", m3, sheared(m3), 10, solver="CG", dt=1e-14, **common)
        dump_blob("cube3_nomass_ctf_kT0", m3, sheared(m3), 20, solver="CG_nomass", dt=1e-12, kT=0.0, calc_noise=0,
                  calc_stokes=1, ctf=ctf)
    # the CPU-runnable benchmark cube: 6^3 cells, 1296 tets, 1000 steps
    m6 = case_mesh(6, seed=12345)
    for solver in ("masslumped", "CG"):
        dump_blob(f"cube6_{solver}_kT0_1000", m6, sheared(m6), 1000, full=False, solver=solver, dt=1e-14,
                  kT=0.0, calc_noise=0)
        dump_blob(f"cube6_{solver}_noise_1000", m6, sheared(m6, 0.0), 1000, full=False, solver=solver,
                  dt=1e-14, kT=4.11e-21, calc_noise=1)
    dump_blob("cube6_nomass_kT0_1000", m6, sheared(m6), 1000, full=False, solver="CG_nomass", dt=1e-12, kT=0.0,
              calc_noise=0)
    dump_blob("cube6_nomass_noise_100", m6, sheared(m6, 0.0), 100, full=False, solver="CG_nomass", dt=1e-12,
              kT=4.11e-21, calc_noise=1)


if __name__ == "__main__":
    main()
