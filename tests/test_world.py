""".ffea script front-end (ffea_gpu_world_*): World::init / World::run for the blob-step path.

* A script run must follow exactly the trajectory of the same blob stepped through the C ABI
  from the World's initial placement with the World's seed (bit-exact, FP64), write the
  checkpoint state the reference would (six (rand() + rand()) mod m seeds from rng_seed, then
  7 draws per element per step), and a frame / measurement row every `check` steps.
* A restart from the checkpoint and the trajectory's last frame continues the same stream;
  positions agree within the trajectory's 7 printed digits (the reference's own restart
  test allows 5e-4).
* Equipartition, as the reference's physics test checks it: the mean strain energy over the
  measurement file is (3N - 6) kT / 2 within 3%.
* Mode variances: over the same run's trajectory, the variance of each of the 3N - 6 internal normal
  modes of the small-strain stiffness (tests/fe.py) is the Boltzmann value kT / lambda_k. Each mode's
  ratio carries a sampling error sqrt(2 / n_eff) (n_eff from its autocorrelation): every mode lies within
  5 of those errors, and the mean ratio over the modes within 3% (the harmonic approximation and the
  Euler step, dt / tau <= 2%, each bias it by about 1%).
"""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

import pyoracle as po
from fe import mode_variance_ratios
from ffea_ci_demo_gb300 import build, lib
from ffea_ci_demo_gb300.mesh import kuhn_cube, write_script, write_structure

M1, M2 = 4294967087, 4294944443


def seeds_from(rng_seed):
    """World::init's package seed: srand(rng_seed), then (rand() + rand()) % m1 (x3) and % m2 (x3)."""
    libc = C.CDLL(None)
    libc.srand(C.c_uint(rng_seed))
    return np.array([(libc.rand() + libc.rand()) % (M1 if k < 3 else M2) for k in range(6)], np.uint32)


def make_script(tmp, name, n=2, **kw):
    m = kuhn_cube(n, side=10.0, seed=4)
    paths = write_structure(m, str(tmp), name)
    path = os.path.join(str(tmp), name + ".ffea")
    write_script(path, paths, scale=1e-9, **kw)
    return m, paths, path


def read_fm(path):
    with open(path) as f:
        lines = f.read().split("\n")
    k = lines.index("Measurements:")
    head = lines[k + 1].split()
    rows = [list(map(float, ln.split())) for ln in lines[k + 2:] if ln.strip()]
    return head, np.array(rows)


def frames(path):
    with open(path) as f:
        txt = f.read()
    return [int(ln.split("step")[1]) for ln in txt.split("\n") if ln.startswith("Blob 0, Conformation 0, step")]


def read_ftj(path, n_take):
    """Positions (m) of the first n_take nodes of blob 0 in every frame of a trajectory file."""
    out = []
    with open(path) as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines):
        if lines[i].startswith("Blob 0, Conformation 0, step"):
            rows = lines[i + 2:i + 2 + n_take]
            out.append([[float(x) for x in r.split()[:3]] for r in rows])
            i += 2 + n_take
        else:
            i += 1
    return np.array(out)


def test_script_refusals(tmp_path):
    build.build()
    _, paths, path = make_script(tmp_path, "c")
    txt = open(path).read()
    L = lib.load()
    h = C.c_void_p()
    for old, new in (("<calc_steric = 0>", "<calc_steric = 1>"), ("<calc_es = 0>", "<calc_es = 1>"),
                     ("<calc_ssint = 0>", ""), ("<num_conformations = (1)>", "<num_conformations = (2)>"),
                     ("<kT = ", "<colour = blue>\n\t<kT = ")):
        bad = os.path.join(str(tmp_path), "bad.ffea")
        with open(bad, "w") as f:
            f.write(txt.replace(old, new))
        assert L.ffea_gpu_world_load(bad.encode(), 0, C.byref(h)) == lib.EINPUT, (old, new)
        assert lib.last_error()


@pytest.mark.gpu
def test_world_run_matches_blob_and_reference_seeding(gpu, oracle_built, tmp_path):
    m, paths, path = make_script(tmp_path, "w", num_steps=20, check=5, rng_seed=777, kT=4.11e-21, calc_noise=1,
                                 dt=1e-12)
    w = lib.World(path)
    x0 = w.blob(0).pos()
    w.run()
    xw = w.blob(0).pos()
    seed = seeds_from(777)
    b = lib.Blob.from_files(paths["node"], paths["top"], paths["mat"], paths["stokes"], paths["pin"], 1e-9,
                            solver="CG_nomass", rng_state=seed, dt=1e-12, kT=4.11e-21, epsilon=1e-10, calc_noise=1,
                            calc_stokes=0, max_iterations_cg=10000)
    b.set_state(pos=x0)
    b.update(21)  # steps 0..num_steps inclusive, as World::run
    assert np.array_equal(xw, b.pos())
    # the checkpoint holds the stream before step 20's forces: the seed advanced by 20 x 7T draws
    o = po.OracleRng()
    o.set_state(seed)
    for _ in range(20 * 7 * m.n_elem):
        o.rand_u01()
    line = open(os.path.join(str(tmp_path), "w.fcp")).read().split("\n")
    assert line[0].startswith("RNGStreams dedicated to the thermal stress:")
    assert np.array_equal(np.array(line[1].split(), np.uint32), o.get_state())
    assert frames(os.path.join(str(tmp_path), "w.ftj")) == [0, 5, 10, 15, 20]
    head, rows = read_fm(os.path.join(str(tmp_path), "w.fm"))
    assert head == ["Time", "StrainEnergy", "Centroid[0]", "Centroid[1]", "Centroid[2]", "RMSD"]
    assert rows.shape == (5, 6) and rows[0, 5] == 0.0 and rows[-1, 5] > 0.0
    # the system centroid sits at the centre of the simulation box (move_into_box)
    assert np.allclose(rows[0, 2:5], rows[0, 2:5].mean(), rtol=1e-6)


@pytest.mark.gpu
def test_world_restart_continues_the_stream(gpu, tmp_path):
    _, _, full = make_script(tmp_path, "full", num_steps=20, check=5, rng_seed=99)
    wa = lib.World(full)
    wa.run()
    xa = wa.blob(0).pos()
    ra = open(os.path.join(str(tmp_path), "full.fcp")).read()
    _, _, first = make_script(tmp_path, "part", num_steps=10, check=5, rng_seed=99)
    lib.World(first).run()
    shutil.copy(os.path.join(str(tmp_path), "part.fcp"), os.path.join(str(tmp_path), "part_in.fcp"))
    txt = open(first).read().replace("<restart = 0>", "<restart = 1>").replace(
        "<num_steps = 10>", "<num_steps = 20>\n\t<checkpoint_in = part_in.fcp>\n\t<checkpoint_out = part.fcp>")
    with open(first, "w") as f:
        f.write(txt)
    wb = lib.World(first)
    wb.run()
    xb = wb.blob(0).pos()
    assert open(os.path.join(str(tmp_path), "part.fcp")).read() == ra
    assert np.abs(xb - xa).max() <= 5e-4 * np.abs(xa).max()
    assert frames(os.path.join(str(tmp_path), "part.ftj")) == [0, 5, 10, 15, 20]
    assert read_fm(os.path.join(str(tmp_path), "part.fm"))[1].shape[0] == 5


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_equipartition_of_strain_energy(gpu, tmp_path, precision):
    n = 2
    steps, check = 120000, 300
    m, _, path = make_script(tmp_path, "eq", n=n, num_steps=steps, check=check, rng_seed=2024, dt=1e-14,
                             kT=4.11e-21, calc_noise=1, epsilon=1e-6)
    import time
    t0 = time.perf_counter()
    lib.World(path, precision=precision).run()
    print(f"{precision}: {(time.perf_counter() - t0) / steps * 1e6:.1f} us per step (27-node blob)")
    head, rows = read_fm(os.path.join(str(tmp_path), "eq.fm"))
    se = rows[40:, head.index("StrainEnergy")]
    nodes = (n + 1) ** 3
    want = 4.11e-21 * (3 * nodes - 6) / 2
    dev = abs(se.mean() / want - 1)
    print(precision, "equipartition: mean strain energy / (3N-6)kT/2 - 1 =", dev, "samples", se.size)
    assert dev < 0.03
    # mode variances over the trajectory frames (the first 40 dropped, as above)
    frames = read_ftj(os.path.join(str(tmp_path), "eq.ftj"), nodes)[40:]
    ratio, neff = mode_variance_ratios(frames, m.pos[:nodes] * 1e-9, m.tets[:, :4], 5.7e8, 2.2e9, 4.11e-21)
    z = (ratio - 1) / np.sqrt(2.0 / neff)
    print(precision, f"mode variances: {ratio.size} modes, mean ratio {ratio.mean():.4f}, range "
          f"[{ratio.min():.3f}, {ratio.max():.3f}], n_eff {neff.min():.0f}-{neff.max():.0f}, max |z| {np.abs(z).max():.2f}")
    assert ratio.size == 3 * nodes - 6
    assert np.abs(z).max() < 5.0
    assert abs(ratio.mean() - 1) < 0.03


GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.gpu
@pytest.mark.parametrize("solver,tol", [("CG", {"KineticEnergy": 0.04, "StrainEnergy": 0.03}),
                                        ("CG_nomass", {"StrainEnergy": 0.03})])
def test_reference_sphere_equipartition(gpu, tmp_path, solver, tol):
    """The reference's physics tests tests/physics/sphere_63_120_mass and _nomass on their own mesh
    (tests/golden/sphere_63_120.npz, made by gen_sphere.py from the reference's structure files): 1e5 steps
    of 1e-14 s with Stokes drag and noise, CG tolerance 1e-2, and the averages of the measurement rows
    40 .. second to last (testAverages.py): kinetic energy within 4% of 3N kT / 2 and strain energy within 3%
    of (3N - 6) kT / 2, N = 63 vertices. The reference's script leaves calc_steric at its default of 1; here
    it is 0, as the front-end refuses surface interactions (they act only when surface faces overlap)."""
    from ffea_ci_demo_gb300.mesh import Mesh

    z = np.load(os.path.join(GOLD, "sphere_63_120.npz"))
    m = Mesh(pos=z["pos"], tets=z["tets"], material=z["material"], stokes_radius=z["stokes_radius"],
             pinned=z["pinned"], scale=float(z["scale"]), n_linear=int(z["n_linear"]))
    paths = write_structure(m, str(tmp_path), "sphere")
    path = os.path.join(str(tmp_path), "sphere.ffea")
    write_script(path, paths, solver=solver, scale=m.scale, dt=1e-14, kT=4.11e-21, epsilon=0.01,
                 max_iterations_cg=1000, calc_noise=1, calc_stokes=1, stokes_visc=1e-3, rng_seed=44,
                 num_steps=100000, check=1000)
    lib.World(path).run()
    head, rows = read_fm(os.path.join(str(tmp_path), "sphere.fm"))
    assert rows.shape[0] == 101
    kT, n = 4.11e-21, 63
    want = {"KineticEnergy": kT * 3 * n / 2, "StrainEnergy": kT * (3 * n - 6) / 2}
    for key, t in tol.items():
        dev = abs(rows[40:-1, head.index(key)].mean() / want[key] - 1)
        print(solver, key, "deviation", dev, "bound", t)
        assert dev < t, (key, dev)


@pytest.mark.gpu
def test_two_blob_script_shares_one_stream(gpu, oracle_built, tmp_path):
    """Two blobs in one script: World::run's single-thread order draws blob 0's elements, then blob 1's, from
    one stream every step. Each blob must follow the oracle stepped on its slice of that stream (FP64 CG to
    rounding, <= 1e-8 of the displacement), and the checkpoint must hold the stream after every step's
    7 (T0 + T1) draws."""
    ma, mb = kuhn_cube(2, side=10.0, seed=4), kuhn_cube(3, side=12.0, seed=9)
    pa = write_structure(ma, str(tmp_path), "a")
    pb = write_structure(mb, str(tmp_path), "b")
    path = os.path.join(str(tmp_path), "two.ffea")
    write_script(path, pa, num_steps=6, check=3, rng_seed=321, dt=1e-12, calc_noise=1, kT=4.11e-21)
    txt = open(path).read()
    blob_b = "\t<blob>\n\t\t<conformation>\n\t\t\t<motion_state = DYNAMIC>\n" + "".join(
        f"\t\t\t<{k} = {os.path.basename(pb[f])}>\n" for k, f in
        (("nodes", "node"), ("topology", "top"), ("material", "mat"), ("stokes", "stokes"), ("pin", "pin"))) + \
        "\t\t</conformation>\n\t\t<solver = CG_nomass>\n\t\t<scale = 1e-09>\n\t\t<centroid = (30.0, 0.0, 0.0)>\n\t</blob>\n"
    txt = txt.replace("<num_blobs = 1>", "<num_blobs = 2>").replace("<num_conformations = (1)>",
                                                                     "<num_conformations = (1,1)>")
    txt = txt.replace("</system>", blob_b + "</system>")
    with open(path, "w") as f:
        f.write(txt)
    w = lib.World(path)
    assert w.num_blobs == 2
    x0 = [w.blob(0).pos(), w.blob(1).pos()]
    w.run()
    T0, T1 = ma.n_elem, mb.n_elem
    state = seeds_from(321)
    kw = dict(dt=1e-12, kT=4.11e-21, calc_noise=1, epsilon=1e-10)
    oa, ob = po.OracleBlob(ma, threads=1, **kw), po.OracleBlob(mb, threads=1, **kw)
    oa.set_pos(x0[0])
    ob.set_pos(x0[1])
    g = po.OracleRng()
    for _ in range(7):  # steps 0..6
        g.set_state(state)
        oa.set_rng_state(state)
        assert oa.step(1) == 0
        for _ in range(7 * T0):
            g.rand_u01()
        ob.set_rng_state(g.get_state())
        assert ob.step(1) == 0
        for _ in range(7 * T1):
            g.rand_u01()
        state = g.get_state()
    for b, o in enumerate((oa, ob)):
        d = np.abs(w.blob(b).pos() - o.pos()).max() / np.abs(o.pos() - x0[b]).max()
        assert d < 1e-8, (b, d)
    # the checkpoint written before step 6's forces: the stream after 6 steps
    g.set_state(seeds_from(321))
    for _ in range(6 * 7 * (T0 + T1)):
        g.rand_u01()
    line = open(os.path.join(str(tmp_path), "two.fcp")).read().split("\n")
    assert np.array_equal(np.array(line[1].split(), np.uint32), g.get_state())
