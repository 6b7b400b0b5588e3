"""Replica batch (ffea_gpu_batch_*): many blobs of uneven size in one graph-captured step.

Each blob of a batch must follow the trajectory the single-blob mixed path gives
for it (same element math, same noise draws; only the CG's cross-node sums are
split over a different set of CTAs, so positions agree to the CG's rounding),
and its noise must come from substream b of the package seed, bit-exact
against the oracle's RngStream restatement (itself pinned to the reference's
known answer).

Tolerances: batch vs single-blob mixed path <= 1e-5 of the largest displacement
after 10 steps at kT > 0 (FP32 CG rounding, the mixed path's own bound against
FP64); batch at kT = 0 vs the FP64 path <= 1e-5 after 200 steps; CG iteration
counts within 2 of the single blob's; RNG states bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
from ffea_ci_demo_gb300 import build, lib
from ffea_ci_demo_gb300.lib import MESO_LENGTH
from ffea_ci_demo_gb300.mesh import write_ctforces
from gen_golden import case_mesh, ctf_case, sheared


def substream_states(n):
    po.OracleRng.set_package_seed([12345] * 6)
    g = po.OracleRng()
    out = []
    for _ in range(n):
        out.append(g.get_state())
        g.reset_next_substream()
    return out


def test_batch_rejects_unsupported_params_without_gpu_work():
    build.build()
    L = lib.load()
    h = C.c_void_p()
    arr = (lib.MeshStruct * 1)()
    for prec, solver in (("fp64", "CG_nomass"), ("mixed", "masslumped")):
        p = lib.make_params(solver=solver, precision=prec)
        assert L.ffea_gpu_batch_create(C.cast(arr, C.c_void_p), 1, C.byref(p), C.byref(h)) == lib.EINPUT
    p = lib.make_params(solver="CG_nomass", precision="mixed")
    assert L.ffea_gpu_batch_create(C.cast(arr, C.c_void_p), 0, C.byref(p), C.byref(h)) == lib.EINPUT
    assert L.ffea_gpu_batch_step(None, 1, None) == lib.EINPUT


MESHES = [(3, 5), (5, 8), (2, 13), (4, 21), (6, 2)]


@pytest.mark.gpu
def test_batch_rng_substreams(gpu, oracle_built):
    meshes = [case_mesh(n, s) for n, s in MESHES]
    bt = lib.Batch(meshes, calc_noise=1)
    want = substream_states(len(meshes))
    for b in range(len(meshes)):
        assert np.array_equal(bt.rng_state(b), want[b]), b
    # after one step each stream has advanced by 7 draws per element of its blob
    bt.update(1)
    for b, m in enumerate(meshes):
        o = po.OracleRng()
        o.set_state(want[b])
        for _ in range(7 * m.n_elem):
            o.rand_u01()
        assert np.array_equal(bt.rng_state(b), o.get_state()), b


@pytest.mark.gpu
def test_batch_matches_single_blobs(gpu, oracle_built):
    meshes = [case_mesh(n, s) for n, s in MESHES]
    kw = dict(dt=1e-12, kT=4.11e-21, calc_noise=1)
    bt = lib.Batch(meshes, **kw)
    x0 = [sheared(m, 0.02, seed=7 + b) for b, m in enumerate(meshes)]
    for b in range(len(meshes)):
        bt.set_state(b, pos=x0[b])
    bt.update(10)
    its, _ = bt.cg_iterations()
    for b, m in enumerate(meshes):
        s = lib.Blob(m, solver="CG_nomass", precision="mixed", cg_poly=-1, rng_state=substream_states(b + 1)[b],
                     **kw)
        s.set_state(pos=x0[b])
        s.update(10)
        err = np.abs(bt.pos(b) - s.pos()).max() / np.abs(s.pos() - x0[b]).max()
        print(f"blob {b}: {m.n_elem} tets, batch vs single error {err:.2e}, iterations {its[b]} / "
              f"{s.cg_iterations()[0]}")
        assert err < 1e-5, b
        assert abs(int(its[b]) - s.cg_iterations()[0]) <= 2, b
        assert np.array_equal(bt.rng_state(b), s.rng_state()), b


@pytest.mark.gpu
def test_batch_stokes_noise_matches_single_blobs(gpu, oracle_built):
    """Stokes drag with noise: each blob draws 3 numbers per node of its own numbering after its elements' 7 per
    element (Blob::aggregate_forces_and_solve, src/Blob.cpp:3190-3219), from its own substream; midpoints' draws
    reach the vertices through the linearise replay. Same bounds as without Stokes noise."""
    meshes = [case_mesh(n, s) for n, s in MESHES]
    kw = dict(dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=1)
    bt = lib.Batch(meshes, **kw)
    x0 = [sheared(m, 0.02, seed=11 + b) for b, m in enumerate(meshes)]
    for b in range(len(meshes)):
        bt.set_state(b, pos=x0[b])
    bt.update(1)
    want = substream_states(len(meshes))
    for b, m in enumerate(meshes):
        o = po.OracleRng()
        o.set_state(want[b])
        for _ in range(7 * m.n_elem + 3 * m.n_nodes):
            o.rand_u01()
        assert np.array_equal(bt.rng_state(b), o.get_state()), b
    bt.update(9)
    its, _ = bt.cg_iterations()
    for b, m in enumerate(meshes):
        s = lib.Blob(m, solver="CG_nomass", precision="mixed", cg_poly=-1, rng_state=want[b], **kw)
        s.set_state(pos=x0[b])
        s.update(10)
        err = np.abs(bt.pos(b) - s.pos()).max() / np.abs(s.pos() - x0[b]).max()
        print(f"blob {b}: {m.n_elem} tets, Stokes noise, batch vs single error {err:.2e}, iterations {its[b]} / "
              f"{s.cg_iterations()[0]}")
        assert err < 1e-5, b
        assert abs(int(its[b]) - s.cg_iterations()[0]) <= 2, b
        assert np.array_equal(bt.rng_state(b), s.rng_state()), b


@pytest.mark.gpu
def test_batch_constant_forces_match_single_blobs(gpu, oracle_built, tmp_path):
    """Constant forces (Blob::apply_ctforces, src/Blob.cpp:1676-1743) per blob of a batch: linear, rotational
    and surface forces on vertices and midpoints, loaded for blob 0 (the file's blob-0 entries) and blob 1 (the
    file's blob-1 entries), none on blob 2; Stokes drag and noise on. Each blob follows the single mixed blob
    given the same files, within the bounds above."""
    meshes = [case_mesh(3, 7, [0, 1, 5, 66]), case_mesh(4, 21), case_mesh(3, 5)]
    files = [ctf_case(meshes[0], str(tmp_path), "b0"), ctf_case(meshes[1], str(tmp_path), "b1"), None]
    kw = dict(dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=1)
    bt = lib.Batch(meshes, **kw)
    x0 = [sheared(m, 0.02, seed=5 + b) for b, m in enumerate(meshes)]
    for b in range(len(meshes)):
        bt.set_state(b, pos=x0[b])
        if files[b]:
            bt.load_ctforces(b, *files[b], blob_index=b)
    bt.update(10)
    its, _ = bt.cg_iterations()
    want = substream_states(len(meshes))
    for b, m in enumerate(meshes):
        s = lib.Blob(m, solver="CG_nomass", precision="mixed", cg_poly=-1, rng_state=want[b], **kw)
        if files[b]:
            s.load_ctforces(*files[b], blob_index=b)
        s.set_state(pos=x0[b])
        s.update(10)
        err = np.abs(bt.pos(b) - s.pos()).max() / np.abs(s.pos() - x0[b]).max()
        print(f"blob {b}: constant forces {'yes' if files[b] else 'no'}, batch vs single error {err:.2e}, "
              f"iterations {its[b]} / {s.cg_iterations()[0]}")
        assert err < 1e-5, b
        assert abs(int(its[b]) - s.cg_iterations()[0]) <= 2, b
        assert np.array_equal(bt.rng_state(b), s.rng_state()), b
    # replacing one blob's forces leaves the others' in place: a file whose only force is another blob's
    # takes blob 1's away
    none = str(tmp_path / "none.ctforces")
    write_ctforces(none, linear=[(1e-12, (1.0, 0.0, 0.0), 7, 0, 3)])
    bt.load_ctforces(1, none, blob_index=1)
    with pytest.raises(lib.FFEAError):
        bt.load_ctforces(0, str(tmp_path / "missing.ctforces"))
    start = [(bt.pos(b), bt.rng_state(b)) for b in range(2)]
    bt.update(5)
    for b in range(2):
        s = lib.Blob(meshes[b], solver="CG_nomass", precision="mixed", cg_poly=-1, rng_state=start[b][1], **kw)
        if b == 0:
            s.load_ctforces(*files[0], blob_index=0)
        s.set_state(pos=start[b][0])
        s.update(5)
        err = np.abs(bt.pos(b) - s.pos()).max() / np.abs(s.pos() - start[b][0]).max()
        print(f"blob {b} after replacing blob 1's forces: batch vs single error {err:.2e}")
        assert err < 1e-5, b


@pytest.mark.gpu
def test_batch_kT0_error_vs_fp64():
    meshes = [case_mesh(n, s) for n, s in ((4, 1), (6, 12345), (3, 9))]
    kw = dict(dt=1e-12, kT=0.0, calc_noise=0)
    bt = lib.Batch(meshes, **kw)
    x0 = [sheared(m, 0.02) for m in meshes]
    for b in range(len(meshes)):
        bt.set_state(b, pos=x0[b])
    bt.update(200)
    for b, m in enumerate(meshes):
        f = lib.Blob(m, solver="CG_nomass", precision="fp64", **kw)
        f.set_state(pos=x0[b])
        f.update(200)
        err = np.abs(bt.pos(b) - f.pos()).max() / np.abs(f.pos() - x0[b]).max()
        print(f"blob {b}: kT=0 200-step error vs FP64 {err:.2e}")
        assert err < 1e-5, b


@pytest.mark.gpu
def test_batch_pinned_blob():
    meshes = [case_mesh(4, 3, [0, 1, 5]), case_mesh(3, 4)]
    kw = dict(kT=0.0, calc_noise=0)
    bt = lib.Batch(meshes, **kw)
    x0 = [sheared(m, 0.02) for m in meshes]
    for b in range(2):
        bt.set_state(b, pos=x0[b])
    bt.update(20)
    for b, m in enumerate(meshes):
        f = lib.Blob(m, solver="CG_nomass", precision="fp64", **kw)
        f.set_state(pos=x0[b])
        f.update(20)
        assert np.abs(bt.pos(b) - f.pos()).max() / np.abs(f.pos() - x0[b]).max() < 1e-5, b
    p = bt.pos(0)
    assert np.array_equal(p[[0, 1, 5]], x0[0][[0, 1, 5]])


@pytest.mark.gpu
def test_batch_tuner_keeps_state():
    meshes = [case_mesh(n, s) for n, s in MESHES]
    bt = lib.Batch(meshes, calc_noise=1)
    bt.update(2)
    before = [bt.state(b) for b in range(len(meshes))]
    rng = [bt.rng_state(b) for b in range(len(meshes))]
    total = bt.cg_iterations()[1]
    best = bt.tune(solves=1)
    cfg = bt.config()
    assert best > 0 and cfg["cg_threads"] in (128, 256, 512, 1024) and cfg["threads_per_row"] in (1, 2, 4, 8)
    assert cfg["element_threads"] in (64, 128, 256) and cfg["assembly_threads"] in (64, 128, 256)
    assert cfg["assembly_split"] in (1, 2) and cfg["gather_threads"] in (64, 128, 256)
    for b in range(len(meshes)):
        p, v = bt.state(b)
        assert np.array_equal(p, before[b][0]) and np.array_equal(v, before[b][1])
        assert np.array_equal(bt.rng_state(b), rng[b])
    assert bt.cg_iterations()[1] == total
    bt.update(2)  # the tuned configuration steps
    # every configuration gives the same trajectory to rounding
    ref = lib.Batch(meshes, calc_noise=1)
    ref.update(4)
    for b, m in enumerate(meshes):
        p0 = m.pos * (m.scale / MESO_LENGTH)
        d = np.abs(bt.pos(b) - ref.pos(b)).max()
        assert d <= 1e-5 * np.abs(ref.pos(b) - p0).max(), b


@pytest.mark.gpu
def test_batch_launch_shapes_give_one_trajectory():
    """Every force-phase launch shape (elements per block, assembly block and split, gather block) steps the
    batch along the default shape's trajectory to FP32 rounding (only the per-block force sums regroup);
    the RNG states stay bit-exact."""
    meshes = [case_mesh(n, s) for n, s in MESHES]
    kw = dict(calc_noise=1, calc_stokes=1)
    ref = lib.Batch(meshes, **kw)
    ref.update(6)
    shapes = [(64, 64, 1, 64), (256, 256, 2, 128), (128, 128, 0, 256), (256, 64, 2, 256)]
    for sh in shapes:
        bt = lib.Batch(meshes, **kw)
        bt.set_shapes(*sh)
        cfg = bt.config()
        assert (cfg["element_threads"], cfg["assembly_threads"], cfg["assembly_split"], cfg["gather_threads"]) == sh
        bt.update(6)
        for b, m in enumerate(meshes):
            p0 = m.pos * (m.scale / MESO_LENGTH)
            d = np.abs(bt.pos(b) - ref.pos(b)).max()
            assert d <= 1e-5 * np.abs(ref.pos(b) - p0).max(), (sh, b)
            assert np.array_equal(bt.rng_state(b), ref.rng_state(b)), (sh, b)
    with pytest.raises(lib.FFEAError):
        bt.set_shapes(96, 128, 0, 256)


@pytest.mark.gpu
def test_batch_bulk_state_matches_per_blob_calls():
    """ffea_gpu_batch_get_states / set_states: every blob's reference-layout array back to back, the same values
    as the per-blob calls (midpoints included), and a bulk set moves each blob as the per-blob set does."""
    meshes = [case_mesh(n, s) for n, s in MESHES]
    bt = lib.Batch(meshes, kT=0.0, calc_noise=0)
    bt.update(2)
    allpos = bt.positions()
    off = np.cumsum([0] + [m.n_nodes for m in meshes])
    for b in range(len(meshes)):
        assert np.array_equal(allpos[off[b]:off[b + 1]], bt.pos(b))
    x0 = np.concatenate([sheared(m, 0.02) for m in meshes])
    bt.set_positions(x0)
    for b, m in enumerate(meshes):
        got, want = bt.pos(b), x0[off[b]:off[b + 1]]
        nv = m.n_linear  # vertices exactly; midpoints as the device linearises them
        assert np.array_equal(got[:nv], want[:nv])
        np.testing.assert_allclose(got[nv:], want[nv:], rtol=1e-14)
    bt.update(5)
    ref = lib.Batch(meshes, kT=0.0, calc_noise=0)
    ref.update(2)  # the same CTA schedule as bt's
    for b, m in enumerate(meshes):
        ref.set_state(b, pos=sheared(m, 0.02))
    ref.update(5)
    assert np.array_equal(bt.positions(), ref.positions())


@pytest.mark.gpu
def test_batch_strain_energies_match_single_blobs():
    """ffea_gpu_batch_strain_energies: each blob's StrainEnergy of Blob::make_measurements, as the single mixed
    blob measures it at the same positions (FP64 sums in another order: 1e-12)."""
    meshes = [case_mesh(n, s) for n, s in MESHES]
    bt = lib.Batch(meshes, kT=0.0, calc_noise=0)
    x0 = [sheared(m, 0.02, seed=3 + b) for b, m in enumerate(meshes)]
    for b in range(len(meshes)):
        bt.set_state(b, pos=x0[b])
    se = bt.strain_energies()
    for b, m in enumerate(meshes):
        s = lib.Blob(m, solver="CG_nomass", precision="mixed", kT=0.0, calc_noise=0)
        s.set_state(pos=x0[b])
        want = s.measurements()["strain_energy"]
        assert want > 0 and abs(se[b] - want) <= 1e-12 * want, b


@pytest.mark.gpu
def test_batch_ragged_edge_cases(gpu, oracle_built):
    """Ragged batches: a batch of one blob, and a batch mixing a one-element blob, a blob with pinned nodes and an
    ordinary one, Stokes drag and noise on; each blob follows the single mixed blob from the same stream state."""
    from test_mixed_elements import one_tet

    kw = dict(dt=1e-12, kT=4.11e-21, calc_noise=1, calc_stokes=1)
    for meshes in ([case_mesh(4, 7)], [one_tet(), case_mesh(3, 4, [0, 1, 5]), case_mesh(5, 2)]):
        bt = lib.Batch(meshes, **kw)
        x0 = [sheared(m, 0.02, seed=21 + b) for b, m in enumerate(meshes)]
        want = substream_states(len(meshes))
        for b in range(len(meshes)):
            bt.set_state(b, pos=x0[b])
        bt.update(6)
        for b, m in enumerate(meshes):
            s = lib.Blob(m, solver="CG_nomass", precision="mixed", cg_poly=-1, rng_state=want[b], **kw)
            s.set_state(pos=x0[b])
            s.update(6)
            scale = np.abs(s.pos() - x0[b]).max()
            assert scale > 0, b
            assert np.abs(bt.pos(b) - s.pos()).max() <= 1e-5 * scale, (len(meshes), b)
            assert np.array_equal(bt.rng_state(b), s.rng_state()), (len(meshes), b)
        if len(meshes) > 1:
            p = bt.pos(1)
            assert np.array_equal(p[[0, 1, 5]], x0[1][[0, 1, 5]])


@pytest.mark.gpu
def test_batch_largest_and_refused_counts(gpu):
    """The most blobs a batch takes: one CG CTA per blob resident at once (the grid of 128-thread CTAs). That many
    small blobs step together, each as its single blob does; one more, and more than FFEA_GPU_BATCH_MAX_BLOBS, are
    refused with EINPUT."""
    import ctypes as C

    probe = lib.Batch([case_mesh(2, 1)], kT=0.0, calc_noise=0)
    probe.set_config(128, 1)
    cap = probe.config()["ctas"]
    probe.close()
    meshes = [case_mesh(2, 1000 + b) for b in range(cap)]
    bt = lib.Batch(meshes, kT=0.0, calc_noise=0)
    assert bt.config()["ctas"] >= cap
    x0 = [sheared(m, 0.02, seed=b) for b, m in enumerate(meshes)]
    bt.set_positions(np.concatenate(x0))
    bt.update(3)
    for b in (0, cap // 2, cap - 1):
        s = lib.Blob(meshes[b], solver="CG_nomass", precision="fp64", kT=0.0, calc_noise=0)
        s.set_state(pos=x0[b])
        s.update(3)
        assert np.abs(bt.pos(b) - s.pos()).max() <= 1e-5 * np.abs(s.pos() - x0[b]).max(), b
    bt.close()
    L = lib.load()
    for n in (cap + 1, 2049):
        many = [case_mesh(2, 7)] * n
        keep: list = []
        arr = (lib.MeshStruct * n)(*[lib._mesh_struct(m, keep) for m in many])
        p = lib.make_params(solver="CG_nomass", precision="mixed")
        h = C.c_void_p()
        assert L.ffea_gpu_batch_create(C.cast(arr, C.c_void_p), n, C.byref(p), C.byref(h)) == lib.EINPUT, n
