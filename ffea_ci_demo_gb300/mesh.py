"""Seeded synthetic FFEA meshes and the FFEA structure-file formats.

The benchmark and parity meshes are cubes split into n^3 cells, each cell
Kuhn-split into 6 linear tetrahedra that share the cell's (0,0,0)-(1,1,1)
diagonal, so the mesh is conforming. FFEA stores "quadratic topology"
tetrahedra: 10 node indices per element, the last six being edge midpoints
in the order fixed by ``tetra_element_linear::linearise_element``
(src/tetra_element_linear.cpp:553-577): n4=(0,1) n5=(0,2) n6=(0,3) n7=(1,2)
n8=(1,3) n9=(2,3).

Node numbering: the (n+1)^3 vertex ("linear") nodes come first in x-fastest
lexicographic order, then one midpoint ("secondary") node per unique edge.
Every node is declared a surface node (``num_interior_nodes 0``) so that the
reference never builds its electrostatics Poisson matrix for these meshes
(src/Blob.cpp:278, only when ``num_interior_nodes > 0``).

File formats follow the reference loaders: ``.node`` Blob::load_nodes
(src/Blob.cpp:1911-1989), ``.top`` Blob::load_topology (:1993-2083),
``.mat`` Blob::load_material_params (:2241-2293), ``.stokes``
Blob::load_stokes_params (:2297-2353), ``.pin`` Blob::load_pinned_nodes
(:3024-3076).
"""
from __future__ import annotations

import itertools
import os
from dataclasses import dataclass, field

import numpy as np

# The six Kuhn tetrahedra of a unit cell, one per permutation of the axes.
_UNIT = np.eye(3, dtype=np.int64)
# local edge (a, b) for midpoint slots 4..9
MID_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))


@dataclass
class Mesh:
    """An FFEA blob's structure in file units (SI material, positions x scale)."""

    pos: np.ndarray            # (N_all, 3) float64, file units
    tets: np.ndarray           # (T, 10) int32, 10-node topology
    material: np.ndarray       # (T, 6) float64: rho, shear_visc, bulk_visc, G, K, dielectric (SI)
    stokes_radius: np.ndarray  # (N_all,) float64, file units
    pinned: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    scale: float = 1e-9        # metres per file unit (the .ffea ``scale`` key)
    n_linear: int = 0          # number of vertex nodes (they come first)

    @property
    def n_nodes(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_elem(self) -> int:
        return int(self.tets.shape[0])


def kuhn_cube(n: int, side: float = 20.0, *, jitter: float = 0.05, seed: int = 12345,
              density: float = 1500.0, shear_mod: float = 5.7e8, bulk_mod: float = 2.2e9,
              shear_visc: float = 1e-3, bulk_visc: float = 1e-3, dielectric: float = 1.0,
              scale: float = 1e-9, stokes_radius: float | None = None) -> Mesh:
    """Cube of side ``side`` (file units) split into n^3 cells x 6 Kuhn tets.

    Interior vertex nodes are jittered uniformly by +-``jitter`` of the cell
    size (seeded); boundary vertex nodes stay on the cube faces. Midpoint
    nodes sit exactly on their edge midpoints. T = 6 n^3, N = (n+1)^3,
    N_all = (2n+1)^3.
    """
    if n < 1:
        raise ValueError("n must be >= 1")
    return kuhn_box(n, n, n, side / n, jitter=jitter, seed=seed, density=density, shear_mod=shear_mod,
                    bulk_mod=bulk_mod, shear_visc=shear_visc, bulk_visc=bulk_visc, dielectric=dielectric,
                    scale=scale, stokes_radius=stokes_radius)


def kuhn_box(nx: int, ny: int, nz: int, h: float, *, jitter: float = 0.05, seed: int = 12345,
             density: float = 1500.0, shear_mod: float = 5.7e8, bulk_mod: float = 2.2e9,
             shear_visc: float = 1e-3, bulk_visc: float = 1e-3, dielectric: float = 1.0,
             scale: float = 1e-9, stokes_radius: float | None = None) -> Mesh:
    """Box of nx x ny x nz cubic cells of edge ``h`` (file units), 6 Kuhn tets per cell, numbered as
    :func:`kuhn_cube` (vertices x fastest, then midpoints in first-appearance order)."""
    if min(nx, ny, nz) < 1:
        raise ValueError("cell counts must be >= 1")
    mx, my, mz = nx + 1, ny + 1, nz + 1
    z, y, x = np.meshgrid(np.arange(mz) * h, np.arange(my) * h, np.arange(mx) * h, indexing="ij")
    pos_lin = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter * h, jitter * h, size=pos_lin.shape)
    ijk = np.stack(np.meshgrid(np.arange(mz), np.arange(my), np.arange(mx), indexing="ij"), -1)
    ijk = ijk.reshape(-1, 3)[:, ::-1]  # (i, j, k) with x fastest, matching pos_lin
    interior = np.all((ijk > 0) & (ijk < np.array([nx, ny, nz])), axis=1)
    pos_lin[interior] += d[interior]

    def vid(i, j, k):
        return i + mx * (j + my * k)

    # 6 tets per cell, orientation made positive (det > 0)
    cells = np.stack(np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij"), -1)
    cells = cells.reshape(-1, 3)[:, ::-1]  # x fastest over cells
    tets4 = []
    for perm in itertools.permutations(range(3)):
        v0 = np.zeros(3, np.int64)
        v1 = _UNIT[perm[0]]
        v2 = _UNIT[perm[0]] + _UNIT[perm[1]]
        v3 = np.ones(3, np.int64)
        det = np.linalg.det(np.stack([v1 - v0, v2 - v0, v3 - v0]).astype(float))
        verts = [v0, v1, v2, v3] if det > 0 else [v0, v2, v1, v3]
        tets4.append(verts)
    t4 = np.empty((cells.shape[0], 6, 4), np.int64)
    for t, verts in enumerate(tets4):
        for a, v in enumerate(verts):
            c = cells + v
            t4[:, t, a] = vid(c[:, 0], c[:, 1], c[:, 2])
    t4 = t4.reshape(-1, 4)
    T = t4.shape[0]
    N = mx * my * mz

    # unique edges -> midpoint nodes, numbered in first-appearance order
    e_all = np.stack([np.stack([t4[:, a], t4[:, b]], 1) for a, b in MID_EDGES], 1)  # (T,6,2)
    lo = e_all.min(-1)
    hi = e_all.max(-1)
    key = (lo * N + hi).ravel()
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    mid_id = N + rank[inv].reshape(T, 6)
    E = uniq.size
    ends = np.stack([uniq // N, uniq % N], 1)[order]
    pos_mid = 0.5 * (pos_lin[ends[:, 0]] + pos_lin[ends[:, 1]])
    pos = np.concatenate([pos_lin, pos_mid], 0)
    tets = np.concatenate([t4, mid_id], 1).astype(np.int32)

    mat = np.tile(np.array([density, shear_visc, bulk_visc, shear_mod, bulk_mod, dielectric]), (T, 1))
    if stokes_radius is None:
        stokes_radius = 0.25 * h
    sr = np.full(N + E, float(stokes_radius))
    return Mesh(pos=pos, tets=tets, material=mat, stokes_radius=sr, scale=scale, n_linear=N)


def apply_shear(mesh: Mesh, strain: float, *, seed: int | None = None) -> np.ndarray:
    """Return vertex positions after a simple shear x += strain * (z - z_mid).

    With ``seed`` the strain of each vertex is scaled by a seeded factor in
    [0.5, 1.5] so that the displacement field is not a pure affine map.
    Midpoint positions are recomputed from the sheared vertices by the
    caller's re-linearisation (FFEA resets midpoints every step).
    """
    p = mesh.pos.copy()
    zc = 0.5 * (p[:, 2].max() + p[:, 2].min())
    f = np.ones(p.shape[0])
    if seed is not None:
        f = np.random.default_rng(seed).uniform(0.5, 1.5, p.shape[0])
    p[:, 0] += strain * f * (p[:, 2] - zc)
    return relinearise(p, mesh.tets)


def relinearise(pos: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Put every midpoint node back on its edge midpoint (linearise_element)."""
    p = pos.copy()
    for s, (a, b) in enumerate(MID_EDGES):
        p[tets[:, 4 + s]] = 0.5 * (p[tets[:, a]] + p[tets[:, b]])
    return p


# ----------------------------------------------------------------------------
# FFEA structure files
# ----------------------------------------------------------------------------

def write_structure(mesh: Mesh, directory: str, name: str, pos: np.ndarray | None = None) -> dict:
    """Write ``name``.node/.top/.mat/.stokes/.pin into ``directory``.

    Values are written with 17 significant digits so that they round-trip
    exactly through the reference's ``fscanf("%le")``.
    """
    os.makedirs(directory, exist_ok=True)
    pos = mesh.pos if pos is None else pos
    paths = {k: os.path.join(directory, f"{name}.{k}") for k in ("node", "top", "mat", "stokes", "pin")}
    N = pos.shape[0]
    with open(paths["node"], "w") as f:
        f.write(f"ffea node file\nnum_nodes {N}\nnum_surface_nodes {N}\nnum_interior_nodes 0\nsurface nodes:\n")
        np.savetxt(f, pos, fmt="%.17e")
        f.write("interior nodes:\n")
    T = mesh.tets.shape[0]
    with open(paths["top"], "w") as f:
        f.write(f"ffea topology file\nnum_elements {T}\nnum_surface_elements {T}\nnum_interior_elements 0\n"
                "surface elements:\n")
        np.savetxt(f, mesh.tets, fmt="%d")
        f.write("interior elements:\n")
    with open(paths["mat"], "w") as f:
        f.write(f"ffea material params file\nnum_elements {T}\n")
        np.savetxt(f, mesh.material, fmt="%.17e")
    with open(paths["stokes"], "w") as f:
        f.write(f"ffea stokes radii file\nnum_nodes {N}\n")
        np.savetxt(f, mesh.stokes_radius, fmt="%.17e")
    with open(paths["pin"], "w") as f:
        f.write(f"ffea pinned nodes file\nnum_pinned_nodes {len(mesh.pinned)}\npinned nodes:\n")
        for p in mesh.pinned:
            f.write(f"{int(p)}\n")
    return paths


def surface_faces(mesh: Mesh) -> np.ndarray:
    """The blob's surface as FFEA surface faces: rows ``element n0 n1 n2`` (global node ids).

    Every tetrahedron face that belongs to one element only is split, as FFEA's second-order surface is,
    into its four triangles through the edge midpoints: the three corner triangles (vertex, two
    midpoints) and the central one. The corners of each boundary face are ordered so that its normal
    points out of the element, and the four triangles keep that orientation. Faces come in element
    order, then by the element's vertex they are opposite to (0..3)."""
    t = np.asarray(mesh.tets, np.int64)
    T = t.shape[0]
    mid = {frozenset(e): 4 + k for k, e in enumerate(MID_EDGES)}
    keys = {}
    for o in range(4):
        tri = np.sort(np.delete(t[:, :4], o, axis=1), axis=1)
        for e in range(T):
            k = tuple(tri[e])
            keys[k] = keys.get(k, 0) + 1
    out = []
    p = mesh.pos
    for e in range(T):
        for o in range(4):
            loc = [a for a in range(4) if a != o]
            if keys[tuple(sorted(int(t[e, a]) for a in loc))] != 1:
                continue
            a, b, c = loc
            n = np.cross(p[t[e, b]] - p[t[e, a]], p[t[e, c]] - p[t[e, a]])
            if np.dot(n, p[t[e, o]] - p[t[e, a]]) > 0:
                b, c = c, b
            mab, mbc, mca = mid[frozenset((a, b))], mid[frozenset((b, c))], mid[frozenset((c, a))]
            for tri in ((a, mab, mca), (b, mbc, mab), (c, mca, mbc), (mab, mbc, mca)):
                out.append([e] + [int(t[e, k]) for k in tri])
    return np.array(out, np.int32).reshape(-1, 4)


def faces_on_plane(mesh: Mesh, faces: np.ndarray, axis: int, value: float, tol: float = 1e-9) -> np.ndarray:
    """Indices of the surface faces whose three nodes lie on the plane x[axis] = value."""
    c = mesh.pos[faces[:, 1:], axis]
    return np.nonzero(np.all(np.abs(c - value) <= tol, axis=1))[0].astype(np.int32)


def write_surface(path: str, faces: np.ndarray) -> None:
    """An FFEA surface file (Blob::load_surface, src/Blob.cpp:2089-2170)."""
    with open(path, "w") as f:
        f.write(f"ffea surface file\nnum_surface_faces {faces.shape[0]}\nfaces:\n")
        np.savetxt(f, np.asarray(faces, np.int64), fmt="%d")


def write_ctforces(path: str, linear=(), surface=(), rotational=()) -> None:
    """An FFEA constant-forces file (Blob::load_ctforces, src/Blob.cpp:2478-2805).

    ``linear``: (F [N], (dx, dy, dz), blob, conformation, node or "all") per force;
    ``rotational``: (F [N], type "pf" or "pt", (px, py, pz) [m], (dx, dy, dz), blob, conformation, node or "all");
    ``surface``: (F [N], (dx, dy, dz), blob, conformation, [face indices]) per set of faces."""
    lines = ["ffea ctforces file", f"num_ctforces {len(linear) + len(rotational) + len(surface)}"]
    if linear:
        lines.append(f"num_linear_forces {len(linear)}")
    if rotational:
        lines.append(f"num_rot_forces {len(rotational)}")
    if surface:
        lines.append(f"num_linear_surface_forces {len(surface)}")
    if linear:
        lines.append("linear forces:")
        for F, d, b, c, n in linear:
            lines.append(f"{F!r} {d[0]!r} {d[1]!r} {d[2]!r} {b} {c} {n}")
    if rotational:
        lines.append("rotational forces:")
        for F, t, pt, d, b, c, n in rotational:
            lines.append(f"{F!r} {t} {pt[0]!r} {pt[1]!r} {pt[2]!r} {d[0]!r} {d[1]!r} {d[2]!r} {b} {c} {n}")
    if surface:
        lines.append("linear surface forces:")
        for F, d, b, c, fs in surface:
            lines.append(f"{F!r} {d[0]!r} {d[1]!r} {d[2]!r} {b} {c} " + " ".join(str(int(x)) for x in fs))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_script(path: str, structure: dict, *, solver: str = "CG_nomass", scale: float = 1e-9,
                 dt: float = 1e-12, kT: float = 4.11e-21, epsilon: float = 1e-10,
                 max_iterations_cg: int = 10000, calc_noise: int = 1, calc_stokes: int = 0,
                 stokes_visc: float = 1e-3, rng_seed: int = 12345, num_steps: int = 1000,
                 check: int | None = None, ctforces: str | None = None, surface: str | None = None) -> None:
    """Write a single-blob ``.ffea`` script with every non-hot-path force off.

    ``calc_ssint`` and ``calc_steric`` default to 1 in the reference
    (src/SimulationParams.cpp:39,44), so they are set to 0 explicitly.
    ``ctforces`` (a constant-forces file) sets ``calc_ctforces = 1`` with an ``<interactions>`` block;
    ``surface`` adds the conformation's surface file.
    """
    check = num_steps if check is None else check
    d = os.path.dirname(os.path.abspath(path))
    rel = {k: os.path.relpath(v, d) for k, v in structure.items()}
    lines = [
        "<param>",
        "\t<restart = 0>",
        f"\t<dt = {dt!r}>",
        f"\t<kT = {kT!r}>",
        f"\t<check = {check}>",
        f"\t<num_steps = {num_steps}>",
        f"\t<rng_seed = {rng_seed}>",
        f"\t<epsilon = {epsilon!r}>",
        f"\t<max_iterations_cg = {max_iterations_cg}>",
        f"\t<calc_noise = {calc_noise}>",
        f"\t<calc_stokes = {calc_stokes}>",
        f"\t<stokes_visc = {stokes_visc!r}>",
        "\t<calc_ssint = 0>", "\t<calc_steric = 0>", "\t<calc_es = 0>", "\t<calc_kinetics = 0>",
        "\t<calc_preComp = 0>", "\t<calc_springs = 0>", f"\t<calc_ctforces = {int(ctforces is not None)}>",
        "\t<num_blobs = 1>", "\t<num_conformations = (1)>", "\t<num_states = (1)>",
        "</param>", "", "<system>", "\t<blob>", "\t\t<conformation>",
        "\t\t\t<motion_state = DYNAMIC>",
        f"\t\t\t<nodes = {rel['node']}>",
        f"\t\t\t<topology = {rel['top']}>",
        f"\t\t\t<material = {rel['mat']}>",
        f"\t\t\t<stokes = {rel['stokes']}>",
        f"\t\t\t<pin = {rel['pin']}>",
    ] + ([f"\t\t\t<surface = {os.path.relpath(surface, d)}>"] if surface else []) + [
        "\t\t</conformation>",
        f"\t\t<solver = {solver}>",
        f"\t\t<scale = {scale!r}>",
        "\t</blob>",
    ] + (["\t<interactions>", "\t\t<ctforces>", f"\t\t\t<ctforces_fname = {os.path.relpath(ctforces, d)}>",
          "\t\t</ctforces>", "\t</interactions>"] if ctforces else []) + [
        "</system>", "",
    ]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def counts(n: int) -> dict:
    """Closed-form sizes of an n^3 Kuhn cube (linear-only CSR nnz included)."""
    N = (n + 1) ** 3
    E = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    return {"T": 6 * n ** 3, "N": N, "E_lin": E, "N_all": (2 * n + 1) ** 3,
            "nnz_linear": 9 * (N + 2 * E), "nnz_blocks": N + 2 * E}


def ensemble_cells(nblobs: int = 256, *, seed: int = 2024, nmin: int = 8, nmax: int = 32) -> np.ndarray:
    """Cells per side of each replica: log-uniform in [nmin, nmax], rounded, seeded."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=nblobs))).astype(int)


def ensemble(nblobs: int = 256, *, seed: int = 2024, nmin: int = 8, nmax: int = 32, cell: float = 5.0,
             g_min: float = 1e8, g_max: float = 1e9, bulk_ratio: float = 3.9) -> list[Mesh]:
    """Replica ensemble of uneven Kuhn cubes: cells per side log-uniform in [nmin, nmax] (so
    6 nmin^3 .. 6 nmax^3 tets per blob), cell size ``cell`` file units, per-blob shear modulus
    uniform in [g_min, g_max] Pa and bulk modulus ``bulk_ratio`` x shear; other material as
    :func:`kuhn_cube`. Every draw comes from ``seed``."""
    cells = ensemble_cells(nblobs, seed=seed, nmin=nmin, nmax=nmax)
    rng = np.random.default_rng(seed + 1)
    gs = rng.uniform(g_min, g_max, size=nblobs)
    out = []
    for b, (n, gmod) in enumerate(zip(cells, gs)):
        out.append(kuhn_cube(int(n), side=cell * int(n), seed=seed + 100 + b, shear_mod=float(gmod),
                             bulk_mod=bulk_ratio * float(gmod)))
    return out
