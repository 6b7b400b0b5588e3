"""Convert the reference's sphere physics-test mesh into a fixture.

Run where the reference sources are (default /root/reference):

    python tests/golden/gen_sphere.py

The reference's equipartition tests (tests/physics/sphere_63_120_mass and sphere_63_120_nomass) run on
tests/physics/sphere_63_120_structure: 120 tetrahedra, 63 vertex nodes, 305 nodes with the edge midpoints.
This reads its .node, .top, .mat, .stokes and .pin files with the reference loaders' formats
(Blob::load_nodes, load_topology, load_material_params, load_stokes_params, load_pinned_nodes,
src/Blob.cpp:1911-2353, 3024-3076) and stores the arrays in sphere_63_120.npz, so that the tests can
rebuild the same structure files where the reference is absent.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("FFEA_REFERENCE", "/root/reference")
SRC = os.path.join(REF, "tests", "physics", "sphere_63_120_structure")


def lines(name):
    with open(os.path.join(SRC, name)) as f:
        return [ln.strip() for ln in f if ln.strip()]


def read_sections(name, cols, dtype):
    """Rows of a file with a count line, two section counts and two labelled sections (nodes or elements)."""
    L = lines(name)
    n = int(L[1].split()[1])
    rows = [ln for ln in L[4:] if ":" not in ln]
    arr = np.array([[dtype(x) for x in r.split()[:cols]] for r in rows])
    assert arr.shape[0] == n, (name, arr.shape, n)
    return arr


def main():
    if not os.path.isdir(SRC):
        raise SystemExit(f"{SRC} not found")
    pos = read_sections("sphere_63_120.node", 3, float).astype(np.float64)
    tets = read_sections("sphere_63_120.top", 10, int).astype(np.int64)
    mat = np.array([[float(x) for x in ln.split()] for ln in lines("sphere_63_120.mat")[2:]])
    stokes = np.array([float(x) for x in lines("sphere_63_120.stokes")[2:]])
    pin_lines = lines("sphere_63_120.pin")
    pinned = np.array([int(x) for x in pin_lines[3:]], np.int64)
    assert mat.shape == (tets.shape[0], 6) and stokes.shape == (pos.shape[0],)
    np.savez_compressed(os.path.join(HERE, "sphere_63_120.npz"), pos=pos, tets=tets.astype(np.int32), material=mat,
                        stokes_radius=stokes, pinned=pinned.astype(np.int32), scale=5e-9,
                        n_linear=len(np.unique(tets[:, :4])))
    print("sphere_63_120:", pos.shape, tets.shape, "vertices", len(np.unique(tets[:, :4])))


if __name__ == "__main__":
    sys.exit(main())
