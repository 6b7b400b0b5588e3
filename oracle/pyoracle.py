"""ctypes bindings for the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.

* ``OracleBlob`` wraps the C restatement (``_build/libffea_oracle.so``, or
  ``libffea_oracle_fast.so`` built with the reference's release optimisation).
* ``RefBlob`` wraps the reference's own hot-path classes
  (``_ref/libffea_ref.so``, built only where the reference sources exist).
Both expose the same methods so that tests can run one against the other.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libffea_oracle.so")
FAST_LIB = os.path.join(HERE, "_build", "libffea_oracle_fast.so")
REF_LIB = os.path.join(HERE, "_ref", "libffea_ref.so")

SOLVERS = {"CG_nomass": 0, "CG": 1, "masslumped": 2}
_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


def build(fast: bool = True, ref: bool = False) -> None:
    """Compile the oracle with its Makefile (the reference build only if asked)."""
    targets = ["port"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("kT", C.c_double), ("epsilon", C.c_double), ("stokes_visc", C.c_double),
                ("max_iterations_cg", C.c_int), ("calc_noise", C.c_int), ("calc_stokes", C.c_int)]


_libs: dict = {}


def _load(path: str):
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} not built (run `make -C {HERE} port` / `ref`)")
    lib = C.CDLL(path)
    _libs[path] = lib
    return lib


def port_lib(fast: bool = False):
    lib = _load(FAST_LIB if fast else PORT_LIB)
    if getattr(lib, "_typed", False):
        return lib
    P = "orc_"
    lib.orc_blob_create.restype = C.c_void_p
    lib.orc_blob_create.argtypes = [C.c_int, _dp, C.c_double, C.c_int, _ip, _dp, _dp, C.c_int, _ip,
                                    C.POINTER(Params), C.c_int, C.c_int, C.POINTER(C.c_int)]
    lib.orc_blob_destroy.argtypes = [C.c_void_p]
    for name, args in {
        "blob_step": [C.c_void_p, C.c_int],
        "blob_update_internal_forces": [C.c_void_p],
        "blob_update_positions": [C.c_void_p],
        "blob_zero_forces": [C.c_void_p],
        "blob_get_pos": [C.c_void_p, _dp], "blob_set_pos": [C.c_void_p, _dp],
        "blob_get_vel": [C.c_void_p, _dp], "blob_get_force": [C.c_void_p, _dp],
        "blob_get_rhs": [C.c_void_p, _dp],
        "blob_get_elem": [C.c_void_p] + [C.c_void_p] * 6,
        "blob_get_rest": [C.c_void_p, C.c_void_p, C.c_void_p],
        "blob_nnz": [C.c_void_p],
        "blob_get_csr": [C.c_void_p] + [C.c_void_p] * 4,
        "blob_n_contrib": [C.c_void_p],
        "blob_get_contrib": [C.c_void_p, _ip, _ip],
        "blob_mass_nnz": [C.c_void_p],
        "blob_get_mass_csr": [C.c_void_p, _ip, _ip, _dp],
        "blob_get_inv_mass": [C.c_void_p, _dp],
        "blob_last_cg_iters": [C.c_void_p],
        "blob_get_rng_state": [C.c_void_p, C.c_int, _up],
        "blob_set_rng_state": [C.c_void_p, C.c_int, _up],
        "blob_measure": [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)],
        "blob_set_ctforces": [C.c_void_p, C.c_int, _ip, _dp, C.c_int, _ip, _ip, _dp, C.c_int, _ip],
        "blob_set_rot_ctforces": [C.c_void_p, C.c_int, _ip, _ip, _dp],
    }.items():
        getattr(lib, P + name).argtypes = args
    lib.orc_blob_total_cg_iters.argtypes = [C.c_void_p]
    lib.orc_blob_total_cg_iters.restype = C.c_longlong
    lib.orc_blob_param.argtypes = [C.c_void_p, C.c_char_p]
    lib.orc_blob_param.restype = C.c_double
    lib.orc_rng_rand_u01.restype = C.c_double
    lib.orc_rng_rand_u01.argtypes = [C.c_void_p]
    lib.orc_rng_rand_int.argtypes = [C.c_void_p, C.c_int, C.c_int]
    for name in ("reset_start_stream", "reset_start_substream", "reset_next_substream", "create"):
        getattr(lib, "orc_rng_" + name).argtypes = [C.c_void_p]
    lib.orc_rng_advance_state.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    lib.orc_rng_set_antithetic.argtypes = [C.c_void_p, C.c_int]
    lib.orc_rng_increased_precis.argtypes = [C.c_void_p, C.c_int]
    lib.orc_rng_get_state.argtypes = [C.c_void_p, _up]
    lib.orc_rng_set_state.argtypes = [C.c_void_p, _up]
    lib.orc_rng_set_package_seed.argtypes = [_up]
    lib.orc_seed_from_rng_seed.argtypes = [C.c_int, _up]
    lib._typed = True
    return lib


def ref_lib():
    lib = _load(REF_LIB)
    if getattr(lib, "_typed", False):
        return lib
    lib.ref_rng_new.restype = C.c_void_p
    lib.ref_rng_free.argtypes = [C.c_void_p]
    lib.ref_rng_rand_u01.restype = C.c_double
    lib.ref_rng_rand_u01.argtypes = [C.c_void_p]
    lib.ref_rng_rand_int.argtypes = [C.c_void_p, C.c_int, C.c_int]
    for name in ("reset_start_stream", "reset_start_substream", "reset_next_substream"):
        getattr(lib, "ref_rng_" + name).argtypes = [C.c_void_p]
    lib.ref_rng_advance_state.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    lib.ref_rng_set_antithetic.argtypes = [C.c_void_p, C.c_int]
    lib.ref_rng_increased_precis.argtypes = [C.c_void_p, C.c_int]
    lib.ref_rng_get_state.argtypes = [C.c_void_p, _up]
    lib.ref_rng_set_package_seed.argtypes = [_up]
    lib.ref_blob_load.restype = C.c_void_p
    lib.ref_blob_load.argtypes = [C.c_char_p] * 7 + [C.c_double] * 5 + [C.c_int] * 5 + [C.POINTER(C.c_int)]
    lib.ref_blob_destroy.argtypes = [C.c_void_p]
    for name, args in {
        "blob_step": [C.c_void_p, C.c_int],
        "blob_get_pos": [C.c_void_p, _dp], "blob_set_pos": [C.c_void_p, _dp],
        "blob_get_vel": [C.c_void_p, _dp], "blob_get_rhs": [C.c_void_p, _dp],
        "blob_get_elem": [C.c_void_p] + [C.c_void_p] * 6,
        "blob_get_rest": [C.c_void_p, C.c_void_p, C.c_void_p],
        "blob_nnz": [C.c_void_p],
        "blob_get_csr": [C.c_void_p] + [C.c_void_p] * 4,
        "blob_n_contrib": [C.c_void_p],
        "blob_get_contrib": [C.c_void_p, _ip, _ip],
        "blob_mass_nnz": [C.c_void_p],
        "blob_get_mass_csr": [C.c_void_p, _ip, _ip, _dp],
        "blob_get_inv_mass": [C.c_void_p, _dp],
        "blob_get_rng_state": [C.c_void_p, C.c_int, _up],
        "blob_measure": [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    }.items():
        getattr(lib, "ref_" + name).argtypes = args
    lib._typed = True
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class _BlobBase:
    """Common accessors; subclasses set self._lib, self._p (prefix) and self._h."""

    n_nodes: int
    n_elem: int

    def _f(self, name):
        return getattr(self._lib, self._p + name)

    def step(self, nsteps: int = 1) -> int:
        return self._f("blob_step")(self._h, nsteps)

    def pos(self) -> np.ndarray:
        o = np.empty((self.n_nodes, 3))
        self._f("blob_get_pos")(self._h, o)
        return o

    def set_pos(self, p) -> None:
        self._f("blob_set_pos")(self._h, np.ascontiguousarray(p, np.float64))

    def vel(self) -> np.ndarray:
        o = np.empty((self.n_nodes, 3))
        self._f("blob_get_vel")(self._h, o)
        return o

    def rhs(self) -> np.ndarray:
        o = np.empty((self.n_nodes, 3))
        self._f("blob_get_rhs")(self._h, o)
        return o

    def elem(self) -> dict:
        T = self.n_elem
        d = {"node_force": np.empty((T, 4, 3)), "dpsi": np.empty((T, 12)), "vol": np.empty(T),
             "vol0": np.empty(T), "visc": np.empty((T, 12, 12)), "stress_mag": np.empty(T)}
        self._f("blob_get_elem")(self._h, *(_ptr(d[k]) for k in ("node_force", "dpsi", "vol", "vol0", "visc",
                                                                  "stress_mag")))
        return d

    def rest(self) -> dict:
        T = self.n_elem
        d = {"jinv0": np.empty((T, 3, 3)), "mat": np.empty((T, 5))}
        self._f("blob_get_rest")(self._h, _ptr(d["jinv0"]), _ptr(d["mat"]))
        return d

    def csr(self) -> dict:
        nnz = self._f("blob_nnz")(self._h)
        d = {"key": np.empty(3 * self.n_nodes + 1, np.int32), "col": np.empty(nnz, np.int32),
             "val": np.empty(nnz), "nsrc": np.empty(nnz, np.int32)}
        self._f("blob_get_csr")(self._h, *(_ptr(d[k]) for k in ("key", "col", "val", "nsrc")))
        return d

    def contrib(self) -> dict:
        m = self._f("blob_n_contrib")(self._h)
        d = {"ptr": np.empty(self.n_nodes + 1, np.int32), "elem_slot": np.empty(m, np.int32)}
        self._f("blob_get_contrib")(self._h, d["ptr"], d["elem_slot"])
        return d

    def mass_csr(self) -> dict:
        nnz = self._f("blob_mass_nnz")(self._h)
        d = {"key": np.empty(self.n_nodes + 1, np.int32), "col": np.empty(nnz, np.int32), "val": np.empty(nnz)}
        self._f("blob_get_mass_csr")(self._h, d["key"], d["col"], d["val"])
        return d

    def inv_mass(self) -> np.ndarray:
        o = np.empty(self.n_nodes)
        self._f("blob_get_inv_mass")(self._h, o)
        return o

    def rng_state(self, t: int = 0) -> np.ndarray:
        o = np.empty(6, np.uint32)
        self._f("blob_get_rng_state")(self._h, t, o)
        return o

    def measure(self) -> tuple[float, float]:
        s, k = C.c_double(), C.c_double()
        self._f("blob_measure")(self._h, C.byref(s), C.byref(k))
        return s.value, k.value

    def set_ctforces(self, ctf: dict, faces: np.ndarray | None = None) -> None:
        """Constant forces from :func:`read_ctforces`; ``faces`` (F, 4) rows ``element n0 n1 n2`` of the
        blob's surface file (:func:`read_surface`)."""
        faces = np.zeros((0, 4), np.int32) if faces is None else np.asarray(faces, np.int32)
        arg = faces[:, 1:] if self._p == "orc_" else faces
        i32 = lambda a: np.ascontiguousarray(a, np.int32) if len(a) else np.zeros(1, np.int32)
        f64 = lambda a: np.ascontiguousarray(a, np.float64).ravel() if len(a) else np.zeros(4)
        st = self._f("blob_set_ctforces")(
            self._h, len(ctf["lin_node"]), i32(ctf["lin_node"]), f64(ctf["lin_fd"]), len(ctf["set_size"]),
            i32(ctf["set_size"]), i32(ctf["set_faces"]), f64(ctf["set_fd"]), faces.shape[0],
            i32(np.ascontiguousarray(arg).ravel()))
        if st != 0:
            raise ValueError(f"set_ctforces failed (status {st})")
        n_rot = len(ctf.get("rot_node", []))
        st = self._f("blob_set_rot_ctforces")(self._h, n_rot, i32(ctf.get("rot_node", [])),
                                               i32(ctf.get("rot_torque", [])),
                                               np.ascontiguousarray(ctf["rot_fpd"], np.float64).ravel()
                                               if n_rot else np.zeros(7))
        if st != 0:
            raise ValueError(f"set_rot_ctforces failed (status {st})")


def read_ctforces(path: str, blob_index: int, n_nodes: int) -> dict:
    """The entries of one blob (conformation 0) of a constant-forces file, as Blob::load_ctforces
    (src/Blob.cpp:2478-2805) selects them: linear forces in file order with "all" expanded over the
    nodes, rotational forces (type, then (F [N], axis point [m], axis direction)) the same way, and the
    linear surface-force sets. Forces stay as read: (F [N], dx, dy, dz)."""
    lines = []
    for ln in open(path).read().split("\n"):
        ln = ln.strip()
        if ln:
            lines.append(ln)
    head = {}
    at = 1
    while at < len(lines) and ":" not in lines[at]:
        w = lines[at].split()
        head[w[0]] = int(w[1])
        at += 1
    nl, nr, ns = (head.get(k, 0) for k in ("num_linear_forces", "num_rot_forces", "num_linear_surface_forces"))
    out = {"lin_node": [], "lin_fd": [], "set_size": [], "set_faces": [], "set_fd": []}
    if lines[at].startswith("linear forces:"):
        at += 1
    for ln in lines[at:at + nl]:
        w = ln.split()
        if int(w[4]) != blob_index or int(w[5]) != 0:
            continue
        fd = [float(x) for x in w[:4]]
        nodes = range(n_nodes) if w[6] == "all" else [int(w[6])]
        for n in nodes:
            out["lin_node"].append(n)
            out["lin_fd"].append(fd)
    at += nl
    rot = {"rot_node": [], "rot_torque": [], "rot_fpd": []}
    if nr:
        at += 1
        for ln in lines[at:at + nr]:
            w = ln.split()
            if int(w[8]) != blob_index or int(w[9]) != 0:
                continue
            if w[1][0] != "p" or w[1][1] not in "ft":
                raise ValueError("only rotational forces about an axis through a point are applied")
            fpd = [float(w[0])] + [float(x) for x in w[2:8]]
            nodes = range(n_nodes) if w[10] == "all" else [int(w[10])]
            for n in nodes:
                rot["rot_node"].append(n)
                rot["rot_torque"].append(1 if w[1][1] == "t" else 0)
                rot["rot_fpd"].append(fpd)
        at += nr
    if ns:
        at += 1
        for ln in lines[at:at + ns]:
            w = ln.split()
            if int(w[4]) != blob_index or int(w[5]) != 0:
                continue
            out["set_fd"].append([float(x) for x in w[:4]])
            out["set_size"].append(len(w) - 6)
            out["set_faces"].extend(int(x) for x in w[6:])
    return {"lin_node": np.array(out["lin_node"], np.int32), "lin_fd": np.array(out["lin_fd"], np.float64),
            "set_size": np.array(out["set_size"], np.int32), "set_faces": np.array(out["set_faces"], np.int32),
            "set_fd": np.array(out["set_fd"], np.float64),
            "rot_node": np.array(rot["rot_node"], np.int32), "rot_torque": np.array(rot["rot_torque"], np.int32),
            "rot_fpd": np.array(rot["rot_fpd"], np.float64).reshape(-1, 7)}


def read_surface(path: str) -> np.ndarray:
    """Faces of an FFEA surface file (Blob::load_surface, src/Blob.cpp:2089-2170): rows element n0 n1 n2."""
    with open(path) as f:
        lines = f.read().split("\n")
    nf = int(lines[1].split()[1])
    return np.array([[int(x) for x in ln.split()] for ln in lines[3:3 + nf]], np.int32).reshape(nf, 4)


def _mesh_args(mesh):
    return (mesh.n_nodes, np.ascontiguousarray(mesh.pos, np.float64).ravel(), float(mesh.scale), mesh.n_elem,
            np.ascontiguousarray(mesh.tets, np.int32).ravel(), np.ascontiguousarray(mesh.material, np.float64).ravel(),
            np.ascontiguousarray(mesh.stokes_radius, np.float64), len(mesh.pinned),
            np.ascontiguousarray(mesh.pinned, np.int32) if len(mesh.pinned) else np.zeros(1, np.int32))


class OracleBlob(_BlobBase):
    """The C restatement of the reference blob (``orc_blob``)."""

    def __init__(self, mesh, *, solver="CG_nomass", dt=1e-12, kT=4.11e-21, epsilon=1e-10, stokes_visc=1e-3,
                 max_iterations_cg=10000, calc_noise=1, calc_stokes=0, threads=1, fast=False,
                 package_seed=(12345,) * 6):
        self._lib = port_lib(fast)
        self._p = "orc_"
        self._lib.orc_rng_set_package_seed(np.asarray(package_seed, np.uint32))
        p = Params(dt, kT, epsilon, stokes_visc, max_iterations_cg, calc_noise, calc_stokes)
        st = C.c_int()
        self._h = self._lib.orc_blob_create(*_mesh_args(mesh), C.byref(p), SOLVERS[solver], threads, C.byref(st))
        if not self._h:
            raise ValueError(f"orc_blob_create failed (status {st.value})")
        self.n_nodes, self.n_elem = mesh.n_nodes, mesh.n_elem

    def update_internal_forces(self) -> int:
        return self._lib.orc_blob_update_internal_forces(self._h)

    def update_positions(self) -> int:
        return self._lib.orc_blob_update_positions(self._h)

    def zero_forces(self) -> None:
        self._lib.orc_blob_zero_forces(self._h)

    def last_cg_iters(self) -> int:
        return self._lib.orc_blob_last_cg_iters(self._h)

    def total_cg_iters(self) -> int:
        return self._lib.orc_blob_total_cg_iters(self._h)

    def set_rng_state(self, s, t: int = 0) -> None:
        self._lib.orc_blob_set_rng_state(self._h, t, np.asarray(s, np.uint32))

    def param(self, name: str) -> float:
        return self._lib.orc_blob_param(self._h, name.encode())

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_blob_destroy(self._h)
            self._h = None


class RefBlob(_BlobBase):
    """The reference's own Blob (Blob::config + Blob::init from structure files, World::run's step) behind the
    same methods (build container only). The mesh is written to the reference's structure files first (17
    significant digits, which the reference's readers parse back exactly); ``ctforces`` is a pair (constant-force
    file, surface file) of the reference's formats, loaded by the reference's own Blob::load_ctforces."""

    def __init__(self, mesh, *, solver="CG_nomass", dt=1e-12, kT=4.11e-21, epsilon=1e-10, stokes_visc=1e-3,
                 max_iterations_cg=10000, calc_noise=1, calc_stokes=0, threads=1, package_seed=(12345,) * 6,
                 ctforces=None):
        import tempfile

        from ffea_ci_demo_gb300.mesh import surface_faces, write_structure, write_surface

        self._lib = ref_lib()
        self._p = "ref_"
        if self._lib.ref_rng_set_package_seed(np.asarray(package_seed, np.uint32)) != 0:
            raise ValueError("invalid package seed")
        with tempfile.TemporaryDirectory() as d:
            paths = write_structure(mesh, d, "blob")
            surf = ctforces[1] if ctforces else os.path.join(d, "blob.surf")
            if not ctforces:
                write_surface(surf, surface_faces(mesh))
            enc = lambda x: None if x is None else str(x).encode()  # noqa: E731
            st = C.c_int()
            self._h = self._lib.ref_blob_load(enc(paths["node"]), enc(paths["top"]), enc(surf), enc(paths["mat"]),
                                              enc(paths["stokes"]), enc(paths["pin"]),
                                              enc(ctforces[0]) if ctforces else None, mesh.scale, dt, kT, epsilon,
                                              stokes_visc, max_iterations_cg, calc_noise, calc_stokes,
                                              SOLVERS[solver], threads, C.byref(st))
        if not self._h:
            raise ValueError(f"ref_blob_load failed (status {st.value})")
        self.n_nodes, self.n_elem = mesh.n_nodes, mesh.n_elem

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ref_blob_destroy(self._h)
            self._h = None


class OracleRng:
    """An ``orc_rng`` stream (RngStream restated); created from the package seed."""

    def __init__(self, lib=None):
        self._lib = lib or port_lib()
        self._buf = C.create_string_buffer(128)
        self._lib.orc_rng_create(self._buf)

    @staticmethod
    def set_package_seed(seed, lib=None):
        (lib or port_lib()).orc_rng_set_package_seed(np.asarray(seed, np.uint32))

    def rand_u01(self):
        return self._lib.orc_rng_rand_u01(self._buf)

    def rand_int(self, lo, hi):
        return self._lib.orc_rng_rand_int(self._buf, lo, hi)

    def reset_start_stream(self):
        self._lib.orc_rng_reset_start_stream(self._buf)

    def reset_start_substream(self):
        self._lib.orc_rng_reset_start_substream(self._buf)

    def reset_next_substream(self):
        self._lib.orc_rng_reset_next_substream(self._buf)

    def advance_state(self, e, c):
        self._lib.orc_rng_advance_state(self._buf, e, c)

    def set_antithetic(self, a):
        self._lib.orc_rng_set_antithetic(self._buf, int(a))

    def increased_precis(self, p):
        self._lib.orc_rng_increased_precis(self._buf, int(p))

    def get_state(self):
        o = np.empty(6, np.uint32)
        self._lib.orc_rng_get_state(self._buf, o)
        return o

    def set_state(self, s):
        self._lib.orc_rng_set_state(self._buf, np.asarray(s, np.uint32))


class RefRng:
    """The reference's RngStream behind the same methods (build container only)."""

    def __init__(self):
        self._lib = ref_lib()
        self._h = self._lib.ref_rng_new()

    @staticmethod
    def set_package_seed(seed):
        ref_lib().ref_rng_set_package_seed(np.asarray(seed, np.uint32))

    def rand_u01(self):
        return self._lib.ref_rng_rand_u01(self._h)

    def rand_int(self, lo, hi):
        return self._lib.ref_rng_rand_int(self._h, lo, hi)

    def reset_start_stream(self):
        self._lib.ref_rng_reset_start_stream(self._h)

    def reset_start_substream(self):
        self._lib.ref_rng_reset_start_substream(self._h)

    def reset_next_substream(self):
        self._lib.ref_rng_reset_next_substream(self._h)

    def advance_state(self, e, c):
        self._lib.ref_rng_advance_state(self._h, e, c)

    def set_antithetic(self, a):
        self._lib.ref_rng_set_antithetic(self._h, int(a))

    def increased_precis(self, p):
        self._lib.ref_rng_increased_precis(self._h, int(p))

    def get_state(self):
        o = np.empty(6, np.uint32)
        self._lib.ref_rng_get_state(self._h, o)
        return o

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ref_rng_free(self._h)
            self._h = None


def rngstream_known_answer(make, set_package_seed) -> float:
    """The call sequence of the reference's RngStream unit test.

    tests/consistency/rngstream/testRngStream.cpp:38-124 drives three streams
    through jumps, substreams, antithetic and increased-precision modes and
    sums the draws; the reference expects the sum to print as 39.697547445251
    at 14 significant digits (:129). ``make`` creates a stream from the
    package seed, ``set_package_seed`` sets it.
    """
    g1, g2, g3 = make(), make(), make()
    s = g2.rand_u01() + g3.rand_u01()
    g1.advance_state(5, 3)
    s += g1.rand_u01()
    g1.reset_start_stream()
    for _ in range(35):
        g1.advance_state(0, 1)
    s += g1.rand_u01()
    g1.reset_start_stream()
    sumi = 0
    for _ in range(35):
        sumi += g1.rand_int(1, 10)
    s += sumi / 100.0
    s3 = 0.0
    for _ in range(100):
        s3 += g3.rand_u01()
    s += s3 / 10.0
    g3.reset_start_stream()
    for _ in range(5):
        s += g3.rand_u01()
    for _ in range(4):
        g3.reset_next_substream()
    for _ in range(5):
        s += g3.rand_u01()
    g3.reset_start_substream()
    for _ in range(5):
        s += g3.rand_u01()
    g2.reset_next_substream()
    s3 = 0.0
    for _ in range(100000):
        s3 += g2.rand_u01()
    s += s3 / 10000.0
    g3.set_antithetic(True)
    s3 = 0.0
    for _ in range(100000):
        s3 += g3.rand_u01()
    s += s3 / 10000.0
    set_package_seed([1, 1, 1, 1, 1, 1])
    gar = [make() for _ in range(4)]
    for g in gar:
        s += g.rand_u01()
    gar[2].advance_state(-127, 0)
    s += gar[2].rand_u01()
    gar[2].reset_next_substream()
    gar[2].increased_precis(True)
    s3 = 0.0
    for _ in range(100000):
        s3 += gar[2].rand_u01()
    s += s3 / 10000.0
    gar[2].set_antithetic(True)
    s3 = 0.0
    for _ in range(100000):
        s3 += gar[2].rand_u01()
    s += s3 / 10000.0
    gar[2].set_antithetic(False)
    gar[2].increased_precis(False)
    for g in gar:
        s += g.rand_u01()
    return s
