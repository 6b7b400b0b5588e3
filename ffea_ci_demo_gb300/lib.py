"""ctypes binding of the C ABI (include/ffea_gpu.h) and a Python ``Blob``.

``Blob`` mirrors the reference's ``Blob`` step surface for the hot path
(include/Blob.h:94-718): construct from a mesh or from the reference's
structure files, then ``update(nsteps)`` runs the per-blob slice of
``World::run`` (zero forces, ``update_internal_forces``, ``update_positions``).
Errors surface as exceptions, as the reference's ``FFEAException`` does.

The CUDA library must be built (``ffea_ci_demo_gb300.build.build()``); there
is no CPU fallback: loading fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from .mesh import Mesh

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "libffea_gpu.so")
HEADER = os.path.join(ROOT, "include", "ffea_gpu.h")

OK, EINVERTED, ECGMAXIT, EINPUT, ENOMEM, ECUDA, ENAN, ETIMEOUT, EFILE = range(9)
SOLVERS = {"CG_nomass": 0, "CG": 1, "masslumped": 2}
PRECISIONS = {"fp64": 0, "mixed": 1}
MESO_LENGTH = 1.7e-10
CG_POLY_DEFAULT = 6  # FFEA_GPU_CG_POLY_DEFAULT: the mixed CG_nomass solve's default Chebyshev degree
CG_POLY_MAX = 8  # FFEA_GPU_CG_POLY_MAX: the highest degree cg_poly accepts (even degrees only)


class FFEAError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        names = {1: "element inverted", 2: "CG did not converge", 3: "invalid input", 4: "out of memory",
                 5: "CUDA error", 6: "non-finite solver output", 7: "device wait timed out", 8: "file error"}
        super().__init__(f"{where}: {names.get(code, code)}" + (f" ({detail})" if detail else ""))


class Params(C.Structure):
    """ffea_gpu_params: the hot-path fields of SimulationParams (meso units)."""

    _fields_ = [("dt", C.c_double), ("kT", C.c_double), ("epsilon2", C.c_double), ("stokes_visc", C.c_double),
                ("max_iterations_cg", C.c_int), ("calc_noise", C.c_int), ("calc_stokes", C.c_int),
                ("solver", C.c_int), ("precision", C.c_int), ("cg_poly", C.c_int),
                ("cg_smem_blocks", C.c_int)]


class MeshStruct(C.Structure):
    _fields_ = [("num_nodes", C.c_int), ("num_elements", C.c_int), ("num_pinned", C.c_int),
                ("pos", C.c_void_p), ("tets", C.c_void_p), ("rho", C.c_void_p), ("A", C.c_void_p),
                ("B", C.c_void_p), ("G", C.c_void_p), ("E", C.c_void_p), ("stokes_radius", C.c_void_p),
                ("pinned", C.c_void_p)]


_lib = None


def header_functions() -> list[str]:
    """Names of every function the C header declares."""
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w]+\s+)+\*?\s*(ffea_gpu_\w+)\s*\(", src, re.M)))


def load():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with ffea_ci_demo_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.c_void_p
    sig = {
        "ffea_gpu_params_default": (C.c_int, [C.POINTER(Params)]),
        "ffea_gpu_params_assign": (C.c_int, [C.POINTER(Params), C.c_char_p, C.c_char_p]),
        "ffea_gpu_material_from_si": (C.c_int, [C.c_int, dp, dp, dp, dp, dp, dp]),
        "ffea_gpu_blob_create": (C.c_int, [C.POINTER(MeshStruct), C.POINTER(Params), C.POINTER(vp)]),
        "ffea_gpu_blob_load": (C.c_int, [C.c_char_p] * 5 + [C.c_double, C.POINTER(Params), C.POINTER(vp)]),
        "ffea_gpu_blob_destroy": (None, [vp]),
        "ffea_gpu_blob_set_rng_state": (C.c_int, [vp, dp]),
        "ffea_gpu_blob_get_rng_state": (C.c_int, [vp, dp]),
        "ffea_gpu_blob_step": (C.c_int, [vp, C.c_int, ip]),
        "ffea_gpu_blob_step_timed": (C.c_int, [vp, C.c_int, C.c_longlong, ip, C.POINTER(C.c_double), dp]),
        "ffea_gpu_blob_get_state": (C.c_int, [vp, dp, dp, dp]),
        "ffea_gpu_blob_set_state": (C.c_int, [vp, dp, dp]),
        "ffea_gpu_blob_measure": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "ffea_gpu_blob_cg_iterations": (C.c_int, [vp, ip, C.POINTER(C.c_longlong)]),
        "ffea_gpu_blob_measurements": (C.c_int, [vp, dp]),
        "ffea_gpu_blob_load_ctforces": (C.c_int, [vp, C.c_char_p, C.c_char_p, C.c_int]),
        "ffea_gpu_blob_set_rmsd_reference": (C.c_int, [vp]),
        "ffea_gpu_blob_sizes": (C.c_int, [vp, ip, ip, C.POINTER(C.c_longlong)]),
        "ffea_gpu_blob_counts": (C.c_int, [vp, ip, ip]),
        "ffea_gpu_blob_cg_history": (C.c_int, [vp, dp, C.c_int, ip]),
        "ffea_gpu_blob_cg_profile": (C.c_int, [vp, dp, C.c_int]),
        "ffea_gpu_blob_cg_preconditioner": (C.c_int, [vp, ip, dp]),
        "ffea_gpu_blob_cg_kernel": (C.c_char_p, [vp]),
        "ffea_gpu_blob_get_pattern": (C.c_int, [vp, dp, dp, dp, dp, C.POINTER(C.c_longlong)]),
        "ffea_gpu_blob_get_connectivity": (C.c_int, [vp, dp, dp, C.POINTER(C.c_longlong)]),
        "ffea_gpu_blob_get_elements": (C.c_int, [vp, dp, dp, dp]),
        "ffea_gpu_blob_get_rhs": (C.c_int, [vp, dp]),
        "ffea_gpu_blob_solve_static": (C.c_int, [vp, dp, dp, ip]),
        "ffea_gpu_adjoint_create": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(vp)]),
        "ffea_gpu_adjoint_forward": (C.c_int, [vp, ip]),
        "ffea_gpu_adjoint_backward": (C.c_int, [vp, dp, dp, dp, dp, dp, dp]),
        "ffea_gpu_adjoint_destroy": (None, [vp]),
        "ffea_gpu_world_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(vp)]),
        "ffea_gpu_world_run": (C.c_int, [vp, C.POINTER(C.c_longlong)]),
        "ffea_gpu_world_num_blobs": (C.c_int, [vp]),
        "ffea_gpu_world_blob": (vp, [vp, C.c_int]),
        "ffea_gpu_world_destroy": (None, [vp]),
        "ffea_gpu_batch_create": (C.c_int, [vp, C.c_int, C.POINTER(Params), C.POINTER(vp)]),
        "ffea_gpu_batch_destroy": (None, [vp]),
        "ffea_gpu_batch_sizes": (C.c_int, [vp, ip, ip, ip, C.POINTER(C.c_longlong)]),
        "ffea_gpu_batch_blob_sizes": (C.c_int, [vp, C.c_int, ip, ip, ip]),
        "ffea_gpu_batch_step": (C.c_int, [vp, C.c_int, ip]),
        "ffea_gpu_batch_step_timed": (C.c_int, [vp, C.c_int, C.c_longlong, ip, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]),
        "ffea_gpu_batch_get_state": (C.c_int, [vp, C.c_int, dp, dp]),
        "ffea_gpu_batch_get_states": (C.c_int, [vp, dp, dp]),
        "ffea_gpu_batch_set_states": (C.c_int, [vp, dp, dp]),
        "ffea_gpu_batch_set_state": (C.c_int, [vp, C.c_int, dp, dp]),
        "ffea_gpu_batch_set_rng_state": (C.c_int, [vp, C.c_int, dp]),
        "ffea_gpu_batch_load_ctforces": (C.c_int, [vp, C.c_int, C.c_char_p, C.c_char_p, C.c_int]),
        "ffea_gpu_batch_strain_energies": (C.c_int, [vp, dp]),
        "ffea_gpu_batch_get_rng_state": (C.c_int, [vp, C.c_int, dp]),
        "ffea_gpu_batch_cg_iterations": (C.c_int, [vp, dp, C.POINTER(C.c_longlong)]),
        "ffea_gpu_batch_config": (C.c_int, [vp, ip, ip, ip]),
        "ffea_gpu_batch_set_config": (C.c_int, [vp, C.c_int, C.c_int]),
        "ffea_gpu_batch_shapes": (C.c_int, [vp, ip, ip, ip, ip]),
        "ffea_gpu_batch_set_shapes": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "ffea_gpu_batch_tune": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
        "ffea_gpu_last_error": (C.c_char_p, []),
        "ffea_gpu_launch_count": (C.c_longlong, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def last_error() -> str:
    return load().ffea_gpu_last_error().decode()


def _out(out, shape):
    if out is None:
        return np.empty(shape)
    if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != int(np.prod(shape)):
        raise ValueError(f"out must be a C-contiguous float64 array of {int(np.prod(shape))} values")
    return out


def _check(rc: int, where: str) -> None:
    if rc != OK:
        raise FFEAError(rc, where, last_error())


def make_params(*, solver: str = "CG_nomass", precision: str = "fp64", **si) -> Params:
    """SimulationParams defaults, then ``assign`` for each SI key (dt, kT, epsilon, ...)."""
    lib = load()
    p = Params()
    _check(lib.ffea_gpu_params_default(C.byref(p)), "params_default")
    for k, v in si.items():
        _check(lib.ffea_gpu_params_assign(C.byref(p), k.encode(), repr(v).encode() if isinstance(v, float)
                                          else str(v).encode()), f"params_assign({k})")
    _check(lib.ffea_gpu_params_assign(C.byref(p), b"solver", solver.encode()), "params_assign(solver)")
    _check(lib.ffea_gpu_params_assign(C.byref(p), b"precision", precision.encode()), "params_assign(precision)")
    return p


def material_from_si(mat6: np.ndarray) -> dict:
    lib = load()
    mat6 = np.ascontiguousarray(mat6, np.float64)
    n = mat6.shape[0]
    out = {k: np.empty(n) for k in ("rho", "A", "B", "G", "E")}
    _check(lib.ffea_gpu_material_from_si(n, _p(mat6), *(_p(out[k]) for k in ("rho", "A", "B", "G", "E"))),
           "material_from_si")
    return out


class Blob:
    """One FFEA blob on the GPU (vertex nodes resident in HBM)."""

    def __init__(self, mesh: Mesh | None = None, *, solver: str = "CG_nomass", precision: str = "fp64",
                 dt: float = 1e-12, kT: float = 4.11e-21, epsilon: float = 1e-10, max_iterations_cg: int = 10000,
                 calc_noise: int = 1, calc_stokes: int = 0, stokes_visc: float = 1e-3, cg_poly: int = 0,
                 cg_smem_blocks: int = 0, rng_state=(12345,) * 6, _handle=None, _n=None):
        """cg_poly: preconditioner of the mixed-precision CG_nomass solve (0: default Chebyshev degree 6,
        -1: Jacobi alone as the reference, 2, 4, 6 or 8: Chebyshev degree); the FP64 path always uses Jacobi.
        cg_smem_blocks: 3x3 matrix blocks per row that the mixed single-reduction CG keeps in shared memory
        (0: as many as fit, n > 0: at most n, -1: none); results do not depend on it."""
        self._lib = load()
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
            self.n_nodes, self.n_elem = _n
        else:
            params = make_params(solver=solver, precision=precision, dt=dt, kT=kT, epsilon=epsilon,
                                 max_iterations_cg=max_iterations_cg, calc_noise=calc_noise,
                                 calc_stokes=calc_stokes, stokes_visc=stokes_visc, cg_poly=cg_poly,
                                 cg_smem_blocks=cg_smem_blocks)
            s = mesh.scale / MESO_LENGTH
            self._keep = [np.ascontiguousarray(mesh.pos * s, np.float64),
                          np.ascontiguousarray(mesh.tets, np.int32),
                          np.ascontiguousarray(mesh.stokes_radius * s, np.float64),
                          np.ascontiguousarray(mesh.pinned, np.int32) if len(mesh.pinned) else None]
            mat = material_from_si(mesh.material)
            self._keep += [mat[k] for k in ("rho", "A", "B", "G", "E")]
            m = MeshStruct(mesh.n_nodes, mesh.n_elem, len(mesh.pinned), _p(self._keep[0]), _p(self._keep[1]),
                           *(_p(mat[k]) for k in ("rho", "A", "B", "G", "E")), _p(self._keep[2]),
                           _p(self._keep[3]))
            _check(self._lib.ffea_gpu_blob_create(C.byref(m), C.byref(params), C.byref(self._h)), "blob_create")
            self._keep = None
            self.n_nodes, self.n_elem = mesh.n_nodes, mesh.n_elem
        self.set_rng_state(rng_state)

    @classmethod
    def from_files(cls, node, top, mat, stokes, pin, scale, *, solver="CG_nomass", precision="fp64",
                   rng_state=(12345,) * 6, **si):
        """Blob::config + Blob::init from the reference's structure files."""
        lib = load()
        params = make_params(solver=solver, precision=precision, **si)
        h = C.c_void_p()
        enc = lambda s: None if s is None else str(s).encode()  # noqa: E731
        _check(lib.ffea_gpu_blob_load(enc(node), enc(top), enc(mat), enc(stokes), enc(pin), float(scale),
                                      C.byref(params), C.byref(h)), "blob_load")
        with open(node) as f:
            f.readline()
            n = int(f.readline().split()[1])
        with open(top) as f:
            f.readline()
            t = int(f.readline().split()[1])
        return cls(_handle=h, _n=(n, t), rng_state=rng_state)

    def close(self) -> None:
        if getattr(self, "_borrowed", False):
            self._h = C.c_void_p()
            return
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ffea_gpu_blob_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()

    # -- the step -------------------------------------------------------------
    def update(self, nsteps: int = 1) -> int:
        """Run nsteps; raises FFEAError at the first failing step. Returns steps done."""
        done = C.c_int(0)
        rc = self._lib.ffea_gpu_blob_step(self._h, int(nsteps), C.byref(done))
        self.steps_done = done.value
        _check(rc, f"step (after {done.value} completed steps)")
        return done.value

    def update_timed(self, nsteps: int, flush_bytes: int = 0, phases: bool = True) -> dict:
        """update() with per-step CUDA-event timing on the blob's stream (flush outside the timed window).
        phases: also time each phase (events between the step's kernels, which cost a little themselves);
        without, the steps run exactly as update() runs them and phase_ms is None."""
        done, ms = C.c_int(0), C.c_double(0)
        ph = np.zeros(5)
        rc = self._lib.ffea_gpu_blob_step_timed(self._h, int(nsteps), int(flush_bytes), C.byref(done), C.byref(ms),
                                                _p(ph) if phases else None)
        _check(rc, f"step_timed (after {done.value} completed steps)")
        return {"steps": done.value, "ms": ms.value,
                "phase_ms": dict(zip(("element", "assemble", "gather", "cg", "euler"), ph.tolist())) if phases
                else None}

    def try_update(self, nsteps: int = 1) -> tuple[int, int]:
        """Like update() but returns (status, steps_done) instead of raising."""
        done = C.c_int(0)
        rc = self._lib.ffea_gpu_blob_step(self._h, int(nsteps), C.byref(done))
        return rc, done.value

    # -- state ------------------------------------------------------------------
    def state(self):
        pos = np.empty((self.n_nodes, 3))
        vel = np.empty((self.n_nodes, 3))
        force = np.empty((self.n_nodes, 3))
        _check(self._lib.ffea_gpu_blob_get_state(self._h, _p(pos), _p(vel), _p(force)), "get_state")
        return pos, vel, force

    def pos(self, out: np.ndarray | None = None) -> np.ndarray:
        """Node positions (num_nodes, 3) in the reference's order; `out` (C-contiguous float64, e.g. a view of
        pinned host memory) is filled in place."""
        o = _out(out, (self.n_nodes, 3))
        _check(self._lib.ffea_gpu_blob_get_state(self._h, _p(o), None, None), "get_state")
        return o

    def vel(self, out: np.ndarray | None = None) -> np.ndarray:
        o = _out(out, (self.n_nodes, 3))
        _check(self._lib.ffea_gpu_blob_get_state(self._h, None, _p(o), None), "get_state")
        return o

    def set_state(self, pos=None, vel=None) -> None:
        pa = None if pos is None else np.ascontiguousarray(pos, np.float64)
        va = None if vel is None else np.ascontiguousarray(vel, np.float64)
        _check(self._lib.ffea_gpu_blob_set_state(self._h, _p(pa), _p(va)), "set_state")

    def set_rng_state(self, s) -> None:
        a = np.ascontiguousarray(s, np.uint32)
        _check(self._lib.ffea_gpu_blob_set_rng_state(self._h, _p(a)), "set_rng_state")

    def rng_state(self) -> np.ndarray:
        a = np.empty(6, np.uint32)
        _check(self._lib.ffea_gpu_blob_get_rng_state(self._h, _p(a)), "get_rng_state")
        return a

    def measure(self) -> tuple[float, float]:
        se, ke = C.c_double(), C.c_double()
        _check(self._lib.ffea_gpu_blob_measure(self._h, C.byref(se), C.byref(ke)), "measure")
        return se.value, ke.value

    def load_ctforces(self, ctforces_file: str, surface_file: str | None = None, blob_index: int = 0) -> None:
        """The reference's constant forces (linear on nodes, linear over surface faces) for this blob."""
        _check(self._lib.ffea_gpu_blob_load_ctforces(self._h, str(ctforces_file).encode(),
                                                     None if surface_file is None else str(surface_file).encode(),
                                                     int(blob_index)), "load_ctforces")

    def measurements(self) -> dict:
        """Blob::make_measurements on the device (meso units)."""
        o = np.zeros(6)
        _check(self._lib.ffea_gpu_blob_measurements(self._h, _p(o)), "measurements")
        return {"strain_energy": o[0], "kinetic_energy": o[1], "centroid": o[2:5].copy(), "rmsd": o[5]}

    def set_rmsd_reference(self) -> None:
        _check(self._lib.ffea_gpu_blob_set_rmsd_reference(self._h), "set_rmsd_reference")

    def cg_iterations(self) -> tuple[int, int]:
        last, total = C.c_int(), C.c_longlong()
        _check(self._lib.ffea_gpu_blob_cg_iterations(self._h, C.byref(last), C.byref(total)), "cg_iterations")
        return last.value, total.value

    def cg_history(self, max_entries: int = 100000) -> np.ndarray:
        """|r|^2/|f|^2 after each CG iteration of the last solve."""
        buf = np.empty(max_entries)
        n = C.c_int()
        _check(self._lib.ffea_gpu_blob_cg_history(self._h, _p(buf), max_entries, C.byref(n)), "cg_history")
        return buf[:n.value].copy()

    CG_PHASES = ("setup", "spmv", "reduce_a", "barrier_a", "sum_a", "update", "reduce_b", "barrier_b", "sum_b",
                 "direction")

    def cg_profile(self) -> dict:
        """Device time (ns) of the last CG solve per phase, as seen by one thread block."""
        buf = np.zeros(len(self.CG_PHASES))
        _check(self._lib.ffea_gpu_blob_cg_profile(self._h, _p(buf), buf.size), "cg_profile")
        return dict(zip(self.CG_PHASES, buf.tolist()))

    def cg_preconditioner(self) -> tuple[int, float]:
        """(Chebyshev degree of the next CG solve, 0 for Jacobi; its lambda_max(D^-1 V) estimate)."""
        d, lm = C.c_int(), np.zeros(1)
        _check(self._lib.ffea_gpu_blob_cg_preconditioner(self._h, C.byref(d), _p(lm)), "cg_preconditioner")
        return d.value, float(lm[0])

    def cg_kernel(self) -> str:
        """Name of the persistent CG kernel this blob's steps launch ("none" for masslumped)."""
        return self._lib.ffea_gpu_blob_cg_kernel(self._h).decode()

    def sizes(self) -> tuple[int, int, int]:
        nl, ne, nb = C.c_int(), C.c_int(), C.c_longlong()
        _check(self._lib.ffea_gpu_blob_sizes(self._h, C.byref(nl), C.byref(ne), C.byref(nb)), "sizes")
        return nl.value, ne.value, nb.value

    def pattern(self, values: bool = True) -> dict:
        nnz = C.c_longlong()
        _check(self._lib.ffea_gpu_blob_get_pattern(self._h, None, None, None, None, C.byref(nnz)), "get_pattern")
        d = {"key": np.empty(3 * self.n_nodes + 1, np.int32), "col": np.empty(nnz.value, np.int32),
             "nsrc": np.empty(nnz.value, np.int32), "val": np.empty(nnz.value) if values else None}
        _check(self._lib.ffea_gpu_blob_get_pattern(self._h, _p(d["key"]), _p(d["col"]), _p(d["val"]), _p(d["nsrc"]),
                                                   C.byref(nnz)), "get_pattern")
        return d

    def connectivity(self) -> dict:
        cnt = C.c_longlong()
        _check(self._lib.ffea_gpu_blob_get_connectivity(self._h, None, None, C.byref(cnt)), "get_connectivity")
        d = {"ptr": np.empty(self.n_nodes + 1, np.int32), "elem_slot": np.empty(cnt.value, np.int32)}
        _check(self._lib.ffea_gpu_blob_get_connectivity(self._h, _p(d["ptr"]), _p(d["elem_slot"]), C.byref(cnt)),
               "get_connectivity")
        return d

    def elements(self, visc: bool = False) -> dict:
        T = self.n_elem
        d = {"node_force": np.empty((T, 4, 3)), "vol": np.empty(T), "visc": np.empty((T, 12, 12)) if visc else None}
        _check(self._lib.ffea_gpu_blob_get_elements(self._h, _p(d["node_force"]), _p(d["vol"]), _p(d["visc"])),
               "get_elements")
        return d

    def rhs(self) -> np.ndarray:
        o = np.empty((self.n_nodes, 3))
        _check(self._lib.ffea_gpu_blob_get_rhs(self._h, _p(o)), "get_rhs")
        return o


class Adjoint:
    """Reverse-mode derivative of a window of CG_nomass steps of a ``Blob``.

    ``forward()`` runs the window (checkpointing every ``checkpoint_every`` steps); ``backward(dl_dx)``
    takes dL/d(final positions) and returns dL/d(G, E, A, B) per element (meso units) and
    dL/d(initial positions)."""

    def __init__(self, blob: "Blob", window_steps: int, checkpoint_every: int):
        self._lib = load()
        self.blob = blob  # the blob stays alive while its adjoint is
        self._h = C.c_void_p()
        _check(self._lib.ffea_gpu_adjoint_create(blob._h, int(window_steps), int(checkpoint_every),
                                                 C.byref(self._h)), "adjoint_create")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ffea_gpu_adjoint_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()

    def forward(self) -> int:
        done = C.c_int(0)
        _check(self._lib.ffea_gpu_adjoint_forward(self._h, C.byref(done)), "adjoint_forward")
        return done.value

    def backward(self, dl_dx_final: np.ndarray) -> dict:
        g = np.ascontiguousarray(dl_dx_final, np.float64).reshape(-1)
        ne, nn = self.blob.n_elem, self.blob.n_nodes
        out = {k: np.zeros(ne) for k in ("G", "E", "A", "B")}
        out["x0"] = np.zeros((nn, 3))
        _check(self._lib.ffea_gpu_adjoint_backward(self._h, _p(g), _p(out["G"]), _p(out["E"]), _p(out["A"]),
                                                   _p(out["B"]), _p(out["x0"])), "adjoint_backward")
        return out


class World:
    """A reference ``.ffea`` script run on the GPU (blob-step path only): ``World(script).run()`` writes the
    trajectory, measurement and checkpoint files the reference writes."""

    def __init__(self, script: str, precision: str = "fp64"):
        self._lib = load()
        self._h = C.c_void_p()
        _check(self._lib.ffea_gpu_world_load(str(script).encode(), PRECISIONS[precision], C.byref(self._h)),
               "world_load")

    def run(self) -> int:
        last = C.c_longlong(0)
        _check(self._lib.ffea_gpu_world_run(self._h, C.byref(last)), f"world_run (stopped at step {last.value})")
        return last.value

    @property
    def num_blobs(self) -> int:
        return int(self._lib.ffea_gpu_world_num_blobs(self._h))

    def blob(self, i: int = 0) -> "Blob":
        """The i-th blob (owned by the World: valid while the World is)."""
        h = self._lib.ffea_gpu_world_blob(self._h, i)
        if not h:
            raise IndexError(i)
        b = Blob.__new__(Blob)
        b._lib, b._h, b._borrowed = self._lib, C.c_void_p(h), True
        n, t = C.c_int(), C.c_int()
        _check(self._lib.ffea_gpu_blob_counts(b._h, C.byref(n), C.byref(t)), "blob_counts")
        b.n_nodes, b.n_elem = n.value, t.value
        return b

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ffea_gpu_world_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()


def meso_to_si_gradients(g: dict) -> dict:
    """Chain rule from dL/d(G, E, A, B) (meso) to the SI material columns of ``Mesh.material``:
    shear/bulk modulus and shear/bulk viscosity (A = eta_s/(P t), B = eta_b/(P t) - 2/3 eta_s,
    G = G_SI/P, E = K_SI/P, as the reference's load_material_params converts them)."""
    P, t = 8.4305832688784826e8, 3.7302915560886126e-13
    return {"shear_mod": g["G"] / P, "bulk_mod": g["E"] / P,
            "shear_visc": g["A"] / (P * t) - (2.0 / 3.0) * g["B"], "bulk_visc": g["B"] / (P * t)}


def _mesh_struct(mesh: Mesh, keep: list) -> MeshStruct:
    """ffea_gpu_mesh of a Mesh in meso units; the arrays it points to are appended to `keep`."""
    s = mesh.scale / MESO_LENGTH
    arrs = [np.ascontiguousarray(mesh.pos * s, np.float64), np.ascontiguousarray(mesh.tets, np.int32),
            np.ascontiguousarray(mesh.stokes_radius * s, np.float64),
            np.ascontiguousarray(mesh.pinned, np.int32) if len(mesh.pinned) else None]
    mat = material_from_si(mesh.material)
    arrs += [mat[k] for k in ("rho", "A", "B", "G", "E")]
    keep += arrs
    return MeshStruct(mesh.n_nodes, mesh.n_elem, len(mesh.pinned), _p(arrs[0]), _p(arrs[1]),
                      *(_p(mat[k]) for k in ("rho", "A", "B", "G", "E")), _p(arrs[2]), _p(arrs[3]))


class Batch:
    """Many independent blobs of uneven size advanced together (mixed precision, CG_nomass).

    Every blob runs the per-blob step of the reference's World::run; blob b's noise is substream b of
    the package seed's stream. One step of the whole batch is one CUDA graph replay."""

    def __init__(self, meshes: list[Mesh], *, dt: float = 1e-12, kT: float = 4.11e-21, epsilon: float = 1e-10,
                 max_iterations_cg: int = 10000, calc_noise: int = 1, calc_stokes: int = 0,
                 stokes_visc: float = 1e-3):
        self._lib = load()
        self._h = C.c_void_p()
        params = make_params(solver="CG_nomass", precision="mixed", dt=dt, kT=kT, epsilon=epsilon,
                             max_iterations_cg=max_iterations_cg, calc_noise=calc_noise, calc_stokes=calc_stokes,
                             stokes_visc=stokes_visc)
        keep: list = []
        arr = (MeshStruct * len(meshes))(*[_mesh_struct(m, keep) for m in meshes])
        _check(self._lib.ffea_gpu_batch_create(C.cast(arr, C.c_void_p), len(meshes), C.byref(params),
                                               C.byref(self._h)), "batch_create")
        self.n_blobs = len(meshes)
        self.n_nodes = [m.n_nodes for m in meshes]

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ffea_gpu_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()

    def update(self, nsteps: int = 1) -> int:
        done = C.c_int(0)
        rc = self._lib.ffea_gpu_batch_step(self._h, int(nsteps), C.byref(done))
        _check(rc, f"batch_step (after {done.value} completed steps)")
        return done.value

    def update_timed(self, nsteps: int, flush_bytes: int = 0, cg: bool = False) -> dict:
        """update() timed by CUDA events around each step; cg: also the steps' CG launches (events inside the
        step), in "cg_ms"."""
        done, ms, mc = C.c_int(0), C.c_double(0), C.c_double(0)
        rc = self._lib.ffea_gpu_batch_step_timed(self._h, int(nsteps), int(flush_bytes), C.byref(done), C.byref(ms),
                                                 C.byref(mc) if cg else None)
        _check(rc, f"batch_step_timed (after {done.value} completed steps)")
        return {"steps": done.value, "ms": ms.value, "cg_ms": mc.value if cg else None}

    def state(self, blob: int):
        pos = np.empty((self.n_nodes[blob], 3))
        vel = np.empty((self.n_nodes[blob], 3))
        _check(self._lib.ffea_gpu_batch_get_state(self._h, blob, _p(pos), _p(vel)), "batch_get_state")
        return pos, vel

    def pos(self, blob: int) -> np.ndarray:
        o = np.empty((self.n_nodes[blob], 3))
        _check(self._lib.ffea_gpu_batch_get_state(self._h, blob, _p(o), None), "batch_get_state")
        return o

    def set_state(self, blob: int, pos=None, vel=None) -> None:
        pa = None if pos is None else np.ascontiguousarray(pos, np.float64)
        va = None if vel is None else np.ascontiguousarray(vel, np.float64)
        _check(self._lib.ffea_gpu_batch_set_state(self._h, blob, _p(pa), _p(va)), "batch_set_state")

    def positions(self, out: np.ndarray | None = None) -> np.ndarray:
        """Every blob's node positions, back to back in blob order: (sum of node counts, 3)."""
        o = _out(out, (int(sum(self.n_nodes)), 3))
        _check(self._lib.ffea_gpu_batch_get_states(self._h, _p(o), None), "batch_get_states")
        return o

    def set_positions(self, pos) -> None:
        pa = np.ascontiguousarray(pos, np.float64)
        if pa.size != 3 * int(sum(self.n_nodes)):
            raise ValueError("positions of every blob, back to back")
        _check(self._lib.ffea_gpu_batch_set_states(self._h, _p(pa), None), "batch_set_states")

    def rng_state(self, blob: int) -> np.ndarray:
        a = np.empty(6, np.uint32)
        _check(self._lib.ffea_gpu_batch_get_rng_state(self._h, blob, _p(a)), "batch_get_rng_state")
        return a

    def set_rng_state(self, blob: int, s) -> None:
        a = np.ascontiguousarray(s, np.uint32)
        _check(self._lib.ffea_gpu_batch_set_rng_state(self._h, blob, _p(a)), "batch_set_rng_state")

    def strain_energies(self) -> np.ndarray:
        """Each blob's strain energy (meso units), as Blob.measurements()["strain_energy"]."""
        out = np.empty(self.n_blobs)
        _check(self._lib.ffea_gpu_batch_strain_energies(self._h, _p(out)), "batch_strain_energies")
        return out

    def load_ctforces(self, blob: int, ctforces_file: str, surface_file: str | None = None,
                      blob_index: int = 0) -> None:
        """The reference's constant forces for one blob of the batch (as Blob.load_ctforces)."""
        _check(self._lib.ffea_gpu_batch_load_ctforces(self._h, int(blob), str(ctforces_file).encode(),
                                                      None if surface_file is None else str(surface_file).encode(),
                                                      int(blob_index)), "batch_load_ctforces")

    def cg_iterations(self) -> tuple[np.ndarray, int]:
        last = np.zeros(self.n_blobs, np.int32)
        total = C.c_longlong()
        _check(self._lib.ffea_gpu_batch_cg_iterations(self._h, _p(last), C.byref(total)), "batch_cg_iterations")
        return last, total.value

    def sizes(self) -> dict:
        nb, nl, ne, blocks = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        _check(self._lib.ffea_gpu_batch_sizes(self._h, C.byref(nb), C.byref(nl), C.byref(ne), C.byref(blocks)),
               "batch_sizes")
        return {"blobs": nb.value, "nodes": nl.value, "elements": ne.value, "blocks": blocks.value}

    def blob_sizes(self, blob: int) -> tuple[int, int, int]:
        n, nv, ne = C.c_int(), C.c_int(), C.c_int()
        _check(self._lib.ffea_gpu_batch_blob_sizes(self._h, blob, C.byref(n), C.byref(nv), C.byref(ne)),
               "batch_blob_sizes")
        return n.value, nv.value, ne.value

    def config(self) -> dict:
        t, p, c = C.c_int(), C.c_int(), C.c_int()
        _check(self._lib.ffea_gpu_batch_config(self._h, C.byref(t), C.byref(p), C.byref(c)), "batch_config")
        e, a, sp, g = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(self._lib.ffea_gpu_batch_shapes(self._h, C.byref(e), C.byref(a), C.byref(sp), C.byref(g)),
               "batch_shapes")
        return {"cg_threads": t.value, "threads_per_row": p.value, "ctas": c.value, "element_threads": e.value,
                "assembly_threads": a.value, "assembly_split": sp.value, "gather_threads": g.value}

    def set_config(self, cg_threads: int, threads_per_row: int) -> None:
        _check(self._lib.ffea_gpu_batch_set_config(self._h, int(cg_threads), int(threads_per_row)),
               "batch_set_config")

    def set_shapes(self, element_threads: int, assembly_threads: int, assembly_split: int,
                   gather_threads: int) -> None:
        _check(self._lib.ffea_gpu_batch_set_shapes(self._h, int(element_threads), int(assembly_threads),
                                                   int(assembly_split), int(gather_threads)), "batch_set_shapes")

    def tune(self, solves: int = 2) -> float:
        """Autotune the force phase's launch shapes (elements per block, assembly and gather blocks) and the CG
        launch (CTA size, threads per row) on the current forces; returns the best CG solve ms."""
        best = C.c_double()
        _check(self._lib.ffea_gpu_batch_tune(self._h, int(solves), C.byref(best)), "batch_tune")
        return best.value


def launch_count() -> int:
    return int(load().ffea_gpu_launch_count())
