"""The C-ABI library: it loads, exports every declared entry point, and its
host-only helpers convert units exactly as the reference's loaders do.
(No device work here: these tests run without a GPU.)"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
from ffea_ci_demo_gb300 import build, lib
from ffea_ci_demo_gb300.mesh import kuhn_cube


@pytest.fixture(scope="module")
def L():
    build.build()
    return lib.load()


def test_exports_every_declared_symbol(L):
    names = lib.header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n


def test_params_assign_matches_simulationparams(L, oracle_built):
    p = lib.make_params(dt=1e-12, kT=4.11e-21, epsilon=1e-10, stokes_visc=1e-3, max_iterations_cg=77,
                        calc_noise=0, calc_stokes=1)
    m = kuhn_cube(1)
    o = po.OracleBlob(m, dt=1e-12, kT=4.11e-21, epsilon=1e-10, stokes_visc=1e-3)
    assert p.dt == o.param("dt") and p.kT == o.param("kT")
    assert p.epsilon2 == o.param("epsilon2") and p.stokes_visc == o.param("stokes_visc")
    assert (p.max_iterations_cg, p.calc_noise, p.calc_stokes) == (77, 0, 1)
    assert L.ffea_gpu_params_assign(C.byref(p), b"calc_ssint", b"1") == lib.EINPUT
    assert L.ffea_gpu_params_assign(C.byref(p), b"solver", b"direct") == lib.EINPUT
    # the mixed CG_nomass preconditioner (an engine key): -1 Jacobi, 0 default, 2, 4, 6 or 8 Chebyshev degree
    for v in (-1, 0, 2, 4, 6, 8):
        assert L.ffea_gpu_params_assign(C.byref(p), b"cg_poly", str(v).encode()) == lib.OK and p.cg_poly == v
    for v in (-2, 1, 3, 5, 10):
        assert L.ffea_gpu_params_assign(C.byref(p), b"cg_poly", str(v).encode()) == lib.EINPUT


def test_params_defaults(L):
    p = lib.Params()
    assert L.ffea_gpu_params_default(C.byref(p)) == 0
    # SimulationParams(): dt 1e-14 s, kT 4.11e-21 J, epsilon2 0.01, 1000 CG iterations, noise and Stokes on
    assert p.max_iterations_cg == 1000 and p.epsilon2 == 0.01 and p.calc_noise == 1 and p.calc_stokes == 1


def test_material_conversion_matches_reference_loader(L, oracle_built):
    m = kuhn_cube(2)
    m.material[:, 3] = np.linspace(1e8, 1e9, m.n_elem)
    got = lib.material_from_si(m.material)
    o = po.OracleBlob(m)
    want = o.rest()["mat"]
    for i, k in enumerate(("rho", "A", "B", "G", "E")):
        assert np.array_equal(got[k], want[:, i]), k
    # the reference's second viscosity: bulk/(P t) - (2/3) shear, shear in SI (src/Blob.cpp:2281)
    assert abs(got["B"][0] - 3.179132) < 1e-5


def test_blob_create_rejects_bad_input_without_gpu_work(L):
    p = lib.make_params()
    h = C.c_void_p()
    m = lib.MeshStruct()
    m.num_nodes, m.num_elements = 0, 0
    assert L.ffea_gpu_blob_create(C.byref(m), C.byref(p), C.byref(h)) == lib.EINPUT
    assert L.ffea_gpu_blob_step(None, 1, None) == lib.EINPUT
    p.cg_poly = 3  # odd degrees are refused: the preconditioner is positive definite for even ones only
    assert L.ffea_gpu_blob_create(C.byref(m), C.byref(p), C.byref(h)) == lib.EINPUT


def test_binding_constants_match_the_header():
    """The binding's status codes and preconditioner constants are the header's #defines."""
    import re
    src = open(lib.HEADER).read()
    defs = {k: int(v) for k, v in re.findall(r"^#define\s+(FFEA_GPU_\w+)\s+(-?\d+)", src, re.M)}
    assert defs["FFEA_GPU_CG_POLY_DEFAULT"] == lib.CG_POLY_DEFAULT
    assert defs["FFEA_GPU_CG_POLY_MAX"] == lib.CG_POLY_MAX
    for name in ("OK", "EINVERTED", "ECGMAXIT", "EINPUT", "ENOMEM", "ECUDA", "ENAN", "ETIMEOUT", "EFILE"):
        assert defs["FFEA_GPU_" + name] == getattr(lib, name), name
