"""The reference-side adapter (tests/integration/blob_gpu_adapter.cpp) compiled against the reference's own headers
and linked against the reference's compiled classes and the GPU library (CPU; build container only).

A maintainer adds three member declarations and the `gpu` handle to class Blob (include/Blob.h:94) and the
adapter's definitions to the reference. The test does the same on a copy of Blob.h in a temporary directory,
compiles the adapter with the reference's release defines (the Boost/Eigen stand-ins of oracle/ref_shim supply the
headers that are absent here), and links it with --no-undefined against the reference's objects (oracle/_ref) and
libffea_gpu.so, so every C ABI call the adapter makes resolves to an exported entry point.
"""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _reference():
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from __graft_entry__ import REFERENCE
    return REFERENCE


PUBLIC = "    void gpu_attach(const SimulationParams &p);\n    void gpu_step();\n    void gpu_pull();\n"
PRIVATE = "    ffea_gpu_blob *gpu = nullptr;\n"


def test_adapter_compiles_and_links_against_the_reference(tmp_path):
    ref = _reference()
    blob_h = os.path.join(ref, "include", "Blob.h")
    ref_lib = os.path.join(ROOT, "oracle", "_ref", "libffea_ref.so")
    gpu_lib = os.path.join(ROOT, "ffea_ci_demo_gb300", "_build", "libffea_gpu.so")
    if not os.path.exists(blob_h) or not os.path.exists(ref_lib):
        pytest.skip("the reference's sources and its compiled classes are only in the build container")
    if not os.path.exists(gpu_lib):
        pytest.skip("libffea_gpu.so is not built")
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = open(blob_h).read()
    # the maintainer's edit: the adapter's members at the top of class Blob's public section, the handle in its
    # private section
    m = re.search(r"class Blob\s*\{\s*public:\s*\n", src)
    assert m, "class Blob { public: not found"
    q = re.compile(r"\nprivate:\s*\n").search(src, m.end())
    assert q, "class Blob's private section not found"
    patched = ('#include "ffea_gpu.h"\n' + src[:m.end()] + PUBLIC + src[m.end():q.end()] + PRIVATE +
               src[q.end():])
    inc = tmp_path / "include"
    inc.mkdir()
    (inc / "Blob.h").write_text(patched)
    flags = ["-std=c++17", "-O1", "-fPIC", "-DUSE_DOUBLE", "-DUSE_OPENMP", "-DFFEA_PARALLEL_WITHIN_BLOB", "-fopenmp",
             "-w", f"-I{inc}", f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ref, 'include')}",
             f"-I{os.path.join(ROOT, 'oracle', 'ref_shim')}", f"-I{os.path.join(ROOT, 'oracle', '_ref', 'shim')}"]
    obj = tmp_path / "adapter.o"
    r = subprocess.run([gxx, *flags, "-c", os.path.join(HERE, "integration", "blob_gpu_adapter.cpp"), "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    so = tmp_path / "adapter.so"
    r = subprocess.run([gxx, "-shared", "-fopenmp", "-o", str(so), str(obj), ref_lib, gpu_lib, "-Wl,--no-undefined",
                        f"-Wl,-rpath,{os.path.dirname(ref_lib)}:{os.path.dirname(gpu_lib)}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # the adapter's members are defined in the object, the C ABI entry points it calls are imported
    nm = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True).stdout
    for sym in ("Blob::gpu_attach(SimulationParams const&)", "Blob::gpu_step()", "Blob::gpu_pull()"):
        assert re.search(r" T " + re.escape(sym), nm), sym
    for sym in ("ffea_gpu_blob_create", "ffea_gpu_blob_step", "ffea_gpu_blob_get_state", "ffea_gpu_blob_set_rng_state",
                "ffea_gpu_params_default", "ffea_gpu_last_error"):
        assert re.search(r" U " + sym + r"\b", nm), sym
