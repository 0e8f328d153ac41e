"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point include/sofa_gb300.h declares; argument checks
that fail before any CUDA call behave like the reference's error handling."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    return capi


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(sgb_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(capi):
    lib = ctypes.CDLL(capi.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string(capi):
    lib = capi.load()
    assert b"sm_103a" in lib.sgb_version()


def test_create_rejects_bad_indices_before_touching_the_gpu(capi):
    lib = capi.load()
    pos = np.zeros((4, 3))
    tets = np.array([[0, 1, 2, 7]], dtype=np.int32)
    h = ctypes.c_void_p()
    y = np.array([5000.0])
    nu = np.array([0.45])
    rc = lib.sgb_tfem_create(ctypes.byref(h), 4, pos.ctypes.data_as(capi._dp), 1, tets.ctypes.data_as(capi._ip),
                             y.ctypes.data_as(capi._dp), 1, nu.ctypes.data_as(capi._dp), 1, None, 0, 1, 0)
    assert rc == -1
    assert "out of range" in capi.last_error()
    rc = lib.sgb_tfem_create(ctypes.byref(h), 4, pos.ctypes.data_as(capi._dp), 1, tets.ctypes.data_as(capi._ip),
                             y.ctypes.data_as(capi._dp), 1, nu.ctypes.data_as(capi._dp), 1, None, 0, 3, 0)
    assert rc == -4  # svd is not supported
    rc = lib.sgb_tfem_create(ctypes.byref(h), 0, pos.ctypes.data_as(capi._dp), 0, None, None, 0, None, 0, None, 0,
                             1, 0)
    assert rc == -1


def test_scene_params_defaults_match_reference_data(capi):
    p = capi.SceneParams()
    capi.load().sgb_scene_params_default(ctypes.byref(p))
    # EulerImplicitSolver.cpp:40-51 and CGLinearSolver.inl:34-46 defaults
    assert p.rayleigh_stiffness == 0.0 and p.rayleigh_mass == 0.0
    assert p.cg_iterations == 25 and p.cg_tolerance == 1e-5 and p.cg_threshold == 1e-5
