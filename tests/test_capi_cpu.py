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
                             y.ctypes.data_as(capi._dp), 1, nu.ctypes.data_as(capi._dp), 1, None, 0, 4, 0)
    assert rc == -4  # no method 4
    rc = lib.sgb_tfem_create(ctypes.byref(h), 0, pos.ctypes.data_as(capi._dp), 0, None, None, 0, None, 0, None, 0,
                             1, 0)
    assert rc == -1
    # the largest mesh: 12 corner terms per tetrahedron must index with 32
    # bits; one more tetrahedron is refused before the array is read
    too_many = 0x7FFFFFFF // 12 + 1
    rc = lib.sgb_tfem_create(ctypes.byref(h), 4, pos.ctypes.data_as(capi._dp), too_many,
                             tets.ctypes.data_as(capi._ip), y.ctypes.data_as(capi._dp), 1,
                             nu.ctypes.data_as(capi._dp), 1, None, 0, 1, 0)
    assert rc == -1 and "too many tetrahedra" in capi.last_error()
    # non-finite rest positions are refused
    bad = pos.copy()
    bad[2, 1] = np.nan
    tets_ok = np.array([[0, 1, 2, 3]], dtype=np.int32)
    rc = lib.sgb_tfem_create(ctypes.byref(h), 4, bad.ctypes.data_as(capi._dp), 1, tets_ok.ctypes.data_as(capi._ip),
                             y.ctypes.data_as(capi._dp), 1, nu.ctypes.data_as(capi._dp), 1, None, 0, 1, 0)
    assert rc == -1 and "non-finite" in capi.last_error()


def test_scene_params_defaults_match_reference_data(capi):
    p = capi.SceneParams()
    capi.load().sgb_scene_params_default(ctypes.byref(p))
    # EulerImplicitSolver.cpp:40-51 and CGLinearSolver.inl:34-46 defaults
    assert p.rayleigh_stiffness == 0.0 and p.rayleigh_mass == 0.0
    assert p.cg_iterations == 25 and p.cg_tolerance == 1e-5 and p.cg_threshold == 1e-5


@pytest.mark.parametrize("n,pe,pn", [((5, 5, 21), 64, 64), ((9, 7, 13), 1024, 1024), ((12, 12, 40), 1024, 1024),
                                      ((6, 6, 6), 7, 20)])
def test_patch_layout_invariants(capi, n, pe, pn):
    """The fused matvec's layout: every element corner is gathered exactly
    once, every node has one owner, shared nodes get one partial slot per
    patch (host logic, no GPU)."""
    from sofa_gb300 import topology as topo

    mesh = topo.beam(n, spacing=0.5, jitter=0.05, seed=1)
    stats = (ctypes.c_int * 5)()
    lib = capi.load()
    lib.sgb_patch_layout_check.argtypes = [ctypes.c_int, capi._dp, ctypes.c_int, capi._ip, ctypes.c_int,
                                           ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    pos = np.ascontiguousarray(mesh.positions)
    tets = np.ascontiguousarray(mesh.tetrahedra, dtype=np.int32)
    rc = lib.sgb_patch_layout_check(mesh.n_nodes, pos.ctypes.data_as(capi._dp), mesh.n_tets,
                                    tets.ctypes.data_as(capi._ip), pe, pn, stats)
    assert rc == 0, capi.last_error()
    patches, max_ln, total_ln, boundary, partials = list(stats)
    assert patches >= mesh.n_tets // pe
    assert max_ln <= pn
    assert total_ln >= mesh.n_nodes
    assert partials >= 2 * boundary


def test_patch_layout_random_soup(capi):
    """Unstructured input: random tetrahedra over random points."""
    rng = np.random.default_rng(3)
    pos = rng.normal(size=(300, 3))
    tets = np.stack([rng.choice(300, 4, replace=False) for _ in range(2000)]).astype(np.int32)
    stats = (ctypes.c_int * 5)()
    lib = capi.load()
    rc = lib.sgb_patch_layout_check(300, pos.ctypes.data_as(capi._dp), 2000, tets.ctypes.data_as(capi._ip), 128, 100,
                                    stats)
    assert rc == 0, capi.last_error()


def test_patch_layout_nodes_of_no_element(capi):
    """Nodes that no tetrahedron uses go into trailing patches without
    elements (each node owned once, no partial slots), so the patch kernels
    form their mass rows; the checker counts every node as touched."""
    from sofa_gb300 import topology as topo

    mesh = topo.beam((6, 6, 20), spacing=0.5, jitter=0.05, seed=2)
    n_old = mesh.n_nodes
    # interleave unused nodes: old node i -> 2 i
    pos = np.zeros((2 * n_old, 3))
    pos[0::2] = mesh.positions
    pos[1::2] = mesh.positions + 0.1
    tets = np.ascontiguousarray(2 * mesh.tetrahedra, dtype=np.int32)
    stats = (ctypes.c_int * 5)()
    lib = capi.load()
    lib.sgb_patch_layout_check.argtypes = [ctypes.c_int, capi._dp, ctypes.c_int, capi._ip, ctypes.c_int,
                                           ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    for pe, pn in ((64, 64), (256, 1024)):
        rc = lib.sgb_patch_layout_check(2 * n_old, np.ascontiguousarray(pos).ctypes.data_as(capi._dp),
                                        mesh.n_tets, tets.ctypes.data_as(capi._ip), pe, pn, stats)
        assert rc == 0, capi.last_error()
        patches, max_ln, total_ln, boundary, partials = list(stats)
        # the unused nodes appear exactly once each, in patches of at most
        # max_ln nodes
        assert patches >= -(-n_old // max_ln) + mesh.n_tets // pe
        assert total_ln >= 2 * n_old


@pytest.mark.parametrize("field,value", [("linear_solver", 1), ("preconditioner", 1), ("warm_start", 1),
                                         ("residual_replacement", 20), ("serial_dots", 1),
                                         ("compute_residual", 1)])
def test_batch_admission_refuses_solver_options_it_does_not_run(capi, field, value):
    """The batch engine runs cold-start CG with block-ordered dots; a mesh
    that asks for PCG, a preconditioner, warmStart, residual replacement or
    serial dots is refused (SGB_ERR_NOT_SUPPORTED) instead of being run as
    plain CG. Planning with a NULL batch runs the same checks host-side."""
    from sofa_gb300 import topology as topo

    lib = capi.load()
    mesh = topo.beam((3, 3, 5), spacing=0.5, jitter=0.05, seed=0)
    d, keep = capi.Batch.mesh_desc(mesh.positions, mesh.tetrahedra, method="polar", fixed=mesh.fixed)
    b = ctypes.c_size_t()
    assert lib.sgb_batch_mesh_bytes(None, ctypes.byref(d), ctypes.byref(b)) == 0
    assert b.value > 0
    setattr(d.params, field, value)
    rc = lib.sgb_batch_mesh_bytes(None, ctypes.byref(d), ctypes.byref(b))
    assert rc == -4, (rc, capi.last_error())
    assert "batched meshes" in capi.last_error()
