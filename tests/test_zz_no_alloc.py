"""The no-allocation addDForce (sgb_tfem_add_dforce_f32_noalloc).

Some callers cannot allocate device memory where they need a force
derivative -- a host framework handing out buffers from its own pool, a
real-time loop that must not hit the synchronisation cudaMalloc/cudaFree
imply. For them the library offers an addDForce whose only scratch is a
fixed array in its own device memory. This test calls it through the C ABI
twice in a row (the second call reuses the array the first one filled) and
checks each result against the handle-based sgb_tfem_add_dforce_f32 on the
same state, within the mixed-precision per-call tolerance of the other GPU
tests (1e-5 relative, on the contribution: the second call accumulates
into a non-zero df). It builds everything it needs itself, so it passes
alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


def node_csr(tets, n_nodes):
    """node -> (tetrahedron*4 + corner) in increasing order."""
    flat = np.asarray(tets, dtype=np.int64).reshape(-1)
    order = np.argsort(flat, kind="stable")
    rowptr = np.zeros(n_nodes + 1, dtype=np.int32)
    np.add.at(rowptr, flat + 1, 1)
    return np.cumsum(rowptr, dtype=np.int64).astype(np.int32), order.astype(np.int32)


def test_noalloc_matches_handle_twice(torch_cuda, capi, oracle):
    torch = torch_cuda
    lib = capi.load()
    fn = lib.sgb_tfem_add_dforce_f32_noalloc
    vp = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_float, vp]

    mesh = cases.beam_mesh((6, 6, 20))
    N, E = mesh.n_nodes, mesh.n_tets
    rng = np.random.default_rng(5)
    x = mesh.positions + rng.normal(scale=5e-3, size=mesh.positions.shape)

    # handle-based path: rotations from add_force at x, then add_dforce
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large", "mixed")
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    fd = torch.zeros((N, 3), dtype=torch.float32, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())

    # the same element data in the no-allocation layout, from the oracle
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large")
    ofem.add_force(x)
    rot = np.empty((9, E), np.float32)
    K = np.empty((3, E), np.float32)
    J = np.empty((12, E), np.float32)
    for e in range(E):
        el = ofem.element(e)
        rot[:, e] = el["rotation"].T.reshape(9)  # rows of R = rotations[e]^T
        K[:, e] = el["K3"]
        J[:, e] = el["J3"].reshape(12)
    rowptr, slots = node_csr(mesh.tetrahedra, N)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
           dict(tets=mesh.tetrahedra.astype(np.int32), rot=rot, K=K, J=J, rowptr=rowptr, slots=slots).items()}

    kfactor = -0.0011
    scale = 0.0
    for call in range(2):
        dx = rng.normal(scale=1e-3, size=(N, 3)).astype(np.float32)
        dxd = torch.from_numpy(dx).cuda()
        # both entry points accumulate (df -= ...): the second call starts
        # from the same non-zero df in both, of the size of a contribution
        df0 = rng.normal(scale=scale, size=(N, 3)).astype(np.float32)
        df_handle = torch.from_numpy(df0.copy()).cuda()
        fem.add_dforce(dxd.data_ptr(), df_handle.data_ptr(), kfactor)
        df_noalloc = torch.from_numpy(df0.copy()).cuda()
        rc = fn(N, E, dev["tets"].data_ptr(), dev["rot"].data_ptr(), dev["K"].data_ptr(), dev["J"].data_ptr(),
                dev["rowptr"].data_ptr(), dev["slots"].data_ptr(), dxd.data_ptr(), df_noalloc.data_ptr(), kfactor,
                None)
        assert rc == 0, capi.last_error()
        torch.cuda.synchronize()
        a = df_noalloc.cpu().double().numpy() - df0
        b = df_handle.cpu().double().numpy() - df0
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= 1e-5, (call, err)
        scale = float(np.sqrt(np.mean(b * b)))
    fem.close()


def test_noalloc_rejects_oversize(capi):
    lib = capi.load()
    fn = lib.sgb_tfem_add_dforce_f32_noalloc
    vp = ctypes.c_void_p
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_float, vp]
    rc = fn(10, (1 << 18) + 1, 16, 16, 16, 16, 16, 16, 16, 16, 1.0, None)
    assert rc == -1
    assert "exceed the fixed scratch" in capi.last_error()
