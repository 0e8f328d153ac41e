"""updateStiffnessMatrix on the GPU against the oracle (methods polar and
svd): every addForce rebuilds each element's strain-displacement matrix from
its deformed positions in its frame (TetrahedronFEMForceField.inl:1063-1067,
1174-1177) and the addDForce that follows uses it. FP64 reference rounding
bit-identical per call and over 10 scene steps with serial dots; FP64-FMA
within 1e-10; mixed within 1e-5 per call (the FP32 rebuild works on the
element's edges, the reference's formula on absolute coordinates: equal in
exact arithmetic) and 1e-4 on the positions after 10 steps. Method large is
refused (SGB_ERR_NOT_SUPPORTED)."""
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
def capi(torch_cuda):
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


def deformed(mesh, seed=4):
    rng = np.random.default_rng(seed)
    u = 0.05 * np.stack([np.sin(0.3 * mesh.positions[:, 2]), np.cos(0.2 * mesh.positions[:, 2]),
                         0.1 * mesh.positions[:, 0]], 1)
    return mesh.positions + u + rng.normal(scale=0.02, size=mesh.positions.shape)


@pytest.mark.parametrize("method", ["polar", "svd"])
@pytest.mark.parametrize("precision,tol", [("fp64", 0.0), ("fp64_fma", 1e-10), ("mixed", 1e-5)])
def test_per_call_against_oracle(torch_cuda, capi, oracle, method, precision, tol):
    torch = torch_cuda
    mesh = cases.beam_mesh()
    x = deformed(mesh)
    dx = np.random.default_rng(5).normal(scale=1e-3, size=x.shape)
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    ofem.set_update_stiffness(True)
    f_ref = ofem.add_force(x)
    df_ref = ofem.add_dforce(dx, -0.01)
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method, precision)
    fem.set_update_stiffness(True)
    dt = torch.float32 if precision == "mixed" else torch.float64
    if precision == "mixed":
        dx = dx.astype(np.float32).astype(np.float64)
        df_ref = ofem.add_dforce(dx, -0.01)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    fd = torch.zeros(x.shape, dtype=dt, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())
    dxd = torch.tensor(dx, dtype=dt, device="cuda")
    dfd = torch.zeros(x.shape, dtype=dt, device="cuda")
    fem.add_dforce(dxd.data_ptr(), dfd.data_ptr(), -0.01)
    torch.cuda.synchronize()
    f, df = fd.cpu().double().numpy(), dfd.cpu().double().numpy()
    fem.close()
    if tol == 0.0:
        assert np.array_equal(f, f_ref), cases.rel_err(f, f_ref)
        assert np.array_equal(df, df_ref), cases.rel_err(df, df_ref)
    else:
        assert cases.rel_err(f, f_ref) <= tol and cases.rel_err(df, df_ref) <= tol
    # the rebuilt matrix changes the result against the initial one
    plain = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    plain.add_force(x)
    assert cases.rel_err(plain.add_dforce(dx, -0.01), df_ref) > 1e-4


@pytest.mark.parametrize("method", ["polar", "svd"])
def test_scene_steps_against_oracle(capi, oracle, method):
    mesh = cases.beam_mesh()
    cfg = cases.BEAM_SMALL
    ofem, osc = cases.oracle_scene(oracle, mesh, method)
    ofem.set_update_stiffness(True)
    osc.step(10)
    xr, vr = osc.state()
    d = np.linalg.norm(xr - mesh.positions)
    for precision in ("fp64", "mixed"):
        fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, cfg["young"], cfg["poisson"], method, precision)
        fem.set_update_stiffness(True)
        sc = capi.Scene(fem, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"],
                        cg_iterations=cfg["cg_iterations"], cg_tolerance=cfg["cg_tolerance"],
                        cg_threshold=cfg["cg_threshold"], gravity=cfg["gravity"],
                        vertex_mass=cfg["total_mass"] / mesh.n_nodes, fixed=mesh.fixed,
                        serial_dots=precision == "fp64")
        sc.step(10)
        it, _ = sc.sync()
        x, v = sc.state()
        sc.close()
        if precision == "fp64":
            assert it == osc.last_iterations
            assert np.array_equal(x, xr) and np.array_equal(v, vr)
        else:
            assert np.linalg.norm(x - xr) / d <= 1e-4


def test_large_is_refused(capi):
    mesh = cases.beam_mesh((3, 3, 6))
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large", "fp64")
    with pytest.raises(capi.SgbError) as e:
        fem.set_update_stiffness(True)
    assert e.value.code == -4
    fem.set_update_stiffness(False)
    fem.close()
    small = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "small", "fp64")
    small.set_update_stiffness(True)  # ignored, as the reference ignores it for method small
    small.close()
