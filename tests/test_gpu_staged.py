"""The bulk-copy staged matvec (opt-in with SGB_PATCH_STAGING=1, read when a
force field is created) against the plain patch kernel: addDForce results
are identical bit for bit (same element arithmetic and gather order), and a
CG step agrees to rounding (the block partials of the dot products are
grouped differently)."""
import numpy as np
import pytest

from sofa_gb300 import topology as topo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    return capi


def _dforce(torch, capi, mesh, dx):
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar", "mixed")
    x = torch.tensor(mesh.positions + 0.01 * np.sin(mesh.positions), dtype=torch.float64, device="cuda")
    f = torch.zeros((mesh.n_nodes, 3), dtype=torch.float32, device="cuda")
    fem.add_force(x.data_ptr(), f.data_ptr())
    d = torch.tensor(dx, dtype=torch.float32, device="cuda")
    df = torch.zeros_like(d)
    fem.add_dforce(d.data_ptr(), df.data_ptr(), -0.5)
    torch.cuda.synchronize()
    assert fem.check_device() == 0
    out = df.cpu().numpy()
    fem.close()
    return out


def test_staged_add_dforce_bit_identical(capi, monkeypatch):
    torch = pytest.importorskip("torch")
    mesh = topo.beam((10, 10, 33), seed=2)
    dx = np.random.default_rng(0).standard_normal((mesh.n_nodes, 3)) * 1e-3
    monkeypatch.setenv("SGB_PATCH_PE", "256")
    monkeypatch.delenv("SGB_PATCH_STAGING", raising=False)
    plain = _dforce(torch, capi, mesh, dx)
    monkeypatch.setenv("SGB_PATCH_STAGING", "1")
    staged = _dforce(torch, capi, mesh, dx)
    assert np.all(np.isfinite(plain)) and np.abs(plain).max() > 0
    np.testing.assert_array_equal(staged, plain)


def test_staged_scene_steps_match(capi, monkeypatch):
    mesh = topo.beam((8, 8, 25), seed=4)

    def run():
        fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar", "mixed")
        sc = capi.Scene(fem, rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=50, cg_tolerance=1e-7,
                        cg_threshold=1e-12, vertex_mass=1.0 / mesh.n_nodes, fixed=mesh.fixed)
        sc.step(20)
        x, _ = sc.state()
        sc.close()
        return x

    monkeypatch.setenv("SGB_PATCH_PE", "256")
    monkeypatch.delenv("SGB_PATCH_STAGING", raising=False)
    plain = run()
    monkeypatch.setenv("SGB_PATCH_STAGING", "1")
    staged = run()
    assert np.linalg.norm(staged - plain) / np.linalg.norm(plain) <= 1e-5
