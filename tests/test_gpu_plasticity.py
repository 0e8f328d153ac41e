"""Plasticity (plasticMaxThreshold > 0, TetrahedronFEMForceField.inl:357-370)
on the GPU against the oracle, through the C ABI.

Tolerances: fp64 (reference rounding) forces and plastic strain
bit-identical per call, and a whole scene with serial dots bit-identical;
fp64_fma within 1e-10 and mixed within 1e-5 of the largest force / plastic
strain per call; mixed scene positions within 1e-4 relative."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

METHODS = ["small", "large", "polar", "svd"]


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


def _deformed(mesh, amp, seed):
    rng = np.random.default_rng(seed)
    x = mesh.positions.copy()
    z = x[:, 2] / x[:, 2].max()
    x[:, 1] += amp * 4.0 * z * z
    x += rng.uniform(-amp, amp, x.shape) * 0.2
    return x


def _settings(oracle, mesh, method, x, creep=0.5):
    """Yield at the 30th and clamp at the 80th percentile of the elements'
    strain norms at x, so that both tests of the update take both branches."""
    probe = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    probe.set_plasticity(1e9, 0.0, 1.0)
    probe.add_force(x)
    norms = np.linalg.norm(probe.plastic_strain(), axis=1)
    return float(np.percentile(norms, 80)), float(np.percentile(norms, 30)), creep


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("precision,tol", [("fp64", 0.0), ("fp64_fma", 1e-10), ("mixed", 1e-5)])
def test_add_force_with_plasticity_per_call(torch_cuda, capi, oracle, method, precision, tol):
    torch = torch_cuda
    mesh = cases.beam_mesh(n=(4, 4, 9))
    xs = [_deformed(mesh, 0.05, 1), _deformed(mesh, 0.1, 2), _deformed(mesh, 0.1, 2), mesh.positions]
    pl = _settings(oracle, mesh, method, xs[1])
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    ofem.set_plasticity(*pl)
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method, precision)
    fem.set_plasticity(*pl)
    dt = torch.float32 if precision == "mixed" else torch.float64
    for k, x in enumerate(xs):
        f_ref = ofem.add_force(x)
        xd = torch.tensor(x, dtype=torch.float64, device="cuda")
        fd = torch.zeros(x.shape, dtype=dt, device="cuda")
        fem.add_force(xd.data_ptr(), fd.data_ptr())
        torch.cuda.synchronize()
        f = fd.cpu().double().numpy()
        ps, ps_ref = fem.plastic_strain(), ofem.plastic_strain()
        if tol == 0.0:
            assert np.array_equal(f, f_ref), (k, np.abs(f - f_ref).max())
            assert np.array_equal(ps, ps_ref), (k, np.abs(ps - ps_ref).max())
        else:
            assert np.abs(f - f_ref).max() <= tol * np.abs(f_ref).max(), k
            assert np.abs(ps - ps_ref).max() <= tol * np.abs(ps_ref).max(), k
    assert np.abs(ofem.plastic_strain()).max() > 0
    fem.reset_plasticity()
    assert not fem.plastic_strain().any()
    fem.close()


def _scene_settings(oracle, mesh, method, steps=20):
    _, sc = cases.oracle_scene(oracle, mesh, method)
    sc.step(steps)
    x, _ = sc.state()
    return _settings(oracle, mesh, method, x, creep=0.3)


def test_scene_with_plasticity_bit_identical_with_serial_dots(torch_cuda, capi, oracle):
    mesh = cases.beam_mesh()
    pl = _scene_settings(oracle, mesh, "large")
    ofem, osc = cases.oracle_scene(oracle, mesh, "large")
    ofem.set_plasticity(*pl)
    sc = cases.gpu_scene(capi, mesh, "large", "fp64", serial_dots=True)
    sc.fem.set_plasticity(*pl)
    for step in range(30):
        osc.step(1)
        sc.step(1)
        it, _ = sc.sync()
        assert it == osc.last_iterations, step
    x, v = sc.state()
    xo, vo = osc.state()
    assert np.array_equal(x, xo), np.abs(x - xo).max()
    assert np.array_equal(v, vo)
    assert np.array_equal(sc.fem.plastic_strain(), ofem.plastic_strain())
    assert np.abs(ofem.plastic_strain()).max() > 0


def test_plasticity_turned_on_between_steps(torch_cuda, capi, oracle):
    """The step is recorded once and replayed; changing the plasticity
    settings between steps records it again."""
    mesh = cases.beam_mesh()
    pl = _scene_settings(oracle, mesh, "polar")
    ofem, osc = cases.oracle_scene(oracle, mesh, "polar")
    sc = cases.gpu_scene(capi, mesh, "polar", "fp64", serial_dots=True)
    osc.step(10)
    sc.step(10)
    ofem.set_plasticity(*pl)
    sc.fem.set_plasticity(*pl)
    osc.step(10)
    sc.step(10)
    ofem.set_plasticity(0.0, pl[1], pl[2])
    sc.fem.set_plasticity(0.0, pl[1], pl[2])
    osc.step(5)
    sc.step(5)
    x, _ = sc.state()
    xo, _ = osc.state()
    assert np.array_equal(x, xo), np.abs(x - xo).max()
    assert np.array_equal(sc.fem.plastic_strain(), ofem.plastic_strain())


@pytest.mark.parametrize("method", ["large", "polar"])
def test_mixed_scene_with_plasticity(torch_cuda, capi, oracle, method):
    mesh = cases.beam_mesh()
    pl = _scene_settings(oracle, mesh, method)
    ofem, osc = cases.oracle_scene(oracle, mesh, method)
    ofem.set_plasticity(*pl)
    osc.step(30)
    sc = cases.gpu_scene(capi, mesh, method, "mixed")
    sc.fem.set_plasticity(*pl)
    sc.step(30)
    x, _ = sc.state()
    xo, _ = osc.state()
    assert cases.rel_err(x, xo) <= 1e-4
    # the mixed run follows the plastic motion, not the elastic one: its
    # distance to the plastic oracle run is a small part of the elastic
    # run's distance to it
    _, el = cases.oracle_scene(oracle, mesh, method)
    el.step(30)
    xe, _ = el.state()
    assert np.linalg.norm(x - xo) < 0.25 * np.linalg.norm(xe - xo)


def test_plasticity_with_residual_replacement_is_refused(torch_cuda, capi):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large", "mixed")
    fem.set_plasticity(0.01, 0.001, 0.5)
    sc = capi.Scene(fem, residual_replacement=10, fixed=mesh.fixed, vertex_mass=1.0 / mesh.n_nodes)
    with pytest.raises(capi.SgbError) as e:
        sc.step(1)
    assert e.value.code == -4
