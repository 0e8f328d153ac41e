"""PCGLinearSolver (+ JacobiPreconditioner) on the GPU against the oracle:
FP64 reference rounding with serial dots bit-identical over 20 steps (with
and without the preconditioner, and with the preconditioner re-assembled
every 3 steps), FP64-FMA within 1e-10, mixed (fused patch kernels) within
1e-4 of the positions; Jacobi cuts the iterations on a stiff inclusion."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

PCG = dict(cases.BEAM_SMALL, cg_iterations=40, cg_tolerance=1e-12)


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


def _oracle(oracle, mesh, method, pre, rate=1, cfg=PCG, young=None):
    _, sc = cases.oracle_scene(oracle, mesh, method, cfg=cfg, young=young)
    sc.set_solver("pcg", pre, rate)
    return sc


@pytest.mark.parametrize("pre,rate", [("jacobi", 1), (None, 1), ("jacobi", 3)])
def test_pcg_fp64_serial_dots_bit_identical(capi, oracle, pre, rate):
    mesh = cases.beam_mesh()
    osc = _oracle(oracle, mesh, "large", pre, rate)
    sc = cases.gpu_scene(capi, mesh, "large", "fp64", cfg=PCG, serial_dots=True, linear_solver="pcg",
                         preconditioner=pre, preconditioner_rate=rate)
    for step in range(20):
        osc.step(1)
        sc.step(1)
        it, _ = sc.sync()
        assert it == osc.last_iterations, step
    x, v = sc.state()
    xo, vo = osc.state()
    assert np.array_equal(x, xo), np.abs(x - xo).max()
    assert np.array_equal(v, vo)


@pytest.mark.parametrize("precision,tol", [("fp64_fma", 1e-10), ("mixed", 1e-4)])
@pytest.mark.parametrize("method", ["large", "polar"])
def test_pcg_jacobi_other_precisions(capi, oracle, precision, tol, method):
    """Tolerance 0, 30 iterations every step: a stopping test sitting on the
    tolerance would otherwise let the rounding of another precision stop one
    iteration earlier or later (a difference of the residual's size)."""
    mesh = cases.beam_mesh()
    cfg = dict(PCG, cg_iterations=30, cg_tolerance=0.0)
    osc = _oracle(oracle, mesh, method, "jacobi", cfg=cfg)
    osc.step(20)
    sc = cases.gpu_scene(capi, mesh, method, precision, cfg=cfg, linear_solver="pcg", preconditioner="jacobi")
    sc.step(20)
    x, _ = sc.state()
    xo, _ = osc.state()
    assert cases.rel_err(x, xo) <= tol
    assert np.linalg.norm(xo - mesh.positions) > 1e-3  # it moved


@pytest.mark.parametrize("pre,rate", [(None, 1), ("jacobi", 3)])
def test_pcg_mixed_patch_kernels(capi, oracle, pre, rate):
    """Mixed precision runs PCG on the fused patch kernels (z = diag^-1 r where
    the direction is formed, r.z in the update); the beam has several patches,
    so shared nodes go through the partial sums."""
    mesh = cases.beam_mesh()
    cfg = dict(PCG, cg_iterations=30, cg_tolerance=0.0)
    osc = _oracle(oracle, mesh, "polar", pre, rate, cfg=cfg)
    osc.step(20)
    sc = cases.gpu_scene(capi, mesh, "polar", "mixed", cfg=cfg, linear_solver="pcg", preconditioner=pre,
                         preconditioner_rate=rate)
    sc.step(20)
    x, _ = sc.state()
    xo, _ = osc.state()
    assert cases.rel_err(x, xo) <= 1e-4
    assert np.linalg.norm(xo - mesh.positions) > 1e-3


def test_pcg_mixed_stops_on_tolerance(capi, oracle):
    """r.z <= tolerance b.b ends the mixed solve early, as in the oracle."""
    mesh = cases.beam_mesh()
    cfg = dict(PCG, cg_iterations=300, cg_tolerance=1e-5)  # the oracle stops after 130-180 iterations
    osc = _oracle(oracle, mesh, "large", "jacobi", cfg=cfg)
    sc = cases.gpu_scene(capi, mesh, "large", "mixed", cfg=cfg, linear_solver="pcg", preconditioner="jacobi")
    for _ in range(5):
        osc.step(1)
        sc.step(1)
        it, _ = sc.sync()
        oi = osc.last_iterations
        assert oi < 300 and abs(it - oi) <= max(3, oi // 20), (it, oi)
    x, _ = sc.state()
    xo, _ = osc.state()
    assert cases.rel_err(x, xo) <= 1e-4


@pytest.mark.parametrize("precision", ["fp64_fma", "mixed"])
def test_pcg_jacobi_fewer_iterations_on_a_stiff_inclusion(capi, precision):
    mesh = cases.beam_mesh(n=(6, 6, 21))
    c = mesh.positions[mesh.tetrahedra].mean(1)
    young = np.where(np.linalg.norm(c - c.mean(0), axis=1) < 1.0, 1e6, 1e3)
    cfg = dict(PCG, cg_iterations=1000, cg_tolerance=1e-16)
    its = {}
    for pre in (None, "jacobi"):
        sc = cases.gpu_scene(capi, mesh, "large", precision, cfg=cfg, young=young, linear_solver="pcg",
                             preconditioner=pre)
        sc.step(1)
        its[pre], _ = sc.sync()
    assert its["jacobi"] < its[None], its


def test_pcg_parameter_errors(capi):
    mesh = cases.beam_mesh(n=(3, 3, 4))
    with pytest.raises(capi.SgbError) as e:
        cases.gpu_scene(capi, mesh, "large", "fp64", preconditioner="jacobi")  # CG with a preconditioner
    assert e.value.code == -1
    with pytest.raises(capi.SgbError) as e:
        fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large", "mixed")
        capi.Scene(fem, linear_solver="pcg", residual_replacement=10)
    assert e.value.code == -4


@pytest.mark.parametrize("precision,tol", [("fp64", 0.0), ("mixed", 1e-4)])
def test_cg_warm_start_against_oracle(capi, oracle, precision, tol):
    """CGLinearSolver warmStart: FP64 reference rounding with serial dots is
    bit-identical to the oracle over 20 steps, iteration counts included;
    mixed is within 1e-4 of the positions."""
    mesh = cases.beam_mesh()
    cfg = dict(cases.BEAM_SMALL, cg_iterations=40, cg_tolerance=1e-8)
    _, osc = cases.oracle_scene(oracle, mesh, "large", cfg=cfg)
    osc.set_warm_start(True)
    sc = cases.gpu_scene(capi, mesh, "large", precision, cfg=cfg, serial_dots=(tol == 0.0), warm_start=True)
    for step in range(20):
        osc.step(1)
        sc.step(1)
        it, _ = sc.sync()
        if tol == 0.0:
            assert it == osc.last_iterations, step
    x, _ = sc.state()
    xo, _ = osc.state()
    if tol == 0.0:
        assert np.array_equal(x, xo), np.abs(x - xo).max()
    else:
        assert cases.rel_err(x, xo) <= tol
