"""EulerImplicitSolver computeResidual on the GPU against the oracle
(EulerImplicitSolver.cpp:314-338; the oracle's restatement is pinned by
tests/test_oracle_residual.py): the Data `residual` after each step and the
trajectory. FP64 reference rounding with serial dots bit-identical (residual,
positions, velocities), with plasticity too, where the residual's extra force
computation advances the plastic strains as the reference's does; FP64-FMA
within 1e-10 and mixed within 1e-4 of the residual. A scene file with
computeResidual="1" reports the same residual."""
import numpy as np
import pytest

from sofa_gb300 import topology as topo
from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


def run_pair(capi, oracle, mesh, method, precision, steps, plastic=False):
    cfg = cases.BEAM_SMALL
    ofem, osc = cases.oracle_scene(oracle, mesh, method)
    if plastic:
        ofem.set_plasticity(1e-3, 1e-7, 0.5)
    osc.set_compute_residual(True)
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, cfg["young"], cfg["poisson"], method, precision)
    if plastic:
        fem.set_plasticity(1e-3, 1e-7, 0.5)
    sc = capi.Scene(fem, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"],
                    cg_iterations=cfg["cg_iterations"], cg_tolerance=cfg["cg_tolerance"],
                    cg_threshold=cfg["cg_threshold"], gravity=cfg["gravity"],
                    vertex_mass=cfg["total_mass"] / mesh.n_nodes, fixed=mesh.fixed,
                    serial_dots=precision == "fp64", compute_residual=True)
    out = []
    for _ in range(steps):
        osc.step(1)
        sc.step(1)
        out.append((osc.residual, sc.residual()))
    x, v = sc.state()
    xr, vr = osc.state()
    sc.close()
    return out, x, v, xr, vr


@pytest.mark.parametrize("method", ["large", "polar"])
def test_fp64_bit_identical(capi, oracle, method):
    mesh = cases.beam_mesh()
    res, x, v, xr, vr = run_pair(capi, oracle, mesh, method, "fp64", 6)
    for r_ref, r in res:
        assert r == r_ref and r > 0.0
    assert np.array_equal(x, xr) and np.array_equal(v, vr)


def test_fp64_with_plasticity_bit_identical(capi, oracle):
    mesh = cases.beam_mesh()
    res, x, v, xr, vr = run_pair(capi, oracle, mesh, "large", "fp64", 6, plastic=True)
    for r_ref, r in res:
        assert r == r_ref
    assert np.array_equal(x, xr) and np.array_equal(v, vr)


@pytest.mark.parametrize("precision,tol", [("fp64_fma", 1e-10), ("mixed", 1e-4)])
def test_fma_and_mixed(capi, oracle, precision, tol):
    mesh = cases.beam_mesh()
    res, _, _, _, _ = run_pair(capi, oracle, mesh, "polar", precision, 4)
    for r_ref, r in res:
        assert abs(r - r_ref) <= tol * r_ref, (r, r_ref)


def test_residual_needs_the_flag(capi):
    mesh = cases.beam_mesh((3, 3, 6))
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large", "fp64")
    sc = capi.Scene(fem, fixed=mesh.fixed)
    sc.step(1)
    with pytest.raises(capi.SgbError) as e:
        sc.residual()
    assert e.value.code == -1
    sc.close()


def test_scene_file_residual(capi, oracle):
    import pathlib

    text = (pathlib.Path(__file__).parent / "scenes" / "grid_fem_4x10x4.scn").read_text()
    assert "<EulerImplicitSolver />" in text
    s = capi.SofaScene(text.replace("<EulerImplicitSolver />", '<EulerImplicitSolver computeResidual="1" />', 1))
    s.animate(10)
    r = s.residual(0)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.set_compute_residual(True)
    osc.step(10)
    assert abs(r - osc.residual) <= 1e-9 * osc.residual
    assert np.max(np.abs(x - osc.state()[0])) <= 1e-10 * np.max(np.abs(osc.state()[0]))
