"""GPU parity of the components' Rayleigh coefficients, EulerImplicitSolver
firstOrder and trapezoidalScheme, and FixedProjectiveConstraint
activate_projectVelocity against
the oracle (tests/test_oracle_options.py pins the oracle's semantics).

Tolerances: FP64 reference rounding with serial dots bit-identical after 20
steps (positions, velocities, CG iterations); FP64-FMA within 1e-10 relative
on the positions; mixed within 1e-4 relative on the positions.
"""
import numpy as np
import pytest

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


OPTIONS = {
    "component_rayleigh": dict(ff_rayleigh_stiffness=0.05, mass_rayleigh_mass=0.03),
    "first_order": dict(first_order=True),
    "project_velocity": dict(project_velocity=True),
    "trapezoidal": dict(trapezoidal_scheme=True),
    "all": dict(ff_rayleigh_stiffness=0.02, mass_rayleigh_mass=0.2, project_velocity=True, trapezoidal_scheme=True),
}


def start_velocity(mesh):
    # non-zero velocities on the fixed nodes too, so that projectVelocity acts
    return np.random.default_rng(8).normal(scale=0.05, size=mesh.positions.shape)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fma", "mixed"])
@pytest.mark.parametrize("option", sorted(OPTIONS))
@pytest.mark.parametrize("method", ["large", "polar"])
def test_options_against_oracle(capi, oracle, precision, option, method):
    mesh = cases.beam_mesh()
    opts = OPTIONS[option]
    v0 = start_velocity(mesh)
    _, osc = cases.oracle_scene(oracle, mesh, method)
    osc.set_options(**opts)
    osc.set_state(mesh.positions, v0)
    osc.step(20)
    xr, vr = osc.state()
    sc = cases.gpu_scene(capi, mesh, method, precision, serial_dots=(precision == "fp64"), **opts)
    sc.set_state(mesh.positions, v0)
    sc.step(20)
    it, _ = sc.sync()
    x, v = sc.state()
    sc.close()
    if precision == "fp64":
        assert np.array_equal(x, xr), cases.rel_err(x, xr)
        assert np.array_equal(v, vr)
        assert it == osc.last_iterations
    elif precision == "fp64_fma":
        assert cases.rel_err(x, xr) <= 1e-10
    else:
        assert cases.rel_err(x, xr) <= 1e-4
    if opts.get("project_velocity"):
        assert np.all(v[mesh.fixed] == 0.0)


def test_options_with_jacobi_pcg(capi, oracle):
    mesh = cases.beam_mesh()
    opts = dict(ff_rayleigh_stiffness=0.05, mass_rayleigh_mass=0.03)
    _, osc = cases.oracle_scene(oracle, mesh, "polar")
    osc.set_options(**opts)
    osc.set_solver("pcg", "jacobi")
    osc.step(10)
    xr, _ = osc.state()
    sc = cases.gpu_scene(capi, mesh, "polar", "fp64", serial_dots=True, linear_solver="pcg",
                         preconditioner="jacobi", **opts)
    sc.step(10)
    x, _ = sc.state()
    assert np.array_equal(x, xr), cases.rel_err(x, xr)


def test_batch_component_rayleigh_matches_scene(capi):
    mesh = cases.beam_mesh()
    kw = dict(young=5000.0, poisson=0.45, method="large", dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1,
              cg_iterations=25, cg_tolerance=1e-9, cg_threshold=1e-9, total_mass=1.0, fixed=mesh.fixed,
              ff_rayleigh_stiffness=0.05, mass_rayleigh_mass=0.03, trapezoidal_scheme=1)
    b = capi.Batch("fp64_fma", budget_bytes=64 << 20, max_meshes=2)
    s = b.add_mesh(mesh.positions, mesh.tetrahedra, **kw)
    b.step(20)
    xb, _ = b.state(s)
    b.close()
    sc = cases.gpu_scene(capi, mesh, "large", "fp64_fma", ff_rayleigh_stiffness=0.05, mass_rayleigh_mass=0.03,
                         trapezoidal_scheme=True)
    sc.step(20)
    x, _ = sc.state()
    assert cases.rel_err(xb, x) <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "fp64_fma", "mixed"])
@pytest.mark.parametrize("method", ["large", "polar"])
def test_separate_gravity_against_oracle(capi, oracle, precision, method):
    """The mass's separateGravity: no weight in the force, v += g dt after the
    position update (the fixed points too). 20 steps against the oracle."""
    mesh = cases.beam_mesh()
    _, osc = cases.oracle_scene(oracle, mesh, method)
    osc.set_separate_gravity(True)
    osc.step(20)
    xr, vr = osc.state()
    sc = cases.gpu_scene(capi, mesh, method, precision, serial_dots=(precision == "fp64"), separate_gravity=True)
    sc.step(20)
    it, _ = sc.sync()
    x, v = sc.state()
    sc.close()
    if precision == "fp64":
        assert np.array_equal(x, xr), cases.rel_err(x, xr)
        assert np.array_equal(v, vr)
        assert it == osc.last_iterations
    elif precision == "fp64_fma":
        assert cases.rel_err(x, xr) <= 1e-10
    else:
        assert cases.rel_err(x, xr) <= 1e-4
    assert np.any(x[mesh.fixed] != mesh.positions[mesh.fixed])  # the reference's drift of the fixed points
