"""The oracle's component Rayleigh coefficients, EulerImplicitSolver
firstOrder and FixedProjectiveConstraint activate_projectVelocity, pinned by
identities that follow from the reference's formulas:

* kFactorIncludingRayleighDamping = kF + bF rs_ff and
  mFactorIncludingRayleighDamping = mF - bF rm_mass (MechanicalParams.h:
  62-64) enter the system matrix only; the solver's rayleighStiffness /
  rayleighMass enter the matrix and the right-hand side (EulerImplicitSolver.
  cpp:151-171). From rest (v = 0) the right-hand side's damping terms vanish,
  so a first step with the coefficient on the component equals a first step
  with it on the solver (to rounding: the factors are summed in another
  order); the second steps differ.
* firstOrder (EulerImplicitSolver.cpp:137-140, 165-171, 200-224) on one node
  held by a spring of stiffness k: (m + h k) v = -k x, x += h v, so
  x_n = x_0 (m / (m + h k))^n.
* projectVelocity (FixedProjectiveConstraint.inl:237-261) zeroes the fixed
  nodes' velocities after the step; their positions have moved with the
  velocity they had (dv is projected to zero there).
"""
import numpy as np
import pytest

from tests import cases


def scene(oracle, mesh, rs=0.0, rm=0.0, **opts):
    cfg = dict(cases.BEAM_SMALL, rs=rs, rm=rm)
    _, sc = cases.oracle_scene(oracle, mesh, "large", cfg=cfg)
    if opts:
        sc.set_options(**opts)
    return sc


@pytest.mark.parametrize("which", ["stiffness", "mass"])
def test_component_rayleigh_equals_solver_rayleigh_from_rest(oracle, which):
    mesh = cases.beam_mesh()
    c = 0.07
    if which == "stiffness":
        a = scene(oracle, mesh, rs=c)
        b = scene(oracle, mesh, ff_rayleigh_stiffness=c)
    else:
        a = scene(oracle, mesh, rm=c)
        b = scene(oracle, mesh, mass_rayleigh_mass=c)
    a.step(1)
    b.step(1)
    xa, _ = a.state()
    xb, _ = b.state()
    d = np.linalg.norm(xa - mesh.positions)
    assert np.linalg.norm(xa - xb) / d <= 1e-9
    a.step(1)
    b.step(1)
    xa, _ = a.state()
    xb, _ = b.state()
    assert np.linalg.norm(xa - xb) / np.linalg.norm(xa - mesh.positions) > 1e-6


def test_component_rayleigh_zero_is_bit_identical(oracle):
    mesh = cases.beam_mesh()
    a = scene(oracle, mesh, rs=0.1, rm=0.1)
    b = scene(oracle, mesh, rs=0.1, rm=0.1, ff_rayleigh_stiffness=0.0, mass_rayleigh_mass=0.0)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.state()[0], b.state()[0])


def test_first_order_spring_closed_form(oracle):
    m, k, h, x0 = 0.5, 40.0, 0.01, 0.3
    sc = oracle.OracleScene(None, n_nodes=1, vertex_mass=m, gravity=(0.0, 0.0, 0.0), dt=h, cg_iterations=10,
                            cg_tolerance=1e-30, cg_threshold=1e-30)
    sc.set_springs(k, np.zeros((1, 3)))
    sc.set_state(np.array([[x0, -x0, 2 * x0]]), np.zeros((1, 3)))
    sc.set_options(first_order=True)
    n = 7
    sc.step(n)
    x, v = sc.state()
    g = m / (m + h * k)
    np.testing.assert_allclose(x[0], np.array([x0, -x0, 2 * x0]) * g ** n, rtol=1e-13)
    np.testing.assert_allclose(v[0], -k * x[0] / (m + h * k) / g, rtol=1e-12)


def test_project_velocity_zeroes_fixed_nodes(oracle):
    mesh = cases.beam_mesh()
    rng = np.random.default_rng(4)
    v0 = rng.normal(scale=0.1, size=mesh.positions.shape)
    res = {}
    for pv in (False, True):
        sc = scene(oracle, mesh, rs=0.1, rm=0.1, project_velocity=pv)
        sc.set_state(mesh.positions, v0)
        sc.step(1)
        res[pv] = sc.state()
    fx = mesh.fixed
    x_off, v_off = res[False]
    x_on, v_on = res[True]
    assert np.array_equal(x_on, x_off)  # positions move with the unprojected velocity
    assert np.all(v_on[fx] == 0.0) and np.any(v_off[fx] != 0.0)
    free = np.setdiff1d(np.arange(mesh.n_nodes), fx)
    assert np.array_equal(v_on[free], v_off[free])
    np.testing.assert_allclose(x_on[fx], mesh.positions[fx] + 0.01 * v0[fx], rtol=0, atol=1e-15)


def test_trapezoidal_spring_recurrence(oracle):
    """trapezoidalScheme (EulerImplicitSolver.cpp:117-171): tr = 0.5 on h in
    the right-hand side's stiffness factor and the system factors. One node
    of mass m held by a spring k: (m + (tr h)^2 k) dv = h (-k x - tr h k v),
    v += dv, x += h v."""
    m, k, h, tr = 0.5, 40.0, 0.01, 0.5
    x = np.array([0.3, -0.3, 0.6])
    v = np.array([0.1, 0.0, -0.2])
    sc = oracle.OracleScene(None, n_nodes=1, vertex_mass=m, gravity=(0.0, 0.0, 0.0), dt=h, cg_iterations=10,
                            cg_tolerance=1e-30, cg_threshold=1e-30)
    sc.set_springs(k, np.zeros((1, 3)))
    sc.set_state(x[None], v[None])
    sc.set_options(trapezoidal_scheme=True)
    for _ in range(6):
        dv = h * (-k * x - tr * h * k * v) / (m + (tr * h) ** 2 * k)
        v = v + dv
        x = x + h * v
    sc.step(6)
    xo, vo = sc.state()
    np.testing.assert_allclose(xo[0], x, rtol=1e-12)
    np.testing.assert_allclose(vo[0], v, rtol=1e-12)


def test_separate_gravity_free_particle(oracle):
    """separateGravity (UniformMass.inl:450-475, EulerImplicitSolver.cpp:296):
    the mass adds no weight; after the position update v += g dt. A free
    particle then lags the plain scheme by one step: x_{n+1} = x_n + h v_n,
    v_{n+1} = v_n + g h, bit for bit."""
    m, h = 0.5, 0.01
    g = np.array([0.0, -9.81, 1.5])
    sc = oracle.OracleScene(None, n_nodes=1, vertex_mass=m, gravity=tuple(g), dt=h, cg_iterations=10,
                            cg_tolerance=1e-30, cg_threshold=1e-30)
    sc.set_separate_gravity(True)
    x = np.array([0.3, 1.0, -2.0])
    v = np.array([0.2, 0.0, 0.1])
    sc.set_state(x[None, :], v[None, :])
    sc.step(6)
    hg = [float(g[k]) * h for k in range(3)]
    xs, vs = [float(c) for c in x], [float(c) for c in v]
    for _ in range(6):
        for k in range(3):
            vv = vs[k] + 0.0  # the solve gives dv = 0: no force
            xs[k] = xs[k] + vv * h
            vs[k] = vv + hg[k]
    xo, vo = sc.state()
    assert np.array_equal(xo[0], np.array(xs)) and np.array_equal(vo[0], np.array(vs))


def test_separate_gravity_fixed_points_drift(oracle):
    """With separateGravity every point's velocity takes g dt, the fixed
    points' too (addGravityToV has no projection), so without
    activate_projectVelocity they move from the second step on, as in the
    reference; with it they stay."""
    mesh = cases.beam_mesh()
    res = {}
    for pv in (False, True):
        sc = scene(oracle, mesh, rs=0.1, rm=0.1, project_velocity=pv)
        sc.set_separate_gravity(True)
        sc.step(3)
        res[pv] = sc.state()[0]
    fx = mesh.fixed
    assert np.any(res[False][fx] != mesh.positions[fx])
    assert np.array_equal(res[True][fx], mesh.positions[fx])
