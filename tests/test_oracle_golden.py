"""Pins the CPU oracle to the reference's own known answers.

Each test replays a reference test (file:line given in its docstring) or
compares against outputs of the reference's own code compiled from its
sources (tests/golden/polar_ref.npz, made by tests/golden/make_polar_golden.py).
"""
import os

import numpy as np
import pytest

from sofa_gb300 import topology as topo
from tests import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_single_tet_large_known_answer(oracle):
    """BaseTetrahedronFEMForceField_test.h:89-114,290-372 (checkInit):
    one tet, E=1000, nu=0.3, method=large, tetra '2 3 1 0'; R0, rotated rest
    coordinates, 6x6 K and 12x6 J to 1e-4."""
    rest = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    fem = oracle.OracleFEM(rest, [[2, 3, 1, 0]], 1000.0, 0.3, "large")
    el = fem.element(0)
    exp_rot = np.array([[0, 0.816497, 0.57735], [-0.707107, -0.408248, 0.57735], [0.707107, -0.408248, 0.57735]])
    exp_pos = np.array([[0, 0, 0], [1.41421, 0, 0], [0.707107, 1.22474, 0], [0.707107, 0.408248, -0.57735]])
    exp_K = np.array([[224.359, 96.1538, 96.1538, 0, 0, 0], [96.1538, 224.359, 96.1538, 0, 0, 0],
                      [96.1538, 96.1538, 224.359, 0, 0, 0], [0, 0, 0, 64.1026, 0, 0], [0, 0, 0, 0, 64.1026, 0],
                      [0, 0, 0, 0, 0, 64.1026]])
    exp_J = np.array([
        [0.707107, 0, 0, 0.408248, 0, -0.57735], [0, 0.408248, 0, 0.707107, -0.57735, 0],
        [0, 0, -0.57735, 0, 0.408248, 0.707107], [-0.707107, 0, 0, 0.408248, 0, -0.57735],
        [0, 0.408248, 0, -0.707107, -0.57735, 0], [0, 0, -0.57735, 0, 0.408248, -0.707107],
        [0, 0, 0, -0.816497, 0, -0.57735], [0, -0.816497, 0, 0, -0.57735, 0],
        [0, 0, -0.57735, 0, -0.816497, 0], [0, 0, 0, 0, 0, 1.73205], [0, 0, 0, 0, 1.73205, 0],
        [0, 0, 1.73205, 0, 0, 0]])
    np.testing.assert_allclose(el["initial_rotation"], exp_rot, atol=1e-4)
    np.testing.assert_allclose(el["rotation"], exp_rot, atol=1e-4)
    np.testing.assert_allclose(el["rotated_rest"], exp_pos, atol=1e-4)
    np.testing.assert_allclose(oracle.full_K(el["K3"]), exp_K, atol=1e-4)
    np.testing.assert_allclose(oracle.full_J(el["J3"]), exp_J, atol=1e-4)


def _grid_scene(oracle):
    """createGridFEMScene (BaseTetrahedronFEMForceField_test.h:117-177)."""
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    # DiagonalMass massDensity=1 with tetrahedron lumping (DiagonalMass.inl:332-376)
    vol = np.abs(topo.signed_volumes(tets, pos))
    masses = np.zeros(len(pos))
    for t, v in zip(tets, vol):
        m = (1.0 * v) / 4.0
        for i in t:
            masses[i] += m
    fixed = topo.box_roi(pos, (-1, -1, 0, 10, 1, 50))
    scene = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01,
                               cg_iterations=20, cg_tolerance=1e-5, cg_threshold=1e-6)
    return pos, tets, fem, scene


def test_grid_100_steps_known_answer(oracle):
    """checkFEMValues (BaseTetrahedronFEMForceField_test.h:379-431): grid
    4x10x4, Hexa2Tetra split, 100 implicit steps; x[159] and element 100's
    rotations, rotated rest coordinates, K and J to 1e-4."""
    pos, tets, fem, scene = _grid_scene(oracle)
    assert len(pos) == 160 and len(tets) == 486
    np.testing.assert_allclose(pos[159], [10, 40, 30], atol=1e-4)
    scene.step(100)
    x, _ = scene.state()
    np.testing.assert_allclose(x[159], [9.99985, 45.0487, 30.0011], atol=1e-4)
    el = fem.element(100)
    np.testing.assert_allclose(el["initial_rotation"], [[-1, 0, 0], [0, -0.8, -0.6], [0, -0.6, 0.8]], atol=1e-4)
    np.testing.assert_allclose(el["rotated_rest"], [[0, 0, 0], [3.33333, 0, 0], [3.33333, 5.55556, 0],
                                                    [0, 3.55556, 2.66667]], atol=1e-4)
    np.testing.assert_allclose(el["rotation"], [[-1, 8.01488e-06, 0.000541687],
                                                [-0.000320764, -0.814541, -0.580106],
                                                [0.000436576, -0.580106, 0.814541]], atol=1e-4)
    K = oracle.full_K(el["K3"])
    np.testing.assert_allclose(K[0, :3], [2.72596, 1.16827, 1.16827], atol=1e-4)
    np.testing.assert_allclose(K[3, 3], 0.778846, atol=1e-4)
    J = oracle.full_J(el["J3"])
    exp_J = np.array([
        [-14.8148, 0, 0, 1.18424e-14, 0, -18.5185], [0, 1.18424e-14, 0, -14.8148, -18.5185, 0],
        [0, 0, -18.5185, 0, 1.18424e-14, -14.8148], [14.8148, 0, 0, -8.88889, 0, 11.8519],
        [0, -8.88889, 0, 14.8148, 11.8519, 0], [0, 0, 11.8519, 0, -8.88889, 14.8148],
        [0, 0, 0, 8.88889, 0, -11.8519], [0, 8.88889, 0, 0, -11.8519, 0], [0, 0, -11.8519, 0, 8.88889, 0],
        [0, 0, 0, -1.18424e-14, 0, 18.5185], [0, -1.18424e-14, 0, 0, 18.5185, 0],
        [0, 0, 18.5185, 0, -1.18424e-14, 0]])
    np.testing.assert_allclose(J, exp_J, atol=1e-4)
    # the reference's own rounding residue in J(0,3) is reproduced to the digit
    assert abs(J[0, 3] - 1.18424e-14) < 1e-18


def test_small_regular_tet_forces(oracle):
    """TetrahedronFEMForceField_stepTest.cpp:58-75 with
    scenes/TetrahedronFEMForceFieldRegularTetra.scn: method=small, E=40,
    nu=0; stretching the apex from z=1 to z=2 gives -sqrt(3)*10/3 on the apex
    and +sqrt(3)*10/9 on each base node (ForceField_test compares f)."""
    rest = np.array([[0, 0, 0], [1, 0, 0], [0.5, 0.86602540378443864676, 0], [0.5, 0.288675134594812882254, 1]])
    x = rest.copy()
    x[2] = [0.5, 0.8660254037, 0]
    x[3] = [0.5, 0.28867513, 2]
    fem = oracle.OracleFEM(rest, [[0, 1, 2, 3]], 40.0, 0.0, "small")
    f = fem.add_force(x)
    fdown = np.sqrt(3.0) * 10.0 / 9.0
    fup = np.sqrt(3.0) * 10.0 / 3.0
    np.testing.assert_allclose(f[:3, 2], [fdown] * 3, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(f[3, 2], -fup, rtol=1e-6)
    np.testing.assert_allclose(f[:, :2], 0, atol=1e-6)


@pytest.mark.parametrize("method", ["small", "large", "polar", "svd"])
def test_dforce_is_derivative_of_force(oracle, method):
    """ForceField_test protocol (SolidMechanics/Testing/.../ForceFieldTestCreation.h,
    run_test): addDForce(dx) matches the finite difference of addForce under a
    seeded random perturbation. For the corotational methods the stiffness of
    the reference is the corotated one (rotation held), so the check is the
    linear one at a configuration near rest."""
    rng = np.random.default_rng(7)
    mesh = topo.beam((3, 3, 4), spacing=0.5, jitter=0.05, seed=3)
    fem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    x0 = mesh.positions + rng.uniform(-1e-3, 1e-3, mesh.positions.shape)
    f0 = fem.add_force(x0)
    dx = rng.uniform(-1e-6, 1e-6, mesh.positions.shape)
    f1 = fem.add_force(x0 + dx)
    fem.add_force(x0)  # rotations at x0 for addDForce
    df = fem.add_dforce(dx, 1.0)
    fd = f1 - f0
    # kFactor=1 gives -K dx; the force change is -K dx too
    rel = np.linalg.norm(df - fd) / np.linalg.norm(fd)
    assert rel < 1e-2, rel


def test_polar_matches_reference_bits(oracle):
    """The oracle's polar decomposition restatement equals the reference's
    Decompose<double>::polarDecomposition bit for bit on 550 matrices
    (tests/golden/polar_ref.npz)."""
    g = np.load(os.path.join(GOLDEN, "polar_ref.npz"))
    for M, Q, det in zip(g["M"], g["Q"], g["det"]):
        q, d = oracle.polar(M)
        assert np.array_equal(q, Q), (M, q, Q)
        assert d == det


def test_polar_stable_matches_reference_bits(oracle):
    """The oracle's restatement of Decompose<double>::polarDecomposition_stable
    (SVD_stable, eigenDecomposition_iterative, QLAlgorithm), used by the svd
    method for inverted or flat elements, equals the reference's bit for bit
    on 600 matrices covering each degenerate branch
    (tests/golden/polar_stable_ref.npz)."""
    g = np.load(os.path.join(GOLDEN, "polar_stable_ref.npz"))
    for M, Q, deg in zip(g["M"], g["Q"], g["degenerate"]):
        q, d = oracle.polar_stable(M)
        assert np.array_equal(q, Q), (M, q, Q)
        assert d == bool(deg)


def test_svd_method_equals_polar_unless_inverted(oracle):
    """accumulateForceSVD (TFEM.inl:1123-1184) takes the polar factor of the
    edge matrix when det(A A0^-1) >= 1e-6, so on a mesh with no inverted or
    flattened element the svd force equals the polar force bit for bit; an
    inverted element takes the stable SVD factor instead."""
    mesh = cases.beam_mesh()
    rng = np.random.default_rng(3)
    x = mesh.positions + rng.normal(scale=1e-2, size=mesh.positions.shape)
    fp = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar").add_force(x)
    fs = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "svd").add_force(x)
    assert np.array_equal(fp, fs)
    # invert element 0: move its node a through the opposite face
    t = mesh.tetrahedra[0]
    xi = x.copy()
    c = x[t[1:]].mean(0)
    xi[t[0]] = c + 1.5 * (c - x[t[0]])
    fp = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar").add_force(xi)
    fs = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "svd").add_force(xi)
    assert np.all(np.isfinite(fs)) and not np.array_equal(fp, fs)
    others = np.setdiff1d(np.arange(mesh.n_nodes), np.unique(mesh.tetrahedra[
        np.any(np.isin(mesh.tetrahedra, t), axis=1)]))
    assert np.array_equal(fp[others], fs[others])


def test_euler_implicit_closed_form(oracle):
    """EulerImplicitSolverDynamic_test.cpp:58-76,150-161: a mass on a linear
    spring under gravity follows the discrete implicit-Euler recurrence with
    Rayleigh damping; replayed on a single node with CG 3000/1e-12/1e-12 as in
    ODESolverSpringTest.h:55-80."""
    for (h, K, m, rm, rk) in [(0.1, 100.0, 10.0, 0.0, 0.0), (0.1, 100.0, 10.0, 0.1, 0.1)]:
        z0, g = 1.0, 10.0
        scene = oracle.OracleScene(None, n_nodes=1, vertex_mass=m, gravity=(0, -g, 0), dt=h,
                                   rayleigh_stiffness=rk, rayleigh_mass=rm, cg_iterations=3000,
                                   cg_tolerance=1e-12, cg_threshold=1e-12)
        scene.set_state(np.array([[0.0, z0, 0.0]]), np.zeros((1, 3)))
        scene.set_springs(K, np.array([[0.0, z0, 0.0]]))
        den = h * (h + rk) * K + (1 + h * rm) * m
        const = -(rk + h) * K - rm * m
        xs, vs = [z0], [0.0]
        for i in range(1, 21):
            vs.append(vs[i - 1] + h * (-K * (xs[i - 1] - z0) - m * g + vs[i - 1] * const) / den)
            xs.append(xs[i - 1] + h * vs[i])
        for i in range(20):
            x, _ = scene.state()
            assert abs(x[0, 1] - xs[i]) <= 5e-16, (i, x[0, 1], xs[i])
            scene.step(1)


def test_uniform_mass_rules(oracle):
    """UniformMass_test.cpp:473-530 / UniformMass.inl:337: vertexMass =
    totalMass / N and f += m g for every node."""
    n = 7
    scene = oracle.OracleScene(None, n_nodes=n, vertex_mass=1.0 / n, gravity=(0, -9.81, 0))
    f = scene.compute_force()
    np.testing.assert_array_equal(f[:, 1], np.full(n, -9.81 * (1.0 / n)))
    assert np.all(f[:, [0, 2]] == 0)


def test_fixed_constraint_constant_force_known_answer(oracle):
    """FixedProjectiveConstraint_test.cpp testTopologicalChanges (before the
    topology change): 5 points at x_i = i + 0.1 k, UniformMass totalMass 1, a
    constant force (10, 10, 10) on every point, points 0-2 fixed,
    EulerImplicitSolver rayleighStiffness 0.01 / rayleighMass 1.0 with CG
    25 / 1e-5 / 1e-5 (SceneCreator createEulerSolverNode), two steps of 0.1:
    x[3][0] = 4.32231, x[4][0] = 5.32231, fixed points unchanged."""
    x0 = np.array([[i + 0.1 * k for k in range(3)] for i in range(5)])
    sc = oracle.OracleScene(None, n_nodes=5, vertex_mass=1.0 / 5, gravity=(0.0, 0.0, 0.0), fixed=[0, 1, 2],
                            dt=0.1, rayleigh_stiffness=0.01, rayleigh_mass=1.0, cg_iterations=25,
                            cg_tolerance=1e-5, cg_threshold=1e-5)
    sc.set_state(x0, np.zeros_like(x0))
    sc.set_external_force(np.full((5, 3), 10.0))
    sc.step(2)
    x, _ = sc.state()
    assert np.array_equal(x[:3], x0[:3])
    np.testing.assert_allclose([x[3, 0], x[4, 0]], [4.32231, 5.32231], atol=1e-4)
