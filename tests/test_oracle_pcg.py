"""PCGLinearSolver with the Jacobi preconditioner in the oracle (CPU):
the inverse diagonal is that of the system operator A = mF M + kF K (probed
with unit vectors through the oracle's own addDForce), fixed DOFs one; a
tightly converged PCG step equals a tightly converged CG step; PCG warm-starts
from the previous step's solution."""
import numpy as np

from sofa_gb300 import topology as topo


def _scene(oracle, mesh, solver, pre, iters=400, tol=1e-30, young=5000.0, method="large"):
    fem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, young, 0.45, method)
    sc = oracle.OracleScene(fem, vertex_mass=1.0 / mesh.n_nodes, fixed=mesh.fixed, dt=0.01,
                            rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=iters, cg_tolerance=tol,
                            cg_threshold=1e-30)
    if solver != "cg":
        sc.set_solver(solver, pre)
    return fem, sc


def test_jacobi_diagonal_is_the_operator_diagonal(oracle):
    mesh = topo.beam((3, 3, 5), spacing=0.5, jitter=0.05, seed=1)
    fem, sc = _scene(oracle, mesh, "pcg", "jacobi", iters=5)
    sc.step(3)  # rotations of a deformed state
    dinv = sc.jacobi()
    h, rs, rm = 0.01, 0.1, 0.1
    mf, kf = 1 + h * rm, -h * (h + rs)
    n = mesh.n_nodes
    diag = np.zeros((n, 3))
    for j in range(n):
        for k in range(3):
            e = np.zeros((n, 3))
            e[j, k] = 1.0
            diag[j, k] = mf / n + fem.add_dforce(e, kf)[j, k]
    free = np.setdiff1d(np.arange(n), mesh.fixed)
    np.testing.assert_allclose(1.0 / dinv[free], diag[free], rtol=1e-12)
    assert np.all(dinv[mesh.fixed] == 1.0)


def test_pcg_jacobi_matches_cg_when_converged(oracle):
    mesh = topo.beam((4, 4, 9), spacing=0.5, jitter=0.05, seed=2)
    _, cg = _scene(oracle, mesh, "cg", None)
    _, pcg = _scene(oracle, mesh, "pcg", "jacobi")
    _, plain = _scene(oracle, mesh, "pcg", None)
    for s in (cg, pcg, plain):
        s.step(5)
    xc, _ = cg.state()
    for s in (pcg, plain):
        x, _ = s.state()
        assert np.linalg.norm(x - xc) / np.linalg.norm(xc - mesh.positions) < 1e-8


def test_pcg_jacobi_fewer_iterations_on_a_stiff_inclusion(oracle):
    """Per-element Young's moduli 1e3 / 1e6: diagonal scaling removes most of
    the contrast, so Jacobi-PCG reaches r.z <= 1e-16 b.b in fewer iterations
    than unpreconditioned PCG."""
    mesh = topo.beam((5, 5, 13), spacing=0.5, jitter=0.05, seed=3)
    c = mesh.positions[mesh.tetrahedra].mean(1)
    young = np.where(np.linalg.norm(c - c.mean(0), axis=1) < 0.6, 1e6, 1e3)
    its = {}
    for pre in (None, "jacobi"):
        _, s = _scene(oracle, mesh, "pcg", pre, iters=2000, tol=1e-16, young=young)
        s.step(1)
        its[pre] = s.last_iterations
    assert its["jacobi"] < its[None], its


def test_pcg_warm_start(oracle):
    """r = b - A x from the previous step's solution: a second solve of the
    same system (state reset) needs no iteration."""
    mesh = topo.beam((3, 3, 5), spacing=0.5, jitter=0.05, seed=4)
    _, s = _scene(oracle, mesh, "pcg", "jacobi", tol=1e-20)
    x0, v0 = s.state()
    s.step(1)
    assert s.last_iterations > 0
    s.set_state(x0, v0)
    s.step(1)
    assert s.last_iterations <= 1
