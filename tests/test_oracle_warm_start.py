"""CGLinearSolver warmStart in the oracle (CGLinearSolver.inl:95-104): each
solve starts from the previous step's solution with r = b - A x. Converged
solves reach the same trajectory as cold starts, in fewer iterations."""
import numpy as np

from tests import cases


def test_warm_start_same_trajectory_fewer_iterations(oracle):
    mesh = cases.beam_mesh(n=(3, 3, 8))
    cfg = dict(cases.BEAM_SMALL, cg_iterations=400, cg_tolerance=1e-12, cg_threshold=1e-30)
    runs = {}
    for warm in (False, True):
        _, sc = cases.oracle_scene(oracle, mesh, "large", cfg=cfg)
        sc.set_warm_start(warm)
        its = 0
        for _ in range(30):
            sc.step(1)
            its += sc.last_iterations
        runs[warm] = (sc.state()[0], its)
    (xc, ic), (xw, iw) = runs[False], runs[True]
    assert np.linalg.norm(xw - xc) <= 1e-8 * np.linalg.norm(xc - mesh.positions)
    assert iw < ic, (iw, ic)
