"""The oracle's exact parallel mode, the checker for meshes too large for one
thread: element terms computed in parallel, then every node adds its terms in
element order. Its addForce, addDForce and whole implicit steps must be
bit-identical to the single-thread oracle (the serial element loop of
TetrahedronFEMForceField::addForce / addDForce, TetrahedronFEMForceField.inl:
1548-1636, and the serial CGLinearSolver of CGLinearSolver.inl:72-315). The
MultiThreading-style mode (thread-local buffers) reorders the sums and is
only close."""
import numpy as np
import pytest

from tests import cases


@pytest.fixture
def threads(oracle):
    yield oracle
    oracle.set_threads(1)


@pytest.mark.parametrize("method", ["small", "large", "polar", "svd"])
def test_exact_parallel_calls_bit_identical(threads, method):
    oracle = threads
    # enough nodes that the vector operations take the threaded path too
    mesh = cases.beam_mesh((26, 26, 70))
    rng = np.random.default_rng(3)
    x = mesh.positions + rng.normal(scale=5e-3, size=mesh.positions.shape)
    dx = rng.normal(scale=1e-3, size=x.shape)
    f0 = rng.normal(size=x.shape)
    out = {}
    for mode in ("serial", "exact", "buffers"):
        oracle.set_threads(1 if mode == "serial" else 7, exact=(mode == "exact"))
        fem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
        out[mode] = (fem.add_force(x, f0), fem.add_dforce(dx, -0.0011, f0))
    for a, b in zip(out["exact"], out["serial"]):
        assert np.array_equal(a, b)
    for a, b in zip(out["buffers"], out["serial"]):
        assert cases.rel_err(a - f0, b - f0) <= 1e-12


@pytest.mark.parametrize("method", ["large", "polar"])
def test_exact_parallel_steps_bit_identical(threads, method):
    oracle = threads
    mesh = cases.beam_mesh((26, 26, 70))
    res = {}
    for mode in ("serial", "exact"):
        oracle.set_threads(1 if mode == "serial" else 5, exact=(mode == "exact"))
        _, sc = cases.oracle_scene(oracle, mesh, method)
        sc.step(3)
        res[mode] = (sc.state(), sc.last_iterations, sc.last_error)
    (xs, vs), its, es = res["serial"]
    (xe, ve), ite, ee = res["exact"]
    assert np.array_equal(xs, xe) and np.array_equal(vs, ve)
    assert its == ite and es == ee
