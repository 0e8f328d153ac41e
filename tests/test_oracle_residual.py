"""The oracle's EulerImplicitSolver computeResidual (EulerImplicitSolver.cpp:
48-49, 314-338): after the step r = 0; r += M (v_new - v_old) with v_new and
v_old the same vector in the animation loop's call (so zero); r += f (-dt)
with f the scene's force at the new state; r projected; residual = r.r
(MechanicalObject::vDot, serial). Checked bit for bit against that formula
evaluated here on the oracle's own force at the new state, and: the residual
does not change the trajectory unless the force field keeps state (plastic
strains), where the extra force computation advances it as the reference's
does."""
import numpy as np

from tests import cases


def residual_formula(f, fixed, dt):
    total = 0.0
    fixed = set(int(i) for i in fixed)
    for n in range(f.shape[0]):
        if n in fixed:
            continue
        r = [float(f[n, k]) * (-dt) for k in range(3)]
        d = r[0] * r[0]
        d += r[1] * r[1]
        d += r[2] * r[2]
        total += d
    return total


def test_residual_is_the_reference_formula(oracle):
    mesh = cases.beam_mesh((4, 4, 9))
    _, osc = cases.oracle_scene(oracle, mesh, "polar")
    osc.set_compute_residual(True)
    osc.step(3)
    res = osc.residual
    f = osc.compute_force()  # the force at the new state, as the residual used it
    assert res == residual_formula(f, mesh.fixed, cases.BEAM_SMALL["dt"])
    assert res > 0.0


def test_residual_leaves_a_stateless_trajectory_alone(oracle):
    mesh = cases.beam_mesh((4, 4, 9))
    _, a = cases.oracle_scene(oracle, mesh, "large")
    _, b = cases.oracle_scene(oracle, mesh, "large")
    b.set_compute_residual(True)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.state()[0], b.state()[0])


def test_residual_advances_plastic_strain_like_the_reference(oracle):
    mesh = cases.beam_mesh((4, 4, 9))
    fa, a = cases.oracle_scene(oracle, mesh, "large")
    fb, b = cases.oracle_scene(oracle, mesh, "large")
    for fem in (fa, fb):
        fem.set_plasticity(1e-3, 1e-7, 0.5)
    b.set_compute_residual(True)
    a.step(5)
    b.step(5)
    assert not np.array_equal(a.state()[0], b.state()[0])
