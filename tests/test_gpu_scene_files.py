"""Scene files on the GPU: the known-answer grid scene run through the
component layer reproduces the reference's checkFEMValues position and the
oracle's trajectory; a mixed-precision scene file runs and stays within the
position tolerance of its FP64 run."""
import os

import numpy as np
import pytest

from sofa_gb300 import topology as topo

pytestmark = pytest.mark.gpu

SCENES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scenes")


def _read(name):
    with open(os.path.join(SCENES, name)) as f:
        return f.read()


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    return capi


def test_grid_scene_file_known_answer(capi, oracle):
    """checkFEMValues (BaseTetrahedronFEMForceField_test.h:379-431) through
    the scene file: x[159] after 100 steps, and the whole trajectory against
    the oracle run of the same scene."""
    s = capi.SofaScene(_read("grid_fem_4x10x4.scn"))
    s.animate(100)
    x = s.positions(0)
    assert s.time == pytest.approx(1.0)
    np.testing.assert_allclose(x[159], [9.99985, 45.0487, 30.0011], atol=1e-4)

    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.step(100)
    xo, _ = osc.state()
    # parallel (non-serial) dot products: not bit-identical, within 1e-10 of the positions
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))


def test_mixed_scene_file_against_its_fp64_run(capi):
    mixed = capi.SofaScene(_read("beam_polar_gpu.scn"))
    fp64 = capi.SofaScene(_read("beam_polar_gpu.scn"), precision=2)
    assert mixed.body_info(0)["precision"] == 1
    mixed.animate(50)
    fp64.animate(50)
    xm, xd = mixed.positions(0), fp64.positions(0)
    assert np.all(np.isfinite(xm))
    rest = topo.regular_grid((12, 4, 4), (0, 0, 0), (6, 1.5, 1.5))[0]
    assert np.linalg.norm(xd - rest) > 1e-3  # it moved
    # a soft beam (E=3000) bending by a quarter of its length under 25
    # unconverged CG iterations: the FP32 and FP64 Krylov sequences part by
    # 1.6e-4 of the positions after 50 steps (measured on a GB300)
    assert np.linalg.norm(xm - xd) / np.linalg.norm(xd) <= 5e-4


def _records(path):
    """WriteState file -> [(t, {tag: values})]."""
    recs = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line.startswith("T="):
                recs.append((float(line.split()[1]), {}))
            elif line:
                tag, _, vals = line.partition("=")
                recs[-1][1][tag] = np.array([float(v) for v in vals.split()]).reshape(-1, 3)
    return recs


def test_write_state_records(capi, tmp_path):
    """WriteState (WriteState.inl:240-380): without time/period it writes at
    the beginning of every step from t = 0; with time="0.02" period="0.03"
    it writes at 0.02, 0.05, 0.08. X0 is the rest position, X the state at
    the record's time, in default stream formatting (6 significant digits)."""
    text = _read("grid_fem_4x10x4.scn")
    every = str(tmp_path / "every.txt")
    timed = str(tmp_path / "timed.txt")
    ws = (f'<WriteState filename="{every}" writeX0="1" writeV="1" />\n'
          f'        <WriteState name="w2" filename="{timed}" time="0.02" period="0.03" />\n'
          '        <TetrahedronFEMForceField')
    s = capi.SofaScene(text.replace("<TetrahedronFEMForceField", ws, 1))
    s.animate(10)
    ref = capi.SofaScene(text)
    ref.animate(9)
    rec = _records(every)
    assert [t for t, _ in rec] == pytest.approx([0.01 * k for k in range(10)])
    rest = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))[0]
    np.testing.assert_allclose(rec[0][1]["X0"], rest, rtol=1e-5)
    np.testing.assert_allclose(rec[0][1]["X"], rest, rtol=1e-5)
    assert np.abs(rec[0][1]["V"]).max() == 0.0
    np.testing.assert_allclose(rec[-1][1]["X"], ref.positions(0), rtol=1e-5, atol=1e-6)
    rec2 = _records(timed)
    assert [t for t, _ in rec2] == pytest.approx([0.02, 0.05, 0.08])
    assert set(rec2[0][1]) == {"X"}


def test_pcg_jacobi_scene_file_against_oracle(capi, oracle):
    """The known-answer grid scene with PCGLinearSolver + JacobiPreconditioner
    (assembled every 4 steps) instead of CG: 30 steps against the oracle's PCG
    on the same inputs (30 iterations every step, tolerance 0: no stopping
    test that dot-product rounding could move)."""
    text = _read("grid_fem_4x10x4.scn").replace(
        '<CGLinearSolver iterations="20" tolerance="1e-5" threshold="1e-6" />',
        '<PreconditionedMatrixFreeSystem assemblingRate="4"/>\n'
        '        <PCGLinearSolver iterations="30" tolerance="0" preconditioner="@precond"/>\n'
        '        <JacobiPreconditioner name="precond"/>')
    s = capi.SofaScene(text)
    s.animate(30)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=30,
                             cg_tolerance=0.0, cg_threshold=1e-6)
    osc.set_solver("pcg", "jacobi", 4)
    osc.step(30)
    xo, _ = osc.state()
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
    assert np.max(np.abs(xo - pos)) > 1e-3


def test_plasticity_scene_file_against_oracle(capi, oracle):
    """The known-answer grid scene with the plasticity settings of the
    reference's TetrahedronFEMForceField_plasticity.scn (yield 0.005, maximum
    0.025, creep 1): 50 steps against the oracle with the same settings."""
    text = _read("grid_fem_4x10x4.scn").replace(
        '<TetrahedronFEMForceField name="FEM"',
        '<TetrahedronFEMForceField plasticYieldThreshold="0.005" plasticMaxThreshold="0.025" plasticCreep="1" '
        'name="FEM"')
    s = capi.SofaScene(text)
    s.animate(50)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    runs = []
    for plastic in (True, False):
        fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
        if plastic:
            fem.set_plasticity(0.025, 0.005, 1.0)
        osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01,
                                 cg_iterations=20, cg_tolerance=1e-5, cg_threshold=1e-6)
        osc.step(50)
        runs.append(osc.state()[0])
        if plastic:
            assert np.abs(fem.plastic_strain()).max() > 0
    xo, xe = runs
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
    assert np.max(np.abs(xe - xo)) > 1e-3 * np.max(np.abs(xo - pos))  # plasticity changed the motion


def test_cg_warm_start_scene_file_against_oracle(capi, oracle):
    """The known-answer grid scene with CGLinearSolver warmStart="1": 30 steps
    against the oracle with warm starts."""
    text = _read("grid_fem_4x10x4.scn").replace(
        '<CGLinearSolver iterations="20" tolerance="1e-5" threshold="1e-6" />',
        '<CGLinearSolver iterations="20" tolerance="1e-5" threshold="1e-6" warmStart="1" />')
    s = capi.SofaScene(text)
    s.animate(30)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.set_warm_start(True)
    osc.step(30)
    xo, _ = osc.state()
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))


@pytest.mark.parametrize("edit,opts", [
    (("<TetrahedronFEMForceField name=\"FEM\"", "<TetrahedronFEMForceField rayleighStiffness=\"0.05\" name=\"FEM\""),
     dict(ff_rayleigh_stiffness=0.05)),
    (("<DiagonalMass name=\"mass\"", "<DiagonalMass rayleighMass=\"0.2\" name=\"mass\""),
     dict(mass_rayleigh_mass=0.2)),
    (("<EulerImplicitSolver />", "<EulerImplicitSolver firstOrder=\"1\" />"), dict(first_order=True)),
    (("<EulerImplicitSolver />", "<EulerImplicitSolver trapezoidalScheme=\"1\" />"), dict(trapezoidal_scheme=True)),
    (("name=\"fixC\"", "name=\"fixC\" activate_projectVelocity=\"1\""), dict(project_velocity=True)),
])
def test_grid_scene_file_with_component_options(capi, oracle, edit, opts):
    """The grid scene with the force field's rayleighStiffness, the mass's
    rayleighMass, the solver's firstOrder or the constraint's
    activate_projectVelocity set: loaded through the component layer, 30
    steps within 1e-10 of the oracle configured the same way."""
    text = _read("grid_fem_4x10x4.scn")
    assert edit[0] in text
    s = capi.SofaScene(text.replace(edit[0], edit[1], 1))
    s.animate(30)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.set_options(**opts)
    osc.step(30)
    xo, _ = osc.state()
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))


def test_grid_scene_file_with_update_stiffness_matrix(capi, oracle):
    """The grid scene with method polar and updateStiffnessMatrix="1" (the
    strain-displacement matrices rebuilt at every addForce): 30 steps within
    1e-10 of the oracle configured the same way."""
    text = _read("grid_fem_4x10x4.scn")
    assert 'method="large"' in text
    s = capi.SofaScene(text.replace('method="large"', 'method="polar" updateStiffnessMatrix="1"', 1))
    s.animate(30)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "polar")
    fem.set_update_stiffness(True)
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.step(30)
    xo, _ = osc.state()
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
    # without the rebuild the trajectory differs
    plain = oracle.OracleScene(oracle.OracleFEM(pos, tets, 600.0, 0.3, "polar"), node_masses=masses,
                               gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20, cg_tolerance=1e-5,
                               cg_threshold=1e-6)
    plain.step(30)
    assert np.max(np.abs(plain.state()[0] - xo)) > 1e-8 * np.max(np.abs(xo))


def test_grid_scene_file_with_separate_gravity(capi, oracle):
    """The grid scene with the mass's separateGravity="1": 30 steps within
    1e-10 of the oracle configured the same way."""
    text = _read("grid_fem_4x10x4.scn")
    assert '<DiagonalMass name="mass"' in text
    s = capi.SofaScene(text.replace('<DiagonalMass name="mass"', '<DiagonalMass separateGravity="1" name="mass"', 1))
    s.animate(30)
    x = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.set_separate_gravity(True)
    osc.step(30)
    xo, _ = osc.state()
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))


def test_reset_and_unload(capi, oracle):
    """SofaPhysicsAPI-style lifecycle. After reset the scene is back at its
    initial state and time 0, and 10 more steps match the oracle run through
    the same history (7 steps, the state put back, 10 steps: the solver keeps
    its time-step count across the reset, as the reference's CGLinearSolver
    does). unload frees the device; the next animate starts over from the
    initial state, bit-identical to a fresh load."""
    text = _read("grid_fem_4x10x4.scn")
    fresh = capi.SofaScene(text)
    fresh.animate(10)
    x_fresh = fresh.positions(0)
    s = capi.SofaScene(text)
    x0 = s.positions(0)
    s.animate(7)
    s.reset()
    assert s.time == 0.0
    assert np.array_equal(s.positions(0), x0)
    s.animate(10)
    x_reset = s.positions(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    _, masses, fixed = s.body_arrays(0)
    fem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(fem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.step(7)
    osc.set_state(pos, np.zeros_like(pos))
    osc.step(10)
    xo, _ = osc.state()
    assert np.max(np.abs(x_reset - xo)) <= 1e-10 * np.max(np.abs(xo))
    s.unload()
    assert s.time == 0.0
    assert np.array_equal(s.positions(0), x0)  # no device objects: the initial positions
    s.animate(10)
    assert np.array_equal(s.positions(0), x_fresh)  # a fresh start: bit-identical to the fresh load
