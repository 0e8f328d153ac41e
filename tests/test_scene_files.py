"""Component layer on the CPU: SOFA scene files parsed into the component
graph, their host initialisation (topology, masses, fixed sets, solver Data)
checked against the oracle-side helpers, the plugin entry points and the
factory, and the errors the reference's factory and components raise.
Nothing here touches a GPU."""
import os

import numpy as np
import pytest

from sofa_gb300 import topology as topo

HERE = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(HERE, "scenes")
# the reference's own benchmark scenes, read in place from the SOFA source
# tree named by SOFA_REFERENCE_ROOT (tests that need them skip without it)
REF_BENCH = os.path.join(os.environ.get("SOFA_REFERENCE_ROOT", ""),
                         "applications/plugins/SofaCUDA/scenes/benchmarks")


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    return capi


def _read(name):
    with open(os.path.join(SCENES, name)) as f:
        return f.read()


def test_plugin_entry_points_and_factory(capi):
    lib = capi.load()
    lib.initExternalModule()
    assert lib.moduleIsInitialized()
    assert lib.getModuleName() == b"SofaGB300"
    comps = lib.getModuleComponentList().decode().split()
    for c in ("TetrahedronFEMForceField", "EulerImplicitSolver", "CGLinearSolver", "UniformMass", "DiagonalMass",
              "FixedProjectiveConstraint", "MechanicalObject", "RegularGridTopology",
              "Hexa2TetraTopologicalMapping", "BoxROI", "TetrahedronSetTopologyContainer", "WriteState"):
        assert c in comps
    f = lib.sgb_object_factory_new()
    try:
        assert lib.sgb_object_factory_count(f) == 0
        lib.registerObjects(f)
        assert lib.sgb_object_factory_count(f) == len(comps)
        assert lib.sgb_object_factory_has(f, b"TetrahedronFEMForceField") == 1
        assert lib.sgb_object_factory_has(f, b"HexahedronFEMForceField") == 0
    finally:
        lib.sgb_object_factory_delete(f)


def test_grid_scene_host_init_matches_oracle_inputs(capi):
    """The known-answer grid scene: topology, lumped masses and the fixed
    set as the oracle test builds them."""
    s = capi.SofaScene(_read("grid_fem_4x10x4.scn"))
    assert s.n_bodies == 1
    info = s.body_info(0)
    assert info == {"n_nodes": 160, "n_tets": 486, "method": 1, "precision": 0, "n_fixed": info["n_fixed"]}
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets_ref = topo.hexa_to_tetra6(hexa, (3, 9))
    tets, masses, fixed = s.body_arrays(0)
    np.testing.assert_array_equal(tets, tets_ref)
    np.testing.assert_array_equal(s.positions(0), pos)
    vol = np.abs(topo.signed_volumes(tets_ref, pos))
    m_ref = np.zeros(len(pos))
    for t, v in zip(tets_ref, vol):
        m_ref[t] += v / 4.0
    np.testing.assert_allclose(masses, m_ref, rtol=1e-13)
    np.testing.assert_array_equal(fixed, topo.box_roi(pos, (-1, -1, 0, 10, 1, 50)))
    d = s.describe()
    b = d["bodies"][0]
    assert d["gravity"] == [0, 10, 0] and d["dt"] == 0.01
    assert (b["cg_iterations"], b["cg_tolerance"], b["cg_threshold"]) == (20, 1e-5, 1e-6)
    assert (b["rayleigh_stiffness"], b["rayleigh_mass"], b["mass_first"]) == (0.0, 0.0, 1)
    assert any("BlockGaussSeidelConstraintSolver" in x for x in d["ignored"])


def test_benchmark_style_scene(capi):
    s = capi.SofaScene(_read("beam_polar_gpu.scn"))
    assert s.n_bodies == 1
    info = s.body_info(0)
    assert info["n_nodes"] == 12 * 4 * 4 and info["n_tets"] == 11 * 3 * 3 * 6
    assert info["method"] == 2 and info["precision"] == 1  # polar, CudaVec3f -> mixed
    pos, _ = topo.regular_grid((12, 4, 4), (0, 0, 0), (6, 1.5, 1.5))
    tets, masses, fixed = s.body_arrays(0)
    np.testing.assert_array_equal(fixed, topo.box_roi(pos, (-0.1, -0.1, -0.1, 0.1, 2, 2)))
    np.testing.assert_allclose(masses, 3.0 / len(pos), rtol=0, atol=0)
    d = s.describe()
    ign = " ".join(d["ignored"])
    for c in ("RequiredPlugin", "VisualStyle", "CollisionPipeline", "OglModel", "IdentityMapping",
              "Tetra2TriangleTopologicalMapping", "TriangleSetTopologyContainer"):
        assert c in ign
    b = d["bodies"][0]
    assert (b["rayleigh_stiffness"], b["rayleigh_mass"], b["cg_iterations"]) == (0.1, 0.1, 25)
    assert d["gravity"] == [0, -9, 0]
    # a precision override
    s64 = capi.SofaScene(_read("beam_polar_gpu.scn"), precision=2)
    assert s64.body_info(0)["precision"] == 2


def test_reference_scene_with_an_out_of_scope_force_field(capi):
    """The 16x16x76 benchmark adds a PlaneForceField (penalty contact with a
    plane), which is not part of this component set: the load fails with
    SGB_ERR_NOT_SUPPORTED naming it, as the reference's factory does for a
    class it does not know."""
    path = os.path.join(REF_BENCH, "TetrahedronFEMForceField_beam16x16x76_gpu.scn")
    if not os.path.exists(path):
        pytest.skip("SOFA_REFERENCE_ROOT does not name the reference tree")
    with open(path) as f, pytest.raises(capi.SgbError) as e:
        capi.SofaScene(f.read())
    assert e.value.code == -4 and "PlaneForceField" in str(e.value)


@pytest.mark.parametrize("name,precision", [("TetrahedronFEMForceField_beam10x10x40_gpu.scn", 1),
                                            ("TetrahedronFEMForceField_beam10x10x40_cpu.scn", 0)])
def test_reference_benchmark_scene_files(capi, name, precision):
    """The reference's own SofaCUDA benchmark scenes, read where the reference
    tree is present, load unchanged."""
    path = os.path.join(REF_BENCH, name)
    if not os.path.exists(path):
        pytest.skip("SOFA_REFERENCE_ROOT does not name the reference tree")
    with open(path) as f:
        s = capi.SofaScene(f.read())
    assert s.n_bodies == 1
    info = s.body_info(0)
    d = s.describe()
    grid = [o for n in d["root"]["children"] for o in n["objects"] if o["class"] == "RegularGridTopology"][0]
    nx, ny, nz = (int(v) for v in grid["data"]["n"].split())
    assert info["n_nodes"] == nx * ny * nz
    assert info["n_tets"] == (nx - 1) * (ny - 1) * (nz - 1) * 6
    assert info["precision"] == precision and info["method"] == 1
    tets, masses, fixed = s.body_arrays(0)
    assert info["n_fixed"] == ny * nz  # the x = 0 face
    assert masses.sum() == pytest.approx(50.0, rel=1e-12)  # DiagonalMass totalMass="50.0"


BAD = {
    "unknown component": ("<Node name='r'><HexahedronFEMForceField/></Node>", -4),
    "unterminated": ("<Node name='r'><EulerImplicitSolver></Node>", -1),
    "not a node root": ("<EulerImplicitSolver/>", -1),
}


@pytest.mark.parametrize("case", sorted(BAD))
def test_scene_errors(capi, case):
    xml, rc = BAD[case]
    with pytest.raises(capi.SgbError) as e:
        capi.SofaScene(xml)
    assert e.value.code == rc


@pytest.mark.parametrize("edit,msg", [
    (('method="large"', 'method="large" updateStiffnessMatrix="1"'), "updateStiffnessMatrix"),
    (('<DiagonalMass name="mass" massDensity="1.0" />', ''), "mass"),
    (('name="fixC"', 'name="fixC" activate_projectVelocity="1"'
      ' />\n        <FixedProjectiveConstraint name="fix2" indices="0"'), "activate_projectVelocity"),
    (('<TetrahedronFEMForceField name="FEM"', '<TetrahedronFEMForceField computeVonMisesStress="3" name="FEM"'),
     "computeVonMisesStress"),
])
def test_unsupported_component_settings(capi, edit, msg):
    xml = _read("grid_fem_4x10x4.scn").replace(*edit)
    with pytest.raises(capi.SgbError) as e:
        capi.SofaScene(xml)
    assert e.value.code == -4 and msg in str(e.value)


def test_initial_points_are_replaced_by_the_rest_positions(capi):
    """TetrahedronFEMForceField initialPoints is accepted and, as in the
    reference, replaced by the MechanicalObject's rest positions at init
    (TetrahedronFEMForceField.inl:1411-1412): the body's rest configuration is
    the one without it."""
    text = _read("grid_fem_4x10x4.scn")
    plain = capi.SofaScene(text)
    with_ip = capi.SofaScene(text.replace('<TetrahedronFEMForceField name="FEM"',
                                          '<TetrahedronFEMForceField initialPoints="0 0 0 1 1 1" name="FEM"', 1))
    assert np.array_equal(plain.positions(0), with_ip.positions(0))
    assert np.array_equal(plain.body_arrays(0)[1], with_ip.body_arrays(0)[1])


PCG_SCENE = ('<CGLinearSolver iterations="20" tolerance="1e-5" threshold="1e-6" />',
             '<PreconditionedMatrixFreeSystem assemblingRate="4"/>\n'
             '        <PCGLinearSolver name="PCG" iterations="30" tolerance="1e-9" preconditioner="@precond"/>\n'
             '        <JacobiPreconditioner name="precond" template="DiagonalMatrix"/>')


def test_pcg_jacobi_scene(capi):
    """PCGLinearSolver + JacobiPreconditioner (+ PreconditionedMatrixFreeSystem
    assemblingRate), as in the reference's FEMBAR_PCG_JacobiPreconditioner.scn."""
    s = capi.SofaScene(_read("grid_fem_4x10x4.scn").replace(*PCG_SCENE))
    assert s.body_solver(0) == {"linear_solver": 1, "preconditioner": 1, "preconditioner_rate": 4,
                                "iterations": 30, "tolerance": pytest.approx(1e-9)}
    plain = capi.SofaScene(_read("grid_fem_4x10x4.scn").replace(
        PCG_SCENE[0], '<PCGLinearSolver iterations="12" use_precond="0" preconditioner="@p"/><JacobiPreconditioner name="p"/>'))
    assert plain.body_solver(0)["preconditioner"] == 0
    with pytest.raises(capi.SgbError) as e:
        capi.SofaScene(_read("grid_fem_4x10x4.scn").replace(
            PCG_SCENE[0], '<PCGLinearSolver preconditioner="@p"/><BlockJacobiPreconditioner name="p"/>'))
    assert e.value.code in (-4,)


DIAG_MASS_SCENE = """<Node name="Root" gravity="0 0 0">
    <RegularGridTopology name="grid" n="2 2 2" min="0 0 0" max="2 2 2" p0="0 0 0" />
    <Node name="Tetra">
        <EulerImplicitSolver />
        <CGLinearSolver />
        <MechanicalObject position="@../grid.position" />
        <TetrahedronSetTopologyContainer name="Container" />
        <Hexa2TetraTopologicalMapping name="default28" input="@../grid" output="@Container" />
        <DiagonalMass name="m_mass" {mass} />
        <TetrahedronFEMForceField />
    </Node>
</Node>"""


@pytest.mark.parametrize("mass,total,first", [
    ('massDensity="1.0"', 8.0, [1.66667, 1.0, 1.0, 0.333333]),
    ('totalMass="10.0"', 10.0, [2.08333, 1.25, 1.25, 0.416667]),
])
def test_diagonal_mass_known_answers(capi, mass, total, first):
    """DiagonalMass on the 2x2x2 grid split into tetrahedra
    (DiagonalMass_test.cpp checkTotalMassFromMassDensity_Tetra and
    checkMassDensityFromTotalMass_Tetra): total mass and the first four
    lumped node masses, to the reference test's 1e-4."""
    s = capi.SofaScene(DIAG_MASS_SCENE.format(mass=mass))
    _, masses, _ = s.body_arrays(0)
    assert len(masses) == 8
    assert masses.sum() == pytest.approx(total, abs=1e-4)
    np.testing.assert_allclose(masses[:4], first, atol=1e-4)
