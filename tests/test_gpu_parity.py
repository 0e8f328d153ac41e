"""GPU parity of the CUDA path against the CPU oracle, through the C ABI.

Tolerances (stated per test):
  fp64      (reference rounding) addForce/addDForce bit-identical; a whole
            step with serial dots bit-identical; with parallel dots positions
            within 1e-10 relative after 100 steps.
  fp64_fma  per call within 1e-10 relative.
  mixed     per call within 1e-5 relative; positions within 1e-4 relative
            to the FP64 trajectory after 100 steps.
"""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


def deformed_state(oracle, mesh, method, steps=10):
    _, sc = cases.oracle_scene(oracle, mesh, method)
    sc.step(steps)
    x, v = sc.state()
    return x, v


def run_calls(torch, capi, mesh, method, precision, x, dx, kfactor):
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method, precision)
    dt = torch.float32 if precision == "mixed" else torch.float64
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    # add_force / add_dforce accumulate: start from non-zero values (zero for
    # mixed, whose FP32 start values would hide the contribution's accuracy)
    scale = 0.0 if precision == "mixed" else 1.0
    f0 = scale * np.random.default_rng(1).normal(size=x.shape)
    fd = torch.tensor(f0, dtype=dt, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())
    dxd = torch.tensor(dx, dtype=dt, device="cuda")
    df0 = scale * np.random.default_rng(2).normal(size=x.shape)
    dfd = torch.tensor(df0, dtype=dt, device="cuda")
    fem.add_dforce(dxd.data_ptr(), dfd.data_ptr(), kfactor)
    torch.cuda.synchronize()
    rot, rot0 = fem.rotations()
    fem.close()
    return f0, fd.cpu().double().numpy(), df0, dfd.cpu().double().numpy(), rot


@pytest.mark.parametrize("method", ["small", "large", "polar", "svd"])
@pytest.mark.parametrize("precision", ["fp64", "fp64_fma", "mixed"])
def test_add_force_add_dforce_per_call(torch_cuda, capi, oracle, method, precision):
    mesh = cases.beam_mesh()
    x, _ = deformed_state(oracle, mesh, method)
    rng = np.random.default_rng(11)
    dx = rng.normal(scale=1e-3, size=x.shape)
    if precision == "mixed":
        # FP32 strain is accurate to ~1e-7 absolute, so the relative bar is
        # checked on a strained state (strains ~1e-2); near rest the force
        # error is that absolute level, which the trajectory test bounds
        x = x + rng.normal(scale=5e-3, size=x.shape)
        dx = dx.astype(np.float32).astype(np.float64)
    kfactor = -0.0011
    f0, f_gpu, df0, df_gpu, rot = run_calls(torch_cuda, capi, mesh, method, precision, x, dx, kfactor)
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    f_ref = ofem.add_force(x, f0)
    df_ref = ofem.add_dforce(dx, kfactor, df0)
    # contribution-only errors (the accumulator start values are random)
    ef = cases.rel_err(f_gpu - f0, f_ref - f0)
    ed = cases.rel_err(df_gpu - df0, df_ref - df0)
    if precision == "fp64":
        assert np.array_equal(f_gpu, f_ref), ef
        assert np.array_equal(df_gpu, df_ref), ed
    elif precision == "fp64_fma":
        assert ef <= 1e-10 and ed <= 1e-10, (ef, ed)
    else:
        assert ef <= 1e-5 and ed <= 1e-5, (ef, ed)
    if method != "small":
        ref_rot = np.stack([ofem.element(e)["rotation"] for e in range(0, mesh.n_tets, 97)])
        tol = 0 if precision == "fp64" else (1e-12 if precision == "fp64_fma" else 1e-5)
        np.testing.assert_allclose(rot[::97], ref_rot, rtol=0, atol=tol)


@pytest.mark.parametrize("method", ["large", "polar"])
def test_mixed_add_force_small_strain(torch_cuda, capi, oracle, method):
    """Mixed addForce at strains of 1e-5..5e-5 on a rotated, translated beam.
    The strain is formed in float-float, so the force matches the FP64
    oracle to the FP32 element arithmetic; FP32 edges and an FP32 rotation
    alone would leave strain noise of ~1e-7 absolute, ~1e-2 of this load."""
    mesh = cases.beam_mesh()
    p = mesh.positions
    u = 1e-5 * np.stack([np.sin(1.3 * p[:, 2]), np.cos(0.7 * p[:, 0]) * p[:, 2], 0.5 * p[:, 1] * p[:, 2]], 1)
    ax = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    kx = np.array([[0.0, -ax[2], ax[1]], [ax[2], 0.0, -ax[0]], [-ax[1], ax[0], 0.0]])
    rot = np.eye(3) + np.sin(0.3) * kx + (1.0 - np.cos(0.3)) * kx @ kx
    x = (p + u) @ rot.T + np.array([7.0, -3.0, 11.0])
    f0, f_gpu, _, _, _ = run_calls(torch_cuda, capi, mesh, method, "mixed", x, np.zeros_like(x), -0.001)
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    f_ref = ofem.add_force(x, f0)
    err = cases.rel_err(f_gpu - f0, f_ref - f0)
    assert err <= 1e-4, err


def _invert(mesh, x, elems, flat=()):
    """Moves node a of each element through the opposite face (inverted,
    det F < 0) or onto its plane (flat, det F = 0)."""
    x = x.copy()
    for e, s in [(e, 1.5) for e in elems] + [(e, 0.0) for e in flat]:
        t = mesh.tetrahedra[e]
        c = x[t[1:]].mean(0)
        x[t[0]] = c + s * (c - x[t[0]])
    return x


@pytest.mark.parametrize("precision", ["fp64", "fp64_fma", "mixed"])
def test_svd_method_inverted_elements(torch_cuda, capi, oracle, precision):
    """method=svd (accumulateForceSVD, TFEM.inl:1123-1184): elements whose
    deformation gradient has det < 1e-6 take the stable SVD polar factor
    (the oracle's restatement is pinned to the reference's bits); the
    others the polar factor. FP64 per call is bit-identical to the oracle
    (a flattened element included), FP64-FMA within 1e-10, mixed within
    1e-5 (inverted elements only: a flat one sits on the FP32 / FP64
    degeneracy thresholds)."""
    mesh = cases.beam_mesh()
    rng = np.random.default_rng(12)
    x = mesh.positions + rng.normal(scale=5e-3, size=mesh.positions.shape)
    x = _invert(mesh, x, [0, 57, 311, 900], flat=[] if precision == "mixed" else [640])
    dx = rng.normal(scale=1e-3, size=x.shape)
    if precision == "mixed":
        dx = dx.astype(np.float32).astype(np.float64)
    kfactor = -0.0011
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "svd")
    f0, f_gpu, df0, df_gpu, rot = run_calls(torch_cuda, capi, mesh, "svd", precision, x, dx, kfactor)
    f_ref = ofem.add_force(x, f0)
    df_ref = ofem.add_dforce(dx, kfactor, df0)
    polar = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar").add_force(x, f0)
    assert not np.array_equal(polar, f_ref)  # the stable frame was taken
    ef = cases.rel_err(f_gpu - f0, f_ref - f0)
    ed = cases.rel_err(df_gpu - df0, df_ref - df0)
    if precision == "fp64":
        assert np.array_equal(f_gpu, f_ref), ef
        assert np.array_equal(df_gpu, df_ref), ed
    elif precision == "fp64_fma":
        assert ef <= 1e-10 and ed <= 1e-10, (ef, ed)
    else:
        assert ef <= 1e-5 and ed <= 1e-5, (ef, ed)
    ref_rot = np.stack([ofem.element(e)["rotation"] for e in (0, 57, 311, 900)])
    tol = 0 if precision == "fp64" else (1e-12 if precision == "fp64_fma" else 1e-5)
    np.testing.assert_allclose(rot[[0, 57, 311, 900]], ref_rot, rtol=0, atol=tol)


def test_scene_100_steps_bit_identical_with_serial_dots(torch_cuda, capi, oracle):
    """FP64 with serial dot products reproduces the reference's rounding
    sequence: positions after 100 steps are bit-identical to the oracle."""
    mesh = cases.beam_mesh()
    _, osc = cases.oracle_scene(oracle, mesh, "large")
    osc.step(100)
    xr, vr = osc.state()
    sc = cases.gpu_scene(capi, mesh, "large", "fp64", serial_dots=True)
    sc.step(100)
    x, v = sc.state()
    it, _ = sc.sync()
    assert np.array_equal(x, xr), np.abs(x - xr).max()
    assert np.array_equal(v, vr)
    assert it == osc.last_iterations


@pytest.mark.parametrize("method", ["large", "polar"])
def test_scene_100_steps_parallel_dots(torch_cuda, capi, oracle, method):
    """FP64 with the parallel deterministic dot products: per-node positions
    within 1e-10 relative (norm-wise) after 100 steps; two runs bit-identical."""
    mesh = cases.beam_mesh()
    _, osc = cases.oracle_scene(oracle, mesh, method)
    osc.step(100)
    xr, _ = osc.state()
    xs = []
    for _ in range(2):
        sc = cases.gpu_scene(capi, mesh, method, "fp64")
        sc.step(100)
        xs.append(sc.state()[0])
        sc.close()
    assert np.array_equal(xs[0], xs[1])  # deterministic: no atomics on the data path
    disp = xr - mesh.positions
    assert cases.rel_err(xs[0], xr) <= 1e-10
    assert np.linalg.norm(xs[0] - xr) / np.linalg.norm(disp) <= 1e-8


# (mesh, method, CG iterations, CG tolerance, bar on the relative L2 position
# error, bar on the displacement-relative error). The small beam is the
# plain-method workload (method=large, CG 25/1e-9); its polar variant and the
# CG 50/1e-7 polar beam (the large-beam workload's solver settings on a
# smaller grid) are checked beside it. With 25 unconverged CG iterations
# (|r|/|b| ~ 1 after the solve) the FP32 Krylov sequence wanders from the
# FP64 one by ~1e-4 of the positions, whatever the FP32 arithmetic details;
# the bars state that.
MIXED_CASES = [
    ((5, 5, 21), "large", 25, 1e-9, 1e-4, 1e-2),
    ((5, 5, 21), "polar", 25, 1e-9, 2e-4, 2e-2),
    ((12, 12, 49), "polar", 50, 1e-7, 1e-4, 2e-1),
]


@pytest.mark.parametrize("n,method,iters,tol,bar_pos,bar_disp", MIXED_CASES)
def test_mixed_precision_trajectory(torch_cuda, capi, n, method, iters, tol, bar_pos, bar_disp):
    """Mixed precision vs the GPU FP64 run of the same scene: relative L2
    position error after 100 steps (the accuracy the benchmark metric is
    quoted at, <= 1e-4) and the stricter
    error relative to the displacement."""
    mesh = cases.beam_mesh(n)
    cfg = dict(cases.BEAM_SMALL, cg_iterations=iters, cg_tolerance=tol)
    ref = cases.gpu_scene(capi, mesh, method, "fp64", cfg=cfg)
    ref.step(100)
    xr, _ = ref.state()
    mx = cases.gpu_scene(capi, mesh, method, "mixed", cfg=cfg)
    mx.step(100)
    x, _ = mx.state()
    err = cases.rel_err(x, xr)
    disp_err = np.linalg.norm(x - xr) / np.linalg.norm(xr - mesh.positions)
    print(f"mixed {n} {method}: rel pos err {err:.3e}, displacement-relative {disp_err:.3e}")
    assert err <= bar_pos
    assert disp_err <= bar_disp


def test_reference_grid_known_answer_on_gpu(torch_cuda, capi, oracle):
    """The reference's checkFEMValues scene (BaseTetrahedronFEMForceField_test.h
    :117-177, :379-431) run on the GPU: x[159] after 100 steps within 1e-4 of
    the reference's expected value and bit-identical to the oracle."""
    from sofa_gb300 import topology as topo

    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    vol = np.abs(topo.signed_volumes(tets, pos))
    masses = np.zeros(len(pos))
    for t, v in zip(tets, vol):
        m = (1.0 * v) / 4.0
        for i in t:
            masses[i] += m
    fixed = topo.box_roi(pos, (-1, -1, 0, 10, 1, 50))
    fem = capi.TetrahedronFEM(pos, tets, 600.0, 0.3, "large", "fp64")
    sc = capi.Scene(fem, dt=0.01, cg_iterations=20, cg_tolerance=1e-5, cg_threshold=1e-6, gravity=(0, 10, 0),
                    node_masses=masses, fixed=fixed, serial_dots=True)
    sc.step(100)
    x, _ = sc.state()
    np.testing.assert_allclose(x[159], [9.99985, 45.0487, 30.0011], atol=1e-4)
    ofem = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large")
    osc = oracle.OracleScene(ofem, node_masses=masses, gravity=(0, 10, 0), fixed=fixed, dt=0.01, cg_iterations=20,
                             cg_tolerance=1e-5, cg_threshold=1e-6)
    osc.step(100)
    assert np.array_equal(x, osc.state()[0])


def test_small_regular_tet_forces_on_gpu(torch_cuda, capi):
    """TetrahedronFEMForceField_stepTest.cpp:58-75 through the C ABI."""
    rest = np.array([[0, 0, 0], [1, 0, 0], [0.5, 0.86602540378443864676, 0], [0.5, 0.288675134594812882254, 1]])
    x = rest.copy()
    x[2] = [0.5, 0.8660254037, 0]
    x[3] = [0.5, 0.28867513, 2]
    fem = capi.TetrahedronFEM(rest, [[0, 1, 2, 3]], 40.0, 0.0, "small", "fp64")
    torch = torch_cuda
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    fd = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())
    torch.cuda.synchronize()
    f = fd.cpu().numpy()
    fdown = np.sqrt(3.0) * 10.0 / 9.0
    np.testing.assert_allclose(f[:3, 2], [fdown] * 3, rtol=1e-6)
    np.testing.assert_allclose(f[3, 2], -np.sqrt(3.0) * 10.0 / 3.0, rtol=1e-6)


def test_empty_and_isolated_nodes(torch_cuda, capi):
    """Edge cases: a mesh with no tetrahedra and nodes with no element leave
    forces untouched; a fully fixed scene does not move."""
    torch = torch_cuda
    pos = np.random.default_rng(0).normal(size=(10, 3))
    fem = capi.TetrahedronFEM(pos, np.zeros((0, 4), np.int32), 5000.0, 0.45, "large", "fp64")
    xd = torch.tensor(pos, dtype=torch.float64, device="cuda")
    fd = torch.ones((10, 3), dtype=torch.float64, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())
    torch.cuda.synchronize()
    assert torch.all(fd == 1)
    mesh = cases.beam_mesh((3, 3, 3))
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "large", "fp64")
    sc = capi.Scene(fem, fix_all=True, cg_iterations=10)
    sc.step(3)
    x, v = sc.state()
    assert np.array_equal(x, mesh.positions) and not v.any()


@pytest.mark.parametrize("method", ["small", "large", "polar", "svd"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp64_fma", 1e-12), ("mixed", 1e-5)])
def test_assembled_stiffness(torch_cuda, capi, oracle, method, precision, tol):
    """sgb_tfem_stiffness_bsr (buildStiffnessMatrix, TFEM.inl:1965-1993): the
    block-sparse df/dx at the rotations of the last addForce times a vector
    equals the oracle's addDForce with kFactor 1; the matrix is symmetric."""
    sp = pytest.importorskip("scipy.sparse")
    mesh = cases.beam_mesh()
    x, _ = deformed_state(oracle, mesh, "large" if method == "small" else method)
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method, precision)
    dt = torch_cuda.float32 if precision == "mixed" else torch_cuda.float64
    xd = torch_cuda.tensor(x, dtype=torch_cuda.float64, device="cuda")
    fd = torch_cuda.zeros(x.shape, dtype=dt, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())
    rowptr, cols, blocks = fem.stiffness_bsr()
    fem.close()
    n3 = 3 * mesh.n_nodes
    Kb = sp.bsr_matrix((blocks, cols, rowptr), shape=(n3, n3))
    v = np.random.default_rng(8).normal(size=x.shape)
    ofem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    ofem.add_force(x)
    ref = ofem.add_dforce(v, 1.0)
    got = (Kb @ v.reshape(-1)).reshape(-1, 3)
    assert cases.rel_err(got, ref) <= tol
    # symmetric to the rounding of the element products (FP32 in mixed)
    assert abs(Kb - Kb.T).max() <= (1e-6 if precision == "mixed" else 1e-12) * abs(Kb).max()


@pytest.mark.parametrize("method", ["large", "polar"])
@pytest.mark.parametrize("precision,tol", [("fp64", 0.0), ("fp64_fma", 1e-10), ("mixed", 1e-5)])
def test_ragged_materials_and_isolated_nodes(torch_cuda, capi, oracle, method, precision, tol):
    """Ragged per-element data (getVecRealInElement,
    BaseLinearElasticityFEMForceField.inl:114-144: entry e when the vector is
    longer than e, else entry 0): a Young's modulus vector of 37 entries, a
    Poisson vector of E entries, a local stiffness factor of 5 entries; plus
    nodes that belong to no element, interleaved with the mesh's nodes (the
    patch layout must leave them out). Per call against the oracle."""
    mesh = cases.beam_mesh((4, 4, 9), seed=3)
    rng = np.random.default_rng(21)
    n0 = mesh.n_nodes
    # interleave isolated nodes: old node i -> 2 i, odd slots unused
    pos = np.zeros((2 * n0, 3))
    pos[0::2] = mesh.positions
    pos[1::2] = rng.normal(size=(n0, 3)) * 10.0
    tets = 2 * mesh.tetrahedra
    E = tets.shape[0]
    young = 10 ** rng.uniform(3, 4, size=37)
    poisson = rng.uniform(0.3, 0.45, size=E)
    lsf = rng.uniform(0.5, 2.0, size=5)
    x = pos + rng.normal(scale=2e-2, size=pos.shape)
    dx = rng.normal(scale=1e-3, size=pos.shape)
    fem = capi.TetrahedronFEM(pos, tets, young, poisson, method, precision, local_stiffness_factor=lsf)
    dt = torch_cuda.float32 if precision == "mixed" else torch_cuda.float64
    if precision == "mixed":
        dx = dx.astype(np.float32).astype(np.float64)
    xd = torch_cuda.tensor(x, dtype=torch_cuda.float64, device="cuda")
    fd = torch_cuda.zeros(x.shape, dtype=dt, device="cuda")
    fem.add_force(xd.data_ptr(), fd.data_ptr())
    dxd = torch_cuda.tensor(dx, dtype=dt, device="cuda")
    dfd = torch_cuda.zeros(x.shape, dtype=dt, device="cuda")
    fem.add_dforce(dxd.data_ptr(), dfd.data_ptr(), -0.01)
    torch_cuda.cuda.synchronize()
    fem.close()
    ofem = oracle.OracleFEM(pos, tets, young, poisson, method, local_stiffness_factor=lsf)
    f_ref = ofem.add_force(x)
    df_ref = ofem.add_dforce(dx, -0.01)
    f, df = fd.cpu().double().numpy(), dfd.cpu().double().numpy()
    assert not f[1::2].any() and not df[1::2].any()  # isolated nodes untouched
    if tol == 0.0:
        assert np.array_equal(f, f_ref) and np.array_equal(df, df_ref)
    else:
        assert cases.rel_err(f, f_ref) <= tol and cases.rel_err(df, df_ref) <= tol


@pytest.mark.parametrize("method", ["large", "polar"])
def test_scene_with_nodes_of_no_element(torch_cuda, capi, oracle, method):
    """A scene whose MechanicalObject has points that no tetrahedron uses:
    those points fall under gravity with their own mass rows. The mixed
    step (fused patch kernels, where such nodes sit in element-free
    patches) against the oracle over 10 steps, the batch engine's mixed step
    beside it, and FP64 with serial dots bit-identical."""
    mesh = cases.beam_mesh((4, 4, 13), seed=5)
    n0 = mesh.n_nodes
    pos = np.zeros((2 * n0, 3))
    pos[0::2] = mesh.positions
    pos[1::2] = mesh.positions + np.array([0.0, 3.0, 0.0])
    tets = 2 * mesh.tetrahedra
    fixed = 2 * np.asarray(mesh.fixed)
    cfg = cases.BEAM_SMALL
    kw = dict(dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"], cg_iterations=cfg["cg_iterations"],
              cg_tolerance=cfg["cg_tolerance"], cg_threshold=cfg["cg_threshold"], gravity=cfg["gravity"])
    vm = cfg["total_mass"] / (2 * n0)
    steps = 10
    ofem = oracle.OracleFEM(pos, tets, cfg["young"], cfg["poisson"], method)
    osc = oracle.OracleScene(ofem, vertex_mass=vm, fixed=fixed, **kw)
    osc.step(steps)
    xr, vr = osc.state()
    it_ref = osc.last_iterations
    d = np.linalg.norm(xr - pos)
    for precision in ("fp64", "mixed"):
        fem = capi.TetrahedronFEM(pos, tets, cfg["young"], cfg["poisson"], method, precision)
        sc = capi.Scene(fem, vertex_mass=vm, fixed=fixed, serial_dots=precision == "fp64", **kw)
        sc.step(steps)
        it, _ = sc.sync()
        x, v = sc.state()
        sc.close()
        if precision == "fp64":
            assert it == it_ref
            assert np.array_equal(x, xr) and np.array_equal(v, vr)
        else:
            assert np.linalg.norm(x - xr) / d <= 1e-4, np.linalg.norm(x - xr) / d
            # the free points: x0 + the FP64 trajectory of a free mass
            np.testing.assert_allclose(x[1::2], xr[1::2], rtol=0, atol=1e-6)
    b = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=2)
    s = b.add_mesh(pos, tets, young=cfg["young"], poisson=cfg["poisson"], method=method, total_mass=cfg["total_mass"],
                   fixed=fixed, **kw)
    b.step(steps)
    x = b.state(s)[0]
    b.close()
    assert np.linalg.norm(x - xr) / d <= 1e-4
    np.testing.assert_allclose(x[1::2], xr[1::2], rtol=0, atol=1e-6)


@pytest.mark.parametrize("precision", ["fp64", "fp64_fma", "mixed"])
def test_fixed_constraint_constant_force_known_answer(torch_cuda, capi, precision):
    """The reference's FixedProjectiveConstraint_test known answer on the GPU
    (a force field with no tetrahedra, the constant force as the external
    force): x[3][0] = 4.32231 and x[4][0] = 5.32231 after two steps of 0.1,
    fixed points unchanged."""
    x0 = np.array([[i + 0.1 * k for k in range(3)] for i in range(5)])
    fem = capi.TetrahedronFEM(x0, np.zeros((0, 4), np.int32), 5000.0, 0.45, "large", precision)
    sc = capi.Scene(fem, dt=0.1, rayleigh_stiffness=0.01, rayleigh_mass=1.0, cg_iterations=25, cg_tolerance=1e-5,
                    cg_threshold=1e-5, gravity=(0.0, 0.0, 0.0), vertex_mass=0.2, fixed=[0, 1, 2])
    sc.set_external_force(np.full((5, 3), 10.0))
    sc.step(2)
    x, _ = sc.state()
    assert np.array_equal(x[:3], x0[:3])
    np.testing.assert_allclose([x[3, 0], x[4, 0]], [4.32231, 5.32231], atol=1e-4)
