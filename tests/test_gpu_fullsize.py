"""GPU parity against the CPU oracle at the benchmark workloads' full size.

The oracle runs in its exact parallel mode (element terms in parallel, every
node summing its terms in element order, dot products serial), which is
bit-identical to the single-thread restatement of the reference's serial
loops (tests/test_oracle_parallel.py), on every host thread.

* Single beam, 64x64x257 nodes, 5,080,320 tetrahedra, polar, CG 50 / 1e-7:
  - addForce / addDForce per call: FP64 reference rounding bit-identical;
    FP64-FMA within 1e-10 relative; mixed within 1e-5 relative.
  - 5 implicit steps: FP64 reference rounding with serial dots bit-identical
    (positions, velocities and CG iterations); FP64-FMA within
    1e-10 relative on the positions; mixed within 1e-4 relative on the
    positions (the metric's norm) and 2e-4 on the displacement (measured
    8.5e-5 after 5 steps).
* Stiff-inclusion block, 48x48x193 nodes, 2,120,640 tetrahedra, E 1e6 in a
  1e3 beam (per-element vector), nu 0.49, tip traction, CG 200 / 1e-10:
  3 steps, FP64 reference rounding with serial dots bit-identical.
* 16 beams of the batched workload's population (both methods, the E/nu
  spread): 3 steps of the FP64 batch within 1e-9 relative on the positions
  of each beam; the mixed batch within 1e-4 (position) of the oracle.
"""
import os

import numpy as np
import pytest

from sofa_gb300 import workloads as wl
from tests import cases

pytestmark = pytest.mark.gpu

STEPS = 5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def capi(torch_cuda):
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


@pytest.fixture(scope="module")
def exact_oracle(oracle):
    oracle.set_threads(max(1, len(os.sched_getaffinity(0))), exact=True)
    yield oracle
    oracle.set_threads(1)


@pytest.fixture(scope="module")
def beam():
    return wl.single_beam_mesh()


@pytest.fixture(scope="module")
def beam_trajectory(exact_oracle, beam):
    """The oracle's state after STEPS steps of the single-beam workload, with
    the CG iterations and residual of the last solve."""
    cfg = wl.SINGLE_BEAM
    fem = exact_oracle.OracleFEM(beam.positions, beam.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"])
    sc = exact_oracle.OracleScene(fem, vertex_mass=cfg["total_mass"] / beam.n_nodes, gravity=cfg["gravity"],
                                  fixed=beam.fixed, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"],
                                  rayleigh_mass=cfg["rm"], cg_iterations=cfg["cg_iterations"],
                                  cg_tolerance=cfg["cg_tolerance"], cg_threshold=cfg["cg_threshold"])
    sc.step(STEPS)
    x, v = sc.state()
    out = dict(x=x, v=v, iterations=sc.last_iterations, residual=sc.last_error)
    del sc, fem
    return out


def gpu_beam_run(capi, beam, precision, serial_dots=False, steps=STEPS):
    cfg = wl.SINGLE_BEAM
    fem = capi.TetrahedronFEM(beam.positions, beam.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"],
                              precision)
    sc = capi.Scene(fem, serial_dots=serial_dots, **wl.single_beam_solver(cfg, beam))
    sc.step(steps)
    it, res = sc.sync()
    x, v = sc.state()
    sc.close()
    return x, v, it, res


def test_single_beam_per_call(torch_cuda, capi, exact_oracle, beam):
    torch = torch_cuda
    cfg = wl.SINGLE_BEAM
    rng = np.random.default_rng(21)
    # a strained, rotated state: the gravity sag of a few steps is too small
    # to exercise the polar factor away from the identity
    u = 2e-3 * np.stack([np.sin(0.05 * beam.positions[:, 2]), np.cos(0.03 * beam.positions[:, 2]),
                         0.01 * beam.positions[:, 0]], 1)
    x = beam.positions + u + rng.normal(scale=5e-3, size=beam.positions.shape)
    dx = rng.normal(scale=1e-3, size=x.shape)
    kfactor = -0.0011
    ofem = exact_oracle.OracleFEM(beam.positions, beam.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"])
    f_ref = ofem.add_force(x)
    df_ref = ofem.add_dforce(dx, kfactor)
    del ofem
    for precision in ("fp64", "fp64_fma", "mixed"):
        fem = capi.TetrahedronFEM(beam.positions, beam.tetrahedra, cfg["young"], cfg["poisson"], cfg["method"],
                                  precision)
        dt = torch.float32 if precision == "mixed" else torch.float64
        xd = torch.tensor(x, dtype=torch.float64, device="cuda")
        fd = torch.zeros(x.shape, dtype=dt, device="cuda")
        fem.add_force(xd.data_ptr(), fd.data_ptr())
        dxd = torch.tensor(dx, dtype=dt, device="cuda")
        dfd = torch.zeros(x.shape, dtype=dt, device="cuda")
        fem.add_dforce(dxd.data_ptr(), dfd.data_ptr(), kfactor)
        torch.cuda.synchronize()
        f = fd.cpu().double().numpy()
        df = dfd.cpu().double().numpy()
        fem.close()
        del xd, fd, dxd, dfd
        if precision == "fp64":
            assert np.array_equal(f, f_ref), cases.rel_err(f, f_ref)
            assert np.array_equal(df, df_ref), cases.rel_err(df, df_ref)
        elif precision == "fp64_fma":
            assert cases.rel_err(f, f_ref) <= 1e-10 and cases.rel_err(df, df_ref) <= 1e-10
        else:
            assert cases.rel_err(f, f_ref) <= 1e-5 and cases.rel_err(df, df_ref) <= 1e-5


def test_single_beam_fp64_steps_bit_identical(capi, beam, beam_trajectory):
    x, v, it, res = gpu_beam_run(capi, beam, "fp64", serial_dots=True)
    assert it == beam_trajectory["iterations"]
    assert np.array_equal(x, beam_trajectory["x"]), cases.rel_err(x, beam_trajectory["x"])
    assert np.array_equal(v, beam_trajectory["v"])


def test_single_beam_fp64_fma_and_mixed_steps(capi, beam, beam_trajectory):
    xr = beam_trajectory["x"]
    d = np.linalg.norm(xr - beam.positions)
    x, _, it, _ = gpu_beam_run(capi, beam, "fp64_fma")
    assert it == beam_trajectory["iterations"]
    assert cases.rel_err(x, xr) <= 1e-10
    x, _, _, _ = gpu_beam_run(capi, beam, "mixed")
    assert cases.rel_err(x, xr) <= 1e-4
    assert np.linalg.norm(x - xr) / d <= 2e-4


def test_inclusion_block_fp64_steps_bit_identical(capi, exact_oracle):
    cfg = wl.INCLUSION
    ib = wl.inclusion_block(cfg)
    m = ib.mesh
    steps = 3
    kw = dict(dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"], cg_iterations=cfg["cg_iterations"],
              cg_tolerance=cfg["cg_tolerance"], cg_threshold=1e-20, gravity=cfg["gravity"])
    ofem = exact_oracle.OracleFEM(m.positions, m.tetrahedra, ib.young, cfg["poisson"], cfg["method"])
    osc = exact_oracle.OracleScene(ofem, vertex_mass=1.0 / m.n_nodes, fixed=m.fixed, **kw)
    osc.set_external_force(ib.tip_force)
    osc.step(steps)
    xr, vr = osc.state()
    it_ref, res_ref = osc.last_iterations, osc.last_error
    del osc, ofem
    fem = capi.TetrahedronFEM(m.positions, m.tetrahedra, ib.young, cfg["poisson"], cfg["method"], "fp64")
    sc = capi.Scene(fem, vertex_mass=1.0 / m.n_nodes, fixed=m.fixed, serial_dots=True, **kw)
    sc.set_external_force(ib.tip_force)
    sc.step(steps)
    it, res = sc.sync()
    x, v = sc.state()
    sc.close()
    assert it == it_ref
    assert np.array_equal(x, xr), cases.rel_err(x, xr)
    assert np.array_equal(v, vr)


def test_batched_population_against_oracle(capi, exact_oracle):
    beams = wl.beam_population(256, seed=3, members=range(0, 256, 16))
    steps = 3
    methods = {kw["method"] for _, kw in beams}
    assert methods == {"large", "polar"}
    ref = []
    for mesh, kw in beams:
        ofem = exact_oracle.OracleFEM(mesh.positions, mesh.tetrahedra, kw["young"], kw["poisson"], kw["method"])
        osc = exact_oracle.OracleScene(ofem, vertex_mass=kw["total_mass"] / mesh.n_nodes, fixed=mesh.fixed,
                                       dt=kw["dt"], rayleigh_stiffness=kw["rayleigh_stiffness"],
                                       rayleigh_mass=kw["rayleigh_mass"], cg_iterations=kw["cg_iterations"],
                                       cg_tolerance=kw["cg_tolerance"], cg_threshold=kw["cg_threshold"])
        osc.step(steps)
        ref.append(osc.state()[0])
        del osc, ofem
    for precision, tol in (("fp64_fma", 1e-9), ("mixed", 1e-4)):
        b = capi.Batch(precision, budget_bytes=4 << 30, max_meshes=len(beams) + 1)
        slots = b.add_meshes([(m.positions, m.tetrahedra, kw) for m, kw in beams], threads=8)
        b.step(steps)
        for s, (mesh, kw), xr in zip(slots, beams, ref):
            x = b.state(s)[0]
            assert cases.rel_err(x, xr) <= tol, (precision, kw["method"], mesh.n_nodes)
        b.close()
