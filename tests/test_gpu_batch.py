"""Batched multi-mesh engine on the GPU: results are independent of the
other meshes in the batch (bit-identical alone and in the mix), match the
FP64 oracle for the FP64 variant, and admission respects the HBM budget."""
import numpy as np
import pytest

from sofa_gb300 import topology as topo
from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


def beam_kw(mesh, young=5000.0, poisson=0.45, method="large", iters=25, tol=1e-9):
    return dict(young=young, poisson=poisson, method=method, dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1,
                cg_iterations=iters, cg_tolerance=tol, cg_threshold=1e-9, total_mass=1.0, fixed=mesh.fixed)


MESHES = [((5, 5, 21), 0, 5000.0, 0.45, "large"), ((4, 6, 17), 1, 2e4, 0.3, "polar"),
          ((7, 5, 12), 2, 1e3, 0.49, "large"), ((3, 3, 30), 3, 1e5, 0.4, "polar")]


@pytest.mark.parametrize("precision", ["mixed", "fp64_fma"])
def test_alone_and_in_mix_bit_identical(capi, precision):
    meshes = [(topo.beam(n, 0.5, 0.05, seed), E, nu, m) for n, seed, E, nu, m in MESHES]
    alone = []
    for mesh, E, nu, m in meshes:
        b = capi.Batch(precision, budget_bytes=64 << 20, max_meshes=4)
        s = b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh, E, nu, m))
        b.step(20)
        alone.append(b.state(s)[0])
        b.close()
    b = capi.Batch(precision, budget_bytes=256 << 20, max_meshes=8)
    slots = [b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh, E, nu, m)) for mesh, E, nu, m in meshes]
    b.step(20)
    for s, xa in zip(slots, alone):
        assert np.array_equal(b.state(s)[0], xa)


def test_fp64_batch_matches_oracle(capi, oracle):
    mesh = cases.beam_mesh()
    _, osc = cases.oracle_scene(oracle, mesh, "large")
    osc.step(100)
    xr, _ = osc.state()
    b = capi.Batch("fp64_fma", budget_bytes=64 << 20, max_meshes=2)
    s = b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    b.step(100)
    x, _ = b.state(s)
    assert cases.rel_err(x, xr) <= 1e-10
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr - mesh.positions) <= 1e-7


def test_mixed_batch_trajectory(capi):
    mesh = cases.beam_mesh()
    ref = capi.Batch("fp64_fma", budget_bytes=64 << 20, max_meshes=2)
    sr = ref.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    ref.step(100)
    xr, _ = ref.state(sr)
    mx = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=2)
    sm = mx.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    mx.step(100)
    x, _ = mx.state(sm)
    assert cases.rel_err(x, xr) <= 1e-4


def test_admission_budget_and_slot_reuse(capi):
    mesh = topo.beam((6, 6, 30), 0.5, 0.05, 0)
    b = capi.Batch("mixed", budget_bytes=16 << 20, max_meshes=64)
    need = b.mesh_bytes(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    fits = (16 << 20) // need
    slots = []
    for _ in range(fits):
        slots.append(b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh)))
    with pytest.raises(capi.SgbError) as e:
        b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    assert e.value.code == -6 and "budget" in str(e.value)
    b.step(3)
    b.remove_mesh(slots[0])
    s_new = b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    assert s_new == slots[0]
    b.step(3)
    # the re-admitted mesh restarted from rest: after 3 steps it equals a mesh
    # that has run 3 steps alone
    x_new = b.state(s_new)[0]
    ref = capi.Batch("mixed", budget_bytes=16 << 20, max_meshes=1)
    sr = ref.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh))
    ref.step(3)
    assert np.array_equal(x_new, ref.state(sr)[0])
    info = b.info()
    assert info["meshes"] == fits and info["budget_used"] <= info["budget_total"]


def test_external_force_and_per_mesh_iterations(capi):
    mesh = cases.beam_mesh((4, 4, 12))
    ext = np.zeros((mesh.n_nodes, 3))
    tip = np.nonzero(np.isclose(mesh.positions[:, 2], mesh.positions[:, 2].max()))[0]
    ext[tip, 1] = -0.5
    b = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=2, max_cg_iterations=40)
    s1 = b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh, iters=10))
    s2 = b.add_mesh(mesh.positions, mesh.tetrahedra, external_force=ext, **beam_kw(mesh, iters=40))
    b.step(5)
    it1, _, st1 = b.stats(s1)
    it2, _, st2 = b.stats(s2)
    assert it1 <= 10 and it2 <= 40 and st1 == st2 == 5
    y1 = b.state(s1)[0][tip, 1].mean()
    y2 = b.state(s2)[0][tip, 1].mean()
    assert y2 < y1  # the traction pulls the tip further down


TILES = [dict(matvec_ctas_per_sm=8, update_nodes_per_thread=1, update_ctas_per_sm=2, elem_ctas_per_sm=8, prefetch=1),
         dict(matvec_ctas_per_sm=5, update_nodes_per_thread=2, update_ctas_per_sm=8, elem_ctas_per_sm=2, prefetch=0)]


@pytest.mark.parametrize("precision", ["mixed", "fp64_fma"])
def test_tiles_are_rounding_neutral(capi, precision):
    """Every launch tile the tuner can pick gives the same bits: the mix with
    non-default tiles equals each mesh run alone with the default tiles."""
    meshes = [(topo.beam(n, 0.5, 0.05, seed), E, nu, m) for n, seed, E, nu, m in MESHES]
    alone = []
    for mesh, E, nu, m in meshes:
        b = capi.Batch(precision, budget_bytes=64 << 20, max_meshes=4)
        s = b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh, E, nu, m))
        b.step(15)
        alone.append(b.state(s)[0])
        b.close()
    for tiles in TILES:
        b = capi.Batch(precision, budget_bytes=256 << 20, max_meshes=8)
        slots = [b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh, E, nu, m))
                 for mesh, E, nu, m in meshes]
        b.set_tiles(**tiles)
        b.step(15)
        for s, xa in zip(slots, alone):
            assert np.array_equal(b.state(s)[0], xa), tiles
        b.close()


def test_tuner_keeps_state_and_results(capi):
    """sgb_batch_tune times whole steps but restores every mesh's state: a
    batch tuned after 5 steps and stepped 5 more equals one stepped 10."""
    meshes = [(topo.beam(n, 0.5, 0.05, seed), E, nu, m) for n, seed, E, nu, m in MESHES]
    res = []
    for tune in (False, True):
        b = capi.Batch("mixed", budget_bytes=256 << 20, max_meshes=8)
        slots = [b.add_mesh(mesh.positions, mesh.tetrahedra, **beam_kw(mesh, E, nu, m))
                 for mesh, E, nu, m in meshes]
        b.step(5)
        if tune:
            info = b.tune(steps_per_trial=2, use_cache=False)
            assert info["trials"] >= 10 and info["tuned_ms_per_step"] > 0
            assert info["tuned_ms_per_step"] <= info["default_ms_per_step"]
            assert all(b.stats(s)[2] == 5 for s in slots)  # step counters restored
            again = b.tune(use_cache=True)  # the same mix: answered by the cache
            assert again["trials"] == 0
        b.step(5)
        res.append([b.state(s) for s in slots])
        b.close()
    for (xa, va), (xb, vb) in zip(*res):
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_patch_size_tuning(capi, monkeypatch):
    """Elements per patch chosen by timing a sample before admission: the
    choice is one of the candidates, a batch admits and steps with it exactly
    as a batch created with that patch size, and the choice is refused once
    meshes are admitted."""
    meshes = [(topo.beam(n, 0.5, 0.05, seed), E, nu, m) for n, seed, E, nu, m in MESHES]
    sample = [(mesh.positions, mesh.tetrahedra, beam_kw(mesh, E, nu, m)) for mesh, E, nu, m in meshes]
    b = capi.Batch("mixed", budget_bytes=256 << 20, max_meshes=8)
    chosen, ms = b.tune_patch_size(sample, steps_per_trial=2)
    assert chosen in (256, 384, 512) and sorted(ms) == [256, 384, 512] and all(v > 0 for v in ms.values())
    assert b.tuning()["elements_per_patch"] == chosen
    slots = [b.add_mesh(pos, tets, **kw) for pos, tets, kw in sample]
    b.step(10)
    got = [b.state(s)[0] for s in slots]
    with pytest.raises(capi.SgbError) as e:
        b.tune_patch_size(sample)
    assert e.value.code == -4
    b.close()
    monkeypatch.setenv("SGB_BATCH_PE", str(chosen))
    ref = capi.Batch("mixed", budget_bytes=256 << 20, max_meshes=8)
    rslots = [ref.add_mesh(pos, tets, **kw) for pos, tets, kw in sample]
    ref.step(10)
    for s, x in zip(rslots, got):
        assert np.array_equal(ref.state(s)[0], x)
    ref.close()
