"""Continuous-batching serving loop on the GPU: requests that overlap on the
device give the same result as the same request run alone (bit-identical:
a mesh's arithmetic does not depend on the other meshes in the batch), an
oversized request fails alone, and latency statistics are reported."""
import time

import numpy as np
import pytest

from sofa_gb300 import topology as topo

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


def request_set(seed=0, count=12):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        n = (int(rng.integers(3, 7)), int(rng.integers(3, 7)), int(rng.integers(8, 25)))
        mesh = topo.beam(n, 0.5, 0.05, int(rng.integers(1 << 20)))
        kw = dict(young=float(10 ** rng.uniform(3, 5)), poisson=float(rng.uniform(0.3, 0.49)),
                  method="large" if i % 2 == 0 else "polar", dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1,
                  cg_iterations=25, cg_tolerance=1e-5, cg_threshold=1e-9, total_mass=1.0, fixed=mesh.fixed)
        reqs.append((mesh, int(rng.integers(1, 40)), kw))
    return reqs


def test_results_same_alone_and_in_the_mix(capi):
    reqs = request_set()
    srv = capi.Server("mixed", budget_bytes=256 << 20, max_meshes=16, prep_threads=3, max_steps_per_launch=4)
    outs = []
    for i, (mesh, k, kw) in enumerate(reqs):
        outs.append(srv.submit(mesh.positions, mesh.tetrahedra, k, **kw))
        if i % 3 == 2:
            time.sleep(0.01)  # arrivals spread out: later ones join running batches
    srv.wait_idle(300)
    done = {c["id"]: c for c in srv.poll()}
    assert len(done) == len(reqs) and all(c["status"] == 0 for c in done.values())
    for (rid, out), (mesh, k, kw) in zip(outs, reqs):
        b = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=1)
        s = b.add_mesh(mesh.positions, mesh.tetrahedra, **kw)
        b.step(k)
        alone = b.state(s)[0]
        b.close()
        assert np.array_equal(out, alone), rid
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()


def test_oversized_request_fails_alone(capi):
    small = topo.beam((4, 4, 10), 0.5, 0.05, 0)
    big = topo.beam((12, 12, 60), 0.5, 0.05, 0)
    kw = lambda m: dict(method="large", dt=0.01, cg_iterations=10, total_mass=1.0, fixed=m.fixed)
    srv = capi.Server("mixed", budget_bytes=8 << 20, max_meshes=4, prep_threads=2)
    a, _ = srv.submit(small.positions, small.tetrahedra, 5, **kw(small))
    b, _ = srv.submit(big.positions, big.tetrahedra, 5, **kw(big))
    c, _ = srv.submit(small.positions, small.tetrahedra, 5, **kw(small))
    srv.wait_idle(120)
    done = {x["id"]: x for x in srv.poll()}
    assert done[a]["status"] == 0 and done[c]["status"] == 0
    assert done[b]["status"] == -6
    srv.close()


def alone_result(capi, mesh, k, kw):
    b = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=1)
    s = b.add_mesh(mesh.positions, mesh.tetrahedra, **kw)
    b.step(k)
    x = b.state(s)[0]
    b.close()
    return x


def small_kw(mesh):
    return dict(method="polar", young=3000.0, poisson=0.4, dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1,
                cg_iterations=25, cg_tolerance=1e-5, cg_threshold=1e-9, total_mass=1.0, fixed=mesh.fixed)


def wait_running_then(srv, rid, action, timeout=5.0):
    """Retries `action(rid)` until the request is on the GPU (the call stops
    raising SGB_ERR_NOT_FOUND)."""
    t0 = time.time()
    while True:
        try:
            action(rid)
            return
        except Exception as e:  # noqa: BLE001 - SgbError(-7) while still queued
            if getattr(e, "code", None) != -7 or time.time() - t0 > timeout:
                raise
            time.sleep(0.005)


def one_mesh_budget(capi, mesh, kw):
    """An HBM budget with room for one such mesh at a time."""
    one = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=1).mesh_bytes(mesh.positions, mesh.tetrahedra, **kw)
    assert one > (1 << 20)  # the smallest budget a batch takes is 1 MiB
    return int(one * 1.5)


def test_cancel_queued_and_running(capi):
    mesh = topo.beam((8, 8, 20), 0.5, 0.05, 3)
    kw = small_kw(mesh)
    # room for one mesh at a time: the later requests wait in the queue
    srv = capi.Server("mixed", budget_bytes=one_mesh_budget(capi, mesh, kw), max_meshes=4, prep_threads=2,
                      max_steps_per_launch=4)
    a, _ = srv.submit(mesh.positions, mesh.tetrahedra, 4000, **kw)
    b, _ = srv.submit(mesh.positions, mesh.tetrahedra, 5, **kw)
    c, out_c = srv.submit(mesh.positions, mesh.tetrahedra, 7, **kw)
    srv.cancel(b)  # queued
    wait_running_then(srv, a, srv.cancel)  # running: removed at the next launch boundary
    srv.wait_idle(120)
    done = {x["id"]: x for x in srv.poll()}
    assert done[a]["status"] == -9 and done[b]["status"] == -9 and done[c]["status"] == 0
    assert np.array_equal(out_c, alone_result(capi, mesh, 7, kw))
    st = srv.stats()
    assert st["cancelled"] == 2 and st["completed"] == 1
    with pytest.raises(capi.SgbError) as e:
        srv.cancel(c)  # already completed
    assert e.value.code == -7
    srv.close()


def test_evicted_request_resumes_bit_exactly(capi):
    mesh = topo.beam((8, 8, 20), 0.5, 0.05, 4)
    other = topo.beam((7, 8, 18), 0.5, 0.05, 5)
    kw, kwo = small_kw(mesh), small_kw(other)
    srv = capi.Server("mixed", budget_bytes=one_mesh_budget(capi, mesh, kw), max_meshes=4, prep_threads=2,
                      max_steps_per_launch=4)
    k = 400
    a, out_a = srv.submit(mesh.positions, mesh.tetrahedra, k, **kw)
    b, out_b = srv.submit(other.positions, other.tetrahedra, 9, **kwo)
    wait_running_then(srv, a, srv.evict)  # a leaves the GPU; b (waiting) runs; then a resumes
    srv.wait_idle(120)
    done = {x["id"]: x for x in srv.poll()}
    assert done[a]["status"] == 0 and done[b]["status"] == 0
    st = srv.stats()
    assert st["evicted"] == 1
    assert np.array_equal(out_a, alone_result(capi, mesh, k, kw))
    assert np.array_equal(out_b, alone_result(capi, other, 9, kwo))
    assert st["step_p99_ms"] >= st["step_p50_ms"] > 0 and st["launches"] > 0
    srv.close()


def test_batch_save_and_restore_mesh(capi):
    mesh = topo.beam((5, 4, 14), 0.5, 0.05, 6)
    kw = small_kw(mesh)
    b = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=2)
    s = b.add_mesh(mesh.positions, mesh.tetrahedra, **kw)
    b.step(12)
    ref = b.state(s)
    b.close()
    b = capi.Batch("mixed", budget_bytes=64 << 20, max_meshes=2)
    s = b.add_mesh(mesh.positions, mesh.tetrahedra, **kw)
    b.step(5)
    x, v, steps = b.save_mesh(s)
    assert steps == 5
    b.remove_mesh(s)
    s2 = b.add_mesh(mesh.positions, mesh.tetrahedra, **kw)
    b.restore_mesh(s2, x, v, steps)
    b.step(7)
    got = b.state(s2)
    b.close()
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


def test_non_finite_input_fails_only_its_mesh(capi):
    """A NaN in one mesh's external force: that mesh reports
    SGB_ERR_NUMERICAL (batch statistics and the server completion), the
    others are bit-identical to their runs alone."""
    reqs = request_set(seed=9, count=4)
    bad = 2
    mesh_bad = reqs[bad][0]
    ext = np.zeros_like(mesh_bad.positions)
    ext[-1, 1] = np.nan
    b = capi.Batch("mixed", budget_bytes=256 << 20, max_meshes=8)
    slots = []
    for i, (mesh, k, kw) in enumerate(reqs):
        extra = dict(external_force=ext) if i == bad else {}
        slots.append(b.add_mesh(mesh.positions, mesh.tetrahedra, **kw, **extra))
    b.step(6)
    for i, (s, (mesh, k, kw)) in enumerate(zip(slots, reqs)):
        if i == bad:
            with pytest.raises(capi.SgbError) as e:
                b.stats(s)
            assert e.value.code == -5
        else:
            assert np.array_equal(b.state(s)[0], alone_result(capi, mesh, 6, kw))
    b.close()
    srv = capi.Server("mixed", budget_bytes=256 << 20, max_meshes=8, prep_threads=2, max_steps_per_launch=3)
    outs = []
    for i, (mesh, k, kw) in enumerate(reqs):
        extra = dict(external_force=ext) if i == bad else {}
        outs.append(srv.submit(mesh.positions, mesh.tetrahedra, k, **kw, **extra))
    srv.wait_idle(120)
    done = {x["id"]: x for x in srv.poll()}
    for i, ((rid, out), (mesh, k, kw)) in enumerate(zip(outs, reqs)):
        if i == bad:
            assert done[rid]["status"] == -5
        else:
            assert done[rid]["status"] == 0
            assert np.array_equal(out, alone_result(capi, mesh, k, kw))
    assert srv.stats()["failed"] == 1
    srv.close()
