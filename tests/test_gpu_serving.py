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
