"""The synthetic workloads the benchmark and the large-mesh parity tests run.

All inputs are seeded synthetic meshes; no dataset is involved.

* ``SINGLE_BEAM``: one cantilever beam of 64x64x257 nodes (1,052,672 nodes,
  5,080,320 tetrahedra), spacing 0.5, interior jitter 0.05*spacing, 5-tet
  split, E=5000, nu=0.45, method polar, total mass 1, gravity -9.81 y, z=0
  fixed, dt=0.01, Rayleigh 0.1/0.1, CG 50 iterations, tolerance 1e-7,
  threshold 1e-9 (the CGLinearSolver default threshold 1e-5 is replaced by
  1e-9, since the tolerance is 1e-7).
* ``beam_population``: the beams of the batched and serving workloads.
* ``INCLUSION``: the ill-conditioned block with a stiff spherical inclusion.
"""
from __future__ import annotations

import numpy as np

from . import topology as topo

SINGLE_BEAM = dict(n=(64, 64, 257), spacing=0.5, jitter=0.05, seed=0, young=5000.0, poisson=0.45, method="polar",
                   dt=0.01, rs=0.1, rm=0.1, cg_iterations=50, cg_tolerance=1e-7, cg_threshold=1e-9, total_mass=1.0,
                   gravity=(0.0, -9.81, 0.0))

INCLUSION = dict(n=(48, 48, 193), young_out=1e3, young_in=1e6, poisson=0.49, method="polar", cg_iterations=200,
                 cg_tolerance=1e-10, replace_every=20, seed=0, dt=0.01, rs=0.1, rm=0.1, gravity=(0.0, -9.81, 0.0))


def single_beam_mesh(cfg=SINGLE_BEAM):
    return topo.beam(cfg["n"], spacing=cfg["spacing"], jitter=cfg["jitter"], seed=cfg["seed"], split=5)


def single_beam_solver(cfg, mesh):
    """Scene keyword arguments of the single-beam workload (capi.Scene)."""
    return dict(dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"],
                cg_iterations=cfg["cg_iterations"], cg_tolerance=cfg["cg_tolerance"],
                cg_threshold=cfg["cg_threshold"], gravity=cfg["gravity"],
                vertex_mass=cfg["total_mass"] / mesh.n_nodes, fixed=mesh.fixed)


def beam_population(n, seed, members=None):
    """Beams of the batched and serving workloads: node counts log-uniform in
    [1e3, 2e5], aspect z:x uniform in [2, 8], youngModulus log-uniform in
    [1e3, 1e5], poissonRatio uniform in [0.3, 0.49], method large or polar at
    50/50; dt 0.01, Rayleigh 0.1/0.1, CG 25 iterations with the
    CGLinearSolver default tolerance and threshold (1e-5), total mass 1,
    z = 0 fixed. Returns [(mesh, keyword arguments of capi.Batch.add_mesh)]
    for the n beams, or for the indices in `members` only (the same beams
    as in the whole population)."""
    rng = np.random.default_rng(seed)
    out = []
    keep = set(range(n)) if members is None else set(members)
    for i in range(n):
        nn = 10 ** rng.uniform(3.0, np.log10(2e5))
        dims = topo.beam_dims(nn, rng.uniform(2.0, 8.0))
        kw = dict(young=float(10 ** rng.uniform(3, 5)), poisson=float(rng.uniform(0.3, 0.49)),
                  method="large" if rng.random() < 0.5 else "polar")
        if i not in keep:
            continue
        mesh = topo.beam(dims, 0.5, 0.05, seed * 100003 + i)
        kw.update(dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=25, cg_tolerance=1e-5,
                  cg_threshold=1e-5, total_mass=1.0, fixed=mesh.fixed)
        out.append((mesh, kw))
    return out


def inclusion_block(cfg=INCLUSION):
    return topo.inclusion_beam(cfg["n"], seed=cfg["seed"], young_out=cfg["young_out"], young_in=cfg["young_in"])
