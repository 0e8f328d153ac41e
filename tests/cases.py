"""Shared scene definitions for the parity tests (seeded, small enough for
the CPU oracle to run in seconds)."""
import numpy as np

from sofa_gb300 import topology as topo

# Cantilever beam of the small plain-method workload: 5x5x21 nodes, spacing
# 0.5, 5-tet split, interior jitter 0.05*spacing, E=5000, nu=0.45, total mass
# 1, gravity -9.81 y, z=0 fixed, dt 0.01, Rayleigh 0.1/0.1, CG 25/1e-9/1e-9.
BEAM_SMALL = dict(n=(5, 5, 21), young=5000.0, poisson=0.45, dt=0.01, rs=0.1, rm=0.1, cg_iterations=25,
                  cg_tolerance=1e-9, cg_threshold=1e-9, total_mass=1.0, gravity=(0.0, -9.81, 0.0))


def beam_mesh(n=(5, 5, 21), seed=0, split=5):
    return topo.beam(n, spacing=0.5, jitter=0.05, seed=seed, split=split)


def oracle_scene(oracle, mesh, method="large", cfg=BEAM_SMALL, young=None, poisson=None):
    fem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, cfg["young"] if young is None else young,
                           cfg["poisson"] if poisson is None else poisson, method)
    sc = oracle.OracleScene(fem, vertex_mass=cfg["total_mass"] / mesh.n_nodes, gravity=cfg["gravity"],
                            fixed=mesh.fixed, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"],
                            cg_iterations=cfg["cg_iterations"], cg_tolerance=cfg["cg_tolerance"],
                            cg_threshold=cfg["cg_threshold"])
    return fem, sc


def gpu_scene(capi, mesh, method="large", precision="fp64", cfg=BEAM_SMALL, serial_dots=False, young=None,
              poisson=None, **solver):
    """`solver`: linear_solver / preconditioner / preconditioner_rate of capi.Scene."""
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, cfg["young"] if young is None else young,
                              cfg["poisson"] if poisson is None else poisson, method, precision)
    return capi.Scene(fem, dt=cfg["dt"], rayleigh_stiffness=cfg["rs"], rayleigh_mass=cfg["rm"],
                      cg_iterations=cfg["cg_iterations"], cg_tolerance=cfg["cg_tolerance"],
                      cg_threshold=cfg["cg_threshold"], gravity=cfg["gravity"],
                      vertex_mass=cfg["total_mass"] / mesh.n_nodes, fixed=mesh.fixed, serial_dots=serial_dots,
                      **solver)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
