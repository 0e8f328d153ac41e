"""ctypes wrapper of the CPU oracle (oracle/tfem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py. The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "libtfem_oracle.so")
_REF_LIB = os.path.join(_HERE, "_ref", "libsofa_ref_math.so")

METHODS = {"small": 0, "large": 1, "polar": 2, "svd": 3}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lib = None


def build():
    """Compile the oracle with its Makefile (gcc, a second or two)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "tfem_oracle.c")):
        build()
    lib = ctypes.CDLL(_LIB)
    vp = ctypes.c_void_p
    lib.orc_fem_create.restype = vp
    lib.orc_fem_create.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _dp, ctypes.c_int, _dp, ctypes.c_int,
                                   _dp, ctypes.c_int, ctypes.c_int]
    lib.orc_fem_destroy.argtypes = [vp]
    lib.orc_fem_add_force.argtypes = [vp, _dp, _dp]
    lib.orc_fem_add_dforce.argtypes = [vp, _dp, _dp, ctypes.c_double]
    lib.orc_fem_element.argtypes = [vp, ctypes.c_int, _dp]
    lib.orc_fem_rest_volume.restype = ctypes.c_double
    lib.orc_fem_rest_volume.argtypes = [vp]
    lib.orc_fem_set_plasticity.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    lib.orc_fem_set_update_stiffness.argtypes = [vp, ctypes.c_int]
    lib.orc_fem_plastic_strain.argtypes = [vp, _dp]
    lib.orc_fem_von_mises.restype = ctypes.c_int
    lib.orc_fem_von_mises.argtypes = [vp, ctypes.c_int, _dp, _dp, _dp]
    lib.orc_polar.restype = ctypes.c_double
    lib.orc_polar.argtypes = [_dp, _dp]
    lib.orc_polar_stable.restype = ctypes.c_int
    lib.orc_polar_stable.argtypes = [_dp, _dp]
    lib.orc_set_threads.argtypes = [ctypes.c_int]
    lib.orc_set_exact_parallel.argtypes = [ctypes.c_int]
    lib.orc_get_threads.restype = ctypes.c_int
    lib.orc_scene_create.restype = vp
    lib.orc_scene_create.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp, _ip, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.orc_scene_destroy.argtypes = [vp]
    lib.orc_scene_set_state.argtypes = [vp, _dp, _dp]
    lib.orc_scene_get_state.argtypes = [vp, _dp, _dp]
    lib.orc_scene_set_external_force.argtypes = [vp, _dp]
    lib.orc_scene_set_springs.argtypes = [vp, ctypes.c_double, _dp]
    lib.orc_scene_step.argtypes = [vp, ctypes.c_int]
    lib.orc_scene_set_solver.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.orc_scene_set_warm_start.argtypes = [vp, ctypes.c_int]
    lib.orc_scene_set_options.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    lib.orc_scene_set_trapezoidal.argtypes = [vp, ctypes.c_int]
    lib.orc_scene_set_compute_residual.argtypes = [vp, ctypes.c_int]
    lib.orc_scene_set_separate_gravity.argtypes = [vp, ctypes.c_int]
    lib.orc_scene_residual.restype = ctypes.c_double
    lib.orc_scene_residual.argtypes = [vp]
    lib.orc_scene_jacobi.argtypes = [vp, _dp]
    lib.orc_scene_compute_force.argtypes = [vp, _dp]
    lib.orc_scene_last_iterations.restype = ctypes.c_int
    lib.orc_scene_last_iterations.argtypes = [vp]
    lib.orc_scene_last_error.restype = ctypes.c_double
    lib.orc_scene_last_error.argtypes = [vp]
    _lib = lib
    return lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


def set_threads(n, exact=False):
    """Threads of the oracle's element loops and vector operations. exact:
    element terms gathered per node in element order, bit-identical to one
    thread (the parity checker for large meshes); otherwise thread-local
    force buffers merged after the loop, as the MultiThreading plugin does
    (the CPU timing baseline)."""
    lib = _load()
    lib.orc_set_threads(int(n))
    lib.orc_set_exact_parallel(1 if exact else 0)


def polar(M):
    lib = _load()
    M, pm = _d(np.asarray(M, dtype=np.float64).reshape(3, 3))
    Q = np.zeros((3, 3))
    _, pq = _d(Q)
    det = lib.orc_polar(pm, Q.ctypes.data_as(_dp))
    return Q, det


def polar_stable(M):
    """Decompose<double>::polarDecomposition_stable restated: (Q, degenerate or inverted)."""
    lib = _load()
    M, pm = _d(np.asarray(M, dtype=np.float64).reshape(3, 3))
    Q = np.zeros((3, 3))
    deg = lib.orc_polar_stable(pm, Q.ctypes.data_as(_dp))
    return Q, bool(deg)


class OracleFEM:
    """TetrahedronFEMForceField restated on the CPU in FP64."""

    def __init__(self, rest, tets, young=5000.0, poisson=0.45, method="large", local_stiffness_factor=None):
        lib = _load()
        self._rest, prest = _d(np.asarray(rest).reshape(-1, 3))
        self._tets, ptets = _i(np.asarray(tets).reshape(-1, 4))
        self._young, py = _d(np.atleast_1d(np.asarray(young, dtype=np.float64)))
        self._poisson, pp = _d(np.atleast_1d(np.asarray(poisson, dtype=np.float64)))
        if local_stiffness_factor is None:
            self._lsf, pl, nl = np.zeros(1), None, 0
        else:
            self._lsf, pl = _d(np.atleast_1d(local_stiffness_factor))
            nl = self._lsf.size
        self.n_nodes = self._rest.shape[0]
        self.n_tets = self._tets.shape[0]
        self.method = method
        self._h = lib.orc_fem_create(self.n_nodes, prest, self.n_tets, ptets, py, self._young.size, pp,
                                     self._poisson.size, pl if pl is not None else _dp(), nl, METHODS[method])

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_fem_destroy(self._h)
            self._h = None

    def add_force(self, x, f=None):
        x, px = _d(np.asarray(x).reshape(-1, 3))
        f = np.zeros_like(x) if f is None else np.array(f, dtype=np.float64, copy=True).reshape(-1, 3)
        _load().orc_fem_add_force(self._h, px, f.ctypes.data_as(_dp))
        return f

    def add_dforce(self, dx, kfactor, df=None):
        dx, pdx = _d(np.asarray(dx).reshape(-1, 3))
        df = np.zeros_like(dx) if df is None else np.array(df, dtype=np.float64, copy=True).reshape(-1, 3)
        _load().orc_fem_add_dforce(self._h, pdx, df.ctypes.data_as(_dp), float(kfactor))
        return df

    def element(self, e):
        out = np.zeros(45)
        _load().orc_fem_element(self._h, int(e), out.ctypes.data_as(_dp))
        return {
            "initial_rotation": out[0:9].reshape(3, 3),  # _initialRotations[e] (R0^T)
            "rotation": out[9:18].reshape(3, 3),  # rotations[e] (R^T)
            "rotated_rest": out[18:30].reshape(4, 3),
            "K3": out[30:33].copy(),
            "J3": out[33:45].reshape(4, 3),
        }

    @property
    def rest_volume(self):
        return _load().orc_fem_rest_volume(self._h)

    def set_plasticity(self, max_threshold, yield_threshold=1e-4, creep=0.9):
        """plasticMaxThreshold / plasticYieldThreshold / plasticCreep."""
        _load().orc_fem_set_plasticity(self._h, max_threshold, yield_threshold, creep)

    def set_update_stiffness(self, on=True):
        """updateStiffnessMatrix (methods polar and svd)."""
        _load().orc_fem_set_update_stiffness(self._h, int(bool(on)))

    def von_mises(self, x, mode):
        """computeVonMisesStress at x: (per element, per node)."""
        x, px = _d(np.asarray(x).reshape(-1, 3))
        e, pe = _d(np.zeros(self.n_tets))
        n, pn = _d(np.zeros(self.n_nodes))
        if _load().orc_fem_von_mises(self._h, int(mode), px, pe, pn) != 0:
            raise ValueError("von Mises mode 1 needs method large, polar or svd")
        return e, n

    def plastic_strain(self):
        """(n_tets, 6) plastic strain."""
        out, pout = _d(np.zeros(6 * self.n_tets))
        _load().orc_fem_plastic_strain(self._h, pout)
        return out.reshape(-1, 6)


def full_K(K3):
    """The 6x6 material stiffness from its three distinct values."""
    k0, k1, k2 = K3
    K = np.zeros((6, 6))
    K[:3, :3] = k1
    np.fill_diagonal(K[:3, :3], k0)
    K[3, 3] = K[4, 4] = K[5, 5] = k2
    return K


def full_J(J3):
    """The 12x6 strain-displacement matrix from its 12 distinct values."""
    J = np.zeros((12, 6))
    for i in range(4):
        a, b, c = J3[i]
        J[3 * i, 0] = J[3 * i + 1, 3] = J[3 * i + 2, 5] = a
        J[3 * i, 3] = J[3 * i + 1, 1] = J[3 * i + 2, 4] = b
        J[3 * i, 5] = J[3 * i + 1, 4] = J[3 * i + 2, 2] = c
    return J


class OracleScene:
    """MechanicalObject + mass + FEM + FixedProjectiveConstraint integrated by
    EulerImplicitSolver / CGLinearSolver, all FP64 on the CPU."""

    def __init__(self, fem, n_nodes=None, vertex_mass=None, node_masses=None, gravity=(0.0, -9.81, 0.0),
                 fixed=(), fix_all=False, dt=0.01, rayleigh_stiffness=0.0, rayleigh_mass=0.0, vdamping=0.0,
                 cg_iterations=25, cg_tolerance=1e-5, cg_threshold=1e-5, mass_first=True):
        lib = _load()
        self.fem = fem
        n = fem.n_nodes if fem is not None else int(n_nodes)
        self.n_nodes = n
        if node_masses is not None:
            kind, vm = 1, 0.0
            self._nm, pnm = _d(node_masses)
        else:
            kind, vm = 0, float(vertex_mass)
            self._nm, pnm = _d(np.zeros(1))
        self._g, pg = _d(np.asarray(gravity, dtype=np.float64))
        self._fixed, pf = _i(np.asarray(fixed, dtype=np.int32) if len(fixed) else np.zeros(1, np.int32))
        self._h = lib.orc_scene_create(fem._h if fem is not None else None, n, kind, vm, pnm, pg, pf, len(fixed),
                                       int(fix_all), dt, rayleigh_stiffness, rayleigh_mass, vdamping,
                                       int(cg_iterations), cg_tolerance, cg_threshold, int(mass_first))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_scene_destroy(self._h)
            self._h = None

    def set_state(self, x=None, v=None):
        xa, px = _d(np.asarray(x).reshape(-1, 3)) if x is not None else (None, _dp())
        va, pv = _d(np.asarray(v).reshape(-1, 3)) if v is not None else (None, _dp())
        _load().orc_scene_set_state(self._h, px, pv)

    def state(self):
        x = np.zeros((self.n_nodes, 3))
        v = np.zeros((self.n_nodes, 3))
        _load().orc_scene_get_state(self._h, x.ctypes.data_as(_dp), v.ctypes.data_as(_dp))
        return x, v

    def set_external_force(self, fext):
        self._ext, p = _d(np.asarray(fext).reshape(-1, 3))
        _load().orc_scene_set_external_force(self._h, p)

    def set_springs(self, k, anchor):
        self._anchor, p = _d(np.asarray(anchor).reshape(-1, 3))
        _load().orc_scene_set_springs(self._h, float(k), p)

    def set_warm_start(self, on=True):
        """CGLinearSolver warmStart."""
        _load().orc_scene_set_warm_start(self._h, int(on))

    def set_options(self, ff_rayleigh_stiffness=0.0, mass_rayleigh_mass=0.0, first_order=False,
                    project_velocity=False, trapezoidal_scheme=False):
        """The force field's and the mass's own Rayleigh coefficients,
        EulerImplicitSolver firstOrder and trapezoidalScheme,
        FixedProjectiveConstraint activate_projectVelocity."""
        lib = _load()
        lib.orc_scene_set_options(self._h, float(ff_rayleigh_stiffness), float(mass_rayleigh_mass),
                                  int(first_order), int(project_velocity))
        lib.orc_scene_set_trapezoidal(self._h, int(trapezoidal_scheme))

    def set_solver(self, solver="cg", preconditioner=None, rate=1):
        """solver "cg" (CGLinearSolver) or "pcg" (PCGLinearSolver, warm start);
        preconditioner None or "jacobi" (JacobiPreconditioner), re-assembled
        every `rate` steps."""
        _load().orc_scene_set_solver(self._h, {"cg": 0, "pcg": 1}[solver],
                                     {None: 0, "jacobi": 1}[preconditioner], int(rate))

    def jacobi(self):
        """The last solve's inverse Jacobi diagonal (n x 3)."""
        out = np.zeros((self.n_nodes, 3))
        _load().orc_scene_jacobi(self._h, out.ctypes.data_as(_dp))
        return out

    def step(self, n=1):
        _load().orc_scene_step(self._h, int(n))

    def compute_force(self):
        f = np.zeros((self.n_nodes, 3))
        _load().orc_scene_compute_force(self._h, f.ctypes.data_as(_dp))
        return f

    @property
    def last_iterations(self):
        return _load().orc_scene_last_iterations(self._h)

    @property
    def last_error(self):
        return _load().orc_scene_last_error(self._h)

    def set_separate_gravity(self, on=True):
        """The mass's separateGravity."""
        _load().orc_scene_set_separate_gravity(self._h, int(bool(on)))

    def set_compute_residual(self, on=True):
        """EulerImplicitSolver computeResidual."""
        _load().orc_scene_set_compute_residual(self._h, int(bool(on)))

    @property
    def residual(self):
        """EulerImplicitSolver's Data `residual` after the last step."""
        return _load().orc_scene_residual(self._h)


def ref_math_lib():
    """The reference's own polar decomposition, compiled from the reference
    sources by oracle/ref/Makefile. The reference tree is named by the
    SOFA_REFERENCE_ROOT environment variable; without it (or without the
    tree) this returns None unless the library was built before."""
    if not os.path.exists(_REF_LIB):
        ref = os.environ.get("SOFA_REFERENCE_ROOT", "")
        if not ref or not os.path.isdir(ref):
            return None
        try:
            subprocess.run(["make", "-s", "-C", os.path.join(_HERE, "ref"), f"REF={ref}"], check=True)
        except Exception:
            return None
    lib = ctypes.CDLL(_REF_LIB)
    lib.ref_polar_decomposition_d.restype = ctypes.c_double
    lib.ref_polar_decomposition_d.argtypes = [_dp, _dp]
    lib.ref_polar_decomposition_f.restype = ctypes.c_float
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ref_polar_decomposition_f.argtypes = [fp, fp]
    lib.ref_polar_decomposition_stable_d.restype = ctypes.c_int
    lib.ref_polar_decomposition_stable_d.argtypes = [_dp, _dp]
    return lib
