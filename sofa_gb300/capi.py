"""ctypes binding of libsofa_gb300.so (the C ABI declared in include/sofa_gb300.h).

This is plumbing for Python callers (tests, benchmarks, notebooks): every
numeric operation runs in the CUDA library. Loading fails loudly when the
library has not been built -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsofa_gb300.so")

SGB_OK = 0
ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "out of device memory",
    -4: "not supported",
    -5: "non-finite value in the CG solve",
    -6: "HBM budget exceeded",
    -7: "not found",
    -8: "a bounded device-side wait ran out",
}
METHODS = {"small": 0, "large": 1, "polar": 2, "svd": 3}
PRECISIONS = {"fp64": 0, "mixed": 1, "fp64_fma": 2}


class SgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SceneParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("rayleigh_stiffness", ctypes.c_double),
        ("rayleigh_mass", ctypes.c_double),
        ("vdamping", ctypes.c_double),
        ("cg_iterations", ctypes.c_int),
        ("cg_tolerance", ctypes.c_double),
        ("cg_threshold", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("vertex_mass", ctypes.c_double),
        ("node_masses_host", ctypes.POINTER(ctypes.c_double)),
        ("fixed_host", ctypes.POINTER(ctypes.c_int32)),
        ("n_fixed", ctypes.c_int),
        ("fix_all", ctypes.c_int),
        ("mass_first", ctypes.c_int),
        ("serial_dots", ctypes.c_int),
        ("residual_replacement", ctypes.c_int),
        ("linear_solver", ctypes.c_int),
        ("preconditioner", ctypes.c_int),
        ("preconditioner_rate", ctypes.c_int),
        ("warm_start", ctypes.c_int),
        ("ff_rayleigh_stiffness", ctypes.c_double),
        ("mass_rayleigh_mass", ctypes.c_double),
        ("first_order", ctypes.c_int),
        ("project_velocity", ctypes.c_int),
        ("trapezoidal_scheme", ctypes.c_int),
        ("compute_residual", ctypes.c_int),
        ("separate_gravity", ctypes.c_int),
    ]


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("n_nodes", ctypes.c_int),
        ("rest_positions_host", ctypes.POINTER(ctypes.c_double)),
        ("n_tets", ctypes.c_int),
        ("tetrahedra_host", ctypes.POINTER(ctypes.c_int32)),
        ("young", ctypes.POINTER(ctypes.c_double)),
        ("n_young", ctypes.c_int),
        ("poisson", ctypes.POINTER(ctypes.c_double)),
        ("n_poisson", ctypes.c_int),
        ("method", ctypes.c_int),
        ("params", SceneParams),
        ("external_force_host", ctypes.POINTER(ctypes.c_double)),
    ]


class Request(ctypes.Structure):
    _fields_ = [
        ("mesh", MeshDesc),
        ("n_steps", ctypes.c_int),
        ("positions_out_host", ctypes.POINTER(ctypes.c_double)),
        ("id", ctypes.c_uint64),
    ]


class Completion(ctypes.Structure):
    _fields_ = [
        ("id", ctypes.c_uint64),
        ("status", ctypes.c_int),
        ("latency_ms", ctypes.c_double),
        ("queue_ms", ctypes.c_double),
        ("cg_iterations_last", ctypes.c_int),
        ("n_tets", ctypes.c_longlong),
        ("n_steps", ctypes.c_int),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_longlong),
        ("completed", ctypes.c_longlong),
        ("failed", ctypes.c_longlong),
        ("tet_steps", ctypes.c_longlong),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("busy_s", ctypes.c_double),
        ("wall_s", ctypes.c_double),
        ("step_p50_ms", ctypes.c_double),
        ("step_p99_ms", ctypes.c_double),
        ("launches", ctypes.c_longlong),
        ("cancelled", ctypes.c_longlong),
        ("evicted", ctypes.c_longlong),
    ]


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p


def load():
    """Load the CUDA library (it must have been built with sofa_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m sofa_gb300.build` "
                          "(this package has no CPU implementation)")
    lib = ctypes.CDLL(LIB_PATH)
    c_int, c_double, c_float = ctypes.c_int, ctypes.c_double, ctypes.c_float
    sig = {
        "sgb_last_error": (ctypes.c_char_p, []),
        "sgb_version": (ctypes.c_char_p, []),
        "sgb_tfem_create": (c_int, [ctypes.POINTER(_vp), c_int, _dp, c_int, _ip, _dp, c_int, _dp, c_int, _dp, c_int,
                                    c_int, c_int]),
        "sgb_tfem_destroy": (c_int, [_vp]),
        "sgb_tfem_add_force": (c_int, [_vp, _vp, _vp, _vp]),
        "sgb_tfem_add_force_f32": (c_int, [_vp, _vp, _vp, _vp]),
        "sgb_tfem_add_dforce": (c_int, [_vp, _vp, _vp, c_double, _vp]),
        "sgb_tfem_add_dforce_f32": (c_int, [_vp, _vp, _vp, c_float, _vp]),
        "sgb_tfem_get_rotations": (c_int, [_vp, _dp, _dp]),
        "sgb_tfem_set_plasticity": (c_int, [_vp, c_double, c_double, c_double]),
        "sgb_tfem_set_update_stiffness": (c_int, [_vp, c_int]),
        "sgb_tfem_reset_plasticity": (c_int, [_vp]),
        "sgb_tfem_get_plastic_strain": (c_int, [_vp, _dp]),
        "sgb_tfem_stiffness_bsr": (c_int, [_vp, ctypes.POINTER(c_int), _ip, _ip, _dp]),
        "sgb_tfem_check_device": (c_int, [_vp]),
        "sgb_tfem_info": (c_int, [_vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                  ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_size_t)]),
        "sgb_scene_params_default": (None, [ctypes.POINTER(SceneParams)]),
        "sgb_scene_create": (c_int, [ctypes.POINTER(_vp), _vp, ctypes.POINTER(SceneParams)]),
        "sgb_scene_destroy": (c_int, [_vp]),
        "sgb_scene_step": (c_int, [_vp, c_int]),
        "sgb_scene_sync": (c_int, [_vp, ctypes.POINTER(c_int), _dp]),
        "sgb_scene_residual": (c_int, [_vp, _dp]),
        "sgb_scene_von_mises": (c_int, [_vp, c_int, _dp, _dp]),
        "sgb_tfem_von_mises": (c_int, [_vp, c_int, _vp, _vp, _vp, _vp]),
        "sgb_scene_get_state": (c_int, [_vp, _dp, _dp]),
        "sgb_scene_set_state": (c_int, [_vp, _dp, _dp]),
        "sgb_scene_set_external_force": (c_int, [_vp, _dp]),
        "sgb_scene_state_device": (c_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
        "sgb_scene_stream": (_vp, [_vp]),
        "sgb_batch_create": (c_int, [ctypes.POINTER(_vp), c_int, ctypes.c_size_t, c_int, c_int]),
        "sgb_batch_destroy": (c_int, [_vp]),
        "sgb_batch_mesh_bytes": (c_int, [_vp, ctypes.POINTER(MeshDesc), ctypes.POINTER(ctypes.c_size_t)]),
        "sgb_batch_add_mesh": (c_int, [_vp, ctypes.POINTER(MeshDesc), ctypes.POINTER(c_int)]),
        "sgb_batch_remove_mesh": (c_int, [_vp, c_int]),
        "sgb_batch_add_meshes": (c_int, [_vp, ctypes.POINTER(MeshDesc), c_int, ctypes.POINTER(c_int), c_int]),
        "sgb_batch_step": (c_int, [_vp, c_int]),
        "sgb_batch_sync": (c_int, [_vp]),
        "sgb_batch_mesh_stats": (c_int, [_vp, c_int, ctypes.POINTER(c_int), _dp, ctypes.POINTER(ctypes.c_longlong)]),
        "sgb_batch_get_state": (c_int, [_vp, c_int, _dp, _dp]),
        "sgb_batch_get_positions_async": (c_int, [_vp, c_int, _dp]),
        "sgb_batch_set_state": (c_int, [_vp, c_int, _dp, _dp]),
        "sgb_batch_info": (c_int, [_vp, ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_longlong),
                                   ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
        "sgb_batch_stream": (_vp, [_vp]),
        "sgb_batch_tune": (c_int, [_vp, c_int, c_int]),
        "sgb_batch_tune_patch_size": (c_int, [_vp, ctypes.POINTER(MeshDesc), c_int, c_int, ctypes.POINTER(c_int),
                                              _dp]),
        "sgb_batch_set_tiles": (c_int, [_vp, ctypes.POINTER(c_int)]),
        "sgb_batch_get_tiles": (c_int, [_vp, ctypes.POINTER(c_int), _dp, _dp, ctypes.POINTER(c_int)]),
        "sgb_server_create": (c_int, [ctypes.POINTER(_vp), c_int, ctypes.c_size_t, c_int, c_int, c_int, c_int]),
        "sgb_server_submit": (c_int, [_vp, ctypes.POINTER(Request)]),
        "sgb_server_poll": (c_int, [_vp, ctypes.POINTER(Completion), c_int, ctypes.POINTER(c_int)]),
        "sgb_server_wait_idle": (c_int, [_vp, c_double]),
        "sgb_server_get_stats": (c_int, [_vp, ctypes.POINTER(ServerStats)]),
        "sgb_server_destroy": (c_int, [_vp]),
        "sgb_server_cancel": (c_int, [_vp, ctypes.c_uint64]),
        "sgb_server_evict": (c_int, [_vp, ctypes.c_uint64]),
        "sgb_batch_save_mesh": (c_int, [_vp, c_int, _dp, _dp, ctypes.POINTER(ctypes.c_longlong)]),
        "sgb_batch_restore_mesh": (c_int, [_vp, c_int, _dp, _dp, ctypes.c_longlong]),
        "sgb_sofa_scene_load": (c_int, [ctypes.POINTER(_vp), ctypes.c_char_p, c_int]),
        "sgb_sofa_scene_destroy": (c_int, [_vp]),
        "sgb_sofa_scene_reset": (c_int, [_vp]),
        "sgb_sofa_scene_unload": (c_int, [_vp]),
        "sgb_sofa_scene_describe": (c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "sgb_sofa_scene_bodies": (c_int, [_vp, ctypes.POINTER(c_int)]),
        "sgb_sofa_scene_body_info": (c_int, [_vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                             ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
        "sgb_sofa_scene_body_arrays": (c_int, [_vp, c_int, _ip, _dp, _ip]),
        "sgb_sofa_scene_body_solver": (c_int, [_vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                               ctypes.POINTER(c_int), ctypes.POINTER(c_int), _dp]),
        "sgb_sofa_scene_init_device": (c_int, [_vp]),
        "sgb_sofa_scene_animate": (c_int, [_vp, c_int]),
        "sgb_sofa_scene_get_positions": (c_int, [_vp, c_int, _dp]),
        "sgb_sofa_scene_get_von_mises": (c_int, [_vp, c_int, _dp, _dp]),
        "sgb_sofa_scene_get_residual": (c_int, [_vp, c_int, _dp]),
        "sgb_sofa_scene_time": (c_int, [_vp, _dp]),
        "sgb_object_factory_new": (_vp, []),
        "sgb_object_factory_delete": (None, [_vp]),
        "sgb_object_factory_has": (c_int, [_vp, ctypes.c_char_p]),
        "sgb_object_factory_count": (c_int, [_vp]),
        "initExternalModule": (None, []),
        "getModuleName": (ctypes.c_char_p, []),
        "getModuleVersion": (ctypes.c_char_p, []),
        "getModuleLicense": (ctypes.c_char_p, []),
        "getModuleDescription": (ctypes.c_char_p, []),
        "getModuleComponentList": (ctypes.c_char_p, []),
        "moduleIsInitialized": (ctypes.c_bool, []),
        "registerObjects": (None, [_vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    return load().sgb_last_error().decode()


def check(rc):
    if rc != SGB_OK:
        raise SgbError(rc, last_error())
    return rc


def _d(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


class TetrahedronFEM:
    """Handle of sgb_tfem_t: a TetrahedronFEMForceField on one mesh, on the GPU."""

    def __init__(self, rest_positions, tetrahedra, young=5000.0, poisson=0.45, method="large", precision="fp64",
                 local_stiffness_factor=None):
        lib = load()
        pos, ppos = _d(np.asarray(rest_positions).reshape(-1, 3))
        tets, ptets = _i(np.asarray(tetrahedra).reshape(-1, 4))
        y, py = _d(np.atleast_1d(young))
        nu, pnu = _d(np.atleast_1d(poisson))
        if local_stiffness_factor is not None:
            lsf, plsf = _d(np.atleast_1d(local_stiffness_factor))
            nl = lsf.size
        else:
            plsf, nl = _dp(), 0
        h = _vp()
        check(lib.sgb_tfem_create(ctypes.byref(h), pos.shape[0], ppos, tets.shape[0], ptets, py, y.size, pnu,
                                  nu.size, plsf, nl, METHODS[method], PRECISIONS[precision]))
        self.warnings = last_error()
        self._h = h
        self.n_nodes = pos.shape[0]
        self.n_tets = tets.shape[0]
        self.method = method
        self.precision = precision
        self._owned = True

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_owned", False) and self._h:
            load().sgb_tfem_destroy(self._h)
        self._h = None
        self._owned = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check_device(self):
        """SGB_OK, or raises for SGB_ERR_DEVICE_TIMEOUT (a bounded device wait of
        an earlier call ran out); synchronises."""
        return check(load().sgb_tfem_check_device(self._h))

    def add_force(self, x_dev, f_dev, stream=None):
        """f += F(x); device pointers (ints). f is FP64 (fp64 handles) or FP32 (mixed)."""
        lib = load()
        if self.precision == "mixed":
            check(lib.sgb_tfem_add_force_f32(self._h, x_dev, f_dev, stream))
        else:
            check(lib.sgb_tfem_add_force(self._h, x_dev, f_dev, stream))

    def add_dforce(self, dx_dev, df_dev, kfactor, stream=None):
        """df += -kfactor K dx; device pointers (ints)."""
        lib = load()
        if self.precision == "mixed":
            check(lib.sgb_tfem_add_dforce_f32(self._h, dx_dev, df_dev, float(kfactor), stream))
        else:
            check(lib.sgb_tfem_add_dforce(self._h, dx_dev, df_dev, float(kfactor), stream))

    def rotations(self):
        r = np.zeros((self.n_tets, 3, 3))
        r0 = np.zeros((self.n_tets, 3, 3))
        check(load().sgb_tfem_get_rotations(self._h, r.ctypes.data_as(_dp), r0.ctypes.data_as(_dp)))
        return r, r0

    def set_plasticity(self, max_threshold, yield_threshold=1e-4, creep=0.9):
        """plasticMaxThreshold / plasticYieldThreshold / plasticCreep: with
        max_threshold > 0 every addForce updates the per-element plastic
        strain (TetrahedronFEMForceField::computeForce)."""
        check(load().sgb_tfem_set_plasticity(self._h, float(max_threshold), float(yield_threshold), float(creep)))

    def set_update_stiffness(self, on=True):
        """updateStiffnessMatrix: every addForce rebuilds the strain-displacement
        matrices from the deformed elements (methods polar and svd)."""
        check(load().sgb_tfem_set_update_stiffness(self._h, int(bool(on))))

    def von_mises(self, x_dev, mode, per_element_dev, per_node_dev=None, stream=None):
        """computeVonMisesStress at positions x_dev (device pointers, FP64)."""
        check(load().sgb_tfem_von_mises(self._h, int(mode), x_dev, per_element_dev, per_node_dev, stream))

    def reset_plasticity(self):
        check(load().sgb_tfem_reset_plasticity(self._h))

    def plastic_strain(self):
        """(n_tets, 6) plastic strain in the caller's element order."""
        out = np.zeros((self.n_tets, 6))
        check(load().sgb_tfem_get_plastic_strain(self._h, out.ctypes.data_as(_dp)))
        return out

    def stiffness_bsr(self):
        """The assembled df/dx at the current rotations as (rowptr, cols,
        blocks[n_blocks, 3, 3]) (buildStiffnessMatrix)."""
        nb = ctypes.c_int()
        check(load().sgb_tfem_stiffness_bsr(self._h, ctypes.byref(nb), None, None, None))
        rowptr = np.zeros(self.n_nodes + 1, np.int32)
        cols = np.zeros(max(nb.value, 1), np.int32)
        vals = np.zeros((max(nb.value, 1), 3, 3))
        check(load().sgb_tfem_stiffness_bsr(self._h, ctypes.byref(nb), rowptr.ctypes.data_as(_ip),
                                             cols.ctypes.data_as(_ip), vals.ctypes.data_as(_dp)))
        return rowptr, cols[: nb.value], vals[: nb.value]

    def device_bytes(self):
        b = ctypes.c_size_t()
        check(load().sgb_tfem_info(self._h, None, None, None, None, ctypes.byref(b)))
        return b.value


class Scene:
    """Handle of sgb_scene_t: mesh + mass + FEM + fixed nodes advanced by
    EulerImplicitSolver / CGLinearSolver on the GPU."""

    def __init__(self, fem: TetrahedronFEM, dt=0.01, rayleigh_stiffness=0.0, rayleigh_mass=0.0, vdamping=0.0,
                 cg_iterations=25, cg_tolerance=1e-5, cg_threshold=1e-5, gravity=(0.0, -9.81, 0.0),
                 vertex_mass=None, total_mass=None, node_masses=None, fixed=(), fix_all=False, mass_first=True,
                 serial_dots=False, residual_replacement=0, linear_solver="cg", preconditioner=None,
                 preconditioner_rate=1, warm_start=False, ff_rayleigh_stiffness=0.0, mass_rayleigh_mass=0.0,
                 first_order=False, project_velocity=False, trapezoidal_scheme=False, compute_residual=False,
                 separate_gravity=False):
        lib = load()
        p = SceneParams()
        lib.sgb_scene_params_default(ctypes.byref(p))
        p.dt = dt
        p.rayleigh_stiffness = rayleigh_stiffness
        p.rayleigh_mass = rayleigh_mass
        p.vdamping = vdamping
        p.cg_iterations = int(cg_iterations)
        p.cg_tolerance = cg_tolerance
        p.cg_threshold = cg_threshold
        for k in range(3):
            p.gravity[k] = float(gravity[k])
        if vertex_mass is None:
            # UniformMass: vertexMass = totalMass / N (UniformMass.inl:337)
            vertex_mass = (1.0 if total_mass is None else float(total_mass)) / fem.n_nodes
        p.vertex_mass = float(vertex_mass)
        self._nm = None
        if node_masses is not None:
            self._nm, p.node_masses_host = _d(node_masses)
        self._fixed, p.fixed_host = _i(np.asarray(fixed, dtype=np.int32).reshape(-1) if len(fixed) else
                                       np.zeros(1, np.int32))
        p.n_fixed = len(fixed)
        p.fix_all = int(fix_all)
        p.mass_first = int(mass_first)
        p.serial_dots = int(serial_dots)
        p.residual_replacement = int(residual_replacement)
        p.linear_solver = {"cg": 0, "pcg": 1}[linear_solver]
        p.preconditioner = {None: 0, "jacobi": 1}[preconditioner]
        p.preconditioner_rate = int(preconditioner_rate)
        p.warm_start = int(warm_start)
        p.ff_rayleigh_stiffness = float(ff_rayleigh_stiffness)
        p.mass_rayleigh_mass = float(mass_rayleigh_mass)
        p.first_order = int(first_order)
        p.project_velocity = int(project_velocity)
        p.trapezoidal_scheme = int(trapezoidal_scheme)
        p.compute_residual = int(compute_residual)
        p.separate_gravity = int(separate_gravity)
        h = _vp()
        check(lib.sgb_scene_create(ctypes.byref(h), fem.handle, ctypes.byref(p)))
        fem._owned = False  # the scene owns the force field now
        self.fem = fem
        self._h = h
        self.n_nodes = fem.n_nodes
        self.params = p

    def close(self):
        if getattr(self, "_h", None):
            load().sgb_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        check(load().sgb_scene_step(self._h, int(n)))

    def von_mises(self, mode=1):
        """(per element, per node) von Mises stress at the current positions
        (computeVonMisesStress mode 1: corotational strain, 2: Green strain)."""
        e = np.zeros(self.fem.n_tets)
        n = np.zeros(self.n_nodes)
        check(load().sgb_scene_von_mises(self._h, int(mode), e.ctypes.data_as(_dp), n.ctypes.data_as(_dp)))
        return e, n

    def sync(self):
        it = ctypes.c_int()
        res = ctypes.c_double()
        check(load().sgb_scene_sync(self._h, ctypes.byref(it), ctypes.byref(res)))
        return it.value, res.value

    def residual(self):
        """EulerImplicitSolver's Data `residual` after the last step
        (scene created with compute_residual=True)."""
        r = ctypes.c_double()
        check(load().sgb_scene_residual(self._h, ctypes.byref(r)))
        return r.value

    def state(self):
        x = np.zeros((self.n_nodes, 3))
        v = np.zeros((self.n_nodes, 3))
        check(load().sgb_scene_get_state(self._h, x.ctypes.data_as(_dp), v.ctypes.data_as(_dp)))
        return x, v

    def state_into(self, x_out=None, v_out=None):
        """Read x and/or v into caller buffers (C-contiguous float64, n x 3;
        pinned buffers give full-speed copies); synchronises."""
        px = x_out.ctypes.data_as(_dp) if x_out is not None else _dp()
        pv = v_out.ctypes.data_as(_dp) if v_out is not None else _dp()
        check(load().sgb_scene_get_state(self._h, px, pv))

    def set_state(self, x=None, v=None):
        xa, px = _d(np.asarray(x).reshape(-1, 3)) if x is not None else (None, _dp())
        va, pv = _d(np.asarray(v).reshape(-1, 3)) if v is not None else (None, _dp())
        self._pending_state = (xa, va)  # kept alive until the stream-ordered copies have run
        check(load().sgb_scene_set_state(self._h, px, pv))

    def set_external_force(self, fext):
        a, p = _d(np.asarray(fext).reshape(-1, 3))
        check(load().sgb_scene_set_external_force(self._h, p))

    def state_device(self):
        x = _vp()
        v = _vp()
        check(load().sgb_scene_state_device(self._h, ctypes.byref(x), ctypes.byref(v)))
        return x.value, v.value

    @property
    def stream(self):
        return load().sgb_scene_stream(self._h)


def scene_params(dt=0.01, rayleigh_stiffness=0.0, rayleigh_mass=0.0, vdamping=0.0, cg_iterations=25,
                 cg_tolerance=1e-5, cg_threshold=1e-5, gravity=(0.0, -9.81, 0.0), vertex_mass=1.0,
                 node_masses=None, fixed=(), fix_all=False, keep=None, linear_solver="cg", preconditioner=None,
                 ff_rayleigh_stiffness=0.0, mass_rayleigh_mass=0.0, trapezoidal_scheme=False):
    """A filled SceneParams; `keep` collects the numpy buffers it points to.
    linear_solver "cg" or "pcg"; preconditioner None or "jacobi" (PCG)."""
    lib = load()
    p = SceneParams()
    lib.sgb_scene_params_default(ctypes.byref(p))
    p.dt = dt
    p.rayleigh_stiffness = rayleigh_stiffness
    p.rayleigh_mass = rayleigh_mass
    p.vdamping = vdamping
    p.cg_iterations = int(cg_iterations)
    p.cg_tolerance = cg_tolerance
    p.cg_threshold = cg_threshold
    for k in range(3):
        p.gravity[k] = float(gravity[k])
    p.vertex_mass = float(vertex_mass)
    keep = [] if keep is None else keep
    if node_masses is not None:
        nm, p.node_masses_host = _d(node_masses)
        keep.append(nm)
    fx, p.fixed_host = _i(np.asarray(fixed, dtype=np.int32).reshape(-1) if len(fixed) else np.zeros(1, np.int32))
    keep.append(fx)
    p.n_fixed = len(fixed)
    p.fix_all = int(fix_all)
    p.mass_first = 1
    p.linear_solver = {"cg": 0, "pcg": 1}[linear_solver]
    p.preconditioner = {None: 0, "jacobi": 1}[preconditioner]
    p.ff_rayleigh_stiffness = float(ff_rayleigh_stiffness)
    p.mass_rayleigh_mass = float(mass_rayleigh_mass)
    p.trapezoidal_scheme = int(trapezoidal_scheme)
    return p


class Batch:
    """Handle of sgb_batch_t: many meshes stepped together in one HBM arena."""

    def __init__(self, precision="mixed", budget_bytes=1 << 30, max_meshes=64, max_cg_iterations=25):
        lib = load()
        h = _vp()
        check(lib.sgb_batch_create(ctypes.byref(h), PRECISIONS[precision], int(budget_bytes), int(max_meshes),
                                   int(max_cg_iterations)))
        self._h = h
        self.precision = precision
        self.n_nodes = {}

    def close(self):
        if getattr(self, "_h", None):
            load().sgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def mesh_desc(positions, tetrahedra, young=5000.0, poisson=0.45, method="large", external_force=None, **params):
        keep = []
        d = MeshDesc()
        pos, d.rest_positions_host = _d(np.asarray(positions).reshape(-1, 3))
        tets, d.tetrahedra_host = _i(np.asarray(tetrahedra).reshape(-1, 4))
        y, d.young = _d(np.atleast_1d(young))
        nu, d.poisson = _d(np.atleast_1d(poisson))
        keep += [pos, tets, y, nu]
        d.n_nodes = pos.shape[0]
        d.n_tets = tets.shape[0]
        d.n_young = y.size
        d.n_poisson = nu.size
        d.method = METHODS[method]
        if "vertex_mass" not in params:
            params["vertex_mass"] = float(params.pop("total_mass", 1.0)) / d.n_nodes
        d.params = scene_params(keep=keep, **params)
        if external_force is not None:
            ext, d.external_force_host = _d(np.asarray(external_force).reshape(-1, 3))
            keep.append(ext)
        return d, keep

    def mesh_bytes(self, positions, tetrahedra, **kw):
        d, keep = self.mesh_desc(positions, tetrahedra, **kw)
        b = ctypes.c_size_t()
        check(load().sgb_batch_mesh_bytes(self._h, ctypes.byref(d), ctypes.byref(b)))
        return b.value

    def add_mesh(self, positions, tetrahedra, **kw):
        """Admits a mesh; returns its slot. Raises SgbError(-6) when it does not fit."""
        d, keep = self.mesh_desc(positions, tetrahedra, **kw)
        slot = ctypes.c_int()
        check(load().sgb_batch_add_mesh(self._h, ctypes.byref(d), ctypes.byref(slot)))
        self.n_nodes[slot.value] = d.n_nodes
        return slot.value

    def add_meshes(self, meshes, threads=8):
        """Admits [(positions, tetrahedra, kwargs), ...], preparing them in
        parallel host threads; returns their slots."""
        descs = (MeshDesc * len(meshes))()
        keep = []
        for i, (pos, tets, kw) in enumerate(meshes):
            d, k = self.mesh_desc(pos, tets, **kw)
            descs[i] = d
            keep.append(k)
        slots = (ctypes.c_int * len(meshes))()
        check(load().sgb_batch_add_meshes(self._h, descs, len(meshes), slots, int(threads)))
        for i in range(len(meshes)):
            self.n_nodes[slots[i]] = descs[i].n_nodes
        return list(slots)

    def remove_mesh(self, slot):
        check(load().sgb_batch_remove_mesh(self._h, int(slot)))
        self.n_nodes.pop(slot, None)

    def step(self, n=1):
        check(load().sgb_batch_step(self._h, int(n)))

    def sync(self):
        check(load().sgb_batch_sync(self._h))

    def stats(self, slot):
        it = ctypes.c_int()
        res = ctypes.c_double()
        steps = ctypes.c_longlong()
        check(load().sgb_batch_mesh_stats(self._h, int(slot), ctypes.byref(it), ctypes.byref(res),
                                          ctypes.byref(steps)))
        return it.value, res.value, steps.value

    def state(self, slot):
        n = self.n_nodes[slot]
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        check(load().sgb_batch_get_state(self._h, int(slot), x.ctypes.data_as(_dp), v.ctypes.data_as(_dp)))
        return x, v

    def positions_async(self, slot, out):
        check(load().sgb_batch_get_positions_async(self._h, int(slot), out.ctypes.data_as(_dp)))

    def set_state(self, slot, x=None, v=None):
        xa, px = _d(np.asarray(x).reshape(-1, 3)) if x is not None else (None, _dp())
        va, pv = _d(np.asarray(v).reshape(-1, 3)) if v is not None else (None, _dp())
        check(load().sgb_batch_set_state(self._h, int(slot), px, pv))

    def save_mesh(self, slot):
        """(x, v, steps) of a mesh: what carries it from one step to the next."""
        n = self.n_nodes[slot]
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        st = ctypes.c_longlong()
        check(load().sgb_batch_save_mesh(self._h, int(slot), x.ctypes.data_as(_dp), v.ctypes.data_as(_dp),
                                         ctypes.byref(st)))
        return x, v, st.value

    def restore_mesh(self, slot, x, v, steps):
        xa, px = _d(np.asarray(x).reshape(-1, 3))
        va, pv = _d(np.asarray(v).reshape(-1, 3))
        check(load().sgb_batch_restore_mesh(self._h, int(slot), px, pv, int(steps)))

    def tune(self, steps_per_trial=2, use_cache=True):
        """Picks the batch step's launch tiles by timing the admitted mix
        (state is restored; results do not change)."""
        check(load().sgb_batch_tune(self._h, int(steps_per_trial), int(use_cache)))
        return self.tuning()

    def tune_patch_size(self, sample, steps_per_trial=2):
        """Elements per patch picked by timing `sample` ([(positions,
        tetrahedra, kwargs), ...]) at each candidate size; call before
        admitting meshes. Returns (chosen, {size: ms per step})."""
        descs = (MeshDesc * len(sample))()
        keep = []
        for i, (pos, tets, kw) in enumerate(sample):
            d, k = self.mesh_desc(pos, tets, **kw)
            descs[i] = d
            keep.append(k)
        chosen = ctypes.c_int()
        ms = (ctypes.c_double * 3)()
        check(load().sgb_batch_tune_patch_size(self._h, descs, len(sample), int(steps_per_trial),
                                               ctypes.byref(chosen), ms))
        cands = (256, 384, 512) if self.precision == "mixed" else (128, 192, 256)
        return chosen.value, {c: ms[i] for i, c in enumerate(cands)}

    def set_tiles(self, matvec_ctas_per_sm=6, update_nodes_per_thread=4, update_ctas_per_sm=4,
                  elem_ctas_per_sm=4, prefetch=0):
        t = (ctypes.c_int * 5)(matvec_ctas_per_sm, update_nodes_per_thread, update_ctas_per_sm, elem_ctas_per_sm,
                               prefetch)
        check(load().sgb_batch_set_tiles(self._h, t))

    def tuning(self):
        t = (ctypes.c_int * 6)()
        d = ctypes.c_double()
        b = ctypes.c_double()
        n = ctypes.c_int()
        check(load().sgb_batch_get_tiles(self._h, t, ctypes.byref(d), ctypes.byref(b), ctypes.byref(n)))
        return {"elements_per_patch": t[0], "matvec_ctas_per_sm": t[1], "update_nodes_per_thread": t[2],
                "update_ctas_per_sm": t[3], "elem_ctas_per_sm": t[4], "prefetch": t[5],
                "default_ms_per_step": d.value, "tuned_ms_per_step": b.value, "trials": n.value}

    def info(self):
        n = ctypes.c_int()
        t = ctypes.c_longlong()
        u = ctypes.c_size_t()
        tot = ctypes.c_size_t()
        check(load().sgb_batch_info(self._h, ctypes.byref(n), ctypes.byref(t), ctypes.byref(u), ctypes.byref(tot)))
        return {"meshes": n.value, "tets": t.value, "budget_used": u.value, "budget_total": tot.value}

    @property
    def stream(self):
        return load().sgb_batch_stream(self._h)


class Server:
    """Handle of sgb_server_t: continuous batching of simulate-K-steps requests."""

    def __init__(self, precision="mixed", budget_bytes=1 << 30, max_meshes=256, max_cg_iterations=25,
                 prep_threads=4, max_steps_per_launch=8):
        lib = load()
        h = _vp()
        check(lib.sgb_server_create(ctypes.byref(h), PRECISIONS[precision], int(budget_bytes), int(max_meshes),
                                    int(max_cg_iterations), int(prep_threads), int(max_steps_per_launch)))
        self._h = h
        self._keep = {}
        self._next = 1

    def close(self):
        if getattr(self, "_h", None):
            load().sgb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, positions, tetrahedra, n_steps, out=None, **kw):
        """Queues a request; returns (id, output array filled at completion)."""
        d, keep = Batch.mesh_desc(positions, tetrahedra, **kw)
        n = d.n_nodes
        out = np.zeros((n, 3)) if out is None else out
        r = Request()
        r.mesh = d
        r.n_steps = int(n_steps)
        r.positions_out_host = out.ctypes.data_as(_dp)
        rid = self._next
        self._next += 1
        r.id = rid
        self._keep[rid] = (keep, out, r)
        check(load().sgb_server_submit(self._h, ctypes.byref(r)))
        return rid, out

    def poll(self, max_out=1024):
        buf = (Completion * max_out)()
        n = ctypes.c_int()
        check(load().sgb_server_poll(self._h, buf, max_out, ctypes.byref(n)))
        res = []
        for i in range(n.value):
            c = buf[i]
            res.append({"id": c.id, "status": c.status, "latency_ms": c.latency_ms, "queue_ms": c.queue_ms,
                        "cg_iterations_last": c.cg_iterations_last, "n_tets": c.n_tets, "n_steps": c.n_steps})
            self._keep.pop(c.id, None)
        return res

    def wait_idle(self, timeout_s=600.0):
        check(load().sgb_server_wait_idle(self._h, float(timeout_s)))

    def cancel(self, rid):
        """Cancels a queued or running request; raises SgbError(-7) when it
        is neither (already completed or unknown)."""
        check(load().sgb_server_cancel(self._h, int(rid)))

    def evict(self, rid):
        """Moves a running request's state to host memory and frees its slot;
        it re-enters the queue and continues bit-exactly."""
        check(load().sgb_server_evict(self._h, int(rid)))

    def stats(self):
        st = ServerStats()
        check(load().sgb_server_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}


class SofaScene:
    """Handle of sgb_sofa_scene_t: a SOFA scene file (.scn XML) parsed into
    the component graph and run on the GPU, one library scene per node that
    holds an EulerImplicitSolver."""

    def __init__(self, xml_text: str, precision: int = -1):
        lib = load()
        h = _vp()
        check(lib.sgb_sofa_scene_load(ctypes.byref(h), xml_text.encode(), int(precision)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().sgb_sofa_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def describe(self) -> dict:
        import json

        lib = load()
        need = ctypes.c_size_t()
        check(lib.sgb_sofa_scene_describe(self._h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        check(lib.sgb_sofa_scene_describe(self._h, buf, need.value, None))
        return json.loads(buf.value.decode())

    @property
    def n_bodies(self) -> int:
        n = ctypes.c_int()
        check(load().sgb_sofa_scene_bodies(self._h, ctypes.byref(n)))
        return n.value

    def body_info(self, body=0) -> dict:
        v = [ctypes.c_int() for _ in range(5)]
        check(load().sgb_sofa_scene_body_info(self._h, int(body), *[ctypes.byref(x) for x in v]))
        return dict(zip(("n_nodes", "n_tets", "method", "precision", "n_fixed"), (x.value for x in v)))

    def body_solver(self, body=0) -> dict:
        v = [ctypes.c_int() for _ in range(4)]
        tol = ctypes.c_double()
        check(load().sgb_sofa_scene_body_solver(self._h, int(body), *[ctypes.byref(x) for x in v], ctypes.byref(tol)))
        names = ("linear_solver", "preconditioner", "preconditioner_rate", "iterations")
        d = dict(zip(names, (x.value for x in v)))
        d["tolerance"] = tol.value
        return d

    def body_arrays(self, body=0):
        info = self.body_info(body)
        tets = np.zeros((info["n_tets"], 4), np.int32)
        masses = np.zeros(info["n_nodes"], np.float64)
        fixed = np.zeros(max(info["n_fixed"], 1), np.int32)
        check(load().sgb_sofa_scene_body_arrays(self._h, int(body), tets.ctypes.data_as(_ip),
                                                 masses.ctypes.data_as(_dp), fixed.ctypes.data_as(_ip)))
        return tets, masses, fixed[: info["n_fixed"]]

    def init_device(self):
        check(load().sgb_sofa_scene_init_device(self._h))

    def reset(self):
        """SofaPhysicsAPI::reset: initial state, plastic strains cleared, time 0."""
        check(load().sgb_sofa_scene_reset(self._h))

    def unload(self):
        """Releases the device objects; the next animate starts again."""
        check(load().sgb_sofa_scene_unload(self._h))

    def animate(self, n_steps=1):
        check(load().sgb_sofa_scene_animate(self._h, int(n_steps)))

    def positions(self, body=0):
        x = np.zeros((self.body_info(body)["n_nodes"], 3), np.float64)
        check(load().sgb_sofa_scene_get_positions(self._h, int(body), x.ctypes.data_as(_dp)))
        return x

    def von_mises(self, body=0):
        """vonMisesPerElement, vonMisesPerNode of a body whose force field sets
        computeVonMisesStress."""
        info = self.body_info(body)
        e = np.zeros(info["n_tets"])
        n = np.zeros(info["n_nodes"])
        check(load().sgb_sofa_scene_get_von_mises(self._h, int(body), e.ctypes.data_as(_dp),
                                                  n.ctypes.data_as(_dp)))
        return e, n

    def residual(self, body=0):
        """The Data `residual` of a body's EulerImplicitSolver with
        computeResidual set, after the last step."""
        r = ctypes.c_double()
        check(load().sgb_sofa_scene_get_residual(self._h, int(body), ctypes.byref(r)))
        return r.value

    @property
    def time(self) -> float:
        t = ctypes.c_double()
        check(load().sgb_sofa_scene_time(self._h, ctypes.byref(t)))
        return t.value
