/*
 * sofa_gb300.h -- C ABI of the GB300-native implicit tetrahedral-FEM step.
 *
 * The library replaces, for one GPU, the hot path of SOFA's soft-body step:
 * TetrahedronFEMForceField (method small/large/polar) integrated by
 * EulerImplicitSolver with a matrix-free CGLinearSolver, UniformMass (or a
 * lumped per-node mass) and FixedProjectiveConstraint. Reference files are
 * cited by their path inside the SOFA source tree (v26.06).
 *
 * Conventions (shared by every entry point):
 *  - Every function returns an int status: SGB_OK (0) or a negative
 *    SGB_ERR_* code; sgb_last_error() gives a message for the calling
 *    thread. Nothing aborts the process. (Error style of
 *    applications/projects/SofaPhysicsAPI/src/SofaPhysicsAPI/SofaPhysicsAPI.h:55-59.)
 *  - Node vectors are arrays of xyz triples (Vec3 AoS, as
 *    Sofa/framework/DefaultType/src/sofa/defaulttype/VecTypes.h).
 *    Tetrahedra are 4 int32 node indices each.
 *  - Pointers named *_dev are device pointers; *_host are host pointers.
 *  - `stream` is a cudaStream_t passed as void* (NULL = the handle's own
 *    stream). Calls are stream-ordered and return without synchronising
 *    unless stated.
 *  - A handle may be used by one host thread at a time.
 */
#ifndef SOFA_GB300_H
#define SOFA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGB_OK 0
#define SGB_ERR_INVALID_ARGUMENT -1
#define SGB_ERR_CUDA -2
#define SGB_ERR_OUT_OF_MEMORY -3
#define SGB_ERR_NOT_SUPPORTED -4
#define SGB_ERR_NUMERICAL -5   /* a non-finite value was met in the CG solve */
#define SGB_ERR_BUDGET -6      /* admission refused: HBM budget exceeded */
#define SGB_ERR_NOT_FOUND -7
#define SGB_ERR_DEVICE_TIMEOUT -8 /* a bounded device-side wait ran out */
#define SGB_ERR_CANCELLED -9   /* the request was cancelled (sgb_server_cancel) */

/* TetrahedronFEMForceField Data "method"
 * (TetrahedronFEMForceField.inl:45): small, large (QR frame), polar, svd
 * (initSVD / accumulateForceSVD, TetrahedronFEMForceField.inl:1090-1184:
 * the polar frame, or for an element whose deformation gradient has
 * determinant below 1e-6 the stable SVD polar factor of that gradient times
 * the initial rotation; the batch engine takes large and polar only). */
#define SGB_METHOD_SMALL 0
#define SGB_METHOD_LARGE 1
#define SGB_METHOD_POLAR 2
#define SGB_METHOD_SVD 3   /* polar, with a stable SVD frame for inverted or flat elements */

/* Precision of the element math and solver vectors.
 *  FP64       FP64 everywhere, rounding like the reference CPU code (no FMA,
 *             the reference's term and summation order per node).
 *  MIXED      FP32 rotation, stiffness apply and vector updates; FP64 dot
 *             products, norms and x/v state accumulation.
 *  FP64_FMA   FP64 with fused multiply-add (faster, within rounding). */
#define SGB_PRECISION_FP64 0
#define SGB_PRECISION_MIXED 1
#define SGB_PRECISION_FP64_FMA 2

const char* sgb_last_error(void);
const char* sgb_version(void);

/* ------------------------------------------------------------------ */
/* TetrahedronFEMForceField                                            */
/* ------------------------------------------------------------------ */
typedef struct sgb_tfem sgb_tfem_t;

/* Creates the force field on a mesh and runs its init/reinit on the GPU:
 * per-element material stiffness (TetrahedronFEMForceField.inl:256-291),
 * strain-displacement matrix (:134-209) and initial rotation plus rotated
 * rest coordinates (initLarge :835-868, initPolar :993-1023, initSmall
 * :526-532); builds the node->(element,corner) gather table.
 * young/poisson have 1 or n_tets entries (entry e, else entry 0, as
 * BaseLinearElasticityFEMForceField.inl:114-132); values out of range
 * (E < 0, nu outside [0, 0.5)) are replaced by 5000 / 0.45 with a warning
 * readable through sgb_last_error(), as
 * BaseLinearElasticityFEMForceField.inl:53-85 does. local_stiffness_factor
 * may be NULL (n_lsf = 0). Replaces the reference's reinit path feeding
 * TetrahedronFEMForceFieldCuda3f_addForce
 * (applications/plugins/SofaCUDA/Component/src/SofaCUDA/component/
 * solidmechanics/fem/elastic/CudaTetrahedronFEMForceField.cu:39-40). */
int sgb_tfem_create(sgb_tfem_t** out, int n_nodes, const double* rest_positions_host, int n_tets,
                    const int32_t* tetrahedra_host, const double* young, int n_young, const double* poisson,
                    int n_poisson, const double* local_stiffness_factor, int n_lsf, int method, int precision);
int sgb_tfem_destroy(sgb_tfem_t* fem);

/* addForce (TetrahedronFEMForceField.inl:1548-1604; SofaCUDA
 * TetrahedronFEMForceFieldCuda3d_addForce, CudaTetrahedronFEMForceField.cu:49):
 * f += internal forces at positions x; updates the element rotations used by
 * the next sgb_tfem_add_dforce. x is FP64 for every precision; f is FP64
 * (FP64 handles) -- use sgb_tfem_add_force_f32 for MIXED handles. */
int sgb_tfem_add_force(sgb_tfem_t* fem, const double* x_dev, double* f_dev, void* stream);
int sgb_tfem_add_force_f32(sgb_tfem_t* fem, const double* x_dev, float* f_dev, void* stream);

/* addDForce (TetrahedronFEMForceField.inl:1606-1636; SofaCUDA
 * TetrahedronFEMForceFieldCuda3d_addDForce, CudaTetrahedronFEMForceField.cu:50):
 * df += -kfactor K dx with the rotations of the last add_force. kfactor is
 * mparams->kFactorIncludingRayleighDamping(rayleighStiffness). */
int sgb_tfem_add_dforce(sgb_tfem_t* fem, const double* dx_dev, double* df_dev, double kfactor, void* stream);
int sgb_tfem_add_dforce_f32(sgb_tfem_t* fem, const float* dx_dev, float* df_dev, float kfactor, void* stream);

/* Per-element rotations in the reference's convention: rotations[e] = R^T,
 * 9 doubles row-major per element (TetrahedronFEMForceField.h
 * getActualTetraRotation / getInitialTetraRotation). Synchronous. */
int sgb_tfem_get_rotations(sgb_tfem_t* fem, double* rotations_host, double* initial_rotations_host);

/* Plasticity of the addForce strain: the Data plasticMaxThreshold,
 * plasticYieldThreshold and plasticCreep of TetrahedronFEMForceField
 * (TetrahedronFEMForceField.inl:51-53; the update in computeForce, :357-370).
 * max_threshold > 0 turns it on; every add_force call (and every scene step,
 * through its force computation) then updates the per-element plastic
 * strain. The strain starts at zero when first turned on; max_threshold = 0
 * turns it off and keeps the strain. Thresholds are 2-norms of the 6-vector
 * strain. Synchronous on the handle's stream when first turned on. */
int sgb_tfem_set_plasticity(sgb_tfem_t* fem, double max_threshold, double yield_threshold, double creep);

/* Data updateStiffnessMatrix of TetrahedronFEMForceField
 * (TetrahedronFEMForceField.inl:49): on (1), every add_force call (and every
 * scene step) rebuilds each element's strain-displacement matrix from its
 * deformed positions in its current frame before forming the force
 * (accumulateForcePolar :1063-1067, accumulateForceSVD :1174-1177), and the
 * later addDForce / CG products use it. Methods polar and svd; method small
 * ignores the flag, as the reference does. Method large returns
 * SGB_ERR_NOT_SUPPORTED: the reference's large update (:908-921) writes only
 * one of the entries J(3i,0) = J(3i+1,3) = J(3i+2,5) (and the like) that it
 * builds equal, which this library stores once. Off (0) keeps the last
 * rebuilt matrix, as the reference does. Synchronous on the handle's stream
 * when first turned on (mixed precision computes a per-element scale). */
int sgb_tfem_set_update_stiffness(sgb_tfem_t* fem, int on);
/* von Mises stress (TetrahedronFEMForceField::computeVonMisesStress,
 * TetrahedronFEMForceField.inl:2197-2374; Data computeVonMisesStress,
 * vonMisesPerElement, vonMisesPerNode) at positions x_dev (n_nodes xyz
 * doubles, device). mode 1: from the corotational strain (methods large,
 * polar, svd; small is refused as in the reference, :1441-1445); mode 2:
 * from the Green strain. per_element_dev: n_tets doubles in the caller's
 * element order; per_node_dev (may be NULL): n_nodes doubles, the mean over
 * each node's elements. FP64 for every precision. The reference also
 * overwrites the element rotations in mode 1; this call leaves them as the
 * last add_force computed them. The first call computes and keeps the
 * elements' Lame coefficients (16 B per element), synchronously; later calls
 * are stream-ordered. */
int sgb_tfem_von_mises(sgb_tfem_t* fem, int mode, const double* x_dev, double* per_element_dev,
                       double* per_node_dev, void* stream);

/* Zeroes the plastic strain (TetrahedronFEMForceField::reset, .inl:1382-1390).
 * Stream-ordered on the handle's stream. */
int sgb_tfem_reset_plasticity(sgb_tfem_t* fem);
/* The plastic strain, 6 doubles per element in the caller's element order
 * (Voigt: xx, yy, zz, then the three shear terms of J^T D); zeros when
 * plasticity was never turned on. Synchronous. */
int sgb_tfem_get_plastic_strain(sgb_tfem_t* fem, double* plastic_strain_host);

/* The assembled stiffness df/dx at the current rotations (those of the last
 * addForce), as TetrahedronFEMForceField::buildStiffnessMatrix assembles it
 * (TetrahedronFEMForceField.inl:1965-1993): block-sparse rows of 3x3 blocks,
 * block (i, j) = - sum over the elements holding nodes i and j (in element
 * order) of R^T S_ij R. rowptr_host: n_nodes + 1 entries; cols_host and
 * values_host (9 doubles per block, row-major): n_blocks entries. Call with
 * NULL arrays to get n_blocks; the pattern is built on the first call.
 * Synchronous. df/dx times dx equals addDForce with kFactor 1. */
int sgb_tfem_stiffness_bsr(sgb_tfem_t* fem, int* n_blocks, int32_t* rowptr_host, int32_t* cols_host,
                           double* values_host);

/* Reads and clears the force field's sticky device error flag (synchronises
 * the device). SGB_OK, or SGB_ERR_DEVICE_TIMEOUT when a bounded device-side
 * wait of an earlier call ran out. No kernel of this version waits on the
 * device (the reductions take no locks and never spin), so it returns
 * SGB_OK after any call that completed; the flag is kept so that callers
 * need no change when a kernel with a bounded wait is added. */
int sgb_tfem_check_device(sgb_tfem_t* fem);

/* Sizes and device footprint of the force field. */
int sgb_tfem_info(const sgb_tfem_t* fem, int* n_nodes, int* n_tets, int* method, int* precision,
                  size_t* device_bytes);

/* addDForce for callers that cannot allocate device memory: a framework
 * that hands out device buffers from its own pool, a real-time loop that
 * must avoid the device synchronisation cudaMalloc/cudaFree imply, or code
 * running where new allocations are not allowed. It calls no cudaMalloc,
 * cudaFree or allocating routine: the caller passes every input and output
 * as device arrays, and the only scratch (12 floats per tetrahedron between
 * the element pass and the node gather) lives in a fixed array of the
 * library's device memory holding 262,144 tetrahedra (12 MiB, kept by every
 * GPU that loads the library until the process exits). Larger meshes are
 * rejected with SGB_ERR_INVALID_ARGUMENT. All calls share that array, so two
 * calls that overlap on the GPU (unordered streams) race and give wrong
 * results; order them on one stream. The first call on a device looks up
 * the array's device address once for that device; make that first call
 * before any stream capture, and make no call after a cudaDeviceReset in
 * the same process (the array may move). Out-of-range node or slot indices
 * are skipped by the kernels (no access outside the arrays; df is then
 * wrong for the nodes concerned). This entry point has no counterpart in the
 * reference: it is a variant of sgb_tfem_add_dforce_f32 for such callers.
 * Computes df -= kfactor R K R^T dx per tetrahedron, FP32, with arrays:
 *   tetrahedra_dev        4 int32 per tetrahedron (node indices < n_nodes), 16-byte aligned
 *   rotations_dev         9 x n_tets floats: entry k of tetrahedron e at [k*n_tets+e] is
 *                         R(k/3, k%3), R's rows being the element frame (R = rotations[e]^T
 *                         of TetrahedronFEMForceField)
 *   stiffness_dev         3 x n_tets: K(0,0), K(0,1), K(3,3) of the 6x6 material stiffness / (36 V)
 *   strain_displacement_dev 12 x n_tets: per node i, J(3i,0), J(3i,3), J(3i,5)
 *   node_rowptr_dev, node_slots_dev  node -> (tetrahedron*4 + corner) table, n_nodes+1
 *                         offsets and 4*n_tets entries, each row in increasing order
 *   dx_dev, df_dev        n_nodes xyz triples; df accumulates. */
int sgb_tfem_add_dforce_f32_noalloc(int n_nodes, int n_tets, const int32_t* tetrahedra_dev, const float* rotations_dev,
                                    const float* stiffness_dev, const float* strain_displacement_dev,
                                    const int32_t* node_rowptr_dev, const int32_t* node_slots_dev,
                                    const float* dx_dev, float* df_dev, float kfactor, void* stream);

/* Host-only check of the element ordering and patch layout the fused
 * kernels use (no GPU needed): every (element, corner) gathered exactly once
 * by one patch, one owner per node, partial-sum slots in patch order.
 * stats (5 ints, may be NULL): patches, largest local node count, local
 * nodes in total, nodes shared by several patches, partial-sum slots.
 * Returns SGB_OK or SGB_ERR_NUMERICAL with the violated invariant in
 * sgb_last_error(). No reference counterpart: it validates this library's
 * own layout. */
int sgb_patch_layout_check(int n_nodes, const double* rest_positions_host, int n_tets, const int32_t* tetrahedra_host,
                           int elements_per_patch, int max_nodes_per_patch, int* stats);

/* ------------------------------------------------------------------ */
/* Scene: MechanicalObject + mass + FEM + fixed constraint, advanced by */
/* EulerImplicitSolver + CGLinearSolver<GraphScattered>.                */
/* ------------------------------------------------------------------ */
typedef struct sgb_scene sgb_scene_t;

typedef struct sgb_scene_params {
    /* EulerImplicitSolver Data (EulerImplicitSolver.cpp:40-51) */
    double dt;
    double rayleigh_stiffness;
    double rayleigh_mass;
    double vdamping;
    /* CGLinearSolver Data (CGLinearSolver.inl:34-46): iterations, tolerance, threshold */
    int cg_iterations;
    double cg_tolerance;
    double cg_threshold;
    /* context gravity */
    double gravity[3];
    /* UniformMass vertexMass (UniformMass.inl:153-340); ignored when node_masses is given */
    double vertex_mass;
    /* optional lumped per-node masses (DiagonalMass-style), host, n_nodes entries, or NULL */
    const double* node_masses_host;
    /* FixedProjectiveConstraint indices / fixAll (FixedProjectiveConstraint.inl:39-48);
     * out-of-range indices are dropped, as checkIndices (:130-160) does */
    const int32_t* fixed_host;
    int n_fixed;
    int fix_all;
    /* 1: the mass component precedes the force field in the node (its
     * forces are accumulated first), 0: after it */
    int mass_first;
    /* 1: dot products summed serially in node order, as
     * MechanicalObject::vDot does (bit-identical to the reference with
     * SGB_PRECISION_FP64; slow on large meshes) */
    int serial_dots;
    /* SGB_PRECISION_MIXED scenes: every residual_replacement CG iterations the
     * FP32 solution increment is accumulated in FP64 and the residual is
     * recomputed as b - A x in FP64 with an FP64 copy of the operator
     * (reliable-update CG: the FP32 recurrence cannot drift from the true
     * residual). 0: off. The FP64 copy doubles the force field's memory. */
    int residual_replacement;
    /* Linear solver: SGB_SOLVER_CG (CGLinearSolver) or SGB_SOLVER_PCG
     * (PCGLinearSolver, PCGLinearSolver.inl:194-262: starts from the previous
     * step's solution, stops when r.z <= tolerance * b.b, no threshold test;
     * cg_iterations / cg_tolerance are its iterations / tolerance), and its
     * preconditioner: SGB_PRECOND_NONE or SGB_PRECOND_JACOBI
     * (JacobiPreconditioner: z = diag(mF M + kF K)^-1 r, the diagonal
     * re-assembled every step, fixed DOFs one). FP64 PCG runs on the
     * element-order kernels, mixed PCG on the fused patch kernels. */
    int linear_solver;
    int preconditioner;
    /* PreconditionedMatrixFreeSystem assemblingRate
     * (PreconditionedMatrixFreeSystem.inl:31-67): the preconditioner is
     * re-assembled on the first step and every this many steps after it
     * (0 or 1: every step). */
    int preconditioner_rate;
    /* CGLinearSolver warmStart (CGLinearSolver.inl:95-104): 1 starts each
     * solve from the previous step's solution, r = b - A x, instead of
     * x = 0, r = b. PCG always starts from it. */
    int warm_start;
    /* The components' own Rayleigh coefficients: the force field's
     * rayleighStiffness (BaseForceField.cpp:34) and the mass's rayleighMass
     * (BaseMass.cpp:33-34). They enter the system matrix only, as
     * kFactorIncludingRayleighDamping = kF + bF * ff_rayleigh_stiffness and
     * mFactorIncludingRayleighDamping = mF - bF * mass_rayleigh_mass
     * (MechanicalParams.h:62-64, BaseForceField.cpp:38-47, Mass.inl:94-104);
     * the right-hand side is built with bF = 0. */
    double ff_rayleigh_stiffness;
    double mass_rayleigh_mass;
    /* EulerImplicitSolver firstOrder (EulerImplicitSolver.cpp:138-171): b = f,
     * (M - h K) v_new = b, x += h v_new; the Rayleigh and bF terms vanish. */
    int first_order;
    /* FixedProjectiveConstraint activate_projectVelocity
     * (FixedProjectiveConstraint.inl:237-261): after each step the velocity
     * of the fixed nodes is set to zero (DefaultAnimationLoop's
     * projectPositionAndVelocity, DefaultAnimationLoop.cpp:228-233, 293). */
    int project_velocity;
    /* EulerImplicitSolver trapezoidalScheme (EulerImplicitSolver.cpp:117-171):
     * the factor tr = 0.5 on h in the right-hand side's stiffness factor
     * (h tr + rs) and in the system factors mF = 1 + tr h rm, bF = -tr h,
     * kF = -tr h (tr h + rs) (first order: kF = -h tr). */
    int trapezoidal_scheme;
    /* EulerImplicitSolver computeResidual (EulerImplicitSolver.cpp:48-49,
     * 314-338): after each step the squared norm of r = M (v_new - v_old) -
     * dt F(x_new), projected, is kept (sgb_scene_residual). In the animation
     * loop's call v_new and v_old are the same vector, so r = -dt F(x_new);
     * the extra force computation runs the force field again (its plastic
     * strains and, with updateStiffnessMatrix, its strain-displacement
     * matrices see it, as in the reference). */
    int compute_residual;
    /* The mass's separateGravity (UniformMass / DiagonalMass; UniformMass.inl:
     * 450-475): the mass adds no weight to the force, and after the position
     * update the step adds g dt to every velocity (EulerImplicitSolver.cpp:
     * 296), before the velocity damping; the fixed points get it too, as in
     * the reference. */
    int separate_gravity;
} sgb_scene_params;

#define SGB_SOLVER_CG 0
#define SGB_SOLVER_PCG 1
#define SGB_PRECOND_NONE 0
#define SGB_PRECOND_JACOBI 1

/* Fills params with the reference Data defaults: dt 0.01, Rayleigh 0, CG
 * 25 / 1e-5 / 1e-5, gravity (0,-9.81,0), vertex mass 1, mass first. */
void sgb_scene_params_default(sgb_scene_params* params);

/* Creates a scene on a force field; the scene takes ownership of `fem`.
 * Positions start at the rest positions, velocities at zero. */
int sgb_scene_create(sgb_scene_t** out, sgb_tfem_t* fem, const sgb_scene_params* params);
int sgb_scene_destroy(sgb_scene_t* scene);

/* Advances n_steps implicit Euler steps (DefaultAnimationLoop::step,
 * Sofa/framework/Simulation/Core/src/sofa/simulation/DefaultAnimationLoop.cpp:273-325).
 * Stream-ordered; the step is recorded once as a CUDA graph and replayed. */
int sgb_scene_step(sgb_scene_t* scene, int n_steps);

/* Waits for the scene's stream and reports the last CG solve: iterations
 * run (the matrix-vector products, including that of an iteration ended by
 * the denominator threshold), last relative residual |r|/|b|, and
 * SGB_ERR_NUMERICAL if a non-finite value was met. */
int sgb_scene_sync(sgb_scene_t* scene, int* cg_iterations, double* cg_residual);
/* The Data `residual` of EulerImplicitSolver after the last step: r.r of the
 * residual above (scene created with compute_residual). Synchronises the
 * scene's stream. SGB_ERR_INVALID_ARGUMENT when compute_residual is off. */
int sgb_scene_residual(sgb_scene_t* scene, double* residual);

/* von Mises stress of the scene's force field at its current positions
 * (sgb_tfem_von_mises; TetrahedronFEMForceField computes it at the end of
 * each step, TetrahedronFEMForceField.inl:2008-2031), into host arrays:
 * n_tets per element, n_nodes per node (may be NULL). Synchronous. */
int sgb_scene_von_mises(sgb_scene_t* scene, int mode, double* per_element_host, double* per_node_host);

/* State access (FP64). get_* synchronise; set_* are stream-ordered: from
 * pinned host memory the copies run asynchronously, and the caller keeps the
 * buffers unchanged until a later synchronising call (get_state,
 * sgb_scene_sync); pageable buffers are consumed before the call returns.
 * Either pointer may be NULL. */
int sgb_scene_get_state(sgb_scene_t* scene, double* x_host, double* v_host);
int sgb_scene_set_state(sgb_scene_t* scene, const double* x_host, const double* v_host);
/* MechanicalObject externalForce (accumulateForce, MechanicalObject.inl:1357-1376). */
int sgb_scene_set_external_force(sgb_scene_t* scene, const double* fext_host);
/* Device pointers of the FP64 state (n_nodes x 3), valid for the scene's lifetime. */
int sgb_scene_state_device(sgb_scene_t* scene, double** x_dev, double** v_dev);
/* The scene's stream (cudaStream_t as void*). */
void* sgb_scene_stream(sgb_scene_t* scene);

/* ------------------------------------------------------------------ */
/* Batch: many meshes advanced together on one GPU                      */
/* ------------------------------------------------------------------ */
/* Every admitted mesh advances one implicit Euler step per sgb_batch_step,
 * through one persistent kernel per phase for all meshes (no reference
 * counterpart: the reference visits each mesh's components one after the
 * other, Sofa/framework/Simulation/Core/src/sofa/simulation/
 * MappingGraphMechanicalOperations.cpp:41-92). Meshes live in a fixed HBM
 * arena whose size is the admission budget; they can be added and removed
 * between steps. Methods large and polar; precision MIXED or FP64_FMA. */
typedef struct sgb_batch sgb_batch_t;

typedef struct sgb_mesh_desc {
    int n_nodes;
    const double* rest_positions_host;  /* 3 n_nodes */
    int n_tets;
    const int32_t* tetrahedra_host;     /* 4 n_tets */
    const double* young;                /* 1 or n_tets values */
    int n_young;
    const double* poisson;              /* 1 or n_tets values */
    int n_poisson;
    int method;                         /* SGB_METHOD_LARGE or SGB_METHOD_POLAR */
    sgb_scene_params params;            /* solver, mass, gravity, fixed nodes */
    const double* external_force_host;  /* optional 3 n_nodes constant external force, or NULL */
} sgb_mesh_desc;

/* hbm_budget_bytes is reserved at once and is the admission budget;
 * max_cg_iterations bounds every mesh's CGLinearSolver iterations. */
int sgb_batch_create(sgb_batch_t** out, int precision, size_t hbm_budget_bytes, int max_meshes,
                     int max_cg_iterations);
int sgb_batch_destroy(sgb_batch_t* batch);
/* Bytes a mesh would take in the budget (host-side planning only; with
 * batch NULL, for a mixed-precision batch with the default patch size).
 * Runs the admission checks: the batch engine runs cold-start
 * CGLinearSolver with block-ordered dot products and the second-order
 * Euler scheme, so a mesh whose params ask for PCG, a preconditioner,
 * warmStart, residual replacement, serial dots, firstOrder or
 * project_velocity is refused with SGB_ERR_NOT_SUPPORTED, here and at
 * admission. The components' Rayleigh coefficients and trapezoidalScheme are
 * supported. */
int sgb_batch_mesh_bytes(const sgb_batch_t* batch, const sgb_mesh_desc* mesh, size_t* bytes);
/* Admission: SGB_ERR_BUDGET when the mesh does not fit or no slot is free.
 * Synchronous; positions start at rest, velocities at zero. */
int sgb_batch_add_mesh(sgb_batch_t* batch, const sgb_mesh_desc* mesh, int* slot);
/* Admits n meshes, preparing them on `threads` host threads; slots[i]
 * receives mesh i's slot. Stops at the first mesh that cannot be admitted
 * (the ones before it stay admitted; the others get slot -1). */
int sgb_batch_add_meshes(sgb_batch_t* batch, const sgb_mesh_desc* meshes, int n, int* slots, int threads);
int sgb_batch_remove_mesh(sgb_batch_t* batch, int slot);
/* Advances every admitted mesh by n_steps (stream-ordered, CUDA graph). */
int sgb_batch_step(sgb_batch_t* batch, int n_steps);
int sgb_batch_sync(sgb_batch_t* batch);
int sgb_batch_mesh_stats(sgb_batch_t* batch, int slot, int* cg_iterations, double* cg_residual, long long* steps);
int sgb_batch_get_state(sgb_batch_t* batch, int slot, double* x_host, double* v_host);
/* Queues the copy of a mesh's positions on the batch stream (no wait). */
int sgb_batch_get_positions_async(sgb_batch_t* batch, int slot, double* x_host);
int sgb_batch_set_state(sgb_batch_t* batch, int slot, const double* x_host, const double* v_host);
/* What carries a mesh from one step to the next -- positions, velocities and
 * its time-step count -- saved to host memory and put back, so that a mesh
 * removed from a batch and admitted again (into this or another batch of the
 * same precision, from the same description) continues bit-exactly; the
 * counterpart of MechanicalObject::writeState / readState
 * (Sofa/Component/StateContainer/src/sofa/component/statecontainer/
 * MechanicalObject.inl:1229-1340) for this library's state. x_host and v_host
 * hold 3 n_nodes doubles. Synchronous. */
int sgb_batch_save_mesh(sgb_batch_t* batch, int slot, double* x_host, double* v_host, long long* steps);
int sgb_batch_restore_mesh(sgb_batch_t* batch, int slot, const double* x_host, const double* v_host,
                           long long steps);
int sgb_batch_info(const sgb_batch_t* batch, int* active_meshes, long long* active_tets, size_t* budget_used,
                   size_t* budget_total);
void* sgb_batch_stream(sgb_batch_t* batch);

/* Launch tiles of the batch step, picked by timing the admitted mix (an
 * autotuner of this library; the reference sets its equivalent knobs by hand:
 * gatherPt / gatherBsize of SofaCUDA's TetrahedronFEMForceField,
 * applications/plugins/SofaCUDA/Component/src/SofaCUDA/component/
 * solidmechanics/fem/elastic/CudaTetrahedronFEMForceField.h:258-266). The
 * tiles are the matvec's resident CTAs per SM (5, 6 or 8: its register cap),
 * the CG update's nodes per thread (1, 2 or 4) and CTAs per SM, the element
 * kernels' CTAs per SM, and an L2 prefetch of each block's next patch. No
 * tile changes a result bit: every per-mesh reduction is formed per work item
 * in an order fixed by the item. sgb_batch_tune times candidates one tile at
 * a time, each over steps_per_trial whole steps from the same saved state,
 * restores every mesh's state afterwards and keeps the fastest; with
 * use_cache it first looks for the choice made for a mix with the same
 * size histogram in this process. Patches keep the size fixed at creation
 * (elements per patch: 512 mixed, 256 FP64), because it fixes each node's
 * gather order. Synchronous. */
int sgb_batch_tune(sgb_batch_t* batch, int steps_per_trial, int use_cache);
/* Elements per patch (the matvec's elements per CTA) picked before any mesh is
 * admitted, by timing a sample of the workload: for each candidate (256, 384,
 * 512 in mixed precision; 128, 192, 256 in FP64) the sample meshes are
 * admitted with that patch size, stepped steps_per_trial times after one
 * warm-up step, and removed. The fastest candidate is kept for the batch's
 * lifetime (it fixes every mesh's gather order, so results depend on it,
 * deterministically). chosen (may be NULL): the patch size kept;
 * ms_per_step (may be NULL): the three candidates' step times.
 * SGB_ERR_NOT_SUPPORTED when meshes are admitted already. Synchronous. */
int sgb_batch_tune_patch_size(sgb_batch_t* batch, const sgb_mesh_desc* sample, int n, int steps_per_trial,
                              int* chosen, double* ms_per_step);
/* tiles: matvec CTAs per SM, update nodes per thread, update CTAs per SM,
 * element CTAs per SM, prefetch (0 / 1). */
int sgb_batch_set_tiles(sgb_batch_t* batch, const int tiles[5]);
/* tiles[6]: elements per patch, then the five tiles above; default_ms and
 * best_ms: step time of the starting and the chosen tiles in the last tuning
 * (0 before any), trials: configurations it timed (0 when the cache
 * answered). Any output but tiles may be NULL. */
int sgb_batch_get_tiles(const sgb_batch_t* batch, int tiles[6], double* default_ms, double* best_ms, int* trials);

/* ------------------------------------------------------------------ */
/* Serving: continuous batching of simulate-K-steps requests            */
/* ------------------------------------------------------------------ */
/* Requests are prepared on host worker threads, admitted in arrival order
 * when the HBM budget and a mesh slot allow, and stepped together with the
 * other admitted meshes; each launch advances every mesh by up to
 * max_steps_per_launch steps, never past the nearest finishing request.
 * Latency is measured from submission to the copy of the final positions.
 * Modelled on the SofaPhysicsAPI load/step/get-positions cycle
 * (applications/projects/SofaPhysicsAPI/src/SofaPhysicsAPI/SofaPhysicsAPI.h:73-152);
 * the continuous batching itself has no reference counterpart. */
typedef struct sgb_server sgb_server_t;

typedef struct sgb_request {
    sgb_mesh_desc mesh;          /* host arrays must stay valid until the request completes */
    int n_steps;                 /* K implicit Euler steps */
    double* positions_out_host;  /* 3 n_nodes doubles, written before completion is reported */
    uint64_t id;
} sgb_request;

typedef struct sgb_completion {
    uint64_t id;
    int status;               /* SGB_OK or the SGB_ERR_* that failed the request */
    double latency_ms;        /* submission -> positions copied */
    double queue_ms;          /* submission -> admission */
    int cg_iterations_last;   /* CG iterations of its last step */
    long long n_tets;
    int n_steps;
} sgb_completion;

typedef struct sgb_server_stats {
    long long submitted, completed, failed;
    long long tet_steps;      /* completed requests: tets x steps */
    double p50_ms, p99_ms, max_ms;  /* request latency: submission -> positions copied */
    double busy_s;            /* time spent in batch launches */
    double wall_s;            /* since the first submission */
    /* step latency: each launch of k steps over the admitted meshes counts k
     * steps of (launch wall time) / k, outputs copied included */
    double step_p50_ms, step_p99_ms;
    long long launches, cancelled, evicted;
} sgb_server_stats;

int sgb_server_create(sgb_server_t** out, int precision, size_t hbm_budget_bytes, int max_meshes,
                      int max_cg_iterations, int prep_threads, int max_steps_per_launch);
int sgb_server_submit(sgb_server_t* server, const sgb_request* request);
/* Non-blocking: moves up to max_out completions into out. */
int sgb_server_poll(sgb_server_t* server, sgb_completion* out, int max_out, int* n_out);
/* Blocks until every submitted request has completed (or timeout_s passes). */
int sgb_server_wait_idle(sgb_server_t* server, double timeout_s);
int sgb_server_get_stats(sgb_server_t* server, sgb_server_stats* stats);
/* Cancels a request: one still queued (being prepared or waiting for
 * admission) is dropped at once, a running one at the next launch boundary
 * (its slot and memory are freed). Its completion carries
 * SGB_ERR_CANCELLED. SGB_ERR_NOT_FOUND when the id is unknown or the request
 * already completed. */
int sgb_server_cancel(sgb_server_t* server, uint64_t id);
/* Evicts a running request at the next launch boundary: its state
 * (sgb_batch_save_mesh) goes to host memory and its slot and HBM are freed;
 * it re-enters the queue behind the requests already waiting and, once
 * admitted again, continues from where it stopped, bit-exactly. Its latency
 * still counts from the first submission. SGB_ERR_NOT_FOUND when the
 * request is not running. */
int sgb_server_evict(sgb_server_t* server, uint64_t id);
int sgb_server_destroy(sgb_server_t* server);

#ifdef __cplusplus
}
#endif

#endif /* SOFA_GB300_H */
