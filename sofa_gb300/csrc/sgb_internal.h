// Internal data structures of the GB300 tetrahedral-FEM library. Device
// buffers are owned by the library; every pointer below is device memory
// unless its name ends in _h.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace sgb {

enum Method { METHOD_SMALL = 0, METHOD_LARGE = 1, METHOD_POLAR = 2, METHOD_SVD = 3 };
enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };

// Blocks used by every node-parallel kernel that produces a dot product: the
// per-block partial sums live in a fixed-size array and the last block to
// finish reduces them in index order, so a dot product is bit-reproducible.
constexpr int kNodeBlock = 256;
constexpr int kMaxNodeBlocks = 152 * 8;
// Largest grid of a kernel that finishes a dot product (size of the per-block
// partial array): the persistent patch kernels run up to 32 small CTAs per SM.
constexpr int kMaxDotBlocks = 152 * 32;
constexpr int kElemBlock = 128;

// Structure-of-arrays view of the per-element data. Arrays of width W are
// stored as W rows of n_tets entries (value k of element e at [k*n_tets+e]),
// so a warp's loads of one value are contiguous.
template <typename R>
struct ElemView {
    const int4* tets;  // node indices a,b,c,d
    R* rot;            // 9 rows: current rotation R (rows x,y,z of the element frame)
    const R* K;        // 3 rows: K(0,0), K(0,1), K(3,3) of the 6x6 material stiffness / (36 V)
    const R* J;        // 12 rows: the distinct values of the 12x6 strain-displacement matrix
    const R* rest;     // 12 rows: rotated rest coordinates (method dependent, see tfem.cu)
    const float2* rest_ff;  // mixed: rows 3..11 (b-a, c-a, d-a) as float-float pairs for the force kernel (or null)
    const R* A0inv;         // svd: inverse rest edge matrix, 9 rows (or null)
    const R* R0;            // svd: initial rotation rows, 9 rows (or null)
    int n_tets;
    int method;
};

// Compact FP32 element format of the matvec: per element only the rotation
// Q = R0^T R from the rest frame to the current element frame (a unit
// quaternion, 16 B), the strain-displacement values being formed from the
// nodes' rest positions in the world frame (float-float, per node) -- for an
// isotropic material K_e(R0 p) = R0 K_e(p) R0^T, so the rotated rest frame
// of the reference and the world frame give the same stiffness.

// Node -> (element*4 + corner) incidence in CSR form, each row sorted by slot.
struct NodeCSR {
    const int* rowptr;  // n_nodes + 1
    const int* slots;   // 4 * n_tets
};

// Patch layout for the fused matvec: elements are stored in patch order
// (Morton order of their centroids, cut into patches of at most `pe`
// elements); each patch lists its nodes (local numbering), its elements'
// corners in local numbering and, per local node, the (element, corner)
// slots that touch it. A node touched by one patch is interior to it; a
// node touched by several patches gets one partial-sum slot per patch and is
// owned by the first of them.
struct PatchView {
    const int* elem_start;      // n_patches + 1, element storage positions
    const int* node_start;      // n_patches + 1, offsets into the local-node arrays
    const int* lnode_gid;       // global node id of each local node
    const int* lnode_info;      // -1: interior; else 2*partial_slot + owner_bit
    const int* lrow;            // per local node: range in lslots (global offsets), size total+1
    const uint16_t* lslots;     // local element*4 + corner, sorted by local element
    const ushort4* lconn;       // per element (storage order): local node indices
    const int* bnd_rowptr;      // per global node: range of its partial slots (empty if interior)
    int n_patches;
    int pe;                     // elements per patch (shared-memory stride)
    int max_lnodes;             // largest local node count of a patch
};

struct PatchLayout {
    int* elem_start = nullptr;
    int* node_start = nullptr;
    int* lnode_gid = nullptr;
    int* lnode_info = nullptr;
    int* lrow = nullptr;
    uint16_t* lslots = nullptr;
    ushort4* lconn = nullptr;
    int* bnd_rowptr = nullptr;
    void* partials = nullptr;   // scratch: 3 reals per partial slot
    int n_patches = 0, pe = 0, max_lnodes = 0, n_partials = 0, n_lnodes = 0, n_boundary = 0;
};

struct TfemMesh {
    int n_nodes = 0, n_tets = 0, method = METHOD_LARGE, precision = PREC_FP64;
    size_t real_size = 8;
    // element data (real type = double for FP64, float for mixed)
    int4* tets = nullptr;
    void* rot = nullptr;
    void* K = nullptr;
    void* J = nullptr;
    void* rest = nullptr;
    float2* rest_ff = nullptr;  // mixed: rest coordinates b-a, c-a, d-a (9 rows) as float-float pairs
    void* R0 = nullptr;       // initial rotation rows (for the rotation getter; the svd method's frame)
    void* A0inv = nullptr;    // svd: inverse rest edge matrix (9 rows)
    double* rest_pos = nullptr;  // rest positions (FP64, n_nodes*3), used by method=small
    int* rowptr = nullptr;
    int* slots = nullptr;
    int* elem_orig = nullptr;      // original element index of each storage position
    std::vector<int> perm_h;       // storage position -> original element index
    // assembled stiffness pattern (built on first use): BSR rows / columns on
    // the host, per-block contribution lists on the device
    std::vector<int> bsr_rowptr_h, bsr_cols_h;
    int* bsr_cptr = nullptr;
    int* bsr_contrib = nullptr;
    double* bsr_values = nullptr;
    PatchLayout pl;
    int max_valence = 0;
    void* eforce = nullptr;   // scratch: 12 reals per element (corner forces)
    int patch_grid = 0;       // CTAs of the persistent patch kernels
    int patch_threads = 128;  // threads per CTA of the patch kernels
    int matvec_minb = 1;      // CG matvec register cap: resident CTAs per SM it is set for (1: none)
    int matvec_db = 0;        // CG matvec with two sets of per-patch tables and no tail barrier
    int adddforce_grid = 0;   // CTAs of the addDForce patch kernel (128 threads)
    int force_patch_grid = 0; // CTAs of the patch force / right-hand side kernel (0: not used)
    int force_threads = 160;  // threads per CTA of that kernel
    int patch_prefetch = 0;   // 1: each CTA prefetches its next patch into L2
    int update_vec4 = 1;      // FP32 CG update: four nodes per thread with 16-byte loads
    int update_minb = 4;      // CG update: resident CTAs per SM the register cap is set for
    int update_grid = 0;      // CG update grid; 0: one thread per group of four nodes
    int* dev_flags = nullptr; // sticky device error flag: 1 = a bounded device wait ran out
    double rest_volume = 0.0;
    // plasticity (plasticMaxThreshold > 0): 6 plastic strain rows per
    // element (allocated when first enabled); mixed: per-element sqrt(K(0,0))
    void* plastic = nullptr;
    void* plastic_scale = nullptr;
    double plastic_max = 0.0, plastic_yield = 1e-4, plastic_creep = 0.9;
    int plastic_version = 0;  // bumped by every change of the settings (a captured step re-records)
    int update_j = 0;         // updateStiffnessMatrix (polar, svd): J rebuilt at every addForce
    double* vm_lame = nullptr;  // von Mises: lambda, mu per element (2 rows, computed on first use)
    std::vector<double> young_h, poisson_h;  // as given (for inspection)
    std::vector<double> lsf_h;               // localStiffnessFactor as given
    size_t device_bytes = 0;
};

// Device-side scalar state of one CG solve plus the reduction scratch.
struct CgScalars {
    double normb;
    double rho, rho_prev, den, alpha, beta;
    double last_err;
    double bnorm2;  // PCG: b.b of the current solve
    long long time_step_count;
    int done;
    int iters;
    int status;  // bit 0: non-finite value seen; bit 1: a bounded device wait ran out
    int pad;
    unsigned int ticket;
    unsigned int pad2;
    // residual replacement: the largest recurrence residual norm since the
    // solve started or was last replaced, and the iteration whose update is
    // followed by a replacement (0: none yet)
    double rmax;
    int replace_it;
    int pad3;
    double residual;  // EulerImplicitSolver computeResidual: r.r after the last step
    double partials[kMaxDotBlocks];
};

struct SceneParams {
    double dt = 0.01, rayleigh_stiffness = 0.0, rayleigh_mass = 0.0, vdamping = 0.0;
    int cg_iterations = 25;
    double cg_tolerance = 1e-5, cg_threshold = 1e-5;
    double gravity[3] = {0.0, -9.81, 0.0};
    double vertex_mass = 1.0;
    int solver = 0;   // 0 CGLinearSolver, 1 PCGLinearSolver
    int precond = 0;  // PCG: 1 Jacobi
    int precond_rate = 1;  // the preconditioner is re-assembled every this many steps
    int warm_start = 0;    // CG: start from the previous solution (warmStart)
    double ff_rs = 0.0;    // the force field's own rayleighStiffness
    double mass_rm = 0.0;  // the mass's own rayleighMass
    int first_order = 0;   // EulerImplicitSolver firstOrder
    int project_velocity = 0;  // FixedProjectiveConstraint activate_projectVelocity
    int trapezoidal = 0;       // EulerImplicitSolver trapezoidalScheme (tr = 0.5)
    int compute_residual = 0;  // EulerImplicitSolver computeResidual
    int separate_gravity = 0;  // the mass's separateGravity
};

// Factors of one EulerImplicitSolver step (EulerImplicitSolver.cpp:117-171,
// trapezoidal factor tr = 0.5 with trapezoidalScheme, else 1): the system
// matrix mF M + bF B + kF K, with the
// components' Rayleigh terms folded into the factors each component applies
// (MechanicalParams::k/mFactorIncludingRayleighDamping, MechanicalParams.h:
// 62-64), and the right-hand side's stiffness factor h + rs (bF = 0 there).
struct StepFactors {
    double mf, bf, kf;  // solver factors
    double kf_ff;       // kF + bF * force-field rayleighStiffness: what the force field's addDForce uses
    double mf_mass;     // mF - bF * mass rayleighMass: what the mass's addMDx uses
    double kf_rhs;      // h + rs, the right-hand side's K factor (second order)
};

inline StepFactors step_factors(const SceneParams& P)
{
    const double h = P.dt, tr = P.trapezoidal ? 0.5 : 1.0;
    StepFactors f;
    if (P.first_order) {
        f.mf = 1;
        f.bf = 0;
        f.kf = -h * tr;
    } else {
        f.mf = 1 + tr * h * P.rayleigh_mass;
        f.bf = -tr * h;
        f.kf = -tr * h * (tr * h + P.rayleigh_stiffness);
    }
    f.kf_ff = f.kf + f.bf * P.ff_rs;
    f.mf_mass = f.mf - f.bf * P.mass_rm;
    f.kf_rhs = h * tr + P.rayleigh_stiffness;
    return f;
}

struct Scene {
    TfemMesh* mesh = nullptr;
    bool owns_mesh = false;
    SceneParams prm;
    int n = 0;
    // state (always FP64)
    double* x = nullptr;
    double* v = nullptr;
    // per-node data
    double* node_mass = nullptr;   // optional per-node masses (DiagonalMass-style), else uniform
    uint8_t* fixed = nullptr;      // 1 = projected to zero
    void* ext = nullptr;           // optional external force (real type)
    // solver vectors (real type of the mesh precision)
    void* f = nullptr;
    void* b = nullptr;
    void* xs = nullptr;
    void* p = nullptr;
    void* p2 = nullptr;            // second CG direction buffer (patch path ping-pong)
    void* q = nullptr;
    void* r = nullptr;
    void* dinv = nullptr;          // PCG + Jacobi: inverse diagonal of the system (3 per node)
    void* eforce_v = nullptr;      // patch step: the right-hand side's K v corner terms (12 per element)
    // the patch step's force and right-hand side passes: 2 one pass over the
    // patches and one over the nodes, 1 one over the elements (eforce_v) and
    // one over the nodes, 0 the four kernels of the element-order step
    int rhs_form = 0;
    CgScalars* cg = nullptr;
    CgScalars* cg_h = nullptr;  // pinned mirror for reads
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    int graph_plastic_version = 0;  // the force field's plasticity settings the graph was recorded with
    int graph_steps = 0;
    size_t device_bytes = 0;
    // residual replacement (FP32 scenes): every `replace_every` CG iterations
    // the FP32 increment is accumulated into x64 and the residual recomputed
    // as b64 - A x64 with an FP64 copy of the operator (`shadow`)
    int replace_every = 0;
    TfemMesh* shadow = nullptr;
    double* b64 = nullptr;
    double* x64 = nullptr;
    double* w64 = nullptr;    // scratch: FP64 forces, then -kf K x64
    double* r64 = nullptr;    // FP64 residual written by the right-hand side gather
    double* ext64 = nullptr;  // external force in FP64
};

// ---------------------------------------------------------------------------
// Batched multi-mesh engine
// ---------------------------------------------------------------------------

// Unit of work of the persistent batch kernels: a patch (a = patch index), a
// range of elements [a, b) or a chunk of nodes [a, b) numbered c in its mesh.
struct WorkItem {
    int slot, a, b, c;
};

enum { WL_PATCH = 0, WL_ELEM = 1, WL_NODE = 2 };
constexpr int kBatchElemChunk = 1024;
constexpr int kBatchNodeChunk = 1024;
constexpr int kBatchMaxLocalNodes = 512;

// Local nodes of one batch patch at most: as many as the patch has elements
// (a 5-tet split of a grid gives about half as many), at most
// kBatchMaxLocalNodes; the matvec's shared memory is sized by it.
__host__ __device__ inline int batch_max_lnodes(int pe)
{
    return pe < kBatchMaxLocalNodes ? pe : kBatchMaxLocalNodes;
}

// Device-resident descriptor of one admitted mesh: its arrays (inside the
// batch's HBM arena), its solver parameters and its CG scalars. Kernels read
// it through the slot index of a work item; reductions update its scalars.
struct BMeshDesc {
    // element data, patch order
    const int4* tets;
    void* rot;
    const void* K;
    const void* J;
    const void* rest;
    const float2* rest_ff;
    void* eforce;
    void* eforce_v;  // the right-hand side's K v corner terms (fused force / right-hand side passes)
    // node -> (element*4+corner) gather table
    const int* rowptr;
    const int* slots;
    // patch layout
    const int* elem_start;
    const int* node_start;
    const int* lnode_gid;
    const int* lnode_info;
    const int* lrow;
    const uint16_t* lslots;
    const ushort4* lconn;
    const int* bnd_rowptr;
    void* partials;
    // node data
    double* x;
    double* v;
    const double* rest_pos;
    const uint8_t* fixed;
    const double* node_mass;
    const void* ext;
    void* f;
    void* b;
    void* r;
    void* p0;
    void* p1;
    void* q;
    void* xs;
    double* patch_energy;
    double* chunk_sum;
    // sizes and parameters
    int n_nodes, n_tets, method, n_patches, n_chunks, cg_iterations;
    double h, kf_rhs, rm_factor, mf, kf, vdamp, tol, thr, vertex_mass;
    double g[3];
    // CG state
    double normb, rho, rho_prev, den, alpha, beta, last_err;
    long long tsc;
    int done, iters, status, active;
    unsigned int ticket_rhs, ticket_den, ticket_rho, ticket_pad;
};

// The register-cap variants of the batch matvec (resident CTAs per SM).
constexpr int kBatchMatvecMinb[3] = {5, 6, 8};

// Launch tiles of a batch step. None of them changes a result bit: every
// per-mesh reduction is formed per work item in an order fixed by the item.
struct BatchTiles {
    int matvec_minb = 6;  // the matvec's register cap: resident CTAs per SM (kBatchMatvecMinb)
    int update_npt = 4;   // nodes per thread of the CG update (1, 2 or 4)
    int update_ctas = 4;  // CG-update CTAs per SM
    int elem_ctas = 4;    // element-kernel CTAs per SM
    int prefetch = 0;     // matvec: L2 prefetch of a block's next patch
};

// Everything a precision variant needs to record one batch step.
struct BatchLaunch {
    BMeshDesc* meshes;
    const WorkItem* items[3];
    const int* counts;
    int grid_patch, grid_elem, grid_node, grid_slots;
    int grid_update;   // CTAs of the CG update
    int matvec_minb;   // register-cap variant of the matvec
    int update_npt;    // nodes per thread of the CG update
    int n_slots;  // mesh slots of the batch (the CG scalar kernels take one block per slot)
    int pe;
    int max_iterations;
    int prefetch;  // FP32 matvec: prefetch the block's next patch into L2
    // forces and right-hand side: 2 by patches and by node chunks (mixed),
    // 1 by elements (the meshes carry eforce_v) and by node chunks, 0 the
    // four passes of the element-order step
    int fused_rhs;
    int grid_force;  // CTAs of the patch force / right-hand side pass
    int* err;    // sticky device error flag of the batch
};

// Forces and right-hand side of the FP32 patch step and of the batch in two
// passes, by patches (2) or by elements (1: SGB_PATCH_RHS=0), or in the four
// passes of the element-order step (0: SGB_FUSED_RHS=0); batch.cu.
int fused_rhs_default();

// von Mises stress (von_mises.cu): per-element lambda and mu, then the
// per-element values (caller's order) and the per-node means.
void launch_lame(const TfemMesh* m, const double* young, int ny, const double* poisson, int np, const double* lsf,
                 int nl, double* lame, cudaStream_t s);
void launch_von_mises(const TfemMesh* m, int mode, const double* x, const double* lame, double* per_element,
                      double* per_node, cudaStream_t s);

}  // namespace sgb
