// Host side of the batched multi-mesh engine: a fixed HBM arena with a
// first-fit allocator (the admission budget), mesh admission and removal,
// the device work lists, and the CUDA graph of one batch step. The graph
// reads the work lists and mesh descriptors from device memory, so meshes can
// join and leave between steps without recording it again.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "batch_internal.h"

namespace sgb {
void set_last_error(const std::string& msg);
}

using namespace sgb;

namespace {

int bfail(int code, const std::string& msg)
{
    set_last_error(msg);
    return code;
}

int bcuda(cudaError_t e, const char* what)
{
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SGB_ERR_OUT_OF_MEMORY : SGB_ERR_CUDA;
}

#define BTRY(expr)                                    \
    do {                                              \
        cudaError_t _e = (expr);                      \
        if (_e != cudaSuccess) return bcuda(_e, #expr); \
    } while (0)

constexpr size_t kAlign = 256;

inline size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Sub-allocations of one mesh inside its arena block.
struct Carve {
    size_t total = 0;
    std::vector<std::pair<void**, size_t>> items;
    template <typename T>
    void add(T** p, size_t bytes)
    {
        items.push_back({(void**)p, align_up(bytes == 0 ? 16 : bytes)});
        total += items.back().second;
    }
    void place(char* base)
    {
        size_t off = 0;
        for (auto& it : items) {
            *it.first = base + off;
            off += it.second;
        }
    }
};

}  // namespace


namespace sgb {
void Arena::reset(char* b, size_t n)
{
    base = b;
    size = n;
    free_.clear();
    free_[0] = n;
    used = 0;
}
bool Arena::alloc(size_t n, size_t* off)
{
    n = (n + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            *off = it->first;
            const size_t rest = it->second - n;
            const size_t o = it->first + n;
            free_.erase(it);
            if (rest) free_[o] = rest;
            used += n;
            return true;
        }
    }
    return false;
}
void Arena::release(size_t off, size_t n)
{
    n = (n + 255) / 256 * 256;
    used -= n;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}
size_t Arena::largest_free() const
{
    size_t m = 0;
    for (auto& kv : free_) m = std::max(m, kv.second);
    return m;
}
}  // namespace sgb

static size_t mesh_plan(sgb_batch* B, int N, int E, const HostLayout& L, bool node_mass, bool ext, Carve& c,
                        BMeshDesc& d, double** young, double** poisson, int** elem_orig, size_t ny, size_t np)
{
    const size_t rs = B->rs;
    const int P = (int)L.elem_start.size() - 1;
    const int chunks = (N + kBatchNodeChunk - 1) / kBatchNodeChunk;
    c.add((int4**)&d.tets, sizeof(int4) * E);
    c.add(&d.rot, rs * 9 * E);
    c.add((void**)&d.K, rs * 3 * E);
    c.add((void**)&d.J, rs * 12 * E);
    c.add((void**)&d.rest, rs * 12 * E);
    d.rest_ff = nullptr;
    if (rs == sizeof(float)) c.add((float2**)&d.rest_ff, sizeof(float2) * 9 * E);
    c.add(&d.eforce, rs * 12 * E);
    d.eforce_v = nullptr;
    if (B->fused_rhs == 1) c.add(&d.eforce_v, rs * 12 * E);
    c.add((int**)&d.rowptr, sizeof(int) * (N + 1));
    c.add((int**)&d.slots, sizeof(int) * 4 * (size_t)E);
    c.add((int**)&d.elem_start, sizeof(int) * (P + 1));
    c.add((int**)&d.node_start, sizeof(int) * (P + 1));
    c.add((int**)&d.lnode_gid, sizeof(int) * L.lnode_gid.size());
    c.add((int**)&d.lnode_info, sizeof(int) * L.lnode_info.size());
    c.add((int**)&d.lrow, sizeof(int) * L.lrow.size());
    c.add((uint16_t**)&d.lslots, sizeof(uint16_t) * (L.lslots.size() + 8));
    c.add((ushort4**)&d.lconn, sizeof(ushort4) * (L.lconn.size() + 2));
    c.add((int**)&d.bnd_rowptr, sizeof(int) * (N + 1));
    c.add(&d.partials, rs * 3 * (size_t)std::max(L.n_partials, 1));
    c.add(&d.x, sizeof(double) * 3 * N);
    c.add(&d.v, sizeof(double) * 3 * N);
    c.add((double**)&d.rest_pos, sizeof(double) * 3 * N);
    c.add((uint8_t**)&d.fixed, (size_t)N);
    if (node_mass) c.add((double**)&d.node_mass, sizeof(double) * N);
    if (ext) c.add((void**)&d.ext, rs * 3 * N);
    c.add(&d.f, rs * 3 * N);
    c.add(&d.b, rs * 3 * N);
    c.add(&d.r, rs * 3 * N);
    c.add(&d.p0, rs * 3 * N);
    c.add(&d.p1, rs * 3 * N);
    c.add(&d.q, rs * 3 * N);
    c.add(&d.xs, rs * 3 * N);
    c.add(&d.patch_energy, sizeof(double) * std::max(P, 1));
    c.add(&d.chunk_sum, sizeof(double) * std::max(chunks, 1));
    c.add(elem_orig, sizeof(int) * E);
    c.add(young, sizeof(double) * ny);
    c.add(poisson, sizeof(double) * np);
    return c.total;
}

// Each mesh's items are contiguous and in mesh-local index order in every
// list: the kernels' per-mesh reductions index their block partials by it.
static void rebuild_work_lists(sgb_batch* B, std::vector<WorkItem> wl[3])
{
    for (int k = 0; k < 3; ++k) wl[k].clear();
    for (int s = 0; s < B->max_slots; ++s) {
        const BatchMeshHost& m = B->slots[(size_t)s];
        if (!m.active) continue;
        for (int p = 0; p < m.n_patches; ++p) wl[WL_PATCH].push_back({s, p, 0, 0});
        for (int e = 0; e < m.n_tets; e += kBatchElemChunk)
            wl[WL_ELEM].push_back({s, e, std::min(m.n_tets, e + kBatchElemChunk), 0});
        for (int c = 0, n = 0; n < m.n_nodes; n += kBatchNodeChunk, ++c)
            wl[WL_NODE].push_back({s, n, std::min(m.n_nodes, n + kBatchNodeChunk), c});
    }
}

static int upload_work_lists(sgb_batch* B)
{
    std::vector<WorkItem> wl[3];
    rebuild_work_lists(B, wl);
    for (int k = 0; k < 3; ++k) {
        const int need = (int)wl[k].size();
        if (need > B->cap[k]) {
            int cap = std::max(need, 2 * B->cap[k]);
            cap = std::max(cap, 1024);
            BTRY(cudaStreamSynchronize(B->stream));
            cudaFree(B->d_items[k]);
            B->d_items[k] = nullptr;
            BTRY(cudaMalloc((void**)&B->d_items[k], sizeof(WorkItem) * cap));
            B->cap[k] = cap;
            B->graph_valid = false;  // the step graph bakes the list pointers
        }
        if (need) BTRY(cudaMemcpyAsync(B->d_items[k], wl[k].data(), sizeof(WorkItem) * need, cudaMemcpyHostToDevice,
                                       B->stream));
        B->counts_h[k] = need;
    }
    BTRY(cudaMemcpyAsync(B->d_counts, B->counts_h, sizeof(int) * 3, cudaMemcpyHostToDevice, B->stream));
    // the host copy must stay valid until the copy has run
    BTRY(cudaStreamSynchronize(B->stream));
    return SGB_OK;
}

extern "C" {

int sgb_batch_create(sgb_batch_t** out, int precision, size_t hbm_budget_bytes, int max_meshes, int max_cg_iterations)
{
    if (!out) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_create: out is NULL");
    *out = nullptr;
    const VariantOps* ops = variant_for(precision);
    if (!ops || !ops->batch_record)
        return bfail(SGB_ERR_NOT_SUPPORTED, "sgb_batch_create: batching needs SGB_PRECISION_MIXED or FP64_FMA");
    if (max_meshes <= 0 || max_cg_iterations < 0 || hbm_budget_bytes < (1u << 20))
        return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_create: invalid capacity");
    sgb_batch* B = new sgb_batch();
    B->ops = ops;
    B->precision = precision;
    B->rs = ops->real_size;
    // elements per patch (512 FP32, 256 FP64); SGB_BATCH_PE overrides the FP32
    // value (even, in [64, 512]); SGB_BATCH_PREFETCH=1 turns on the L2
    // prefetch of a block's next patch
    B->pe = B->rs == 4 ? 512 : 256;
    if (B->rs == 4)
        if (const char* e = getenv("SGB_BATCH_PE")) {
            const int v = atoi(e);
            if (v >= 64 && v <= 512 && v % 2 == 0) B->pe = v;
        }
    if (const char* e = getenv("SGB_BATCH_PREFETCH")) B->tiles.prefetch = (e[0] == '1');
    B->fused_rhs = batch_rhs_form(fused_rhs_default(), B->rs);
    B->max_slots = max_meshes;
    B->max_iterations = max_cg_iterations;
    B->slots.resize((size_t)max_meshes);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc((void**)&B->arena_mem, hbm_budget_bytes)) != cudaSuccess ||
        (e = cudaMalloc((void**)&B->d_meshes, sizeof(BMeshDesc) * max_meshes)) != cudaSuccess ||
        (e = cudaMalloc((void**)&B->d_counts, sizeof(int) * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&B->d_err, sizeof(int))) != cudaSuccess ||
        (e = cudaMemset(B->d_meshes, 0, sizeof(BMeshDesc) * max_meshes)) != cudaSuccess ||
        (e = cudaMemset(B->d_counts, 0, sizeof(int) * 4)) != cudaSuccess ||
        (e = cudaMemset(B->d_err, 0, sizeof(int))) != cudaSuccess) {
        int rc = bcuda(e, "sgb_batch_create");
        sgb_batch_destroy(B);
        return rc;
    }
    B->arena.reset(B->arena_mem, hbm_budget_bytes);
    B->device_bytes = hbm_budget_bytes + sizeof(BMeshDesc) * max_meshes;
    B->sms = ops->batch_prepare(B->pe, B->grid_patch_v);
    if (B->sms <= 0) {
        sgb_batch_destroy(B);
        return bfail(SGB_ERR_CUDA, "sgb_batch_create: kernel attributes");
    }
    int rc = upload_work_lists(B);
    if (rc) {
        sgb_batch_destroy(B);
        return rc;
    }
    *out = B;
    return SGB_OK;
}

int sgb_batch_destroy(sgb_batch_t* B)
{
    if (!B) return SGB_OK;
    if (B->stream) cudaStreamSynchronize(B->stream);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    for (int k = 0; k < 3; ++k) cudaFree(B->d_items[k]);
    cudaFree(B->d_counts);
    cudaFree(B->d_err);
    cudaFree(B->d_meshes);
    cudaFree(B->arena_mem);
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
    return SGB_OK;
}

static int validate_mesh(const sgb_mesh_desc* m)
{
    if (!m) return bfail(SGB_ERR_INVALID_ARGUMENT, "mesh description is NULL");
    if (m->n_nodes <= 0 || !m->rest_positions_host || m->n_tets <= 0 || !m->tetrahedra_host)
        return bfail(SGB_ERR_INVALID_ARGUMENT, "a batched mesh needs nodes and tetrahedra");
    if (m->method != SGB_METHOD_LARGE && m->method != SGB_METHOD_POLAR)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes use method large or polar");
    for (size_t i = 0; i < (size_t)m->n_tets * 4; ++i)
        if (m->tetrahedra_host[i] < 0 || m->tetrahedra_host[i] >= m->n_nodes)
            return bfail(SGB_ERR_INVALID_ARGUMENT, "tetrahedron node index out of range");
    for (size_t i = 0; i < (size_t)m->n_nodes * 3; ++i)
        if (!std::isfinite(m->rest_positions_host[i]))
            return bfail(SGB_ERR_INVALID_ARGUMENT, "non-finite rest position");
    const sgb_scene_params& p = m->params;
    if (!(p.dt > 0) || p.cg_iterations < 0 || !(p.cg_tolerance >= 0) || !(p.cg_threshold >= 0))
        return bfail(SGB_ERR_INVALID_ARGUMENT, "invalid solver parameters");
    if (p.n_fixed < 0 || (p.n_fixed > 0 && !p.fixed_host))
        return bfail(SGB_ERR_INVALID_ARGUMENT, "invalid fixed indices");
    // the batch kernels run plain cold-start CGLinearSolver with block-ordered
    // dot products: options that would change the solve are refused rather
    // than ignored
    if (p.linear_solver != SGB_SOLVER_CG)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes use CGLinearSolver (linear_solver = SGB_SOLVER_CG)");
    if (p.preconditioner != SGB_PRECOND_NONE)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes take no preconditioner");
    if (p.warm_start) return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes do not support CG warmStart");
    if (p.residual_replacement > 0)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes do not support residual replacement");
    if (p.serial_dots)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes sum dot products per block, not serially (serial_dots)");
    if (p.first_order) return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes run the second-order Euler scheme");
    if (p.compute_residual)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes do not compute EulerImplicitSolver's residual");
    if (p.separate_gravity) return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes add gravity as a force");
    if (p.project_velocity)
        return bfail(SGB_ERR_NOT_SUPPORTED, "batched meshes do not support activate_projectVelocity");
    if (!std::isfinite(p.ff_rayleigh_stiffness) || !std::isfinite(p.mass_rayleigh_mass))
        return bfail(SGB_ERR_INVALID_ARGUMENT, "non-finite component Rayleigh coefficient");
    return SGB_OK;
}

int sgb_batch_mesh_bytes(const sgb_batch_t* B, const sgb_mesh_desc* m, size_t* bytes)
{
    if (!bytes) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_mesh_bytes: NULL argument");
    // no batch: plan for a mixed-precision batch with the default patch size
    const int pe = B ? B->pe : 512;
    const size_t rs = B ? B->rs : sizeof(float);
    PreparedMesh pm;
    int rc = prepare_mesh(m, pe, rs, pm, B ? B->fused_rhs : fused_rhs_default());
    if (rc) return rc;
    *bytes = pm.bytes;
    return SGB_OK;
}

int sgb_batch_add_mesh(sgb_batch_t* B, const sgb_mesh_desc* m, int* slot_out)
{
    if (!B || !slot_out) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_add_mesh: NULL argument");
    *slot_out = -1;
    PreparedMesh pm;
    int rc = prepare_mesh(m, B->pe, B->rs, pm, B->fused_rhs);
    if (rc) return rc;
    return admit_prepared(B, pm, slot_out);
}

}  // extern "C"

namespace sgb {

// SGB_FUSED_RHS=0: the force and right-hand side run as four passes (the
// same operations); SGB_PATCH_RHS=0: as one pass over the elements (the
// meshes carry eforce_v) and one over the nodes; else by patches.
int fused_rhs_default()
{
    const char* e = getenv("SGB_FUSED_RHS");
    if (e && e[0] == '0') return 0;
    const char* p = getenv("SGB_PATCH_RHS");
    return (p && p[0] == '0') ? 1 : 2;
}

// The batch's form of those passes: by patches in mixed precision only (the
// FP64 batch keeps the element-order pair).
int batch_rhs_form(int fused_rhs, size_t rs) { return (fused_rhs == 2 && rs != sizeof(float)) ? 1 : fused_rhs; }

// Host-only part of admission: validation, material checks like the
// reference (BaseLinearElasticityFEMForceField.inl:53-85), element order,
// patch layout, gather tables and the byte count. Safe on any thread.

int prepare_mesh(const sgb_mesh_desc* m, int pe, size_t rs, PreparedMesh& pm, int fused_rhs)
{
    int rc = validate_mesh(m);
    if (rc) return rc;
    const int N = m->n_nodes, E = m->n_tets;
    pm.N = N;
    pm.E = E;
    pm.method = m->method;
    pm.P = m->params;
    pm.rest.assign(m->rest_positions_host, m->rest_positions_host + 3 * (size_t)N);
    if (m->young && m->n_young > 0) pm.Eh.assign(m->young, m->young + m->n_young);
    if (m->poisson && m->n_poisson > 0) pm.nuh.assign(m->poisson, m->poisson + m->n_poisson);
    if (pm.Eh.empty()) pm.Eh.push_back(5000.0);
    if (pm.nuh.empty()) pm.nuh.push_back(0.45);
    for (double& y : pm.Eh)
        if (!(y >= 0)) y = 5000.0;
    for (double& v : pm.nuh)
        if (!(v >= 0 && v < 0.5)) v = 0.45;
    build_patch_layout(N, E, m->tetrahedra_host, m->rest_positions_host, pe, batch_max_lnodes(pe), pm.L);
    int maxval = 0;
    build_node_csr(N, E, m->tetrahedra_host, pm.L.inv, pm.rowptr, pm.slots, maxval);
    pm.tets_store.resize((size_t)E * 4);
    for (size_t s = 0; s < (size_t)E; ++s)
        for (int c = 0; c < 4; ++c) pm.tets_store[4 * s + c] = m->tetrahedra_host[4 * (size_t)pm.L.perm[s] + c];
    pm.fixed.assign((size_t)N, 0);
    const sgb_scene_params& P = m->params;
    if (P.fix_all)
        std::fill(pm.fixed.begin(), pm.fixed.end(), 1);
    else
        for (int i = 0; i < P.n_fixed; ++i)
            if (P.fixed_host[i] >= 0 && P.fixed_host[i] < N) pm.fixed[(size_t)P.fixed_host[i]] = 1;
    if (P.node_masses_host) pm.node_mass.assign(P.node_masses_host, P.node_masses_host + N);
    if (m->external_force_host) pm.ext.assign(m->external_force_host, m->external_force_host + 3 * (size_t)N);
    pm.P.fixed_host = nullptr;
    pm.P.node_masses_host = nullptr;
    Carve c;
    BMeshDesc d{};
    double *y, *p;
    int* eo;
    sgb_batch tmp;
    tmp.rs = rs;
    tmp.fused_rhs = batch_rhs_form(fused_rhs, rs);
    pm.bytes = align_up(mesh_plan(&tmp, N, E, pm.L, !pm.node_mass.empty(), !pm.ext.empty(), c, d, &y, &p, &eo,
                                  pm.Eh.size(), pm.nuh.size()));
    return SGB_OK;
}

// Device part of admission: arena block, uploads, per-element init,
// descriptor and work lists. Synchronous on the batch stream.
int admit_prepared(sgb_batch* B, PreparedMesh& pm, int* slot_out)
{
    *slot_out = -1;
    int slot = -1;
    for (int s = 0; s < B->max_slots; ++s)
        if (!B->slots[(size_t)s].active) {
            slot = s;
            break;
        }
    if (slot < 0) return bfail(SGB_ERR_BUDGET, "sgb_batch_add_mesh: every mesh slot is taken");
    const int N = pm.N, E = pm.E;
    const sgb_scene_params& P = pm.P;
    const HostLayout& L = pm.L;
    Carve c;
    BMeshDesc d{};
    double *d_young = nullptr, *d_poisson = nullptr;
    int* d_elem_orig = nullptr;
    const size_t bytes = mesh_plan(B, N, E, L, !pm.node_mass.empty(), !pm.ext.empty(), c, d, &d_young, &d_poisson,
                                   &d_elem_orig, pm.Eh.size(), pm.nuh.size());
    size_t off = 0;
    if (!B->arena.alloc(bytes, &off))
        return bfail(SGB_ERR_BUDGET, "sgb_batch_add_mesh: the mesh needs " + std::to_string(bytes) +
                                         " bytes, the HBM budget has " + std::to_string(B->arena.largest_free()) +
                                         " contiguous bytes left");
    c.place(B->arena.base + off);
    const size_t rs = B->rs;
    const int Pn = (int)L.elem_start.size() - 1;
    const int chunks = (N + kBatchNodeChunk - 1) / kBatchNodeChunk;
    cudaStream_t s = B->stream;
    std::vector<float> ext32;
    auto fail_free = [&](int code) {
        cudaStreamSynchronize(s);
        B->arena.release(off, bytes);
        return code;
    };
#define BUP(dst, src, n)                                                                                      \
    do {                                                                                                      \
        if ((n) > 0) {                                                                                        \
            cudaError_t _e = cudaMemcpyAsync((void*)(dst), (const void*)(src), (n), cudaMemcpyHostToDevice, s); \
            if (_e != cudaSuccess) return fail_free(bcuda(_e, "upload"));                                     \
        }                                                                                                     \
    } while (0)
    BUP(d.tets, pm.tets_store.data(), sizeof(int4) * E);
    BUP(d_elem_orig, L.perm.data(), sizeof(int) * E);
    BUP(d.rowptr, pm.rowptr.data(), sizeof(int) * pm.rowptr.size());
    BUP(d.slots, pm.slots.data(), sizeof(int) * pm.slots.size());
    BUP(d.elem_start, L.elem_start.data(), sizeof(int) * L.elem_start.size());
    BUP(d.node_start, L.node_start.data(), sizeof(int) * L.node_start.size());
    BUP(d.lnode_gid, L.lnode_gid.data(), sizeof(int) * L.lnode_gid.size());
    BUP(d.lnode_info, L.lnode_info.data(), sizeof(int) * L.lnode_info.size());
    BUP(d.lrow, L.lrow.data(), sizeof(int) * L.lrow.size());
    BUP(d.lslots, L.lslots.data(), sizeof(uint16_t) * L.lslots.size());
    BUP(d.lconn, L.lconn.data(), sizeof(ushort4) * L.lconn.size());
    BUP(d.bnd_rowptr, L.bnd_rowptr.data(), sizeof(int) * L.bnd_rowptr.size());
    BUP(d.rest_pos, pm.rest.data(), sizeof(double) * 3 * N);
    BUP(d.x, pm.rest.data(), sizeof(double) * 3 * N);
    BUP(d.fixed, pm.fixed.data(), (size_t)N);
    BUP(d_young, pm.Eh.data(), sizeof(double) * pm.Eh.size());
    BUP(d_poisson, pm.nuh.data(), sizeof(double) * pm.nuh.size());
    if (!pm.node_mass.empty()) BUP(d.node_mass, pm.node_mass.data(), sizeof(double) * N);
    if (!pm.ext.empty()) {
        if (rs == sizeof(double)) {
            BUP(d.ext, pm.ext.data(), sizeof(double) * 3 * N);
        } else {
            ext32.resize((size_t)3 * N);
            for (size_t i = 0; i < ext32.size(); ++i) ext32[i] = (float)pm.ext[i];
            BUP(d.ext, ext32.data(), sizeof(float) * ext32.size());
        }
    }
#undef BUP
    cudaError_t ce;
    if ((ce = cudaMemsetAsync(d.v, 0, sizeof(double) * 3 * N, s)) || (ce = cudaMemsetAsync(d.p0, 0, rs * 3 * N, s)) ||
        (ce = cudaMemsetAsync(d.p1, 0, rs * 3 * N, s)) || (ce = cudaMemsetAsync(d.xs, 0, rs * 3 * N, s)))
        return fail_free(bcuda(ce, "cudaMemsetAsync"));
    // per-element init (TetrahedronFEMForceField::reinit) through the variant's kernel
    TfemMesh tmp;
    tmp.n_nodes = N;
    tmp.n_tets = E;
    tmp.method = pm.method;
    tmp.precision = B->precision;
    tmp.real_size = rs;
    tmp.tets = (int4*)d.tets;
    tmp.rot = d.rot;
    tmp.K = (void*)d.K;
    tmp.J = (void*)d.J;
    tmp.rest = (void*)d.rest;
    tmp.rest_ff = const_cast<float2*>(d.rest_ff);
    tmp.R0 = d.eforce;  // the initial rotation is not kept: the scratch takes it
    tmp.rest_pos = (double*)d.rest_pos;
    tmp.elem_orig = d_elem_orig;
    // element volumes land in the scratch too, after the initial rotations
    double* vol = (double*)((char*)d.eforce + ((rs * 9 * (size_t)E + 7) & ~(size_t)7));
    B->ops->init(&tmp, d_young, (int)pm.Eh.size(), d_poisson, (int)pm.nuh.size(), nullptr, 0, vol, s);
    tmp = TfemMesh();  // the arena owns these buffers
    if ((ce = cudaGetLastError()) != cudaSuccess) return fail_free(bcuda(ce, "init kernel"));
    d.n_nodes = N;
    d.n_tets = E;
    d.method = pm.method;
    d.n_patches = Pn;
    d.n_chunks = chunks;
    d.cg_iterations = std::min(P.cg_iterations, B->max_iterations);
    const double h = P.dt;
    d.h = h;
    // solver factors with the components' own Rayleigh terms folded in
    // (kFactor/mFactorIncludingRayleighDamping, MechanicalParams.h:62-64)
    SceneParams sp;
    sp.dt = h;
    sp.rayleigh_stiffness = P.rayleigh_stiffness;
    sp.rayleigh_mass = P.rayleigh_mass;
    sp.ff_rs = P.ff_rayleigh_stiffness;
    sp.mass_rm = P.mass_rayleigh_mass;
    sp.trapezoidal = P.trapezoidal_scheme ? 1 : 0;
    const StepFactors F = step_factors(sp);
    d.kf_rhs = F.kf_rhs;
    d.rm_factor = -P.rayleigh_mass;
    d.mf = F.mf_mass;
    d.kf = F.kf_ff;
    d.vdamp = (P.vdamping != 0.0) ? std::exp(-h * P.vdamping) : 1.0;
    d.tol = P.cg_tolerance;
    d.thr = P.cg_threshold;
    d.vertex_mass = P.vertex_mass;
    for (int k = 0; k < 3; ++k) d.g[k] = P.gravity[k];
    d.active = 1;
    if ((ce = cudaMemcpyAsync(&B->d_meshes[slot], &d, sizeof(BMeshDesc), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return fail_free(bcuda(ce, "descriptor upload"));
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return fail_free(bcuda(ce, "admission"));
    BatchMeshHost& hm = B->slots[(size_t)slot];
    hm.active = true;
    hm.off = off;
    hm.bytes = bytes;
    hm.n_nodes = N;
    hm.n_tets = E;
    hm.n_patches = Pn;
    hm.n_chunks = chunks;
    hm.steps = 0;
    hm.perm = L.perm;
    hm.d = d;
    int rc = upload_work_lists(B);
    if (rc) return rc;
    *slot_out = slot;
    return SGB_OK;
}

}  // namespace sgb

extern "C" {

int sgb_batch_add_meshes(sgb_batch_t* B, const sgb_mesh_desc* meshes, int n, int* slots, int threads)
{
    if (!B || n < 0 || (n > 0 && (!meshes || !slots)))
        return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_add_meshes: invalid argument");
    if (threads < 1) threads = 1;
    std::vector<PreparedMesh> pms((size_t)n);
    std::vector<int> rcs((size_t)n, SGB_OK);
    std::vector<std::string> errs((size_t)n);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (int i = t; i < n; i += threads) {
                rcs[(size_t)i] = prepare_mesh(&meshes[i], B->pe, B->rs, pms[(size_t)i], B->fused_rhs);
                if (rcs[(size_t)i]) errs[(size_t)i] = sgb_last_error();
            }
        });
    for (auto& th : pool) th.join();
    for (int i = 0; i < n; ++i) slots[i] = -1;
    for (int i = 0; i < n; ++i) {
        if (rcs[(size_t)i]) return bfail(rcs[(size_t)i], "mesh " + std::to_string(i) + ": " + errs[(size_t)i]);
        int rc = admit_prepared(B, pms[(size_t)i], &slots[i]);
        pms[(size_t)i] = PreparedMesh();
        if (rc) return rc;
    }
    return SGB_OK;
}

int sgb_batch_remove_mesh(sgb_batch_t* B, int slot)
{
    if (!B || slot < 0 || slot >= B->max_slots || !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_remove_mesh: no mesh in that slot");
    BatchMeshHost& hm = B->slots[(size_t)slot];
    BTRY(cudaStreamSynchronize(B->stream));
    BMeshDesc zero{};
    BTRY(cudaMemcpy(&B->d_meshes[slot], &zero, sizeof(BMeshDesc), cudaMemcpyHostToDevice));
    B->arena.release(hm.off, hm.bytes);
    hm = BatchMeshHost();
    return upload_work_lists(B);
}

int sgb_batch_step(sgb_batch_t* B, int n_steps)
{
    if (!B || n_steps < 0) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_step: invalid argument");
    if (!B->graph_valid) {
        if (B->graph) {
            cudaGraphExecDestroy(B->graph);
            B->graph = nullptr;
        }
        BatchLaunch L;
        L.meshes = B->d_meshes;
        for (int k = 0; k < 3; ++k) L.items[k] = B->d_items[k];
        L.counts = B->d_counts;
        const BatchTiles& T = B->tiles;
        const int mi = T.matvec_minb == kBatchMatvecMinb[0] ? 0 : (T.matvec_minb == kBatchMatvecMinb[2] ? 2 : 1);
        L.grid_patch = B->grid_patch_v[mi];
        L.matvec_minb = kBatchMatvecMinb[mi];
        L.grid_elem = B->sms * T.elem_ctas;
        L.grid_node = B->sms * 4;
        L.grid_update = B->sms * T.update_ctas;
        L.update_npt = T.update_npt;
        L.n_slots = B->max_slots;
        L.grid_slots = std::min(B->max_slots, B->sms * 8);
        L.pe = B->pe;
        L.max_iterations = B->max_iterations;
        L.prefetch = T.prefetch;
        L.fused_rhs = B->fused_rhs;
        L.grid_force = B->grid_patch_v[3];
        L.err = B->d_err;
        cudaGraph_t g;
        BTRY(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
        B->ops->batch_record(L, B->stream);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(B->stream, &g);
        if (le != cudaSuccess) return bcuda(le, "batch step launch");
        if (ce != cudaSuccess) return bcuda(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&B->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return bcuda(ce, "cudaGraphInstantiate");
        B->graph_valid = true;
    }
    for (int i = 0; i < n_steps; ++i) BTRY(cudaGraphLaunch(B->graph, B->stream));
    for (auto& m : B->slots)
        if (m.active) m.steps += n_steps;
    return SGB_OK;
}

int sgb_batch_sync(sgb_batch_t* B)
{
    if (!B) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_sync: NULL batch");
    int err = 0;
    BTRY(cudaMemcpyAsync(&err, B->d_err, sizeof(int), cudaMemcpyDeviceToHost, B->stream));
    BTRY(cudaStreamSynchronize(B->stream));
    if (err) return bfail(SGB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait ran out in the batch step");
    return SGB_OK;
}

int sgb_batch_mesh_stats(sgb_batch_t* B, int slot, int* cg_iterations, double* cg_residual, long long* steps)
{
    if (!B || slot < 0 || slot >= B->max_slots || !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_mesh_stats: no mesh in that slot");
    BMeshDesc d;
    BTRY(cudaMemcpyAsync(&d, &B->d_meshes[slot], sizeof(BMeshDesc), cudaMemcpyDeviceToHost, B->stream));
    BTRY(cudaStreamSynchronize(B->stream));
    if (cg_iterations) *cg_iterations = d.iters;
    if (cg_residual) *cg_residual = d.last_err;
    if (steps) *steps = B->slots[(size_t)slot].steps;
    if (d.status & 1) return bfail(SGB_ERR_NUMERICAL, "non-finite value in this mesh's CG solve");
    if (d.status & 2) return bfail(SGB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait ran out in this mesh's solve");
    return SGB_OK;
}

int sgb_batch_get_state(sgb_batch_t* B, int slot, double* x_host, double* v_host)
{
    if (!B || slot < 0 || slot >= B->max_slots || !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_get_state: no mesh in that slot");
    const BatchMeshHost& hm = B->slots[(size_t)slot];
    const size_t bytes = sizeof(double) * 3 * (size_t)hm.n_nodes;
    if (x_host) BTRY(cudaMemcpyAsync(x_host, hm.d.x, bytes, cudaMemcpyDeviceToHost, B->stream));
    if (v_host) BTRY(cudaMemcpyAsync(v_host, hm.d.v, bytes, cudaMemcpyDeviceToHost, B->stream));
    BTRY(cudaStreamSynchronize(B->stream));
    return SGB_OK;
}

int sgb_batch_get_positions_async(sgb_batch_t* B, int slot, double* x_host)
{
    if (!B || !x_host || slot < 0 || slot >= B->max_slots || !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_get_positions_async: no mesh in that slot");
    const BatchMeshHost& hm = B->slots[(size_t)slot];
    BTRY(cudaMemcpyAsync(x_host, hm.d.x, sizeof(double) * 3 * (size_t)hm.n_nodes, cudaMemcpyDeviceToHost,
                         B->stream));
    return SGB_OK;
}

int sgb_batch_set_state(sgb_batch_t* B, int slot, const double* x_host, const double* v_host)
{
    if (!B || slot < 0 || slot >= B->max_slots || !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_set_state: no mesh in that slot");
    const BatchMeshHost& hm = B->slots[(size_t)slot];
    const size_t bytes = sizeof(double) * 3 * (size_t)hm.n_nodes;
    if (x_host) BTRY(cudaMemcpyAsync(hm.d.x, x_host, bytes, cudaMemcpyHostToDevice, B->stream));
    if (v_host) BTRY(cudaMemcpyAsync(hm.d.v, v_host, bytes, cudaMemcpyHostToDevice, B->stream));
    BTRY(cudaStreamSynchronize(B->stream));
    return SGB_OK;
}

// ---- launch-tile tuner ------------------------------------------------------
// The batch step's launch tiles (the matvec's register cap, the CG update's
// nodes per thread and grid, the element kernels' grid, the L2 prefetch) are
// picked by timing the admitted mix: one coordinate at a time from the
// current choice, each candidate timed with CUDA events over a few whole
// steps that all start from the same saved state, which is put back
// afterwards. Every tile is rounding-neutral, so tuning changes no result.
// The reference sets its equivalent knobs by hand (gatherPt / gatherBsize of
// SofaCUDA's TetrahedronFEMForceField). Choices are cached per process by the
// mix's size histogram, so a batch with the same kind of mix skips the timing.

namespace {

std::mutex g_tile_cache_mutex;
std::map<std::string, BatchTiles> g_tile_cache;

std::string mix_key(const sgb_batch* B)
{
    // meshes per power-of-two size class of their tetrahedron count, the
    // counts themselves rounded to powers of two
    int hist[40] = {0};
    for (auto& m : B->slots)
        if (m.active) {
            int b = 0;
            while (b < 39 && (1LL << (b + 1)) <= (long long)m.n_tets) ++b;
            hist[b]++;
        }
    std::string key = std::to_string(B->precision) + "/" + std::to_string(B->pe) + "/" + std::to_string(B->sms) + ":";
    for (int b = 0; b < 40; ++b)
        if (hist[b]) {
            int q = 0;
            while ((1 << (q + 1)) <= hist[b]) ++q;
            key += std::to_string(b) + "x" + std::to_string(q) + ",";
        }
    return key;
}

// What a step changes: every mesh's positions and velocities, the device
// descriptors (time-step counts, CG scalars, status), the host step counters
// and the device error flag.
struct BatchSnapshot {
    std::vector<BMeshDesc> desc;
    std::vector<std::vector<double>> x, v;
    std::vector<long long> steps;
    int err = 0;
};

int snapshot_take(sgb_batch* B, BatchSnapshot& S)
{
    BTRY(cudaStreamSynchronize(B->stream));
    S.desc.resize((size_t)B->max_slots);
    BTRY(cudaMemcpy(S.desc.data(), B->d_meshes, sizeof(BMeshDesc) * B->max_slots, cudaMemcpyDeviceToHost));
    BTRY(cudaMemcpy(&S.err, B->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    S.x.assign((size_t)B->max_slots, {});
    S.v.assign((size_t)B->max_slots, {});
    S.steps.assign((size_t)B->max_slots, 0);
    for (int i = 0; i < B->max_slots; ++i) {
        const BatchMeshHost& m = B->slots[(size_t)i];
        if (!m.active) continue;
        const size_t n = 3 * (size_t)m.n_nodes;
        S.x[(size_t)i].resize(n);
        S.v[(size_t)i].resize(n);
        BTRY(cudaMemcpy(S.x[(size_t)i].data(), m.d.x, sizeof(double) * n, cudaMemcpyDeviceToHost));
        BTRY(cudaMemcpy(S.v[(size_t)i].data(), m.d.v, sizeof(double) * n, cudaMemcpyDeviceToHost));
        S.steps[(size_t)i] = m.steps;
    }
    return SGB_OK;
}

int snapshot_restore(sgb_batch* B, const BatchSnapshot& S)
{
    BTRY(cudaStreamSynchronize(B->stream));
    BTRY(cudaMemcpy(B->d_meshes, S.desc.data(), sizeof(BMeshDesc) * B->max_slots, cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(B->d_err, &S.err, sizeof(int), cudaMemcpyHostToDevice));
    for (int i = 0; i < B->max_slots; ++i) {
        BatchMeshHost& m = B->slots[(size_t)i];
        if (!m.active) continue;
        const size_t n = 3 * (size_t)m.n_nodes;
        BTRY(cudaMemcpy(m.d.x, S.x[(size_t)i].data(), sizeof(double) * n, cudaMemcpyHostToDevice));
        BTRY(cudaMemcpy(m.d.v, S.v[(size_t)i].data(), sizeof(double) * n, cudaMemcpyHostToDevice));
        m.steps = S.steps[(size_t)i];
    }
    return SGB_OK;
}

int valid_tiles(const BatchTiles& t)
{
    const bool minb = t.matvec_minb == kBatchMatvecMinb[0] || t.matvec_minb == kBatchMatvecMinb[1] ||
                      t.matvec_minb == kBatchMatvecMinb[2];
    const bool npt = t.update_npt == 1 || t.update_npt == 2 || t.update_npt == 4;
    return minb && npt && t.update_ctas >= 1 && t.update_ctas <= 16 && t.elem_ctas >= 1 && t.elem_ctas <= 16 &&
           (t.prefetch == 0 || t.prefetch == 1);
}

}  // namespace

int sgb_batch_tune_patch_size(sgb_batch_t* B, const sgb_mesh_desc* sample, int n, int steps_per_trial,
                              int* chosen, double* ms_per_step)
{
    if (!B || !sample || n <= 0 || steps_per_trial < 1)
        return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_tune_patch_size: invalid argument");
    for (auto& m : B->slots)
        if (m.active)
            return bfail(SGB_ERR_NOT_SUPPORTED, "sgb_batch_tune_patch_size: the patch size is chosen before any "
                                                "mesh is admitted (it fixes each mesh's gather order)");
    // elements per patch: 256, 384, 512 (FP32); 128, 192, 256 (FP64)
    const int cand[3] = {B->rs == 4 ? 256 : 128, B->rs == 4 ? 384 : 192, B->rs == 4 ? 512 : 256};
    const int start = B->pe;
    cudaEvent_t e0, e1;
    BTRY(cudaEventCreate(&e0));
    BTRY(cudaEventCreate(&e1));
    std::vector<int> slots((size_t)n, -1);
    int best = start, rc = SGB_OK;
    double best_ms = 0.0;
    for (int c = 0; c < 3 && rc == SGB_OK; ++c) {
        B->pe = cand[c];
        B->sms = B->ops->batch_prepare(B->pe, B->grid_patch_v);
        B->graph_valid = false;
        if (B->sms <= 0) {
            rc = bfail(SGB_ERR_CUDA, "sgb_batch_tune_patch_size: kernel attributes");
            break;
        }
        rc = sgb_batch_add_meshes(B, sample, n, slots.data(), 8);
        if (rc == SGB_OK) rc = sgb_batch_step(B, 1);  // records the graph; warms up
        float f = 0.f;
        if (rc == SGB_OK) {
            cudaError_t ce;
            if ((ce = cudaEventRecord(e0, B->stream)) != cudaSuccess) rc = bcuda(ce, "cudaEventRecord");
            if (rc == SGB_OK) rc = sgb_batch_step(B, steps_per_trial);
            if (rc == SGB_OK && ((ce = cudaEventRecord(e1, B->stream)) != cudaSuccess ||
                                 (ce = cudaEventSynchronize(e1)) != cudaSuccess ||
                                 (ce = cudaEventElapsedTime(&f, e0, e1)) != cudaSuccess))
                rc = bcuda(ce, "timing");
        }
        for (int i = 0; i < n; ++i)
            if (slots[(size_t)i] >= 0) sgb_batch_remove_mesh(B, slots[(size_t)i]);
        const double ms = (double)f / steps_per_trial;
        if (ms_per_step) ms_per_step[c] = ms;
        if (rc == SGB_OK && (c == 0 || ms < best_ms)) {
            best = cand[c];
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->pe = rc == SGB_OK ? best : start;
    B->sms = B->ops->batch_prepare(B->pe, B->grid_patch_v);
    B->graph_valid = false;
    if (chosen) *chosen = B->pe;
    return rc;
}

int sgb_batch_set_tiles(sgb_batch_t* B, const int tiles[5])
{
    if (!B || !tiles) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_set_tiles: NULL argument");
    BatchTiles t;
    t.matvec_minb = tiles[0];
    t.update_npt = tiles[1];
    t.update_ctas = tiles[2];
    t.elem_ctas = tiles[3];
    t.prefetch = tiles[4];
    if (!valid_tiles(t))
        return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_set_tiles: matvec CTAs per SM must be 5, 6 or 8, update "
                                               "nodes per thread 1, 2 or 4, grids 1..16 CTAs per SM, prefetch 0 or 1");
    B->tiles = t;
    B->graph_valid = false;
    return SGB_OK;
}

int sgb_batch_get_tiles(const sgb_batch_t* B, int tiles[6], double* default_ms, double* best_ms, int* trials)
{
    if (!B || !tiles) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_get_tiles: NULL argument");
    tiles[0] = B->pe;
    tiles[1] = B->tiles.matvec_minb;
    tiles[2] = B->tiles.update_npt;
    tiles[3] = B->tiles.update_ctas;
    tiles[4] = B->tiles.elem_ctas;
    tiles[5] = B->tiles.prefetch;
    if (default_ms) *default_ms = B->tune_default_ms;
    if (best_ms) *best_ms = B->tune_best_ms;
    if (trials) *trials = B->tune_trials;
    return SGB_OK;
}

int sgb_batch_tune(sgb_batch_t* B, int steps_per_trial, int use_cache)
{
    if (!B || steps_per_trial < 1) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_tune: invalid argument");
    bool any = false;
    for (auto& m : B->slots) any = any || m.active;
    if (!any) return SGB_OK;  // nothing admitted: nothing to time
    const std::string key = mix_key(B);
    if (use_cache) {
        std::lock_guard<std::mutex> lk(g_tile_cache_mutex);
        auto it = g_tile_cache.find(key);
        if (it != g_tile_cache.end()) {
            B->tiles = it->second;
            B->graph_valid = false;
            B->tune_trials = 0;
            return SGB_OK;
        }
    }
    BatchSnapshot S;
    int rc = snapshot_take(B, S);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    BTRY(cudaEventCreate(&e0));
    BTRY(cudaEventCreate(&e1));
    int trials = 0;
    auto trial = [&](const BatchTiles& t, double* ms) -> int {
        B->tiles = t;
        B->graph_valid = false;
        int r = snapshot_restore(B, S);
        if (!r) r = sgb_batch_step(B, 1);  // records the graph of these tiles; warms up
        if (!r) r = snapshot_restore(B, S);
        if (r) return r;
        BTRY(cudaEventRecord(e0, B->stream));
        if ((r = sgb_batch_step(B, steps_per_trial))) return r;
        BTRY(cudaEventRecord(e1, B->stream));
        BTRY(cudaEventSynchronize(e1));
        float f = 0.f;
        BTRY(cudaEventElapsedTime(&f, e0, e1));
        *ms = (double)f / steps_per_trial;
        trials++;
        return SGB_OK;
    };
    const BatchTiles start = B->tiles;
    BatchTiles best = start;
    double best_ms = 0.0, default_ms = 0.0;
    rc = trial(best, &best_ms);
    default_ms = best_ms;
    // one coordinate at a time; a candidate must win by 1 % to be taken
    const int minbs[3] = {kBatchMatvecMinb[0], kBatchMatvecMinb[1], kBatchMatvecMinb[2]};
    const int npts[3] = {4, 2, 1};
    const int ctas[3] = {2, 4, 8};
    for (int knob = 0; knob < 5 && !rc; ++knob) {
        const int n = knob == 4 ? 2 : 3;
        for (int c = 0; c < n && !rc; ++c) {
            BatchTiles t = best;
            if (knob == 0) t.matvec_minb = minbs[c];
            if (knob == 1) t.update_npt = npts[c];
            if (knob == 2) t.update_ctas = ctas[c];
            if (knob == 3) t.elem_ctas = ctas[c];
            if (knob == 4) t.prefetch = c;
            if (std::memcmp(&t, &best, sizeof(t)) == 0) continue;
            double ms = 0.0;
            rc = trial(t, &ms);
            if (!rc && ms < 0.99 * best_ms) {
                best = t;
                best_ms = ms;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->tiles = rc ? start : best;
    B->graph_valid = false;
    const int rr = snapshot_restore(B, S);
    if (rc) return rc;
    if (rr) return rr;
    B->tune_default_ms = default_ms;
    B->tune_best_ms = best_ms;
    B->tune_trials = trials;
    {
        std::lock_guard<std::mutex> lk(g_tile_cache_mutex);
        g_tile_cache[key] = best;
    }
    return SGB_OK;
}

int sgb_batch_save_mesh(sgb_batch_t* B, int slot, double* x_host, double* v_host, long long* steps)
{
    if (!B || !x_host || !v_host || !steps || slot < 0 || slot >= B->max_slots || !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_save_mesh: no mesh in that slot, or a NULL output");
    int rc = sgb_batch_get_state(B, slot, x_host, v_host);
    if (rc) return rc;
    *steps = B->slots[(size_t)slot].steps;
    return SGB_OK;
}

int sgb_batch_restore_mesh(sgb_batch_t* B, int slot, const double* x_host, const double* v_host, long long steps)
{
    if (!B || !x_host || !v_host || steps < 0 || slot < 0 || slot >= B->max_slots ||
        !B->slots[(size_t)slot].active)
        return bfail(SGB_ERR_NOT_FOUND, "sgb_batch_restore_mesh: no mesh in that slot, or an invalid argument");
    int rc = sgb_batch_set_state(B, slot, x_host, v_host);
    if (rc) return rc;
    // the solver's time-step count (CGLinearSolver exempts the very first
    // iteration of the first time step from its tests)
    BTRY(cudaMemcpy((char*)&B->d_meshes[slot] + offsetof(BMeshDesc, tsc), &steps, sizeof(long long),
                    cudaMemcpyHostToDevice));
    B->slots[(size_t)slot].steps = steps;
    return SGB_OK;
}

int sgb_batch_info(const sgb_batch_t* B, int* active_meshes, long long* active_tets, size_t* budget_used,
                   size_t* budget_total)
{
    if (!B) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_info: NULL batch");
    int n = 0;
    long long t = 0;
    for (auto& m : B->slots)
        if (m.active) {
            n++;
            t += m.n_tets;
        }
    if (active_meshes) *active_meshes = n;
    if (active_tets) *active_tets = t;
    if (budget_used) *budget_used = B->arena.used;
    if (budget_total) *budget_total = B->arena.size;
    return SGB_OK;
}

void* sgb_batch_stream(sgb_batch_t* B) { return B ? (void*)B->stream : nullptr; }

}  // extern "C"
