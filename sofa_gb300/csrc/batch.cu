// Host side of the batched multi-mesh engine: a fixed HBM arena with a
// first-fit allocator (the admission budget), mesh admission and removal,
// the device work lists, and the CUDA graph of one batch step. The graph
// reads the work lists and mesh descriptors from device memory, so meshes can
// join and leave between steps without recording it again.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
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
    if (const char* e = getenv("SGB_BATCH_PREFETCH")) B->prefetch = (e[0] == '1');
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
    B->sms = ops->batch_prepare(B->pe, &B->grid_patch);
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
    return SGB_OK;
}

int sgb_batch_mesh_bytes(const sgb_batch_t* B, const sgb_mesh_desc* m, size_t* bytes)
{
    if (!bytes) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_mesh_bytes: NULL argument");
    // no batch: plan for a mixed-precision batch with the default patch size
    const int pe = B ? B->pe : 512;
    const size_t rs = B ? B->rs : sizeof(float);
    PreparedMesh pm;
    int rc = prepare_mesh(m, pe, rs, pm);
    if (rc) return rc;
    *bytes = pm.bytes;
    return SGB_OK;
}

int sgb_batch_add_mesh(sgb_batch_t* B, const sgb_mesh_desc* m, int* slot_out)
{
    if (!B || !slot_out) return bfail(SGB_ERR_INVALID_ARGUMENT, "sgb_batch_add_mesh: NULL argument");
    *slot_out = -1;
    PreparedMesh pm;
    int rc = prepare_mesh(m, B->pe, B->rs, pm);
    if (rc) return rc;
    return admit_prepared(B, pm, slot_out);
}

}  // extern "C"

namespace sgb {

// Host-only part of admission: validation, material checks like the
// reference (BaseLinearElasticityFEMForceField.inl:53-85), element order,
// patch layout, gather tables and the byte count. Safe on any thread.
int prepare_mesh(const sgb_mesh_desc* m, int pe, size_t rs, PreparedMesh& pm)
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
    build_patch_layout(N, E, m->tetrahedra_host, m->rest_positions_host, pe, kBatchMaxLocalNodes, pm.L);
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
    d.kf_rhs = h * 1.0 + P.rayleigh_stiffness;
    d.rm_factor = -P.rayleigh_mass;
    d.mf = 1 + 1.0 * h * P.rayleigh_mass;
    d.kf = -1.0 * h * (1.0 * h + P.rayleigh_stiffness);
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
                rcs[(size_t)i] = prepare_mesh(&meshes[i], B->pe, B->rs, pms[(size_t)i]);
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
        L.grid_patch = B->grid_patch;
        L.grid_elem = B->sms * 4;
        L.grid_node = B->sms * 4;
        L.n_slots = B->max_slots;
        L.grid_slots = std::min(B->max_slots, B->sms * 8);
        L.pe = B->pe;
        L.max_iterations = B->max_iterations;
        L.prefetch = B->prefetch;
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
