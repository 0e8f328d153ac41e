// C ABI of the GB300 tetrahedral-FEM library: handle management, input
// validation, the node->slot gather table, scene orchestration and CUDA
// graph capture. Kernels live in tfem_impl.cuh (one instance per precision).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <cstdlib>
#include <vector>

#include "../../include/sofa_gb300.h"
#include "mesh_layout.h"
#include "sgb_internal.h"
#include "variants.h"

using namespace sgb;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? SGB_ERR_OUT_OF_MEMORY : SGB_ERR_CUDA;
}

#define SGB_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, #expr);  \
    } while (0)

template <typename T>
int dev_alloc(T** p, size_t count, size_t* acc)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if (acc) *acc += sizeof(T) * count;
    return SGB_OK;
}

int dev_alloc_bytes(void** p, size_t bytes, size_t* acc)
{
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if (acc) *acc += bytes;
    return SGB_OK;
}

}  // namespace

struct sgb_tfem {
    TfemMesh m;
    const VariantOps* ops = nullptr;
    cudaStream_t stream = nullptr;
    std::string warnings;
};

struct sgb_scene {
    Scene s;
    sgb_tfem* fem = nullptr;
    sgb_tfem* shadow = nullptr;  // FP64 copy of the force field (residual replacement)
    const VariantOps* ops = nullptr;
    double* dot_terms = nullptr;
    int serial_dots = 0;
    int mass_first = 1;
};

namespace sgb {
void set_last_error(const std::string& msg) { g_last_error = msg; }

const VariantOps* variant_for(int precision)
{
    switch (precision) {
        case SGB_PRECISION_FP64: return &ops_fp64_exact;
        case SGB_PRECISION_MIXED: return &ops_mixed;
        case SGB_PRECISION_FP64_FMA: return &ops_fp64_fast;
        default: return nullptr;
    }
}
}  // namespace sgb

static void free_mesh(TfemMesh& m)
{
    cudaFree(m.plastic);
    cudaFree(m.plastic_scale);
    cudaFree(m.vm_lame);
    cudaFree(m.bsr_cptr);
    cudaFree(m.bsr_contrib);
    cudaFree(m.bsr_values);
    cudaFree(m.tets);
    cudaFree(m.rot);
    cudaFree(m.K);
    cudaFree(m.J);
    cudaFree(m.rest);
    cudaFree(m.rest_ff);
    cudaFree(m.R0);
    cudaFree(m.A0inv);
    cudaFree(m.rest_pos);
    cudaFree(m.rowptr);
    cudaFree(m.slots);
    cudaFree(m.eforce);
    cudaFree(m.elem_orig);
    cudaFree(m.pl.elem_start);
    cudaFree(m.pl.node_start);
    cudaFree(m.pl.lnode_gid);
    cudaFree(m.pl.lnode_info);
    cudaFree(m.pl.lrow);
    cudaFree(m.pl.lslots);
    cudaFree(m.pl.lconn);
    cudaFree(m.pl.bnd_rowptr);
    cudaFree(m.pl.partials);
    cudaFree(m.dev_flags);
    m = TfemMesh();
}

extern "C" {

const char* sgb_last_error(void) { return g_last_error.c_str(); }

const char* sgb_version(void) { return "sofa_gb300 0.1 (sm_103a)"; }

int sgb_tfem_create(sgb_tfem_t** out, int n_nodes, const double* rest_positions_host, int n_tets,
                    const int32_t* tetrahedra_host, const double* young, int n_young, const double* poisson,
                    int n_poisson, const double* local_stiffness_factor, int n_lsf, int method, int precision)
{
    if (!out) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: out is NULL");
    *out = nullptr;
    if (n_nodes <= 0 || !rest_positions_host)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: the mesh needs at least one node");
    if (n_tets < 0 || (n_tets > 0 && !tetrahedra_host))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: invalid tetrahedra");
    if (method < SGB_METHOD_SMALL || method > SGB_METHOD_SVD)
        return fail(SGB_ERR_NOT_SUPPORTED, "sgb_tfem_create: method must be small, large, polar or svd");
    const VariantOps* ops = variant_for(precision);
    if (!ops) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: unknown precision");
    if ((size_t)n_tets * 12 > (size_t)0x7fffffff)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: too many tetrahedra for one mesh");
    for (size_t i = 0; i < (size_t)n_tets * 4; ++i)
        if (tetrahedra_host[i] < 0 || tetrahedra_host[i] >= n_nodes)
            return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: tetrahedron node index out of range");
    for (size_t i = 0; i < (size_t)n_nodes * 3; ++i)
        if (!std::isfinite(rest_positions_host[i]))
            return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: non-finite rest position");
    if (n_lsf < 0 || (n_lsf > 0 && !local_stiffness_factor))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_create: invalid localStiffnessFactor");

    std::string warn;
    // BaseLinearElasticityFEMForceField::checkYoungModulus / checkPoissonRatio
    std::vector<double> E_h, nu_h;
    if (young && n_young > 0) E_h.assign(young, young + n_young);
    if (poisson && n_poisson > 0) nu_h.assign(poisson, poisson + n_poisson);
    if (E_h.empty()) {
        E_h.push_back(5000.0);
        warn += "youngModulus empty, using 5000; ";
    }
    if (nu_h.empty()) {
        nu_h.push_back(0.45);
        warn += "poissonRatio empty, using 0.45; ";
    }
    for (double& y : E_h)
        if (!(y >= 0)) {
            warn += "negative youngModulus replaced by 5000; ";
            y = 5000.0;
        }
    for (double& p : nu_h)
        if (!(p >= 0 && p < 0.5)) {
            warn += "poissonRatio outside [0,0.5) replaced by 0.45; ";
            p = 0.45;
        }

    sgb_tfem* h = new sgb_tfem();
    TfemMesh& m = h->m;
    h->ops = ops;
    m.n_nodes = n_nodes;
    m.n_tets = n_tets;
    m.method = method;
    m.precision = precision;
    m.real_size = ops->real_size;
    m.young_h = E_h;
    if (n_lsf > 0) m.lsf_h.assign(local_stiffness_factor, local_stiffness_factor + n_lsf);
    m.poisson_h = nu_h;
    int rc = SGB_OK;
    // element storage order and patch layout (Morton-ordered patches) for
    // the fused variants; the reference-rounding variant keeps the caller's
    // element order
    HostLayout L;
    // elements per patch: 320 for FP32 (the fastest implicit step on a
    // GB300 among 256..512: 10.42 ms per step of the 64x64x257 beam against
    // 10.75 at 256, where fewer shared nodes make the CG update cheaper; a
    // lone addDForce call is 2 % faster at 256) and 256 for FP64;
    // SGB_PATCH_PE overrides the FP32 value (an even count in [32, 1024])
    int pe = ops->real_size == 4 ? 320 : 256;
    if (ops->real_size == 4)
        if (const char* e = getenv("SGB_PATCH_PE")) {
            const int v = atoi(e);
            if (v >= 32 && v <= 1024 && v % 2 == 0) pe = v;
        }
    if (ops->uses_patches && method != SGB_METHOD_SMALL && n_tets > 0) {
        build_patch_layout(n_nodes, n_tets, tetrahedra_host, rest_positions_host, pe, 1024, L);
    } else {
        L.perm.resize((size_t)n_tets);
        L.inv.resize((size_t)n_tets);
        for (int e = 0; e < n_tets; ++e) L.perm[(size_t)e] = L.inv[(size_t)e] = e;
    }
    std::vector<int> rowptr, slots;
    build_node_csr(n_nodes, n_tets, tetrahedra_host, L.inv, rowptr, slots, m.max_valence);
    std::vector<int32_t> tets_store((size_t)n_tets * 4);
    for (size_t s = 0; s < (size_t)n_tets; ++s)
        for (int c = 0; c < 4; ++c) tets_store[4 * s + c] = tetrahedra_host[4 * (size_t)L.perm[s] + c];
    m.perm_h = L.perm;
    const size_t rs = ops->real_size, E = (size_t)n_tets;
    size_t* acc = &m.device_bytes;
    double *d_y = nullptr, *d_p = nullptr, *d_l = nullptr, *d_vol = nullptr;
    cudaError_t ce;
    ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        rc = cuda_fail(ce, "cudaStreamCreate");
        goto fail_out;
    }
    if ((rc = dev_alloc(&m.tets, E, acc)) || (rc = dev_alloc_bytes(&m.rot, rs * 9 * E, acc)) ||
        (rc = dev_alloc_bytes(&m.R0, rs * 9 * E, acc)) || (rc = dev_alloc_bytes(&m.K, rs * 3 * E, acc)) ||
        (rc = dev_alloc_bytes(&m.J, rs * 12 * E, acc)) || (rc = dev_alloc_bytes(&m.rest, rs * 12 * E, acc)) ||
        (rc = dev_alloc_bytes(&m.eforce, rs * 12 * E, acc)) || (rc = dev_alloc(&m.rest_pos, 3 * (size_t)n_nodes, acc)) ||
        (rc = dev_alloc(&m.rowptr, (size_t)n_nodes + 1, acc)) || (rc = dev_alloc(&m.slots, 4 * E, acc)) ||
        (rc = dev_alloc(&m.elem_orig, E, acc)) || (rc = dev_alloc(&m.dev_flags, 1, acc)) ||
        (precision == SGB_PRECISION_MIXED && method != SGB_METHOD_SMALL && (rc = dev_alloc(&m.rest_ff, 9 * E, acc))) ||
        (method == SGB_METHOD_SVD && (rc = dev_alloc_bytes(&m.A0inv, rs * 9 * E, acc))))
        goto fail_out;
    if ((ce = cudaMemsetAsync(m.dev_flags, 0, sizeof(int), h->stream)) != cudaSuccess) {
        rc = cuda_fail(ce, "cudaMemsetAsync");
        goto fail_out;
    }
    if (!L.elem_start.empty()) {
        PatchLayout& pl = m.pl;
        pl.n_patches = (int)L.elem_start.size() - 1;
        pl.pe = pe;
        pl.max_lnodes = L.max_lnodes;
        pl.n_partials = L.n_partials;
        pl.n_lnodes = (int)L.lnode_gid.size();
        pl.n_boundary = L.n_boundary;
        if ((rc = dev_alloc(&pl.elem_start, L.elem_start.size(), acc)) ||
            (rc = dev_alloc(&pl.node_start, L.node_start.size(), acc)) ||
            (rc = dev_alloc(&pl.lnode_gid, L.lnode_gid.size(), acc)) ||
            (rc = dev_alloc(&pl.lnode_info, L.lnode_info.size(), acc)) ||
            (rc = dev_alloc(&pl.lrow, L.lrow.size(), acc)) || (rc = dev_alloc(&pl.lslots, L.lslots.size() + 8, acc)) ||
            (rc = dev_alloc(&pl.lconn, L.lconn.size() + 2, acc)) ||
            (rc = dev_alloc(&pl.bnd_rowptr, L.bnd_rowptr.size(), acc)) ||
            (rc = dev_alloc_bytes(&pl.partials, rs * 3 * (size_t)std::max(L.n_partials, 1), acc)))
            goto fail_out;
        struct {
            void* dst;
            const void* src;
            size_t bytes;
        } up[] = {
            {pl.elem_start, L.elem_start.data(), sizeof(int) * L.elem_start.size()},
            {pl.node_start, L.node_start.data(), sizeof(int) * L.node_start.size()},
            {pl.lnode_gid, L.lnode_gid.data(), sizeof(int) * L.lnode_gid.size()},
            {pl.lnode_info, L.lnode_info.data(), sizeof(int) * L.lnode_info.size()},
            {pl.lrow, L.lrow.data(), sizeof(int) * L.lrow.size()},
            {pl.lslots, L.lslots.data(), sizeof(uint16_t) * L.lslots.size()},
            {pl.lconn, L.lconn.data(), sizeof(ushort4) * L.lconn.size()},
            {pl.bnd_rowptr, L.bnd_rowptr.data(), sizeof(int) * L.bnd_rowptr.size()},
        };
        for (auto& u : up) {
            if (u.bytes == 0) continue;
            if ((ce = cudaMemcpyAsync(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess) {
                rc = cuda_fail(ce, "cudaMemcpyAsync");
                goto fail_out;
            }
        }
        m.patch_grid = ops->prepare(&m);
        if ((ce = cudaGetLastError()) != cudaSuccess) {
            rc = cuda_fail(ce, "patch kernel attributes");
            goto fail_out;
        }
    }
    if ((rc = dev_alloc(&d_y, E_h.size(), nullptr)) || (rc = dev_alloc(&d_p, nu_h.size(), nullptr)) ||
        (rc = dev_alloc(&d_l, (size_t)std::max(n_lsf, 1), nullptr)) || (rc = dev_alloc(&d_vol, E, nullptr)))
        goto fail_out;
    if ((ce = cudaMemcpyAsync(m.tets, tets_store.data(), sizeof(int4) * E, cudaMemcpyHostToDevice, h->stream)) ||
        (ce = cudaMemcpyAsync(m.elem_orig, L.perm.data(), sizeof(int) * E, cudaMemcpyHostToDevice, h->stream)) ||
        (ce = cudaMemcpyAsync(m.rest_pos, rest_positions_host, sizeof(double) * 3 * n_nodes, cudaMemcpyHostToDevice,
                              h->stream)) ||
        (ce = cudaMemcpyAsync(m.rowptr, rowptr.data(), sizeof(int) * rowptr.size(), cudaMemcpyHostToDevice,
                              h->stream)) ||
        (!slots.empty() && (ce = cudaMemcpyAsync(m.slots, slots.data(), sizeof(int) * slots.size(),
                                                 cudaMemcpyHostToDevice, h->stream))) ||
        (ce = cudaMemcpyAsync(d_y, E_h.data(), sizeof(double) * E_h.size(), cudaMemcpyHostToDevice, h->stream)) ||
        (ce = cudaMemcpyAsync(d_p, nu_h.data(), sizeof(double) * nu_h.size(), cudaMemcpyHostToDevice, h->stream))) {
        rc = cuda_fail(ce, "cudaMemcpyAsync");
        goto fail_out;
    }
    if (n_lsf > 0 && (ce = cudaMemcpyAsync(d_l, local_stiffness_factor, sizeof(double) * n_lsf,
                                           cudaMemcpyHostToDevice, h->stream))) {
        rc = cuda_fail(ce, "cudaMemcpyAsync");
        goto fail_out;
    }
    ops->init(&m, d_y, (int)E_h.size(), d_p, (int)nu_h.size(), d_l, n_lsf, d_vol, h->stream);
    if ((ce = cudaGetLastError()) != cudaSuccess) {
        rc = cuda_fail(ce, "init kernel launch");
        goto fail_out;
    }
    {
        std::vector<double> vol(E);
        if (E) {
            ce = cudaMemcpyAsync(vol.data(), d_vol, sizeof(double) * E, cudaMemcpyDeviceToHost, h->stream);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
            if (ce != cudaSuccess) {
                rc = cuda_fail(ce, "init");
                goto fail_out;
            }
        }
        size_t degenerate = 0;
        double total = 0.0;
        for (double v : vol) {
            total += v;
            if (!(v > 0)) degenerate++;
        }
        m.rest_volume = total;
        if (degenerate) warn += std::to_string(degenerate) + " degenerate (zero-volume) tetrahedra; ";
    }
    cudaFree(d_y);
    cudaFree(d_p);
    cudaFree(d_l);
    cudaFree(d_vol);
    h->warnings = warn;
    g_last_error = warn;
    *out = h;
    return SGB_OK;
fail_out:
    cudaFree(d_y);
    cudaFree(d_p);
    cudaFree(d_l);
    cudaFree(d_vol);
    free_mesh(m);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return rc;
}

int sgb_tfem_destroy(sgb_tfem_t* fem)
{
    if (!fem) return SGB_OK;
    cudaStreamSynchronize(fem->stream);
    free_mesh(fem->m);
    cudaStreamDestroy(fem->stream);
    delete fem;
    return SGB_OK;
}

static cudaStream_t pick(sgb_tfem_t* fem, void* stream)
{
    return stream ? (cudaStream_t)stream : fem->stream;
}

int sgb_tfem_add_force(sgb_tfem_t* fem, const double* x_dev, double* f_dev, void* stream)
{
    if (!fem || !x_dev || !f_dev) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_force: NULL argument");
    if (fem->m.real_size != sizeof(double))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_force: MIXED handle, use sgb_tfem_add_force_f32");
    fem->ops->add_force(&fem->m, x_dev, f_dev, pick(fem, stream));
    SGB_CUDA_TRY(cudaGetLastError());
    return SGB_OK;
}

int sgb_tfem_add_force_f32(sgb_tfem_t* fem, const double* x_dev, float* f_dev, void* stream)
{
    if (!fem || !x_dev || !f_dev) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_force_f32: NULL argument");
    if (fem->m.real_size != sizeof(float))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_force_f32: FP64 handle, use sgb_tfem_add_force");
    fem->ops->add_force(&fem->m, x_dev, f_dev, pick(fem, stream));
    SGB_CUDA_TRY(cudaGetLastError());
    return SGB_OK;
}

int sgb_tfem_add_dforce(sgb_tfem_t* fem, const double* dx_dev, double* df_dev, double kfactor, void* stream)
{
    if (!fem || !dx_dev || !df_dev) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_dforce: NULL argument");
    if (fem->m.real_size != sizeof(double))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_dforce: MIXED handle, use sgb_tfem_add_dforce_f32");
    fem->ops->add_dforce(&fem->m, dx_dev, df_dev, kfactor, pick(fem, stream));
    SGB_CUDA_TRY(cudaGetLastError());
    return SGB_OK;
}

int sgb_tfem_add_dforce_f32(sgb_tfem_t* fem, const float* dx_dev, float* df_dev, float kfactor, void* stream)
{
    if (!fem || !dx_dev || !df_dev) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_dforce_f32: NULL argument");
    if (fem->m.real_size != sizeof(float))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_add_dforce_f32: FP64 handle, use sgb_tfem_add_dforce");
    fem->ops->add_dforce(&fem->m, dx_dev, df_dev, (double)kfactor, pick(fem, stream));
    SGB_CUDA_TRY(cudaGetLastError());
    return SGB_OK;
}

int sgb_tfem_stiffness_bsr(sgb_tfem_t* fem, int* n_blocks, int32_t* rowptr_host, int32_t* cols_host,
                           double* values_host)
{
    if (!fem || !n_blocks) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_stiffness_bsr: NULL argument");
    TfemMesh& m = fem->m;
    const int N = m.n_nodes, E = m.n_tets;
    if ((size_t)E * 16 >= ((size_t)1 << 31) || (size_t)E >= ((size_t)1 << 27))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_stiffness_bsr: too many tetrahedra");
    if (m.bsr_rowptr_h.empty()) {
        // pattern: per node row, the nodes sharing an element with it
        // (itself included), ascending; per block, its contributions in the
        // caller's element order
        std::vector<int32_t> st((size_t)E * 4);
        if (E > 0) SGB_CUDA_TRY(cudaMemcpy(st.data(), m.tets, sizeof(int32_t) * st.size(), cudaMemcpyDeviceToHost));
        std::vector<int> inv((size_t)E);
        for (int s = 0; s < E; ++s) inv[(size_t)m.perm_h[(size_t)s]] = s;
        std::vector<std::vector<int>> adj((size_t)N);
        for (int s = 0; s < E; ++s)
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) adj[(size_t)st[4 * (size_t)s + a]].push_back(st[4 * (size_t)s + b]);
        std::vector<int> rowptr((size_t)N + 1, 0), cols;
        for (int n = 0; n < N; ++n) {
            auto& v = adj[(size_t)n];
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            rowptr[(size_t)n + 1] = rowptr[(size_t)n] + (int)v.size();
            cols.insert(cols.end(), v.begin(), v.end());
            std::vector<int>().swap(v);
        }
        const int nb = rowptr[(size_t)N];
        auto block_of = [&](int r, int c) {
            auto b0 = cols.begin() + rowptr[(size_t)r], b1 = cols.begin() + rowptr[(size_t)r + 1];
            return (int)(std::lower_bound(b0, b1, c) - cols.begin());
        };
        std::vector<int> cptr((size_t)nb + 1, 0), contrib((size_t)E * 16);
        for (int s = 0; s < E; ++s)
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) cptr[(size_t)block_of(st[4 * (size_t)s + a], st[4 * (size_t)s + b]) + 1]++;
        for (int k = 0; k < nb; ++k) cptr[(size_t)k + 1] += cptr[(size_t)k];
        std::vector<int> fill(cptr.begin(), cptr.end() - 1);
        for (int e = 0; e < E; ++e) {  // caller order
            const int s = inv[(size_t)e];
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) {
                    const int k = block_of(st[4 * (size_t)s + a], st[4 * (size_t)s + b]);
                    contrib[(size_t)fill[(size_t)k]++] = (s << 4) | (a << 2) | b;
                }
        }
        size_t acc = 0;
        int rc;
        if ((rc = dev_alloc(&m.bsr_cptr, (size_t)nb + 1, &acc)) ||
            (rc = dev_alloc(&m.bsr_contrib, std::max<size_t>(contrib.size(), 1), &acc)) ||
            (rc = dev_alloc(&m.bsr_values, std::max<size_t>((size_t)nb * 9, 1), &acc))) {
            cudaFree(m.bsr_cptr);
            cudaFree(m.bsr_contrib);
            cudaFree(m.bsr_values);
            m.bsr_cptr = m.bsr_contrib = nullptr;
            m.bsr_values = nullptr;
            return rc;
        }
        SGB_CUDA_TRY(cudaMemcpy(m.bsr_cptr, cptr.data(), sizeof(int) * cptr.size(), cudaMemcpyHostToDevice));
        if (!contrib.empty())
            SGB_CUDA_TRY(
                cudaMemcpy(m.bsr_contrib, contrib.data(), sizeof(int) * contrib.size(), cudaMemcpyHostToDevice));
        m.bsr_rowptr_h.assign(rowptr.begin(), rowptr.end());
        m.bsr_cols_h.swap(cols);
    }
    const int nb = (int)m.bsr_cols_h.size();
    *n_blocks = nb;
    if (rowptr_host) std::memcpy(rowptr_host, m.bsr_rowptr_h.data(), sizeof(int32_t) * ((size_t)N + 1));
    if (cols_host && nb) std::memcpy(cols_host, m.bsr_cols_h.data(), sizeof(int32_t) * (size_t)nb);
    if (values_host && nb) {
        fem->ops->stiffness_blocks(&m, m.bsr_cptr, m.bsr_contrib, nb, m.bsr_values, fem->stream);
        SGB_CUDA_TRY(cudaGetLastError());
        SGB_CUDA_TRY(cudaMemcpyAsync(values_host, m.bsr_values, sizeof(double) * 9 * (size_t)nb,
                                     cudaMemcpyDeviceToHost, fem->stream));
        SGB_CUDA_TRY(cudaStreamSynchronize(fem->stream));
    }
    return SGB_OK;
}

int sgb_tfem_get_rotations(sgb_tfem_t* fem, double* rotations_host, double* initial_rotations_host)
{
    if (!fem) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_get_rotations: NULL handle");
    const size_t E = (size_t)fem->m.n_tets, rs = fem->m.real_size;
    std::vector<unsigned char> buf(rs * 9 * std::max<size_t>(E, 1));
    void* src[2] = {fem->m.rot, fem->m.R0};
    double* dst[2] = {rotations_host, initial_rotations_host};
    SGB_CUDA_TRY(cudaStreamSynchronize(fem->stream));
    for (int w = 0; w < 2; ++w) {
        if (!dst[w] || E == 0) continue;
        if (w == 0 && rs == sizeof(float)) {
            // FP32 keeps the current rotation as a unit quaternion (x, y, z, w;
            // w <= -2 flags a reflection)
            std::vector<float> q(4 * E);
            SGB_CUDA_TRY(cudaMemcpy(q.data(), src[w], sizeof(float) * 4 * E, cudaMemcpyDeviceToHost));
            for (size_t e = 0; e < E; ++e) {
                double x = q[4 * e], y = q[4 * e + 1], z = q[4 * e + 2], ww = q[4 * e + 3], sg = 1.0;
                if (ww <= -1.5) {
                    sg = -1.0;
                    ww = -ww - 2.0;
                }
                const double Rm[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - ww * z), 2 * (x * z + ww * y),
                                      2 * (x * y + ww * z), 1 - 2 * (x * x + z * z), 2 * (y * z - ww * x),
                                      2 * (x * z - ww * y), 2 * (y * z + ww * x), 1 - 2 * (x * x + y * y)};
                const size_t o = (size_t)fem->m.perm_h[e];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) dst[w][9 * o + 3 * i + j] = sg * Rm[3 * j + i];
            }
            continue;
        }
        SGB_CUDA_TRY(cudaMemcpy(buf.data(), src[w], rs * 9 * E, cudaMemcpyDeviceToHost));
        for (size_t e = 0; e < E; ++e) {
            const size_t o = (size_t)fem->m.perm_h[e];  // caller's element index
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    // stored: rows of R, SoA; reference convention: R^T row-major
                    size_t k = (size_t)(3 * j + i) * E + e;
                    double v = (rs == 8) ? ((double*)buf.data())[k] : (double)((float*)buf.data())[k];
                    dst[w][9 * o + 3 * i + j] = v;
                }
        }
    }
    return SGB_OK;
}

// Temporary device copies of the material vectors as given at creation
// (Young's moduli, Poisson ratios, localStiffnessFactor), for kernels that
// recompute per-element material values after initialisation. The caller
// frees all three, also on failure.
static cudaError_t upload_materials(const TfemMesh& m, double** d_y, double** d_p, double** d_l)
{
    cudaError_t ce = cudaMalloc(d_y, sizeof(double) * m.young_h.size());
    if (ce == cudaSuccess) ce = cudaMalloc(d_p, sizeof(double) * m.poisson_h.size());
    if (ce == cudaSuccess) ce = cudaMalloc(d_l, sizeof(double) * std::max<size_t>(m.lsf_h.size(), 1));
    if (ce == cudaSuccess)
        ce = cudaMemcpy(*d_y, m.young_h.data(), sizeof(double) * m.young_h.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
        ce = cudaMemcpy(*d_p, m.poisson_h.data(), sizeof(double) * m.poisson_h.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && !m.lsf_h.empty())
        ce = cudaMemcpy(*d_l, m.lsf_h.data(), sizeof(double) * m.lsf_h.size(), cudaMemcpyHostToDevice);
    return ce;
}

// Mixed precision: the per-element sqrt(K(0,0)) the packed J carries,
// computed once (plasticity and updateStiffnessMatrix share it).
static int ensure_k_scale(sgb_tfem_t* fem)
{
    TfemMesh& m = fem->m;
    const size_t E = (size_t)m.n_tets;
    if (m.real_size != sizeof(float) || m.plastic_scale || E == 0) return SGB_OK;
    SGB_CUDA_TRY(cudaStreamSynchronize(fem->stream));
    SGB_CUDA_TRY(cudaMalloc(&m.plastic_scale, sizeof(float) * E));
    m.device_bytes += sizeof(float) * E;
    double *d_y = nullptr, *d_p = nullptr, *d_l = nullptr;
    cudaError_t ce = upload_materials(m, &d_y, &d_p, &d_l);
    if (ce == cudaSuccess) {
        fem->ops->plastic_scale(&m, d_y, (int)m.young_h.size(), d_p, (int)m.poisson_h.size(), d_l,
                                (int)m.lsf_h.size(), fem->stream);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(fem->stream);
    cudaFree(d_y);
    cudaFree(d_p);
    cudaFree(d_l);
    if (ce != cudaSuccess) return cuda_fail(ce, "per-element strain scale");
    return SGB_OK;
}

int sgb_tfem_set_update_stiffness(sgb_tfem_t* fem, int on)
{
    if (!fem) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_set_update_stiffness: NULL handle");
    TfemMesh& m = fem->m;
    if (on && m.method == METHOD_LARGE)
        return fail(SGB_ERR_NOT_SUPPORTED,
                    "sgb_tfem_set_update_stiffness: method large (the reference rebuilds only some of the "
                    "strain-displacement entries it builds equal)");
    if (on && m.method != METHOD_SMALL) {
        int rc = ensure_k_scale(fem);
        if (rc) return rc;
    }
    const int v = (on && m.method != METHOD_SMALL) ? 1 : 0;
    if (v != m.update_j) {
        m.update_j = v;
        m.plastic_version++;  // captured steps re-record with the new force kernel arguments
    }
    return SGB_OK;
}

int sgb_tfem_set_plasticity(sgb_tfem_t* fem, double max_threshold, double yield_threshold, double creep)
{
    if (!fem) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_set_plasticity: NULL handle");
    if (!(max_threshold >= 0.0) || !(yield_threshold >= 0.0) || !std::isfinite(max_threshold) ||
        !std::isfinite(yield_threshold) || !std::isfinite(creep))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_set_plasticity: thresholds must be finite and >= 0");
    TfemMesh& m = fem->m;
    const size_t E = (size_t)m.n_tets;
    if (max_threshold > 0.0 && !m.plastic && E > 0) {
        // first enabled: zero plastic strain; mixed also computes its
        // per-element strain scale
        SGB_CUDA_TRY(cudaStreamSynchronize(fem->stream));
        SGB_CUDA_TRY(cudaMalloc(&m.plastic, m.real_size * 6 * E));
        m.device_bytes += m.real_size * 6 * E;
        SGB_CUDA_TRY(cudaMemsetAsync(m.plastic, 0, m.real_size * 6 * E, fem->stream));
        int rc = ensure_k_scale(fem);
        if (rc) return rc;
    }
    m.plastic_max = max_threshold;
    m.plastic_yield = yield_threshold;
    m.plastic_creep = creep;
    m.plastic_version++;
    return SGB_OK;
}

int sgb_tfem_von_mises(sgb_tfem_t* fem, int mode, const double* x_dev, double* per_element_dev,
                       double* per_node_dev, void* stream)
{
    if (!fem || !x_dev || !per_element_dev)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_von_mises: NULL argument");
    if (mode != 1 && mode != 2)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_von_mises: mode must be 1 (corotational) or 2 (Green)");
    TfemMesh& m = fem->m;
    if (mode == 1 && m.method == METHOD_SMALL)
        return fail(SGB_ERR_NOT_SUPPORTED,
                    "sgb_tfem_von_mises: method small computes von Mises stress with the Green strain only (mode 2)");
    const size_t E = (size_t)m.n_tets;
    if (!m.vm_lame && E > 0) {
        SGB_CUDA_TRY(cudaStreamSynchronize(fem->stream));
        SGB_CUDA_TRY(cudaMalloc(&m.vm_lame, sizeof(double) * 2 * E));
        m.device_bytes += sizeof(double) * 2 * E;
        double *d_y = nullptr, *d_p = nullptr, *d_l = nullptr;
        cudaError_t ce = upload_materials(m, &d_y, &d_p, &d_l);
        if (ce == cudaSuccess) {
            launch_lame(&m, d_y, (int)m.young_h.size(), d_p, (int)m.poisson_h.size(), d_l, (int)m.lsf_h.size(),
                        m.vm_lame, fem->stream);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(fem->stream);
        cudaFree(d_y);
        cudaFree(d_p);
        cudaFree(d_l);
        if (ce != cudaSuccess) {
            cudaFree(m.vm_lame);
            m.vm_lame = nullptr;
            return cuda_fail(ce, "sgb_tfem_von_mises");
        }
    }
    launch_von_mises(&m, mode, x_dev, m.vm_lame, per_element_dev, per_node_dev, pick(fem, stream));
    SGB_CUDA_TRY(cudaGetLastError());
    return SGB_OK;
}

int sgb_tfem_reset_plasticity(sgb_tfem_t* fem)
{
    if (!fem) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_reset_plasticity: NULL handle");
    if (fem->m.plastic)
        SGB_CUDA_TRY(cudaMemsetAsync(fem->m.plastic, 0, fem->m.real_size * 6 * (size_t)fem->m.n_tets, fem->stream));
    return SGB_OK;
}

int sgb_tfem_get_plastic_strain(sgb_tfem_t* fem, double* plastic_strain_host)
{
    if (!fem || !plastic_strain_host)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_get_plastic_strain: NULL argument");
    TfemMesh& m = fem->m;
    const size_t E = (size_t)m.n_tets, rs = m.real_size;
    if (!m.plastic) {
        std::fill(plastic_strain_host, plastic_strain_host + 6 * E, 0.0);
        return SGB_OK;
    }
    std::vector<unsigned char> buf(rs * 6 * std::max<size_t>(E, 1));
    std::vector<float> scale;
    SGB_CUDA_TRY(cudaStreamSynchronize(fem->stream));
    SGB_CUDA_TRY(cudaMemcpy(buf.data(), m.plastic, rs * 6 * E, cudaMemcpyDeviceToHost));
    if (m.plastic_scale) {
        scale.resize(E);
        SGB_CUDA_TRY(cudaMemcpy(scale.data(), m.plastic_scale, sizeof(float) * E, cudaMemcpyDeviceToHost));
    }
    for (size_t e = 0; e < E; ++e) {
        const size_t o = (size_t)m.perm_h[e];
        for (int i = 0; i < 6; ++i) {
            const size_t k = (size_t)i * E + e;
            double v = (rs == 8) ? ((double*)buf.data())[k] : (double)((float*)buf.data())[k];
            if (!scale.empty()) v /= (double)scale[e];  // mixed keeps it in J's scaling
            plastic_strain_host[6 * o + i] = v;
        }
    }
    return SGB_OK;
}

int sgb_tfem_check_device(sgb_tfem_t* fem)
{
    if (!fem) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_check_device: NULL handle");
    int flag = 0;
    const int zero = 0;
    SGB_CUDA_TRY(cudaDeviceSynchronize());
    SGB_CUDA_TRY(cudaMemcpy(&flag, fem->m.dev_flags, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        SGB_CUDA_TRY(cudaMemcpy(fem->m.dev_flags, &zero, sizeof(int), cudaMemcpyHostToDevice));
        return fail(SGB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait ran out in an earlier add_dforce");
    }
    return SGB_OK;
}

int sgb_tfem_info(const sgb_tfem_t* fem, int* n_nodes, int* n_tets, int* method, int* precision, size_t* device_bytes)
{
    if (!fem) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_tfem_info: NULL handle");
    if (n_nodes) *n_nodes = fem->m.n_nodes;
    if (n_tets) *n_tets = fem->m.n_tets;
    if (method) *method = fem->m.method;
    if (precision) *precision = fem->m.precision;
    if (device_bytes) *device_bytes = fem->m.device_bytes;
    return SGB_OK;
}

// ---------------------------------------------------------------------------
// scene
// ---------------------------------------------------------------------------

int sgb_patch_layout_check(int n_nodes, const double* rest_positions_host, int n_tets, const int32_t* tetrahedra_host,
                           int elements_per_patch, int max_nodes_per_patch, int* stats)
{
    if (n_nodes <= 0 || n_tets < 0 || !rest_positions_host || (n_tets > 0 && !tetrahedra_host) ||
        elements_per_patch < 2 || elements_per_patch > 16384 || max_nodes_per_patch < 8 ||
        max_nodes_per_patch > 65535)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_patch_layout_check: invalid argument");
    for (size_t i = 0; i < (size_t)n_tets * 4; ++i)
        if (tetrahedra_host[i] < 0 || tetrahedra_host[i] >= n_nodes)
            return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_patch_layout_check: node index out of range");
    HostLayout L;
    build_patch_layout(n_nodes, n_tets, tetrahedra_host, rest_positions_host, elements_per_patch,
                       max_nodes_per_patch, L);
    const int P = (int)L.elem_start.size() - 1;
    // patches with elements first, then the patches of nodes of no element
    int P_elem = 0;
    while (P_elem < P && L.elem_start[P_elem + 1] > L.elem_start[P_elem]) ++P_elem;
    // every (element, corner) is gathered exactly once, by the patch that
    // holds the element, at the local node that is that corner's node
    std::vector<int> seen((size_t)n_tets * 4, 0);
    std::vector<int> owners((size_t)n_nodes, 0), touched((size_t)n_nodes, 0);
    for (int p = 0; p < P; ++p) {
        const int e0 = L.elem_start[p], e1 = L.elem_start[p + 1];
        if (e1 - e0 > elements_per_patch || (p < P_elem ? e1 <= e0 : (e0 != n_tets || e1 != n_tets)))
            return fail(SGB_ERR_NUMERICAL, "patch element range");
        if (p + 1 < P_elem && ((e1 - e0) & 1))
            return fail(SGB_ERR_NUMERICAL, "odd element count before the last patch");
        const int n0 = L.node_start[p], n1 = L.node_start[p + 1];
        if (n1 - n0 > max_nodes_per_patch || (p >= P_elem && (n1 <= n0 || n1 - n0 > L.max_lnodes)))
            return fail(SGB_ERR_NUMERICAL, "patch node count");
        for (int l = n0; l < n1; ++l) {
            const int g = L.lnode_gid[(size_t)l];
            if (l > n0 && g <= L.lnode_gid[(size_t)l - 1]) return fail(SGB_ERR_NUMERICAL, "local nodes not sorted");
            touched[(size_t)g]++;
            const int info = L.lnode_info[(size_t)l];
            if (info < 0 || (info & 1)) owners[(size_t)g]++;
            if (info >= 0) {
                const int slot = info >> 1;
                if (slot < L.bnd_rowptr[(size_t)g] || slot >= L.bnd_rowptr[(size_t)g + 1])
                    return fail(SGB_ERR_NUMERICAL, "partial slot outside the node's range");
            }
            int prev = -1;
            for (int s = L.lrow[(size_t)l]; s < L.lrow[(size_t)l + 1]; ++s) {
                const int slot = L.lslots[(size_t)s];
                const int le = slot >> 2, c = slot & 3;
                if (le >= e1 - e0 || slot <= prev) return fail(SGB_ERR_NUMERICAL, "local slot order");
                prev = slot;
                const int st = e0 + le;
                const int orig = L.perm[(size_t)st];
                if (tetrahedra_host[4 * (size_t)orig + c] != g) return fail(SGB_ERR_NUMERICAL, "slot node mismatch");
                const ushort4 lc = L.lconn[(size_t)st];
                const int ln[4] = {lc.x, lc.y, lc.z, lc.w};
                if (n0 + ln[c] != l) return fail(SGB_ERR_NUMERICAL, "local connectivity mismatch");
                seen[4 * (size_t)orig + c]++;
            }
        }
    }
    int boundary = 0;
    for (int n = 0; n < n_nodes; ++n) {
        const int cnt = L.bnd_rowptr[(size_t)n + 1] - L.bnd_rowptr[(size_t)n];
        if ((P > 0 && touched[(size_t)n] == 0) || (touched[(size_t)n] > 0 && owners[(size_t)n] != 1))
            return fail(SGB_ERR_NUMERICAL, "node owner count");
        if (touched[(size_t)n] > 1 ? cnt != touched[(size_t)n] : cnt != 0)
            return fail(SGB_ERR_NUMERICAL, "partial slot count");
        boundary += cnt > 0;
    }
    for (size_t i = 0; i < seen.size(); ++i)
        if (seen[i] != 1) return fail(SGB_ERR_NUMERICAL, "element corner not gathered exactly once");
    if (stats) {
        stats[0] = P;
        stats[1] = L.max_lnodes;
        stats[2] = (int)L.lnode_gid.size();
        stats[3] = boundary;
        stats[4] = L.n_partials;
    }
    return SGB_OK;
}

void sgb_scene_params_default(sgb_scene_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dt = 0.01;
    p->cg_iterations = 25;
    p->cg_tolerance = 1e-5;
    p->cg_threshold = 1e-5;
    p->gravity[1] = -9.81;
    p->vertex_mass = 1.0;
    p->mass_first = 1;
}

static void free_scene(sgb_scene* sc)
{
    Scene& s = sc->s;
    if (s.graph) cudaGraphExecDestroy(s.graph);
    cudaFree(s.x);
    cudaFree(s.v);
    cudaFree(s.node_mass);
    cudaFree(s.fixed);
    cudaFree(s.dinv);
    cudaFree(s.ext);
    cudaFree(s.f);
    cudaFree(s.b);
    cudaFree(s.xs);
    cudaFree(s.p);
    cudaFree(s.p2);
    cudaFree(s.q);
    cudaFree(s.r);
    cudaFree(s.eforce_v);
    cudaFree(s.cg);
    cudaFree(sc->dot_terms);
    cudaFree(s.b64);
    cudaFree(s.x64);
    cudaFree(s.w64);
    cudaFree(s.r64);
    cudaFree(s.ext64);
    if (s.cg_h) cudaFreeHost(s.cg_h);
    if (sc->shadow) sgb_tfem_destroy(sc->shadow);
    sc->shadow = nullptr;
    s.shadow = nullptr;
}

int sgb_scene_create(sgb_scene_t** out, sgb_tfem_t* fem, const sgb_scene_params* params)
{
    if (!out || !fem || !params) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: NULL argument");
    *out = nullptr;
    const sgb_scene_params& P = *params;
    if (!(P.dt > 0) || P.cg_iterations < 0 || !(P.cg_tolerance >= 0) || !(P.cg_threshold >= 0))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: invalid solver parameters");
    if (P.n_fixed < 0 || (P.n_fixed > 0 && !P.fixed_host))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: invalid fixed indices");
    if (P.residual_replacement < 0)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: residual_replacement must be >= 0");
    if (P.linear_solver != SGB_SOLVER_CG && P.linear_solver != SGB_SOLVER_PCG)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: unknown linear_solver");
    if (P.preconditioner != SGB_PRECOND_NONE && P.preconditioner != SGB_PRECOND_JACOBI)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: unknown preconditioner");
    if (P.preconditioner != SGB_PRECOND_NONE && P.linear_solver != SGB_SOLVER_PCG)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: a preconditioner needs linear_solver = PCG");
    if (P.warm_start && P.residual_replacement > 0)
        return fail(SGB_ERR_NOT_SUPPORTED, "sgb_scene_create: residual replacement starts each solve from x = 0");
    if (P.first_order && P.residual_replacement > 0)
        return fail(SGB_ERR_NOT_SUPPORTED, "sgb_scene_create: residual replacement runs the second-order scheme");
    if (!std::isfinite(P.ff_rayleigh_stiffness) || !std::isfinite(P.mass_rayleigh_mass))
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_create: non-finite component Rayleigh coefficient");
    if (P.linear_solver == SGB_SOLVER_PCG && P.residual_replacement > 0)
        return fail(SGB_ERR_NOT_SUPPORTED, "sgb_scene_create: residual replacement runs with CG only");
    if (P.residual_replacement > 0 &&
        (fem->m.precision != SGB_PRECISION_MIXED || fem->m.pl.n_patches == 0 || fem->m.method == SGB_METHOD_SMALL))
        return fail(SGB_ERR_NOT_SUPPORTED,
                    "sgb_scene_create: residual replacement needs a mixed-precision large/polar force field");
    sgb_scene* sc = new sgb_scene();
    Scene& s = sc->s;
    const int N = fem->m.n_nodes;
    const size_t rs = fem->m.real_size;
    s.mesh = &fem->m;
    s.n = N;
    s.prm.dt = P.dt;
    s.prm.rayleigh_stiffness = P.rayleigh_stiffness;
    s.prm.rayleigh_mass = P.rayleigh_mass;
    s.prm.vdamping = P.vdamping;
    s.prm.cg_iterations = P.cg_iterations;
    s.prm.cg_tolerance = P.cg_tolerance;
    s.prm.cg_threshold = P.cg_threshold;
    for (int k = 0; k < 3; ++k) s.prm.gravity[k] = P.gravity[k];
    s.prm.vertex_mass = P.vertex_mass;
    s.prm.solver = P.linear_solver;
    s.prm.precond = P.preconditioner;
    s.prm.precond_rate = P.preconditioner_rate > 1 ? P.preconditioner_rate : 1;
    s.prm.warm_start = P.warm_start ? 1 : 0;
    s.prm.ff_rs = P.ff_rayleigh_stiffness;
    s.prm.mass_rm = P.mass_rayleigh_mass;
    s.prm.first_order = P.first_order ? 1 : 0;
    s.prm.project_velocity = P.project_velocity ? 1 : 0;
    s.prm.trapezoidal = P.trapezoidal_scheme ? 1 : 0;
    s.prm.compute_residual = P.compute_residual ? 1 : 0;
    s.prm.separate_gravity = P.separate_gravity ? 1 : 0;
    s.stream = fem->stream;
    sc->fem = fem;
    sc->ops = fem->ops;
    sc->serial_dots = P.serial_dots;
    sc->mass_first = P.mass_first;
    size_t* acc = &s.device_bytes;
    int rc;
    std::vector<uint8_t> fixed((size_t)N, 0);
    if (P.fix_all)
        std::fill(fixed.begin(), fixed.end(), 1);
    else
        for (int i = 0; i < P.n_fixed; ++i)
            if (P.fixed_host[i] >= 0 && P.fixed_host[i] < N) fixed[(size_t)P.fixed_host[i]] = 1;
    cudaError_t ce;
    if ((rc = dev_alloc(&s.x, 3 * (size_t)N, acc)) || (rc = dev_alloc(&s.v, 3 * (size_t)N, acc)) ||
        (rc = dev_alloc(&s.fixed, (size_t)N, acc)) || (rc = dev_alloc_bytes(&s.f, rs * 3 * N, acc)) ||
        (rc = dev_alloc_bytes(&s.b, rs * 3 * N, acc)) || (rc = dev_alloc_bytes(&s.xs, rs * 3 * N, acc)) ||
        (rc = dev_alloc_bytes(&s.p, rs * 3 * N, acc)) || (rc = dev_alloc_bytes(&s.p2, rs * 3 * N, acc)) ||
        (rc = dev_alloc_bytes(&s.q, rs * 3 * N, acc)) ||
        (rc = dev_alloc_bytes(&s.r, rs * 3 * N, acc)) || (rc = dev_alloc(&s.cg, 1, acc)))
        goto fail_out;
    if (P.node_masses_host && (rc = dev_alloc(&s.node_mass, (size_t)N, acc))) goto fail_out;
    if (P.serial_dots && (rc = dev_alloc(&sc->dot_terms, (size_t)N, acc))) goto fail_out;
    if (P.preconditioner == SGB_PRECOND_JACOBI && (rc = dev_alloc_bytes(&s.dinv, rs * 3 * N, acc))) goto fail_out;
    // the patch step's force and right-hand side passes (FP32 large / polar /
    // svd): by patches where the force field set that kernel up, else over
    // the elements with a second corner-term buffer; SGB_FUSED_RHS=0 runs
    // the four separate kernels (the same operations)
    if (fem->m.precision == SGB_PRECISION_MIXED && fem->m.pl.n_patches > 0 && fem->m.method != SGB_METHOD_SMALL &&
        fused_rhs_default()) {
        if (fem->m.force_patch_grid > 0) {
            s.rhs_form = 2;
        } else {
            if ((rc = dev_alloc_bytes(&s.eforce_v, rs * 12 * std::max<size_t>((size_t)fem->m.n_tets, 1), acc)))
                goto fail_out;
            s.rhs_form = 1;
        }
    }
    if (P.residual_replacement > 0) {
        // the FP64 copy of the operator, created from the force field's
        // inputs (rest positions and tetrahedra read back, caller order)
        const TfemMesh& fm = fem->m;
        std::vector<double> rest((size_t)N * 3);
        std::vector<int32_t> store((size_t)fm.n_tets * 4), tets((size_t)fm.n_tets * 4);
        if ((ce = cudaMemcpy(rest.data(), fm.rest_pos, sizeof(double) * rest.size(), cudaMemcpyDeviceToHost)) ||
            (ce = cudaMemcpy(store.data(), fm.tets, sizeof(int32_t) * store.size(), cudaMemcpyDeviceToHost))) {
            rc = cuda_fail(ce, "residual replacement set-up");
            goto fail_out;
        }
        for (size_t st = 0; st < (size_t)fm.n_tets; ++st)
            for (int c = 0; c < 4; ++c) tets[4 * (size_t)fm.perm_h[st] + c] = store[4 * st + c];
        if ((rc = sgb_tfem_create(&sc->shadow, N, rest.data(), fm.n_tets, tets.data(), fm.young_h.data(),
                                  (int)fm.young_h.size(), fm.poisson_h.data(), (int)fm.poisson_h.size(),
                                  fm.lsf_h.empty() ? nullptr : fm.lsf_h.data(), (int)fm.lsf_h.size(), fm.method,
                                  SGB_PRECISION_FP64_FMA)))
            goto fail_out;
        s.shadow = &sc->shadow->m;
        s.replace_every = P.residual_replacement;
        *acc += sc->shadow->m.device_bytes;
        if ((rc = dev_alloc(&s.b64, 3 * (size_t)N, acc)) || (rc = dev_alloc(&s.x64, 3 * (size_t)N, acc)) ||
            (rc = dev_alloc(&s.w64, 3 * (size_t)N, acc)) || (rc = dev_alloc(&s.r64, 3 * (size_t)N, acc)))
            goto fail_out;
    }
    if ((ce = cudaMallocHost((void**)&s.cg_h, sizeof(CgScalars))) != cudaSuccess) {
        rc = cuda_fail(ce, "cudaMallocHost");
        goto fail_out;
    }
    if ((ce = cudaMemcpyAsync(s.x, fem->m.rest_pos, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s.stream)) ||
        (ce = cudaMemsetAsync(s.v, 0, sizeof(double) * 3 * N, s.stream)) ||
        (ce = cudaMemsetAsync(s.p, 0, rs * 3 * N, s.stream)) || (ce = cudaMemsetAsync(s.p2, 0, rs * 3 * N, s.stream)) ||
        (ce = cudaMemsetAsync(s.xs, 0, rs * 3 * N, s.stream)) ||
        (ce = cudaMemsetAsync(s.cg, 0, sizeof(CgScalars), s.stream)) ||
        (ce = cudaMemcpyAsync(s.fixed, fixed.data(), (size_t)N, cudaMemcpyHostToDevice, s.stream))) {
        rc = cuda_fail(ce, "scene init copy");
        goto fail_out;
    }
    if (P.node_masses_host &&
        (ce = cudaMemcpyAsync(s.node_mass, P.node_masses_host, sizeof(double) * N, cudaMemcpyHostToDevice, s.stream))) {
        rc = cuda_fail(ce, "scene init copy");
        goto fail_out;
    }
    if ((ce = cudaStreamSynchronize(s.stream)) != cudaSuccess) {
        rc = cuda_fail(ce, "scene init");
        goto fail_out;
    }
    *out = sc;
    return SGB_OK;
fail_out:
    free_scene(sc);
    delete sc;
    return rc;
}

int sgb_scene_destroy(sgb_scene_t* scene)
{
    if (!scene) return SGB_OK;
    cudaStreamSynchronize(scene->s.stream);
    free_scene(scene);
    sgb_tfem_destroy(scene->fem);
    delete scene;
    return SGB_OK;
}

int sgb_scene_step(sgb_scene_t* scene, int n_steps)
{
    if (!scene || n_steps < 0) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_step: invalid argument");
    Scene& s = scene->s;
    const TfemMesh& fm = *s.mesh;
    if (s.replace_every > 0 && fm.plastic && fm.plastic_max > 0.0)
        return fail(SGB_ERR_NOT_SUPPORTED, "sgb_scene_step: plasticity runs without residual replacement");
    if (s.graph_valid && s.graph_plastic_version != fm.plastic_version) s.graph_valid = false;
    if (!s.graph_valid) {
        if (s.graph) {
            cudaGraphExecDestroy(s.graph);
            s.graph = nullptr;
        }
        s.graph_plastic_version = fm.plastic_version;
        cudaGraph_t g;
        SGB_CUDA_TRY(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
        scene->ops->scene_step(&s, scene->dot_terms, scene->mass_first, s.stream);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(s.stream, &g);
        if (le != cudaSuccess) return cuda_fail(le, "scene step launch");
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&s.graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
        s.graph_valid = true;
    }
    for (int i = 0; i < n_steps; ++i) SGB_CUDA_TRY(cudaGraphLaunch(s.graph, s.stream));
    return SGB_OK;
}

int sgb_scene_von_mises(sgb_scene_t* scene, int mode, double* per_element_host, double* per_node_host)
{
    if (!scene || !per_element_host) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_von_mises: NULL argument");
    const TfemMesh& m = scene->fem->m;
    const size_t E = (size_t)m.n_tets, N = (size_t)m.n_nodes;
    double *d_e = nullptr, *d_n = nullptr;
    cudaError_t ce = cudaMalloc(&d_e, sizeof(double) * std::max<size_t>(E, 1));
    if (ce == cudaSuccess && per_node_host) ce = cudaMalloc(&d_n, sizeof(double) * std::max<size_t>(N, 1));
    int rc = SGB_OK;
    if (ce == cudaSuccess) {
        rc = sgb_tfem_von_mises(scene->fem, mode, scene->s.x, d_e, d_n, scene->s.stream);
        if (rc == SGB_OK) {
            ce = cudaMemcpyAsync(per_element_host, d_e, sizeof(double) * E, cudaMemcpyDeviceToHost, scene->s.stream);
            if (ce == cudaSuccess && per_node_host)
                ce = cudaMemcpyAsync(per_node_host, d_n, sizeof(double) * N, cudaMemcpyDeviceToHost,
                                     scene->s.stream);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(scene->s.stream);
        }
    }
    cudaFree(d_e);
    cudaFree(d_n);
    if (rc != SGB_OK) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "sgb_scene_von_mises");
    return SGB_OK;
}

int sgb_scene_sync(sgb_scene_t* scene, int* cg_iterations, double* cg_residual)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_sync: NULL scene");
    Scene& s = scene->s;
    SGB_CUDA_TRY(cudaMemcpyAsync(s.cg_h, s.cg, offsetof(CgScalars, partials), cudaMemcpyDeviceToHost, s.stream));
    SGB_CUDA_TRY(cudaStreamSynchronize(s.stream));
    if (cg_iterations) *cg_iterations = s.cg_h->iters;
    if (cg_residual) *cg_residual = s.cg_h->last_err;
    if (s.cg_h->status & 1) return fail(SGB_ERR_NUMERICAL, "non-finite value in the CG solve");
    if (s.cg_h->status & 2) return fail(SGB_ERR_DEVICE_TIMEOUT, "a bounded device-side wait ran out in the CG solve");
    return SGB_OK;
}

int sgb_scene_residual(sgb_scene_t* scene, double* residual)
{
    if (!scene || !residual) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_residual: NULL argument");
    Scene& s = scene->s;
    if (!s.prm.compute_residual)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_residual: the scene was created without compute_residual");
    SGB_CUDA_TRY(cudaMemcpyAsync(s.cg_h, s.cg, offsetof(CgScalars, partials), cudaMemcpyDeviceToHost, s.stream));
    SGB_CUDA_TRY(cudaStreamSynchronize(s.stream));
    *residual = s.cg_h->residual;
    return SGB_OK;
}

int sgb_scene_get_state(sgb_scene_t* scene, double* x_host, double* v_host)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_get_state: NULL scene");
    Scene& s = scene->s;
    const size_t bytes = sizeof(double) * 3 * (size_t)s.n;
    if (x_host) SGB_CUDA_TRY(cudaMemcpyAsync(x_host, s.x, bytes, cudaMemcpyDeviceToHost, s.stream));
    if (v_host) SGB_CUDA_TRY(cudaMemcpyAsync(v_host, s.v, bytes, cudaMemcpyDeviceToHost, s.stream));
    SGB_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return SGB_OK;
}

int sgb_scene_set_state(sgb_scene_t* scene, const double* x_host, const double* v_host)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_set_state: NULL scene");
    Scene& s = scene->s;
    const size_t bytes = sizeof(double) * 3 * (size_t)s.n;
    // stream-ordered: with pinned host buffers the copies run asynchronously
    // (the caller keeps the buffers unchanged until a later synchronising
    // call); pageable buffers are copied before the call returns
    if (x_host) SGB_CUDA_TRY(cudaMemcpyAsync(s.x, x_host, bytes, cudaMemcpyHostToDevice, s.stream));
    if (v_host) SGB_CUDA_TRY(cudaMemcpyAsync(s.v, v_host, bytes, cudaMemcpyHostToDevice, s.stream));
    return SGB_OK;
}

int sgb_scene_set_external_force(sgb_scene_t* scene, const double* fext_host)
{
    if (!scene || !fext_host) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_set_external_force: NULL argument");
    Scene& s = scene->s;
    const size_t n3 = 3 * (size_t)s.n, rs = s.mesh->real_size;
    if (!s.ext) {
        int rc = dev_alloc_bytes(&s.ext, rs * n3, &s.device_bytes);
        if (rc) return rc;
        s.graph_valid = false;  // the force gather reads ext: re-record the step
        if (s.graph) {
            cudaGraphExecDestroy(s.graph);
            s.graph = nullptr;
        }
    }
    if (s.shadow) {
        if (!s.ext64) {
            int rc = dev_alloc(&s.ext64, n3, &s.device_bytes);
            if (rc) return rc;
            s.graph_valid = false;
            if (s.graph) {
                cudaGraphExecDestroy(s.graph);
                s.graph = nullptr;
            }
        }
        SGB_CUDA_TRY(cudaMemcpyAsync(s.ext64, fext_host, sizeof(double) * n3, cudaMemcpyHostToDevice, s.stream));
    }
    if (rs == sizeof(double)) {
        SGB_CUDA_TRY(cudaMemcpyAsync(s.ext, fext_host, sizeof(double) * n3, cudaMemcpyHostToDevice, s.stream));
    } else {
        std::vector<float> tmp(n3);
        for (size_t i = 0; i < n3; ++i) tmp[i] = (float)fext_host[i];
        SGB_CUDA_TRY(cudaMemcpyAsync(s.ext, tmp.data(), sizeof(float) * n3, cudaMemcpyHostToDevice, s.stream));
        SGB_CUDA_TRY(cudaStreamSynchronize(s.stream));
    }
    SGB_CUDA_TRY(cudaStreamSynchronize(s.stream));
    return SGB_OK;
}

int sgb_scene_state_device(sgb_scene_t* scene, double** x_dev, double** v_dev)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_scene_state_device: NULL scene");
    if (x_dev) *x_dev = scene->s.x;
    if (v_dev) *v_dev = scene->s.v;
    return SGB_OK;
}

void* sgb_scene_stream(sgb_scene_t* scene) { return scene ? (void*)scene->s.stream : nullptr; }

}  // extern "C"
