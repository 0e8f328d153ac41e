// Batched multi-mesh kernels: every admitted mesh advances one implicit
// Euler step through the same launches. Each launch is a persistent grid
// that walks a device-resident work list (patches, element ranges or node
// chunks of all active meshes); the mesh of an item is found through its
// slot's BMeshDesc. Per-mesh dot products are reduced without float atomics:
// inside the CG loop every item writes its partial sum and a small kernel
// with one block per mesh slot adds them in index order and updates that
// mesh's CG scalars (CGLinearSolver::solve, Sofa/Component/LinearSolver/
// Iterative/src/sofa/component/linearsolver/iterative/CGLinearSolver.inl:
// 102-272); the once-per-step start of CG reduces with a per-mesh ticket.
// Meshes whose CG has stopped skip their items. Every partial belongs to one
// work item (a patch or a node chunk) and is formed in an order fixed by the
// item alone, so neither the grid sizes nor the register caps and nodes per
// thread the tile tuner picks change a single bit of the results.
//
// Included by the variant translation units after tfem_impl.cuh, inside
// SGB_NS, for R = float (mixed) and R = double (FP64 with FMA).
#pragma once

namespace SGB_NS {

constexpr int kBatchThreads = 256;

template <typename R>
__device__ __forceinline__ ElemView<R> bm_elem_view(const BMeshDesc& m)
{
    ElemView<R> ev;
    ev.tets = m.tets;
    ev.rot = (R*)m.rot;
    ev.K = (const R*)m.K;
    ev.J = (const R*)m.J;
    ev.rest = (const R*)m.rest;
    ev.rest_ff = m.rest_ff;
    ev.A0inv = nullptr;  // the batch engine admits large and polar meshes
    ev.R0 = nullptr;
    ev.n_tets = m.n_tets;
    ev.method = m.method;
    return ev;
}

__device__ __forceinline__ PatchView bm_patch_view(const BMeshDesc& m, int pe)
{
    PatchView pv;
    pv.elem_start = m.elem_start;
    pv.node_start = m.node_start;
    pv.lnode_gid = m.lnode_gid;
    pv.lnode_info = m.lnode_info;
    pv.lrow = m.lrow;
    pv.lslots = m.lslots;
    pv.lconn = m.lconn;
    pv.bnd_rowptr = m.bnd_rowptr;
    pv.n_patches = m.n_patches;
    pv.pe = pe;
    pv.max_lnodes = batch_max_lnodes(pe);
    return pv;
}

__device__ __forceinline__ bool bm_cg_skip(const BMeshDesc& m, int it)
{
    return m.done || it > m.cg_iterations || !m.active;
}

// Canonical sum of a node chunk's per-node terms: the terms of nodes
// 32g .. 32g+31 (chunk-local) are added as a balanced pairwise tree,
// neighbours first, and the chunk's group sums are then added in group order.
// A thread holding NPT consecutive nodes adds the first log2(NPT) tree levels
// itself and the warp butterfly adds the rest, so every group sum -- and the
// chunk sum -- is the same for NPT = 1, 2 or 4 (IEEE addition is
// commutative). group_tree_store: this thread's NPT terms (node order) of
// the pass starting at chunk-local node `base`; every thread of the block
// calls it. Groups past the chunk's end hold zeros.
template <int NPT>
__device__ __forceinline__ void group_tree_store(const double t[NPT], int base, double* gsum)
{
    double v;
    if constexpr (NPT == 4)
        v = (t[0] + t[1]) + (t[2] + t[3]);
    else if constexpr (NPT == 2)
        v = t[0] + t[1];
    else
        v = t[0];
    constexpr int lanes = 32 / NPT;  // lanes holding one group of 32 nodes
#pragma unroll
    for (int o = 1; o < lanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x % lanes) == 0) gsum[(base + (int)threadIdx.x * NPT) / 32] = v;
}

// The chunk sum from its group sums, in group order (thread 0), after a
// block barrier.
__device__ __forceinline__ double groups_sum(const double* gsum, int n_groups)
{
    double total = 0.0;
    if (threadIdx.x == 0)
        for (int g = 0; g < n_groups; ++g) total += gsum[g];
    return total;
}

// Block-wide: store this item's partial, take the mesh's ticket; when this
// is the mesh's last item, returns true in every thread with the mesh total
// in `total` (valid in thread 0).
__device__ __forceinline__ bool bm_ticket_sum(double mine, double* partials, int idx, unsigned int* ticket,
                                              int count, double* total)
{
    __shared__ int last;
    const double bsum = block_sum(mine);
    if (threadIdx.x == 0) {
        partials[idx] = bsum;
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        last = (t == (unsigned int)count - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double v = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) v += __ldcg(&partials[i]);
    *total = block_sum(v);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// CG start: rho = r.r, |b|. Every node chunk of the mesh calls it with its
// share; the last one to arrive adds the chunk partials in chunk order.
__device__ __forceinline__ void rhs_done(BMeshDesc& m, int chunk, double mine)
{
    double total;
    if (bm_ticket_sum(mine, m.chunk_sum, chunk, &m.ticket_rhs, m.n_chunks, &total) && threadIdx.x == 0) {
        m.rho = total;
        m.normb = sqrt(total);
        m.iters = 0;
        m.last_err = 0.0;
        m.den = 0.0;
        if (!isfinite(total)) {
            m.status |= 1;
            m.done = 1;
        } else if (m.normb == 0.0 || m.cg_iterations <= 0) {
            m.done = 1;
        } else {
            const double err = sqrt(total) / m.normb;
            m.last_err = err;
            m.done = (err <= m.tol && m.tsc != 0) ? 1 : 0;
        }
    }
    __syncthreads();
}

// ---- force: f = ext + m g + internal forces --------------------------------
template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_force_elem(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                               const int* __restrict__ counts)
{
    const int L = counts[WL_ELEM];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        const BMeshDesc& m = M[it.slot];
        const ElemView<R> ev = bm_elem_view<R>(m);
        R* ef = (R*)m.eforce;
        for (int e = it.a + threadIdx.x; e < it.b; e += blockDim.x) {
            if (m.method == METHOD_LARGE)
                elem_force_body<R, METHOD_LARGE>(ev, e, m.x, m.rest_pos, ef);
            else
                elem_force_body<R, METHOD_POLAR>(ev, e, m.x, m.rest_pos, ef);
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_force_gather(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                                 const int* __restrict__ counts)
{
    const int L = counts[WL_NODE];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        const BMeshDesc& m = M[it.slot];
        const R* ef = (const R*)m.eforce;
        const R* ext = (const R*)m.ext;
        R* f = (R*)m.f;
        const R mg0 = (R)(m.g[0] * m.vertex_mass), mg1 = (R)(m.g[1] * m.vertex_mass),
                mg2 = (R)(m.g[2] * m.vertex_mass);
        for (int n = it.a + threadIdx.x; n < it.b; n += blockDim.x) {
            R a0 = R(0), a1 = R(0), a2 = R(0);
            if (ext) {
                a0 += ext[3 * (size_t)n];
                a1 += ext[3 * (size_t)n + 1];
                a2 += ext[3 * (size_t)n + 2];
            }
            if (m.node_mass) {
                const double mm = m.node_mass[n];
                a0 += (R)(m.g[0] * mm);
                a1 += (R)(m.g[1] * mm);
                a2 += (R)(m.g[2] * mm);
            } else {
                a0 += mg0;
                a1 += mg1;
                a2 += mg2;
            }
            for (int s = m.rowptr[n]; s < m.rowptr[n + 1]; ++s) {
                const R* c = ef + 3 * (size_t)m.slots[s];
                a0 += c[0];
                a1 += c[1];
                a2 += c[2];
            }
            f[3 * (size_t)n] = a0;
            f[3 * (size_t)n + 1] = a1;
            f[3 * (size_t)n + 2] = a2;
        }
    }
}

// ---- right-hand side b = h (f - (h+rs) K v - rm M v), CG start -------------
template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_rhs_elem(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                             const int* __restrict__ counts)
{
    const int L = counts[WL_ELEM];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        const BMeshDesc& m = M[it.slot];
        const ElemView<R> ev = bm_elem_view<R>(m);
        for (int e = it.a + threadIdx.x; e < it.b; e += blockDim.x)
            elem_dforce_body<R, double, METHOD_LARGE, 0>(ev, e, m.v, nullptr, R(0), (R)m.kf_rhs, (R*)m.eforce);
    }
}

template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_rhs_gather(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                               const int* __restrict__ counts)
{
    const int L = counts[WL_NODE];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        BMeshDesc& m = M[it.slot];
        const R* ef = (const R*)m.eforce;
        const R* f = (const R*)m.f;
        R* b = (R*)m.b;
        R* r = (R*)m.r;
        R* xs = (R*)m.xs;
        const double rmf = m.rm_factor;  // -rm
        const R mmu = (R)(rmf != 1.0 ? m.vertex_mass * rmf : m.vertex_mass);
        const R hr = (R)m.h;
        double dlocal = 0.0;
        for (int n = it.a + threadIdx.x; n < it.b; n += blockDim.x) {
            R a[3] = {f[3 * (size_t)n], f[3 * (size_t)n + 1], f[3 * (size_t)n + 2]};
            const R vv[3] = {(R)m.v[3 * (size_t)n], (R)m.v[3 * (size_t)n + 1], (R)m.v[3 * (size_t)n + 2]};
            if (rmf != 0.0) {
                const R mm = m.node_mass ? (R)(m.node_mass[n] * rmf) : mmu;
#pragma unroll
                for (int k = 0; k < 3; ++k) a[k] += vv[k] * mm;
            }
            for (int s = m.rowptr[n]; s < m.rowptr[n + 1]; ++s) {
                const R* c = ef + 3 * (size_t)m.slots[s];
                a[0] -= c[0];
                a[1] -= c[1];
                a[2] -= c[2];
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] *= hr;
            if (m.fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                b[3 * (size_t)n + k] = a[k];
                r[3 * (size_t)n + k] = a[k];
                xs[3 * (size_t)n + k] = R(0);
            }
            dlocal += (double)(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        }
        rhs_done(m, it.c, dlocal);  // the chunk's partial at its own index
    }
}

// ---- forces and right-hand side in one element pass and one node pass ------
// The operations of kb_force_elem + kb_rhs_elem (force terms into eforce, the
// (h + rs) K v terms into eforce_v) and of kb_force_gather + kb_rhs_gather
// (f kept in registers): the same operations in two launches instead of
// four (FMA contraction may differ between the kernels: equal to rounding).
template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_force_rhs_elem(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                                   const int* __restrict__ counts)
{
    const int L = counts[WL_ELEM];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        const BMeshDesc& m = M[it.slot];
        const ElemView<R> ev = bm_elem_view<R>(m);
        R* ef = (R*)m.eforce;
        R* efv = (R*)m.eforce_v;
        const R kf = (R)m.kf_rhs;
        for (int e = it.a + threadIdx.x; e < it.b; e += blockDim.x) {
            R Rm[9], K[3], J[12];
            if (m.method == METHOD_LARGE)
                elem_force_body<R, METHOD_LARGE, true>(ev, e, m.x, m.rest_pos, ef, PlasticArgs<R>{}, Rm, K, J);
            else
                elem_force_body<R, METHOD_POLAR, true>(ev, e, m.x, m.rest_pos, ef, PlasticArgs<R>{}, Rm, K, J);
            rhs_v_terms(ev, e, m.v, Rm, K, J, kf, efv);
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_force_rhs_gather(BMeshDesc* M,
                                                                     const WorkItem* __restrict__ items,
                                                                     const int* __restrict__ counts)
{
    const int L = counts[WL_NODE];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        BMeshDesc& m = M[it.slot];
        const R* ef = (const R*)m.eforce;
        const R* efv = (const R*)m.eforce_v;
        const R* ext = (const R*)m.ext;
        R* b = (R*)m.b;
        R* r = (R*)m.r;
        R* xs = (R*)m.xs;
        const R mg0 = (R)(m.g[0] * m.vertex_mass), mg1 = (R)(m.g[1] * m.vertex_mass),
                mg2 = (R)(m.g[2] * m.vertex_mass);
        const double rmf = m.rm_factor;  // -rm
        const R mmu = (R)(rmf != 1.0 ? m.vertex_mass * rmf : m.vertex_mass);
        const R hr = (R)m.h;
        double dlocal = 0.0;
        for (int n = it.a + threadIdx.x; n < it.b; n += blockDim.x) {
            R a0 = R(0), a1 = R(0), a2 = R(0);
            if (ext) {
                a0 += ext[3 * (size_t)n];
                a1 += ext[3 * (size_t)n + 1];
                a2 += ext[3 * (size_t)n + 2];
            }
            if (m.node_mass) {
                const double mm = m.node_mass[n];
                a0 += (R)(m.g[0] * mm);
                a1 += (R)(m.g[1] * mm);
                a2 += (R)(m.g[2] * mm);
            } else {
                a0 += mg0;
                a1 += mg1;
                a2 += mg2;
            }
            const int s0 = m.rowptr[n], s1 = m.rowptr[n + 1];
            for (int s = s0; s < s1; ++s) {
                const R* c = ef + 3 * (size_t)m.slots[s];
                a0 += c[0];
                a1 += c[1];
                a2 += c[2];
            }
            R a[3] = {a0, a1, a2};
            const R vv[3] = {(R)m.v[3 * (size_t)n], (R)m.v[3 * (size_t)n + 1], (R)m.v[3 * (size_t)n + 2]};
            if (rmf != 0.0) {
                const R mm = m.node_mass ? (R)(m.node_mass[n] * rmf) : mmu;
#pragma unroll
                for (int k = 0; k < 3; ++k) a[k] += vv[k] * mm;
            }
            for (int s = s0; s < s1; ++s) {
                const R* c = efv + 3 * (size_t)m.slots[s];
                a[0] -= c[0];
                a[1] -= c[1];
                a[2] -= c[2];
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] *= hr;
            if (m.fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                b[3 * (size_t)n + k] = a[k];
                r[3 * (size_t)n + k] = a[k];
                xs[3 * (size_t)n + k] = R(0);
            }
            dlocal += (double)(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        }
        rhs_done(m, it.c, dlocal);  // the chunk's partial at its own index
    }
}

// ---- forces and right-hand side by patches (mixed precision) ---------------
// The operations of kb_force_rhs_elem + kb_force_rhs_gather with each
// element's force terms less its (h + rs) K v terms summed per local node in
// shared memory, as k_patch_force_rhs does for one mesh: interior nodes into
// the mesh's q, shared nodes into their partial slots; kb_rhs_finish_patch
// then forms b per node chunk. Every sum belongs to one patch or one node
// chunk, so the results do not depend on the other meshes of the batch.
template <typename R>
struct BRhsArgs {
    const double* x;
    const double* v;
    R kf;
    int method;
    R* own;
    R* partials;
};

template <typename R>
size_t batch_force_smem(int pe)
{
    return force_patch_smem_size<R>(pe, batch_max_lnodes(pe));
}

// 80 registers (no spills): 6 resident CTAs of 128 threads per SM instead of
// 5 at 96, 0.3 % faster batch steps
template <typename R>
__global__ void __maxnreg__(80) kb_force_rhs_patch(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                                    const int* __restrict__ counts, int pe)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* ef;
    R* lp;
    uint16_t* sl;
    int* lr;
    patch_smem_carve<R>(smem_raw, pe, batch_max_lnodes(pe), &ef, &sl, &lr, &lp);
    float2* lv = reinterpret_cast<float2*>(lp);
    // the open mesh's views and operands, read where they are used
    __shared__ PatchView spv;
    __shared__ ElemView<R> sev;
    __shared__ BRhsArgs<R> sa;
    const int L = counts[WL_PATCH];
    int open_slot = -1;
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem wi = items[w];
        if (open_slot != wi.slot) {
            open_slot = wi.slot;
            // the previous patch ended with a block barrier
            if (threadIdx.x == 0) {
                const BMeshDesc& m = M[wi.slot];
                spv = bm_patch_view(m, pe);
                sev = bm_elem_view<R>(m);
                sa = BRhsArgs<R>{m.x, m.v, (R)m.kf_rhs, m.method, (R*)m.q, (R*)m.partials};
            }
            __syncthreads();
        }
        if (sa.method == METHOD_LARGE)
            patch_force_rhs_body<R, METHOD_LARGE>(spv, sev, wi.a, sa.x, sa.v, PlasticArgs<R>{}, sa.kf, 0, sa.own,
                                                  sa.partials, ef, lv, sl, lr);
        else
            patch_force_rhs_body<R, METHOD_POLAR>(spv, sev, wi.a, sa.x, sa.v, PlasticArgs<R>{}, sa.kf, 0, sa.own,
                                                  sa.partials, ef, lv, sl, lr);
    }
}

template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_rhs_finish_patch(BMeshDesc* M,
                                                                     const WorkItem* __restrict__ items,
                                                                     const int* __restrict__ counts)
{
    const int L = counts[WL_NODE];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem it = items[w];
        BMeshDesc& m = M[it.slot];
        const R* own = (const R*)m.q;
        const R* part = (const R*)m.partials;
        const R* ext = (const R*)m.ext;
        R* b = (R*)m.b;
        R* r = (R*)m.r;
        R* xs = (R*)m.xs;
        const R mg0 = (R)(m.g[0] * m.vertex_mass), mg1 = (R)(m.g[1] * m.vertex_mass),
                mg2 = (R)(m.g[2] * m.vertex_mass);
        const double rmf = m.rm_factor;  // -rm
        const R mmu = (R)(rmf != 1.0 ? m.vertex_mass * rmf : m.vertex_mass);
        const R hr = (R)m.h;
        double dlocal = 0.0;
        for (int n = it.a + threadIdx.x; n < it.b; n += blockDim.x) {
            const int b0 = m.bnd_rowptr[n], b1 = m.bnd_rowptr[n + 1];
            R s0 = R(0), s1 = R(0), s2 = R(0);
            if (b0 == b1) {
                s0 = own[3 * (size_t)n];
                s1 = own[3 * (size_t)n + 1];
                s2 = own[3 * (size_t)n + 2];
            } else {
                for (int k = b0; k < b1; ++k) {
                    s0 += part[3 * (size_t)k];
                    s1 += part[3 * (size_t)k + 1];
                    s2 += part[3 * (size_t)k + 2];
                }
            }
            R a[3] = {R(0), R(0), R(0)};
            if (ext) {
                a[0] += ext[3 * (size_t)n];
                a[1] += ext[3 * (size_t)n + 1];
                a[2] += ext[3 * (size_t)n + 2];
            }
            if (m.node_mass) {
                const double mm = m.node_mass[n];
                a[0] += (R)(m.g[0] * mm);
                a[1] += (R)(m.g[1] * mm);
                a[2] += (R)(m.g[2] * mm);
            } else {
                a[0] += mg0;
                a[1] += mg1;
                a[2] += mg2;
            }
            a[0] += s0;
            a[1] += s1;
            a[2] += s2;
            if (rmf != 0.0) {
                const R mm = m.node_mass ? (R)(m.node_mass[n] * rmf) : mmu;
                const R vv[3] = {(R)m.v[3 * (size_t)n], (R)m.v[3 * (size_t)n + 1], (R)m.v[3 * (size_t)n + 2]};
#pragma unroll
                for (int k = 0; k < 3; ++k) a[k] += vv[k] * mm;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] *= hr;
            if (m.fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                b[3 * (size_t)n + k] = a[k];
                r[3 * (size_t)n + k] = a[k];
                xs[3 * (size_t)n + k] = R(0);
            }
            dlocal += (double)(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        }
        rhs_done(m, it.c, dlocal);  // the chunk's partial at its own index
    }
}

// ---- CG matvec over patches ------------------------------------------------
// MINB: resident CTAs per SM the register cap is set for (a tile of the
// tuner; the arithmetic is the same for every value)
template <typename R, int MODE, int MINB>
__global__ void __launch_bounds__(kPatchThreads, MINB) kb_matvec(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                           const int* __restrict__ counts, int it, int pe,
                                                           int prefetch)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* ef;
    R* lp;
    uint16_t* sl;
    int* lr;
    patch_smem_carve<R>(smem_raw, pe, batch_max_lnodes(pe), &ef, &sl, &lr, &lp);
    // the open mesh's views and operands, read where they are used
    __shared__ PatchView spv;
    __shared__ ElemView<R> sev;
    __shared__ PatchArgs<R> sa;
    const int L = counts[WL_PATCH];
    int open_slot = -1;
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem wi = items[w];
        BMeshDesc& m = M[wi.slot];
        if (bm_cg_skip(m, it)) continue;  // uniform over the block
        if (open_slot != wi.slot) {
            open_slot = wi.slot;
            // the previous patch ended with a block barrier: no thread still
            // reads the shared copies
            if (threadIdx.x == 0) {
                spv = bm_patch_view(m, pe);
                sev = bm_elem_view<R>(m);
                const double mf = m.mf;
                sa.rin = (const R*)m.r;
                sa.pold = (const R*)((it & 1) ? m.p1 : m.p0);
                sa.pnew = (R*)((it & 1) ? m.p0 : m.p1);
                sa.beta = (MODE == 2) ? (R)m.beta : R(0);
                sa.kf = (R)m.kf;
                sa.mmu = (R)(mf != 1.0 ? m.vertex_mass * mf : m.vertex_mass);
                sa.ma = MassArgs{m.node_mass, m.vertex_mass, {m.g[0], m.g[1], m.g[2]}};
                sa.mf = mf;
                sa.fixed = m.fixed;
                sa.qout = (R*)m.q;
                sa.partials = (R*)m.partials;
            }
            __syncthreads();
        }
        if constexpr (is_mixed<R>::value) {
            // the block's next item into L2 while this one computes
            const int wn = w + (int)gridDim.x;
            if (prefetch && threadIdx.x == 0 && wn < L) {
                const WorkItem ni = items[wn];
                const BMeshDesc& nm = M[ni.slot];
                prefetch_patch(bm_patch_view(nm, pe), bm_elem_view<R>(nm), ni.a);
            }
        }
        // the patch's p^T A p share, stored at the patch's own index
        const double e = block_sum((double)patch_body<R, MODE>(spv, sev, wi.a, sa, ef, lp, sl, lr));
        if (threadIdx.x == 0) m.patch_energy[wi.a] = e;
    }
}

// ---- CG update: shared-node q, x += alpha p, r -= alpha q, rho -------------
// NPT 4: a register cap for 4 resident CTAs per SM (64 registers, a few
// spilled; without it 95 registers and 2 CTAs per SM, 2.4 % slower steps)
template <typename R, int NPT>
__global__ void __launch_bounds__(kBatchThreads, NPT == 4 ? 4 : 1) kb_update(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                           const int* __restrict__ counts, int it)
{
    __shared__ double gsum[kBatchNodeChunk / 32];
    const int L = counts[WL_NODE];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem wi = items[w];
        BMeshDesc& m = M[wi.slot];
        if (bm_cg_skip(m, it)) continue;  // uniform over the block
        const R alpha = (R)m.alpha;
        const R* p = (const R*)((it & 1) ? m.p0 : m.p1);
        const R* q = (const R*)m.q;
        const R* partials = (const R*)m.partials;
        R* xs = (R*)m.xs;
        R* r = (R*)m.r;
        const double mf = m.mf;
        const R mmu = (R)(mf != 1.0 ? m.vertex_mass * mf : m.vertex_mass);
        // chunk-local passes of blockDim * NPT nodes; thread t takes NPT
        // consecutive nodes of each pass
        for (int base = 0; base < kBatchNodeChunk; base += kBatchThreads * NPT) {
            const int n0 = wi.a + base + (int)threadIdx.x * NPT;
            double t[NPT];
            if constexpr (is_mixed<R>::value && NPT == 4) {
                if (n0 + 4 <= wi.b) {
                    cg_update4_terms(4 * (size_t)(n0 >> 2), xs, r, p, q, partials, m.bnd_rowptr, m.node_mass, mmu, mf,
                                     m.fixed, alpha, t);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        t[j] = (n0 + j < wi.b)
                                   ? (double)cg_update1<R>((size_t)(n0 + j), xs, r, p, q, partials, m.bnd_rowptr,
                                                           m.node_mass, mmu, mf, m.fixed, alpha)
                                   : 0.0;
                }
            } else {
#pragma unroll
                for (int j = 0; j < NPT; ++j)
                    t[j] = (n0 + j < wi.b) ? (double)cg_update1<R>((size_t)(n0 + j), xs, r, p, q, partials,
                                                                   m.bnd_rowptr, m.node_mass, mmu, mf, m.fixed, alpha)
                                           : 0.0;
            }
            group_tree_store<NPT>(t, base, gsum);
        }
        __syncthreads();
        const double tot = groups_sum(gsum, kBatchNodeChunk / 32);
        if (threadIdx.x == 0) m.chunk_sum[wi.c] = tot;  // the chunk's partial at its own index
        __syncthreads();
    }
}

// ---- per-mesh CG scalars of one iteration ----------------------------------
// One block per mesh slot adds the mesh's partials (one per block run, at
// the run's first item index: min(grid, items) of them) in a fixed order
// (thread-strided, then the block tree). Which items share a partial depends
// only on the item index modulo the grid, so the sum does not depend on the
// other meshes of the batch.
// WHAT 0, after the matvec: den = p.Ap, the threshold test, alpha.
// WHAT 1, after the update: rho = r.r, beta, the tolerance and iteration tests.
template <int WHAT>
__global__ void __launch_bounds__(kBatchThreads) kb_cg_scalars(BMeshDesc* M, int n_slots, int it)
{
    for (int s = blockIdx.x; s < n_slots; s += gridDim.x) {
        BMeshDesc& m = M[s];
        if (bm_cg_skip(m, it)) continue;  // uniform over the block
        const double* part = (WHAT == 0) ? m.patch_energy : m.chunk_sum;
        const int items_m = (WHAT == 0) ? m.n_patches : m.n_chunks;
        const int n = items_m;  // one partial per item
        // thread t adds entries t, t + blockDim, ... in that order; eight
        // loads are issued before their additions
        double v = 0.0;
        for (int i0 = threadIdx.x; i0 < n; i0 += 8 * blockDim.x) {
            double a[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int i = i0 + j * (int)blockDim.x;
                a[j] = i < n ? __ldcg(&part[i]) : 0.0;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) v += a[j];
        }
        const double total = block_sum(v);
        if (threadIdx.x == 0) {
            if (WHAT == 0) {
                m.den = total;
                const bool first_of_first = (it == 1 && m.tsc == 0);
                if (!isfinite(total)) {
                    m.status |= 1;
                    m.done = 1;
                } else if (total != 0.0) {
                    if (fabs(total) <= m.thr && !first_of_first) {
                        m.done = 1;
                        m.iters = it;  // the matvecs run, as the single-mesh count
                    } else {
                        m.alpha = m.rho / total;
                    }
                } else {
                    m.done = 1;
                    m.iters = it;
                }
            } else {
                m.rho_prev = m.rho;
                m.rho = total;
                m.iters = it;
                m.beta = total / m.rho_prev;
                const double err = sqrt(total) / m.normb;
                m.last_err = err;
                if (!isfinite(total)) {
                    m.status |= 1;
                    m.done = 1;
                } else if (err <= m.tol || it >= m.cg_iterations) {
                    m.done = 1;
                }
            }
        }
        __syncthreads();
    }
}

// ---- v += dv, x += h v -------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBatchThreads) kb_euler(BMeshDesc* M, const WorkItem* __restrict__ items,
                                                          const int* __restrict__ counts)
{
    const int L = counts[WL_NODE];
    for (int w = blockIdx.x; w < L; w += gridDim.x) {
        const WorkItem wi = items[w];
        BMeshDesc& m = M[wi.slot];
        const R* xs = (const R*)m.xs;
        const double h = m.h, vd = m.vdamp;
        for (int n = wi.a + threadIdx.x; n < wi.b; n += blockDim.x) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const size_t i = 3 * (size_t)n + k;
                double vv = m.v[i] + (double)xs[i];
                m.x[i] = m.x[i] + vv * h;
                if (vd != 1.0) vv *= vd;
                m.v[i] = vv;
            }
        }
        if (wi.c == 0 && threadIdx.x == 0) m.tsc += 1;
    }
}

// ---- host side: record one step of the whole batch ---------------------------
template <typename R>
size_t batch_patch_smem(int pe)
{
    return patch_smem_size<R>(pe, batch_max_lnodes(pe));
}

// Kernel attributes of the batch step; grid_patch[i]: resident matvec CTAs
// over the device for the register-cap variant kBatchMatvecMinb[i]. Returns
// the SM count, -1 on failure.
template <typename R, int MINB>
int matvec_grid(size_t smem, int sms)
{
    int nb1 = 0, nb2 = 0;
    if (cudaFuncSetAttribute(kb_matvec<R, 1, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaFuncSetAttribute(kb_matvec<R, 2, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
        return -1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb1, kb_matvec<R, 1, MINB>, kPatchThreads, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, kb_matvec<R, 2, MINB>, kPatchThreads, smem);
    const int nb = nb1 < nb2 ? nb1 : nb2;
    return (nb < 1 ? 1 : nb) * sms;
}

template <typename R>
int batch_prepare(int pe, int* grid_patch)
{
    const size_t smem = batch_patch_smem<R>(pe);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_patch[0] = matvec_grid<R, kBatchMatvecMinb[0]>(smem, sms);
    grid_patch[1] = matvec_grid<R, kBatchMatvecMinb[1]>(smem, sms);
    grid_patch[2] = matvec_grid<R, kBatchMatvecMinb[2]>(smem, sms);
    if (grid_patch[0] < 0 || grid_patch[1] < 0 || grid_patch[2] < 0) return -1;
    // grid_patch[3]: resident CTAs of the patch force / right-hand side pass
    // (mixed precision)
    grid_patch[3] = 0;
    if constexpr (is_mixed<R>::value) {
        const size_t fsmem = batch_force_smem<R>(pe);
        if (cudaFuncSetAttribute(kb_force_rhs_patch<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem) !=
            cudaSuccess)
            return -1;
        int nf = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nf, kb_force_rhs_patch<R>, kPatchThreads, fsmem);
        grid_patch[3] = (nf < 1 ? 1 : nf) * sms;
    }
    return sms;
}

template <typename R, int MODE>
void launch_kb_matvec(const BatchLaunch& B, size_t smem, int it, cudaStream_t s)
{
    const WorkItem* pit = B.items[WL_PATCH];
    if (B.matvec_minb == kBatchMatvecMinb[0])
        kb_matvec<R, MODE, kBatchMatvecMinb[0]>
            <<<B.grid_patch, kPatchThreads, smem, s>>>(B.meshes, pit, B.counts, it, B.pe, B.prefetch);
    else if (B.matvec_minb == kBatchMatvecMinb[2])
        kb_matvec<R, MODE, kBatchMatvecMinb[2]>
            <<<B.grid_patch, kPatchThreads, smem, s>>>(B.meshes, pit, B.counts, it, B.pe, B.prefetch);
    else
        kb_matvec<R, MODE, kBatchMatvecMinb[1]>
            <<<B.grid_patch, kPatchThreads, smem, s>>>(B.meshes, pit, B.counts, it, B.pe, B.prefetch);
}

template <typename R>
void launch_kb_update(const BatchLaunch& B, int it, cudaStream_t s)
{
    const WorkItem* nit = B.items[WL_NODE];
    if (B.update_npt == 1)
        kb_update<R, 1><<<B.grid_update, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts, it);
    else if (B.update_npt == 2)
        kb_update<R, 2><<<B.grid_update, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts, it);
    else
        kb_update<R, 4><<<B.grid_update, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts, it);
}

template <typename R>
void batch_record_step(const BatchLaunch& B, cudaStream_t s)
{
    const WorkItem* eit = B.items[WL_ELEM];
    const WorkItem* nit = B.items[WL_NODE];
    if (B.fused_rhs == 2) {
        if constexpr (is_mixed<R>::value) {
            kb_force_rhs_patch<R><<<B.grid_force, kPatchThreads, batch_force_smem<R>(B.pe), s>>>(
                B.meshes, B.items[WL_PATCH], B.counts, B.pe);
            kb_rhs_finish_patch<R><<<B.grid_node, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts);
        }
    } else if (B.fused_rhs) {
        kb_force_rhs_elem<R><<<B.grid_elem, kBatchThreads, 0, s>>>(B.meshes, eit, B.counts);
        kb_force_rhs_gather<R><<<B.grid_node, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts);
    } else {
        kb_force_elem<R><<<B.grid_elem, kBatchThreads, 0, s>>>(B.meshes, eit, B.counts);
        kb_force_gather<R><<<B.grid_node, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts);
        kb_rhs_elem<R><<<B.grid_elem, kBatchThreads, 0, s>>>(B.meshes, eit, B.counts);
        kb_rhs_gather<R><<<B.grid_node, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts);
    }
    const size_t smem = batch_patch_smem<R>(B.pe);
    for (int it = 1; it <= B.max_iterations; ++it) {
        if (it == 1)
            launch_kb_matvec<R, 1>(B, smem, it, s);
        else
            launch_kb_matvec<R, 2>(B, smem, it, s);
        kb_cg_scalars<0><<<B.grid_slots, kBatchThreads, 0, s>>>(B.meshes, B.n_slots, it);
        launch_kb_update<R>(B, it, s);
        kb_cg_scalars<1><<<B.grid_slots, kBatchThreads, 0, s>>>(B.meshes, B.n_slots, it);
    }
    kb_euler<R><<<B.grid_node, kBatchThreads, 0, s>>>(B.meshes, nit, B.counts);
}

}  // namespace SGB_NS
