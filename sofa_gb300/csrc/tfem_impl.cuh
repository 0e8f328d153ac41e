// Kernels of one precision variant of the tetrahedral-FEM implicit step.
//
// This header is compiled three times, each time inside its own namespace
// (SGB_NS):
//   tfem_fp64_exact.cu  R = double, no FMA contraction (-fmad=false): the
//                       element math, node gathers and vector updates round
//                       exactly like the reference's CPU code, so with
//                       serial dot products a whole step is bit-identical to
//                       it;
//   tfem_fp64_fast.cu   R = double with FMA contraction;
//   tfem_mixed.cu       R = float element math and solver vectors, FP64 state
//                       (positions, velocities) and FP64 dot products.
//
// Data flow of one addForce / addDForce (reference: Sofa/Component/
// SolidMechanics/FEM/Elastic/src/sofa/component/solidmechanics/fem/elastic/
// TetrahedronFEMForceField.inl:1548-1636, "TFEM.inl"):
//   element kernel   one thread per tetrahedron: rotation, strain, K J^T,
//                    the four corner forces R^T F into `eforce` (12 reals);
//   gather kernel    one thread per node: sums its (element, corner) slots
//                    from the node->slot CSR in element order, no atomics.
// The solver kernels fuse the mass term, the fixed-node projection, the CG
// vector updates and the dot products into the gathers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "sgb_internal.h"
#include "tfem_math.cuh"

#ifndef SGB_NS
#error "define SGB_NS before including tfem_impl.cuh"
#endif

namespace SGB_NS {
using namespace sgb;

template <typename R>
using is_mixed = std::is_same<R, float>;

__device__ __forceinline__ void ld3(const double* p, long long i, double o[3])
{
    o[0] = p[3 * i];
    o[1] = p[3 * i + 1];
    o[2] = p[3 * i + 2];
}
__device__ __forceinline__ void ld3(const float* p, long long i, float o[3])
{
    o[0] = p[3 * i];
    o[1] = p[3 * i + 1];
    o[2] = p[3 * i + 2];
}

// ------------------------------------------------------------------------
// Element-data access. FP64 keeps the reference's quantities as rows of
// n_tets entries: R (9), K(0,0), K(0,1), K(3,3) (3), J (12). FP32 packs
// what every CG matvec reads into 64 bytes: the rotation as a unit
// quaternion (one float4 in `rot`; a reflection, which the polar factor of an
// inverted element can be, is flagged by w <= -2), and in `J` three float4
// planes holding J scaled by sqrt(K(0,0)) for nodes b, c, d and the ratios
// K(0,1)/K(0,0), K(3,3)/K(0,0). Node a's J is minus the sum of the other
// three (the columns of J sum to zero over the nodes), so a translation
// gives exactly zero strain.
// ------------------------------------------------------------------------
__device__ __forceinline__ float4 rot_to_quat(const float Rm[9])
{
    // Shepperd's method on the largest of the trace and the diagonal
    float det = Rm[0] * (Rm[4] * Rm[8] - Rm[5] * Rm[7]) - Rm[1] * (Rm[3] * Rm[8] - Rm[5] * Rm[6]) +
                Rm[2] * (Rm[3] * Rm[7] - Rm[4] * Rm[6]);
    const float sg = det < 0.f ? -1.f : 1.f;
    float M[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = sg * Rm[i];
    const float tr = M[0] + M[4] + M[8];
    // with t = 2 sqrt(s): 0.25 t = 0.5 s / sqrt(s) and 1 / t = 0.5 / sqrt(s),
    // from the approximate reciprocal square root (the normalisation below
    // absorbs its error)
    float x, y, z, w;
    if (tr > 0.f) {
        const float sq = tr + 1.f, h = 0.5f * rsqrtf(sq);
        w = sq * h;
        x = (M[7] - M[5]) * h;
        y = (M[2] - M[6]) * h;
        z = (M[3] - M[1]) * h;
    } else if (M[0] > M[4] && M[0] > M[8]) {
        const float sq = 1.f + M[0] - M[4] - M[8], h = 0.5f * rsqrtf(sq);
        w = (M[7] - M[5]) * h;
        x = sq * h;
        y = (M[1] + M[3]) * h;
        z = (M[2] + M[6]) * h;
    } else if (M[4] > M[8]) {
        const float sq = 1.f + M[4] - M[0] - M[8], h = 0.5f * rsqrtf(sq);
        w = (M[2] - M[6]) * h;
        x = (M[1] + M[3]) * h;
        y = sq * h;
        z = (M[5] + M[7]) * h;
    } else {
        const float sq = 1.f + M[8] - M[0] - M[4], h = 0.5f * rsqrtf(sq);
        w = (M[3] - M[1]) * h;
        x = (M[2] + M[6]) * h;
        y = (M[5] + M[7]) * h;
        z = sq * h;
    }
    const float n = rsqrtf(x * x + y * y + z * z + w * w);
    x *= n;
    y *= n;
    z *= n;
    w *= n;
    if (w < 0.f) {  // q and -q are the same rotation: keep w >= 0
        x = -x;
        y = -y;
        z = -z;
        w = -w;
    }
    if (sg < 0.f) w = -w - 2.f;  // reflection flag
    return make_float4(x, y, z, w);
}

__device__ __forceinline__ void quat_to_rot(float4 q, float Rm[9])
{
    float sg = 1.f;
    float w = q.w;
    if (w <= -1.5f) {
        sg = -1.f;
        w = -w - 2.f;
    }
    const float x = q.x, y = q.y, z = q.z;
    const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y,
                wz = w * z;
    Rm[0] = sg * (1.f - 2.f * (yy + zz));
    Rm[1] = sg * (2.f * (xy - wz));
    Rm[2] = sg * (2.f * (xz + wy));
    Rm[3] = sg * (2.f * (xy + wz));
    Rm[4] = sg * (1.f - 2.f * (xx + zz));
    Rm[5] = sg * (2.f * (yz - wx));
    Rm[6] = sg * (2.f * (xz - wy));
    Rm[7] = sg * (2.f * (yz + wx));
    Rm[8] = sg * (1.f - 2.f * (xx + yy));
}

// ---- float-float arithmetic for the mixed-precision strain ----------------
// The strain D = rest - R e is a small difference of edge-sized terms, so the
// mixed variant forms it with about 47 significant bits: values are carried
// as unevaluated sums hi + lo of two floats, built from the error-free
// transformations TwoSum (Knuth) and TwoProduct (one FMA). GB300 runs FP64
// arithmetic and FP64<->FP32 conversions at about 2 per clock per SM against
// 128 FP32 FMAs, so none of this touches the FP64 pipe.
struct ff {
    float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff two_prod(float a, float b)
{
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

// FP64 -> hi + lo floats by bit manipulation (integer pipe only): hi keeps
// the leading 24 significant bits, lo the next 23 (both truncated), so
// hi + lo equals v to 2^-47 relative. Below 2^-80 in magnitude lo is zero
// and below 2^-126 the value is flushed to zero; from 2^128 on (and for
// infinities and NaNs) the value goes through the FP64 conversion, which
// keeps non-finite states visible.
__device__ __forceinline__ ff split_f64(double v)
{
    const unsigned hw = (unsigned)__double2hiint(v);
    const unsigned lw = (unsigned)__double2loint(v);
    const int E = (int)((hw >> 20) & 0x7FFu);
    const unsigned sgn = hw & 0x80000000u;
    if ((unsigned)(E - 897) > 253u) {
        if (E < 897) return {__uint_as_float(sgn), 0.f};
        return {__double2float_rn(v), 0.f};
    }
    const unsigned mant = ((hw & 0xFFFFFu) << 3) | (lw >> 29);
    const float h = __uint_as_float(sgn | ((unsigned)(E - 896) << 23) | mant);
    // the next 23 mantissa bits as an integer r < 2^23, worth r * 2^(E - 1069)
    const unsigned r = (lw & 0x1FFFFFFFu) >> 6;
    const float rf = __uint_as_float(0x4B000000u | r) - 8388608.0f;
    const int k = E - 1069;
    const float scale = k >= -126 ? __uint_as_float((unsigned)(k + 127) << 23) : 0.f;
    const float l = rf * scale;
    return {h, sgn ? -l : l};
}

// One Newton step of the polar iteration X <- (X + X^-T) / 2 = X/2 + cof(X)
// / (2 det X) on an FP32 matrix X that is a rotation to FP32 precision; the
// result X + dX is orthonormal to about 1e-14. The cofactors and the
// determinant are formed in float-float; dX (of the size of X's rounding)
// then needs only FP32: with det = 1 + d,
// dX = (cof - X)/2 + (d^2 - d) cof / 2.
__device__ __forceinline__ void orthonormalize_ff(const float X[9], float dX[9])
{
    const int cidx[9][4] = {{4, 8, 5, 7}, {5, 6, 3, 8}, {3, 7, 4, 6}, {7, 2, 8, 1}, {8, 0, 6, 2},
                            {6, 1, 7, 0}, {1, 5, 2, 4}, {2, 3, 0, 5}, {0, 4, 1, 3}};
    ff c[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const ff p = two_prod(X[cidx[i][0]], X[cidx[i][1]]);
        const ff q = two_prod(X[cidx[i][2]], X[cidx[i][3]]);
        const ff s = two_sum(p.h, -q.h);
        c[i] = {s.h, s.l + (p.l - q.l)};
    }
    const ff t0 = two_prod(X[0], c[0].h), t1 = two_prod(X[1], c[1].h), t2 = two_prod(X[2], c[2].h);
    const ff s01 = two_sum(t0.h, t1.h);
    const ff s = two_sum(s01.h, t2.h);
    const float lo = s01.l + s.l + t0.l + t1.l + t2.l + X[0] * c[0].l + X[1] * c[1].l + X[2] * c[2].l;
    const float d = (s.h - 1.0f) + lo;  // s.h is within 2^-20 of 1: exact subtraction
    const float g = 0.5f * (d * d - d);
#pragma unroll
    for (int i = 0; i < 9; ++i) dX[i] = 0.5f * ((c[i].h - X[i]) + c[i].l) + g * c[i].h;
}

template <typename R>
__device__ __forceinline__ void load_rot(const ElemView<R>& ev, size_t e, R Rm[9])
{
    if constexpr (is_mixed<R>::value) {
        quat_to_rot(reinterpret_cast<const float4*>(ev.rot)[e], Rm);
    } else {
        const size_t En = (size_t)ev.n_tets;
#pragma unroll
        for (int i = 0; i < 9; ++i) Rm[i] = ev.rot[i * En + e];
    }
}

template <typename R>
__device__ __forceinline__ void store_rot(const ElemView<R>& ev, size_t e, const R Rm[9])
{
    if constexpr (is_mixed<R>::value) {
        reinterpret_cast<float4*>(ev.rot)[e] = rot_to_quat(Rm);
    } else {
        const size_t En = (size_t)ev.n_tets;
#pragma unroll
        for (int i = 0; i < 9; ++i) ev.rot[i * En + e] = Rm[i];
    }
}

template <typename R>
__device__ __forceinline__ void load_KJ(const ElemView<R>& ev, size_t e, R K[3], R J[12])
{
    const size_t En = (size_t)ev.n_tets;
    if constexpr (is_mixed<R>::value) {
        const float4* P = reinterpret_cast<const float4*>(ev.J);
        const float4 a = P[e], b = P[En + e], c = P[2 * En + e];
        J[3] = a.x;
        J[4] = a.y;
        J[5] = a.z;
        J[6] = a.w;
        J[7] = b.x;
        J[8] = b.y;
        J[9] = b.z;
        J[10] = b.w;
        J[11] = c.x;
        J[0] = -(J[3] + J[6] + J[9]);
        J[1] = -(J[4] + J[7] + J[10]);
        J[2] = -(J[5] + J[8] + J[11]);
        K[0] = 1.f;
        K[1] = c.y;
        K[2] = c.z;
    } else {
#pragma unroll
        for (int i = 0; i < 3; ++i) K[i] = ev.K[i * En + e];
#pragma unroll
        for (int i = 0; i < 12; ++i) J[i] = ev.J[i * En + e];
    }
}

// ------------------------------------------------------------------------
// initialisation: per-element K, J, initial rotation and rotated rest
// coordinates, computed in FP64 (computeMaterialStiffness TFEM.inl:256-291,
// initSmall/initLarge/initPolar TFEM.inl:526-532, 835-868, 993-1023) and
// stored in R.
// ------------------------------------------------------------------------
// computeMaterialStiffness (TFEM.inl:256-291) of element s (storage order;
// e its index in the caller's order): K(0,0), K(0,1), K(3,3) divided by
// 36 V, and V.
__device__ __forceinline__ void material_stiffness(const double pa[3], const double pb[3], const double pc[3],
                                                   const double pd[3], int e, int E,
                                                   const double* __restrict__ young, int n_young,
                                                   const double* __restrict__ poisson, int n_poisson,
                                                   const double* __restrict__ lsf, int n_lsf, double k[3], double* vol)
{
    // getVecRealInElement (BaseLinearElasticityFEMForceField.inl:114-132)
    double Ey = (n_young > e) ? young[e] : young[0];
    double nu = (n_poisson > e) ? poisson[e] : poisson[0];
    double f = (n_lsf > 0) ? lsf[(size_t)e * (size_t)n_lsf / (size_t)E] : 1.0;
    Ey = f * Ey;
    double sc = (Ey * (1 - nu)) / ((1 + nu) * (1 - 2 * nu));
    double k0 = 1.0, k1 = nu / (1 - nu), k2 = (1 - 2 * nu) / (2 * (1 - nu));
    k0 *= sc;
    k1 *= sc;
    k2 *= sc;
    double ea[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    double eb[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
    double ec[3] = {pd[0] - pa[0], pd[1] - pa[1], pd[2] - pa[2]};
    double cr[3];
    cross3(ea, eb, cr);
    double dt = cr[0] * ec[0];
    dt += cr[1] * ec[1];
    dt += cr[2] * ec[2];
    double v = fabs(dt / 6.0);
    *vol = v;
    k[0] = k0 / (v * 36);
    k[1] = k1 / (v * 36);
    k[2] = k2 / (v * 36);
}

template <typename R>
__global__ void k_init_elements(const double* __restrict__ rest_pos, const int4* __restrict__ tets,
                                const int* __restrict__ elem_orig, int E, int method,
                                const double* __restrict__ young, int n_young, const double* __restrict__ poisson,
                                int n_poisson, const double* __restrict__ lsf, int n_lsf, R* K, R* J, R* rest,
                                float2* rest_ff, R* rot, R* A0inv,
                                R* R0, double* vol)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= E) return;
    const int e = elem_orig[s];  // material data is indexed by the caller's element order
    const int4 t = tets[s];
    double pa[3], pb[3], pc[3], pd[3];
    ld3(rest_pos, t.x, pa);
    ld3(rest_pos, t.y, pb);
    ld3(rest_pos, t.z, pc);
    ld3(rest_pos, t.w, pd);
    double kk[3];
    material_stiffness(pa, pb, pc, pd, e, E, young, n_young, poisson, n_poisson, lsf, n_lsf, kk, &vol[s]);
    const double k0 = kk[0], k1 = kk[1], k2 = kk[2];
    double ea[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    double eb[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
    double ec[3] = {pd[0] - pa[0], pd[1] - pa[1], pd[2] - pa[2]};
    const size_t En = (size_t)E;
    K[0 * En + s] = (R)k0;
    K[1 * En + s] = (R)k1;
    K[2 * En + s] = (R)k2;

    double Jd[12], rr[12];
    double Rm[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (method == METHOD_SMALL) {
        strain_displacement(pa, pb, pc, pd, Jd);
        for (int i = 0; i < 12; ++i) rr[i] = 0.0;
    } else {
        if (method == METHOD_LARGE) {
            rotation_large(ea, eb, Rm);
        } else {
            double A[9] = {ea[0], ea[1], ea[2], eb[0], eb[1], eb[2], ec[0], ec[1], ec[2]};
            if (method == METHOD_SVD && A0inv) {
                // initSVD (TFEM.inl:1090-1119): the polar init plus the
                // inverse rest edge matrix (_initialTransformation)
                double Ai[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
                (void)invert3(A, Ai);
                for (int i = 0; i < 9; ++i) A0inv[(size_t)i * E + s] = (R)Ai[i];
            }
            polar3(A, Rm, 1000);
        }
        const double* P[4] = {pa, pb, pc, pd};
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) {
                double acc = Rm[3 * k] * P[i][0];
                acc += Rm[3 * k + 1] * P[i][1];
                acc += Rm[3 * k + 2] * P[i][2];
                rr[3 * i + k] = acc;
            }
        if (method == METHOD_LARGE) {
            for (int i = 1; i < 4; ++i)
                for (int k = 0; k < 3; ++k) rr[3 * i + k] -= rr[k];
            rr[0] = rr[1] = rr[2] = 0.0;
        }
        strain_displacement(&rr[0], &rr[3], &rr[6], &rr[9], Jd);
        if ((method == METHOD_POLAR || method == METHOD_SVD) && is_mixed<R>::value) {
            // mixed precision drops the rigid translation (J's columns sum to
            // zero): keep rest coordinates relative to node a
            for (int i = 1; i < 4; ++i)
                for (int k = 0; k < 3; ++k) rr[3 * i + k] -= rr[k];
            rr[0] = rr[1] = rr[2] = 0.0;
        }
    }
    if constexpr (is_mixed<R>::value) {
        const double sk = sqrt(k0);
        float4* P = reinterpret_cast<float4*>(J);
        P[s] = make_float4((float)(sk * Jd[3]), (float)(sk * Jd[4]), (float)(sk * Jd[5]), (float)(sk * Jd[6]));
        P[En + s] = make_float4((float)(sk * Jd[7]), (float)(sk * Jd[8]), (float)(sk * Jd[9]), (float)(sk * Jd[10]));
        P[2 * En + s] = make_float4((float)(sk * Jd[11]), (float)(k1 / k0), (float)(k2 / k0), 0.f);
        float Rf[9];
        for (int i = 0; i < 9; ++i) Rf[i] = (float)Rm[i];
        reinterpret_cast<float4*>(rot)[s] = rot_to_quat(Rf);
    } else {
        for (int i = 0; i < 12; ++i) J[(size_t)i * En + s] = (R)Jd[i];
        for (int i = 0; i < 9; ++i) rot[(size_t)i * En + s] = (R)Rm[i];
    }
    for (int i = 0; i < 12; ++i) rest[(size_t)i * En + s] = (R)rr[i];
    if (rest_ff)  // rows b-a, c-a, d-a (rr[0..2] are zero) as float-float pairs
        for (int i = 3; i < 12; ++i) {
            const float hi = (float)rr[i];
            rest_ff[(size_t)(i - 3) * En + s] = make_float2(hi, (float)(rr[i] - (double)hi));
        }
    for (int i = 0; i < 9; ++i) R0[(size_t)i * En + s] = (R)Rm[i];
}

// ------------------------------------------------------------------------
// element kernels
// ------------------------------------------------------------------------

template <typename R>
__device__ __forceinline__ void store_eforce(R* eforce, int e, const R c[12])
{
    R* o = eforce + (size_t)e * 12;
#pragma unroll
    for (int i = 0; i < 12; ++i) o[i] = c[i];
}

// The svd method's frame of element e from its stored inverse rest edge
// matrix and initial rotation (svd_frame); false: the element takes the
// polar factor of its edges, as the polar method does.
template <typename R, typename T>
__device__ __forceinline__ bool svd_frame_elem(const ElemView<R>& ev, size_t e, const T A[9], T Rout[9])
{
    const size_t En = (size_t)ev.n_tets;
    T Ai[9], R0[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        Ai[i] = (T)ev.A0inv[i * En + e];
        R0[i] = (T)ev.R0[i * En + e];
    }
    return svd_frame(A, Ai, R0, Rout);
}

// Plasticity of the addForce strain (plasticMaxThreshold > 0): per element
// six plastic strain components that every addForce call updates.
// FP64 stores the strain as the reference does; mixed precision stores it in
// the scaling of its strain-displacement values (J sqrt(K(0,0)), so J^T D is
// sqrt(K(0,0)) times the strain) and scales the thresholds by the same
// per-element factor.
template <typename R>
struct PlasticArgs {
    R* strain = nullptr;         // 6 rows x n_tets; null: plasticity off
    const R* scale = nullptr;    // mixed: sqrt(K(0,0)) per element; null for FP64
    R max_threshold = R(0), yield_threshold = R(0), creep = R(0);
    // updateStiffnessMatrix (polar, svd): the element's strain-displacement
    // values rebuilt from its deformed positions in its current frame at
    // every addForce (TFEM.inl:1063-1067, 1174-1177) and stored here (the
    // mesh's J array; mixed: scaled by `scale`); null: J stays as built
    R* update_J = nullptr;
};

// computeForce's plastic step (TFEM.inl:357-370): the elastic part of the
// strain J^T D minus the plastic strain; above the yield threshold the
// plastic strain creeps towards it, it is clamped to the maximum norm, and
// the force uses the strain minus the plastic strain.
template <typename R>
__device__ __forceinline__ void plastic_step(R jd[6], const PlasticArgs<R>& pl, size_t e, size_t En)
{
    R ps[6], el[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        ps[i] = pl.strain[i * En + e];
        el[i] = jd[i] - ps[i];
    }
    R yield = pl.yield_threshold, mx = pl.max_threshold;
    if (pl.scale) {
        const R k = pl.scale[e];
        yield = yield * k;
        mx = mx * k;
    }
    R n2 = el[0] * el[0];
#pragma unroll
    for (int i = 1; i < 6; ++i) n2 += el[i] * el[i];
    if (n2 > yield * yield) {
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const R c = el[i] * pl.creep;
            ps[i] += c;
        }
    }
    R p2 = ps[0] * ps[0];
#pragma unroll
    for (int i = 1; i < 6; ++i) p2 += ps[i] * ps[i];
    if (p2 > mx * mx) {
        const R f = mx / sqrt(p2);
#pragma unroll
        for (int i = 0; i < 6; ++i) ps[i] *= f;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        pl.strain[i * En + e] = ps[i];
        jd[i] -= ps[i];
    }
}

// computeForce of addForce (TFEM.inl:293-415), with the plastic step when
// plasticity is on.
template <typename R>
__device__ __forceinline__ void addforce_element(R F[12], const R D[12], const R K[3], const R J[12],
                                                 const PlasticArgs<R>& pl, size_t e, size_t En)
{
    R jd[6];
    strain_jtd(D, J, jd);
    if (pl.strain) plastic_step(jd, pl, e, En);
    force_from_strain(F, jd, K, J);
}

// addForce element part: accumulateForceSmall / Large / Polar
// (TFEM.inl:534-623, 870-986, 1025-1079). Writes rotations and the corner
// forces R^T F (method=small: F).
// updateStiffnessMatrix, FP32: J from the element's deformed edges in its
// frame (node a at the origin: the cofactors are translation invariant, and
// relative coordinates keep them accurate in FP32), scaled by sqrt(K(0,0))
// and packed as the init kernel packs it; J (registers) takes the new
// values, node a's as minus the sum of the others like load_KJ.
template <typename R>
__device__ __forceinline__ void update_j_mixed(const float ew[3][3], float sk, const R K[3], R J[12], R* Jout,
                                               size_t e, size_t En)
{
    if constexpr (is_mixed<R>::value) {
        const float o[3] = {0.f, 0.f, 0.f};
        float Jn[12];
        strain_displacement(o, ew[0], ew[1], ew[2], Jn);
#pragma unroll
        for (int i = 3; i < 12; ++i) J[i] = sk * Jn[i];
        J[0] = -(J[3] + J[6] + J[9]);
        J[1] = -(J[4] + J[7] + J[10]);
        J[2] = -(J[5] + J[8] + J[11]);
        float4* P = reinterpret_cast<float4*>(Jout);
        P[e] = make_float4(J[3], J[4], J[5], J[6]);
        P[En + e] = make_float4(J[7], J[8], J[9], J[10]);
        P[2 * En + e] = make_float4(J[11], K[1], K[2], 0.f);
    }
}

// The mixed strain of a rotated element (float-float rest coordinates) from
// its edges x_i - x_a (i = b, c, d) as float-float pairs: the FP32 frame
// (large: the QR frame, polar: the polar factor) from the edges' high parts,
// made orthonormal to ~1e-14 by one float-float Newton step, and D = rest -
// R e per component from TwoProducts and TwoSums, rounded once. Rm is the
// corrected frame; updateStiffnessMatrix rebuilds J (and K) from the edges
// in the element frame.
template <typename R, int METHOD>
__device__ __forceinline__ void strain_ff(const ElemView<R>& ev, int e, const ff eg[3][3], const PlasticArgs<R>& pl,
                                          R K[3], R J[12], R Rm[9], R D[12])
{
    const size_t En = (size_t)ev.n_tets;
    float X[9], dX[9];
    if (METHOD == METHOD_LARGE) {
        const float eab[3] = {eg[0][0].h, eg[0][1].h, eg[0][2].h};
        const float eac[3] = {eg[1][0].h, eg[1][1].h, eg[1][2].h};
        rotation_large_fast(eab, eac, X);
    } else {
        float A[9] = {eg[0][0].h, eg[0][1].h, eg[0][2].h, eg[1][0].h, eg[1][1].h,
                      eg[1][2].h, eg[2][0].h, eg[2][1].h, eg[2][2].h};
        if (!(METHOD == METHOD_SVD && svd_frame_elem(ev, (size_t)e, A, X))) polar3(A, X);
    }
    orthonormalize_ff(X, dX);
#pragma unroll
    for (int i = 0; i < 9; ++i) Rm[i] = X[i] + dX[i];
    D[0] = D[1] = D[2] = R(0);
    float ew[3][3];  // the edges in the element frame (updateStiffnessMatrix)
#pragma unroll
    for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float* xr = &X[3 * k];
            const float* dr = &dX[3 * k];
            const ff* ei = eg[i - 1];
            const ff t0 = two_prod(xr[0], ei[0].h), t1 = two_prod(xr[1], ei[1].h);
            const ff t2 = two_prod(xr[2], ei[2].h);
            const ff s01 = two_sum(t0.h, t1.h);
            const ff s = two_sum(s01.h, t2.h);
            float lo = s01.l + s.l + t0.l + t1.l + t2.l;
            lo += xr[0] * ei[0].l + xr[1] * ei[1].l + xr[2] * ei[2].l;
            lo += dr[0] * ei[0].h + dr[1] * ei[1].h + dr[2] * ei[2].h;
            const float2 rv = ev.rest_ff[(size_t)(3 * (i - 1) + k) * En + e];
            D[3 * i + k] = (rv.x - s.h) + (rv.y - lo);
            ew[i - 1][k] = s.h + lo;
        }
    if constexpr (METHOD == METHOD_POLAR || METHOD == METHOD_SVD)
        if (pl.update_J) update_j_mixed(ew, pl.scale[e], K, J, pl.update_J, (size_t)e, En);
}

// The corner terms R^T F of a rotated mixed element from its edges as
// float-float pairs (strain_ff), with the frame packed for the matvec;
// Rm, K and J are handed back for the right-hand side's K v terms.
template <typename R, int METHOD>
__device__ __forceinline__ void elem_force_edges(const ElemView<R>& ev, int e, const ff eg[3][3],
                                                 const PlasticArgs<R>& pl, R Rm[9], R K[3], R J[12], R c[12])
{
    const size_t En = (size_t)ev.n_tets;
    load_KJ(ev, (size_t)e, K, J);
    R D[12], F[12];
    strain_ff<R, METHOD>(ev, e, eg, pl, K, J, Rm, D);
    store_rot(ev, (size_t)e, Rm);
    addforce_element(F, D, K, J, pl, (size_t)e, En);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R acc = Rm[k] * F[3 * i];
            acc += Rm[3 + k] * F[3 * i + 1];
            acc += Rm[6 + k] * F[3 * i + 2];
            c[3 * i + k] = acc;
        }
}

// KEEP: also hands the rotation (before packing), K and J to the caller
// (rotated methods only).
template <typename R, int METHOD, bool KEEP = false>
__device__ __forceinline__ void elem_force_body(const ElemView<R>& ev, int e, const double* __restrict__ x,
                                                const double* __restrict__ rest_pos, R* __restrict__ eforce,
                                                const PlasticArgs<R>& pl = PlasticArgs<R>{}, R* keep_rot = nullptr,
                                                R* keep_K = nullptr, R* keep_J = nullptr)
{
    const size_t En = (size_t)ev.n_tets;
    const int4 t = ev.tets[e];
    double p[4][3];
    ld3(x, t.x, p[0]);
    ld3(x, t.y, p[1]);
    ld3(x, t.z, p[2]);
    ld3(x, t.w, p[3]);
    R K[3], J[12];
    load_KJ(ev, (size_t)e, K, J);
    R D[12], F[12], c[12];
    if (METHOD == METHOD_SMALL) {
        double q[4][3];
        ld3(rest_pos, t.x, q[0]);
        ld3(rest_pos, t.y, q[1]);
        ld3(rest_pos, t.z, q[2]);
        ld3(rest_pos, t.w, q[3]);
        D[0] = D[1] = D[2] = R(0);
#pragma unroll
        for (int i = 1; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) D[3 * i + k] = (R)(q[i][k] - q[0][k] - p[i][k] + p[0][k]);
        addforce_element(F, D, K, J, pl, (size_t)e, En);
#pragma unroll
        for (int i = 0; i < 12; ++i) c[i] = F[i];
        store_eforce(eforce, e, c);
        return;
    }
    R Rm[9];
    R rr[12];
#pragma unroll
    for (int i = 0; i < 12; ++i) rr[i] = ev.rest[i * En + e];
    if constexpr (!is_mixed<R>::value) {
        // FP64: the reference's formulation on absolute positions
        R eab[3] = {R(p[1][0] - p[0][0]), R(p[1][1] - p[0][1]), R(p[1][2] - p[0][2])};
        R eac[3] = {R(p[2][0] - p[0][0]), R(p[2][1] - p[0][1]), R(p[2][2] - p[0][2])};
        if (METHOD == METHOD_LARGE) {
            rotation_large(eab, eac, Rm);
        } else {
            R ead[3] = {R(p[3][0] - p[0][0]), R(p[3][1] - p[0][1]), R(p[3][2] - p[0][2])};
            R A[9] = {eab[0], eab[1], eab[2], eac[0], eac[1], eac[2], ead[0], ead[1], ead[2]};
            if (!(METHOD == METHOD_SVD && svd_frame_elem(ev, (size_t)e, A, Rm))) polar3(A, Rm);
        }
        R def[12];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                R acc = Rm[3 * k] * (R)p[i][0];
                acc += Rm[3 * k + 1] * (R)p[i][1];
                acc += Rm[3 * k + 2] * (R)p[i][2];
                def[3 * i + k] = acc;
            }
        if constexpr (METHOD == METHOD_POLAR || METHOD == METHOD_SVD) {
            // updateStiffnessMatrix: computeStrainDisplacement on the
            // deformed positions in the element frame (absolute, as the
            // reference passes them)
            if (pl.update_J) {
                strain_displacement(&def[0], &def[3], &def[6], &def[9], J);
#pragma unroll
                for (int i = 0; i < 12; ++i) pl.update_J[i * En + e] = J[i];
            }
        }
        if (METHOD == METHOD_LARGE) {
            def[3] -= def[0];
            def[6] -= def[0];
            def[7] -= def[1];
            def[9] -= def[0];
            def[10] -= def[1];
            def[11] -= def[2];
            D[0] = D[1] = D[2] = D[4] = D[5] = D[8] = R(0);
            D[3] = rr[3] - def[3];
            D[6] = rr[6] - def[6];
            D[7] = rr[7] - def[7];
            D[9] = rr[9] - def[9];
            D[10] = rr[10] - def[10];
            D[11] = rr[11] - def[11];
        } else {
#pragma unroll
            for (int i = 0; i < 12; ++i) D[i] = rr[i] - def[i];
        }
    } else {
        if (ev.rest_ff) {
            // mixed: D = rest - R e is a small difference of edge-sized terms,
            // formed in float-float (about 47 bits) from the FP64 edges and
            // float-float rest coordinates. R is the FP32 frame (large: the QR
            // frame, polar: the polar factor) made orthonormal to ~1e-14 by one
            // float-float Newton step. A residual error of R that is a rotation
            // adds no first-order strain, so all nine components of D are
            // computed (for large the reference's zero components D[4], D[5],
            // D[8] come out at that rotation's size instead of being forced to
            // zero, which would leave them inconsistent with R); a
            // non-orthonormal R would add strain noise of the size of the
            // edges' FP32 rounding, on stiff, lightly loaded meshes as large as
            // the load itself.
            // edges: one FP64 subtraction each (exact to the edge's own
            // rounding, however far the mesh is from the origin), then split
            ff eg[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) eg[i][k] = split_f64(p[i + 1][k] - p[0][k]);
            strain_ff<R, METHOD>(ev, e, eg, pl, K, J, Rm, D);
        } else {
            // mixed without float-float rest coordinates: edges formed in FP64
            // and rounded once, the strain in FP32 on positions relative to node a
            R ed[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) ed[i][k] = (R)(p[i + 1][k] - p[0][k]);
            if (METHOD == METHOD_LARGE) {
                rotation_large(ed[0], ed[1], Rm);
            } else {
                R A[9] = {ed[0][0], ed[0][1], ed[0][2], ed[1][0], ed[1][1], ed[1][2], ed[2][0], ed[2][1], ed[2][2]};
                if (!(METHOD == METHOD_SVD && svd_frame_elem(ev, (size_t)e, A, Rm))) polar3(A, Rm);
            }
            D[0] = D[1] = D[2] = R(0);
            float ew[3][3];  // the edges in the element frame (updateStiffnessMatrix)
#pragma unroll
            for (int i = 1; i < 4; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    R d = Rm[3 * k] * ed[i - 1][0] + Rm[3 * k + 1] * ed[i - 1][1] + Rm[3 * k + 2] * ed[i - 1][2];
                    D[3 * i + k] = rr[3 * i + k] - d;
                    ew[i - 1][k] = (float)d;
                }
            if (METHOD == METHOD_LARGE) D[4] = D[5] = D[8] = R(0);
            if constexpr (METHOD == METHOD_POLAR || METHOD == METHOD_SVD)
                if (pl.update_J) update_j_mixed(ew, pl.scale[e], K, J, pl.update_J, (size_t)e, En);
        }
    }
    store_rot(ev, (size_t)e, Rm);
    addforce_element(F, D, K, J, pl, (size_t)e, En);
    // f[node] += rotations[e] * F_node, rotations[e] = R^T
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R acc = Rm[k] * F[3 * i];
            acc += Rm[3 + k] * F[3 * i + 1];
            acc += Rm[6 + k] * F[3 * i + 2];
            c[3 * i + k] = acc;
        }
    store_eforce(eforce, e, c);
    if constexpr (KEEP) {
#pragma unroll
        for (int i = 0; i < 9; ++i) keep_rot[i] = Rm[i];
#pragma unroll
        for (int i = 0; i < 3; ++i) keep_K[i] = K[i];
#pragma unroll
        for (int i = 0; i < 12; ++i) keep_J[i] = J[i];
    }
}

template <typename R, int METHOD>
__global__ void __launch_bounds__(kElemBlock) k_elem_force(ElemView<R> ev, const double* __restrict__ x,
                                                           const double* __restrict__ rest_pos,
                                                           R* __restrict__ eforce, PlasticArgs<R> pl)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ev.n_tets) return;
    elem_force_body<R, METHOD>(ev, e, x, rest_pos, eforce, pl);
}

// Direction of the CG step for the matvec element pass. DIR 0: the input
// vector itself; DIR 1: p = r (first iteration); DIR 2: p = p_old*beta + r
// (vOp_avf, Sofa/Component/StateContainer/src/sofa/component/statecontainer/
// MechanicalObject.inl:1999-2013).
template <typename R>
__device__ __forceinline__ R cg_dir(R r, R pold, R beta)
{
    R t = pold * beta;
    return t + r;
}

// addDForce element inputs: the four nodes' values of dx (DIR 0), of the
// CG direction p = r (DIR 1) or p = p_old*beta + r (DIR 2).
template <typename R, typename VIN, int METHOD, int DIR, int PC = 0>
__device__ __forceinline__ void dforce_inputs(const int node[4], const VIN* __restrict__ dx,
                                              const R* __restrict__ pold, R beta, const R* __restrict__ dinv,
                                              R xin[4][3])
{
    VIN v0[3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        VIN v3[3];
        ld3(dx, node[i], v3);
        if constexpr (PC != 0 && DIR != 0) {
            // PCG: the direction is built from z = diag^-1 r (Jacobi)
            R dv[3];
            ld3(dinv, node[i], dv);
#pragma unroll
            for (int k = 0; k < 3; ++k) v3[k] = (VIN)(dv[k] * (R)v3[k]);
        }
        if (DIR == 2) {
            R po[3];
            ld3(pold, node[i], po);
#pragma unroll
            for (int k = 0; k < 3; ++k) xin[i][k] = cg_dir((R)v3[k], po[k], beta);
        } else if (is_mixed<R>::value && !std::is_same<VIN, R>::value) {
            // FP64 input (velocities): form the differences to node a in
            // FP64 before rounding to FP32
            if (i == 0) {
#pragma unroll
                for (int k = 0; k < 3; ++k) v0[k] = v3[k];
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) xin[i][k] = (R)(v3[k] - v0[k]);
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) xin[i][k] = (R)v3[k];
        }
    }
    if (is_mixed<R>::value && METHOD != METHOD_SMALL) {
        // FP32: J^T annihilates rigid translations (each column of J sums to
        // zero over the four nodes), so work on values relative to node a;
        // smooth CG directions then keep their strain bits
#pragma unroll
        for (int i = 3; i >= 0; --i)
#pragma unroll
            for (int k = 0; k < 3; ++k) xin[i][k] -= xin[0][k];
    }
}

// addDForce corner terms of one element from its inputs:
// applyStiffnessSmall / applyStiffnessCorotational (TFEM.inl:721-749,
// 1193-1237), c = R K (R^T x) fact, which the gather subtracts. Rm is
// unused for method small.
template <typename R, int METHOD>
__device__ __forceinline__ void dforce_terms(const R xin[4][3], const R Rm[9], const R K[3], const R J[12], R fact,
                                             R c[12])
{
    R X[12], F[12];
    if (METHOD == METHOD_SMALL) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) X[3 * i + k] = xin[i][k];
        element_force(F, X, K, J, fact);
#pragma unroll
        for (int i = 0; i < 12; ++i) c[i] = F[i];
        return;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R acc = Rm[3 * k] * xin[i][0];
            acc += Rm[3 * k + 1] * xin[i][1];
            acc += Rm[3 * k + 2] * xin[i][2];
            X[3 * i + k] = acc;
        }
    element_force(F, X, K, J, fact);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R acc = Rm[k] * F[3 * i];
            acc += Rm[3 + k] * F[3 * i + 1];
            acc += Rm[6 + k] * F[3 * i + 2];
            c[3 * i + k] = acc;
        }
}

// addDForce element part: the inputs, the element's stored rotation and
// stiffness, the corner terms into eforce.
template <typename R, typename VIN, int METHOD, int DIR, int PC = 0>
__device__ __forceinline__ void elem_dforce_body(const ElemView<R>& ev, int e, const VIN* __restrict__ dx,
                                                 const R* __restrict__ pold, R beta, R fact,
                                                 R* __restrict__ eforce, const R* __restrict__ dinv = nullptr)
{
    const int4 t = ev.tets[e];
    const int node[4] = {t.x, t.y, t.z, t.w};
    R xin[4][3];
    dforce_inputs<R, VIN, METHOD, DIR, PC>(node, dx, pold, beta, dinv, xin);
    R K[3], J[12], Rm[9], c[12];
    load_KJ(ev, (size_t)e, K, J);
    if (METHOD != METHOD_SMALL) load_rot(ev, (size_t)e, Rm);
    dforce_terms<R, METHOD>(xin, Rm, K, J, fact, c);
    store_eforce(eforce, e, c);
}

template <typename R, typename VIN, int METHOD, int DIR, int PC = 0>
__global__ void __launch_bounds__(kElemBlock) k_elem_dforce(ElemView<R> ev, const VIN* __restrict__ dx,
                                                            const R* __restrict__ pold, const CgScalars* cg,
                                                            R fact, R* __restrict__ eforce,
                                                            const R* __restrict__ dinv)
{
    if (DIR != 0 && cg->done) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ev.n_tets) return;
    const R beta = (DIR == 2) ? (R)cg->beta : R(0);
    elem_dforce_body<R, VIN, METHOD, DIR, PC>(ev, e, dx, pold, beta, fact, eforce, dinv);
}

// The right-hand side's (h + rs) K v corner terms of element e (rotated
// methods) from the rotation elem_force_body formed (Rm, before packing) and
// its K, J: the rotation as the packed copy gives it back, then the
// operations of elem_dforce_body on the FP64 velocities.
template <typename R>
__device__ __forceinline__ void rhs_v_terms_c(const ElemView<R>& ev, int e, const double* __restrict__ v,
                                              const R Rm[9], const R K[3], const R J[12], R kf_rhs, R c[12])
{
    R Rq[9];
    if constexpr (is_mixed<R>::value) {
        quat_to_rot(rot_to_quat(Rm), Rq);
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) Rq[i] = Rm[i];
    }
    const int4 t = ev.tets[e];
    const int node[4] = {t.x, t.y, t.z, t.w};
    R xin[4][3];
    dforce_inputs<R, double, METHOD_LARGE, 0>(node, v, nullptr, R(0), nullptr, xin);
    dforce_terms<R, METHOD_LARGE>(xin, Rq, K, J, kf_rhs, c);
}

template <typename R>
__device__ __forceinline__ void rhs_v_terms(const ElemView<R>& ev, int e, const double* __restrict__ v,
                                            const R Rm[9], const R K[3], const R J[12], R kf_rhs,
                                            R* __restrict__ eforce_v)
{
    R c[12];
    rhs_v_terms_c(ev, e, v, Rm, K, J, kf_rhs, c);
    store_eforce(eforce_v, e, c);
}

// addForce and the right-hand side's stiffness term of one implicit step in
// one pass over the elements (rotated methods): the force corner terms as
// k_elem_force forms them into eforce, then the terms (h + rs) K v of
// EulerImplicitSolver's right-hand side (EulerImplicitSolver.cpp:137-160) into
// eforce_v, with the rotation as the stored copy gives it back and K, J from
// registers; the values are those of k_elem_force followed by k_elem_dforce
// on v.
template <typename R, int METHOD>
__global__ void __launch_bounds__(kElemBlock) k_elem_force_rhs(ElemView<R> ev, const double* __restrict__ x,
                                                               const double* __restrict__ rest_pos,
                                                               R* __restrict__ eforce, PlasticArgs<R> pl,
                                                               const double* __restrict__ v, R kf_rhs,
                                                               R* __restrict__ eforce_v)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ev.n_tets) return;
    R Rm[9], K[3], J[12];
    elem_force_body<R, METHOD, true>(ev, e, x, rest_pos, eforce, pl, Rm, K, J);
    rhs_v_terms(ev, e, v, Rm, K, J, kf_rhs, eforce_v);
}

// ------------------------------------------------------------------------
// node-centric gathers
// ------------------------------------------------------------------------

// out[n] += sum (ADD) or out[n] -= each term (SUB), terms in element order:
// the reference's serial scatter, restated per node.
template <typename R, typename VO, bool SUB>
__global__ void __launch_bounds__(kNodeBlock) k_gather_accumulate(NodeCSR csr, const R* __restrict__ eforce,
                                                                  VO* __restrict__ out, int N)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R a0 = (R)out[3 * (size_t)n], a1 = (R)out[3 * (size_t)n + 1], a2 = (R)out[3 * (size_t)n + 2];
        const int s0 = csr.rowptr[n], s1 = csr.rowptr[n + 1];
        for (int s = s0; s < s1; ++s) {
            const R* c = eforce + 3 * (size_t)csr.slots[s];
            if (SUB) {
                a0 -= c[0];
                a1 -= c[1];
                a2 -= c[2];
            } else {
                a0 += c[0];
                a1 += c[1];
                a2 += c[2];
            }
        }
        out[3 * (size_t)n] = (VO)a0;
        out[3 * (size_t)n + 1] = (VO)a1;
        out[3 * (size_t)n + 2] = (VO)a2;
    }
}

// ---- deterministic dot products -----------------------------------------

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block in a fixed tree; the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double red[kNodeBlock / 32];
    __syncthreads();
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Vec3 dot in the reference order ((x x' + y y') + z z'), FP64.
template <typename A, typename B>
__device__ __forceinline__ double dot3(const A a[3], const B b[3])
{
    double r = (double)a[0] * (double)b[0];
    r += (double)a[1] * (double)b[1];
    r += (double)a[2] * (double)b[2];
    return r;
}

enum Finish {
    FIN_RHS = 0,
    FIN_DEN = 1,
    FIN_RHO = 2,
    FIN_REPLACE = 3,
    FIN_PCG_START = 4,
    FIN_WARM_START = 5,
    FIN_RESIDUAL = 6
};

struct SolveConsts {
    double tol, threshold;
    int it;   // CG iteration this kernel belongs to (1-based)
    int pcg;  // 1: PCGLinearSolver bookkeeping (r.z, tolerance * b.b, no threshold test)
    int warm; // 1: CG warmStart (the solve starts from the previous solution)
    int replace_every = 0;  // residual replacement: check every this many iterations (0: off)
};

// Residual replacement condition (van der Vorst and Ye, SIAM J. Sci. Comput.
// 22(3), 2000, with their epsilon-hat = sqrt(u) for the FP32 unit roundoff
// u = 2^-24): the residual is recomputed in FP64 only once the recurrence
// residual has fallen below kReplaceEps times its largest norm since the
// last replacement (the drift between recurrence and true residual then
// matters), or when the recurrence says the solve has converged (the true
// residual decides). A solve whose residual does not decrease -- a truncated
// solve of a badly conditioned system -- is left to the FP32 recurrence, so
// a replacement never perturbs a Krylov sequence that is still far from
// converged.
constexpr double kReplaceEps = 1.0 / 4096.0;

// Last-block finish of a dot product: every block writes its partial; the
// last block to arrive (integer ticket) adds the partials in block order and
// applies the CG bookkeeping of CGLinearSolver::solve
// (Sofa/Component/LinearSolver/Iterative/src/sofa/component/linearsolver/
// iterative/CGLinearSolver.inl:102-272). With `terms` non-null the sum is
// instead the serial node-order sum of per-node terms, as MechanicalObject::vDot
// (MechanicalObject.inl:2334-2356) computes it.
template <int FIN>
__device__ void finish_dot(double local, CgScalars* cg, const double* terms, int N, SolveConsts sc)
{
    __shared__ int is_last;
    double bsum = block_sum(local);
    if (threadIdx.x == 0) {
        cg->partials[blockIdx.x] = bsum;
        __threadfence();
        unsigned t = atomicAdd(&cg->ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double total;
    if (terms) {
        total = 0.0;
        if (threadIdx.x == 0)
            for (int i = 0; i < N; ++i) total += __ldcg(&terms[i]);
    } else {
        double v = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) v += __ldcg(&cg->partials[i]);
        total = block_sum(v);
    }
    if (threadIdx.x != 0) return;
    cg->ticket = 0;
    if (FIN == FIN_RESIDUAL) {  // the Data `residual` only; the solve is over
        cg->residual = total;
        return;
    }
    if (!isfinite(total)) {
        cg->status |= 1;
        cg->done = 1;
        return;
    }
    const bool first_of_first = (sc.it == 1 && cg->time_step_count == 0);
    if (sc.pcg) {
        // PCGLinearSolver::solve (PCGLinearSolver.inl:194-262): r_norm = r.z,
        // tol = tolerance * b.b, loop while r_norm > tol, no threshold test
        const double bb = cg->bnorm2;
        if (FIN == FIN_RHS) {
            cg->bnorm2 = total;
            cg->normb = sqrt(total);
            cg->iters = 0;
            cg->last_err = 0.0;
            cg->done = 0;
        } else if (FIN == FIN_PCG_START) {
            cg->rho = total;
            cg->last_err = bb != 0.0 ? total / bb : 0.0;
            cg->done = (total > sc.tol * bb) ? 0 : 1;
        } else if (FIN == FIN_DEN) {
            cg->den = total;
            if (total != 0.0)
                cg->alpha = cg->rho / total;
            else
                cg->done = 1;
        } else if (FIN == FIN_RHO) {
            cg->rho_prev = cg->rho;
            cg->rho = total;
            cg->iters = sc.it;
            cg->beta = total / cg->rho_prev;
            cg->last_err = bb != 0.0 ? total / bb : 0.0;
            cg->done = (total > sc.tol * bb) ? 0 : 1;
        }
        return;
    }
    if (FIN == FIN_RHS) {
        // x = 0; r = b; normb = |b|; iteration 1 starts with rho = r.r
        cg->rho = total;
        cg->normb = sqrt(total);
        cg->iters = 0;
        cg->last_err = 0.0;
        cg->rmax = sqrt(total);
        cg->replace_it = 0;
        if (cg->normb == 0.0) {
            cg->done = 1;
        } else {
            double err = sqrt(total) / cg->normb;
            cg->last_err = err;
            cg->done = (err <= sc.tol && !first_of_first) ? 1 : 0;
        }
    } else if (FIN == FIN_DEN) {
        // a break here comes after iteration sc.it's matvec: the iteration
        // count is that of the matvecs run (the update is skipped)
        cg->den = total;
        if (total != 0.0) {
            if (fabs(total) <= sc.threshold && !first_of_first) {
                cg->done = 1;
                cg->iters = sc.it;
            } else {
                cg->alpha = cg->rho / total;
            }
        } else {
            cg->done = 1;
            cg->iters = sc.it;
        }
    } else if (FIN == FIN_RHO) {
        cg->rho_prev = cg->rho;
        cg->rho = total;
        cg->iters = sc.it;
        cg->beta = total / cg->rho_prev;
        double err = sqrt(total) / cg->normb;
        cg->last_err = err;
        if (sc.replace_every > 0) {
            const double nr = sqrt(total);
            if (nr > cg->rmax) cg->rmax = nr;
            if (sc.it % sc.replace_every == 0 && (nr <= kReplaceEps * cg->rmax || err <= sc.tol))
                cg->replace_it = sc.it;
        }
        if (err <= sc.tol) cg->done = 1;
    } else if (FIN == FIN_WARM_START) {
        // warmStart (CGLinearSolver.inl:95-99): r = b - A x; iteration 1
        // starts with rho = r.r; b = 0 runs no iteration and keeps x
        if (cg->normb != 0.0) {
            cg->rho = total;
            double err = sqrt(total) / cg->normb;
            cg->last_err = err;
            cg->done = (err <= sc.tol && !first_of_first) ? 1 : 0;
        }
    } else {
        // residual replacement after the update of iteration sc.it: the true
        // residual's r.r replaces the recurrence's, for beta and for the
        // stopping test (which may now continue a solve the recurrence ended)
        cg->rho = total;
        cg->beta = total / cg->rho_prev;
        double err = sqrt(total) / cg->normb;
        cg->last_err = err;
        cg->done = (err <= sc.tol) ? 1 : 0;
        cg->rmax = sqrt(total);
    }
}

struct MassArgs {
    const double* node_mass;  // per-node masses, or null for a uniform vertex mass
    double vertex_mass;
    double g[3];
};

// computeForce of the scene (MappingGraphMechanicalOperations.cpp:41-92):
// f = ext + (mass m g and FEM forces in component order).
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_gather_force(NodeCSR csr, const R* __restrict__ eforce,
                                                             const R* __restrict__ ext, MassArgs ma,
                                                             int mass_first, R* __restrict__ f, int N)
{
    // UniformMass::addForce: mg = g * vertexMass (UniformMass.inl:471-496)
    const R mg0 = (R)(ma.g[0] * ma.vertex_mass), mg1 = (R)(ma.g[1] * ma.vertex_mass),
            mg2 = (R)(ma.g[2] * ma.vertex_mass);
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R a0 = R(0), a1 = R(0), a2 = R(0);
        if (ext) {
            a0 += ext[3 * (size_t)n];
            a1 += ext[3 * (size_t)n + 1];
            a2 += ext[3 * (size_t)n + 2];
        }
        R m0 = mg0, m1 = mg1, m2 = mg2;
        if (ma.node_mass) {
            const double m = ma.node_mass[n];
            m0 = (R)(ma.g[0] * m);
            m1 = (R)(ma.g[1] * m);
            m2 = (R)(ma.g[2] * m);
        }
        if (mass_first) {
            a0 += m0;
            a1 += m1;
            a2 += m2;
        }
        const int s0 = csr.rowptr[n], s1 = csr.rowptr[n + 1];
        for (int s = s0; s < s1; ++s) {
            const R* c = eforce + 3 * (size_t)csr.slots[s];
            a0 += c[0];
            a1 += c[1];
            a2 += c[2];
        }
        if (!mass_first) {
            a0 += m0;
            a1 += m1;
            a2 += m2;
        }
        f[3 * (size_t)n] = a0;
        f[3 * (size_t)n + 1] = a1;
        f[3 * (size_t)n + 2] = a2;
    }
}

// res += factor M dx for one node (UniformMass::addMDx UniformMass.inl:403-419,
// DiagonalMass::addMDx DiagonalMass.inl:536-559).
template <typename R>
__device__ __forceinline__ void add_mdx(R a[3], const R d[3], const MassArgs& ma, double factor, R mm_uniform, int n)
{
    if (ma.node_mass) {
        const R m = (R)ma.node_mass[n];
        if (factor == 1.0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] += d[k] * m;
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] += (d[k] * m) * (R)factor;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; ++k) a[k] += d[k] * mm_uniform;
    }
}

// Right-hand side of EulerImplicitSolver (EulerImplicitSolver.cpp:130-163):
// b = h (f + (-rm M + (h+rs) K) v), projected; then the CG start r = b,
// x = 0 and the dot b.b.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_gather_rhs(NodeCSR csr, const R* __restrict__ eforce,
                                                           const R* __restrict__ f, const double* __restrict__ v,
                                                           MassArgs ma, double mfac, int mass_first, double h,
                                                           const uint8_t* __restrict__ fixed, R* __restrict__ b,
                                                           R* __restrict__ r, R* __restrict__ xs, CgScalars* cg,
                                                           double* terms, int N, SolveConsts sc, int first_order = 0)
{
    const R mm = (R)(mfac != 1.0 ? ma.vertex_mass * mfac : ma.vertex_mass);
    const R hr = (R)h;
    double local = 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) cg->done = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R a[3] = {f[3 * (size_t)n], f[3 * (size_t)n + 1], f[3 * (size_t)n + 2]};
        if (!first_order) {
            // b = h (f + (-rm M + (h + rs) K) v); firstOrder: b = f
            // (EulerImplicitSolver.cpp:137-160)
            R vv[3] = {(R)v[3 * (size_t)n], (R)v[3 * (size_t)n + 1], (R)v[3 * (size_t)n + 2]};
            if (mass_first && mfac != 0.0) add_mdx(a, vv, ma, mfac, mm, n);
            const int s0 = csr.rowptr[n], s1 = csr.rowptr[n + 1];
            for (int s = s0; s < s1; ++s) {
                const R* c = eforce + 3 * (size_t)csr.slots[s];
                a[0] -= c[0];
                a[1] -= c[1];
                a[2] -= c[2];
            }
            if (!mass_first && mfac != 0.0) add_mdx(a, vv, ma, mfac, mm, n);
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] *= hr;
        }
        if (fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            b[3 * (size_t)n + k] = a[k];
            r[3 * (size_t)n + k] = a[k];
            if (!sc.pcg && !sc.warm) xs[3 * (size_t)n + k] = R(0);  // PCG / warmStart keep the previous solution
        }
        double d = dot3(a, a);
        if (terms) terms[n] = d;
        local += d;
    }
    finish_dot<FIN_RHS>(local, cg, terms, N, sc);
}

// computeForce and the right-hand side in one pass over the nodes, with the
// operations of k_gather_force followed by k_gather_rhs (f stays in
// registers): eforce holds the force corner terms, eforce_v the (h + rs) K v
// terms (unused with firstOrder).
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_gather_force_rhs(NodeCSR csr, const R* __restrict__ eforce,
                                                                 const R* __restrict__ eforce_v,
                                                                 const R* __restrict__ ext,
                                                                 const double* __restrict__ v, MassArgs ma,
                                                                 double mfac, int mass_first, double h,
                                                                 const uint8_t* __restrict__ fixed,
                                                                 R* __restrict__ b, R* __restrict__ r,
                                                                 R* __restrict__ xs, CgScalars* cg, int N,
                                                                 SolveConsts sc, int first_order)
{
    const R mg0 = (R)(ma.g[0] * ma.vertex_mass), mg1 = (R)(ma.g[1] * ma.vertex_mass),
            mg2 = (R)(ma.g[2] * ma.vertex_mass);
    const R mm = (R)(mfac != 1.0 ? ma.vertex_mass * mfac : ma.vertex_mass);
    const R hr = (R)h;
    double local = 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) cg->done = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R a0 = R(0), a1 = R(0), a2 = R(0);
        if (ext) {
            a0 += ext[3 * (size_t)n];
            a1 += ext[3 * (size_t)n + 1];
            a2 += ext[3 * (size_t)n + 2];
        }
        R m0 = mg0, m1 = mg1, m2 = mg2;
        if (ma.node_mass) {
            const double m = ma.node_mass[n];
            m0 = (R)(ma.g[0] * m);
            m1 = (R)(ma.g[1] * m);
            m2 = (R)(ma.g[2] * m);
        }
        if (mass_first) {
            a0 += m0;
            a1 += m1;
            a2 += m2;
        }
        const int s0 = csr.rowptr[n], s1 = csr.rowptr[n + 1];
        for (int s = s0; s < s1; ++s) {
            const R* c = eforce + 3 * (size_t)csr.slots[s];
            a0 += c[0];
            a1 += c[1];
            a2 += c[2];
        }
        if (!mass_first) {
            a0 += m0;
            a1 += m1;
            a2 += m2;
        }
        R a[3] = {a0, a1, a2};
        if (!first_order) {
            R vv[3] = {(R)v[3 * (size_t)n], (R)v[3 * (size_t)n + 1], (R)v[3 * (size_t)n + 2]};
            if (mass_first && mfac != 0.0) add_mdx(a, vv, ma, mfac, mm, n);
            for (int s = s0; s < s1; ++s) {
                const R* c = eforce_v + 3 * (size_t)csr.slots[s];
                a[0] -= c[0];
                a[1] -= c[1];
                a[2] -= c[2];
            }
            if (!mass_first && mfac != 0.0) add_mdx(a, vv, ma, mfac, mm, n);
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] *= hr;
        }
        if (fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            b[3 * (size_t)n + k] = a[k];
            r[3 * (size_t)n + k] = a[k];
            if (!sc.pcg && !sc.warm) xs[3 * (size_t)n + k] = R(0);  // PCG / warmStart keep the previous solution
        }
        local += dot3(a, a);
    }
    finish_dot<FIN_RHS>(local, cg, nullptr, N, sc);
}

// q = A p for GraphScatteredMatrix::apply (GraphScatteredTypes.cpp:33-45):
// q = mF M p - (K p terms), projected; also stores the direction p and
// the dot p.q.
template <typename R, int DIR, int PC = 0>
__global__ void __launch_bounds__(kNodeBlock) k_gather_matvec(NodeCSR csr, const R* __restrict__ eforce,
                                                              const R* __restrict__ r, R* __restrict__ p,
                                                              MassArgs ma, double mf, int mass_first,
                                                              const uint8_t* __restrict__ fixed,
                                                              R* __restrict__ q, CgScalars* cg, double* terms,
                                                              int N, SolveConsts sc,
                                                              const R* __restrict__ dinv = nullptr)
{
    if (cg->done) return;
    const R mm = (R)(mf != 1.0 ? ma.vertex_mass * mf : ma.vertex_mass);
    const R beta = (DIR == 2) ? (R)cg->beta : R(0);
    double local = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R pp[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R rv = r[3 * (size_t)n + k];
            if constexpr (PC != 0) rv = dinv[3 * (size_t)n + k] * rv;  // PCG: z = diag^-1 r
            pp[k] = (DIR == 2) ? cg_dir(rv, p[3 * (size_t)n + k], beta) : rv;
        }
        R a[3] = {R(0), R(0), R(0)};
        if (mass_first) add_mdx(a, pp, ma, mf, mm, n);
        const int s0 = csr.rowptr[n], s1 = csr.rowptr[n + 1];
        for (int s = s0; s < s1; ++s) {
            const R* c = eforce + 3 * (size_t)csr.slots[s];
            a[0] -= c[0];
            a[1] -= c[1];
            a[2] -= c[2];
        }
        if (!mass_first) add_mdx(a, pp, ma, mf, mm, n);
        if (fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            p[3 * (size_t)n + k] = pp[k];
            q[3 * (size_t)n + k] = a[k];
        }
        double d = dot3(pp, a);
        if (terms) terms[n] = d;
        local += d;
    }
    finish_dot<FIN_DEN>(local, cg, terms, N, sc);
}

// cgstep_alpha (CGLinearSolver.cpp:47-63): x += alpha p; r += -alpha q; then
// rho = r.r for the next iteration.
template <typename R, int PC = 0>
__global__ void __launch_bounds__(kNodeBlock) k_cg_update(R* __restrict__ xs, R* __restrict__ r,
                                                          const R* __restrict__ p, const R* __restrict__ q,
                                                          CgScalars* cg, double* terms, int N, SolveConsts sc,
                                                          const R* __restrict__ dinv = nullptr)
{
    if (cg->done) return;
    const R alpha = (R)cg->alpha;
    const R nalpha = -alpha;
    double local = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R rr[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const size_t i = 3 * (size_t)n + k;
            R t = p[i] * alpha;
            xs[i] = xs[i] + t;
            R u = q[i] * nalpha;
            rr[k] = r[i] + u;
            r[i] = rr[k];
        }
        double d;
        if constexpr (PC != 0) {
            R zz[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) zz[k] = dinv[3 * (size_t)n + k] * rr[k];
            d = dot3(rr, zz);
        } else {
            d = dot3(rr, rr);
        }
        if (terms) terms[n] = d;
        local += d;
    }
    finish_dot<FIN_RHO>(local, cg, terms, N, sc);
}

// ---- PCGLinearSolver with the Jacobi preconditioner ------------------------
// (PCGLinearSolver.inl:194-262, JacobiPreconditioner.inl:41-51) on the
// element-order kernels.

// Jacobi diagonal, element part: for node i of element e the diagonal of
// R^T S R, S = B_i^T C B_i its 3x3 stiffness block (B_i from the node's
// strain-displacement values, C the isotropic material matrix), times -kF:
// the element's contribution to diag(mF M + kF K).
template <typename R, int METHOD>
__global__ void __launch_bounds__(kElemBlock) k_elem_jacobi(ElemView<R> ev, R nkf, R* __restrict__ eforce,
                                                             const CgScalars* cg, int rate)
{
    if (cg->time_step_count % rate != 0) return;  // assembled on the first step and every `rate` steps
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ev.n_tets) return;
    R K[3], J[12], Rm[9];
    load_KJ(ev, (size_t)e, K, J);
    if (METHOD == METHOD_SMALL) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Rm[i] = (i % 4 == 0) ? R(1) : R(0);
    } else {
        load_rot(ev, (size_t)e, Rm);
    }
    const R k0 = K[0], k1 = K[1], k2 = K[2], k12 = k1 + k2;
    R c[12];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const R a = J[3 * i], b = J[3 * i + 1], cc = J[3 * i + 2];
        const R S[9] = {a * a * k0 + b * b * k2 + cc * cc * k2, a * b * k12, a * cc * k12,
                        a * b * k12, b * b * k0 + a * a * k2 + cc * cc * k2, b * cc * k12,
                        a * cc * k12, b * cc * k12, cc * cc * k0 + b * b * k2 + a * a * k2};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R acc = R(0);
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                const R sr = S[3 * p] * Rm[k] + S[3 * p + 1] * Rm[3 + k] + S[3 * p + 2] * Rm[6 + k];
                acc += Rm[3 * p + k] * sr;
            }
            c[3 * i + k] = nkf * acc;
        }
    }
    store_eforce(eforce, e, c);
}

// Jacobi diagonal, node part: dinv = 1 / (mF m + element terms in element
// order; mass first or last as in the node), fixed DOFs one.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_gather_jacobi(NodeCSR csr, const R* __restrict__ eforce, MassArgs ma,
                                                              double mf, int mass_first,
                                                              const uint8_t* __restrict__ fixed,
                                                              R* __restrict__ dinv, int N, const CgScalars* cg,
                                                              int rate)
{
    if (cg->time_step_count % rate != 0) return;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const R mm = (R)((ma.node_mass ? ma.node_mass[n] : ma.vertex_mass) * mf);
        R d[3] = {R(0), R(0), R(0)};
        if (mass_first)
#pragma unroll
            for (int k = 0; k < 3; ++k) d[k] += mm;
        for (int s = csr.rowptr[n]; s < csr.rowptr[n + 1]; ++s) {
            const R* c = eforce + 3 * (size_t)csr.slots[s];
            d[0] += c[0];
            d[1] += c[1];
            d[2] += c[2];
        }
        if (!mass_first)
#pragma unroll
            for (int k = 0; k < 3; ++k) d[k] += mm;
#pragma unroll
        for (int k = 0; k < 3; ++k) dinv[3 * (size_t)n + k] = fixed[n] ? R(1) : R(1) / d[k];
    }
}

// PCG start: r = b - A x with x the previous step's solution (its K terms
// in eforce), z = diag^-1 r (or r), r.z; FIN_WARM_START: the same start for
// CG with warmStart (r.r).
template <typename R, int FIN = FIN_PCG_START>
__global__ void __launch_bounds__(kNodeBlock) k_pcg_start(NodeCSR csr, const R* __restrict__ eforce,
                                                          const R* __restrict__ xs, const R* __restrict__ b,
                                                          MassArgs ma, double mf, int mass_first,
                                                          const uint8_t* __restrict__ fixed,
                                                          const R* __restrict__ dinv, R* __restrict__ r,
                                                          CgScalars* cg, double* terms, int N, SolveConsts sc)
{
    const R mm = (R)(mf != 1.0 ? ma.vertex_mass * mf : ma.vertex_mass);
    double local = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        R pp[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) pp[k] = xs[3 * (size_t)n + k];
        R a[3] = {R(0), R(0), R(0)};
        if (mass_first) add_mdx(a, pp, ma, mf, mm, n);
        for (int s = csr.rowptr[n]; s < csr.rowptr[n + 1]; ++s) {
            const R* c = eforce + 3 * (size_t)csr.slots[s];
            a[0] -= c[0];
            a[1] -= c[1];
            a[2] -= c[2];
        }
        if (!mass_first) add_mdx(a, pp, ma, mf, mm, n);
        if (fixed[n]) a[0] = a[1] = a[2] = R(0);
        R rr[3], z[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const size_t i = 3 * (size_t)n + k;
            R t = a[k] * R(-1);  // r = b + (A x) * -1 (vOp_avf)
            rr[k] = t + b[i];
            r[i] = rr[k];
            z[k] = dinv ? dinv[i] * rr[k] : rr[k];
        }
        double d = dot3(rr, z);
        if (terms) terms[n] = d;
        local += d;
    }
    finish_dot<FIN>(local, cg, terms, N, sc);
}

// Euler update (MechanicalObject::vMultiOp fast path, MechanicalObject.inl:
// 2206-2240): v += dv; x += v h; optional v *= exp(-h vdamping).
// firstOrder (EulerImplicitSolver.cpp:200-224): v = dv, then x += v h.
// project_velocity: FixedProjectiveConstraint::projectVelocity
// (FixedProjectiveConstraint.inl:237-261), after the solve: fixed nodes'
// velocities set to zero (their positions have moved with the unprojected v).
// EulerImplicitSolver computeResidual (EulerImplicitSolver.cpp:314-338),
// after the step: r = 0; r += M (v_new - v_old), zero because the animation
// loop passes the state's own velocity as both; r += f (-dt) with f the
// scene's force at the new state (computeForce, just formed into f); r
// projected; r.r (MechanicalObject::vDot, serial with `terms`).
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_residual_dot(const R* __restrict__ f,
                                                             const uint8_t* __restrict__ fixed, double dt,
                                                             CgScalars* cg, double* terms, int N, SolveConsts sc)
{
    double local = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        double r[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) r[k] = fixed[n] ? 0.0 : (double)f[3 * (size_t)n + k] * (-dt);
        const double d = dot3(r, r);
        if (terms) terms[n] = d;
        local += d;
    }
    finish_dot<FIN_RESIDUAL>(local, cg, terms, N, sc);
}

// EulerImplicitSolver's addSeparateGravity (EulerImplicitSolver.cpp:296;
// UniformMass::addGravityToV, UniformMass.inl:450-468): v += g dt after the
// position update, before the velocity damping.
struct SepGravity {
    double hg[3];
    int on;
};

template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_euler_update(double* __restrict__ x, double* __restrict__ v,
                                                             const R* __restrict__ xs, double h, double vdamp,
                                                             CgScalars* cg, int N, int first_order = 0,
                                                             const uint8_t* __restrict__ project_fixed = nullptr,
                                                             SepGravity sg = SepGravity{{0.0, 0.0, 0.0}, 0})
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const bool zero_v = project_fixed && project_fixed[n];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const size_t i = 3 * (size_t)n + k;
            double vv = first_order ? (double)xs[i] : v[i] + (double)xs[i];
            double t = vv * h;
            x[i] = x[i] + t;
            if (sg.on) vv = vv + sg.hg[k];
            if (vdamp != 1.0) vv *= vdamp;
            v[i] = zero_v ? 0.0 : vv;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cg->time_step_count += 1;
}

// ------------------------------------------------------------------------
// fused patch matvec: one CTA per patch of elements (persistent over
// patches). Phase 0 loads the patch's nodal values into shared memory (and
// forms the CG direction p); phase 1 computes every element's four corner
// terms R K R^T (p_i - p_a) into shared memory; phase 2 sums, for each local
// node, its (element, corner) slots in element order -- a deterministic
// gather with no atomics. Nodes touched by this patch only are finished
// here; nodes shared with other patches leave one partial sum per patch.
// MODE 0: addDForce of the C ABI (df -= sum); MODE 1/2: CG matvec with p = r
// (first iteration) or p = p_old*beta + r, q = mF M p - sum, projected, and
// p^T A p from element energies plus the mass term.
// ------------------------------------------------------------------------
constexpr int kPatchThreads = 128;     // batch patch kernels
constexpr int kPatchMaxThreads = 256;  // single-mesh patch kernels: 64, 128 or 256 threads

// L2 prefetch of [lo, hi) by the bulk-copy unit (cp.async.bulk.prefetch.L2),
// trimmed to whole 16-byte chunks inside the range's allocation: the start
// is rounded down (allocations are 256-byte aligned), the end rounded down.
__device__ __forceinline__ void l2_prefetch(const void* lo, const void* hi)
{
    const unsigned long long a = (unsigned long long)lo & ~15ull;
    const unsigned long long b = (unsigned long long)hi & ~15ull;
    if (b > a) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(b - a)) : "memory");
}

// Issued by one thread: the element data (FP32 compressed form) and the
// local tables of patch P into L2, so that the block's next patch starts on
// L2 hits instead of DRAM latency.
template <typename R>
__device__ __forceinline__ void prefetch_patch(const PatchView& pv, const ElemView<R>& ev, int P)
{
    const int e0 = pv.elem_start[P], e1 = pv.elem_start[P + 1];
    const int n0 = pv.node_start[P], n1 = pv.node_start[P + 1];
    const size_t En = (size_t)ev.n_tets;
    const float4* q = reinterpret_cast<const float4*>(ev.rot);
    const float4* J = reinterpret_cast<const float4*>(ev.J);
    l2_prefetch(q + e0, q + e1);
#pragma unroll
    for (int k = 0; k < 3; ++k) l2_prefetch(J + k * En + e0, J + k * En + e1);
    l2_prefetch(pv.lconn + e0, pv.lconn + e1);
    l2_prefetch(pv.lslots + 4 * (size_t)e0, pv.lslots + 4 * (size_t)e1);
    l2_prefetch(pv.lnode_gid + n0, pv.lnode_gid + n1);
    l2_prefetch(pv.lnode_info + n0, pv.lnode_info + n1);
    l2_prefetch(pv.lrow + n0, pv.lrow + n1 + 1);
}

// Shared memory of the patch kernels: ef[12][pe] corner terms, sl[4*pe]
// slot lists, lr[max_lnodes+1] row starts (padded to 16 bytes), then
// lp[max_lnodes][3] nodal values. pe is even, so every region starts on a
// 16-byte boundary.
template <typename R>
__host__ __device__ __forceinline__ size_t patch_smem_size(int pe, int max_lnodes)
{
    return sizeof(R) * 12 * (size_t)pe + 8 * (size_t)pe + ((4 * ((size_t)max_lnodes + 1) + 15) & ~(size_t)15) +
           sizeof(R) * 3 * (size_t)max_lnodes;
}

// Shared memory of the matvec with two sets of slot lists and node values
// (no row starts): ef, set 1, then set 2 from the next 16-byte boundary (the
// slot lists take 16-byte asynchronous copies).
template <typename R>
__host__ __device__ __forceinline__ size_t patch_smem_set_db(int pe, int max_lnodes)
{
    return (8 * (size_t)pe + sizeof(R) * 3 * (size_t)max_lnodes + 15) & ~(size_t)15;
}
template <typename R>
__host__ __device__ __forceinline__ size_t patch_smem_size_db(int pe, int max_lnodes)
{
    return sizeof(R) * 12 * (size_t)pe + 2 * patch_smem_set_db<R>(pe, max_lnodes);
}
template <typename R>
__device__ __forceinline__ void patch_smem_carve_db(unsigned char* base, int pe, int max_lnodes, int set, R** ef,
                                                    uint16_t** sl, R** lp)
{
    *ef = reinterpret_cast<R*>(base);
    unsigned char* p = base + sizeof(R) * 12 * (size_t)pe + (size_t)set * patch_smem_set_db<R>(pe, max_lnodes);
    *sl = reinterpret_cast<uint16_t*>(p);
    *lp = reinterpret_cast<R*>(p + 8 * (size_t)pe);
}

template <typename R>
__device__ __forceinline__ void patch_smem_carve(unsigned char* base, int pe, int max_lnodes, R** ef, uint16_t** sl,
                                                 int** lr, R** lp)
{
    unsigned char* p = base;
    *ef = reinterpret_cast<R*>(p);
    p += sizeof(R) * 12 * (size_t)pe;
    *sl = reinterpret_cast<uint16_t*>(p);
    p += 8 * (size_t)pe;
    *lr = reinterpret_cast<int*>(p);
    p += (4 * ((size_t)max_lnodes + 1) + 15) & ~(size_t)15;
    *lp = reinterpret_cast<R*>(p);
}

// One element of a patch: nodal values relative to node a (J^T annihilates
// translations), rotated into the element frame, F = J K J^T X (computeForce,
// TFEM.inl:417-521), and the four corner terms R^T F_i into ef[12][pe];
// `pen` collects -p_rel^T (R^T F) for the CG modes.
template <typename R, int MODE>
__device__ __forceinline__ void patch_element(int le, ushort4 c, const R Rm[9], const R K[3], const R J[12], R kf,
                                              int pe, const R* lp, R* ef, R& pen)
{
    const int ln[4] = {c.x, c.y, c.z, c.w};
    R xr[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) xr[i][k] = lp[3 * ln[i] + k];
#pragma unroll
    for (int i = 3; i >= 0; --i)
#pragma unroll
        for (int k = 0; k < 3; ++k) xr[i][k] -= xr[0][k];
    R X[12], F[12];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k)
            X[3 * i + k] = Rm[3 * k] * xr[i][0] + Rm[3 * k + 1] * xr[i][1] + Rm[3 * k + 2] * xr[i][2];
    element_force(F, X, K, J, kf);
    R en = R(0);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const R ck = Rm[k] * F[3 * i] + Rm[3 + k] * F[3 * i + 1] + Rm[6 + k] * F[3 * i + 2];
            ef[(3 * i + k) * pe + le] = ck;
            en += xr[i][k] * ck;
        }
    if (MODE != 0) pen -= en;
}

// Per-call operands of the fused matvec. The single-mesh kernels build it
// from their parameters; the batch kernel keeps one per mesh in shared
// memory, so that its pointers are read where they are used instead of
// being held in registers across the patch.
template <typename R>
struct PatchArgs {
    const R* __restrict__ rin;   // input vector (r for the CG modes)
    const R* __restrict__ pold;  // previous direction (MODE 2)
    R* __restrict__ pnew;        // new direction (CG modes)
    R beta, kf, mmu;
    MassArgs ma;
    double mf;
    const uint8_t* __restrict__ fixed;
    R* __restrict__ qout;
    R* __restrict__ partials;
    const R* __restrict__ dinv;  // PCG: Jacobi inverse diagonal (PC = 1)
};

// One patch of the fused matvec, executed by the whole block (it contains
// block barriers). Returns this thread's share of the patch's p^T A p.
// One 16-byte global-to-shared copy that does not hold up the thread
// (cp.async, completed by cp_async_wait_all before the block barrier).
__device__ __forceinline__ void cp_async16(void* dst_smem, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst_smem, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// DB: the caller alternates two sets of slot lists and node values between
// consecutive patches (patch_smem_carve_db); the row starts are read from
// global memory and no barrier follows phase 2 (the next patch's phase-0
// barrier orders its phase 1 after this phase 2's reads of ef).
template <typename R, int MODE, int PC = 0, bool DB = false>
__device__ __forceinline__ R patch_body(const PatchView& pv, const ElemView<R>& ev, int P, const PatchArgs<R>& a, R* ef,
                                        R* lp, uint16_t* sl, int* lr)
{
    const size_t En = (size_t)ev.n_tets;
    R pen = R(0);
    const int e0 = pv.elem_start[P], ne = pv.elem_start[P + 1] - e0;
    const int n0 = pv.node_start[P], nn = pv.node_start[P + 1] - n0;
    // phase 0: the patch's slot lists (4 per element, from slot 4*e0; e0 is
    // even, so the 16-byte copies start on a 16-byte boundary and may read 8
    // bytes of padding past the end; a patch without elements copies
    // nothing) and row starts (global offsets; phase 2 subtracts 4*e0) into
    // shared memory, so that the gather of phase 2 runs on shared memory only
    {
        const uint4* src = reinterpret_cast<const uint4*>(pv.lslots + 4 * (size_t)e0);
        uint4* dst = reinterpret_cast<uint4*>(sl);
        const int n16 = (8 * ne + 15) >> 4;
        // asynchronous copies: the node loads below go out without waiting
        // for them (0.35 % faster CG steps than copies through registers)
        for (int k = threadIdx.x; k < n16; k += blockDim.x) cp_async16(dst + k, src + k);
        if constexpr (!DB)
            for (int l = threadIdx.x; l <= nn; l += blockDim.x) cp_async4(lr + l, pv.lrow + n0 + l);
    }
    // phase 0: nodal values of the patch
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const int g = pv.lnode_gid[n0 + l];
        R v[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            R rv = a.rin[3 * (size_t)g + k];
            if constexpr (PC != 0) rv = a.dinv[3 * (size_t)g + k] * rv;  // PCG: z = diag^-1 r
            v[k] = (MODE == 2) ? cg_dir(rv, a.pold[3 * (size_t)g + k], a.beta) : rv;
            lp[3 * l + k] = v[k];
        }
        if (MODE != 0) {
            const int info = pv.lnode_info[n0 + l];
            if (info < 0 || (info & 1)) {
#pragma unroll
                for (int k = 0; k < 3; ++k) a.pnew[3 * (size_t)g + k] = v[k];
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // phase 1: element terms
    for (int le = threadIdx.x; le < ne; le += blockDim.x) {
        const size_t e = (size_t)(e0 + le);
        R Rm[9], K[3], J[12];
        load_rot(ev, e, Rm);
        load_KJ(ev, e, K, J);
        patch_element<R, MODE>(le, pv.lconn[e], Rm, K, J, a.kf, pv.pe, lp, ef, pen);
    }
    __syncthreads();
    // phase 2: per local node, its slots in element order. The node's
    // global loads (id, layout word, then what its finish reads: df for
    // addDForce, mass and fixed flag for the CG modes) go out before the
    // shared-memory sum, so that they arrive while it runs.
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const int g = pv.lnode_gid[n0 + l];
        const int info = pv.lnode_info[n0 + l];
        R d0 = R(0), d1 = R(0), d2 = R(0), mm = a.mmu;
        bool fx = false;
        if (MODE == 0) {
            if (info < 0) {
                d0 = a.qout[3 * (size_t)g];
                d1 = a.qout[3 * (size_t)g + 1];
                d2 = a.qout[3 * (size_t)g + 2];
            }
        } else if (info < 0 || (info & 1)) {
            if (a.ma.node_mass) mm = (R)(a.ma.node_mass[g] * a.mf);
            if (info < 0) fx = a.fixed[g] != 0;
        }
        int s0, s1;
        if constexpr (DB) {
            s0 = pv.lrow[n0 + l] - 4 * e0;
            s1 = pv.lrow[n0 + l + 1] - 4 * e0;
        } else {
            s0 = lr[l] - 4 * e0;
            s1 = lr[l + 1] - 4 * e0;
        }
        R a0 = R(0), a1 = R(0), a2 = R(0);
        for (int s = s0; s < s1; ++s) {
            const int slot = sl[s];
            const int le = slot >> 2, cc = slot & 3;
            a0 += ef[(3 * cc + 0) * pv.pe + le];
            a1 += ef[(3 * cc + 1) * pv.pe + le];
            a2 += ef[(3 * cc + 2) * pv.pe + le];
        }
        if (info >= 0) {
            R* o = a.partials + 3 * (size_t)(info >> 1);
            o[0] = a0;
            o[1] = a1;
            o[2] = a2;
        }
        if (MODE == 0) {
            if (info < 0) {
                a.qout[3 * (size_t)g] = d0 - a0;
                a.qout[3 * (size_t)g + 1] = d1 - a1;
                a.qout[3 * (size_t)g + 2] = d2 - a2;
            }
        } else if (info < 0 || (info & 1)) {
            const R p0 = lp[3 * l], p1 = lp[3 * l + 1], p2 = lp[3 * l + 2];
            pen += mm * (p0 * p0 + p1 * p1 + p2 * p2);
            if (info < 0) {
                R q0 = mm * p0 - a0, q1 = mm * p1 - a1, q2 = mm * p2 - a2;
                if (fx) q0 = q1 = q2 = R(0);
                a.qout[3 * (size_t)g] = q0;
                a.qout[3 * (size_t)g + 1] = q1;
                a.qout[3 * (size_t)g + 2] = q2;
            }
        }
    }
    if constexpr (!DB) __syncthreads();
    return pen;
}

// MINB > 1: 128-thread CTAs with the register cap for MINB resident CTAs
// per SM (FP32 only; 9 gives 56 registers without spills); MINB = 1: no cap,
// 64, 128 or 256 threads.
template <typename R, int MODE, int PC = 0, int MINB = 1, bool DB = false>
__global__ void __launch_bounds__(MINB > 1 ? kPatchThreads : kPatchMaxThreads, sizeof(R) == 4 && MINB > 1 ? MINB : 0)
    k_patch_matvec(PatchView pv, ElemView<R> ev,
                                                                   const R* __restrict__ rin,
                                                                   const R* __restrict__ pold, R* __restrict__ pnew,
                                                                   CgScalars* cg, R kf, MassArgs ma, double mf,
                                                                   const uint8_t* __restrict__ fixed,
                                                                   R* __restrict__ qout, R* __restrict__ partials,
                                                                   SolveConsts sc, int prefetch,
                                                                   const R* __restrict__ dinv = nullptr)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* ef;
    R* lp;
    uint16_t* sl;
    int* lr;
    patch_smem_carve<R>(smem_raw, pv.pe, pv.max_lnodes, &ef, &sl, &lr, &lp);
    if (MODE != 0 && cg->done) return;
    // MODE 0 with a CG state: run only if iteration sc.it of the solve ran
    // (residual replacement inside a captured step)
    if (MODE == 0 && cg && cg->iters != sc.it) return;
    const R beta = (MODE == 2) ? (R)cg->beta : R(0);
    const R mmu = (R)(mf != 1.0 ? ma.vertex_mass * mf : ma.vertex_mass);
    const PatchArgs<R> args{rin, pold, pnew, beta, kf, mmu, ma, mf, fixed, qout, partials, dinv};
    double energy = 0.0;  // FP64 across patches; FP32 within one patch
    int k = 0;
    for (int P = blockIdx.x; P < pv.n_patches; P += gridDim.x, ++k) {
        if constexpr (is_mixed<R>::value)
            if (prefetch && threadIdx.x == 0 && P + (int)gridDim.x < pv.n_patches)
                prefetch_patch(pv, ev, P + gridDim.x);
        if constexpr (DB) {
            patch_smem_carve_db<R>(smem_raw, pv.pe, pv.max_lnodes, k & 1, &ef, &sl, &lp);
            energy += (double)patch_body<R, MODE, PC, true>(pv, ev, P, args, ef, lp, sl, nullptr);
        } else {
            energy += (double)patch_body<R, MODE, PC>(pv, ev, P, args, ef, lp, sl, lr);
        }
    }
    if (MODE != 0) finish_dot<FIN_DEN>(energy, cg, nullptr, 0, sc);
}

// addDForce (MODE 0) as its own kernel so that it can carry its own register
// cap: 128-thread CTAs, at least 10 per SM in FP32 (51 registers), measured
// faster than the 64 the CG modes need. `gate`: run only if *gate equals
// gate_it (residual replacement inside a captured step: the iteration a
// replacement was decided for).
template <typename R>
__global__ void __launch_bounds__(kPatchThreads, sizeof(R) == 4 ? 10 : 1)
    k_patch_adddforce(PatchView pv, ElemView<R> ev, const R* __restrict__ dx, R kf, R* __restrict__ df,
                      R* __restrict__ partials, const int* gate, int gate_it)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* ef;
    R* lp;
    uint16_t* sl;
    int* lr;
    patch_smem_carve<R>(smem_raw, pv.pe, pv.max_lnodes, &ef, &sl, &lr, &lp);
    if (gate && *gate != gate_it) return;
    const PatchArgs<R> args{dx, nullptr, nullptr, R(0), kf, R(0), {nullptr, 0.0, {0.0, 0.0, 0.0}}, 1.0, nullptr, df,
                            partials, nullptr};
    for (int P = blockIdx.x; P < pv.n_patches; P += gridDim.x) (void)patch_body<R, 0>(pv, ev, P, args, ef, lp, sl, lr);
}

// C ABI addDForce, second pass: nodes shared by several patches subtract
// their partial sums in patch order.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_patch_fixup(const int* __restrict__ bnd_rowptr,
                                                            const R* __restrict__ partials, R* __restrict__ df, int N,
                                                            const int* gate = nullptr, int gate_it = 0)
{
    if (gate && *gate != gate_it) return;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const int b0 = bnd_rowptr[n], b1 = bnd_rowptr[n + 1];
        if (b0 == b1) continue;
        R a0 = R(0), a1 = R(0), a2 = R(0);
        for (int b = b0; b < b1; ++b) {
            a0 += partials[3 * (size_t)b];
            a1 += partials[3 * (size_t)b + 1];
            a2 += partials[3 * (size_t)b + 2];
        }
        df[3 * (size_t)n] -= a0;
        df[3 * (size_t)n + 1] -= a1;
        df[3 * (size_t)n + 2] -= a2;
    }
}

// The float-float difference b - a of two float-float values.
__device__ __forceinline__ ff ff_sub(float2 b, float2 a)
{
    const ff s = two_sum(b.x, -a.x);
    const float t = s.l + (b.y - a.y);
    const float h = s.h + t;
    return {h, t - (h - s.h)};
}

// Shared memory of the patch force / right-hand side pass: the matvec's
// regions, then per local node three float-float pairs (v relative to the
// patch's first local node).
template <typename R>
__host__ __device__ __forceinline__ size_t force_patch_smem_size(int pe, int max_lnodes)
{
    return patch_smem_size<R>(pe, max_lnodes) - sizeof(R) * 3 * (size_t)max_lnodes +
           sizeof(float2) * 3 * (size_t)max_lnodes;
}

// One patch of computeForce and the right-hand side's stiffness term (mixed
// precision, rotated methods; executed by the whole block). Phase 0: each
// local node's velocity relative to the patch's first local node, formed in
// FP64 and split into a float-float pair in shared memory (the FP64
// subtraction and conversion once per local node instead of once per
// element corner). Phase 1: per element the force corner terms from its FP64
// edges (elem_force_edges; the edges stay per element: relative to a patch
// point they would lose the bits the strain of stiff, lightly loaded meshes
// needs), less the (h + rs) K v terms on the velocities relative to node a
// (the float-float differences rounded once, as the FP64 differences were),
// into ef[12][pe] (firstOrder: the force terms alone). Phase 2: per local
// node its slots summed there, interior nodes into own[], nodes shared by
// several patches into their partial slot.
template <typename R, int METHOD>
__device__ __forceinline__ void patch_force_rhs_body(const PatchView& pv, const ElemView<R>& ev, int P,
                                                     const double* __restrict__ x, const double* __restrict__ v,
                                                     const PlasticArgs<R>& pl, R kf_rhs, int first_order,
                                                     R* __restrict__ own, R* __restrict__ partials, R* ef,
                                                     float2* lv, uint16_t* sl, int* lr)
{
    const int e0 = pv.elem_start[P], ne = pv.elem_start[P + 1] - e0;
    const int n0 = pv.node_start[P], nn = pv.node_start[P + 1] - n0;
    {
        const uint4* src = reinterpret_cast<const uint4*>(pv.lslots + 4 * (size_t)e0);
        uint4* dst = reinterpret_cast<uint4*>(sl);
        const int n16 = (8 * ne + 15) >> 4;
        for (int k = threadIdx.x; k < n16; k += blockDim.x) cp_async16(dst + k, src + k);
        for (int l = threadIdx.x; l <= nn; l += blockDim.x) cp_async4(lr + l, pv.lrow + n0 + l);
    }
    if (ne > 0 && !first_order) {
        double v0[3];
        ld3(v, pv.lnode_gid[n0], v0);
        for (int l = threadIdx.x; l < nn; l += blockDim.x) {
            const int g = pv.lnode_gid[n0 + l];
            double vv[3];
            ld3(v, g, vv);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const ff b = split_f64(vv[k] - v0[k]);
                lv[3 * l + k] = make_float2(b.h, b.l);
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
    for (int le = threadIdx.x; le < ne; le += blockDim.x) {
        const int e = e0 + le;
        ff eg[3][3];
        {
            // edges: one FP64 subtraction each, then split (elem_force_body)
            const int4 t = ev.tets[e];
            double p[4][3];
            ld3(x, t.x, p[0]);
            ld3(x, t.y, p[1]);
            ld3(x, t.z, p[2]);
            ld3(x, t.w, p[3]);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) eg[i][k] = split_f64(p[i + 1][k] - p[0][k]);
        }
        R Rm[9], K[3], J[12], c[12];
        elem_force_edges<R, METHOD>(ev, e, eg, pl, Rm, K, J, c);
        if (!first_order) {
            // the K v terms with the rotation as the packed copy gives it back
            const ushort4 cn = pv.lconn[e];
            const float2* na = lv + 3 * (int)cn.x;
            const float2* nb[3] = {lv + 3 * (int)cn.y, lv + 3 * (int)cn.z, lv + 3 * (int)cn.w};
            R xin[4][3], Rq[9], cv[12];
#pragma unroll
            for (int k = 0; k < 3; ++k) xin[0][k] = R(0);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const ff d = ff_sub(nb[i][k], na[k]);
                    xin[i + 1][k] = d.h + d.l;
                }
            quat_to_rot(rot_to_quat(Rm), Rq);
            dforce_terms<R, METHOD_LARGE>(xin, Rq, K, J, kf_rhs, cv);
#pragma unroll
            for (int i = 0; i < 12; ++i) c[i] -= cv[i];
        }
#pragma unroll
        for (int i = 0; i < 12; ++i) ef[i * pv.pe + le] = c[i];
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const int g = pv.lnode_gid[n0 + l];
        const int info = pv.lnode_info[n0 + l];
        const int s0 = lr[l] - 4 * e0, s1 = lr[l + 1] - 4 * e0;
        R a0 = R(0), a1 = R(0), a2 = R(0);
        for (int s = s0; s < s1; ++s) {
            const int slot = sl[s];
            const int le = slot >> 2, cc = slot & 3;
            a0 += ef[(3 * cc + 0) * pv.pe + le];
            a1 += ef[(3 * cc + 1) * pv.pe + le];
            a2 += ef[(3 * cc + 2) * pv.pe + le];
        }
        R* o = info >= 0 ? partials + 3 * (size_t)(info >> 1) : own + 3 * (size_t)g;
        o[0] = a0;
        o[1] = a1;
        o[2] = a2;
    }
    __syncthreads();
}

// computeForce and the right-hand side's stiffness term by patches (mixed
// precision, rotated methods, persistent CTAs): the operations of
// k_elem_force_rhs and k_gather_force_rhs, summed per patch instead of in
// element order, with no corner-term buffers in HBM; k_rhs_finish_patch
// then forms b.
// 64 registers (no spills for large and polar; svd keeps 80): 6 resident
// CTAs of 160 threads per SM instead of 4, 0.2 % faster steps
template <typename R, int METHOD>
__global__ void __maxnreg__(METHOD == METHOD_SVD ? 80 : 64) k_patch_force_rhs(PatchView pv, ElemView<R> ev,
                                                                   const double* __restrict__ x,
                                                                   PlasticArgs<R> pl, const double* __restrict__ v,
                                                                   R kf_rhs, int first_order, R* __restrict__ own,
                                                                   R* __restrict__ partials)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* ef;
    R* lp;
    uint16_t* sl;
    int* lr;
    patch_smem_carve<R>(smem_raw, pv.pe, pv.max_lnodes, &ef, &sl, &lr, &lp);
    float2* lv = reinterpret_cast<float2*>(lp);
    for (int P = blockIdx.x; P < pv.n_patches; P += gridDim.x)
        patch_force_rhs_body<R, METHOD>(pv, ev, P, x, v, pl, kf_rhs, first_order, own, partials, ef, lv, sl, lr);
}

// The right-hand side per node after k_patch_force_rhs: the element sum
// (own[] or the node's partial sums in patch order), external and gravity
// forces, the Rayleigh mass term on v, times h; projected; b = r, x = 0
// (cold start) and |b|^2 as k_gather_force_rhs forms them.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_rhs_finish_patch(const R* __restrict__ own,
                                                                 const R* __restrict__ partials,
                                                                 const int* __restrict__ bnd_rowptr,
                                                                 const R* __restrict__ ext,
                                                                 const double* __restrict__ v, MassArgs ma,
                                                                 double mfac, double h,
                                                                 const uint8_t* __restrict__ fixed,
                                                                 R* __restrict__ b, R* __restrict__ r,
                                                                 R* __restrict__ xs, CgScalars* cg, int N,
                                                                 SolveConsts sc, int first_order)
{
    const R mg0 = (R)(ma.g[0] * ma.vertex_mass), mg1 = (R)(ma.g[1] * ma.vertex_mass),
            mg2 = (R)(ma.g[2] * ma.vertex_mass);
    const R mm = (R)(mfac != 1.0 ? ma.vertex_mass * mfac : ma.vertex_mass);
    const R hr = (R)h;
    double local = 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) cg->done = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const int b0 = bnd_rowptr[n], b1 = bnd_rowptr[n + 1];
        R s0 = R(0), s1 = R(0), s2 = R(0);
        if (b0 == b1) {
            s0 = own[3 * (size_t)n];
            s1 = own[3 * (size_t)n + 1];
            s2 = own[3 * (size_t)n + 2];
        } else {
            for (int k = b0; k < b1; ++k) {
                s0 += partials[3 * (size_t)k];
                s1 += partials[3 * (size_t)k + 1];
                s2 += partials[3 * (size_t)k + 2];
            }
        }
        R a[3] = {mg0, mg1, mg2};
        if (ma.node_mass) {
            const double m = ma.node_mass[n];
            a[0] = (R)(ma.g[0] * m);
            a[1] = (R)(ma.g[1] * m);
            a[2] = (R)(ma.g[2] * m);
        }
        if (ext) {
            a[0] += ext[3 * (size_t)n];
            a[1] += ext[3 * (size_t)n + 1];
            a[2] += ext[3 * (size_t)n + 2];
        }
        a[0] += s0;
        a[1] += s1;
        a[2] += s2;
        if (!first_order) {
            R vv[3] = {(R)v[3 * (size_t)n], (R)v[3 * (size_t)n + 1], (R)v[3 * (size_t)n + 2]};
            if (mfac != 0.0) add_mdx(a, vv, ma, mfac, mm, n);
#pragma unroll
            for (int k = 0; k < 3; ++k) a[k] *= hr;
        }
        if (fixed[n]) a[0] = a[1] = a[2] = R(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            b[3 * (size_t)n + k] = a[k];
            r[3 * (size_t)n + k] = a[k];
            if (!sc.pcg && !sc.warm) xs[3 * (size_t)n + k] = R(0);  // PCG / warmStart keep the previous solution
        }
        local += dot3(a, a);
    }
    finish_dot<FIN_RHS>(local, cg, nullptr, N, sc);
}

// A node's r.r, with the roundings spelled out (two fused multiply-adds), so
// that every kernel forming it gets the same bits.
__device__ __forceinline__ float node_rr(const float r[3]) { return __fmaf_rn(r[2], r[2], __fmaf_rn(r[1], r[1], r[0] * r[0])); }
__device__ __forceinline__ double node_rr(const double r[3]) { return __fma_rn(r[2], r[2], __fma_rn(r[1], r[1], r[0] * r[0])); }

// CG update of one node after a patch matvec: completes q on a shared node
// (mass term minus the patches' partial sums, projected), then x += alpha p,
// r += -alpha q. Returns the node's r.r, or r.z with z = diag^-1 r for PCG
// (three-term sum in R).
template <typename R, int PC = 0>
__device__ __forceinline__ R cg_update1(size_t n, R* __restrict__ xs, R* __restrict__ r, const R* __restrict__ p,
                                        const R* __restrict__ q, const R* __restrict__ partials,
                                        const int* __restrict__ bnd_rowptr, const double* __restrict__ node_mass,
                                        R mmu, double mf, const uint8_t* __restrict__ fixed, R alpha,
                                        const R* __restrict__ dinv = nullptr)
{
    const size_t i3 = 3 * n;
    const R pp[3] = {p[i3], p[i3 + 1], p[i3 + 2]};
    R qq[3];
    const int b0 = bnd_rowptr[n], b1 = bnd_rowptr[n + 1];
    if (b0 == b1) {
        qq[0] = q[i3];
        qq[1] = q[i3 + 1];
        qq[2] = q[i3 + 2];
    } else {
        R a0 = R(0), a1 = R(0), a2 = R(0);
        for (int b = b0; b < b1; ++b) {
            a0 += partials[3 * (size_t)b];
            a1 += partials[3 * (size_t)b + 1];
            a2 += partials[3 * (size_t)b + 2];
        }
        const R mm = node_mass ? (R)(node_mass[n] * mf) : mmu;
        qq[0] = mm * pp[0] - a0;
        qq[1] = mm * pp[1] - a1;
        qq[2] = mm * pp[2] - a2;
        if (fixed[n]) qq[0] = qq[1] = qq[2] = R(0);
    }
    const R nalpha = -alpha;
    R rr[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        xs[i3 + k] = xs[i3 + k] + pp[k] * alpha;
        rr[k] = r[i3 + k] + qq[k] * nalpha;
        r[i3 + k] = rr[k];
    }
    if constexpr (PC != 0) {
        R zz[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) zz[k] = dinv[i3 + k] * rr[k];
        return rr[0] * zz[0] + rr[1] * zz[1] + rr[2] * zz[2];
    }
    return node_rr(rr);
}

__device__ __forceinline__ void ld12(const float* __restrict__ a, size_t n0, float v[12])
{
    const float4* s = reinterpret_cast<const float4*>(a + 3 * n0);
    const float4 x = s[0], y = s[1], z = s[2];
    v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w;
    v[4] = y.x, v[5] = y.y, v[6] = y.z, v[7] = y.w;
    v[8] = z.x, v[9] = z.y, v[10] = z.z, v[11] = z.w;
}

__device__ __forceinline__ void st12(float* __restrict__ a, size_t n0, const float v[12])
{
    float4* d = reinterpret_cast<float4*>(a + 3 * n0);
    d[0] = make_float4(v[0], v[1], v[2], v[3]);
    d[1] = make_float4(v[4], v[5], v[6], v[7]);
    d[2] = make_float4(v[8], v[9], v[10], v[11]);
}

// The same update for four consecutive nodes n0..n0+3 (n0 a multiple of 4)
// with 16-byte loads, every load of the group issued before the first use.
// Returns the group's r.r (PCG: r.z, z = diag^-1 r): the twelve products
// summed in FP32 in node order (the caller's running sum is FP64).
template <int PC = 0>
__device__ __forceinline__ double cg_update4(size_t n0, float* __restrict__ xs, float* __restrict__ r,
                                             const float* __restrict__ p, const float* __restrict__ q,
                                             const float* __restrict__ partials, const int* __restrict__ bnd_rowptr,
                                             const double* __restrict__ node_mass, float mmu, double mf,
                                             const uint8_t* __restrict__ fixed, float alpha,
                                             const float* __restrict__ dinv = nullptr)
{
    float pp[12], qq[12], xx[12], rr[12];
    ld12(p, n0, pp);
    ld12(q, n0, qq);
    ld12(xs, n0, xx);
    ld12(r, n0, rr);
    const int4 br = *reinterpret_cast<const int4*>(bnd_rowptr + n0);
    const int bb[5] = {br.x, br.y, br.z, br.w, bnd_rowptr[n0 + 4]};
    const uchar4 fx = *reinterpret_cast<const uchar4*>(fixed + n0);
    const uint8_t ff[4] = {fx.x, fx.y, fx.z, fx.w};
    // x needs no partial sum: advanced and stored first, which frees its
    // registers before the partial loop
#pragma unroll
    for (int k = 0; k < 12; ++k) xx[k] = xx[k] + pp[k] * alpha;
    st12(xs, n0, xx);
    // the group's partial slots are one contiguous range (node-major CSR):
    // one unrolled loop over it, each slot added to its node in slot order,
    // so the loads of several slots are in flight together
    float ps[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) ps[k] = 0.f;
#pragma unroll 4
    for (int b = bb[0]; b < bb[4]; ++b) {
        const float v0 = partials[3 * (size_t)b], v1 = partials[3 * (size_t)b + 1], v2 = partials[3 * (size_t)b + 2];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (b >= bb[j] && b < bb[j + 1]) {
                ps[3 * j] += v0;
                ps[3 * j + 1] += v1;
                ps[3 * j + 2] += v2;
            }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (bb[j + 1] > bb[j]) {
            const float mm = node_mass ? (float)(node_mass[n0 + j] * mf) : mmu;
            qq[3 * j] = mm * pp[3 * j] - ps[3 * j];
            qq[3 * j + 1] = mm * pp[3 * j + 1] - ps[3 * j + 1];
            qq[3 * j + 2] = mm * pp[3 * j + 2] - ps[3 * j + 2];
            if (ff[j]) qq[3 * j] = qq[3 * j + 1] = qq[3 * j + 2] = 0.f;
        }
    }
    const float nalpha = -alpha;
#pragma unroll
    for (int k = 0; k < 12; ++k) rr[k] = rr[k] + qq[k] * nalpha;
    st12(r, n0, rr);
    float zz[12];
    if constexpr (PC != 0) {
        ld12(dinv, n0, zz);
#pragma unroll
        for (int k = 0; k < 12; ++k) zz[k] = zz[k] * rr[k];
    } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) zz[k] = rr[k];
    }
    float local = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        local += rr[3 * j] * zz[3 * j] + rr[3 * j + 1] * zz[3 * j + 1] + rr[3 * j + 2] * zz[3 * j + 2];
    return (double)local;
}

// cg_update4 for the batch engine: the four nodes' r.r in t[0..3], each
// formed as node_rr forms it (cg_update1 gives the same per node).
__device__ __forceinline__ void cg_update4_terms(size_t n0, float* __restrict__ xs, float* __restrict__ r,
                                                 const float* __restrict__ p, const float* __restrict__ q,
                                                 const float* __restrict__ partials,
                                                 const int* __restrict__ bnd_rowptr,
                                                 const double* __restrict__ node_mass, float mmu, double mf,
                                                 const uint8_t* __restrict__ fixed, float alpha, double t[4])
{
    float pp[12], qq[12], xx[12], rr[12];
    ld12(p, n0, pp);
    ld12(q, n0, qq);
    ld12(xs, n0, xx);
    ld12(r, n0, rr);
    const int4 br = *reinterpret_cast<const int4*>(bnd_rowptr + n0);
    const int bb[5] = {br.x, br.y, br.z, br.w, bnd_rowptr[n0 + 4]};
    const uchar4 fx = *reinterpret_cast<const uchar4*>(fixed + n0);
    const uint8_t ff[4] = {fx.x, fx.y, fx.z, fx.w};
    // x needs no partial sum: advanced and stored first, which frees its
    // registers before the partial loop
#pragma unroll
    for (int k = 0; k < 12; ++k) xx[k] = xx[k] + pp[k] * alpha;
    st12(xs, n0, xx);
    float ps[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) ps[k] = 0.f;
#pragma unroll 4
    for (int b = bb[0]; b < bb[4]; ++b) {
        const float v0 = partials[3 * (size_t)b], v1 = partials[3 * (size_t)b + 1], v2 = partials[3 * (size_t)b + 2];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (b >= bb[j] && b < bb[j + 1]) {
                ps[3 * j] += v0;
                ps[3 * j + 1] += v1;
                ps[3 * j + 2] += v2;
            }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (bb[j + 1] > bb[j]) {
            const float mm = node_mass ? (float)(node_mass[n0 + j] * mf) : mmu;
            qq[3 * j] = mm * pp[3 * j] - ps[3 * j];
            qq[3 * j + 1] = mm * pp[3 * j + 1] - ps[3 * j + 1];
            qq[3 * j + 2] = mm * pp[3 * j + 2] - ps[3 * j + 2];
            if (ff[j]) qq[3 * j] = qq[3 * j + 1] = qq[3 * j + 2] = 0.f;
        }
    }
    const float nalpha = -alpha;
#pragma unroll
    for (int k = 0; k < 12; ++k) rr[k] = rr[k] + qq[k] * nalpha;
    st12(r, n0, rr);
#pragma unroll
    for (int j = 0; j < 4; ++j) t[j] = (double)node_rr(rr + 3 * j);
}

template <typename R, int PC>
__device__ __forceinline__ double cg_update4g(size_t n0, R* xs, R* r, const R* p, const R* q, const R* partials,
                                              const int* bnd_rowptr, const double* node_mass, R mmu, double mf,
                                              const uint8_t* fixed, R alpha, const R* dinv)
{
    if constexpr (is_mixed<R>::value) {
        return cg_update4<PC>(n0, xs, r, p, q, partials, bnd_rowptr, node_mass, mmu, mf, fixed, alpha, dinv);
    } else {
        double local = 0.0;
        for (int j = 0; j < 4; ++j)
            local += (double)cg_update1<R, PC>(n0 + j, xs, r, p, q, partials, bnd_rowptr, node_mass, mmu, mf, fixed,
                                               alpha, dinv);
        return local;
    }
}

// CG update after a patch matvec over all nodes, then rho = r.r (PCG: r.z).
// FP32: one thread per group of four nodes (16-byte loads), the N % 4 last
// nodes one per thread.
template <typename R, int MINB, int PC = 0>
__global__ void __launch_bounds__(kNodeBlock, MINB) k_cg_update_patch(R* __restrict__ xs, R* __restrict__ r,
                                                                const R* __restrict__ p, const R* __restrict__ q,
                                                                const R* __restrict__ partials,
                                                                const int* __restrict__ bnd_rowptr, MassArgs ma,
                                                                double mf, const uint8_t* __restrict__ fixed,
                                                                CgScalars* cg, int N, SolveConsts sc, int vec4,
                                                                const R* __restrict__ dinv = nullptr)
{
    if (cg->done) return;
    const R alpha = (R)cg->alpha;
    const R mmu = (R)(mf != 1.0 ? ma.vertex_mass * mf : ma.vertex_mass);
    double local = 0.0;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (is_mixed<R>::value && vec4) {
        const int G4 = N >> 2;
        for (int g = tid; g < G4; g += stride)
            local += cg_update4g<R, PC>(4 * (size_t)g, xs, r, p, q, partials, bnd_rowptr, ma.node_mass, mmu, mf,
                                        fixed, alpha, dinv);
        for (int n = 4 * G4 + tid; n < N; n += stride)
            local += (double)cg_update1<R, PC>((size_t)n, xs, r, p, q, partials, bnd_rowptr, ma.node_mass, mmu, mf,
                                               fixed, alpha, dinv);
    } else {
        for (int n = tid; n < N; n += stride)
            local += (double)cg_update1<R, PC>((size_t)n, xs, r, p, q, partials, bnd_rowptr, ma.node_mass, mmu, mf,
                                               fixed, alpha, dinv);
    }
    finish_dot<FIN_RHO>(local, cg, nullptr, N, sc);
}

// ------------------------------------------------------------------------
// Residual replacement for FP32 scenes (reliable-update CG, after van der
// Vorst and Ye, "Residual replacement strategies for Krylov subspace
// iterative methods for the convergence of true residuals", SIAM J. Sci.
// Comput. 22(3), 2000): the FP32 recurrence r -= alpha q drifts from
// b - A x; every few iterations the FP32 increment is folded into an FP64
// solution x64 and the residual recomputed from b64 in FP64 with an FP64
// copy of the operator.
// ------------------------------------------------------------------------

// x64 += xs32, xs32 = 0, if a replacement was decided after iteration `it`.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_refine_accumulate(double* __restrict__ x64, R* __restrict__ xs,
                                                                  const CgScalars* cg, int it, int N)
{
    if (cg->replace_it != it) return;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < 3 * (size_t)N;
         i += (size_t)gridDim.x * blockDim.x) {
        x64[i] += (double)xs[i];
        xs[i] = R(0);
    }
}

// r = b64 - (mF M x64 - kF K x64), with w64 = -kF K x64 from the FP64
// operator; projected; r32 = r (rounded); r.r in FP64 replaces rho.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_refine_residual(const double* __restrict__ b64,
                                                                const double* __restrict__ x64,
                                                                const double* __restrict__ w64, MassArgs ma,
                                                                double mf, const uint8_t* __restrict__ fixed,
                                                                R* __restrict__ r, CgScalars* cg, int N,
                                                                SolveConsts sc)
{
    if (cg->replace_it != sc.it) return;
    const double mmu = ma.vertex_mass * mf;
    double local = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const double mm = ma.node_mass ? ma.node_mass[n] * mf : mmu;
        double rr[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const size_t i = 3 * (size_t)n + k;
            rr[k] = fixed[n] ? 0.0 : b64[i] - (mm * x64[i] + w64[i]);
            r[i] = (R)rr[k];
        }
        local += dot3(rr, rr);
    }
    finish_dot<FIN_REPLACE>(local, cg, nullptr, N, sc);
}

// v += x64 + xs32, x += h v (EulerImplicitSolver.cpp:256-295 with the
// solution split in two parts).
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_euler_refined(double* __restrict__ x, double* __restrict__ v,
                                                              const double* __restrict__ x64,
                                                              const R* __restrict__ xs, double h, double vdamp,
                                                              CgScalars* cg, int N,
                                                              const uint8_t* __restrict__ project_fixed = nullptr,
                                                              SepGravity sg = SepGravity{{0.0, 0.0, 0.0}, 0})
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const bool zero_v = project_fixed && project_fixed[n];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const size_t i = 3 * (size_t)n + k;
            double vv = v[i] + (x64[i] + (double)xs[i]);
            double t = vv * h;
            x[i] = x[i] + t;
            if (sg.on) vv = vv + sg.hg[k];
            if (vdamp != 1.0) vv *= vdamp;
            v[i] = zero_v ? 0.0 : vv;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cg->time_step_count += 1;
}

// ------------------------------------------------------------------------
// host launchers
// ------------------------------------------------------------------------
inline int node_grid(int N)
{
    int g = (N + kNodeBlock - 1) / kNodeBlock;
    if (g > kMaxNodeBlocks) g = kMaxNodeBlocks;
    return g < 1 ? 1 : g;
}
inline int elem_grid(int E) { return (E + kElemBlock - 1) / kElemBlock; }

template <typename R>
ElemView<R> view(TfemMesh* m)
{
    ElemView<R> ev;
    ev.tets = m->tets;
    ev.rot = (R*)m->rot;
    ev.K = (const R*)m->K;
    ev.J = (const R*)m->J;
    ev.rest = (const R*)m->rest;
    ev.rest_ff = m->rest_ff;
    ev.A0inv = (const R*)m->A0inv;
    ev.R0 = m->method == METHOD_SVD ? (const R*)m->R0 : nullptr;
    ev.n_tets = m->n_tets;
    ev.method = m->method;
    return ev;
}

template <typename R>
void launch_init(TfemMesh* m, const double* young, int ny, const double* poisson, int np, const double* lsf, int nl,
                 double* vol, cudaStream_t s)
{
    if (m->n_tets == 0) return;
    k_init_elements<R><<<elem_grid(m->n_tets), kElemBlock, 0, s>>>(
        m->rest_pos, m->tets, m->elem_orig, m->n_tets, m->method, young, ny, poisson, np, lsf, nl, (R*)m->K,
        (R*)m->J, (R*)m->rest, m->rest_ff, (R*)m->rot, (R*)m->A0inv, (R*)m->R0, vol);
}

// Mixed precision: the per-element factor sqrt(K(0,0)) of the stored
// strain-displacement values, for the plastic thresholds.
template <typename R>
__global__ void k_plastic_scale(const double* __restrict__ rest_pos, const int4* __restrict__ tets,
                                const int* __restrict__ elem_orig, int E, const double* __restrict__ young,
                                int n_young, const double* __restrict__ poisson, int n_poisson,
                                const double* __restrict__ lsf, int n_lsf, R* __restrict__ scale)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= E) return;
    const int4 t = tets[s];
    double pa[3], pb[3], pc[3], pd[3], k[3], v;
    ld3(rest_pos, t.x, pa);
    ld3(rest_pos, t.y, pb);
    ld3(rest_pos, t.z, pc);
    ld3(rest_pos, t.w, pd);
    material_stiffness(pa, pb, pc, pd, elem_orig[s], E, young, n_young, poisson, n_poisson, lsf, n_lsf, k, &v);
    scale[s] = (R)sqrt(k[0]);
}

template <typename R>
void launch_plastic_scale(TfemMesh* m, const double* young, int ny, const double* poisson, int np, const double* lsf,
                          int nl, cudaStream_t s)
{
    if (m->n_tets == 0 || !m->plastic_scale) return;
    k_plastic_scale<R><<<elem_grid(m->n_tets), kElemBlock, 0, s>>>(m->rest_pos, m->tets, m->elem_orig, m->n_tets,
                                                                   young, ny, poisson, np, lsf, nl,
                                                                   (R*)m->plastic_scale);
}

// The force kernels' plasticity and updateStiffnessMatrix operands.
template <typename R>
PlasticArgs<R> plastic_args(TfemMesh* m)
{
    PlasticArgs<R> pl;
    if (m->plastic && m->plastic_max > 0.0) {
        pl.strain = (R*)m->plastic;
        pl.scale = (const R*)m->plastic_scale;
        pl.max_threshold = (R)m->plastic_max;
        pl.yield_threshold = (R)m->plastic_yield;
        pl.creep = (R)m->plastic_creep;
    }
    if (m->update_j) {
        pl.update_J = (R*)m->J;
        pl.scale = (const R*)m->plastic_scale;
    }
    return pl;
}

template <typename R>
void launch_elem_force(TfemMesh* m, const double* x, cudaStream_t s)
{
    if (m->n_tets == 0) return;
    ElemView<R> ev = view<R>(m);
    const int g = elem_grid(m->n_tets);
    const PlasticArgs<R> pl = plastic_args<R>(m);
    if (m->method == METHOD_SMALL)
        k_elem_force<R, METHOD_SMALL><<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl);
    else if (m->method == METHOD_LARGE)
        k_elem_force<R, METHOD_LARGE><<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl);
    else if (m->method == METHOD_SVD)
        k_elem_force<R, METHOD_SVD><<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl);
    else
        k_elem_force<R, METHOD_POLAR><<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl);
}

// k_elem_force_rhs for the rotated methods (the patch step's force field).
template <typename R>
void launch_elem_force_rhs(TfemMesh* m, const double* x, const double* v, R kf_rhs, R* eforce_v, cudaStream_t s)
{
    if (m->n_tets == 0) return;
    ElemView<R> ev = view<R>(m);
    const int g = elem_grid(m->n_tets);
    const PlasticArgs<R> pl = plastic_args<R>(m);
    if (m->method == METHOD_LARGE)
        k_elem_force_rhs<R, METHOD_LARGE>
            <<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl, v, kf_rhs, eforce_v);
    else if (m->method == METHOD_SVD)
        k_elem_force_rhs<R, METHOD_SVD>
            <<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl, v, kf_rhs, eforce_v);
    else
        k_elem_force_rhs<R, METHOD_POLAR>
            <<<g, kElemBlock, 0, s>>>(ev, x, m->rest_pos, (R*)m->eforce, pl, v, kf_rhs, eforce_v);
}

template <typename R, typename VIN, int DIR>
void launch_elem_dforce(TfemMesh* m, const VIN* dx, const R* pold, const CgScalars* cg, R fact, cudaStream_t s,
                        const R* dinv = nullptr)
{
    if (m->n_tets == 0) return;
    ElemView<R> ev = view<R>(m);
    const int g = elem_grid(m->n_tets);
    // the preconditioned variant is a separate instantiation: the CG
    // kernels carry no test for it
    if (m->method == METHOD_SMALL) {
        if (dinv)
            k_elem_dforce<R, VIN, METHOD_SMALL, DIR, 1>
                <<<g, kElemBlock, 0, s>>>(ev, dx, pold, cg, fact, (R*)m->eforce, dinv);
        else
            k_elem_dforce<R, VIN, METHOD_SMALL, DIR, 0>
                <<<g, kElemBlock, 0, s>>>(ev, dx, pold, cg, fact, (R*)m->eforce, nullptr);
    } else {
        if (dinv)
            k_elem_dforce<R, VIN, METHOD_LARGE, DIR, 1>
                <<<g, kElemBlock, 0, s>>>(ev, dx, pold, cg, fact, (R*)m->eforce, dinv);
        else
            k_elem_dforce<R, VIN, METHOD_LARGE, DIR, 0>
                <<<g, kElemBlock, 0, s>>>(ev, dx, pold, cg, fact, (R*)m->eforce, nullptr);
    }
}

// ---- assembled stiffness (buildStiffnessMatrix, TFEM.inl:1965-1993) --------
// One thread per 3x3 block (row node n1, column node n2) of df/dx: minus the
// sum, over the elements holding both nodes in element index order, of
// R^T S R with S = B1^T C B2 the element's coupling block in its frame (B
// from the nodes' strain-displacement values, C isotropic; R the element's
// current rotation rows, identity for method small). contrib holds the
// element storage slot << 4 | n1 << 2 | n2 per contribution.
template <typename R>
__global__ void __launch_bounds__(kNodeBlock) k_stiffness_blocks(ElemView<R> ev, int small,
                                                                 const int* __restrict__ cptr,
                                                                 const int* __restrict__ contrib, int n_blocks,
                                                                 double* __restrict__ out)
{
    for (int blk = blockIdx.x * blockDim.x + threadIdx.x; blk < n_blocks; blk += gridDim.x * blockDim.x) {
        double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int c = cptr[blk]; c < cptr[blk + 1]; ++c) {
            const int code = contrib[c];
            const size_t e = (size_t)(code >> 4);
            const int n1 = (code >> 2) & 3, n2 = code & 3;
            R K[3], J[12], Rm[9];
            load_KJ(ev, e, K, J);
            if (small) {
#pragma unroll
                for (int i = 0; i < 9; ++i) Rm[i] = (i % 4 == 0) ? R(1) : R(0);
            } else {
                load_rot(ev, e, Rm);
            }
            const R k0 = K[0], k1 = K[1], k2 = K[2];
            const R a1 = J[3 * n1], b1 = J[3 * n1 + 1], c1 = J[3 * n1 + 2];
            const R a2 = J[3 * n2], b2 = J[3 * n2 + 1], c2 = J[3 * n2 + 2];
            const R S[9] = {a1 * k0 * a2 + b1 * k2 * b2 + c1 * k2 * c2, a1 * k1 * b2 + b1 * k2 * a2,
                            a1 * k1 * c2 + c1 * k2 * a2,
                            b1 * k1 * a2 + a1 * k2 * b2, b1 * k0 * b2 + a1 * k2 * a2 + c1 * k2 * c2,
                            b1 * k1 * c2 + c1 * k2 * b2,
                            c1 * k1 * a2 + a1 * k2 * c2, c1 * k1 * b2 + b1 * k2 * c2,
                            c1 * k0 * c2 + b1 * k2 * b2 + a1 * k2 * a2};
            // W = R^T S R (world frame)
            R SR[9];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    SR[3 * i + j] = S[3 * i] * Rm[j] + S[3 * i + 1] * Rm[3 + j] + S[3 * i + 2] * Rm[6 + j];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const R w = Rm[i] * SR[j] + Rm[3 + i] * SR[3 + j] + Rm[6 + i] * SR[6 + j];
                    acc[3 * i + j] -= (double)w;
                }
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) out[9 * (size_t)blk + i] = acc[i];
    }
}

template <typename R>
void launch_stiffness_blocks(TfemMesh* m, const int* cptr, const int* contrib, int n_blocks, double* out,
                             cudaStream_t s)
{
    if (n_blocks <= 0) return;
    k_stiffness_blocks<R><<<node_grid(n_blocks), kNodeBlock, 0, s>>>(view<R>(m), m->method == METHOD_SMALL, cptr,
                                                                     contrib, n_blocks, out);
}

inline PatchView patch_view(TfemMesh* m)
{
    PatchView pv;
    pv.elem_start = m->pl.elem_start;
    pv.node_start = m->pl.node_start;
    pv.lnode_gid = m->pl.lnode_gid;
    pv.lnode_info = m->pl.lnode_info;
    pv.lrow = m->pl.lrow;
    pv.lslots = m->pl.lslots;
    pv.lconn = m->pl.lconn;
    pv.bnd_rowptr = m->pl.bnd_rowptr;
    pv.n_patches = m->pl.n_patches;
    pv.pe = m->pl.pe;
    pv.max_lnodes = m->pl.max_lnodes;
    return pv;
}

template <typename R>
size_t patch_smem_bytes(const TfemMesh* m)
{
    return patch_smem_size<R>(m->pl.pe, m->pl.max_lnodes);
}

// The CG update with the register cap chosen at preparation (MINB resident
// CTAs of kNodeBlock threads per SM).
template <typename R, int PC = 0, typename... A>
void launch_cg_update(const TfemMesh* m, int grid, cudaStream_t s, A... a)
{
    if (m->update_minb == 2)
        k_cg_update_patch<R, 2, PC><<<grid, kNodeBlock, 0, s>>>(a...);
    else if (m->update_minb == 3)
        k_cg_update_patch<R, 3, PC><<<grid, kNodeBlock, 0, s>>>(a...);
    else
        k_cg_update_patch<R, 4, PC><<<grid, kNodeBlock, 0, s>>>(a...);
}

// The CG matvec with the register cap chosen at preparation.
template <typename R, int MODE, int PC = 0, typename... A>
void launch_patch_matvec(const TfemMesh* m, size_t smem, cudaStream_t s, A... a)
{
    if (m->matvec_db)
        k_patch_matvec<R, MODE, PC, 9, true>
            <<<m->patch_grid, m->patch_threads, patch_smem_size_db<R>(m->pl.pe, m->pl.max_lnodes), s>>>(a...);
    else if (m->matvec_minb == 9)
        k_patch_matvec<R, MODE, PC, 9><<<m->patch_grid, m->patch_threads, smem, s>>>(a...);
    else
        k_patch_matvec<R, MODE, PC, 1><<<m->patch_grid, m->patch_threads, smem, s>>>(a...);
}

template <typename K>
int resident_grid(K kernel, int threads, size_t smem, int sms, int n_patches)
{
    int nb = 0;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem);
    long long g = (long long)(nb < 1 ? 1 : nb) * sms;
    if (g > kMaxDotBlocks) g = kMaxDotBlocks;
    if (g > n_patches) g = n_patches;
    return (int)(g < 1 ? 1 : g);
}

// Dynamic shared memory of a patch matvec kernel, with the largest
// shared-memory carve-out so that its resident CTAs are bounded by
// registers rather than by the L1 split.
template <typename K>
void patch_matvec_attrs(K kernel, size_t smem)
{
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
}

// k_patch_force_rhs for the rotated methods (mixed precision; the grid is
// set by prepare_patch).
template <typename R>
size_t force_patch_smem_bytes(const TfemMesh* m)
{
    return force_patch_smem_size<R>(m->pl.pe, m->pl.max_lnodes);
}

template <typename R>
void launch_patch_force_rhs(TfemMesh* m, const double* x, const double* v, R kf_rhs, int first_order, R* own,
                            R* partials, cudaStream_t s)
{
    if constexpr (is_mixed<R>::value) {
        const PlasticArgs<R> pl = plastic_args<R>(m);
        const PatchView pv = patch_view(m);
        const ElemView<R> ev = view<R>(m);
        const size_t smem = force_patch_smem_bytes<R>(m);
        const int g = m->force_patch_grid;
        if (m->method == METHOD_LARGE)
            k_patch_force_rhs<R, METHOD_LARGE>
                <<<g, m->force_threads, smem, s>>>(pv, ev, x, pl, v, kf_rhs, first_order, own, partials);
        else if (m->method == METHOD_SVD)
            k_patch_force_rhs<R, METHOD_SVD>
                <<<g, m->force_threads, smem, s>>>(pv, ev, x, pl, v, kf_rhs, first_order, own, partials);
        else
            k_patch_force_rhs<R, METHOD_POLAR>
                <<<g, m->force_threads, smem, s>>>(pv, ev, x, pl, v, kf_rhs, first_order, own, partials);
    }
}

// Sets the shared-memory attribute of the patch kernels and returns the grid
// (CTAs resident at once, capped by the dot-product partial array).
template <typename R>
int prepare_patch(TfemMesh* m)
{
    const size_t smem = patch_smem_bytes<R>(m);
    int dev = 0, sms = 0, nb1 = 0, nb2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // launch-shape knobs: threads per CTA (a multiple of 32 in [64, 256]), L2 prefetch of the
    // next patch, vectorised FP32 update
    int threads = 128;
    if (const char* e = getenv("SGB_PATCH_THREADS")) {
        const int t = atoi(e);
        if (t >= 64 && t <= kPatchMaxThreads && t % 32 == 0) threads = t;
    }
    m->patch_threads = threads;
    if (const char* e = getenv("SGB_PATCH_PREFETCH")) m->patch_prefetch = (e[0] == '1');
    if (const char* e = getenv("SGB_UPDATE_VEC4")) m->update_vec4 = (e[0] != '0');
    // CG update: register cap (2, 3 or 4 resident CTAs per SM; 4 measured
    // best) and a persistent grid (resident CTAs x SMs; 1.3 % faster steps
    // than one thread per group of four nodes, SGB_UPDATE_PERSIST=0)
    if (const char* e = getenv("SGB_UPDATE_MINB")) {
        const int v = atoi(e);
        if (v >= 2 && v <= 4) m->update_minb = v;
    }
    m->update_grid = 0;
    {
        const char* e = getenv("SGB_UPDATE_PERSIST");
        if (!e || e[0] != '0') {
            int nu = 0;
            if (m->update_minb == 2)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nu, k_cg_update_patch<R, 2>, kNodeBlock, 0);
            else if (m->update_minb == 3)
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nu, k_cg_update_patch<R, 3>, kNodeBlock, 0);
            else
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nu, k_cg_update_patch<R, 4>, kNodeBlock, 0);
            long long gu = (long long)(nu < 1 ? 1 : nu) * sms;
            if (gu > kMaxDotBlocks) gu = kMaxDotBlocks;
            m->update_grid = (int)gu;
        }
    }
    // CG matvec register cap: 9 resident 128-thread CTAs per SM (56
    // registers, no spills) or none (64 registers, 8 per SM). More warps pay
    // where the element data streams from DRAM: the 5.08 M-tet beam (0.4 GB of
    // element data, 3x L2) steps 2 % faster with the cap at 320 tets per
    // patch, while the 2.12 M-tet block (1.3x L2) and 256-tet patches step
    // slower. Hence the cap from 288 tets per patch and at least twice L2 of
    // element data (80 B per tet); SGB_MATVEC_MINB = 1 or 9 overrides.
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    m->matvec_minb = (m->pl.pe >= 288 && (double)m->n_tets * 80.0 >= 2.0 * (double)l2) ? 9 : 1;
    if (const char* e = getenv("SGB_MATVEC_MINB")) {
        const int v = atoi(e);
        if (v == 1 || v == 9) m->matvec_minb = v;
    }
    if (sizeof(R) != 4 || threads != kPatchThreads) m->matvec_minb = 1;
    // with the 9-CTA cap: two sets of slot lists and node values and no
    // barrier after phase 2 (24.4 KB per CTA at 320 tets still fits 9 per
    // SM; 0.2 % faster steps); SGB_MATVEC_DB=0 keeps one set
    m->matvec_db = m->matvec_minb == 9 ? 1 : 0;
    if (const char* e = getenv("SGB_MATVEC_DB"))
        if (e[0] == '0') m->matvec_db = 0;
    if (m->matvec_db) {
        const size_t sdb = patch_smem_size_db<R>(m->pl.pe, m->pl.max_lnodes);
        patch_matvec_attrs(k_patch_matvec<R, 1, 0, 9, true>, sdb);
        patch_matvec_attrs(k_patch_matvec<R, 2, 0, 9, true>, sdb);
        patch_matvec_attrs(k_patch_matvec<R, 1, 1, 9, true>, sdb);
        patch_matvec_attrs(k_patch_matvec<R, 2, 1, 9, true>, sdb);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb1, k_patch_matvec<R, 1, 0, 9, true>, threads, sdb);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, k_patch_matvec<R, 2, 0, 9, true>, threads, sdb);
    } else if (m->matvec_minb == 9) {
        patch_matvec_attrs(k_patch_matvec<R, 1, 0, 9>, smem);
        patch_matvec_attrs(k_patch_matvec<R, 2, 0, 9>, smem);
        patch_matvec_attrs(k_patch_matvec<R, 1, 1, 9>, smem);
        patch_matvec_attrs(k_patch_matvec<R, 2, 1, 9>, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb1, k_patch_matvec<R, 1, 0, 9>, threads, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, k_patch_matvec<R, 2, 0, 9>, threads, smem);
    } else {
        patch_matvec_attrs(k_patch_matvec<R, 1>, smem);
        patch_matvec_attrs(k_patch_matvec<R, 2>, smem);
        patch_matvec_attrs(k_patch_matvec<R, 1, 1>, smem);
        patch_matvec_attrs(k_patch_matvec<R, 2, 1>, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb1, k_patch_matvec<R, 1>, threads, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, k_patch_matvec<R, 2>, threads, smem);
    }
    int nb = nb1;
    nb = nb < nb2 ? nb : nb2;
    if (nb < 1) nb = 1;
    long long g = (long long)nb * sms;
    if (g > kMaxDotBlocks) g = kMaxDotBlocks;
    if (g > m->pl.n_patches) g = m->pl.n_patches;
    if (g < 1) g = 1;
    // the patch force / right-hand side pass (mixed precision, rotated
    // methods; SGB_PATCH_RHS=0 keeps the element-order pair of kernels)
    m->force_patch_grid = 0;
    if constexpr (is_mixed<R>::value) {
        const char* e = getenv("SGB_PATCH_RHS");
        if (m->method != METHOD_SMALL && !(e && e[0] == '0')) {
            const size_t fsmem = force_patch_smem_bytes<R>(m);
            // 160 threads: a 320-tet patch in two full element rounds and its
            // ~140 local nodes in one (128: a half-empty third element round
            // and a nearly empty second node round; 0.3 % faster steps)
            int ft = 160;
            if (const char* te = getenv("SGB_FORCE_THREADS")) {
                const int t = atoi(te);
                if (t >= 64 && t <= kPatchMaxThreads && t % 32 == 0) ft = t;
            }
            m->force_threads = ft;
            int nf = 0;
            if (m->method == METHOD_LARGE) {
                patch_matvec_attrs(k_patch_force_rhs<R, METHOD_LARGE>, fsmem);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nf, k_patch_force_rhs<R, METHOD_LARGE>, ft,
                                                              fsmem);
            } else if (m->method == METHOD_SVD) {
                patch_matvec_attrs(k_patch_force_rhs<R, METHOD_SVD>, fsmem);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nf, k_patch_force_rhs<R, METHOD_SVD>, ft,
                                                              fsmem);
            } else {
                patch_matvec_attrs(k_patch_force_rhs<R, METHOD_POLAR>, fsmem);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nf, k_patch_force_rhs<R, METHOD_POLAR>, ft,
                                                              fsmem);
            }
            long long gf = (long long)(nf < 1 ? 1 : nf) * sms;
            if (gf > m->pl.n_patches) gf = m->pl.n_patches;
            m->force_patch_grid = (int)(gf < 1 ? 1 : gf);
        }
    }
    {
        int na = 0;
        cudaFuncSetAttribute(k_patch_adddforce<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&na, k_patch_adddforce<R>, kPatchThreads, smem);
        long long ga = (long long)(na < 1 ? 1 : na) * sms;
        if (ga > m->pl.n_patches) ga = m->pl.n_patches;
        m->adddforce_grid = (int)(ga < 1 ? 1 : ga);
    }
    return (int)g;
}

// Public per-call operations (the drop-in for
// TetrahedronFEMForceFieldCuda3{f,d}_addForce / _addDForce).
template <typename R, typename VO>
void api_add_force(TfemMesh* m, const double* x, VO* f, cudaStream_t s)
{
    launch_elem_force<R>(m, x, s);
    NodeCSR csr{m->rowptr, m->slots};
    k_gather_accumulate<R, VO, false><<<node_grid(m->n_nodes), kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, f,
                                                                                   m->n_nodes);
}

template <typename R>
void api_add_dforce(TfemMesh* m, const R* dx, R* df, R kfactor, cudaStream_t s)
{
    if (m->pl.n_patches > 0 && m->method != METHOD_SMALL) {
        PatchView pv = patch_view(m);
        k_patch_adddforce<R><<<m->adddforce_grid, kPatchThreads, patch_smem_bytes<R>(m), s>>>(
                pv, view<R>(m), dx, kfactor, df, (R*)m->pl.partials, nullptr, 0);
        k_patch_fixup<R><<<node_grid(m->n_nodes), kNodeBlock, 0, s>>>(m->pl.bnd_rowptr, (const R*)m->pl.partials, df,
                                                                      m->n_nodes);
        return;
    }
    launch_elem_dforce<R, R, 0>(m, dx, nullptr, nullptr, kfactor, s);
    NodeCSR csr{m->rowptr, m->slots};
    k_gather_accumulate<R, R, true><<<node_grid(m->n_nodes), kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, df,
                                                                                 m->n_nodes);
}

// PCG before its first iteration (PCGLinearSolver.inl:194-214): the Jacobi
// diagonal from this step's rotations when a preconditioner is set (it
// returns at once on the steps between re-assemblies), then r = b - A x from
// the previous step's solution and r.z. CG with warmStart
// (CGLinearSolver.inl:95-99): the same start with r.r. Element-order
// kernels: once per step.

// The scene's mass operands. With separateGravity (UniformMass::addForce,
// UniformMass.inl:471-475) the mass adds no weight to the force; gravity
// enters the velocity after the position update instead (k_euler_update).
inline MassArgs scene_mass_args(const Scene* sc)
{
    const SceneParams& P = sc->prm;
    const double z = 0.0;
    return MassArgs{sc->node_mass, P.vertex_mass,
                    {P.separate_gravity ? z : P.gravity[0], P.separate_gravity ? z : P.gravity[1],
                     P.separate_gravity ? z : P.gravity[2]}};
}


inline SepGravity scene_sep_gravity(const Scene* sc)
{
    const SceneParams& P = sc->prm;
    SepGravity sg{{0.0, 0.0, 0.0}, P.separate_gravity ? 1 : 0};
    if (sg.on)
        for (int k = 0; k < 3; ++k) sg.hg[k] = P.gravity[k] * P.dt;
    return sg;
}

template <typename R>
void pcg_begin(Scene* sc, int mass_first, double mf, double kf, const SolveConsts& cons, double* dot_terms,
               cudaStream_t s)
{
    TfemMesh* m = sc->mesh;
    const int N = sc->n;
    const SceneParams& P = sc->prm;
    NodeCSR csr{m->rowptr, m->slots};
    const MassArgs ma = scene_mass_args(sc);
    const int ng = node_grid(N);
    R* dinv = (R*)sc->dinv;  // null: no preconditioner
    if (P.solver != 1) {
        launch_elem_dforce<R, R, 0>(m, (const R*)sc->xs, nullptr, sc->cg, (R)kf, s);
        k_pcg_start<R, FIN_WARM_START><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->xs,
                                                                 (const R*)sc->b, ma, mf, mass_first, sc->fixed,
                                                                 nullptr, (R*)sc->r, sc->cg, dot_terms, N, cons);
        return;
    }
    if (dinv) {
        ElemView<R> ev = view<R>(m);
        const int ge = elem_grid(m->n_tets);
        if (m->n_tets > 0) {
            if (m->method == METHOD_SMALL)
                k_elem_jacobi<R, METHOD_SMALL>
                    <<<ge, kElemBlock, 0, s>>>(ev, (R)(-kf), (R*)m->eforce, sc->cg, P.precond_rate);
            else
                k_elem_jacobi<R, METHOD_LARGE>
                    <<<ge, kElemBlock, 0, s>>>(ev, (R)(-kf), (R*)m->eforce, sc->cg, P.precond_rate);
        }
        k_gather_jacobi<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, ma, mf, mass_first, sc->fixed, dinv,
                                                     N, sc->cg, P.precond_rate);
    }
    launch_elem_dforce<R, R, 0>(m, (const R*)sc->xs, nullptr, sc->cg, (R)kf, s);
    k_pcg_start<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->xs, (const R*)sc->b, ma, mf,
                                             mass_first, sc->fixed, dinv, (R*)sc->r, sc->cg, dot_terms, N, cons);
}

// computeResidual at the end of a step: the scene's force at the new state
// (the force field runs again, with its side effects on plastic strains
// and rebuilt strain-displacement matrices, as the reference's computeForce
// does), then the residual's r.r into cg->residual.
template <typename R>
void launch_step_residual(Scene* sc, double* dot_terms, int mass_first, cudaStream_t s)
{
    TfemMesh* m = sc->mesh;
    const int N = sc->n;
    const SceneParams& P = sc->prm;
    NodeCSR csr{m->rowptr, m->slots};
    const MassArgs ma = scene_mass_args(sc);
    const int ng = node_grid(N);
    SolveConsts cons{P.cg_tolerance, P.cg_threshold, 1, 0, 0};
    launch_elem_force<R>(m, sc->x, s);
    k_gather_force<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->ext, ma, mass_first,
                                                (R*)sc->f, N);
    k_residual_dot<R><<<ng, kNodeBlock, 0, s>>>((const R*)sc->f, sc->fixed, P.dt, sc->cg, dot_terms, N, cons);
}

// One implicit Euler step of a scene (EulerImplicitSolver::solve,
// Sofa/Component/ODESolver/Backward/src/sofa/component/odesolver/backward/
// EulerImplicitSolver.cpp:83-341) as a fixed sequence of launches: the CG
// loop is unrolled to `iterations` and the kernels after convergence return
// at once, so the step can be captured in a CUDA graph.
template <typename R>
void scene_step(Scene* sc, double* dot_terms, int mass_first, cudaStream_t s)
{
    TfemMesh* m = sc->mesh;
    const int N = sc->n;
    const SceneParams& P = sc->prm;
    const double h = P.dt;
    NodeCSR csr{m->rowptr, m->slots};
    const MassArgs ma = scene_mass_args(sc);
    const int ng = node_grid(N);
    R* f = (R*)sc->f;
    R* b = (R*)sc->b;
    R* r = (R*)sc->r;
    R* p = (R*)sc->p;
    R* q = (R*)sc->q;
    R* xs = (R*)sc->xs;
    const bool pcg = P.solver == 1;
    R* dinv = pcg ? (R*)sc->dinv : nullptr;  // null: no preconditioner
    SolveConsts cons{P.cg_tolerance, P.cg_threshold, 1, pcg ? 1 : 0, P.warm_start};
    // f = F(x)
    launch_elem_force<R>(m, sc->x, s);
    k_gather_force<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->ext, ma, mass_first, f, N);
    // b = h (f - (h+rs) K v - rm M v); firstOrder: b = f
    const StepFactors F = step_factors(P);
    if (!P.first_order) launch_elem_dforce<R, double, 0>(m, sc->v, nullptr, sc->cg, (R)F.kf_rhs, s);
    k_gather_rhs<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, f, sc->v, ma, -P.rayleigh_mass, mass_first,
                                              h, sc->fixed, b, r, xs, sc->cg, dot_terms, N, cons, P.first_order);
    // CG (or PCG) on (mF M + kF K) dv = b, each component with its own
    // Rayleigh term folded into its factor
    const double mf = F.mf_mass;
    const double kf = F.kf_ff;
    if (pcg || P.warm_start) pcg_begin<R>(sc, mass_first, mf, kf, cons, dot_terms, s);
    for (int it = 1; it <= P.cg_iterations; ++it) {
        cons.it = it;
        if (it == 1) {
            launch_elem_dforce<R, R, 1>(m, r, p, sc->cg, (R)kf, s, dinv);
            if (dinv)
                k_gather_matvec<R, 1, 1><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, r, p, ma, mf,
                                                                   mass_first, sc->fixed, q, sc->cg, dot_terms, N,
                                                                   cons, dinv);
            else
                k_gather_matvec<R, 1><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, r, p, ma, mf,
                                                                mass_first, sc->fixed, q, sc->cg, dot_terms, N, cons);
        } else {
            launch_elem_dforce<R, R, 2>(m, r, p, sc->cg, (R)kf, s, dinv);
            if (dinv)
                k_gather_matvec<R, 2, 1><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, r, p, ma, mf,
                                                                   mass_first, sc->fixed, q, sc->cg, dot_terms, N,
                                                                   cons, dinv);
            else
                k_gather_matvec<R, 2><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, r, p, ma, mf,
                                                                mass_first, sc->fixed, q, sc->cg, dot_terms, N, cons);
        }
        if (dinv)
            k_cg_update<R, 1><<<ng, kNodeBlock, 0, s>>>(xs, r, p, q, sc->cg, dot_terms, N, cons, dinv);
        else
            k_cg_update<R><<<ng, kNodeBlock, 0, s>>>(xs, r, p, q, sc->cg, dot_terms, N, cons);
    }
    const double vd = (P.vdamping != 0.0) ? exp(-h * P.vdamping) : 1.0;
    k_euler_update<R><<<ng, kNodeBlock, 0, s>>>(sc->x, sc->v, xs, h, vd, sc->cg, N, P.first_order,
                                                P.project_velocity ? (const uint8_t*)sc->fixed : nullptr,
                                                scene_sep_gravity(sc));
    if (P.compute_residual) launch_step_residual<R>(sc, dot_terms, mass_first, s);
}

// The same step with the fused patch matvec: two launches per CG iteration
// (patch matvec + update), the CG direction p ping-pongs between two buffers.
// PCG (linear_solver = PCG) adds the warm start of pcg_begin and, with the
// Jacobi preconditioner, the PC = 1 kernels (z = diag^-1 r where the direction
// is formed, r.z in the update).
template <typename R>
void scene_step_patch(Scene* sc, int mass_first, cudaStream_t s)
{
    TfemMesh* m = sc->mesh;
    const int N = sc->n;
    const SceneParams& P = sc->prm;
    const double h = P.dt;
    NodeCSR csr{m->rowptr, m->slots};
    const MassArgs ma = scene_mass_args(sc);
    const int ng = node_grid(N);
    R* b = (R*)sc->b;
    R* r = (R*)sc->r;
    R* pb[2] = {(R*)sc->p, (R*)sc->p2};
    R* q = (R*)sc->q;
    R* xs = (R*)sc->xs;
    R* partials = (R*)m->pl.partials;
    const bool pcg = P.solver == 1;
    const R* dinv = pcg ? (const R*)sc->dinv : nullptr;
    SolveConsts cons{P.cg_tolerance, P.cg_threshold, 1, pcg ? 1 : 0, P.warm_start};
    const StepFactors F = step_factors(P);
    // forces and the right-hand side (sc->rhs_form): one pass over the
    // patches (element force and (h + rs) K v terms summed per patch in
    // shared memory) and one over the nodes; or one pass over the elements
    // (eforce_v) and one over the nodes in element order; or the four
    // kernels of scene_step. The same operations, equal to rounding
    // (summation order; the FP32 build may contract multiply-adds
    // differently in the fused kernels).
    if (sc->rhs_form == 2) {
        launch_patch_force_rhs<R>(m, sc->x, sc->v, (R)F.kf_rhs, P.first_order, q, partials, s);
        k_rhs_finish_patch<R><<<ng, kNodeBlock, 0, s>>>(q, partials, (const int*)m->pl.bnd_rowptr, (const R*)sc->ext,
                                                        sc->v, ma, -P.rayleigh_mass, h, sc->fixed, b, r, xs, sc->cg,
                                                        N, cons, P.first_order);
    } else if (sc->rhs_form == 1) {
        if (P.first_order)
            launch_elem_force<R>(m, sc->x, s);
        else
            launch_elem_force_rhs<R>(m, sc->x, sc->v, (R)F.kf_rhs, (R*)sc->eforce_v, s);
        k_gather_force_rhs<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->eforce_v,
                                                        (const R*)sc->ext, sc->v, ma, -P.rayleigh_mass, mass_first,
                                                        h, sc->fixed, b, r, xs, sc->cg, N, cons, P.first_order);
    } else {
        R* f = (R*)sc->f;
        launch_elem_force<R>(m, sc->x, s);
        k_gather_force<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->ext, ma, mass_first, f,
                                                    N);
        if (!P.first_order) launch_elem_dforce<R, double, 0>(m, sc->v, nullptr, sc->cg, (R)F.kf_rhs, s);
        k_gather_rhs<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, f, sc->v, ma, -P.rayleigh_mass,
                                                  mass_first, h, sc->fixed, b, r, xs, sc->cg, nullptr, N, cons,
                                                  P.first_order);
    }
    const double mf = F.mf_mass;
    const double kf = F.kf_ff;
    if (pcg || P.warm_start) pcg_begin<R>(sc, mass_first, mf, kf, cons, nullptr, s);
    PatchView pv = patch_view(m);
    ElemView<R> ev = view<R>(m);
    const size_t smem = patch_smem_bytes<R>(m);
    const int ng_update = is_mixed<R>::value ? node_grid((N + 3) / 4) : ng;
    const int gu = m->update_grid > 0 ? m->update_grid : (m->update_vec4 ? ng_update : ng);
    for (int it = 1; it <= P.cg_iterations; ++it) {
        cons.it = it;
        R* pold = pb[it & 1];
        R* pnew = pb[(it + 1) & 1];
        if (dinv) {
            if (it == 1)
                launch_patch_matvec<R, 1, 1>(m, smem, s, pv, ev, (const R*)r, (const R*)pold, pnew, sc->cg, (R)kf,
                                             ma, mf, (const uint8_t*)sc->fixed, q, partials, cons,
                                             m->patch_prefetch, (const R*)dinv);
            else
                launch_patch_matvec<R, 2, 1>(m, smem, s, pv, ev, (const R*)r, (const R*)pold, pnew, sc->cg, (R)kf,
                                             ma, mf, (const uint8_t*)sc->fixed, q, partials, cons,
                                             m->patch_prefetch, (const R*)dinv);
            launch_cg_update<R, 1>(m, gu, s, xs, r, (const R*)pnew, (const R*)q, (const R*)partials,
                                   (const int*)m->pl.bnd_rowptr, ma, mf, (const uint8_t*)sc->fixed, sc->cg, N, cons,
                                   m->update_vec4, dinv);
            continue;
        }
        if (it == 1)
            launch_patch_matvec<R, 1>(m, smem, s, pv, ev, (const R*)r, (const R*)pold, pnew, sc->cg, (R)kf, ma, mf,
                                      (const uint8_t*)sc->fixed, q, partials, cons, m->patch_prefetch);
        else
            launch_patch_matvec<R, 2>(m, smem, s, pv, ev, (const R*)r, (const R*)pold, pnew, sc->cg, (R)kf, ma, mf,
                                      (const uint8_t*)sc->fixed, q, partials, cons, m->patch_prefetch);
        launch_cg_update<R>(m, gu, s, xs, r, (const R*)pnew, (const R*)q, (const R*)partials,
                            (const int*)m->pl.bnd_rowptr, ma, mf, (const uint8_t*)sc->fixed, sc->cg, N, cons,
                            m->update_vec4);
    }
    const double vd = (P.vdamping != 0.0) ? exp(-h * P.vdamping) : 1.0;
    k_euler_update<R><<<ng, kNodeBlock, 0, s>>>(sc->x, sc->v, xs, h, vd, sc->cg, N, P.first_order,
                                                P.project_velocity ? (const uint8_t*)sc->fixed : nullptr,
                                                scene_sep_gravity(sc));
    if (P.compute_residual) launch_step_residual<R>(sc, nullptr, mass_first, s);
}

// The FP32 patch step with residual replacement every sc->replace_every CG
// iterations: forces, right-hand side and the replaced residuals in FP64 on
// the FP64 copy of the operator (sc->shadow), the CG iterations in FP32.
template <typename R>
void scene_step_refined(Scene* sc, int mass_first, cudaStream_t s)
{
    TfemMesh* m = sc->mesh;
    TfemMesh* sh = sc->shadow;
    const int N = sc->n;
    const SceneParams& P = sc->prm;
    const double h = P.dt;
    const MassArgs ma = scene_mass_args(sc);
    const int ng = node_grid(N);
    R* r = (R*)sc->r;
    R* pb[2] = {(R*)sc->p, (R*)sc->p2};
    R* q = (R*)sc->q;
    R* xs = (R*)sc->xs;
    R* partials = (R*)m->pl.partials;
    SolveConsts cons{P.cg_tolerance, P.cg_threshold, 1, 0, 0, sc->replace_every};
    // FP64: f = F(x) and b = h (f - (h+rs) K v - rm M v) on the FP64 operator
    NodeCSR csr64{sh->rowptr, sh->slots};
    launch_elem_force<double>(sh, sc->x, s);
    k_gather_force<double><<<ng, kNodeBlock, 0, s>>>(csr64, (const double*)sh->eforce, sc->ext64, ma, mass_first,
                                                     sc->w64, N);
    const StepFactors F = step_factors(P);
    launch_elem_dforce<double, double, 0>(sh, sc->v, nullptr, sc->cg, F.kf_rhs, s);
    k_gather_rhs<double><<<ng, kNodeBlock, 0, s>>>(csr64, (const double*)sh->eforce, sc->w64, sc->v, ma,
                                                   -P.rayleigh_mass, mass_first, h, sc->fixed, sc->b64, sc->r64,
                                                   sc->x64, sc->cg, nullptr, N, cons);
    // FP32: the plain mixed step's forces and right-hand side (b, r = b,
    // xs = 0); its CG start replaces the FP64 one's, so that a step whose
    // solve never meets the replacement condition is the plain mixed step,
    // bit for bit; b64 is used only by the replacements
    NodeCSR csr{m->rowptr, m->slots};
    launch_elem_force<R>(m, sc->x, s);
    k_gather_force<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->ext, ma, mass_first,
                                                (R*)sc->f, N);
    launch_elem_dforce<R, double, 0>(m, sc->v, nullptr, sc->cg, (R)F.kf_rhs, s);
    k_gather_rhs<R><<<ng, kNodeBlock, 0, s>>>(csr, (const R*)m->eforce, (const R*)sc->f, sc->v, ma,
                                              -P.rayleigh_mass, mass_first, h, sc->fixed, (R*)sc->b, r, xs, sc->cg,
                                              nullptr, N, cons);
    const double mf = F.mf_mass;
    const double kf = F.kf_ff;
    PatchView pv = patch_view(m);
    ElemView<R> ev = view<R>(m);
    const size_t smem = patch_smem_bytes<R>(m);
    const int ng_update = m->update_vec4 ? node_grid((N + 3) / 4) : ng;
    const int k = sc->replace_every;
    for (int it = 1; it <= P.cg_iterations; ++it) {
        cons.it = it;
        R* pold = pb[it & 1];
        R* pnew = pb[(it + 1) & 1];
        if (it == 1)
            launch_patch_matvec<R, 1>(m, smem, s, pv, ev, (const R*)r, (const R*)pold, pnew, sc->cg, (R)kf, ma, mf,
                                      (const uint8_t*)sc->fixed, q, partials, cons, m->patch_prefetch);
        else
            launch_patch_matvec<R, 2>(m, smem, s, pv, ev, (const R*)r, (const R*)pold, pnew, sc->cg, (R)kf, ma, mf,
                                      (const uint8_t*)sc->fixed, q, partials, cons, m->patch_prefetch);
        launch_cg_update<R>(m, m->update_grid > 0 ? m->update_grid : ng_update, s, xs, r, (const R*)pnew,
                            (const R*)q, (const R*)partials, (const int*)m->pl.bnd_rowptr, ma, mf,
                            (const uint8_t*)sc->fixed, sc->cg, N, cons, m->update_vec4);
        if (k > 0 && it % k == 0 && it < P.cg_iterations) {
            k_refine_accumulate<R><<<node_grid(3 * N), kNodeBlock, 0, s>>>(sc->x64, xs, sc->cg, it, N);
            cudaMemsetAsync(sc->w64, 0, sizeof(double) * 3 * (size_t)N, s);
            k_patch_adddforce<double><<<sh->patch_grid, kPatchThreads, patch_smem_bytes<double>(sh), s>>>(
                patch_view(sh), view<double>(sh), sc->x64, kf, sc->w64, (double*)sh->pl.partials,
                &sc->cg->replace_it, it);
            k_patch_fixup<double><<<ng, kNodeBlock, 0, s>>>(sh->pl.bnd_rowptr, (const double*)sh->pl.partials,
                                                            sc->w64, N, &sc->cg->replace_it, it);
            k_refine_residual<R><<<ng, kNodeBlock, 0, s>>>(sc->b64, sc->x64, sc->w64, ma, mf, sc->fixed, r, sc->cg,
                                                           N, cons);
        }
    }
    const double vd = (P.vdamping != 0.0) ? exp(-h * P.vdamping) : 1.0;
    k_euler_refined<R><<<ng, kNodeBlock, 0, s>>>(sc->x, sc->v, sc->x64, xs, h, vd, sc->cg, N,
                                                 P.project_velocity ? (const uint8_t*)sc->fixed : nullptr,
                                                 scene_sep_gravity(sc));
    if (P.compute_residual) launch_step_residual<R>(sc, nullptr, mass_first, s);
}

}  // namespace SGB_NS
