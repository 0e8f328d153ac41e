// Per-element math of the corotational tetrahedral FEM, as device functions
// templated on the real type. The term order follows the reference CPU path
// (Sofa/Component/SolidMechanics/FEM/Elastic/src/sofa/component/solidmechanics/
// fem/elastic/TetrahedronFEMForceField.inl, cited as TFEM.inl below) so the
// FP64 instantiation stays within rounding of it; the FP32 instantiation is
// the mixed-precision path's element math.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

namespace sgb {

template <typename T> struct RealTraits;
template <> struct RealTraits<double> {
    // Decompose<double>::zeroTolerance (Sofa/framework/Helper/src/sofa/helper/decompose.h:384-387)
    static __host__ __device__ constexpr double polar_tol() { return 1e-8; }
    static __host__ __device__ constexpr double eps() { return 2.220446049250313e-16; }
};
template <> struct RealTraits<float> {
    // Decompose<float>::zeroTolerance (decompose.h:378-381)
    static __host__ __device__ constexpr float polar_tol() { return 1e-6f; }
    static __host__ __device__ constexpr float eps() { return 1.1920929e-07f; }
};

template <typename T> __device__ __forceinline__ T rsqrt_div_norm(T n2);

template <typename T>
__device__ __forceinline__ void cross3(const T a[3], const T b[3], T r[3])
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

// Vec::normalize with the epsilon threshold (Sofa/framework/Type/src/sofa/type/Vec.h:548-562).
template <typename T>
__device__ __forceinline__ void normalize3(T v[3])
{
    T n = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n > RealTraits<T>::eps()) {
        v[0] /= n;
        v[1] /= n;
        v[2] /= n;
    }
}

// computeRotationLarge (TFEM.inl:755-778) from the two edges ab and ac:
// rows of R are the unit edge ab, the in-plane unit vector and the normal.
template <typename T>
__device__ __forceinline__ void rotation_large(const T eab[3], const T eac[3], T R[9])
{
    T ex[3] = {eab[0], eab[1], eab[2]};
    normalize3(ex);
    T ez[3];
    cross3(ex, eac, ez);
    normalize3(ez);
    T ey[3];
    cross3(ez, ex, ey);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R[k] = ex[k];
        R[3 + k] = ey[k];
        R[6 + k] = ez[k];
    }
}

template <typename T>
__device__ __forceinline__ T one_norm3(const T a[9])
{
    T n = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T s = fabs(a[i]) + fabs(a[3 + i]) + fabs(a[6 + i]);
        n = s > n ? s : n;
    }
    return n;
}

template <typename T>
__device__ __forceinline__ T inf_norm3(const T a[9])
{
    T n = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T s = fabs(a[3 * i]) + fabs(a[3 * i + 1]) + fabs(a[3 * i + 2]);
        n = s > n ? s : n;
    }
    return n;
}

// Orthogonal polar factor by Higham's scaled Newton iteration on M^T with
// adjugate rows from cross products and gamma from one/inf norms, stopping
// when ||E_k||_1 <= ||M_k||_1 * tol (the published method the reference uses,
// Sofa/framework/Helper/src/sofa/helper/decompose.inl:672-723). A row-major,
// Q row-major. The iteration count is capped (max_iter) so a degenerate
// element cannot stall a warp; the cap is far above the 3-8 iterations near
// rotations need.
template <typename T>
__device__ __forceinline__ void polar3(const T A[9], T Q[9], int max_iter = 64)
{
    // FP32 runs one Newton step past the reference's float tolerance (1e-6):
    // the step is quadratic, so the factor ends orthogonal to FP32 rounding
    // instead of to the tolerance, which keeps the corotated strain bits
    int extra = std::is_same<T, float>::value ? 1 : 0;
    T Mk[9], Madj[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Mk[3 * i + j] = A[3 * j + i];
    T m_one = one_norm3(Mk), m_inf = inf_norm3(Mk);
    const T tol = RealTraits<T>::polar_tol();
    for (int it = 0; it < max_iter; ++it) {
        cross3(&Mk[3], &Mk[6], &Madj[0]);
        cross3(&Mk[6], &Mk[0], &Madj[3]);
        cross3(&Mk[0], &Mk[3], &Madj[6]);
        T det = Mk[0] * Madj[0] + Mk[1] * Madj[1] + Mk[2] * Madj[2];
        if (det == T(0)) break;
        T a_one = one_norm3(Madj), a_inf = inf_norm3(Madj);
        T gamma = sqrt(sqrt((a_one * a_inf) / (m_one * m_inf)) / fabs(det));
        T g1 = gamma * T(0.5);
        T g2 = T(0.5) / (gamma * det);
        T e_one = T(0);
        T colsum[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            T prev = Mk[i];
            Mk[i] = Mk[i] * g1 + Madj[i] * g2;
            colsum[i % 3] += fabs(prev - Mk[i]);
        }
        e_one = colsum[0];
        e_one = colsum[1] > e_one ? colsum[1] : e_one;
        e_one = colsum[2] > e_one ? colsum[2] : e_one;
        m_one = one_norm3(Mk);
        m_inf = inf_norm3(Mk);
        if (!(e_one > m_one * tol)) {
            if (extra-- <= 0) break;
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Q[3 * i + j] = Mk[3 * j + i];
}

// peudo_determinant_for_coef (TFEM.inl:211-215) of [m00 m01 m02; m10 m11 m12].
template <typename T>
__host__ __device__ __forceinline__ T pdet(T m00, T m01, T m02, T m10, T m11, T m12)
{
    return m01 * m12 - m11 * m02 - m00 * m12 + m10 * m02 + m00 * m11 - m10 * m01;
}

// computeStrainDisplacement (TFEM.inl:134-209): the 12 distinct values of J,
// three per node (J(3i,0), J(3i,3), J(3i,5)).
template <typename T>
__host__ __device__ __forceinline__ void strain_displacement(const T* a, const T* b, const T* c, const T* d, T J[12])
{
    J[0] = -pdet(b[1], c[1], d[1], b[2], c[2], d[2]);
    J[1] = pdet(b[0], c[0], d[0], b[2], c[2], d[2]);
    J[2] = -pdet(b[0], c[0], d[0], b[1], c[1], d[1]);
    J[3] = pdet(c[1], d[1], a[1], c[2], d[2], a[2]);
    J[4] = -pdet(c[0], d[0], a[0], c[2], d[2], a[2]);
    J[5] = pdet(c[0], d[0], a[0], c[1], d[1], a[1]);
    J[6] = -pdet(d[1], a[1], b[1], d[2], a[2], b[2]);
    J[7] = pdet(d[0], a[0], b[0], d[2], a[2], b[2]);
    J[8] = -pdet(d[0], a[0], b[0], d[1], a[1], b[1]);
    J[9] = pdet(a[1], b[1], c[1], a[2], b[2], c[2]);
    J[10] = -pdet(a[0], b[0], c[0], a[2], b[2], c[2]);
    J[11] = pdet(a[0], b[0], c[0], a[1], b[1], c[1]);
}

// computeForce (TFEM.inl:417-521): F = J (fact K) J^T D on J's sparsity
// pattern. K = {K(0,0), K(0,1), K(3,3)}; J = the 12 distinct values.
template <typename T>
__device__ __forceinline__ void element_force(T F[12], const T D[12], const T K[3], const T J[12], T fact)
{
    T jd0 = J[0] * D[0] + J[3] * D[3] + J[6] * D[6] + J[9] * D[9];
    T jd1 = J[1] * D[1] + J[4] * D[4] + J[7] * D[7] + J[10] * D[10];
    T jd2 = J[2] * D[2] + J[5] * D[5] + J[8] * D[8] + J[11] * D[11];
    T jd3 = J[1] * D[0] + J[0] * D[1] + J[4] * D[3] + J[3] * D[4] + J[7] * D[6] + J[6] * D[7] + J[10] * D[9] +
            J[9] * D[10];
    T jd4 = J[2] * D[1] + J[1] * D[2] + J[5] * D[4] + J[4] * D[5] + J[8] * D[7] + J[7] * D[8] + J[11] * D[10] +
            J[10] * D[11];
    T jd5 = J[2] * D[0] + J[0] * D[2] + J[5] * D[3] + J[3] * D[5] + J[8] * D[6] + J[6] * D[8] + J[11] * D[9] +
            J[9] * D[11];
    const T k0 = K[0], k1 = K[1], k2 = K[2];
    T s0 = (k0 * jd0 + k1 * jd1 + k1 * jd2) * fact;
    T s1 = (k1 * jd0 + k0 * jd1 + k1 * jd2) * fact;
    T s2 = (k1 * jd0 + k1 * jd1 + k0 * jd2) * fact;
    T s3 = (k2 * jd3) * fact;
    T s4 = (k2 * jd4) * fact;
    T s5 = (k2 * jd5) * fact;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const T a = J[3 * i], b = J[3 * i + 1], c = J[3 * i + 2];
        F[3 * i + 0] = a * s0 + b * s3 + c * s5;
        F[3 * i + 1] = b * s1 + a * s3 + c * s4;
        F[3 * i + 2] = c * s2 + b * s4 + a * s5;
    }
}

// computeForce without the factor (the addForce variant, TFEM.inl:293-415,
// plasticity off).
template <typename T>
__device__ __forceinline__ void element_force_nofact(T F[12], const T D[12], const T K[3], const T J[12])
{
    T jd0 = J[0] * D[0] + J[3] * D[3] + J[6] * D[6] + J[9] * D[9];
    T jd1 = J[1] * D[1] + J[4] * D[4] + J[7] * D[7] + J[10] * D[10];
    T jd2 = J[2] * D[2] + J[5] * D[5] + J[8] * D[8] + J[11] * D[11];
    T jd3 = J[1] * D[0] + J[0] * D[1] + J[4] * D[3] + J[3] * D[4] + J[7] * D[6] + J[6] * D[7] + J[10] * D[9] +
            J[9] * D[10];
    T jd4 = J[2] * D[1] + J[1] * D[2] + J[5] * D[4] + J[4] * D[5] + J[8] * D[7] + J[7] * D[8] + J[11] * D[10] +
            J[10] * D[11];
    T jd5 = J[2] * D[0] + J[0] * D[2] + J[5] * D[3] + J[3] * D[5] + J[8] * D[6] + J[6] * D[8] + J[11] * D[9] +
            J[9] * D[11];
    const T k0 = K[0], k1 = K[1], k2 = K[2];
    T s0 = k0 * jd0 + k1 * jd1 + k1 * jd2;
    T s1 = k1 * jd0 + k0 * jd1 + k1 * jd2;
    T s2 = k1 * jd0 + k1 * jd1 + k0 * jd2;
    T s3 = k2 * jd3, s4 = k2 * jd4, s5 = k2 * jd5;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const T a = J[3 * i], b = J[3 * i + 1], c = J[3 * i + 2];
        F[3 * i + 0] = a * s0 + b * s3 + c * s5;
        F[3 * i + 1] = b * s1 + a * s3 + c * s4;
        F[3 * i + 2] = c * s2 + b * s4 + a * s5;
    }
}

}  // namespace sgb
