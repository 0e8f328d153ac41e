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

// rotation_large for the FP32 frame of the mixed path, which is made
// orthonormal to ~1e-14 afterwards: the unit vectors from the approximate
// reciprocal square root (an error of it turns the frame slightly, which
// adds no first-order strain), the same epsilon threshold.
__device__ __forceinline__ void normalize3_fast(float v[3])
{
    const float n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (n2 > RealTraits<float>::eps() * RealTraits<float>::eps()) {
        const float r = rsqrtf(n2);
        v[0] *= r;
        v[1] *= r;
        v[2] *= r;
    }
}

__device__ __forceinline__ void rotation_large_fast(const float eab[3], const float eac[3], float R[9])
{
    float ex[3] = {eab[0], eab[1], eab[2]};
    normalize3_fast(ex);
    float ez[3];
    cross3(ex, eac, ez);
    normalize3_fast(ez);
    float ey[3];
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
        T gamma, g2;
        if constexpr (std::is_same<T, float>::value) {
            // FP32: the scale gamma only sets how fast the iteration
            // converges, not where to, so it comes from the hardware's
            // approximate reciprocal square root and quotient; an error e in
            // 1/(gamma det) scales the converged factor by 1 + e/2, within
            // FP32 rounding (the mixed path then makes the factor orthonormal
            // to ~1e-14 in float-float)
            gamma = rsqrtf(fabsf(det) * rsqrtf(__fdividef(a_one * a_inf, m_one * m_inf)));
            g2 = __fdividef(0.5f, gamma * det);
        } else {
            gamma = sqrt(sqrt((a_one * a_inf) / (m_one * m_inf)) / fabs(det));
            g2 = T(0.5) / (gamma * det);
        }
        T g1 = gamma * T(0.5);
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

// J^T D on J's sparsity pattern (computeForce, TFEM.inl:329-355): the six
// strain components in the reference's term order.
template <typename T>
__device__ __forceinline__ void strain_jtd(const T D[12], const T J[12], T jd[6])
{
    jd[0] = J[0] * D[0] + J[3] * D[3] + J[6] * D[6] + J[9] * D[9];
    jd[1] = J[1] * D[1] + J[4] * D[4] + J[7] * D[7] + J[10] * D[10];
    jd[2] = J[2] * D[2] + J[5] * D[5] + J[8] * D[8] + J[11] * D[11];
    jd[3] = J[1] * D[0] + J[0] * D[1] + J[4] * D[3] + J[3] * D[4] + J[7] * D[6] + J[6] * D[7] + J[10] * D[9] +
            J[9] * D[10];
    jd[4] = J[2] * D[1] + J[1] * D[2] + J[5] * D[4] + J[4] * D[5] + J[8] * D[7] + J[7] * D[8] + J[11] * D[10] +
            J[10] * D[11];
    jd[5] = J[2] * D[0] + J[0] * D[2] + J[5] * D[3] + J[3] * D[5] + J[8] * D[6] + J[6] * D[8] + J[11] * D[9] +
            J[9] * D[11];
}

// F = J K jd (computeForce, TFEM.inl:374-412) without the factor.
template <typename T>
__device__ __forceinline__ void force_from_strain(T F[12], const T jd[6], const T K[3], const T J[12])
{
    const T k0 = K[0], k1 = K[1], k2 = K[2];
    T s0 = k0 * jd[0] + k1 * jd[1] + k1 * jd[2];
    T s1 = k1 * jd[0] + k0 * jd[1] + k1 * jd[2];
    T s2 = k1 * jd[0] + k1 * jd[1] + k0 * jd[2];
    T s3 = k2 * jd[3], s4 = k2 * jd[4], s5 = k2 * jd[5];
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
    T jd[6];
    strain_jtd(D, J, jd);
    force_from_strain(F, jd, K, J);
}

// ---- svd method: stable polar factor through a 3x3 SVD ---------------------
// Decompose<Real>::polarDecomposition_stable / SVD_stable /
// eigenDecomposition_iterative / QLAlgorithm
// (Sofa/framework/Helper/src/sofa/helper/decompose.inl:756-765, 1664-1825,
// 1563-1608, 1488-1558), for the inverted or nearly flat elements of the svd
// method. Row-major 3x3; operations in the reference's order.

// determinant(Mat<3,3>) (Sofa/framework/Type/src/sofa/type/Mat.h:987-996)
template <typename T>
__device__ __forceinline__ T det3(const T m[9])
{
    return m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[6] * m[1] * m[5] - m[0] * m[7] * m[5] - m[3] * m[1] * m[8] -
           m[6] * m[4] * m[2];
}

// operator*(Mat<3,3>, Mat<3,3>) (Mat.h:1443-1481)
template <typename T>
__device__ __forceinline__ void mul3(const T a[9], const T b[9], T r[9])
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}

// a * b^T (Mat::multTransposed, Mat.h:623-635)
template <typename T>
__device__ __forceinline__ void mul3_bt(const T a[9], const T b[9], T r[9])
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T s = a[3 * i] * b[3 * j];
            s += a[3 * i + 1] * b[3 * j + 1];
            s += a[3 * i + 2] * b[3 * j + 2];
            r[3 * i + j] = s;
        }
}

// invertMatrix(Mat<3,3>) (Mat.h:1170-1192): adjugate entries over det
template <typename T>
__host__ __device__ inline bool invert3(const T f[9], T d[9])
{
    const T det = f[0] * f[4] * f[8] + f[3] * f[7] * f[2] + f[6] * f[1] * f[5] - f[0] * f[7] * f[5] -
                  f[3] * f[1] * f[8] - f[6] * f[4] * f[2];
    if (fabs(det) <= RealTraits<T>::eps()) return false;
    d[0] = (f[4] * f[8] - f[7] * f[5]) / det;
    d[3] = (f[5] * f[6] - f[8] * f[3]) / det;
    d[6] = (f[3] * f[7] - f[6] * f[4]) / det;
    d[1] = (f[7] * f[2] - f[1] * f[8]) / det;
    d[4] = (f[8] * f[0] - f[2] * f[6]) / det;
    d[7] = (f[6] * f[1] - f[0] * f[7]) / det;
    d[2] = (f[1] * f[5] - f[4] * f[2]) / det;
    d[5] = (f[2] * f[3] - f[5] * f[0]) / det;
    d[8] = (f[0] * f[4] - f[3] * f[1]) / det;
    return true;
}

// QL with implicit shifts on a symmetric tridiagonal matrix (at most 32
// sweeps per eigenvalue), rotations accumulated into V
template <typename T>
__device__ inline void ql_tridiagonal(T diag[3], T sub[3], T V[9])
{
    for (int i0 = 0; i0 < 3; ++i0) {
        int i1;
        for (i1 = 0; i1 < 32; ++i1) {
            int i2;
            for (i2 = i0; i2 <= 1; ++i2) {
                const T tmp = fabs(diag[i2]) + fabs(diag[i2 + 1]);
                if (fabs(sub[i2]) + tmp == tmp) break;
            }
            if (i2 == i0) break;
            T g = (diag[i0 + 1] - diag[i0]) / (T(2) * sub[i0]);
            T r = sqrt(g * g + T(1));
            if (g < T(0))
                g = diag[i2] - diag[i0] + sub[i0] / (g - r);
            else
                g = diag[i2] - diag[i0] + sub[i0] / (g + r);
            T sn = T(1), cs = T(1), p = T(0);
            for (int i3 = i2 - 1; i3 >= i0; --i3) {
                T f = sn * sub[i3];
                const T b = cs * sub[i3];
                if (fabs(f) >= fabs(g)) {
                    cs = g / f;
                    r = sqrt(cs * cs + T(1));
                    sub[i3 + 1] = f * r;
                    sn = T(1) / r;
                    cs *= sn;
                } else {
                    sn = f / g;
                    r = sqrt(sn * sn + T(1));
                    sub[i3 + 1] = g * r;
                    cs = T(1) / r;
                    sn *= cs;
                }
                g = diag[i3 + 1] - p;
                r = (diag[i3] - g) * sn + T(2) * b * cs;
                p = sn * r;
                diag[i3 + 1] = g + p;
                g = cs * r - b;
                for (int i4 = 0; i4 < 3; ++i4) {
                    f = V[3 * i4 + i3 + 1];
                    V[3 * i4 + i3 + 1] = sn * V[3 * i4 + i3] + cs * f;
                    V[3 * i4 + i3] = cs * V[3 * i4 + i3] - sn * f;
                }
            }
            diag[i0] -= p;
            sub[i0] = g;
            sub[i2] = T(0);
        }
        if (i1 == 32) return;
    }
}

// Householder tridiagonalisation of the symmetric M, then QL
template <typename T>
__device__ inline void eigen_iterative3(const T M[9], T V[9], T diag[3])
{
    T sub[3];
    T m01 = M[1], m02 = M[2];
    const T m00 = M[0], m11 = M[4], m12 = M[5], m22 = M[8];
    diag[0] = m00;
    sub[2] = T(0);
    if (m02 != T(0)) {
        const T len = sqrt(m01 * m01 + m02 * m02);
        const T inv = T(1) / len;
        m01 *= inv;
        m02 *= inv;
        const T q = T(2) * m01 * m12 + m02 * (m22 - m11);
        diag[1] = m11 + m02 * q;
        diag[2] = m22 - m02 * q;
        sub[0] = len;
        sub[1] = m12 - m01 * q;
        V[0] = T(1), V[1] = T(0), V[2] = T(0);
        V[3] = T(0), V[4] = m01, V[5] = m02;
        V[6] = T(0), V[7] = m02, V[8] = -m01;
    } else {
        diag[1] = m11;
        diag[2] = m22;
        sub[0] = m01;
        sub[1] = m12;
#pragma unroll
        for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? T(1) : T(0);
    }
    ql_tridiagonal(diag, sub, V);
}

// SVD_stable: F = U diag(S) V^T with rotations U, V. Null singular values
// (S^2 below the zero tolerance) are rebuilt (one: cross product of the two
// valid columns; two: a frame around the valid column, with the reference's
// choice of components; three: identity) and an inversion goes into the
// smallest singular value.
template <typename T>
__device__ inline void svd_stable3(const T F[9], T U[9], T S[3], T V[9])
{
    T FtF[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) FtF[3 * i + j] = F[i] * F[j] + F[3 + i] * F[3 + j] + F[6 + i] * F[6 + j];
    eigen_iterative3(FtF, V, S);
    if (det3(V) < T(0))
        for (int i = 0; i < 3; ++i) V[3 * i] = -V[3 * i];
    int degenerated = 0;
    T S_1[3];
    for (int i = 0; i < 3; ++i) {
        if (S[i] < RealTraits<T>::polar_tol()) {
            degenerated++;
            S[i] = T(0);
            S_1[i] = T(1);
        } else {
            S[i] = sqrt(S[i]);
            S_1[i] = T(1) / S[i];
        }
    }
    int o0, o1, o2;
    if (S[0] < S[1]) {
        if (S[0] < S[2]) {
            o0 = 0;
            if (S[1] < S[2]) o1 = 1, o2 = 2;
            else o1 = 2, o2 = 1;
        } else {
            o0 = 2, o1 = 0, o2 = 1;
        }
    } else {
        if (S[1] < S[2]) {
            o0 = 1;
            if (S[0] < S[2]) o1 = 0, o2 = 2;
            else o1 = 2, o2 = 0;
        } else {
            o0 = 2, o1 = 1, o2 = 0;
        }
    }
    if (degenerated == 3) {
        for (int i = 0; i < 9; ++i) U[i] = (i % 4 == 0) ? T(1) : T(0);
    } else {
        T VS[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) VS[3 * i + j] = V[3 * i + j] * S_1[j];
        mul3(F, VS, U);
        if (degenerated == 1) {
            const T a[3] = {U[o1], U[3 + o1], U[6 + o1]};
            const T b[3] = {U[o2], U[3 + o2], U[6 + o2]};
            T c[3];
            cross3(a, b, c);
            U[o0] = c[0], U[3 + o0] = c[1], U[6 + o0] = c[2];
        } else if (degenerated == 2) {
            const T e2[3] = {U[o2], U[3 + o0], U[6 + o0]};
            T e0[3], e1[3];
            const T a0 = fabs(e2[0]), a1 = fabs(e2[1]), a2 = fabs(e2[2]);
            if (a0 > a1) {
                if (a0 > a2) e0[0] = T(0), e0[1] = T(1), e0[2] = T(0);
                else e0[0] = T(1), e0[1] = T(0), e0[2] = T(0);
            } else {
                if (a1 > a2) e0[0] = T(0), e0[1] = T(0), e0[2] = T(1);
                else e0[0] = T(1), e0[1] = T(0), e0[2] = T(0);
            }
            cross3(e2, e0, e1);
            normalize3(e1);
            cross3(e1, e2, e0);
            U[o0] = e0[0], U[3 + o0] = e0[1], U[6 + o0] = e0[2];
            U[o1] = e1[0], U[3 + o1] = e1[1], U[6 + o1] = e1[2];
        }
    }
    if (det3(U) < T(0)) {
        U[o0] *= T(-1);
        U[3 + o0] *= T(-1);
        U[6 + o0] *= T(-1);
        S[o0] *= T(-1);
    }
}

// polarDecomposition_stable: Q = U V^T
template <typename T>
__device__ inline void polar_stable3(const T M[9], T Q[9])
{
    T U[9], S[3], V[9];
    svd_stable3(M, U, S, V);
    mul3_bt(U, V, Q);
}

// The svd method's frame (accumulateForceSVD, TFEM.inl:1123-1150): with the
// edge rows A and the inverse rest edge matrix A0inv, F = A A0inv; when
// det F < 1e-6 (inverted or nearly flat) R = polar_stable(F) R0 (R0 = the
// initial rotation rows) and the function returns true; otherwise the
// caller takes the polar factor of A, as the polar method does.
template <typename T>
__device__ inline bool svd_frame(const T A[9], const T A0inv[9], const T R0[9], T R[9])
{
    T F[9];
    mul3(A, A0inv, F);
    if (!(det3(F) < T(1e-6))) return false;
    T Rs[9];
    polar_stable3(F, Rs);
    // Rs.multTransposed(initialRotations) with initialRotations = R0^T
    T R0t[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) R0t[3 * i + j] = R0[3 * j + i];
    mul3_bt(Rs, R0t, R);
    return true;
}


}  // namespace sgb
