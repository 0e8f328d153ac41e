/*
 * CPU oracle for the implicit corotational tetrahedral FEM step.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA path is
 * compared against; only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py may load it. The product (sofa_gb300/) never calls it.
 *
 * It restates, in plain C and in the reference's operation order, the CPU
 * path of SOFA v26.06 (file:line citations are paths inside that project):
 *
 *   TetrahedronFEMForceField   Sofa/Component/SolidMechanics/FEM/Elastic/src/
 *                              sofa/component/solidmechanics/fem/elastic/
 *                              TetrahedronFEMForceField.inl (cited as TFEM.inl)
 *   polar decomposition        Sofa/framework/Helper/src/sofa/helper/decompose.inl
 *   3x3 norms                  Sofa/framework/Type/src/sofa/type/Mat.h:1056-1080
 *   UniformMass                Sofa/Component/Mass/src/sofa/component/mass/UniformMass.inl
 *   DiagonalMass (tet lumping) Sofa/Component/Mass/src/sofa/component/mass/DiagonalMass.inl
 *   FixedProjectiveConstraint  Sofa/Component/Constraint/Projective/src/sofa/component/
 *                              constraint/projective/FixedProjectiveConstraint.inl
 *   CGLinearSolver             Sofa/Component/LinearSolver/Iterative/src/sofa/component/
 *                              linearsolver/iterative/CGLinearSolver.inl (+ .cpp)
 *   EulerImplicitSolver        Sofa/Component/ODESolver/Backward/src/sofa/component/
 *                              odesolver/backward/EulerImplicitSolver.cpp
 *   MechanicalObject vOps      Sofa/Component/StateContainer/src/sofa/component/
 *                              statecontainer/MechanicalObject.inl
 *
 * It is compiled with -ffp-contract=off so that every a*b+c rounds twice, as
 * the reference does on a target without fused multiply-add; the results are
 * then identical on x86-64 and aarch64.
 *
 * The multi-threaded mode (orc_set_threads > 1) follows the MultiThreading
 * plugin's ParallelTetrahedronFEMForceField (thread-local force buffers merged
 * after the element loop, applications/plugins/MultiThreading/src/
 * MultiThreading/component/solidmechanics/fem/elastic/
 * ParallelTetrahedronFEMForceField.inl:53-124); its sums are reordered, so it
 * is used for timing, not as the parity reference. The exact parallel mode
 * (orc_set_exact_parallel(1) with orc_set_threads > 1) computes each
 * element's corner terms in parallel into a per-element buffer and then lets
 * every node add its terms in element order, which is the serial loop's
 * order: its results are bit-identical to one thread, so it checks large
 * meshes. In both modes the element-wise vector operations of the solver run
 * in parallel (they have no reductions, so their bits do not change) and the
 * dot products stay serial, as MechanicalObject::vDot computes them.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_SMALL 0
#define ORC_LARGE 1
#define ORC_POLAR 2
#define ORC_SVD 3

/* ------------------------------------------------------------------------- */
/* small fixed-size helpers                                                   */
/* ------------------------------------------------------------------------- */

/* Vec::norm2 then sqrt, Vec::normalizeWithNorm with the default epsilon
 * threshold (Sofa/framework/Type/src/sofa/type/Vec.h:496-562). */
static void vec_normalize(double v[3])
{
    double n2 = v[0] * v[0];
    n2 += v[1] * v[1];
    n2 += v[2] * v[2];
    double n = sqrt(n2);
    if (n > 2.220446049250313e-16) {
        v[0] /= n;
        v[1] /= n;
        v[2] /= n;
    }
}

/* type::cross (Vec.h:775-780) */
static void vec_cross(const double a[3], const double b[3], double r[3])
{
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

/* Vec dot (Vec::operator*(Vec), Vec.h:406-412): left to right. */
static double vec_dot(const double a[3], const double b[3])
{
    double r = a[0] * b[0];
    r += a[1] * b[1];
    r += a[2] * b[2];
    return r;
}

/* Mat * Vec (Mat.h:577-587): r(i) = m(i,0)v0; r(i) += m(i,1)v1; ... */
static void mat_vec(const double m[9], const double v[3], double r[3])
{
    for (int i = 0; i < 3; ++i) {
        double s = m[3 * i + 0] * v[0];
        s += m[3 * i + 1] * v[1];
        s += m[3 * i + 2] * v[2];
        r[i] = s;
    }
}

static void mat_transpose(const double m[9], double t[9])
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[3 * i + j] = m[3 * j + i];
}

/* oneNorm / infNorm of a 3x3 (Mat.h:1056-1080). */
static double mat_one_norm(const double a[9])
{
    double norm = 0.0;
    for (int i = 0; i < 3; ++i) {
        double s = fabs(a[0 * 3 + i]) + fabs(a[1 * 3 + i]) + fabs(a[2 * 3 + i]);
        if (s > norm) norm = s;
    }
    return norm;
}

static double mat_inf_norm(const double a[9])
{
    double norm = 0.0;
    for (int i = 0; i < 3; ++i) {
        double s = fabs(a[i * 3 + 0]) + fabs(a[i * 3 + 1]) + fabs(a[i * 3 + 2]);
        if (s > norm) norm = s;
    }
    return norm;
}

/* Higham's scaled Newton iteration for the orthogonal polar factor, as in
 * Decompose<double>::polarDecomposition(M, Q) (decompose.inl:672-723) with
 * the FP64 tolerance 1e-8 (decompose.h:384-387). M and Q are row-major 3x3.
 * Returns the determinant of the last iterate. */
double orc_polar(const double M[9], double Q[9])
{
    double Mk[9], Ek[9], Madj[9];
    double det = 0.0, M_one, M_inf, E_one;
    const double tol = 1e-8;
    mat_transpose(M, Mk);
    M_one = mat_one_norm(Mk);
    M_inf = mat_inf_norm(Mk);
    do {
        vec_cross(&Mk[3], &Mk[6], &Madj[0]);
        vec_cross(&Mk[6], &Mk[0], &Madj[3]);
        vec_cross(&Mk[0], &Mk[3], &Madj[6]);
        det = Mk[0] * Madj[0] + Mk[1] * Madj[1] + Mk[2] * Madj[2];
        if (det == 0.0) break;
        double adj_one = mat_one_norm(Madj);
        double adj_inf = mat_inf_norm(Madj);
        double gamma = sqrt(sqrt((adj_one * adj_inf) / (M_one * M_inf)) / fabs(det));
        double g1 = gamma * 0.5;
        double g2 = 0.5 / (gamma * det);
        for (int i = 0; i < 9; ++i) {
            Ek[i] = Mk[i];
            Mk[i] = Mk[i] * g1 + Madj[i] * g2;
            Ek[i] -= Mk[i];
        }
        E_one = mat_one_norm(Ek);
        M_one = mat_one_norm(Mk);
        M_inf = mat_inf_norm(Mk);
    } while (E_one > M_one * tol);
    mat_transpose(Mk, Q);
    return det;
}

/* ------------------------------------------------------------------------- */
/* svd method: stable polar decomposition through a 3x3 SVD                   */
/* (Decompose<double>::polarDecomposition_stable, SVD_stable,                 */
/* eigenDecomposition_iterative and QLAlgorithm, decompose.inl:756-765,       */
/* 1664-1825, 1563-1608, 1488-1558). Matrices are row-major m[3*i+j].         */
/* ------------------------------------------------------------------------- */

/* determinant(Mat<3,3>) (Mat.h:987-996), terms in the reference's order */
static double mat_det(const double m[9])
{
    return m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[6] * m[1] * m[5] - m[0] * m[7] * m[5] -
           m[3] * m[1] * m[8] - m[6] * m[4] * m[2];
}

/* operator*(Mat<3,3>, Mat<3,3>) (Mat.h:1443-1481) */
static void mat_mul(const double a[9], const double b[9], double r[9])
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}

/* a * b^T (Mat::multTransposed, Mat.h:623-635) */
static void mat_mul_bt(const double a[9], const double b[9], double r[9])
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = a[3 * i] * b[3 * j];
            s += a[3 * i + 1] * b[3 * j + 1];
            s += a[3 * i + 2] * b[3 * j + 2];
            r[3 * i + j] = s;
        }
}

/* invertMatrix(Mat<3,3>) (Mat.h:1170-1192), each entry divided by det */
int orc_invert3(const double f[9], double d[9])
{
    const double det = mat_det(f);
    if (fabs(det) <= 2.220446049250313e-16) return 0; /* equalsZero (Mat.h:44-48) */
    d[0] = (f[4] * f[8] - f[7] * f[5]) / det;
    d[3] = (f[5] * f[6] - f[8] * f[3]) / det;
    d[6] = (f[3] * f[7] - f[6] * f[4]) / det;
    d[1] = (f[7] * f[2] - f[1] * f[8]) / det;
    d[4] = (f[8] * f[0] - f[2] * f[6]) / det;
    d[7] = (f[6] * f[1] - f[0] * f[7]) / det;
    d[2] = (f[1] * f[5] - f[4] * f[2]) / det;
    d[5] = (f[2] * f[3] - f[5] * f[0]) / det;
    d[8] = (f[0] * f[4] - f[3] * f[1]) / det;
    return 1;
}

/* QLAlgorithm for a symmetric tridiagonal matrix (decompose.inl:1488-1558):
 * implicit shifts, at most 32 sweeps per eigenvalue, rotations applied to V */
static void ql_algorithm(double diag[3], double sub[3], double V[9])
{
    for (int i0 = 0; i0 < 3; ++i0) {
        int i1;
        for (i1 = 0; i1 < 32; ++i1) {
            int i2;
            for (i2 = i0; i2 <= 1; ++i2) {
                const double tmp = fabs(diag[i2]) + fabs(diag[i2 + 1]);
                if (fabs(sub[i2]) + tmp == tmp) break;
            }
            if (i2 == i0) break;
            double g = (diag[i0 + 1] - diag[i0]) / (2.0 * sub[i0]);
            double r = sqrt(g * g + 1.0);
            if (g < 0.0)
                g = diag[i2] - diag[i0] + sub[i0] / (g - r);
            else
                g = diag[i2] - diag[i0] + sub[i0] / (g + r);
            double sn = 1.0, cs = 1.0, p = 0.0;
            for (int i3 = i2 - 1; i3 >= i0; --i3) {
                double f = sn * sub[i3];
                const double b = cs * sub[i3];
                if (fabs(f) >= fabs(g)) {
                    cs = g / f;
                    r = sqrt(cs * cs + 1.0);
                    sub[i3 + 1] = f * r;
                    sn = 1.0 / r;
                    cs *= sn;
                } else {
                    sn = f / g;
                    r = sqrt(sn * sn + 1.0);
                    sub[i3 + 1] = g * r;
                    cs = 1.0 / r;
                    sn *= cs;
                }
                g = diag[i3 + 1] - p;
                r = (diag[i3] - g) * sn + 2.0 * b * cs;
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
            sub[i2] = 0.0;
        }
        if (i1 == 32) return;
    }
}

/* eigenDecomposition_iterative (decompose.inl:1563-1608): Householder
 * tridiagonalisation of the symmetric M, then QL */
static void eigen_iterative(const double M[9], double V[9], double diag[3])
{
    double sub[3];
    double m01 = M[1], m02 = M[2];
    const double m00 = M[0], m11 = M[4], m12 = M[5], m22 = M[8];
    diag[0] = m00;
    sub[2] = 0.0;
    if (m02 != 0.0) {
        const double len = sqrt(m01 * m01 + m02 * m02);
        const double inv = 1.0 / len;
        m01 *= inv;
        m02 *= inv;
        const double q = 2.0 * m01 * m12 + m02 * (m22 - m11);
        diag[1] = m11 + m02 * q;
        diag[2] = m22 - m02 * q;
        sub[0] = len;
        sub[1] = m12 - m01 * q;
        V[0] = 1.0, V[1] = 0.0, V[2] = 0.0;
        V[3] = 0.0, V[4] = m01, V[5] = m02;
        V[6] = 0.0, V[7] = m02, V[8] = -m01;
    } else {
        diag[1] = m11;
        diag[2] = m22;
        sub[0] = m01;
        sub[1] = m12;
        for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    ql_algorithm(diag, sub, V);
}

/* SVD_stable (decompose.inl:1664-1825): F = U diag(S) V^T with U and V
 * rotations; a null singular value (S^2 below 1e-8) is rebuilt (one: from
 * the cross product of the two valid columns; two: an arbitrary orthogonal
 * frame around the valid column; three: identity) and an inversion is moved
 * into the smallest singular value. Returns 1 when degenerate or inverted. */
static int svd_stable(const double F[9], double U[9], double S[3], double V[9])
{
    double FtF[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) FtF[3 * i + j] = F[i] * F[j] + F[3 + i] * F[3 + j] + F[6 + i] * F[6 + j];
    eigen_iterative(FtF, V, S);
    if (mat_det(V) < 0.0)
        for (int i = 0; i < 3; ++i) V[3 * i] = -V[3 * i];
    int degenerated = 0;
    double S_1[3];
    for (int i = 0; i < 3; ++i) {
        if (S[i] < 1e-8) {
            degenerated++;
            S[i] = 0.0;
            S_1[i] = 1.0;
        } else {
            S[i] = sqrt(S[i]);
            S_1[i] = 1.0 / S[i];
        }
    }
    int o[3];
    if (S[0] < S[1]) {
        if (S[0] < S[2]) {
            o[0] = 0;
            if (S[1] < S[2]) o[1] = 1, o[2] = 2;
            else o[1] = 2, o[2] = 1;
        } else {
            o[0] = 2, o[1] = 0, o[2] = 1;
        }
    } else {
        if (S[1] < S[2]) {
            o[0] = 1;
            if (S[0] < S[2]) o[1] = 0, o[2] = 2;
            else o[1] = 2, o[2] = 0;
        } else {
            o[0] = 2, o[1] = 1, o[2] = 0;
        }
    }
    if (degenerated == 3) {
        for (int i = 0; i < 9; ++i) U[i] = (i % 4 == 0) ? 1.0 : 0.0;
    } else {
        double VS[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) VS[3 * i + j] = V[3 * i + j] * S_1[j];
        mat_mul(F, VS, U);
        if (degenerated == 1) {
            const double a[3] = {U[o[1]], U[3 + o[1]], U[6 + o[1]]};
            const double b[3] = {U[o[2]], U[3 + o[2]], U[6 + o[2]]};
            double c[3];
            vec_cross(a, b, c);
            U[o[0]] = c[0];
            U[3 + o[0]] = c[1];
            U[6 + o[0]] = c[2];
        } else if (degenerated == 2) {
            /* the reference takes edge2 = (U(0,o2), U(1,o0), U(2,o0)) */
            const double e2[3] = {U[o[2]], U[3 + o[0]], U[6 + o[0]]};
            double e0[3], e1[3];
            const double a0 = fabs(e2[0]), a1 = fabs(e2[1]), a2 = fabs(e2[2]);
            if (a0 > a1) {
                if (a0 > a2) e0[0] = 0, e0[1] = 1, e0[2] = 0;
                else e0[0] = 1, e0[1] = 0, e0[2] = 0;
            } else {
                if (a1 > a2) e0[0] = 0, e0[1] = 0, e0[2] = 1;
                else e0[0] = 1, e0[1] = 0, e0[2] = 0;
            }
            vec_cross(e2, e0, e1);
            vec_normalize(e1);
            vec_cross(e1, e2, e0);
            U[o[0]] = e0[0], U[3 + o[0]] = e0[1], U[6 + o[0]] = e0[2];
            U[o[1]] = e1[0], U[3 + o[1]] = e1[1], U[6 + o[1]] = e1[2];
        }
    }
    const int inverted = mat_det(U) < 0.0;
    if (inverted) {
        U[o[0]] *= -1.0;
        U[3 + o[0]] *= -1.0;
        U[6 + o[0]] *= -1.0;
        S[o[0]] *= -1.0;
    }
    return degenerated || inverted;
}

/* polarDecomposition_stable (decompose.inl:756-765): Q = U V^T */
int orc_polar_stable(const double M[9], double Q[9])
{
    double U[9], S[3], V[9];
    const int deg = svd_stable(M, U, S, V);
    mat_mul_bt(U, V, Q);
    return deg;
}

/* computeRotationLarge (TFEM.inl:755-778): rows of R are the unit edge
 * ab, the in-plane unit vector and the normal. */
static void rotation_large(const double* pa, const double* pb, const double* pc, double R[9])
{
    double ex[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    vec_normalize(ex);
    double ey[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
    double ez[3];
    vec_cross(ex, ey, ez);
    vec_normalize(ez);
    vec_cross(ez, ex, ey);
    for (int k = 0; k < 3; ++k) {
        R[0 + k] = ex[k];
        R[3 + k] = ey[k];
        R[6 + k] = ez[k];
    }
}

/* peudo_determinant_for_coef (TFEM.inl:211-215); m = [m00 m01 m02; m10 m11 m12]. */
static double pdet(double m00, double m01, double m02, double m10, double m11, double m12)
{
    return m01 * m12 - m11 * m02 - m00 * m12 + m10 * m02 + m00 * m11 - m10 * m01;
}

/* computeStrainDisplacement (TFEM.inl:134-209). The 12x6 J has three
 * distinct values per node i, stored as J3[3i+0] = J(3i,0) = J(3i+1,3) =
 * J(3i+2,5), J3[3i+1] = J(3i,3) = J(3i+1,1) = J(3i+2,4) and J3[3i+2] =
 * J(3i,5) = J(3i+1,4) = J(3i+2,2). */
static void strain_displacement(const double* a, const double* b, const double* c, const double* d,
                                double J3[12])
{
    J3[0] = -pdet(b[1], c[1], d[1], b[2], c[2], d[2]);
    J3[1] = pdet(b[0], c[0], d[0], b[2], c[2], d[2]);
    J3[2] = -pdet(b[0], c[0], d[0], b[1], c[1], d[1]);

    J3[3] = pdet(c[1], d[1], a[1], c[2], d[2], a[2]);
    J3[4] = -pdet(c[0], d[0], a[0], c[2], d[2], a[2]);
    J3[5] = pdet(c[0], d[0], a[0], c[1], d[1], a[1]);

    J3[6] = -pdet(d[1], a[1], b[1], d[2], a[2], b[2]);
    J3[7] = pdet(d[0], a[0], b[0], d[2], a[2], b[2]);
    J3[8] = -pdet(d[0], a[0], b[0], d[1], a[1], b[1]);

    J3[9] = pdet(a[1], b[1], c[1], a[2], b[2], c[2]);
    J3[10] = -pdet(a[0], b[0], c[0], a[2], b[2], c[2]);
    J3[11] = pdet(a[0], b[0], c[0], a[1], b[1], c[1]);
}

/* Plasticity settings of computeForce (TFEM.inl:51-53): max_threshold > 0
 * turns the plastic step on. */
typedef struct {
    double max_threshold, yield_threshold, creep;
} orc_plastic;

/* computeForce (TFEM.inl:293-415, and :417-521 with `fact`): F = J K J^T D
 * using only J's non-zero pattern, in the reference's term order.
 * K3 = {K(0,0), K(0,1), K(3,3)}. fact is applied to K J^T D when use_fact is
 * set. With `ps` (the element's plastic strain) and plasticity on, the
 * plastic step of :357-370 updates ps and the force uses J^T D - ps. */
static void compute_force_pl(double F[12], const double D[12], const double K3[3], const double J3[12],
                             int use_fact, double fact, double* ps, const orc_plastic* pl)
{
#define JA(i) J3[3 * (i) + 0]
#define JB(i) J3[3 * (i) + 1]
#define JC(i) J3[3 * (i) + 2]
    double JtD[6], KJtD[6];
    JtD[0] = JA(0) * D[0] + JA(1) * D[3] + JA(2) * D[6] + JA(3) * D[9];
    JtD[1] = JB(0) * D[1] + JB(1) * D[4] + JB(2) * D[7] + JB(3) * D[10];
    JtD[2] = JC(0) * D[2] + JC(1) * D[5] + JC(2) * D[8] + JC(3) * D[11];
    JtD[3] = JB(0) * D[0] + JA(0) * D[1] + JB(1) * D[3] + JA(1) * D[4] + JB(2) * D[6] + JA(2) * D[7] +
             JB(3) * D[9] + JA(3) * D[10];
    JtD[4] = JC(0) * D[1] + JB(0) * D[2] + JC(1) * D[4] + JB(1) * D[5] + JC(2) * D[7] + JB(2) * D[8] +
             JC(3) * D[10] + JB(3) * D[11];
    JtD[5] = JC(0) * D[0] + JA(0) * D[2] + JC(1) * D[3] + JA(1) * D[5] + JC(2) * D[6] + JA(2) * D[8] +
             JC(3) * D[9] + JA(3) * D[11];

    if (ps && pl && pl->max_threshold > 0) {
        double el[6], n2, p2;
        for (int i = 0; i < 6; ++i) el[i] = JtD[i] - ps[i]; /* elasticStrain = JtD - plasticStrain */
        n2 = el[0] * el[0];                                  /* Vec::norm2 (Vec.h:483-493) */
        for (int i = 1; i < 6; ++i) n2 += el[i] * el[i];
        if (n2 > pl->yield_threshold * pl->yield_threshold)
            for (int i = 0; i < 6; ++i) ps[i] += el[i] * pl->creep;
        p2 = ps[0] * ps[0];
        for (int i = 1; i < 6; ++i) p2 += ps[i] * ps[i];
        if (p2 > pl->max_threshold * pl->max_threshold) {
            const double s = pl->max_threshold / sqrt(p2); /* helper::rsqrt(double) is sqrt (rmath.h:131-138) */
            for (int i = 0; i < 6; ++i) ps[i] *= s;
        }
        for (int i = 0; i < 6; ++i) JtD[i] -= ps[i];
    }

    const double k0 = K3[0], k1 = K3[1], k2 = K3[2];
    KJtD[0] = k0 * JtD[0] + k1 * JtD[1] + k1 * JtD[2];
    KJtD[1] = k1 * JtD[0] + k0 * JtD[1] + k1 * JtD[2];
    KJtD[2] = k1 * JtD[0] + k1 * JtD[1] + k0 * JtD[2];
    KJtD[3] = k2 * JtD[3];
    KJtD[4] = k2 * JtD[4];
    KJtD[5] = k2 * JtD[5];
    if (use_fact)
        for (int i = 0; i < 6; ++i) KJtD[i] *= fact;

    for (int i = 0; i < 4; ++i) {
        F[3 * i + 0] = JA(i) * KJtD[0] + JB(i) * KJtD[3] + JC(i) * KJtD[5];
        F[3 * i + 1] = JB(i) * KJtD[1] + JA(i) * KJtD[3] + JC(i) * KJtD[4];
        F[3 * i + 2] = JC(i) * KJtD[2] + JB(i) * KJtD[4] + JA(i) * KJtD[5];
    }
#undef JA
#undef JB
#undef JC
}

static void compute_force(double F[12], const double D[12], const double K3[3], const double J3[12],
                          int use_fact, double fact)
{
    compute_force_pl(F, D, K3, J3, use_fact, fact, NULL, NULL);
}

/* ------------------------------------------------------------------------- */
/* thread pool (one parallel region at a time)                               */
/* ------------------------------------------------------------------------- */

static int g_threads = 1;
static int g_exact = 0;

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int orc_get_threads(void) { return g_threads; }
void orc_set_exact_parallel(int on) { g_exact = on ? 1 : 0; }

typedef void (*orc_task_fn)(void* ctx, int tid, int nthreads);
typedef struct {
    orc_task_fn fn;
    void* ctx;
    int tid, n;
} orc_task;

static void* orc_task_main(void* p)
{
    orc_task* t = (orc_task*)p;
    t->fn(t->ctx, t->tid, t->n);
    return NULL;
}

static void parallel_run(orc_task_fn fn, void* ctx, int n)
{
    if (n <= 1) {
        fn(ctx, 0, 1);
        return;
    }
    pthread_t th[256];
    orc_task tk[256];
    if (n > 256) n = 256;
    for (int t = 0; t < n; ++t) {
        tk[t].fn = fn;
        tk[t].ctx = ctx;
        tk[t].tid = t;
        tk[t].n = n;
        if (t > 0) pthread_create(&th[t], NULL, orc_task_main, &tk[t]);
    }
    fn(ctx, 0, n);
    for (int t = 1; t < n; ++t) pthread_join(th[t], NULL);
}

static void chunk(long total, int tid, int n, long* b, long* e)
{
    long per = (total + n - 1) / n;
    *b = per * tid;
    *e = *b + per;
    if (*b > total) *b = total;
    if (*e > total) *e = total;
}

/* ------------------------------------------------------------------------- */
/* TetrahedronFEMForceField                                                   */
/* ------------------------------------------------------------------------- */

typedef struct orc_fem {
    int n_nodes, n_tets, method;
    int32_t* tets;     /* 4 per element */
    double* rest;      /* initialPoints, 3 per node */
    double* K3;        /* 3 per element */
    double* J3;        /* 12 per element */
    double* R0t;       /* _initialRotations, 9 per element */
    double* rot;       /* rotations (= R^T), 9 per element */
    double* rest_rot;  /* _rotatedInitialElements, 12 per element */
    double* A0inv;     /* svd: _initialTransformation (inverse rest edge matrix), 9 per element */
    double rest_volume;
    double* plastic;   /* _plasticStrains, 6 per element (NULL until plasticity is turned on) */
    double* lame;      /* elemLambda, elemMu (TFEM.inl:278-282), 2 per element */
    orc_plastic pl;
    double* tl_buf;    /* thread-local force buffers for the threaded mode */
    int tl_threads;
    double* ebuf;      /* exact parallel mode: 12 corner terms per element */
    int32_t* nrow;     /* exact parallel mode: node -> (element*4 + corner) CSR, */
    int32_t* nslot;    /* rows in increasing order */
    int update_stiffness; /* Data updateStiffnessMatrix (polar, svd) */
} orc_fem;

/* BaseLinearElasticityFEMForceField::getVecRealInElement
 * (BaseLinearElasticityFEMForceField.inl:114-144): entry e when the vector is
 * longer than e, else entry 0. */
static double per_element(const double* v, int n, int e, int n_tets)
{
    (void)n_tets;
    return (n > e) ? v[e] : v[0];
}

orc_fem* orc_fem_create(int n_nodes, const double* rest, int n_tets, const int32_t* tets,
                        const double* young, int n_young, const double* poisson, int n_poisson,
                        const double* lsf, int n_lsf, int method)
{
    orc_fem* m = (orc_fem*)calloc(1, sizeof(orc_fem));
    m->n_nodes = n_nodes;
    m->n_tets = n_tets;
    m->method = method;
    m->tets = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)n_tets);
    memcpy(m->tets, tets, sizeof(int32_t) * 4 * (size_t)n_tets);
    m->rest = (double*)malloc(sizeof(double) * 3 * (size_t)n_nodes);
    memcpy(m->rest, rest, sizeof(double) * 3 * (size_t)n_nodes);
    m->K3 = (double*)calloc(3 * (size_t)n_tets, sizeof(double));
    m->J3 = (double*)calloc(12 * (size_t)n_tets, sizeof(double));
    m->R0t = (double*)calloc(9 * (size_t)n_tets, sizeof(double));
    m->rot = (double*)calloc(9 * (size_t)n_tets, sizeof(double));
    m->rest_rot = (double*)calloc(12 * (size_t)n_tets, sizeof(double));
    if (method == ORC_SVD) m->A0inv = (double*)calloc(9 * (size_t)n_tets, sizeof(double));
    m->lame = (double*)calloc(2 * (size_t)n_tets + 1, sizeof(double));

    for (int e = 0; e < n_tets; ++e) {
        const int32_t* t = &tets[4 * e];
        const double *pa = &rest[3 * t[0]], *pb = &rest[3 * t[1]], *pc = &rest[3 * t[2]],
                     *pd = &rest[3 * t[3]];
        /* computeMaterialStiffness (TFEM.inl:256-291) */
        double E = per_element(young, n_young, e, n_tets);
        double nu = per_element(poisson, n_poisson, e, n_tets);
        double f = (n_lsf > 0) ? lsf[(size_t)e * (size_t)n_lsf / (size_t)n_tets] : 1.0;
        E = f * E;
        double s = (E * (1 - nu)) / ((1 + nu) * (1 - 2 * nu));
        double k0 = 1.0, k1 = nu / (1 - nu), k2 = (1 - 2 * nu) / (2 * (1 - nu));
        k0 *= s;
        k1 *= s;
        k2 *= s;
        m->lame[2 * e] = k1; /* elemLambda = K(0,1), elemMu = K(3,3) before the volume division */
        m->lame[2 * e + 1] = k2;
        /* geometry::Tetrahedron::volume (Geometry/.../Tetrahedron.h:55-83) */
        double ea[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
        double eb[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
        double ec[3] = {pd[0] - pa[0], pd[1] - pa[1], pd[2] - pa[2]};
        double cr[3];
        vec_cross(ea, eb, cr);
        double vol = fabs(vec_dot(cr, ec) / 6.0);
        m->rest_volume += vol;
        k0 /= vol * 36;
        k1 /= vol * 36;
        k2 /= vol * 36;
        m->K3[3 * e + 0] = k0;
        m->K3[3 * e + 1] = k1;
        m->K3[3 * e + 2] = k2;

        double* rr = &m->rest_rot[12 * e];
        if (method == ORC_SMALL) {
            /* initSmall (TFEM.inl:526-532) */
            strain_displacement(pa, pb, pc, pd, &m->J3[12 * e]);
            for (int i = 0; i < 9; ++i) m->R0t[9 * e + i] = m->rot[9 * e + i] = (i % 4 == 0);
        } else {
            double R[9];
            if (method == ORC_LARGE) {
                /* initLarge (TFEM.inl:835-868) */
                rotation_large(pa, pb, pc, R);
            } else {
                /* initPolar (TFEM.inl:993-1023); initSVD (:1090-1119) also
                 * keeps the inverse of the rest edge matrix */
                double A[9] = {ea[0], ea[1], ea[2], eb[0], eb[1], eb[2], ec[0], ec[1], ec[2]};
                if (method == ORC_SVD) (void)orc_invert3(A, &m->A0inv[9 * e]);
                orc_polar(A, R);
            }
            mat_transpose(R, &m->R0t[9 * e]);
            memcpy(&m->rot[9 * e], &m->R0t[9 * e], sizeof(double) * 9);
            mat_vec(R, pa, &rr[0]);
            mat_vec(R, pb, &rr[3]);
            mat_vec(R, pc, &rr[6]);
            mat_vec(R, pd, &rr[9]);
            if (method == ORC_LARGE) {
                for (int i = 1; i < 4; ++i)
                    for (int k = 0; k < 3; ++k) rr[3 * i + k] -= rr[k];
                rr[0] = rr[1] = rr[2] = 0.0;
            }
            strain_displacement(&rr[0], &rr[3], &rr[6], &rr[9], &m->J3[12 * e]);
        }
    }
    return m;
}

void orc_fem_destroy(orc_fem* m)
{
    if (!m) return;
    free(m->tets);
    free(m->rest);
    free(m->K3);
    free(m->J3);
    free(m->R0t);
    free(m->rot);
    free(m->rest_rot);
    free(m->A0inv);
    free(m->plastic);
    free(m->lame);
    free(m->tl_buf);
    free(m->ebuf);
    free(m->nrow);
    free(m->nslot);
    free(m);
}

/* Element e's contribution to addForce (TFEM.inl:534-623 small, :870-986
 * large, :1025-1079 polar): out[3i+k] is what the element adds to f at its
 * node i. Also stores rotations[e]. */
static void element_force_terms(orc_fem* m, int e, const double* p, double out[12])
{
    const int32_t* t = &m->tets[4 * e];
    const double* K3 = &m->K3[3 * e];
    const double* J3 = &m->J3[12 * e];
    const double* rr = &m->rest_rot[12 * e];
    double D[12], F[12];
    if (m->method == ORC_SMALL) {
        const double* ip = m->rest;
        const int a = t[0];
        D[0] = D[1] = D[2] = 0.0;
        for (int i = 1; i < 4; ++i)
            for (int k = 0; k < 3; ++k)
                D[3 * i + k] = ip[3 * t[i] + k] - ip[3 * a + k] - p[3 * t[i] + k] + p[3 * a + k];
        compute_force_pl(F, D, K3, J3, 0, 0.0, m->plastic ? &m->plastic[6 * e] : NULL, &m->pl);
        memcpy(out, F, sizeof(double) * 12);
        return;
    }
    double R[9], def[12];
    if (m->method == ORC_LARGE) {
        rotation_large(&p[3 * t[0]], &p[3 * t[1]], &p[3 * t[2]], R);
    } else {
        const double *p0 = &p[3 * t[0]], *p1 = &p[3 * t[1]], *p2 = &p[3 * t[2]], *p3 = &p[3 * t[3]];
        double A[9] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], p2[0] - p0[0], p2[1] - p0[1],
                       p2[2] - p0[2], p3[0] - p0[0], p3[1] - p0[1], p3[2] - p0[2]};
        int stable = 0;
        if (m->method == ORC_SVD) {
            /* accumulateForceSVD (TFEM.inl:1123-1184): F = A A0^-1; an
             * inverted or nearly flat element (det F < 1e-6) takes the
             * stable SVD polar factor of F times the initial rotation */
            double F[9];
            mat_mul(A, &m->A0inv[9 * e], F);
            if (mat_det(F) < 1e-6) {
                double Rs[9];
                orc_polar_stable(F, Rs);
                mat_mul_bt(Rs, &m->R0t[9 * e], R);
                stable = 1;
            }
        }
        if (!stable) orc_polar(A, R);
    }
    double* rot = &m->rot[9 * e];
    mat_transpose(R, rot);
    for (int i = 0; i < 4; ++i) mat_vec(R, &p[3 * t[i]], &def[3 * i]);
    if (m->method == ORC_LARGE) {
        def[3] -= def[0];
        def[6] -= def[0];
        def[7] -= def[1];
        def[9] -= def[0];
        def[10] -= def[1];
        def[11] -= def[2];
        D[0] = D[1] = D[2] = 0.0;
        D[3] = rr[3] - def[3];
        D[4] = D[5] = 0.0;
        D[6] = rr[6] - def[6];
        D[7] = rr[7] - def[7];
        D[8] = 0.0;
        D[9] = rr[9] - def[9];
        D[10] = rr[10] - def[10];
        D[11] = rr[11] - def[11];
    } else {
        for (int i = 0; i < 12; ++i) D[i] = rr[i] - def[i];
        /* updateStiffnessMatrix: computeStrainDisplacement on the deformed
         * positions in the element frame before the force
         * (accumulateForcePolar TFEM.inl:1063-1067, accumulateForceSVD
         * :1174-1177) */
        if (m->update_stiffness) strain_displacement(&def[0], &def[3], &def[6], &def[9], &m->J3[12 * e]);
    }
    compute_force_pl(F, D, K3, J3, 0, 0.0, m->plastic ? &m->plastic[6 * e] : NULL, &m->pl);
    for (int i = 0; i < 4; ++i) mat_vec(rot, &F[3 * i], &out[3 * i]);
}

/* f += element e's addForce terms, node by node in corner order */
static void element_force(orc_fem* m, int e, const double* p, double* f)
{
    const int32_t* t = &m->tets[4 * e];
    double c[12];
    element_force_terms(m, e, p, c);
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 3; ++k) f[3 * t[i] + k] += c[3 * i + k];
}

/* applyStiffnessSmall / applyStiffnessCorotational (TFEM.inl:721-749,
 * 1193-1237): R K (R^T dx) * fact for element e; out[3i+k] is what the
 * element subtracts from df at its node i (df += -F for small is the same
 * operation: x + (-y) and x - y round alike). */
static void element_dforce_terms(const orc_fem* m, int e, const double* x, double fact, double out[12])
{
    const int32_t* t = &m->tets[4 * e];
    const double* K3 = &m->K3[3 * e];
    const double* J3 = &m->J3[12 * e];
    double X[12], F[12];
    if (m->method == ORC_SMALL) {
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) X[3 * i + k] = x[3 * t[i] + k];
        compute_force(F, X, K3, J3, 1, fact);
        memcpy(out, F, sizeof(double) * 12);
        return;
    }
    const double* r = &m->rot[9 * e]; /* rotations[i] = R^T */
    for (int i = 0; i < 4; ++i) {
        const double* xi = &x[3 * t[i]];
        for (int k = 0; k < 3; ++k) X[3 * i + k] = r[0 * 3 + k] * xi[0] + r[1 * 3 + k] * xi[1] + r[2 * 3 + k] * xi[2];
    }
    compute_force(F, X, K3, J3, 1, fact);
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 3; ++k)
            out[3 * i + k] = r[k * 3 + 0] * F[3 * i + 0] + r[k * 3 + 1] * F[3 * i + 1] + r[k * 3 + 2] * F[3 * i + 2];
}

/* df -= element e's addDForce terms, node by node in corner order */
static void element_dforce(const orc_fem* m, int e, const double* x, double* df, double fact)
{
    const int32_t* t = &m->tets[4 * e];
    double c[12];
    element_dforce_terms(m, e, x, fact, c);
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 3; ++k) df[3 * t[i] + k] -= c[3 * i + k];
}

typedef struct {
    orc_fem* m;
    const double* in;
    double* out;
    double fact;
    int dforce;
} fem_job;

static void fem_job_run(void* ctx, int tid, int n)
{
    fem_job* j = (fem_job*)ctx;
    long b, e;
    chunk(j->m->n_tets, tid, n, &b, &e);
    double* buf = j->m->tl_buf + (size_t)tid * 3 * (size_t)j->m->n_nodes;
    memset(buf, 0, sizeof(double) * 3 * (size_t)j->m->n_nodes);
    for (long i = b; i < e; ++i) {
        if (j->dforce)
            element_dforce(j->m, (int)i, j->in, buf, j->fact);
        else
            element_force(j->m, (int)i, j->in, buf);
    }
}

typedef struct {
    orc_fem* m;
    double* out;
    int nt;
} merge_job;

static void merge_job_run(void* ctx, int tid, int n)
{
    merge_job* j = (merge_job*)ctx;
    long b, e;
    long len = 3L * j->m->n_nodes;
    chunk(len, tid, n, &b, &e);
    for (int t = 0; t < j->nt; ++t) {
        const double* buf = j->m->tl_buf + (size_t)t * (size_t)len;
        for (long i = b; i < e; ++i) j->out[i] += buf[i];
    }
}

static void fem_threaded(orc_fem* m, const double* in, double* out, double fact, int dforce)
{
    int nt = g_threads;
    if (m->tl_threads < nt) {
        free(m->tl_buf);
        m->tl_buf = (double*)malloc(sizeof(double) * 3 * (size_t)m->n_nodes * (size_t)nt);
        m->tl_threads = nt;
    }
    fem_job j = {m, in, out, fact, dforce};
    parallel_run(fem_job_run, &j, nt);
    merge_job mj = {m, out, nt};
    parallel_run(merge_job_run, &mj, nt);
}

/* Exact parallel mode: element terms into ebuf (parallel over elements),
 * then each node adds or subtracts its terms in increasing (element, corner)
 * order (parallel over nodes) -- the serial element loop's order for every
 * node, so the sums are bit-identical to one thread. */
typedef struct {
    orc_fem* m;
    const double* in;
    double* out;
    double fact;
    int dforce;
} exact_job;

static void exact_elem_run(void* ctx, int tid, int n)
{
    exact_job* j = (exact_job*)ctx;
    long b, e;
    chunk(j->m->n_tets, tid, n, &b, &e);
    for (long i = b; i < e; ++i) {
        if (j->dforce)
            element_dforce_terms(j->m, (int)i, j->in, j->fact, &j->m->ebuf[12 * (size_t)i]);
        else
            element_force_terms(j->m, (int)i, j->in, &j->m->ebuf[12 * (size_t)i]);
    }
}

static void exact_node_run(void* ctx, int tid, int n)
{
    exact_job* j = (exact_job*)ctx;
    const orc_fem* m = j->m;
    long b, e;
    chunk(m->n_nodes, tid, n, &b, &e);
    for (long v = b; v < e; ++v) {
        double* o = &j->out[3 * (size_t)v];
        for (int32_t s = m->nrow[v]; s < m->nrow[v + 1]; ++s) {
            const double* c = &m->ebuf[3 * (size_t)m->nslot[s]];
            for (int k = 0; k < 3; ++k) {
                if (j->dforce)
                    o[k] -= c[k];
                else
                    o[k] += c[k];
            }
        }
    }
}

static void fem_exact(orc_fem* m, const double* in, double* out, double fact, int dforce)
{
    if (!m->ebuf) {
        const size_t E = (size_t)m->n_tets, N = (size_t)m->n_nodes;
        m->ebuf = (double*)malloc(sizeof(double) * 12 * E + 1);
        m->nrow = (int32_t*)calloc(N + 1, sizeof(int32_t));
        m->nslot = (int32_t*)malloc(sizeof(int32_t) * 4 * E + 1);
        for (size_t s = 0; s < 4 * E; ++s) m->nrow[m->tets[s] + 1]++;
        for (size_t v = 0; v < N; ++v) m->nrow[v + 1] += m->nrow[v];
        int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (N + 1));
        memcpy(fill, m->nrow, sizeof(int32_t) * (N + 1));
        for (size_t s = 0; s < 4 * E; ++s) m->nslot[fill[m->tets[s]]++] = (int32_t)s;
        free(fill);
    }
    exact_job j = {m, in, out, fact, dforce};
    parallel_run(exact_elem_run, &j, g_threads);
    parallel_run(exact_node_run, &j, g_threads);
}

/* addForce (TFEM.inl:1548-1604): f += internal forces at positions x. */
void orc_fem_add_force(orc_fem* m, const double* x, double* f)
{
    if (g_threads > 1 && g_exact) {
        fem_exact(m, x, f, 0.0, 0);
        return;
    }
    if (g_threads > 1) {
        fem_threaded(m, x, f, 0.0, 0);
        return;
    }
    for (int e = 0; e < m->n_tets; ++e) element_force(m, e, x, f);
}

/* addDForce (TFEM.inl:1606-1636): df += -kFactor K dx. */
void orc_fem_add_dforce(orc_fem* m, const double* dx, double* df, double kfactor)
{
    if (g_threads > 1 && g_exact) {
        fem_exact(m, dx, df, kfactor, 1);
        return;
    }
    if (g_threads > 1) {
        fem_threaded(m, dx, df, kfactor, 1);
        return;
    }
    for (int e = 0; e < m->n_tets; ++e) element_dforce(m, e, dx, df, kfactor);
}

/* Element data for the known-answer tests: out[0:9] initial rotation (R0^T),
 * out[9:18] current rotation (R^T), out[18:30] rotated rest coordinates,
 * out[30:33] K(0,0), K(0,1), K(3,3), out[33:45] the 12 distinct J values. */
void orc_fem_element(const orc_fem* m, int e, double* out)
{
    memcpy(out, &m->R0t[9 * e], 9 * sizeof(double));
    memcpy(out + 9, &m->rot[9 * e], 9 * sizeof(double));
    memcpy(out + 18, &m->rest_rot[12 * e], 12 * sizeof(double));
    memcpy(out + 30, &m->K3[3 * e], 3 * sizeof(double));
    memcpy(out + 33, &m->J3[12 * e], 12 * sizeof(double));
}

double orc_fem_rest_volume(const orc_fem* m) { return m->rest_volume; }

/* updateStiffnessMatrix (TFEM.inl:49) for methods polar and svd: every
 * addForce rebuilds J from the deformed element (see element_force_terms).
 * The large method's partial rebuild (:908-921) is not restated. */
void orc_fem_set_update_stiffness(orc_fem* m, int on)
{
    m->update_stiffness = (on && (m->method == ORC_POLAR || m->method == ORC_SVD)) ? 1 : 0;
}

/* plasticMaxThreshold / plasticYieldThreshold / plasticCreep; the plastic
 * strain starts at zero when plasticity is first turned on. */
void orc_fem_set_plasticity(orc_fem* m, double max_threshold, double yield_threshold, double creep)
{
    if (max_threshold > 0 && !m->plastic) m->plastic = (double*)calloc(6 * (size_t)m->n_tets + 1, sizeof(double));
    m->pl.max_threshold = max_threshold;
    m->pl.yield_threshold = yield_threshold;
    m->pl.creep = creep;
}

/* invertMatrix, general square case (Sofa/framework/Type/src/sofa/type/
 * Mat.h:1102-1168), for 4x4: Gauss-Jordan with full pivoting. Returns 0 when
 * a pivot is within machine epsilon of zero (equalsZero, Mat.h:46-49). */
static int invert4(const double from[16], double dest[16])
{
    double m1[16], m2[16];
    int r[4] = {0}, c[4] = {0}, row[4] = {0}, col[4] = {0};
    for (int i = 0; i < 16; ++i) {
        m1[i] = from[i];
        m2[i] = (i % 5 == 0) ? 1.0 : 0.0;
    }
    for (int k = 0; k < 4; ++k) {
        double pivot = 0;
        for (int i = 0; i < 4; ++i) {
            if (row[i]) continue;
            for (int j = 0; j < 4; ++j) {
                double t;
                if (col[j]) continue;
                t = m1[4 * i + j];
                if (t < 0) t = -t;
                if (t > pivot) {
                    pivot = t;
                    r[k] = i;
                    c[k] = j;
                }
            }
        }
        if (fabs(pivot) <= DBL_EPSILON) return 0;
        row[r[k]] = col[c[k]] = 1;
        pivot = m1[4 * r[k] + c[k]];
        for (int j = 0; j < 4; ++j) m1[4 * r[k] + j] /= pivot;
        m1[4 * r[k] + c[k]] = 1;
        for (int j = 0; j < 4; ++j) m2[4 * r[k] + j] /= pivot;
        for (int i = 0; i < 4; ++i) {
            if (i == r[k]) continue;
            double f = m1[4 * i + c[k]];
            for (int j = 0; j < 4; ++j) m1[4 * i + j] -= m1[4 * r[k] + j] * f;
            m1[4 * i + c[k]] = 0;
            for (int j = 0; j < 4; ++j) m2[4 * i + j] -= m2[4 * r[k] + j] * f;
        }
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            if (c[j] == i) row[i] = r[j];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) dest[4 * i + j] = m2[4 * row[i] + j];
    return 1;
}

/* computeVonMisesStress (TFEM.inl:2197-2374): per element von Mises stress
 * from the corotational strain (mode 1, large/polar/svd) or the Green strain
 * (mode 2), and per node the mean over the node's elements in element order.
 * vmn may be NULL. Returns 0, or -1 for mode 1 with method small (the
 * reference marks the component invalid, :1441-1445). */
int orc_fem_von_mises(const orc_fem* m, int mode, const double* X, double* vme, double* vmn)
{
    if (mode == 1 && m->method == ORC_SMALL) return -1;
    for (int el = 0; el < m->n_tets; ++el) {
        const int32_t* t = &m->tets[4 * el];
        double mv[16], shf[16] = {0}, g[9], strain[9], v[6], sg[6], tr = 0.0, q;
        /* elemShapeFun (:1527-1541) */
        for (int k = 0; k < 4; ++k) {
            mv[4 * k] = 1.0;
            for (int l = 1; l < 4; ++l) mv[4 * k + l] = m->rest[3 * t[k] + l - 1];
        }
        if (!invert4(mv, shf)) memset(shf, 0, sizeof(shf));
        if (mode == 2) {
            double U[4][3];
            for (int i = 0; i < 4; ++i)
                for (int k = 0; k < 3; ++k) U[i][k] = X[3 * t[i] + k] - m->rest[3 * t[i] + k];
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    g[3 * k + l] = 0.0;
                    for (int i = 0; i < 4; ++i) g[3 * k + l] += shf[4 * (l + 1) + i] * U[i][k];
                }
            /* 0.5 (gradU + gradU^T + gradU^T gradU) */
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double sym = g[3 * i + j] + g[3 * j + i];
                    double tt = g[i] * g[j] + g[3 + i] * g[3 + j] + g[6 + i] * g[6 + j];
                    strain[3 * i + j] = 0.5 * (sym + tt);
                }
        } else {
            double R[9], def[12], D[12];
            const double* rr = &m->rest_rot[12 * el];
            const double *p0 = &X[3 * t[0]], *p1 = &X[3 * t[1]], *p2 = &X[3 * t[2]], *p3 = &X[3 * t[3]];
            if (m->method == ORC_LARGE) {
                rotation_large(p0, p1, p2, R);
            } else {
                double A[9] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], p2[0] - p0[0], p2[1] - p0[1],
                               p2[2] - p0[2], p3[0] - p0[0], p3[1] - p0[1], p3[2] - p0[2]};
                orc_polar(A, R);
            }
            for (int i = 0; i < 4; ++i) mat_vec(R, &X[3 * t[i]], &def[3 * i]);
            if (m->method == ORC_LARGE) {
                def[3] -= def[0];
                def[6] -= def[0];
                def[7] -= def[1];
                def[9] -= def[0];
                def[10] -= def[1];
                def[11] -= def[2];
                for (int i = 0; i < 12; ++i) D[i] = 0.0;
                D[3] = rr[3] - def[3];
                D[6] = rr[6] - def[6];
                D[7] = rr[7] - def[7];
                D[9] = rr[9] - def[9];
                D[10] = rr[10] - def[10];
                D[11] = rr[11] - def[11];
            } else {
                for (int i = 0; i < 12; ++i) D[i] = rr[i] - def[i];
            }
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) {
                    g[3 * k + l] = 0.0;
                    for (int i = 0; i < 4; ++i) g[3 * k + l] += shf[4 * (l + 1) + i] * D[3 * i + k];
                }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) strain[3 * i + j] = 0.5 * (g[3 * i + j] + g[3 * j + i]);
        }
        v[0] = strain[0];
        v[1] = strain[4];
        v[2] = strain[8];
        v[3] = strain[5];
        v[4] = strain[2];
        v[5] = strain[1];
        for (int k = 0; k < 3; ++k) {
            tr += v[k];
            sg[k] = v[k] * 2 * m->lame[2 * el + 1];
        }
        for (int k = 3; k < 6; ++k) sg[k] = v[k] * 2 * m->lame[2 * el + 1];
        for (int k = 0; k < 3; ++k) sg[k] += m->lame[2 * el] * tr;
        q = sg[0] * sg[0] + sg[1] * sg[1] + sg[2] * sg[2] - sg[0] * sg[1] - sg[1] * sg[2] - sg[2] * sg[0] +
            3 * sg[3] * sg[3] + 3 * sg[4] * sg[4] + 3 * sg[5] * sg[5];
        vme[el] = sqrt(q);
        if (vme[el] < 1e-10) vme[el] = 0.0;
    }
    if (vmn) {
        int* cnt = (int*)calloc((size_t)m->n_nodes + 1, sizeof(int));
        memset(vmn, 0, sizeof(double) * (size_t)m->n_nodes);
        for (int el = 0; el < m->n_tets; ++el)
            for (int c = 0; c < 4; ++c) {
                vmn[m->tets[4 * el + c]] += vme[el];
                cnt[m->tets[4 * el + c]]++;
            }
        for (int n = 0; n < m->n_nodes; ++n)
            if (cnt[n]) vmn[n] /= (double)cnt[n];
        free(cnt);
    }
    return 0;
}

/* _plasticStrains, 6 per element (zeros before plasticity is turned on). */
void orc_fem_plastic_strain(const orc_fem* m, double* out)
{
    for (size_t i = 0; i < 6 * (size_t)m->n_tets; ++i) out[i] = m->plastic ? m->plastic[i] : 0.0;
}

/* ------------------------------------------------------------------------- */
/* Scene: MechanicalObject + mass + force fields + projective constraint,    */
/* integrated by EulerImplicitSolver with CGLinearSolver<GraphScattered>.    */
/* ------------------------------------------------------------------------- */

typedef struct orc_scene {
    int n;               /* nodes */
    orc_fem* fem;        /* borrowed, may be NULL */
    int mass_kind;       /* 0: UniformMass, 1: DiagonalMass */
    double vertex_mass;  /* UniformMass vertexMass */
    double* node_mass;   /* DiagonalMass per-node masses */
    double g[3];
    int* fixed;
    int n_fixed;
    int fix_all;
    double* ext;         /* MechanicalObject externalForce, may be NULL */
    /* optional isotropic anchor springs: f -= k (x - anchor) (test helper) */
    double spring_k;
    double* anchor;
    int mass_first;      /* component order in the node: mass before the FEM */
    /* EulerImplicitSolver data */
    double dt, rs, rm, vdamping;
    /* CGLinearSolver data */
    int cg_iters;
    double cg_tol, cg_threshold;
    long time_step_count;
    /* state + solver vectors */
    double *x, *v, *f, *b, *xs, *p, *q, *r;
    /* statistics of the last solve */
    int last_iters;
    double last_err;
    /* linear solver: 0 CGLinearSolver, 1 PCGLinearSolver; Jacobi preconditioner */
    int solver, precond, precond_rate;
    int warm_start; /* CGLinearSolver warmStart */
    double* dinv;
    /* the components' own Rayleigh coefficients (force field rayleighStiffness,
     * mass rayleighMass), EulerImplicitSolver firstOrder,
     * FixedProjectiveConstraint activate_projectVelocity */
    double ff_rs, mass_rm;
    int first_order, project_velocity, trapezoidal;
    double cur_bf; /* bFactor of the matrix being applied (0 for the right-hand side) */
    int compute_residual; /* EulerImplicitSolver computeResidual */
    double residual;      /* its Data `residual` after the last step */
    int separate_gravity; /* the mass's separateGravity */
} orc_scene;

orc_scene* orc_scene_create(orc_fem* fem, int n_nodes, int mass_kind, double vertex_mass,
                            const double* node_mass, const double* gravity, const int32_t* fixed,
                            int n_fixed, int fix_all, double dt, double rs, double rm, double vdamping,
                            int cg_iters, double cg_tol, double cg_threshold, int mass_first)
{
    orc_scene* s = (orc_scene*)calloc(1, sizeof(orc_scene));
    size_t n3 = 3 * (size_t)n_nodes;
    s->n = n_nodes;
    s->fem = fem;
    s->mass_kind = mass_kind;
    s->vertex_mass = vertex_mass;
    if (mass_kind == 1) {
        s->node_mass = (double*)malloc(sizeof(double) * (size_t)n_nodes);
        memcpy(s->node_mass, node_mass, sizeof(double) * (size_t)n_nodes);
    }
    memcpy(s->g, gravity, sizeof(double) * 3);
    s->n_fixed = n_fixed;
    s->fixed = (int*)malloc(sizeof(int) * (size_t)(n_fixed > 0 ? n_fixed : 1));
    for (int i = 0; i < n_fixed; ++i) s->fixed[i] = fixed[i];
    s->fix_all = fix_all;
    s->dt = dt;
    s->rs = rs;
    s->rm = rm;
    s->vdamping = vdamping;
    s->cg_iters = cg_iters;
    s->cg_tol = cg_tol;
    s->cg_threshold = cg_threshold;
    s->mass_first = mass_first;
    s->x = (double*)calloc(n3, sizeof(double));
    s->v = (double*)calloc(n3, sizeof(double));
    s->f = (double*)calloc(n3, sizeof(double));
    s->b = (double*)calloc(n3, sizeof(double));
    s->xs = (double*)calloc(n3, sizeof(double));
    s->p = (double*)calloc(n3, sizeof(double));
    s->q = (double*)calloc(n3, sizeof(double));
    s->r = (double*)calloc(n3, sizeof(double));
    if (fem) memcpy(s->x, fem->rest, sizeof(double) * n3);
    return s;
}

void orc_scene_destroy(orc_scene* s)
{
    if (!s) return;
    free(s->node_mass);
    free(s->fixed);
    free(s->ext);
    free(s->dinv);
    free(s->anchor);
    free(s->x);
    free(s->v);
    free(s->f);
    free(s->b);
    free(s->xs);
    free(s->p);
    free(s->q);
    free(s->r);
    free(s);
}

void orc_scene_set_state(orc_scene* s, const double* x, const double* v)
{
    size_t n3 = 3 * (size_t)s->n;
    if (x) memcpy(s->x, x, sizeof(double) * n3);
    if (v) memcpy(s->v, v, sizeof(double) * n3);
}

void orc_scene_get_state(const orc_scene* s, double* x, double* v)
{
    size_t n3 = 3 * (size_t)s->n;
    if (x) memcpy(x, s->x, sizeof(double) * n3);
    if (v) memcpy(v, s->v, sizeof(double) * n3);
}

void orc_scene_set_external_force(orc_scene* s, const double* fext)
{
    size_t n3 = 3 * (size_t)s->n;
    if (!s->ext) s->ext = (double*)malloc(sizeof(double) * n3);
    memcpy(s->ext, fext, sizeof(double) * n3);
}

void orc_scene_set_springs(orc_scene* s, double k, const double* anchor)
{
    size_t n3 = 3 * (size_t)s->n;
    s->spring_k = k;
    if (!s->anchor) s->anchor = (double*)malloc(sizeof(double) * n3);
    memcpy(s->anchor, anchor, sizeof(double) * n3);
}

int orc_scene_last_iterations(const orc_scene* s) { return s->last_iters; }
double orc_scene_last_error(const orc_scene* s) { return s->last_err; }

/* Element-wise vector operations (MechanicalObject::vOp,
 * MechanicalObject.inl:1999-2205), split over the threads for long vectors:
 * each entry is computed by the same expression whatever the split. */
enum { VOP_COPY, VOP_ZERO, VOP_AVF, VOP_INC, VOP_INTEGRATE };
typedef struct {
    int kind;
    double* out;
    const double* a;
    double* x; /* VOP_INTEGRATE: positions (out = v, a = dv) */
    double f;
    long n3;
} vop_job;

static void vop_range(const vop_job* j, long b, long e)
{
    double* out = j->out;
    const double* a = j->a;
    const double f = j->f;
    switch (j->kind) {
    case VOP_COPY:
        memcpy(out + b, a + b, sizeof(double) * (size_t)(e - b));
        break;
    case VOP_ZERO:
        memset(out + b, 0, sizeof(double) * (size_t)(e - b));
        break;
    case VOP_AVF: /* out = out * f + a (f == 1: out += a) */
        if (f == 1.0)
            for (long i = b; i < e; ++i) out[i] += a[i];
        else
            for (long i = b; i < e; ++i) {
                out[i] *= f;
                out[i] += a[i];
            }
        break;
    case VOP_INC: /* out += a * f (f == 1: out += a) */
        if (f == 1.0)
            for (long i = b; i < e; ++i) out[i] += a[i];
        else
            for (long i = b; i < e; ++i) out[i] += a[i] * f;
        break;
    case VOP_INTEGRATE: /* v += dv; x += v h */
        for (long i = b; i < e; ++i) {
            out[i] += a[i];
            j->x[i] += out[i] * f;
        }
        break;
    }
}

static void vop_job_run(void* ctx, int tid, int n)
{
    const vop_job* j = (const vop_job*)ctx;
    long b, e;
    chunk(j->n3, tid, n, &b, &e);
    vop_range(j, b, e);
}

static void vop_run(int kind, double* out, const double* a, double f, long n3, double* x)
{
    vop_job j = {kind, out, a, x, f, n3};
    if (g_threads > 1 && n3 >= (1L << 17))
        parallel_run(vop_job_run, &j, g_threads);
    else
        vop_range(&j, 0, n3);
}

/* UniformMass::addForce (UniformMass.inl:471-496) / DiagonalMass::addForce
 * (DiagonalMass.inl:1393-1413): f += m g. */
static void mass_add_force(const orc_scene* s, double* f)
{
    /* separateGravity: UniformMass::addForce returns at once
     * (UniformMass.inl:471-475), DiagonalMass::addForce likewise */
    if (s->separate_gravity) return;
    if (s->mass_kind == 0) {
        double mg[3] = {s->g[0] * s->vertex_mass, s->g[1] * s->vertex_mass, s->g[2] * s->vertex_mass};
        for (int i = 0; i < s->n; ++i)
            for (int k = 0; k < 3; ++k) f[3 * i + k] += mg[k];
    } else {
        for (int i = 0; i < s->n; ++i)
            for (int k = 0; k < 3; ++k) f[3 * i + k] += s->g[k] * s->node_mass[i];
    }
}

/* UniformMass::addMDx (UniformMass.inl:403-419) / DiagonalMass::addMDx
 * (DiagonalMass.inl:536-559): res += factor M dx. */
static void mass_add_mdx(const orc_scene* s, double* res, const double* dx, double factor)
{
    if (s->mass_kind == 0) {
        double m = s->vertex_mass;
        if (factor != 1.0) m *= factor;
        vop_run(VOP_INC, res, dx, m, 3L * s->n, NULL);
    } else if (factor == 1.0) {
        for (int i = 0; i < s->n; ++i)
            for (int k = 0; k < 3; ++k) res[3 * i + k] += dx[3 * i + k] * s->node_mass[i];
    } else {
        for (int i = 0; i < s->n; ++i)
            for (int k = 0; k < 3; ++k) res[3 * i + k] += (dx[3 * i + k] * s->node_mass[i]) * factor;
    }
}

static void spring_add_force(const orc_scene* s, const double* x, double* f)
{
    if (s->spring_k == 0.0) return;
    for (long i = 0; i < 3L * s->n; ++i) f[i] += -s->spring_k * (x[i] - s->anchor[i]);
}

static void spring_add_dforce(const orc_scene* s, const double* dx, double* df, double kf)
{
    if (s->spring_k == 0.0) return;
    for (long i = 0; i < 3L * s->n; ++i) df[i] += -s->spring_k * dx[i] * kf;
}

/* FixedProjectiveConstraint::projectResponse (FixedProjectiveConstraint.inl:184-207). */
static void project_response(const orc_scene* s, double* res)
{
    if (s->fix_all) {
        memset(res, 0, sizeof(double) * 3 * (size_t)s->n);
        return;
    }
    for (int i = 0; i < s->n_fixed; ++i) {
        int j = s->fixed[i];
        if (j >= 0 && j < s->n) res[3 * j] = res[3 * j + 1] = res[3 * j + 2] = 0.0;
    }
}

/* MechanicalObject::vDot (MechanicalObject.inl:2334-2356). */
static double vdot(const double* a, const double* b, int n)
{
    double r = 0.0;
    for (int i = 0; i < n; ++i) r += vec_dot(&a[3 * i], &b[3 * i]);
    return r;
}

/* addMBKdx with the forcefield order of the node: mass (Mass::addMBKdx,
 * Mass.inl:94-104) and the FEM (BaseForceField::addMBKdx,
 * BaseForceField.cpp:38-47). mf and kf are the factors each component
 * applies, their own Rayleigh terms already folded in
 * (k/mFactorIncludingRayleighDamping, MechanicalParams.h:62-64); the force
 * field runs when its factor or the matrix's bFactor is non-zero. */
static void add_mbkdx(orc_scene* s, double* df, const double* dx, double mf, double kf)
{
    const int ff = (kf != 0.0 || s->cur_bf != 0.0) && s->fem;
    if (s->mass_first) {
        if (mf != 0.0) mass_add_mdx(s, df, dx, mf);
        if (ff) orc_fem_add_dforce(s->fem, dx, df, kf);
    } else {
        if (ff) orc_fem_add_dforce(s->fem, dx, df, kf);
        if (mf != 0.0) mass_add_mdx(s, df, dx, mf);
    }
    if (kf != 0.0) spring_add_dforce(s, dx, df, kf);
}

/* GraphScatteredMatrix::apply (GraphScatteredTypes.cpp:33-45):
 * q = (mF M + kF K) p, then projected. */
static void matvec(orc_scene* s, double* q, const double* p, double mf, double kf)
{
    vop_run(VOP_ZERO, q, NULL, 0.0, 3L * s->n, NULL);
    add_mbkdx(s, q, p, mf, kf);
    project_response(s, q);
}

/* CGLinearSolver::solve (CGLinearSolver.inl:72-315) with the GraphScattered
 * cgstep_beta / cgstep_alpha (CGLinearSolver.cpp:40-63), warmStart off. */
static void vop_avf(double* out, const double* a, double f, long n3);

static void cg_solve(orc_scene* s, double mf, double kf)
{
    const int n = s->n;
    const long n3 = 3L * n;
    double *x = s->xs, *b = s->b, *p = s->p, *q = s->q, *r = s->r;
    double rho, rho_1 = 0.0, alpha, beta;
    if (s->warm_start) {
        /* CGLinearSolver.inl:95-99: r = A x; r = b + r * -1 */
        matvec(s, r, x, mf, kf);
        vop_avf(r, b, -1.0, n3);
    } else {
        vop_run(VOP_ZERO, x, NULL, 0.0, n3, NULL);
        vop_run(VOP_COPY, r, b, 0.0, n3, NULL);
    }
    const double normb = sqrt(vdot(b, b, n));
    int nb_iter = 0, n_matvec = 0;
    s->last_err = 0.0;
    if (normb != 0.0) {
        for (nb_iter = 1; nb_iter <= s->cg_iters; nb_iter++) {
            rho = vdot(r, r, n);
            const double err = sqrt(rho) / normb;
            s->last_err = err;
            if (err <= s->cg_tol) {
                if (!(nb_iter == 1 && s->time_step_count == 0)) break;
            }
            if (nb_iter == 1) {
                vop_run(VOP_COPY, p, r, 0.0, n3, NULL);
            } else {
                beta = rho / rho_1;
                /* vOp_avf (MechanicalObject.inl:1999-2013): p *= beta; p += r */
                vop_run(VOP_AVF, p, r, beta, n3, NULL);
            }
            matvec(s, q, p, mf, kf);
            n_matvec++;
            const double den = vdot(p, q, n);
            if (den != 0.0) {
                if (fabs(den) <= s->cg_threshold) {
                    if (!(nb_iter == 1 && s->time_step_count == 0)) break;
                }
                alpha = rho / den;
                /* vOp_v_inc_bf (MechanicalObject.inl:2018-2032) */
                vop_run(VOP_INC, x, p, alpha, n3, NULL);
                vop_run(VOP_INC, r, q, -alpha, n3, NULL);
            } else {
                break;
            }
            rho_1 = rho;
        }
    }
    s->time_step_count++;
    s->last_iters = n_matvec;
}

/* ------------------------------------------------------------------------- */
/* PCGLinearSolver (PCGLinearSolver.inl:194-262) with an optional Jacobi     */
/* preconditioner (JacobiPreconditioner.inl:41-51: z = diag(A)^-1 r, the     */
/* diagonal of the assembled system A = mF M + kF K with fixed DOFs set to   */
/* one). The diagonal is re-assembled every solve from this step's           */
/* rotations. Its summation order is this restatement's (component order,    */
/* elements in index order); the reference assembles it through addKToMatrix */
/* and addMToMatrix, which cannot be run here.                               */
/* ------------------------------------------------------------------------- */

/* diag(R^T S R) of node i's 3x3 stiffness block S = B^T C B of element e,
 * with B from node i's strain-displacement values (a, b, c) and C the
 * isotropic K3 = (k0, k1, k2); R = rot^T (rot holds rotations[e] = R^T). */
static void element_stiffness_diag(const double* rot, const double* K3, const double* J3i, double dk[3])
{
    const double a = J3i[0], b = J3i[1], c = J3i[2];
    const double k0 = K3[0], k1 = K3[1], k2 = K3[2];
    const double k12 = k1 + k2;
    const double S[9] = {a * a * k0 + b * b * k2 + c * c * k2, a * b * k12, a * c * k12,
                         a * b * k12, b * b * k0 + a * a * k2 + c * c * k2, b * c * k12,
                         a * c * k12, b * c * k12, c * c * k0 + b * b * k2 + a * a * k2};
    for (int k = 0; k < 3; ++k) {
        double acc = 0.0;
        for (int p = 0; p < 3; ++p) {
            double sr = S[3 * p] * rot[3 * k] + S[3 * p + 1] * rot[3 * k + 1] + S[3 * p + 2] * rot[3 * k + 2];
            acc += rot[3 * k + p] * sr;
        }
        dk[k] = acc;
    }
}

static void mass_diag_add(const orc_scene* s, double* d, double mf)
{
    for (int i = 0; i < s->n; ++i) {
        const double m = (s->mass_kind == 1) ? s->node_mass[i] : s->vertex_mass;
        for (int k = 0; k < 3; ++k) d[3 * i + k] += m * mf;
    }
}

/* dinv = 1 / diag(mF M + kF K), fixed DOFs 1 */
static void jacobi_inverse_diagonal(orc_scene* s, double mf, double kf, double* dinv)
{
    const long n3 = 3L * s->n;
    memset(dinv, 0, sizeof(double) * (size_t)n3);
    if (s->mass_first) mass_diag_add(s, dinv, mf);
    if (s->fem) {
        const orc_fem* m = s->fem;
        for (int e = 0; e < m->n_tets; ++e)
            for (int i = 0; i < 4; ++i) {
                double dk[3];
                element_stiffness_diag(&m->rot[9 * e], &m->K3[3 * e], &m->J3[12 * e + 3 * i], dk);
                const int node = m->tets[4 * e + i];
                for (int k = 0; k < 3; ++k) dinv[3 * node + k] += -kf * dk[k];
            }
    }
    if (!s->mass_first) mass_diag_add(s, dinv, mf);
    for (long i = 0; i < n3; ++i) dinv[i] = 1.0 / dinv[i];
    if (s->fix_all) {
        for (long i = 0; i < n3; ++i) dinv[i] = 1.0;
    } else {
        for (int f = 0; f < s->n_fixed; ++f)
            if (s->fixed[f] >= 0 && s->fixed[f] < s->n)
                for (int k = 0; k < 3; ++k) dinv[3 * s->fixed[f] + k] = 1.0;
    }
}

/* out = a + out * f (vOp_avf, MechanicalObject.inl:1997-2011; f == 1: out += a) */
static void vop_avf(double* out, const double* a, double f, long n3)
{
    if (f == 1.0)
        for (long i = 0; i < n3; ++i) out[i] += a[i];
    else
        for (long i = 0; i < n3; ++i) {
            out[i] *= f;
            out[i] += a[i];
        }
}

/* out += a * f (vOp_v_inc_bf; f == 1: out += a) */
static void vop_inc(double* out, const double* a, double f, long n3)
{
    if (f == 1.0)
        for (long i = 0; i < n3; ++i) out[i] += a[i];
    else
        for (long i = 0; i < n3; ++i) out[i] += a[i] * f;
}

static void precond_apply(const orc_scene* s, double* z, const double* r, long n3)
{
    if (s->precond)
        for (long i = 0; i < n3; ++i) z[i] = s->dinv[i] * r[i];
    else
        memcpy(z, r, sizeof(double) * (size_t)n3);
}

/* The solution vector xs keeps the previous step's solution (the solver's
 * x is not cleared between steps): r = b - A x starts from it. */
static void pcg_solve(orc_scene* s, double mf, double kf)
{
    const int n = s->n;
    const long n3 = 3L * n;
    double *x = s->xs, *b = s->b, *r = s->r, *w = s->p, *sv = s->q;
    /* PreconditionedMatrixFreeSystem assemblingRate (PreconditionedMatrixFreeSystem.inl:
     * 48, 60-71): assembled on the first solve and every precond_rate solves */
    if (s->precond && s->time_step_count % s->precond_rate == 0) jacobi_inverse_diagonal(s, mf, kf, s->dinv);
    const double b_norm = vdot(b, b, n);
    const double tol = s->cg_tol * b_norm;
    matvec(s, r, x, mf, kf);
    vop_avf(r, b, -1.0, n3); /* r = b - A x */
    precond_apply(s, w, r, n3);
    double r_norm = vdot(r, w, n);
    int iter = 1;
    while (iter <= s->cg_iters && r_norm > tol) {
        matvec(s, sv, w, mf, kf);
        const double dtq = vdot(w, sv, n);
        const double alpha = r_norm / dtq;
        vop_inc(x, w, alpha, n3);
        vop_inc(r, sv, -alpha, n3);
        precond_apply(s, sv, r, n3);
        const double delta_old = r_norm;
        r_norm = vdot(r, sv, n);
        const double beta = r_norm / delta_old;
        vop_avf(w, sv, beta, n3);
        iter++;
    }
    s->last_iters = iter - 1;
    s->last_err = (b_norm != 0.0) ? r_norm / b_norm : 0.0;
    s->time_step_count++;
}

/* Selects the linear solver: 0 CGLinearSolver, 1 PCGLinearSolver; precond
 * 1 = JacobiPreconditioner. */
void orc_scene_set_solver(orc_scene* s, int solver, int precond, int precond_rate)
{
    s->solver = solver;
    s->precond = precond;
    s->precond_rate = precond_rate > 1 ? precond_rate : 1;
    if (precond && !s->dinv) s->dinv = (double*)calloc(3 * (size_t)s->n, sizeof(double));
}

/* CGLinearSolver warmStart: each CG solve starts from the previous solution. */
void orc_scene_set_warm_start(orc_scene* s, int on) { s->warm_start = on ? 1 : 0; }

/* EulerImplicitSolver trapezoidalScheme. */
void orc_scene_set_trapezoidal(orc_scene* s, int on) { s->trapezoidal = on ? 1 : 0; }

/* The components' own Rayleigh coefficients, EulerImplicitSolver firstOrder and
 * FixedProjectiveConstraint activate_projectVelocity. */
void orc_scene_set_options(orc_scene* s, double ff_rayleigh_stiffness, double mass_rayleigh_mass, int first_order,
                           int project_velocity)
{
    s->ff_rs = ff_rayleigh_stiffness;
    s->mass_rm = mass_rayleigh_mass;
    s->first_order = first_order ? 1 : 0;
    s->project_velocity = project_velocity ? 1 : 0;
}

/* the last solve's Jacobi inverse diagonal (zeros before the first) */
void orc_scene_jacobi(const orc_scene* s, double* out)
{
    if (s->dinv) memcpy(out, s->dinv, sizeof(double) * 3 * (size_t)s->n);
    else memset(out, 0, sizeof(double) * 3 * (size_t)s->n);
}

/* computeForce (MappingGraphMechanicalOperations.cpp:41-92): f = 0,
 * f += externalForce, f += sum of the force fields' addForce. */
static void scene_compute_force(orc_scene* s)
{
    const long n3 = 3L * s->n;
    memset(s->f, 0, sizeof(double) * (size_t)n3);
    if (s->ext)
        for (long i = 0; i < n3; ++i) s->f[i] += s->ext[i];
    if (s->mass_first) {
        mass_add_force(s, s->f);
        if (s->fem) orc_fem_add_force(s->fem, s->x, s->f);
    } else {
        if (s->fem) orc_fem_add_force(s->fem, s->x, s->f);
        mass_add_force(s, s->f);
    }
    spring_add_force(s, s->x, s->f);
}

/* One EulerImplicitSolver::solve (EulerImplicitSolver.cpp:83-341) in its
 * second-order, non-trapezoidal form, followed by the animation loop's
 * projectPositionAndVelocity (no-op for FixedProjectiveConstraint with
 * activate_projectVelocity off). */
static void euler_step(orc_scene* s)
{
    const long n3 = 3L * s->n;
    /* trapezoidalScheme: tr = 0.5 on some uses of h (EulerImplicitSolver.cpp:117-123) */
    const double h = s->dt, tr = s->trapezoidal ? 0.5 : 1.0;
    scene_compute_force(s);
    memcpy(s->b, s->f, sizeof(double) * (size_t)n3);
    if (!s->first_order) {
        /* b = f; b += (-rm M + (h + rs) K) v with bFactor 0; b *= h
         * (EulerImplicitSolver.cpp:141-158); firstOrder: b = f (:137-140) */
        s->cur_bf = 0.0;
        add_mbkdx(s, s->b, s->v, -s->rm, h * tr + s->rs);
        for (long i = 0; i < n3; ++i) s->b[i] *= h;
    }
    project_response(s, s->b);
    /* setSystemMBKMatrix (EulerImplicitSolver.cpp:165-171): second order
     * mF = 1 + h rm, bF = -h, kF = -h (h + rs); first order mF = 1, bF = 0,
     * kF = -h. Each component adds its own Rayleigh term to its factor. */
    double mf, bf, kf;
    if (s->first_order) {
        mf = 1;
        bf = 0;
        kf = -h * tr;
    } else {
        mf = 1 + tr * h * s->rm;
        bf = -tr * h;
        kf = -tr * h * (tr * h + s->rs);
    }
    const double kf_ff = kf + bf * s->ff_rs;
    const double mf_mass = mf - bf * s->mass_rm;
    s->cur_bf = bf;
    if (s->solver == 1)
        pcg_solve(s, mf_mass, kf_ff);
    else
        cg_solve(s, mf_mass, kf_ff);
    if (s->first_order) {
        /* v = x; x = x + v h (the generic vMultiOp, :248-256) */
        vop_run(VOP_COPY, s->v, s->xs, 0.0, n3, NULL);
        vop_run(VOP_INC, s->x, s->v, h, n3, NULL);
    } else {
        /* vMultiOp fast path (MechanicalObject.inl:2206-2240): v += dv; x += v h */
        vop_run(VOP_INTEGRATE, s->v, s->xs, h, n3, s->x);
    }
    if (s->separate_gravity) {
        /* addSeparateGravity (EulerImplicitSolver.cpp:296; UniformMass::
         * addGravityToV, UniformMass.inl:450-468): v += g dt, every point */
        double hg[3];
        for (int k = 0; k < 3; ++k) hg[k] = s->g[k] * h;
        for (long i = 0; i < n3; ++i) s->v[i] += hg[i % 3];
    }
    if (s->vdamping != 0.0) {
        const double d = exp(-h * s->vdamping);
        for (long i = 0; i < n3; ++i) s->v[i] *= d;
    }
    if (s->compute_residual) {
        /* computeResidual (EulerImplicitSolver.cpp:314-338): r = 0;
         * r += M (newVel - vel), zero, the animation loop passing the
         * state's velocity as both; f = computeForce at the new state (the
         * force field runs again, plastic strains and rebuilt J included);
         * r += f (-dt); projectResponse(r); residual = r.r (vDot) */
        scene_compute_force(s);
        for (long i = 0; i < n3; ++i) s->r[i] = 0.0 + s->f[i] * (-h);
        project_response(s, s->r);
        s->residual = vdot(s->r, s->r, s->n);
    }
    /* DefaultAnimationLoop::projectPositionAndVelocity (DefaultAnimationLoop.cpp:
     * 228-233, 293): FixedProjectiveConstraint::projectVelocity
     * (FixedProjectiveConstraint.inl:237-261) zeroes the fixed nodes' velocity
     * when activate_projectVelocity is set; projectPosition does nothing */
    if (s->project_velocity) project_response(s, s->v);
}

void orc_scene_set_compute_residual(orc_scene* s, int on) { s->compute_residual = on ? 1 : 0; }
void orc_scene_set_separate_gravity(orc_scene* s, int on) { s->separate_gravity = on ? 1 : 0; }
double orc_scene_residual(const orc_scene* s) { return s->residual; }

void orc_scene_step(orc_scene* s, int n_steps)
{
    for (int i = 0; i < n_steps; ++i) euler_step(s);
}

/* Exposed pieces of the step for per-call parity checks. */
void orc_scene_compute_force(orc_scene* s, double* f_out)
{
    scene_compute_force(s);
    if (f_out) memcpy(f_out, s->f, sizeof(double) * 3 * (size_t)s->n);
}
