// von Mises stress of TetrahedronFEMForceField (computeVonMisesStress,
// Sofa/Component/SolidMechanics/FEM/Elastic/src/sofa/component/solidmechanics/
// fem/elastic/TetrahedronFEMForceField.inl:2197-2374), per element and per
// node, in FP64 for every precision of the force field. Compiled without FMA
// contraction: the operations follow the reference's order.
#include <cuda_runtime.h>
#include <math.h>

#include "sgb_internal.h"
#include "tfem_math.cuh"

namespace sgb {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void ld3d(const double* p, int i, double o[3])
{
    o[0] = p[3 * (size_t)i];
    o[1] = p[3 * (size_t)i + 1];
    o[2] = p[3 * (size_t)i + 2];
}

// invertMatrix for a general square matrix (Sofa/framework/Type/src/sofa/type/
// Mat.h:1102-1168): Gauss-Jordan with full pivoting, the pivot the first
// largest |entry| in row-major order among the unused rows and columns.
// Returns false (leaving dest untouched) when a pivot is within machine
// epsilon of zero (equalsZero, Mat.h:46-49).
__device__ bool invert4(const double from[16], double dest[16])
{
    double m1[16], m2[16];
    int r[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0}, row[4] = {0, 0, 0, 0}, col[4] = {0, 0, 0, 0};
    for (int i = 0; i < 16; ++i) {
        m1[i] = from[i];
        m2[i] = (i % 5 == 0) ? 1.0 : 0.0;
    }
    for (int k = 0; k < 4; ++k) {
        double pivot = 0.0;
        for (int i = 0; i < 4; ++i) {
            if (row[i]) continue;
            for (int j = 0; j < 4; ++j) {
                if (col[j]) continue;
                double t = m1[4 * i + j];
                if (t < 0) t = -t;
                if (t > pivot) {
                    pivot = t;
                    r[k] = i;
                    c[k] = j;
                }
            }
        }
        if (fabs(pivot) <= 2.220446049250313e-16) return false;
        row[r[k]] = col[c[k]] = 1;
        pivot = m1[4 * r[k] + c[k]];
        for (int j = 0; j < 4; ++j) m1[4 * r[k] + j] /= pivot;
        m1[4 * r[k] + c[k]] = 1.0;
        for (int j = 0; j < 4; ++j) m2[4 * r[k] + j] /= pivot;
        for (int i = 0; i < 4; ++i) {
            if (i == r[k]) continue;
            const double f = m1[4 * i + c[k]];
            for (int j = 0; j < 4; ++j) {
                const double t = m1[4 * r[k] + j] * f;
                m1[4 * i + j] -= t;
            }
            m1[4 * i + c[k]] = 0.0;
            for (int j = 0; j < 4; ++j) {
                const double t = m2[4 * r[k] + j] * f;
                m2[4 * i + j] -= t;
            }
        }
    }
    int rw[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            if (c[j] == i) rw[i] = r[j];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) dest[4 * i + j] = m2[4 * rw[i] + j];
    return true;
}

// Mat<3,3> * Vec3 (Mat.h:576-586)
__device__ __forceinline__ void matvec3(const double R[9], const double v[3], double o[3])
{
    for (int i = 0; i < 3; ++i) {
        double a = R[3 * i] * v[0];
        a += R[3 * i + 1] * v[1];
        a += R[3 * i + 2] * v[2];
        o[i] = a;
    }
}

// Per element (storage order s): lambda and mu of the element's material
// (computeMaterialStiffness: K(0,1) and K(3,3) before the division by 36 V,
// TetrahedronFEMForceField.inl:256-284).
__global__ void k_lame(const int* __restrict__ elem_orig, int E, const double* __restrict__ young, int n_young,
                       const double* __restrict__ poisson, int n_poisson, const double* __restrict__ lsf, int n_lsf,
                       double* __restrict__ lame)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= E) return;
    const int e = elem_orig[s];
    double Ey = (n_young > e) ? young[e] : young[0];
    const double nu = (n_poisson > e) ? poisson[e] : poisson[0];
    const double f = (n_lsf > 0) ? lsf[(size_t)e * (size_t)n_lsf / (size_t)E] : 1.0;
    Ey = f * Ey;
    const double sc = (Ey * (1 - nu)) / ((1 + nu) * (1 - 2 * nu));
    double k1 = nu / (1 - nu), k2 = (1 - 2 * nu) / (2 * (1 - nu));
    k1 *= sc;
    k2 *= sc;
    lame[s] = k1;
    lame[(size_t)E + s] = k2;
}

// computeVonMisesStress's element loop (:2223-2358) for element s; the
// result goes to the caller's element index.
__global__ void k_von_mises_elem(int mode, int method, const double* __restrict__ rest_pos,
                                 const double* __restrict__ x, const int4* __restrict__ tets,
                                 const int* __restrict__ elem_orig, const double* __restrict__ lame, int E,
                                 double* __restrict__ vme)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= E) return;
    const int4 t = tets[s];
    const int idx[4] = {t.x, t.y, t.z, t.w};
    double X0[4][3], X[4][3];
    for (int i = 0; i < 4; ++i) {
        ld3d(rest_pos, idx[i], X0[i]);
        ld3d(x, idx[i], X[i]);
    }
    // elemShapeFun: inverse of the rows (1, x, y, z) of the rest corners (:1527-1541)
    double mv[16], shf[16];
    for (int k = 0; k < 4; ++k) {
        mv[4 * k] = 1.0;
        for (int l = 1; l < 4; ++l) mv[4 * k + l] = X0[k][l - 1];
    }
    if (!invert4(mv, shf))
        for (int i = 0; i < 16; ++i) shf[i] = 0.0;
    double g[9];  // gradU(k,l) row-major
    double strain[9];
    if (mode == 2) {
        double U[4][3];
        for (int m = 0; m < 4; ++m)
            for (int k = 0; k < 3; ++k) U[m][k] = X[m][k] - X0[m][k];
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) {
                double a = 0.0;
                for (int m = 0; m < 4; ++m) {
                    const double p = shf[4 * (l + 1) + m] * U[m][k];
                    a += p;
                }
                g[3 * k + l] = a;
            }
        // 0.5 (gradU + gradU^T + gradU^T gradU), the product by Mat.h:1443-1475
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const double sym = g[3 * i + j] + g[3 * j + i];
                double tt = g[i] * g[j];
                tt += g[3 + i] * g[3 + j];
                tt += g[6 + i] * g[6 + j];
                const double sum = sym + tt;
                strain[3 * i + j] = sum * 0.5;
            }
    } else {
        // corotational strain: the element's rotation at x and its rotated
        // rest corners (initLarge / initPolar, :835-868, 993-1023)
        double R[9], R0[9], rr[12], def[12], D[12];
        double e0[3], e1[3], e2[3];
        for (int k = 0; k < 3; ++k) {
            e0[k] = X0[1][k] - X0[0][k];
            e1[k] = X0[2][k] - X0[0][k];
            e2[k] = X0[3][k] - X0[0][k];
        }
        if (method == METHOD_LARGE) {
            rotation_large(e0, e1, R0);
        } else {
            const double A0[9] = {e0[0], e0[1], e0[2], e1[0], e1[1], e1[2], e2[0], e2[1], e2[2]};
            polar3(A0, R0, 1000);
        }
        for (int i = 0; i < 4; ++i) matvec3(R0, X0[i], &rr[3 * i]);
        if (method == METHOD_LARGE) {
            for (int i = 1; i < 4; ++i)
                for (int k = 0; k < 3; ++k) rr[3 * i + k] -= rr[k];
            rr[0] = rr[1] = rr[2] = 0.0;
        }
        double a0[3], a1[3], a2[3];
        for (int k = 0; k < 3; ++k) {
            a0[k] = X[1][k] - X[0][k];
            a1[k] = X[2][k] - X[0][k];
            a2[k] = X[3][k] - X[0][k];
        }
        if (method == METHOD_LARGE) {
            rotation_large(a0, a1, R);
        } else {
            const double A[9] = {a0[0], a0[1], a0[2], a1[0], a1[1], a1[2], a2[0], a2[1], a2[2]};
            polar3(A, R);
        }
        for (int i = 0; i < 4; ++i) matvec3(R, X[i], &def[3 * i]);
        if (method == METHOD_LARGE) {
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
                double a = 0.0;
                for (int m = 0; m < 4; ++m) {
                    const double p = shf[4 * (l + 1) + m] * D[3 * m + k];
                    a += p;
                }
                g[3 * k + l] = a;
            }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const double sym = g[3 * i + j] + g[3 * j + i];
                strain[3 * i + j] = sym * 0.5;
            }
    }
    const double v[6] = {strain[0], strain[4], strain[8], strain[5], strain[2], strain[1]};
    const double lambda = lame[s], mu = lame[(size_t)E + s];
    double sg[6];
    double tr = 0.0;
    for (int k = 0; k < 3; ++k) {
        tr += v[k];
        const double a = v[k] * 2;
        sg[k] = a * mu;
    }
    for (int k = 3; k < 6; ++k) {
        const double a = v[k] * 2;
        sg[k] = a * mu;
    }
    for (int k = 0; k < 3; ++k) {
        const double a = lambda * tr;
        sg[k] += a;
    }
    double q = sg[0] * sg[0];
    q += sg[1] * sg[1];
    q += sg[2] * sg[2];
    q -= sg[0] * sg[1];
    q -= sg[1] * sg[2];
    q -= sg[2] * sg[0];
    q += 3 * sg[3] * sg[3];
    q += 3 * sg[4] * sg[4];
    q += 3 * sg[5] * sg[5];
    double r = sqrt(q);
    if (r < 1e-10) r = 0.0;
    vme[elem_orig[s]] = r;
}

// Per node: the mean of its elements' values (:2363-2372), its elements in
// the node table's order.
__global__ void k_von_mises_node(const int* __restrict__ rowptr, const int* __restrict__ slots,
                                 const int* __restrict__ elem_orig, const double* __restrict__ vme, int N,
                                 double* __restrict__ vmn)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int b = rowptr[n], e = rowptr[n + 1];
    double a = 0.0;
    for (int k = b; k < e; ++k) a += vme[elem_orig[slots[k] >> 2]];
    if (e > b) a /= (double)(e - b);
    vmn[n] = a;
}

}  // namespace

void launch_lame(const TfemMesh* m, const double* young, int ny, const double* poisson, int np, const double* lsf,
                 int nl, double* lame, cudaStream_t s)
{
    if (m->n_tets == 0) return;
    k_lame<<<(m->n_tets + kBlock - 1) / kBlock, kBlock, 0, s>>>(m->elem_orig, m->n_tets, young, ny, poisson, np,
                                                                lsf, nl, lame);
}

void launch_von_mises(const TfemMesh* m, int mode, const double* x, const double* lame, double* per_element,
                      double* per_node, cudaStream_t s)
{
    if (m->n_tets > 0)
        k_von_mises_elem<<<(m->n_tets + kBlock - 1) / kBlock, kBlock, 0, s>>>(
            mode, m->method, m->rest_pos, x, m->tets, m->elem_orig, lame, m->n_tets, per_element);
    if (m->n_nodes > 0 && per_node)
        k_von_mises_node<<<(m->n_nodes + kBlock - 1) / kBlock, kBlock, 0, s>>>(m->rowptr, m->slots, m->elem_orig,
                                                                              per_element, m->n_nodes, per_node);
}

}  // namespace sgb
