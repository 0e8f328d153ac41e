// Reference harness: exposes the reference's own Higham/Shoemake polar
// decomposition (Sofa/framework/Helper/src/sofa/helper/decompose.inl:672-723,
// tolerance decompose.h:378-387) with C linkage so tests can check the
// oracle's restatement (oracle/tfem_oracle.c, orc_polar) against it bit for
// bit. The reference sources are compiled where they lie; nothing is copied.
#include <sofa/helper/decompose.inl>

extern "C" {

// M, Q: 3x3 row-major. Returns the determinant of the last iterate, as the
// reference does.
double ref_polar_decomposition_d(const double* M, double* Q)
{
    sofa::type::Mat<3, 3, double> m, q;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m(i, j) = M[3 * i + j];
    double det = sofa::helper::Decompose<double>::polarDecomposition(m, q);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Q[3 * i + j] = q(i, j);
    return det;
}

float ref_polar_decomposition_f(const float* M, float* Q)
{
    sofa::type::Mat<3, 3, float> m, q;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m(i, j) = M[3 * i + j];
    float det = sofa::helper::Decompose<float>::polarDecomposition(m, q);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Q[3 * i + j] = q(i, j);
    return det;
}

// Stable polar factor through the 3x3 SVD (decompose.inl:756-765, SVD_stable
// 1664-1825), used by the svd method for inverted or flat elements. Returns
// whether the reference flagged the matrix degenerate or inverted.
int ref_polar_decomposition_stable_d(const double* M, double* Q)
{
    sofa::type::Mat<3, 3, double> m, q;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m(i, j) = M[3 * i + j];
    const bool deg = sofa::helper::Decompose<double>::polarDecomposition_stable(m, q);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Q[3 * i + j] = q(i, j);
    return deg ? 1 : 0;
}

// Reference 3x3 norms (Sofa/framework/Type/src/sofa/type/Mat.h:1056-1080).
double ref_one_norm_d(const double* A)
{
    sofa::type::Mat<3, 3, double> a;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a(i, j) = A[3 * i + j];
    return sofa::type::oneNorm(a);
}

}
