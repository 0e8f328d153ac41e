"""Generates tests/golden/polar_stable_ref.npz: outputs of the reference's own
Decompose<double>::polarDecomposition_stable (SVD_stable path,
Sofa/framework/Helper/src/sofa/helper/decompose.inl:756-765, 1664-1825),
compiled from the reference sources by oracle/ref/Makefile, on seeded 3x3
matrices covering each branch the svd method reaches: regular, inverted,
nearly inverted, flat (rank 2), collapsed to an edge (rank 1) and to a
point, and flat or inverted deformation gradients of tetrahedra.

Run with SOFA_REFERENCE_ROOT naming the SOFA source tree:
    SOFA_REFERENCE_ROOT=<tree> python tests/golden/make_polar_stable_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import pyoracle  # noqa: E402


def main():
    lib = pyoracle.ref_math_lib()
    if lib is None:
        raise SystemExit("reference tree not found; cannot build the reference math library")
    rng = np.random.default_rng(20261205)
    mats = []
    for i in range(600):
        M = rng.normal(size=(3, 3))
        k = i % 8
        if k == 1:
            M[0] *= -1.0  # inverted
        elif k == 2:
            M[2] = 0.3 * M[0] + 0.7 * M[1]  # flat
        elif k == 3:
            M[1] = 2.0 * M[0]
            M[2] = -M[0]  # collapsed to an edge
        elif k == 4:
            M[:] = 0.0  # collapsed to a point
        elif k == 5:
            M = np.eye(3) + 1e-5 * rng.normal(size=(3, 3))
            M[1] *= -1.0  # inverted, nearly a reflection
        elif k == 6:
            M = np.eye(3) + 0.1 * rng.normal(size=(3, 3))
            M[2] *= 1e-7  # nearly flat (det below the 1e-6 switch)
        elif k == 7:
            M = np.diag([1.0, 1e-5, 1e-6]) @ rng.normal(size=(3, 3))  # two tiny singular values
        mats.append(M)
    mats = np.array(mats)
    dp = ctypes.POINTER(ctypes.c_double)
    Q = np.zeros_like(mats)
    deg = np.zeros(len(mats), dtype=np.int32)
    for i in range(len(mats)):
        m = np.ascontiguousarray(mats[i])
        q = np.zeros((3, 3))
        deg[i] = lib.ref_polar_decomposition_stable_d(m.ctypes.data_as(dp), q.ctypes.data_as(dp))
        Q[i] = q
    np.savez_compressed(os.path.join(HERE, "polar_stable_ref.npz"), M=mats, Q=Q, degenerate=deg)
    print("wrote", len(mats), "cases,", int(deg.sum()), "degenerate or inverted")


if __name__ == "__main__":
    main()
