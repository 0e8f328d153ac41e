"""Generates tests/golden/polar_ref.npz: outputs of the reference's own
Decompose<double>/Decompose<float>::polarDecomposition
(Sofa/framework/Helper/src/sofa/helper/decompose.inl:672-723), compiled from
the reference sources by oracle/ref/Makefile, on seeded 3x3 matrices shaped
like the edge matrices of deformed tetrahedra (rotation x stretch x shear),
plus generic random ones.

Run with SOFA_REFERENCE_ROOT naming the SOFA source tree:
    SOFA_REFERENCE_ROOT=<tree> python tests/golden/make_polar_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import pyoracle  # noqa: E402


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def main():
    lib = pyoracle.ref_math_lib()
    if lib is None:
        raise SystemExit("reference tree not found; cannot build the reference math library")
    rng = np.random.default_rng(20261204)
    mats = []
    for _ in range(400):  # tetra-like: R * (I + small strain) * edge scale
        R = random_rotation(rng)
        S = np.eye(3) + rng.normal(scale=0.05, size=(3, 3))
        mats.append(0.5 * R @ S)
    for _ in range(100):  # large deformation
        mats.append(random_rotation(rng) @ (np.eye(3) + rng.normal(scale=0.5, size=(3, 3))))
    for _ in range(50):  # generic
        mats.append(rng.normal(size=(3, 3)) * 10.0 ** rng.uniform(-3, 3))
    mats = np.array(mats)
    dp = ctypes.POINTER(ctypes.c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    Qd = np.zeros_like(mats)
    detd = np.zeros(len(mats))
    mf = mats.astype(np.float32)
    Qf = np.zeros_like(mf)
    detf = np.zeros(len(mats), dtype=np.float32)
    for i in range(len(mats)):
        m = np.ascontiguousarray(mats[i])
        q = np.zeros((3, 3))
        detd[i] = lib.ref_polar_decomposition_d(m.ctypes.data_as(dp), q.ctypes.data_as(dp))
        Qd[i] = q
        m32 = np.ascontiguousarray(mf[i])
        q32 = np.zeros((3, 3), dtype=np.float32)
        detf[i] = lib.ref_polar_decomposition_f(m32.ctypes.data_as(fp), q32.ctypes.data_as(fp))
        Qf[i] = q32
    np.savez_compressed(os.path.join(HERE, "polar_ref.npz"), M=mats, Q=Qd, det=detd, M32=mf, Q32=Qf, det32=detf)
    print("wrote", len(mats), "cases")


if __name__ == "__main__":
    main()
