"""The oracle's updateStiffnessMatrix (TetrahedronFEMForceField.inl:49; polar
:1063-1067, svd :1174-1177): after an addForce each element's 12 distinct
strain-displacement values are computeStrainDisplacement (TFEM.inl:134-209)
of its deformed positions in its current frame, R p_i with the absolute
positions. Checked bit for bit against the same formula evaluated here, and
the rebuilt matrix must be what addDForce then uses."""
import numpy as np
import pytest

from tests import cases


def pdet(m00, m01, m02, m10, m11, m12):
    # peudo_determinant_for_coef (TFEM.inl:211-215), the reference's term order
    return m01 * m12 - m11 * m02 - m00 * m12 + m10 * m02 + m00 * m11 - m10 * m01


def strain_displacement(a, b, c, d):
    return np.array([
        -pdet(b[1], c[1], d[1], b[2], c[2], d[2]), pdet(b[0], c[0], d[0], b[2], c[2], d[2]),
        -pdet(b[0], c[0], d[0], b[1], c[1], d[1]),
        pdet(c[1], d[1], a[1], c[2], d[2], a[2]), -pdet(c[0], d[0], a[0], c[2], d[2], a[2]),
        pdet(c[0], d[0], a[0], c[1], d[1], a[1]),
        -pdet(d[1], a[1], b[1], d[2], a[2], b[2]), pdet(d[0], a[0], b[0], d[2], a[2], b[2]),
        -pdet(d[0], a[0], b[0], d[1], a[1], b[1]),
        pdet(a[1], b[1], c[1], a[2], b[2], c[2]), -pdet(a[0], b[0], c[0], a[2], b[2], c[2]),
        pdet(a[0], b[0], c[0], a[1], b[1], c[1])])


def frame_positions(R, p):
    # deforme[i] = R p[index[i]] with Mat*Vec's left-to-right sums
    out = []
    for pi in p:
        out.append([float(R[k, 0] * pi[0] + R[k, 1] * pi[1] + R[k, 2] * pi[2]) for k in range(3)])
    return out


def deformed(mesh, seed=4):
    rng = np.random.default_rng(seed)
    u = 0.05 * np.stack([np.sin(0.3 * mesh.positions[:, 2]), np.cos(0.2 * mesh.positions[:, 2]),
                         0.1 * mesh.positions[:, 0]], 1)
    return mesh.positions + u + rng.normal(scale=0.02, size=mesh.positions.shape)


@pytest.mark.parametrize("method", ["polar", "svd"])
def test_rebuilt_strain_displacement_is_the_reference_formula(oracle, method):
    mesh = cases.beam_mesh((3, 3, 6))
    x = deformed(mesh)
    fem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
    j0 = [fem.element(e)["J3"].copy() for e in range(mesh.n_tets)]
    fem.set_update_stiffness(True)
    fem.add_force(x)
    for e in range(mesh.n_tets):
        el = fem.element(e)
        R = el["rotation"].T  # rotations[e] holds R^T
        t = mesh.tetrahedra[e]
        a, b, c, d = frame_positions(R, [x[t[0]], x[t[1]], x[t[2]], x[t[3]]])
        got = el["J3"].reshape(-1)
        assert np.array_equal(got, strain_displacement(a, b, c, d)), e
        assert not np.array_equal(got, j0[e].reshape(-1))


def test_rebuilt_matrix_enters_add_dforce(oracle):
    mesh = cases.beam_mesh((3, 3, 6))
    x = deformed(mesh)
    dx = np.random.default_rng(5).normal(scale=1e-3, size=x.shape)
    plain = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar")
    upd = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar")
    upd.set_update_stiffness(True)
    f0, f1 = plain.add_force(x), upd.add_force(x)
    df0, df1 = plain.add_dforce(dx, -0.01), upd.add_dforce(dx, -0.01)
    assert not np.array_equal(f0, f1) and not np.array_equal(df0, df1)
    # at the rest state the rebuilt J is the initial one up to the rounding of
    # the frame: forces stay zero to rounding
    rest = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "polar")
    rest.set_update_stiffness(True)
    assert np.max(np.abs(rest.add_force(mesh.positions))) < 1e-9


def test_large_and_small_keep_their_matrix(oracle):
    mesh = cases.beam_mesh((3, 3, 6))
    x = deformed(mesh)
    for method in ("large", "small"):
        fem = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)
        j0 = fem.element(3)["J3"].copy()
        fem.set_update_stiffness(True)
        fem.add_force(x)
        assert np.array_equal(fem.element(3)["J3"], j0)
