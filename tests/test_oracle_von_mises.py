"""The oracle's von Mises stress (computeVonMisesStress,
TetrahedronFEMForceField.inl:2197-2374) against answers that follow from
the formulas alone:
  * at rest, and after a rigid motion, both strains vanish, so every value
    is zero;
  * a uniform stretch x_z -> (1 + e) x_z has the Green strain e + e^2/2
    along z in every element, so every element's value is
    2 mu (e + e^2/2) = E/(1+nu) (e + e^2/2) (mode 2); the corotational
    value (mode 1) is of first order in a small stretch;
  * a node's value is the mean of its elements';
  * mode 1 with method small is refused, as in the reference."""
import numpy as np
import pytest

from tests import cases

YOUNG, NU = 5000.0, 0.45


def _fem(oracle, mesh, method):
    return oracle.OracleFEM(mesh.positions, mesh.tetrahedra, YOUNG, NU, method)


def _rotation(a=0.7, b=-0.4):
    ca, sa, cb, sb = np.cos(a), np.sin(a), np.cos(b), np.sin(b)
    return np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]]) @ np.array([[1, 0, 0], [0, cb, -sb], [0, sb, cb]])


@pytest.mark.parametrize("method,mode", [("large", 1), ("polar", 1), ("svd", 1), ("large", 2), ("small", 2)])
def test_rest_and_rigid_motion_give_zero(oracle, method, mode):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    fem = _fem(oracle, mesh, method)
    for x in (mesh.positions, mesh.positions @ _rotation().T + np.array([1.0, -2.0, 0.5])):
        e, n = fem.von_mises(x, mode)
        assert np.abs(e).max() <= 1e-9 * YOUNG and np.abs(n).max() <= 1e-9 * YOUNG


@pytest.mark.parametrize("method", ["large", "polar", "small"])
def test_uniform_stretch_green_strain(oracle, method):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    eps = 0.02
    x = mesh.positions.copy()
    x[:, 2] *= 1 + eps
    e, _ = _fem(oracle, mesh, method).von_mises(x, 2)
    expect = YOUNG / (1 + NU) * (eps + eps * eps / 2)
    np.testing.assert_allclose(e, expect, rtol=1e-9)


@pytest.mark.parametrize("method", ["large", "polar"])
def test_corotational_strain_is_first_order_in_the_stretch(oracle, method):
    """Mode 1 takes the shape-function gradients in the world frame and the
    displacements in the element's rotated frame (:2316-2324), so its value
    depends on each element's initial rotation and has no frame-free closed
    form; it is homogeneous of degree one in a small stretch."""
    mesh = cases.beam_mesh(n=(3, 3, 6))
    fem = _fem(oracle, mesh, method)
    vals = []
    for eps in (1e-6, 2e-6):
        x = mesh.positions.copy()
        x[:, 2] *= 1 + eps
        vals.append(fem.von_mises(x, 1)[0])
    assert (vals[0] > 0).all()
    np.testing.assert_allclose(vals[1], 2 * vals[0], rtol=1e-4)


def test_node_values_are_element_means(oracle):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    rng = np.random.default_rng(3)
    x = mesh.positions + rng.uniform(-0.02, 0.02, mesh.positions.shape)
    e, n = _fem(oracle, mesh, "polar").von_mises(x, 1)
    acc = np.zeros(mesh.n_nodes)
    cnt = np.zeros(mesh.n_nodes)
    for t, v in zip(mesh.tetrahedra, e):
        acc[t] += v
        cnt[t] += 1
    np.testing.assert_allclose(n, np.where(cnt > 0, acc / np.maximum(cnt, 1), 0.0), rtol=1e-14)
    assert (e > 0).all()


def test_corotational_mode_refused_for_small(oracle):
    mesh = cases.beam_mesh(n=(3, 3, 4))
    with pytest.raises(ValueError):
        _fem(oracle, mesh, "small").von_mises(mesh.positions, 1)
