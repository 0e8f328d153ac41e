"""The oracle's plasticity (TetrahedronFEMForceField.inl:357-370) against
answers that follow from the reference's update rule alone:
  * plasticMaxThreshold = 0 leaves addForce unchanged;
  * creep 1 with yield 0 makes all of the strain plastic, so every force is
    zero (exactly on the first call, to rounding after);
  * creep c with yield 0 and no clamp scales the force of one call at a
    fixed position by (1 - c), and of n calls by (1 - c)^n (the force is
    linear in the elastic strain);
  * the clamp keeps the plastic strain's norm at plasticMaxThreshold;
  * below the yield threshold nothing changes."""
import numpy as np
import pytest

from tests import cases

METHODS = ["small", "large", "polar", "svd"]


def _deformed(mesh, amp=0.05, seed=1):
    rng = np.random.default_rng(seed)
    x = mesh.positions.copy()
    z = x[:, 2] / x[:, 2].max()
    x[:, 1] += amp * 4.0 * z * z
    x += rng.uniform(-amp, amp, x.shape) * 0.2
    return x


def _fem(oracle, mesh, method):
    return oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method)


def _add(fem, x):
    return fem.add_force(x)


@pytest.mark.parametrize("method", METHODS)
def test_plasticity_off_changes_nothing(oracle, method):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    x = _deformed(mesh)
    a, b = _fem(oracle, mesh, method), _fem(oracle, mesh, method)
    b.set_plasticity(0.0, 0.01, 0.5)
    assert np.array_equal(_add(a, x), _add(b, x))
    assert not b.plastic_strain().any()


@pytest.mark.parametrize("method", METHODS)
def test_full_creep_makes_every_force_zero(oracle, method):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    fem = _fem(oracle, mesh, method)
    fem.set_plasticity(1e9, 0.0, 1.0)
    x = _deformed(mesh)
    scale = np.abs(_add(_fem(oracle, mesh, method), x)).max()
    assert not _add(fem, x).any()  # first call: the plastic strain is the strain itself
    assert not _add(fem, x).any()
    # at other positions the plastic strain follows to rounding
    # (ps + (JtD - ps) need not equal JtD exactly)
    for x in (_deformed(mesh, 0.1, seed=2), mesh.positions):
        assert np.abs(_add(fem, x)).max() <= 1e-12 * scale


@pytest.mark.parametrize("method", METHODS)
def test_partial_creep_scales_the_force(oracle, method):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    x = _deformed(mesh)
    f_el = _add(_fem(oracle, mesh, method), x)
    c = 0.25
    fem = _fem(oracle, mesh, method)
    fem.set_plasticity(1e9, 0.0, c)
    scale = np.abs(f_el).max()
    for n in (1, 2, 3):
        f = _add(fem, x)
        assert np.abs(f - (1 - c) ** n * f_el).max() <= 1e-12 * scale, n


@pytest.mark.parametrize("method", METHODS)
def test_clamp_keeps_the_plastic_norm_at_the_maximum(oracle, method):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    x = _deformed(mesh, 0.1)
    free = _fem(oracle, mesh, method)
    free.set_plasticity(1e9, 0.0, 1.0)
    _add(free, x)
    strain = np.linalg.norm(free.plastic_strain(), axis=1)  # the total strain of each element
    mx = float(np.median(strain))
    fem = _fem(oracle, mesh, method)
    fem.set_plasticity(mx, 0.0, 1.0)
    _add(fem, x)
    ps = np.linalg.norm(fem.plastic_strain(), axis=1)
    big = strain > mx
    assert big.any() and (~big).any()
    assert np.allclose(ps[big], mx, rtol=1e-12)
    assert np.allclose(ps[~big], strain[~big], rtol=1e-12)


@pytest.mark.parametrize("method", METHODS)
def test_below_yield_nothing_changes(oracle, method):
    mesh = cases.beam_mesh(n=(3, 3, 6))
    x = _deformed(mesh)
    f_el = _add(_fem(oracle, mesh, method), x)
    fem = _fem(oracle, mesh, method)
    fem.set_plasticity(1.0, 1e9, 1.0)
    assert np.array_equal(_add(fem, x), f_el)
    assert not fem.plastic_strain().any()
