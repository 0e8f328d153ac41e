"""von Mises stress (computeVonMisesStress, TetrahedronFEMForceField.inl:
2197-2374) on the GPU against the oracle, through the C ABI. The kernels run
in FP64 without FMA contraction for every precision of the force field, so
the per-element values are bit-identical to the oracle's; the per-node means
sum in the node table's order, which follows the element storage order of
the precision (bit-identical for the reference-rounding variant, within
1e-14 relative otherwise)."""
import os

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def capi():
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


@pytest.mark.parametrize("method,mode", [("large", 1), ("polar", 1), ("svd", 1), ("large", 2), ("polar", 2),
                                         ("small", 2)])
@pytest.mark.parametrize("precision", ["fp64", "fp64_fma", "mixed"])
def test_von_mises_against_oracle(torch_cuda, capi, oracle, method, mode, precision):
    torch = torch_cuda
    mesh = cases.beam_mesh()
    _, osc = cases.oracle_scene(oracle, mesh, "polar" if method == "small" else method)
    osc.step(15)
    x, _ = osc.state()
    e_ref, n_ref = oracle.OracleFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method).von_mises(x, mode)
    fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method, precision)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    ed = torch.zeros(mesh.n_tets, dtype=torch.float64, device="cuda")
    nd = torch.zeros(mesh.n_nodes, dtype=torch.float64, device="cuda")
    for _ in range(2):  # the second call reuses the kept Lame coefficients
        fem.von_mises(xd.data_ptr(), mode, ed.data_ptr(), nd.data_ptr())
        torch.cuda.synchronize()
        e, n = ed.cpu().numpy(), nd.cpu().numpy()
        assert np.array_equal(e, e_ref), np.abs(e - e_ref).max()
        if precision == "fp64":
            assert np.array_equal(n, n_ref)
        else:
            assert np.abs(n - n_ref).max() <= 1e-14 * np.abs(n_ref).max()
    assert e_ref.max() > 0
    fem.close()


def test_von_mises_mode_errors(torch_cuda, capi):
    torch = torch_cuda
    mesh = cases.beam_mesh(n=(3, 3, 4))
    xd = torch.tensor(mesh.positions, dtype=torch.float64, device="cuda")
    ed = torch.zeros(mesh.n_tets, dtype=torch.float64, device="cuda")
    small = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, "small", "fp64")
    with pytest.raises(capi.SgbError) as e:
        small.von_mises(xd.data_ptr(), 1, ed.data_ptr())
    assert e.value.code == -4
    with pytest.raises(capi.SgbError) as e:
        small.von_mises(xd.data_ptr(), 3, ed.data_ptr())
    assert e.value.code == -1


def test_von_mises_scene_file(capi, oracle):
    """computeVonMisesStress="2" on the known-answer grid scene: after 20 steps
    the body's vonMisesPerElement / vonMisesPerNode equal the oracle's at the
    same positions."""
    from sofa_gb300 import topology as topo

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "scenes", "grid_fem_4x10x4.scn")
    with open(path) as f:
        text = f.read().replace('<TetrahedronFEMForceField name="FEM"',
                                '<TetrahedronFEMForceField computeVonMisesStress="2" name="FEM"')
    s = capi.SofaScene(text)
    s.animate(20)
    x = s.positions(0)
    e, n = s.von_mises(0)
    pos, hexa = topo.regular_grid((4, 10, 4), (0, 0, 20), (10, 40, 30))
    tets = topo.hexa_to_tetra6(hexa, (3, 9))
    e_ref, n_ref = oracle.OracleFEM(pos, tets, 600.0, 0.3, "large").von_mises(x, 2)
    assert np.array_equal(e, e_ref)
    assert np.array_equal(n, n_ref)
    assert e.max() > 0
