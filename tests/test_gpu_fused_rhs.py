"""The mixed patch step forms the forces and the right-hand side in two
passes instead of the four kernels of the element-order step (k_elem_force,
k_gather_force, k_elem_dforce on v, k_gather_rhs): by default one pass over
the patches that sums each element's force and (h + rs) K v terms per local
node in shared memory (k_patch_force_rhs) and one over the nodes
(k_rhs_finish_patch); with SGB_PATCH_RHS=0 one pass over the elements and
one over the nodes in element order (k_elem_force_rhs, k_gather_force_rhs);
SGB_FUSED_RHS=0 at creation selects the four kernels. All three perform the
same operations on the same values, but the patch form sums in patch order,
and in the FMA-contracting FP32 build the compiler fuses multiply-adds per
kernel, so the fused element passes can come out with other contractions
than the separate ones (they did for polar and svd once the
updateStiffnessMatrix path joined the force kernel): the trajectories agree
to the rounding of the element terms (displacement-relative difference
within 1e-4 after 8 steps, the bar of the mixed path against FP64; measured
up to 1.6e-5 for the element-order pair, with the velocity projection and
vdamping), not necessarily bit for bit. Checked over 8 steps for the rotated
methods and the options that enter the right-hand side: the components'
Rayleigh coefficients, firstOrder, trapezoidalScheme, projectVelocity,
vdamping, per-node masses, mass_first, an external force, plasticity.
"""
import os

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sofa_gb300 import build, capi

    build.build()
    capi.load()
    return capi


CASES = {
    "plain": dict(),
    "component_rayleigh": dict(ff_rayleigh_stiffness=0.05, mass_rayleigh_mass=0.03),
    "first_order": dict(first_order=True),
    "trapezoidal_project": dict(trapezoidal_scheme=True, project_velocity=True, vdamping=0.5),
    "node_masses_mass_last": dict(node_masses="ramp", mass_first=False),
    "external_force": dict(external="tip"),
    "plasticity": dict(plastic=True),
}


# the three forms of the force and right-hand side passes: the
# environment at creation
FORMS = {"patch": {"SGB_FUSED_RHS": "1", "SGB_PATCH_RHS": "1"},
         "element": {"SGB_FUSED_RHS": "1", "SGB_PATCH_RHS": "0"},
         "four": {"SGB_FUSED_RHS": "0", "SGB_PATCH_RHS": "0"}}


def run(capi, mesh, method, case, form, steps=8):
    opts = dict(CASES[case])
    ext = opts.pop("external", None)
    plastic = opts.pop("plastic", False)
    if opts.get("node_masses") == "ramp":
        opts["node_masses"] = np.linspace(0.5, 1.5, mesh.n_nodes) / mesh.n_nodes
    old = {k: os.environ.get(k) for k in FORMS[form]}
    os.environ.update(FORMS[form])
    try:
        fem = capi.TetrahedronFEM(mesh.positions, mesh.tetrahedra, 5000.0, 0.45, method, "mixed")
        if plastic:
            fem.set_plasticity(1e-2, 1e-6, 0.5)
        sc = capi.Scene(fem, dt=0.01, rayleigh_stiffness=0.1, rayleigh_mass=0.1, cg_iterations=25,
                        cg_tolerance=1e-9, cg_threshold=1e-9, gravity=(0.0, -9.81, 0.0),
                        vertex_mass=1.0 / mesh.n_nodes, fixed=mesh.fixed, **opts)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v
    v0 = np.random.default_rng(8).normal(scale=0.05, size=mesh.positions.shape)
    sc.set_state(mesh.positions, v0)
    if ext is not None:
        f = np.zeros_like(mesh.positions)
        tip = mesh.positions[:, 2] >= mesh.positions[:, 2].max() - 1e-9
        f[tip] = (0.0, -2e-3, 1e-3)
        sc.set_external_force(f)
    sc.step(steps)
    it, res = sc.sync()
    x, v = sc.state()
    sc.close()
    return x, v, it, res


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("method", ["large", "polar", "svd"])
def test_fused_force_and_rhs(capi, method, case):
    mesh = cases.beam_mesh()
    b = run(capi, mesh, method, case, "four")
    d = np.linalg.norm(b[0] - mesh.positions)
    assert d > 0  # the scene moved
    for form in ("patch", "element"):
        a = run(capi, mesh, method, case, form)
        assert np.linalg.norm(a[0] - b[0]) / d <= 1e-4, (form, np.linalg.norm(a[0] - b[0]) / d)


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-4), ("fp64_fma", 1e-12)])
def test_batch_fused_force_and_rhs(capi, precision, tol):
    """The batch engine's two passes against its four (SGB_FUSED_RHS=0 at
    batch creation), on beams of the batched workload's population (both
    methods), 5 steps: by patches (kb_force_rhs_patch, kb_rhs_finish_patch;
    mixed precision only, the FP64 batch keeps the element-order pair) and by
    elements (kb_force_rhs_elem, kb_force_rhs_gather; SGB_PATCH_RHS=0). The
    passes do the same operations, but the patch form sums in patch order,
    and in these FMA-contracting builds the compiler fuses multiply-adds per
    kernel, so the batch's fused element pass (both methods and the
    right-hand side in one kernel) comes out with other contractions than
    its two separate passes: the trajectories agree to the rounding of the
    element terms (displacement-relative difference within `tol`), not bit
    for bit."""
    from sofa_gb300 import workloads as wl

    beams = wl.beam_population(64, seed=5, members=range(0, 64, 8))
    out = {}
    for form in ("four", "element", "patch"):
        old = {k: os.environ.get(k) for k in FORMS[form]}
        os.environ.update(FORMS[form])
        try:
            b = capi.Batch(precision, budget_bytes=4 << 30, max_meshes=len(beams) + 1)
        finally:
            for k, v in old.items():
                if v is None:
                    del os.environ[k]
                else:
                    os.environ[k] = v
        slots = b.add_meshes([(m.positions, m.tetrahedra, kw) for m, kw in beams], threads=8)
        b.step(5)
        out[form] = [b.state(s) for s in slots]
        b.close()
    for form in ("element", "patch"):
        worst = 0.0
        for (m, _), (xa, _), (xb, _) in zip(beams, out[form], out["four"]):
            d = np.linalg.norm(xb - m.positions)
            worst = max(worst, float(np.linalg.norm(xa - xb) / d))
        assert worst <= tol, (form, worst)


def test_batch_patch_form_as_accurate_as_element_form(capi):
    """Accuracy guard of the patch form: against an FP64-FMA batch of the
    same beams (5 steps), the mixed patch form's error stays within 1.5x the
    mixed element form's (measured 2.16e-5 against 2.11e-5). Forming the
    edges from positions relative to a patch point instead of per element
    (about 2^-44 of the edge instead of 2^-47) gave 1.34e-4 here: the strain
    of stiff, lightly loaded beams needs those bits."""
    from sofa_gb300 import workloads as wl

    beams = wl.beam_population(64, seed=5, members=range(0, 64, 8))

    def run(precision, form):
        old = {k: os.environ.get(k) for k in FORMS[form]}
        os.environ.update(FORMS[form])
        try:
            b = capi.Batch(precision, budget_bytes=4 << 30, max_meshes=len(beams) + 1)
        finally:
            for k, v in old.items():
                if v is None:
                    del os.environ[k]
                else:
                    os.environ[k] = v
        slots = b.add_meshes([(m.positions, m.tetrahedra, kw) for m, kw in beams], threads=8)
        b.step(5)
        out = [b.state(s)[0] for s in slots]
        b.close()
        return out

    ref = run("fp64_fma", "element")

    def worst(xs):
        return max(float(np.linalg.norm(x - r) / np.linalg.norm(r - m.positions))
                   for (m, _), x, r in zip(beams, xs, ref))

    e_elem = worst(run("mixed", "element"))
    e_patch = worst(run("mixed", "patch"))
    assert e_patch <= 1.5 * e_elem + 1e-6, (e_patch, e_elem)
