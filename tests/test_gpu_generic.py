"""GPU parity of the generic kernels (forms outside the coefficient
channels) through the public API, against scikit-fem's own outputs
(tests/golden, generic_cases of make_golden.py).  The local values are the
reference's bit for bit; CSR patterns are compared bit-exact, CSR values
within the usual bounds (the segmented sum's fixed order is not scipy's),
interpolated fields and per-cell functional values bitwise where every
operation is correctly rounded."""
import numpy as np
import pytest
import torch

import oracle as O
import skfem_gb300 as F
from skfem_gb300 import helpers as H
from skfem_gb300.models.poisson import laplace, mass
from _generic import (SCALAR_CASES, energy, fixture_csr, newton, newton_res, qp_coef,
                      reference_csr, trig_load, vec_conv, vec_energy)
from _util import REL_FRO, REL_MAX, csr_diff, golden

pytestmark = pytest.mark.gpu

MESH = {3: F.MeshTri, 4: F.MeshTet, 8: F.MeshHex}


def basis_of(g, elem, intorder=None):
    b = F.Basis(MESH[g["t"].shape[0]](g["p"], g["t"]), elem, intorder=intorder)
    np.testing.assert_array_equal(b.element_dofs, g["element_dofs"])
    np.testing.assert_array_equal(b.X, g["X"])
    return b


def check_csr(K, ip, ix, d):
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, ip, ix, d,
                                                   K.shape)
    assert same, "pattern differs: %d extra, %d missing (max %.3g)" % (extra, missing, noise)
    assert rf <= REL_FRO, rf
    assert rm <= REL_MAX, rm


@pytest.mark.parametrize("name,elem,forms", SCALAR_CASES, ids=[c[0] for c in SCALAR_CASES])
def test_generic_forms_vs_reference(name, elem, forms):
    g = golden(name)
    b = basis_of(g, elem())
    for suffix, form in forms.items():
        check_csr(form.assemble(b), *fixture_csr(g, suffix))
    check_csr(qp_coef.assemble(b, c=g["c"]), *fixture_csr(g, "qp"))
    # a DOF vector, its DiscreteField and a device tensor give the same matrix
    Ks = [newton.assemble(b, s=g["s"]), newton.assemble(b, s=b.interpolate(g["s"])),
          newton.assemble(b, s=torch.as_tensor(g["s"], device="cuda"))]
    for K in Ks:
        check_csr(K, *fixture_csr(g, "newton"))
        np.testing.assert_array_equal(K.data, Ks[0].data)
    bn = newton_res.assemble(b, s=g["s"])
    np.testing.assert_allclose(bn, g["b_newton"], rtol=0, atol=1e-13 * np.abs(bn).max())
    if "b_trig" in g:
        bt = trig_load.assemble(b)
        np.testing.assert_allclose(bt, g["b_trig"], rtol=0, atol=1e-13 * np.abs(bt).max())


@pytest.mark.parametrize("name,elem", [(c[0], c[1]) for c in SCALAR_CASES],
                         ids=[c[0] for c in SCALAR_CASES])
def test_interpolate_and_functional_vs_reference(name, elem):
    g = golden(name)
    b = basis_of(g, elem())
    f = b.interpolate(g["s"])
    np.testing.assert_array_equal(np.asarray(f), g["s_value"])
    np.testing.assert_array_equal(f.grad, g["s_grad"])
    e = energy.elemental(b, s=g["s"])
    tot = energy.assemble(b, s=g["s"])
    if b.mesh.p.shape[0] == 2:
        # every operation correctly rounded (h = sqrt|det|): bitwise
        np.testing.assert_array_equal(e, g["e_energy"])
        assert tot == g["f_energy"]
    else:
        # h = |det|**(1/3) through the CUDA math library
        np.testing.assert_allclose(e, g["e_energy"], rtol=1e-15, atol=0)
        assert abs(tot - g["f_energy"]) <= 1e-14 * abs(g["f_energy"])
    assert isinstance(tot, np.float64)


def test_vector_generic_vs_reference():
    g = golden("tet_p2_vec_generic")
    b = basis_of(g, F.ElementVector(F.ElementTetP2()), intorder=4)
    f = b.interpolate(g["d"])
    np.testing.assert_array_equal(np.asarray(f), g["d_value"])
    np.testing.assert_array_equal(f.grad, g["d_grad"])
    check_csr(vec_conv.assemble(b, d=g["d"]), *fixture_csr(g, "conv"))
    np.testing.assert_array_equal(vec_energy.elemental(b, d=g["d"]), g["e_energy"])
    assert vec_energy.assemble(b, d=g["d"]) == g["f_energy"]


def test_generic_local_matrices_are_the_reference_bitwise():
    """elemental_torch on the generic path returns the reference's local
    matrices: scipy's own COO -> CSR of them reproduces the fixture
    bit for bit, values included."""
    g = golden("tri_p2_generic")
    b = basis_of(g, F.ElementTriP2())
    from _generic import aniso_adv
    local = aniso_adv.elemental_torch(b).cpu().numpy()
    K = reference_csr(local, b.element_dofs, b.N)
    ip, ix, d = fixture_csr(g, "aniso")
    np.testing.assert_array_equal(K.indptr, ip)
    np.testing.assert_array_equal(K.indices, ix)
    np.testing.assert_array_equal(K.data, d)


def test_generic_reruns_bitwise_and_stale_pattern():
    g = golden("tet_p1_generic")
    b = basis_of(g, F.ElementTetP1())
    c = g["c"].copy()
    K1 = qp_coef.assemble(b, c=c)
    K1b = qp_coef.assemble(b, c=c)
    np.testing.assert_array_equal(K1.data, K1b.data)
    c[:10] = 0.0                        # exact zeros: entries leave the pattern
    K2 = qp_coef.assemble(b, c=c)
    local = qp_coef.elemental_torch(b, c=c).cpu().numpy()
    Kr = reference_csr(local, b.element_dofs, b.N)
    assert K2.nnz < K1.nnz
    np.testing.assert_array_equal(K2.indptr, Kr.indptr)
    np.testing.assert_array_equal(K2.indices, Kr.indices)
    np.testing.assert_allclose(K2.data, Kr.data, rtol=0, atol=1e-13 * np.abs(Kr.data).max())


@pytest.mark.parametrize("kind,elem,intorder", [("tri", "TriP1", 1), ("tri", "TriP2", 2),
                                                ("tet", "TetP2", 3), ("hex", "Hex1", 3)])
def test_other_quadrature_orders_vs_oracle(kind, elem, intorder):
    """A basis whose rule the channel kernels do not integrate with (too low
    an order, another Hex1 rule) assembles through the generic kernels with
    the reference's quadrature."""
    rng = np.random.default_rng(3)
    if kind == "tri":
        m = F.MeshTri.init_tensor(np.linspace(0, 1, 7), np.linspace(0, 1, 6))
    elif kind == "tet":
        m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 4),) * 3)
    else:
        m = F.MeshHex.init_tensor(*(np.linspace(0, 1, 4),) * 3)
    p = m.p + rng.uniform(-0.02, 0.02, m.p.shape) * (np.abs(m.p - 0.5) < 0.49).all(axis=0)
    m = type(m)(p, m.t)
    b = F.Basis(m, getattr(F, "Element" + elem)(), intorder=intorder)
    assert not b._fast_ok
    bo = O.OBasis(O.OMesh(m.p, m.t, kind), getattr(O, elem)(), intorder=intorder)
    np.testing.assert_array_equal(b.X, bo.X)
    for f, fo in ((laplace, O.laplace), (mass, O.mass)):
        K = f.assemble(b)
        Ko = O.bilinear_assemble(fo, bo)
        same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data,
                                                       Ko.indptr, Ko.indices, Ko.data, K.shape)
        assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)
        assert noise <= REL_MAX


def test_asm_and_functional_api():
    g = golden("tri_p2_generic")
    b = basis_of(g, F.ElementTriP2())
    tot = F.asm(energy, b, s=g["s"])
    assert tot == g["f_energy"]
    area = F.Functional(lambda w: 1.0 + 0.0 * w.x[0]).assemble(b)
    assert abs(area - 1.0) < 1e-14
    # a Functional on a plain per-cell coefficient
    k = np.arange(b.nelems, dtype=np.float64)
    e = F.Functional(lambda w: w.k).elemental(b, k=b.zero_w() + k[:, None])
    cell_area = F.Functional(lambda w: 1.0 + 0.0 * w.x[0]).elemental(b)
    np.testing.assert_allclose(e, k * cell_area, rtol=1e-14)


def test_helpers_mul_and_trace_in_generic_forms():
    """A form with an explicit anisotropic tensor A (mul, transpose) against
    the oracle evaluating the same callable on numpy arrays."""
    A = np.array([[2.0, 0.3], [0.3, 0.5]])

    def form(u, v, w):
        Au = H.mul(np.array([[A[0, 0], A[0, 1]], [A[1, 0], A[1, 1]]]), H.grad(u))
        return H.dot(Au, H.grad(v)) + w.x[1] * u * v

    m = F.MeshTri.init_tensor(np.linspace(0, 1, 9), np.linspace(0, 1, 5))
    b = F.Basis(m, F.ElementTriP2())
    K = F.BilinearForm(form).assemble(b)
    bo = O.OBasis(O.OMesh(m.p, m.t, "tri"), O.TriP2())
    Ko = O.bilinear_assemble(form, bo)
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, Ko.indptr,
                                                   Ko.indices, Ko.data, K.shape)
    assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)


def test_compiled_programs_equal_the_interpreter(monkeypatch):
    """Programs compiled to straight-line code (NVRTC, -fmad=false) give the
    interpreter's local matrices, vectors and functional values bit for bit."""
    from _facet import robin, s_energy
    from skfem_gb300.tracer import FieldSpec  # noqa: F401
    g = golden("tri_p2_generic")
    b = basis_of(g, F.ElementTriP2())
    gf = golden("tet_p1_facet")
    fb = F.FacetBasis(F.MeshTet(gf["p"], gf["t"]), F.ElementTetP1())
    runs = []
    for jit in ("1", "0"):
        monkeypatch.setenv("SKFEM_GB300_JIT", jit)
        runs.append([newton.elemental_torch(b, s=g["s"]).cpu().numpy(),
                     qp_coef.elemental_torch(b, c=g["c"]).cpu().numpy(),
                     energy.elemental(b, s=g["s"]),
                     robin.elemental_torch(fb).cpu().numpy(),
                     s_energy.elemental(fb, s=gf["s"]),
                     newton_res.assemble(b, s=g["s"])])
    for a, c in zip(*runs):
        np.testing.assert_array_equal(a, c)


def test_mixed_bases_vs_reference():
    """Different trial and test bases (Stokes divergence block, its
    transpose, a P2 x P1 coupling with a trial-side DOF vector) against the
    reference: rectangular CSR, pattern bit-exact, values within the bounds."""
    from _generic import bdiv, bdiv_t, coupling
    g = golden("tri_mixed")
    m = F.MeshTri(g["p"], g["t"])
    ub = F.Basis(m, F.ElementVector(F.ElementTriP2()))
    pb = F.Basis(m, F.ElementTriP1(), intorder=4)
    sb = F.Basis(m, F.ElementTriP2())
    for K, sfx in ((bdiv.assemble(ub, pb), "bdiv"), (bdiv_t.assemble(pb, ub), "bdivt"),
                   (coupling.assemble(sb, pb, s=g["s"]), "coupling")):
        assert tuple(K.shape) == tuple(g["shape_" + sfx])
        same, extra, missing, noise, rf, rm = csr_diff(
            K.indptr, K.indices, K.data, g["indptr_" + sfx], g["indices_" + sfx],
            g["data_" + sfx], K.shape)
        assert same and rf <= REL_FRO and rm <= REL_MAX, (sfx, extra, missing, rf, rm)
    T = bdiv.assemble_torch(ub, pb)
    assert tuple(T.shape) == (pb.N, ub.N)
    with pytest.raises(ValueError):
        bdiv.assemble(ub, F.Basis(m, F.ElementTriP1()))       # quadrature mismatch
    gt = golden("tet_mixed")
    mt = F.MeshTet(gt["p"], gt["t"])
    K = bdiv.assemble(F.Basis(mt, F.ElementVector(F.ElementTetP2())),
                      F.Basis(mt, F.ElementTetP1(), intorder=4))
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, gt["indptr_bdiv"],
                                                   gt["indices_bdiv"], gt["data_bdiv"], K.shape)
    assert same and rf <= REL_FRO and rm <= REL_MAX


def test_asm_sums_over_lists_of_bases():
    """asm(form, [b1, b2]) sums the assemblies over both bases (here two
    element subsets covering the mesh), as COOData addition does."""
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 7), np.linspace(0, 1, 6))
    left = F.Basis(m, F.ElementTriP2(), elements=lambda x: x[0] < 0.5)
    right = F.Basis(m, F.ElementTriP2(), elements=lambda x: x[0] >= 0.5)
    full = F.Basis(m, F.ElementTriP2())
    K = F.asm(laplace, [left, right])
    Kf = laplace.assemble(full)
    np.testing.assert_array_equal(K.indptr, Kf.indptr)
    np.testing.assert_array_equal(K.indices, Kf.indices)
    np.testing.assert_allclose(K.data, Kf.data, rtol=0, atol=1e-13 * np.abs(Kf.data).max())
    b = F.asm(F.LinearForm(lambda v, w: 1.0 * v), [left, right])
    np.testing.assert_allclose(b, F.LinearForm(lambda v, w: 1.0 * v).assemble(full), atol=1e-15)


def test_vector_hex_vs_reference():
    """ElementVector(ElementHex1) on the generic kernels: elasticity matrix,
    FacetBasis traction load and interpolation against the reference."""
    from skfem_gb300.models.elasticity import linear_elasticity
    g = golden("hex1_vec")
    m = F.MeshHex(g["p"], g["t"])
    e = F.ElementVector(F.ElementHex1())
    b = F.Basis(m, e)
    np.testing.assert_array_equal(b.element_dofs, g["element_dofs"])
    check_csr(linear_elasticity(1.0, 0.5).assemble(b), *fixture_csr(g, "elast"))
    f = b.interpolate(g["d"])
    np.testing.assert_array_equal(np.asarray(f), g["d_value"])
    np.testing.assert_array_equal(f.grad, g["d_grad"])
    fb = F.FacetBasis(m, e)
    traction = F.LinearForm(lambda v, w: (1.0 + w.x[2]) * H.dot(w.n, v))
    bt = traction.assemble(fb)
    np.testing.assert_allclose(bt, g["b_traction"], rtol=0, atol=1e-13 * np.abs(bt).max())
