"""Pin the CPU oracle against fixtures produced by scikit-fem itself."""
import os

import numpy as np
import pytest

import oracle as O

G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return dict(np.load(os.path.join(G, name + ".npz")))


def check_csr(K, g, rtol=1e-12):
    np.testing.assert_array_equal(K.indptr, g["indptr"])
    np.testing.assert_array_equal(K.indices, g["indices"])
    d, gd = K.data, g["data"]
    assert np.linalg.norm(d - gd) <= rtol * np.linalg.norm(gd)
    assert np.max(np.abs(d - gd)) <= 1e-13 * np.max(np.abs(gd))


def basis_from(g, elem, kind, intorder=None):
    m = O.OMesh(g["p"], g["t"], kind)
    b = O.OBasis(m, elem, intorder=intorder)
    np.testing.assert_array_equal(b.element_dofs, g["element_dofs"])
    np.testing.assert_array_equal(b.X, g["X"])
    np.testing.assert_array_equal(b.W, g["W"])
    return b


def test_meshes_match_reference_constructors():
    g = load("tri_p1_laplace")
    m = O.mesh_tri_tensor(np.linspace(0, 1, 17), np.linspace(0, 1, 17))
    np.testing.assert_array_equal(m.p, g["p"])
    np.testing.assert_array_equal(m.t, g["t"])
    g = load("tet_p1_k_laplace_mass")
    m = O.mesh_tet_tensor(*(np.linspace(0, 1, 7),) * 3)
    np.testing.assert_array_equal(m.p, g["p"])
    np.testing.assert_array_equal(m.t, g["t"])
    g = load("hex1_laplace_8")
    m = O.mesh_hex_tensor(*(np.linspace(0, 1, 9),) * 3)
    np.testing.assert_array_equal(m.p, g["p"])
    np.testing.assert_array_equal(m.t, g["t"])
    g = load("tri_default_mass")
    m = O.mesh_tri_default()
    np.testing.assert_array_equal(m.t, g["t"])


def test_tri_default_mass():
    g = load("tri_default_mass")
    b = basis_from(g, O.TriP1(), "tri")
    check_csr(O.bilinear_assemble(O.mass, b), g)


def test_tri_p1_laplace_and_load():
    g = load("tri_p1_laplace")
    b = basis_from(g, O.TriP1(), "tri")
    check_csr(O.bilinear_assemble(O.laplace, b), g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=0)


def test_tet_p1_k_laplace_mass():
    g = load("tet_p1_k_laplace_mass")
    b = basis_from(g, O.TetP1(), "tet")
    k = b.zero_w() + g["k"][:, None]
    check_csr(O.bilinear_assemble(O.k_laplace_mass, b, k=k), g)
    np.testing.assert_allclose(O.linear_assemble(O.f_load, b, f=k), g["b"], rtol=1e-13, atol=0)


def test_tet_p2_vec_elasticity():
    g = load("tet_p2_vec_elasticity")
    b = basis_from(g, O.Vector(O.TetP2()), "tet", intorder=4)
    check_csr(O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), b), g)


def test_tet_p2_laplace_exact_zeros():
    g = load("tet_p2_laplace")
    b = basis_from(g, O.TetP2(), "tet")
    check_csr(O.bilinear_assemble(O.laplace, b), g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=1e-17)


def test_tri_p2_k_laplace():
    g = load("tri_p2_k_laplace")
    b = basis_from(g, O.TriP2(), "tri")
    k = b.zero_w() + g["k"][:, None]
    check_csr(O.bilinear_assemble(O.k_laplace, b, k=k), g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=1e-17)


def test_hex1_theta_laplace_and_gradients():
    g = load("hex1_theta_laplace")
    b = basis_from(g, O.Hex1(), "hex")
    th = b.zero_w() + g["theta"][:, None]
    check_csr(O.bilinear_assemble(O.theta_laplace, b, theta=th), g)
    dth = O.theta_gradient(O.laplace, b, g["wv"], g["uv"])
    np.testing.assert_allclose(dth, g["dtheta"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(O.linear_assemble(O.f_load, b, f=th), g["b"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("name,elem,kind", [
    ("hex1_laplace_8", O.Hex1(), "hex"),
    ("tet_p1_jitter_laplace", O.TetP1(), "tet"),
])
def test_laplace_cases(name, elem, kind):
    g = load(name)
    b = basis_from(g, elem, kind)
    check_csr(O.bilinear_assemble(O.laplace, b), g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=1e-17)


@pytest.mark.parametrize("refdom,order", [("tri", 2), ("tri", 4), ("tet", 2), ("tet", 4)])
def test_closed_form_rules_match_reference_tables(refdom, order):
    X, W = O.quadrature(refdom, order)
    Xc, Wc = O.skfem_oracle.quadrature_closed_form(refdom, order)
    np.testing.assert_allclose(Xc, X, rtol=0, atol=2e-15)
    np.testing.assert_allclose(Wc, W, rtol=0, atol=2e-15)


def test_element_subsets():
    g = load("tri_p2_subset")
    m = O.OMesh(g["p"], g["t"], "tri")
    b = O.OBasis(m, O.TriP2(), elements=lambda x: x[0] < 0.5)
    np.testing.assert_array_equal(b.element_dofs, g["element_dofs"])
    check_csr(O.bilinear_assemble(O.k_laplace, b, k=b.zero_w() + g["k"][:, None]), g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=1e-17)
    g = load("tet_p1_subset")
    b = O.OBasis(O.OMesh(g["p"], g["t"], "tet"), O.TetP1(), elements=g["tind"])
    check_csr(O.bilinear_assemble(O.laplace, b), g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=1e-17)


def test_oracle_generic_forms_vs_reference():
    """The oracle's default parameters (w.x, w.h), DOF-vector interpolation
    and per-point coefficients against scikit-fem's outputs on the forms of
    the generic kernels."""
    from _generic import SCALAR_CASES, fixture_csr, newton, qp_coef
    kinds = {3: "tri", 4: "tet", 8: "hex"}
    elems = {"tri_p2_generic": O.TriP2(), "tet_p1_generic": O.TetP1(),
             "hex1_generic": O.Hex1()}
    for name, _, forms in SCALAR_CASES:
        g = load(name)
        bo = O.OBasis(O.OMesh(g["p"], g["t"], kinds[g["t"].shape[0]]), elems[name])
        d = bo.default_parameters()
        np.testing.assert_array_equal(d["x"], g["x"])
        np.testing.assert_allclose(d["h"], g["h"], rtol=1e-15, atol=0)
        f = bo.interpolate(g["s"])
        np.testing.assert_array_equal(np.asarray(f), g["s_value"])
        np.testing.assert_array_equal(f.grad, g["s_grad"])
        cases = [(forms["aniso"], {}, "aniso"), (qp_coef, {"c": g["c"]}, "qp"),
                 (newton, {"s": g["s"]}, "newton")]
        for form, kw, suffix in cases:
            K = O.bilinear_assemble(form.form, bo, **kw)
            ip, ix, dat = fixture_csr(g, suffix)
            np.testing.assert_array_equal(K.indptr, ip)
            np.testing.assert_array_equal(K.indices, ix)
            np.testing.assert_array_equal(K.data, dat)


def test_oracle_mixed_bases_vs_reference():
    """BilinearForm.assemble(ubasis, vbasis) with different trial and test
    bases (bilinear_form.py:58-128): the oracle's two-basis loop against the
    reference, bit for bit."""
    from _generic import bdiv, bdiv_t, coupling
    g = load("tri_mixed")
    m = O.OMesh(g["p"], g["t"], "tri")
    ub = O.OBasis(m, O.Vector(O.TriP2()))
    pb = O.OBasis(m, O.TriP1(), intorder=4)
    sb = O.OBasis(m, O.TriP2())
    for form, u, v, kw, sfx in ((bdiv, ub, pb, {}, "bdiv"), (bdiv_t, pb, ub, {}, "bdivt"),
                                (coupling, sb, pb, {"s": g["s"]}, "coupling")):
        K = O.bilinear_assemble(form.form, u, v, **kw)
        np.testing.assert_array_equal(K.indptr, g["indptr_" + sfx])
        np.testing.assert_array_equal(K.indices, g["indices_" + sfx])
        np.testing.assert_array_equal(K.data, g["data_" + sfx])


def _edge(name, g):
    sub = {k[len(name) + 1:]: v for k, v in g.items() if k.startswith(name + "_")}
    return sub


@pytest.mark.parametrize("name", ["unused_node", "single", "empty_subset"])
def test_edge_cases(name):
    """A node no cell uses (no DOF: the reference numbers up to max(t)), a
    single cell, an empty element subset -- CSR and load as the reference."""
    g = _edge(name, load("edge_cases"))
    m = O.OMesh(g["p"], g["t"], "tet")
    b = O.OBasis(m, O.TetP1(), elements=np.array([], dtype=np.int64)
                 if name == "empty_subset" else None)
    assert b.N == int(g["N"])
    K = O.bilinear_assemble(O.k_laplace_mass, b, k=b.zero_w() + g["k"][:, None])
    assert K.shape == tuple(g["shape"])
    np.testing.assert_array_equal(K.indptr, g["indptr"])
    np.testing.assert_array_equal(K.indices, g["indices"])
    if K.nnz:
        check_csr(K, g)
    np.testing.assert_allclose(O.linear_assemble(O.unit_load, b), g["b"], rtol=1e-13, atol=0)
