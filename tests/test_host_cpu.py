"""Host-side logic that needs no GPU: meshes, DOF numbering, quadrature and
form tracing against the reference's fixtures and conventions."""
import numpy as np
import pytest

import skfem_gb300 as F
from skfem_gb300 import helpers as H
from skfem_gb300.tracer import bilinear_channels, linear_channels, trace_bilinear, trace_linear
from skfem_gb300.models.elasticity import linear_elasticity
from _util import golden


def test_tensor_meshes_and_dofs_match_reference():
    g = golden("tri_p1_laplace")
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 17), np.linspace(0, 1, 17))
    np.testing.assert_array_equal(m.p, g["p"])
    np.testing.assert_array_equal(m.t, g["t"])
    g = golden("tet_p1_k_laplace_mass")
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 7),) * 3)
    np.testing.assert_array_equal(m.p, g["p"])
    np.testing.assert_array_equal(m.t, g["t"])
    g = golden("hex1_laplace_8")
    m = F.MeshHex.init_tensor(*(np.linspace(0, 1, 9),) * 3)
    np.testing.assert_array_equal(m.p, g["p"])
    np.testing.assert_array_equal(m.t, g["t"])


@pytest.mark.parametrize("name,elem", [
    ("tet_p2_vec_elasticity", lambda: F.ElementVector(F.ElementTetP2())),
    ("tet_p2_laplace", F.ElementTetP2),
    ("tri_p2_k_laplace", F.ElementTriP2),
    ("hex1_theta_laplace", F.ElementHex1),
])
def test_element_dofs_match_reference(name, elem):
    g = golden(name)
    kind = {3: F.MeshTri, 4: F.MeshTet, 8: F.MeshHex}[g["t"].shape[0]]
    d = F.Dofs(kind(g["p"], g["t"]), elem())
    np.testing.assert_array_equal(d.element_dofs, g["element_dofs"])


@pytest.mark.parametrize("refdom,order,name", [
    ("tri", 2, "tri_p1_laplace"), ("tri", 4, "tri_p2_k_laplace"),
    ("tet", 2, "tet_p1_k_laplace_mass"), ("tet", 4, "tet_p2_vec_elasticity"),
    ("hex", 6, "hex1_laplace_8")])
def test_quadrature_matches_reference(refdom, order, name):
    g = golden(name)
    X, W = F.get_quadrature(refdom, order)
    np.testing.assert_allclose(X, g["X"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(W, g["W"], rtol=0, atol=1e-15)


def test_trace_scalar_forms():
    e = F.ElementTetP1()
    s = trace_bilinear(lambda u, v, w: w.k * H.dot(H.grad(u), H.grad(v)) + u * v, e, 3,
                       {"k": None}, {})
    assert bilinear_channels(s, e, 3) == {"diff": {("k",): 1.0}, "mass": {(): 1.0}}
    s = trace_bilinear(lambda u, v, w: 2.0 * (u.grad[0] * v.grad[0] + u.grad[1] * v.grad[1]
                                              + u.grad[2] * v.grad[2]), e, 3, {}, {})
    assert bilinear_channels(s, e, 3)["diff"] == {(): 2.0}
    s = trace_linear(lambda v, w: w.f * v, e, 3, {"f": None}, {})
    assert linear_channels(s, e, 3) == {"load": {("f",): 1.0}}


def test_trace_elasticity():
    e = F.ElementVector(F.ElementTetP2())
    ch = bilinear_channels(trace_bilinear(linear_elasticity(1.0, 0.5).form, e, 3, {}, {}), e, 3)
    assert ch["lam"] == {(): 1.0} and ch["lap"] == {(): 0.5} and ch["tr"] == {(): 0.5}


def test_trace_rejects_unsupported_forms():
    e = F.ElementTetP1()
    with pytest.raises(NotImplementedError):
        bilinear_channels(trace_bilinear(lambda u, v, w: u.grad[0] * v, e, 3, {}, {}), e, 3)
    with pytest.raises(NotImplementedError):
        bilinear_channels(trace_bilinear(lambda u, v, w: u.grad[0] * v.grad[0], e, 3, {}, {}),
                          e, 3)
    with pytest.raises(NotImplementedError):
        trace_bilinear(lambda u, v, w: u * u * v, e, 3, {}, {})
    with pytest.raises(NotImplementedError):
        trace_bilinear(lambda u, v, w: w.x[0] * u * v, e, 3, {}, {})


def test_basis_rejects_mismatch_without_gpu():
    with pytest.raises(ValueError):
        F.Basis(F.MeshTri(), F.ElementTetP1())


def test_get_dofs_match_reference():
    """Basis.get_dofs: boundary facets, a facet callable, a cell callable,
    for every element family and its vector version (dofs.py:539-662)."""
    import numpy as np
    import skfem_gb300 as F
    from skfem_gb300.dofs import Dofs
    from _util import golden
    g = golden("get_dofs")
    meshes = {"tri": F.MeshTri.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 4)),
              "tet": F.MeshTet.init_tensor(*(np.linspace(0, 1, 4),) * 3),
              "hex": F.MeshHex.init_tensor(*(np.linspace(0, 1, 4),) * 3)}
    elems = {"tri": ("ElementTriP1", "ElementTriP2"), "tet": ("ElementTetP1", "ElementTetP2"),
             "hex": ("ElementHex1",)}
    for kind, m in meshes.items():
        for name in elems[kind]:
            for vec in (0, 1):
                e = getattr(F, name)()
                d = Dofs(m, F.ElementVector(e) if vec else e)
                key = "%s_%s_%d" % (kind, name, vec)
                np.testing.assert_array_equal(
                    d.get_facet_dofs(m.normalize_facets(None)).flatten(), g[key + "_boundary"])
                np.testing.assert_array_equal(
                    d.get_facet_dofs(m.normalize_facets(lambda x: np.isclose(x[1], 0))).flatten(),
                    g[key + "_y0"])
                np.testing.assert_array_equal(
                    d.get_element_dofs(m.normalize_elements(lambda x: x[0] < 0.5)).flatten(),
                    g[key + "_left"])


def _host_basis(m, elem):
    """A CellBasis's host-side attributes only (no device arrays)."""
    from skfem_gb300.basis import CellBasis
    from skfem_gb300.dofs import Dofs
    b = CellBasis.__new__(CellBasis)
    b.mesh, b.elem, b.dofs = m, elem, Dofs(m, elem)
    return b


def test_doflocs_match_reference():
    """Basis.doflocs (abstract_basis.py:60-71) on jittered meshes, bit for bit."""
    import skfem_gb300 as F
    g = golden("doflocs")
    meshes = {"tri": F.MeshTri, "tet": F.MeshTet, "hex": F.MeshHex}
    elems = {"tri": (F.ElementTriP1, F.ElementTriP2), "tet": (F.ElementTetP1, F.ElementTetP2),
             "hex": (F.ElementHex1,)}
    for kind, cls in meshes.items():
        m = cls(g[kind + "_p"], g[kind + "_t"])
        for E in elems[kind]:
            for vec in (0, 1):
                b = _host_basis(m, F.ElementVector(E()) if vec else E())
                np.testing.assert_array_equal(b.doflocs, g["%s_%s_%d" % (kind, E.__name__, vec)],
                                              err_msg="%s %s %d" % (kind, E.__name__, vec))


def test_complement_dofs():
    import skfem_gb300 as F
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 4), np.linspace(0, 1, 3))
    b = _host_basis(m, F.ElementTriP1())
    D = np.array([0, 3, 5])
    np.testing.assert_array_equal(b.complement_dofs(D), np.setdiff1d(np.arange(b.N), D))
    np.testing.assert_array_equal(b.complement_dofs(np.array([1]), np.array([2, 7])),
                                  np.setdiff1d(np.arange(b.N), [1, 2, 7]))


def test_autotune_candidates_per_family():
    """The autotuner times every block size, grid and unroll; the scalar
    bases with an even number of local functions (TetP1, TriP2, TetP2) also
    try two columns per lane in the fused sum, the P1 simplex families the
    three forms of the one-pass sum and the scalar P2 families the two
    forms of the one-pass node-block sum (bitwise equal), the others and
    every vector basis one of each."""
    from skfem_gb300 import autotune
    base = 3 * 2 * 3
    for fam in ("TriP2", "TetP2"):
        c = autotune.candidates(fam)
        assert len(c) == 4 * base and {x["sum_cols"] for x in c} == {1, 2}
        assert {x["onepass"] for x in c} == {1, 2}
        v = autotune.candidates(fam, vector=True)
        assert len(v) == base and {x["onepass"] for x in v} == {1}
    c = autotune.candidates("TetP1")
    assert len(c) == 6 * base and {x["sum_cols"] for x in c} == {1, 2}
    assert {x["onepass"] for x in c} == {0, 1, 2}
    assert len(autotune.candidates("TetP1", vector=True)) == base
    c = autotune.candidates("TriP1")
    assert len(c) == 3 * base and {x["onepass"] for x in c} == {0, 1, 2}
    c = autotune.candidates("Hex1")
    assert len(c) == base and {x["sum_cols"] for x in c} == {1}
    c = autotune.candidates("TetP1")
    assert len({tuple(sorted(x.items())) for x in c}) == len(c)


def test_coodata_host_side_matches_reference_layout():
    """COOData's host-side operations on the reference's own arrays
    (coo_api.npz): tolocal / fromlocal reshape exactly as coo_data.py does,
    __add__ concatenates and widens the shape, sum() starts from 0."""
    from skfem_gb300.coo import COOData
    from _util import golden
    g = golden("coo_api")
    A = COOData(g["lap_indices"], g["lap_data"], tuple(g["lap_shape"]),
                tuple(g["lap_local_shape"]))
    np.testing.assert_array_equal(A.tolocal(), g["lap_tolocal"])
    np.testing.assert_array_equal(A.fromlocal(A.tolocal()).data, A.data)
    B = sum([A, A])
    assert B.indices.shape == (2, 2 * A.indices.shape[1]) and B.local_shape is None
    assert B.shape == A.shape
    idx, data, shape = A.astuple()
    assert idx is A.indices and data is A.data and shape == A.shape


def test_condense_dof_sets_match_setdiff1d():
    """The kept DOFs and their map that condense forms on the device (here
    with CPU tensors) equal the reference's np.setdiff1d(np.arange(n), D)
    (utils.py _init_bc), for empty, partial and full sets given as D, as I,
    as boolean masks and with duplicates; indices outside [0, n) raise."""
    import torch
    from skfem_gb300.utils import _bc_sets, _kept_map
    rng = np.random.default_rng(1)
    for n in (1, 5, 100, 10007):
        for k in sorted({0, 1, 3, n // 2, n}):
            if k > n:
                continue
            D = rng.choice(n, k, replace=False)
            ref = np.setdiff1d(np.arange(n), D)
            mask = np.zeros(n, dtype=bool)
            mask[D] = True
            for kw in ({"D": D}, {"D": np.concatenate([D, D[:2]])}, {"D": mask}, {"I": ref}):
                In, mp = _kept_map(n, kw.get("I"), kw.get("D"), "cpu")
                assert np.array_equal(In.numpy(), ref)
                want = np.full(n, -1)
                want[ref] = np.arange(len(ref))
                assert np.array_equal(mp.numpy(), want) and mp.dtype == torch.int32
            assert np.array_equal(_bc_sets(n, ref, None, "cpu").numpy(), np.unique(D))
    for bad in ([0, 5], [-1]):
        with pytest.raises(IndexError):
            _kept_map(5, None, np.array(bad), "cpu")
