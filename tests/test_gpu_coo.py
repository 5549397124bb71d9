"""COOData and the elemental API on the GPU against scikit-fem's own results
(tests/golden/coo_api.npz, made by make_golden.py --coo): Form.elemental /
coo_data (indices and data in the reference's order), COOData.tolocal
(cells and facets), tocsr / toarray / todefault on the device, inverse,
Form.block, and asm over lists of bases with the default and a custom
reducer (coo_data.py:19-242, form.py:53-89, assembly/__init__.py:69-97)."""
import numpy as np
import pytest

import skfem_gb300 as F
from skfem_gb300 import helpers as H
from skfem_gb300.models.poisson import laplace, mass, unit_load
from _util import golden

pytestmark = pytest.mark.gpu

G = golden("coo_api")
TOL = 1e-13


def _mesh():
    return F.MeshTri.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 4))


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.max(np.abs(a - b), initial=0.0) <= TOL * max(1.0, np.max(np.abs(b), initial=0.0))


def test_bilinear_elemental_and_coodata():
    b = F.Basis(_mesh(), F.ElementTriP1())
    A = laplace.elemental(b)
    np.testing.assert_array_equal(A.indices, G["lap_indices"])
    np.testing.assert_array_equal(A.data, G["lap_data"])          # the reference's, bitwise
    assert tuple(A.shape) == tuple(G["lap_shape"])
    assert tuple(A.local_shape) == tuple(G["lap_local_shape"])
    _close(A.tolocal(), G["lap_tolocal"])
    K = A.tocsr()
    np.testing.assert_array_equal(K.indptr, G["lap_indptr"])
    np.testing.assert_array_equal(K.indices, G["lap_csr_indices"])
    _close(K.data, G["lap_csr_data"])
    # coo_data is the older name; todefault of a 2-tensor is tocsr
    K2 = laplace.coo_data(b).todefault()
    np.testing.assert_array_equal(K2.data, K.data)
    # fromlocal(tolocal()) round trip
    np.testing.assert_array_equal(A.fromlocal(A.tolocal()).data, A.data)


def test_linear_elemental_and_toarray():
    b = F.Basis(_mesh(), F.ElementTriP1())
    L = unit_load.elemental(b)
    np.testing.assert_array_equal(L.indices, G["load_indices"])
    _close(L.data, G["load_data"])
    _close(L.toarray(), G["load_array"])
    _close(L.todefault(), G["load_array"])


def test_inverse_of_local_mass_matrices():
    b = F.Basis(_mesh(), F.ElementTriP1())
    _close(mass.coo_data(b).inverse().tocsr().toarray(), G["mass_inverse"])


def test_mixed_pair_elemental():
    m = _mesh()
    pb = F.Basis(m, F.ElementTriP2())
    qb = F.Basis(m, F.ElementTriP1(), intorder=4)

    @F.BilinearForm
    def mixed(u, v, w):
        return u.grad[0] * v + 0.5 * u * v.grad[1]
    C = mixed.elemental(pb, qb)
    np.testing.assert_array_equal(C.indices, G["mixed_indices"])
    _close(C.data, G["mixed_data"])
    assert tuple(C.shape) == tuple(G["mixed_shape"])
    assert tuple(C.local_shape) == tuple(G["mixed_local_shape"])


def test_asm_lists_and_reducers():
    m = _mesh()
    b1 = F.Basis(m, F.ElementTriP1(), elements=lambda x: x[0] < 0.5)
    b2 = F.Basis(m, F.ElementTriP1(), elements=lambda x: x[0] >= 0.5)
    S = F.asm(laplace, [b1, b2])
    np.testing.assert_array_equal(S.indptr, G["asm_sum_indptr"])
    np.testing.assert_array_equal(S.indices, G["asm_sum_indices"])
    _close(S.data, G["asm_sum_data"])
    parts = F.asm(laplace, [b1, b2], to=list)
    _close(parts[0].todefault().toarray(), G["asm_to_list_0"])
    _close(parts[1].todefault().toarray(), G["asm_to_list_1"])
    _close(F.asm(unit_load, [b1, b2]), G["asm_load_sum"])

    @F.BilinearForm
    def with_idx(u, v, w):
        return (1.0 + w.idx[0]) * u * v
    _close(F.asm(with_idx, [b1, b2]).toarray(), G["asm_idx"])


def test_block_of_a_product_form():
    b = F.Basis(_mesh(), F.ElementTriP1())

    @F.BilinearForm
    def prod(u1, u2, v1, v2, w):
        return H.dot(H.grad(u1), H.grad(v1)) + 2.0 * u2 * v2 + u1 * v2
    for i in (0, 1):
        for j in (0, 1):
            _close(F.asm(prod.block(i, j), b).toarray(), G["block_%d%d" % (i, j)])


def test_facet_matrices_summed_per_cell():
    m = _mesh()
    fb = F.FacetBasis(m, F.ElementTriP1())
    _close(mass.elemental(fb).tolocal(fb), G["facet_tolocal"])


def test_functional_coo_and_device_coo_sum():
    from skfem_gb300.coo import COOData
    b = F.Basis(_mesh(), F.ElementTriP1())

    @F.Functional
    def area(w):
        return 1.0 + 0.0 * w.x[0]
    c = area.coo_data(b)
    assert c.shape == () and abs(c.todefault() - 1.0) <= 1e-14
    # a general COO with duplicates, an exact zero and an entry that sums to 0
    rows = np.array([0, 1, 1, 2, 0, 2, 2], dtype=np.int32)
    cols = np.array([0, 1, 1, 0, 0, 2, 1], dtype=np.int32)
    data = np.array([1.0, 2.0, 3.0, 4.0, -1.0, 0.0, 5.0])
    K = COOData(np.stack([rows, cols]), data, (3, 3), None).tocsr()
    import scipy.sparse as sp
    R = sp.coo_matrix((data, (rows, cols)), shape=(3, 3))
    R.eliminate_zeros()
    R = R.tocsr()
    np.testing.assert_array_equal(K.indptr, R.indptr)
    np.testing.assert_array_equal(K.indices, R.indices)
    np.testing.assert_array_equal(K.data, R.data)
