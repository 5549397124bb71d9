"""GPU parity of FacetBasis assembly (boundary, interior facets from either
side, callable facet subsets) through the public API against scikit-fem's
own outputs: CSR patterns bit-exact, values within the usual bounds,
interpolated fields and per-facet functional values bitwise."""
import numpy as np
import pytest

import skfem_gb300 as F
from skfem_gb300.models.poisson import laplace
from _facet import (CASES, VARIANTS, facet_args, fmass, length, neumann, robin, s_energy,
                    traction, vmass)
from _util import REL_FRO, REL_MAX, csr_diff, golden

pytestmark = pytest.mark.gpu


def check_csr(K, g, pre, suffix):
    same, extra, missing, noise, rf, rm = csr_diff(
        K.indptr, K.indices, K.data, g[pre + "indptr_" + suffix], g[pre + "indices_" + suffix],
        g[pre + "data_" + suffix], K.shape)
    assert same, "%s%s: pattern differs (%d extra, %d missing)" % (pre, suffix, extra, missing)
    assert rf <= REL_FRO and rm <= REL_MAX, (pre, suffix, rf, rm)


@pytest.mark.parametrize("name,mesh_cls,elem", CASES, ids=[c[0] for c in CASES])
def test_facet_basis_vs_reference(name, mesh_cls, elem):
    g = golden(name)
    m = mesh_cls(g["p"], g["t"])
    for pre in VARIANTS:
        fb = F.FacetBasis(m, elem(), **facet_args(m, g, pre))
        np.testing.assert_array_equal(fb.find, g[pre + "find"])
        np.testing.assert_array_equal(fb.tind, g[pre + "tind"])
        np.testing.assert_array_equal(fb.X, g[pre + "X"])
        check_csr(fmass.assemble(fb), g, pre, "mass")
        check_csr(robin.assemble(fb), g, pre, "robin")
        b = neumann.assemble(fb)
        np.testing.assert_allclose(b, g[pre + "b_neumann"], rtol=0,
                                   atol=1e-13 * np.abs(b).max())
        np.testing.assert_array_equal(length.elemental(fb), g[pre + "e_length"])
        assert length.assemble(fb) == g[pre + "f_length"]
        np.testing.assert_array_equal(s_energy.elemental(fb, s=g["s"]), g[pre + "e_energy"])
        assert s_energy.assemble(fb, s=g["s"]) == g[pre + "f_energy"]
        f = fb.interpolate(g["s"])
        np.testing.assert_array_equal(np.asarray(f), g[pre + "s_value"])
        np.testing.assert_array_equal(f.grad, g[pre + "s_grad"])


def test_vector_facet_basis_vs_reference():
    g = golden("tet_p2_vec_facet")
    m = F.MeshTet(g["p"], g["t"])
    fb = F.FacetBasis(m, F.ElementVector(F.ElementTetP2()))
    np.testing.assert_array_equal(fb.find, g["find"])
    check_csr(vmass.assemble(fb), g, "", "vmass")
    b = traction.assemble(fb)
    np.testing.assert_allclose(b, g["b_traction"], rtol=0, atol=1e-13 * np.abs(b).max())


def test_robin_problem_cell_plus_facet():
    """A Robin problem assembled from a CellBasis and a FacetBasis of the
    same mesh: the matrices add (same DOF numbering), and the solution of
    -lap u = 0, du/dn + u = g with g from u = x + 2y is reproduced."""
    import scipy.sparse.linalg as spla
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 9), np.linspace(0, 1, 9))
    ib = F.Basis(m, F.ElementTriP2())
    fb = F.FacetBasis(m, F.ElementTriP2())
    rob = F.BilinearForm(lambda u, v, w: u * v)
    rhs = F.LinearForm(lambda v, w: (w.n[0] + 2.0 * w.n[1] + w.x[0] + 2.0 * w.x[1]) * v)
    K = laplace.assemble(ib) + rob.assemble(fb)
    b = rhs.assemble(fb)
    u = spla.spsolve(K.tocsc(), b)
    x, y = m.p
    dofs = ib.element_dofs[:3]       # vertex DOFs of P2 on this mesh are 0..nverts-1
    np.testing.assert_allclose(u[:m.p.shape[1]], x + 2 * y, atol=1e-10)
    assert dofs.max() < ib.N
