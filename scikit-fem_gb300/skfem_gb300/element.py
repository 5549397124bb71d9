"""Element descriptors: the metadata of the reference's element classes the
kernels specialise on (the basis polynomials themselves live in the CUDA
kernels and the exact reference tensors of csrc/fem_tables.cuh).

  ElementTriP1 skfem/element/element_tri/element_tri_p1.py
  ElementTriP2 skfem/element/element_tri/element_tri_p2.py
  ElementTetP1 skfem/element/element_tet/element_tet_p1.py
  ElementTetP2 skfem/element/element_tet/element_tet_p2.py
  ElementHex1  skfem/element/element_hex/element_hex1.py
  ElementVector skfem/element/element_vector.py
"""

import numpy as np

__all__ = ["Element", "ElementTriP1", "ElementTriP2", "ElementTetP1", "ElementTetP2",
           "ElementHex1", "ElementVector", "ElementH1"]


class Element:
    family = ""
    refdom = ""
    dim = 0
    maxdeg = 0
    nodal_dofs = 0
    edge_dofs = 0
    facet_dofs = 0
    interior_dofs = 0
    nbfun_scalar = 0
    vector = False

    @property
    def nbfun(self):
        return self.nbfun_scalar

    def __repr__(self):
        return type(self).__name__ + "()"


class ElementH1(Element):
    pass


class ElementTriP1(ElementH1):
    family, refdom, dim, maxdeg = "TriP1", "tri", 2, 1
    nodal_dofs, nbfun_scalar = 1, 3
    # reference DOF locations (element_tri_p1.py:13-15)
    doflocs = np.array([[0., 0.], [1., 0.], [0., 1.]])


class ElementTriP2(ElementH1):
    family, refdom, dim, maxdeg = "TriP2", "tri", 2, 2
    nodal_dofs, facet_dofs, nbfun_scalar = 1, 1, 6
    # vertices, then edge midpoints (element_tri_p2.py:14-19)
    doflocs = np.array([[0., 0.], [1., 0.], [0., 1.], [.5, 0.], [.5, .5], [0., .5]])


class ElementTetP1(ElementH1):
    family, refdom, dim, maxdeg = "TetP1", "tet", 3, 1
    nodal_dofs, nbfun_scalar = 1, 4
    # element_tet_p1.py:13-16
    doflocs = np.array([[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.]])


class ElementTetP2(ElementH1):
    family, refdom, dim, maxdeg = "TetP2", "tet", 3, 2
    nodal_dofs, edge_dofs, nbfun_scalar = 1, 1, 10
    # vertices, then edge midpoints in the reference's edge order (element_tet_p2.py:14-23)
    doflocs = np.array([[0., 0., 0.], [1., 0., 0.], [0., 1., 0.], [0., 0., 1.],
                        [.5, 0., 0.], [.5, .5, 0.], [0., .5, 0.], [0., 0., .5],
                        [.5, 0., .5], [0., .5, .5]])


class ElementHex1(ElementH1):
    family, refdom, dim, maxdeg = "Hex1", "hex", 3, 3
    nodal_dofs, nbfun_scalar = 1, 8
    # element_hex1.py:13-20 (node k at the corner of refdom.py's node k)
    doflocs = np.array([[1., 1., 1.], [1., 1., 0.], [1., 0., 1.], [0., 1., 1.],
                        [1., 0., 0.], [0., 1., 0.], [0., 0., 1.], [0., 0., 0.]])


class ElementVector(Element):
    """Same scalar element per component; vector function i is component
    i % dim of scalar function i // dim (element_vector.py:36-48)."""

    vector = True

    def __init__(self, elem, dim=None):
        if elem.vector:
            raise NotImplementedError("nested ElementVector")
        self.elem = elem
        self.family = elem.family
        self.refdom = elem.refdom
        self.dim = elem.dim if dim is None else dim
        if self.dim != elem.dim:
            raise NotImplementedError("ElementVector with dim != element dim")
        self.maxdeg = elem.maxdeg
        self.nodal_dofs = elem.nodal_dofs * self.dim
        self.edge_dofs = elem.edge_dofs * self.dim
        self.facet_dofs = elem.facet_dofs * self.dim
        self.interior_dofs = elem.interior_dofs * self.dim
        self.nbfun_scalar = elem.nbfun_scalar
        # each scalar location once per component (element_vector.py:26-29)
        self.doflocs = np.array([elem.doflocs[i // self.dim]
                                 for i in range(self.dim * elem.doflocs.shape[0])])

    @property
    def nbfun(self):
        return self.nbfun_scalar * self.dim

    def __repr__(self):
        return "ElementVector(%r)" % self.elem
