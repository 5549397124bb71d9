"""CellBasis: a mesh and an element resident on the GPU.

Mirrors skfem/assembly/basis/cell_basis.py:42-106 and abstract_basis.py:45-88
for the API a form needs (``N``, ``Nbfun``, ``nelems``, ``element_dofs``,
``X``, ``W``, ``zero_w``, ``mesh``, ``elem``).  Unlike the reference it does
not precompute basis values and gradients at every quadrature point: the
kernels evaluate geometry and bases per element from the mesh arrays kept
in HBM (``p``, ``t``, ``element_dofs``), uploaded once here.
"""

import numpy as np
import torch

from . import _native as N
from .dofs import Dofs
from .element import ElementHex1
from .field import DiscreteField
from .mesh import as_mesh
from .quadrature import get_quadrature

__all__ = ["CellBasis", "Basis", "FacetBasis"]

MAX_POINTS = 128    # quadrature points per cell of the generic kernels


class CellBasis:
    def __init__(self, mesh, elem, mapping=None, intorder=None, elements=None,
                 quadrature=None, dofs=None, disable_doflocs=False, device=None):
        mesh = as_mesh(mesh)
        if mesh.refdom != elem.refdom:
            raise ValueError("Incompatible Mesh and Element.")      # abstract_basis.py:55-56
        if mapping is not None:
            raise NotImplementedError("custom mappings are not supported; the kernels use the "
                                      "mesh's own affine / isoparametric mapping")
        self.mesh = mesh
        self.elem = elem
        self.dofs = Dofs(mesh, elem) if dofs is None else dofs
        self.Nbfun = self.dofs.element_dofs.shape[0]
        # element subset (cell_basis.py:94-99): the kernels run over the
        # selected cells only, with the global DOF numbering unchanged
        if elements is None:
            self.tind = None
            self.nelems = mesh.nelements
        else:
            self.tind = mesh.normalize_elements(elements)
            if self.tind.size and (self.tind.min() < 0 or self.tind.max() >= mesh.nelements):
                raise ValueError("element index out of range")
            self.nelems = len(self.tind)
        self.intorder = intorder if intorder is not None else 2 * elem.maxdeg
        if quadrature is not None:
            X, W = quadrature
            self.X = np.ascontiguousarray(X, dtype=np.float64)
            self.W = np.ascontiguousarray(W, dtype=np.float64)
            if self.X.ndim != 2 or self.X.shape[0] != mesh.p.shape[0] or \
                    self.W.shape != (self.X.shape[1],):
                raise ValueError("quadrature must be (X (dim, nqp), W (nqp,))")
        else:
            self.X, self.W = get_quadrature(elem.refdom, self.intorder)
        if self.X.shape[1] > MAX_POINTS:
            raise NotImplementedError("%d quadrature points per cell (limit %d)"
                                      % (self.X.shape[1], MAX_POINTS))
        # The coefficient-channel kernels integrate exactly (simplices) or
        # with the default 4x4x4 rule (Hex1); a basis whose rule gives other
        # numbers -- too low an order, a custom rule, another Hex1 rule --
        # assembles every form through the generic per-point kernels.
        if elem.refdom == "hex":
            self._fast_ok = quadrature is None and self.X.shape[1] == 64 and not elem.vector
        else:
            min_order = {1: 2, 2: 4}.get(elem.maxdeg, 0)
            self._fast_ok = quadrature is None and self.intorder >= min_order
        self.device = N.require_cuda(device)
        self._patterns = {}
        self._upload()

    # -------------------------------------------------------------- device
    def _upload(self):
        dev = self.device
        t = self.mesh.t if self.tind is None else self.mesh.t[:, self.tind]
        ed = self.element_dofs
        self.p_dev = torch.from_numpy(np.ascontiguousarray(self.mesh.p)).to(dev)
        self.t_dev = torch.from_numpy(np.ascontiguousarray(t)).to(dev)
        if ed.shape == t.shape and np.array_equal(ed, t):
            self.ed_dev = self.t_dev
        else:
            self.ed_dev = torch.from_numpy(np.ascontiguousarray(ed)).to(dev)
        dim = self.mesh.p.shape[0]
        self.c_mesh = N.FemMesh(dim, self.mesh.t.shape[0], self.mesh.p.shape[1],
                                self.nelems, self.p_dev.data_ptr(), self.t_dev.data_ptr())
        self.c_basis = N.FemBasis(N.FAMILY[self.elem.family], int(self.elem.vector),
                                  self.Nbfun, 0, self.N, self.ed_dev.data_ptr())
        self.X_dev = torch.from_numpy(np.ascontiguousarray(self.X, dtype=np.float64)).to(dev)
        self.W_dev = torch.from_numpy(np.ascontiguousarray(self.W, dtype=np.float64)).to(dev)
        # the (mesh, basis) pair the CSR pattern is built over
        self.c_mesh_pat, self.c_basis_pat = self.c_mesh, self.c_basis

    @property
    def doflocs(self):
        """Global DOF locations (abstract_basis.py:60-71): the mesh's mapping
        F of the element's reference DOF locations, cell by cell, written
        into the global numbering (a DOF shared by cells takes the value of
        the last cell and local DOF to reach it, as numpy's fancy assignment
        does).  Host arrays, computed once; every cell of the mesh, as the
        reference maps them all."""
        if getattr(self, "_doflocs", None) is None:
            p, t = self.mesh.p, self.mesh.t
            X = self.elem.doflocs                       # (nloc, dim)
            dim = p.shape[0]
            if self.elem.refdom == "hex":
                # MappingIsoparametric.F: sum over the nodes of p(t_n) phi_n(X)
                corner = ElementHex1.doflocs
                x = np.zeros((dim, X.shape[0], t.shape[1]))
                for n in range(t.shape[0]):
                    f = np.ones(X.shape[0])
                    for a in range(3):
                        f = f * (X[:, a] if corner[n, a] else 1.0 - X[:, a])
                    x = x + p[:, t[n]][:, None, :] * f[None, :, None]
            else:
                # MappingAffine.F: sum_j A_ij X_j + b_i, A = [p(t_j+1) - p(t_0)], b = p(t_0)
                A = np.stack([p[:, t[j + 1]] - p[:, t[0]] for j in range(dim)], axis=1)
                x = np.einsum('ijk,lj->ilk', A, X) + p[:, t[0]][:, None, :]
            ed = self.dofs.element_dofs
            out = np.zeros((dim, self.N))
            for itr in range(dim):
                for jtr in range(ed.shape[0]):
                    out[itr, ed[jtr]] = x[itr, jtr, :]
            self._doflocs = out
        return self._doflocs

    def complement_dofs(self, *D):
        """abstract_basis.py:119-123: the DOFs outside D (arrays of DOFs, DOF
        views, or one dict of them)."""
        if type(D[0]) is dict:
            D = tuple(D[0][key].all() for key in D[0])
        D = tuple(d if isinstance(d, np.ndarray) else d.all() for d in D)
        return np.setdiff1d(np.arange(self.N), np.concatenate(D))

    def _run_program(self, kind, prog, out, status):
        """The generic kernel of a traced program over this basis's cells."""
        fn = {"bilinear": "fem_program_local_matrices", "linear": "fem_program_local_vectors",
              "functional": "fem_program_elemental"}[kind]
        N.check(getattr(N.lib(), fn)(N.byref(self.c_mesh), N.byref(self.c_basis), N.byref(prog),
                                     N.ptr(out), N.ptr(status), N.stream_ptr()))

    def update_coordinates(self, p):
        """Replace the node coordinates (same topology) -- used by shape
        optimisation loops; patterns stay valid if the zero structure does."""
        p = torch.as_tensor(p, dtype=torch.float64, device=self.device).contiguous()
        if tuple(p.shape) != tuple(self.p_dev.shape):
            raise ValueError("coordinate array has the wrong shape")
        self.p_dev = p
        self.c_mesh.p = p.data_ptr()

    # ----------------------------------------------------------------- API
    @property
    def N(self):
        return self.dofs.N

    @property
    def element_dofs(self):
        """abstract_basis.py:110-117 (restricted to the element subset)."""
        if self.tind is None:
            return self.dofs.element_dofs
        return self.dofs.element_dofs[:, self.tind]

    def zero_w(self, dtype=None):
        """abstract_basis.py:378-382."""
        return np.zeros((self.nelems, 0 if self.W is None else len(self.W)), dtype=dtype)

    def zeros(self, dtype=None):
        return np.zeros(self.N, dtype=dtype)

    def quadrature(self):
        return self.X, self.W

    def get_dofs(self, facets=None, elements=None):
        """Global DOF numbers on facets (default: the boundary) or of cells
        (abstract_basis.py:125-260): a DofsView, ``.flatten()`` for the
        sorted array condense / enforce take."""
        if elements is not None:
            if facets is not None:
                raise ValueError("Give only facets or only elements")
            return self.dofs.get_element_dofs(self.mesh.normalize_elements(elements))
        return self.dofs.get_facet_dofs(self.mesh.normalize_facets(facets))

    def interpolate_torch(self, w):
        """Device interpolation of the DOF vector w: (nquant, nelems, nqp)
        float64, quantity-major -- scalar bases value then the dim
        derivatives; vector bases the components then grad[c][k] at
        dim + c*dim + k (abstract_basis.py:271-322 arithmetic)."""
        w = torch.as_tensor(w, dtype=torch.float64).to(self.device).contiguous()
        if w.dim() != 1 or w.shape[0] != self.N:
            raise ValueError("Input array has wrong size.")       # abstract_basis.py:284-285
        dim = self.mesh.p.shape[0]
        nquant = dim + dim * dim if self.elem.vector else 1 + dim
        nq = self.X.shape[1]
        out = torch.empty((nquant, self.nelems, nq), dtype=torch.float64, device=self.device)
        N.check(N.lib().fem_interpolate(N.byref(self.c_mesh), N.byref(self.c_basis), nq,
                                        N.ptr(self.X_dev), N.ptr(w), N.ptr(out),
                                        N.stream_ptr()))
        return out

    def interpolate(self, w):
        """Basis.interpolate (abstract_basis.py:271-322): a DiscreteField of
        the values at the quadrature points, with ``grad``; computed on the
        device (and kept there for forms that receive it)."""
        if isinstance(w, np.ndarray) and (w.ndim != 1 or w.shape[0] != self.N):
            raise ValueError("Input array has wrong size.")
        dev = self.interpolate_torch(w)
        host = dev.cpu().numpy()
        dim = self.mesh.p.shape[0]
        if self.elem.vector:
            value = host[:dim]
            grad = host[dim:].reshape((dim, dim) + host.shape[1:])
        else:
            value, grad = host[0], host[1:]
        f = DiscreteField(value, grad)
        f._dev = (dev, self)
        return f

    def default_parameters(self):
        return {}

    def __repr__(self):
        return "CellBasis(%r, %r) on %s: %d DOFs" % (self.mesh, self.elem, self.device, self.N)


BOUNDARY_REFDOM = {"tri": "line", "tet": "tri", "hex": "quad"}


class FacetBasis(CellBasis):
    """FacetBasis (skfem/assembly/basis/facet_basis.py:21-110) on affine
    simplex meshes: integrates over a set of facets -- by default the
    boundary -- with the basis of the cell on ``side`` (f2t[side]) and the
    outward normal of the cell f2t[0].  Forms see ``w.x``, ``w.h`` and
    ``w.n``; every form runs on the generic per-point kernels, over facets
    instead of cells."""

    def __init__(self, mesh, elem, mapping=None, intorder=None, quadrature=None, facets=None,
                 dofs=None, side=0, disable_doflocs=False, device=None):
        mesh = as_mesh(mesh)
        if mesh.refdom != elem.refdom:
            raise ValueError("Incompatible Mesh and Element.")
        if mapping is not None:
            raise NotImplementedError("custom mappings are not supported")
        if mesh.refdom not in BOUNDARY_REFDOM:
            raise NotImplementedError("FacetBasis on %s meshes is not implemented"
                                      % type(mesh).__name__)
        self.mesh, self.elem = mesh, elem
        self.dofs = Dofs(mesh, elem) if dofs is None else dofs
        self.Nbfun = self.dofs.element_dofs.shape[0]
        self.find = np.asarray(mesh.normalize_facets(facets), dtype=np.int32)
        f2t = mesh.f2t
        self.tind = f2t[side, self.find]
        self.tind_normals = f2t[0, self.find]
        if np.any(self.tind < 0):
            raise ValueError("side=%d has no cell on %d of the facets (boundary facets have "
                             "one side)" % (side, int(np.sum(self.tind < 0))))
        self.nelems = len(self.find)
        self.intorder = intorder if intorder is not None else 2 * elem.maxdeg
        brefdom = BOUNDARY_REFDOM[mesh.refdom]
        if quadrature is not None:
            self.X = np.ascontiguousarray(quadrature[0], dtype=np.float64)
            self.W = np.ascontiguousarray(quadrature[1], dtype=np.float64)
        else:
            self.X, self.W = get_quadrature(brefdom, self.intorder)
        if self.X.shape[0] != mesh.p.shape[0] - 1 or self.X.shape[1] > MAX_POINTS:
            raise ValueError("facet quadrature must be (dim-1, nqp) with nqp <= %d" % MAX_POINTS)
        self._fast_ok = False
        self.device = N.require_cuda(device)
        self._patterns = {}
        self._upload_facets()

    def _upload_facets(self):
        dev = self.device
        m = self.mesh
        dim = m.p.shape[0]
        t2f = m.t2f
        lf = np.argmax(t2f[:, self.tind_normals] == self.find[None, :], axis=0).astype(np.int32)

        def up(a, dtype=np.int32):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev)

        self.p_dev = up(m.p, np.float64)
        self.t_dev = up(m.t)
        self.ed_full_dev = up(self.dofs.element_dofs)
        self.fv_dev = up(m.facets[:, self.find])
        self.tind_dev = up(self.tind)
        self.tindn_dev = up(self.tind_normals)
        self.lf_dev = up(lf)
        self.ed_dev = up(self.element_dofs)
        fam = N.FAMILY[self.elem.family]
        self.c_mesh = N.FemMesh(dim, m.t.shape[0], m.p.shape[1], m.t.shape[1],
                                self.p_dev.data_ptr(), self.t_dev.data_ptr())
        self.c_basis = N.FemBasis(fam, int(self.elem.vector), self.Nbfun, 0, self.N,
                                  self.ed_full_dev.data_ptr())
        self.c_facets = N.FemFacets(self.nelems, self.fv_dev.data_ptr(), self.tind_dev.data_ptr(),
                                    self.tindn_dev.data_ptr(), self.lf_dev.data_ptr(), None)
        # the pattern is built over the facets with their cells' DOFs
        self.c_mesh_pat = N.FemMesh(dim, m.t.shape[0], m.p.shape[1], self.nelems,
                                    self.p_dev.data_ptr(), self.t_dev.data_ptr())
        self.c_basis_pat = N.FemBasis(fam, int(self.elem.vector), self.Nbfun, 0, self.N,
                                      self.ed_dev.data_ptr())
        self.X_dev = up(self.X, np.float64)
        self.W_dev = up(self.W, np.float64)
        if m.refdom == "hex":
            # isoparametric facets: the point geometry (Newton-iterated
            # reference points, normals) once, as the reference precomputes it
            nq = self.X.shape[1]
            self.geo_dev = torch.empty(max(1, self.nelems * nq * 20), dtype=torch.float64,
                                       device=dev)
            status = torch.zeros(1, dtype=torch.int32, device=dev)
            N.check(N.lib().fem_facet_geometry(N.byref(self.c_mesh), N.byref(self.c_basis),
                                               N.byref(self.c_facets), nq, N.ptr(self.X_dev),
                                               N.ptr(self.geo_dev), N.ptr(status),
                                               N.stream_ptr()))
            st = int(status.item())
            if st & (1 << N.FEM_ERR_ZERO_JACOBIAN):
                raise N.ZeroJacobianError("Zero Jacobian determinant")
            if st & (1 << N.FEM_ERR_NEWTON):
                raise Exception("Newton iteration didn't converge up to TOL=1e-12")
            if st:
                raise ValueError("invalid facet arrays")
            self.c_facets.geo = self.geo_dev.data_ptr()

    def update_coordinates(self, p):
        raise NotImplementedError("FacetBasis.update_coordinates is not supported")

    @property
    def element_dofs(self):
        """The DOFs of each facet's cell (abstract_basis.py:110-117 with tind)."""
        return self.dofs.element_dofs[:, self.tind]

    def _run_program(self, kind, prog, out, status):
        fn = {"bilinear": "fem_facet_program_local_matrices",
              "linear": "fem_facet_program_local_vectors",
              "functional": "fem_facet_program_elemental"}[kind]
        N.check(getattr(N.lib(), fn)(N.byref(self.c_mesh), N.byref(self.c_basis),
                                     N.byref(self.c_facets), N.byref(prog), N.ptr(out),
                                     N.ptr(status), N.stream_ptr()))

    def interpolate_torch(self, w):
        w = torch.as_tensor(w, dtype=torch.float64).to(self.device).contiguous()
        if w.dim() != 1 or w.shape[0] != self.N:
            raise ValueError("Input array has wrong size.")
        dim = self.mesh.p.shape[0]
        nquant = dim + dim * dim if self.elem.vector else 1 + dim
        nq = self.X.shape[1]
        out = torch.empty((nquant, self.nelems, nq), dtype=torch.float64, device=self.device)
        N.check(N.lib().fem_facet_interpolate(N.byref(self.c_mesh), N.byref(self.c_basis),
                                              N.byref(self.c_facets), nq, N.ptr(self.X_dev),
                                              N.ptr(w), N.ptr(out), N.stream_ptr()))
        return out

    def __repr__(self):
        return "FacetBasis(%r, %r) on %s: %d facets, %d DOFs" % (
            self.mesh, self.elem, self.device, self.nelems, self.N)


Basis = CellBasis
