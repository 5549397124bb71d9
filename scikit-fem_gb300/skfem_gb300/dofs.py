"""Global DOF numbering (Dofs, skfem/assembly/dofs.py:264-334): nodal DOFs
numbered vertex-major (nodal_dofs per vertex), then edge DOFs (3-D), then
facet DOFs (the triangle's edges), in the same interleaving, so that the
element_dofs array -- and therefore the CSR pattern -- is the reference's."""

import numpy as np

from .mesh import TET_EDGES, TRI_FACETS

__all__ = ["Dofs", "DofsView"]


class Dofs:
    def __init__(self, topo, element, offset=0):
        self.topo = topo
        self.element = element
        nv = topo.nvertices
        nd = element.nodal_dofs
        t = topo.t
        # nodal: dof(c, v) = c + nd * v + offset  (Fortran reshape of arange)
        rows = []
        for itr in range(t.shape[0]):
            base = nd * t[itr].astype(np.int64) + offset
            for c in range(nd):
                rows.append(base + c)
        offset += nd * nv
        if element.dim == 3 and element.edge_dofs > 0:
            edges, t2e = topo._build("edges", TET_EDGES)[:2]
            ed = element.edge_dofs
            for itr in range(t2e.shape[0]):
                base = ed * t2e[itr].astype(np.int64) + offset
                for c in range(ed):
                    rows.append(base + c)
            offset += ed * edges.shape[1]
        self.facet_offset = offset
        if element.dim == 2 and element.facet_dofs > 0:
            facets, t2f = topo._build("facets", TRI_FACETS)[:2]
            fd = element.facet_dofs
            for itr in range(t2f.shape[0]):
                base = fd * t2f[itr].astype(np.int64) + offset
                for c in range(fd):
                    rows.append(base + c)
            offset += fd * facets.shape[1]
        self.edge_offset = nd * nv
        ed_all = np.vstack(rows) if rows else np.zeros((0, t.shape[1]), dtype=np.int64)
        if ed_all.size and ed_all.max() >= np.iinfo(np.int32).max:
            raise ValueError("more DOFs than int32 indices can hold")
        self.element_dofs = np.ascontiguousarray(ed_all, dtype=np.int32)
        self.N = int(self.element_dofs.max()) + 1 if self.element_dofs.size else 0

    # DOF subsets (dofs.py:539-662)
    def _nodal(self, vertices):
        nd = self.element.nodal_dofs
        v = np.asarray(vertices, dtype=np.int64)
        return (nd * v[None, :] + np.arange(nd)[:, None]).ravel()

    def _entity(self, ix, per, offset):
        i = np.asarray(ix, dtype=np.int64)
        return (offset + per * i[None, :] + np.arange(per)[:, None]).ravel()

    def get_facet_dofs(self, facets):
        """DOFs on the given facets: their vertices' nodal DOFs, in 3-D the
        DOFs of their edges, in 2-D their own (facet) DOFs."""
        topo, el = self.topo, self.element
        facets = np.asarray(facets, dtype=np.int64)
        fv = topo.facets[:, facets]
        parts = [self._nodal(np.unique(fv))] if el.nodal_dofs else []
        if el.dim == 3 and el.edge_dofs:
            edges = topo._build("edges", TET_EDGES)[0]
            n = max(topo.nvertices, 1)
            keys = edges[0].astype(np.int64) * n + edges[1]
            pairs = [(0, 1), (1, 2), (0, 2)]
            fk = np.concatenate([np.minimum(fv[a], fv[b]).astype(np.int64) * n +
                                 np.maximum(fv[a], fv[b]) for a, b in pairs])
            parts.append(self._entity(np.unique(np.searchsorted(keys, fk)), el.edge_dofs,
                                      self.edge_offset))
        if el.dim == 2 and el.facet_dofs:
            parts.append(self._entity(facets, el.facet_dofs, self.facet_offset))
        return DofsView(np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64))

    def get_element_dofs(self, elements):
        """DOFs of the given cells (their vertices, edges and facets)."""
        ed = self.element_dofs[:, np.asarray(elements, dtype=np.int64)]
        return DofsView(ed.ravel())


class DofsView:
    """A set of global DOF numbers (skfem/assembly/dofs.py:12-260):
    ``flatten()`` / ``all()`` / ``np.asarray`` give them sorted and unique."""

    def __init__(self, dofs):
        self._dofs = np.unique(np.asarray(dofs, dtype=np.int64)).astype(np.int32)

    def flatten(self):
        return self._dofs.copy()

    def all(self, key=None):
        if key is not None:
            raise NotImplementedError("DOF names are not distinguished (H1 elements have one)")
        return self.flatten()

    def __array__(self, dtype=None, copy=None):
        return self._dofs if dtype is None else self._dofs.astype(dtype)

    def __len__(self):
        return len(self._dofs)

    def __repr__(self):
        return "DofsView(%d DOFs)" % len(self._dofs)
