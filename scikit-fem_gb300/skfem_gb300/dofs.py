"""Global DOF numbering (Dofs, skfem/assembly/dofs.py:264-334): nodal DOFs
numbered vertex-major (nodal_dofs per vertex), then edge DOFs (3-D), then
facet DOFs (the triangle's edges), in the same interleaving, so that the
element_dofs array -- and therefore the CSR pattern -- is the reference's."""

import numpy as np

from .mesh import TET_EDGES, TRI_FACETS

__all__ = ["Dofs"]


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
        if element.dim == 2 and element.facet_dofs > 0:
            facets, t2f = topo._build("facets", TRI_FACETS)[:2]
            fd = element.facet_dofs
            for itr in range(t2f.shape[0]):
                base = fd * t2f[itr].astype(np.int64) + offset
                for c in range(fd):
                    rows.append(base + c)
            offset += fd * facets.shape[1]
        ed_all = np.vstack(rows) if rows else np.zeros((0, t.shape[1]), dtype=np.int64)
        if ed_all.size and ed_all.max() >= np.iinfo(np.int32).max:
            raise ValueError("more DOFs than int32 indices can hold")
        self.element_dofs = np.ascontiguousarray(ed_all, dtype=np.int32)
        self.N = int(self.element_dofs.max()) + 1 if self.element_dofs.size else 0
