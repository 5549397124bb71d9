"""Meshes: the reference's data layout (p (dim, nverts) float64, t (nloc,
nelems) int32) and the tensor-mesh constructors the workloads use.

Node and cell numbering must match scikit-fem's for the CSR pattern to be
bit-identical, so the constructors follow (in our own code):
  MeshTri1.init_tensor   skfem/mesh/mesh_tri_1.py:31-80 (+ sort_t, :28)
  MeshTet1.init_tensor   skfem/mesh/mesh_tet_1.py:327-393
  MeshHex1.init_tensor   skfem/mesh/mesh_hex_1.py:98-155
  Mesh.__post_init__     skfem/mesh/mesh.py:544-591 (sort_t, dtypes)
  Mesh.build_entities    skfem/mesh/mesh.py:1065-1082 (edges / facets)
"""

import numpy as np

__all__ = ["Mesh", "MeshTri", "MeshTri1", "MeshTet", "MeshTet1", "MeshHex", "MeshHex1",
           "as_mesh"]

# local vertices of the entities, in the reference's order
TRI_FACETS = np.array([[0, 1], [1, 2], [0, 2]])                           # refdom.py:60-62
TET_EDGES = np.array([[0, 1], [1, 2], [0, 2], [0, 3], [1, 3], [2, 3]])    # refdom.py:101-106
TET_FACETS = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]])       # refdom.py:96-99
# outward normals of the reference cell's facets (refdom.py:60-62, 107-110)
TRI_NORMALS = np.array([[0., -1.], [1., 1.], [-1., 0.]])
TET_NORMALS = np.array([[0., 0., -1.], [0., -1., 0.], [-1., 0., 0.], [1., 1., 1.]])
HEX_FACETS = np.array([[0, 1, 4, 2], [0, 2, 6, 3], [0, 3, 5, 1], [2, 4, 7, 6], [1, 5, 7, 4],
                       [3, 6, 7, 5]])                                     # refdom.py:188-193
HEX_NORMALS = np.array([[1., 0., 0.], [0., 0., 1.], [0., 1., 0.], [0., -1., 0.], [0., 0., -1.],
                        [-1., 0., 0.]])                                   # refdom.py:182-187


class Mesh:
    """Base class: ``p`` (dim, nverts) float64 and ``t`` (nloc, nelems) int32."""

    kind = ""
    refdom = ""
    affine = False
    sort_t = False
    nloc = 0

    def __init__(self, doflocs, t, **kwargs):
        p = np.ascontiguousarray(np.asarray(doflocs, dtype=np.float64))
        t = np.asarray(t)
        if self.sort_t:
            t = np.sort(t, axis=0)
        t = np.ascontiguousarray(t, dtype=np.int32)
        if p.ndim != 2 or t.ndim != 2 or t.shape[0] != self.nloc:
            raise ValueError("Mesh expects p (dim, nverts) and t (%d, nelems)" % self.nloc)
        self.doflocs = p
        self.t = t
        self._entities = {}

    @property
    def p(self):
        return self.doflocs

    @property
    def nelements(self):
        return self.t.shape[1]

    @property
    def nvertices(self):
        return int(self.t.max()) + 1 if self.t.size else 0

    def dim(self):
        return self.p.shape[0]

    def elements_satisfying(self, test):
        """Cells whose midpoints satisfy ``test`` (mesh.py:481-493)."""
        midp = self.p[:, self.t].mean(axis=1)
        return np.nonzero(test(midp))[0].astype(np.int32)

    def normalize_elements(self, elements):
        """Element indices from the reference's selectors (mesh.py:1331-1369):
        True, an index, an index array (a boolean mask selects its True
        cells), a callable on cell midpoints, or a list of those."""
        if isinstance(elements, bool) and elements:
            return np.arange(self.nelements, dtype=np.int32)
        if isinstance(elements, (int, np.integer)):
            return np.array([elements], dtype=np.int32)
        if isinstance(elements, np.ndarray):
            if elements.dtype == bool:
                return np.nonzero(elements)[0].astype(np.int32)
            return elements.astype(np.int32)
        if callable(elements):
            return self.elements_satisfying(elements)
        if isinstance(elements, (tuple, list, set)):
            return np.unique(np.concatenate([self.normalize_elements(e) for e in elements]))
        if isinstance(elements, str):
            raise ValueError("Subdomain '{}' not found.".format(elements))
        raise NotImplementedError

    # ------------------------------------------------------------ entities
    def _build(self, name, local, sort=True):
        """Mesh.build_entities (mesh.py:1065-1082): every cell's local vertex
        tuples, made unique in the lexicographic order of the sorted tuples
        and stored sorted (sort=True) or in the vertex order of their first
        occurrence (sort=False, MeshHex1 facets, mesh_hex_1.py:49-55); plus
        the inverse map (cell -> entity) and, as Mesh.build_inverse
        (mesh.py:1084-1100) does, the first and last cell that contain each
        entity (-1 when only one does)."""
        if name not in self._entities:
            t = self.t
            ne = t.shape[1]
            raw = np.hstack([t[list(ix)] for ix in local])
            cols = np.sort(raw, axis=0)
            M = cols.shape[1]
            order = np.lexsort(cols[::-1])          # stable: positions ascend in a group
            sc = cols[:, order]
            new = np.ones(M, dtype=bool)
            if M > 1:
                new[1:] = np.any(sc[:, 1:] != sc[:, :-1], axis=0)
            ids = np.cumsum(new) - 1
            if sort:
                ent = np.ascontiguousarray(sc[:, new]).astype(np.int32)
            else:
                ent = np.ascontiguousarray(raw[:, order[new]]).astype(np.int32)
            inv = np.empty(M, dtype=np.int64)
            inv[order] = ids
            starts = np.nonzero(new)[0]
            ends = np.r_[starts[1:], M] - 1
            cell = np.tile(np.arange(ne, dtype=np.int32), len(local))
            inverse = np.vstack((cell[order[starts]], cell[order[ends]])).astype(np.int32)
            inverse[1, inverse[0] == inverse[1]] = -1
            self._entities[name] = (ent, inv.reshape(len(local), ne).astype(np.int32), inverse)
        return self._entities[name]

    # facets (mesh.py:98-113, 197-199, 426-456, 1291-1329)
    facet_tuples = None
    facet_sort = True
    normals_ref = None

    @property
    def facets(self):
        if self.facet_tuples is None:
            raise NotImplementedError("facets of %s are not supported" % type(self).__name__)
        return self._build("facets", self.facet_tuples, self.facet_sort)[0]

    @property
    def t2f(self):
        return self._build("facets", self.facet_tuples, self.facet_sort)[1]

    @property
    def f2t(self):
        return self._build("facets", self.facet_tuples, self.facet_sort)[2]

    def boundary_facets(self):
        return np.nonzero(self.f2t[1] == -1)[0].astype(np.int32)

    def facets_satisfying(self, test, boundaries_only=False):
        midp = self.p[:, self.facets].mean(axis=1)
        facets = np.nonzero(test(midp))[0].astype(np.int32)
        if boundaries_only:
            facets = np.intersect1d(facets, self.boundary_facets())
        return facets

    def normalize_facets(self, facets):
        if isinstance(facets, (int, np.integer)):
            return np.array([facets])
        if isinstance(facets, np.ndarray):
            return facets
        if facets is None:
            return self.boundary_facets()
        if isinstance(facets, (tuple, list, set)):
            return np.unique(np.concatenate([self.normalize_facets(f) for f in facets]))
        if callable(facets):
            return self.facets_satisfying(facets)
        if isinstance(facets, str):
            raise ValueError("Boundary '{}' not found.".format(facets))
        raise NotImplementedError

    def __repr__(self):
        return "%s(%d vertices, %d elements)" % (type(self).__name__, self.p.shape[1],
                                                 self.nelements)


class MeshTri1(Mesh):
    """Triangular mesh (MeshTri1, mesh_tri_1.py:13-28): affine, sort_t."""

    kind = refdom = "tri"
    affine = True
    sort_t = True
    nloc = 3

    def __init__(self, doflocs=None, t=None, **kwargs):
        if doflocs is None:
            doflocs = np.array([[0., 0.], [1., 0.], [0., 1.], [1., 1.]]).T
            t = np.array([[0, 1, 2], [1, 3, 2]]).T
        super().__init__(doflocs, t, **kwargs)

    facet_tuples = TRI_FACETS
    normals_ref = TRI_NORMALS

    @classmethod
    def init_tensor(cls, x, y):
        x = np.sort(np.asarray(x, dtype=np.float64))
        y = np.sort(np.asarray(y, dtype=np.float64))
        nx, ny = len(x), len(y)
        # vertex (ix, iy) -> iy + ny*ix
        p = np.vstack((np.repeat(x, ny), np.tile(y, nx)))
        cx = np.repeat(np.arange(nx - 1), ny - 1)
        cy = np.tile(np.arange(ny - 1), nx - 1)
        v00 = cy + ny * cx
        v01 = v00 + 1
        v10 = v00 + ny
        v11 = v10 + 1
        t = np.hstack((np.vstack((v00, v01, v11)), np.vstack((v00, v10, v11))))
        return cls(p, t)


class MeshTet1(Mesh):
    """Tetrahedral mesh (MeshTet1, mesh_tet_1.py:13-44): affine."""

    kind = refdom = "tet"
    affine = True
    nloc = 4

    def __init__(self, doflocs=None, t=None, **kwargs):
        if doflocs is None:
            doflocs = np.array([[0., 0., 0.], [0., 0., 1.], [0., 1., 0.], [1., 0., 0.],
                                [0., 1., 1.], [1., 0., 1.], [1., 1., 0.], [1., 1., 1.]]).T
            t = np.array([[0, 1, 2, 3], [3, 5, 1, 7], [2, 3, 6, 7], [2, 3, 1, 7],
                          [1, 2, 4, 7]]).T
        super().__init__(doflocs, t, **kwargs)

    facet_tuples = TET_FACETS
    normals_ref = TET_NORMALS

    @property
    def edges(self):
        return self._build("edges", TET_EDGES)[0]

    @property
    def t2e(self):
        return self._build("edges", TET_EDGES)[1]

    @classmethod
    def init_tensor(cls, x, y, z):
        p, c = _box_cells(x, y, z)
        t = np.hstack([c[[0, 1, 5, 7]], c[[0, 1, 4, 7]], c[[0, 2, 4, 7]],
                       c[[0, 3, 5, 7]], c[[0, 2, 6, 7]], c[[0, 3, 6, 7]]])
        return cls(p, t)


class MeshHex1(Mesh):
    """Trilinear hexahedral mesh (MeshHex1, mesh_hex_1.py:13-47): isoparametric."""

    kind = refdom = "hex"
    affine = False
    nloc = 8
    facet_tuples = HEX_FACETS
    facet_sort = False
    normals_ref = HEX_NORMALS

    def __init__(self, doflocs=None, t=None, **kwargs):
        if doflocs is None:
            doflocs = np.array([[0., 0., 0.], [0., 0., 1.], [0., 1., 0.], [1., 0., 0.],
                                [0., 1., 1.], [1., 0., 1.], [1., 1., 0.], [1., 1., 1.]]).T
            t = np.array([[0, 1, 2, 3, 4, 5, 6, 7]]).T
        super().__init__(doflocs, t, **kwargs)

    @classmethod
    def init_tensor(cls, x, y, z):
        p, c = _box_cells(x, y, z)
        return cls(p, c)


def _box_cells(x, y, z):
    """Vertices of a tensor grid and the 8 corners of every cell in the
    reference's numbering: vertex (ix, iy, iz) -> iy + ny*ix + ny*nx*iz,
    cell (cx, cy, cz) -> cy + (ny-1)*cx + (ny-1)*(nx-1)*cz."""
    x = np.sort(np.asarray(x, dtype=np.float64))
    y = np.sort(np.asarray(y, dtype=np.float64))
    z = np.sort(np.asarray(z, dtype=np.float64))
    nx, ny, nz = len(x), len(y), len(z)
    iz, ix, iy = np.meshgrid(np.arange(nz), np.arange(nx), np.arange(ny), indexing="ij")
    p = np.vstack((x[ix.ravel()], y[iy.ravel()], z[iz.ravel()]))
    cz, cx, cy = np.meshgrid(np.arange(nz - 1), np.arange(nx - 1), np.arange(ny - 1),
                             indexing="ij")
    cx, cy, cz = cx.ravel(), cy.ravel(), cz.ravel()

    def n(a, b, c):
        return b + ny * a + ny * nx * c

    corners = np.array([
        n(cx, cy, cz), n(cx, cy + 1, cz), n(cx + 1, cy, cz), n(cx, cy, cz + 1),
        n(cx + 1, cy + 1, cz), n(cx, cy + 1, cz + 1), n(cx + 1, cy, cz + 1),
        n(cx + 1, cy + 1, cz + 1),
    ])
    return p, corners


MeshTri = MeshTri1
MeshTet = MeshTet1
MeshHex = MeshHex1


def as_mesh(m):
    """Accept our meshes or any object with ``p``/``t`` arrays (e.g. a
    scikit-fem mesh); the cell type is read from ``t``'s rows and the
    dimension."""
    if isinstance(m, Mesh):
        return m
    p, t = np.asarray(m.p), np.asarray(m.t)
    kinds = {(2, 3): MeshTri1, (3, 4): MeshTet1, (3, 8): MeshHex1}
    cls = kinds.get((p.shape[0], t.shape[0]))
    if cls is None:
        raise NotImplementedError("mesh with dim %d and %d vertices per cell is not supported"
                                  % (p.shape[0], t.shape[0]))
    out = cls.__new__(cls)
    out.doflocs = np.ascontiguousarray(p, dtype=np.float64)
    out.t = np.ascontiguousarray(t, dtype=np.int32)  # already sorted by its own class
    out._entities = {}
    return out
