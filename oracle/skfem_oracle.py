"""Numpy restatement of scikit-fem 12.0.1 cell assembly (the oracle).

Test infrastructure only: imported by ``tests/``, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline leg, never by the product package.

Every block cites the reference (paths relative to the scikit-fem project).
The restatement keeps the reference's structure on purpose -- eager
per-basis-function fields, the Nbfun x Nbfun Python loop with one vectorised
numpy evaluation per local entry, and scipy's ``coo_matrix`` ->
``eliminate_zeros`` -> ``tocsr`` -- so that its results and its cost profile
both stand in for the reference's on machines where scikit-fem is absent.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
from scipy.sparse import coo_matrix

__all__ = [
    "OMesh", "mesh_tri_tensor", "mesh_tet_tensor", "mesh_hex_tensor",
    "mesh_tri_default", "mesh_unit_square_jittered",
    "TriP1", "TriP2", "TetP1", "TetP2", "Hex1", "Vector", "OElement",
    "build_entities", "element_dofs", "quadrature", "OBasis", "DField",
    "grad", "dot", "ddot", "sym_grad", "trace", "eye", "transpose",
    "laplace", "mass", "unit_load", "linear_elasticity", "k_laplace_mass",
    "theta_laplace", "k_laplace", "f_load",
    "bilinear_local", "bilinear_assemble", "linear_local", "linear_assemble",
    "theta_gradient", "fd_x_gradient",
]


# --------------------------------------------------------------------------
# Meshes: p (dim, nverts) float64, t (nloc, nelems) int32
# --------------------------------------------------------------------------

@dataclass
class OMesh:
    p: np.ndarray
    t: np.ndarray
    kind: str  # "tri" | "tet" | "hex"

    @property
    def affine(self) -> bool:
        # mesh_tri_1.py:27, mesh_tet_1.py:44 (affine=True); MeshHex1 keeps
        # the Mesh default affine=False (mesh.py:32) -> isoparametric.
        return self.kind in ("tri", "tet")

    @property
    def nelements(self) -> int:
        return self.t.shape[1]

    @property
    def nvertices(self) -> int:
        # mesh.py:72  (np.max(t) + 1)
        return int(np.max(self.t)) + 1


def _finish(p, t, kind, sort_t):
    # mesh.py:555-559: optional per-column sort, then float64 / int32.
    t = np.asarray(t)
    if sort_t:
        t = np.sort(t, axis=0)
    return OMesh(np.ascontiguousarray(p, dtype=np.float64),
                 np.ascontiguousarray(t, dtype=np.int32), kind)


def mesh_tri_tensor(x, y) -> OMesh:
    """MeshTri1.init_tensor (mesh_tri_1.py:31-80); sort_t=True (:28).

    Node (ix, iy) gets id ``iy + npy*ix`` (meshgrid flattened in Fortran
    order); cell (cx, cy) has index ``cy + (npy-1)*cx`` and is cut into
    [(cx,cy),(cx,cy+1),(cx+1,cy+1)] and, offset by nt,
    [(cx,cy),(cx+1,cy),(cx+1,cy+1)].
    """
    x = np.sort(np.asarray(x, dtype=np.float64))
    y = np.sort(np.asarray(y, dtype=np.float64))
    npx, npy = len(x), len(y)
    IX, IY = np.meshgrid(np.arange(npx), np.arange(npy), indexing="ij")
    p = np.vstack((x[IX.ravel()], y[IY.ravel()]))
    cx, cy = np.meshgrid(np.arange(npx - 1), np.arange(npy - 1), indexing="ij")
    cx, cy = cx.ravel(), cy.ravel()

    def n(ix, iy):
        return iy + npy * ix

    t1 = np.array([n(cx, cy), n(cx, cy + 1), n(cx + 1, cy + 1)])
    t2 = np.array([n(cx, cy), n(cx + 1, cy), n(cx + 1, cy + 1)])
    return _finish(p, np.hstack((t1, t2)), "tri", sort_t=True)


def _box_corners(x, y, z):
    # Shared by mesh_tet_1.py:327-380 and mesh_hex_1.py:98-154: node
    # (ix,iy,iz) -> iy + npy*ix + npy*npx*iz; cell (cx,cy,cz) ->
    # cy + (npy-1)*cx + (npy-1)*(npx-1)*cz; eight corners in the order
    # t[0..7] of those functions.
    x = np.sort(np.asarray(x, dtype=np.float64))
    y = np.sort(np.asarray(y, dtype=np.float64))
    z = np.sort(np.asarray(z, dtype=np.float64))
    npx, npy, npz = len(x), len(y), len(z)
    IX, IY, IZ = np.meshgrid(np.arange(npx), np.arange(npy), np.arange(npz),
                             indexing="ij")
    # node id = iy + npy*ix + npy*npx*iz -> iterate iz slowest, ix, iy fastest
    IZf = np.transpose(IZ, (2, 0, 1)).ravel()
    IXf = np.transpose(IX, (2, 0, 1)).ravel()
    IYf = np.transpose(IY, (2, 0, 1)).ravel()
    p = np.vstack((x[IXf], y[IYf], z[IZf]))
    CX, CY, CZ = np.meshgrid(np.arange(npx - 1), np.arange(npy - 1),
                             np.arange(npz - 1), indexing="ij")
    cx = np.transpose(CX, (2, 0, 1)).ravel()
    cy = np.transpose(CY, (2, 0, 1)).ravel()
    cz = np.transpose(CZ, (2, 0, 1)).ravel()

    def n(ix, iy, iz):
        return iy + npy * ix + npy * npx * iz

    t = np.array([
        n(cx, cy, cz), n(cx, cy + 1, cz), n(cx + 1, cy, cz),
        n(cx, cy, cz + 1), n(cx + 1, cy + 1, cz), n(cx, cy + 1, cz + 1),
        n(cx + 1, cy, cz + 1), n(cx + 1, cy + 1, cz + 1),
    ])
    return p, t


def mesh_tet_tensor(x, y, z) -> OMesh:
    """MeshTet1.init_tensor (mesh_tet_1.py:327-393): six tets per cell with
    corner tuples (0,1,5,7) (0,1,4,7) (0,2,4,7) (0,3,5,7) (0,2,6,7)
    (0,3,6,7), stacked block by block (:386-392).  No per-column sort."""
    p, t = _box_corners(x, y, z)
    T = np.hstack([t[[0, 1, 5, 7]], t[[0, 1, 4, 7]], t[[0, 2, 4, 7]],
                   t[[0, 3, 5, 7]], t[[0, 2, 6, 7]], t[[0, 3, 6, 7]]])
    return _finish(p, T, "tet", sort_t=False)


def mesh_hex_tensor(x, y, z) -> OMesh:
    """MeshHex1.init_tensor (mesh_hex_1.py:98-155)."""
    p, t = _box_corners(x, y, z)
    return _finish(p, t, "hex", sort_t=False)


def mesh_tri_default() -> OMesh:
    """MeshTri1 default (mesh_tri_1.py:16-25): unit square, two triangles."""
    p = np.array([[0., 0.], [1., 0.], [0., 1.], [1., 1.]]).T
    t = np.array([[0, 1, 2], [1, 3, 2]]).T
    return _finish(p, t, "tri", sort_t=True)


def mesh_unit_square_jittered(n: int, rng: np.random.Generator,
                              amp: float = 0.2) -> OMesh:
    """Tensor triangle mesh of the unit square, interior nodes jittered by
    U(-amp*h, amp*h) per coordinate (h = 1/n)."""
    m = mesh_tri_tensor(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1))
    p = m.p.copy()
    h = 1.0 / n
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += rng.uniform(-amp * h, amp * h, size=(2, int(inner.sum())))
    return OMesh(p, m.t, "tri")


# --------------------------------------------------------------------------
# Topological entities (mesh.py:1065-1082)
# --------------------------------------------------------------------------

REF_TRI_FACETS = [[0, 1], [1, 2], [0, 2]]                       # refdom.py:60-62
REF_TET_EDGES = [[0, 1], [1, 2], [0, 2], [0, 3], [1, 3], [2, 3]]  # refdom.py:101-106


def build_entities(t, indices):
    """Mesh.build_entities (mesh.py:1065-1082): gather the local vertex tuples,
    sort each tuple, unique over columns (lexicographic), return the sorted
    entities and the element-to-entity map (len(indices), nelems)."""
    indexing = np.hstack(tuple(t[ix] for ix in indices))
    s = np.sort(indexing, axis=0)
    ent, inv = np.unique(s, axis=1, return_inverse=True)
    return ent, inv.reshape(len(indices), t.shape[1])


# --------------------------------------------------------------------------
# Reference elements: lbasis(X, i) -> (phi, dphi)
# --------------------------------------------------------------------------

class OElement:
    name = ""
    refdom = ""
    maxdeg = 1
    nodal_dofs = 1
    edge_dofs = 0
    facet_dofs = 0
    interior_dofs = 0
    dim = 2
    nbfun = 3
    vector = False

    def lbasis(self, X, i):
        raise NotImplementedError


class TriP1(OElement):
    """element_tri_p1.py:18-33."""
    name, refdom, maxdeg, dim, nbfun = "TriP1", "tri", 1, 2, 3

    def lbasis(self, X, i):
        x, y = X
        if i == 0:
            return 1. - x - y, np.array([-1. + 0. * x, -1. + 0. * x])
        if i == 1:
            return x, np.array([1. + 0. * x, 0. * x])
        if i == 2:
            return y, np.array([0. * x, 1. + 0. * x])
        raise ValueError(i)


class TriP2(OElement):
    """element_tri_p2.py:22-48 (DOFs: 3 vertices, then facets 0-1, 1-2, 0-2)."""
    name, refdom, maxdeg, dim, nbfun = "TriP2", "tri", 2, 2, 6
    facet_dofs = 1

    def lbasis(self, X, i):
        x, y = X
        if i == 0:
            return (1. - 3. * x - 3. * y + 2. * x ** 2 + 4. * x * y + 2. * y ** 2,
                    np.array([-3 + 4. * x + 4. * y, -3 + 4. * x + 4. * y]))
        if i == 1:
            return 2. * x ** 2 - x, np.array([4. * x - 1, 0. * x])
        if i == 2:
            return 2. * y ** 2 - y, np.array([0. * x, 4. * y - 1])
        if i == 3:
            return (4. * x - 4. * x ** 2 - 4. * x * y,
                    np.array([4 - 8. * x - 4. * y, -4. * x]))
        if i == 4:
            return 4. * x * y, np.array([4. * y, 4. * x])
        if i == 5:
            return (4. * y - 4. * x * y - 4. * y ** 2,
                    np.array([-4. * y, 4 - 4. * x - 8. * y]))
        raise ValueError(i)


class TetP1(OElement):
    """element_tet_p1.py:19-45."""
    name, refdom, maxdeg, dim, nbfun = "TetP1", "tet", 1, 3, 4

    def lbasis(self, X, i):
        x, y, z = X
        o, zz = 1. + 0. * x, 0. * x
        if i == 0:
            return 1. - x - y - z, np.array([-o, -o, -o])
        if i == 1:
            return x, np.array([o, zz, zz])
        if i == 2:
            return y, np.array([zz, o, zz])
        if i == 3:
            return z, np.array([zz, zz, o])
        raise ValueError(i)


class TetP2(OElement):
    """element_tet_p2.py:26-103 (DOFs: 4 vertices, then edges
    01, 12, 02, 03, 13, 23 as in refdom.py:101-106)."""
    name, refdom, maxdeg, dim, nbfun = "TetP2", "tet", 2, 3, 10
    edge_dofs = 1

    def lbasis(self, X, i):
        x, y, z = X
        zz = 0. * x
        if i == 0:
            g = -3. + 4. * x + 4. * y + 4. * z
            return (1. - 3. * x + 2. * x ** 2 - 3. * y + 4. * x * y + 2. * y ** 2
                    - 3. * z + 4. * x * z + 4. * y * z + 2. * z ** 2,
                    np.array([g, g, g]))
        if i == 1:
            return -1. * x + 2. * x ** 2, np.array([-1 + 4 * x, zz, zz])
        if i == 2:
            return -1. * y + 2. * y ** 2, np.array([zz, -1. + 4. * y, zz])
        if i == 3:
            return -1. * z + 2. * z ** 2, np.array([zz, zz, -1. + 4. * z])
        if i == 4:
            return (4. * x - 4. * x ** 2 - 4. * x * y - 4 * x * z,
                    np.array([4. - 8. * x - 4. * y - 4. * z, -4. * x, -4. * x]))
        if i == 5:
            return 4. * x * y, np.array([4. * y, 4. * x, zz])
        if i == 6:
            return (4. * y - 4. * x * y - 4. * y ** 2 - 4. * y * z,
                    np.array([-4. * y, 4. - 4. * x - 8. * y - 4. * z, -4. * y]))
        if i == 7:
            return (4. * z - 4. * x * z - 4. * y * z - 4. * z ** 2,
                    np.array([-4. * z, -4. * z, 4. - 4. * x - 4. * y - 8. * z]))
        if i == 8:
            return 4. * x * z, np.array([4. * z, zz, 4 * x])
        if i == 9:
            return 4. * y * z, np.array([zz, 4 * z, 4 * y])
        raise ValueError(i)


class Hex1(OElement):
    """element_hex1.py:23-69 (trilinear; node k sits at the reference vertex
    refdom.py:173-180, i.e. node 0 at (1,1,1) and node 7 at (0,0,0)).
    maxdeg=3 (:11) gives the default intorder 6."""
    name, refdom, maxdeg, dim, nbfun = "Hex1", "hex", 3, 3, 8
    # corner coordinates of node k in the reference cube
    corners = np.array([[1., 1., 1.], [1., 1., 0.], [1., 0., 1.], [0., 1., 1.],
                        [1., 0., 0.], [0., 1., 0.], [0., 0., 1.], [0., 0., 0.]])

    def lbasis(self, X, i):
        x, y, z = X
        cx, cy, cz = self.corners[i]
        # factor s(t) = t if the corner coordinate is 1 else (1 - t)
        fx = x if cx else 1 - x
        fy = y if cy else 1 - y
        fz = z if cz else 1 - z
        sx = 1. if cx else -1.
        sy = 1. if cy else -1.
        sz = 1. if cz else -1.
        return fx * fy * fz, np.array([sx * fy * fz, sy * fx * fz, sz * fx * fy])


class Vector(OElement):
    """ElementVector (element_vector.py:9-48): component c of scalar function
    k is vector function i = dim*k + c."""
    vector = True

    def __init__(self, elem: OElement):
        self.elem = elem
        self.name = "Vector" + elem.name
        self.refdom = elem.refdom
        self.maxdeg = elem.maxdeg
        self.dim = elem.dim
        self.nodal_dofs = elem.nodal_dofs * self.dim
        self.edge_dofs = elem.edge_dofs * self.dim
        self.facet_dofs = elem.facet_dofs * self.dim
        self.interior_dofs = elem.interior_dofs * self.dim
        self.nbfun = elem.nbfun * self.dim


# --------------------------------------------------------------------------
# DOF numbering (dofs.py:264-334)
# --------------------------------------------------------------------------

def element_dofs(mesh: OMesh, elem: OElement) -> Tuple[np.ndarray, int]:
    """Dofs.__init__ (dofs.py:264-334): nodal dofs reshaped (nodal_dofs,
    nverts) in Fortran order, then 3-D edge dofs (t2e), then facet dofs
    (t2f; the triangle's edges are its facets), then interior dofs."""
    nv = mesh.nvertices
    nodal = np.arange(elem.nodal_dofs * nv, dtype=np.int32).reshape(
        (elem.nodal_dofs, nv), order="F")
    offset = elem.nodal_dofs * nv
    rows = [nodal[:, mesh.t[itr]] for itr in range(mesh.t.shape[0])]
    if elem.dim == 3 and elem.edge_dofs > 0:
        edges, t2e = build_entities(mesh.t, REF_TET_EDGES)
        ne = edges.shape[1]
        ed = np.arange(elem.edge_dofs * ne, dtype=np.int32).reshape(
            (elem.edge_dofs, ne), order="F") + offset
        offset += elem.edge_dofs * ne
        rows += [ed[:, t2e[itr]] for itr in range(t2e.shape[0])]
    if elem.dim == 2 and elem.facet_dofs > 0:
        facets, t2f = build_entities(mesh.t, REF_TRI_FACETS)
        nf = facets.shape[1]
        fd = np.arange(elem.facet_dofs * nf, dtype=np.int32).reshape(
            (elem.facet_dofs, nf), order="F") + offset
        offset += elem.facet_dofs * nf
        rows += [fd[:, t2f[itr]] for itr in range(t2f.shape[0])]
    ed = np.vstack(rows).astype(np.int32)
    return ed, int(ed.max()) + 1


# --------------------------------------------------------------------------
# Quadrature (quadrature.py:12-78, 80-845, 847-2836, 2839-2844)
# --------------------------------------------------------------------------

def _line(order):
    # quadrature.py:2839-2844: Gauss-Legendre with ceil((n+1)/2) points on [0,1]
    if order <= 1:
        order = 2
    X, W = np.polynomial.legendre.leggauss(int(math.ceil((order + 1.0) / 2.0)))
    return 0.5 * X + 0.5, W / 2.0


_RULES_FILE = __import__("os").path.join(
    __import__("os").path.dirname(__import__("os").path.dirname(
        __import__("os").path.abspath(__file__))), "tests", "golden", "quadrature_rules.npz")
_RULES = None


def quadrature(refdom: str, order: int) -> Tuple[np.ndarray, np.ndarray]:
    """get_quadrature (quadrature.py:12-78).

    Triangle / tetrahedron rules are read from ``tests/golden/quadrature_rules.npz``,
    which ``tests/golden/make_golden.py`` writes by calling the reference's
    ``get_quadrature_tri`` / ``get_quadrature_tet``: the reference tabulates
    its nodes to 15-16 decimals, and which rounding-noise local entries come
    out exactly 0.0 (and are dropped by ``eliminate_zeros``) depends on those
    last bits.  The hexahedral rule is generated as the reference does.
    ``quadrature_closed_form`` restates the same rules from their published
    closed forms; a test checks both agree to a few ulps.
    """
    global _RULES
    if refdom in ("tri", "tet"):
        if _RULES is None:
            _RULES = dict(np.load(_RULES_FILE))
        o = max(order, 1) if refdom == "tet" else max(order, 2)
        key = "%s%d" % (refdom, o)
        if key + "_X" in _RULES:
            return _RULES[key + "_X"].copy(), _RULES[key + "_W"].copy()
    return quadrature_closed_form(refdom, order)


def quadrature_closed_form(refdom: str, order: int) -> Tuple[np.ndarray, np.ndarray]:
    """The rules the configs use, from their published closed forms.

    tri 2: 3-point rule at (1/6,1/6),(2/3,1/6),(1/6,2/3), weight 1/6 each.
    tri 4: the 6-point degree-4 symmetric rule (two S21 orbits, Dunavant 1985),
           orbit parameters obtained here by Newton on the moment equations.
    tet 2: 4-point rule with a = (5+3*sqrt5)/20, b = (5-sqrt5)/20.
    tet 4: Keast's 11-point rule: centroid, S31 orbit at 1/14, S22 orbit at
           (1 +- sqrt(5/14))/4; weights -74/5625, 343/45000, 56/2250.
    hex n: tensor Gauss-Legendre, meshgrid(X,X,X) flattened Fortran order
           (quadrature.py:64-74).
    Point order follows the reference tables.
    """
    if refdom == "tri":
        if order <= 2:
            a, b = 1 / 6, 2 / 3
            X = np.array([[a, b, a], [a, a, b]])
            return X, np.full(3, 1 / 6)
        if order <= 4:
            a1, w1, a2, w2 = _dunavant4()
            c1, c2 = 1 - 2 * a1, 1 - 2 * a2
            X = np.array([[a1, a2, c1, c2, a1, a2],
                          [c1, c2, a1, a2, a1, a2]])
            # w1, w2 are whole-orbit weights (sum 1); three points per orbit, area 1/2
            W = np.array([w1, w2, w1, w2, w1, w2]) / 6
            return X, W
    if refdom == "tet":
        if order <= 2:
            a = (5 + 3 * math.sqrt(5)) / 20
            b = (5 - math.sqrt(5)) / 20
            X = np.array([[a, b, b, b], [b, b, b, a], [b, b, a, b]])
            return X, np.full(4, 0.25 / 6)
        if order <= 4:
            s = 1 / 14
            c = 1 - 3 * s
            p = (1 + math.sqrt(5 / 14)) / 4
            q = (1 - math.sqrt(5 / 14)) / 4
            X = np.array([
                [.25, c, s, s, s, q, p, p, p, q, q],
                [.25, s, s, s, c, p, q, p, q, p, q],
                [.25, s, s, c, s, p, p, q, q, q, p],
            ])
            W = np.array([-74 / 5625] + [343 / 45000] * 4 + [56 / 2250] * 6)
            return X, W
    if refdom == "hex":
        x, w = _line(order)
        A, B, C = np.meshgrid(x, x, x)
        X = np.vstack((A.flatten("F"), B.flatten("F"), C.flatten("F")))
        A, B, C = np.meshgrid(w, w, w)
        return X, (A * B * C).flatten("F")
    raise NotImplementedError((refdom, order))


def _dunavant4():
    """Orbit parameters of the symmetric 6-point degree-4 triangle rule:
    weights w1, w2 (summing to 1) at barycentric (a,a,1-2a).  Solved by
    Newton from the moment equations of the symmetric invariants
    1, e2, e3, e2^2 over the unit-area triangle."""
    from math import factorial

    def mono(a, b, c):
        # average over the triangle of l1^a l2^b l3^c
        return 2.0 * factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 2)

    # exact averages of the invariants
    e2 = 3 * mono(1, 1, 0)
    e3 = mono(1, 1, 1)
    e22 = 3 * mono(2, 2, 0) + 6 * mono(2, 1, 1)
    target = np.array([1.0, e2, e3, e22])

    def inv(a):
        l = np.array([a, a, 1 - 2 * a])
        s2 = l[0] * l[1] + l[1] * l[2] + l[0] * l[2]
        return np.array([1.0, s2, l[0] * l[1] * l[2], s2 * s2])

    def F(v):
        a1, w1, a2, w2 = v
        return w1 * inv(a1) + w2 * inv(a2) - target

    v = np.array([0.445, 0.22, 0.09, 0.11])
    for _ in range(60):
        f = F(v)
        J = np.zeros((4, 4))
        for k in range(4):
            dv = np.zeros(4)
            dv[k] = 1e-7
            J[:, k] = (F(v + dv) - F(v - dv)) / 2e-7
        v = v - np.linalg.solve(J, f)
        if np.max(np.abs(f)) < 1e-17:
            break
    return tuple(float(q) for q in v)


# --------------------------------------------------------------------------
# DiscreteField and form helpers (discrete_field.py, helpers.py)
# --------------------------------------------------------------------------

class DField(np.ndarray):
    """Minimal DiscreteField (discrete_field.py:7-110): value array with a
    ``grad`` attribute; ufunc results drop the attribute (:61-66)."""

    def __new__(cls, value, grad=None):
        obj = np.asarray(value).view(cls)
        obj.grad = grad
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self.grad = getattr(obj, "grad", None)

    def __array_wrap__(self, out_arr, context=None, return_scalar=False):
        return np.array(out_arr)


def grad(u):          # helpers.py:22-24
    return u.grad


def dot(u, v):        # helpers.py:108-110
    return np.einsum("i...,i...", u, v)


def ddot(u, v):       # helpers.py:113-115
    return np.einsum("ij...,ij...", u, v)


def transpose(T):     # helpers.py:142-144
    return np.einsum("ij...->ji...", T)


def sym_grad(u):      # helpers.py:71-73
    return .5 * (u.grad + transpose(u.grad))


def trace(T):         # helpers.py:137-139
    return np.einsum("ii...", T)


def eye(w, n):        # helpers.py:147-150
    return np.array([[w if i == j else 0. * w for i in range(n)]
                     for j in range(n)])


def laplace(u, v, w):            # models/poisson.py:7-9
    return dot(grad(u), grad(v))


def mass(u, v, w):               # models/poisson.py:17-19
    return u * v


def unit_load(v, w):             # models/poisson.py:22-24
    return v


def linear_elasticity(Lambda=1., Mu=1.):
    """models/elasticity.py:35-53."""
    def C(T):
        return 2. * Mu * T + Lambda * eye(trace(T), T.shape[0])

    def weakform(u, v, w):
        return ddot(C(sym_grad(u)), sym_grad(v))
    return weakform


def k_laplace_mass(u, v, w):
    """k * dot(grad u, grad v) + u * v with a coefficient field ``k``."""
    return w["k"] * dot(grad(u), grad(v)) + u * v


def k_laplace(u, v, w):
    return w["k"] * dot(grad(u), grad(v))


def theta_laplace(u, v, w):
    return w["theta"] * dot(grad(u), grad(v))


def f_load(v, w):
    return w["f"] * v


# --------------------------------------------------------------------------
# Basis (abstract_basis.py:45-88, cell_basis.py:42-106)
# --------------------------------------------------------------------------

class OBasis:
    """CellBasis restated: eager per-basis-function value/grad fields at all
    quadrature points, and dx = |detDF| * W (cell_basis.py:101-105)."""

    def __init__(self, mesh: OMesh, elem: OElement, intorder: Optional[int] = None,
                 elements=None):
        refdom = {"tri": "tri", "tet": "tet", "hex": "hex"}[mesh.kind]
        if refdom != elem.refdom:
            raise ValueError("Incompatible Mesh and Element.")  # abstract_basis.py:55-56
        self.mesh, self.elem = mesh, elem
        self.element_dofs, self.N = element_dofs(mesh, elem)
        self.Nbfun = self.element_dofs.shape[0]
        self.nelems = mesh.nelements
        if elements is not None:
            # CellBasis(elements=...) (cell_basis.py:94-99): normalize_elements
            # (mesh.py:1331-1369) with callables tested on cell midpoints
            # (mesh.py:481-493); geometry and DOFs restricted to the subset
            if callable(elements):
                tind = np.nonzero(elements(mesh.p[:, mesh.t].mean(axis=1)))[0].astype(np.int32)
            else:
                tind = np.asarray(elements)
            self.element_dofs = self.element_dofs[:, tind]
            self.mesh = mesh = OMesh(mesh.p, mesh.t[:, tind], mesh.kind)
            self.nelems = len(tind)
        self.X, self.W = quadrature(refdom, intorder if intorder is not None
                                    else 2 * elem.maxdeg)
        self.dim = mesh.p.shape[0]
        self._geometry()
        self.basis = [self._gbasis(j) for j in range(self.Nbfun)]
        self.dx = np.abs(self.detDF) * np.broadcast_to(self.W, (self.nelems, self.W.shape[-1]))

    # -- mappings --------------------------------------------------------
    def _geometry(self):
        m, X, dim = self.mesh, self.X, self.dim
        nq = X.shape[1]
        if m.affine:
            # MappingAffine._init_Ab / _init_invA (mapping_affine.py:55-131)
            p, t = m.p, m.t
            A = np.empty((dim, dim, m.nelements))
            for i in range(dim):
                for j in range(dim):
                    A[i, j] = p[i, t[j + 1]] - p[i, t[0]]
            if dim == 2:
                det = A[0, 0] * A[1, 1] - A[0, 1] * A[1, 0]
                inv = np.empty_like(A)
                inv[0, 0] = A[1, 1] / det
                inv[0, 1] = -A[0, 1] / det
                inv[1, 0] = -A[1, 0] / det
                inv[1, 1] = A[0, 0] / det
            else:
                det = (A[0, 0] * (A[1, 1] * A[2, 2] - A[1, 2] * A[2, 1])
                       - A[0, 1] * (A[1, 0] * A[2, 2] - A[1, 2] * A[2, 0])
                       + A[0, 2] * (A[1, 0] * A[2, 1] - A[1, 1] * A[2, 0]))
                inv = np.empty_like(A)
                inv[0, 0] = (-A[1, 2] * A[2, 1] + A[1, 1] * A[2, 2]) / det
                inv[1, 0] = (A[1, 2] * A[2, 0] - A[1, 0] * A[2, 2]) / det
                inv[2, 0] = (-A[1, 1] * A[2, 0] + A[1, 0] * A[2, 1]) / det
                inv[0, 1] = (A[0, 2] * A[2, 1] - A[0, 1] * A[2, 2]) / det
                inv[1, 1] = (-A[0, 2] * A[2, 0] + A[0, 0] * A[2, 2]) / det
                inv[2, 1] = (A[0, 1] * A[2, 0] - A[0, 0] * A[2, 1]) / det
                inv[0, 2] = (-A[0, 2] * A[1, 1] + A[0, 1] * A[1, 2]) / det
                inv[1, 2] = (A[0, 2] * A[1, 0] - A[0, 0] * A[1, 2]) / det
                inv[2, 2] = (-A[0, 1] * A[1, 0] + A[0, 0] * A[1, 1]) / det
            self.A, self.b = A, p[:, t[0]]
            self.detDF = np.tile(det, (nq, 1)).T                 # :205-211
            self.invDF = np.einsum("ijk,l->ijkl", inv, np.ones(nq))  # :225-232
        else:
            # MappingIsoparametric._J / detDF / invDF (mapping_isoparametric.py:112-226)
            p, t = m.p, m.t
            el = Hex1()
            J = [[np.zeros((m.nelements, nq)) for _ in range(dim)] for _ in range(dim)]
            for i in range(dim):
                for j in range(dim):
                    for itr in range(t.shape[0]):
                        _, dphi = el.lbasis(X, itr)
                        J[i][j] += p[i, t[itr]][:, None] * dphi[j]
            det = (J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1])
                   - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0])
                   + J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]))
            if np.sum(det == 0) > 0:
                raise Exception("Zero Jacobian determinant")     # :195-196
            inv = np.empty((dim, dim) + det.shape)
            inv[0, 0] = -J[1][2] * J[2][1] + J[1][1] * J[2][2]
            inv[1, 0] = J[1][2] * J[2][0] - J[1][0] * J[2][2]
            inv[2, 0] = -J[1][1] * J[2][0] + J[1][0] * J[2][1]
            inv[0, 1] = J[0][2] * J[2][1] - J[0][1] * J[2][2]
            inv[1, 1] = -J[0][2] * J[2][0] + J[0][0] * J[2][2]
            inv[2, 1] = J[0][1] * J[2][0] - J[0][0] * J[2][1]
            inv[0, 2] = -J[0][2] * J[1][1] + J[0][1] * J[1][2]
            inv[1, 2] = J[0][2] * J[1][0] - J[0][0] * J[1][2]
            inv[2, 2] = -J[0][1] * J[1][0] + J[0][0] * J[1][1]
            self.detDF = det
            self.invDF = inv / det

    def _gbasis(self, j):
        # ElementH1.gbasis (element_h1.py:10-24) and ElementVector.gbasis
        # (element_vector.py:36-48)
        elem = self.elem
        scalar = elem.elem if elem.vector else elem
        k = j // self.dim if elem.vector else j
        phi, dphi = scalar.lbasis(self.X, k)
        value = np.broadcast_to(phi, (self.nelems, self.X.shape[1]))
        g = np.einsum("ijkl,il->jkl", self.invDF, dphi)
        if not elem.vector:
            return (DField(value, g),)
        c = j - self.dim * k
        v = np.zeros((self.dim,) + value.shape)
        v[c] = value
        G = np.zeros((self.dim,) + g.shape)
        G[c] = g
        return (DField(v, G),)

    def default_parameters(self):
        """CellBasis.default_parameters (cell_basis.py:124-141): global
        coordinates of the quadrature points (MappingAffine.F,
        mapping_affine.py:183-193; MappingIsoparametric.F,
        mapping_isoparametric.py:50-58, 170-171) and the mesh parameter
        h = |detDF|**(1/dim)."""
        m, X, dim = self.mesh, self.X, self.dim
        if m.affine:
            x = np.empty((dim, self.nelems, X.shape[1]))
            for i in range(dim):
                s = 0.0
                for j in range(dim):
                    s = s + self.A[i, j][:, None] * X[j][None, :]
                x[i] = s + self.b[i][:, None]
        else:
            x = np.zeros((dim, self.nelems, X.shape[1]))
            el = Hex1()
            for itr in range(m.t.shape[0]):
                phi, _ = el.lbasis(X, itr)
                for i in range(dim):
                    x[i] += m.p[i, m.t[itr]][:, None] * phi
        h = np.abs(self.detDF) ** (1.0 / dim)
        return {"x": DField(x), "h": DField(h)}

    def zero_w(self):
        # abstract_basis.py:378-382
        return np.zeros((self.nelems, len(self.W)))

    def interpolate(self, w):
        # abstract_basis.py:271-322 (scalar elements)
        if w.shape[0] != self.N:
            raise ValueError("Input array has wrong size.")
        val = 0.
        gr = 0.
        for i in range(self.Nbfun):
            vals = w[self.element_dofs[i]]
            val = val + vals[:, None] * np.asarray(self.basis[i][0])
            gr = gr + vals[:, None] * self.basis[i][0].grad
        return DField(val, gr)


# --------------------------------------------------------------------------
# Assembly (bilinear_form.py:58-128, linear_form.py:18-49, coo_data.py:27-36,
# 102-108, form.py:91-121)
# --------------------------------------------------------------------------

class OParams(dict):
    """FormExtraParams (form.py:13-26): keys also readable as attributes."""

    def __getattr__(self, name):
        if name in self:
            return self[name]
        raise AttributeError("Attribute '{}' not found in 'w'.".format(name))


def _normalize_w(basis: OBasis, w: Dict) -> Dict:
    # form.py:91-121: numbers pass through, 1-D arrays are DOF vectors that
    # get interpolated, 2-D arrays become fields (checked against nqp); the
    # basis's default parameters come first (bilinear_form.py:77-80).
    out = OParams(basis.default_parameters())
    for k, v in w.items():
        if isinstance(v, np.ndarray) and v.ndim == 1:
            out[k] = basis.interpolate(v)
        elif isinstance(v, np.ndarray):
            if v.shape[-1] != basis.X.shape[-1]:
                raise ValueError("Quadrature mismatch")
            out[k] = DField(v)
        else:
            out[k] = v
    return out


def bilinear_local(form: Callable, ubasis: OBasis, vbasis: Optional[OBasis] = None,
                   nthreads: int = 0, **w):
    """BilinearForm._assemble (bilinear_form.py:58-128): returns
    ``data`` of shape (Nu, Nv, nelems), ``rows``/``cols`` in the reference's
    COO order (index nt*(Nv*j + i) + e), and the shape (Nv_dofs, Nu_dofs).
    nthreads > 0 splits the (j, i) loop over Python threads as the
    reference does (bilinear_form.py:100-119)."""
    vbasis = ubasis if vbasis is None else vbasis
    nt = ubasis.nelems
    dx = ubasis.dx
    wd = _normalize_w(ubasis, w)
    Nu, Nv = ubasis.Nbfun, vbasis.Nbfun
    data = np.zeros((Nu, Nv, nt))
    rows = np.zeros(Nu * Nv * nt, dtype=np.int32)
    cols = np.zeros(Nu * Nv * nt, dtype=np.int32)
    for j in range(Nu):
        for i in range(Nv):
            ixs = slice(nt * (Nv * j + i), nt * (Nv * j + i + 1))
            rows[ixs] = vbasis.element_dofs[i]
            cols[ixs] = ubasis.element_dofs[j]
            if nthreads <= 0:
                data[j, i, :] = np.sum(form(*ubasis.basis[j], *vbasis.basis[i], wd) * dx, axis=1)
    if nthreads > 0:
        from threading import Thread
        pairs = np.array([[i, j] for j in range(Nu) for i in range(Nv)])

        def work(ix):
            for i, j in ix:
                data[j, i] = np.sum(form(*ubasis.basis[j], *vbasis.basis[i], wd) * dx, axis=1)

        ths = [Thread(target=work, args=(ix,)) for ix in np.array_split(pairs, nthreads, axis=0)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    return data, rows, cols, (vbasis.N, ubasis.N)


def bilinear_assemble(form: Callable, ubasis: OBasis, vbasis: Optional[OBasis] = None,
                      nthreads: int = 0, **w):
    """Form -> COO -> eliminate_zeros -> CSR (coo_data.py:27-36)."""
    data, rows, cols, shape = bilinear_local(form, ubasis, vbasis, nthreads=nthreads, **w)
    K = coo_matrix((data.flatten("C"), (rows, cols)), shape=shape)
    K.eliminate_zeros()
    return K.tocsr()


def linear_local(form: Callable, basis: OBasis, **w):
    """LinearForm._assemble (linear_form.py:18-46)."""
    nt = basis.nelems
    wd = _normalize_w(basis, w)
    data = np.zeros(basis.Nbfun * nt)
    rows = np.zeros(basis.Nbfun * nt, dtype=np.int32)
    for i in range(basis.Nbfun):
        ixs = slice(nt * i, nt * (i + 1))
        rows[ixs] = basis.element_dofs[i]
        data[ixs] = np.sum(form(*basis.basis[i], wd) * basis.dx, axis=1)
    return data, rows


def linear_assemble(form: Callable, basis: OBasis, **w) -> np.ndarray:
    """COOData.toarray for 1-D shape (coo_data.py:102-108)."""
    data, rows = linear_local(form, basis, **w)
    return coo_matrix((data, (rows, np.zeros_like(rows))),
                      shape=(basis.N, 1)).toarray().T[0]


# --------------------------------------------------------------------------
# Gradient oracles for the adjoint (no reference counterpart: scikit-fem
# differentiates only with respect to the solution field)
# --------------------------------------------------------------------------

def theta_gradient(form_unit: Callable, basis: OBasis, wvec, uvec, **w):
    """d(w^T K(theta) u)/d theta_e for K = sum_e theta_e K_e: the element
    functional  a_e(u_h, w_h)  (the same value Functional.elemental gives,
    functional.py:26-34) computed from the local matrices of ``form_unit``."""
    data, _, _, _ = bilinear_local(form_unit, basis, **w)
    ed = basis.element_dofs
    # data[j, i, e] = a(phi_j, phi_i) on e ; row i (test) pairs with w
    return np.einsum("jie,ie,je->e", data, wvec[ed], uvec[ed])


def fd_x_gradient(assemble_scalar: Callable[[np.ndarray], float], p: np.ndarray,
                  h: float = 1e-6) -> np.ndarray:
    """Central differences of a scalar function of the node coordinates."""
    g = np.zeros_like(p)
    for a in range(p.shape[0]):
        for n in range(p.shape[1]):
            pp = p.copy()
            pp[a, n] += h
            fp = assemble_scalar(pp)
            pp[a, n] -= 2 * h
            fm = assemble_scalar(pp)
            g[a, n] = (fp - fm) / (2 * h)
    return g
