"""Quadrature rules (get_quadrature, skfem/quadrature.py:12-78).

The affine-simplex kernels integrate with exact reference tensors and need
no points; the rules here give ``Basis.X`` / ``Basis.W`` (and so the shape
of ``zero_w()``), the hexahedral rule of the isoparametric kernel and the
nodes of the exact-zero mask.  Triangle / tetrahedron rules of orders 1-4
are the reference's own tables, bit-exact (``_refquad.py``, generated from
fixtures recorded by running the reference): which rounding-noise local
entries the reference computes as exactly 0.0 depends on the last bits of
its nodes.  The closed forms below derive the same rules (to a few ulps)
and are used for orders the tables do not hold.

  tri order <= 2: 3-point rule at (1/6, 1/6), (2/3, 1/6), (1/6, 2/3)
  tri order 3, 4: the symmetric 6-point degree-4 rule (Dunavant 1985; two
                  S21 orbits), orbit parameters solved from the moment
                  equations below
  tet order <= 2: 4-point rule, a = (5 + 3 sqrt 5)/20, b = (5 - sqrt 5)/20
  tet order 3, 4: Keast's 11-point degree-4 rule
  hex order n:    tensor Gauss-Legendre with ceil((n+1)/2) points per axis
                  (numpy's leggauss, as quadrature.py:2839-2844),
                  meshgrid(X, X, X) flattened in Fortran order (:64-74)
Point order follows the reference tables.
"""

import math

import numpy as np

__all__ = ["get_quadrature", "gauss_line"]


def gauss_line(order):
    if order <= 1:
        order = 2
    x, w = np.polynomial.legendre.leggauss(int(math.ceil((order + 1.0) / 2.0)))
    return 0.5 * x + 0.5, w / 2.0


def _tri_degree4():
    """Whole-orbit weights (w1, w2; sum 1) and parameters (a1, a2) of the
    degree-4 rule with points (a, a, 1-2a): Newton on the averages of the
    symmetric invariants 1, e2, e3, e2^2 over the triangle."""
    f = math.factorial

    def avg(a, b, c):
        return 2.0 * f(a) * f(b) * f(c) / f(a + b + c + 2)

    target = np.array([1.0, 3 * avg(1, 1, 0), avg(1, 1, 1), 3 * avg(2, 2, 0) + 6 * avg(2, 1, 1)])

    def inv(a):
        s2 = a * a + 2 * a * (1 - 2 * a)
        return np.array([1.0, s2, a * a * (1 - 2 * a), s2 * s2])

    def F(v):
        return v[1] * inv(v[0]) + v[3] * inv(v[2]) - target

    v = np.array([0.445, 0.22, 0.09, 0.11])
    for _ in range(50):
        r = F(v)
        J = np.empty((4, 4))
        for k in range(4):
            d = np.zeros(4)
            d[k] = 1e-7
            J[:, k] = (F(v + d) - F(v - d)) / 2e-7
        step = np.linalg.solve(J, r)
        v = v - step
        if np.max(np.abs(step)) < 1e-17:
            break
    return v


def _table(refdom, norder):
    from ._refquad import RULES
    key = "%s%d" % (refdom, max(norder, 1 if refdom == "tet" else 2))
    if key not in RULES:
        return None
    X, W = RULES[key]
    return (np.array([[float.fromhex(v) for v in row] for row in X]),
            np.array([float.fromhex(v) for v in W]))


def get_quadrature(refdom, norder):
    if refdom in ("tri", "tet"):
        t = _table(refdom, norder)
        if t is not None:
            return t
    if refdom == "line":
        from ._refquad import RULES
        key = "line%d" % max(norder, 1)
        if key in RULES:
            X, W = RULES[key]
            return (np.array([[float.fromhex(v) for v in row] for row in X]),
                    np.array([float.fromhex(v) for v in W]))
        x, w = gauss_line(norder)
        return x[None, :], w
    if refdom == "quad":
        # tensor product of the line rule (quadrature.py:55-62)
        x, w = get_quadrature("line", norder)
        A, B = np.meshgrid(x[0], x[0])
        X = np.vstack((A.flatten(order="F"), B.flatten(order="F")))
        A, B = np.meshgrid(w, w)
        return X, (A * B).flatten(order="F")
    if refdom == "hex" and norder in (6, 7):
        # the reference's default Hex1 rule as recorded (leggauss's last bits
        # depend on the platform's eigenvalue solver)
        from ._refquad import RULES
        X, W = RULES["hex6"]
        return (np.array([[float.fromhex(v) for v in row] for row in X]),
                np.array([float.fromhex(v) for v in W]))
    return closed_form_quadrature(refdom, norder)


def closed_form_quadrature(refdom, norder):
    if refdom == "tri":
        if norder <= 2:
            a, b = 1.0 / 6.0, 2.0 / 3.0
            return np.array([[a, b, a], [a, a, b]]), np.full(3, 1.0 / 6.0)
        if norder <= 4:
            a1, w1, a2, w2 = _tri_degree4()
            c1, c2 = 1 - 2 * a1, 1 - 2 * a2
            X = np.array([[a1, a2, c1, c2, a1, a2], [c1, c2, a1, a2, a1, a2]])
            return X, np.array([w1, w2, w1, w2, w1, w2]) / 6.0
    elif refdom == "tet":
        if norder <= 2:
            a = (5 + 3 * math.sqrt(5)) / 20
            b = (5 - math.sqrt(5)) / 20
            return np.array([[a, b, b, b], [b, b, b, a], [b, b, a, b]]), np.full(4, 1.0 / 24.0)
        if norder <= 4:
            s, c = 1.0 / 14.0, 11.0 / 14.0
            p = (1 + math.sqrt(5.0 / 14.0)) / 4
            q = (1 - math.sqrt(5.0 / 14.0)) / 4
            X = np.array([[.25, c, s, s, s, q, p, p, p, q, q],
                          [.25, s, s, s, c, p, q, p, q, p, q],
                          [.25, s, s, c, s, p, p, q, q, q, p]])
            W = np.array([-74 / 5625] + [343 / 45000] * 4 + [56 / 2250] * 6)
            return X, W
    elif refdom == "hex":
        x, w = gauss_line(norder)
        A, B, C = np.meshgrid(x, x, x)
        X = np.vstack((A.flatten("F"), B.flatten("F"), C.flatten("F")))
        A, B, C = np.meshgrid(w, w, w)
        return X, (A * B * C).flatten("F")
    raise NotImplementedError("quadrature of order %d on %s" % (norder, refdom))
