"""Generate fem_tables.cuh: exact reference tensors for the element families.

The tensor representation of a bilinear form on affine cells (Kirby & Logg,
"A compiler for variational forms", ACM TOMS 2006) splits each local matrix
into element-independent integrals over the reference cell, computed here in
exact rational arithmetic, and a few geometric factors the kernels compute
per element.  The basis functions restate scikit-fem 12.0.1:

  TriP1  element_tri_p1.py:18-33     TriP2 element_tri_p2.py:22-48
  TetP1  element_tet_p1.py:19-45     TetP2 element_tet_p2.py:26-103
  Hex1   element_hex1.py:23-69 (node k at the reference corner refdom.py:173-180)

Simplices are written in barycentric coordinates l_0 = 1 - sum(x), l_{m+1} =
x_m; for every function grad(phi_i) = sum_a p_ia(l) grad(l_a).  The tables
hold, with |T| the cell measure,

  BB[i][j][a][b] = (1/|T|) int_T p_ia p_jb        (stiffness, vector coupling)
  MM[i][j]       = (1/|T|) int_T phi_i phi_j        (mass)
  LV[i]          = (1/|T|) int_T phi_i              (load)

and for the trilinear hexahedron on the unit cube

  HS[k][l][i][j] = int d_k phi_i d_l phi_j,  HM[i][j] = int phi_i phi_j,
  HL[i] = int phi_i.

The 4-point Gauss-Legendre rule of the isoparametric path comes from
numpy.polynomial.legendre.leggauss, the same routine the reference calls
(quadrature.py:2839-2844), so both use bit-identical nodes.

Run:  python gen_tables.py  (writes fem_tables.cuh next to this file).
"""

import os
from fractions import Fraction as F
from itertools import product
from math import factorial

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# ---- polynomials over barycentric coordinates: {exponent tuple: Fraction}
def padd(p, q, s=F(1)):
    r = dict(p)
    for k, v in q.items():
        r[k] = r.get(k, F(0)) + s * v
    return {k: v for k, v in r.items() if v != 0}


def pmul(p, q):
    r = {}
    for (ka, va), (kb, vb) in product(p.items(), q.items()):
        k = tuple(x + y for x, y in zip(ka, kb))
        r[k] = r.get(k, F(0)) + va * vb
    return {k: v for k, v in r.items() if v != 0}


def lam(a, n):
    e = [0] * n
    e[a] = 1
    return {tuple(e): F(1)}


def const(c, n):
    return {tuple([0] * n): F(c)}


def integ(p, d):
    """(1/|T|) int_T p over a d-simplex with n = d+1 barycentrics."""
    tot = F(0)
    for k, v in p.items():
        num = factorial(d)
        for x in k:
            num *= factorial(x)
        tot += v * F(num, factorial(sum(k) + d))
    return tot


def simplex_p1(d):
    n = d + 1
    phi = [lam(a, n) for a in range(n)]
    grads = [{a: const(1, n)} for a in range(n)]  # grad phi_a = grad l_a
    return phi, grads


def simplex_p2(d):
    n = d + 1
    edges = [(0, 1), (1, 2), (0, 2)] if d == 2 else \
        [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
    phi, grads = [], []
    for a in range(n):  # vertex: l_a (2 l_a - 1)
        phi.append(pmul(lam(a, n), padd(pmul(const(2, n), lam(a, n)), const(1, n), F(-1))))
        grads.append({a: padd(pmul(const(4, n), lam(a, n)), const(1, n), F(-1))})
    for (a, b) in edges:  # edge: 4 l_a l_b
        phi.append(pmul(const(4, n), pmul(lam(a, n), lam(b, n))))
        grads.append({a: pmul(const(4, n), lam(b, n)), b: pmul(const(4, n), lam(a, n))})
    return phi, grads


def simplex_tables(d, order):
    phi, grads = simplex_p1(d) if order == 1 else simplex_p2(d)
    nb, n = len(phi), d + 1
    BB = [[[[F(0)] * n for _ in range(n)] for _ in range(nb)] for _ in range(nb)]
    for i, j in product(range(nb), range(nb)):
        for a, pa in grads[i].items():
            for b, pb in grads[j].items():
                BB[i][j][a][b] = integ(pmul(pa, pb), d)
    MM = [[integ(pmul(phi[i], phi[j]), d) for j in range(nb)] for i in range(nb)]
    LV = [integ(phi[i], d) for i in range(nb)]
    return BB, MM, LV


# ---- trilinear hexahedron on [0,1]^3 ------------------------------------
HEX_CORNERS = [(1, 1, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1),
               (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 0, 0)]


def hex_tables():
    # 1-D factor f_c(t) = t (c=1) or 1-t (c=0): int f f' = 1/3 same, 1/6 diff;
    # int f = 1/2; int f' f'' (derivatives) = +-1; int f * g' = +-1/2.
    def i_ff(a, b):
        return F(1, 3) if a == b else F(1, 6)

    def i_dd(a, b):
        return F(1) if a == b else F(-1)

    def i_fd(a, b):  # int f_a * d f_b
        return F(1, 2) if b == 1 else F(-1, 2)

    HS = [[[[F(0)] * 8 for _ in range(8)] for _ in range(3)] for _ in range(3)]
    for k, l, i, j in product(range(3), range(3), range(8), range(8)):
        ci, cj = HEX_CORNERS[i], HEX_CORNERS[j]
        v = F(1)
        for ax in range(3):
            if ax == k and ax == l:
                v *= i_dd(ci[ax], cj[ax])
            elif ax == k:
                v *= i_fd(cj[ax], ci[ax])
            elif ax == l:
                v *= i_fd(ci[ax], cj[ax])
            else:
                v *= i_ff(ci[ax], cj[ax])
        HS[k][l][i][j] = v
    HM = [[F(1) for _ in range(8)] for _ in range(8)]
    for i, j in product(range(8), range(8)):
        v = F(1)
        for ax in range(3):
            v *= i_ff(HEX_CORNERS[i][ax], HEX_CORNERS[j][ax])
        HM[i][j] = v
    HL = [F(1, 8)] * 8
    return HS, HM, HL


def dlit(x):
    x = float(x)
    if x == 0.0:
        return "0.0"
    return repr(x)


def emit_array(name, arr, ctype="double"):
    a = np.array(arr, dtype=object)
    lit = dlit if ctype == "double" else (lambda v: str(int(v)))
    flat = [lit(v) for v in a.reshape(-1)]
    dims = "".join("[%d]" % s for s in a.shape)
    lines = []
    for k in range(0, len(flat), 6):
        lines.append("  " + ", ".join(flat[k:k + 6]) + ",")
    return "__constant__ %s %s%s = {\n%s\n};\n" % (ctype, name, dims, "\n".join(lines))


def emit_simplex_contractions(tag, d, order):
    """Straight-line code of  out_ij = sum_ab BB[i][j][a][b] * G(a,b)  for
    i <= j, where G(a,b) is a caller macro; zero terms are omitted."""
    BB, MM, LV = simplex_tables(d, order)
    nb, n = len(BB), d + 1
    out = ["// %s: K(i,j) = sum_ab BB[i][j][a][b] G(a,b); symmetric in (i,j)" % tag,
           "#define %s_NB %d" % (tag, nb)]
    body = []
    for i in range(nb):
        for j in range(i, nb):
            terms = []
            for a in range(n):
                for b in range(n):
                    c = BB[i][j][a][b]
                    if c != 0:
                        terms.append("(%s)*G(%d,%d)" % (dlit(c), a, b))
            expr = " + ".join(terms) if terms else "0.0"
            body.append("  K(%d,%d, %s);" % (i, j, expr))
    out.append("#define %s_STIFF(G, K) do { \\\n%s \\\n} while (0)" % (tag, " \\\n".join(body)))
    mbody = []
    for i in range(nb):
        for j in range(i, nb):
            mbody.append("  K(%d,%d, %s);" % (i, j, dlit(MM[i][j])))
    out.append("#define %s_MASS(K) do { \\\n%s \\\n} while (0)" % (tag, " \\\n".join(mbody)))
    out.append("__device__ __forceinline__ double %s_load(int i) { switch (i) { %s default: return 0.0; } }"
               % (tag.lower(), " ".join("case %d: return %s;" % (i, dlit(LV[i])) for i in range(nb))))
    return "\n".join(out) + "\n"


def reduced_terms(BB, i, j, d):
    """sum_ab BB[i][j][a][b] G(a,b) rewritten over G(m,n), 1 <= m <= n <= d,
    using grad l_0 = -sum_m grad l_m (so G(0,n) = -sum_m G(m,n))."""
    n = d + 1
    out = {}

    def expand(a):
        return [(a, F(1))] if a > 0 else [(m, F(-1)) for m in range(1, n)]

    for a in range(n):
        for b in range(n):
            c = BB[i][j][a][b]
            if c == 0:
                continue
            for (m, sm) in expand(a):
                for (k, sk) in expand(b):
                    key = (min(m, k), max(m, k))
                    out[key] = out.get(key, F(0)) + c * sm * sk
    return {k: v for k, v in out.items() if v != 0}


def emit_reduced(tag, d, order):
    """K(i, j, stiffness over reduced Gram GR(m,n), mass constant) for i <= j."""
    BB, MM, LV = simplex_tables(d, order)
    nb = len(BB)
    body = []
    for i in range(nb):
        for j in range(i, nb):
            t = reduced_terms(BB, i, j, d)
            expr = " + ".join("(%s)*GR(%d,%d)" % (dlit(c), m, k) for (m, k), c in sorted(t.items()))
            body.append("  K(%d,%d, %s, %s);" % (i, j, expr if expr else "0.0", dlit(MM[i][j])))
    return "#define %s_KRED(GR, K) do { \\\n%s \\\n} while (0)\n" % (tag, " \\\n".join(body))


def emit_bb_terms(tag, d):
    """For the vector P2 kernel: per (i,j) block, the list of (a, b, coef)."""
    BB, _, _ = simplex_tables(d, 2)
    nb, n = len(BB), d + 1
    lines = ["// %s: BLOCK(i,j,T) with T(a,b,c) terms of BB[i][j]" % tag]
    body = []
    for i in range(nb):
        for j in range(nb):
            terms = []
            for a in range(n):
                for b in range(n):
                    c = BB[i][j][a][b]
                    if c != 0:
                        terms.append("T(%d,%d,%s)" % (a, b, dlit(c)))
            body.append("  if (J == %d) { %s }" % (j, " ".join(terms)))
    # macro over j for fixed i is emitted per i
    for i in range(nb):
        parts = []
        for j in range(nb):
            terms = []
            for a in range(n):
                for b in range(n):
                    c = BB[i][j][a][b]
                    if c != 0:
                        terms.append("T(%d,%d,%s);" % (a, b, dlit(c)))
            parts.append("case %d: { %s } break;" % (j, " ".join(terms)))
        lines.append("#define %s_ROW%d(J, T) switch (J) { %s default: break; }" % (tag, i, " ".join(parts)))
    return "\n".join(lines) + "\n"


def emit_qacc(tag, d, order):
    """Q(a,b) += BB[i][j][a][b] * W(i) * U(j) over all (i, j): the gradient of
    E = w^T K u with respect to the Gram entries G(a,b) (adjoint kernels)."""
    BB, MM, LV = simplex_tables(d, order)
    nb, n = len(BB), d + 1
    body = []
    for i in range(nb):
        for j in range(nb):
            for a in range(n):
                for b in range(n):
                    c = BB[i][j][a][b]
                    if c != 0:
                        body.append("  Q(%d,%d) += (%s) * (W(%d) * U(%d));" % (a, b, dlit(c), i, j))
    mbody = []
    for i in range(nb):
        for j in range(nb):
            if MM[i][j] != 0:
                mbody.append("  MU += (%s) * (W(%d) * U(%d));" % (dlit(MM[i][j]), i, j))
    lbody = ["  LW += (%s) * W(%d);" % (dlit(LV[i]), i) for i in range(nb) if LV[i] != 0]
    return ("#define %s_QACC(W, U, Q) do { \\\n%s \\\n} while (0)\n"
            "#define %s_MACC(W, U, MU) do { \\\n%s \\\n} while (0)\n"
            "#define %s_LACC(W, LW) do { \\\n%s \\\n} while (0)\n"
            % (tag, " \\\n".join(body), tag, " \\\n".join(mbody), tag,
               " \\\n".join(lbody) if lbody else ""))


def main():
    out = ["// Generated by gen_tables.py -- exact reference tensors (do not edit).",
           "#pragma once", ""]
    out.append(emit_simplex_contractions("TRI1", 2, 1))
    out.append(emit_simplex_contractions("TRI2", 2, 2))
    out.append(emit_simplex_contractions("TET1", 3, 1))
    out.append(emit_simplex_contractions("TET2", 3, 2))
    for tag, d, o in (("TRI1", 2, 1), ("TRI2", 2, 2), ("TET1", 3, 1), ("TET2", 3, 2)):
        out.append(emit_qacc(tag, d, o))
        out.append(emit_reduced(tag, d, o))
    out.append(emit_bb_terms("TET2BB", 3))
    out.append(emit_bb_terms("TRI2BB", 2))
    for tag, d, o in (("tri1", 2, 1), ("tri2", 2, 2), ("tet1", 3, 1), ("tet2", 3, 2)):
        _, MM, _ = simplex_tables(d, o)
        out.append(emit_array("c_%s_mm" % tag, MM))
    HS, HM, HL = hex_tables()
    out.append(emit_array("c_hex_S", HS))
    out.append(emit_array("c_hex_M", HM))
    # Gauss-Legendre (leggauss) on [0,1] with 2 and 4 points
    for npt in (2, 4):
        x, w = np.polynomial.legendre.leggauss(npt)
        out.append(emit_array("c_gl%d_x" % npt, list(0.5 * x + 0.5)))
        out.append(emit_array("c_gl%d_w" % npt, list(w / 2.0)))
    out.append(emit_array("c_hex_corner", HEX_CORNERS, ctype="int"))
    path = os.path.join(HERE, "fem_tables.cuh")
    with open(path, "w") as f:
        f.write("\n".join(out))
    return path


if __name__ == "__main__":
    print(main())
