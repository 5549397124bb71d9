"""Generate fem_refquad.cuh: the reference's quadrature rules bit-exactly.

scikit-fem tabulates its triangle / tetrahedron rules to 15-16 decimals
(quadrature.py:80-2836) and builds the hexahedral rule from numpy's
leggauss (:64-74, :2839-2844).  The exact-zero mask of the pattern build
replays the reference's arithmetic, so it needs the very same doubles:
they are read here from the fixtures tests/golden/make_golden.py recorded
by calling the reference itself, and emitted as hexadecimal literals.
Run once (the header is committed); the build does not regenerate it.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(os.path.dirname(os.path.dirname(HERE)), "tests", "golden")


def lit(x):
    return float(x).hex()


def arr(name, a):
    a = np.asarray(a, dtype=np.float64).ravel()
    body = ", ".join(lit(v) for v in a)
    return "__constant__ double %s[%d] = {%s};\n" % (name, a.size, body)


def main():
    q = dict(np.load(os.path.join(GOLD, "quadrature_rules.npz")))
    hexg = dict(np.load(os.path.join(GOLD, "hex1_laplace_8.npz")))
    out = ["// Generated by gen_refquad.py from reference-recorded fixtures (do not edit).",
           "#pragma once", ""]
    for key, nq in (("tri2", 3), ("tri4", 6), ("tet2", 4), ("tet4", 11)):
        X, W = q[key + "_X"], q[key + "_W"]
        assert X.shape[1] == nq
        out.append(arr("c_rq_%s_X" % key, X))   # (dim, nq) row-major
        out.append(arr("c_rq_%s_W" % key, W))
    X, W = hexg["X"], hexg["W"]
    assert X.shape == (3, 64)
    out.append(arr("c_rq_hex6_X", X))
    out.append(arr("c_rq_hex6_W", W))
    path = os.path.join(HERE, "fem_refquad.cuh")
    open(path, "w").write("\n".join(out))
    # the same rules for the Python side (Basis.X / Basis.W)
    py = ['"""Generated by csrc/gen_refquad.py from reference-recorded fixtures (do not',
          'edit): scikit-fem\'s triangle (orders 1-19) / tetrahedron (1-9) quadrature rules,',
          'its line rules of orders 1-10 and its default hexahedral rule, bit-exact, as',
          'hexadecimal floats."""', "",
          "RULES = {"]
    for key in sorted((k[:-2] for k in q if k.endswith("_X")),
                      key=lambda k: (k[:3], int(k[3:]))):
        X, W = q[key + "_X"], q[key + "_W"]
        py.append("    %r: (%r,\n           %r)," % (
            key, [[float(v).hex() for v in row] for row in X], [float(v).hex() for v in W]))
    # the default Hex1 rule (intorder 6-7, 4x4x4 leggauss points)
    # Gauss-Legendre line rules (FacetBasis quadrature of triangle meshes)
    lines = dict(np.load(os.path.join(GOLD, "line_rules.npz")))
    for key in sorted((k[:-2] for k in lines if k.endswith("_X")), key=lambda k: int(k[4:])):
        X, W = lines[key + "_X"], lines[key + "_W"]
        py.append("    %r: (%r,\n           %r)," % (
            key, [[float(v).hex() for v in row] for row in X], [float(v).hex() for v in W]))
    Xh, Wh = hexg["X"], hexg["W"]
    py.append("    %r: (%r,\n           %r)," % (
        "hex6", [[float(v).hex() for v in row] for row in Xh], [float(v).hex() for v in Wh]))
    py.append("}")
    pkg = os.path.join(os.path.dirname(HERE), "skfem_gb300", "_refquad.py")
    open(pkg, "w").write("\n".join(py) + "\n")
    return path


if __name__ == "__main__":
    print(main())
