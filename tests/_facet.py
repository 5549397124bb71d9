"""Forms of the FacetBasis fixtures (tests/golden/make_golden.py,
facet_cases) written with this package's helpers."""
import skfem_gb300 as F
from skfem_gb300.helpers import dot, grad

# the FacetBasis variants each fixture holds: prefix -> (facets, side)
VARIANTS = ("", "in0_", "in1_", "cb_")


@F.BilinearForm
def fmass(u, v, w):
    return u * v


@F.BilinearForm
def robin(u, v, w):
    return (1.0 + w.x[0]) * u * v + dot(w.n, grad(u)) * v


@F.LinearForm
def neumann(v, w):
    return dot(w.n, w.x) * v + w.h * v


@F.Functional
def length(w):
    return 1.0 + 0.0 * w.x[0]


@F.Functional
def s_energy(w):
    return w['s'] ** 2 + dot(w.n, grad(w['s']))


@F.BilinearForm
def vmass(u, v, w):
    return dot(u, v)


@F.LinearForm
def traction(v, w):
    return (1.0 + w.x[2]) * dot(w.n, v)


CASES = [("tri_p1_facet", F.MeshTri, F.ElementTriP1),
         ("tri_p2_facet", F.MeshTri, F.ElementTriP2),
         ("tet_p1_facet", F.MeshTet, F.ElementTetP1),
         ("tet_p2_facet", F.MeshTet, F.ElementTetP2),
         ("hex1_facet", F.MeshHex, F.ElementHex1)]


def facet_args(m, g, prefix):
    """FacetBasis arguments reproducing the fixture's variant."""
    import numpy as np
    if prefix == "":
        return {}
    if prefix in ("in0_", "in1_"):
        return {"facets": np.nonzero(m.f2t[1] >= 0)[0].astype(np.int32),
                "side": int(prefix[2])}
    return {"facets": lambda x: x[1] < 0.3}
