"""Generate golden fixtures by running scikit-fem itself (run in a container
where the scikit-fem source tree is importable; the fixtures travel, the
reference does not).

    PYTHONPATH=<scikit-fem checkout> python tests/golden/make_golden.py

Each case stores the mesh (p, t), the reference's element_dofs, its
quadrature (X, W), the coefficient arrays it was given, the assembled CSR
(indptr, indices, data) and, where the case has one, the load vector b or
the adjoint oracles.  Sizes are small so the fixtures stay a few hundred KB.
"""

import os
import sys

import numpy as np

import skfem
from skfem import (Basis, BilinearForm, ElementHex1, ElementTetP1,
                   ElementTetP2, ElementTriP1, ElementTriP2, ElementVector,
                   Functional, LinearForm, MeshHex, MeshTet, MeshTri)
from skfem.helpers import dot, grad
from skfem.models.elasticity import linear_elasticity
from skfem.models.poisson import laplace, mass, unit_load

OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, **arrs):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrs)
    print(name, {k: getattr(v, "shape", v) for k, v in arrs.items()})


def csr_arrays(K):
    K = K.tocsr()
    return dict(indptr=K.indptr, indices=K.indices, data=K.data,
                shape=np.array(K.shape))


@BilinearForm
def k_laplace_mass(u, v, w):
    return w.k * dot(grad(u), grad(v)) + u * v


@BilinearForm
def k_laplace(u, v, w):
    return w.k * dot(grad(u), grad(v))


@BilinearForm
def theta_laplace(u, v, w):
    return w.theta * dot(grad(u), grad(v))


@LinearForm
def f_load(v, w):
    return w.f * v


def jitter(m, rng, amp):
    p = m.p.copy()
    lo, hi = p.min(axis=1, keepdims=True), p.max(axis=1, keepdims=True)
    inner = np.all((p > lo + 1e-12) & (p < hi - 1e-12), axis=0)
    return inner


def main():
    rng = np.random.default_rng(20261203)

    # 1. doctest case: MeshTri() default, mass matrix (bilinear_form.py:26-30)
    m = MeshTri()
    ib = Basis(m, ElementTriP1())
    save("tri_default_mass", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, **csr_arrays(mass.assemble(ib)))

    # 2. TriP1 Laplace + unit load on a 16x16 tensor mesh (the CPU-sized Poisson case)
    m = MeshTri.init_tensor(np.linspace(0, 1, 17), np.linspace(0, 1, 17))
    ib = Basis(m, ElementTriP1())
    save("tri_p1_laplace", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, b=unit_load.assemble(ib), **csr_arrays(laplace.assemble(ib)))

    # 3. TetP1 k*Laplace + mass, 6x6x6 cells, k ~ lognormal(0,1) per element
    m = MeshTet.init_tensor(*(np.linspace(0, 1, 7),) * 3)
    ib = Basis(m, ElementTetP1())
    k = rng.lognormal(0.0, 1.0, m.t.shape[1])
    K = k_laplace_mass.assemble(ib, k=ib.zero_w() + k[:, None])
    b = f_load.assemble(ib, f=ib.zero_w() + k[:, None])
    save("tet_p1_k_laplace_mass", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, k=k, b=b, **csr_arrays(K))

    # 4. vector TetP2 elasticity, 3x3x3 cells jittered +-0.2h, lambda=1, mu=0.5
    n = 3
    m = MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    m = MeshTet(p, m.t)
    ib = Basis(m, ElementVector(ElementTetP2()), intorder=4)
    K = linear_elasticity(1.0, 0.5).assemble(ib)
    save("tet_p2_vec_elasticity", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, **csr_arrays(K))

    # 5. scalar TetP2 Laplace on an unjittered 3x3x3 mesh (exact-zero entries)
    m = MeshTet.init_tensor(*(np.linspace(0, 1, 4),) * 3)
    ib = Basis(m, ElementTetP2())
    save("tet_p2_laplace", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, b=unit_load.assemble(ib), **csr_arrays(laplace.assemble(ib)))

    # 6. TriP2 k*Laplace on a jittered 8x8 unit square, k ~ lognormal(0,0.5)
    n = 8
    m = MeshTri.init_tensor(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1))
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(2, int(inner.sum())))
    m = MeshTri(p, m.t)
    ib = Basis(m, ElementTriP2())
    k = rng.lognormal(0.0, 0.5, m.t.shape[1])
    K = k_laplace.assemble(ib, k=ib.zero_w() + k[:, None])
    save("tri_p2_k_laplace", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, k=k, b=unit_load.assemble(ib), **csr_arrays(K))

    # 7. Hex1 theta*Laplace on the 4^3 cube (a small SIMP-style case) + adjoint oracles
    m = MeshHex.init_tensor(*(np.linspace(0, 1, 5),) * 3)
    ib = Basis(m, ElementHex1())
    theta = rng.uniform(0.01, 1.0, m.t.shape[1])
    wv = rng.standard_normal(ib.N)
    uv = rng.standard_normal(ib.N)
    K = theta_laplace.assemble(ib, theta=ib.zero_w() + theta[:, None])

    @Functional
    def a_wu(w):
        return dot(grad(w['wh']), grad(w['uh']))
    dtheta = a_wu.elemental(ib, wh=ib.interpolate(wv), uh=ib.interpolate(uv))

    def J_of(pp):
        mm = MeshHex(pp, m.t)
        bb = Basis(mm, ElementHex1())
        KK = theta_laplace.assemble(bb, theta=bb.zero_w() + theta[:, None])
        return wv @ (KK @ uv)

    h = 1e-6
    dX = np.zeros_like(m.p)
    for a in range(3):
        for q in range(m.p.shape[1]):
            pp = m.p.copy()
            pp[a, q] += h
            fp = J_of(pp)
            pp[a, q] -= 2 * h
            dX[a, q] = (fp - J_of(pp)) / (2 * h)
    # load-vector VJP: d(w^T b(f, X))/d f_e and /dX for b = f*v
    bvec = f_load.assemble(ib, f=ib.zero_w() + theta[:, None])

    def L_of(pp):
        mm = MeshHex(pp, m.t)
        bb = Basis(mm, ElementHex1())
        return wv @ f_load.assemble(bb, f=bb.zero_w() + theta[:, None])

    dXb = np.zeros_like(m.p)
    for a in range(3):
        for q in range(m.p.shape[1]):
            pp = m.p.copy()
            pp[a, q] += h
            fp = L_of(pp)
            pp[a, q] -= 2 * h
            dXb[a, q] = (fp - L_of(pp)) / (2 * h)
    save("hex1_theta_laplace", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, theta=theta, wv=wv, uv=uv, dtheta=dtheta, dX=dX,
         b=bvec, dXb=dXb, **csr_arrays(K))

    # 8. Hex1 Laplace on an unjittered 8^3 cube: rounding-noise entries
    m = MeshHex.init_tensor(*(np.linspace(0, 1, 9),) * 3)
    ib = Basis(m, ElementHex1())
    save("hex1_laplace_8", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, b=unit_load.assemble(ib), **csr_arrays(laplace.assemble(ib)))

    # 9. TetP1 Laplace on a jittered 5^3 mesh, two different bases of one mesh
    n = 5
    m = MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    m = MeshTet(p, m.t)
    ib = Basis(m, ElementTetP1())
    save("tet_p1_jitter_laplace", p=m.p, t=m.t, element_dofs=ib.element_dofs,
         X=ib.X, W=ib.W, b=unit_load.assemble(ib), **csr_arrays(laplace.assemble(ib)))

    # 10. element subset: TriP2 k*Laplace on the cells with midpoint x < 0.5,
    #     and TetP1 Laplace + load on an index subset
    m = MeshTri.init_tensor(np.linspace(0, 1, 9), np.linspace(0, 1, 9))
    ib = Basis(m, ElementTriP2(), elements=lambda x: x[0] < 0.5)
    k = rng.lognormal(0.0, 0.5, ib.nelems)
    K = k_laplace.assemble(ib, k=ib.zero_w() + k[:, None])
    save("tri_p2_subset", p=m.p, t=m.t, element_dofs=ib.element_dofs, tind=ib.tind,
         X=ib.X, W=ib.W, k=k, b=unit_load.assemble(ib), **csr_arrays(K))
    m = MeshTet.init_tensor(*(np.linspace(0, 1, 5),) * 3)
    tind = np.arange(0, m.t.shape[1], 3).astype(np.int32)
    ib = Basis(m, ElementTetP1(), elements=tind)
    save("tet_p1_subset", p=m.p, t=m.t, element_dofs=ib.element_dofs, tind=ib.tind,
         X=ib.X, W=ib.W, b=unit_load.assemble(ib), **csr_arrays(laplace.assemble(ib)))

    generic_cases()
    facet_cases()
    mixed_cases()
    vector_hex_case()
    dofs_case()
    poisson_case()

    quadrature_rules()

    with open(os.path.join(OUT, "VERSION"), "w") as f:
        f.write("scikit-fem %s, numpy %s, python %s\n"
                % (skfem.__version__, np.__version__, sys.version.split()[0]))


def quadrature_rules():
    """Every triangle (orders 1-19) and tetrahedron (orders 1-9) rule the
    reference tabulates (quadrature.py:80-2836), exactly as it returns them."""
    from skfem.quadrature import get_quadrature_tet, get_quadrature_tri
    rules = {}
    for o in range(1, 20):
        X, W = get_quadrature_tri(o)
        rules["tri%d_X" % o], rules["tri%d_W" % o] = X, W
    for o in range(1, 10):
        X, W = get_quadrature_tet(o)
        rules["tet%d_X" % o], rules["tet%d_W" % o] = X, W
    save("quadrature_rules", **rules)


def generic_cases():
    """Forms outside the isotropic coefficient channels: anisotropic and
    advection terms, w.x / w.h, per-point coefficients, interpolated DOF
    vectors, numpy functions, Functional; with the reference's interpolate
    output and global coordinates."""
    from skfem.helpers import ddot, div, sym_grad
    rng = np.random.default_rng(20261204)

    @BilinearForm
    def aniso_adv(u, v, w):
        x = w.x
        return ((1.0 + x[0] * x[1]) * grad(u)[0] * grad(v)[0] + 0.5 * grad(u)[1] * grad(v)[1]
                + (x[0] * grad(u)[0] + 2.0 * grad(u)[1]) * v + w.h * u * v)

    @BilinearForm
    def qp_coef(u, v, w):
        return w.c * dot(grad(u), grad(v)) + w.c ** 2 * u * v

    @BilinearForm
    def newton(u, v, w):
        s = w['s']
        return (1.0 + s ** 2) * dot(grad(u), grad(v)) + 2.0 * s * u * dot(grad(s), grad(v))

    @LinearForm
    def trig_load(v, w):
        return np.sin(np.pi * w.x[0]) * np.cos(np.pi * w.x[1]) * v

    @LinearForm
    def newton_res(v, w):
        s = w['s']
        return (1.0 + s ** 2) * dot(grad(s), grad(v)) - w.x[0] * v

    @Functional
    def energy(w):
        s = w['s']
        return s ** 2 + dot(grad(s), grad(s)) + w.x[0] * w.h

    # TriP2 on a jittered 6x6 square
    n = 6
    m = MeshTri.init_tensor(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1))
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(2, int(inner.sum())))
    m = MeshTri(p, m.t)
    ib = Basis(m, ElementTriP2())
    c = rng.uniform(0.5, 2.0, (ib.nelems, ib.X.shape[1]))
    s = rng.standard_normal(ib.N)
    sf = ib.interpolate(s)
    K1 = aniso_adv.assemble(ib)
    K2 = qp_coef.assemble(ib, c=c)
    K3 = newton.assemble(ib, s=s)
    save("tri_p2_generic", p=m.p, t=m.t, element_dofs=ib.element_dofs, X=ib.X, W=ib.W,
         c=c, s=s, s_value=np.asarray(sf), s_grad=sf.grad,
         x=np.asarray(ib.global_coordinates()), h=np.asarray(ib.mesh_parameters()),
         b_trig=trig_load.assemble(ib), b_newton=newton_res.assemble(ib, s=s),
         e_energy=energy.elemental(ib, s=s), f_energy=np.float64(energy.assemble(ib, s=s)),
         **{k + "_aniso": v for k, v in csr_arrays(K1).items()},
         **{k + "_qp": v for k, v in csr_arrays(K2).items()},
         **{k + "_newton": v for k, v in csr_arrays(K3).items()})

    # TetP1 (4-point rule) and Hex1 (64 points) on jittered meshes
    for name, mesh_cls, elem, n in (("tet_p1_generic", MeshTet, ElementTetP1(), 3),
                                    ("hex1_generic", MeshHex, ElementHex1(), 3)):
        m = mesh_cls.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
        p = m.p.copy()
        inner = jitter(m, rng, 0.2)
        p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
        m = mesh_cls(p, m.t)
        ib = Basis(m, elem)
        c = rng.uniform(0.5, 2.0, (ib.nelems, ib.X.shape[1]))
        s = rng.standard_normal(ib.N)
        sf = ib.interpolate(s)

        @BilinearForm
        def aniso3(u, v, w):
            x = w.x
            return ((1.0 + x[2]) * grad(u)[0] * grad(v)[0] + grad(u)[1] * grad(v)[1]
                    + 0.25 * grad(u)[2] * grad(v)[2] + x[1] * grad(u)[2] * v)

        save(name, p=m.p, t=m.t, element_dofs=ib.element_dofs, X=ib.X, W=ib.W, c=c, s=s,
             s_value=np.asarray(sf), s_grad=sf.grad, x=np.asarray(ib.global_coordinates()),
             h=np.asarray(ib.mesh_parameters()),
             b_newton=newton_res.assemble(ib, s=s), e_energy=energy.elemental(ib, s=s),
             f_energy=np.float64(energy.assemble(ib, s=s)),
             **{k + "_aniso": v for k, v in csr_arrays(aniso3.assemble(ib)).items()},
             **{k + "_qp": v for k, v in csr_arrays(qp_coef.assemble(ib, c=c)).items()},
             **{k + "_newton": v for k, v in csr_arrays(newton.assemble(ib, s=s)).items()})

    # vector TetP2: elasticity plus a convection-like term with an
    # interpolated vector field d
    n = 2
    m = MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    m = MeshTet(p, m.t)
    ib = Basis(m, ElementVector(ElementTetP2()), intorder=4)
    d = rng.standard_normal(ib.N)
    df = ib.interpolate(d)

    @BilinearForm
    def vec_conv(u, v, w):
        return (ddot(sym_grad(u), sym_grad(v)) + div(u) * div(v)
                + dot(np.einsum('ij...,j...->i...', grad(u), w['d']), v))

    @Functional
    def vec_energy(w):
        return ddot(grad(w['d']), grad(w['d'])) + dot(w['d'], w['d'])

    save("tet_p2_vec_generic", p=m.p, t=m.t, element_dofs=ib.element_dofs, X=ib.X, W=ib.W,
         d=d, d_value=np.asarray(df), d_grad=df.grad,
         e_energy=vec_energy.elemental(ib, d=d), f_energy=np.float64(vec_energy.assemble(ib, d=d)),
         **{k + "_conv": v for k, v in csr_arrays(vec_conv.assemble(ib, d=d)).items()})


def facet_cases():
    """FacetBasis (boundary, interior with side 0/1, callable subsets) on
    affine simplices: boundary mass, Robin / normal-derivative terms,
    Neumann loads with w.n / w.x / w.h, Functional, interpolate; plus the
    reference's line rules (FacetBasis quadrature of triangle meshes)."""
    from skfem import FacetBasis
    from skfem.quadrature import get_quadrature_line
    rng = np.random.default_rng(20261205)

    @BilinearForm
    def robin(u, v, w):
        return (1.0 + w.x[0]) * u * v + dot(w.n, grad(u)) * v

    @LinearForm
    def neumann(v, w):
        return dot(w.n, w.x) * v + w.h * v

    @Functional
    def length(w):
        return 1.0 + 0.0 * w.x[0]

    @Functional
    def s_energy(w):
        return w['s'] ** 2 + dot(w.n, grad(w['s']))

    def facet_arrays(fb, s, prefix=""):
        sf = fb.interpolate(s)
        out = dict(find=fb.find, tind=fb.tind, X=fb.X, W=fb.W,
                   x=np.asarray(fb.global_coordinates()), h=np.asarray(fb.mesh_parameters()),
                   n=np.asarray(fb.normals), s_value=np.asarray(sf), s_grad=sf.grad,
                   b_neumann=neumann.assemble(fb), e_length=length.elemental(fb),
                   f_length=np.float64(length.assemble(fb)),
                   e_energy=s_energy.elemental(fb, s=s),
                   f_energy=np.float64(s_energy.assemble(fb, s=s)))
        out.update({k + "_mass": v for k, v in csr_arrays(mass.assemble(fb)).items()})
        out.update({k + "_robin": v for k, v in csr_arrays(robin.assemble(fb)).items()})
        return {prefix + k: v for k, v in out.items()}

    for name, mesh_cls, elem, shape in (
            ("tri_p1_facet", MeshTri, ElementTriP1(), (7, 6)),
            ("tri_p2_facet", MeshTri, ElementTriP2(), (5, 5)),
            ("tet_p1_facet", MeshTet, ElementTetP1(), (4, 4, 4)),
            ("tet_p2_facet", MeshTet, ElementTetP2(), (3, 3, 3))):
        m = mesh_cls.init_tensor(*[np.linspace(0, 1, k) for k in shape])
        p = m.p.copy()
        inner = jitter(m, rng, 0.2)
        hh = 1.0 / (max(shape) - 1)
        p[:, inner] += rng.uniform(-0.2 * hh, 0.2 * hh, size=(p.shape[0], int(inner.sum())))
        m = mesh_cls(p, m.t)
        s = rng.standard_normal(Basis(m, elem).N)
        arrs = dict(p=m.p, t=m.t, facets=m.facets, f2t=m.f2t, t2f=m.t2f, s=s)
        arrs.update(facet_arrays(FacetBasis(m, elem), s))
        interior = np.nonzero(m.f2t[1] >= 0)[0].astype(np.int32)
        arrs.update(facet_arrays(FacetBasis(m, elem, facets=interior, side=0), s, "in0_"))
        arrs.update(facet_arrays(FacetBasis(m, elem, facets=interior, side=1), s, "in1_"))
        arrs.update(facet_arrays(FacetBasis(m, elem, facets=lambda x: x[1] < 0.3), s, "cb_"))
        save(name, **arrs)

    # vector TetP2: boundary mass and a traction load
    m = MeshTet.init_tensor(*(np.linspace(0, 1, 3),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.1, 0.1, size=(3, int(inner.sum())))
    m = MeshTet(p, m.t)
    fb = FacetBasis(m, ElementVector(ElementTetP2()))

    @BilinearForm
    def vmass(u, v, w):
        return dot(u, v)

    @LinearForm
    def traction(v, w):
        return (1.0 + w.x[2]) * dot(w.n, v)

    save("tet_p2_vec_facet", p=m.p, t=m.t, X=fb.X, W=fb.W, find=fb.find,
         b_traction=traction.assemble(fb),
         **{k + "_vmass": v for k, v in csr_arrays(vmass.assemble(fb)).items()})

    rules = {}
    for o in range(1, 11):
        X, W = get_quadrature_line(o)
        rules["line%d_X" % o], rules["line%d_W" % o] = X, W
    save("line_rules", **rules)
    hex_facet_case()


def hex_facet_case():
    """FacetBasis on a jittered Hex1 mesh: quadrilateral facets, Newton
    iterated reference points, normals of the isoparametric cells."""
    from skfem import FacetBasis
    rng = np.random.default_rng(20261206)

    @BilinearForm
    def robin(u, v, w):
        return (1.0 + w.x[0]) * u * v + dot(w.n, grad(u)) * v

    @LinearForm
    def neumann(v, w):
        return dot(w.n, w.x) * v + w.h * v

    @Functional
    def length(w):
        return 1.0 + 0.0 * w.x[0]

    @Functional
    def s_energy(w):
        return w['s'] ** 2 + dot(w.n, grad(w['s']))

    n = 3
    m = MeshHex.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
    m = MeshHex(p, m.t)
    s = rng.standard_normal(Basis(m, ElementHex1()).N)
    arrs = dict(p=m.p, t=m.t, facets=m.facets, f2t=m.f2t, t2f=m.t2f, s=s)
    interior = np.nonzero(m.f2t[1] >= 0)[0].astype(np.int32)
    for pre, kw in (("", {}), ("in0_", dict(facets=interior, side=0)),
                    ("in1_", dict(facets=interior, side=1)),
                    ("cb_", dict(facets=lambda x: x[1] < 0.3))):
        fb = FacetBasis(m, ElementHex1(), **kw)
        sf = fb.interpolate(s)
        out = dict(find=fb.find, tind=fb.tind, X=fb.X, W=fb.W,
                   x=np.asarray(fb.global_coordinates()), h=np.asarray(fb.mesh_parameters()),
                   n=np.asarray(fb.normals), s_value=np.asarray(sf), s_grad=sf.grad,
                   b_neumann=neumann.assemble(fb), e_length=length.elemental(fb),
                   f_length=np.float64(length.assemble(fb)),
                   e_energy=s_energy.elemental(fb, s=s),
                   f_energy=np.float64(s_energy.assemble(fb, s=s)))
        out.update({k + "_mass": v for k, v in csr_arrays(mass.assemble(fb)).items()})
        out.update({k + "_robin": v for k, v in csr_arrays(robin.assemble(fb)).items()})
        arrs.update({pre + k: v for k, v in out.items()})
    save("hex1_facet", **arrs)


def mixed_cases():
    """BilinearForm.assemble(ubasis, vbasis) with different trial and test
    bases on one mesh (mixed methods): the Stokes divergence block and its
    transpose, a P2 x P1 coupling with an interpolated trial-side field."""
    from skfem.helpers import div
    rng = np.random.default_rng(20261207)

    @BilinearForm
    def bdiv(u, v, w):
        return div(u) * v

    @BilinearForm
    def bdiv_t(u, v, w):
        return u * div(v)

    @BilinearForm
    def coupling(u, v, w):
        return (1.0 + w['s'] ** 2) * u * v + dot(grad(u), grad(v)) + w.x[0] * grad(u)[0] * v

    n = 5
    m = MeshTri.init_tensor(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1))
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(2, int(inner.sum())))
    m = MeshTri(p, m.t)
    ub = Basis(m, ElementVector(ElementTriP2()))
    pb = Basis(m, ElementTriP1(), intorder=4)
    sb = Basis(m, ElementTriP2())
    s = rng.standard_normal(sb.N)
    save("tri_mixed", p=m.p, t=m.t, s=s,
         **{k + "_bdiv": v for k, v in csr_arrays(bdiv.assemble(ub, pb)).items()},
         **{k + "_bdivt": v for k, v in csr_arrays(bdiv_t.assemble(pb, ub)).items()},
         **{k + "_coupling": v for k, v in csr_arrays(coupling.assemble(sb, pb, s=s)).items()})
    m = MeshTet.init_tensor(*(np.linspace(0, 1, 3),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.1, 0.1, size=(3, int(inner.sum())))
    m = MeshTet(p, m.t)
    ub = Basis(m, ElementVector(ElementTetP2()))
    pb = Basis(m, ElementTetP1(), intorder=4)
    save("tet_mixed", p=m.p, t=m.t,
         **{k + "_bdiv": v for k, v in csr_arrays(bdiv.assemble(ub, pb)).items()})


def vector_hex_case():
    """ElementVector(ElementHex1): linear elasticity on a jittered Hex1 mesh,
    a traction load on its boundary, the interpolated displacement."""
    from skfem import FacetBasis
    rng = np.random.default_rng(20261208)
    n = 2
    m = MeshHex.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    p = m.p.copy()
    inner = jitter(m, rng, 0.2)
    p[:, inner] += rng.uniform(-0.1, 0.1, size=(3, int(inner.sum())))
    m = MeshHex(p, m.t)
    e = ElementVector(ElementHex1())
    ib = Basis(m, e)
    fb = FacetBasis(m, e)
    d = rng.standard_normal(ib.N)
    df = ib.interpolate(d)

    @LinearForm
    def traction(v, w):
        return (1.0 + w.x[2]) * dot(w.n, v)

    save("hex1_vec", p=m.p, t=m.t, element_dofs=ib.element_dofs, d=d, d_value=np.asarray(df),
         d_grad=df.grad, b_traction=traction.assemble(fb),
         **{k + "_elast": v for k, v in csr_arrays(linear_elasticity(1.0, 0.5).assemble(ib)).items()})


def dofs_case():
    """Basis.get_dofs (abstract_basis.py:125-260): boundary DOFs, DOFs on the
    facets a callable selects, DOFs of the cells a callable selects."""
    out = {}
    meshes = {"tri": MeshTri.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 4)),
              "tet": MeshTet.init_tensor(*(np.linspace(0, 1, 4),) * 3),
              "hex": MeshHex.init_tensor(*(np.linspace(0, 1, 4),) * 3)}
    elems = {"tri": (ElementTriP1, ElementTriP2), "tet": (ElementTetP1, ElementTetP2),
             "hex": (ElementHex1,)}
    for kind, m in meshes.items():
        for E in elems[kind]:
            for vec in (0, 1):
                b = Basis(m, ElementVector(E()) if vec else E())
                key = "%s_%s_%d" % (kind, E.__name__, vec)
                out[key + "_boundary"] = b.get_dofs().flatten()
                out[key + "_y0"] = b.get_dofs(lambda x: np.isclose(x[1], 0)).flatten()
                out[key + "_left"] = b.get_dofs(elements=lambda x: x[0] < 0.5).flatten()
    save("get_dofs", **out)


def poisson_case():
    """A whole solve as users write it (docs/examples/ex01.py): -lap u = 1 on
    the unit square, u = 0 on the boundary, condense and spsolve."""
    from skfem import condense, solve
    m = MeshTri.init_tensor(np.linspace(0, 1, 33), np.linspace(0, 1, 33))
    b = Basis(m, ElementTriP2())
    A = laplace.assemble(b)
    f = unit_load.assemble(b)
    u = solve(*condense(A, f, D=b.get_dofs()))
    save("poisson_tri_p2", u=u)


def edge_cases():
    """Meshes at the edges of the path: a node no cell uses (the reference
    numbers DOFs up to max(t), mesh.py nvertices), a single cell, an empty
    element subset (cell_basis.py:94-99), for TetP1 k*laplace + mass, the
    unit load and TriP2 Laplace."""
    out = {}
    m = MeshTet()
    p = np.hstack([m.p, [[2.0], [2.0], [2.0]]])
    k9 = np.linspace(0.5, 1.5, m.t.shape[1])
    for name, mesh, elements in (("unused_node", MeshTet(p, m.t), None),
                                 ("single", MeshTet(m.p[:, m.t[:, 0]],
                                                    np.arange(4).reshape(4, 1)), None),
                                 ("empty_subset", m, np.array([], dtype=np.int64))):
        b = Basis(mesh, ElementTetP1(), elements=elements)
        k = np.ones(b.nelems) if name != "unused_node" else k9
        K = k_laplace_mass.assemble(b, k=b.zero_w() + k[:, None])
        f = unit_load.assemble(b)
        out[name + "_p"] = mesh.p
        out[name + "_t"] = mesh.t
        out[name + "_k"] = k
        out[name + "_N"] = np.array(b.N)
        for key, val in csr_arrays(K).items():
            out[name + "_" + key] = val
        out[name + "_b"] = f
    mt = MeshTri()
    b = Basis(MeshTri(mt.p[:, mt.t[:, 0]], np.arange(3).reshape(3, 1)), ElementTriP2())
    for key, val in csr_arrays(laplace.assemble(b)).items():
        out["tri2_single_" + key] = val
    save("edge_cases", **out)


def doflocs_case():
    """Basis.doflocs (abstract_basis.py:60-71) on jittered meshes."""
    rng = np.random.default_rng(11)
    out = {}
    meshes = {"tri": MeshTri.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 4)),
              "tet": MeshTet.init_tensor(*(np.linspace(0, 1, 4),) * 3),
              "hex": MeshHex.init_tensor(*(np.linspace(0, 1, 4),) * 3)}
    elems = {"tri": (ElementTriP1, ElementTriP2), "tet": (ElementTetP1, ElementTetP2),
             "hex": (ElementHex1,)}
    for kind, m0 in meshes.items():
        p = m0.p + rng.uniform(-0.05, 0.05, m0.p.shape)
        m = type(m0)(p, m0.t)
        out[kind + "_p"] = m.p
        out[kind + "_t"] = m.t
        for E in elems[kind]:
            for vec in (0, 1):
                b = Basis(m, ElementVector(E()) if vec else E())
                out["%s_%s_%d" % (kind, E.__name__, vec)] = b.doflocs
    save("doflocs", **out)


def _digest(a):
    import hashlib
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(),
                         dtype=np.uint8).copy()


def config_cases():
    """The benchmark configurations at the sizes the GPU tests assemble them
    (bench.py's own seeded workloads), run through scikit-fem: per case the
    nnz, SHA-256 digests of indptr and indices (int32) and the Frobenius norm
    and sum of the values.  The matrices are too large to store; the digests
    pin the reference's exact CSR pattern, which the GPU reproduces by
    replaying numpy's arithmetic of this platform (noise-level local entries
    that come out exactly 0.0 are dropped by eliminate_zeros)."""
    root = os.path.dirname(os.path.dirname(OUT))
    for q in (root, os.path.join(root, "scikit-fem_gb300")):
        if q not in sys.path:
            sys.path.insert(0, q)
    import bench as B

    out = {}

    def record(name, K, **extra):
        K = K.tocsr()
        out[name + "__nnz"] = np.array(K.nnz)
        out[name + "__indptr"] = _digest(K.indptr.astype(np.int32))
        out[name + "__indices"] = _digest(K.indices.astype(np.int32))
        out[name + "__fro"] = np.array(np.linalg.norm(K.data))
        out[name + "__sum"] = np.array(K.data.sum())
        for k, v in extra.items():
            out[name + "__" + k] = v
        print(name, K.nnz)

    # TriP1 Laplace + unit load, 256 x 256 squares
    m = MeshTri.init_tensor(*(np.linspace(0, 1, 257),) * 2)
    ib = Basis(m, ElementTriP1())
    record("tri_p1_256", laplace.assemble(ib), b=unit_load.assemble(ib))
    # TetP1 k*Laplace + mass, the 61^3-node sample of the 101^3 workload
    _, k = B.build_workload(61)
    m = MeshTet.init_tensor(*(np.linspace(0, 1, 61),) * 3)
    ib = Basis(m, ElementTetP1())
    record("tet_p1_61", k_laplace_mass.assemble(ib, k=ib.zero_w() + k[:, None]))
    # Hex1 theta*Laplace, 64^3 cells
    _, theta, _, _ = B.hex_cube_workload(64)
    m = MeshHex.init_tensor(*(np.linspace(0, 1, 65),) * 3)
    ib = Basis(m, ElementHex1())
    record("hex1_64", theta_laplace.assemble(ib, theta=ib.zero_w() + theta[:, None]))
    # vector TetP2 elasticity, jittered 16^3 cells, intorder 4
    fm = B.jittered_tet_cube(16)
    ib = Basis(MeshTet(fm.p, fm.t), ElementVector(ElementTetP2()), intorder=4)
    record("vec_tet_p2_16", linear_elasticity(1.0, 0.5).assemble(ib))
    # four meshes of the batched TriP2 workload
    meshes, ks = B.trip2_batch(4)
    for i, (fmm, kk) in enumerate(zip(meshes, ks)):
        ib = Basis(MeshTri(fmm.p, fmm.t), ElementTriP2())
        record("trip2_batch_%d" % i, k_laplace.assemble(ib, k=ib.zero_w() + kk[:, None]))
    np.savez_compressed(os.path.join(OUT, "config_patterns.npz"), **out)


def capacity_cases():
    """Rows of high-valence DOFs at the pattern build's candidate limit:
    vector TetP2 elasticity on the double cone of 273 ring vertices (546
    cells share the origin) and TriP2 k*Laplace on a fan of 1,500 triangles,
    run through scikit-fem -- nnz, digests of indptr / indices, Frobenius
    norm and sum, as config_cases records them."""
    sys.path.insert(0, os.path.dirname(OUT))
    from _util import double_cone_arrays, fan_arrays, fan_coefficient

    out = {}

    def record(name, K):
        # the whole pattern too: on these symmetric meshes the oracle's
        # exact zeros differ from the reference's in a few noise entries
        K = K.tocsr()
        out[name + "__nnz"] = np.array(K.nnz)
        out[name + "__indptr"] = _digest(K.indptr.astype(np.int32))
        out[name + "__indices"] = _digest(K.indices.astype(np.int32))
        out[name + "__fro"] = np.array(np.linalg.norm(K.data))
        out[name + "__sum"] = np.array(K.data.sum())
        out[name + "__pattern_indptr"] = K.indptr.astype(np.int32)
        out[name + "__pattern_indices"] = K.indices.astype(np.int32)
        print(name, K.nnz)

    p, t = double_cone_arrays(273)
    ib = Basis(MeshTet(p, t), ElementVector(ElementTetP2()))
    record("cone_273_vec_tet_p2", linear_elasticity(1.0, 0.5).assemble(ib))
    p, t = fan_arrays(1500)
    ib = Basis(MeshTri(p, t), ElementTriP2())
    k = fan_coefficient(t.shape[1])
    record("fan_1500_tri_p2", k_laplace.assemble(ib, k=ib.zero_w() + k[:, None]))
    np.savez_compressed(os.path.join(OUT, "capacity_patterns.npz"), **out)


def coo_cases():
    """COOData / Form.elemental / Form.block / asm(to=...) results of
    scikit-fem (coo_data.py, form.py:53-89, assembly/__init__.py:69-97)."""
    from skfem import FacetBasis, asm
    from skfem.helpers import dot as hdot
    out = {}
    m = MeshTri.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 4))
    ib = Basis(m, ElementTriP1())
    A = laplace.elemental(ib)
    out["lap_indices"], out["lap_data"] = A.indices, A.data
    out["lap_shape"], out["lap_local_shape"] = np.array(A.shape), np.array(A.local_shape)
    out["lap_tolocal"] = A.tolocal()
    K = A.tocsr()
    out["lap_indptr"], out["lap_csr_indices"], out["lap_csr_data"] = K.indptr, K.indices, K.data
    b = unit_load.elemental(ib)
    out["load_indices"], out["load_data"], out["load_array"] = b.indices, b.data, b.toarray()
    # mass matrices inverted cell by cell, then assembled
    out["mass_inverse"] = mass.coo_data(ib).inverse().tocsr().toarray()
    # trial P2 / test P1 pair
    pb = Basis(m, ElementTriP2())
    ib2 = Basis(m, ElementTriP1(), intorder=4)     # the trial basis's quadrature

    @BilinearForm
    def mixed(u, v, w):
        return u.grad[0] * v + 0.5 * u * v.grad[1]
    C = mixed.elemental(pb, ib2)
    out["mixed_indices"], out["mixed_data"] = C.indices, C.data
    out["mixed_shape"], out["mixed_local_shape"] = np.array(C.shape), np.array(C.local_shape)
    # asm over lists of bases (element subsets), summed; and a custom reducer
    b1 = Basis(m, ElementTriP1(), elements=lambda x: x[0] < 0.5)
    b2 = Basis(m, ElementTriP1(), elements=lambda x: x[0] >= 0.5)
    S = asm(laplace, [b1, b2])
    out["asm_sum_indptr"], out["asm_sum_indices"], out["asm_sum_data"] = S.indptr, S.indices, S.data
    parts = asm(laplace, [b1, b2], to=list)
    out["asm_to_list_0"] = parts[0].todefault().toarray()
    out["asm_to_list_1"] = parts[1].todefault().toarray()
    out["asm_load_sum"] = asm(unit_load, [b1, b2])

    @BilinearForm
    def with_idx(u, v, w):
        return (1.0 + w.idx[0]) * u * v
    out["asm_idx"] = asm(with_idx, [b1, b2]).toarray()
    # blocks of a form written on a product space
    @BilinearForm
    def prod(u1, u2, v1, v2, w):
        return hdot(grad(u1), grad(v1)) + 2.0 * u2 * v2 + u1 * v2
    for i in (0, 1):
        for j in (0, 1):
            out["block_%d%d" % (i, j)] = asm(prod.block(i, j), ib).toarray()
    # facet matrices summed per cell
    fb = FacetBasis(m, ElementTriP1())
    F_ = mass.elemental(fb)
    out["facet_tolocal"] = F_.tolocal(fb)
    np.savez_compressed(os.path.join(OUT, "coo_api.npz"), **out)
    print("coo_api", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if sys.argv[1:] == ["--coo"]:
        coo_cases()
    elif sys.argv[1:] == ["--configs"]:
        config_cases()
    elif sys.argv[1:] == ["--capacity"]:
        capacity_cases()
    elif sys.argv[1:] == ["--quadrature"]:
        quadrature_rules()
    elif sys.argv[1:] == ["--doflocs"]:
        doflocs_case()
    elif sys.argv[1:] == ["--edge"]:
        edge_cases()
    elif sys.argv[1:] == ["--generic"]:
        generic_cases()
    elif sys.argv[1:] == ["--facet"]:
        facet_cases()
    elif sys.argv[1:] == ["--hex-facet"]:
        hex_facet_case()
    elif sys.argv[1:] == ["--mixed"]:
        mixed_cases()
    elif sys.argv[1:] == ["--vector-hex"]:
        vector_hex_case()
    elif sys.argv[1:] == ["--dofs"]:
        dofs_case()
    elif sys.argv[1:] == ["--poisson"]:
        poisson_case()
    else:
        main()
