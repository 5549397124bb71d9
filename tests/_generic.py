"""Forms of the generic-kernel fixtures (tests/golden/make_golden.py,
generic_cases) written with this package's helpers, and the reference's
COO -> CSR steps for comparing replayed local matrices with the fixtures."""
import numpy as np
import scipy.sparse as sp

import skfem_gb300 as F
from skfem_gb300.helpers import ddot, div, dot, grad, sym_grad


@F.BilinearForm
def aniso_adv(u, v, w):
    x = w.x
    return ((1.0 + x[0] * x[1]) * grad(u)[0] * grad(v)[0] + 0.5 * grad(u)[1] * grad(v)[1]
            + (x[0] * grad(u)[0] + 2.0 * grad(u)[1]) * v + w.h * u * v)


@F.BilinearForm
def aniso3(u, v, w):
    x = w.x
    return ((1.0 + x[2]) * grad(u)[0] * grad(v)[0] + grad(u)[1] * grad(v)[1]
            + 0.25 * grad(u)[2] * grad(v)[2] + x[1] * grad(u)[2] * v)


@F.BilinearForm
def qp_coef(u, v, w):
    return w.c * dot(grad(u), grad(v)) + w.c ** 2 * u * v


@F.BilinearForm
def newton(u, v, w):
    s = w['s']
    return (1.0 + s ** 2) * dot(grad(u), grad(v)) + 2.0 * s * u * dot(grad(s), grad(v))


@F.LinearForm
def trig_load(v, w):
    return np.sin(np.pi * w.x[0]) * np.cos(np.pi * w.x[1]) * v


@F.LinearForm
def newton_res(v, w):
    s = w['s']
    return (1.0 + s ** 2) * dot(grad(s), grad(v)) - w.x[0] * v


@F.Functional
def energy(w):
    s = w['s']
    return s ** 2 + dot(grad(s), grad(s)) + w.x[0] * w.h


@F.BilinearForm
def vec_conv(u, v, w):
    return (ddot(sym_grad(u), sym_grad(v)) + div(u) * div(v)
            + dot(np.einsum('ij...,j...->i...', grad(u), w['d']), v))


@F.Functional
def vec_energy(w):
    return ddot(grad(w['d']), grad(w['d'])) + dot(w['d'], w['d'])


# (fixture, element, bilinear forms {suffix: (form, kwargs names)}, has 2-D trig load)
SCALAR_CASES = [
    ("tri_p2_generic", F.ElementTriP2, {"aniso": aniso_adv}),
    ("tet_p1_generic", F.ElementTetP1, {"aniso": aniso3}),
    ("hex1_generic", F.ElementHex1, {"aniso": aniso3}),
]


def reference_csr(local, element_dofs, n):
    """bilinear_form.py:84-128 + coo_data.py:27-36 on local matrices
    local[e, i, j] (row i = test function): data[j, i, e] in C order, COO,
    eliminate_zeros, tocsr."""
    nt, nv, nu = local.shape
    data = np.transpose(local, (2, 1, 0)).reshape(-1)
    rows = np.zeros(nu * nv * nt, dtype=np.int32)
    cols = np.zeros(nu * nv * nt, dtype=np.int32)
    for j in range(nu):
        for i in range(nv):
            ixs = slice(nt * (nv * j + i), nt * (nv * j + i + 1))
            rows[ixs] = element_dofs[i]
            cols[ixs] = element_dofs[j]
    K = sp.coo_matrix((data, (rows, cols)), shape=(n, n))
    K.eliminate_zeros()
    return K.tocsr()


def reference_vector(local, element_dofs, n):
    """linear_form.py:18-46 + coo_data.py:102-108 on local vectors local[e, i]."""
    nt, nv = local.shape
    data = np.transpose(local).reshape(-1)
    rows = np.concatenate([element_dofs[i] for i in range(nv)]).astype(np.int32)
    return sp.coo_matrix((data, (rows, np.zeros_like(rows))), shape=(n, 1)).toarray().T[0]


def fixture_csr(g, suffix):
    return (g["indptr_" + suffix], g["indices_" + suffix], g["data_" + suffix])


@F.BilinearForm
def bdiv(u, v, w):
    return div(u) * v


@F.BilinearForm
def bdiv_t(u, v, w):
    return u * div(v)


@F.BilinearForm
def coupling(u, v, w):
    return (1.0 + w['s'] ** 2) * u * v + dot(grad(u), grad(v)) + w.x[0] * grad(u)[0] * v
