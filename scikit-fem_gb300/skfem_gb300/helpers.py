"""Form helpers with the reference's semantics (skfem/helpers.py): they act
on the symbolic fields the tracer passes to forms, through numpy einsum on
object arrays exactly as the reference's versions act on its arrays."""

import numpy as np

__all__ = ["grad", "div", "dot", "ddot", "dddot", "sym_grad", "transpose", "trace", "eye",
           "identity", "mul", "prod", "inner", "d"]


def grad(u):                       # helpers.py:22-24
    return u.grad


d = grad


def div(u):                        # helpers.py:27-37 (vector fields)
    return np.einsum("ii...", u.grad)


def dot(u, v):                     # helpers.py:108-110
    return np.einsum("i...,i...", u, v)


def ddot(u, v):                    # helpers.py:113-115
    return np.einsum("ij...,ij...", u, v)


def dddot(u, v):                   # helpers.py:118-120
    return np.einsum("ijk...,ijk...", u, v)


def prod(u, v, w=None):            # helpers.py:123-129
    if w is None:
        return np.einsum("i...,j...->ij...", u, v)
    return np.einsum("i...,j...,k...->ijk...", u, v, w)


def mul(A, x):                     # helpers.py:132-134
    return np.einsum("ij...,j...->i...", A, x)


def trace(T):                      # helpers.py:137-139
    return np.einsum("ii...", T)


def transpose(T):                  # helpers.py:142-144
    return np.einsum("ij...->ji...", T)


def eye(w, n):                     # helpers.py:147-150
    return np.array([[w if i == j else 0. * w for i in range(n)] for j in range(n)])


def identity(w, N=None):
    if N is None:
        N = np.shape(w)[0] if np.ndim(w) > 0 else None
        if N is None:
            raise ValueError("Cannot deduce the size of the identity matrix. "
                             "Give an explicit keyword argument N.")
    return eye(1.0, N)


def sym_grad(u):                   # helpers.py:71-73
    return .5 * (u.grad + transpose(u.grad))


def inner(u, v):                   # helpers.py:93-105
    nd = np.ndim(u)
    if nd == 0:
        return u * v
    if nd == 1:
        return dot(u, v)
    if nd == 2:
        return ddot(u, v)
    raise NotImplementedError
