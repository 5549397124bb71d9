"""skfem/models/elasticity.py:7-53."""
from ..form import BilinearForm
from ..helpers import ddot, eye, sym_grad, trace


def lame_parameters(E, nu):
    return E * nu / ((1. + nu) * (1. - 2. * nu)), E / (2. * (1. + nu))


def linear_stress(Lambda=1., Mu=1.):
    def C(T):
        return 2. * Mu * T + Lambda * eye(trace(T), T.shape[0])
    return C


def linear_elasticity(Lambda=1., Mu=1.):
    C = linear_stress(Lambda, Mu)

    @BilinearForm
    def weakform(u, v, w):
        return ddot(C(sym_grad(u)), sym_grad(v))

    return weakform
