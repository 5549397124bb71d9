"""DiscreteField: a function's values (and derivatives) at quadrature points.

Mirrors skfem/element/discrete_field.py:7-120 -- an ndarray of values with
``grad`` (and the reference's other derivative slots, unused by the H1
elements here) as attributes.  A field produced by ``CellBasis.interpolate``
also keeps its device copy, quantity-major (nquant, nelems, nq), so that
passing it back into a form does not upload it again.
"""

import warnings

import numpy as np

__all__ = ["DiscreteField"]


class DiscreteField(np.ndarray):

    _extra_attrs = ("grad", "div", "curl", "hess", "grad3", "grad4", "grad5", "grad6")

    def __new__(cls, value=None, grad=None, div=None, curl=None, hess=None, grad3=None,
                grad4=None, grad5=None, grad6=None):
        if value is None:
            value = np.array([0])
        obj = np.asarray(value).view(cls)
        obj.grad, obj.div, obj.curl, obj.hess = grad, div, curl, hess
        obj.grad3, obj.grad4, obj.grad5, obj.grad6 = grad3, grad4, grad5, grad6
        obj._dev = None
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        for a in self._extra_attrs:
            setattr(self, a, getattr(obj, a, None))
        self._dev = None

    def __getitem__(self, key):
        return np.array(self)[key]

    def __array_wrap__(self, out_arr, context=None, return_scalar=False):
        return np.array(out_arr)

    def get(self, n):
        if n == 0:
            return np.array(self)
        return getattr(self, self._extra_attrs[n - 1])

    @property
    def astuple(self):
        return tuple(self.get(i) for i in range(len(self._extra_attrs) + 1))

    @property
    def value(self):
        warnings.warn("Writing 'u.value' is unnecessary and can be replaced by 'u'.",
                      DeprecationWarning)
        return np.array(self)

    def zeros(self):
        return DiscreteField(*tuple(None if c is None else np.zeros_like(c)
                                    for c in self.astuple))
