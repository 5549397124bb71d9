"""Differentiable assembly: J = w^T K(coef, X) u and J = w^T b(coef, X).

The reference has no derivative of an assembled operator with respect to its
coefficients or the mesh (skfem/autodiff/__init__.py:124-213 differentiates a
nonlinear form with respect to the solution field only).  These functions
wrap the CUDA adjoint kernels (fem_bilinear_vjp / fem_linear_vjp) in a
``torch.autograd.Function``: the forward pass assembles on the device, the
backward pass recomputes each cell's geometry and returns
  d J / d coefficient field (per element),  d J / d X (node coordinates),
  d J / d w = K u,  d J / d u = K^T w.
"""

import ctypes

import torch

from . import _native as N
from .form import BilinearForm, LinearForm, _Coefficients

__all__ = ["assemble_vjp", "assemble_linear_vjp"]


def _vertex_incidence(basis):
    h = getattr(basis, "_vinc", None)
    if h is None:
        hv = ctypes.c_void_p()
        N.check(N.lib().fem_vertex_incidence_build(N.byref(basis.c_mesh), ctypes.byref(hv),
                                                   N.stream_ptr()))
        h = N.Pattern(hv.value)
        basis._vinc = h
    return h


def _mesh_with(basis, X):
    m = N.FemMesh()
    ctypes.memmove(ctypes.addressof(m), ctypes.addressof(basis.c_mesh), ctypes.sizeof(m))
    if X is not None:
        m.p = X.data_ptr()
    return m


def _channel_fields(ch):
    """{channel: field name} for channels that are const * one field."""
    out = {}
    for name, poly in ch.items():
        items = [(k, c) for k, c in poly.items() if c != 0.0]
        fields = [k for k, c in items if k != ()]
        if not fields:
            continue
        if len(items) != 1 or len(fields[0]) != 1:
            raise NotImplementedError("the adjoint supports coefficients of the form c * field")
        out[name] = fields[0][0]
    return out


class _BilinearJ(torch.autograd.Function):
    @staticmethod
    def forward(ctx, form, basis, names, w, u, X, *fields):
        kw = dict(zip(names, [f.detach() for f in fields]))
        Xd = X.detach().contiguous() if X is not None else None
        old_p = basis.c_mesh.p
        if Xd is not None:
            basis.c_mesh.p = Xd.data_ptr()
        try:
            K = form.assemble_torch(basis, **kw)
            coeffs = _Coefficients(basis, kw)
            ch = form._trace(basis, coeffs, "bilinear")
            c_form = form._setup(basis, None, kw)[2]
        finally:
            basis.c_mesh.p = old_p
        Ku = torch.mv(K, u)
        J = torch.dot(w, Ku)
        ctx.save_for_backward(w, u, Xd if Xd is not None else torch.empty(0), *fields)
        ctx.form, ctx.basis, ctx.names, ctx.K, ctx.ch, ctx.coeffs = form, basis, names, K, ch, coeffs
        ctx.c_form = c_form
        ctx.has_X = X is not None
        return J

    @staticmethod
    def backward(ctx, g):
        w, u, Xd, *fields = ctx.saved_tensors
        basis = ctx.basis
        dev = basis.device
        ne = basis.nelems
        chf = _channel_fields(ctx.ch)
        if basis.elem.vector:
            raise NotImplementedError("the adjoint is implemented for scalar bases")
        dcd = torch.zeros(ne, dtype=torch.float64, device=dev) if "diff" in chf else None
        dcm = torch.zeros(ne, dtype=torch.float64, device=dev) if "mass" in chf else None
        need_X = ctx.has_X and ctx.needs_input_grad[5]
        dX = torch.empty_like(Xd) if need_X else None
        scratch = (torch.empty(ne * basis.mesh.t.shape[0] * basis.mesh.p.shape[0],
                               dtype=torch.float64, device=dev) if need_X else None)
        vinc = _vertex_incidence(basis) if need_X else None
        m = _mesh_with(basis, Xd if ctx.has_X else None)
        wc, uc = w.contiguous(), u.contiguous()
        N.check(N.lib().fem_bilinear_vjp(N.byref(m), N.byref(basis.c_basis), N.byref(ctx.c_form),
                                         vinc.handle if vinc else None, N.ptr(wc), N.ptr(uc),
                                         N.ptr(dcd), N.ptr(dcm), N.ptr(dX), N.ptr(scratch),
                                         N.stream_ptr()))
        grads = {n: None for n in ctx.names}
        for chan, fname in chf.items():
            d = dcd if chan == "diff" else dcm
            grads[fname] = d * g if grads[fname] is None else grads[fname] + d * g
        K = ctx.K
        gw = torch.mv(K, u) * g if ctx.needs_input_grad[3] else None
        # every form the kernels implement is symmetric (isotropic diffusion +
        # mass, isotropic elasticity), so K^T w = K w
        gu = torch.mv(K, w) * g if ctx.needs_input_grad[4] else None
        return (None, None, None, gw, gu, dX * g if dX is not None else None,
                *[grads[n] for n in ctx.names])


class _LinearJ(torch.autograd.Function):
    @staticmethod
    def forward(ctx, form, basis, names, w, X, *fields):
        kw = dict(zip(names, [f.detach() for f in fields]))
        Xd = X.detach().contiguous() if X is not None else None
        old_p = basis.c_mesh.p
        if Xd is not None:
            basis.c_mesh.p = Xd.data_ptr()
        try:
            b = form.assemble_torch(basis, **kw)
            coeffs = _Coefficients(basis, kw)
            ch = form._trace(basis, coeffs, "linear")
            c_form = form._setup(basis, kw)[1]
        finally:
            basis.c_mesh.p = old_p
        ctx.save_for_backward(w, Xd if Xd is not None else torch.empty(0), b, *fields)
        ctx.form, ctx.basis, ctx.names, ctx.ch, ctx.c_form = form, basis, names, ch, c_form
        ctx.has_X = X is not None
        ctx.coeffs = coeffs
        return torch.dot(w, b)

    @staticmethod
    def backward(ctx, g):
        w, Xd, b, *fields = ctx.saved_tensors
        basis = ctx.basis
        dev = basis.device
        ne = basis.nelems
        chf = _channel_fields(ctx.ch)
        dl = torch.zeros(ne, dtype=torch.float64, device=dev) if "load" in chf else None
        need_X = ctx.has_X and ctx.needs_input_grad[4]
        dX = torch.empty_like(Xd) if need_X else None
        scratch = (torch.empty(ne * basis.mesh.t.shape[0] * basis.mesh.p.shape[0],
                               dtype=torch.float64, device=dev) if need_X else None)
        vinc = _vertex_incidence(basis) if need_X else None
        m = _mesh_with(basis, Xd if ctx.has_X else None)
        N.check(N.lib().fem_linear_vjp(N.byref(m), N.byref(basis.c_basis), N.byref(ctx.c_form),
                                       vinc.handle if vinc else None, N.ptr(w.contiguous()),
                                       N.ptr(dl), N.ptr(dX), N.ptr(scratch), N.stream_ptr()))
        grads = {n: None for n in ctx.names}
        if "load" in chf:
            grads[chf["load"]] = dl * g
        gw = b * g if ctx.needs_input_grad[3] else None
        return (None, None, None, gw, dX * g if dX is not None else None,
                *[grads[n] for n in ctx.names])


def _fields(basis, coefs):
    names, vals = [], []
    for k, v in coefs.items():
        t = torch.as_tensor(v, dtype=torch.float64, device=basis.device)
        if t.dim() != 1 or t.shape[0] != basis.nelems:
            raise ValueError("assemble_vjp takes one value per element for '%s'" % k)
        names.append(k)
        vals.append(t)
    return tuple(names), vals


def assemble_vjp(form: BilinearForm, basis, w, u, X=None, **coefs):
    """J = w^T K u, differentiable in w, u, X (node coordinates, shape
    (dim, nverts)) and the per-element coefficient fields in ``coefs``."""
    names, vals = _fields(basis, coefs)
    return _BilinearJ.apply(form, basis, names, w, u, X, *vals)


def assemble_linear_vjp(form: LinearForm, basis, w, X=None, **coefs):
    """J = w^T b, differentiable in w, X and the coefficient fields."""
    names, vals = _fields(basis, coefs)
    return _LinearJ.apply(form, basis, names, w, X, *vals)
