"""The generic kernels' arithmetic (csrc/fem_faithful_core.cuh), built for
the host, against scikit-fem's own outputs on forms outside the coefficient
channels: interpolated DOF vectors, global coordinates and mesh parameter,
per-point coefficients, anisotropic / advection terms, Functional.  Every
operation these forms use is correctly rounded, so the comparison is
bitwise (the trigonometric load and the 3-D mesh parameter, which go
through libm, within 1e-15)."""
import ctypes

import numpy as np
import pytest

import skfem_gb300 as F
from skfem_gb300 import _native as N
from skfem_gb300.tracer import FieldSpec, trace_tape
from _generic import (SCALAR_CASES, energy, fixture_csr, newton, newton_res, qp_coef,
                      reference_csr, reference_vector, trig_load, vec_conv, vec_energy)
from _util import golden
from test_faithful_cpu import harness


def _lib():
    lib = harness()
    lib.faithful_program_host.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
    lib.faithful_interpolate_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.faithful_points_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p]
    lib.faithful_sum_host.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    lib.faithful_sum_host.restype = ctypes.c_double
    return lib


class HostCase:
    """A golden fixture's mesh / basis as host FemMesh / FemBasis structs."""

    def __init__(self, g, elem):
        self.g = g
        self.elem = elem
        self.p = np.ascontiguousarray(g["p"], dtype=np.float64)
        self.t = np.ascontiguousarray(g["t"], dtype=np.int32)
        self.ed = np.ascontiguousarray(g["element_dofs"], dtype=np.int32)
        self.X = np.ascontiguousarray(g["X"], dtype=np.float64)
        self.W = np.ascontiguousarray(g["W"], dtype=np.float64)
        self.dim = self.p.shape[0]
        self.nel = self.t.shape[1]
        self.nq = self.X.shape[1]
        self.N = int(self.ed.max()) + 1
        self.mesh = N.FemMesh(self.dim, self.t.shape[0], self.p.shape[1], self.nel,
                              self.p.ctypes.data, self.t.ctypes.data)
        self.basis = N.FemBasis(N.FAMILY[elem.family], int(elem.vector), self.ed.shape[0], 0,
                                self.N, self.ed.ctypes.data)
        self.keep = []

    def interpolate(self, w):
        w = np.ascontiguousarray(w, dtype=np.float64)
        nquant = self.dim + self.dim ** 2 if self.elem.vector else 1 + self.dim
        out = np.zeros((nquant, self.nel, self.nq))
        _lib().faithful_interpolate_host(ctypes.byref(self.mesh), ctypes.byref(self.basis),
                                         self.nq, self.X.ctypes.data, w.ctypes.data,
                                         out.ctypes.data)
        return out

    def points(self):
        out = np.zeros((4, self.nel, self.nq))
        _lib().faithful_points_host(ctypes.byref(self.mesh), ctypes.byref(self.basis), self.nq,
                                    self.X.ctypes.data, out.ctypes.data)
        return out

    def run(self, form, kind, fields):
        """fields: name -> per-point array (nel, nq) or DOF vector (N,)."""
        specs, arrays = {}, {}
        for k, a in fields.items():
            if a.ndim == 1:
                q = self.interpolate(a)
                specs[k] = FieldSpec("field", self.dim if self.elem.vector else 0, True)
                arrays[k] = q
            else:
                specs[k] = FieldSpec("qp")
                arrays[k] = np.ascontiguousarray(a, dtype=np.float64)
        ins, out, names = trace_tape(form.form, self.elem, self.dim, specs, {}, kind=kind,
                                     defaults=True)
        arr = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm) for op, a, b, imm in ins])
        prog = N.FemProgram(len(ins), out, len(names), self.nq, ctypes.addressof(arr))
        for k, n in enumerate(names):
            if isinstance(n, tuple):
                a = np.ascontiguousarray(arrays[n[0]][n[1]])
            else:
                a = arrays[n]
            self.keep.append(a)
            prog.coef[k] = a.ctypes.data
            prog.coef_stride[k] = self.nq
        prog.qX, prog.qW = self.X.ctypes.data, self.W.ctypes.data
        mode = {"bilinear": 0, "linear": 1, "functional": 2}[kind]
        nb = self.ed.shape[0]
        L = nb * nb if mode == 0 else (nb if mode == 1 else 1)
        res = np.zeros(self.nel * L)
        rc = _lib().faithful_program_host(mode, ctypes.byref(self.mesh), ctypes.byref(self.basis),
                                          ctypes.byref(prog), res.ctypes.data)
        assert rc == 0
        if mode == 0:
            return res.reshape(self.nel, nb, nb)
        if mode == 1:
            return res.reshape(self.nel, nb)
        return res


ELEMS = {"tri_p2_generic": F.ElementTriP2(), "tet_p1_generic": F.ElementTetP1(),
         "hex1_generic": F.ElementHex1()}


@pytest.mark.parametrize("name", list(ELEMS))
def test_interpolate_and_points_bitwise(name):
    g = golden(name)
    h = HostCase(g, ELEMS[name])
    q = h.interpolate(g["s"])
    np.testing.assert_array_equal(q[0], g["s_value"])
    np.testing.assert_array_equal(q[1:], g["s_grad"])
    pts = h.points()
    np.testing.assert_array_equal(pts[:h.dim], g["x"])
    if h.dim == 2:
        np.testing.assert_array_equal(pts[3], g["h"])       # **0.5 is sqrt
    else:
        np.testing.assert_allclose(pts[3], g["h"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("name,elem,forms", SCALAR_CASES, ids=[c[0] for c in SCALAR_CASES])
def test_generic_bilinear_bitwise(name, elem, forms):
    g = golden(name)
    h = HostCase(g, ELEMS[name])
    cases = dict(forms)
    cases["qp"] = qp_coef
    cases["newton"] = newton
    args = {"qp": {"c": g["c"]}, "newton": {"s": g["s"]}}
    for suffix, form in cases.items():
        local = h.run(form, "bilinear", args.get(suffix, {}))
        K = reference_csr(local, h.ed, h.N)
        ip, ix, d = fixture_csr(g, suffix)
        np.testing.assert_array_equal(K.indptr, ip, err_msg=suffix)
        np.testing.assert_array_equal(K.indices, ix, err_msg=suffix)
        np.testing.assert_array_equal(K.data, d, err_msg=suffix)


@pytest.mark.parametrize("name", list(ELEMS))
def test_generic_linear_and_functional(name):
    g = golden(name)
    h = HostCase(g, ELEMS[name])
    b = reference_vector(h.run(newton_res, "linear", {"s": g["s"]}), h.ed, h.N)
    np.testing.assert_array_equal(b, g["b_newton"])
    e = h.run(energy, "functional", {"s": g["s"]})
    if h.dim == 2:
        np.testing.assert_array_equal(e, g["e_energy"])
        assert _lib().faithful_sum_host(e.ctypes.data, len(e)) == g["f_energy"]
    else:
        np.testing.assert_allclose(e, g["e_energy"], rtol=1e-15, atol=0)
        assert abs(_lib().faithful_sum_host(e.ctypes.data, len(e)) - g["f_energy"]) <= \
            1e-14 * abs(g["f_energy"])
    if name == "tri_p2_generic":
        bt = reference_vector(h.run(trig_load, "linear", {}), h.ed, h.N)
        np.testing.assert_allclose(bt, g["b_trig"], rtol=1e-14, atol=1e-15 * np.abs(bt).max())


def test_vector_field_bitwise():
    g = golden("tet_p2_vec_generic")
    h = HostCase(g, F.ElementVector(F.ElementTetP2()))
    q = h.interpolate(g["d"])
    np.testing.assert_array_equal(q[:3], g["d_value"])
    np.testing.assert_array_equal(q[3:].reshape(3, 3, h.nel, h.nq), g["d_grad"])
    local = h.run(vec_conv, "bilinear", {"d": g["d"]})
    K = reference_csr(local, h.ed, h.N)
    ip, ix, d = fixture_csr(g, "conv")
    np.testing.assert_array_equal(K.indptr, ip)
    np.testing.assert_array_equal(K.indices, ix)
    np.testing.assert_array_equal(K.data, d)
    e = h.run(vec_energy, "functional", {"d": g["d"]})
    np.testing.assert_array_equal(e, g["e_energy"])
    assert _lib().faithful_sum_host(e.ctypes.data, len(e)) == g["f_energy"]


def test_numpy_pairwise_sum_order():
    """np.sum of a vector: leaves of <= 128 values (8 accumulators), split
    at n/2 rounded down to a multiple of 8 -- checked on sizes where the
    order changes the result."""
    rng = np.random.default_rng(5)
    for n in (0, 1, 7, 8, 127, 128, 129, 1000, 4097, 100_003):
        x = rng.standard_normal(n) * np.exp(rng.uniform(-30, 30, n))
        assert _lib().faithful_sum_host(x.ctypes.data, n) == np.sum(x)


def test_vector_hex_bitwise():
    """ElementVector(ElementHex1) (generic kernels only): interpolation and
    linear elasticity replayed on the host equal the reference bit for bit."""
    from skfem_gb300.models.elasticity import linear_elasticity
    g = golden("hex1_vec")
    e = F.ElementVector(F.ElementHex1())
    X, W = F.get_quadrature("hex", 6)
    g = dict(g, X=X, W=W)
    h = HostCase(g, e)
    q = h.interpolate(g["d"])
    np.testing.assert_array_equal(q[:3], g["d_value"])
    np.testing.assert_array_equal(q[3:].reshape(3, 3, h.nel, h.nq), g["d_grad"])
    local = h.run(linear_elasticity(1.0, 0.5), "bilinear", {})
    K = reference_csr(local, h.ed, h.N)
    ip, ix, d = fixture_csr(g, "elast")
    np.testing.assert_array_equal(K.indptr, ip)
    np.testing.assert_array_equal(K.indices, ix)
    np.testing.assert_array_equal(K.data, d)
