"""FacetBasis on the host: the mesh's facets / f2t / t2f, the facet-point
geometry (coordinates, h, outward normals; on Hex1 meshes the reference's
Newton-iterated inverse map) and the replayed facet integrals, against
scikit-fem's own outputs (tests/golden facet cases), bit for bit -- every
operation on this path is correctly rounded."""
import ctypes

import numpy as np
import pytest

from skfem_gb300 import _native as N
from skfem_gb300.tracer import FieldSpec, trace_tape
from _facet import CASES, VARIANTS, facet_args, fmass, length, neumann, robin, s_energy
from _generic import reference_csr, reference_vector
from _util import golden
from test_faithful_cpu import harness

V = ctypes.c_void_p


def _lib():
    lib = harness()
    lib.faithful_facet_program_host.argtypes = [ctypes.c_int] + [V] * 5
    lib.faithful_facet_points_host.argtypes = [V, V, ctypes.c_int, V, V]
    lib.faithful_facet_interpolate_host.argtypes = [V, V, V, ctypes.c_int, V, V, V]
    lib.faithful_hex_facet_geometry_host.argtypes = [V, V, ctypes.c_int, V, V]
    lib.faithful_sum_host.argtypes = [V, ctypes.c_int64]
    lib.faithful_sum_host.restype = ctypes.c_double
    return lib


class HostFacets:
    def __init__(self, m, elem, find, tind, X, W):
        from skfem_gb300.dofs import Dofs
        self.m, self.elem = m, elem
        self.dim = m.p.shape[0]
        self.p = np.ascontiguousarray(m.p)
        self.t = np.ascontiguousarray(m.t)
        self.ed = np.ascontiguousarray(Dofs(m, elem).element_dofs)
        self.N = int(self.ed.max()) + 1
        self.find = np.asarray(find, dtype=np.int32)
        self.tind = np.ascontiguousarray(tind, dtype=np.int32)
        self.tindn = np.ascontiguousarray(m.f2t[0, self.find], dtype=np.int32)
        self.lf = np.ascontiguousarray(np.argmax(m.t2f[:, self.tindn] == self.find[None, :],
                                                 axis=0), dtype=np.int32)
        self.fv = np.ascontiguousarray(m.facets[:, self.find], dtype=np.int32)
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.W = np.ascontiguousarray(W, dtype=np.float64)
        self.nf, self.nq = len(self.find), self.X.shape[1]
        self.mesh = N.FemMesh(self.dim, self.t.shape[0], self.p.shape[1], self.t.shape[1],
                              self.p.ctypes.data, self.t.ctypes.data)
        self.basis = N.FemBasis(N.FAMILY[elem.family], int(elem.vector), self.ed.shape[0], 0,
                                self.N, self.ed.ctypes.data)
        self.fc = N.FemFacets(self.nf, self.fv.ctypes.data, self.tind.ctypes.data,
                              self.tindn.ctypes.data, self.lf.ctypes.data, None)
        self.keep = []
        if elem.refdom == "hex":
            # Newton-iterated point geometry, as fem_facet_geometry computes it
            self.geo = np.zeros(self.nf * self.nq * 20)
            assert _lib().faithful_hex_facet_geometry_host(
                ctypes.byref(self.mesh), ctypes.byref(self.fc), self.nq, self.X.ctypes.data,
                self.geo.ctypes.data) == 0
            self.fc.geo = self.geo.ctypes.data

    def points(self):
        out = np.zeros((7, self.nf, self.nq))
        assert _lib().faithful_facet_points_host(ctypes.byref(self.mesh), ctypes.byref(self.fc),
                                                 self.nq, self.X.ctypes.data,
                                                 out.ctypes.data) == 0
        return out

    def interpolate(self, w):
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros((1 + self.dim, self.nf, self.nq))
        _lib().faithful_facet_interpolate_host(ctypes.byref(self.mesh), ctypes.byref(self.basis),
                                               ctypes.byref(self.fc), self.nq, self.X.ctypes.data,
                                               w.ctypes.data, out.ctypes.data)
        return out

    def run(self, form, kind, fields):
        specs, arrays = {}, {}
        for k, a in fields.items():
            specs[k] = FieldSpec("field", 0, True)
            arrays[k] = self.interpolate(a)
        ins, out, names = trace_tape(form.form, self.elem, self.dim, specs, {}, kind=kind,
                                     defaults="facet")
        arr = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm) for op, a, b, imm in ins])
        prog = N.FemProgram(len(ins), out, len(names), self.nq, ctypes.addressof(arr))
        for k, n in enumerate(names):
            a = np.ascontiguousarray(arrays[n[0]][n[1]])
            self.keep.append(a)
            prog.coef[k], prog.coef_stride[k] = a.ctypes.data, self.nq
        prog.qX, prog.qW = self.X.ctypes.data, self.W.ctypes.data
        mode = {"bilinear": 0, "linear": 1, "functional": 2}[kind]
        nb = self.ed.shape[0]
        L = nb * nb if mode == 0 else (nb if mode == 1 else 1)
        res = np.zeros(self.nf * L)
        assert _lib().faithful_facet_program_host(mode, ctypes.byref(self.mesh),
                                                  ctypes.byref(self.basis), ctypes.byref(self.fc),
                                                  ctypes.byref(prog), res.ctypes.data) == 0
        return res.reshape((self.nf, nb, nb) if mode == 0 else (self.nf, nb) if mode == 1
                           else (self.nf,))


@pytest.mark.parametrize("name,mesh_cls,elem", CASES, ids=[c[0] for c in CASES])
def test_mesh_facets_match_reference(name, mesh_cls, elem):
    g = golden(name)
    m = mesh_cls(g["p"], g["t"])
    np.testing.assert_array_equal(m.facets, g["facets"])
    np.testing.assert_array_equal(m.f2t, g["f2t"])
    np.testing.assert_array_equal(m.t2f, g["t2f"])
    for pre in VARIANTS:
        a = facet_args(m, g, pre)
        find = m.normalize_facets(a.get("facets"))
        np.testing.assert_array_equal(find, g[pre + "find"])
        np.testing.assert_array_equal(m.f2t[a.get("side", 0), find], g[pre + "tind"])


@pytest.mark.parametrize("name,mesh_cls,elem", CASES, ids=[c[0] for c in CASES])
def test_facet_replay_bitwise(name, mesh_cls, elem):
    g = golden(name)
    m = mesh_cls(g["p"], g["t"])
    for pre in VARIANTS:
        h = HostFacets(m, elem(), g[pre + "find"], g[pre + "tind"], g[pre + "X"], g[pre + "W"])
        pts = h.points()
        np.testing.assert_array_equal(pts[:h.dim], g[pre + "x"], err_msg=pre + "x")
        np.testing.assert_array_equal(pts[3], g[pre + "h"], err_msg=pre + "h")
        np.testing.assert_array_equal(pts[4:4 + h.dim], g[pre + "n"], err_msg=pre + "n")
        q = h.interpolate(g["s"])
        np.testing.assert_array_equal(q[0], g[pre + "s_value"])
        np.testing.assert_array_equal(q[1:], g[pre + "s_grad"])
        ed = h.ed[:, h.tind]
        for form, suffix in ((fmass, "mass"), (robin, "robin")):
            K = reference_csr(h.run(form, "bilinear", {}), ed, h.N)
            np.testing.assert_array_equal(K.indptr, g[pre + "indptr_" + suffix])
            np.testing.assert_array_equal(K.indices, g[pre + "indices_" + suffix])
            np.testing.assert_array_equal(K.data, g[pre + "data_" + suffix])
        b = reference_vector(h.run(neumann, "linear", {}), ed, h.N)
        np.testing.assert_array_equal(b, g[pre + "b_neumann"])
        for form, key, kw in ((length, "length", {}), (s_energy, "energy", {"s": g["s"]})):
            e = h.run(form, "functional", kw)
            np.testing.assert_array_equal(e, g[pre + "e_" + key])
            assert _lib().faithful_sum_host(e.ctypes.data, len(e)) == g[pre + "f_" + key]
