"""The exact-zero replay (csrc/fem_faithful_core.cuh) reproduces the
reference's arithmetic bit for bit: built for the host, it must return
exactly the oracle's local matrices (themselves bit-exact to scikit-fem on
the golden cases) for every entry -- not only the noise-level ones the GPU
pattern build replays."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle as O
import skfem_gb300 as F
from skfem_gb300 import _native as N
from skfem_gb300 import helpers as H
from skfem_gb300.models.elasticity import linear_elasticity
from skfem_gb300.models.poisson import laplace, mass
from skfem_gb300.tracer import trace_tape
from _util import ROOT, golden

_LIB = None


def harness():
    global _LIB
    if _LIB is None:
        src = os.path.join(ROOT, "tests", "native", "faithful_harness.cpp")
        out = os.path.join(tempfile.mkdtemp(), "faithful_harness.so")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                        src, "-o", out], check=True)
        _LIB = ctypes.CDLL(out)
        _LIB.faithful_replay_host.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int,
                                                                      ctypes.c_void_p]
    return _LIB


def replay(g, elem, form, fields, nq_X, nq_W):
    p = np.ascontiguousarray(g["p"], dtype=np.float64)
    t = np.ascontiguousarray(g["t"], dtype=np.int32)
    ed = np.ascontiguousarray(g["element_dofs"], dtype=np.int32)
    dim = p.shape[0]
    mesh = N.FemMesh(dim, t.shape[0], p.shape[1], t.shape[1], p.ctypes.data, t.ctypes.data)
    basis = N.FemBasis(N.FAMILY[elem.family], int(elem.vector), ed.shape[0], 0,
                       int(ed.max()) + 1, ed.ctypes.data)
    ins, out, names = trace_tape(form.form, elem, dim, list(fields), {})
    arr = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm) for op, a, b, imm in ins])
    prog = N.FemProgram(len(ins), out, len(names), nq_X.shape[1], ctypes.addressof(arr))
    keep = []
    for k, n in enumerate(names):
        a = np.ascontiguousarray(fields[n], dtype=np.float64)
        keep.append(a)
        prog.coef[k] = a.ctypes.data
    X = np.ascontiguousarray(nq_X, dtype=np.float64)
    W = np.ascontiguousarray(nq_W, dtype=np.float64)
    nb = ed.shape[0]
    res = np.zeros(t.shape[1] * nb * nb)
    rc = harness().faithful_replay_host(ctypes.byref(mesh), ctypes.byref(basis),
                                        ctypes.byref(prog), X.ctypes.data, W.ctypes.data,
                                        X.shape[1], res.ctypes.data)
    assert rc == 0
    return res.reshape(t.shape[1], nb, nb)


@F.BilinearForm
def k_laplace_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


@F.BilinearForm
def k_laplace(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v))


@F.BilinearForm
def theta_laplace(u, v, w):
    return w.theta * H.dot(H.grad(u), H.grad(v))


CASES = [
    ("tri_default_mass", F.ElementTriP1(), O.TriP1(), "tri", mass, O.mass, {}),
    ("tri_p1_laplace", F.ElementTriP1(), O.TriP1(), "tri", laplace, O.laplace, {}),
    ("tet_p1_k_laplace_mass", F.ElementTetP1(), O.TetP1(), "tet", k_laplace_mass,
     O.k_laplace_mass, {"k": "k"}),
    ("tri_p2_k_laplace", F.ElementTriP2(), O.TriP2(), "tri", k_laplace, O.k_laplace, {"k": "k"}),
    ("tet_p2_laplace", F.ElementTetP2(), O.TetP2(), "tet", laplace, O.laplace, {}),
    ("tet_p2_vec_elasticity", F.ElementVector(F.ElementTetP2()), O.Vector(O.TetP2()), "tet",
     linear_elasticity(1.0, 0.5), O.linear_elasticity(1.0, 0.5), {}),
    ("hex1_theta_laplace", F.ElementHex1(), O.Hex1(), "hex", theta_laplace, O.theta_laplace,
     {"theta": "theta"}),
    ("hex1_laplace_8", F.ElementHex1(), O.Hex1(), "hex", laplace, O.laplace, {}),
]


@pytest.mark.parametrize("name,ep,eo,kind,fp,fo,fields", CASES, ids=[c[0] for c in CASES])
def test_replay_is_bitwise_the_reference_arithmetic(name, ep, eo, kind, fp, fo, fields):
    g = golden(name)
    bo = O.OBasis(O.OMesh(g["p"], g["t"], kind), eo,
                  intorder=4 if name == "tet_p2_vec_elasticity" else None)
    w = {k: bo.zero_w() + g[v][:, None] for k, v in fields.items()}
    data, _, _, _ = O.bilinear_local(fo, bo, **w)      # (Nu, Nv, nel): data[j, i, e]
    ref = np.transpose(data, (2, 1, 0))                 # [e][i][j]
    got = replay(g, ep, fp, {k: g[v] for k, v in fields.items()}, g["X"], g["W"])
    assert np.array_equal(got == 0.0, ref == 0.0), "exact-zero sets differ"
    np.testing.assert_array_equal(got, ref)
