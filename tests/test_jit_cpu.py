"""Run-time compiled form programs: the source fem_program_source writes for
traced forms compiles with NVRTC for sm_103a (no GPU needed for that), with
the same options and headers fem_program_compile uses."""
import ctypes
import os

import pytest

import skfem_gb300 as F
from skfem_gb300 import _native as N
from skfem_gb300.tracer import FieldSpec, trace_tape
from _facet import robin, s_energy
from _generic import newton, trig_load, vec_conv
from _util import ROOT


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("libnvrtc not available")


HEADERS = [("fem_faithful_core.cuh", os.path.join(ROOT, "scikit-fem_gb300", "csrc",
                                                  "fem_faithful_core.cuh")),
           ("fem_program_kernel.cuh", os.path.join(ROOT, "scikit-fem_gb300", "csrc",
                                                   "fem_program_kernel.cuh")),
           ("../../include/skfem_gb300.h", os.path.join(ROOT, "include", "skfem_gb300.h"))]


def source_of(form, elem, dim, specs, kind, mode, facet):
    ins, out, names = trace_tape(form.form, elem, dim, specs, {}, kind=kind,
                                 defaults="facet" if facet else "cell")
    arr = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm) for op, a, b, imm in ins])
    need = ctypes.c_int64()
    lib = N.lib()
    v = int(elem.vector)
    assert lib.fem_program_source(ctypes.addressof(arr), len(ins), out, len(names), dim, v, v,
                                  mode, int(facet), None, 0, ctypes.byref(need)) == 0
    buf = ctypes.create_string_buffer(need.value)
    assert lib.fem_program_source(ctypes.addressof(arr), len(ins), out, len(names), dim, v, v,
                                  mode, int(facet), buf, need.value, None) == 0
    return buf.value.decode(), len(ins)


CASES = [
    ("newton_tri_p2", newton, F.ElementTriP2(), 2, {"s": FieldSpec("field", 0, True)},
     "bilinear", 0, False),
    ("trig_load", trig_load, F.ElementTriP1(), 2, {}, "linear", 1, False),
    ("vec_conv", vec_conv, F.ElementVector(F.ElementTetP2()), 3,
     {"d": FieldSpec("field", 3, True)}, "bilinear", 0, False),
    ("robin_facet", robin, F.ElementTetP1(), 3, {}, "bilinear", 0, True),
    ("s_energy_facet", s_energy, F.ElementTriP2(), 2, {"s": FieldSpec("field", 0, True)},
     "functional", 2, True),
]


@pytest.mark.parametrize("name,form,elem,dim,specs,kind,mode,facet", CASES,
                         ids=[c[0] for c in CASES])
def test_program_source_compiles_for_sm103a(name, form, elem, dim, specs, kind, mode, facet):
    src, n = source_of(form, elem, dim, specs, kind, mode, facet)
    for k in range(n):                                  # every instruction is written out
        assert ("const double r%d = " % k) in src
    nv = _nvrtc()
    prog = ctypes.c_void_p()
    hdr_src = (ctypes.c_char_p * 3)(*[open(p, "rb").read() for _, p in HEADERS])
    hdr_names = (ctypes.c_char_p * 3)(*[h.encode() for h, _ in HEADERS])
    assert nv.nvrtcCreateProgram(ctypes.byref(prog), src.encode(), b"fem_jit_program.cu", 3,
                                 hdr_src, hdr_names) == 0
    opts = (ctypes.c_char_p * 4)(b"--gpu-architecture=sm_103a", b"-fmad=false", b"--std=c++17",
                                 b"-default-device")
    rc = nv.nvrtcCompileProgram(prog, 4, opts)
    if rc != 0:
        size = ctypes.c_size_t()
        nv.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
        log = ctypes.create_string_buffer(size.value)
        nv.nvrtcGetProgramLog(prog, log)
        pytest.fail(log.value.decode()[:3000])
    size = ctypes.c_size_t()
    assert nv.nvrtcGetCUBINSize(prog, ctypes.byref(size)) == 0 and size.value > 0
    nv.nvrtcDestroyProgram(ctypes.byref(prog))


def test_program_source_rejects_bad_operands():
    bad = (N.FemInstr * 2)(N.FemInstr(1, 0, -1, 0, 0.0), N.FemInstr(4, 0, 5, 0, 0.0))
    assert N.lib().fem_program_source(ctypes.addressof(bad), 2, 1, 0, 2, 0, 0, 0, 0, None, 0,
                                      None) == N.FEM_ERR_ARGUMENT
