"""ctypes binding of libskfem_gb300.so (the C ABI in include/skfem_gb300.h).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every assembly call raises -- there is no CPU fallback.
"""

import ctypes
import os
import threading

import torch

from . import _build

FEM_OK = 0
FEM_ERR_ARGUMENT = 1
FEM_ERR_UNSUPPORTED = 2
FEM_ERR_CUDA = 3
FEM_ERR_ZERO_JACOBIAN = 4
FEM_ERR_STALE_PATTERN = 5
FEM_ERR_CAPACITY = 6
FEM_ERR_VARYING = 7
FEM_ERR_NEWTON = 8
FEM_ERR_TIMEOUT = 9

FAMILY = {"TriP1": 1, "TriP2": 2, "TetP1": 3, "TetP2": 4, "Hex1": 5}


class FemMesh(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("nloc", ctypes.c_int32),
                ("nverts", ctypes.c_int64), ("nelems", ctypes.c_int64),
                ("p", ctypes.c_void_p), ("t", ctypes.c_void_p)]


class FemBasis(ctypes.Structure):
    _fields_ = [("family", ctypes.c_int32), ("vector", ctypes.c_int32),
                ("nbfun", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("ndofs", ctypes.c_int64), ("element_dofs", ctypes.c_void_p)]


class FemCoef(ctypes.Structure):
    _fields_ = [("scale", ctypes.c_double), ("field", ctypes.c_void_p),
                ("stride", ctypes.c_int64)]


class FemHostRows(ctypes.Structure):
    _fields_ = [("host", ctypes.c_void_p), ("dev", ctypes.c_void_p), ("stride", ctypes.c_int64)]


class FemBilinear(ctypes.Structure):
    _fields_ = [("diff", FemCoef), ("mass", FemCoef), ("lam", FemCoef),
                ("lap", FemCoef), ("tr", FemCoef)]


class FemLinear(ctypes.Structure):
    _fields_ = [("load", FemCoef)]


class FemInstr(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("pad_", ctypes.c_int32), ("imm", ctypes.c_double)]


class FemFacets(ctypes.Structure):
    _fields_ = [("nfacets", ctypes.c_int64), ("fverts", ctypes.c_void_p),
                ("tind", ctypes.c_void_p), ("tind_n", ctypes.c_void_p),
                ("lfacet_n", ctypes.c_void_p), ("geo", ctypes.c_void_p)]


class FemProgram(ctypes.Structure):
    _fields_ = [("ninstr", ctypes.c_int32), ("out", ctypes.c_int32), ("ncoef", ctypes.c_int32),
                ("nq", ctypes.c_int32), ("ins", ctypes.c_void_p), ("coef", ctypes.c_void_p * 16),
                ("coef_stride", ctypes.c_int32 * 16), ("qX", ctypes.c_void_p),
                ("qW", ctypes.c_void_p), ("compiled", ctypes.c_void_p)]


class FemError(RuntimeError):
    pass


class ZeroJacobianError(Exception):
    pass


_lib = None
_lock = threading.Lock()

_P = ctypes.c_void_p
_I64P = ctypes.POINTER(ctypes.c_int64)

_SIGS = {
    "fem_last_error": (ctypes.c_char_p, []),
    "fem_version": (ctypes.c_char_p, []),
    "fem_local_matrices": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "fem_local_vectors": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "fem_pattern_build": (ctypes.c_int, [_P, _P, _P, _P, ctypes.POINTER(ctypes.c_void_p), _P]),
    "fem_pattern_info": (ctypes.c_int, [_P, _I64P, _I64P, _I64P]),
    "fem_pattern_export": (ctypes.c_int, [_P, _P, _P, _P]),
    "fem_pattern_destroy": (None, [_P]),
    "fem_assemble": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "fem_csr_sum": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "fem_csr_sum_staged": (ctypes.c_int, [_P, _P, _P, _P]),
    "fem_vector_sum": (ctypes.c_int, [_P, _P, _P, _P]),
    "fem_assemble_vector": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "fem_bilinear_vjp": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "fem_linear_vjp": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "fem_vertex_incidence_build": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_void_p), _P]),
    "fem_condense_pattern": (ctypes.c_int, [_P, _P, ctypes.c_int64, _P, ctypes.c_int64, _P,
                                            _I64P, _P]),
    "fem_condense_values": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, _P, _P, _P, _P, _P, _P,
                                           _P, _P]),
    "fem_program_local_matrices": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "fem_program_local_vectors": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "fem_program_elemental": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "fem_pattern_build_local": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(ctypes.c_void_p), _P]),
    "fem_csr_sum_checked": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "fem_interpolate": (ctypes.c_int, [_P, _P, ctypes.c_int32, _P, _P, _P, _P]),
    "fem_sum_pairwise": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P]),
    "fem_facet_program_local_matrices": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "fem_facet_program_local_vectors": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "fem_facet_program_elemental": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "fem_facet_interpolate": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P, _P, _P, _P]),
    "fem_assemble_to_host": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, ctypes.c_int32,
                                            _P, _P]),
    "fem_program_compile": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.c_int32,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "fem_program_local_matrices_mixed": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "fem_pattern_build_local_mixed": (ctypes.c_int, [_P, _P, _P, _P,
                                                     ctypes.POINTER(ctypes.c_void_p), _P]),
    "fem_program_release": (None, [_P]),
    "fem_program_source": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p,
                                          ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "fem_assemble_local": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, ctypes.c_int64, ctypes.c_int64,
                                          _P]),
    "fem_csr_sum_to_host": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int32, _P, _P]),
    "fem_host_memory_access": (ctypes.c_int, [_P]),
    "fem_pattern_cache_geometry": (ctypes.c_int, [_P, _P, _P, _P]),
    "fem_pattern_drop_geometry": (None, [_P]),
    "fem_pattern_cache_coefficient_update": (ctypes.c_int, [_P, _P, _P, _P]),
    "fem_pattern_drop_coefficient_update": (None, [_P]),
    "fem_assemble_to_host_pipelined": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P,
                                                      ctypes.c_int32, ctypes.c_int32, _P, _P,
                                                      _P]),
    "fem_facet_geometry": (ctypes.c_int, [_P, _P, _P, ctypes.c_int32, _P, _P, _P, _P]),
    "fem_enforce": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, _P, ctypes.c_int64,
                                   ctypes.c_double, _P, _P, _P, _P]),
    "fem_set_tuning": (ctypes.c_int, [ctypes.c_int] * 5),
    "fem_set_onepass": (ctypes.c_int, [ctypes.c_int] * 2),
    "fem_set_local_tma": (ctypes.c_int, [ctypes.c_int] * 2),
    "fem_assemble_noalloc": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "fem_batch_plan_build": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_void_p)]),
    "fem_batch_plan_destroy": (None, [_P]),
    "fem_batch_plan_info": (ctypes.c_int, [_P, _I64P, _I64P]),
    "fem_batched_assemble_vjp": (ctypes.c_int, [_P] * 14),
    "fem_coo_pattern_build": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64,
                                             ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p),
                                             _P]),
}


def lib():
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) or os.environ.get("SKFEM_GB300_REBUILD"):
            path = _build.build()
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


_host_access = None


def host_memory_access():
    """Whether kernels on the current device read pageable host memory."""
    global _host_access
    if _host_access is None:
        v = ctypes.c_int32(0)
        check(lib().fem_host_memory_access(ctypes.byref(v)))
        _host_access = bool(v.value)
    return _host_access


def require_cuda(device=None):
    if not torch.cuda.is_available():
        raise RuntimeError(
            "skfem_gb300 assembles on a CUDA GPU (GB300, sm_103a) and has no CPU "
            "fallback; no CUDA device is visible")
    return torch.device("cuda", torch.cuda.current_device() if device is None else
                        torch.device(device).index or 0)


def check(rc):
    if rc == FEM_OK:
        return
    msg = lib().fem_last_error().decode(errors="replace")
    if rc == FEM_ERR_ARGUMENT:
        raise ValueError(msg)
    if rc == FEM_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == FEM_ERR_ZERO_JACOBIAN:
        raise ZeroJacobianError("Zero Jacobian determinant")
    raise FemError(msg)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def byref(s):
    return ctypes.byref(s)


class Pattern:
    """Owns a FemPattern handle."""

    def __init__(self, handle):
        self.handle = handle
        nnz, nrows, stg = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().fem_pattern_info(handle, ctypes.byref(nnz), ctypes.byref(nrows),
                                     ctypes.byref(stg)))
        self.nnz, self.nrows, self.staging_bytes = nnz.value, nrows.value, stg.value

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h and _lib is not None:
            try:
                torch.cuda.synchronize()
            except Exception:
                pass
            _lib.fem_pattern_destroy(h)
