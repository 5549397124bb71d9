"""fem_assemble_noalloc: the assembly entry point for callers that cannot
allocate GPU memory (a framework owning the device's memory, or a program
that allows no allocation after start-up).  It must produce what
fem_assemble produces, call after call, from its static scratch array, and
refuse meshes too large for that array.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from _util import REL_FRO, REL_MAX

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    fn = lib.fem_assemble_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 7
    return fn


def _setup(nodes):
    import skfem_gb300 as F
    from skfem_gb300 import helpers as H

    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, nodes),) * 3)
    b = F.Basis(m, F.ElementTetP1())
    k = torch.from_numpy(np.random.default_rng(5).lognormal(0, 1, m.nelements)).cuda()

    @F.BilinearForm
    def form(u, v, w):
        return w.k * H.dot(H.grad(u), H.grad(v)) + u * v

    K = form.assemble_torch(b, k=k)          # builds the pattern through the normal path
    entry = next(iter(b._patterns.values()))
    c_form = form._setup(b, None, {"k": k})[2]
    return b, k, K, entry, c_form


def test_noalloc_matches_fem_assemble_twice():
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, k, K, entry, c_form = _setup(17)           # 24,576 cells: 3 MiB of scratch
    ref = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                             entry.pat.handle, N.ptr(entry.staging), N.ptr(ref), N.ptr(status),
                             N.stream_ptr()))
    for _ in range(2):
        out = torch.full((entry.nnz,), np.nan, dtype=torch.float64, device="cuda")
        status.zero_()
        rc = fn(ctypes.byref(b.c_mesh), ctypes.byref(b.c_basis), ctypes.byref(c_form),
                entry.pat.handle, N.ptr(out), N.ptr(status), N.stream_ptr())
        assert rc == 0, lib.fem_last_error()
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        d = (out - ref).abs()
        assert torch.linalg.norm(out - ref) <= REL_FRO * torch.linalg.norm(ref)
        assert d.max() <= REL_MAX * ref.abs().max()


def test_noalloc_rejects_meshes_beyond_its_scratch():
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, k, K, entry, c_form = _setup(83)           # 3,176,523 cells: 388 MiB > 64 MiB
    out = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    rc = fn(ctypes.byref(b.c_mesh), ctypes.byref(b.c_basis), ctypes.byref(c_form),
            entry.pat.handle, N.ptr(out), None, N.stream_ptr())
    assert rc == N.FEM_ERR_CAPACITY
    assert b"static scratch" in lib.fem_last_error()
