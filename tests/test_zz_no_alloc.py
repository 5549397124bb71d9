"""fem_assemble_noalloc: the assembly entry point for callers that cannot
allocate GPU memory (a framework owning the device's memory, or a program
that allows no allocation after start-up).  It must produce what
fem_assemble produces, call after call, from its static scratch array, take
meshes up to that array's size and refuse larger ones, and reject bad
arguments on the host before any kernel runs.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from _util import REL_FRO, REL_MAX

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20


def _noalloc(lib):
    fn = lib.fem_assemble_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 7
    return fn


def _setup(nodes, vector=False):
    import skfem_gb300 as F
    from skfem_gb300 import helpers as H
    from skfem_gb300.models.elasticity import linear_elasticity

    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, nodes),) * 3)
    if vector:
        p = m.p.copy()
        inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
        rng = np.random.default_rng(11)
        h = 1.0 / (nodes - 1)
        p[:, inner] += rng.uniform(-0.2 * h, 0.2 * h, size=(3, int(inner.sum())))
        m = F.MeshTet(p, m.t)
        b = F.Basis(m, F.ElementVector(F.ElementTetP1()))
        form = linear_elasticity(1.0, 0.5)
        coefs = {}
    else:
        b = F.Basis(m, F.ElementTetP1())
        k = torch.from_numpy(np.random.default_rng(5).lognormal(0, 1, m.nelements)).cuda()

        @F.BilinearForm
        def form(u, v, w):
            return w.k * H.dot(H.grad(u), H.grad(v)) + u * v
        coefs = {"k": k}

    form.assemble_torch(b, **coefs)          # builds the pattern through the normal path
    entry = next(iter(b._patterns.values()))
    c_form = form._setup(b, None, coefs)[2]
    return b, entry, c_form


def _reference_values(lib, N, b, entry, c_form):
    ref = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                             entry.pat.handle, N.ptr(entry.staging), N.ptr(ref), N.ptr(status),
                             N.stream_ptr()))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return ref


def _check_twice(lib, N, fn, b, entry, c_form, ref):
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
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


def test_noalloc_matches_fem_assemble_twice():
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, entry, c_form = _setup(17)                 # 24,576 cells: 3 MiB of scratch
    ref = _reference_values(lib, N, b, entry, c_form)
    _check_twice(lib, N, fn, b, entry, c_form, ref)


def test_noalloc_vector_basis_matches_fem_assemble():
    # vector TetP1 elasticity: fem_assemble sums block-upper staging, the
    # no-alloc path the full local matrices; the values agree within the bound
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, entry, c_form = _setup(7, vector=True)     # 1,296 cells, 12 x 12 local matrices
    ref = _reference_values(lib, N, b, entry, c_form)
    _check_twice(lib, N, fn, b, entry, c_form, ref)


def test_noalloc_at_its_capacity():
    # 45 nodes per axis: 511,104 TetP1 cells x 128 B = 62.4 MiB, inside the
    # 64 MiB array -- accepted, and equal to fem_assemble
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, entry, c_form = _setup(45)
    assert b.nelems * 16 * 8 <= SCRATCH_BYTES
    ref = _reference_values(lib, N, b, entry, c_form)
    _check_twice(lib, N, fn, b, entry, c_form, ref)


def test_noalloc_rejects_meshes_beyond_its_scratch():
    # 46 nodes per axis: 546,750 cells x 128 B = 66.7 MiB > 64 MiB
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, entry, c_form = _setup(46)
    assert b.nelems * 16 * 8 > SCRATCH_BYTES
    out = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    rc = fn(ctypes.byref(b.c_mesh), ctypes.byref(b.c_basis), ctypes.byref(c_form),
            entry.pat.handle, N.ptr(out), None, N.stream_ptr())
    assert rc == N.FEM_ERR_CAPACITY
    assert b"static scratch" in lib.fem_last_error()


def test_noalloc_rejects_bad_arguments_on_the_host():
    # a null coordinate array, or a vertex count that does not match the
    # element, is refused before any kernel is launched
    from skfem_gb300 import _native as N
    lib = N.lib()
    fn = _noalloc(lib)
    b, entry, c_form = _setup(5)
    out = torch.full((entry.nnz,), 7.0, dtype=torch.float64, device="cuda")
    mesh = type(b.c_mesh).from_buffer_copy(b.c_mesh)
    mesh.p = None
    rc = fn(ctypes.byref(mesh), ctypes.byref(b.c_basis), ctypes.byref(c_form),
            entry.pat.handle, N.ptr(out), None, N.stream_ptr())
    assert rc == N.FEM_ERR_ARGUMENT
    mesh = type(b.c_mesh).from_buffer_copy(b.c_mesh)
    mesh.nloc = 3
    rc = fn(ctypes.byref(mesh), ctypes.byref(b.c_basis), ctypes.byref(c_form),
            entry.pat.handle, N.ptr(out), None, N.stream_ptr())
    assert rc == N.FEM_ERR_ARGUMENT
    torch.cuda.synchronize()
    assert bool((out == 7.0).all())               # nothing was written
