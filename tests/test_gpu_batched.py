"""Batched multi-mesh assembly: the block-diagonal batch reproduces each
mesh's own assembly bit for bit, the CUDA-graph replay reproduces the eager
launch bit for bit, and the batched adjoint matches the per-mesh adjoint."""
import numpy as np
import pytest
import torch

import skfem_gb300 as F
from skfem_gb300 import helpers as H
from skfem_gb300.batched import BatchedBasis, GraphedAssembly

pytestmark = pytest.mark.gpu


@F.BilinearForm
def k_laplace(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v))


def jittered_square(n, rng):
    m = F.MeshTri.init_tensor(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1))
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(2, int(inner.sum())))
    return F.MeshTri(p, m.t)


def make_batch(sizes, seed=0):
    rng = np.random.default_rng(seed)
    meshes = [jittered_square(n, rng) for n in sizes]
    ks = [rng.lognormal(0, 0.5, m.nelements) for m in meshes]
    return meshes, ks


def test_batch_blocks_equal_per_mesh_assembly():
    meshes, ks = make_batch([3, 7, 12, 5, 9])
    bb = BatchedBasis(meshes, F.ElementTriP2())
    kcat = np.concatenate(ks)
    K = k_laplace.assemble(bb, k=bb.zero_w() + kcat[:, None])
    for m, k, blk in zip(meshes, ks, bb.split(K)):
        b = F.Basis(m, F.ElementTriP2())
        Km = k_laplace.assemble(b, k=b.zero_w() + k[:, None])
        np.testing.assert_array_equal(blk.indptr, Km.indptr)
        np.testing.assert_array_equal(blk.indices, Km.indices)
        np.testing.assert_array_equal(blk.data, Km.data)


def test_graph_replay_forward_and_adjoint():
    """The separate-kernel path with the coordinate gradient: graph replay
    equals the eager launch bit for bit, and the adjoint the autograd path."""
    from skfem_gb300.autodiff import assemble_vjp
    meshes, ks = make_batch([4, 6, 10], seed=3)
    bb = BatchedBasis(meshes, F.ElementTriP2())
    rng = np.random.default_rng(9)
    k = torch.tensor(np.concatenate(ks), device="cuda")
    w = torch.tensor(rng.standard_normal(bb.N), device="cuda")
    u = torch.tensor(rng.standard_normal(bb.N), device="cuda")
    ga = GraphedAssembly(k_laplace, bb, {"k": k}, w=w, u=u, with_dX=True)
    assert ga.plan is None and ga.launches_per_step() == 4
    ga.run_eager()
    torch.cuda.synchronize()
    v_eager = ga.values.clone()
    dk_eager = ga.dcoef["k"].clone()
    dX_eager = ga.dX.clone()
    ga.values.zero_()
    ga.dcoef["k"].zero_()
    ga.dX.zero_()
    ga.capture()
    ga.replay()
    torch.cuda.synchronize()
    ga.check()
    assert torch.equal(ga.values, v_eager)
    assert torch.equal(ga.dcoef["k"], dk_eager)
    assert torch.equal(ga.dX, dX_eager)
    # new coefficients through the same graph
    ga.coef["k"].mul_(2.0)
    ga.replay()
    torch.cuda.synchronize()
    torch.testing.assert_close(ga.values, 2.0 * v_eager, rtol=1e-15, atol=0)
    # adjoint of the batch equals the autograd path
    kt = k.clone().requires_grad_(True)
    X = bb.p_dev.clone().requires_grad_(True)
    J = assemble_vjp(k_laplace, bb, w, u, X=X, k=kt)
    J.backward()
    torch.testing.assert_close(kt.grad, dk_eager, rtol=1e-13, atol=1e-15)
    torch.testing.assert_close(X.grad, dX_eager, rtol=1e-13, atol=1e-15)


@F.BilinearForm
def k_laplace_c_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + w.c * u * v


@pytest.mark.parametrize("elem,dim", [(F.ElementTriP2, 2), (F.ElementTriP1, 2),
                                      (F.ElementTetP1, 3), (F.ElementTetP2, 3)])
def test_persistent_launch_equals_separate_kernels(elem, dim):
    """One persistent work-queue launch (cell units, then row units waiting
    on their mesh's cells) gives the CSR values of fem_assemble's path for the
    family -- TriP1 / TetP1: the split entry points' (bit for bit), TriP2 /
    TetP2: the one-pass node-block sum's (bit for bit; its row-block units
    wait on every mesh their rows belong to) -- and the separate adjoint
    kernel's gradients within 1e-13; graph replay equals the eager launch bit
    for bit; meshes of very uneven size, and repeated replays with new
    coefficients, keep the status word clear."""
    rng = np.random.default_rng(12)
    if dim == 2:
        meshes, _ = make_batch([1, 17, 3, 40, 2, 9], seed=7)
    else:
        meshes = []
        for n in (2, 7, 1, 5):
            m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
            p = m.p.copy()
            inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
            p[:, inner] += rng.uniform(-0.2 / n, 0.2 / n, size=(3, int(inner.sum())))
            meshes.append(F.MeshTet(p, m.t))
    bb = BatchedBasis(meshes, elem())
    k = torch.tensor(rng.lognormal(0, 0.5, bb.nelems), device="cuda")
    c = torch.tensor(rng.uniform(0.5, 2.0, bb.nelems), device="cuda")
    w = torch.tensor(rng.standard_normal(bb.N), device="cuda")
    u = torch.tensor(rng.standard_normal(bb.N), device="cuda")
    sep = GraphedAssembly(k_laplace_c_mass, bb, {"k": k, "c": c}, w=w, u=u, persistent=False)
    per = GraphedAssembly(k_laplace_c_mass, bb, {"k": k, "c": c}, w=w, u=u)
    assert per.plan is not None and per.launches_per_step() == 1
    sep.run_eager()
    per.run_eager()
    torch.cuda.synchronize()
    per.check()
    sep.check()
    ref = _reference(per, elem)
    _same(per.values, ref, elem)
    for name in ("k", "c"):
        scale = sep.dcoef[name].abs().max()
        assert (per.dcoef[name] - sep.dcoef[name]).abs().max() <= 1e-13 * scale
    v0, dk0 = per.values.clone(), per.dcoef["k"].clone()
    per.capture()
    for _ in range(3):
        per.values.zero_()
        per.replay()
        torch.cuda.synchronize()
        per.check()
        assert torch.equal(per.values, v0)
        assert torch.equal(per.dcoef["k"], dk0)
    per.coef["k"].mul_(0.5)
    per.replay()
    torch.cuda.synchronize()
    per.check()
    _same(per.values, _reference(per, elem), elem)


@pytest.mark.parametrize("elem,dim", [(F.ElementTriP2, 2), (F.ElementTetP2, 3)])
def test_persistent_two_pass_form_for_p2(elem, dim):
    """With the family's one-pass sums off (fem_set_onepass 0) the
    persistent launch runs its two-pass form for P2 too: local matrices in
    the cell units, the staging sum in the row units -- the split entry
    points' values (bit for bit for TriP2, within 1e-14 of max|K| for TetP2,
    whose longer tensor sums the compiler may contract differently)."""
    from skfem_gb300 import _native as N
    rng = np.random.default_rng(21)
    if dim == 2:
        meshes, _ = make_batch([5, 12, 3], seed=8)
    else:
        meshes = [F.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3) for n in (3, 2, 4)]
    bb = BatchedBasis(meshes, elem())
    k = torch.tensor(rng.lognormal(0, 0.5, bb.nelems), device="cuda")
    c = torch.tensor(rng.uniform(0.5, 2.0, bb.nelems), device="cuda")
    w = torch.tensor(rng.standard_normal(bb.N), device="cuda")
    u = torch.tensor(rng.standard_normal(bb.N), device="cuda")
    fam = N.FAMILY["TriP2" if dim == 2 else "TetP2"]
    lib = N.lib()
    try:
        lib.fem_set_onepass(fam, 0)
        per = GraphedAssembly(k_laplace_c_mass, bb, {"k": k, "c": c}, w=w, u=u)
        per.run_eager()
        torch.cuda.synchronize()
        per.check()
        ref = _two_pass(per)
    finally:
        lib.fem_set_onepass(fam, 1)
    if elem is F.ElementTetP2:
        assert (per.values - ref).abs().max() <= 1e-14 * ref.abs().max()
    else:
        assert torch.equal(per.values, ref)


def _same(a, b, elem):
    """Bitwise (the one-pass forms of TriP2 / TetP2 add the same terms in
    the same order in both kernels)."""
    assert torch.equal(a, b)


def _reference(ga, elem):
    if elem in (F.ElementTriP2, F.ElementTetP2):
        return _one_pass(ga)
    return _two_pass(ga)


def _one_pass(ga):
    """The CSR values of fem_assemble (the one-pass node-block sum for
    scalar P2 bases)."""
    from skfem_gb300 import _native as N
    b, e = ga.basis, ga.entry
    out = torch.full_like(ga.values, float("nan"))
    staging = torch.empty_like(e.staging)
    N.check(N.lib().fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(ga.c_form),
                                 e.pat.handle, N.ptr(staging), N.ptr(out), None, N.stream_ptr()))
    torch.cuda.synchronize()
    return out


def _two_pass(ga):
    """The CSR values of the split entry points (local kernel on the cached
    geometry, then the staging sum) -- the persistent kernel's order."""
    from skfem_gb300 import _native as N
    b, e = ga.basis, ga.entry
    lib = N.lib()
    out = torch.full_like(ga.values, float("nan"))
    N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(ga.c_form),
                                   e.pat.handle, N.ptr(e.staging), None, 0, b.nelems,
                                   N.stream_ptr()))
    N.check(lib.fem_csr_sum_staged(e.pat.handle, N.ptr(e.staging), N.ptr(out), N.stream_ptr()))
    torch.cuda.synchronize()
    return out


def test_autotune_applies_a_configuration(tmp_path, monkeypatch):
    from skfem_gb300 import autotune
    monkeypatch.setenv("SKFEM_GB300_CACHE", str(tmp_path))
    meshes, ks = make_batch([8, 16], seed=5)
    bb = BatchedBasis(meshes, F.ElementTriP2())
    k = torch.tensor(np.concatenate(ks), device="cuda")
    K0 = k_laplace.assemble(bb, k=k)
    best, timings = autotune.tune(k_laplace, bb, {"k": k}, reps=1)
    assert len(timings) == len(autotune.candidates("TriP2")) and best in [c for _, c in timings]
    K1 = k_laplace.assemble(bb, k=k)
    np.testing.assert_array_equal(K0.data, K1.data)   # launch shape never changes results
    best2, _ = autotune.tune(k_laplace, bb, {"k": k}, reps=1)   # from the cache
    assert best2 == best
