"""The staging layouts of the channel kernels (full local matrices cell
after cell for scalar bases, block-upper matrices for vector bases): the
split entry points fem_assemble_local + fem_csr_sum_staged give
fem_assemble's values bit for bit, over the whole mesh and cell range by
cell range, in the reference's cell order and in a shuffled one."""
import numpy as np
import pytest
import torch

import skfem_gb300 as F
from skfem_gb300 import _native as N
from skfem_gb300 import helpers as H

pytestmark = pytest.mark.gpu


@F.BilinearForm
def k_lap_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


CASES = {
    "TetP1": (F.MeshTet, 3, 13, F.ElementTetP1, False),
    "Hex1": (F.MeshHex, 3, 9, F.ElementHex1, False),
    "TriP2": (F.MeshTri, 2, 33, F.ElementTriP2, False),
    "TetP1-vector": (F.MeshTet, 3, 9, F.ElementTetP1, True),
}


def _basis(name, shuffle):
    cls, dim, n, elem, vector = CASES[name]
    m = cls.init_tensor(*(np.linspace(0, 1, n),) * dim)
    if shuffle:
        perm = np.random.default_rng(4).permutation(m.t.shape[1])
        m = cls(m.p, np.ascontiguousarray(m.t[:, perm]))
    e = F.ElementVector(elem()) if vector else elem()
    return F.Basis(m, e)


@pytest.mark.parametrize("shuffle", [False, True])
@pytest.mark.parametrize("name", list(CASES))
def test_split_entry_points_equal_fem_assemble(name, shuffle):
    b = _basis(name, shuffle)
    vector = CASES[name][4]
    if vector:
        from skfem_gb300.models.elasticity import linear_elasticity
        form, kw = linear_elasticity(1.0, 0.5), {}
    else:
        k = torch.from_numpy(np.random.default_rng(1).lognormal(0, 1, b.nelems)).cuda()
        form, kw = k_lap_mass, {"k": k}
    K = form.assemble_torch(b, **kw)
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    coeffs, ch, c_form = form._setup(b, None, kw)
    lib = N.lib()
    s = N.stream_ptr()
    # without the geometry cache (and the fused sum it enables), and with the
    # family's one-pass sums off, fem_assemble runs the local kernel and the
    # staging sum, as the split entry points do
    lib.fem_pattern_drop_geometry(entry.pat.handle)
    entry.geo_key = None
    ref = torch.full_like(K.values(), np.nan)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    fam = N.FAMILY[name.split("-")[0]]
    try:
        lib.fem_set_onepass(fam, 0)
        N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                 entry.pat.handle, N.ptr(entry.staging), N.ptr(ref),
                                 N.ptr(status), s))
    finally:
        lib.fem_set_onepass(fam, 1)
    vals = torch.full_like(ref, np.nan)
    # whole mesh
    N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                   entry.pat.handle, N.ptr(entry.staging), N.ptr(status), 0,
                                   b.nelems, s))
    N.check(lib.fem_csr_sum_staged(entry.pat.handle, N.ptr(entry.staging), N.ptr(vals), s))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(vals, ref)
    # three cell ranges into a cleared staging, then one sum
    entry.staging.fill_(np.nan)
    vals.fill_(np.nan)
    cuts = [0, b.nelems // 3, (2 * b.nelems) // 3, b.nelems]
    for c0, c1 in zip(cuts[:-1], cuts[1:]):
        N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                       entry.pat.handle, N.ptr(entry.staging), N.ptr(status),
                                       c0, c1, s))
    N.check(lib.fem_csr_sum_staged(entry.pat.handle, N.ptr(entry.staging), N.ptr(vals), s))
    torch.cuda.synchronize()
    assert torch.equal(vals, ref)
    del coeffs, ch


@F.BilinearForm
def lap_mass_const(u, v, w):
    return 2.5 * H.dot(H.grad(u), H.grad(v)) + 0.75 * u * v


@F.BilinearForm
def mass_only(u, v, w):
    return 3.0 * u * v


FUSED = [(F.MeshTri, 2, 33, F.ElementTriP1), (F.MeshTri, 2, 17, F.ElementTriP2),
         (F.MeshTet, 3, 11, F.ElementTetP1), (F.MeshTet, 3, 7, F.ElementTetP2)]


@F.BilinearForm
def k_lap_cmass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + w.c * u * v


@pytest.mark.parametrize("path", ["default", "coefficient_update"])
@pytest.mark.parametrize("form", ["k_lap_mass", "lap_mass_const", "mass_only", "k_lap_cmass"])
@pytest.mark.parametrize("cls,dim,n,elem", FUSED, ids=[c[3].__name__ for c in FUSED])
def test_one_pass_sums_equal_staging_sum(cls, dim, n, elem, form, path):
    """The one-pass assemblies of scalar simplex forms -- TriP1 / TetP1 by
    default (each CSR row contracting k_e G_e from the geometry cache and
    summing |det_e| in exact fixed point, or m_e |det_e| in FP64 for a mass
    field), and the opt-in coefficient-update cache (K = diff * sum_e k_e S_e
    + mass * M over cached unit-coefficient rows, constant mass only) -- are
    equal to the local kernel plus staging sum within 1e-14 of max|K| (the
    additions are grouped differently), with the same CSR structure, and
    bitwise on reruns."""
    m = cls.init_tensor(*(np.linspace(0, 1, n),) * dim)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += np.random.default_rng(5).uniform(-0.2 / n, 0.2 / n, (dim, int(inner.sum())))
    b = F.Basis(cls(p, m.t), elem())
    f = {"k_lap_mass": k_lap_mass, "lap_mass_const": lap_mass_const, "mass_only": mass_only,
         "k_lap_cmass": k_lap_cmass}[form]
    rng = np.random.default_rng(6)
    kw = {}
    if form in ("k_lap_mass", "k_lap_cmass"):
        kw["k"] = torch.from_numpy(rng.lognormal(0, 1, b.nelems)).cuda()
    if form == "k_lap_cmass":
        kw["c"] = torch.from_numpy(rng.uniform(0.5, 2.0, b.nelems)).cuda()
    if path == "coefficient_update":
        f.cache_coefficient_update(b, **kw)
    Kf = f.assemble_torch(b, **kw)
    Kf2 = f.assemble_torch(b, **kw)
    assert torch.equal(Kf.values(), Kf2.values())
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    coeffs, ch, c_form = f._setup(b, None, kw)
    lib = N.lib()
    lib.fem_pattern_drop_geometry(entry.pat.handle)
    entry.geo_key = None
    entry.coef_update = False
    ref = torch.full_like(Kf.values(), np.nan)
    N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                             entry.pat.handle, N.ptr(entry.staging), N.ptr(ref), None,
                             N.stream_ptr()))
    torch.cuda.synchronize()
    a, r = Kf.values().cpu().numpy(), ref.cpu().numpy()
    assert np.isfinite(r).all()
    assert np.abs(a - r).max() <= 1e-14 * np.abs(r).max()
    del coeffs, ch


@pytest.mark.parametrize("elem,n", [(F.ElementTetP1, 9), (F.ElementTetP2, 5)],
                         ids=["TetP1", "TetP2"])
def test_fused_checks_report_stale_and_varying(elem, n):
    """The coefficient checks of the fused path and of the one-pass sums
    (TetP1: folded into the sum; TetP2: in the pair-value kernel): a
    coefficient that became exactly zero on some cells sets
    FEM_ERR_STALE_PATTERN, a per-point coefficient that varies inside a cell
    sets FEM_ERR_VARYING, and a constant per-point row (with +0.0 / -0.0
    taken as equal) sets neither -- the same bits as the local kernel's
    checks without the cache."""
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n),) * 3)
    b = F.Basis(m, elem())
    rng = np.random.default_rng(7)
    k = rng.lognormal(0, 1, b.nelems)
    k_lap_mass.assemble_torch(b, k=torch.from_numpy(k).cuda())
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    nq = b.zero_w().shape[1]
    k_zero = k.copy()
    k_zero[[3, 17, 200]] = 0.0
    k_vary = np.repeat(k[:, None], nq, axis=1)
    k_vary[5, 1] *= 1.5
    k_signed = np.repeat(k_zero[:, None], nq, axis=1)
    k_signed[3, 2] = -0.0
    cases = [(torch.from_numpy(k_zero).cuda(), 1 << N.FEM_ERR_STALE_PATTERN),
             (torch.from_numpy(k_vary).cuda(), 1 << N.FEM_ERR_VARYING),
             (torch.from_numpy(k_signed).cuda(), 1 << N.FEM_ERR_STALE_PATTERN),
             (torch.from_numpy(k).cuda(), 0)]
    lib = N.lib()
    vals = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    seen = []
    for cached in ("coefficient_update", "geometry", None):
        if cached == "coefficient_update":
            k_lap_mass.cache_coefficient_update(b, k=torch.from_numpy(k).cuda())
        elif cached == "geometry":
            lib.fem_pattern_drop_coefficient_update(entry.pat.handle)
        else:
            lib.fem_pattern_drop_geometry(entry.pat.handle)
            entry.geo_key = None
        for kd, want in cases:
            k1 = kd[:, 0].contiguous() if kd.dim() > 1 else kd
            coeffs, ch, c_form = k_lap_mass._setup(b, None, {"k": k1})
            if kd.dim() > 1:
                # per-point rows (nelems, nqp), as the host path hands them over
                c_form.diff = N.FemCoef(c_form.diff.scale, kd.data_ptr(), kd.shape[1])
            status.zero_()
            N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                     entry.pat.handle, N.ptr(entry.staging), N.ptr(vals),
                                     N.ptr(status), N.stream_ptr()))
            torch.cuda.synchronize()
            seen.append(int(status.item()))
            assert seen[-1] == want, (cached, want, seen[-1])
            del coeffs, ch


COLS = [("TetP1", F.MeshTet, 3, 15, F.ElementTetP1), ("TriP2", F.MeshTri, 2, 41, F.ElementTriP2),
        ("TetP2", F.MeshTet, 3, 8, F.ElementTetP2)]


@pytest.mark.parametrize("form", ["k_lap_mass", "lap_mass_const"])
@pytest.mark.parametrize("fam,cls,dim,n,elem", COLS, ids=[c[0] for c in COLS])
def test_fused_sum_columns_per_lane_are_bitwise_equal(fam, cls, dim, n, elem, form):
    """The coefficient-update cache's fused sum with two columns per lane
    (TetP1, TriP2, TetP2) adds every slot's contributions in the same order
    as the one-column kernel: equal bit for bit for every unroll, on the
    device path and through the pipelined host path, in a shuffled cell
    order."""
    from skfem_gb300 import autotune
    m = cls.init_tensor(*(np.linspace(0, 1, n),) * dim)
    perm = np.random.default_rng(8).permutation(m.t.shape[1])
    b = F.Basis(cls(m.p, np.ascontiguousarray(m.t[:, perm])), elem())
    f = k_lap_mass if form == "k_lap_mass" else lap_mass_const
    k = np.random.default_rng(9).lognormal(0, 1, b.nelems)
    kw = {"k": torch.from_numpy(k).cuda()} if form == "k_lap_mass" else {}
    kh = {"k": b.zero_w() + k[:, None]} if form == "k_lap_mass" else {}
    f.cache_coefficient_update(b, **kw)
    code = N.FAMILY[fam]
    base = {"local_block": 128, "persistent": 0, "sum_unroll": 8, "sum_cols": 1}
    try:
        autotune.apply(code, base)
        ref = f.assemble_torch(b, **kw).values().clone()
        ref_host = f.assemble(b, **kh)
        for unroll in (4, 8, 16):
            autotune.apply(code, dict(base, sum_unroll=unroll, sum_cols=2))
            assert torch.equal(f.assemble_torch(b, **kw).values(), ref)
            Kh = f.assemble(b, **kh)
            np.testing.assert_array_equal(Kh.data, ref_host.data)
        np.testing.assert_array_equal(ref_host.data, ref.cpu().numpy())
    finally:
        autotune.apply(code, base)


P1 = [("TriP1", F.MeshTri, 2, 41, F.ElementTriP1), ("TetP1", F.MeshTet, 3, 13, F.ElementTetP1)]


@pytest.mark.parametrize("form", ["k_lap_mass", "lap_mass_const", "k_lap_cmass"])
@pytest.mark.parametrize("fam,cls,dim,n,elem", P1, ids=[c[0] for c in P1])
def test_one_pass_forms_agree(fam, cls, dim, n, elem, form):
    """The one-pass P1 sum's two forms -- two lanes per row adding into
    shared-memory slots, and a lane per upper entry walking its list in
    registers and writing the entry and its transpose -- add every entry's
    contributions in the same order: on a jittered mesh (cells around a
    vertex within a factor 8 in |det|, so the fixed-point mass sums are
    exact in both) they agree bit for bit, on the device path and through
    the pipelined host path, for every unroll; on a strongly graded mesh
    within 1e-15 of max|K|."""
    from skfem_gb300 import autotune
    code = N.FAMILY[fam]
    f = {"k_lap_mass": k_lap_mass, "lap_mass_const": lap_mass_const,
         "k_lap_cmass": k_lap_cmass}[form]
    base = {"local_block": 128, "persistent": 0, "sum_unroll": 8, "sum_cols": 1, "onepass": 0}
    for graded in (False, True):
        m = cls.init_tensor(*(np.linspace(0, 1, n),) * dim)
        p = m.p.copy()
        if graded:
            p = p ** 4                     # cell sizes over four orders of magnitude
        else:
            inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
            p[:, inner] += np.random.default_rng(3).uniform(-0.2 / n, 0.2 / n,
                                                            (dim, int(inner.sum())))
        perm = np.random.default_rng(8).permutation(m.t.shape[1])
        b = F.Basis(cls(p, np.ascontiguousarray(m.t[:, perm])), elem())
        rng = np.random.default_rng(10)
        k = rng.lognormal(0, 1, b.nelems)
        c = rng.uniform(0.5, 2.0, b.nelems)
        kw, kh = {}, {}
        if form != "lap_mass_const":
            kw["k"] = torch.from_numpy(k).cuda()
            kh["k"] = b.zero_w() + k[:, None]
        if form == "k_lap_cmass":
            kw["c"] = torch.from_numpy(c).cuda()
            kh["c"] = b.zero_w() + c[:, None]
        try:
            autotune.apply(code, base)
            ref = f.assemble_torch(b, **kw).values().clone()
            ref_host = f.assemble(b, **kh).data
            for unroll, variant in ((4, 1), (8, 1), (4, 2), (8, 2)):
                autotune.apply(code, dict(base, sum_unroll=unroll, onepass=variant))
                got = f.assemble_torch(b, **kw).values()
                got_host = f.assemble(b, **kh).data
                if graded:
                    scale = ref.abs().max().item()
                    assert (got - ref).abs().max().item() <= 1e-15 * scale
                    assert np.abs(got_host - ref_host).max() <= 1e-15 * scale
                else:
                    assert torch.equal(got, ref)
                    np.testing.assert_array_equal(got_host, ref_host)
        finally:
            autotune.apply(code, dict(base, onepass=1))


@pytest.mark.parametrize("fam,cls,dim,n,elem", [
    ("TriP1", F.MeshTri, 2, 40, F.ElementTriP1), ("TriP2", F.MeshTri, 2, 30, F.ElementTriP2),
    ("TetP1", F.MeshTet, 3, 12, F.ElementTetP1), ("TetP2", F.MeshTet, 3, 8, F.ElementTetP2)])
def test_local_kernel_tma_staged_geometry_is_bitwise_the_same(fam, cls, dim, n, elem):
    """fem_set_local_tma: the local kernel on the geometry cache with each
    tile's geometry brought in by one 2-D TMA tensor copy writes the same
    local matrices, bit for bit, as with per-thread loads; the status word
    stays clean (no bounded wait ran out)."""
    m = cls.init_tensor(*(np.linspace(0, 1, n),) * dim)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += np.random.default_rng(4).uniform(-0.2 / n, 0.2 / n, (dim, int(inner.sum())))
    b = F.Basis(cls(p, m.t), elem())
    assert b.nelems % 2 == 0                  # the tensor map's row stride
    k = torch.from_numpy(np.random.default_rng(6).lognormal(0, 1, b.nelems)).cuda()
    c = torch.from_numpy(np.random.default_rng(7).uniform(0.5, 2.0, b.nelems)).cuda()
    K = k_lap_cmass.assemble_torch(b, k=k, c=c)
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    c_form = k_lap_cmass._setup(b, None, {"k": k, "c": c})[2]
    lib = N.lib()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")

    def local():
        out = torch.full_like(entry.staging, np.nan)
        N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                       entry.pat.handle, N.ptr(out), N.ptr(status), 0, b.nelems,
                                       N.stream_ptr()))
        torch.cuda.synchronize()
        return out
    ref = local()
    try:
        lib.fem_set_local_tma(N.FAMILY[fam], 1)
        got = local()
    finally:
        lib.fem_set_local_tma(N.FAMILY[fam], 0)
    assert int(status.item()) == 0
    nloc = b.nelems * b.Nbfun * b.Nbfun
    assert torch.equal(got[:nloc], ref[:nloc])
    assert K.values().numel() > 0
