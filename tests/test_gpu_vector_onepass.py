"""The one-pass vector sum (simplex ElementVector bases: the cells' pair
blocks, then one lane per node block contracting the reference tensor and
summing in ascending cell order) against the two-pass path (local matrices
into the staging, then the fixed-order segmented sum) and the oracle.

Bounds: CSR pattern unchanged (it is the pattern's), values within 1e-14 of
max|K| of the two-pass path (the additions are grouped differently:
per-cell blocks first there, straight into the node block here), within the
parity bounds of the oracle (its pattern up to noise-level entries, where
this machine's numpy rounds a mathematically-zero entry differently), and
repeated assemblies bitwise identical."""
import numpy as np
import pytest
import torch

import oracle as O
import skfem_gb300 as F
from skfem_gb300 import _native as N
from skfem_gb300 import helpers as H
from skfem_gb300.models.elasticity import linear_elasticity
from _util import REL_FRO, REL_MAX, csr_diff

pytestmark = pytest.mark.gpu


def _jitter(m, kind, seed, amp=0.2):
    p = np.array(m.p, dtype=np.float64)
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    rng = np.random.default_rng(seed)
    h = float(np.min(np.linalg.norm(p[:, m.t[1]] - p[:, m.t[0]], axis=0)))
    p[:, inner] += rng.uniform(-amp * h, amp * h, size=(p.shape[0], int(inner.sum())))
    return (F.MeshTet if kind == "tet" else F.MeshTri)(p, m.t)


CASES = [
    ("tri", "TriP1", lambda: F.ElementTriP1(), lambda: O.TriP1(), 24),
    ("tri", "TriP2", lambda: F.ElementTriP2(), lambda: O.TriP2(), 16),
    ("tet", "TetP1", lambda: F.ElementTetP1(), lambda: O.TetP1(), 7),
    ("tet", "TetP2", lambda: F.ElementTetP2(), lambda: O.TetP2(), 5),
]


@F.BilinearForm
def elastic_mass(u, v, w):
    return (w.lam * H.div(u) * H.div(v) + w.mu * H.ddot(H.grad(u), H.grad(v))
            + w.mu * H.ddot(H.grad(u), H.transpose(H.grad(v))) + w.rho * H.dot(u, v))


def _mesh(kind, n, seed):
    if kind == "tet":
        m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    else:
        m = F.MeshTri.init_tensor(*(np.linspace(0, 1, n + 1),) * 2)
    return _jitter(m, kind, seed)


def _both_paths(form, b, fam, **kw):
    lib = N.lib()
    one = form.assemble(b, **kw)
    again = form.assemble(b, **kw)
    np.testing.assert_array_equal(one.data, again.data)
    try:
        # the cooperative form of the one-pass sum: the same values bit for bit
        lib.fem_set_onepass(N.FAMILY[fam], 2)
        coop = form.assemble(b, **kw)
        np.testing.assert_array_equal(one.data, coop.data)
        lib.fem_set_onepass(N.FAMILY[fam], 0)
        two = form.assemble(b, **kw)
    finally:
        lib.fem_set_onepass(N.FAMILY[fam], 1)
    np.testing.assert_array_equal(one.indptr, two.indptr)
    np.testing.assert_array_equal(one.indices, two.indices)
    return one, two


@pytest.mark.parametrize("kind,fam,elem,oelem,n", CASES, ids=[c[1] for c in CASES])
def test_vector_elasticity_onepass_vs_two_pass_and_oracle(kind, fam, elem, oelem, n):
    m = _mesh(kind, n, 5)
    b = F.Basis(m, F.ElementVector(elem()))
    form = linear_elasticity(1.0, 0.5)
    one, two = _both_paths(form, b, fam)
    scale = np.abs(two.data).max()
    assert np.abs(one.data - two.data).max() <= 1e-14 * scale
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), kind), O.Vector(oelem()))
    Ko = O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), ob)
    # the oracle runs on this machine's numpy, whose rounding of the
    # mathematically-zero entries of the unjittered boundary cells may
    # differ from the reference platform's: such entries are noise
    same, extra, missing, noise, rf, rm = csr_diff(one.indptr, one.indices, one.data, Ko.indptr,
                                                   Ko.indices, Ko.data, one.shape)
    assert same or noise <= REL_MAX, (extra, missing, noise)
    assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)


@pytest.mark.parametrize("kind,fam,elem,oelem,n", CASES, ids=[c[1] for c in CASES])
def test_vector_fields_and_mass_onepass_vs_two_pass(kind, fam, elem, oelem, n):
    # per-cell lambda, mu and density: every channel of the vector forms,
    # the mass term through the block diagonals
    m = _mesh(kind, n, 6)
    b = F.Basis(m, F.ElementVector(elem()))
    rng = np.random.default_rng(7)
    lam, mu, rho = (rng.lognormal(0.0, 0.5, m.nelements) for _ in range(3))
    kw = {"lam": b.zero_w() + lam[:, None], "mu": b.zero_w() + mu[:, None],
          "rho": b.zero_w() + rho[:, None]}
    one, two = _both_paths(elastic_mass, b, fam, **kw)
    scale = np.abs(two.data).max()
    assert np.abs(one.data - two.data).max() <= 1e-14 * scale


def test_vector_onepass_device_and_host_coefficients_agree():
    # per-cell coefficients given on the device and as the reference's
    # (nelems, nqp) host arrays give the same CSR values bit for bit
    m = _mesh("tet", 4, 8)
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()))
    rng = np.random.default_rng(9)
    lam, mu, rho = (rng.lognormal(0.0, 0.5, m.nelements) for _ in range(3))
    Kh = elastic_mass.assemble(b, lam=b.zero_w() + lam[:, None], mu=b.zero_w() + mu[:, None],
                               rho=b.zero_w() + rho[:, None])
    T = elastic_mass.assemble_torch(b, lam=torch.tensor(lam, device="cuda"),
                                    mu=torch.tensor(mu, device="cuda"),
                                    rho=torch.tensor(rho, device="cuda"))
    np.testing.assert_array_equal(T.values().cpu().numpy(), Kh.data)


def test_vector_onepass_coefficient_checks():
    # the pair-block kernel runs the coefficient checks: a density that
    # became exactly zero on some cells sets FEM_ERR_STALE_PATTERN, a
    # per-point density varying inside a cell FEM_ERR_VARYING
    m = _mesh("tet", 4, 10)
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()))
    rng = np.random.default_rng(11)
    lam, mu, rho = (rng.lognormal(0.0, 0.5, m.nelements) for _ in range(3))
    dev = {k: torch.tensor(v, device="cuda") for k, v in (("lam", lam), ("mu", mu), ("rho", rho))}
    elastic_mass.assemble_torch(b, **dev)
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    nq = b.zero_w().shape[1]
    rho_zero = rho.copy()
    rho_zero[[2, 50, 300]] = 0.0
    rho_vary = np.repeat(rho[:, None], nq, axis=1)
    rho_vary[7, 1] *= 1.5
    lib = N.lib()
    vals = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    for rd, want in ((torch.tensor(rho_zero, device="cuda"), 1 << N.FEM_ERR_STALE_PATTERN),
                     (torch.tensor(rho_vary, device="cuda"), 1 << N.FEM_ERR_VARYING),
                     (dev["rho"], 0)):
        r1 = rd[:, 0].contiguous() if rd.dim() > 1 else rd
        coeffs, ch, c_form = elastic_mass._setup(b, None, {**dev, "rho": r1})
        if rd.dim() > 1:
            c_form.mass = N.FemCoef(c_form.mass.scale, rd.data_ptr(), rd.shape[1])
        status.zero_()
        N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                 entry.pat.handle, N.ptr(entry.staging), N.ptr(vals),
                                 N.ptr(status), N.stream_ptr()))
        torch.cuda.synchronize()
        assert int(status.item()) == want
        del coeffs, ch


@F.BilinearForm
def _k_lap_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


TICKET_CASES = [
    # (mesh kind, family, vector basis, cells per axis): sizes whose node-block
    # sums exceed eight resident waves of work, where the slices come from a
    # ticket instead of a fixed grid stride
    ("tet", "TetP2", True, 28),     # 131,712 cells, vector elasticity
    ("tet", "TetP2", False, 36),    # 279,936 cells, scalar k*Laplace + mass
    ("tri", "TriP2", False, 420),   # 352,800 cells, scalar k*Laplace + mass
]


@pytest.mark.parametrize("kind,fam,vec,n", TICKET_CASES,
                         ids=["vecTetP2", "TetP2", "TriP2"])
def test_onepass_ticket_path_at_size(kind, fam, vec, n):
    """Device assemblies large enough for the node-block sums to take their
    slices from a ticket: the result equals the other one-pass form bit for
    bit (the vector cooperative form on the fixed grid; the scalar form with
    one FMA per step), repeated calls are bitwise identical, and the two-pass
    path agrees within 1e-14 of max|K|."""
    m = _mesh(kind, n, 11)
    elem = (F.ElementTetP2() if kind == "tet" else F.ElementTriP2())
    b = F.Basis(m, F.ElementVector(elem) if vec else elem)
    if vec:
        form, kw = linear_elasticity(1.0, 0.5), {}
    else:
        k = np.random.default_rng(12).lognormal(0, 1, b.nelems)
        form, kw = _k_lap_mass, {"k": torch.from_numpy(k).cuda()}
    lib = N.lib()
    code = N.FAMILY[fam]
    one = form.assemble_torch(b, **kw).values().clone()
    again = form.assemble_torch(b, **kw).values()
    assert torch.equal(one, again)
    try:
        lib.fem_set_onepass(code, 2)
        other = form.assemble_torch(b, **kw).values()
        assert torch.equal(one, other)
        lib.fem_set_onepass(code, 0)
        two = form.assemble_torch(b, **kw).values()
    finally:
        lib.fem_set_onepass(code, 1)
    scale = one.abs().max().item()
    assert (one - two).abs().max().item() <= 1e-14 * scale
