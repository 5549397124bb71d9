"""GPU parity: the CUDA path against scikit-fem's own results (golden
fixtures made by tests/golden/make_golden.py) and against the CPU oracle on
seeded inputs.  Bounds: CSR indptr/indices bit-exact, values within 1e-12
relative Frobenius and 1e-13 * max|K| entrywise, load vectors the same,
repeated runs bitwise identical."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import oracle as O
import skfem_gb300 as F
from skfem_gb300 import helpers as H
from skfem_gb300.models.elasticity import linear_elasticity
from skfem_gb300.models.poisson import laplace, mass, unit_load
from _util import REL_FRO, REL_MAX, csr_diff, golden

pytestmark = pytest.mark.gpu


@F.BilinearForm
def k_laplace_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


@F.BilinearForm
def k_laplace(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v))


@F.BilinearForm
def theta_laplace(u, v, w):
    return w.theta * H.dot(H.grad(u), H.grad(v))


@F.LinearForm
def f_load(v, w):
    return w.f * v


MESH = {3: F.MeshTri, 4: F.MeshTet, 8: F.MeshHex}


def basis_of(g, elem, intorder=None):
    m = MESH[g["t"].shape[0]](g["p"], g["t"])
    return F.Basis(m, elem, intorder=intorder)


def check_matrix(K, g, pattern_exact=True):
    same, extra, missing, noise, rf, rm = csr_diff(
        K.indptr, K.indices, K.data, g["indptr"], g["indices"], g["data"], K.shape)
    assert rf <= REL_FRO, rf
    assert rm <= REL_MAX, rm
    if pattern_exact:
        assert same, "pattern differs: %d extra, %d missing, max |value| %.3g of max|K|" % (
            extra, missing, noise)
    else:
        # entries present on one side only must be rounding noise of
        # mathematically-zero local entries
        assert noise <= REL_MAX, noise


CASES = [
    # name, element factory, form, kwargs builder, exact pattern expected
    ("tri_default_mass", F.ElementTriP1, mass, lambda b, g: {}, True),
    ("tri_p1_laplace", F.ElementTriP1, laplace, lambda b, g: {}, True),
    ("tet_p1_k_laplace_mass", F.ElementTetP1, k_laplace_mass,
     lambda b, g: {"k": b.zero_w() + g["k"][:, None]}, True),
    ("tet_p1_jitter_laplace", F.ElementTetP1, laplace, lambda b, g: {}, True),
    ("tri_p2_k_laplace", F.ElementTriP2, k_laplace,
     lambda b, g: {"k": b.zero_w() + g["k"][:, None]}, True),
    ("tet_p2_laplace", F.ElementTetP2, laplace, lambda b, g: {}, True),
    ("tet_p2_vec_elasticity", lambda: F.ElementVector(F.ElementTetP2()),
     linear_elasticity(1.0, 0.5), lambda b, g: {}, True),
    ("hex1_theta_laplace", F.ElementHex1, theta_laplace,
     lambda b, g: {"theta": b.zero_w() + g["theta"][:, None]}, True),
    ("hex1_laplace_8", F.ElementHex1, laplace, lambda b, g: {}, True),
]


@pytest.mark.parametrize("name,elem,form,kw,exact", CASES, ids=[c[0] for c in CASES])
def test_matrix_vs_reference_values(name, elem, form, kw, exact):
    """Values within tolerance; entries present on one side only are noise."""
    g = golden(name)
    b = basis_of(g, elem(), intorder=4 if name == "tet_p2_vec_elasticity" else None)
    K = form.assemble(b, **kw(b, g))
    check_matrix(K, g, pattern_exact=False)


@pytest.mark.parametrize("name,elem,form,kw,exact", CASES, ids=[c[0] for c in CASES])
def test_matrix_vs_reference_pattern(name, elem, form, kw, exact):
    """indptr / indices bit-exact against scikit-fem."""
    g = golden(name)
    b = basis_of(g, elem(), intorder=4 if name == "tet_p2_vec_elasticity" else None)
    K = form.assemble(b, **kw(b, g))
    check_matrix(K, g, pattern_exact=True)


@pytest.mark.parametrize("name,elem,form,kw", [
    ("tri_p1_laplace", F.ElementTriP1, unit_load, lambda b, g: {}),
    ("tet_p1_k_laplace_mass", F.ElementTetP1, f_load, lambda b, g: {"f": b.zero_w() + g["k"][:, None]}),
    ("tri_p2_k_laplace", F.ElementTriP2, unit_load, lambda b, g: {}),
    ("tet_p2_laplace", F.ElementTetP2, unit_load, lambda b, g: {}),
    ("hex1_theta_laplace", F.ElementHex1, f_load, lambda b, g: {"f": b.zero_w() + g["theta"][:, None]}),
    ("hex1_laplace_8", F.ElementHex1, unit_load, lambda b, g: {}),
])
def test_load_vector_vs_reference(name, elem, form, kw):
    g = golden(name)
    b = basis_of(g, elem())
    vec = form.assemble(b, **kw(b, g))
    ref = g["b"]
    assert np.linalg.norm(vec - ref) <= REL_FRO * np.linalg.norm(ref)
    assert np.max(np.abs(vec - ref)) <= REL_MAX * np.max(np.abs(ref))


def test_repeated_runs_bitwise_identical():
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 13),) * 3)
    b = F.Basis(m, F.ElementTetP1())
    k = np.random.default_rng(1).lognormal(0, 1, m.nelements)
    kw = {"k": b.zero_w() + k[:, None]}
    K1 = k_laplace_mass.assemble(b, **kw)
    K2 = k_laplace_mass.assemble(b, **kw)
    assert np.array_equal(K1.data, K2.data)
    T = k_laplace_mass.assemble_torch(b, **kw)
    assert torch.equal(T.values().cpu(), torch.from_numpy(K1.data))


def _oracle_case(kind, n, elem_o, elem_p, seed, jitter=0.0):
    rng = np.random.default_rng(seed)
    if kind == "tri":
        m = O.mesh_tri_tensor(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1))
    elif kind == "tet":
        m = O.mesh_tet_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    else:
        m = O.mesh_hex_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    if jitter:
        p = m.p.copy()
        inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
        p[:, inner] += rng.uniform(-jitter / n, jitter / n, size=(p.shape[0], int(inner.sum())))
        m = O.OMesh(p, m.t, m.kind)
    bo = O.OBasis(m, elem_o)
    bp = F.Basis(MESH[m.t.shape[0]](m.p, m.t), elem_p)
    return m, bo, bp, rng


@pytest.mark.parametrize("kind,n,eo,ep,jit", [
    ("tri", 40, O.TriP1(), F.ElementTriP1(), 0.25),
    ("tri", 24, O.TriP2(), F.ElementTriP2(), 0.25),
    ("tet", 10, O.TetP1(), F.ElementTetP1(), 0.2),
    ("tet", 5, O.TetP2(), F.ElementTetP2(), 0.2),
    ("hex", 6, O.Hex1(), F.ElementHex1(), 0.2),
])
def test_k_laplace_mass_vs_oracle(kind, n, eo, ep, jit):
    m, bo, bp, rng = _oracle_case(kind, n, eo, ep, 7, jit)
    k = rng.lognormal(0, 1, m.nelements)
    c = rng.uniform(0.5, 2.0, m.nelements)
    Ko = O.bilinear_assemble(lambda u, v, w: w["k"] * O.dot(O.grad(u), O.grad(v))
                             + w["c"] * (u * v), bo,
                             k=bo.zero_w() + k[:, None], c=bo.zero_w() + c[:, None])

    @F.BilinearForm
    def form(u, v, w):
        return w.k * H.dot(H.grad(u), H.grad(v)) + w.c * u * v

    Kp = form.assemble(bp, k=bp.zero_w() + k[:, None], c=bp.zero_w() + c[:, None])
    same, extra, missing, noise, rf, rm = csr_diff(Kp.indptr, Kp.indices, Kp.data, Ko.indptr,
                                                   Ko.indices, Ko.data, Kp.shape)
    assert same and rf <= REL_FRO and rm <= REL_MAX, (extra, missing, rf, rm)
    bo_ = O.linear_assemble(O.f_load, bo, f=bo.zero_w() + k[:, None])
    bp_ = f_load.assemble(bp, f=bp.zero_w() + k[:, None])
    assert np.max(np.abs(bp_ - bo_)) <= REL_MAX * np.max(np.abs(bo_))


def test_vector_elasticity_vs_oracle():
    m, bo, bp, rng = _oracle_case("tet", 4, O.Vector(O.TetP2()),
                                  F.ElementVector(F.ElementTetP2()), 3, 0.2)
    Ko = O.bilinear_assemble(O.linear_elasticity(2.0, 0.7), bo)
    Kp = linear_elasticity(2.0, 0.7).assemble(bp)
    same, extra, missing, noise, rf, rm = csr_diff(Kp.indptr, Kp.indices, Kp.data, Ko.indptr,
                                                   Ko.indices, Ko.data, Kp.shape)
    assert rf <= REL_FRO and rm <= REL_MAX and noise <= REL_MAX, (rf, rm, noise)


def test_hex1_adjoint_vs_reference_oracles():
    """d(w^T K(theta, X) u)/d theta and /d X against Functional.elemental and
    central differences (h = 1e-6) of the reference's assemble (4^3 cells)."""
    from skfem_gb300.autodiff import assemble_vjp
    g = golden("hex1_theta_laplace")
    b = basis_of(g, F.ElementHex1())
    theta = torch.tensor(g["theta"], device="cuda", requires_grad=True)
    X = torch.tensor(g["p"], device="cuda", requires_grad=True)
    w = torch.tensor(g["wv"], device="cuda")
    u = torch.tensor(g["uv"], device="cuda")
    J = assemble_vjp(theta_laplace, b, w, u, X=X, theta=theta)
    J.backward()
    np.testing.assert_allclose(theta.grad.cpu().numpy(), g["dtheta"], rtol=1e-12, atol=1e-14)
    # FD reference has truncation + cancellation error ~1e-8 relative
    dX = X.grad.cpu().numpy()
    assert np.max(np.abs(dX - g["dX"])) <= 1e-6 * np.max(np.abs(g["dX"]))


def test_hex1_load_adjoint_vs_fd():
    from skfem_gb300.autodiff import assemble_linear_vjp
    g = golden("hex1_theta_laplace")
    b = basis_of(g, F.ElementHex1())
    f = torch.tensor(g["theta"], device="cuda", requires_grad=True)
    X = torch.tensor(g["p"], device="cuda", requires_grad=True)
    w = torch.tensor(g["wv"], device="cuda")
    J = assemble_linear_vjp(f_load, b, w, X=X, f=f)
    J.backward()
    dX = X.grad.cpu().numpy()
    assert np.max(np.abs(dX - g["dXb"])) <= 1e-6 * np.max(np.abs(g["dXb"]))


@pytest.mark.parametrize("kind,n,eo,ep", [
    ("tri", 4, O.TriP1(), F.ElementTriP1()),
    ("tri", 3, O.TriP2(), F.ElementTriP2()),
    ("tet", 2, O.TetP1(), F.ElementTetP1()),
    ("tet", 2, O.TetP2(), F.ElementTetP2()),
    ("hex", 2, O.Hex1(), F.ElementHex1()),
])
def test_simplex_and_hex_adjoint_vs_fd(kind, n, eo, ep):
    from skfem_gb300.autodiff import assemble_vjp
    m, bo, bp, rng = _oracle_case(kind, n, eo, ep, 11, 0.2)
    k = rng.uniform(0.5, 2.0, m.nelements)
    c = rng.uniform(0.5, 2.0, m.nelements)
    wv = rng.standard_normal(bo.N)
    uv = rng.standard_normal(bo.N)

    def form_o(u, v, w):
        return w["k"] * O.dot(O.grad(u), O.grad(v)) + w["c"] * (u * v)

    def J_of(p):
        bb = O.OBasis(O.OMesh(p, m.t, m.kind), eo)
        K = O.bilinear_assemble(form_o, bb, k=bb.zero_w() + k[:, None], c=bb.zero_w() + c[:, None])
        return wv @ (K @ uv)

    dX_fd = O.fd_x_gradient(J_of, m.p, 1e-6)

    @F.BilinearForm
    def form(u, v, w):
        return w.k * H.dot(H.grad(u), H.grad(v)) + w.c * u * v

    kt = torch.tensor(k, device="cuda", requires_grad=True)
    ct = torch.tensor(c, device="cuda", requires_grad=True)
    X = torch.tensor(m.p, device="cuda", requires_grad=True)
    J = assemble_vjp(form, bp, torch.tensor(wv, device="cuda"), torch.tensor(uv, device="cuda"),
                     X=X, k=kt, c=ct)
    assert abs(J.item() - J_of(m.p)) <= 1e-12 * abs(J_of(m.p)) + 1e-14
    J.backward()
    assert np.max(np.abs(X.grad.cpu().numpy() - dX_fd)) <= 1e-6 * np.max(np.abs(dX_fd))
    # coefficient gradients: exact (local quadratic forms)
    dk = O.theta_gradient(O.laplace, bo, wv, uv)
    dc = O.theta_gradient(O.mass, bo, wv, uv)
    np.testing.assert_allclose(kt.grad.cpu().numpy(), dk, rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(ct.grad.cpu().numpy(), dc, rtol=1e-11, atol=1e-13)


def test_zero_jacobian_raises_like_reference():
    """mapping_isoparametric.py:195-196: a degenerate hexahedron raises."""
    m = F.MeshHex()
    p = m.p.copy()
    p[2, :] = 0.0  # flatten the cell: detDF == 0 at every quadrature point
    m = F.MeshHex(p, m.t)
    b = F.Basis(m, F.ElementHex1())
    with pytest.raises(Exception, match="Zero Jacobian determinant"):
        laplace.assemble(b)


def test_errors_match_reference_types():
    b = F.Basis(F.MeshTri(), F.ElementTriP1())
    with pytest.raises(ValueError):
        k_laplace.assemble(b, k=np.zeros((b.nelems, 7)))     # quadrature mismatch
    with pytest.raises(ValueError):
        k_laplace.assemble(b, k=np.zeros(b.N + 1))            # wrong DOF-vector length
    with pytest.raises(NotImplementedError):
        F.BilinearForm(lambda u, v, w: np.arcsinh(u) * v).assemble(b)
    with pytest.raises(NotImplementedError):
        F.BilinearForm(lambda u, v, w: u * v, dtype=np.complex128)


def test_stale_pattern_is_rebuilt():
    """A coefficient that becomes exactly zero removes entries, as
    eliminate_zeros does in the reference."""
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 5), np.linspace(0, 1, 5))
    b = F.Basis(m, F.ElementTriP1())
    k = np.ones(m.nelements)
    K1 = k_laplace.assemble(b, k=b.zero_w() + k[:, None])
    k[:4] = 0.0
    K2 = k_laplace.assemble(b, k=b.zero_w() + k[:, None])
    bo = O.OBasis(O.OMesh(m.p, m.t, "tri"), O.TriP1())
    Ko = O.bilinear_assemble(O.k_laplace, bo, k=bo.zero_w() + k[:, None])
    assert K2.nnz < K1.nnz
    np.testing.assert_array_equal(K2.indptr, Ko.indptr)
    np.testing.assert_array_equal(K2.indices, Ko.indices)


def test_element_subsets_vs_reference():
    """CellBasis(elements=...) (cell_basis.py:94-99): a callable on cell
    midpoints and an index array, against scikit-fem's own results."""
    g = golden("tri_p2_subset")
    b = F.Basis(F.MeshTri(g["p"], g["t"]), F.ElementTriP2(), elements=lambda x: x[0] < 0.5)
    np.testing.assert_array_equal(b.tind, g["tind"])
    check_matrix(k_laplace.assemble(b, k=b.zero_w() + g["k"][:, None]), g)
    vec = unit_load.assemble(b)
    assert np.max(np.abs(vec - g["b"])) <= REL_MAX * np.max(np.abs(g["b"]))
    g = golden("tet_p1_subset")
    b = F.Basis(F.MeshTet(g["p"], g["t"]), F.ElementTetP1(), elements=g["tind"])
    check_matrix(laplace.assemble(b), g)
    vec = unit_load.assemble(b)
    assert np.max(np.abs(vec - g["b"])) <= REL_MAX * np.max(np.abs(g["b"]))


def test_condense_on_device_matches_reference_semantics():
    """utils.condense (utils.py:462-600) on the device CSR: A[I][:, I] and
    b[I] - A[I][:, D] x[D], against scipy applied to the same matrix."""
    from skfem_gb300.utils import condense
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 7),) * 3)
    b = F.Basis(m, F.ElementTetP1())
    rng = np.random.default_rng(2)
    k = rng.lognormal(0, 1, m.nelements)
    A = k_laplace_mass.assemble_torch(b, k=b.zero_w() + k[:, None])
    rhs = torch.tensor(rng.standard_normal(b.N), device="cuda")
    x = torch.tensor(rng.standard_normal(b.N), device="cuda")
    p = m.p
    D = np.nonzero(np.any((p < 1e-12) | (p > 1 - 1e-12), axis=0))[0]
    AII, bI, xr, I = condense(A, rhs, x=x, D=D)
    Ks = k_laplace_mass.assemble(b, k=b.zero_w() + k[:, None])
    Iref = np.setdiff1d(np.arange(b.N), D)
    Aref = Ks[Iref][:, Iref].tocsr()
    bref = rhs.cpu().numpy()[Iref] - Ks[Iref][:, D] @ x.cpu().numpy()[D]
    np.testing.assert_array_equal(AII.crow_indices().cpu().numpy(), Aref.indptr)
    np.testing.assert_array_equal(AII.col_indices().cpu().numpy(), Aref.indices)
    np.testing.assert_array_equal(AII.values().cpu().numpy(), Aref.data)
    np.testing.assert_allclose(bI.cpu().numpy(), bref, rtol=1e-13, atol=1e-13 * np.abs(bref).max())
    np.testing.assert_array_equal(I.cpu().numpy(), Iref)
    # only A: the reference returns the matrix alone when b is None and expand=False
    assert isinstance(condense(A, D=D, expand=False), torch.Tensor)
    # the same sets given as I, as a boolean mask, as a device tensor, with
    # duplicates: the same condensed system
    mask = np.zeros(b.N, dtype=bool)
    mask[D] = True
    for kw in ({"I": Iref}, {"D": mask}, {"D": torch.as_tensor(D, device="cuda")},
               {"D": np.concatenate([D, D[:5]])}):
        A2, b2, _, I2 = condense(A, rhs, x=x, **kw)
        np.testing.assert_array_equal(A2.values().cpu().numpy(), Aref.data)
        np.testing.assert_array_equal(b2.cpu().numpy(), bI.cpu().numpy())
        np.testing.assert_array_equal(I2.cpu().numpy(), Iref)
    # x without b: b is zero, as the reference's _init_bc makes it
    A3, b3 = condense(A, x=x, D=D, expand=False)
    b3ref = -(Ks[Iref][:, D] @ x.cpu().numpy()[D])
    np.testing.assert_allclose(b3.cpu().numpy(), b3ref, rtol=1e-13,
                               atol=1e-13 * np.abs(b3ref).max())
    # indices outside the matrix are refused on the host side
    for bad in (np.array([0, b.N]), np.array([-1, 3])):
        with pytest.raises(IndexError):
            condense(A, rhs, D=bad)
    with pytest.raises(Exception, match="Give only I or only D"):
        condense(A, rhs, I=Iref, D=D)


def test_host_coefficients_checked_in_kernel():
    """assemble() with (nelems, nqp) host coefficient arrays: the rows are
    checked inside the local kernel and the values stream to pinned host
    memory by row ranges -- the same bits as the device-resident call; a row
    that varies inside a cell falls back to the generic kernels."""
    g = golden("tet_p1_k_laplace_mass")
    b = basis_of(g, F.ElementTetP1())
    kw = b.zero_w() + g["k"][:, None]
    K1 = k_laplace_mass.assemble(b, k=kw)
    K2 = k_laplace_mass.assemble_torch(b, k=torch.as_tensor(g["k"], device="cuda"))
    np.testing.assert_array_equal(K1.indptr, K2.crow_indices().cpu().numpy())
    np.testing.assert_array_equal(K1.indices, K2.col_indices().cpu().numpy())
    np.testing.assert_array_equal(K1.data, K2.values().cpu().numpy())
    check_matrix(K1, g)
    kv = kw.copy()
    kv[5, 2] *= 3.0
    kv[40, 0] = 0.0
    Kv = k_laplace_mass.assemble(b, k=kv)
    bo = O.OBasis(O.OMesh(g["p"], g["t"], "tet"), O.TetP1())
    Ko = O.bilinear_assemble(O.k_laplace_mass, bo, k=kv)
    same, extra, missing, noise, rf, rm = csr_diff(Kv.indptr, Kv.indices, Kv.data, Ko.indptr,
                                                   Ko.indices, Ko.data, Kv.shape)
    assert same and rf <= REL_FRO and rm <= REL_MAX, (extra, missing, rf, rm)
    # the plain call afterwards is back on the channel kernels
    K3 = k_laplace_mass.assemble(b, k=kw)
    np.testing.assert_array_equal(K3.data, K1.data)


def test_enforce_on_device_matches_reference_semantics():
    """enforce (utils.py:327-400): rows D zero with 1 on the diagonal,
    entries kept as stored zeros, b[D] = x[D] -- compared with scipy doing the
    same on the host copy."""
    from skfem_gb300.utils import enforce
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 9), np.linspace(0, 1, 7))
    b = F.Basis(m, F.ElementTriP2())
    A = laplace.assemble_torch(b)
    rhs = unit_load.assemble_torch(b)
    D = np.unique(b.element_dofs[:, :5])
    x = np.arange(b.N, dtype=np.float64)
    Ae, be = enforce(A, rhs, x=x, D=D)
    Ah = laplace.assemble(b).tolil()
    for r in D:
        Ah[r, :] = 0.0
        Ah[r, r] = 1.0
    Ah = Ah.tocsr()
    Ae_h = sp.csr_matrix((Ae.values().cpu().numpy(), Ae.col_indices().cpu().numpy(),
                          Ae.crow_indices().cpu().numpy()), shape=Ah.shape)
    np.testing.assert_array_equal(Ae_h.toarray(), Ah.toarray())
    assert Ae._nnz() == A._nnz()                              # pattern kept
    bh = unit_load.assemble(b)
    bh[D] = x[D]
    np.testing.assert_array_equal(be.cpu().numpy(), bh)
    # a mass matrix as b: its rows D are zeroed with a zero diagonal
    M = mass.assemble_torch(b)
    _, Me = enforce(A, M, D=D)
    Mh = Me.to_dense().cpu().numpy()
    assert np.all(Mh[D] == 0.0)


def test_poisson_solve_as_users_write_it():
    """ex01-style: assemble on the GPU, condense on the device with the
    boundary DOFs of get_dofs, solve with scipy; the solution equals the
    reference's own solve."""
    import scipy.sparse.linalg as spla
    from skfem_gb300.utils import condense
    g = golden("poisson_tri_p2")
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 33), np.linspace(0, 1, 33))
    b = F.Basis(m, F.ElementTriP2())
    A = laplace.assemble_torch(b)
    f = unit_load.assemble_torch(b)
    D = b.get_dofs()
    AII, fI, x, I = condense(A, f, D=D)
    Kh = sp.csr_matrix((AII.values().cpu().numpy(), AII.col_indices().cpu().numpy(),
                        AII.crow_indices().cpu().numpy()), shape=AII.shape)
    u = np.zeros(b.N)
    u[I.cpu().numpy()] = spla.spsolve(Kh.tocsc(), fI.cpu().numpy())
    np.testing.assert_allclose(u, g["u"], rtol=0, atol=1e-12)


def test_device_csr_feeds_a_device_solver():
    """The device CSR goes to a solver without a host copy: condensed on the
    device, handed over by DLPack (what CuPy / cuDSS-style consumers take)
    and solved by conjugate gradients on the GPU; the solution equals the
    reference's own solve."""
    from torch.utils.dlpack import from_dlpack, to_dlpack
    from skfem_gb300.utils import condense
    g = golden("poisson_tri_p2")
    m = F.MeshTri.init_tensor(np.linspace(0, 1, 33), np.linspace(0, 1, 33))
    b = F.Basis(m, F.ElementTriP2())
    A = laplace.assemble_torch(b)
    f = unit_load.assemble_torch(b)
    AII, fI, x, I = condense(A, f, D=b.get_dofs())
    crow, col, val = AII.crow_indices(), AII.col_indices(), AII.values()
    assert crow.dtype == torch.int32 and col.dtype == torch.int32 and val.dtype == torch.float64
    assert crow.is_cuda and col.is_cuda and val.is_cuda
    # the consumer's view: the same device arrays, no copy
    crow2, col2, val2 = (from_dlpack(to_dlpack(t)) for t in (crow, col, val))
    assert (crow2.data_ptr(), col2.data_ptr(), val2.data_ptr()) == \
        (crow.data_ptr(), col.data_ptr(), val.data_ptr())
    K = torch.sparse_csr_tensor(crow2, col2, val2, size=AII.shape)
    u = torch.zeros_like(fI)
    r = fI.clone()
    p = r.clone()
    rr = torch.dot(r, r)
    for _ in range(2000):
        Kp = torch.mv(K, p)
        alpha = rr / torch.dot(p, Kp)
        u += alpha * p
        r -= alpha * Kp
        rr_new = torch.dot(r, r)
        if float(rr_new.sqrt()) <= 1e-14 * float(fI.norm()):
            break
        p = r + (rr_new / rr) * p
        rr = rr_new
    full = np.zeros(b.N)
    full[I.cpu().numpy()] = u.cpu().numpy()
    np.testing.assert_allclose(full, g["u"], rtol=0, atol=1e-11)


@pytest.mark.parametrize("name", ["unused_node", "single", "empty_subset"])
def test_edge_cases(name):
    """A node no cell uses (no DOF: the reference numbers DOFs up to
    max(t)), a single cell and an empty element subset, through the public
    API on both paths: CSR and load vector as the reference's."""
    g = {k[len(name) + 1:]: v for k, v in golden("edge_cases").items()
         if k.startswith(name + "_")}
    m = F.MeshTet(g["p"], g["t"])
    b = F.Basis(m, F.ElementTetP1(), elements=np.array([], dtype=np.int64)
                if name == "empty_subset" else None)
    assert b.N == int(g["N"])
    kw = {"k": b.zero_w() + g["k"][:, None]}
    for K in (k_laplace_mass.assemble(b, **kw),
              _host(k_laplace_mass.assemble_torch(b, k=torch.as_tensor(g["k"], device="cuda")))):
        assert K.shape == tuple(g["shape"])
        np.testing.assert_array_equal(K.indptr, g["indptr"])
        np.testing.assert_array_equal(K.indices, g["indices"])
        if len(g["data"]):
            *_, fro, mx = csr_diff(K.indptr, K.indices, K.data, g["indptr"], g["indices"],
                                   g["data"], K.shape)
            assert fro <= REL_FRO and mx <= REL_MAX
    np.testing.assert_allclose(unit_load.assemble(b), g["b"], rtol=1e-13, atol=0)


def _host(T):
    return sp.csr_matrix((T.values().cpu().numpy(), T.col_indices().cpu().numpy(),
                          T.crow_indices().cpu().numpy()), shape=tuple(T.shape))


def test_single_tri_p2_cell():
    g = {k[len("tri2_single_"):]: v for k, v in golden("edge_cases").items()
         if k.startswith("tri2_single_")}
    mt = F.MeshTri()
    b = F.Basis(F.MeshTri(mt.p[:, mt.t[:, 0]], np.arange(3).reshape(3, 1)), F.ElementTriP2())
    K = laplace.assemble(b)
    np.testing.assert_array_equal(K.indptr, g["indptr"])
    np.testing.assert_array_equal(K.indices, g["indices"])
    *_, fro, mx = csr_diff(K.indptr, K.indices, K.data, g["indptr"], g["indices"], g["data"],
                           K.shape)
    assert fro <= REL_FRO and mx <= REL_MAX


def test_empty_cell_and_facet_sets():
    """No cells / no facets on every path, as the reference: an (N, N)
    matrix without entries, a zero load, a functional of 0.0."""
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 3),) * 3)
    none = np.array([], dtype=np.int64)

    @F.BilinearForm
    def gx(u, v, w):
        return (1 + w.x[0]) * H.dot(H.grad(u), H.grad(v))

    @F.Functional
    def fx(w):
        return w.x[0]

    b = F.Basis(m, F.ElementTetP1(), elements=none)
    for K in (gx.assemble(b), k_laplace_mass.assemble(b, k=b.zero_w())):
        assert K.shape == (27, 27) and K.nnz == 0
    assert fx.assemble(b) == 0.0
    np.testing.assert_array_equal(unit_load.assemble(b), np.zeros(27))
    fb = F.FacetBasis(m, F.ElementTetP1(), facets=none)
    K = gx.assemble(fb)
    assert K.shape == (27, 27) and K.nnz == 0
    assert fx.assemble(fb) == 0.0
    bv = F.Basis(m, F.ElementVector(F.ElementTetP2()), elements=none)
    K = linear_elasticity(1.0, 0.5).assemble(bv)
    assert K.shape == (375, 375) and K.nnz == 0


PATCH_CASES = [
    # (mesh, element, exact harmonic functions the element reproduces)
    (lambda: F.MeshTri.init_tensor(*(np.linspace(0, 1, 9),) * 2), F.ElementTriP1,
     [lambda x: 1 + x[0] + 2 * x[1]]),
    (lambda: F.MeshTri.init_tensor(*(np.linspace(0, 1, 9),) * 2), F.ElementTriP2,
     [lambda x: 1 + x[0] * x[1], lambda x: x[0] ** 2 - x[1] ** 2 + x[0]]),
    (lambda: F.MeshTet.init_tensor(*(np.linspace(0, 1, 5),) * 3), F.ElementTetP1,
     [lambda x: 1 + x[0] - x[1] + 3 * x[2]]),
    (lambda: F.MeshTet.init_tensor(*(np.linspace(0, 1, 5),) * 3), F.ElementTetP2,
     [lambda x: 1 + x[0] * x[1] + x[1] * x[2], lambda x: x[0] ** 2 - x[2] ** 2]),
    (lambda: F.MeshHex.init_tensor(*(np.linspace(0, 1, 9),) * 3), F.ElementHex1,
     [lambda x: 1 + x[0] * x[1] * x[2], lambda x: 1 + x[0] * x[1] + x[1] * x[2] + x[0]]),
]


@pytest.mark.parametrize("mesh,elem,funs", PATCH_CASES,
                         ids=[c[1].__name__ for c in PATCH_CASES])
def test_patch_exact_solutions(mesh, elem, funs):
    """tests/test_manufactured.py:142-232 of the reference: Laplace with the
    exact values of a harmonic function the element holds on the boundary
    reproduces it inside to 1e-10."""
    import scipy.sparse.linalg as spla
    b = F.Basis(mesh(), elem())
    A = laplace.assemble(b)
    D = b.get_dofs().all()
    I = b.complement_dofs(D)
    for fun in funs:
        x = fun(b.doflocs)
        u = x.copy()
        u[I] = spla.spsolve(A[I][:, I].tocsc(), -(A[I][:, D] @ x[D]))
        assert np.max(np.abs(u - x)) <= 1e-10


@pytest.mark.parametrize("elem,rate", [(F.ElementTriP1, 2.0), (F.ElementTriP2, 3.0)],
                         ids=["TriP1", "TriP2"])
def test_convergence_rate(elem, rate):
    """tests/test_convergence.py of the reference, on the GPU path end to
    end: -lap u = f with u = sin(pi x) sin(pi y) (a load of w.x, the generic
    kernels), the L2 error by a Functional of the interpolated solution;
    the rate over three halvings of h is the element's."""
    import scipy.sparse.linalg as spla

    @F.LinearForm
    def load(v, w):
        x = w.x
        return 2 * np.pi ** 2 * np.sin(np.pi * x[0]) * np.sin(np.pi * x[1]) * v

    @F.Functional
    def l2err(w):
        x = w.x
        return (w["uh"] - np.sin(np.pi * x[0]) * np.sin(np.pi * x[1])) ** 2

    errs, hs = [], []
    for n in (8, 16, 32):
        m = F.MeshTri.init_tensor(*(np.linspace(0, 1, n + 1),) * 2)
        b = F.Basis(m, elem(), intorder=6)
        A = laplace.assemble(b)
        f = load.assemble(b)
        D = b.get_dofs().all()
        I = b.complement_dofs(D)
        u = np.zeros(b.N)
        u[I] = spla.spsolve(A[I][:, I].tocsc(), f[I])
        errs.append(np.sqrt(l2err.assemble(b, uh=b.interpolate(u))))
        hs.append(1.0 / n)
    rates = np.log(np.array(errs[:-1]) / np.array(errs[1:])) / np.log(2.0)
    assert np.all(np.abs(rates - rate) < 0.15), rates
