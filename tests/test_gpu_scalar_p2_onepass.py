"""The one-pass node-block sum on scalar TriP2 / TetP2 bases (per cell the
numbers k_e |det| / d! grad(lambda_p) . grad(lambda_q) and m_e |det| / d!,
then one lane per CSR entry on and above the diagonal contracting the
element's reference tensor while it sums its cells in ascending order)
against the two-pass path (local matrices into the staging, then the
fixed-order segmented sum) and the oracle.

Bounds: CSR pattern unchanged (it is the pattern's), values within 1e-14 of
max|K| of the two-pass path (the products are grouped differently), within
the parity bounds of the oracle (its pattern up to noise-level entries, where
this machine's numpy rounds a mathematically-zero entry differently), and
repeated assemblies bitwise identical."""
import numpy as np
import pytest
import torch

import oracle as O
import skfem_gb300 as F
from skfem_gb300 import _native as N
from skfem_gb300 import helpers as H
from _util import REL_FRO, REL_MAX, csr_diff

pytestmark = pytest.mark.gpu


@F.BilinearForm
def k_laplace_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


@F.BilinearForm
def k_laplace(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v))


@F.BilinearForm
def k_laplace_rho_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + w.rho * u * v


CASES = [
    ("tri", "TriP2", lambda: F.ElementTriP2(), lambda: O.TriP2(), 20),
    ("tet", "TetP2", lambda: F.ElementTetP2(), lambda: O.TetP2(), 6),
]


def _mesh(kind, n, seed, amp=0.2):
    if kind == "tet":
        m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
    else:
        m = F.MeshTri.init_tensor(*(np.linspace(0, 1, n + 1),) * 2)
    if amp == 0.0:
        return m
    p = np.array(m.p, dtype=np.float64)
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    rng = np.random.default_rng(seed)
    h = float(np.min(np.linalg.norm(p[:, m.t[1]] - p[:, m.t[0]], axis=0)))
    p[:, inner] += rng.uniform(-amp * h, amp * h, size=(p.shape[0], int(inner.sum())))
    return (F.MeshTet if kind == "tet" else F.MeshTri)(p, m.t)


def _both_paths(form, b, fam, **kw):
    lib = N.lib()
    one = form.assemble(b, **kw)
    again = form.assemble(b, **kw)
    np.testing.assert_array_equal(one.data, again.data)
    try:
        # the flattened form of the sum (one FMA per step): the same bits
        lib.fem_set_onepass(N.FAMILY[fam], 2)
        flat = form.assemble(b, **kw)
        np.testing.assert_array_equal(one.data, flat.data)
        lib.fem_set_onepass(N.FAMILY[fam], 0)
        two = form.assemble(b, **kw)
    finally:
        lib.fem_set_onepass(N.FAMILY[fam], 1)
    np.testing.assert_array_equal(one.indptr, two.indptr)
    np.testing.assert_array_equal(one.indices, two.indices)
    scale = np.abs(two.data).max()
    assert np.abs(one.data - two.data).max() <= 1e-14 * scale
    return one, two


def _oracle_parity(K, m, kind, oelem, oform, **kw):
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), kind), oelem())
    okw = {k: ob.zero_w() + v[:, None] for k, v in kw.items()}
    Ko = O.bilinear_assemble(oform, ob, **okw)
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, Ko.indptr,
                                                   Ko.indices, Ko.data, K.shape)
    assert same or noise <= REL_MAX, (extra, missing, noise)
    assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)


@pytest.mark.parametrize("kind,fam,elem,oelem,n", CASES, ids=[c[1] for c in CASES])
@pytest.mark.parametrize("amp", [0.0, 0.2], ids=["regular", "jittered"])
def test_scalar_p2_k_laplace_mass_onepass_vs_two_pass_and_oracle(kind, fam, elem, oelem, n, amp):
    m = _mesh(kind, n, 11, amp)
    b = F.Basis(m, elem())
    k = np.random.default_rng(12).lognormal(0.0, 1.0, m.nelements)
    one, _ = _both_paths(k_laplace_mass, b, fam, k=b.zero_w() + k[:, None])
    _oracle_parity(one, m, kind, oelem, O.k_laplace_mass, k=k)


@pytest.mark.parametrize("kind,fam,elem,oelem,n", CASES, ids=[c[1] for c in CASES])
def test_scalar_p2_stiffness_only_and_mass_field(kind, fam, elem, oelem, n):
    # without a mass term (the sum's MASS = false form), and with a per-cell
    # mass coefficient (a field on the mass channel)
    m = _mesh(kind, n, 13)
    b = F.Basis(m, elem())
    rng = np.random.default_rng(14)
    k, rho = rng.lognormal(0.0, 0.5, m.nelements), rng.lognormal(0.0, 0.5, m.nelements)
    one, _ = _both_paths(k_laplace, b, fam, k=b.zero_w() + k[:, None])
    _oracle_parity(one, m, kind, oelem, O.k_laplace, k=k)
    _both_paths(k_laplace_rho_mass, b, fam, k=b.zero_w() + k[:, None],
                rho=b.zero_w() + rho[:, None])


def test_scalar_p2_device_and_host_coefficients_agree():
    # the device call (pair values from the geometry cache) and the host
    # (nelems, nqp) call (chunked pipeline) give the same values bit for bit
    m = _mesh("tet", 5, 15)
    b = F.Basis(m, F.ElementTetP2())
    k = np.random.default_rng(16).lognormal(0.0, 1.0, m.nelements)
    Kh = k_laplace_mass.assemble(b, k=b.zero_w() + k[:, None])
    T = k_laplace_mass.assemble_torch(b, k=torch.tensor(k, device="cuda"))
    np.testing.assert_array_equal(T.values().cpu().numpy(), Kh.data)
    np.testing.assert_array_equal(T.crow_indices().cpu().numpy(), Kh.indptr)
