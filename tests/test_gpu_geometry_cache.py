"""The per-cell geometry cache of the scalar simplex kernels
(fem_pattern_cache_geometry): assembling from the cache equals assembling
from the coordinates, and a change of the coordinates -- in place or by
replacement -- reaches the next assembly."""
import ctypes

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


def _jittered(cls, n, dim, seed):
    m = cls.init_tensor(*(np.linspace(0, 1, n),) * dim)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p[:, inner] += np.random.default_rng(seed).uniform(-0.2 / n, 0.2 / n, (dim, int(inner.sum())))
    return cls(p, m.t)


CASES = [(F.MeshTri, 2, F.ElementTriP1, 65), (F.MeshTri, 2, F.ElementTriP2, 33),
         (F.MeshTet, 3, F.ElementTetP1, 17), (F.MeshTet, 3, F.ElementTetP2, 9)]


def _uncached(form, b, **kw):
    """The same assembly with the kernels computing the geometry: the mesh
    points at a copy of the coordinates, which the cache does not match."""
    p2 = b.p_dev.clone()
    old = b.c_mesh.p
    b.c_mesh.p = p2.data_ptr()
    try:
        return form.assemble_torch(b, **kw)
    finally:
        b.c_mesh.p = old


@pytest.mark.parametrize("cls,dim,elem,n", CASES, ids=[c[2].__name__ for c in CASES])
def test_cached_geometry_equals_computed(cls, dim, elem, n):
    m = _jittered(cls, n, dim, 0)
    b = F.Basis(m, elem())
    k = torch.from_numpy(np.random.default_rng(1).lognormal(0, 1, m.nelements)).cuda()
    Kc = k_lap_mass.assemble_torch(b, k=k)
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    assert entry.geo_key is not None
    Ku = _uncached(k_lap_mass, b, k=k)
    a, c = Kc.values().cpu().numpy(), Ku.values().cpu().numpy()
    np.testing.assert_array_equal(Kc.col_indices().cpu().numpy(), Ku.col_indices().cpu().numpy())
    assert np.abs(a - c).max() <= 1e-14 * np.abs(c).max()


def test_coordinates_changed_in_place_and_replaced():
    m = _jittered(F.MeshTet, 13, 3, 2)
    b = F.Basis(m, F.ElementTetP1())
    k = torch.from_numpy(np.random.default_rng(3).lognormal(0, 1, m.nelements)).cuda()
    k_lap_mass.assemble_torch(b, k=k)
    # in place: scale the coordinates (the zero structure does not change)
    with torch.no_grad():
        b.p_dev.mul_(1.5)
    K1 = k_lap_mass.assemble_torch(b, k=k)
    ref1 = k_lap_mass.assemble_torch(F.Basis(F.MeshTet(m.p * 1.5, m.t), F.ElementTetP1()), k=k)
    v1, r1 = K1.values().cpu().numpy(), ref1.values().cpu().numpy()
    assert np.abs(v1 - r1).max() <= 1e-13 * np.abs(r1).max()
    # replaced: update_coordinates
    p2 = m.p * 0.75
    b.update_coordinates(p2)
    K2 = k_lap_mass.assemble_torch(b, k=k)
    ref2 = k_lap_mass.assemble_torch(F.Basis(F.MeshTet(p2, m.t), F.ElementTetP1()), k=k)
    v2, r2 = K2.values().cpu().numpy(), ref2.values().cpu().numpy()
    assert np.abs(v2 - r2).max() <= 1e-13 * np.abs(r2).max()


def test_cache_is_a_no_op_for_families_without_one():
    m = F.MeshHex.init_tensor(*(np.linspace(0, 1, 5),) * 3)
    b = F.Basis(m, F.ElementHex1())
    k_lap_mass.assemble_torch(b, k=torch.ones(m.nelements, dtype=torch.float64, device="cuda"))
    entry = next(e for key, e in b._patterns.items() if key[0] == "bilinear")
    assert N.lib().fem_pattern_cache_geometry(entry.pat.handle, N.byref(b.c_mesh),
                                              N.byref(b.c_basis), N.stream_ptr()) == 0
