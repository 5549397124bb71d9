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
    ref = K.values()
    coeffs, ch, c_form = form._setup(b, None, kw)
    lib = N.lib()
    s = N.stream_ptr()
    vals = torch.full_like(ref, np.nan)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
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
