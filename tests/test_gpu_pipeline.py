"""The host path of BilinearForm.assemble (strided host coefficients, the
pipelined upload / local kernel / row-range sum / copy back in order of the
cells' smallest DOF) against the device path on the same inputs: bit for
bit, on meshes large enough for several chunks, in the reference's cell
order and in a shuffled one."""
import numpy as np
import pytest
import torch

import skfem_gb300 as F
from skfem_gb300 import form as FM
from skfem_gb300 import helpers as H

pytestmark = pytest.mark.gpu


@F.BilinearForm
def k_lap_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


def _mesh(kind, shuffle, seed=0):
    rng = np.random.default_rng(seed)
    if kind == "tet":
        m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 33),) * 3)      # 196,608 cells
        e = F.ElementTetP1()
    elif kind == "tri2":
        m = F.MeshTri.init_tensor(*(np.linspace(0, 1, 257),) * 2)    # 131,072 cells
        e = F.ElementTriP2()
    else:
        m = F.MeshHex.init_tensor(*(np.linspace(0, 1, 33),) * 3)      # 32,768 cells
        e = F.ElementHex1()
    if shuffle:
        t = m.t[:, rng.permutation(m.t.shape[1])]
        m = type(m)(m.p, np.ascontiguousarray(t))
    return m, e


@pytest.mark.parametrize("kind", ["tet", "tri2", "hex"])
@pytest.mark.parametrize("shuffle", [False, True])
def test_host_pipeline_equals_device_path(kind, shuffle):
    m, e = _mesh(kind, shuffle)
    b = F.Basis(m, e)
    k = np.random.default_rng(1).lognormal(0, 1, m.nelements)
    Kd = k_lap_mass.assemble_torch(b, k=torch.from_numpy(k).cuda())
    old = FM.UPLOAD_CHUNKS
    try:
        for chunks in (1, 3, 8, 16):
            FM.UPLOAD_CHUNKS = chunks
            Kh = k_lap_mass.assemble(b, k=b.zero_w() + k[:, None])
            np.testing.assert_array_equal(Kh.indptr, Kd.crow_indices().cpu().numpy())
            np.testing.assert_array_equal(Kh.indices, Kd.col_indices().cpu().numpy())
            np.testing.assert_array_equal(Kh.data, Kd.values().cpu().numpy())
    finally:
        FM.UPLOAD_CHUNKS = old


def test_host_pipeline_varying_rows_fall_back_to_generic():
    """A per-point coefficient varying inside the cells, passed from the host
    at a size with several chunks, takes the generic kernels (the pipeline
    reports FEM_ERR_VARYING) and matches them."""
    m, e = _mesh("tet", False)
    b = F.Basis(m, e)
    rng = np.random.default_rng(2)
    kq = rng.lognormal(0, 1, b.zero_w().shape)
    K = k_lap_mass.assemble(b, k=kq)
    Kg = k_lap_mass.assemble_torch(b, k=torch.from_numpy(kq).cuda())
    np.testing.assert_array_equal(K.indices, Kg.col_indices().cpu().numpy())
    np.testing.assert_array_equal(K.data, Kg.values().cpu().numpy())


def test_host_pipeline_vector_elasticity():
    """Vector TetP2 linear elasticity (no coefficient fields: the pipeline
    runs with no host rows) on 34,992 cells, eight chunks, against the
    device path."""
    from skfem_gb300.models.elasticity import linear_elasticity
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, 19),) * 3)
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()))
    form = linear_elasticity(1.0, 0.5)
    Kd = form.assemble_torch(b)
    Kh = form.assemble(b)
    np.testing.assert_array_equal(Kh.indptr, Kd.crow_indices().cpu().numpy())
    np.testing.assert_array_equal(Kh.indices, Kd.col_indices().cpu().numpy())
    np.testing.assert_array_equal(Kh.data, Kd.values().cpu().numpy())
