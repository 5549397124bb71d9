"""Rows of high-valence DOFs.  The pattern build gathers a row's candidate
columns (cells sharing the row's DOF x local columns) in one warp's shared
memory, at most 16,384 of them; a vector TetP2 row has 30 candidates per
cell, so a DOF may be shared by at most 546 cells.  At that edge the
assembly must still match the oracle; beyond it the build must refuse the
mesh with a message naming the limit (FEM_ERR_CAPACITY) -- no fault, no
truncated row.  Rows whose shared-memory accumulators do not fit four warps
per block run with fewer warps per block.

The tet mesh is a double cone: a ring of n vertices around the origin, an
apex above and below; every tet (origin, ring_i, ring_i+1, apex) holds the
origin, which is shared by 2n cells.  The triangle mesh is a fan of n
triangles around the origin."""
import numpy as np
import pytest

import oracle as O
import skfem_gb300 as F
from skfem_gb300.models.elasticity import linear_elasticity
from _util import REL_FRO, REL_MAX, csr_diff

pytestmark = pytest.mark.gpu


def double_cone(n):
    ang = 2 * np.pi * np.arange(n) / n
    ring = np.vstack((np.cos(ang), np.sin(ang), np.zeros(n)))
    p = np.hstack((np.zeros((3, 1)), ring, [[0.0], [0.0], [1.0]], [[0.0], [0.0], [-1.1]]))
    top, bot = n + 1, n + 2
    t = []
    for i in range(n):
        a, b = 1 + i, 1 + (i + 1) % n
        t.append((0, a, b, top))
        t.append((0, a, b, bot))
    return F.MeshTet(p, np.array(t, dtype=np.int64).T)


def fan(n):
    ang = 2 * np.pi * np.arange(n) / n
    p = np.hstack((np.zeros((2, 1)), np.vstack((np.cos(ang), np.sin(ang)))))
    t = np.array([(0, 1 + i, 1 + (i + 1) % n) for i in range(n)], dtype=np.int64).T
    return F.MeshTri(p, t)


def test_vector_tetp2_row_at_the_candidate_limit_matches_oracle():
    m = double_cone(273)                          # 546 cells share the origin: 16,380 candidates
    assert int((m.t == 0).any(axis=0).sum()) == 546
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()))
    K = linear_elasticity(1.0, 0.5).assemble(b)
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), "tet"), O.Vector(O.TetP2()))
    Ko = O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), ob)
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, Ko.indptr,
                                                   Ko.indices, Ko.data, K.shape)
    assert same, "pattern differs: %d extra, %d missing" % (extra, missing)
    assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)


def test_vector_tetp2_row_beyond_the_candidate_limit_is_refused():
    from skfem_gb300._native import FemError
    m = double_cone(274)                          # 548 cells: 16,440 candidates
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()))
    with pytest.raises(FemError, match="limit 16384"):
        linear_elasticity(1.0, 0.5).assemble(b)


def test_trip2_hub_row_sums_with_fewer_warps_per_block():
    # 1,500 triangles around one vertex: its TriP2 row holds 4,501 entries,
    # 144 KB of accumulators for a warp's 4 rows -- one warp per block
    from skfem_gb300 import helpers as H
    m = fan(1500)
    k = np.random.default_rng(3).lognormal(0.0, 1.0, m.nelements)

    @F.BilinearForm
    def k_laplace(u, v, w):
        return w.k * H.dot(H.grad(u), H.grad(v))
    b = F.Basis(m, F.ElementTriP2())
    K = k_laplace.assemble(b, k=b.zero_w() + k[:, None])
    assert np.diff(K.indptr).max() == 4501
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), "tri"), O.TriP2())
    Ko = O.bilinear_assemble(O.k_laplace, ob, k=ob.zero_w() + k[:, None])
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, Ko.indptr,
                                                   Ko.indices, Ko.data, K.shape)
    assert same, "pattern differs: %d extra, %d missing" % (extra, missing)
    assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)
