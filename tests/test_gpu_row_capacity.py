"""Rows of high-valence DOFs.  The pattern build gathers a row's candidate
columns (cells sharing the row's DOF x local columns) in one warp's shared
memory, at most 16,384 of them; a vector TetP2 row has 30 candidates per
cell, so a DOF may be shared by at most 546 cells.  At that edge the
assembly must still give scikit-fem's CSR pattern (digests recorded by
running it, tests/golden/make_golden.py --capacity) and the oracle's values;
beyond it the build must refuse the mesh with a message naming the limit
(FEM_ERR_CAPACITY) -- no fault, no truncated row.  Rows whose shared-memory
accumulators do not fit four warps per block run with fewer warps per block.

The meshes (tests/_util.py): a double cone whose origin 2n tets share, and a
fan of n triangles around the origin.  Both are symmetric, so many of their
local entries are mathematically zero: where this platform's numpy rounds
such an entry differently from the platform the reference ran on, the
oracle's pattern may differ from the reference's by noise-level entries."""
import hashlib

import numpy as np
import pytest

import oracle as O
import skfem_gb300 as F
from skfem_gb300.models.elasticity import linear_elasticity
from _util import (REL_FRO, REL_MAX, csr_diff, double_cone_arrays, fan_arrays, fan_coefficient,
                   golden)

pytestmark = pytest.mark.gpu

REF = golden("capacity_patterns")


def _digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes())
                         .digest(), dtype=np.uint8)


def assert_reference_pattern_and_oracle_values(name, K, Ko):
    # the GPU replays the reference platform's arithmetic for exact zeros:
    # its pattern is the reference's, entry for entry
    assert K.nnz == int(REF[name + "__nnz"])
    np.testing.assert_array_equal(K.indptr, REF[name + "__pattern_indptr"])
    np.testing.assert_array_equal(K.indices, REF[name + "__pattern_indices"])
    assert np.array_equal(_digest(K.indptr), REF[name + "__indptr"])
    assert np.array_equal(_digest(K.indices), REF[name + "__indices"])
    fro = float(REF[name + "__fro"])
    assert abs(np.linalg.norm(K.data) - fro) <= REL_FRO * fro
    same, extra, missing, noise, rf, rm = csr_diff(K.indptr, K.indices, K.data, Ko.indptr,
                                                   Ko.indices, Ko.data, K.shape)
    assert rf <= REL_FRO and rm <= REL_MAX, (rf, rm)
    assert same or noise <= REL_MAX, (extra, missing, noise)


def double_cone(n):
    p, t = double_cone_arrays(n)
    return F.MeshTet(p, t)


def fan(n):
    p, t = fan_arrays(n)
    return F.MeshTri(p, t)


def test_vector_tetp2_row_at_the_candidate_limit_matches_oracle():
    m = double_cone(273)                          # 546 cells share the origin: 16,380 candidates
    assert int((m.t == 0).any(axis=0).sum()) == 546
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()))
    K = linear_elasticity(1.0, 0.5).assemble(b)
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), "tet"), O.Vector(O.TetP2()))
    Ko = O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), ob)
    assert_reference_pattern_and_oracle_values("cone_273_vec_tet_p2", K, Ko)


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
    k = fan_coefficient(m.nelements)

    @F.BilinearForm
    def k_laplace(u, v, w):
        return w.k * H.dot(H.grad(u), H.grad(v))
    b = F.Basis(m, F.ElementTriP2())
    K = k_laplace.assemble(b, k=b.zero_w() + k[:, None])
    assert np.diff(K.indptr).max() == 4501
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), "tri"), O.TriP2())
    Ko = O.bilinear_assemble(O.k_laplace, ob, k=ob.zero_w() + k[:, None])
    assert_reference_pattern_and_oracle_values("fan_1500_tri_p2", K, Ko)
