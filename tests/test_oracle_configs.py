"""The oracle against scikit-fem's own CSR patterns at the benchmark
configurations' sizes (digests recorded by tests/golden/make_golden.py
--configs): nnz, indptr and indices bit-exact, Frobenius norm of the values
within 1e-12.  Runs on the CPU; it pins the oracle that the GPU tests and
the benchmark's parity check compare with, at full size on this platform."""
import hashlib
import os

import numpy as np
import pytest

import bench as B
import oracle as O
from _util import golden

REF = golden("config_patterns")
THREADS = max(1, min(16, os.cpu_count() or 1))


def _digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes())
                         .digest(), dtype=np.uint8)


def _check(name, K):
    assert K.nnz == int(REF[name + "__nnz"])
    assert np.array_equal(_digest(K.indptr), REF[name + "__indptr"])
    assert np.array_equal(_digest(K.indices), REF[name + "__indices"])
    fro = float(REF[name + "__fro"])
    assert abs(np.linalg.norm(K.data) - fro) <= 1e-12 * fro


def test_oracle_tri_p1_256():
    ob = O.OBasis(O.mesh_tri_tensor(*(np.linspace(0, 1, 257),) * 2), O.TriP1())
    _check("tri_p1_256", O.bilinear_assemble(O.laplace, ob))
    b = O.linear_assemble(O.unit_load, ob)
    assert np.max(np.abs(b - REF["tri_p1_256__b"])) <= 1e-13 * np.max(np.abs(b))


def test_oracle_tet_p1_61():
    m = O.mesh_tet_tensor(*(np.linspace(0, 1, 61),) * 3)
    k = np.random.default_rng(B.SEED).lognormal(0.0, 1.0, m.nelements)
    ob = O.OBasis(m, O.TetP1())
    _check("tet_p1_61", O.bilinear_assemble(O.k_laplace_mass, ob, k=ob.zero_w() + k[:, None],
                                            nthreads=THREADS))


@pytest.mark.parametrize("i", range(4))
def test_oracle_trip2_batch_meshes(i):
    meshes, ks = B.trip2_batch(4)
    m = meshes[i]
    ob = O.OBasis(O.OMesh(np.asarray(m.p), np.asarray(m.t), "tri"), O.TriP2())
    _check("trip2_batch_%d" % i, O.bilinear_assemble(O.k_laplace, ob,
                                                     k=ob.zero_w() + ks[i][:, None],
                                                     nthreads=THREADS))
