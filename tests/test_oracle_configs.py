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


CAP = golden("capacity_patterns")


def _pattern_diff(indptr, indices, rindptr, rindices, nrows):
    """(extra, missing) entry coordinates of a CSR pattern against another."""
    def coords(ip, ix):
        rows = np.repeat(np.arange(nrows, dtype=np.int64), np.diff(ip))
        return rows * (nrows + 1) + ix.astype(np.int64)
    a, b = coords(indptr, indices), coords(rindptr, rindices)
    return np.setdiff1d(a, b), np.setdiff1d(b, a)


@pytest.mark.parametrize("name", ["cone_273_vec_tet_p2", "fan_1500_tri_p2"])
def test_oracle_high_valence_rows(name):
    # the rows at the pattern build's candidate limit (tests/test_gpu_row_capacity.py):
    # the oracle against scikit-fem's pattern -- on these symmetric meshes
    # its exact zeros may differ from the reference's in a few noise-level
    # entries (an entry only the oracle has is at most 1e-13 of max|K|; one
    # only the reference has is an exact zero of the oracle's)
    from _util import double_cone_arrays, fan_arrays, fan_coefficient
    if name.startswith("cone"):
        p, t = double_cone_arrays(273)
        ob = O.OBasis(O.OMesh(p, np.sort(t, axis=0), "tet"), O.Vector(O.TetP2()))
        K = O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), ob)
    else:
        p, t = fan_arrays(1500)
        ob = O.OBasis(O.OMesh(p, np.sort(t, axis=0), "tri"), O.TriP2())
        k = fan_coefficient(t.shape[1])
        K = O.bilinear_assemble(O.k_laplace, ob, k=ob.zero_w() + k[:, None])
    rip, rix = CAP[name + "__pattern_indptr"], CAP[name + "__pattern_indices"]
    assert np.array_equal(_digest(rip), CAP[name + "__indptr"])
    assert np.array_equal(_digest(rix), CAP[name + "__indices"])
    extra, missing = _pattern_diff(K.indptr, K.indices, rip, rix, K.shape[0])
    assert len(extra) + len(missing) <= 1e-3 * K.nnz
    if len(extra):
        Kd = K.tocsr()
        vals = np.abs(np.asarray(Kd[extra // (K.shape[0] + 1), extra % (K.shape[0] + 1)]))
        assert vals.max() <= 1e-13 * np.abs(K.data).max()
    fro = float(CAP[name + "__fro"])
    assert abs(np.linalg.norm(K.data) - fro) <= 1e-12 * fro
