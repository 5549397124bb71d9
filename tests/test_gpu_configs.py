"""Parity at the benchmark configurations' own sizes: the public API on the
GPU against scikit-fem's own CSR patterns of the same seeded inputs the
benchmark builds (digests recorded by running scikit-fem) and against the
CPU oracle (the numpy restatement of scikit-fem's assembly, pinned to the
reference's fixtures) run beside it.  Bounds: CSR indptr / indices
bit-exact, values within 1e-12 relative Frobenius and 1e-13 * max|K|
entrywise, load vectors the same, and repeated GPU assemblies bitwise
identical.

  - TriP1 Laplace + unit load on the 256 x 256 square (131,072 cells), full size
  - TetP1 k*Laplace + mass on the 61^3-node cube (1,296,000 cells), the
    benchmark's CPU sample of the 101^3 workload, lognormal k: through the
    device path and the host (nelems, nqp) path
  - Hex1 theta*Laplace on the 64^3-cell cube (262,144 cells), full size, and
    the theta-gradient of w^T K(theta) u against Functional.elemental's
  - vector TetP2 elasticity on a jittered 16^3-cell cube (intorder 4)
  - four meshes of the batched TriP2 workload, each with its own k, taken
    out of one batched assembly (CUDA-graph replay)
"""
import hashlib
import os

import numpy as np
import pytest
import torch

import bench as B
import oracle as O
import skfem_gb300 as F
from skfem_gb300 import helpers as H
from skfem_gb300.models.elasticity import linear_elasticity
from skfem_gb300.models.poisson import laplace, unit_load
from _util import REL_FRO, REL_MAX, csr_diff, golden

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


@F.BilinearForm
def k_laplace_mass(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v)) + u * v


@F.BilinearForm
def theta_laplace(u, v, w):
    return w.theta * H.dot(H.grad(u), H.grad(v))


@F.BilinearForm
def k_laplace(u, v, w):
    return w.k * H.dot(H.grad(u), H.grad(v))


# scikit-fem's own results for these cases, run where it is installed
# (tests/golden/make_golden.py --configs): nnz, SHA-256 of indptr / indices,
# Frobenius norm and sum of the values
REF = golden("config_patterns")


def _digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes())
                         .digest(), dtype=np.uint8)


def _pattern_is_reference(name, K):
    return (K.nnz == int(REF[name + "__nnz"])
            and np.array_equal(_digest(K.indptr), REF[name + "__indptr"])
            and np.array_equal(_digest(K.indices), REF[name + "__indices"]))


def assert_parity(name, Kp, Ko):
    """Kp (GPU): CSR pattern bit-exact with scikit-fem's (digests), values
    within the bounds of the oracle's.  The oracle runs on this machine's
    numpy: where its compiled loops round a mathematically-zero local entry
    differently from the platform the reference ran on (numpy's aarch64
    build may contract multiply-adds), its pattern can differ from the
    reference's by such noise entries -- then those entries must be noise
    (at most 1e-13 of max|K|) and the rest within the bounds."""
    assert _pattern_is_reference(name, Kp), "GPU pattern differs from scikit-fem's"
    fro = np.linalg.norm(Kp.data)
    assert abs(fro - float(REF[name + "__fro"])) <= REL_FRO * float(REF[name + "__fro"])
    same, extra, missing, noise, rf, rm = csr_diff(Kp.indptr, Kp.indices, Kp.data, Ko.indptr,
                                                   Ko.indices, Ko.data, Kp.shape)
    assert rf <= REL_FRO, rf
    assert rm <= REL_MAX, rm
    if _pattern_is_reference(name, Ko):
        assert same, "pattern differs: %d extra, %d missing" % (extra, missing)
    else:
        assert noise <= REL_MAX, noise


def omesh(m, kind):
    return O.OMesh(np.asarray(m.p), np.asarray(m.t), kind)


def test_tri_p1_laplace_and_load_256():
    m = B.tri_square(256)
    om = O.mesh_tri_tensor(*(np.linspace(0, 1, 257),) * 2)
    np.testing.assert_array_equal(m.p, om.p)
    np.testing.assert_array_equal(m.t, om.t)
    b = F.Basis(m, F.ElementTriP1())
    K = laplace.assemble(b)
    K2 = laplace.assemble(b)
    np.testing.assert_array_equal(K.data, K2.data)
    f = unit_load.assemble(b)
    ob = O.OBasis(om, O.TriP1())
    Ko = O.bilinear_assemble(O.laplace, ob)
    fo = O.linear_assemble(O.unit_load, ob)
    assert K.nnz == Ko.nnz == 329217
    assert_parity("tri_p1_256", K, Ko)
    assert np.max(np.abs(f - fo)) <= REL_MAX * np.max(np.abs(fo))
    assert np.max(np.abs(f - REF["tri_p1_256__b"])) <= REL_MAX * np.max(np.abs(fo))


def test_tet_p1_k_laplace_mass_61_cube():
    m, k = B.build_workload(61)
    om = O.mesh_tet_tensor(*(np.linspace(0, 1, 61),) * 3)
    np.testing.assert_array_equal(m.p, om.p)
    np.testing.assert_array_equal(m.t, om.t)
    b = F.Basis(m, F.ElementTetP1())
    ob = O.OBasis(om, O.TetP1())
    Ko = O.bilinear_assemble(O.k_laplace_mass, ob, k=ob.zero_w() + k[:, None], nthreads=THREADS)
    # host (nelems, nqp) coefficient, as the reference takes it -> scipy CSR
    Kh = k_laplace_mass.assemble(b, k=b.zero_w() + k[:, None])
    assert_parity("tet_p1_61", Kh, Ko)
    # device per-cell coefficient -> device CSR, twice
    kd = torch.from_numpy(k).cuda()
    T1 = k_laplace_mass.assemble_torch(b, k=kd)
    T2 = k_laplace_mass.assemble_torch(b, k=kd)
    assert torch.equal(T1.values(), T2.values())
    np.testing.assert_array_equal(T1.values().cpu().numpy(), Kh.data)
    np.testing.assert_array_equal(T1.crow_indices().cpu().numpy(), Ko.indptr)
    np.testing.assert_array_equal(T1.col_indices().cpu().numpy(), Ko.indices)


def test_hex1_theta_laplace_64_cube_and_theta_gradient():
    m, theta, wv, uv = B.hex_cube_workload(64)
    om = O.mesh_hex_tensor(*(np.linspace(0, 1, 65),) * 3)
    np.testing.assert_array_equal(m.p, om.p)
    np.testing.assert_array_equal(m.t, om.t)
    b = F.Basis(m, F.ElementHex1())
    ob = O.OBasis(om, O.Hex1())
    Ko = O.bilinear_assemble(O.theta_laplace, ob, theta=ob.zero_w() + theta[:, None],
                             nthreads=THREADS)
    K = theta_laplace.assemble(b, theta=b.zero_w() + theta[:, None])
    K2 = theta_laplace.assemble(b, theta=b.zero_w() + theta[:, None])
    np.testing.assert_array_equal(K.data, K2.data)
    assert_parity("hex1_64", K, Ko)
    # d(w^T K(theta) u)/d theta_e = w_e^T K_e(1) u_e (Functional.elemental's)
    from skfem_gb300.autodiff import assemble_vjp
    th = torch.tensor(theta, device="cuda", requires_grad=True)
    J = assemble_vjp(theta_laplace, b, torch.tensor(wv, device="cuda"),
                     torch.tensor(uv, device="cuda"), theta=th)
    J.backward()
    dth = O.theta_gradient(O.laplace, ob, wv, uv, nthreads=THREADS)
    np.testing.assert_allclose(th.grad.cpu().numpy(), dth, rtol=1e-11,
                               atol=1e-13 * np.abs(dth).max())
    assert abs(J.item() - wv @ (Ko @ uv)) <= 1e-12 * abs(wv @ (Ko @ uv)) + 1e-14


def test_vector_tet_p2_elasticity_jittered_16():
    m = B.jittered_tet_cube(16)
    b = F.Basis(m, F.ElementVector(F.ElementTetP2()), intorder=4)
    ob = O.OBasis(omesh(m, "tet"), O.Vector(O.TetP2()), intorder=4)
    Ko = O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), ob, nthreads=THREADS)
    form = linear_elasticity(1.0, 0.5)
    K = form.assemble(b)
    K2 = form.assemble(b)
    np.testing.assert_array_equal(K.data, K2.data)
    assert_parity("vec_tet_p2_16", K, Ko)


def test_batched_trip2_meshes_against_oracle():
    from skfem_gb300.batched import BatchedBasis, GraphedAssembly
    meshes, ks = B.trip2_batch(4)
    bb = BatchedBasis(meshes, F.ElementTriP2())
    kk = torch.tensor(np.concatenate(ks), device="cuda")
    rng = np.random.default_rng(2)
    ga = GraphedAssembly(k_laplace, bb, {"k": kk},
                         w=torch.tensor(rng.standard_normal(bb.N), device="cuda"),
                         u=torch.tensor(rng.standard_normal(bb.N), device="cuda")).capture()
    ga.replay()
    torch.cuda.synchronize()
    ga.check()
    first = ga.values.clone()
    ga.replay()
    torch.cuda.synchronize()
    assert torch.equal(first, ga.values)
    blocks = bb.split(ga.csr())
    for i, (m, k, blk) in enumerate(zip(meshes, ks, blocks)):
        ob = O.OBasis(omesh(m, "tri"), O.TriP2())
        Ko = O.bilinear_assemble(O.k_laplace, ob, k=ob.zero_w() + k[:, None], nthreads=THREADS)
        assert_parity("trip2_batch_%d" % i, blk, Ko)
