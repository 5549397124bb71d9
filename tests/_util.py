"""Shared helpers for the parity tests."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
HEADER = os.path.join(ROOT, "include", "skfem_gb300.h")

# Parity bounds (values): relative Frobenius and entrywise vs max |K|.
REL_FRO = 1e-12
REL_MAX = 1e-13


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fem_[a-z0-9_]+)\s*\(", src)))


def csr_diff(indptr, indices, data, gindptr, gindices, gdata, shape):
    """Compare two CSR matrices: returns (pattern_equal, extra, missing,
    maxnoise, rel_fro, rel_max) where extra/missing count entries present in
    only one of them and maxnoise is the largest |value| among those, relative
    to max |K|."""
    import scipy.sparse as sp
    A = sp.csr_matrix((data, indices, indptr), shape=shape)
    B = sp.csr_matrix((gdata, gindices, gindptr), shape=shape)
    same = (len(indptr) == len(gindptr) and np.array_equal(indptr, gindptr)
            and np.array_equal(indices, gindices))
    Ap = sp.csr_matrix((np.ones_like(data), indices, indptr), shape=shape)
    Bp = sp.csr_matrix((np.ones_like(gdata), gindices, gindptr), shape=shape)
    onlyA = (Ap - Ap.multiply(Bp)).tocoo()
    onlyB = (Bp - Bp.multiply(Ap)).tocoo()
    kmax = np.max(np.abs(gdata)) if len(gdata) else 1.0
    noise = 0.0
    if onlyA.nnz:
        noise = max(noise, np.max(np.abs(np.asarray(A[onlyA.row, onlyA.col]).ravel())))
    if onlyB.nnz:
        noise = max(noise, np.max(np.abs(np.asarray(B[onlyB.row, onlyB.col]).ravel())))
    D = (A - B)
    rel_fro = sp.linalg.norm(D) / max(sp.linalg.norm(B), 1e-300)
    rel_max = (abs(D).max() if D.nnz else 0.0) / kmax
    return same, onlyA.nnz, onlyB.nnz, noise / kmax, rel_fro, rel_max


def double_cone_arrays(n):
    """(p, t) of a double cone: a ring of n vertices around the origin, an
    apex above (z = 1) and below (z = -1.1); every tet (origin, ring_i,
    ring_i+1, apex) holds the origin, which 2n cells share."""
    ang = 2 * np.pi * np.arange(n) / n
    ring = np.vstack((np.cos(ang), np.sin(ang), np.zeros(n)))
    p = np.hstack((np.zeros((3, 1)), ring, [[0.0], [0.0], [1.0]], [[0.0], [0.0], [-1.1]]))
    top, bot = n + 1, n + 2
    t = []
    for i in range(n):
        a, b = 1 + i, 1 + (i + 1) % n
        t.append((0, a, b, top))
        t.append((0, a, b, bot))
    return p, np.array(t, dtype=np.int64).T


def fan_arrays(n):
    """(p, t) of n triangles around the origin."""
    ang = 2 * np.pi * np.arange(n) / n
    p = np.hstack((np.zeros((2, 1)), np.vstack((np.cos(ang), np.sin(ang)))))
    t = np.array([(0, 1 + i, 1 + (i + 1) % n) for i in range(n)], dtype=np.int64).T
    return p, t


def fan_coefficient(n):
    """The per-cell k of the fan case (seeded)."""
    return np.random.default_rng(3).lognormal(0.0, 1.0, n)
