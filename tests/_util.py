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
