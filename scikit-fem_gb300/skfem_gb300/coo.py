"""COOData: the reference's elemental-result container, summed on the GPU.

  COOData                      skfem/assembly/form/coo_data.py:19-242
  Form.elemental / coo_data    skfem/assembly/form/form.py:82-89

Holds what the reference holds -- ``indices`` ((1 or 2, n) int32 rows /
columns), ``data`` (n float64 values in the reference's order: block (j, i)
of a bilinear form's (Nu, Nv, nelems) local values, then cells), ``shape``
and ``local_shape`` -- as host numpy arrays, so code written against the
reference reads and combines them unchanged.  Every reduction runs on the
GPU: ``tocsr`` uploads the entries and builds the CSR with the library's
COO pattern build (exact +-0.0 entries dropped first, as
``eliminate_zeros``) and fixed-order segmented sum; ``toarray`` of a 1-D
COOData is the same sum into an N x 1 matrix; a 0-D COOData sums with
numpy's pairwise order on the device.
"""

import ctypes
from dataclasses import dataclass, replace
from typing import Optional, Tuple

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as N

__all__ = ["COOData"]


def _device():
    N.require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def _device_csr(rows, cols, data, shape):
    """Device COO -> CSR (eliminate_zeros, then duplicates summed in
    ascending entry order): (indptr, indices, values) torch tensors."""
    dev = _device()
    r = torch.as_tensor(np.ascontiguousarray(rows, dtype=np.int32)).to(dev)
    c = torch.as_tensor(np.ascontiguousarray(cols, dtype=np.int32)).to(dev)
    v = torch.as_tensor(np.ascontiguousarray(data, dtype=np.float64)).to(dev)
    lib = N.lib()
    h = ctypes.c_void_p()
    s = N.stream_ptr()
    if r.numel() and (int(r.min()) < 0 or int(r.max()) >= shape[0]):
        raise ValueError("row index out of range")
    N.check(lib.fem_coo_pattern_build(N.ptr(r), N.ptr(c), N.ptr(v), r.numel(), int(shape[0]),
                                      int(shape[1]), ctypes.byref(h), s))
    pat = N.Pattern(h.value)
    indptr = torch.empty(pat.nrows + 1, dtype=torch.int32, device=dev)
    indices = torch.empty(max(pat.nnz, 1), dtype=torch.int32, device=dev)[:pat.nnz]
    vals = torch.empty(max(pat.nnz, 1), dtype=torch.float64, device=dev)[:pat.nnz]
    N.check(lib.fem_pattern_export(pat.handle, N.ptr(indptr), N.ptr(indices), s))
    if pat.nnz:
        N.check(lib.fem_csr_sum(pat.handle, N.ptr(v), N.ptr(vals), None, s))
    torch.cuda.current_stream().synchronize()
    del pat
    return indptr, indices, vals


@dataclass
class COOData:
    """coo_data.py:19-242 on the GPU (see the module docstring)."""

    indices: np.ndarray
    data: np.ndarray
    shape: Tuple[int, ...]
    local_shape: Optional[Tuple[int, ...]]

    # ---------------------------------------------------------- combining
    def __radd__(self, other):
        return self.__add__(other)

    def __add__(self, other):
        if isinstance(other, int):
            return self
        return replace(self,
                       indices=np.hstack((self.indices, other.indices)),
                       data=np.hstack((self.data, other.data)),
                       shape=tuple(max(self.shape[i], other.shape[i])
                                   for i in range(len(self.shape))),
                       local_shape=None)

    def __array__(self, dtype=None, copy=None):
        a = self.toarray()
        return a if dtype is None else a.astype(dtype)

    # ----------------------------------------------------- local matrices
    def tolocal(self, basis=None):
        """The local matrices, (nelems,) + local_shape, as the reference
        reshapes them; with a FacetBasis the facet matrices are scattered to
        the mesh's facets and summed per cell over its facets (t2f)."""
        if self.local_shape is None:
            raise NotImplementedError("Cannot build local matrices if "
                                      "local_shape is not specified.")
        local = np.moveaxis(self.data.reshape(tuple(self.local_shape) + (-1,), order="C"), -1, 0)
        if basis is not None:
            dev = _device()
            nfacets = int(np.asarray(basis.mesh.facets).shape[1])
            out = torch.zeros((nfacets,) + local.shape[1:], dtype=torch.float64, device=dev)
            out[torch.as_tensor(np.asarray(basis.find), device=dev).long()] = \
                torch.as_tensor(np.ascontiguousarray(local), device=dev)
            t2f = torch.as_tensor(np.asarray(basis.mesh.t2f), device=dev).long()
            acc = out[t2f[0]].clone()
            for k in range(1, t2f.shape[0]):          # np.sum(axis=0): in facet order
                acc = acc + out[t2f[k]]
            local = acc.cpu().numpy()
        return local

    def fromlocal(self, local):
        """Reverse of tolocal."""
        return replace(self, data=np.moveaxis(np.asarray(local), 0, -1).flatten("C"))

    def inverse(self):
        """Every local matrix inverted (on the device, batched)."""
        loc = torch.as_tensor(np.ascontiguousarray(self.tolocal()), device=_device())
        return self.fromlocal(torch.linalg.inv(loc).cpu().numpy())

    # --------------------------------------------------------- reductions
    def tocsr_torch(self):
        """The CSR as a device torch.sparse_csr_tensor (int32 indices)."""
        if len(self.shape) != 2:
            raise ValueError("tocsr needs a 2-tensor")
        indptr, indices, vals = _device_csr(self.indices[0], self.indices[1], self.data,
                                            self.shape)
        return torch.sparse_csr_tensor(indptr, indices, vals, size=tuple(self.shape))

    def tocsr(self):
        """scipy.sparse.csr_matrix (coo_data.py:94-100): exact zeros dropped
        before duplicates are summed, canonical format."""
        if len(self.shape) != 2:
            raise ValueError("tocsr needs a 2-tensor")
        indptr, indices, vals = _device_csr(self.indices[0], self.indices[1], self.data,
                                            self.shape)
        K = sp.csr_matrix((vals.cpu().numpy(), indices.cpu().numpy(), indptr.cpu().numpy()),
                          shape=tuple(self.shape))
        K.has_sorted_indices = True
        K.has_canonical_format = True
        return K

    def toarray(self):
        """Dense result (coo_data.py:102-118)."""
        if len(self.shape) == 1:
            rows = self.indices[0]
            indptr, indices, vals = _device_csr(rows, np.zeros_like(rows), self.data,
                                                (self.shape[0], 1))
            out = torch.zeros(self.shape[0], dtype=torch.float64, device=vals.device)
            counts = indptr[1:] - indptr[:-1]
            nz = torch.nonzero(counts, as_tuple=True)[0]
            out[nz] = vals            # one CSR entry (column 0) per nonempty row
            return out.cpu().numpy()
        if len(self.shape) == 2:
            return self.tocsr().toarray()
        raise NotImplementedError("toarray of a %d-tensor" % len(self.shape))

    def todefault(self):
        """Scalar for a 0-tensor, ndarray for a 1-tensor, scipy CSR for a
        2-tensor, self otherwise (coo_data.py:177-190)."""
        if len(self.shape) == 0:
            v = torch.as_tensor(np.ascontiguousarray(self.data, dtype=np.float64),
                                device=_device())
            total = torch.empty(1, dtype=torch.float64, device=v.device)
            N.check(N.lib().fem_sum_pairwise(N.ptr(v), v.numel(), N.ptr(total), N.stream_ptr()))
            return np.float64(total.item())
        if len(self.shape) == 1:
            return self.toarray()
        if len(self.shape) == 2:
            return self.tocsr()
        return self

    def astuple(self):
        return self.indices, self.data, self.shape

    def topetsc(self, dofs=None):
        raise NotImplementedError("PETSc export is not part of the GPU assembly path; hand the "
                                  "device CSR (tocsr_torch) to the solver instead")

    # ------------------------------------------------- matrix operations
    def dot(self, x, D=None):
        """Matrix-vector product of the (unassembled) COO matrix on the
        device; D: DOFs kept unchanged (coo_data.py:192-209)."""
        dev = _device()
        xt = torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev)
        A = self.tocsr_torch()
        z = A.matmul(xt[:, None])[:, 0]
        if D is not None:
            Dt = torch.as_tensor(np.asarray(D), device=dev).long()
            z[Dt] = xt[Dt]
        return z.cpu().numpy()

    def solve(self, b, D=None, tol=1e-10, maxiters=500):
        """Conjugate gradients on the device (coo_data.py:211-242)."""
        dev = _device()
        A = self.tocsr_torch()
        Dt = torch.as_tensor(np.asarray(D), device=dev).long() if D is not None else None

        def mv(v):
            z = A.matmul(v[:, None])[:, 0]
            if Dt is not None:
                z[Dt] = v[Dt]
            return z
        x = torch.as_tensor(np.asarray(b, dtype=np.float64), device=dev).clone()
        r = x - mv(x)
        p = r
        rsold = torch.dot(r, r)
        for _ in range(maxiters):
            Ap = mv(p)
            alpha = rsold / torch.dot(p, Ap)
            x = x + alpha * p
            r = r - alpha * Ap
            rsnew = torch.dot(r, r)
            if float(torch.sqrt(rsnew)) < tol:
                break
            p = r + (rsnew / rsold) * p
            rsold = rsnew
        return x.cpu().numpy()
