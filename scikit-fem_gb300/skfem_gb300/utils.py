"""Consumers of the assembled system, on the device.

``condense`` follows skfem.utils.condense (skfem/utils.py:462-600) and
``enforce`` skfem.utils.enforce (skfem/utils.py:327-400) for the
device-resident results of ``assemble_torch``: a torch sparse CSR matrix and
torch vectors stay in HBM; the condensed matrix is again a canonical CSR.
"""

import numpy as np
import torch

from . import _native as N

__all__ = ["condense", "enforce"]


def _device_dofs(S, n, device):
    """A DOF set (index array, list, bool mask or tensor) as a sorted,
    duplicate-free int64 tensor on the device; indices outside [0, n) raise
    IndexError here, before any device indexing uses them."""
    if S is None:
        return None
    if not isinstance(S, torch.Tensor):
        S = torch.from_numpy(np.ascontiguousarray(np.asarray(S)))
    S = S.to(device)
    if S.dtype == torch.bool:
        if S.numel() != n:
            raise IndexError("boolean DOF mask of length %d for %d DOFs" % (S.numel(), n))
        return torch.nonzero(S).squeeze(1)
    S = torch.unique(S.to(torch.int64))          # sorted
    if S.numel() and (int(S[0]) < 0 or int(S[-1]) >= n):
        raise IndexError("DOF index out of range for %d DOFs" % n)
    return S


def _kept_map(n, I, D, device):
    """(In, map): the kept DOFs In (sorted, device int64) and the int32 map
    DOF -> its index in In (-1 for eliminated DOFs), built on the device."""
    Dn, In = _device_dofs(D, n, device), _device_dofs(I, n, device)
    if In is None and Dn is None:
        raise Exception("Either I or D must be given!")
    if In is not None and Dn is not None:
        raise Exception("Give only I or only D!")
    if In is None:
        keep = torch.ones(n, dtype=torch.bool, device=device)
        keep[Dn] = False
        In = torch.nonzero(keep).squeeze(1)
    mp = torch.full((n,), -1, dtype=torch.int32, device=device)
    mp[In] = torch.arange(In.numel(), dtype=torch.int32, device=device)
    return In, mp


def condense(A, b=None, x=None, I=None, D=None, expand=True):
    """Eliminate DOFs: returns (A_II, b_I[, x, I]) with
    A_II = A[I][:, I] and b_I = b[I] - A[I][:, D] x[D] (utils.py:578-598).

    ``A`` is a torch sparse CSR tensor on the GPU (``assemble_torch``);
    ``b`` and ``x`` are torch vectors (``b`` may also be a sparse mass matrix
    for generalized eigenproblems: then ``B[I][:, I]`` is returned); with
    ``x`` given and no ``b``, ``b`` is zero (utils.py:319-322).  ``I`` / ``D``
    are index arrays, boolean masks, tensors or DofsViews; the sets are
    formed on the device, and an index outside the matrix raises IndexError.
    """
    if not (isinstance(A, torch.Tensor) and A.layout == torch.sparse_csr):
        raise TypeError("condense on the GPU takes the torch CSR of assemble_torch")
    n = A.shape[0]
    dev = A.device
    In, mp_d = _kept_map(n, I, D, dev)
    nk = In.numel()
    if x is None:
        x = torch.zeros(n, dtype=torch.float64, device=dev)
    elif b is None:
        b = torch.zeros(n, dtype=torch.float64, device=dev)
    x = torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()

    def sub(M, rhs=None):
        crow = M.crow_indices().to(torch.int32).contiguous()
        col = M.col_indices().to(torch.int32).contiguous()
        val = M.values().contiguous()
        lib = N.lib()
        out_ptr = torch.empty(nk + 1, dtype=torch.int32, device=dev)
        nnz = N.ctypes.c_int64()
        s = N.stream_ptr()
        N.check(lib.fem_condense_pattern(N.ptr(crow), N.ptr(col), n, N.ptr(mp_d), nk,
                                         N.ptr(out_ptr), N.ctypes.byref(nnz), s))
        out_ind = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)[:nnz.value]
        out_val = torch.empty(max(nnz.value, 1), dtype=torch.float64, device=dev)[:nnz.value]
        out_b = torch.empty(nk, dtype=torch.float64, device=dev) if rhs is not False else None
        bb = rhs if isinstance(rhs, torch.Tensor) else None
        N.check(lib.fem_condense_values(N.ptr(crow), N.ptr(col), N.ptr(val), n, N.ptr(mp_d),
                                        N.ptr(bb), N.ptr(x), N.ptr(out_ptr), N.ptr(out_ind),
                                        N.ptr(out_val), N.ptr(out_b), s))
        Mc = torch.sparse_csr_tensor(out_ptr, out_ind, out_val, size=(nk, nk))
        return Mc, out_b

    I_t = In
    if b is None:
        AII, _ = sub(A, rhs=False)
        ret = (AII,)
    elif isinstance(b, torch.Tensor) and b.layout == torch.sparse_csr:
        AII, _ = sub(A, rhs=False)
        BII, _ = sub(b, rhs=False)
        ret = (AII, BII)
    else:
        bt = torch.as_tensor(b, dtype=torch.float64, device=dev).contiguous()
        AII, bI = sub(A, rhs=bt)
        ret = (AII, bI)
    if expand:
        ret += (x, I_t)
    return ret if len(ret) > 1 else ret[0]


def _bc_sets(n, I, D, device):
    """The constrained DOFs (sorted, device int64) of enforce's I / D."""
    Dn, In = _device_dofs(D, n, device), _device_dofs(I, n, device)
    if In is None and Dn is None:
        raise Exception("Either I or D must be given!")
    if In is not None and Dn is not None:
        raise Exception("Give only I or only D!")
    if Dn is None:
        rest = torch.ones(n, dtype=torch.bool, device=device)
        rest[In] = False
        Dn = torch.nonzero(rest).squeeze(1)
    return Dn


def _rows_to_identity(M, rows, nd, d, rhs, x, overwrite):
    dev = M.device
    crow = M.crow_indices().to(torch.int32).contiguous()
    col = M.col_indices().to(torch.int32).contiguous()
    val = M.values() if overwrite else M.values().clone()
    missing = torch.zeros(1, dtype=torch.int32, device=dev)
    N.check(N.lib().fem_enforce(N.ptr(crow), N.ptr(col), N.ptr(val), M.shape[0], N.ptr(rows),
                                nd, float(d), N.ptr(rhs), N.ptr(x), N.ptr(missing),
                                N.stream_ptr()))
    if int(missing.item()):
        raise NotImplementedError("enforce: %d constrained rows have no diagonal entry in the "
                                  "pattern" % int(missing.item()))
    if overwrite:
        return M
    return torch.sparse_csr_tensor(M.crow_indices(), M.col_indices(), val, size=M.shape)


def enforce(A, b=None, x=None, I=None, D=None, diag=1., overwrite=False):
    """Set the rows D of A to zero with ``diag`` on the diagonal and b[D] =
    x[D] (utils.py:327-400) on a device CSR (torch sparse CSR of
    ``assemble_torch``); a sparse ``b`` (mass matrix) gets its rows D
    zeroed with a zero diagonal.  Returns (A, b) or A like the reference;
    ``overwrite`` modifies the inputs in place."""
    if not (isinstance(A, torch.Tensor) and A.layout == torch.sparse_csr):
        raise TypeError("enforce on the GPU takes the torch CSR of assemble_torch")
    n = A.shape[0]
    dev = A.device
    Dn = _bc_sets(n, I, D, dev)
    rows = Dn.to(torch.int32)
    if x is not None:
        x = torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
        if b is None:
            b = torch.zeros(n, dtype=torch.float64, device=dev)     # utils.py:321-322
    sparse_b = isinstance(b, torch.Tensor) and b.layout == torch.sparse_csr
    bout = None
    if b is not None and not sparse_b:
        bt = torch.as_tensor(b, dtype=torch.float64, device=dev)
        bout = bt if (overwrite and bt.is_contiguous()) else bt.clone().contiguous()
    Aout = _rows_to_identity(A, rows, rows.numel(), diag, bout, x, overwrite)
    if b is None:
        return Aout
    if sparse_b:
        return Aout, _rows_to_identity(b, rows, rows.numel(), 0.0, None, None, overwrite)
    return Aout, bout
