"""Consumers of the assembled system, on the device.

``condense`` follows skfem.utils.condense (skfem/utils.py:462-600) for the
device-resident results of ``assemble_torch``: a torch sparse CSR matrix and
torch vectors stay in HBM; the condensed matrix is again a canonical CSR.
"""

import numpy as np
import torch

from . import _native as N

__all__ = ["condense"]


def _dofs(S, n, device):
    if S is None:
        return None
    if isinstance(S, torch.Tensor):
        S = S.detach().cpu().numpy()
    S = np.asarray(S)
    if S.dtype == bool:
        S = np.nonzero(S)[0]
    return np.unique(S.astype(np.int64))


def condense(A, b=None, x=None, I=None, D=None, expand=True):
    """Eliminate DOFs: returns (A_II, b_I[, x, I]) with
    A_II = A[I][:, I] and b_I = b[I] - A[I][:, D] x[D] (utils.py:578-598).

    ``A`` is a torch sparse CSR tensor on the GPU (``assemble_torch``);
    ``b`` and ``x`` are torch vectors (``b`` may also be a sparse mass matrix
    for generalized eigenproblems: then ``B[I][:, I]`` is returned).
    """
    if not (isinstance(A, torch.Tensor) and A.layout == torch.sparse_csr):
        raise TypeError("condense on the GPU takes the torch CSR of assemble_torch")
    n = A.shape[0]
    dev = A.device
    Dn, In = _dofs(D, n, dev), _dofs(I, n, dev)
    if In is None and Dn is None:
        raise Exception("Either I or D must be given!")
    if In is not None and Dn is not None:
        raise Exception("Give only I or only D!")
    if In is None:
        In = np.setdiff1d(np.arange(n), Dn)
    mp = np.full(n, -1, dtype=np.int32)
    mp[In] = np.arange(len(In), dtype=np.int32)
    mp_d = torch.from_numpy(mp).to(dev)
    if x is None:
        x = torch.zeros(n, dtype=torch.float64, device=dev)
    x = torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()

    def sub(M, rhs=None):
        crow = M.crow_indices().to(torch.int32).contiguous()
        col = M.col_indices().to(torch.int32).contiguous()
        val = M.values().contiguous()
        lib = N.lib()
        out_ptr = torch.empty(len(In) + 1, dtype=torch.int32, device=dev)
        nnz = N.ctypes.c_int64()
        s = N.stream_ptr()
        N.check(lib.fem_condense_pattern(N.ptr(crow), N.ptr(col), n, N.ptr(mp_d), len(In),
                                         N.ptr(out_ptr), N.ctypes.byref(nnz), s))
        out_ind = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)[:nnz.value]
        out_val = torch.empty(max(nnz.value, 1), dtype=torch.float64, device=dev)[:nnz.value]
        out_b = torch.empty(len(In), dtype=torch.float64, device=dev) if rhs is not False else None
        bb = rhs if isinstance(rhs, torch.Tensor) else None
        N.check(lib.fem_condense_values(N.ptr(crow), N.ptr(col), N.ptr(val), n, N.ptr(mp_d),
                                        N.ptr(bb), N.ptr(x), N.ptr(out_ptr), N.ptr(out_ind),
                                        N.ptr(out_val), N.ptr(out_b), s))
        Mc = torch.sparse_csr_tensor(out_ptr, out_ind, out_val, size=(len(In), len(In)))
        return Mc, out_b

    I_t = torch.from_numpy(In).to(dev)
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
