"""BilinearForm / LinearForm / asm: the reference's assembly API on the GPU.

  Form.__init__ / decorator       skfem/assembly/form/form.py:32-71
  Form._normalize_asm_kwargs      form.py:91-121 (coefficient formats)
  BilinearForm.assemble           bilinear_form.py:130-148 -> scipy CSR
  LinearForm.assemble             form.py:73-80 + linear_form.py:18-46 -> ndarray
  asm                             skfem/assembly/__init__.py:69-97

``assemble`` returns what the reference returns (scipy.sparse.csr_matrix /
numpy array, canonical CSR with the reference's pattern); ``assemble_torch``
returns the device-resident result (torch sparse CSR / tensor) without a
host round trip.  The form callable is traced once (tracer.py) and mapped to
the CUDA kernels' coefficient channels; per-element coefficient fields stay
on the device.
"""

import ctypes
import numbers

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as N
from .tracer import (bilinear_channels, linear_channels, trace_bilinear, trace_linear,
                     trace_tape)

__all__ = ["Form", "BilinearForm", "LinearForm", "asm", "ElementField"]


class ElementField:
    """An explicit per-element coefficient (one value per cell), accepted
    wherever the reference takes a (nelems, nqp) array that is constant in
    each cell.  Holds a host array or a device tensor."""

    def __init__(self, values):
        self.values = values


class _Coefficients:
    """Form arguments normalised to device tensors (one value per element)."""

    def __init__(self, basis, kwargs):
        self.fields = {}
        self.numbers = {}
        self.keep = []
        dev = basis.device
        ne = basis.nelems
        nqp = basis.X.shape[-1]
        for k, v in kwargs.items():
            if isinstance(v, numbers.Number) or isinstance(v, tuple):
                self.numbers[k] = v
                continue
            if isinstance(v, ElementField):
                t = torch.as_tensor(v.values, dtype=torch.float64).to(dev).reshape(-1)
                if t.numel() != ne:
                    raise ValueError("ElementField '%s' has %d values for %d elements"
                                     % (k, t.numel(), ne))
                self.fields[k] = t.contiguous()
                continue
            if isinstance(v, torch.Tensor):
                t = v.to(device=dev, dtype=torch.float64)
            elif isinstance(v, np.ndarray):
                if v.ndim == 1:
                    if v.shape[0] != basis.N:
                        raise ValueError("Input array has wrong size.")  # abstract_basis.py:284-285
                    raise NotImplementedError(
                        "DOF-vector coefficients ('%s', interpolated by the reference) are not "
                        "supported yet; pass per-element values (nelems, nqp) or ElementField" % k)
                t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(dev)
            elif isinstance(v, list):
                raise NotImplementedError("list-valued coefficients are not supported")
            else:
                raise ValueError("The given type '{}' for the list of extra form parameters w "
                                 "cannot be converted to DiscreteField.".format(type(v)))
            if t.dim() == 1 and t.shape[0] == ne:
                self.fields[k] = t.contiguous()
                continue
            if t.dim() != 2 or t.shape[0] != ne:
                raise ValueError("coefficient '%s' must have shape (nelems, nqp)" % k)
            if t.shape[1] != nqp:
                raise ValueError("Quadrature mismatch: '{}' should have same number of "
                                 "integration points as the basis object.".format(k))
            col = t[:, 0].contiguous()
            if nqp > 1 and not bool(torch.equal(t[:, 1:], col[:, None].expand(-1, nqp - 1))):
                raise NotImplementedError(
                    "coefficient '%s' varies inside cells; the kernels take per-element "
                    "coefficients (constant over each cell's quadrature points)" % k)
            self.fields[k] = col

    def coef(self, poly, ne, device):
        """Poly -> FemCoef (scale, field pointer)."""
        items = [(names, c) for names, c in poly.items() if c != 0.0]
        if not items:
            return N.FemCoef(0.0, None)
        if len(items) == 1:
            names, c = items[0]
            if names == ():
                return N.FemCoef(c, None)
            if len(names) == 1:
                return N.FemCoef(c, self.fields[names[0]].data_ptr())
        acc = torch.zeros(ne, dtype=torch.float64, device=device)
        for names, c in items:
            term = torch.full((ne,), c, dtype=torch.float64, device=device)
            for n in names:
                term = term * self.fields[n]
            acc = acc + term
        self.keep.append(acc)
        return N.FemCoef(1.0, acc.data_ptr())


class Form:
    """form.py:29-89 (decorator, partial, dtype / nthreads / params)."""

    form = None

    def __init__(self, form=None, dtype=np.float64, nthreads=0, **params):
        self.form = form.form if isinstance(form, Form) else form
        if dtype is not np.float64 and np.dtype(dtype) != np.float64:
            raise NotImplementedError("only float64 forms are assembled on the GPU")
        self.dtype = dtype
        self.nthreads = nthreads
        self.params = params
        self._traces = {}

    def __call__(self, *args):
        if self.form is None:
            return type(self)(form=args[0], dtype=self.dtype, nthreads=self.nthreads,
                              **self.params)
        raise TypeError("call .assemble(basis, ...) to assemble")

    def partial(self, *args, **kwargs):
        import functools
        f = type(self)(form=functools.partial(self.form, *args, **kwargs), dtype=self.dtype,
                       nthreads=self.nthreads, **self.params)
        return f

    @property
    def __name__(self):
        return getattr(self.form, "__name__", "form")

    # tracing is cached per (element kind, field names, numbers)
    def _trace(self, basis, coeffs, kind):
        key = (basis.elem.family, basis.elem.vector, basis.mesh.p.shape[0],
               tuple(sorted(coeffs.fields)), tuple(sorted(coeffs.numbers.items(), key=repr)))
        ch = self._traces.get(key)
        if ch is None:
            dim = basis.mesh.p.shape[0]
            if kind == "bilinear":
                sym = trace_bilinear(self.form, basis.elem, dim, coeffs.fields, coeffs.numbers)
                ch = bilinear_channels(sym, basis.elem, dim)
            else:
                sym = trace_linear(self.form, basis.elem, dim, coeffs.fields, coeffs.numbers)
                ch = linear_channels(sym, basis.elem, dim)
            self._traces[key] = ch
        return ch


def _structure_key(ch):
    return tuple(sorted((name, tuple(sorted(names for names, c in p.items() if c != 0.0)))
                        for name, p in ch.items()))


def _program(form, basis, coeffs):
    """The form's exact-order program (tracer.trace_tape) on the device."""
    try:
        ins, out, names = trace_tape(form.form, basis.elem, basis.mesh.p.shape[0],
                                     list(coeffs.fields), coeffs.numbers)
    except NotImplementedError:
        # an operation the replay cannot reproduce bit for bit: the mask then
        # comes from the separately rounded tensor-form evaluation alone
        return None, None
    if len(ins) > 512 or len(names) > 8:
        return None, None
    arr = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm) for op, a, b, imm in ins])
    dev = torch.frombuffer(bytearray(arr), dtype=torch.uint8).to(basis.device)
    prog = N.FemProgram(len(ins), out, len(names), basis.X.shape[1], dev.data_ptr())
    for k, n in enumerate(names):
        prog.coef[k] = coeffs.fields[n].data_ptr()
    return prog, dev


class _PatternEntry:
    def __init__(self, basis, c_form, stream, program=None):
        lib = N.lib()
        h = ctypes.c_void_p()
        N.check(lib.fem_pattern_build(N.byref(basis.c_mesh), N.byref(basis.c_basis),
                                      N.byref(c_form) if c_form is not None else None,
                                      N.byref(program) if program is not None else None,
                                      ctypes.byref(h), stream))
        self.pat = N.Pattern(h.value)
        dev = basis.device
        self.nrows = self.pat.nrows
        self.nnz = self.pat.nnz
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        if c_form is not None:
            self.indptr = torch.empty(self.nrows + 1, dtype=torch.int32, device=dev)
            self.indices = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=dev)[:self.nnz]
            N.check(lib.fem_pattern_export(self.pat.handle, N.ptr(self.indptr),
                                           N.ptr(self.indices), stream))
            self.staging = torch.empty(max(1, self.pat.staging_bytes // 8), dtype=torch.float64,
                                       device=dev)
            torch.cuda.current_stream().synchronize()
        else:
            self.staging = torch.empty(max(1, basis.nelems * basis.Nbfun), dtype=torch.float64,
                                       device=dev)


class BilinearForm(Form):
    """bilinear_form.py:19-151."""

    def _setup(self, ubasis, vbasis, kwargs):
        if vbasis is not None and vbasis is not ubasis:
            raise NotImplementedError("different trial and test bases are not supported yet")
        coeffs = _Coefficients(ubasis, kwargs)
        ch = self._trace(ubasis, coeffs, "bilinear")
        ne, dev = ubasis.nelems, ubasis.device
        z = N.FemCoef(0.0, None)
        if ubasis.elem.vector:
            f = N.FemBilinear(z, coeffs.coef(ch["mass"], ne, dev), coeffs.coef(ch["lam"], ne, dev),
                              coeffs.coef(ch["lap"], ne, dev), coeffs.coef(ch["tr"], ne, dev))
        else:
            f = N.FemBilinear(coeffs.coef(ch["diff"], ne, dev), coeffs.coef(ch["mass"], ne, dev),
                              z, z, z)
        return coeffs, ch, f

    def _device_assemble(self, ubasis, vbasis=None, **kwargs):
        coeffs, ch, c_form = self._setup(ubasis, vbasis, kwargs)
        stream = N.stream_ptr()
        key = ("bilinear", _structure_key(ch))
        entry = ubasis._patterns.get(key)
        if entry is None:
            prog, keep = _program(self, ubasis, coeffs)
            entry = _PatternEntry(ubasis, c_form, stream, prog)
            del keep
            ubasis._patterns[key] = entry
        vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64, device=ubasis.device)[:entry.nnz]
        entry.status.zero_()
        N.check(N.lib().fem_assemble(N.byref(ubasis.c_mesh), N.byref(ubasis.c_basis),
                                     N.byref(c_form), entry.pat.handle, N.ptr(entry.staging),
                                     N.ptr(vals), N.ptr(entry.status), stream))
        return entry, vals, coeffs, key, c_form

    def _check_status(self, ubasis, entry, key):
        st = int(entry.status.item())
        if st & (1 << N.FEM_ERR_ZERO_JACOBIAN):
            raise N.ZeroJacobianError("Zero Jacobian determinant")
        if st & (1 << N.FEM_ERR_STALE_PATTERN):
            del ubasis._patterns[key]
            return False
        return True

    def assemble(self, ubasis, vbasis=None, **kwargs):
        """Assemble into a scipy.sparse.csr_matrix (bilinear_form.py:130-148)."""
        for _ in range(2):
            entry, vals, coeffs, key, _f = self._device_assemble(ubasis, vbasis, **kwargs)
            if self._check_status(ubasis, entry, key):
                break
        # Device -> pinned host copies (torch's caching host allocator reuses
        # the blocks of matrices the caller has dropped); the returned matrix
        # owns its arrays through their numpy views.
        data = torch.empty(entry.nnz, dtype=torch.float64, pin_memory=True)
        indices = torch.empty(entry.nnz, dtype=torch.int32, pin_memory=True)
        indptr = torch.empty(entry.nrows + 1, dtype=torch.int32, pin_memory=True)
        data.copy_(vals, non_blocking=True)
        indices.copy_(entry.indices, non_blocking=True)
        indptr.copy_(entry.indptr, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        K = sp.csr_matrix((data.numpy(), indices.numpy(), indptr.numpy()),
                          shape=(ubasis.N, ubasis.N), copy=False)
        K.has_sorted_indices = True
        K.has_canonical_format = True
        return K

    def assemble_torch(self, ubasis, vbasis=None, check=True, **kwargs):
        """Device-resident result: torch.sparse_csr_tensor (int32 indices,
        float64 values) sharing the cached pattern arrays."""
        entry, vals, coeffs, key, _f = self._device_assemble(ubasis, vbasis, **kwargs)
        if check and not self._check_status(ubasis, entry, key):
            entry, vals, coeffs, key, _f = self._device_assemble(ubasis, vbasis, **kwargs)
        return torch.sparse_csr_tensor(entry.indptr, entry.indices, vals,
                                       size=(ubasis.N, ubasis.N))

    def elemental_torch(self, ubasis, **kwargs):
        """Local matrices (nelems, Nbfun, Nbfun), row = test function."""
        coeffs, ch, c_form = self._setup(ubasis, None, kwargs)
        nb = ubasis.Nbfun
        out = torch.empty((ubasis.nelems, nb, nb), dtype=torch.float64, device=ubasis.device)
        N.check(N.lib().fem_local_matrices(N.byref(ubasis.c_mesh), N.byref(ubasis.c_basis),
                                           N.byref(c_form), N.ptr(out), N.stream_ptr()))
        return out

    def pattern(self, ubasis, **kwargs):
        """(indptr, indices) device tensors of the cached CSR pattern."""
        entry, _, _, _, _ = self._device_assemble(ubasis, None, **kwargs)
        return entry.indptr, entry.indices


class LinearForm(Form):
    """linear_form.py:10-49."""

    def _setup(self, basis, kwargs):
        coeffs = _Coefficients(basis, kwargs)
        ch = self._trace(basis, coeffs, "linear")
        return coeffs, N.FemLinear(coeffs.coef(ch["load"], basis.nelems, basis.device))

    def _device_assemble(self, basis, vbasis=None, **kwargs):
        if vbasis is not None:
            raise ValueError("LinearForm takes one basis")
        coeffs, c_form = self._setup(basis, kwargs)
        stream = N.stream_ptr()
        key = ("incidence",)
        entry = basis._patterns.get(key)
        if entry is None:
            entry = _PatternEntry(basis, None, stream, None)
            basis._patterns[key] = entry
        b = torch.empty(basis.N, dtype=torch.float64, device=basis.device)
        N.check(N.lib().fem_assemble_vector(N.byref(basis.c_mesh), N.byref(basis.c_basis),
                                            N.byref(c_form), entry.pat.handle,
                                            N.ptr(entry.staging), N.ptr(b), stream))
        return b, coeffs

    def assemble(self, basis, vbasis=None, **kwargs):
        b, _ = self._device_assemble(basis, vbasis, **kwargs)
        out = torch.empty(basis.N, dtype=torch.float64, pin_memory=True)
        out.copy_(b, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out.numpy()

    def assemble_torch(self, basis, vbasis=None, **kwargs):
        b, _ = self._device_assemble(basis, vbasis, **kwargs)
        return b


def asm(form, *args, **kwargs):
    """skfem/assembly/__init__.py:69-97 for a single basis (no list products)."""
    if not isinstance(form, Form):
        import inspect
        nargs = len(inspect.signature(form).parameters)
        form = BilinearForm(form) if nargs == 3 else LinearForm(form)
    if any(isinstance(a, (list, tuple)) for a in args):
        raise NotImplementedError("asm over lists of bases is not supported")
    return form.assemble(*args, **kwargs)
