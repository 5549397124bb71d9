"""BilinearForm / LinearForm / asm: the reference's assembly API on the GPU.

  Form.__init__ / decorator       skfem/assembly/form/form.py:32-71
  Form._normalize_asm_kwargs      form.py:91-121 (coefficient formats)
  BilinearForm.assemble           bilinear_form.py:130-148 -> scipy CSR
  LinearForm.assemble             form.py:73-80 + linear_form.py:18-46 -> ndarray
  Functional.elemental/assemble   functional.py:19-61 -> ndarray / float64
  asm                             skfem/assembly/__init__.py:69-97

``assemble`` returns what the reference returns (scipy.sparse.csr_matrix /
numpy array, canonical CSR with the reference's pattern); ``assemble_torch``
returns the device-resident result (torch sparse CSR / tensor) without a
host round trip.  The form callable is traced once (tracer.py).  Forms of
the isotropic coefficient families run on the channel kernels (exact
reference tensors, FP64); every other form -- anisotropic or advection
terms, coefficients varying inside cells, interpolated DOF vectors, w.x and
w.h, numpy functions -- runs on the generic kernels, which evaluate the
traced program per quadrature point with the reference's own operation
order.  Coefficients stay on the device.
"""

import ctypes
import numbers
import os

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as N
from .field import DiscreteField
from .tracer import (FieldSpec, bilinear_channels, linear_channels, trace_bilinear, trace_linear,
                     trace_tape)

__all__ = ["Form", "BilinearForm", "LinearForm", "Functional", "asm", "ElementField"]


def _zeros_like(x):
    """A zero argument of the same kind as a form argument x (the traced
    stand-ins of the GPU path, or a DiscreteField), for Form.block: the
    reference passes ``arg.zeros()``."""
    from .tracer import Sym, SymField, TapeNode
    if isinstance(x, DiscreteField):
        return x.zeros()
    if isinstance(x, SymField):
        z = SymField(np.vectorize(lambda c: _zeros_like(c), otypes=[object])(np.asarray(x)))
        if getattr(x, "grad", None) is not None:
            z.grad = np.vectorize(lambda c: _zeros_like(c), otypes=[object])(x.grad)
        return z
    if isinstance(x, Sym):
        z = Sym()
        if getattr(x, "grad", None) is not None:
            z.grad = np.array([Sym() for _ in x.grad], dtype=object)
        return z
    if isinstance(x, TapeNode):
        z = x.tape.const(0.0)
        if getattr(x, "grad", None) is not None:
            z.grad = np.array([x.tape.const(0.0) for _ in x.grad], dtype=object)
        return z
    if isinstance(x, np.ndarray):
        return np.zeros_like(x)
    return 0.0 * x


class ElementField:
    """An explicit per-element coefficient (one value per cell), accepted
    wherever the reference takes a (nelems, nqp) array that is constant in
    each cell.  Holds a host array or a device tensor."""

    def __init__(self, values):
        self.values = values


class _Coefficients:
    """Form arguments normalised to device tensors (form.py:91-121):

      fields   name -> (nelems,)        one value per cell
      qfields  name -> (nelems, nqp)    values varying inside cells
      dfields  name -> (tensor (nquant, nelems, nqp), FieldSpec)
               DiscreteFields: interpolated DOF vectors (1-D arrays of
               length N, abstract_basis.py:271-322) or given fields
    """

    def __init__(self, basis, kwargs, strided=False):
        self.fields = {}
        self.qfields = {}
        self.dfields = {}
        self.numbers = {}
        self.strided = {}   # name -> (nelems, nqp) device copy checked inside the kernels
        self.strided_host = {}   # name -> its host array, not yet uploaded
        self.keep = []
        dev = basis.device
        ne = basis.nelems
        nqp = basis.X.shape[-1]
        dim = basis.mesh.p.shape[0]
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
            if isinstance(v, DiscreteField) or hasattr(v, "grad") and isinstance(v, np.ndarray):
                self._discrete_field(k, v, basis, dim, ne, nqp)
                continue
            if isinstance(v, torch.Tensor):
                t = v.to(device=dev, dtype=torch.float64)
                if t.dim() == 1 and t.shape[0] != ne:
                    if t.shape[0] != basis.N:
                        raise ValueError("Input array has wrong size.")
                    self._dof_vector(k, t, basis, dim)
                    continue
            elif isinstance(v, np.ndarray):
                if v.ndim == 1:
                    if v.shape[0] != basis.N:
                        raise ValueError("Input array has wrong size.")  # abstract_basis.py:284-285
                    self._dof_vector(k, v, basis, dim)
                    continue
                if strided and v.shape == (ne, nqp) and nqp > 1 and ne > 0:
                    # the channel kernels read column 0 and check each row
                    # is constant (FEM_ERR_VARYING), no separate pass; the
                    # upload is left to the caller (pipelined with the kernels)
                    self.strided[k] = torch.empty((ne, nqp), dtype=torch.float64, device=dev)
                    self.strided_host[k] = np.ascontiguousarray(v, dtype=np.float64)
                    self.fields[k] = None
                    continue
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
                self.qfields[k] = t.contiguous()      # varies inside cells: generic kernels
            else:
                self.fields[k] = col

    def _dof_vector(self, name, w, basis, dim):
        t = basis.interpolate_torch(w)
        self.dfields[name] = (t, FieldSpec("field", dim if basis.elem.vector else 0, True))

    def _discrete_field(self, name, v, basis, dim, ne, nqp):
        dev = getattr(v, "_dev", None)
        if dev is not None and dev[1] is basis:
            self.dfields[name] = (dev[0], FieldSpec("field", dim if basis.elem.vector else 0,
                                                    True))
            return
        value = np.asarray(v, dtype=np.float64)
        if value.shape[-2:] != (ne, nqp):
            raise ValueError("Quadrature mismatch: '{}' should have same number of "
                             "integration points as the basis object.".format(name))
        if value.ndim == 2:
            ncomp, parts = 0, [value[None]]
        elif value.ndim == 3:
            ncomp, parts = value.shape[0], [value]
        else:
            raise NotImplementedError("fields of rank > 1 are not supported")
        grad = getattr(v, "grad", None)
        if grad is not None:
            grad = np.asarray(grad, dtype=np.float64)
            parts.append(grad.reshape((-1, ne, nqp)))
        t = torch.from_numpy(np.ascontiguousarray(np.concatenate(parts, axis=0))).to(basis.device)
        self.dfields[name] = (t, FieldSpec("field", ncomp, grad is not None))

    def upload(self, begin=0, end=None, stream=None):
        """Copy rows [begin, end) of the strided host arrays to the device."""
        for k, t in self.strided.items():
            h = torch.from_numpy(self.strided_host[k][begin:end])
            if stream is None:
                t[begin:end].copy_(h)
            else:
                with torch.cuda.stream(stream):
                    t[begin:end].copy_(h, non_blocking=True)

    @property
    def generic(self):
        """Arguments only the generic per-point kernels take."""
        return bool(self.qfields or self.dfields)

    def specs(self):
        s = {k: FieldSpec("elem") for k in self.fields}
        s.update({k: FieldSpec("qp") for k in self.qfields})
        s.update({k: spec for k, (_, spec) in self.dfields.items()})
        return s

    def slot(self, key, ne, nq):
        """Device pointer and stride of a program coefficient slot."""
        if isinstance(key, tuple):
            t, _ = self.dfields[key[0]]
            return t.data_ptr() + key[1] * ne * nq * 8, nq
        if key in self.qfields:
            return self.qfields[key].data_ptr(), nq
        return self.fields[key].data_ptr(), 0

    def coef(self, poly, ne, device):
        """Poly -> FemCoef (scale, field pointer, stride)."""
        items = [(names, c) for names, c in poly.items() if c != 0.0]
        if not items:
            return N.FemCoef(0.0, None)
        if len(items) == 1:
            names, c = items[0]
            if names == ():
                return N.FemCoef(c, None)
            if len(names) == 1:
                n = names[0]
                if n in self.strided:
                    a = self.strided[n]
                    return N.FemCoef(c, a.data_ptr(), a.shape[1])
                return N.FemCoef(c, self.fields[n].data_ptr())
        if any(n in self.strided for names, _ in items for n in names):
            raise _StridedFieldInProduct()
        acc = torch.zeros(ne, dtype=torch.float64, device=device)
        for names, c in items:
            term = torch.full((ne,), c, dtype=torch.float64, device=device)
            for n in names:
                term = term * self.fields[n]
            acc = acc + term
        self.keep.append(acc)
        return N.FemCoef(1.0, acc.data_ptr())


class _StridedFieldInProduct(Exception):
    """A strided (unchecked) coefficient enters a product of fields: the
    caller normalises the coefficients with a separate check instead."""


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

    def block(self, *args):
        """form.py:53-60: the block of a form written on product spaces --
        block(i, j) of form(u0, u1, ..., v0, v1, ..., w) is the form of
        (u, v, w) that passes u as u_i, v as v_j and zero fields in the
        other slots."""
        import inspect
        orig = self.form
        nargs = len(inspect.signature(orig).parameters)

        def blk(*arg):
            per = (nargs - 1) // (len(arg) - 1)
            return orig(*[arg[k] if args[k] == j else _zeros_like(arg[k])
                          for k in range(len(arg) - 1) for j in range(per)], arg[-1])
        blk.__name__ = getattr(orig, "__name__", "form")
        return type(self)(form=blk, dtype=self.dtype, nthreads=self.nthreads, **self.params)

    def elemental(self, *args, **kwargs):
        """form.py:82-85: the unassembled element values as a COOData."""
        return self._coo(*args, **kwargs)

    def coo_data(self, *args, **kwargs):
        """form.py:87-89 (the older name of elemental)."""
        return self._coo(*args, **kwargs)

    # tracing is cached per (element kind, field names, numbers)
    def _key(self, basis, coeffs, kind):
        return (kind, type(basis).__name__, basis.elem.family, basis.elem.vector,
                basis.mesh.p.shape[0],
                tuple(sorted((k, s.kind, s.ncomp, s.grad) for k, s in coeffs.specs().items())),
                tuple(sorted(coeffs.numbers.items(), key=repr)))

    def _trace(self, basis, coeffs, kind):
        """The form's coefficient channels, or None when only the generic
        per-point kernels can assemble it (a form outside the isotropic
        channel families, arguments varying inside cells, w.x / w.h, numpy
        functions, or a basis whose quadrature rule the channel kernels do
        not integrate with)."""
        if coeffs.generic or not basis._fast_ok:
            return None
        key = ("channels",) + self._key(basis, coeffs, kind)
        if key in self._traces:
            return self._traces[key]
        dim = basis.mesh.p.shape[0]
        try:
            if kind == "bilinear":
                sym = trace_bilinear(self.form, basis.elem, dim, coeffs.fields, coeffs.numbers)
                ch = bilinear_channels(sym, basis.elem, dim)
            else:
                sym = trace_linear(self.form, basis.elem, dim, coeffs.fields, coeffs.numbers)
                ch = linear_channels(sym, basis.elem, dim)
        except (NotImplementedError, TypeError):
            ch = None
        self._traces[key] = ch
        return ch

    def _generic(self, basis, coeffs, kind, ubasis=None):
        """The form's program for the generic kernels (cached per argument
        structure) and its cache key.  basis: the test basis; ubasis: a trial
        basis of its own (bilinear forms)."""
        key = ("program",) + self._key(basis, coeffs, kind)
        if ubasis is not None:
            key += ("trial", ubasis.elem.family, ubasis.elem.vector)
        g = self._traces.get(key)
        if g is None:
            ins, out, names = trace_tape(self.form, basis.elem, basis.mesh.p.shape[0],
                                         coeffs.specs(), coeffs.numbers, kind=kind,
                                         defaults="facet" if hasattr(basis, "c_facets")
                                         else "cell",
                                         uelem=ubasis.elem if ubasis is not None else None)
            g = _GenericProgram(ins, out, names)
            self._traces[key] = g
        return g, key


class _GenericProgram:
    """A traced form program and its per-device instruction arrays."""

    def __init__(self, ins, out, names):
        if len(ins) > MAX_PROGRAM:
            raise NotImplementedError("the form traces to %d operations per point (limit %d)"
                                      % (len(ins), MAX_PROGRAM))
        if len(names) > MAX_COEF:
            raise NotImplementedError("the form reads %d coefficient quantities (limit %d)"
                                      % (len(names), MAX_COEF))
        self.ins, self.out, self.names = ins, out, names
        self._host = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm)
                                               for op, a, b, imm in ins])
        self._dev = {}
        self._compiled = {}

    def struct(self, basis, coeffs, kind, ubasis=None):
        dev = self._dev.get(basis.device)
        if dev is None:
            dev = torch.frombuffer(bytearray(self._host), dtype=torch.uint8).to(basis.device)
            self._dev[basis.device] = dev
        nq = basis.X.shape[1]
        prog = N.FemProgram(len(self.ins), self.out, len(self.names), nq, dev.data_ptr())
        for k, n in enumerate(self.names):
            prog.coef[k], prog.coef_stride[k] = coeffs.slot(n, basis.nelems, nq)
        prog.qX = basis.X_dev.data_ptr()
        prog.qW = basis.W_dev.data_ptr()
        prog.compiled = self._kernel(basis, kind, ubasis)
        return prog

    def _kernel(self, basis, kind, ubasis=None):
        """The program compiled to straight-line code for this basis kind
        (once; None keeps the interpreter: compilation disabled with
        SKFEM_GB300_JIT=0 or unavailable)."""
        if os.environ.get("SKFEM_GB300_JIT", "1") == "0":
            return None
        mode = {"bilinear": 0, "linear": 1, "functional": 2}[kind]
        facet = int(hasattr(basis, "c_facets"))
        dim = basis.mesh.p.shape[0]
        vec_u = int((ubasis if ubasis is not None else basis).elem.vector)
        key = (str(basis.device), dim, int(basis.elem.vector), vec_u, mode, facet)
        if key not in self._compiled:
            h = ctypes.c_void_p()
            with torch.cuda.device(basis.device):
                rc = N.lib().fem_program_compile(ctypes.addressof(self._host), len(self.ins),
                                                 self.out, len(self.names), dim,
                                                 int(basis.elem.vector), vec_u, mode, facet,
                                                 ctypes.byref(h))
            if rc == N.FEM_ERR_UNSUPPORTED:
                self._compiled[key] = None
            else:
                N.check(rc)
                self._compiled[key] = h
        h = self._compiled[key]
        return h.value if h is not None else None

    def __del__(self):
        try:
            for h in self._compiled.values():
                if h is not None:
                    N.lib().fem_program_release(h)
        except Exception:
            pass


MAX_PROGRAM = 512
MAX_COEF = 16


def _structure_key(ch):
    return tuple(sorted((name, tuple(sorted(names for names, c in p.items() if c != 0.0)))
                        for name, p in ch.items()))


def _program(form, basis, coeffs):
    """The form's exact-order program (tracer.trace_tape) on the device, for
    the exact-zero mask of the channel kernels' pattern build."""
    try:
        ins, out, names = trace_tape(form.form, basis.elem, basis.mesh.p.shape[0],
                                     list(coeffs.fields), coeffs.numbers)
    except NotImplementedError:
        # an operation the replay cannot reproduce bit for bit: the mask then
        # comes from the separately rounded tensor-form evaluation alone
        return None, None
    if len(ins) > MAX_PROGRAM or len(names) > MAX_COEF:
        return None, None
    arr = (N.FemInstr * len(ins))(*[N.FemInstr(op, a, b, 0, imm) for op, a, b, imm in ins])
    dev = torch.frombuffer(bytearray(arr), dtype=torch.uint8).to(basis.device)
    prog = N.FemProgram(len(ins), out, len(names), basis.X.shape[1], dev.data_ptr())
    for k, n in enumerate(names):
        if n in coeffs.strided:
            prog.coef[k] = coeffs.strided[n].data_ptr()
            prog.coef_stride[k] = coeffs.strided[n].shape[1]
        else:
            prog.coef[k] = coeffs.fields[n].data_ptr()
    prog.qX = basis.X_dev.data_ptr()
    prog.qW = basis.W_dev.data_ptr()
    return prog, dev


class _PatternEntry:
    def __init__(self, basis, c_form, stream, program=None, local=None, ubasis=None):
        lib = N.lib()
        h = ctypes.c_void_p()
        if ubasis is not None:
            # basis: the test basis (rows), ubasis: the trial basis (columns)
            N.check(lib.fem_pattern_build_local_mixed(N.byref(basis.c_mesh), N.byref(basis.c_basis),
                                                      N.byref(ubasis.c_basis), N.ptr(local),
                                                      ctypes.byref(h), stream))
        elif local is not None:
            N.check(lib.fem_pattern_build_local(N.byref(basis.c_mesh_pat),
                                                N.byref(basis.c_basis_pat), N.ptr(local),
                                                ctypes.byref(h), stream))
        else:
            N.check(lib.fem_pattern_build(N.byref(basis.c_mesh_pat), N.byref(basis.c_basis_pat),
                                          N.byref(c_form) if c_form is not None else None,
                                          N.byref(program) if program is not None else None,
                                          ctypes.byref(h), stream))
        self.pat = N.Pattern(h.value)
        dev = basis.device
        self.nrows = self.pat.nrows
        self.nnz = self.pat.nnz
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        if c_form is not None or local is not None or ubasis is not None:
            self.indptr = torch.empty(self.nrows + 1, dtype=torch.int32, device=dev)
            self.indices = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=dev)[:self.nnz]
            N.check(lib.fem_pattern_export(self.pat.handle, N.ptr(self.indptr),
                                           N.ptr(self.indices), stream))
            if local is None:
                self.staging = torch.empty(max(1, self.pat.staging_bytes // 8),
                                           dtype=torch.float64, device=dev)
            torch.cuda.current_stream().synchronize()
        else:
            self.staging = torch.empty(max(1, basis.nelems * basis.Nbfun), dtype=torch.float64,
                                       device=dev)
        self.geo_key = None
        if c_form is not None and local is None and ubasis is None:
            self.refresh_geometry(basis, stream)

    def refresh_geometry(self, basis, stream=None):
        """The channel pattern's per-cell geometry cache of scalar simplex
        bases -- CellBasis keeps its mapping the same way -- recomputed when
        the basis's coordinates changed: in place (the tensor's version
        counter) or replaced (its pointer); an opted-in coefficient-update
        cache is refreshed with it.  While the mesh points at other
        coordinates (the adjoint's X) the kernels compute the geometry and
        run the two-pass assembly."""
        p = basis.p_dev
        if basis.c_mesh.p != p.data_ptr():
            return
        key = (p.data_ptr(), p._version)
        if key == self.geo_key:
            return
        N.check(N.lib().fem_pattern_cache_geometry(
            self.pat.handle, N.byref(basis.c_mesh), N.byref(basis.c_basis),
            stream if stream is not None else N.stream_ptr()))
        self.geo_key = key

    def ensure_caches(self, basis, key, stream):
        """The geometry cache, and the coefficient-update cache when the
        basis asked for one on this form structure (kept across pattern
        rebuilds)."""
        self.refresh_geometry(basis, stream)
        if key in basis.__dict__.get("_coef_update", ()) and not getattr(self, "coef_update", False):
            if self.geo_key is None:
                return
            N.check(N.lib().fem_pattern_cache_coefficient_update(
                self.pat.handle, N.byref(basis.c_mesh), N.byref(basis.c_basis), stream))
            self.coef_update = True


_SIDE = {}
_COPY = {}
HOST_CHUNKS = 16    # row ranges whose device->host copies overlap the segmented sum
# cell ranges whose coefficient uploads overlap the kernels (6M TetP1 cells:
# 1.86 ms per call, against 1.91 ms with 8, 1.99 ms with 4, 1.93 ms with 32)
UPLOAD_CHUNKS = 16


def _copy_stream(device):
    """A per-device stream for host->device coefficient uploads, at the
    highest priority: its kernels (host-row gathers) take SMs ahead of the
    local kernels that wait for them."""
    s = _COPY.get(device)
    if s is None:
        hi = torch.cuda.Stream.priority_range()[1]
        s = _COPY[device] = torch.cuda.Stream(device=device, priority=hi)
    return s


def _side_stream(device):
    """A per-device stream for copies that overlap the assembly kernels."""
    s = _SIDE.get(device)
    if s is None:
        s = _SIDE[device] = torch.cuda.Stream(device=device)
    return s


def _raise_status(st):
    if st & (1 << N.FEM_ERR_ZERO_JACOBIAN):
        raise N.ZeroJacobianError("Zero Jacobian determinant")
    if st & (1 << N.FEM_ERR_ARGUMENT):
        raise ValueError("a facet's cell index is out of range")


def _host_csr(entry, vals, n, ncols=None):
    """Device CSR -> scipy.sparse.csr_matrix through pinned host buffers
    (torch's caching host allocator reuses the blocks of matrices the
    caller has dropped); the matrix owns its arrays through numpy views."""
    data = torch.empty(entry.nnz, dtype=torch.float64, pin_memory=True)
    indices = torch.empty(entry.nnz, dtype=torch.int32, pin_memory=True)
    indptr = torch.empty(entry.nrows + 1, dtype=torch.int32, pin_memory=True)
    data.copy_(vals, non_blocking=True)
    indices.copy_(entry.indices, non_blocking=True)
    indptr.copy_(entry.indptr, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    K = sp.csr_matrix((data.numpy(), indices.numpy(), indptr.numpy()),
                      shape=(n, n if ncols is None else ncols), copy=False)
    K.has_sorted_indices = True
    K.has_canonical_format = True
    return K


class BilinearForm(Form):
    """bilinear_form.py:19-151."""

    def _setup(self, ubasis, vbasis, kwargs):
        """Coefficients, channels and FemBilinear of a form the channel
        kernels take (NotImplementedError otherwise)."""
        if vbasis is not None and vbasis is not ubasis:
            raise NotImplementedError("different trial and test bases are not supported yet")
        coeffs = _Coefficients(ubasis, kwargs)
        ch = self._trace(ubasis, coeffs, "bilinear")
        if ch is None:
            raise NotImplementedError("this form / basis is assembled by the generic per-point "
                                      "kernels only (no coefficient-channel form)")
        return (coeffs, ch) + (self._c_form(ubasis, coeffs, ch),)

    @staticmethod
    def _c_form(ubasis, coeffs, ch):
        ne, dev = ubasis.nelems, ubasis.device
        z = N.FemCoef(0.0, None)
        if ubasis.elem.vector:
            return N.FemBilinear(z, coeffs.coef(ch["mass"], ne, dev),
                                 coeffs.coef(ch["lam"], ne, dev), coeffs.coef(ch["lap"], ne, dev),
                                 coeffs.coef(ch["tr"], ne, dev))
        return N.FemBilinear(coeffs.coef(ch["diff"], ne, dev), coeffs.coef(ch["mass"], ne, dev),
                             z, z, z)

    # ---------------------------------------------------- channel kernels
    def _fast_once(self, ubasis, coeffs, ch):
        c_form = self._c_form(ubasis, coeffs, ch)
        stream = N.stream_ptr()
        key = ("bilinear", _structure_key(ch))
        entry = ubasis._patterns.get(key)
        if entry is None:
            prog, keep = _program(self, ubasis, coeffs)
            entry = _PatternEntry(ubasis, c_form, stream, prog)
            del keep
            ubasis._patterns[key] = entry
        entry.ensure_caches(ubasis, key, stream)
        vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64, device=ubasis.device)[:entry.nnz]
        entry.status.zero_()
        N.check(N.lib().fem_assemble(N.byref(ubasis.c_mesh), N.byref(ubasis.c_basis),
                                     N.byref(c_form), entry.pat.handle, N.ptr(entry.staging),
                                     N.ptr(vals), N.ptr(entry.status), stream))
        return entry, vals, key

    # ---------------------------------------------------- generic kernels
    def _local_generic(self, basis, coeffs):
        g, key = self._generic(basis, coeffs, "bilinear")
        prog = g.struct(basis, coeffs, "bilinear")
        nb = basis.Nbfun
        local = torch.empty(max(1, basis.nelems * nb * nb), dtype=torch.float64,
                            device=basis.device)
        status = torch.zeros(1, dtype=torch.int32, device=basis.device)
        basis._run_program("bilinear", prog, local, status)
        return local, status, key

    def _generic_assemble(self, basis, coeffs, check):
        local, status, key = self._local_generic(basis, coeffs)
        stream = N.stream_ptr()
        entry = basis._patterns.get(key)
        fresh = entry is None
        if fresh:
            entry = _PatternEntry(basis, None, stream, local=local)
            basis._patterns[key] = entry
        vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64, device=basis.device)[:entry.nnz]
        N.check(N.lib().fem_csr_sum_checked(entry.pat.handle, N.ptr(local), N.ptr(vals),
                                            N.ptr(status), stream))
        if check or fresh:
            st = int(status.item())
            _raise_status(st)
            if st & (1 << N.FEM_ERR_STALE_PATTERN):
                # the exact-zero structure changed: rebuild from these local
                # matrices (they are exact, so the new pattern is final)
                entry = _PatternEntry(basis, None, stream, local=local)
                basis._patterns[key] = entry
                vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64,
                                   device=basis.device)[:entry.nnz]
                N.check(N.lib().fem_csr_sum(entry.pat.handle, N.ptr(local), N.ptr(vals), None,
                                            stream))
        return entry, vals

    # ---------------------------------------------- different trial / test
    def _check_pair(self, ubasis, vbasis):
        """bilinear_form.py:64-70: both bases on the same cells and points."""
        if hasattr(ubasis, "c_facets") or hasattr(vbasis, "c_facets"):
            raise NotImplementedError("different trial and test FacetBases are not supported")
        if ubasis.X.shape[1] != vbasis.X.shape[1] or not np.array_equal(ubasis.X, vbasis.X):
            raise ValueError("Quadrature mismatch: trial and test functions should have "
                             "same number of integration points.")
        same_mesh = ubasis.mesh is vbasis.mesh or (
            np.array_equal(ubasis.mesh.p, vbasis.mesh.p) and
            np.array_equal(ubasis.mesh.t, vbasis.mesh.t))
        same_cells = (ubasis.tind is None and vbasis.tind is None) or (
            ubasis.tind is not None and vbasis.tind is not None and
            np.array_equal(ubasis.tind, vbasis.tind))
        if not (same_mesh and same_cells):
            raise NotImplementedError("trial and test bases on different cells are not supported")

    def _mixed_assemble(self, ubasis, vbasis, kwargs, check=True):
        self._check_pair(ubasis, vbasis)
        coeffs = _Coefficients(ubasis, kwargs)                 # form.py:91-121 (ubasis)
        g, key = self._generic(vbasis, coeffs, "bilinear", ubasis)
        prog = g.struct(vbasis, coeffs, "bilinear", ubasis)
        nl = vbasis.nelems * vbasis.Nbfun * ubasis.Nbfun
        local = torch.empty(max(1, nl), dtype=torch.float64, device=vbasis.device)
        status = torch.zeros(1, dtype=torch.int32, device=vbasis.device)
        stream = N.stream_ptr()
        N.check(N.lib().fem_program_local_matrices_mixed(
            N.byref(vbasis.c_mesh), N.byref(vbasis.c_basis), N.byref(ubasis.c_basis),
            N.byref(prog), N.ptr(local), N.ptr(status), stream))
        pkey = key + ("trial-dofs", ubasis.N)
        entry = vbasis._patterns.get(pkey)
        fresh = entry is None
        if fresh:
            entry = _PatternEntry(vbasis, None, stream, local=local, ubasis=ubasis)
            vbasis._patterns[pkey] = entry
        vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64, device=vbasis.device)[:entry.nnz]
        N.check(N.lib().fem_csr_sum_checked(entry.pat.handle, N.ptr(local), N.ptr(vals),
                                            N.ptr(status), stream))
        if check or fresh:
            st = int(status.item())
            _raise_status(st)
            if st & (1 << N.FEM_ERR_STALE_PATTERN):
                entry = _PatternEntry(vbasis, None, stream, local=local, ubasis=ubasis)
                vbasis._patterns[pkey] = entry
                vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64,
                                   device=vbasis.device)[:entry.nnz]
                N.check(N.lib().fem_csr_sum(entry.pat.handle, N.ptr(local), N.ptr(vals), None,
                                            stream))
        return entry, vals

    # ------------------------------------------------------------- driver
    def _assemble_device(self, ubasis, vbasis, kwargs, check=True, coeffs=None):
        if vbasis is not None and vbasis is not ubasis:
            raise NotImplementedError("different trial and test bases are not supported yet")
        if coeffs is None:
            coeffs = _Coefficients(ubasis, kwargs)
        ch = self._trace(ubasis, coeffs, "bilinear")
        if ch is None:
            return self._generic_assemble(ubasis, coeffs, check)
        for attempt in range(2):
            entry, vals, key = self._fast_once(ubasis, coeffs, ch)
            if not check:
                break
            st = int(entry.status.item())
            _raise_status(st)
            if not st & (1 << N.FEM_ERR_STALE_PATTERN):
                break
            del ubasis._patterns[key]
        return entry, vals

    def assemble(self, ubasis, vbasis=None, **kwargs):
        """Assemble into a scipy.sparse.csr_matrix (bilinear_form.py:130-148).

        On the channel kernels (nelems, nqp) coefficient arrays are copied
        whole and their rows checked inside the local kernel, the pattern's
        index arrays are copied to the host on a side stream while the
        kernels run, and the call synchronises once before returning."""
        if vbasis is not None and vbasis is not ubasis:
            entry, vals = self._mixed_assemble(ubasis, vbasis, kwargs)
            return _host_csr(entry, vals, vbasis.N, ubasis.N)
        coeffs = _Coefficients(ubasis, kwargs, strided=True)
        ch = self._trace(ubasis, coeffs, "bilinear")
        if ch is not None:
            try:
                K = self._assemble_to_host(ubasis, coeffs, ch)
            except _StridedFieldInProduct:
                K = None
            if K is not None:
                return K
        if coeffs.strided or ch is not None:
            coeffs = _Coefficients(ubasis, kwargs)          # rows checked up front
        entry, vals = self._assemble_device(ubasis, None, kwargs, coeffs=coeffs)
        return _host_csr(entry, vals, ubasis.N)

    def _assemble_to_host(self, ubasis, coeffs, ch):
        """Channel kernels, results copied to pinned host memory; None when
        a per-point coefficient varies inside a cell.

        One native call queues the pipeline: the cells in order of their
        smallest DOF, in UPLOAD_CHUNKS chunks; per chunk the strided host
        coefficients' rows are read from host memory by a kernel on a copy
        stream, the chunk's coefficient checks (with the fused cache) or
        local kernel follow, and the rows it completes are summed and copied
        back behind their sum -- the upload, the kernels and the copy of the
        values overlap.  Where kernels cannot read pageable host memory the
        coefficients are uploaded first."""
        main = torch.cuda.current_stream()
        uploaded = False
        for attempt in range(2):
            c_form = self._c_form(ubasis, coeffs, ch)
            stream = N.stream_ptr(main)
            key = ("bilinear", _structure_key(ch))
            entry = ubasis._patterns.get(key)
            if entry is None:
                if not uploaded:
                    coeffs.upload()
                    uploaded = True
                prog, keep = _program(self, ubasis, coeffs)
                entry = _PatternEntry(ubasis, c_form, stream, prog)
                del keep
                ubasis._patterns[key] = entry
            entry.ensure_caches(ubasis, key, stream)
            data = torch.empty(entry.nnz, dtype=torch.float64, pin_memory=True)
            indices = torch.empty(entry.nnz, dtype=torch.int32, pin_memory=True)
            indptr = torch.empty(entry.nrows + 1, dtype=torch.int32, pin_memory=True)
            side = _side_stream(ubasis.device)
            side.wait_stream(main)
            with torch.cuda.stream(side):
                indices.copy_(entry.indices, non_blocking=True)
                indptr.copy_(entry.indptr, non_blocking=True)
            vals = torch.empty(max(entry.nnz, 1), dtype=torch.float64, device=ubasis.device)
            entry.status.zero_()
            lib = N.lib()
            ne = ubasis.nelems
            nch = UPLOAD_CHUNKS if ne >= UPLOAD_CHUNKS * 4096 else 1
            rows, nrows = None, 0
            if coeffs.strided and not uploaded:
                if entry.nnz and N.host_memory_access():
                    fields = [(coeffs.strided_host[k], t) for k, t in coeffs.strided.items()]
                    rows = (N.FemHostRows * len(fields))(*[
                        N.FemHostRows(h.ctypes.data, t.data_ptr(), h.shape[1] if h.ndim > 1 else 0)
                        for h, t in fields])
                    nrows = len(fields)
                else:
                    coeffs.upload()
                uploaded = True
            if entry.nnz:
                up = _copy_stream(ubasis.device)
                rc = lib.fem_assemble_to_host_pipelined(
                    N.byref(ubasis.c_mesh), N.byref(ubasis.c_basis), N.byref(c_form),
                    entry.pat.handle, N.ptr(entry.staging), N.ptr(vals),
                    ctypes.c_void_p(data.data_ptr()), N.ptr(entry.status), rows, nrows, nch,
                    stream, N.stream_ptr(up), N.stream_ptr(side))
                if rc:
                    # gathers already queued read the host arrays and write the
                    # device ones: let them finish before either can be freed
                    up.synchronize()
                    N.check(rc)
            else:
                N.check(lib.fem_assemble_local(
                    N.byref(ubasis.c_mesh), N.byref(ubasis.c_basis), N.byref(c_form),
                    entry.pat.handle, N.ptr(entry.staging), N.ptr(entry.status), 0, ne, stream))
            st_h = torch.empty(1, dtype=torch.int32, pin_memory=True)
            st_h.copy_(entry.status, non_blocking=True)
            main.synchronize()
            side.synchronize()
            st = int(st_h[0])
            _raise_status(st)
            if st & (1 << N.FEM_ERR_VARYING):
                return None
            if st & (1 << N.FEM_ERR_STALE_PATTERN):
                del ubasis._patterns[key]
                continue
            K = sp.csr_matrix((data.numpy(), indices.numpy(), indptr.numpy()),
                              shape=(ubasis.N, ubasis.N), copy=False)
            K.has_sorted_indices = True
            K.has_canonical_format = True
            return K
        raise RuntimeError("the CSR pattern went stale twice in one call")

    def assemble_torch(self, ubasis, vbasis=None, check=True, **kwargs):
        """Device-resident result: torch.sparse_csr_tensor (int32 indices,
        float64 values) sharing the cached pattern arrays."""
        if vbasis is not None and vbasis is not ubasis:
            entry, vals = self._mixed_assemble(ubasis, vbasis, kwargs, check=check)
            return torch.sparse_csr_tensor(entry.indptr, entry.indices, vals,
                                           size=(vbasis.N, ubasis.N))
        entry, vals = self._assemble_device(ubasis, vbasis, kwargs, check=check)
        return torch.sparse_csr_tensor(entry.indptr, entry.indices, vals,
                                       size=(ubasis.N, ubasis.N))

    def _coo(self, ubasis, vbasis=None, idx=None, **kwargs):
        """bilinear_form.py:58-128's COO triplet: data[j, i, e] (trial j,
        test i, cell e) flattened in C order, rows = the test basis's DOFs,
        cols = the trial basis's.  The local values come from the generic
        kernels, which evaluate the form with the reference's own sequence
        of operations: the data are the reference's bit for bit, so the
        exact zeros that COOData.tocsr drops (eliminate_zeros) are its."""
        from .coo import COOData
        if idx is not None:
            kwargs["idx"] = idx
        if vbasis is None or vbasis is ubasis:
            vbasis = ubasis
            nb = ubasis.Nbfun
            flat, status, _ = self._local_generic(ubasis, _Coefficients(ubasis, kwargs))
            _raise_status(int(status.item()))
            local = flat[:ubasis.nelems * nb * nb].view(ubasis.nelems, nb, nb)   # (ne, Nv, Nu)
        else:
            local = self._mixed_local(ubasis, vbasis, kwargs)
        dev = local.device
        ne, nv, nu = local.shape
        data = local.permute(2, 1, 0).reshape(-1)
        edv = torch.as_tensor(np.ascontiguousarray(vbasis.element_dofs), device=dev)
        edu = torch.as_tensor(np.ascontiguousarray(ubasis.element_dofs), device=dev)
        rows = edv[None, :, :].expand(nu, nv, ne).reshape(-1)
        cols = edu[:, None, :].expand(nu, nv, ne).reshape(-1)
        return COOData(np.stack([rows.cpu().numpy(), cols.cpu().numpy()]).astype(np.int32),
                       data.cpu().numpy(), (vbasis.N, ubasis.N), (vbasis.Nbfun, ubasis.Nbfun))

    def _mixed_local(self, ubasis, vbasis, kwargs):
        """Local matrices (ne, Nv, Nu) of a trial / test basis pair (generic
        kernels, as _mixed_assemble computes them)."""
        self._check_pair(ubasis, vbasis)
        coeffs = _Coefficients(ubasis, kwargs)
        g, _ = self._generic(vbasis, coeffs, "bilinear", ubasis)
        prog = g.struct(vbasis, coeffs, "bilinear", ubasis)
        nl = vbasis.nelems * vbasis.Nbfun * ubasis.Nbfun
        local = torch.empty(max(1, nl), dtype=torch.float64, device=vbasis.device)
        status = torch.zeros(1, dtype=torch.int32, device=vbasis.device)
        N.check(N.lib().fem_program_local_matrices_mixed(
            N.byref(vbasis.c_mesh), N.byref(vbasis.c_basis), N.byref(ubasis.c_basis),
            N.byref(prog), N.ptr(local), N.ptr(status), N.stream_ptr()))
        _raise_status(int(status.item()))
        return local[:nl].view(vbasis.nelems, vbasis.Nbfun, ubasis.Nbfun)

    def elemental_torch(self, ubasis, **kwargs):
        """Local matrices (nelems, Nbfun, Nbfun), row = test function."""
        coeffs = _Coefficients(ubasis, kwargs)
        ch = self._trace(ubasis, coeffs, "bilinear")
        nb = ubasis.Nbfun
        if ch is None:
            local, status, _ = self._local_generic(ubasis, coeffs)
            _raise_status(int(status.item()))
            return local[:ubasis.nelems * nb * nb].view(ubasis.nelems, nb, nb)
        c_form = self._c_form(ubasis, coeffs, ch)
        out = torch.empty((ubasis.nelems, nb, nb), dtype=torch.float64, device=ubasis.device)
        N.check(N.lib().fem_local_matrices(N.byref(ubasis.c_mesh), N.byref(ubasis.c_basis),
                                           N.byref(c_form), N.ptr(out), N.stream_ptr()))
        return out

    def cache_coefficient_update(self, ubasis, **kwargs):
        """Opt into the coefficient-update cache of this form on ``ubasis``
        (no counterpart in the reference): the cells' unit-coefficient
        stiffness rows in the sum's order and the unit-coefficient mass
        matrix are kept, and later assemblies with new per-cell stiffness
        coefficients (and one constant mass coefficient) run as one fused
        sum over them.  For loops that re-assemble one form many times; it
        costs nelems * Nbfun^2 + nnz doubles of device memory.  Scalar
        simplex bases only; elsewhere a no-op."""
        coeffs = _Coefficients(ubasis, kwargs)
        ch = self._trace(ubasis, coeffs, "bilinear")
        if ch is None or ubasis.elem.vector:
            return self
        key = ("bilinear", _structure_key(ch))
        ubasis.__dict__.setdefault("_coef_update", set()).add(key)
        entry, _vals, _key = self._fast_once(ubasis, coeffs, ch)
        return self

    def pattern(self, ubasis, **kwargs):
        """(indptr, indices) device tensors of the cached CSR pattern."""
        entry, _ = self._assemble_device(ubasis, None, kwargs)
        return entry.indptr, entry.indices


class LinearForm(Form):
    """linear_form.py:10-49."""

    def _setup(self, basis, kwargs):
        coeffs = _Coefficients(basis, kwargs)
        ch = self._trace(basis, coeffs, "linear")
        if ch is None:
            raise NotImplementedError("this form / basis is assembled by the generic per-point "
                                      "kernels only (no coefficient-channel form)")
        return coeffs, N.FemLinear(coeffs.coef(ch["load"], basis.nelems, basis.device))

    def _incidence(self, basis, stream):
        key = ("incidence",)
        entry = basis._patterns.get(key)
        if entry is None:
            entry = _PatternEntry(basis, None, stream, None)
            basis._patterns[key] = entry
        return entry

    def _local_generic(self, basis, coeffs):
        g, _ = self._generic(basis, coeffs, "linear")
        prog = g.struct(basis, coeffs, "linear")
        local = torch.empty(max(1, basis.nelems * basis.Nbfun), dtype=torch.float64,
                            device=basis.device)
        status = torch.zeros(1, dtype=torch.int32, device=basis.device)
        basis._run_program("linear", prog, local, status)
        return local, status

    def _device_assemble(self, basis, vbasis=None, **kwargs):
        if vbasis is not None:
            raise ValueError("LinearForm takes one basis")
        coeffs = _Coefficients(basis, kwargs)
        ch = self._trace(basis, coeffs, "linear")
        stream = N.stream_ptr()
        entry = self._incidence(basis, stream)
        b = torch.empty(basis.N, dtype=torch.float64, device=basis.device)
        if ch is None:
            local, status = self._local_generic(basis, coeffs)
            N.check(N.lib().fem_vector_sum(entry.pat.handle, N.ptr(local), N.ptr(b), stream))
            _raise_status(int(status.item()))
            return b, coeffs
        c_form = N.FemLinear(coeffs.coef(ch["load"], basis.nelems, basis.device))
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

    def elemental_torch(self, basis, **kwargs):
        """Local load vectors (nelems, Nbfun) on the device."""
        coeffs = _Coefficients(basis, kwargs)
        ch = self._trace(basis, coeffs, "linear")
        nb = basis.Nbfun
        if ch is None:
            local, status = self._local_generic(basis, coeffs)
            _raise_status(int(status.item()))
            return local[:basis.nelems * nb].view(basis.nelems, nb)
        c_form = N.FemLinear(coeffs.coef(ch["load"], basis.nelems, basis.device))
        out = torch.empty((basis.nelems, nb), dtype=torch.float64, device=basis.device)
        N.check(N.lib().fem_local_vectors(N.byref(basis.c_mesh), N.byref(basis.c_basis),
                                          N.byref(c_form), N.ptr(out), N.stream_ptr()))
        return out

    def _coo(self, basis, vbasis=None, idx=None, **kwargs):
        """linear_form.py:18-46's COO pair: data[i, e] flattened, rows =
        the basis's DOFs (local values from the generic kernels: the
        reference's bit for bit)."""
        from .coo import COOData
        if vbasis is not None:
            raise ValueError("LinearForm takes one basis")
        if idx is not None:
            kwargs["idx"] = idx
        nb = basis.Nbfun
        flat, status = self._local_generic(basis, _Coefficients(basis, kwargs))
        _raise_status(int(status.item()))
        local = flat[:basis.nelems * nb].view(basis.nelems, nb)         # (ne, Nb)
        data = local.t().reshape(-1)
        rows = np.ascontiguousarray(basis.element_dofs, dtype=np.int32).reshape(-1)
        return COOData(rows[None, :], data.cpu().numpy(), (basis.N,), (basis.Nbfun,))


class Functional(Form):
    """functional.py:10-61: a form of ``w`` alone, integrated per cell
    (``elemental``) or over the mesh (``assemble``, numpy's pairwise sum of
    the per-cell values)."""

    def _device_elemental(self, basis, kwargs):
        coeffs = _Coefficients(basis, kwargs)
        g, _ = self._generic(basis, coeffs, "functional")
        prog = g.struct(basis, coeffs, "functional")
        out = torch.empty(max(1, basis.nelems), dtype=torch.float64, device=basis.device)
        status = torch.zeros(1, dtype=torch.int32, device=basis.device)
        basis._run_program("functional", prog, out, status)
        return out[:basis.nelems], status

    def elemental_torch(self, basis, **kwargs):
        out, status = self._device_elemental(basis, kwargs)
        _raise_status(int(status.item()))
        return out

    def elemental(self, v, **kwargs):
        """Per-cell values (functional.py:26-34) as a numpy array."""
        return self.elemental_torch(v, **kwargs).cpu().numpy()

    def assemble_torch(self, ubasis, vbasis=None, **kwargs):
        assert vbasis is None
        e, status = self._device_elemental(ubasis, kwargs)
        total = torch.empty(1, dtype=torch.float64, device=ubasis.device)
        N.check(N.lib().fem_sum_pairwise(N.ptr(e), ubasis.nelems, N.ptr(total), N.stream_ptr()))
        _raise_status(int(status.item()))
        return total[0]

    def assemble(self, ubasis, vbasis=None, **kwargs):
        """The functional's value (functional.py:36-61) as a numpy float64."""
        return np.float64(self.assemble_torch(ubasis, vbasis, **kwargs).item())

    def _coo(self, ubasis, vbasis=None, idx=None, **kwargs):
        """functional.py:36-61's COO form: no indices, one datum (the
        functional's value), a 0-tensor."""
        from .coo import COOData
        if idx is not None:
            kwargs["idx"] = idx
        return COOData(np.array([]), np.array([self.assemble(ubasis, vbasis, **kwargs)]), (), ())


def _sum_blocks(blocks):
    out = sum(blocks)
    assert not isinstance(out, int)
    return out.todefault()


def asm(form, *args, to=_sum_blocks, **kwargs):
    """skfem/assembly/__init__.py:69-97: assemble ``form`` on its bases; an
    argument that is a list of bases assembles every combination (the
    product over the lists), each block told its position as ``w.idx``,
    and ``to`` reduces the blocks' COOData (default: their sum, as
    COOData.__add__ concatenates them, assembled on the GPU).  A single
    combination with the default reducer goes straight to ``assemble``."""
    from itertools import product
    if not isinstance(form, Form):
        import inspect
        nargs = len(inspect.signature(form).parameters)
        form = {3: BilinearForm, 2: LinearForm, 1: Functional}[nargs](form)
    lists = [a if isinstance(a, list) else [a] for a in args]
    if to is _sum_blocks and all(len(a) == 1 for a in lists) and not any(
            isinstance(a, list) for a in args):
        return form.assemble(*[a[0] for a in lists], **kwargs)
    return to(map(lambda a: form.coo_data(*a[1], idx=a[0], **kwargs),
                  zip(product(*(range(len(x)) for x in lists)), product(*lists))))
