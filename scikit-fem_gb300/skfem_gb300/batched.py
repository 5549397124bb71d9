"""Batched assembly of many meshes in one launch, replayed from a CUDA graph.

The reference assembles one mesh per call (a Python loop over meshes is the
batched baseline).  Here meshes of one element family become a single
block-diagonal system: vertices, cells and DOFs are offset per mesh while
each mesh keeps the reference's own numbering (so block m of the result is,
bit for bit, mesh m's scipy CSR).  One pattern build covers all meshes.

Every later step of a scalar simplex basis (TriP1/P2, TetP1/P2) is ONE
persistent launch (fem_batched_assemble_vjp) whose blocks take work units
from a device queue -- per mesh, units of 128 cells (local matrices from the
geometry cache and, with the adjoint, the cells' coefficient gradients from
the same matrices) queued before units of rows (the fixed-order segmented
sum, waiting on the mesh's cell units) -- captured once in a CUDA graph
(a counter reset and the kernel) and replayed.  Other bases, and the
coordinate gradient (with_dX), run the separate local / sum / adjoint
kernels over the union.
"""

import ctypes

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as N
from .basis import CellBasis
from .dofs import Dofs
from .form import _Coefficients
from .mesh import as_mesh

__all__ = ["BatchedBasis", "GraphedAssembly"]


class _Plan:
    """Owns a FemBatchPlan handle."""

    def __init__(self, handle):
        self.handle = handle

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h and N._lib is not None:
            try:
                torch.cuda.synchronize()
            except Exception:
                pass
            N._lib.fem_batch_plan_destroy(h)


class _UnionDofs:
    def __init__(self, element_dofs, N):
        self.element_dofs = element_dofs
        self.N = N


class BatchedBasis(CellBasis):
    """A CellBasis over the disjoint union of ``meshes`` (same element)."""

    def __init__(self, meshes, elem, device=None):
        meshes = [as_mesh(m) for m in meshes]
        if len({type(m) for m in meshes}) != 1:
            raise ValueError("all meshes of a batch must have the same cell type")
        dofs = [Dofs(m, elem) for m in meshes]
        nv = np.array([m.p.shape[1] for m in meshes], dtype=np.int64)
        ne = np.array([m.nelements for m in meshes], dtype=np.int64)
        nd = np.array([d.N for d in dofs], dtype=np.int64)
        self.vert_offsets = np.concatenate(([0], np.cumsum(nv)))
        self.elem_offsets = np.concatenate(([0], np.cumsum(ne)))
        self.dof_offsets = np.concatenate(([0], np.cumsum(nd)))
        if self.dof_offsets[-1] >= np.iinfo(np.int32).max:
            raise ValueError("batch has more DOFs than int32 indices hold")
        p = np.hstack([m.p for m in meshes])
        t = np.hstack([m.t.astype(np.int64) + self.vert_offsets[k]
                       for k, m in enumerate(meshes)]).astype(np.int32)
        ed = np.hstack([d.element_dofs.astype(np.int64) + self.dof_offsets[k]
                        for k, d in enumerate(dofs)]).astype(np.int32)
        union = type(meshes[0]).__new__(type(meshes[0]))
        union.doflocs = np.ascontiguousarray(p)
        union.t = np.ascontiguousarray(t)
        union._entities = {}
        self.meshes = meshes
        super().__init__(union, elem, dofs=_UnionDofs(ed, int(self.dof_offsets[-1])),
                         device=device)

    @property
    def nmeshes(self):
        return len(self.meshes)

    def split(self, K):
        """Per-mesh scipy CSR blocks of a block-diagonal batch matrix."""
        K = K.tocsr()
        out = []
        for k in range(self.nmeshes):
            a, b = int(self.dof_offsets[k]), int(self.dof_offsets[k + 1])
            p0, p1 = K.indptr[a], K.indptr[b]
            blk = sp.csr_matrix((K.data[p0:p1].copy(), K.indices[p0:p1] - a,
                                 K.indptr[a:b + 1] - p0), shape=(b - a, b - a))
            out.append(blk)
        return out

    def split_elements(self, x):
        return [x[self.elem_offsets[k]:self.elem_offsets[k + 1]] for k in range(self.nmeshes)]


ROWS_PER_UNIT = 1024


class GraphedAssembly:
    """Forward assembly (+ optional adjoint) of one form over a basis,
    captured in a CUDA graph.  Static device buffers: ``coef[name]``
    (per-element fields), ``w``, ``u`` (adjoint vectors); outputs ``values``
    (CSR values in the cached pattern), ``dcoef[name]`` (d(w^T K u) / d
    coefficient field) and, with ``with_dX``, ``dX`` (/ d node coordinates).
    ``persistent`` (default: wherever supported) runs forward + coefficient
    adjoint as one persistent work-queue launch; False runs the separate
    kernels."""

    def __init__(self, form, basis, coefs, w=None, u=None, adjoint=True, with_dX=False,
                 persistent=None):
        self.form, self.basis = form, basis
        dev = basis.device
        self.coef = {k: torch.as_tensor(v, dtype=torch.float64, device=dev).clone()
                     for k, v in coefs.items()}
        # first assembly builds (and caches) the pattern eagerly
        K = form.assemble_torch(basis, **self.coef)
        self.key, self.entry = next((key, e) for key, e in basis._patterns.items()
                                    if key[0] == "bilinear")
        self.indptr, self.indices = K.crow_indices(), K.col_indices()
        self.values = torch.empty(self.entry.nnz, dtype=torch.float64, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        coeffs, ch, self.c_form = form._setup(basis, None, self.coef)
        self._coeffs = coeffs
        self.adjoint = adjoint
        if adjoint:
            from .autodiff import _channel_fields, _vertex_incidence
            chf = _channel_fields(ch)
            self.w = torch.as_tensor(w, dtype=torch.float64, device=dev).clone()
            self.u = torch.as_tensor(u, dtype=torch.float64, device=dev).clone()
            ne = basis.nelems
            self.dcd = torch.zeros(ne, dtype=torch.float64, device=dev) if "diff" in chf else None
            self.dcm = torch.zeros(ne, dtype=torch.float64, device=dev) if "mass" in chf else None
            self.dcoef = {}
            if "diff" in chf:
                self.dcoef[chf["diff"]] = self.dcd
            if "mass" in chf:
                self.dcoef.setdefault(chf["mass"], self.dcm)
            self.with_dX = with_dX
            if with_dX:
                self.dX = torch.empty_like(basis.p_dev)
                self.scratch = torch.empty(ne * basis.mesh.t.shape[0] * basis.mesh.p.shape[0],
                                           dtype=torch.float64, device=dev)
                self.vinc = _vertex_incidence(basis)
            else:
                self.dX = self.scratch = self.vinc = None
        else:
            self.with_dX = False
        supported = (not basis.elem.vector and basis.elem.family in
                     ("TriP1", "TriP2", "TetP1", "TetP2"))
        if persistent is None:
            persistent = supported and not self.with_dX
        if persistent and (not supported or self.with_dX):
            raise NotImplementedError("the persistent batched launch takes scalar simplex "
                                      "bases and the coefficient adjoint only")
        self.plan = None
        if persistent:
            self._build_plan()
        self.graph = None

    def _build_plan(self):
        b = self.basis
        if isinstance(b, BatchedBasis):
            cells = np.ascontiguousarray(b.elem_offsets, dtype=np.int64)
            rows = np.ascontiguousarray(b.dof_offsets, dtype=np.int64)
        else:
            cells = np.array([0, b.nelems], dtype=np.int64)
            rows = np.array([0, b.N], dtype=np.int64)
        h = ctypes.c_void_p()
        N.check(N.lib().fem_batch_plan_build(cells.ctypes.data, rows.ctypes.data, len(cells) - 1,
                                             ROWS_PER_UNIT, ctypes.byref(h)))
        self.plan = _Plan(h.value)
        nu, nc = ctypes.c_int64(), ctypes.c_int64()
        N.check(N.lib().fem_batch_plan_info(self.plan.handle, ctypes.byref(nu), ctypes.byref(nc)))
        self.counters = torch.zeros(nc.value, dtype=torch.int32, device=b.device)

    @property
    def nunits(self):
        """Work units of the queue the persistent launch runs (the one-pass
        queue of scalar P2 bases once it has run), or None without a plan."""
        if self.plan is None:
            return None
        nu, nc = ctypes.c_int64(), ctypes.c_int64()
        N.check(N.lib().fem_batch_plan_info(self.plan.handle, ctypes.byref(nu), ctypes.byref(nc)))
        return nu.value

    def _launch(self):
        lib = N.lib()
        b = self.basis
        s = N.stream_ptr()
        self.entry.ensure_caches(b, self.key, s)
        if self.plan is not None:
            adj = self.adjoint
            N.check(lib.fem_batched_assemble_vjp(
                N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(self.c_form),
                self.entry.pat.handle, self.plan.handle, N.ptr(self.entry.staging),
                N.ptr(self.values), N.ptr(self.w) if adj else None,
                N.ptr(self.u) if adj else None, N.ptr(self.dcd) if adj else None,
                N.ptr(self.dcm) if adj else None, N.ptr(self.counters), N.ptr(self.status), s))
            return
        N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(self.c_form),
                                 self.entry.pat.handle, N.ptr(self.entry.staging),
                                 N.ptr(self.values), N.ptr(self.status), s))
        if self.adjoint:
            N.check(lib.fem_bilinear_vjp(N.byref(b.c_mesh), N.byref(b.c_basis),
                                         N.byref(self.c_form),
                                         self.vinc.handle if self.vinc else None, N.ptr(self.w),
                                         N.ptr(self.u), N.ptr(self.dcd), N.ptr(self.dcm),
                                         N.ptr(self.dX), N.ptr(self.scratch), s))

    def launches_per_step(self):
        """Kernel launches one step issues (the persistent path: one kernel
        after a counter reset)."""
        if self.plan is not None:
            return 1
        fwd = 2
        adj = (1 + (1 if self.with_dX else 0)) if self.adjoint else 0
        return fwd + adj

    def run_eager(self):
        self._launch()

    def capture(self):
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(2):
                self._launch()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._launch()
        torch.cuda.synchronize()
        return self

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def check(self):
        st = int(self.status.item())
        if st & (1 << N.FEM_ERR_TIMEOUT):
            raise N.FemError("a wait of the persistent batched launch ran out: its results are "
                             "not valid")
        if st:
            raise N.FemError("batched assembly status %d" % st)

    def csr(self):
        return sp.csr_matrix((self.values.cpu().numpy(), self.indices.cpu().numpy(),
                              self.indptr.cpu().numpy()), shape=(self.basis.N, self.basis.N))
