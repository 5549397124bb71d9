// The generic-form kernel body (program_kernel in fem_faithful.cu, and the
// kernels compiled at run time from traced programs in fem_jit.cu).  Needs
// fem_faithful_core.cuh first.
#pragma once

namespace fem_faithful {

// ------------------------------------------------------------ generic forms
// One block takes EPB cells (or facets).  Stage 1: the geometry of every
// (cell, point) pair into shared memory.  Stage 2: form * dx for every
// (cell, entry, point) triple into shared memory.  Stage 3: numpy's
// pairwise sum over the points of each entry.  MODE 0: bilinear (L =
// nbfun^2 entries, row = test function), 1: linear (L = nbfun), 2:
// functional (L = 1).  FACET: the cells are a FacetBasis's facets.
constexpr int kGeo = 20;  // inv 9, det, qx 7, reference point 3
constexpr int kCell = 22; // affine cell map: inv 9, det, A 9, x0 3

template <int D, bool FACET>
__device__ bool geometry_at(const FemMesh& m, const FemBasis& b, const FemFacets& fc,
                            const Rule& rule, ProgFlags f, int64_t e, int q, double Y[3],
                            PointGeo& g, const double* cell = nullptr) {
  if (FACET) {
    if (fc.geo) {   // Hex1 facets: precomputed by fem_facet_geometry
      const double* G = fc.geo + ((size_t)e * rule.nq + q) * kGeo;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) g.inv[i][j] = G[i * 3 + j];
      g.det = G[9];
      for (int i = 0; i < 7; ++i) g.qx[i] = G[10 + i];
      for (int i = 0; i < 3; ++i) Y[i] = G[17 + i];
      return true;
    }
    double Xf[2] = {rule.X[q], D == 3 ? rule.X[rule.nq + q] : 0.0};
    return facet_point<D>(m, fc, e, Xf, Y, g);
  }
  const bool hex = b.family == FEM_HEX_1;
  CellGeo c;
  if (cell && !hex) {   // the cell's affine map, computed once per cell
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        c.inv[i][j] = cell[i * 3 + j];
        c.A[i][j] = cell[10 + i * 3 + j];
      }
    c.det = cell[9];
    for (int i = 0; i < 3; ++i) c.x0[i] = cell[19 + i];
  } else {
    cell_geometry<D>(m, e, hex, c);
  }
  Y[0] = rule.X[q];
  Y[1] = rule.X[rule.nq + q];
  Y[2] = D == 3 ? rule.X[2 * rule.nq + q] : 0.0;
  point_geometry<D>(m, e, hex, c, f, Y[0], Y[1], Y[2], g);
  return true;
}

// Shared-memory layout of one block of program_kernel.
struct GenericLayout {
  int epb, L, nq, nb, nquant;
  bool cells, quants;  // per-cell affine maps staged; basis quantities staged
  int npoint;          // compiled programs: values hoisted per point (0: none)
  bool mixed;          // a trial basis of its own (nbu functions, nquantu quantities)
  int nbu, nquantu;
  bool entry_loop;     // one thread per entry looping over the points (no value stage)
  bool uv;             // compiled bilinear programs: trial-only / test-only values staged
  int nuval, nvval;    // ... per (point, trial function) / (point, test function)
  __host__ __device__ size_t geo() const { return 0; }
  __host__ __device__ size_t val() const { return (size_t)epb * nq * kGeo; }
  __host__ __device__ size_t cell() const {
    return val() + (entry_loop ? 0 : (size_t)epb * L * nq);
  }
  __host__ __device__ size_t quant() const { return cell() + (cells ? (size_t)epb * kCell : 0); }
  __host__ __device__ size_t quantu() const {
    return quant() + (quants ? (size_t)epb * nq * nb * nquant : 0);
  }
  __host__ __device__ size_t point() const {
    return quantu() + (mixed ? (size_t)epb * nq * nbu * nquantu : 0);
  }
  __host__ __device__ size_t uval() const { return point() + (size_t)epb * nq * npoint; }
  __host__ __device__ size_t vval() const {
    return uval() + (uv ? (size_t)epb * nq * (mixed ? nbu : nb) * nuval : 0);
  }
  __host__ __device__ size_t dx() const {
    return vval() + (uv ? (size_t)epb * nq * nb * nvval : 0);
  }
  __host__ __device__ size_t total() const { return dx() + (size_t)epb * nq; }
};

// b: the test basis (and trial basis unless s.mixed); bu: the trial basis.
template <int D, int MODE, bool FACET, bool VEC, bool VECU>
__device__ __forceinline__ void program_body(const FemMesh& m, const FemBasis& b,
                                             const FemBasis& bu,
                                             const FemFacets& fc, const FemProgram& prog,
                                             const Rule& rule, const GenericLayout& s,
                                             int64_t ncells, double* __restrict__ out,
                                             int32_t* __restrict__ status) {
  extern __shared__ double gsm[];
  double* geo = gsm + s.geo();
  double* val = gsm + s.val();
  double* cgeo = gsm + s.cell();
  double* Q = gsm + s.quant();
  double* dxs = gsm + s.dx();   // |det| W_q per (cell, point): dx, the same for every entry
  const bool hex = b.family == FEM_HEX_1;
  constexpr bool vec = VEC;
  constexpr int NQ = VEC ? D + D * D : 1 + D;   // quantities per basis function
  constexpr int NQU = VECU ? D + D * D : 1 + D; // ... of the trial basis
  const ProgFlags f = prog_flags(prog);
  const int64_t e0 = (int64_t)blockIdx.x * s.epb;
  const int nb = b.nbfun;
  const int nbu = s.mixed ? bu.nbfun : nb;      // trial functions
  double* Qu = s.mixed ? gsm + s.quantu() : Q;
  // stage 0: affine cell maps (9 divisions each), once per cell
  if (s.cells) {
    for (int el = threadIdx.x; el < s.epb; el += blockDim.x) {
      const int64_t e = e0 + el;
      if (e >= ncells) continue;
      CellGeo c;
      cell_geometry<D>(m, e, false, c);
      double* C = cgeo + (size_t)el * kCell;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          C[i * 3 + j] = c.inv[i][j];
          C[10 + i * 3 + j] = c.A[i][j];
        }
      C[9] = c.det;
      for (int i = 0; i < 3; ++i) C[19 + i] = c.x0[i];
    }
    __syncthreads();
  }
  // stage 1: point geometry
  for (int k = threadIdx.x; k < s.epb * s.nq; k += blockDim.x) {
    const int el = k / s.nq, q = k - el * s.nq;
    const int64_t e = e0 + el;
    if (e >= ncells) continue;
    PointGeo g;
    double Y[3];
    if (!geometry_at<D, FACET>(m, b, fc, rule, f, e, q, Y, g,
                               s.cells ? cgeo + (size_t)el * kCell : nullptr)) {
      atomicOr(status, 1 << FEM_ERR_ARGUMENT);
      g = PointGeo{};
      Y[0] = Y[1] = Y[2] = 0.0;
    }
    if (!FACET && hex && g.det == 0.0) atomicOr(status, 1 << FEM_ERR_ZERO_JACOBIAN);
    double* G = geo + (size_t)k * kGeo;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) G[i * 3 + j] = g.inv[i][j];
    G[9] = g.det;
    for (int i = 0; i < 7; ++i) G[10 + i] = g.qx[i];
    for (int i = 0; i < 3; ++i) G[17 + i] = Y[i];
    dxs[k] = fabs(g.det) * rule.W[q];
  }
  __syncthreads();
  // stage 1b: every basis function's quantities at every point, once.  P1
  // on affine cells: the full quantities at each cell's first point, then
  // at the other points the values with the same derivative part
  if (s.quants) {
    const bool p1 = !FACET && s.cells && point_free_gradients(b.family);
    for (int k = threadIdx.x; k < s.epb * s.nq * nb; k += blockDim.x) {
      const int p = k / nb, fn = k - p * nb;    // p = el * nq + q
      if (e0 + p / s.nq >= ncells) continue;
      if (p1 && p % s.nq != 0) continue;
      const double* G = geo + (size_t)p * kGeo;
      double inv[3][3];
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) inv[a][c] = G[a * 3 + c];
      double qq[D + D * D];
      quantities<D>(b.family, vec, fn, G[17], G[18], G[19], inv, qq);
#pragma unroll
      for (int a = 0; a < NQ; ++a) Q[(size_t)k * NQ + a] = qq[a];
    }
    if (p1) {
      __syncthreads();
      for (int k = threadIdx.x; k < s.epb * s.nq * nb; k += blockDim.x) {
        const int p = k / nb, fn = k - p * nb;
        if (e0 + p / s.nq >= ncells || p % s.nq == 0) continue;
        const double* G = geo + (size_t)p * kGeo;
        const size_t k0 = ((size_t)(p - p % s.nq) * nb + fn) * NQ;   // first point, same fn
        double qq[D + D * D];
        quantities_values<D>(b.family, vec, fn, G[17], G[18], G[19], Q + k0, qq);
#pragma unroll
        for (int a = 0; a < NQ; ++a) Q[(size_t)k * NQ + a] = qq[a];
      }
    }
    if (s.mixed) {
      for (int k = threadIdx.x; k < s.epb * s.nq * nbu; k += blockDim.x) {
        const int p = k / nbu, fn = k - p * nbu;
        if (e0 + p / s.nq >= ncells) continue;
        const double* G = geo + (size_t)p * kGeo;
        double inv[3][3];
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c) inv[a][c] = G[a * 3 + c];
        double qq[D + D * D];
        quantities<D>(bu.family, VECU, fn, G[17], G[18], G[19], inv, qq);
#pragma unroll
        for (int a = 0; a < NQU; ++a) Qu[(size_t)k * NQU + a] = qq[a];
      }
    }
    __syncthreads();
  }
#ifdef FEM_JIT_HOIST
  // stage 1c (compiled programs): the instructions that depend on neither
  // the trial nor the test function, once per point
  double* P = gsm + s.point();
  for (int k = threadIdx.x; k < s.epb * s.nq; k += blockDim.x) {
    const int el = k / s.nq, q = k - el * s.nq;
    const int64_t e = e0 + el;
    if (e >= ncells) continue;
    double cq[kMaxCoef];
#pragma unroll
    for (int c = 0; c < kMaxCoef; ++c)
      cq[c] = (c < prog.ncoef && prog.coef[c])
                  ? prog.coef[c][prog.coef_stride[c] ? e * prog.coef_stride[c] + q : e]
                  : 0.0;
    jit_point(cq, geo + (size_t)k * kGeo + 10, P + (size_t)k * s.npoint);
  }
  __syncthreads();
#endif
#ifdef FEM_JIT_HOIST_UV
  // stage 1d (compiled bilinear programs): the instructions that depend on the
  // trial function only, once per point and trial function, and those on the
  // test function only, once per point and test function
  double* UU = gsm + s.uval();
  double* VV = gsm + s.vval();
  if (s.uv) {
    for (int k = threadIdx.x; k < s.epb * s.nq * nbu; k += blockDim.x) {
      const int p = k / nbu;                    // p = el * nq + q
      if (e0 + p / s.nq >= ncells) continue;
      double qu[D + D * D];
#pragma unroll
      for (int a = 0; a < NQU; ++a) qu[a] = Qu[(size_t)k * NQU + a];
      jit_u(qu, P + (size_t)p * s.npoint, UU + (size_t)k * s.nuval);
    }
    for (int k = threadIdx.x; k < s.epb * s.nq * nb; k += blockDim.x) {
      const int p = k / nb;
      if (e0 + p / s.nq >= ncells) continue;
      double qv[D + D * D];
#pragma unroll
      for (int a = 0; a < NQ; ++a) qv[a] = Q[(size_t)k * NQ + a];
      jit_v(qv, P + (size_t)p * s.npoint, VV + (size_t)k * s.nvval);
    }
    __syncthreads();
  }
#endif
  if (s.entry_loop) {
    // large local matrices: a thread takes an entry, its points in turn
    double R[kMaxProgram];
    double vals[kMaxPoints];
    for (int k = threadIdx.x; k < s.epb * s.L; k += blockDim.x) {
      const int el = k / s.L, r = k - el * s.L;
      const int64_t e = e0 + el;
      if (e >= ncells) continue;
      const int i = MODE == 0 ? r / nbu : (MODE == 1 ? r : 0);
      const int j = MODE == 0 ? r - i * nbu : 0;
      for (int q = 0; q < s.nq; ++q) {
        const double* G = geo + ((size_t)el * s.nq + q) * kGeo;
        PointGeo g;
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c) g.inv[a][c] = G[a * 3 + c];
        g.det = G[9];
        for (int a = 0; a < 7; ++a) g.qx[a] = G[10 + a];
        double qu[D + D * D], qv[D + D * D];
        if (s.quants) {
          const double* Qp = Q + ((size_t)(el * s.nq + q) * nb) * NQ;
          const double* Qup = Qu + ((size_t)(el * s.nq + q) * nbu) * NQU;
#pragma unroll
          for (int a = 0; a < NQU; ++a) qu[a] = Qup[(size_t)j * NQU + a];
#pragma unroll
          for (int a = 0; a < NQ; ++a) qv[a] = Qp[(size_t)i * NQ + a];
        } else {
#pragma unroll
          for (int a = 0; a < NQU; ++a) qu[a] = 0.0;
#pragma unroll
          for (int a = 0; a < NQ; ++a) qv[a] = 0.0;
        }
#if defined(FEM_JIT_HOIST_UV)
        const double* Pp = P + ((size_t)el * s.nq + q) * s.npoint;
        double Ut[FEM_JIT_NUVAL], Vt[FEM_JIT_NVVAL];
        jit_u(qu, Pp, Ut);
        jit_v(qv, Pp, Vt);
        const double fq = jit_form_uv(Pp, Ut, Vt);
        vals[q] = fq * dxs[(size_t)el * s.nq + q];
        (void)R;
#elif defined(FEM_JIT_HOIST)
        const double fq = jit_form_hoisted(qu, qv, P + ((size_t)el * s.nq + q) * s.npoint);
        vals[q] = fq * dxs[(size_t)el * s.nq + q];
        (void)R;
#else
        vals[q] = point_value_q(prog, e, q, qu, qv, g, rule.W[q], R);
#endif
      }
      out[e0 * s.L + k] = np_pairwise_sum(vals, s.nq);
    }
    return;
  }
  // stage 2: form * dx
  double R[kMaxProgram];
  const int per = s.L * s.nq;
  for (int k = threadIdx.x; k < s.epb * per; k += blockDim.x) {
    const int el = k / per;
    const int rq = k - el * per;
    const int r = rq / s.nq, q = rq - r * s.nq;
    const int64_t e = e0 + el;
    if (e >= ncells) continue;
    const int i = MODE == 0 ? r / nbu : (MODE == 1 ? r : 0);
    const int j = MODE == 0 ? r - i * nbu : 0;
#if defined(FEM_JIT_HOIST_UV)
    if (s.uv) {
      const size_t p = (size_t)el * s.nq + q;
      const double fq = jit_form_uv(P + p * s.npoint, UU + (p * nbu + j) * s.nuval,
                                    VV + (p * nb + i) * s.nvval);
      val[k] = fq * dxs[p];
      continue;
    }
#endif
    const double* G = geo + ((size_t)el * s.nq + q) * kGeo;
    PointGeo g;
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) g.inv[a][c] = G[a * 3 + c];
    g.det = G[9];
    for (int a = 0; a < 7; ++a) g.qx[a] = G[10 + a];
    double qu[D + D * D], qv[D + D * D];
    if (s.quants) {
      const double* Qp = Q + ((size_t)(el * s.nq + q) * nb) * NQ;
      const double* Qup = Qu + ((size_t)(el * s.nq + q) * nbu) * NQU;
#pragma unroll
      for (int a = 0; a < NQU; ++a) qu[a] = Qup[(size_t)j * NQU + a];
#pragma unroll
      for (int a = 0; a < NQ; ++a) qv[a] = Qp[(size_t)i * NQ + a];
    } else {
#pragma unroll
      for (int a = 0; a < NQU; ++a) qu[a] = 0.0;
#pragma unroll
      for (int a = 0; a < NQ; ++a) qv[a] = 0.0;
    }
#if defined(FEM_JIT_HOIST_UV)
    {
      const double* Pp = P + ((size_t)el * s.nq + q) * s.npoint;
      double Ut[FEM_JIT_NUVAL], Vt[FEM_JIT_NVVAL];
      jit_u(qu, Pp, Ut);
      jit_v(qv, Pp, Vt);
      val[k] = jit_form_uv(Pp, Ut, Vt) * dxs[(size_t)el * s.nq + q];
      (void)R;
    }
#elif defined(FEM_JIT_HOIST)
    const double fq = jit_form_hoisted(qu, qv, P + ((size_t)el * s.nq + q) * s.npoint);
    val[k] = fq * dxs[(size_t)el * s.nq + q];
    (void)R;
#else
    val[k] = point_value_q(prog, e, q, qu, qv, g, rule.W[q], R);
#endif
  }
  __syncthreads();
  for (int k = threadIdx.x; k < s.epb * s.L; k += blockDim.x) {
    const int el = k / s.L;
    const int64_t e = e0 + el;
    if (e >= ncells) continue;
    out[e0 * s.L + k] = np_pairwise_sum(val + (size_t)k * s.nq, s.nq);
  }
}

}  // namespace fem_faithful
