// Fused local-matrix kernels: geometry + basis + form + quadrature in one
// FP64 pass per element, writing element matrices K_e[i][j] (i = test row,
// j = trial column) to an element-major staging array.
//
// Replaces, per element family, the chain
//   MappingAffine._init_Ab/_init_invA (skfem/mapping/mapping_affine.py:55-131)
//   MappingIsoparametric._J/detDF/invDF (skfem/mapping/mapping_isoparametric.py:112-226)
//   ElementH1.gbasis / ElementVector.gbasis (skfem/element/element_h1.py:10-24,
//                                            skfem/element/element_vector.py:36-48)
//   CellBasis dx = |detDF| * W (skfem/assembly/basis/cell_basis.py:104-105)
//   BilinearForm._kernel / LinearForm._kernel (bilinear_form.py:150-151, linear_form.py:48-49)
//
// Affine simplices use the tensor representation (exact reference
// integrals from fem_tables.cuh contracted with the barycentric-gradient
// Gram matrix of each cell), which integrates the same polynomials the
// reference's quadrature integrates exactly, in far fewer FP64 operations.
// The trilinear hexahedron takes a closed form on parallelepipeds (where
// the Jacobian is constant and the 4x4x4 rule is exact) and the full
// 64-point isoparametric quadrature otherwise.
//
// This file is compiled twice: the default build lets the compiler fuse
// multiply-adds (the values path), the FEM_EXACT build disables
// contraction (-fmad=false) so that products that cancel exactly in
// separately rounded arithmetic -- as numpy evaluates them -- come out as
// exact zeros; that build feeds the eliminate_zeros mask of the pattern.

#include <cuda.h>   // CUtensorMap (the TMA-staged local kernel)
#include <cstring>
#include <type_traits>

#include "fem_common.cuh"
#include "fem_tables.cuh"

#ifdef FEM_EXACT
#define FEM_NS fem_exact
#else
#define FEM_NS fem_fast
#endif

namespace FEM_NS {

using fem::coef_at;
using fem::hex_corner;

constexpr int kBlock = 128;

// Compile-time loop: f(std::integral_constant<int, I>) for I = 0 .. N-1, so
// that array indices derived from I are constants (registers, not memory).
template <int I, int N, typename F>
__device__ __forceinline__ void static_for_impl(F& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for_impl<I + 1, N>(f);
  }
}
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl<0, N>(f);
}

// --------------------------------------------------------------- geometry
// c[a] = det(A) * grad(lambda_a) for the barycentric coordinates of the
// cell, with A[i][j] = p_i(t_{j+1}) - p_i(t_0) (mapping_affine.py:64-70)
// and the cofactor expressions of mapping_affine.py:92-129.
template <int D>
struct Simplex {
  double c[D + 1][D];
  double det;
};

template <int D>
__device__ __forceinline__ void simplex_geometry(const FemMesh& m, int64_t e, Simplex<D>& s) {
  double x[D + 1][D];
#pragma unroll
  for (int a = 0; a <= D; ++a) {
    const int64_t v = m.t[a * m.nelems + e];
#pragma unroll
    for (int k = 0; k < D; ++k) x[a][k] = m.p[k * m.nverts + v];
  }
  double A[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) A[i][j] = x[j + 1][i] - x[0][i];
  if constexpr (D == 2) {
    s.c[1][0] = A[1][1];
    s.c[1][1] = -A[0][1];
    s.c[2][0] = -A[1][0];
    s.c[2][1] = A[0][0];
    s.det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  } else {
    s.c[1][0] = -A[1][2] * A[2][1] + A[1][1] * A[2][2];
    s.c[2][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    s.c[3][0] = -A[1][1] * A[2][0] + A[1][0] * A[2][1];
    s.c[1][1] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
    s.c[2][1] = -A[0][2] * A[2][0] + A[0][0] * A[2][2];
    s.c[3][1] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
    s.c[1][2] = -A[0][2] * A[1][1] + A[0][1] * A[1][2];
    s.c[2][2] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
    s.c[3][2] = -A[0][1] * A[1][0] + A[0][0] * A[1][1];
    // first row of A times first column of adj(A)
    s.det = A[0][0] * s.c[1][0] + A[0][1] * s.c[2][0] + A[0][2] * s.c[3][0];
  }
}

// c[0] = -(c[1] + ... + c[D]) (grad lambda_0 = -sum grad lambda_m)
template <int D>
__device__ __forceinline__ void simplex_c0(Simplex<D>& s) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    double acc = s.c[1][k];
#pragma unroll
    for (int a = 2; a <= D; ++a) acc = acc + s.c[a][k];
    s.c[0][k] = -acc;
  }
}

template <int D>
__device__ __forceinline__ double dotc(const double* a, const double* b) {
  double r = a[0] * b[0];
#pragma unroll
  for (int k = 1; k < D; ++k) r = r + a[k] * b[k];
  return r;
}

// ----------------------------------------------------------- smem epilogue
// The cells of a launch: positions [ebeg, eend) of the list `cells`, or the
// cells ebeg .. eend-1 themselves when cells is null.
__device__ __forceinline__ int64_t cell_at(const int32_t* __restrict__ cells, int64_t pos) {
  return cells ? (int64_t)__ldg(cells + pos) : pos;
}

// Each thread writes its element's matrix into a padded row of shared
// memory; the block then streams the rows out (each cell's row contiguous,
// consecutive cells contiguous without a cell list).  With a cell list the
// block's cell ids sit in shared memory (cid, one per thread, written by
// the thread that computed the cell).
template <int L, int BS = kBlock>
__device__ __forceinline__ void flush_rows(double* smem, double* __restrict__ out, int64_t e0,
                                           int64_t nelems, const int64_t* cid) {
  __syncthreads();
  const int64_t nb = ((nelems - e0) < (int64_t)BS ? (nelems - e0) : (int64_t)BS);
  const int64_t total = nb * L;
  if (!cid) {
    double* dst = out + e0 * L;
    for (int64_t g = threadIdx.x; g < total; g += blockDim.x) {
      const int el = (int)(g / L);
      const int k = (int)(g - (int64_t)el * L);
      dst[g] = smem[el * (L + 1) + k];
    }
  } else {
    for (int64_t g = threadIdx.x; g < total; g += blockDim.x) {
      const int el = (int)(g / L);
      const int k = (int)(g - (int64_t)el * L);
      out[cid[el] * L + k] = smem[el * (L + 1) + k];
    }
  }
  __syncthreads();
}

// Shared-memory bytes of a cell-list launch beyond the row buffer.
template <int BS>
constexpr size_t kCidBytes = (size_t)BS * sizeof(int64_t);

// ------------------------------------------------ simplex, scalar P1 / P2
template <int D, int ORDER>
struct SimplexTraits;
template <> struct SimplexTraits<2, 1> { static constexpr int NB = 3; static constexpr double FACT = 2.0; };
template <> struct SimplexTraits<2, 2> { static constexpr int NB = 6; static constexpr double FACT = 2.0; };
template <> struct SimplexTraits<3, 1> { static constexpr int NB = 4; static constexpr double FACT = 6.0; };
template <> struct SimplexTraits<3, 2> { static constexpr int NB = 10; static constexpr double FACT = 6.0; };

// Status bits of one element's coefficients: FEM_ERR_VARYING for a strided
// row that is not constant; with ref, FEM_ERR_STALE_PATTERN when the zero
// bits (bit k: channel k of diff, mass, lam, lap, tr is exactly 0) differ
// from the ones recorded at pattern build -- the zero structure may have
// changed.  No side effects: the kernels OR the bits into a register and
// publish them once (an atomic in the middle of the element would make
// every later load re-read memory the atomic may have written).
// ref is the element's recorded byte, or -1 without a record; the kernels
// load it before the element's geometry and call this after its values, so
// that the load's latency overlaps the arithmetic.
__device__ __forceinline__ int32_t coef_status(const FemBilinear& f, int64_t e, int ref) {
  int32_t st = fem::row_status(f.diff, e) | fem::row_status(f.mass, e) |
               fem::row_status(f.lam, e) | fem::row_status(f.lap, e) | fem::row_status(f.tr, e);
  if (ref < 0) return st;
  int bits = 0;
  bits |= fem::coef_zero(f.diff, e) ? 1 : 0;
  bits |= fem::coef_zero(f.mass, e) ? 2 : 0;
  bits |= fem::coef_zero(f.lam, e) ? 4 : 0;
  bits |= fem::coef_zero(f.lap, e) ? 8 : 0;
  bits |= fem::coef_zero(f.tr, e) ? 16 : 0;
  if (bits != ref) st |= 1 << FEM_ERR_STALE_PATTERN;
  return st;
}

__device__ __forceinline__ int ref_byte(const uint8_t* __restrict__ ref, int64_t e) {
  return ref ? (int)__ldg(ref + e) : -1;
}

// The coefficient-free geometry of a simplex: the Gram matrix of
// c_a = det(A) grad(lambda_a) (entries a <= b; row 0 from c_0 = -sum c_m),
// |det A| and its reciprocal.  The scalar kernels compute it per cell, or
// read it from a per-cell cache (simplex_geometry_cache_kernel): the Gram
// entries already scaled by 1/(d! |det|), and |det|.
template <int D>
constexpr int kGramCount = (D + 1) * (D + 2) / 2;
template <int D>
constexpr int kGeoCount = kGramCount<D> + 1;  // scaled Gram entries, |det|
template <int D>
constexpr double kInvFact = D == 2 ? 0.5 : 1.0 / 6.0;

template <int D>
__device__ __forceinline__ void simplex_gram(const FemMesh& m, int64_t e, double gram[D + 1][D + 1],
                                             double& adet, double& rinv) {
  Simplex<D> s;
  simplex_geometry<D>(m, e, s);
  adet = fem::abs_bits(s.det);
  rinv = 1.0 / adet;
#pragma unroll
  for (int a = 1; a <= D; ++a)
#pragma unroll
    for (int b = a; b <= D; ++b) gram[a][b] = dotc<D>(s.c[a], s.c[b]);
#pragma unroll
  for (int b = 1; b <= D; ++b) {
    double acc = (1 <= b ? gram[1][b] : gram[b][1]);
#pragma unroll
    for (int a = 2; a <= D; ++a) acc = acc + (a <= b ? gram[a][b] : gram[b][a]);
    gram[0][b] = -acc;
  }
  {
    double acc = gram[0][1];
#pragma unroll
    for (int b = 2; b <= D; ++b) acc = acc + gram[0][b];
    gram[0][0] = -acc;
  }
}

// geo[k * nelems + e]: the Gram entries (a <= b, row-major) times
// 1/(d! |det|) -- the stiffness per unit coefficient -- then |det|
template <int D>
__global__ void simplex_geometry_cache_kernel(FemMesh m, double* __restrict__ geo) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  double gram[D + 1][D + 1], adet, rinv;
  simplex_gram<D>(m, e, gram, adet, rinv);
  const double s = rinv * kInvFact<D>;
  int k = 0;
#pragma unroll
  for (int a = 0; a <= D; ++a)
#pragma unroll
    for (int b = a; b <= D; ++b) geo[(int64_t)(k++) * m.nelems + e] = gram[a][b] * s;
  geo[(int64_t)k * m.nelems + e] = adet;
}

// Bounded mbarrier wait (the TMA-staged kernel): false when it gave up.
__device__ __forceinline__ bool tile_wait(uint32_t bar, uint32_t parity, long long limit) {
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// CACHED: the geometry comes from geo (simplex_geometry_cache_kernel on the
// same coordinates) instead of the mesh -- coefficient changes then cost
// the ~14 FP64 operations per cell of the form alone.
// TMA (with CACHED, no cell list): each tile's geometry -- the (NG+1) x BS
// box of the SoA cache at column e0 -- comes into shared memory by one
// cp.async.bulk.tensor.2d copy (tensor map tmap) instead of per-thread
// loads; the wait is bounded (FEM_ERR_TIMEOUT in *status, after a second
// bounded wait for the copy in flight).
template <int D, int ORDER, int BS, bool CACHED, bool TMA = false>
__global__ void __launch_bounds__(BS) simplex_scalar_kernel(FemMesh m, FemBilinear f,
                                                                FemCoef kdiff,
                                                                double* __restrict__ out,
                                                                const uint8_t* __restrict__ ref_bits,
                                                                int32_t* __restrict__ status,
                                                                const int32_t* __restrict__ cells,
                                                                const double* __restrict__ geo,
                                                                int64_t ebeg, int64_t eend,
                                                                const __grid_constant__ CUtensorMap tmap) {
  constexpr int NB = SimplexTraits<D, ORDER>::NB;
  constexpr int L = NB * NB;
  constexpr int NGEO = kGeoCount<D>;
  constexpr double INV_FACT = 1.0 / SimplexTraits<D, ORDER>::FACT;
  extern __shared__ double smem[];
  int64_t* cid = cells ? reinterpret_cast<int64_t*>(smem + (size_t)BS * (L + 1)) : nullptr;
  // TMA: the geometry tile after the row buffer (128-byte aligned), then the mbarrier
  constexpr size_t kTileOff = (((size_t)BS * (L + 1) * sizeof(double)) + 127) / 128 * 128;
  double* sgeo = reinterpret_cast<double*>(reinterpret_cast<char*>(smem) + kTileOff);
  uint64_t* sbar = reinterpret_cast<uint64_t*>(sgeo + (size_t)NGEO * BS);
  uint32_t phase = 0;
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"((uint32_t)__cvta_generic_to_shared(sbar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
  }
  int32_t flags = 0;
  // grid-stride over element tiles of BS cells (persistent when the grid is
  // smaller than the number of tiles)
  for (int64_t e0 = ebeg + (int64_t)blockIdx.x * BS; e0 < eend; e0 += (int64_t)gridDim.x * BS) {
  if constexpr (TMA) {
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(sbar);
    if (threadIdx.x == 0) {
      // the previous tile's reads (generic proxy) before the copy's writes (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      unsigned long long state;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                   : "=l"(state) : "r"(bar), "r"((uint32_t)(NGEO * BS * sizeof(double))) : "memory");
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
          "[%0], [%1, {%2, %3}], [%4];"
          :: "r"((uint32_t)__cvta_generic_to_shared(sgeo)), "l"(&tmap), "r"((int32_t)e0), "r"(0),
             "r"(bar) : "memory");
      (void)state;
    }
    // every thread waits (bounded); the outcome is made block-uniform
    if (!__syncthreads_and(tile_wait(bar, phase, 1ll << 22) ? 1 : 0)) {
      // gave up: report, let this tile's copy land (bounded), stop
      if (threadIdx.x == 0) {
        fem::publish_status(status, 1 << FEM_ERR_TIMEOUT);
        tile_wait(bar, phase, 1ll << 22);
      }
      __syncthreads();
      return;
    }
    phase ^= 1u;
  }
  const int64_t pos = e0 + threadIdx.x;
  if (pos < eend) {
    const int64_t e = cell_at(cells, pos);
    if (cid) cid[threadIdx.x] = e;
    const int rb = ref_byte(ref_bits, e);
    // stiffness scale sd times the Gram entries: kd / (d! |det|) (kdiff is
    // f.diff with its scale multiplied by 1/d! on the host; the cache holds
    // the Gram entries already scaled by 1/(d! |det|)); mass scale km |det|
    // (the 1/d! of the mass goes into the table constants, folded at
    // compile time)
    double gram[D + 1][D + 1], adet, sd;
    if constexpr (CACHED && TMA) {
      int k = 0;
#pragma unroll
      for (int a = 0; a <= D; ++a)
#pragma unroll
        for (int b = a; b <= D; ++b) gram[a][b] = sgeo[(k++) * BS + threadIdx.x];
      adet = sgeo[k * BS + threadIdx.x];
      sd = coef_at(f.diff, e);
    } else if constexpr (CACHED) {
      int k = 0;
#pragma unroll
      for (int a = 0; a <= D; ++a)
#pragma unroll
        for (int b = a; b <= D; ++b) gram[a][b] = __ldg(geo + (int64_t)(k++) * m.nelems + e);
      adet = __ldg(geo + (int64_t)k * m.nelems + e);
      sd = coef_at(f.diff, e);
    } else {
      double rinv;
      simplex_gram<D>(m, e, gram, adet, rinv);
      sd = coef_at(kdiff, e) * rinv;
    }
    const double sm = coef_at(f.mass, e) * adet;
    double* row = smem + threadIdx.x * (L + 1);
    double kst[NB][NB];
#define G(a, b) ((a) <= (b) ? gram[a][b] : gram[b][a])
#define KS(i, j, v) { kst[i][j] = (v); }
#define KM(i, j, v) { constexpr double _m = (v) * INV_FACT; const double _v = __fma_rn(sd, kst[i][j], sm * _m); row[(i) * NB + (j)] = _v; row[(j) * NB + (i)] = _v; }
    if constexpr (D == 2 && ORDER == 1) { TRI1_STIFF(G, KS); TRI1_MASS(KM); }
    if constexpr (D == 2 && ORDER == 2) { TRI2_STIFF(G, KS); TRI2_MASS(KM); }
    if constexpr (D == 3 && ORDER == 1) { TET1_STIFF(G, KS); TET1_MASS(KM); }
    if constexpr (D == 3 && ORDER == 2) { TET2_STIFF(G, KS); TET2_MASS(KM); }
#undef G
#undef KS
#undef KM
    if (status) flags |= coef_status(f, e, rb);
  }
  flush_rows<L, BS>(smem, out, e0, eend, cid);
  }
  fem::publish_status(status, flags);
}

// -------------------------------------------- simplex, vector P2 (and P1)
// K[(i a)(j b)] = sum_{p,q} BB[i][j][p][q] * E_pq[a][b]
// E_pq[a][b] = s0 (lam c_p[a] c_q[b] + tr c_p[b] c_q[a] + lap delta_ab c_p.c_q),
// s0 = 1/(d! |det|), E_qp = E_pq^T; plus mass delta_ab sm MM[i][j].
// The element's 3 (or 2) rows of one scalar node are produced at a time
// and streamed out through shared memory.
template <int D, int ORDER, bool UPPER>
__global__ void __launch_bounds__(64) simplex_vector_kernel(FemMesh m, FemBilinear f,
                                                            double* __restrict__ out,
                                                            const uint8_t* __restrict__ ref_bits,
                                                            int32_t* __restrict__ status,
                                                            const int32_t* __restrict__ cells,
                                                            int64_t ebeg, int64_t eend) {
  constexpr int BS = 64;
  constexpr int NS = SimplexTraits<D, ORDER>::NB;  // scalar functions
  constexpr int NB = NS * D;                        // vector functions
  constexpr int NV = D + 1;
  constexpr int RB = D * NB;                        // values per node row block
  constexpr double FACT = SimplexTraits<D, ORDER>::FACT;
  extern __shared__ double smem[];
  double* rows = smem;                               // [BS][RB+1]
  int64_t* cid = cells ? reinterpret_cast<int64_t*>(smem + (size_t)BS * (RB + 1)) : nullptr;
  const int64_t e0 = ebeg + (int64_t)blockIdx.x * BS;
  const int tid = threadIdx.x;
  const bool live = e0 + tid < eend;
  const int64_t e = live ? cell_at(cells, e0 + tid) : 0;
  if (cid) cid[tid] = e;
  double sm = 0.0;
  // E[p][q][a][b] for p <= q, kept in registers: every index below is a
  // compile-time constant once the block loops are unrolled.
  double E[NV][NV][D][D];
  int32_t flags = 0;
  if (live) {
    const int rb = ref_byte(ref_bits, e);
    Simplex<D> s;
    simplex_geometry<D>(m, e, s);
    simplex_c0<D>(s);
    const double adet = fem::abs_bits(s.det);
    const double s0 = 1.0 / (FACT * adet);
    const double lam = coef_at(f.lam, e) * s0;
    const double lap = coef_at(f.lap, e) * s0;
    const double tr = coef_at(f.tr, e) * s0;
    sm = coef_at(f.mass, e) * (adet / FACT);
#pragma unroll
    for (int p = 0; p < NV; ++p)
#pragma unroll
      for (int q = p; q < NV; ++q) {
        const double g = lap * dotc<D>(s.c[p], s.c[q]);
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
          for (int b = 0; b < D; ++b) {
            double v = lam * (s.c[p][a] * s.c[q][b]) + tr * (s.c[p][b] * s.c[q][a]);
            if (a == b) v = v + g;
            E[p][q][a][b] = v;
          }
      }
    if (status) flags = coef_status(f, e, rb);
  }
  static_for<NS>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    if (live) {
      double* row = rows + tid * (RB + 1);
      static_for<NS>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (!UPPER || j >= i) {
        double blk[D][D];
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
          for (int b = 0; b < D; ++b) blk[a][b] = 0.0;
#define T(p, q, c)                                                                   \
  {                                                                                  \
    _Pragma("unroll") for (int a = 0; a < D; ++a) _Pragma("unroll") for (int b = 0; b < D; ++b) { \
      const double ev = (p) <= (q) ? E[(p)][(q)][a][b] : E[(q)][(p)][b][a];          \
      blk[a][b] = blk[a][b] + (c) * ev;                                              \
    }                                                                                \
  }
        if constexpr (D == 3 && ORDER == 2) {
          if constexpr (i == 0) { TET2BB_ROW0(j, T); }
          if constexpr (i == 1) { TET2BB_ROW1(j, T); }
          if constexpr (i == 2) { TET2BB_ROW2(j, T); }
          if constexpr (i == 3) { TET2BB_ROW3(j, T); }
          if constexpr (i == 4) { TET2BB_ROW4(j, T); }
          if constexpr (i == 5) { TET2BB_ROW5(j, T); }
          if constexpr (i == 6) { TET2BB_ROW6(j, T); }
          if constexpr (i == 7) { TET2BB_ROW7(j, T); }
          if constexpr (i == 8) { TET2BB_ROW8(j, T); }
          if constexpr (i == 9) { TET2BB_ROW9(j, T); }
        } else if constexpr (D == 2 && ORDER == 2) {
          if constexpr (i == 0) { TRI2BB_ROW0(j, T); }
          if constexpr (i == 1) { TRI2BB_ROW1(j, T); }
          if constexpr (i == 2) { TRI2BB_ROW2(j, T); }
          if constexpr (i == 3) { TRI2BB_ROW3(j, T); }
          if constexpr (i == 4) { TRI2BB_ROW4(j, T); }
          if constexpr (i == 5) { TRI2BB_ROW5(j, T); }
        } else {
          // P1: grad phi_i = grad lambda_i, BB[i][j][p][q] = delta_ip delta_jq
          T(i, j, 1.0);
        }
#undef T
        // mass: delta_ab sm MM[i][j] (elasticity has none: uniform branch)
        double mij = 0.0;
        if (!fem::zero_bits(sm)) {
          if constexpr (D == 3 && ORDER == 2) mij = c_tet2_mm[i][j];
          else if constexpr (D == 2 && ORDER == 2) mij = c_tri2_mm[i][j];
          else if constexpr (D == 3) mij = c_tet1_mm[i][j];
          else mij = c_tri1_mm[i][j];
        }
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
          for (int b = 0; b < D; ++b) {
            double v = blk[a][b];
            if (a == b) v = v + sm * mij;
            row[a * NB + j * D + b] = v;
          }
        }
      });
    }
    // stream rows (i*D .. i*D+D-1) of every element of the block (UPPER:
    // their columns from i*D on, the blocks on and above the diagonal)
    __syncthreads();
    const int64_t nb = ((eend - e0) < (int64_t)BS ? (eend - e0) : (int64_t)BS);
    constexpr int W = UPPER ? NB - i * D : NB;  // columns streamed per row
    constexpr int C0 = NB - W;                  // first column streamed
    for (int64_t g = threadIdx.x; g < nb * (D * W); g += blockDim.x) {
      const int el = (int)(g / (D * W));
      const int kk = (int)(g - (int64_t)el * (D * W));
      const int a = kk / W;
      const int k = a * NB + C0 + (kk - a * W);
      out[(cid ? cid[el] : e0 + el) * (int64_t)(NB * NB) + (int64_t)i * RB + k] =
          rows[el * (RB + 1) + k];
    }
    __syncthreads();
  });
  fem::publish_status(status, flags);
}

// Per-cell pair blocks of the vector channel forms, the inputs of the
// one-pass vector sum (fem_vecsum.cu): for the vertex pairs p <= q in
// row-major upper order k, out[e * R + k * D * D + a * D + b] = E_pq[a][b]
// = lam c_p[a] c_q[b] + tr c_p[b] c_q[a] + lap (c_p . c_q) delta_ab (the
// coefficients times 1/(d! |det|)), evaluated as fma(lam c_p[a], c_q[b],
// (tr c_p[b]) c_q[a]) -- 2 FP64 operations per entry, 1 on the symmetric
// blocks p = q -- and out[e * R + NP * D * D] the mass scale m_e |det| / d!.
// R = NP * D * D + 1, NP = (D + 1)(D + 2) / 2.
// Cells: positions [ebeg, eend) of the list `cells` (null: the cells
// themselves), each written at its own cell's row.
template <int D, int BS>
__global__ void __launch_bounds__(BS) vector_pair_blocks_kernel(FemMesh m, FemBilinear f,
                                                                double* __restrict__ out,
                                                                const int32_t* __restrict__ cells,
                                                                int64_t ebeg, int64_t eend,
                                                                const uint8_t* __restrict__ ref_bits,
                                                                int32_t* __restrict__ status) {
  constexpr int NV = D + 1;
  constexpr int NP = NV * (NV + 1) / 2;
  constexpr int R = NP * D * D + 1;
  constexpr double FACT = D == 3 ? 6.0 : 2.0;
  extern __shared__ double smem[];
  int64_t* cid = cells ? reinterpret_cast<int64_t*>(smem + (size_t)BS * (R + 1)) : nullptr;
  const int64_t e0 = ebeg + (int64_t)blockIdx.x * BS;
  const int64_t pos = e0 + threadIdx.x;
  int32_t flags = 0;
  if (pos < eend) {
    const int64_t e = cell_at(cells, pos);
    if (cid) cid[threadIdx.x] = e;
    const int rb = ref_byte(ref_bits, e);
    Simplex<D> s;
    simplex_geometry<D>(m, e, s);
    simplex_c0<D>(s);
    const double adet = fem::abs_bits(s.det);
    const double s0 = 1.0 / (FACT * adet);
    const double lam = coef_at(f.lam, e) * s0;
    const double lap = coef_at(f.lap, e) * s0;
    const double tr = coef_at(f.tr, e) * s0;
    double* row = smem + threadIdx.x * (R + 1);
    double L[NV][D], T[NV][D];
#pragma unroll
    for (int p = 0; p < NV; ++p)
#pragma unroll
      for (int a = 0; a < D; ++a) {
        L[p][a] = lam * s.c[p][a];
        T[p][a] = tr * s.c[p][a];
      }
    const double lt = lam + tr;
    int k = 0;
#pragma unroll
    for (int p = 0; p < NV; ++p)
#pragma unroll
      for (int q = p; q < NV; ++q) {
        const double g = lap * dotc<D>(s.c[p], s.c[q]);
        if (p == q) {
          // symmetric: (lam + tr) c_p[a] c_p[b] + g delta_ab
#pragma unroll
          for (int a = 0; a < D; ++a) {
            const double la = lt * s.c[p][a];
#pragma unroll
            for (int b = a; b < D; ++b) {
              double v = la * s.c[p][b];
              if (a == b) v = v + g;
              row[k * D * D + a * D + b] = v;
              row[k * D * D + b * D + a] = v;
            }
          }
        } else {
#pragma unroll
          for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b < D; ++b) {
              double v = __fma_rn(L[p][a], s.c[q][b], T[p][b] * s.c[q][a]);
              if (a == b) v = v + g;
              row[k * D * D + a * D + b] = v;
            }
        }
        ++k;
      }
    row[NP * D * D] = coef_at(f.mass, e) * (adet / FACT);
    if (status) flags = coef_status(f, e, rb);
  }
  flush_rows<R, BS>(smem, out, e0, eend, cid);
  fem::publish_status(status, flags);
}

// ------------------------------------- simplex, scalar P2 (one-pass sum)
// The scalar forms k_e dot(grad u, grad v) + m_e u v on TriP2 / TetP2 as the
// one-pass node-block sum reads them: per cell the NP numbers
//   E_pq = k_e |det| / d! grad(lambda_p) . grad(lambda_q)   (p <= q)
// and m_e |det| / d!.  The Gram entries come from the geometry cache when
// geo is given, else from the coordinates with the cache kernel's rounding
// (the scaled Gram entries, then the coefficient), so both give the same bits.
template <int D, int BS>
__global__ void __launch_bounds__(BS) scalar_pair_kernel(FemMesh m, FemBilinear f,
                                                         const double* __restrict__ geo,
                                                         double* __restrict__ out,
                                                         const int32_t* __restrict__ cells,
                                                         int64_t ebeg, int64_t eend,
                                                         const uint8_t* __restrict__ ref_bits,
                                                         int32_t* __restrict__ status) {
  constexpr int NP = kGramCount<D>;
  constexpr int R = NP + 1;
  extern __shared__ double smem[];
  int64_t* cid = cells ? reinterpret_cast<int64_t*>(smem + (size_t)BS * (R + 1)) : nullptr;
  const int64_t e0 = ebeg + (int64_t)blockIdx.x * BS;
  const int64_t pos = e0 + threadIdx.x;
  int32_t flags = 0;
  if (pos < eend) {
    const int64_t e = cell_at(cells, pos);
    if (cid) cid[threadIdx.x] = e;
    const int rb = ref_byte(ref_bits, e);
    double* row = smem + threadIdx.x * (R + 1);
    const double sd = coef_at(f.diff, e);
    double adet;
    if (geo) {
#pragma unroll
      for (int k = 0; k < NP; ++k) row[k] = sd * __ldg(geo + (int64_t)k * m.nelems + e);
      adet = __ldg(geo + (int64_t)NP * m.nelems + e);
    } else {
      double gram[D + 1][D + 1], rinv;
      simplex_gram<D>(m, e, gram, adet, rinv);
      const double s = rinv * kInvFact<D>;
      int k = 0;
#pragma unroll
      for (int a = 0; a <= D; ++a)
#pragma unroll
        for (int b = a; b <= D; ++b) row[k++] = sd * (gram[a][b] * s);
    }
    row[NP] = coef_at(f.mass, e) * (adet * kInvFact<D>);
    if (status) flags = coef_status(f, e, rb);
  }
  flush_rows<R, BS>(smem, out, e0, eend, cid);
  fem::publish_status(status, flags);
}

// ----------------------------------------------------------- hexahedron Q1
// Reference node k sits at corner c_hex_corner[k] (refdom.py:173-180);
// phi_k = prod_ax f(c, x_ax) with f(1,t) = t, f(0,t) = 1 - t.
struct Hex {
  double x[8][3];
};

__device__ __forceinline__ void hex_load(const FemMesh& m, int64_t e, Hex& h) {
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int64_t v = m.t[n * m.nelems + e];
#pragma unroll
    for (int k = 0; k < 3; ++k) h.x[n][k] = m.p[k * m.nverts + v];
  }
}

// Parallelepiped test: every node equals x7 + J c_n with J's columns the
// edges from node 7 (corner 000) to nodes 4 (100), 5 (010), 6 (001).
__device__ __forceinline__ bool hex_affine(const Hex& h, double J[3][3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    J[k][0] = h.x[4][k] - h.x[7][k];
    J[k][1] = h.x[5][k] - h.x[7][k];
    J[k][2] = h.x[6][k] - h.x[7][k];
  }
  bool ok = true;
#pragma unroll
  for (int n = 0; n < 8; ++n) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double v = h.x[7][k];
      if (hex_corner(n, 0)) v = v + J[k][0];
      if (hex_corner(n, 1)) v = v + J[k][1];
      if (hex_corner(n, 2)) v = v + J[k][2];
      ok = ok && (v == h.x[n][k]);
    }
  }
  return ok;
}

// adj(J) (so that J^{-1} = adj / det), as mapping_isoparametric.py:216-224
__device__ __forceinline__ double adj3(const double J[3][3], double ad[3][3]) {
  ad[0][0] = -J[1][2] * J[2][1] + J[1][1] * J[2][2];
  ad[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  ad[2][0] = -J[1][1] * J[2][0] + J[1][0] * J[2][1];
  ad[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  ad[1][1] = -J[0][2] * J[2][0] + J[0][0] * J[2][2];
  ad[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  ad[0][2] = -J[0][2] * J[1][1] + J[0][1] * J[1][2];
  ad[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  ad[2][2] = -J[0][1] * J[1][0] + J[0][0] * J[1][1];
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

// M = |det| J^{-1} J^{-T} = adj adj^T / |det|  (symmetric)
__device__ __forceinline__ void hex_metric(const double ad[3][3], double det, double w,
                                           double M[3][3]) {
  const double s = w / fem::abs_bits(det);
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int l = k; l < 3; ++l) {
      const double v = s * (ad[k][0] * ad[l][0] + ad[k][1] * ad[l][1] + ad[k][2] * ad[l][2]);
      M[k][l] = v;
      M[l][k] = v;
    }
}

__device__ __forceinline__ void hex_shape(double x, double y, double z, double phi[8],
                                          double dphi[8][3]) {
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int cx = hex_corner(n, 0), cy = hex_corner(n, 1), cz = hex_corner(n, 2);
    const double fx = cx ? x : 1.0 - x, fy = cy ? y : 1.0 - y, fz = cz ? z : 1.0 - z;
    const double sx = cx ? 1.0 : -1.0, sy = cy ? 1.0 : -1.0, sz = cz ? 1.0 : -1.0;
    phi[n] = fx * fy * fz;
    dphi[n][0] = sx * (fy * fz);
    dphi[n][1] = sy * (fx * fz);
    dphi[n][2] = sz * (fx * fy);
  }
}

__global__ void __launch_bounds__(kBlock) hex_scalar_kernel(FemMesh m, FemBilinear f,
                                                            double* __restrict__ out,
                                                            const uint8_t* __restrict__ ref_bits,
                                                            int32_t* __restrict__ status,
                                                            const int32_t* __restrict__ cells,
                                                            int64_t ebeg, int64_t eend) {
  constexpr int L = 64;
  extern __shared__ double smem[];
  int64_t* cid = cells ? reinterpret_cast<int64_t*>(smem + (size_t)kBlock * (L + 1)) : nullptr;
  const int64_t e0 = ebeg + (int64_t)blockIdx.x * kBlock;
  int32_t flags = 0;
  const bool live = e0 + threadIdx.x < eend;
  int64_t e = 0;
  Hex h;
  double J[3][3];
  bool affine = true;
  if (live) {
    e = cell_at(cells, e0 + threadIdx.x);
    hex_load(m, e, h);
    affine = hex_affine(h, J);
  }
  // the reference element's values and gradients at the 64 points and the
  // points' weights, once per block that holds a general cell (every cell
  // reads them: broadcasts)
  double* tab = smem + (size_t)kBlock * (L + 1) + kBlock;   // after the rows and the cell ids
  double* sphi = tab;                 // [64][8]
  double* sdphi = tab + 64 * 8;       // [64][8][3]
  double* sw = tab + 64 * 32;         // [64]
  if (__syncthreads_or(affine ? 0 : 1)) {
    for (int q = threadIdx.x; q < 64; q += blockDim.x) {
      const int qx = q & 3, qy = (q >> 2) & 3, qz = q >> 4;
      double phi[8], dphi[8][3];
      hex_shape(c_gl4_x[qx], c_gl4_x[qy], c_gl4_x[qz], phi, dphi);
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        sphi[q * 8 + n] = phi[n];
#pragma unroll
        for (int k = 0; k < 3; ++k) sdphi[(q * 8 + n) * 3 + k] = dphi[n][k];
      }
      sw[q] = c_gl4_w[qx] * c_gl4_w[qy] * c_gl4_w[qz];
    }
    __syncthreads();
  }
  if (live) {
    if (cid) cid[threadIdx.x] = e;
    const int rb = ref_byte(ref_bits, e);
    const double kd = coef_at(f.diff, e);
    const double km = coef_at(f.mass, e);
    double* row = smem + threadIdx.x * (L + 1);
    if (affine) {
      double ad[3][3];
      const double det = adj3(J, ad);
      if (fem::zero_bits(det)) flags |= 1 << FEM_ERR_ZERO_JACOBIAN;
      double M[3][3];
      hex_metric(ad, det, kd, M);
      const double sm = km * fem::abs_bits(det);
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = i; j < 8; ++j) {
          double v = 0.0;
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int l = 0; l < 3; ++l) v = v + M[k][l] * c_hex_S[k][l][i][j];
          v = v + sm * c_hex_M[i][j];
          row[i * 8 + j] = v;
          row[j * 8 + i] = v;
        }
    } else {
#pragma unroll
      for (int k = 0; k < 64; ++k) row[k] = 0.0;
      const bool mass = !fem::zero_bits(km);
#pragma unroll 1
      for (int q = 0; q < 64; ++q) {
            const double* phi = sphi + q * 8;
            const double (*dphi)[3] = reinterpret_cast<const double (*)[3]>(sdphi + q * 24);
            const double w = sw[q];
            double Jq[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
              for (int b = 0; b < 3; ++b) {
                double acc = 0.0;
#pragma unroll
                for (int n = 0; n < 8; ++n) acc = acc + h.x[n][a] * dphi[n][b];
                Jq[a][b] = acc;
              }
            double ad[3][3];
            const double det = adj3(Jq, ad);
            if (fem::zero_bits(det)) {
              flags |= 1 << FEM_ERR_ZERO_JACOBIAN;
              continue;
            }
            double M[3][3];
            hex_metric(ad, det, w * kd, M);
            const double sm = w * km * fem::abs_bits(det);
            double hv[8][3];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
              for (int k = 0; k < 3; ++k)
                hv[i][k] = M[k][0] * dphi[i][0] + M[k][1] * dphi[i][1] + M[k][2] * dphi[i][2];
            if (mass) {
#pragma unroll
              for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = i; j < 8; ++j) {
                  const double v = hv[i][0] * dphi[j][0] + hv[i][1] * dphi[j][1] +
                                   hv[i][2] * dphi[j][2] + sm * (phi[i] * phi[j]);
                  row[i * 8 + j] += v;
                }
            } else {
              // no mass term (a zero mass coefficient): the stiffness alone
#pragma unroll
              for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = i; j < 8; ++j)
                  row[i * 8 + j] += hv[i][0] * dphi[j][0] + hv[i][1] * dphi[j][1] +
                                    hv[i][2] * dphi[j][2];
            }
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < i; ++j) row[i * 8 + j] = row[j * 8 + i];
    }
    if (status) flags |= coef_status(f, e, rb);
  }
  fem::publish_status(status, flags);
  flush_rows<L>(smem, out, e0, eend, cid);
}

// ------------------------------------------------------------ load vectors
template <int D, int ORDER>
__global__ void simplex_load_kernel(FemMesh m, FemLinear f, int ncomp, double* __restrict__ out) {
  constexpr int NS = SimplexTraits<D, ORDER>::NB;
  constexpr double FACT = SimplexTraits<D, ORDER>::FACT;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  double x[D + 1][D];
#pragma unroll
  for (int a = 0; a <= D; ++a) {
    const int64_t v = m.t[a * m.nelems + e];
#pragma unroll
    for (int k = 0; k < D; ++k) x[a][k] = m.p[k * m.nverts + v];
  }
  double det;
  if constexpr (D == 2) {
    det = (x[1][0] - x[0][0]) * (x[2][1] - x[0][1]) - (x[2][0] - x[0][0]) * (x[1][1] - x[0][1]);
  } else {
    double A[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) A[i][j] = x[j + 1][i] - x[0][i];
    det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
          A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
          A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  }
  const double s = coef_at(f.load, e) * (fem::abs_bits(det) / FACT);
#pragma unroll
  for (int i = 0; i < NS; ++i) {
    double lv;
    if constexpr (D == 2 && ORDER == 1) lv = tri1_load(i);
    else if constexpr (D == 2) lv = tri2_load(i);
    else if constexpr (ORDER == 1) lv = tet1_load(i);
    else lv = tet2_load(i);
    const double v = s * lv;
    for (int c = 0; c < ncomp; ++c) out[e * (int64_t)(NS * ncomp) + i * ncomp + c] = v;
  }
}

__global__ void hex_load_kernel(FemMesh m, FemLinear f, int ncomp, double* __restrict__ out,
                                int32_t* __restrict__ status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  Hex h;
  hex_load(m, e, h);
  const double fe = coef_at(f.load, e);
  double b[8];
  double J[3][3];
  if (hex_affine(h, J)) {
    double ad[3][3];
    const double det = adj3(J, ad);
    if (fem::zero_bits(det)) if (status) atomicOr(status, 1 << FEM_ERR_ZERO_JACOBIAN);
    const double v = fe * fem::abs_bits(det) * 0.125;
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = v;
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = 0.0;
    for (int q = 0; q < 64; ++q) {
      const int qx = q & 3, qy = (q >> 2) & 3, qz = q >> 4;
      double phi[8], dphi[8][3];
      hex_shape(c_gl4_x[qx], c_gl4_x[qy], c_gl4_x[qz], phi, dphi);
      const double w = c_gl4_w[qx] * c_gl4_w[qy] * c_gl4_w[qz];
      double Jq[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
          double acc = 0.0;
#pragma unroll
          for (int n = 0; n < 8; ++n) acc = acc + h.x[n][a] * dphi[n][bb];
          Jq[a][bb] = acc;
        }
      double ad[3][3];
      const double det = adj3(Jq, ad);
      if (fem::zero_bits(det)) if (status) atomicOr(status, 1 << FEM_ERR_ZERO_JACOBIAN);
      const double s = fe * w * fem::abs_bits(det);
#pragma unroll
      for (int i = 0; i < 8; ++i) b[i] = b[i] + s * phi[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
    for (int c = 0; c < ncomp; ++c) out[e * (int64_t)(8 * ncomp) + i * ncomp + c] = b[i];
}

// ------------------------------------------------------------------ launch
template <typename K>
static int set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    cudaError_t err =
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err != cudaSuccess) return fem::check_cuda(err, "cudaFuncSetAttribute");
  }
  return 0;
}

// The 2-D tensor map of the SoA geometry cache (ng rows of nelems doubles)
// with a box of ng x bs: encoded through the driver's cuTensorMapEncodeTiled
// (looked up once through the runtime).  False when it cannot be made
// (the row stride must be a multiple of 16 bytes: nelems even).
static bool geometry_tensor_map(const double* geo, int64_t nelems, int ng, int bs,
                                CUtensorMap* map) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                              const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                              const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<Encode>(fn);
    cudaGetLastError();
  }
  if (!encode || nelems <= 0 || (nelems * 8) % 16 != 0 || ((uintptr_t)geo % 16) != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nelems, (cuuint64_t)ng};
  const cuuint64_t strides[1] = {(cuuint64_t)nelems * sizeof(double)};
  const cuuint32_t box[2] = {(cuuint32_t)bs, (cuuint32_t)ng};
  const cuuint32_t estr[2] = {1, 1};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(geo), dims, strides,
                box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

template <int D, int O, int BS>
static int launch_scalar(const FemMesh& m, const FemBilinear& f, double* out,
                         const uint8_t* ref_bits, int32_t* status, int persistent,
                         cudaStream_t st, int64_t ebeg, int64_t eend, const int32_t* cells,
                         const double* geo, bool tma) {
  constexpr int NB = SimplexTraits<D, O>::NB;
  const size_t sm = (size_t)BS * (NB * NB + 1) * sizeof(double) + (cells ? kCidBytes<BS> : 0);
  int64_t grid = fem::ceil_div(eend - ebeg, BS);
  if (persistent > 0) grid = std::min<int64_t>(grid, (int64_t)persistent * fem::num_sms());
  FemCoef kdiff = f.diff;
  kdiff.scale = f.diff.scale * (1.0 / SimplexTraits<D, O>::FACT);
  CUtensorMap tmap;
  std::memset(&tmap, 0, sizeof(tmap));
  if (geo && tma && status && !cells && ebeg % 2 == 0 &&
      geometry_tensor_map(geo, m.nelems, kGeoCount<D>, BS, &tmap)) {
    // the TMA-staged form: the row buffer, the geometry tile (128-byte aligned), the mbarrier
    const size_t tile_off = ((size_t)BS * (NB * NB + 1) * sizeof(double) + 127) / 128 * 128;
    const size_t smt = tile_off + (size_t)kGeoCount<D> * BS * sizeof(double) + 16;
    int rc = set_smem(simplex_scalar_kernel<D, O, BS, true, true>, smt);
    if (rc) return rc;
    simplex_scalar_kernel<D, O, BS, true, true><<<(unsigned)grid, BS, smt, st>>>(
        m, f, kdiff, out, ref_bits, status, cells, geo, ebeg, eend, tmap);
  } else if (geo) {
    int rc = set_smem(simplex_scalar_kernel<D, O, BS, true>, sm);
    if (rc) return rc;
    simplex_scalar_kernel<D, O, BS, true><<<(unsigned)grid, BS, sm, st>>>(
        m, f, kdiff, out, ref_bits, status, cells, geo, ebeg, eend, tmap);
  } else {
    int rc = set_smem(simplex_scalar_kernel<D, O, BS, false>, sm);
    if (rc) return rc;
    simplex_scalar_kernel<D, O, BS, false><<<(unsigned)grid, BS, sm, st>>>(
        m, f, kdiff, out, ref_bits, status, cells, nullptr, ebeg, eend, tmap);
  }
  return 0;
}

template <int D, int O>
static int launch_scalar_tuned(const FemMesh& m, const FemBilinear& f, double* out,
                               const uint8_t* ref_bits, int32_t* status, cudaStream_t st,
                               int64_t ebeg, int64_t eend, const int32_t* cells,
                               const double* geo) {
  const fem::Tuning t = fem::tuning_for(D == 2 ? (O == 1 ? FEM_TRI_P1 : FEM_TRI_P2)
                                               : (O == 1 ? FEM_TET_P1 : FEM_TET_P2));
  const bool tma = t.local_tma != 0;
  switch (t.local_block) {
    case 64: return launch_scalar<D, O, 64>(m, f, out, ref_bits, status, t.persistent, st, ebeg, eend, cells, geo, tma);
    case 256: return launch_scalar<D, O, 256>(m, f, out, ref_bits, status, t.persistent, st, ebeg, eend, cells, geo, tma);
    default: return launch_scalar<D, O, 128>(m, f, out, ref_bits, status, t.persistent, st, ebeg, eend, cells, geo, tma);
  }
}

int local_matrices_checked(const FemMesh& m, const FemBasis& b, const FemBilinear& f, double* out,
                           const uint8_t* ref_bits, int32_t* status, cudaStream_t st,
                           int64_t ebeg, int64_t eend, const int32_t* cells, int upper,
                           const double* geo) {
  if (eend < 0 || eend > m.nelems) eend = m.nelems;
  if (ebeg < 0) ebeg = 0;
  if (eend <= ebeg) return 0;
  const int fam = b.family;
  const int64_t grid = fem::ceil_div(eend - ebeg, kBlock);
  int rc = 0;
  if (!b.vector) {
    switch (fam) {
      case FEM_TRI_P1: rc = launch_scalar_tuned<2, 1>(m, f, out, ref_bits, status, st, ebeg, eend, cells, geo); break;
      case FEM_TRI_P2: rc = launch_scalar_tuned<2, 2>(m, f, out, ref_bits, status, st, ebeg, eend, cells, geo); break;
      case FEM_TET_P1: rc = launch_scalar_tuned<3, 1>(m, f, out, ref_bits, status, st, ebeg, eend, cells, geo); break;
      case FEM_TET_P2: rc = launch_scalar_tuned<3, 2>(m, f, out, ref_bits, status, st, ebeg, eend, cells, geo); break;
      case FEM_HEX_1: {
        // the rows, room for the cell ids, the 64 points' tables
        const size_t sm = ((size_t)kBlock * 65 + kBlock + 64 * 33) * sizeof(double);
        if ((rc = set_smem(hex_scalar_kernel, sm))) return rc;
        hex_scalar_kernel<<<(unsigned)grid, kBlock, sm, st>>>(m, f, out, ref_bits, status, cells,
                                                              ebeg, eend);
        break;
      }
      default:
        fem::set_error(FEM_ERR_UNSUPPORTED, "unsupported element family %d", fam);
        return FEM_ERR_UNSUPPORTED;
    }
    if (rc) return rc;
  } else {
    const int64_t vgrid = fem::ceil_div(eend - ebeg, 64);
    switch (fam) {
#define LAUNCH_V(D, O)                                                                 \
  {                                                                                    \
    constexpr int NS = SimplexTraits<D, O>::NB, NB = NS * D;                          \
    constexpr int RB = D * NB;                                                         \
    const size_t sm = (size_t)64 * (RB + 1) * sizeof(double) + (cells ? kCidBytes<64> : 0); \
    if (upper) {                                                                       \
      if ((rc = set_smem(simplex_vector_kernel<D, O, true>, sm))) return rc;           \
      simplex_vector_kernel<D, O, true><<<(unsigned)vgrid, 64, sm, st>>>(m, f, out, ref_bits, status, cells, ebeg, eend); \
    } else {                                                                           \
      if ((rc = set_smem(simplex_vector_kernel<D, O, false>, sm))) return rc;          \
      simplex_vector_kernel<D, O, false><<<(unsigned)vgrid, 64, sm, st>>>(m, f, out, ref_bits, status, cells, ebeg, eend); \
    }                                                                                  \
    break;                                                                             \
  }
      case FEM_TRI_P1: LAUNCH_V(2, 1)
      case FEM_TRI_P2: LAUNCH_V(2, 2)
      case FEM_TET_P1: LAUNCH_V(3, 1)
      case FEM_TET_P2: LAUNCH_V(3, 2)
#undef LAUNCH_V
      default:
        fem::set_error(FEM_ERR_UNSUPPORTED,
                       "vector bases are implemented for simplex P1/P2 families (got family %d)", fam);
        return FEM_ERR_UNSUPPORTED;
    }
  }
  FEM_LAUNCH_CHECK("local matrix kernel");
  return 0;
}

// The coefficient checks of the channel kernels (coef_status) without the
// local matrices, for assemblies that take the matrices from a cache.  The
// host splits the form once per call: the channels with a field (pointer,
// stride, whether the scale is 0) are read per cell; the zero bits of the
// others follow from their scales alone (const_bits).  Each cell gets the
// status coef_status gives it: FEM_ERR_VARYING for a strided row that is not
// constant, FEM_ERR_STALE_PATTERN when its zero bits differ from ref.
struct FieldChecks {
  const double* field[5];
  int64_t stride[5];
  int bit[5];
  int scale_zero[5];
  int n;
  int const_bits;
};

__global__ void coef_fields_kernel(FieldChecks c, const uint8_t* __restrict__ ref_bits,
                                   int32_t* __restrict__ status, const int32_t* __restrict__ cells,
                                   int64_t ebeg, int64_t eend) {
  const int64_t pos = ebeg + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= eend) return;
  const int64_t e = cell_at(cells, pos);
  const int rb = ref_byte(ref_bits, e);
  int32_t st = 0;
  int bits = c.const_bits;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    if (k < c.n) {
      const int64_t s = c.stride[k];
      const double* r = c.field[k] + (s > 1 ? e * s : e);
      const unsigned long long v0 = fem::dbits(__ldg(r));
      if (s > 1) {
        bool same = true;
        for (int64_t q = 1; q < s; ++q) {
          const unsigned long long vq = fem::dbits(__ldg(r + q));
          same = same && (vq == v0 || ((vq | v0) << 1) == 0ull);
        }
        if (!same) st |= 1 << FEM_ERR_VARYING;
      }
      if (c.scale_zero[k] || (v0 << 1) == 0ull) bits |= 1 << c.bit[k];
    }
  }
  if (rb >= 0 && bits != rb) st |= 1 << FEM_ERR_STALE_PATTERN;
  fem::publish_status(status, st);
}

int coef_checks(const FemBilinear& f, const uint8_t* ref_bits, int32_t* status, cudaStream_t st,
                int64_t ebeg, int64_t eend, const int32_t* cells) {
  if (!status || eend <= ebeg) return 0;
  const FemCoef* ch[5] = {&f.diff, &f.mass, &f.lam, &f.lap, &f.tr};
  FieldChecks c{};
  for (int k = 0; k < 5; ++k) {
    if (ch[k]->field) {
      c.field[c.n] = ch[k]->field;
      c.stride[c.n] = ch[k]->stride;
      c.bit[c.n] = k;
      c.scale_zero[c.n] = ch[k]->scale == 0.0;
      ++c.n;
    } else if (ch[k]->scale == 0.0) {
      c.const_bits |= 1 << k;
    }
  }
  if (c.n == 0 && !ref_bits) return 0;   // nothing varies per cell, nothing to compare
  // one cell per thread: every cell's loads are in flight at once
  const int64_t grid = fem::ceil_div(eend - ebeg, 256);
  coef_fields_kernel<<<(unsigned)grid, 256, 0, st>>>(c, ref_bits, status, cells, ebeg, eend);
  FEM_LAUNCH_CHECK("coef_fields_kernel");
  return 0;
}

int vector_pair_blocks(const FemMesh& m, const FemBasis& b, const FemBilinear& f, double* out,
                       cudaStream_t st, int64_t ebeg, int64_t eend, const int32_t* cells,
                       const uint8_t* ref_bits, int32_t* status) {
  if (eend < 0) eend = m.nelems;
  if (eend <= ebeg) return 0;
  constexpr int BS = 64;
  const unsigned grid = (unsigned)fem::ceil_div(eend - ebeg, BS);
  const size_t cid = cells ? kCidBytes<BS> : 0;
  if (m.dim == 3) {
    const size_t sm = (size_t)BS * (10 * 9 + 2) * sizeof(double) + cid;
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(vector_pair_blocks_kernel<3, BS>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return fem::check_cuda(e, "vector_pair_blocks smem");
    }
    vector_pair_blocks_kernel<3, BS><<<grid, BS, sm, st>>>(m, f, out, cells, ebeg, eend,
                                                           ref_bits, status);
  } else if (m.dim == 2) {
    const size_t sm = (size_t)BS * (6 * 4 + 2) * sizeof(double) + cid;
    vector_pair_blocks_kernel<2, BS><<<grid, BS, sm, st>>>(m, f, out, cells, ebeg, eend,
                                                           ref_bits, status);
  } else {
    fem::set_error(FEM_ERR_UNSUPPORTED, "vector pair blocks of a %d-D mesh", m.dim);
    return FEM_ERR_UNSUPPORTED;
  }
  (void)b;
  FEM_LAUNCH_CHECK("vector_pair_blocks_kernel");
  return 0;
}

int scalar_pair_values(const FemMesh& m, const FemBasis& b, const FemBilinear& f,
                       const double* geo, double* out, cudaStream_t st, int64_t ebeg,
                       int64_t eend, const int32_t* cells, const uint8_t* ref_bits,
                       int32_t* status) {
  if (eend < 0) eend = m.nelems;
  if (eend <= ebeg) return 0;
  if (b.vector || (b.family != FEM_TRI_P2 && b.family != FEM_TET_P2) ||
      fem::basis_dim(b.family) != m.dim) {
    fem::set_error(FEM_ERR_UNSUPPORTED, "scalar pair values: not a scalar TriP2 / TetP2 basis");
    return FEM_ERR_UNSUPPORTED;
  }
  constexpr int BS = 128;
  const unsigned grid = (unsigned)fem::ceil_div(eend - ebeg, BS);
  const size_t cid = cells ? kCidBytes<BS> : 0;
  if (m.dim == 3) {
    const size_t sm = (size_t)BS * (kGramCount<3> + 2) * sizeof(double) + cid;
    scalar_pair_kernel<3, BS><<<grid, BS, sm, st>>>(m, f, geo, out, cells, ebeg, eend,
                                                    ref_bits, status);
  } else {
    const size_t sm = (size_t)BS * (kGramCount<2> + 2) * sizeof(double) + cid;
    scalar_pair_kernel<2, BS><<<grid, BS, sm, st>>>(m, f, geo, out, cells, ebeg, eend,
                                                    ref_bits, status);
  }
  FEM_LAUNCH_CHECK("scalar_pair_kernel");
  return 0;
}

int local_matrices(const FemMesh& m, const FemBasis& b, const FemBilinear& f, double* out,
                   int32_t* status, cudaStream_t st) {
  return local_matrices_checked(m, b, f, out, nullptr, status, st, 0, -1, nullptr, 0, nullptr);
}

// Doubles per cell of the geometry cache of the scalar simplex kernels (0:
// the family has none).
int geometry_count(const FemMesh& m, const FemBasis& b) {
  if (b.vector) return 0;
  switch (b.family) {
    case FEM_TRI_P1: case FEM_TRI_P2: return m.dim == 2 ? kGeoCount<2> : 0;
    case FEM_TET_P1: case FEM_TET_P2: return m.dim == 3 ? kGeoCount<3> : 0;
    default: return 0;
  }
}

int geometry_cache(const FemMesh& m, const FemBasis& b, double* geo, cudaStream_t st) {
  if (!geometry_count(m, b) || m.nelems == 0) return 0;
  const unsigned grid = (unsigned)fem::ceil_div(m.nelems, 128);
  if (m.dim == 2) simplex_geometry_cache_kernel<2><<<grid, 128, 0, st>>>(m, geo);
  else simplex_geometry_cache_kernel<3><<<grid, 128, 0, st>>>(m, geo);
  FEM_LAUNCH_CHECK("simplex_geometry_cache_kernel");
  return 0;
}

int local_vectors(const FemMesh& m, const FemBasis& b, const FemLinear& f, double* out,
                  int32_t* status, cudaStream_t st) {
  if (m.nelems == 0) return 0;
  const int ncomp = b.vector ? m.dim : 1;
  const unsigned grid = (unsigned)fem::ceil_div(m.nelems, 128);
  switch (b.family) {
    case FEM_TRI_P1: simplex_load_kernel<2, 1><<<grid, 128, 0, st>>>(m, f, ncomp, out); break;
    case FEM_TRI_P2: simplex_load_kernel<2, 2><<<grid, 128, 0, st>>>(m, f, ncomp, out); break;
    case FEM_TET_P1: simplex_load_kernel<3, 1><<<grid, 128, 0, st>>>(m, f, ncomp, out); break;
    case FEM_TET_P2: simplex_load_kernel<3, 2><<<grid, 128, 0, st>>>(m, f, ncomp, out); break;
    case FEM_HEX_1: hex_load_kernel<<<grid, 128, 0, st>>>(m, f, ncomp, out, status); break;
    default:
      fem::set_error(FEM_ERR_UNSUPPORTED, "unsupported element family %d", b.family);
      return FEM_ERR_UNSUPPORTED;
  }
  FEM_LAUNCH_CHECK("local vector kernel");
  return 0;
}

}  // namespace FEM_NS
