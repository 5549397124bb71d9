// Shared definitions of the skfem_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/skfem_gb300.h"

namespace fem {

// ---------------------------------------------------------------- errors
void set_error(int code, const char* fmt, ...);
int check_cuda(cudaError_t err, const char* what);

#define FEM_TRY_CUDA(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return ::fem::check_cuda(_e, #expr); \
  } while (0)

#define FEM_LAUNCH_CHECK(what)                                      \
  do {                                                              \
    cudaError_t _e = cudaGetLastError();                            \
    if (_e != cudaSuccess) return ::fem::check_cuda(_e, what);      \
  } while (0)

// ---------------------------------------------------------------- pattern
// Row incidence: for row r, inc[inc_ptr[r] .. inc_ptr[r+1]) lists the
// (element, local index) pairs whose DOF is r, encoded e * nbfun + i and
// sorted ascending -- the fixed summation order of every later call.
// CSR: indptr/indices as scipy returns them.  slot[(q) * nbfun_u + j] is
// the offset of local column j of incidence entry q inside its row
// (0xFFFF: exact-zero local entry, no CSR slot).
struct Pattern {
  int64_t nrows = 0;
  int64_t nelems = 0;
  int32_t nbfun_v = 0;   // local rows per element
  int32_t nbfun_u = 0;   // local columns per element
  int64_t ninc = 0;      // incidence entries = nelems * nbfun_v
  int64_t nnz = 0;
  int32_t max_row_nnz = 0;
  int32_t max_row_inc = 0;
  int32_t* inc_ptr = nullptr;   // nrows + 1
  int32_t* inc = nullptr;       // ninc
  int32_t* indptr = nullptr;    // nrows + 1 (matrix patterns only)
  int32_t* indices = nullptr;   // nnz
  uint16_t* slot = nullptr;     // ninc * nbfun_u
  bool has_matrix = false;
  int sum_unroll = 8;    // set from the family's tuning when the pattern is built
  int sum_cols = 1;      // fused sum: columns per lane (1, or 2 for an even row length)
  // Layout of the staging that fem_assemble_local writes for this pattern:
  // 0 full local matrices; D > 0 (vector bases of dimension D) the local
  // matrices' D x D blocks on and above the block diagonal only -- the
  // sum reads the others at their transposed positions (the vector
  // channel forms are symmetric).
  int staging_sym = 0;
};

// ---------------------------------------------------------------- helpers
inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Stream-ordered scratch that is released on every return path of the
// function that owns it (cudaFreeAsync on the stream it was taken on).
struct AsyncScratch {
  cudaStream_t st;
  void* ptrs[16] = {};
  int n = 0;
  explicit AsyncScratch(cudaStream_t s) : st(s) {}
  AsyncScratch(const AsyncScratch&) = delete;
  AsyncScratch& operator=(const AsyncScratch&) = delete;
  template <typename T>
  cudaError_t alloc(T** p, size_t bytes) {
    *p = nullptr;
    if (n >= 16) return cudaErrorInvalidValue;
    cudaError_t e = cudaMallocAsync((void**)p, bytes, st);
    if (e == cudaSuccess) ptrs[n++] = (void*)*p;
    return e;
  }
  ~AsyncScratch() {
    for (int i = n - 1; i >= 0; --i) cudaFreeAsync(ptrs[i], st);
  }
};

inline int num_sms();
// Blocks of a grid-stride kernel: enough for work_blocks, at most one wave
// of resident blocks (kern's occupancy at this block size and dynamic
// shared memory), so that every block runs from the start and no partial
// last wave idles the SMs.  Used by the one-pass P1 sums, whose slices
// carry about equal work (6M TetP1 cells: 0.338 ms in one wave against
// 0.369 ms in 3.5 waves of a 32-blocks-per-SM grid); the node-block sums,
// whose slices differ in work, keep an oversubscribed grid that the block
// scheduler balances (one wave measured slower there).
// The occupancy is looked up once per (kernel, block size, shared memory,
// device) and cached.
int resident_blocks_per_sm(const void* kern, int threads, size_t smem);
template <typename K>
inline int resident_grid(K kern, int threads, size_t smem, int64_t work_blocks) {
  const int per_sm = resident_blocks_per_sm(reinterpret_cast<const void*>(kern), threads, smem);
  return (int)std::max<int64_t>(1, std::min<int64_t>(work_blocks, (int64_t)per_sm * num_sms()));
}

inline int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

__device__ __forceinline__ double coef_at(const FemCoef& c, int64_t e) {
  return c.field ? c.scale * c.field[c.stride > 1 ? e * c.stride : e] : c.scale;
}

// Bit tests and |x| on the integer pipes: the FP64 pipe bounds the local
// kernels, so comparisons and sign masks stay off it.  The bit pattern is
// moved through an inline-PTX mov, which the optimizer cannot see through
// (it would otherwise fold the integer test back into an FP64 compare).
// zero_bits(x) is x == 0.0 (either sign; false for NaN).
__device__ __forceinline__ unsigned long long dbits(double x) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
}
__device__ __forceinline__ double dfrombits(unsigned long long u) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
}
__device__ __forceinline__ bool zero_bits(double x) { return (dbits(x) << 1) == 0ull; }
__device__ __forceinline__ double abs_bits(double x) {
  return dfrombits(dbits(x) & 0x7fffffffffffffffull);
}

// coef_at(c, e) is zero because its scale or its field value is exactly 0
// (either sign) -- the zero bit of a channel, tested without forming the
// product (an underflow of the product itself is not tracked).  The
// pattern build and every later call use this same definition.
__device__ __forceinline__ bool coef_zero(const FemCoef& c, int64_t e) {
  if (zero_bits(c.scale)) return true;
  return c.field ? zero_bits(c.field[c.stride > 1 ? e * c.stride : e]) : false;
}

// A strided (per-point) coefficient must be constant over the cell's points
// for the channel kernels -- bitwise, with +0.0 and -0.0 taken as equal --
// otherwise the status bit FEM_ERR_VARYING (the caller then takes the
// generic path).  Returns the bit instead of publishing it, so the kernels
// keep their flags in a register and issue one atomic at the end.
__device__ __forceinline__ int32_t row_status(const FemCoef& c, int64_t e) {
  if (!c.field || c.stride <= 1) return 0;
  const double* r = c.field + e * c.stride;
  const unsigned long long v0 = dbits(r[0]);
  bool same = true;
  for (int64_t q = 1; q < c.stride; ++q) {
    const unsigned long long vq = dbits(r[q]);
    same = same && (vq == v0 || ((vq | v0) << 1) == 0ull);
  }
  return same ? 0 : (1 << FEM_ERR_VARYING);
}

// Publishes a thread's accumulated status bits (one atomic per thread).
__device__ __forceinline__ void publish_status(int32_t* status, int32_t bits) {
  if (bits && status) atomicOr(status, bits);
}

// Reference-cube corner (0/1 per axis) of Hex1 node n: node 0 sits at
// (1,1,1) and node 7 at (0,0,0) (refdom.py:173-180).  constexpr so that
// unrolled loops index registers, not memory.
__host__ __device__ constexpr int hex_corner(int n, int ax) {
  constexpr int tab[8][3] = {{1, 1, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1},
                             {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}};
  return tab[n][ax];
}

// Exclusive scan of n int32 counts into out (n+1 entries); device scratch
// from the caller's allocation helper.  Returns the total via *total (host).
int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int64_t* total,
                       cudaStream_t stream);

// Launch parameters chosen by the autotuner (fem_set_tuning), per family.
struct Tuning {
  int local_block = 128;  // threads (= cells) per CTA of the local kernel
  int persistent = 0;     // >0: grid capped at persistent * SMs (grid-stride)
  int sum_unroll = 8;     // incidence entries loaded together in the sum
  int sum_cols = 1;       // fused sum: columns per lane (1, or 2 for an even row length)
  int onepass = 1;        // one-pass P1 sum: 0 two lanes per row, 1 a lane per upper entry,
                          // 2 the same with its codes staged in shared memory by TMA
  int local_tma = 0;      // local kernel on the geometry cache: 1 each tile's geometry
                          // staged by a 2-D TMA tensor copy (fem_set_local_tma)
};
Tuning tuning_for(int family);

// Fixed-order segmented sum of local matrices into CSR values, rows
// [row0, row1) (row1 < 0: to the last row); check_status non-null: also
// verify the exact-zero structure (FEM_ERR_STALE_PATTERN).  sym > 0: the
// local matrices hold their sym x sym blocks on and above the block
// diagonal only (Pattern::staging_sym), square patterns.
int csr_sum(const Pattern& P, const double* local, double* vals, cudaStream_t st,
            int64_t row0 = 0, int64_t row1 = -1, int32_t* check_status = nullptr, int sym = 0);

// Fused assembly of a scalar form k_e * S_e + mscale * M on cached geometry
// (rows [row0, row1)): stiff = the cells' geometry-only stiffness rows in
// incidence order (incidence_rows), mass1 = the CSR values of the
// unit-coefficient mass matrix (null: no mass part); the stiffness factor
// is diff (scale and per-cell field).
int csr_sum_scaled(const Pattern& P, const double* stiff, const FemCoef& diff,
                   const double* mass1, double mscale, double* vals, cudaStream_t st,
                   int64_t row0 = 0, int64_t row1 = -1);
// Element-major full local rows (nelems x nbfun x nbfun) into incidence
// order (ninc x nbfun) for csr_sum_scaled.
int incidence_rows(const Pattern& P, const double* local, double* out, cudaStream_t st);

// One-pass assembly of a scalar P1 simplex form k_e S_e + m M_e (rows
// [row0, row1)) from the per-cell geometry cache geo (Gram entries scaled
// by 1/(d! |det|), then |det|); mbase: the rows' fixed-point binary points
// of the constant-coefficient mass sums (row_mass_base; unused when the
// mass coefficient has a field).
int csr_sum_geometry_p1(const Pattern& P, int dim, const double* geo, const FemCoef& diff,
                        const FemCoef& mass, const int16_t* mbase, double* vals, cudaStream_t st,
                        int64_t row0 = 0, int64_t row1 = -1);
// The rows' binary points for csr_sum_geometry_p1 from the cells' |det|
// (adet: nelems doubles); *ok false when some |det| is outside the range
// the fixed point covers (degenerate or non-finite cells).
int row_mass_base(const Pattern& P, const double* adet, int16_t* mbase, int* shmax, bool* ok,
                  cudaStream_t st);

// The one-pass P1 sum in its upper-gather form (csr_upper_p1_kernel): per
// CSR entry on or above the diagonal, the (cell, local pair) contributions
// in the sum's order, sliced 32 entries at a time.  Pattern-only data.
struct UpperLists {
  int64_t nd = 0, nupper = 0, nslices = 0, ncodes = 0;
  // 0: diagonal entries first, then the others; > 0: rows in blocks of
  // block_rows, each block's diagonal entries then its others (upper_slot)
  int64_t block_rows = 0;
  int32_t max_len = 0;          // the longest slice (codes per lane)
  int32_t* dpos = nullptr;      // nrows + 1: row -> first diagonal entry
  int32_t* opos = nullptr;      // nrows + 1: row -> first off-diagonal entry (after nd)
  int32_t* pos = nullptr;       // nupper: CSR index of (i, j)
  int32_t* tpos = nullptr;      // nupper: CSR index of (j, i); -1 on the diagonal
  int32_t* row = nullptr;       // nupper: i
  int32_t* slice_len = nullptr;   // nslices
  int32_t* slice_base = nullptr;  // nslices: first code row (32 codes) of the slice
  // ncodes, 0xFFFFFFFF padding: e * 16 + k, k the Gram entry of the local
  // pair (li, lj) (at most 4 local functions, narrow codes), or
  // e * 128 + li * nu + lj (wide codes, nu <= 11)
  uint32_t* codes = nullptr;
  std::vector<int32_t> dpos_h, opos_h;
};
// wide: codes e * 128 + li * nu + lj whatever nu (always for nu > 4);
// block_rows: the row-block layout (UpperLists::block_rows)
int build_upper_lists(const Pattern& P, UpperLists* U, cudaStream_t st, bool wide = false,
                      int64_t block_rows = 0);
// Rows per block of the one-pass P1 sum's upper lists
constexpr int64_t kUpperBlockRows = 4096;
void free_upper_lists(UpperLists* U);
// tma: stage each warp's slice codes in shared memory with bulk copies
// (needs status for its bounded waits' error bit)
// ref_bits / const_bits: the coefficient checks folded into the plain form
// (a per-cell stiffness field of stride 1 and a nonzero constant mass; the
// cells' zero bits against the pattern's, FEM_ERR_STALE_PATTERN in *status)
int csr_sum_upper_p1(const Pattern& P, const UpperLists& U, int dim, const double* geo,
                     const FemCoef& diff, const FemCoef& mass, const int16_t* mbase, double* vals,
                     cudaStream_t st, int64_t row0 = 0, int64_t row1 = -1,
                     int32_t* status = nullptr, bool tma = false,
                     const uint8_t* ref_bits = nullptr, int const_bits = 0);
// True when csr_sum_upper_p1 checks the coefficients itself for this form
// (the plain form, not TMA-staged)
inline bool upper_p1_checks(const FemCoef& diff, const FemCoef& mass, bool tma) {
  return !tma && diff.field && diff.stride <= 1 && !mass.field && mass.scale != 0.0;
}

int basis_nb_scalar(int family);
int basis_dim(int family);

int build_incidence(const int32_t* dofs, int64_t nelems, int nb, int64_t nrows, Pattern* P,
                    cudaStream_t st);
// local == nullptr: every (row, column) pair of a cell is an entry
int build_csr(const int32_t* udofs, int nu, int64_t ncols, const double* local, Pattern* P,
              cudaStream_t st);
void free_pattern(Pattern* P);

// One-pass sum of the vector channel forms on simplex ElementVector bases
// (fem_vecsum.cu): per node block (I, J), I <= J, its contribution list (the
// node-level pattern's upper lists, codes e * 128 + i * ns + j) and the
// vector CSR positions and presence mask of its entries.
struct VecUpper {
  int dim = 0, ns = 0;          // dim: the block size (the mesh dimension; 1 for scalar bases)
  int sdim = 0;                 // the mesh dimension
  int64_t block_rows = 0;       // node rows per block of the lists' row-block layout
  int64_t nelems = 0;
  UpperLists U;                 // pos / tpos / row released after the build
  int32_t* vpos = nullptr;      // dim * nupper: rows D*I + a, first entry of the block
  int32_t* vposT = nullptr;     // dim * nupper: rows D*J + b (transposed block; -1 if I == J)
  uint16_t* vmask = nullptr;    // nupper: bit a*D + b, entry (D*I + a, D*J + b) present
  void* terms = nullptr;        // reference-tensor terms per local node pair
  int32_t* count = nullptr;
  double* mm = nullptr;         // mass table per local node pair
};
// dim: the block size -- the family's dimension (ElementVector bases) or 1
// (scalar TriP2 / TetP2 bases)
int build_vec_upper(const Pattern& P, const int32_t* udofs, int family, int dim, VecUpper* V,
                    cudaStream_t st);
void free_vec_upper(VecUpper* V);
// doubles per cell of the pair blocks the sum reads (vector_pair_blocks,
// scalar_pair_values): sdim the mesh dimension, dim the block size
inline int64_t vec_pair_stride(int sdim, int dim) {
  const int np = (sdim + 1) * (sdim + 2) / 2;
  return (int64_t)np * dim * dim + 1;
}
// DOF rows [row0, row1) (multiples of dim; row1 < 0: to the last row): the
// node blocks of their node rows, which also complete the rows' entries
// left of the diagonal (written by earlier node rows' blocks)
// DOF rows per window of the node blocks' work-sorted layout: row ranges of
// vec_upper_sum start and end on multiples of it (or end at the last row)
int64_t vec_window_rows(const VecUpper& V);
// coop: the D*D lanes of a node block cooperate (vec_upper_coop_kernel).
// E: the caller's staging (nelems x nbfun^2 doubles) holding the pair values
// in its first nelems x vec_pair_stride doubles; the 4 bytes after them are
// written (the slices' ticket).
int vec_upper_sum(const VecUpper& V, const double* E, bool mass, double* vals, cudaStream_t st,
                  int64_t row0 = 0, int64_t row1 = -1, bool coop = false);

}  // namespace fem
