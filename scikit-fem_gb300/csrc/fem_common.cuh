// Shared definitions of the skfem_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <string>

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
};

// ---------------------------------------------------------------- helpers
inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

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

// A strided (per-point) coefficient must be constant over the cell's points
// for the channel kernels; otherwise flag FEM_ERR_VARYING.
__device__ __forceinline__ void check_row(const FemCoef& c, int64_t e, int32_t* status) {
  if (!c.field || c.stride <= 1) return;
  const double* r = c.field + e * c.stride;
  const double v0 = r[0];
  bool same = true;
  for (int64_t q = 1; q < c.stride; ++q) same = same && r[q] == v0;
  if (!same && status) atomicOr(status, 1 << FEM_ERR_VARYING);
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
};
Tuning tuning_for(int family);

// Fixed-order segmented sum of local matrices into CSR values, rows
// [row0, row1) (row1 < 0: to the last row); check_status non-null: also
// verify the exact-zero structure (FEM_ERR_STALE_PATTERN).
int csr_sum(const Pattern& P, const double* local, double* vals, cudaStream_t st,
            int64_t row0 = 0, int64_t row1 = -1, int32_t* check_status = nullptr);

int basis_nb_scalar(int family);
int basis_dim(int family);

}  // namespace fem
