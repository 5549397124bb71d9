// Dirichlet condensation on the device: skfem.utils.condense
// (skfem/utils.py:462-600) for a CSR matrix already in HBM,
//   A_II = A[I][:, I],   b_I = b[I] - A[I][:, D] x[D],
// with I the kept DOFs in ascending order.  `map` gives each DOF its index
// in I, or -1 for eliminated DOFs.  Column order inside a row is preserved
// (the map is increasing on I), so the result is a canonical CSR like
// scipy's A[I][:, I]; the right-hand-side correction of each row is summed
// in the row's column order (deterministic).

#include "fem_common.cuh"

namespace {

__global__ void condense_count_kernel(const int32_t* __restrict__ indptr,
                                      const int32_t* __restrict__ indices, int64_t nrows,
                                      const int32_t* __restrict__ map, int32_t* __restrict__ cnt) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t nr = map[r];
  if (nr < 0) return;
  int32_t c = 0;
  for (int32_t p = indptr[r]; p < indptr[r + 1]; ++p) c += map[indices[p]] >= 0;
  cnt[nr] = c;
}

__global__ void condense_fill_kernel(const int32_t* __restrict__ indptr,
                                     const int32_t* __restrict__ indices,
                                     const double* __restrict__ vals, int64_t nrows,
                                     const int32_t* __restrict__ map, const double* __restrict__ b,
                                     const double* __restrict__ x,
                                     const int32_t* __restrict__ out_ptr,
                                     int32_t* __restrict__ out_ind, double* __restrict__ out_val,
                                     double* __restrict__ out_b) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t nr = map[r];
  if (nr < 0) return;
  int32_t o = out_ptr[nr];
  double corr = 0.0;
  for (int32_t p = indptr[r]; p < indptr[r + 1]; ++p) {
    const int32_t c = indices[p];
    const int32_t nc = map[c];
    if (nc >= 0) {
      out_ind[o] = nc;
      out_val[o] = vals[p];
      ++o;
    } else if (x) {
      corr += vals[p] * x[c];
    }
  }
  if (out_b) out_b[nr] = (b ? b[r] : 0.0) - corr;
}

}  // namespace

// enforce (utils.py:327-400): the rows D become zero with `diag` on their
// diagonal, in place (the pattern keeps its entries, as scipy keeps explicit
// zeros); b[D] = x[D].  missing counts D rows without a diagonal entry.
__global__ void enforce_kernel(const int32_t* __restrict__ indptr,
                               const int32_t* __restrict__ indices, double* __restrict__ vals,
                               const int32_t* __restrict__ rows, int64_t nd, double diag,
                               double* __restrict__ b, const double* __restrict__ x,
                               int32_t* __restrict__ missing) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nd) return;
  const int32_t r = rows[k];
  bool found = false;
  for (int32_t p = indptr[r]; p < indptr[r + 1]; ++p) {
    const bool d = indices[p] == r;
    vals[p] = d ? diag : 0.0;
    found = found || d;
  }
  if (!found) atomicAdd(missing, 1);
  if (b) b[r] = x ? x[r] : 0.0;
}

extern "C" {

int fem_enforce(const int32_t* indptr, const int32_t* indices, double* vals, int64_t nrows,
                const int32_t* rows, int64_t nd, double diag, double* b, const double* x,
                int32_t* missing, fem_stream_t stream) {
  if (!indptr || !indices || !vals || (!rows && nd > 0) || nd < 0 || nrows < 0 || !missing) {
    fem::set_error(FEM_ERR_ARGUMENT, "invalid enforce arguments");
    return FEM_ERR_ARGUMENT;
  }
  if (nd == 0) return 0;
  enforce_kernel<<<(unsigned)fem::ceil_div(nd, 256), 256, 0, (cudaStream_t)stream>>>(
      indptr, indices, vals, rows, nd, diag, b, x, missing);
  FEM_LAUNCH_CHECK("enforce_kernel");
  return 0;
}

int fem_condense_pattern(const int32_t* indptr, const int32_t* indices, int64_t nrows,
                         const int32_t* map, int64_t nkeep, int32_t* out_indptr, int64_t* out_nnz,
                         fem_stream_t stream) {
  if (!indptr || !map || !out_indptr || !out_nnz || nrows < 0 || nkeep < 0 || nkeep > nrows) {
    fem::set_error(FEM_ERR_ARGUMENT, "invalid condense arguments");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int32_t* cnt = nullptr;
  FEM_TRY_CUDA(cudaMallocAsync(&cnt, (nkeep + 1) * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(cnt, 0, (nkeep + 1) * sizeof(int32_t), st));
  if (nrows > 0) {
    condense_count_kernel<<<(unsigned)fem::ceil_div(nrows, 256), 256, 0, st>>>(indptr, indices,
                                                                               nrows, map, cnt);
    FEM_LAUNCH_CHECK("condense_count_kernel");
  }
  int rc = fem::exclusive_scan_i32(cnt, out_indptr, nkeep, out_nnz, st);
  cudaFreeAsync(cnt, st);
  return rc;
}

int fem_condense_values(const int32_t* indptr, const int32_t* indices, const double* vals,
                        int64_t nrows, const int32_t* map, const double* b, const double* x,
                        const int32_t* out_indptr, int32_t* out_indices, double* out_vals,
                        double* out_b, fem_stream_t stream) {
  if (!indptr || !indices || !vals || !map || !out_indptr || !out_indices || !out_vals) {
    fem::set_error(FEM_ERR_ARGUMENT, "invalid condense arguments");
    return FEM_ERR_ARGUMENT;
  }
  if (nrows == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  condense_fill_kernel<<<(unsigned)fem::ceil_div(nrows, 256), 256, 0, st>>>(
      indptr, indices, vals, nrows, map, b, x, out_indptr, out_indices, out_vals, out_b);
  FEM_LAUNCH_CHECK("condense_fill_kernel");
  return 0;
}

}  // extern "C"
