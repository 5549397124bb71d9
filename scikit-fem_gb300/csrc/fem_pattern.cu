// One-time CSR pattern build and the per-call fixed-order segmented sum.
//
// Replaces COOData._assemble_scipy_csr (skfem/assembly/form/coo_data.py:27-36):
//   coo_matrix((data, (rows, cols))).eliminate_zeros().tocsr()
// whose result is a canonical CSR (sorted column indices, duplicates summed)
// in which a (row, col) pair exists iff at least one of its local entries is
// nonzero -- eliminate_zeros drops exact +-0.0 local entries before the
// duplicates are summed.  And COOData.toarray for load vectors
// (coo_data.py:102-108).
//
// Build (once per mesh / basis / zero structure):
//   1. row incidence: for every global row r the (element, local row) pairs
//      that map to r, counted, scanned, filled and sorted so that every later
//      summation runs in ascending (element, local row) order;
//   2. per row, one warp gathers the candidate columns of its incidence
//      entries whose local value is nonzero, sorts them in shared memory
//      (bitonic), counts the unique ones (row length), and after a scan
//      writes the column indices and, for each local entry, the offset of
//      its column inside the row (the slot map).
// Every call afterwards: one row group per CSR row walks the row's
// incidence list in order and adds each local row into shared-memory
// accumulators at the precomputed slots -- deterministic, no atomics.

#include "fem_common.cuh"

#include <type_traits>

namespace fem {

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr size_t kMaxBlockSmem = 227 * 1024;
// candidate columns a warp gathers and sorts for one CSR row (a power of two;
// 2 x 16384 words = 128 KB of shared memory, one warp per block at that size)
constexpr int kMaxRowCandidates = 16384;

// Warps per block of a kernel whose warps each hold bytes_per_warp of shared
// memory (candidate columns, row accumulators): kWarpsPerBlock, or fewer when
// that does not fit the 227 KB a block may use; 0 when one warp does not fit.
static int smem_block_warps(size_t bytes_per_warp) {
  for (int w = kWarpsPerBlock; w >= 1; --w)
    if ((size_t)w * bytes_per_warp <= kMaxBlockSmem) return w;
  return 0;
}

static int row_smem_error(int row_nnz) {
  set_error(FEM_ERR_CAPACITY,
            "a CSR row of %d entries needs more shared memory for its accumulators than a "
            "block has (227 KB)", row_nnz);
  return FEM_ERR_CAPACITY;
}

__global__ void count_rows_kernel(const int32_t* __restrict__ dofs, int64_t nelems, int nb,
                                  int64_t nrows, int32_t* __restrict__ cnt,
                                  int32_t* __restrict__ err) {
  const int64_t n = nelems * nb;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = dofs[idx];
    if (r < 0 || r >= nrows) {
      atomicOr(err, 1);
      continue;
    }
    atomicAdd(&cnt[r], 1);
  }
}

__global__ void fill_rows_kernel(const int32_t* __restrict__ dofs, int64_t nelems, int nb,
                                 int64_t nrows, const int32_t* __restrict__ ptr,
                                 int32_t* __restrict__ cursor, int32_t* __restrict__ inc) {
  const int64_t n = nelems * nb;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = dofs[idx];
    if (r < 0 || r >= nrows) continue;
    const int64_t i = idx / nelems;
    const int64_t e = idx - i * nelems;
    const int32_t pos = ptr[r] + atomicAdd(&cursor[r], 1);
    inc[pos] = (int32_t)(e * nb + i);
  }
}

// Sort each row's incidence segment ascending (segments are short: the
// number of cells sharing a DOF).
__global__ void sort_segments_kernel(const int32_t* __restrict__ ptr, int64_t nrows,
                                     int32_t* __restrict__ inc, int32_t* __restrict__ maxlen) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t b = ptr[r], n = ptr[r + 1] - b;
  int32_t* s = inc + b;
  for (int k = 1; k < n; ++k) {
    const int32_t v = s[k];
    int m = k - 1;
    while (m >= 0 && s[m] > v) {
      s[m + 1] = s[m];
      --m;
    }
    s[m + 1] = v;
  }
  atomicMax(maxlen, n);
}

// Bitonic sort of `n2` (power of two) int32 keys in shared memory by one warp.
__device__ void warp_bitonic_sort(int32_t* a, int n2) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n2; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int32_t x = a[i], y = a[ixj];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
  }
}

// Candidate columns of row r at fixed positions q*nu + j (masked: INT_MAX),
// sorted copy in `srt`, original order in `cand`.  Returns unique count.
__device__ int row_columns(int64_t r, const int32_t* __restrict__ inc_ptr,
                           const int32_t* __restrict__ inc, const int32_t* __restrict__ udofs,
                           const double* __restrict__ local, int64_t nelems, int nv, int nu,
                           int cap, int32_t* cand, int32_t* srt) {
  const int lane = threadIdx.x & 31;
  const int32_t b = inc_ptr[r], len = inc_ptr[r + 1] - b;
  const int n = len * nu;
  int n2 = 1;
  while (n2 < n) n2 <<= 1;
  for (int k = lane; k < n2; k += 32) {
    int32_t c = INT32_MAX;
    if (k < n) {
      const int q = k / nu, j = k - q * nu;
      const int32_t code = inc[b + q];
      const int64_t e = code / nv;
      const int64_t i = code - e * nv;
      // without local matrices every (row, column) pair is an entry
      if (!local || local[(e * nv + i) * nu + j] != 0.0) c = udofs[(int64_t)j * nelems + e];
    }
    if (k < n) cand[k] = c;
    srt[k] = c;
  }
  __syncwarp();
  warp_bitonic_sort(srt, n2);
  // unique count of the non-sentinel prefix
  int cnt = 0;
  for (int base = 0; base < n; base += 32) {
    const int k = base + lane;
    bool first = false;
    if (k < n) {
      const int32_t c = srt[k];
      first = (c != INT32_MAX) && (k == 0 || srt[k - 1] != c);
    }
    cnt += __popc(__ballot_sync(0xffffffffu, first));
  }
  return cnt;
}

__global__ void row_nnz_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                               const int32_t* __restrict__ udofs, const double* __restrict__ local,
                               int64_t nrows, int64_t nelems, int nv, int nu, int cap,
                               int32_t* __restrict__ row_nnz, int32_t* __restrict__ maxnnz) {
  extern __shared__ int32_t ismem[];
  const int w = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  int32_t* cand = ismem + (size_t)w * 2 * cap;
  int32_t* srt = cand + cap;
  for (int64_t r = (int64_t)blockIdx.x * nw + w; r < nrows; r += (int64_t)gridDim.x * nw) {
    const int cnt = row_columns(r, inc_ptr, inc, udofs, local, nelems, nv, nu, cap, cand, srt);
    if ((threadIdx.x & 31) == 0) {
      row_nnz[r] = cnt;
      atomicMax(maxnnz, cnt);
    }
    __syncwarp();
  }
}

__global__ void row_fill_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                const int32_t* __restrict__ udofs, const double* __restrict__ local,
                                int64_t nrows, int64_t nelems, int nv, int nu, int cap,
                                const int32_t* __restrict__ indptr, int32_t* __restrict__ indices,
                                uint16_t* __restrict__ slot) {
  extern __shared__ int32_t ismem[];
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  int32_t* cand = ismem + (size_t)w * 2 * cap;
  int32_t* srt = cand + cap;
  for (int64_t r = (int64_t)blockIdx.x * nw + w; r < nrows; r += (int64_t)gridDim.x * nw) {
    row_columns(r, inc_ptr, inc, udofs, local, nelems, nv, nu, cap, cand, srt);
    const int32_t b = inc_ptr[r], len = inc_ptr[r + 1] - b;
    const int n = len * nu;
    // compact unique columns to the front of srt (ballot-based stream compaction)
    int out = 0;
    for (int base = 0; base < n; base += 32) {
      const int k = base + lane;
      int32_t c = INT32_MAX;
      bool first = false;
      if (k < n) {
        c = srt[k];
        first = (c != INT32_MAX) && (k == 0 || srt[k - 1] != c);
      }
      const unsigned m = __ballot_sync(0xffffffffu, first);
      __syncwarp();
      if (first) {
        const int pos = out + __popc(m & ((1u << lane) - 1u));
        srt[pos] = c;  // pos <= k: never overwrites an unread element of this chunk
      }
      out += __popc(m);
      __syncwarp();
    }
    const int32_t row0 = indptr[r];
    for (int k = lane; k < out; k += 32) indices[row0 + k] = srt[k];
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
      const int32_t c = cand[k];
      uint16_t s = 0xFFFF;
      if (c != INT32_MAX) {
        int lo = 0, hi = out - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (srt[mid] < c) lo = mid + 1;
          else hi = mid;
        }
        s = (uint16_t)lo;
      }
      slot[(int64_t)b * nu + k] = s;
    }
    __syncwarp();
  }
}

// Fixed-order segmented sum.  G lanes per row (G = power of two >= nu);
// shared accumulators of `stride` doubles per row.  Incidence entries are
// taken U at a time: their index, slot and value loads are issued together
// (independent of each other), then added in order -- entry q's additions
// complete (__syncwarp) before entry q+1's, so every slot sums its
// contributions in ascending (element, local row) order.
// CHECK: also verify the zero structure (exact local masks, generic path):
// a nonzero local entry without a slot, or a CSR entry that no nonzero
// local entry reaches, sets FEM_ERR_STALE_PATTERN in *status.
// SYM > 0: the local matrices hold their SYM x SYM blocks on and above the
// block diagonal only; entry (i, j) of a block below it is read at (j, i).
// The cell of an incidence code is code / nu (square patterns), taken as
// the high word of code * div_magic (div_magic = ceil(2^64 / nu), exact
// for codes below 2^32).
template <int G, int U, bool CHECK, int SYM = 0>
__global__ void csr_sum_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                               const uint16_t* __restrict__ slot, const int32_t* __restrict__ indptr,
                               const double* __restrict__ local, int64_t row0, int64_t nrows,
                               int nu, int stride, double* __restrict__ vals,
                               int32_t* __restrict__ status, unsigned long long div_magic = 0) {
  extern __shared__ double acc_smem[];
  constexpr int RPW = 32 / G;  // rows per warp
  const int lane = threadIdx.x & 31;
  const int sub = lane / G;      // row within warp
  const int j = lane - sub * G;  // local column
  const int wib = threadIdx.x >> 5;
  double* acc = acc_smem + ((size_t)wib * RPW + sub) * stride;
  uint8_t* seen = reinterpret_cast<uint8_t*>(acc_smem + (size_t)(blockDim.x >> 5) * RPW * stride) +
                  ((size_t)wib * RPW + sub) * stride;
  bool stale = false;
  const int64_t rows_per_block = (int64_t)(blockDim.x >> 5) * RPW;
  for (int64_t rb = row0 + (int64_t)blockIdx.x * rows_per_block; rb < nrows;
       rb += (int64_t)gridDim.x * rows_per_block) {
    const int64_t r = rb + (int64_t)wib * RPW + sub;
    const bool live = r < nrows;
    int32_t b = 0, len = 0, p0 = 0, nnz = 0;
    if (live) {
      b = inc_ptr[r];
      len = inc_ptr[r + 1] - b;
      p0 = indptr[r];
      nnz = indptr[r + 1] - p0;
    }
    for (int k = j; k < nnz; k += G) {
      acc[k] = 0.0;
      if (CHECK) seen[k] = 0;
    }
    int maxlen = len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
    __syncwarp();
    for (int q0 = 0; q0 < maxlen; q0 += U) {
      double v[U];
      int s[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = q0 + u;
        s[u] = 0xFFFF;
        v[u] = 0.0;
        if (q < len && j < nu) {
          const int64_t code = __ldg(inc + b + q);
          s[u] = __ldg(slot + ((int64_t)b + q) * nu + j);
          int64_t at = code * nu + j;
          if constexpr (SYM > 0) {
            const int64_t e = (int64_t)__umul64hi((unsigned long long)code, div_magic);
            const int il = (int)(code - e * nu);
            if (j / SYM < il / SYM) at = (e * nu + j) * nu + il;
          }
          v[u] = __ldg(local + at);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (s[u] != 0xFFFF) {
          acc[s[u]] += v[u];
          if (CHECK && !zero_bits(v[u])) seen[s[u]] = 1;
        } else if (CHECK && !zero_bits(v[u])) {
          stale = true;
        }
        __syncwarp();
      }
    }
    for (int k = j; k < nnz; k += G) {
      vals[p0 + k] = acc[k];
      if (CHECK) stale = stale || !seen[k];
    }
    __syncwarp();
  }
  if (CHECK && stale) atomicOr(status, 1 << FEM_ERR_STALE_PATTERN);
}

// Fused assembly of a scalar form  k_e * S_e + m * M_e  on cached geometry:
// stiff holds every cell's geometry-only stiffness rows in incidence order
// (row q of the incidence list at stiff + q * nu), mass1 the CSR values of
// the unit-coefficient mass matrix.  Per CSR row the slots accumulate
// fma(k_e, S_e[il][j], acc) in ascending (element, local row) order, as
// csr_sum_kernel adds local entries, then the entry is
// fma(mscale, mass1[p], dscale * acc).  field: the per-cell factor k_e of
// the stiffness (field[e * fstride]; null: 1); stiff null: no stiffness
// part.  The cell of an incidence code is code / NU when the row length is
// a compile-time NU (a shift for TetP1's 4), else code / nu by the same
// magic division as the block-upper sum.
template <int G, int U, int NU = 0>
__global__ void csr_scaled_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                  const uint16_t* __restrict__ slot, const int32_t* __restrict__ indptr,
                                  const double* __restrict__ stiff, const double* __restrict__ field,
                                  int64_t fstride, double dscale, const double* __restrict__ mass1,
                                  double mscale, int64_t row0, int64_t nrows, int nu, int stride,
                                  double* __restrict__ vals, unsigned long long div_magic) {
  extern __shared__ double acc_smem[];
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int sub = lane / G;
  const int j = lane - sub * G;
  const int wib = threadIdx.x >> 5;
  double* acc = acc_smem + ((size_t)wib * RPW + sub) * stride;
  const int64_t rows_per_block = (int64_t)(blockDim.x >> 5) * RPW;
  for (int64_t rb = row0 + (int64_t)blockIdx.x * rows_per_block; rb < nrows;
       rb += (int64_t)gridDim.x * rows_per_block) {
    const int64_t r = rb + (int64_t)wib * RPW + sub;
    const bool live = r < nrows;
    int32_t b = 0, len = 0, p0 = 0, nnz = 0;
    if (live) {
      b = inc_ptr[r];
      len = stiff ? inc_ptr[r + 1] - b : 0;
      p0 = indptr[r];
      nnz = indptr[r + 1] - p0;
    }
    for (int k = j; k < nnz; k += G) acc[k] = 0.0;
    int maxlen = len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
    __syncwarp();
    for (int q0 = 0; q0 < maxlen; q0 += U) {
      double v[U], kv[U];
      int s[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = q0 + u;
        s[u] = 0xFFFF;
        v[u] = 0.0;
        kv[u] = 1.0;
        if (q < len && j < nu) {
          const int64_t at = ((int64_t)b + q) * nu + j;
          s[u] = __ldg(slot + at);
          v[u] = __ldg(stiff + at);
          if (field) {
            const unsigned long long code = (unsigned long long)__ldg(inc + b + q);
            const int64_t e = NU > 0 ? (int64_t)(code / NU) : (int64_t)__umul64hi(code, div_magic);
            kv[u] = __ldg(field + e * fstride);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (s[u] != 0xFFFF) acc[s[u]] = __fma_rn(kv[u], v[u], acc[s[u]]);
        __syncwarp();
      }
    }
    for (int k = j; k < nnz; k += G) {
      double a = dscale * acc[k];
      if (mass1) a = __fma_rn(mscale, __ldg(mass1 + p0 + k), a);
      vals[p0 + k] = a;
    }
    __syncwarp();
  }
}

// csr_scaled_kernel for an even number NU of local functions (TetP1 4,
// TriP2 6, TetP2 10) with two columns per lane: NU / 2 lanes per CSR row,
// lane h takes columns 2h and 2h+1 of each incidence entry -- one 16-byte
// load of its two stiffness values, one 4-byte load of their two slots, one
// coefficient gather for both -- so a warp keeps 32 / (NU / 2) rows'
// entries in flight (the lanes beyond them idle).  The columns of an entry
// have distinct slots, and entries are still added in ascending order
// (__syncwarp between them): the values are bit for bit those of
// csr_scaled_kernel.
template <int NU, int U>
__global__ void csr_scaled_pair_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                       const uint16_t* __restrict__ slot, const int32_t* __restrict__ indptr,
                                       const double* __restrict__ stiff, const double* __restrict__ field,
                                       int64_t fstride, double dscale, const double* __restrict__ mass1,
                                       double mscale, int64_t row0, int64_t nrows, int stride,
                                       double* __restrict__ vals) {
  extern __shared__ double acc_smem[];
  constexpr int LPR = NU / 2;        // lanes per row
  constexpr int RPW = 32 / LPR;      // rows per warp
  static_assert(NU % 2 == 0 && LPR <= 32, "two columns per lane need an even row length");
  const int lane = threadIdx.x & 31;
  const int sub = lane / LPR;        // RPW for the idle lanes
  const int h = lane - sub * LPR;
  const int wib = threadIdx.x >> 5;
  const bool row_lane = sub < RPW;
  double* acc = acc_smem + ((size_t)wib * RPW + (row_lane ? sub : 0)) * stride;
  const int64_t rows_per_block = (int64_t)(blockDim.x >> 5) * RPW;
  for (int64_t rb = row0 + (int64_t)blockIdx.x * rows_per_block; rb < nrows;
       rb += (int64_t)gridDim.x * rows_per_block) {
    const int64_t r = rb + (int64_t)wib * RPW + sub;
    int32_t b = 0, len = 0, p0 = 0, nnz = 0;
    if (row_lane && r < nrows) {
      b = inc_ptr[r];
      len = stiff ? inc_ptr[r + 1] - b : 0;
      p0 = indptr[r];
      nnz = indptr[r + 1] - p0;
    }
    for (int k = h; k < nnz; k += LPR) acc[k] = 0.0;
    int maxlen = len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
    __syncwarp();
    for (int q0 = 0; q0 < maxlen; q0 += U) {
      double2 v[U];
      double kv[U];
      uint32_t s[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = q0 + u;
        s[u] = 0xFFFFFFFFu;
        v[u] = make_double2(0.0, 0.0);
        kv[u] = 1.0;
        if (q < len) {
          const int64_t at = ((int64_t)b + q) * NU + 2 * h;
          s[u] = __ldg(reinterpret_cast<const uint32_t*>(slot + at));
          v[u] = __ldg(reinterpret_cast<const double2*>(stiff + at));
          if (field) kv[u] = __ldg(field + (int64_t)((uint32_t)__ldg(inc + b + q) / NU) * fstride);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t s0 = s[u] & 0xFFFFu, s1 = s[u] >> 16;
        if (s0 != 0xFFFFu) acc[s0] = __fma_rn(kv[u], v[u].x, acc[s0]);
        if (s1 != 0xFFFFu) acc[s1] = __fma_rn(kv[u], v[u].y, acc[s1]);
        __syncwarp();
      }
    }
    for (int k = h; k < nnz; k += LPR) {
      double a = dscale * acc[k];
      if (mass1) a = __fma_rn(mscale, __ldg(mass1 + p0 + k), a);
      vals[p0 + k] = a;
    }
    __syncwarp();
  }
}

// ------------------------------------------------ one-pass P1 assembly
// Assembly of a scalar P1 simplex form  k_e * dot(grad u, grad v) + m * u v
// in one pass over the CSR rows, from the basis's per-cell geometry cache
// (geo[g * nelems + e]: the Gram entries of the barycentric gradients scaled
// by 1/(d! |det|), row-major upper, then |det| -- what CellBasis keeps of
// its mapping, cell_basis.py:101-105).  Every call contracts the form per
// cell row as it sums: for CSR row r and each incidence entry (cell e, local
// row il) in ascending order, local column j adds
//   stiffness  k_e * G_e[il][j]                  -> acc_k[slot], one DFMA
//   mass       |det_e| (twice on the diagonal)  -> acc_m[slot]
// and the entry is  kscale * acc_k + m * c_P1 * acc_m  (c_P1 the P1 mass
// integral per unit |det| off the diagonal, 1/((d+1)(d+2) d!)).
//
// With a constant mass coefficient (MFIELD false) acc_m is an exact int64
// fixed-point sum of |det_e|: each row has its own binary point
// (mbase[r], from the largest |det| among the row's cells, with shmax bits
// of headroom for the row's entries), so the row's mass sums are exact and
// rounded once when converted back -- order-independent, and FP64-free in
// the loop (GB300's FP64 pipe runs 1/58 of its FP32 rate; the integer pipes
// take the mass term).  With a per-cell mass field, acc_m sums m_e |det_e|
// in FP64 in the same fixed order.
//
// Two lanes per row, lane h taking columns 2h and 2h+1 (TriP1: lane 1 only
// column 2), 16 rows per warp, U entries' loads in flight; entries are
// added in ascending (cell, local row) order (__syncwarp between them), so
// every call gives the same bits.  The local entries are the two-pass
// kernels' up to rounding: k_e G and |det| c are combined per CSR entry
// instead of per cell (within 1e-14 of max|K|, tested).
__device__ __forceinline__ long long fixed_of(double x, int base) {
  const unsigned long long bits = dbits(x);            // x > 0, normal
  const int ex = (int)(bits >> 52);
  const unsigned long long man = (bits & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  const int sh = ex - base;
  return sh >= 0 ? (long long)(man << sh) : (long long)(man >> min(-sh, 63));
}

// x == 0.0 of either sign, on the integer pipes.
__device__ __forceinline__ bool fem_zero(double x) { return (dbits(x) << 1) == 0ull; }

// Packed symmetric index of Gram entry (a, b) (row-major upper triangle).
__host__ __device__ constexpr int gram_index(int nu, int a, int b) {
  return a <= b ? a * (2 * nu + 1 - a) / 2 + b - a : b * (2 * nu + 1 - b) / 2 + a - b;
}

// Bit k set when Gram entry k is a diagonal one (gram_index(nu, a, a)).
template <int NU>
constexpr uint32_t gram_diag_mask() {
  uint32_t m = 0;
  for (int a = 0; a < NU; ++a) m |= 1u << gram_index(NU, a, a);
  return m;
}
template <int NU>
constexpr uint32_t kGramDiag = gram_diag_mask<NU>();

template <int NU, int U, bool MFIELD>
__global__ void __launch_bounds__(128) csr_geometry_p1_kernel(
    const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
    const uint16_t* __restrict__ slot, const int32_t* __restrict__ indptr,
    const double* __restrict__ geo, int64_t nelems, const double* __restrict__ kfield,
    int64_t kstride, double kscale, const double* __restrict__ mfield, int64_t mstride,
    double mscale, double moff, const int16_t* __restrict__ mbase, int64_t row0, int64_t nrows,
    int stride, double* __restrict__ vals) {
  constexpr int NG = NU * (NU + 1) / 2;    // Gram entries; geo[NG] is |det|
  constexpr int RPW = 16;
  using MAcc = typename std::conditional<MFIELD, double, long long>::type;
  extern __shared__ double acc_smem[];
  const int lane = threadIdx.x & 31;
  const int sub = lane >> 1;
  const int h = lane & 1;
  const int wib = threadIdx.x >> 5;
  double* acck = acc_smem + ((size_t)wib * RPW + sub) * stride;
  MAcc* accm = reinterpret_cast<MAcc*>(acc_smem + (size_t)(blockDim.x >> 5) * RPW * stride) +
               ((size_t)wib * RPW + sub) * stride;
  const int j0 = 2 * h, j1 = 2 * h + 1;
  const bool has1 = j1 < NU;
  // this lane's Gram arrays for local rows l = 0 .. NU-1, 4 bits each
  uint32_t tab0 = 0, tab1 = 0;
#pragma unroll
  for (int l = 0; l < NU; ++l) {
    tab0 |= (uint32_t)gram_index(NU, l, j0) << (4 * l);
    if (has1) tab1 |= (uint32_t)gram_index(NU, l, j1) << (4 * l);
  }
  const double* __restrict__ adet_arr = geo + (int64_t)NG * nelems;
  const int64_t rows_per_block = (int64_t)(blockDim.x >> 5) * RPW;
  for (int64_t rb = row0 + (int64_t)blockIdx.x * rows_per_block; rb < nrows;
       rb += (int64_t)gridDim.x * rows_per_block) {
    const int64_t r = rb + (int64_t)wib * RPW + sub;
    int32_t b = 0, len = 0, p0 = 0, nnz = 0, base = 0;
    if (r < nrows) {
      b = inc_ptr[r];
      len = inc_ptr[r + 1] - b;
      p0 = indptr[r];
      nnz = indptr[r + 1] - p0;
      if (!MFIELD) base = mbase[r];
    }
    for (int k = h; k < nnz; k += 2) {
      acck[k] = 0.0;
      accm[k] = (MAcc)0;
    }
    int maxlen = len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
    __syncwarp();
    // the incidence codes of the next U entries are loaded one batch ahead,
    // so that each batch waits for one round of gathers, not two
    uint32_t cnext[U];
#pragma unroll
    for (int u = 0; u < U; ++u) cnext[u] = u < len ? (uint32_t)__ldg(inc + b + u) : 0u;
    for (int q0 = 0; q0 < maxlen; q0 += U) {
      uint32_t code[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        code[u] = cnext[u];
        const int qn = q0 + U + u;
        cnext[u] = qn < len ? (uint32_t)__ldg(inc + b + qn) : 0u;
      }
      double kv[U], g0[U], g1[U];
      MAcc mv[U];
      uint32_t sp[U];
      int il[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = q0 + u;
        sp[u] = 0xFFFFFFFFu;
        kv[u] = 0.0;
        g0[u] = 0.0;
        g1[u] = 0.0;
        mv[u] = (MAcc)0;
        il[u] = -1;
        if (q < len) {
          const uint32_t e = NU == 4 ? (code[u] >> 2) : (__umulhi(code[u], 0xAAAAAAABu) >> 1);
          const int l = (int)(code[u] - e * NU);
          il[u] = l;
          const uint16_t* sq = slot + ((int64_t)b + q) * NU;
          if constexpr (NU % 2 == 0) {
            sp[u] = __ldg(reinterpret_cast<const uint32_t*>(sq + j0));
          } else {
            sp[u] = (uint32_t)__ldg(sq + j0) | (has1 ? (uint32_t)__ldg(sq + j1) << 16 : 0xFFFF0000u);
          }
          kv[u] = kfield ? __ldg(kfield + (int64_t)e * kstride) : 1.0;
          g0[u] = __ldg(geo + (int64_t)((tab0 >> (4 * l)) & 15u) * nelems + e);
          if (has1) g1[u] = __ldg(geo + (int64_t)((tab1 >> (4 * l)) & 15u) * nelems + e);
          const double adet = __ldg(adet_arr + e);
          if constexpr (MFIELD) mv[u] = __ldg(mfield + (int64_t)e * mstride) * adet;
          else mv[u] = fixed_of(adet, base);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t s0 = sp[u] & 0xFFFFu, s1 = sp[u] >> 16;
        if (s0 != 0xFFFFu) {
          acck[s0] = __fma_rn(kv[u], g0[u], acck[s0]);
          accm[s0] += il[u] == j0 ? mv[u] + mv[u] : mv[u];
        }
        if (s1 != 0xFFFFu) {
          acck[s1] = __fma_rn(kv[u], g1[u], acck[s1]);
          accm[s1] += il[u] == j1 ? mv[u] + mv[u] : mv[u];
        }
        __syncwarp();
      }
    }
    double mc;
    if constexpr (MFIELD) {
      mc = moff;
    } else {
      // 2^(base - 1075): the value of one unit of the row's fixed point
      const double unit = dfrombits((unsigned long long)(base - 1075 + 1023) << 52);
      mc = (mscale * moff) * unit;
    }
    for (int k = h; k < nnz; k += 2) {
      const double m = MFIELD ? (double)accm[k] : __ll2double_rn((long long)accm[k]);
      vals[p0 + k] = __fma_rn(mc, m, kscale * acck[k]);
    }
    __syncwarp();
  }
}

// ------------------------------------------ one-pass P1, upper gather form
// The same assembly as csr_geometry_p1_kernel with one lane per CSR entry
// on or above the diagonal (an "upper entry" (i, j), j >= i) instead of
// two lanes per row: the lane walks the entry's contribution list -- every
// (cell e, local pair (li, lj)) with dof(li) = i, dof(lj) = j whose local
// entry is not an exact zero, in ascending (e, li) order, the order in
// which the row kernel adds them into the slot -- accumulating
//   acc_k = fma(k_e, G_e[li][lj], acc_k)      (FP64, in registers)
//   acc_m += |det_e| (twice on the diagonal)  (exact fixed point / FP64)
// and writes the entry to (i, j) and, off the diagonal, to (j, i): the
// symmetric forms' local matrices are symmetric bit for bit
// (G_e[li][lj] is one cached number), so the two positions receive the
// same additions in the same order.  Each cell's 10 (TetP1) or 6 (TriP1)
// Gram entries are read and multiplied once, and there is no shared-memory
// accumulation or warp barrier: every lane's sum lives in its registers.
// The values equal csr_geometry_p1_kernel's bit for bit.
//
// Lists are stored sliced: 32 consecutive upper entries form a slice of
// len = the longest list among them; code p of the slice's lane l sits at
// codes[(base + p) * 32 + l] (coalesced), padded with 0xFFFFFFFF.  A code
// is e * 16 + k, k the Gram entry gram_index(li, lj) of the cell's local
// pair (diagonal ones flagged by kGramDiag).  Upper entries are numbered diagonal entries
// first (by row), then the others by (row, column), so list lengths within
// a slice are alike (a vertex's cells vs an edge's cells).
// TMA (bulk-copy engine) helpers for the staged form below.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// One bulk copy of `bytes` (a multiple of 16, both ends 16-byte aligned)
// from global memory into this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes,
                                            uint64_t* bar) {
  unsigned long long state;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(state) : "r"(smem_addr(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
  (void)state;
}
// Bounded wait for the phase `parity` of `bar`; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// One slice of upper entries: lane `lane` walks codes cp[p * 32], p < len.
// CHECK (a per-cell stiffness field of stride 1, a nonzero constant mass):
// the coefficient checks ride along -- at each cell's contribution of Gram
// entry 0 (its local diagonal (0, 0), which the mass keeps in every list)
// the cell's zero bits, const_bits | (k_e == 0), are compared with the
// pattern's ref_bits[e]; a difference sets FEM_ERR_STALE_PATTERN in *stale.
template <int NU, int U, bool MFIELD, bool SMEM, bool CHECK = false>
__device__ __forceinline__ void upper_slice(
    const uint32_t* __restrict__ cp, int len, int64_t u, bool live,
    const int32_t* __restrict__ pos, const int32_t* __restrict__ tpos,
    const int32_t* __restrict__ urow, const double* __restrict__ geo, int64_t nelems,
    const double* __restrict__ kfield, int64_t kstride, double kscale,
    const double* __restrict__ mfield, int64_t mstride, double mscale, double moff,
    const int16_t* __restrict__ mbase, double* __restrict__ vals,
    const uint8_t* __restrict__ ref_bits = nullptr, int const_bits = 0,
    int32_t* stale = nullptr) {
  constexpr int NG = NU * (NU + 1) / 2;
  using MAcc = typename std::conditional<MFIELD, double, long long>::type;
  const double* __restrict__ adet_arr = geo + (int64_t)NG * nelems;
  auto code_at = [&](int p) -> uint32_t {
    if constexpr (SMEM) return cp[p * 32];
    else return __ldg(cp + (int64_t)p * 32);
  };
  int mb = 0;
  if (!MFIELD && live) mb = mbase[urow[u]];
  double acck = 0.0;
  MAcc accm = (MAcc)0;
  uint32_t cn[U];
#pragma unroll
  for (int v = 0; v < U; ++v) cn[v] = v < len ? code_at(v) : 0xFFFFFFFFu;
  for (int p0 = 0; p0 < len; p0 += U) {
    uint32_t c[U];
#pragma unroll
    for (int v = 0; v < U; ++v) {
      c[v] = cn[v];
      const int pn = p0 + U + v;
      cn[v] = pn < len ? code_at(pn) : 0xFFFFFFFFu;
    }
    double kv[U], g[U];
    MAcc mv[U];
#pragma unroll
    for (int v = 0; v < U; ++v) {
      kv[v] = 0.0;
      g[v] = 0.0;
      mv[v] = (MAcc)0;
      if (live && c[v] != 0xFFFFFFFFu) {
        const uint32_t e = c[v] >> 4;
        const int gk = (int)(c[v] & 15u);        // the pair's Gram entry
        const bool diag = (kGramDiag<NU> >> gk) & 1u;
        kv[v] = kfield ? __ldg(kfield + (int64_t)e * kstride) : 1.0;
        g[v] = __ldg(geo + (int64_t)gk * nelems + e);
        if constexpr (CHECK) {
          if (gk == 0) {
            const int bits = const_bits | (fem_zero(kv[v]) ? 1 : 0);
            if (bits != (int)__ldg(ref_bits + e)) *stale = 1 << FEM_ERR_STALE_PATTERN;
          }
        }
        const double adet = __ldg(adet_arr + e);
        MAcc m;
        if constexpr (MFIELD) m = __ldg(mfield + (int64_t)e * mstride) * adet;
        else m = fixed_of(adet, mb);
        mv[v] = diag ? m + m : m;
      }
    }
#pragma unroll
    for (int v = 0; v < U; ++v) {
      acck = __fma_rn(kv[v], g[v], acck);
      accm += mv[v];
    }
  }
  if (live) {
    double mc;
    if constexpr (MFIELD) {
      mc = moff;
    } else {
      // mcoef * 2^(mb - 1075) (mcoef = mscale * moff): a power-of-two scaling,
      // done on the exponent field (integer pipes) while the result stays
      // normal -- the same value as the FP64 product
      const double mcoef = mscale * moff;
      const unsigned long long cb = dbits(mcoef);
      const int sh = mb - 1075;
      const int ex = (int)((cb >> 52) & 0x7ffu) + sh;
      if (ex >= 1 && ex <= 2046 && ((cb >> 52) & 0x7ffu) != 0u)
        mc = dfrombits(cb + ((unsigned long long)(long long)sh << 52));
      else
        mc = mcoef * dfrombits((unsigned long long)(sh + 1023) << 52);
    }
    const double m = MFIELD ? (double)accm : __ll2double_rn((long long)accm);
    if (kscale != 1.0) acck = kscale * acck;
    const double val = __fma_rn(mc, m, acck);
    vals[pos[u]] = val;
    const int32_t t = tpos[u];
    if (t >= 0) vals[t] = val;
  }
}

template <int NU, int U, bool MFIELD, bool CHECK = false>
__global__ void __launch_bounds__(128) csr_upper_p1_kernel(
    int64_t ua, int64_t ub, const int32_t* __restrict__ slice_len,
    const int32_t* __restrict__ slice_base, const uint32_t* __restrict__ codes,
    const int32_t* __restrict__ pos, const int32_t* __restrict__ tpos,
    const int32_t* __restrict__ urow, const double* __restrict__ geo, int64_t nelems,
    const double* __restrict__ kfield, int64_t kstride, double kscale,
    const double* __restrict__ mfield, int64_t mstride, double mscale, double moff,
    const int16_t* __restrict__ mbase, double* __restrict__ vals,
    const uint8_t* __restrict__ ref_bits = nullptr, int const_bits = 0,
    int32_t* __restrict__ status = nullptr) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t s0 = ua >> 5, s1 = (ub + 31) >> 5;
  int32_t stale = 0;
  for (int64_t sl = s0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); sl < s1;
       sl += warps) {
    const int64_t u = sl * 32 + lane;
    upper_slice<NU, U, MFIELD, false, CHECK>(
        codes + (int64_t)slice_base[sl] * 32 + lane, slice_len[sl], u, u >= ua && u < ub, pos,
        tpos, urow, geo, nelems, kfield, kstride, kscale, mfield, mstride, mscale, moff, mbase,
        vals, ref_bits, const_bits, &stale);
  }
  if constexpr (CHECK) fem::publish_status(status, stale);
}

// The same sum with each warp's slice codes staged in shared memory by the
// TMA bulk-copy engine: lane 0 of the warp issues one cp.async.bulk of the
// next slice's codes (len x 128 bytes, contiguous) while the warp works on
// the current one, double-buffered on two mbarriers, so the lanes read their
// codes from shared memory and only the geometry gathers go to L2 / HBM.
// cap: the longest slice (codes per lane) the buffers hold.  Every wait is
// bounded; past the limit the warp sets FEM_ERR_TIMEOUT in *status and
// stops, after a second bounded wait for its copies in flight.
template <int NU, int U, bool MFIELD>
__global__ void __launch_bounds__(128) csr_upper_p1_tma_kernel(
    int64_t ua, int64_t ub, const int32_t* __restrict__ slice_len,
    const int32_t* __restrict__ slice_base, const uint32_t* __restrict__ codes, int cap,
    const int32_t* __restrict__ pos, const int32_t* __restrict__ tpos,
    const int32_t* __restrict__ urow, const double* __restrict__ geo, int64_t nelems,
    const double* __restrict__ kfield, int64_t kstride, double kscale,
    const double* __restrict__ mfield, int64_t mstride, double mscale, double moff,
    const int16_t* __restrict__ mbase, double* __restrict__ vals, int32_t* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  constexpr long long kWaitLimit = 1ll << 24;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  uint32_t* const buf0 = reinterpret_cast<uint32_t*>(tma_smem) + (size_t)wib * 2 * cap * 32;
  uint32_t* const buf1 = buf0 + (size_t)cap * 32;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tma_smem + (size_t)nw * 2 * cap * 32 * 4) + wib * 2;
  if (lane == 0) {
    mbar_init(bar);
    mbar_init(bar + 1);
    mbar_init_fence();
  }
  __syncwarp();
  const int64_t warps = (int64_t)gridDim.x * nw;
  const int64_t s0 = ua >> 5, s1 = (ub + 31) >> 5;
  int64_t sl = s0 + (int64_t)blockIdx.x * nw + wib;
  uint32_t ph0 = 0u, ph1 = 0u;    // the phase each buffer's barrier waits for next
  auto issue = [&](int64_t s, int k) {
    if (s < s1 && lane == 0) {
      const int len = slice_len[s];
      if (len > 0)
        tma_load_1d(k ? buf1 : buf0, codes + (int64_t)slice_base[s] * 32, (uint32_t)len * 128u,
                    bar + k);
    }
  };
  issue(sl, 0);
  int k = 0;
  while (sl < s1) {
    const int64_t next = sl + warps;
    issue(next, k ^ 1);          // that buffer was released by the __syncwarp below
    const int len = slice_len[sl];
    if (len > 0) {
      const uint32_t ph = k ? ph1 : ph0;
      if (!mbar_wait(bar + k, ph, kWaitLimit)) {
        if (lane == 0 && status) atomicOr(status, 1 << FEM_ERR_TIMEOUT);
        // the copies still in flight must land before the block exits
        mbar_wait(bar + k, ph, kWaitLimit);
        if (next < s1 && slice_len[next] > 0)
          mbar_wait(bar + (k ^ 1), k ? ph0 : ph1, kWaitLimit);
        return;
      }
      if (k) ph1 ^= 1u;
      else ph0 ^= 1u;
    }
    const int64_t u = sl * 32 + lane;
    upper_slice<NU, U, MFIELD, true>((k ? buf1 : buf0) + lane, len, u, u >= ua && u < ub, pos,
                                     tpos, urow, geo, nelems, kfield, kstride, kscale, mfield,
                                     mstride, mscale, moff, mbase, vals);
    __syncwarp();
    sl = next;
    k ^= 1;
  }
}

// Upper-entry numbering of a square pattern, one thread per row: the
// offset of the diagonal (or of the first column above it) in row i, and
// whether the diagonal is present; then the number of upper entries.
// Slot of row i's upper entries: its diagonal (k < 0) or its k-th entry
// above the diagonal.  block_rows == 0: every diagonal entry first (by row),
// then the others by (row, column).  block_rows > 0: the rows in blocks of
// block_rows, each block's diagonal entries, then its other entries -- the
// entries of neighbouring rows, diagonal or not, are summed at about the
// same time, so each cell's geometry is read about once.
__device__ __forceinline__ int64_t upper_slot(const int32_t* __restrict__ dpos,
                                              const int32_t* __restrict__ opos, int64_t nd,
                                              int64_t nrows, int64_t block_rows, int64_t i,
                                              int k) {
  if (block_rows <= 0) return k < 0 ? (int64_t)dpos[i] : nd + opos[i] + k;
  const int64_t b0 = i / block_rows * block_rows;
  const int64_t b1 = b0 + block_rows < nrows ? b0 + block_rows : nrows;
  const int64_t start = (int64_t)dpos[b0] + opos[b0];
  if (k < 0) return start + (dpos[i] - dpos[b0]);
  return start + (dpos[b1] - dpos[b0]) + (opos[i] - opos[b0]) + k;
}

__global__ void upper_count_kernel(const int32_t* __restrict__ indptr,
                                   const int32_t* __restrict__ indices, int64_t nrows,
                                   int32_t* __restrict__ ndiag, int32_t* __restrict__ noff) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  const int32_t p0 = indptr[i], p1 = indptr[i + 1];
  int lo = p0, hi = p1;                     // first column >= i
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (indices[mid] < i) lo = mid + 1;
    else hi = mid;
  }
  const bool d = lo < p1 && indices[lo] == i;
  ndiag[i] = d ? 1 : 0;
  noff[i] = p1 - lo - (d ? 1 : 0);
}

// Per row i: pos / tpos / row of its upper entries, and the length of each
// entry's contribution list (cnt, indexed by upper entry).
__global__ void upper_fill_kernel(const int32_t* __restrict__ indptr,
                                  const int32_t* __restrict__ indices,
                                  const int32_t* __restrict__ inc_ptr,
                                  const int32_t* __restrict__ inc,
                                  const uint16_t* __restrict__ slot, int nu, int64_t nrows,
                                  const int32_t* __restrict__ dpos, const int32_t* __restrict__ opos,
                                  int64_t nd, int64_t block_rows, int32_t* __restrict__ pos,
                                  int32_t* __restrict__ tpos,
                                  int32_t* __restrict__ urow, int32_t* __restrict__ cnt,
                                  int32_t* __restrict__ asym) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  const int32_t p0 = indptr[i], p1 = indptr[i + 1];
  int lo = p0, hi = p1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (indices[mid] < i) lo = mid + 1;
    else hi = mid;
  }
  const bool d = lo < p1 && indices[lo] == i;
  const int sd = lo - p0;                   // offset of the diagonal / first upper column
  const int so = sd + (d ? 1 : 0);          // offset of the first column above the diagonal
  if (d) {
    const int64_t u = upper_slot(dpos, opos, nd, nrows, block_rows, i, -1);
    pos[u] = lo;
    tpos[u] = -1;
    urow[u] = (int32_t)i;
    cnt[u] = 0;
  }
  for (int s = so; s < p1 - p0; ++s) {
    const int64_t u = upper_slot(dpos, opos, nd, nrows, block_rows, i, s - so);
    const int32_t j = indices[p0 + s];
    pos[u] = p0 + s;
    // (j, i) in row j: i < j is among its columns (the pattern is symmetric)
    int a = indptr[j], z = indptr[j + 1];
    while (a < z) {
      const int mid = (a + z) >> 1;
      if (indices[mid] < i) a = mid + 1;
      else z = mid;
    }
    const bool found = a < indptr[j + 1] && indices[a] == i;
    tpos[u] = found ? a : -1;
    if (!found) atomicOr(asym, 1);      // not a symmetric pattern: no upper form
    urow[u] = (int32_t)i;
    cnt[u] = 0;
  }
  const int32_t b = inc_ptr[i], len = inc_ptr[i + 1] - b;
  for (int q = 0; q < len; ++q)
    for (int j = 0; j < nu; ++j) {
      const uint16_t sv = slot[((int64_t)b + q) * nu + j];
      if (sv == 0xFFFF || (int)sv < sd) continue;
      const int64_t u = upper_slot(dpos, opos, nd, nrows, block_rows, i,
                                   ((int)sv == sd && d) ? -1 : (int)sv - so);
      cnt[u] += 1;
    }
}

// slice_len[sl] = longest list among the slice's 32 entries
__global__ void upper_slice_len_kernel(const int32_t* __restrict__ cnt, int64_t nupper,
                                       int64_t nslices, int32_t* __restrict__ slice_len) {
  const int64_t sl = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sl >= nslices) return;
  const int64_t u = sl * 32 + lane;
  int v = u < nupper ? cnt[u] : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) slice_len[sl] = v;
}

// Codes of every list, in ascending (cell, local row) order: one thread per
// row walks the row's incidence (ascending) and appends to its entries.
__global__ void upper_codes_kernel(const int32_t* __restrict__ indptr,
                                   const int32_t* __restrict__ indices,
                                   const int32_t* __restrict__ inc_ptr,
                                   const int32_t* __restrict__ inc,
                                   const uint16_t* __restrict__ slot, int nu, int64_t nrows,
                                   const int32_t* __restrict__ dpos,
                                   const int32_t* __restrict__ opos, int64_t nd,
                                   int64_t block_rows,
                                   const int32_t* __restrict__ slice_base,
                                   int32_t* __restrict__ cursor, uint32_t* __restrict__ codes,
                                   bool wide) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  const int32_t p0 = indptr[i], p1 = indptr[i + 1];
  int lo = p0, hi = p1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (indices[mid] < i) lo = mid + 1;
    else hi = mid;
  }
  const bool d = lo < p1 && indices[lo] == i;
  const int sd = lo - p0, so = sd + (d ? 1 : 0);
  const int32_t b = inc_ptr[i], len = inc_ptr[i + 1] - b;
  for (int q = 0; q < len; ++q) {
    const uint32_t code = (uint32_t)inc[b + q];
    const uint32_t e = code / (uint32_t)nu;
    const uint32_t li = code - e * (uint32_t)nu;
    for (int j = 0; j < nu; ++j) {
      const uint16_t sv = slot[((int64_t)b + q) * nu + j];
      if (sv == 0xFFFF || (int)sv < sd) continue;
      const int64_t u = upper_slot(dpos, opos, nd, nrows, block_rows, i,
                                   ((int)sv == sd && d) ? -1 : (int)sv - so);
      const int c = cursor[u]++;
      codes[((int64_t)slice_base[u >> 5] + c) * 32 + (u & 31)] =
          wide ? (e << 7) | (li * (uint32_t)nu + (uint32_t)j)
               : (e << 4) | (uint32_t)gram_index(nu, (int)li, j);
    }
  }
}

// mbase[r] = (largest exponent field of |det_e| over the cells of row r)
// - shmax, the binary point of row r's fixed-point mass sums; *minexp the
// smallest exponent field of any |det| (0: a degenerate cell), *maxexp the
// largest (2047: inf / nan) -- the host then leaves the fixed-point path.
__global__ void row_mass_base_kernel(const int32_t* __restrict__ inc_ptr,
                                     const int32_t* __restrict__ inc, int64_t nrows, int nu,
                                     const double* __restrict__ adet, int shmax,
                                     int16_t* __restrict__ mbase, int32_t* __restrict__ ext) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t b = inc_ptr[r], n = inc_ptr[r + 1] - b;
  int emax = 0, emin = 2047;
  for (int q = 0; q < n; ++q) {
    const uint32_t e = (uint32_t)inc[b + q] / (uint32_t)nu;
    const int ex = (int)((dbits(adet[e]) >> 52) & 0x7FF);
    emax = max(emax, ex);
    emin = min(emin, ex);
  }
  mbase[r] = (int16_t)(n > 0 ? emax - shmax : 1075);
  if (n > 0) {
    atomicMin(ext, emin);
    atomicMax(ext + 1, emax);
  }
}

// out[q * nu + j] = local[inc[q] * nu + j]: element-major local rows
// gathered into incidence order.
__global__ void incidence_rows_kernel(const int32_t* __restrict__ inc, int64_t ninc, int nu,
                                      const double* __restrict__ local, double* __restrict__ out) {
  const int64_t n = ninc * nu;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = idx / nu;
    const int j = (int)(idx - q * nu);
    out[idx] = local[(int64_t)__ldg(inc + q) * nu + j];
  }
}

__global__ void vector_sum_kernel(const int32_t* __restrict__ inc_ptr, const int32_t* __restrict__ inc,
                                  const double* __restrict__ local, int64_t nrows,
                                  double* __restrict__ b) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t p0 = inc_ptr[r], p1 = inc_ptr[r + 1];
  double s = 0.0;
  for (int32_t q = p0; q < p1; ++q) s += local[inc[q]];
  b[r] = s;
}

int grid_for(int64_t n, int block) {
  const int64_t g = ceil_div(n, block);
  const int64_t cap = (int64_t)num_sms() * 32;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

}  // namespace

// ----------------------------------------------------------------- scan
// Exclusive scan, 1024 int32 per block (warp shuffles + one shared pass),
// block totals scanned recursively, then added back.
namespace {
constexpr int kScanBlock = 1024;

__global__ void scan_blocks_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out,
                                   int64_t n, int32_t* __restrict__ sums) {
  __shared__ int32_t wsum[32];
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t v = i < n ? in[i] : 0;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    wsum[lane] = s;
  }
  __syncthreads();
  const int32_t incl = x + (w > 0 ? wsum[w - 1] : 0);
  if (i < n) out[i] = incl - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = incl;
}

__global__ void scan_add_kernel(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ offs) {
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

int scan_rec(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st) {
  const int64_t nb = ceil_div(n, kScanBlock);
  AsyncScratch scratch(st);
  int32_t *sums = nullptr, *offs = nullptr;
  FEM_TRY_CUDA(scratch.alloc(&sums, nb * sizeof(int32_t)));
  FEM_TRY_CUDA(scratch.alloc(&offs, nb * sizeof(int32_t)));
  scan_blocks_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(in, out, n, sums);
  FEM_LAUNCH_CHECK("scan_blocks_kernel");
  if (nb > 1) {
    int rc = scan_rec(sums, offs, nb, st);
    if (rc) return rc;
    scan_add_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(out, n, offs);
    FEM_LAUNCH_CHECK("scan_add_kernel");
  }
  return 0;
}

// 64-bit total of n nonnegative int32 counts (one atomic per block), so that
// a total beyond int32 is reported instead of wrapping in the scan.
__global__ void count_total_kernel(const int32_t* __restrict__ in, int64_t n,
                                   unsigned long long* __restrict__ total) {
  unsigned long long s = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += (unsigned long long)(uint32_t)max(in[i], 0);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ unsigned long long ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += ws[w];
    atomicAdd(total, b);
  }
}
}  // namespace

int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int64_t* total,
                       cudaStream_t stream) {
  // out[0..n]: out[k] = sum(in[0..k)); out[n] = total.  `in` must hold n+1
  // entries with in[n] == 0 (callers allocate counts with one spare slot).
  // A total beyond INT32_MAX (the int32 offsets of the reference's CSR)
  // returns FEM_ERR_CAPACITY before any offset is written.
  if (n + 1 > INT32_MAX) {
    set_error(FEM_ERR_CAPACITY, "scan of %lld entries exceeds int32", (long long)n);
    return FEM_ERR_CAPACITY;
  }
  {
    AsyncScratch scratch(stream);
    unsigned long long* dtot = nullptr;
    FEM_TRY_CUDA(scratch.alloc(&dtot, sizeof(unsigned long long)));
    FEM_TRY_CUDA(cudaMemsetAsync(dtot, 0, sizeof(unsigned long long), stream));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256),
                                                                (int64_t)num_sms() * 8));
    count_total_kernel<<<grid, 256, 0, stream>>>(in, n, dtot);
    FEM_LAUNCH_CHECK("count_total_kernel");
    unsigned long long t64 = 0;
    FEM_TRY_CUDA(cudaMemcpyAsync(&t64, dtot, sizeof(t64), cudaMemcpyDeviceToHost, stream));
    FEM_TRY_CUDA(cudaStreamSynchronize(stream));
    if (t64 > (unsigned long long)INT32_MAX) {
      set_error(FEM_ERR_CAPACITY, "total of %llu entries exceeds the int32 offsets of the CSR",
                t64);
      return FEM_ERR_CAPACITY;
    }
  }
  int rc = scan_rec(in, out, n + 1, stream);
  if (rc) return rc;
  if (total) {
    int32_t t = 0;
    FEM_TRY_CUDA(cudaMemcpyAsync(&t, out + n, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    FEM_TRY_CUDA(cudaStreamSynchronize(stream));
    *total = t;
  }
  return 0;
}

// Build row incidence of `dofs` (nb, nelems) over nrows rows.
int build_incidence(const int32_t* dofs, int64_t nelems, int nb, int64_t nrows, Pattern* P,
                    cudaStream_t st) {
  P->nrows = nrows;
  P->nelems = nelems;
  P->nbfun_v = nb;
  P->ninc = nelems * nb;
  if (P->ninc >= INT32_MAX) {
    set_error(FEM_ERR_CAPACITY, "nelems * nbfun = %lld exceeds int32 incidence codes",
              (long long)P->ninc);
    return FEM_ERR_CAPACITY;
  }
  // scratch released on every return; the pattern's own arrays are
  // released by the caller's free_pattern on failure
  AsyncScratch scratch(st);
  int32_t *cnt = nullptr, *cursor = nullptr, *flags = nullptr;
  FEM_TRY_CUDA(cudaMallocAsync(&P->inc_ptr, (nrows + 1) * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMallocAsync(&P->inc, std::max<int64_t>(1, P->ninc) * sizeof(int32_t), st));
  FEM_TRY_CUDA(scratch.alloc(&cnt, (nrows + 1) * sizeof(int32_t)));
  FEM_TRY_CUDA(scratch.alloc(&cursor, (nrows + 1) * sizeof(int32_t)));
  FEM_TRY_CUDA(scratch.alloc(&flags, 2 * sizeof(int32_t)));
  FEM_TRY_CUDA(cudaMemsetAsync(cnt, 0, (nrows + 1) * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(cursor, 0, (nrows + 1) * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int32_t), st));
  if (P->ninc > 0) {
    count_rows_kernel<<<grid_for(P->ninc, 256), 256, 0, st>>>(dofs, nelems, nb, nrows, cnt, flags);
    FEM_LAUNCH_CHECK("count_rows_kernel");
  }
  int64_t total = 0;
  int rc = exclusive_scan_i32(cnt, P->inc_ptr, nrows, &total, st);
  if (rc) return rc;
  if (P->ninc > 0) {
    fill_rows_kernel<<<grid_for(P->ninc, 256), 256, 0, st>>>(dofs, nelems, nb, nrows, P->inc_ptr,
                                                             cursor, P->inc);
    FEM_LAUNCH_CHECK("fill_rows_kernel");
  }
  if (nrows > 0) {
    sort_segments_kernel<<<(unsigned)ceil_div(nrows, 128), 128, 0, st>>>(P->inc_ptr, nrows, P->inc,
                                                                        flags + 1);
    FEM_LAUNCH_CHECK("sort_segments_kernel");
  }
  int32_t h[2] = {0, 0};
  FEM_TRY_CUDA(cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, st));
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  if (h[0]) {
    set_error(FEM_ERR_ARGUMENT, "element_dofs holds an index outside [0, %lld)", (long long)nrows);
    return FEM_ERR_ARGUMENT;
  }
  if (total != P->ninc) {
    set_error(FEM_ERR_ARGUMENT, "incidence count mismatch (%lld vs %lld)", (long long)total,
              (long long)P->ninc);
    return FEM_ERR_ARGUMENT;
  }
  P->max_row_inc = h[1];
  return 0;
}

int build_csr(const int32_t* udofs, int nu, int64_t ncols, const double* local, Pattern* P,
              cudaStream_t st) {
  P->nbfun_u = nu;
  const int nv = P->nbfun_v;
  int cap = 1;
  while (cap < P->max_row_inc * nu) cap <<= 1;
  cap = std::max(cap, 32);
  if (cap > kMaxRowCandidates) {
    set_error(FEM_ERR_CAPACITY,
              "a row gathers %d candidate columns (limit %d): the mesh has a DOF shared by "
              "%d cells", P->max_row_inc * nu, kMaxRowCandidates, P->max_row_inc);
    return FEM_ERR_CAPACITY;
  }
  // a warp sorts its row's candidates in shared memory (2 x cap words)
  const int rwarps = smem_block_warps((size_t)2 * cap * sizeof(int32_t));
  const size_t smem = (size_t)rwarps * 2 * cap * sizeof(int32_t);
  if (smem > 48 * 1024) {
    FEM_TRY_CUDA(cudaFuncSetAttribute(row_nnz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    FEM_TRY_CUDA(cudaFuncSetAttribute(row_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  }
  AsyncScratch scratch(st);
  int32_t *row_nnz = nullptr, *flags = nullptr;
  FEM_TRY_CUDA(scratch.alloc(&row_nnz, (P->nrows + 1) * sizeof(int32_t)));
  FEM_TRY_CUDA(scratch.alloc(&flags, sizeof(int32_t)));
  FEM_TRY_CUDA(cudaMemsetAsync(flags, 0, sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(row_nnz, 0, (P->nrows + 1) * sizeof(int32_t), st));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(P->nrows, rwarps),
                                                              (int64_t)num_sms() * 16));
  if (P->nrows > 0) {
    row_nnz_kernel<<<grid, 32 * rwarps, smem, st>>>(P->inc_ptr, P->inc, udofs, local,
                                                           P->nrows, P->nelems, nv, nu, cap,
                                                           row_nnz, flags);
    FEM_LAUNCH_CHECK("row_nnz_kernel");
  }
  FEM_TRY_CUDA(cudaMallocAsync(&P->indptr, (P->nrows + 1) * sizeof(int32_t), st));
  int64_t nnz = 0;
  int rc = exclusive_scan_i32(row_nnz, P->indptr, P->nrows, &nnz, st);
  if (rc) return rc;
  int32_t maxnnz = 0;
  FEM_TRY_CUDA(cudaMemcpyAsync(&maxnnz, flags, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  if (maxnnz > 0xFFFE) {
    set_error(FEM_ERR_CAPACITY, "a CSR row has %d entries (limit 65534)", maxnnz);
    return FEM_ERR_CAPACITY;
  }
  P->nnz = nnz;
  P->max_row_nnz = maxnnz;
  FEM_TRY_CUDA(cudaMallocAsync(&P->indices, std::max<int64_t>(1, nnz) * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMallocAsync(&P->slot, std::max<int64_t>(1, P->ninc * nu) * sizeof(uint16_t), st));
  if (P->nrows > 0) {
    row_fill_kernel<<<grid, 32 * rwarps, smem, st>>>(P->inc_ptr, P->inc, udofs, local,
                                                            P->nrows, P->nelems, nv, nu, cap,
                                                            P->indptr, P->indices, P->slot);
    FEM_LAUNCH_CHECK("row_fill_kernel");
  }
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  (void)ncols;
  P->has_matrix = true;
  return 0;
}

int csr_sum(const Pattern& P, const double* local, double* vals, cudaStream_t st, int64_t row0,
            int64_t row1, int32_t* check_status, int sym) {
  if (!P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern has no CSR structure (built without local matrices)");
    return FEM_ERR_ARGUMENT;
  }
  if (row1 < 0 || row1 > P.nrows) row1 = P.nrows;
  if (row0 < 0) row0 = 0;
  if (row1 <= row0 || (P.nnz == 0 && !check_status)) return 0;
  const int nu = P.nbfun_u;
  const int stride = std::max(1, P.max_row_nnz);
  int rc = 0;
  auto launch = [&](auto kern, int G) -> int {
    const int rpw = 32 / G;
    const size_t per_warp = (size_t)rpw * stride * (sizeof(double) + (check_status ? 1 : 0));
    const int warps = smem_block_warps(per_warp);
    if (!warps) return row_smem_error(stride);
    const int threads = 32 * warps;
    const size_t smem = warps * per_warp;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return check_cuda(e, "csr_sum smem");
    }
    const int64_t rows_per_block = (int64_t)warps * rpw;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(row1 - row0, rows_per_block),
                                                                (int64_t)num_sms() * 64));
    kern<<<grid, threads, smem, st>>>(P.inc_ptr, P.inc, P.slot, P.indptr, local, row0, row1, nu,
                                      stride, vals, check_status, 0ull);
    return 0;
  };
  const int U = P.sum_unroll;
  auto pick = [&](auto check_tag) -> int {
    constexpr bool C = decltype(check_tag)::value;
    if (nu <= 2) return U >= 16 ? launch(csr_sum_kernel<2, 16, C>, 2) : U >= 8 ? launch(csr_sum_kernel<2, 8, C>, 2) : launch(csr_sum_kernel<2, 4, C>, 2);
    if (nu <= 4) return U >= 16 ? launch(csr_sum_kernel<4, 16, C>, 4) : U >= 8 ? launch(csr_sum_kernel<4, 8, C>, 4) : launch(csr_sum_kernel<4, 4, C>, 4);
    if (nu <= 8) return U >= 16 ? launch(csr_sum_kernel<8, 16, C>, 8) : U >= 8 ? launch(csr_sum_kernel<8, 8, C>, 8) : launch(csr_sum_kernel<8, 4, C>, 8);
    if (nu <= 16) return U >= 8 ? launch(csr_sum_kernel<16, 8, C>, 16) : launch(csr_sum_kernel<16, 4, C>, 16);
    return U >= 8 ? launch(csr_sum_kernel<32, 8, C>, 32) : launch(csr_sum_kernel<32, 4, C>, 32);
  };
  if (nu > 32) {
    set_error(FEM_ERR_UNSUPPORTED, "more than 32 local functions per cell (%d)", nu);
    return FEM_ERR_UNSUPPORTED;
  }
  if (sym > 0) {
    // block-upper staging of vector channel kernels (no zero-structure check)
    if (check_status || (sym != 2 && sym != 3) || P.nbfun_u != P.nbfun_v || nu % sym) {
      set_error(FEM_ERR_ARGUMENT, "block-symmetric staging needs a square pattern, blocks of 2 or 3");
      return FEM_ERR_ARGUMENT;
    }
    const int64_t ncodes = P.nelems * (int64_t)P.nbfun_v;
    if (ncodes >= ((int64_t)1 << 32)) {
      set_error(FEM_ERR_CAPACITY, "%lld incidence codes exceed 2^32", (long long)ncodes);
      return FEM_ERR_CAPACITY;
    }
    const unsigned long long magic = ~0ull / (unsigned long long)nu + 1ull;
    auto launch_sym = [&](auto kern, int G) -> int {
      const int rpw = 32 / G;
      const size_t per_warp = (size_t)rpw * stride * sizeof(double);
      const int warps = smem_block_warps(per_warp);
      if (!warps) return row_smem_error(stride);
      const int threads = 32 * warps;
      const size_t smem = warps * per_warp;
      if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return check_cuda(e, "csr_sum smem");
      }
      const int64_t rows_per_block = (int64_t)warps * rpw;
      const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(row1 - row0, rows_per_block),
                                                                  (int64_t)num_sms() * 64));
      kern<<<grid, threads, smem, st>>>(P.inc_ptr, P.inc, P.slot, P.indptr, local, row0, row1, nu,
                                        stride, vals, nullptr, magic);
      return 0;
    };
#define FEM_SYM_PICK(S)                                                                        \
    if (nu <= 8) rc = U >= 8 ? launch_sym(csr_sum_kernel<8, 8, false, S>, 8) : launch_sym(csr_sum_kernel<8, 4, false, S>, 8); \
    else if (nu <= 16) rc = U >= 8 ? launch_sym(csr_sum_kernel<16, 8, false, S>, 16) : launch_sym(csr_sum_kernel<16, 4, false, S>, 16); \
    else rc = U >= 8 ? launch_sym(csr_sum_kernel<32, 8, false, S>, 32) : launch_sym(csr_sum_kernel<32, 4, false, S>, 32);
    if (sym == 2) { FEM_SYM_PICK(2) }
    else { FEM_SYM_PICK(3) }
#undef FEM_SYM_PICK
  } else {
    rc = check_status ? pick(std::true_type{}) : pick(std::false_type{});
  }
  if (rc) return rc;
  FEM_LAUNCH_CHECK("csr_sum_kernel");
  return 0;
}


int incidence_rows(const Pattern& P, const double* local, double* out, cudaStream_t st) {
  const int64_t n = P.ninc * (int64_t)P.nbfun_u;
  if (n == 0) return 0;
  incidence_rows_kernel<<<grid_for(n, 256), 256, 0, st>>>(P.inc, P.ninc, P.nbfun_u, local, out);
  FEM_LAUNCH_CHECK("incidence_rows_kernel");
  return 0;
}

int csr_sum_scaled(const Pattern& P, const double* stiff, const FemCoef& diff,
                   const double* mass1, double mscale, double* vals, cudaStream_t st,
                   int64_t row0, int64_t row1) {
  if (!P.has_matrix || P.nbfun_u != P.nbfun_v) {
    set_error(FEM_ERR_ARGUMENT, "the fused sum needs a square matrix pattern");
    return FEM_ERR_ARGUMENT;
  }
  if (row1 < 0 || row1 > P.nrows) row1 = P.nrows;
  if (row0 < 0) row0 = 0;
  if (row1 <= row0 || P.nnz == 0) return 0;
  const int nu = P.nbfun_u;
  if (nu > 32) {
    set_error(FEM_ERR_UNSUPPORTED, "more than 32 local functions per cell (%d)", nu);
    return FEM_ERR_UNSUPPORTED;
  }
  const int64_t ncodes = P.nelems * (int64_t)nu;
  if (ncodes >= ((int64_t)1 << 32)) {
    set_error(FEM_ERR_CAPACITY, "%lld incidence codes exceed 2^32", (long long)ncodes);
    return FEM_ERR_CAPACITY;
  }
  const unsigned long long magic = ~0ull / (unsigned long long)nu + 1ull;
  const double* field = diff.field;
  const int64_t fstride = diff.stride > 1 ? diff.stride : 1;
  const int stride = std::max(1, P.max_row_nnz);
  auto launch = [&](auto kern, int G) -> int {
    const int rpw = 32 / G;
    const size_t per_warp = (size_t)rpw * stride * sizeof(double);
    const int warps = smem_block_warps(per_warp);
    if (!warps) return row_smem_error(stride);
    const int threads = 32 * warps;
    const size_t smem = warps * per_warp;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return check_cuda(e, "csr_scaled smem");
    }
    const int64_t rows_per_block = (int64_t)warps * rpw;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(row1 - row0, rows_per_block),
                                                                (int64_t)num_sms() * 64));
    kern<<<grid, threads, smem, st>>>(P.inc_ptr, P.inc, P.slot, P.indptr, stiff, field, fstride,
                                      diff.scale, mass1, mscale, row0, row1, nu, stride, vals,
                                      magic);
    return 0;
  };
  const int U = P.sum_unroll;
  int rc;
  if (P.sum_cols == 2 && (nu == 4 || nu == 6 || nu == 10)) {
    using Kern = decltype(&csr_scaled_pair_kernel<4, 4>);
    Kern kern;
    int rpw;
    if (nu == 4) {
      kern = U >= 16 ? csr_scaled_pair_kernel<4, 16> : U >= 8 ? csr_scaled_pair_kernel<4, 8> : csr_scaled_pair_kernel<4, 4>;
      rpw = 16;
    } else if (nu == 6) {
      kern = U >= 16 ? csr_scaled_pair_kernel<6, 16> : U >= 8 ? csr_scaled_pair_kernel<6, 8> : csr_scaled_pair_kernel<6, 4>;
      rpw = 10;
    } else {
      kern = U >= 8 ? csr_scaled_pair_kernel<10, 8> : csr_scaled_pair_kernel<10, 4>;
      rpw = 6;
    }
    const size_t per_warp = (size_t)rpw * stride * sizeof(double);
    const int warps = smem_block_warps(per_warp);
    if (!warps) return row_smem_error(stride);
    const int threads = 32 * warps;
    const size_t smem = warps * per_warp;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return check_cuda(e, "csr_scaled smem");
    }
    const int64_t rows_per_block = (int64_t)warps * rpw;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(row1 - row0, rows_per_block),
                                                                (int64_t)num_sms() * 64));
    kern<<<grid, threads, smem, st>>>(P.inc_ptr, P.inc, P.slot, P.indptr, stiff, field, fstride,
                                      diff.scale, mass1, mscale, row0, row1, stride, vals);
    FEM_LAUNCH_CHECK("csr_scaled_pair_kernel");
    return 0;
  }
  if (nu == 4) rc = U >= 16 ? launch(csr_scaled_kernel<4, 16, 4>, 4) : U >= 8 ? launch(csr_scaled_kernel<4, 8, 4>, 4) : launch(csr_scaled_kernel<4, 4, 4>, 4);
  else if (nu < 4) rc = U >= 16 ? launch(csr_scaled_kernel<4, 16>, 4) : U >= 8 ? launch(csr_scaled_kernel<4, 8>, 4) : launch(csr_scaled_kernel<4, 4>, 4);
  else if (nu <= 8) rc = U >= 16 ? launch(csr_scaled_kernel<8, 16>, 8) : U >= 8 ? launch(csr_scaled_kernel<8, 8>, 8) : launch(csr_scaled_kernel<8, 4>, 8);
  else if (nu <= 16) rc = U >= 8 ? launch(csr_scaled_kernel<16, 8>, 16) : launch(csr_scaled_kernel<16, 4>, 16);
  else rc = U >= 8 ? launch(csr_scaled_kernel<32, 8>, 32) : launch(csr_scaled_kernel<32, 4>, 32);
  if (rc) return rc;
  FEM_LAUNCH_CHECK("csr_scaled_kernel");
  return 0;
}

int vector_sum(const Pattern& P, const double* local, double* b, cudaStream_t st) {
  if (P.nrows == 0) return 0;
  vector_sum_kernel<<<(unsigned)ceil_div(P.nrows, 256), 256, 0, st>>>(P.inc_ptr, P.inc, local,
                                                                     P.nrows, b);
  FEM_LAUNCH_CHECK("vector_sum_kernel");
  return 0;
}

void free_pattern(Pattern* P) {
  if (!P) return;
  cudaFree(P->inc_ptr);
  cudaFree(P->inc);
  cudaFree(P->indptr);
  cudaFree(P->indices);
  cudaFree(P->slot);
  delete P;
}


int row_mass_base(const Pattern& P, const double* adet, int16_t* mbase, int* shmax_out,
                  bool* ok, cudaStream_t st) {
  // headroom: a row adds at most max_row_inc entries of at most 2 * 2^(53 + shmax)
  int lg = 0;
  while ((1 << lg) < std::max(1, P.max_row_inc)) ++lg;
  const int shmax = 8 - lg;
  *shmax_out = shmax;
  *ok = false;
  if (P.nrows == 0) {
    *ok = true;
    return 0;
  }
  AsyncScratch scratch(st);
  int32_t* ext = nullptr;
  FEM_TRY_CUDA(scratch.alloc(&ext, 2 * sizeof(int32_t)));
  const int32_t init[2] = {2047, 0};
  FEM_TRY_CUDA(cudaMemcpyAsync(ext, init, sizeof(init), cudaMemcpyHostToDevice, st));
  row_mass_base_kernel<<<(unsigned)ceil_div(P.nrows, 256), 256, 0, st>>>(
      P.inc_ptr, P.inc, P.nrows, P.nbfun_v, adet, shmax, mbase, ext);
  FEM_LAUNCH_CHECK("row_mass_base_kernel");
  int32_t h[2] = {0, 0};
  FEM_TRY_CUDA(cudaMemcpyAsync(h, ext, sizeof(h), cudaMemcpyDeviceToHost, st));
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  // the unit 2^(base - 1075) must be a normal double: base = exponent - shmax
  // in [53 + ..., 2046]; degenerate (0) or non-finite (2047) cells excluded
  *ok = shmax >= 0 && h[0] >= 64 + shmax && h[1] <= 2000;
  return 0;
}

int csr_sum_geometry_p1(const Pattern& P, int dim, const double* geo, const FemCoef& diff,
                        const FemCoef& mass, const int16_t* mbase, double* vals, cudaStream_t st,
                        int64_t row0, int64_t row1) {
  const int nu = dim + 1;
  if (!P.has_matrix || P.nbfun_u != nu || P.nbfun_v != nu || (dim != 2 && dim != 3)) {
    set_error(FEM_ERR_ARGUMENT, "the one-pass P1 sum needs a square P1 simplex pattern");
    return FEM_ERR_ARGUMENT;
  }
  if (!mass.field && !mbase) {
    set_error(FEM_ERR_ARGUMENT, "the one-pass P1 sum needs the rows' mass binary points");
    return FEM_ERR_ARGUMENT;
  }
  if (row1 < 0 || row1 > P.nrows) row1 = P.nrows;
  if (row0 < 0) row0 = 0;
  if (row1 <= row0 || P.nnz == 0) return 0;
  if (P.nelems * (int64_t)nu >= ((int64_t)1 << 32)) {
    set_error(FEM_ERR_CAPACITY, "%lld incidence codes exceed 2^32", (long long)(P.nelems * nu));
    return FEM_ERR_CAPACITY;
  }
  // off-diagonal P1 mass per unit |det|: 1/((d+1)(d+2) d!) -- 1/120 (tet), 1/24 (tri)
  const double moff = dim == 3 ? 0.05 * (1.0 / 6.0) : (1.0 / 12.0) * 0.5;
  const int stride = std::max(1, P.max_row_nnz);
  const int rpw = 16;
  const size_t per_warp = (size_t)rpw * stride * (sizeof(double) + 8);
  const int warps = smem_block_warps(per_warp);
  if (!warps) return row_smem_error(stride);
  const int threads = 32 * warps;
  const size_t smem = warps * per_warp;
  const int64_t rows_per_block = (int64_t)warps * rpw;
  const double* kf = diff.field;
  const int64_t ks = diff.stride > 1 ? diff.stride : 1;
  const double* mf = mass.field;
  const int64_t ms = mass.stride > 1 ? mass.stride : 1;
  const int U = P.sum_unroll >= 8 ? 8 : 4;
  auto launch = [&](auto kern) -> int {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return check_cuda(e, "csr_geometry_p1 smem");
    }
    const int grid = resident_grid(kern, threads, smem, ceil_div(row1 - row0, rows_per_block));
    kern<<<grid, threads, smem, st>>>(P.inc_ptr, P.inc, P.slot, P.indptr, geo, P.nelems, kf, ks,
                                      diff.scale, mf, ms, mass.scale, moff, mbase, row0, row1,
                                      stride, vals);
    return 0;
  };
  int rc;
#define FEM_GEO_PICK(NU)                                                                      \
  if (mf) rc = U == 8 ? launch(csr_geometry_p1_kernel<NU, 8, true>) : launch(csr_geometry_p1_kernel<NU, 4, true>); \
  else rc = U == 8 ? launch(csr_geometry_p1_kernel<NU, 8, false>) : launch(csr_geometry_p1_kernel<NU, 4, false>);
  if (nu == 4) { FEM_GEO_PICK(4) }
  else { FEM_GEO_PICK(3) }
#undef FEM_GEO_PICK
  if (rc) return rc;
  FEM_LAUNCH_CHECK("csr_geometry_p1_kernel");
  return 0;
}


int build_upper_lists(const Pattern& P, UpperLists* U, cudaStream_t st, bool wide,
                      int64_t block_rows) {
  *U = UpperLists();
  U->block_rows = block_rows > 0 ? block_rows : 0;
  const int nu = P.nbfun_u;
  wide = wide || nu > 4;
  if (!P.has_matrix || P.nbfun_v != nu || nu > 11) {
    set_error(FEM_ERR_ARGUMENT, "upper lists need a square pattern of at most 11 local functions");
    return FEM_ERR_ARGUMENT;
  }
  const int cell_bits = wide ? 25 : 28;
  if (P.nelems >= ((int64_t)1 << cell_bits)) {
    set_error(FEM_ERR_CAPACITY, "%lld cells exceed the upper lists' %d-bit cell codes",
              (long long)P.nelems, cell_bits);
    return FEM_ERR_CAPACITY;
  }
  const int64_t n = P.nrows;
  AsyncScratch scratch(st);
  int32_t *nd = nullptr, *no = nullptr, *cnt = nullptr;
  FEM_TRY_CUDA(scratch.alloc(&nd, (n + 1) * sizeof(int32_t)));
  FEM_TRY_CUDA(scratch.alloc(&no, (n + 1) * sizeof(int32_t)));
  FEM_TRY_CUDA(cudaMemsetAsync(nd, 0, (n + 1) * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(no, 0, (n + 1) * sizeof(int32_t), st));
  if (n > 0) {
    upper_count_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(P.indptr, P.indices, n, nd, no);
    FEM_LAUNCH_CHECK("upper_count_kernel");
  }
  auto fail = [&](int rc) {
    free_upper_lists(U);
    return rc;
  };
  int64_t tot_d = 0, tot_o = 0;
  FEM_TRY_CUDA(cudaMalloc(&U->dpos, (n + 1) * sizeof(int32_t)));
  FEM_TRY_CUDA(cudaMalloc(&U->opos, (n + 1) * sizeof(int32_t)));
  int rc = exclusive_scan_i32(nd, U->dpos, n, &tot_d, st);
  if (!rc) rc = exclusive_scan_i32(no, U->opos, n, &tot_o, st);
  if (rc) return fail(rc);
  U->nd = tot_d;
  U->nupper = tot_d + tot_o;
  U->nslices = ceil_div(U->nupper, 32);
  const int64_t nup1 = std::max<int64_t>(1, U->nupper);
  cudaError_t e = cudaMalloc(&U->pos, nup1 * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&U->tpos, nup1 * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&U->row, nup1 * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&U->slice_len, (U->nslices + 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&U->slice_base, (U->nslices + 1) * sizeof(int32_t));
  if (e != cudaSuccess) return fail(check_cuda(e, "cudaMalloc(upper lists)"));
  int32_t* asym = nullptr;
  e = scratch.alloc(&cnt, nup1 * sizeof(int32_t));
  if (e == cudaSuccess) e = scratch.alloc(&asym, sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMemsetAsync(asym, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return fail(check_cuda(e, "cudaMallocAsync(upper list lengths)"));
  if (n > 0) {
    upper_fill_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, st>>>(
        P.indptr, P.indices, P.inc_ptr, P.inc, P.slot, nu, n, U->dpos, U->opos, U->nd,
        U->block_rows, U->pos, U->tpos, U->row, cnt, asym);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(check_cuda(e, "upper_fill_kernel"));
    int32_t h = 0;
    e = cudaMemcpyAsync(&h, asym, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(check_cuda(e, "upper_fill_kernel"));
    if (h) {
      set_error(FEM_ERR_UNSUPPORTED, "the CSR pattern is not symmetric: no upper lists");
      return fail(FEM_ERR_UNSUPPORTED);
    }
  }
  FEM_TRY_CUDA(cudaMemsetAsync(U->slice_len, 0, (U->nslices + 1) * sizeof(int32_t), st));
  if (U->nslices > 0) {
    upper_slice_len_kernel<<<(unsigned)ceil_div(U->nslices * 32, 256), 256, 0, st>>>(
        cnt, U->nupper, U->nslices, U->slice_len);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(check_cuda(e, "upper_slice_len_kernel"));
  }
  int64_t rows32 = 0;
  rc = exclusive_scan_i32(U->slice_len, U->slice_base, U->nslices, &rows32, st);
  if (rc) return fail(rc);
  if (rows32 * 32 >= INT32_MAX) {
    set_error(FEM_ERR_CAPACITY, "upper lists of %lld codes exceed int32 offsets",
              (long long)(rows32 * 32));
    return fail(FEM_ERR_CAPACITY);
  }
  U->ncodes = rows32 * 32;
  {
    std::vector<int32_t> lens(U->nslices);
    e = cudaMemcpyAsync(lens.data(), U->slice_len, U->nslices * sizeof(int32_t),
                        cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(check_cuda(e, "upper slice lengths"));
    U->max_len = 0;
    for (int32_t v : lens) U->max_len = std::max(U->max_len, v);
  }
  e = cudaMalloc(&U->codes, std::max<int64_t>(1, U->ncodes) * sizeof(uint32_t));
  if (e != cudaSuccess) return fail(check_cuda(e, "cudaMalloc(upper codes)"));
  FEM_TRY_CUDA(cudaMemsetAsync(U->codes, 0xFF, std::max<int64_t>(1, U->ncodes) * sizeof(uint32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(cnt, 0, nup1 * sizeof(int32_t), st));
  if (n > 0) {
    upper_codes_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, st>>>(
        P.indptr, P.indices, P.inc_ptr, P.inc, P.slot, nu, n, U->dpos, U->opos, U->nd,
        U->block_rows, U->slice_base, cnt, U->codes, wide);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(check_cuda(e, "upper_codes_kernel"));
  }
  // host copies of the row -> upper-entry offsets (row ranges of the
  // pipelined host path)
  U->dpos_h.resize(n + 1);
  U->opos_h.resize(n + 1);
  e = cudaMemcpyAsync(U->dpos_h.data(), U->dpos, (n + 1) * sizeof(int32_t),
                      cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(U->opos_h.data(), U->opos, (n + 1) * sizeof(int32_t),
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(check_cuda(e, "upper lists"));
  return 0;
}

void free_upper_lists(UpperLists* U) {
  if (!U) return;
  cudaFree(U->dpos);
  cudaFree(U->opos);
  cudaFree(U->pos);
  cudaFree(U->tpos);
  cudaFree(U->row);
  cudaFree(U->slice_len);
  cudaFree(U->slice_base);
  cudaFree(U->codes);
  *U = UpperLists();
}

int csr_sum_upper_p1(const Pattern& P, const UpperLists& U, int dim, const double* geo,
                     const FemCoef& diff, const FemCoef& mass, const int16_t* mbase, double* vals,
                     cudaStream_t st, int64_t row0, int64_t row1, int32_t* status, bool tma,
                     const uint8_t* ref_bits, int const_bits) {
  const int nu = dim + 1;
  if (!U.codes || P.nbfun_u != nu || (dim != 2 && dim != 3)) {
    set_error(FEM_ERR_ARGUMENT, "the upper-gather P1 sum needs the pattern's upper lists");
    return FEM_ERR_ARGUMENT;
  }
  if (!mass.field && !mbase) {
    set_error(FEM_ERR_ARGUMENT, "the one-pass P1 sum needs the rows' mass binary points");
    return FEM_ERR_ARGUMENT;
  }
  if (row1 < 0 || row1 > P.nrows) row1 = P.nrows;
  if (row0 < 0) row0 = 0;
  if (row1 <= row0 || U.nupper == 0) return 0;
  const double moff = dim == 3 ? 0.05 * (1.0 / 6.0) : (1.0 / 12.0) * 0.5;
  const double* kf = diff.field;
  const int64_t ks = diff.stride > 1 ? diff.stride : 1;
  const double* mf = mass.field;
  const int64_t ms = mass.stride > 1 ? mass.stride : 1;
  const int Un = P.sum_unroll >= 8 ? 8 : 4;
  // upper entries of rows [row0, row1): a diagonal range and an off-diagonal
  // one (all rows: the two are adjacent, one launch); in the row-block
  // layout one range, the rows' blocks
  const bool all = row0 == 0 && row1 == P.nrows;
  int64_t ranges[2][2] = {{all ? 0 : U.dpos_h[row0], all ? U.nupper : U.dpos_h[row1]},
                          {all ? 0 : U.nd + U.opos_h[row0], all ? 0 : U.nd + U.opos_h[row1]}};
  if (U.block_rows > 0 && !all) {
    if (row0 % U.block_rows || (row1 % U.block_rows && row1 != P.nrows)) {
      set_error(FEM_ERR_ARGUMENT, "upper-list rows [%lld, %lld) off the %lld-row blocks",
                (long long)row0, (long long)row1, (long long)U.block_rows);
      return FEM_ERR_ARGUMENT;
    }
    ranges[0][0] = (int64_t)U.dpos_h[row0] + U.opos_h[row0];
    ranges[0][1] = (int64_t)U.dpos_h[row1] + U.opos_h[row1];
    ranges[1][0] = ranges[1][1] = 0;
  }
  const int threads = 128;
  for (int k = 0; k < 2; ++k) {
    const int64_t ua = ranges[k][0], ub = ranges[k][1];
    if (ub <= ua) continue;
    const int64_t nsl = ((ub + 31) >> 5) - (ua >> 5);
    const int64_t work = ceil_div(nsl, threads / 32);
    // the staged form: two buffers of the longest slice per warp + 2 mbarriers
    const size_t tma_smem = (size_t)(threads / 32) * (2 * (size_t)U.max_len * 128 + 16);
    const bool staged = tma && status && U.max_len > 0 && tma_smem <= 96 * 1024;
    auto launch = [&](auto kern) {
      const int grid = resident_grid(kern, threads, 0, work);
      kern<<<grid, threads, 0, st>>>(ua, ub, U.slice_len, U.slice_base, U.codes, U.pos, U.tpos,
                                     U.row, geo, P.nelems, kf, ks, diff.scale, mf, ms, mass.scale,
                                     moff, mbase, vals, ref_bits, const_bits, status);
    };
    const bool check = ref_bits && status && kf && ks == 1 && !mf && mass.scale != 0.0;
    auto launch_tma = [&](auto kern) -> int {
      if (tma_smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)tma_smem);
        if (e != cudaSuccess) return check_cuda(e, "csr_upper_p1_tma smem");
      }
      const int grid = resident_grid(kern, threads, tma_smem, work);
      kern<<<grid, threads, tma_smem, st>>>(ua, ub, U.slice_len, U.slice_base, U.codes,
                                            U.max_len, U.pos, U.tpos, U.row, geo, P.nelems, kf, ks,
                                            diff.scale, mf, ms, mass.scale, moff, mbase, vals,
                                            status);
      return 0;
    };
    int rc = 0;
#define FEM_UP_PICK(NU)                                                                     \
    if (staged) { \
      if (mf) rc = Un == 8 ? launch_tma(csr_upper_p1_tma_kernel<NU, 8, true>) : launch_tma(csr_upper_p1_tma_kernel<NU, 4, true>); \
      else rc = Un == 8 ? launch_tma(csr_upper_p1_tma_kernel<NU, 8, false>) : launch_tma(csr_upper_p1_tma_kernel<NU, 4, false>); \
    } else if (mf) { if (Un == 8) launch(csr_upper_p1_kernel<NU, 8, true>); else launch(csr_upper_p1_kernel<NU, 4, true>); } \
    else if (check) { if (Un == 8) launch(csr_upper_p1_kernel<NU, 8, false, true>); else launch(csr_upper_p1_kernel<NU, 4, false, true>); } \
    else { if (Un == 8) launch(csr_upper_p1_kernel<NU, 8, false>); else launch(csr_upper_p1_kernel<NU, 4, false>); }
    if (nu == 4) { FEM_UP_PICK(4) }
    else { FEM_UP_PICK(3) }
#undef FEM_UP_PICK
    if (rc) return rc;
    FEM_LAUNCH_CHECK("csr_upper_p1_kernel");
  }
  return 0;
}

}  // namespace fem
