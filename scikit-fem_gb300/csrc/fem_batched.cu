// Batched assembly of many meshes in one persistent launch over a device
// work queue: forward (local matrices + fixed-order segmented sum) and the
// coefficient adjoint, for scalar simplex bases (TriP1/P2, TetP1/P2) on the
// per-cell geometry cache.
//
// The reference assembles one mesh per BilinearForm.assemble call
// (skfem/assembly/form/bilinear_form.py:130-148), so a batch is a Python
// loop over meshes; here the meshes are one block-diagonal union (each
// keeps its own numbering inside its block) and the launch processes a
// queue of work units:
//   cell unit (mesh m, cells [a, b), at most one block's worth): each thread
//     one cell -- its local matrix k_e S_e + m_e M_e from the cached
//     geometry into the element-major staging (as fem_assemble's local
//     kernel writes it), and the adjoint of J = w^T K u with respect to the
//     cell's coefficients, dJ/dk_e = w_e^T S_e u_e and dJ/dm_e = w_e^T M_e
//     u_e, from the same matrices (no second pass over the geometry);
//   row unit (mesh m, rows [a, b)): the fixed-order segmented sum of those
//     rows (csr_sum_kernel's order: ascending (cell, local row) per slot).
// Blocks take units in queue order from an atomic ticket.  A row unit of
// mesh m first waits until every cell unit of mesh m has published its
// staging (a per-mesh counter); the queue lists all of a mesh's cell units
// before its row units (and the next mesh's cell units before them, so the
// waits are short), so a block only ever waits for units that blocks
// already running hold and that never wait themselves -- no deadlock,
// whatever the grid size.  Every wait is bounded: past the limit the block
// sets FEM_ERR_TIMEOUT in the status word and skips the unit.

#include "fem_common.cuh"
#include "fem_nodesum.cuh"
#include "fem_tables.cuh"

#include <algorithm>
#include <vector>

struct FemBatchPlan {
  int32_t nmeshes = 0;
  int64_t nunits = 0;
  int32_t cells_per_unit = 128, rows_per_unit = 256;
  int64_t* unit_begin = nullptr;  // nunits
  int64_t* unit_end = nullptr;    // nunits
  int32_t* unit_kind_mesh = nullptr;  // nunits: kind (bit 0) | mesh << 1
  int32_t* cell_units = nullptr;  // nmeshes: cell units of each mesh
  std::vector<int64_t> cell_off, row_off;   // the meshes' offsets (host)
  // The one-pass queue (scalar TriP2 / TetP2 patterns with node-block
  // lists), built on first use for the lists it was built from: cell units
  // as above, then row-block units (kind 1, mesh = the block's last mesh,
  // [begin, end) = the block's slots of the lists) waiting on the meshes
  // [op_mesh_lo, mesh] of the block's rows.
  const void* op_lists = nullptr;
  int64_t op_nunits = 0;
  int64_t* op_begin = nullptr;
  int64_t* op_end = nullptr;
  int32_t* op_kind_mesh = nullptr;
  int32_t* op_mesh_lo = nullptr;
};

namespace fem_batched {

using fem::coef_at;
using fem::dbits;

constexpr int kBlock = 128;
constexpr long long kSpinLimit = 1ll << 22;   // x 128 ns: about half a second

template <int D, int ORDER>
struct Traits;
template <> struct Traits<2, 1> { static constexpr int NB = 3; static constexpr double FACT = 2.0; };
template <> struct Traits<2, 2> { static constexpr int NB = 6; static constexpr double FACT = 2.0; };
template <> struct Traits<3, 1> { static constexpr int NB = 4; static constexpr double FACT = 6.0; };
template <> struct Traits<3, 2> { static constexpr int NB = 10; static constexpr double FACT = 6.0; };

__device__ __forceinline__ int load_acquire(const int32_t* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// The status bits of one cell's coefficients, as the local kernels give
// them (FEM_ERR_VARYING for a per-point row that is not constant,
// FEM_ERR_STALE_PATTERN for zero bits that differ from the pattern's).
__device__ __forceinline__ int32_t cell_status(const FemBilinear& f, int64_t e, int ref) {
  int32_t st = fem::row_status(f.diff, e) | fem::row_status(f.mass, e);
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

struct SumArgs {
  const int32_t* inc_ptr;
  const int32_t* inc;
  const uint16_t* slot;
  const int32_t* indptr;
  int nu;
  int stride;
};

template <int D, int ORDER, int G, int U>
__global__ void __launch_bounds__(kBlock) batched_forward_vjp_kernel(
    FemMesh m, FemBasis b, FemBilinear f, const double* __restrict__ geo, SumArgs sa,
    const int32_t* __restrict__ kind_mesh, const int64_t* __restrict__ ubeg,
    const int64_t* __restrict__ uend, int64_t nunits, const int32_t* __restrict__ cell_units,
    int32_t* __restrict__ counters, const uint8_t* __restrict__ ref_bits,
    double* __restrict__ staging, double* __restrict__ vals, const double* __restrict__ w,
    const double* __restrict__ u, double* __restrict__ dcd, double* __restrict__ dcm,
    int32_t* __restrict__ status) {
  constexpr int NB = Traits<D, ORDER>::NB;
  constexpr int L = NB * NB;
  constexpr double INV_FACT = 1.0 / Traits<D, ORDER>::FACT;
  constexpr int NG = (D + 1) * (D + 2) / 2;
  constexpr int RPW = 32 / G;
  extern __shared__ double smem[];
  __shared__ long long s_unit;
  __shared__ int s_skip;
  int32_t* ticket = counters;
  int32_t* done = counters + 1;
  int32_t flags = 0;
  for (;;) {
    if (threadIdx.x == 0) s_unit = atomicAdd(ticket, 1);
    __syncthreads();
    const long long k = s_unit;
    __syncthreads();
    if (k >= nunits) break;
    const int km = kind_mesh[k];
    const int mesh = km >> 1;
    const int64_t a = ubeg[k], z = uend[k];
    if ((km & 1) == 0) {
      // ---------------------------------------------------- cell unit
      // each thread writes its cell's matrix straight into the staging (the
      // rows of one cell contiguous; the L2 merges the lanes' partial
      // sectors), so the block needs no shared memory for the cell units
      const int64_t e = a + threadIdx.x;
      double* row = staging + e * L;
      if (e < z) {
        const int rb = ref_bits ? (int)__ldg(ref_bits + e) : -1;
        double gram[D + 1][D + 1];
        int q = 0;
#pragma unroll
        for (int i = 0; i <= D; ++i)
#pragma unroll
          for (int j = i; j <= D; ++j) gram[i][j] = __ldg(geo + (int64_t)(q++) * m.nelems + e);
        const double adet = __ldg(geo + (int64_t)NG * m.nelems + e);
        const double sd = coef_at(f.diff, e);
        const double sm = coef_at(f.mass, e) * adet;
        double kst[NB][NB];
        double mm[NB][NB];
#define G_(i, j) ((i) <= (j) ? gram[i][j] : gram[j][i])
#define KS(i, j, v) { kst[i][j] = (v); }
#define KM(i, j, v) { constexpr double _m = (v) * INV_FACT; mm[i][j] = _m; mm[j][i] = _m; const double _v = __fma_rn(sd, kst[i][j], sm * _m); row[(i) * NB + (j)] = _v; row[(j) * NB + (i)] = _v; }
        if constexpr (D == 2 && ORDER == 1) { TRI1_STIFF(G_, KS); TRI1_MASS(KM); }
        if constexpr (D == 2 && ORDER == 2) { TRI2_STIFF(G_, KS); TRI2_MASS(KM); }
        if constexpr (D == 3 && ORDER == 1) { TET1_STIFF(G_, KS); TET1_MASS(KM); }
        if constexpr (D == 3 && ORDER == 2) { TET2_STIFF(G_, KS); TET2_MASS(KM); }
#undef G_
#undef KS
#undef KM
        if (w && u && (dcd || dcm)) {
          double wl[NB], ul[NB];
#pragma unroll
          for (int i = 0; i < NB; ++i) {
            const int64_t dof = b.element_dofs[(int64_t)i * m.nelems + e];
            wl[i] = w[dof];
            ul[i] = u[dof];
          }
          if (dcd) {
            double js = 0.0;
#pragma unroll
            for (int i = 0; i < NB; ++i) {
              double ks = 0.0;
#pragma unroll
              for (int j = 0; j < NB; ++j) ks = __fma_rn(i <= j ? kst[i][j] : kst[j][i], ul[j], ks);
              js = __fma_rn(wl[i], ks, js);
            }
            dcd[e] = f.diff.scale * js;
          }
          if (dcm) {
            double jm = 0.0;
#pragma unroll
            for (int i = 0; i < NB; ++i) {
              double ms = 0.0;
#pragma unroll
              for (int j = 0; j < NB; ++j) ms = __fma_rn(mm[i][j], ul[j], ms);
              jm = __fma_rn(wl[i], ms, jm);
            }
            dcm[e] = f.mass.scale * adet * jm;
          }
        }
        flags |= cell_status(f, e, rb);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(done + mesh, 1);
      }
    } else {
      // ----------------------------------------------------- row unit
      if (threadIdx.x == 0) {
        const int need = cell_units[mesh];
        long long it = 0;
        while (load_acquire(done + mesh) < need && it < kSpinLimit) {
          __nanosleep(128);
          ++it;
        }
        s_skip = load_acquire(done + mesh) < need;
        if (s_skip) atomicOr(status, 1 << FEM_ERR_TIMEOUT);
        __threadfence();
      }
      __syncthreads();
      if (!s_skip) {
        const int lane = threadIdx.x & 31;
        const int sub = lane / G;
        const int j = lane - sub * G;
        const int wib = threadIdx.x >> 5;
        double* acc = smem + ((size_t)wib * RPW + sub) * sa.stride;
        const int64_t rows_per_block = (int64_t)(blockDim.x >> 5) * RPW;
        for (int64_t rb = a; rb < z; rb += rows_per_block) {
          const int64_t r = rb + (int64_t)wib * RPW + sub;
          int32_t bb = 0, len = 0, p0 = 0, nnz = 0;
          if (r < z) {
            bb = sa.inc_ptr[r];
            len = sa.inc_ptr[r + 1] - bb;
            p0 = sa.indptr[r];
            nnz = sa.indptr[r + 1] - p0;
          }
          for (int c = j; c < nnz; c += G) acc[c] = 0.0;
          int maxlen = len;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1)
            maxlen = max(maxlen, __shfl_xor_sync(0xffffffffu, maxlen, o));
          __syncwarp();
          for (int q0 = 0; q0 < maxlen; q0 += U) {
            double v[U];
            int s[U];
#pragma unroll
            for (int uu = 0; uu < U; ++uu) {
              const int q = q0 + uu;
              s[uu] = 0xFFFF;
              v[uu] = 0.0;
              if (q < len && j < sa.nu) {
                const int64_t code = __ldg(sa.inc + bb + q);
                s[uu] = __ldg(sa.slot + ((int64_t)bb + q) * sa.nu + j);
                // staging written in this launch by other blocks: L2, not L1
                v[uu] = __ldcg(staging + code * sa.nu + j);
              }
            }
#pragma unroll
            for (int uu = 0; uu < U; ++uu) {
              if (s[uu] != 0xFFFF) acc[s[uu]] += v[uu];
              __syncwarp();
            }
          }
          for (int c = j; c < nnz; c += G) vals[p0 + c] = acc[c];
          __syncwarp();
        }
      }
      __syncthreads();
    }
  }
  fem::publish_status(status, flags);
}

// The one-pass form for scalar TriP2 / TetP2 (ORDER 2) patterns with
// node-block lists -- the batched form of the one-pass node-block sum:
//   cell unit: each thread one cell -- its pair values E[e] (the scaled Gram
//     entries times k_e, then m_e |det| / d!; scalar_pair_kernel's rounding)
//     into the staging, and dJ/dk_e = w_e^T S_e u_e, dJ/dm_e = w_e^T M_e u_e
//     from the cached geometry, as the two-pass form computes them;
//   row-block unit (the lists' slots of one block of rows): after a bounded
//     acquire-wait on the cell units of every mesh the block's rows belong
//     to, the block's slices, one lane per CSR entry (scalar_entry_sum: the
//     reference-tensor terms and mass of its cells in ascending order).
// The same values bit for bit as fem_assemble's one-pass sum.
struct NodeArgs {
  const int32_t* slice_len;
  const int32_t* slice_base;
  const uint32_t* codes;
  const int32_t* vpos;
  const int32_t* vposT;
  const uint16_t* vmask;
  const fem::VecTerm* terms;
  const int32_t* count;
  const double* mm;
  int npairs;
};

// Triangles: at most 64 registers (60, no spills) for eight resident blocks
// per SM -- the kernel waits on its gathers (about 23 long-scoreboard
// stalls per issue), so more warps per SM pay (9.73 -> 9.28 ms on 512
// TriP2 meshes); tetrahedra keep their registers (a bound spills).
template <int D, bool MASS>
__global__ void __launch_bounds__(kBlock, D == 2 ? 8 : 1) batched_onepass_vjp_kernel(
    FemMesh m, FemBasis b, FemBilinear f, const double* __restrict__ geo, NodeArgs na,
    const int32_t* __restrict__ kind_mesh, const int32_t* __restrict__ mesh_lo,
    const int64_t* __restrict__ ubeg, const int64_t* __restrict__ uend, int64_t nunits,
    const int32_t* __restrict__ cell_units, int32_t* __restrict__ counters,
    const uint8_t* __restrict__ ref_bits, double* __restrict__ staging,
    double* __restrict__ vals, const double* __restrict__ w, const double* __restrict__ u,
    double* __restrict__ dcd, double* __restrict__ dcm, int32_t* __restrict__ status) {
  constexpr int NB = Traits<D, 2>::NB;
  constexpr double INV_FACT = 1.0 / Traits<D, 2>::FACT;
  constexpr int NG = (D + 1) * (D + 2) / 2;
  constexpr int R = NG + 1;
  __shared__ fem::VecTerm terms[fem::kMaxNodePairs * fem::kMaxTerms];
  __shared__ int32_t count[fem::kMaxNodePairs];
  __shared__ double mmt[fem::kMaxNodePairs];
  __shared__ long long s_unit;
  __shared__ int s_skip;
  for (int k = threadIdx.x; k < na.npairs * fem::kMaxTerms; k += blockDim.x)
    terms[k] = na.terms[k];
  for (int k = threadIdx.x; k < na.npairs; k += blockDim.x) {
    count[k] = na.count[k];
    mmt[k] = na.mm[k];
  }
  __syncthreads();
  int32_t* ticket = counters;
  int32_t* done = counters + 1;
  int32_t flags = 0;
  for (;;) {
    if (threadIdx.x == 0) s_unit = atomicAdd(ticket, 1);
    __syncthreads();
    const long long k = s_unit;
    __syncthreads();
    if (k >= nunits) break;
    const int km = kind_mesh[k];
    const int mesh = km >> 1;
    const int64_t a = ubeg[k], z = uend[k];
    if ((km & 1) == 0) {
      // ---------------------------------------------------- cell unit
      const int64_t e = a + threadIdx.x;
      if (e < z) {
        const int rb = ref_bits ? (int)__ldg(ref_bits + e) : -1;
        double gram[D + 1][D + 1];
        int q = 0;
#pragma unroll
        for (int i = 0; i <= D; ++i)
#pragma unroll
          for (int j = i; j <= D; ++j) gram[i][j] = __ldg(geo + (int64_t)(q++) * m.nelems + e);
        const double adet = __ldg(geo + (int64_t)NG * m.nelems + e);
        const double sd = coef_at(f.diff, e);
        double* row = staging + e * R;
        q = 0;
#pragma unroll
        for (int i = 0; i <= D; ++i)
#pragma unroll
          for (int j = i; j <= D; ++j) {
            row[q] = sd * gram[i][j];
            ++q;
          }
        row[NG] = coef_at(f.mass, e) * (adet * INV_FACT);
        if (w && u && (dcd || dcm)) {
          double kst[NB][NB];
          double mm[NB][NB];
#define G_(i, j) ((i) <= (j) ? gram[i][j] : gram[j][i])
#define KS(i, j, v) { kst[i][j] = (v); }
#define KM(i, j, v) { constexpr double _m = (v) * INV_FACT; mm[i][j] = _m; mm[j][i] = _m; }
          if constexpr (D == 2) { TRI2_STIFF(G_, KS); TRI2_MASS(KM); }
          if constexpr (D == 3) { TET2_STIFF(G_, KS); TET2_MASS(KM); }
#undef G_
#undef KS
#undef KM
          double wl[NB], ul[NB];
#pragma unroll
          for (int i = 0; i < NB; ++i) {
            const int64_t dof = b.element_dofs[(int64_t)i * m.nelems + e];
            wl[i] = w[dof];
            ul[i] = u[dof];
          }
          if (dcd) {
            double js = 0.0;
#pragma unroll
            for (int i = 0; i < NB; ++i) {
              double ks = 0.0;
#pragma unroll
              for (int j = 0; j < NB; ++j) ks = __fma_rn(i <= j ? kst[i][j] : kst[j][i], ul[j], ks);
              js = __fma_rn(wl[i], ks, js);
            }
            dcd[e] = f.diff.scale * js;
          }
          if (dcm) {
            double jm = 0.0;
#pragma unroll
            for (int i = 0; i < NB; ++i) {
              double ms = 0.0;
#pragma unroll
              for (int j = 0; j < NB; ++j) ms = __fma_rn(mm[i][j], ul[j], ms);
              jm = __fma_rn(wl[i], ms, jm);
            }
            dcm[e] = f.mass.scale * adet * jm;
          }
        }
        flags |= cell_status(f, e, rb);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(done + mesh, 1);
      }
    } else {
      // ------------------------------------------------ row-block unit
      if (threadIdx.x == 0) {
        int skip = 0;
        for (int mm = mesh_lo[k]; mm <= mesh && !skip; ++mm) {
          const int need = cell_units[mm];
          long long it = 0;
          while (load_acquire(done + mm) < need && it < kSpinLimit) {
            __nanosleep(128);
            ++it;
          }
          skip = load_acquire(done + mm) < need;
        }
        s_skip = skip;
        if (skip) atomicOr(status, 1 << FEM_ERR_TIMEOUT);
        __threadfence();
      }
      __syncthreads();
      if (!s_skip) {
        const int lane = threadIdx.x & 31;
        const int64_t s1 = (z + 31) >> 5;
        for (int64_t sl = (a >> 5) + (threadIdx.x >> 5); sl < s1; sl += kBlock / 32) {
          const int64_t slot = sl * 32 + lane;
          const bool inr = slot >= a && slot < z;
          const int len = inr ? __ldg(na.slice_len + sl) : 0;
          const uint32_t* cp = na.codes + (int64_t)__ldg(na.slice_base + sl) * 32 + lane;
          fem::scalar_entry_sum<D, MASS, true>(inr, slot, len, cp, m.nelems, na.npairs, terms,
                                               count, mmt, na.vpos, na.vposT, na.vmask, staging,
                                               vals);
        }
      }
      __syncthreads();
    }
  }
  fem::publish_status(status, flags);
}

}  // namespace fem_batched

namespace fem {
const VecUpper* pattern_node_lists(const FemPattern* h);
const Pattern* pattern_of(const FemPattern* h);
const uint8_t* pattern_coef_bits(const FemPattern* h);
int validate_mesh_basis(const FemMesh* m, const FemBasis* b);
const double* pattern_geometry(const FemPattern* h, const FemMesh* m);
}  // namespace fem

namespace {

// The one-pass queue of a plan for node-block lists V (one node per row):
// per mesh its cell units, then the row blocks whose rows all belong to
// earlier meshes -- every row-block unit's cells are queued before it.
int build_onepass_queue(FemBatchPlan* P, const fem::VecUpper& V) {
  if (P->op_lists == &V) return 0;
  cudaFree(P->op_begin);
  cudaFree(P->op_end);
  cudaFree(P->op_kind_mesh);
  cudaFree(P->op_mesh_lo);
  P->op_begin = P->op_end = nullptr;
  P->op_kind_mesh = P->op_mesh_lo = nullptr;
  P->op_lists = nullptr;
  P->op_nunits = 0;
  const int M = P->nmeshes;
  const int64_t nrows = (int64_t)V.U.dpos_h.size() - 1;
  if (M <= 0 || P->row_off[M] != nrows || V.block_rows <= 0) {
    fem::set_error(FEM_ERR_ARGUMENT, "batch plan rows do not match the pattern's lists");
    return FEM_ERR_ARGUMENT;
  }
  const int cpu = fem_batched::kBlock;
  auto mesh_of = [&](int64_t r) {
    return (int)(std::upper_bound(P->row_off.begin(), P->row_off.end(), r) -
                 P->row_off.begin()) - 1;
  };
  std::vector<int32_t> km, lo;
  std::vector<int64_t> ub, ue;
  const int64_t nb = (nrows + V.block_rows - 1) / V.block_rows;
  int64_t next = 0;   // the next row block to queue
  auto blocks_upto = [&](int last_mesh) {
    for (; next < nb; ++next) {
      const int64_t n0 = next * V.block_rows, n1 = std::min(nrows, n0 + V.block_rows);
      const int mh = mesh_of(n1 - 1);
      if (mh > last_mesh) break;
      const int64_t a = (int64_t)V.U.dpos_h[n0] + V.U.opos_h[n0];
      const int64_t z = (int64_t)V.U.dpos_h[n1] + V.U.opos_h[n1];
      if (z <= a) continue;
      km.push_back((mh << 1) | 1);
      lo.push_back(mesh_of(n0));
      ub.push_back(a);
      ue.push_back(z);
    }
  };
  for (int m = 0; m < M; ++m) {
    for (int64_t a = P->cell_off[m]; a < P->cell_off[m + 1]; a += cpu) {
      km.push_back(m << 1);
      lo.push_back(m);
      ub.push_back(a);
      ue.push_back(std::min<int64_t>(a + cpu, P->cell_off[m + 1]));
    }
    blocks_upto(m - 1);
  }
  blocks_upto(M - 1);
  const size_t n = std::max<size_t>(1, km.size());
  cudaError_t e = cudaMalloc(&P->op_kind_mesh, n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&P->op_mesh_lo, n * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&P->op_begin, n * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&P->op_end, n * sizeof(int64_t));
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->op_kind_mesh, km.data(), km.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->op_mesh_lo, lo.data(), lo.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->op_begin, ub.data(), ub.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->op_end, ue.data(), ue.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(P->op_begin);
    cudaFree(P->op_end);
    cudaFree(P->op_kind_mesh);
    cudaFree(P->op_mesh_lo);
    P->op_begin = P->op_end = nullptr;
    P->op_kind_mesh = P->op_mesh_lo = nullptr;
    return fem::check_cuda(e, "batch one-pass queue");
  }
  P->op_nunits = (int64_t)km.size();
  P->op_lists = &V;
  return 0;
}

}  // namespace

extern "C" {

int fem_batch_plan_build(const int64_t* cell_offsets, const int64_t* row_offsets,
                         int32_t nmeshes, int32_t rows_per_unit, FemBatchPlan** out) {
  if (!out || !cell_offsets || !row_offsets || nmeshes < 0 || rows_per_unit < 1) {
    fem::set_error(FEM_ERR_ARGUMENT, "null offsets or output, or a non-positive unit size");
    return FEM_ERR_ARGUMENT;
  }
  *out = nullptr;
  const int cpu = fem_batched::kBlock;
  std::vector<int32_t> km;
  std::vector<int64_t> ub, ue;
  std::vector<int32_t> ncell(std::max(1, nmeshes), 0);
  for (int m = 0; m < nmeshes; ++m)
    if (cell_offsets[m + 1] < cell_offsets[m] || row_offsets[m + 1] < row_offsets[m]) {
      fem::set_error(FEM_ERR_ARGUMENT, "offsets of mesh %d decrease", m);
      return FEM_ERR_ARGUMENT;
    }
  auto cells = [&](int m) {
    for (int64_t a = cell_offsets[m]; a < cell_offsets[m + 1]; a += cpu) {
      km.push_back(m << 1);
      ub.push_back(a);
      ue.push_back(std::min<int64_t>(a + cpu, cell_offsets[m + 1]));
      ++ncell[m];
    }
  };
  auto rows = [&](int m) {
    for (int64_t a = row_offsets[m]; a < row_offsets[m + 1]; a += rows_per_unit) {
      km.push_back((m << 1) | 1);
      ub.push_back(a);
      ue.push_back(std::min<int64_t>(a + rows_per_unit, row_offsets[m + 1]));
    }
  };
  // mesh m's cell units, then mesh m-1's row units: every row unit's cells
  // are queued before it, one mesh ahead
  for (int m = 0; m < nmeshes; ++m) {
    cells(m);
    if (m > 0) rows(m - 1);
  }
  if (nmeshes > 0) rows(nmeshes - 1);
  FemBatchPlan* P = new FemBatchPlan();
  P->nmeshes = nmeshes;
  P->nunits = (int64_t)km.size();
  P->cell_off.assign(cell_offsets, cell_offsets + nmeshes + 1);
  P->row_off.assign(row_offsets, row_offsets + nmeshes + 1);
  P->cells_per_unit = cpu;
  P->rows_per_unit = rows_per_unit;
  const size_t nu1 = std::max<size_t>(1, km.size());
  cudaError_t e = cudaMalloc(&P->unit_kind_mesh, nu1 * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&P->unit_begin, nu1 * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&P->unit_end, nu1 * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&P->cell_units, ncell.size() * sizeof(int32_t));
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->unit_kind_mesh, km.data(), km.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->unit_begin, ub.data(), ub.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !km.empty())
    e = cudaMemcpy(P->unit_end, ue.data(), ue.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(P->cell_units, ncell.data(), ncell.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(P->unit_kind_mesh);
    cudaFree(P->unit_begin);
    cudaFree(P->unit_end);
    cudaFree(P->cell_units);
    delete P;
    return fem::check_cuda(e, "batch plan");
  }
  *out = P;
  return 0;
}

void fem_batch_plan_destroy(FemBatchPlan* P) {
  if (!P) return;
  cudaFree(P->unit_kind_mesh);
  cudaFree(P->unit_begin);
  cudaFree(P->unit_end);
  cudaFree(P->cell_units);
  cudaFree(P->op_begin);
  cudaFree(P->op_end);
  cudaFree(P->op_kind_mesh);
  cudaFree(P->op_mesh_lo);
  delete P;
}

int fem_batch_plan_info(const FemBatchPlan* P, int64_t* nunits, int64_t* ncounters) {
  if (!P) {
    fem::set_error(FEM_ERR_ARGUMENT, "null plan");
    return FEM_ERR_ARGUMENT;
  }
  if (nunits) *nunits = P->op_lists ? P->op_nunits : P->nunits;
  if (ncounters) *ncounters = 1 + (int64_t)P->nmeshes;
  return 0;
}

int fem_batched_assemble_vjp(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                             const FemPattern* pat, const FemBatchPlan* plan, double* staging,
                             double* csr_values, const double* w, const double* u,
                             double* dcoef_diff, double* dcoef_mass, int32_t* counters,
                             int32_t* status, fem_stream_t stream) {
  int rc = fem::validate_mesh_basis(mesh, basis);
  if (rc) return rc;
  if (!form || !pat || !plan || !staging || !counters || !status ||
      (!csr_values && fem::pattern_of(pat)->nnz > 0)) {
    fem::set_error(FEM_ERR_ARGUMENT, "null form, pattern, plan or buffer");
    return FEM_ERR_ARGUMENT;
  }
  const fem::Pattern& P = *fem::pattern_of(pat);
  if (!P.has_matrix || P.nelems != mesh->nelems || P.nbfun_v != basis->nbfun ||
      P.nbfun_u != P.nbfun_v || P.staging_sym) {
    fem::set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  if (basis->vector || form->lam.field || form->lam.scale != 0.0 || form->lap.field ||
      form->lap.scale != 0.0 || form->tr.field || form->tr.scale != 0.0) {
    fem::set_error(FEM_ERR_UNSUPPORTED, "the persistent batched kernel takes scalar forms");
    return FEM_ERR_UNSUPPORTED;
  }
  const double* geo = fem::pattern_geometry(pat, mesh);
  if (!geo) {
    fem::set_error(FEM_ERR_UNSUPPORTED, "the persistent batched kernel needs the pattern's "
                   "geometry cache of this mesh's coordinates (fem_pattern_cache_geometry)");
    return FEM_ERR_UNSUPPORTED;
  }
  if (mesh->nelems * (int64_t)P.nbfun_u >= ((int64_t)1 << 31)) {
    fem::set_error(FEM_ERR_CAPACITY, "too many incidence codes for the batched kernel");
    return FEM_ERR_CAPACITY;
  }
  cudaStream_t st = (cudaStream_t)stream;
  FEM_TRY_CUDA(cudaMemsetAsync(counters, 0, (1 + (size_t)plan->nmeshes) * sizeof(int32_t), st));
  if (plan->nunits == 0) return 0;
  const uint8_t* ref = fem::pattern_coef_bits(pat);
  // scalar TriP2 / TetP2 with the pattern's node-block lists: the one-pass
  // form, unless the family's tuning selects the two-pass path
  const fem::VecUpper* V = fem::pattern_node_lists(pat);
  if (V && V->dim == 1 && V->sdim == mesh->dim &&
      (basis->family == FEM_TRI_P2 || basis->family == FEM_TET_P2) &&
      fem::tuning_for(basis->family).onepass >= 1) {
    if (mesh->nelems * (int64_t)(V->sdim == 3 ? 11 : 7) >
        mesh->nelems * (int64_t)P.nbfun_u * P.nbfun_v) {
      fem::set_error(FEM_ERR_CAPACITY, "staging too small for the pair values");
      return FEM_ERR_CAPACITY;
    }
    rc = build_onepass_queue(const_cast<FemBatchPlan*>(plan), *V);
    if (rc) return rc;
    fem_batched::NodeArgs na{V->U.slice_len, V->U.slice_base, V->U.codes, V->vpos, V->vposT,
                             V->vmask, static_cast<const fem::VecTerm*>(V->terms), V->count,
                             V->mm, V->ns * V->ns};
    const bool mass = form->mass.field || form->mass.scale != 0.0;
    auto launch1 = [&](auto kern) -> int {
      int per_sm = 0;
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern,
                                                                    fem_batched::kBlock, 0);
      if (e != cudaSuccess) return fem::check_cuda(e, "batched kernel occupancy");
      const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(
          (int64_t)std::max(1, per_sm) * fem::num_sms(), plan->op_nunits));
      kern<<<(unsigned)grid, fem_batched::kBlock, 0, st>>>(
          *mesh, *basis, *form, geo, na, plan->op_kind_mesh, plan->op_mesh_lo, plan->op_begin,
          plan->op_end, plan->op_nunits, plan->cell_units, counters, ref, staging, csr_values,
          w, u, dcoef_diff, dcoef_mass, status);
      return 0;
    };
    if (mesh->dim == 3)
      rc = mass ? launch1(fem_batched::batched_onepass_vjp_kernel<3, true>)
                : launch1(fem_batched::batched_onepass_vjp_kernel<3, false>);
    else
      rc = mass ? launch1(fem_batched::batched_onepass_vjp_kernel<2, true>)
                : launch1(fem_batched::batched_onepass_vjp_kernel<2, false>);
    if (rc) return rc;
    FEM_LAUNCH_CHECK("batched_onepass_vjp_kernel");
    return 0;
  }
  fem_batched::SumArgs sa{P.inc_ptr, P.inc, P.slot, P.indptr, P.nbfun_u,
                          std::max(1, P.max_row_nnz)};
  const int tU = fem::tuning_for(basis->family).sum_unroll >= 8 ? 8 : 4;
  auto launch = [&](auto kern, int L, int G) -> int {
    const int rpw = 32 / G;
    (void)L;
    const size_t smem = (size_t)(fem_batched::kBlock / 32) * rpw * sa.stride * sizeof(double);
    if (smem > 227 * 1024) {
      fem::set_error(FEM_ERR_CAPACITY, "a CSR row of %d entries needs more shared memory for "
                     "the batched kernel's row accumulators than a block has", sa.stride);
      return FEM_ERR_CAPACITY;
    }
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return fem::check_cuda(e, "batched kernel smem");
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern,
                                                                  fem_batched::kBlock, smem);
    if (e != cudaSuccess) return fem::check_cuda(e, "batched kernel occupancy");
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(
        (int64_t)std::max(1, per_sm) * fem::num_sms(), plan->nunits));
    kern<<<(unsigned)grid, fem_batched::kBlock, smem, st>>>(
        *mesh, *basis, *form, geo, sa, plan->unit_kind_mesh, plan->unit_begin, plan->unit_end,
        plan->nunits, plan->cell_units, counters, ref, staging, csr_values, w, u, dcoef_diff,
        dcoef_mass, status);
    return 0;
  };
#define FEM_BATCH_PICK(D, O, NB, G)                                                          \
  rc = tU == 8 ? launch(fem_batched::batched_forward_vjp_kernel<D, O, G, 8>, NB * NB, G)     \
               : launch(fem_batched::batched_forward_vjp_kernel<D, O, G, 4>, NB * NB, G);
  switch (basis->family) {
    case FEM_TRI_P1: FEM_BATCH_PICK(2, 1, 3, 4) break;
    case FEM_TRI_P2: FEM_BATCH_PICK(2, 2, 6, 8) break;
    case FEM_TET_P1: FEM_BATCH_PICK(3, 1, 4, 4) break;
    case FEM_TET_P2: FEM_BATCH_PICK(3, 2, 10, 16) break;
    default:
      fem::set_error(FEM_ERR_UNSUPPORTED, "the persistent batched kernel takes simplex families");
      return FEM_ERR_UNSUPPORTED;
  }
#undef FEM_BATCH_PICK
  if (rc) return rc;
  FEM_LAUNCH_CHECK("batched_forward_vjp_kernel");
  return 0;
}

}  // extern "C"
