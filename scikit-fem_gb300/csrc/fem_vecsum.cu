// One-pass assembly of the vector channel forms on simplex ElementVector
// bases (vector TriP1/P2, TetP1/P2: linear elasticity and its relatives).
//
// The reference builds each cell's (D*NS)^2 local matrix, then sums the COO
// triplets (bilinear_form.py:130-148, coo_data.py:27-36).  Here the local
// matrices are never stored: their D x D node blocks are contracted while
// the CSR entries are summed.
//
//   K_e[(i a)(j b)] = sum_{p,q} BB[i][j][p][q] E_pq[a][b]      (D x D block (i, j))
//
// with BB the element's exact reference tensor (fem_tables.cuh, at most 2 x 2
// vertex pairs per node pair) and E_pq the cell's pair blocks, computed per
// call from the coordinates and coefficients (vector_pair_blocks_kernel).
//
// Scalar TriP2 / TetP2 bases take the same path with D = 1: E_pq is then the
// number k_e |det| / d! grad(lambda_p) . grad(lambda_q) (scalar_pair_values)
// and a node block is one CSR entry.
//
// Work unit: one node block (I, J), I <= J, of the CSR (DOF D*node + a, the
// reference's interleaved numbering).  A lane owns a block, walks its
// contribution list -- the cells holding both nodes, ascending, each with
// its local pair (i, j) -- and accumulates the D*D entries in registers in
// that fixed order, then writes them to (I, J) and, transposed, to (J, I).
// Entries that the reference's eliminate_zeros left out of the pattern are
// skipped through the block's presence mask.  Lists are sliced 32 blocks at a
// time (code p of lane l at codes[(base + p) * 32 + l]), as the scalar
// one-pass sum's; they come from the upper lists of the node-level pattern.

#include "fem_common.cuh"
#include "fem_nodesum.cuh"
#include "fem_tables.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <vector>

namespace fem {

namespace {

int pair_index(int nv, int p, int q) { return p * nv - p * (p - 1) / 2 + (q - p); }

// terms[(i * ns + j) * kMaxTerms + t], count[i * ns + j]: the BB[i][j]
// terms of the element's reference tensor; mm[i * ns + j] its mass table.
// scalar: the pair values are numbers (E_qp = E_pq), so the terms of BB[i][j]
// on (p, q) and (q, p) are one term with the coefficients' sum (exact for
// the tables' coefficients, which are equal there).
int fill_terms(int family, int dim, bool scalar, std::vector<VecTerm>* terms,
               std::vector<int32_t>* count, std::vector<double>* mm) {
  const int ns = basis_nb_scalar(family);
  const int nv = dim + 1;
  terms->assign((size_t)ns * ns * kMaxTerms, VecTerm{0, 0, 0.0});
  count->assign((size_t)ns * ns, 0);
  mm->assign((size_t)ns * ns, 0.0);
  bool over = false;
  auto add = [&](int i, int j, int p, int q, double c) {
    int& n = (*count)[i * ns + j];
    if (scalar) {
      const int k = pair_index(nv, std::min(p, q), std::max(p, q));
      for (int t = 0; t < n; ++t) {
        VecTerm& tm = (*terms)[(size_t)(i * ns + j) * kMaxTerms + t];
        if (tm.k == k) {
          tm.c += c;
          return;
        }
      }
    }
    if (n >= kMaxTerms) {
      over = true;
      return;
    }
    const bool tr = p > q;
    (*terms)[(size_t)(i * ns + j) * kMaxTerms + n] =
        VecTerm{pair_index(nv, tr ? q : p, tr ? p : q), tr ? 1 : 0, c};
    ++n;
  };
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j < ns; ++j) {
#define VT(p, q, c) add(i, j, (p), (q), (c));
      if (family == FEM_TET_P2) {
        switch (i) {
          case 0: TET2BB_ROW0(j, VT) break;
          case 1: TET2BB_ROW1(j, VT) break;
          case 2: TET2BB_ROW2(j, VT) break;
          case 3: TET2BB_ROW3(j, VT) break;
          case 4: TET2BB_ROW4(j, VT) break;
          case 5: TET2BB_ROW5(j, VT) break;
          case 6: TET2BB_ROW6(j, VT) break;
          case 7: TET2BB_ROW7(j, VT) break;
          case 8: TET2BB_ROW8(j, VT) break;
          case 9: TET2BB_ROW9(j, VT) break;
          default: break;
        }
      } else if (family == FEM_TRI_P2) {
        switch (i) {
          case 0: TRI2BB_ROW0(j, VT) break;
          case 1: TRI2BB_ROW1(j, VT) break;
          case 2: TRI2BB_ROW2(j, VT) break;
          case 3: TRI2BB_ROW3(j, VT) break;
          case 4: TRI2BB_ROW4(j, VT) break;
          case 5: TRI2BB_ROW5(j, VT) break;
          default: break;
        }
      } else {
        // P1: grad phi_i = grad lambda_i, BB[i][j][p][q] = delta_ip delta_jq
        add(i, j, i, j, 1.0);
      }
#undef VT
    }
  if (over) {
    set_error(FEM_ERR_UNSUPPORTED, "more than %d reference-tensor terms per node pair", kMaxTerms);
    return FEM_ERR_UNSUPPORTED;
  }
  // the mass tables live in constant memory: read them back to the host
  const void* sym = family == FEM_TET_P2 ? (const void*)&c_tet2_mm
                    : family == FEM_TRI_P2 ? (const void*)&c_tri2_mm
                    : family == FEM_TET_P1 ? (const void*)&c_tet1_mm
                                           : (const void*)&c_tri1_mm;
  FEM_TRY_CUDA(cudaMemcpyFromSymbol(mm->data(), sym, (size_t)ns * ns * sizeof(double)));
  return 0;
}

// node[i][e] = element_dofs[D i][e] / D; *bad set when a cell's DOFs are not
// D consecutive numbers D*node + a per scalar node (the interleaved layout)
__global__ void node_dofs_kernel(const int32_t* __restrict__ udofs, int64_t nelems, int ns,
                                 int dim, int32_t* __restrict__ node, int32_t* __restrict__ bad) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nelems * ns) return;
  const int i = (int)(idx / nelems);
  const int64_t e = idx - (int64_t)i * nelems;
  const int32_t d0 = udofs[(int64_t)(dim * i) * nelems + e];
  bool ok = d0 >= 0 && d0 % dim == 0;
  for (int a = 1; a < dim; ++a) ok = ok && udofs[(int64_t)(dim * i + a) * nelems + e] == d0 + a;
  if (!ok) atomicOr(bad, 1);
  node[idx] = d0 / dim;
}

// first position of row r of the vector CSR with a column >= col
__device__ __forceinline__ int32_t row_lower_bound(const int32_t* __restrict__ indptr,
                                                   const int32_t* __restrict__ indices, int64_t r,
                                                   int32_t col) {
  int32_t lo = indptr[r], hi = indptr[r + 1];
  while (lo < hi) {
    const int32_t mid = (lo + hi) >> 1;
    if (indices[mid] < col) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The node blocks' layout: node rows in blocks of kBlockRows (the upper
// lists' row-block layout: each block's diagonal node blocks, then its
// others, so a cell's pair blocks are read in one sweep), and inside each
// block the diagonal node blocks, then each row's others, sorted by
// descending list length x terms -- the lanes of a slice carry about the
// same FP64 work and stay on neighbouring rows, whose node blocks share cells
// (their pair blocks hit L1) and whose values are written side by side.
// Sorting across rows evens the work further but loses that locality
// (measured at 384k cells: 1.71 ms per step sorting within each row, 1.74 /
// 1.86 / 1.90 ms across 8 / 64 / 512 rows, 1.80 ms unsorted).
constexpr int64_t kBlockRows = 512;

// Per node block u (natural order): its list length and the sort key of
// the work-sorted layout -- (segment << 32) | ~(length x terms); segment
// (b, 0) for row block b's diagonal node blocks, (b, 1 + r) for row r's
// others (r counted in the block): the natural order's ranges.
// by_terms (scalar bases, 1 x 1 blocks): segment (b, 1) for all of row
// block b's others, and the key's low word ordered by the terms per
// contribution (fewest first), then by descending length: the terms per
// contribution are fixed by the two nodes' kinds (vertex / edge), so the
// lanes of a slice add the same number of terms per step (measured at 1.3M
// TetP2 cells: 0.91 ms per step against 1.13 ms sorted by length x terms
// within each row; sorting within windows of 8 / 32 / 128 rows 1.02 / 0.95 /
// 0.96 ms; blocks of 2,048 / 8,192 rows 0.95 / 0.95 ms).
__global__ void block_work_kernel(const int32_t* __restrict__ slice_len,
                                  const int32_t* __restrict__ slice_base,
                                  const uint32_t* __restrict__ codes,
                                  const int32_t* __restrict__ urow,
                                  const int32_t* __restrict__ utpos, int64_t nupper,
                                  const int32_t* __restrict__ count, int npairs,
                                  int64_t block_rows, bool by_terms, int32_t* __restrict__ len, unsigned long long* __restrict__ key,
                                  int32_t* __restrict__ ident) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nupper) return;
  const int64_t sl = u >> 5;
  const uint32_t* cp = codes + (int64_t)slice_base[sl] * 32 + (u & 31);
  const int sl_len = slice_len[sl];
  int n = 0;
  while (n < sl_len && cp[(int64_t)n * 32] != 0xFFFFFFFFu) ++n;
  int nt = 1;
  if (n > 0) {
    const int ij = (int)(cp[0] & 127u);
    nt = ij < npairs ? max(1, count[ij]) : 1;
  }
  len[u] = n;
  const int64_t row = urow[u];
  const int64_t b = row / block_rows;
  const bool diag = utpos[u] < 0;
  ident[u] = (int32_t)u;
  if (by_terms) {
    const unsigned long long seg = (unsigned long long)(b * 2 + (diag ? 0 : 1));
    const unsigned long long lo = ((unsigned long long)min(nt, 15) << 28) |
                                  (0x0FFFFFFFull - (unsigned long long)min(n, 0x0FFFFFFF));
    key[u] = (seg << 32) | lo;
    return;
  }
  const unsigned long long seg =
      (unsigned long long)(b * (block_rows + 1) + (diag ? 0 : 1 + (row - b * block_rows)));
  const unsigned long long work = (unsigned long long)n * (unsigned long long)nt;
  key[u] = (seg << 32) | (0xFFFFFFFFull - (work > 0xFFFFFFFFull ? 0xFFFFFFFFull : work));
}

// Longest list of each slice of 32 slots of the sorted layout.
__global__ void sorted_slice_len_kernel(const int32_t* __restrict__ perm,
                                        const int32_t* __restrict__ len, int64_t nupper,
                                        int64_t nslices, int32_t* __restrict__ slice_len) {
  const int64_t sl = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sl >= nslices) return;
  const int64_t s = sl * 32 + lane;
  int v = s < nupper ? len[perm[s]] : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) slice_len[sl] = v;
}

// Every slot's list copied from its block's natural position.
__global__ void sorted_codes_kernel(const int32_t* __restrict__ perm,
                                    const int32_t* __restrict__ len,
                                    const int32_t* __restrict__ old_base,
                                    const uint32_t* __restrict__ old_codes,
                                    const int32_t* __restrict__ new_base, int64_t nupper,
                                    uint32_t* __restrict__ new_codes) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nupper) return;
  const int64_t u = perm[s];
  const uint32_t* src = old_codes + (int64_t)old_base[u >> 5] * 32 + (u & 31);
  uint32_t* dst = new_codes + (int64_t)new_base[s >> 5] * 32 + (s & 31);
  const int n = len[u];
  for (int p = 0; p < n; ++p) dst[(int64_t)p * 32] = src[(int64_t)p * 32];
}

// Per node block u = (I, J): the vector CSR position of each row's first
// entry in the block (vpos[a][u], rows D*I + a) and of the transposed
// block's (vposT[b][u], rows D*J + b; I < J), and the entries present
// (bit a*D + b).  *asym when the transposed block's entries differ.
__global__ void vec_block_pos_kernel(const int32_t* __restrict__ perm,
                                     const int32_t* __restrict__ urow,
                                     const int32_t* __restrict__ upos,
                                     const int32_t* __restrict__ nindices, int64_t nupper,
                                     int64_t nd, int dim, const int32_t* __restrict__ indptr,
                                     const int32_t* __restrict__ indices,
                                     int32_t* __restrict__ vpos, int32_t* __restrict__ vposT,
                                     uint16_t* __restrict__ vmask, int32_t* __restrict__ asym) {
  // u: the slot (the sorted layout's position); b0: its block's natural index
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nupper) return;
  const int64_t b0 = perm[u];
  const int64_t I = urow[b0];
  const int64_t J = nindices[upos[b0]];
  const bool off = I != J;
  unsigned mask = 0, maskT = 0;
  for (int a = 0; a < dim; ++a) {
    const int64_t r = dim * I + a;
    int32_t p = row_lower_bound(indptr, indices, r, (int32_t)(dim * J));
    vpos[a * nupper + u] = p;
    const int32_t end = indptr[r + 1];
    for (int b = 0; b < dim; ++b)
      if (p < end && indices[p] == (int32_t)(dim * J + b)) {
        mask |= 1u << (a * dim + b);
        ++p;
      }
  }
  if (off) {
    for (int b = 0; b < dim; ++b) {
      const int64_t r = dim * J + b;
      int32_t p = row_lower_bound(indptr, indices, r, (int32_t)(dim * I));
      vposT[b * nupper + u] = p;
      const int32_t end = indptr[r + 1];
      for (int a = 0; a < dim; ++a)
        if (p < end && indices[p] == (int32_t)(dim * I + a)) {
          maskT |= 1u << (a * dim + b);
          ++p;
        }
    }
    if (maskT != mask) atomicOr(asym, 1);
  } else {
    for (int b = 0; b < dim; ++b) vposT[b * nupper + u] = -1;
  }
  vmask[u] = (uint16_t)(mask | (off ? kOffDiagBit : 0u));
}

// The sum.  MASS: add m_e |det| / d! * MM[i][j] on the block diagonals.
// S: the spatial dimension (S + 1 vertices, the pair blocks' count); D: the
// block size (S for vector bases, 1 for scalar ones).  D = 1: per step a
// contribution's terms (predicated up to kMaxTerms) and its mass; FLAT: one
// FMA per step -- a term, or the mass after a contribution's terms -- with
// the next step's operand loaded before this one's FMA (the same FMAs in the
// same order, bitwise the same values; as fast once the lanes of a slice
// carry the same terms per contribution, at 37 against 32 registers).
// DYN: one wave of resident blocks whose warps take their slices in order
// from a ticket (*ticket, zero at launch) instead of a fixed grid stride:
// the slices in flight stay a narrow band of node rows (their cells' pair
// values shared in L2), and a warp with a long slice does not hold up the
// others.  Each slice's sums are the same whichever warp runs it.
template <int S, int D, bool MASS, bool FLAT = false, bool DYN = false>
__global__ void __launch_bounds__(128) vec_upper_kernel(
    int64_t ua, int64_t ub, int64_t nupper, int64_t nd, int64_t nelems, int ns,
    const int32_t* __restrict__ slice_len,
    const int32_t* __restrict__ slice_base, const uint32_t* __restrict__ codes,
    const int32_t* __restrict__ vpos, const int32_t* __restrict__ vposT,
    const uint16_t* __restrict__ vmask, const VecTerm* __restrict__ terms_g,
    const int32_t* __restrict__ count_g, const double* __restrict__ mm_g,
    const double* __restrict__ E, double* __restrict__ vals,
    int32_t* __restrict__ ticket = nullptr, int chunk = 1) {
  constexpr int DD = D * D;
  constexpr int NP = (S + 1) * (S + 2) / 2;
  constexpr int R = NP * DD + 1;
  __shared__ VecTerm terms[kMaxNodePairs * kMaxTerms];
  __shared__ int32_t count[kMaxNodePairs];
  __shared__ double mm[kMaxNodePairs];
  const int npairs = ns * ns;
  for (int k = threadIdx.x; k < npairs * kMaxTerms; k += blockDim.x) terms[k] = terms_g[k];
  for (int k = threadIdx.x; k < npairs; k += blockDim.x) {
    count[k] = count_g[k];
    mm[k] = mm_g[k];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t s1 = (ub + 31) >> 5;
  // the warp's next slice (warp-uniform); without a ticket the fixed
  // grid stride
  // grid stride.  A ticket hands out `chunk` consecutive slices.
  const bool dyn = DYN && ticket != nullptr;
  int64_t chunk_end = 0;
  auto next_slice = [&](int64_t cur) -> int64_t {
    if (dyn) {
      if (cur + 1 < chunk_end) return cur + 1;
      int t = 0;
      if (lane == 0) t = atomicAdd(ticket, 1);
      const int64_t b = (ua >> 5) + (int64_t)__shfl_sync(0xffffffffu, t, 0) * chunk;
      chunk_end = b + chunk;
      return b;
    }
    return cur + warps;
  };
  const int64_t first =
      dyn ? next_slice(-1) : (ua >> 5) + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int64_t sl = first; sl < s1; sl = next_slice(sl)) {
    const int64_t u = sl * 32 + lane;
    // a lane whose block belongs to the neighbouring range takes part in
    // the warp's votes with an empty list and writes nothing
    const bool inr = u >= ua && u < ub;
    const int len = inr ? slice_len[sl] : 0;
    const uint32_t* cp = codes + (int64_t)slice_base[sl] * 32 + lane;
    if constexpr (D == 1 && !FLAT) {
      scalar_entry_sum<S, MASS, false>(inr, u, len, cp, nelems, npairs, terms, count, mm, vpos,
                                       vposT, vmask, E, vals);
      continue;
    }
    double acc[DD];
#pragma unroll
    for (int q = 0; q < DD; ++q) acc[q] = 0.0;
    // One loop over (contribution, term) steps: a lane moves to its next
    // contribution as soon as it has done the current one's terms, so the
    // warp runs max over its lanes of (list length x terms) steps, not
    // (longest list) x (most terms).  Per contribution: its terms, then its
    // mass, in that order.
    uint32_t cur = len > 0 ? __ldg(cp) : 0xFFFFFFFFu;
    uint32_t nxt = len > 1 ? __ldg(cp + 32) : 0xFFFFFFFFu;
    int p = 0, t = 0, nt = 0, ij = 0;
    bool valid = false;
    const double* Eb = E;
    auto decode = [&]() {
      const int64_t e = cur >> 7;
      ij = (int)(cur & 127u);
      valid = e < nelems && ij < npairs;   // never false for the lists this file builds
      nt = valid ? count[ij] : 0;
      Eb = E + (valid ? e : 0) * R;
    };
    bool live = cur != 0xFFFFFFFFu;        // this lane's list is not done
    if (live) decode();
    if constexpr (D == 1 && FLAT) {
      // One FMA per step, software-pipelined: the next step's operand is
      // loaded before this step's FMA, so that a lane has two gathers in
      // flight.  Steps: each contribution's terms, then its mass.
      auto advance = [&]() {
        t = 0;
        ++p;
        cur = nxt;
        nxt = p + 1 < len ? __ldg(cp + (int64_t)(p + 1) * 32) : 0xFFFFFFFFu;
        live = cur != 0xFFFFFFFFu;
        if (live) decode();
      };
      // the lane's next step (false: its list is done); a null operand
      // address is a step without an FMA (a contribution without terms or
      // mass, or a code out of range)
      auto fetch = [&](double& c, const double*& a) -> bool {
        if (!live) return false;
        a = nullptr;
        if (valid && t < nt) {
          const VecTerm tm = terms[ij * kMaxTerms + t];
          c = tm.c;
          a = Eb + tm.k;
          if (++t >= nt && !MASS) advance();
          return true;
        }
        if (MASS && valid) {
          c = mm[ij];
          a = Eb + NP;
        }
        advance();
        return true;
      };
      double ca = 0.0, va = 0.0;
      const double* aa = nullptr;
      bool ha = fetch(ca, aa);
      if (ha && aa) va = __ldg(aa);
      while (__any_sync(0xffffffffu, ha)) {
        double cb = 0.0, vb = 0.0;
        const double* ab = nullptr;
        const bool hb = fetch(cb, ab);
        if (hb && ab) vb = __ldg(ab);
        if (ha && aa) acc[0] = __fma_rn(ca, va, acc[0]);
        ca = cb;
        va = vb;
        aa = ab;
        ha = hb;
      }
    }
    while (!(D == 1 && FLAT) && __any_sync(0xffffffffu, live)) {
      if (live) {
        if (t < nt) {
          const VecTerm tm = terms[ij * kMaxTerms + t];
          const double* Ep = Eb + tm.k * DD;
          double v[DD];
#pragma unroll
          for (int q = 0; q < DD; ++q) v[q] = __ldg(Ep + q);
          if (tm.tr) {
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
              for (int b = a + 1; b < D; ++b) {
                const double x = v[a * D + b];
                v[a * D + b] = v[b * D + a];
                v[b * D + a] = x;
              }
          }
#pragma unroll
          for (int q = 0; q < DD; ++q) acc[q] = __fma_rn(tm.c, v[q], acc[q]);
          ++t;
        }
        if (t >= nt) {
          if (MASS && valid) {
            const double sm = __ldg(Eb + NP * DD);
            const double mv = mm[ij];
#pragma unroll
            for (int a = 0; a < D; ++a) acc[a * D + a] = __fma_rn(sm, mv, acc[a * D + a]);
          }
          t = 0;
          ++p;
          cur = nxt;
          nxt = p + 1 < len ? __ldg(cp + (int64_t)(p + 1) * 32) : 0xFFFFFFFFu;   // one code ahead
          live = cur != 0xFFFFFFFFu;
          if (live) decode();
        }
      }
    }
    if (inr) {
      const unsigned mk = vmask[u];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        int32_t pos = vpos[a * nupper + u];
#pragma unroll
        for (int b = 0; b < D; ++b)
          if ((mk >> (a * D + b)) & 1u) vals[pos++] = acc[a * D + b];
      }
      if (mk & kOffDiagBit) {
#pragma unroll
        for (int b = 0; b < D; ++b) {
          int32_t pos = vposT[b * nupper + u];
#pragma unroll
          for (int a = 0; a < D; ++a)
            if ((mk >> (a * D + b)) & 1u) vals[pos++] = acc[a * D + b];
        }
      }
    }
  }
}

// The same sum with the D*D lanes of a node block's entries cooperating:
// 32 / (D*D) blocks per warp, lane (a, b) of a block accumulates entry
// (a, b) over the block's cells -- one coalesced load of the cell's pair
// block per term for the block, where the lane-per-block form issues D*D
// scattered loads per lane.  Same terms in the same order per entry: the
// values are bitwise those of vec_upper_kernel.
template <int D, bool MASS>
__global__ void __launch_bounds__(128) vec_upper_coop_kernel(
    int64_t ua, int64_t ub, int64_t nupper, int64_t nd, int64_t nelems, int ns,
    const int32_t* __restrict__ slice_len, const int32_t* __restrict__ slice_base,
    const uint32_t* __restrict__ codes, const int32_t* __restrict__ vpos,
    const int32_t* __restrict__ vposT, const uint16_t* __restrict__ vmask,
    const VecTerm* __restrict__ terms_g, const int32_t* __restrict__ count_g,
    const double* __restrict__ mm_g, const double* __restrict__ E, double* __restrict__ vals) {
  constexpr int DD = D * D;
  constexpr int BPW = 32 / DD;   // node blocks per warp
  constexpr int NP = (D + 1) * (D + 2) / 2;
  constexpr int R = NP * DD + 1;
  __shared__ VecTerm terms[kMaxNodePairs * kMaxTerms];
  __shared__ int32_t count[kMaxNodePairs];
  __shared__ double mm[kMaxNodePairs];
  const int npairs = ns * ns;
  for (int k = threadIdx.x; k < npairs * kMaxTerms; k += blockDim.x) terms[k] = terms_g[k];
  for (int k = threadIdx.x; k < npairs; k += blockDim.x) {
    count[k] = count_g[k];
    mm[k] = mm_g[k];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int sub = lane / DD;            // block of the warp
  const int q = lane - sub * DD;        // entry of the block
  const int a = q / D, b = q - a * D;
  const int qt = b * D + a;             // the entry's position in a transposed pair block
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int64_t u0 = ua + gw * BPW; u0 < ub; u0 += nwarps * BPW) {
    const int64_t u = u0 + sub;
    if (sub >= BPW || u >= ub) continue;
    const int len = slice_len[u >> 5];
    const uint32_t* cp = codes + (int64_t)slice_base[u >> 5] * 32 + (u & 31);
    double acc = 0.0;
    uint32_t next = len > 0 ? __ldg(cp) : 0xFFFFFFFFu;
    for (int p = 0; p < len; ++p) {
      const uint32_t code = next;
      if (code == 0xFFFFFFFFu) break;                               // the block's list ended
      if (p + 1 < len) next = __ldg(cp + (int64_t)(p + 1) * 32);    // one code ahead
      const int64_t e = code >> 7;
      const int ij = (int)(code & 127u);
      if (e >= nelems || ij >= npairs) continue;   // never for the lists this file builds
      const double* Eb = E + e * R;
      const int nt = count[ij];
      for (int t = 0; t < nt; ++t) {
        const VecTerm tm = terms[ij * kMaxTerms + t];
        acc = __fma_rn(tm.c, __ldg(Eb + tm.k * DD + (tm.tr ? qt : q)), acc);
      }
      if (MASS && a == b) acc = __fma_rn(__ldg(Eb + NP * DD), mm[ij], acc);
    }
    const unsigned mk = vmask[u];
    if ((mk >> q) & 1u) {
      const unsigned row = (mk >> (a * D)) & ((1u << D) - 1u);
      vals[vpos[a * nupper + u] + __popc(row & ((1u << b) - 1u))] = acc;
      if (mk & kOffDiagBit) {
        unsigned col = 0;
#pragma unroll
        for (int a2 = 0; a2 < D; ++a2) col |= ((mk >> (a2 * D + b)) & 1u) << a2;
        vals[vposT[b * nupper + u] + __popc(col & ((1u << a) - 1u))] = acc;
      }
    }
  }
}

}  // namespace

void free_vec_upper(VecUpper* V) {
  if (!V) return;
  free_upper_lists(&V->U);
  cudaFree(V->vpos);
  cudaFree(V->vposT);
  cudaFree(V->vmask);
  cudaFree(V->terms);
  cudaFree(V->count);
  cudaFree(V->mm);
  *V = VecUpper();
}

int build_vec_upper(const Pattern& P, const int32_t* udofs, int family, int dim, VecUpper* V,
                    cudaStream_t st) {
  *V = VecUpper();
  const int ns = basis_nb_scalar(family);
  const int sdim = basis_dim(family);
  if ((sdim != 2 && sdim != 3) || (dim != 1 && dim != sdim) || ns <= 0 || ns > 10 ||
      P.nbfun_u != dim * ns || P.nbfun_v != dim * ns || !P.has_matrix || P.nrows % dim) {
    set_error(FEM_ERR_UNSUPPORTED, "one-pass node-block sum: not a simplex pattern");
    return FEM_ERR_UNSUPPORTED;
  }
  V->dim = dim;
  V->sdim = sdim;
  V->ns = ns;
  V->nelems = P.nelems;
  const int64_t nelems = P.nelems, nnodes = P.nrows / dim;
  std::vector<VecTerm> terms;
  std::vector<int32_t> count;
  std::vector<double> mm;
  int rc = fill_terms(family, sdim, dim == 1, &terms, &count, &mm);
  if (rc) return rc;
  auto fail = [&](int code) {
    free_vec_upper(V);
    return code;
  };
  // node-level pattern: every pair of nodes sharing a cell
  Pattern N;
  AsyncScratch scratch(st);
  int32_t *node = nullptr, *flag = nullptr;
  FEM_TRY_CUDA(scratch.alloc(&node, std::max<int64_t>(1, nelems * ns) * sizeof(int32_t)));
  FEM_TRY_CUDA(scratch.alloc(&flag, sizeof(int32_t)));
  FEM_TRY_CUDA(cudaMemsetAsync(flag, 0, sizeof(int32_t), st));
  if (nelems > 0) {
    node_dofs_kernel<<<(unsigned)ceil_div(nelems * ns, 256), 256, 0, st>>>(udofs, nelems, ns, dim,
                                                                           node, flag);
    FEM_LAUNCH_CHECK("node_dofs_kernel");
  }
  int32_t h = 0;
  FEM_TRY_CUDA(cudaMemcpyAsync(&h, flag, sizeof(h), cudaMemcpyDeviceToHost, st));
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  if (h) {
    set_error(FEM_ERR_UNSUPPORTED, "one-pass node-block sum: DOFs are not interleaved by node");
    return FEM_ERR_UNSUPPORTED;
  }
  rc = build_incidence(node, nelems, ns, nnodes, &N, st);
  if (!rc) rc = build_csr(node, ns, nnodes, nullptr, &N, st);
  V->block_rows = kBlockRows;
  if (!rc) rc = build_upper_lists(N, &V->U, st, /*wide=*/true, V->block_rows);
  if (rc) {
    free_pattern(new Pattern(N));   // releases N's device arrays
    return fail(rc);
  }
  const int64_t nu = V->U.nupper;
  cudaError_t e = cudaMalloc(&V->vpos, std::max<int64_t>(1, nu * dim) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&V->vposT, std::max<int64_t>(1, nu * dim) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&V->vmask, std::max<int64_t>(1, nu) * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&V->terms, terms.size() * sizeof(VecTerm));
  if (e == cudaSuccess) e = cudaMalloc(&V->count, count.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&V->mm, mm.size() * sizeof(double));
  if (e != cudaSuccess) {
    free_pattern(new Pattern(N));   // releases N's device arrays
    return fail(check_cuda(e, "cudaMalloc(vector one-pass lists)"));
  }
  e = cudaMemcpyAsync(V->terms, terms.data(), terms.size() * sizeof(VecTerm),
                      cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(V->count, count.data(), count.size() * sizeof(int32_t),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(V->mm, mm.data(), mm.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    free_pattern(new Pattern(N));   // releases N's device arrays
    return fail(check_cuda(e, "vector one-pass tables"));
  }
  // The work-sorted layout: inside each window of node rows (its diagonal
  // blocks, then its blocks above the diagonal) the blocks are ordered by
  // descending list length x terms, so that a slice's 32 lanes carry about
  // the same FP64 work (the lanes of a warp share the FP64 pipe's issue).
  // perm[slot] = the block's natural index; a window's slots stay its range.
  int32_t* perm = nullptr;
  if (nu > 0) {
    int32_t *len = nullptr, *ident = nullptr;
    unsigned long long *key = nullptr, *key2 = nullptr;
    e = scratch.alloc(&len, nu * sizeof(int32_t));
    if (e == cudaSuccess) e = scratch.alloc(&ident, nu * sizeof(int32_t));
    if (e == cudaSuccess) e = scratch.alloc(&perm, nu * sizeof(int32_t));
    if (e == cudaSuccess) e = scratch.alloc(&key, nu * sizeof(unsigned long long));
    if (e == cudaSuccess) e = scratch.alloc(&key2, nu * sizeof(unsigned long long));
    if (e == cudaSuccess) {
      block_work_kernel<<<(unsigned)ceil_div(nu, 256), 256, 0, st>>>(
          V->U.slice_len, V->U.slice_base, V->U.codes, V->U.row, V->U.tpos, nu, V->count,
          ns * ns, V->block_rows, dim == 1, len, key, ident);
      e = cudaGetLastError();
    }
    size_t tmp_bytes = 0;
    void* tmp = nullptr;
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key, key2, ident, perm, nu, 0, 64,
                                          st);
    if (e == cudaSuccess) e = scratch.alloc(&tmp, std::max<size_t>(1, tmp_bytes));
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key2, ident, perm, nu, 0, 64, st);
    // slices of the sorted slots, and their codes
    int32_t *nlen = nullptr, *nbase = nullptr;
    uint32_t* ncodes = nullptr;
    const int64_t nsl = V->U.nslices;
    if (e == cudaSuccess) e = cudaMalloc(&nlen, (nsl + 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&nbase, (nsl + 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(nlen, 0, (nsl + 1) * sizeof(int32_t), st);
    if (e == cudaSuccess) {
      sorted_slice_len_kernel<<<(unsigned)ceil_div(nsl * 32, 256), 256, 0, st>>>(perm, len, nu,
                                                                                 nsl, nlen);
      e = cudaGetLastError();
    }
    int64_t rows32 = 0;
    if (e == cudaSuccess) {
      rc = exclusive_scan_i32(nlen, nbase, nsl, &rows32, st);
      if (rc) e = cudaErrorUnknown;
    }
    if (e == cudaSuccess && rows32 * 32 >= INT32_MAX) e = cudaErrorInvalidValue;
    if (e == cudaSuccess) e = cudaMalloc(&ncodes, std::max<int64_t>(1, rows32 * 32) * sizeof(uint32_t));
    if (e == cudaSuccess)
      e = cudaMemsetAsync(ncodes, 0xFF, std::max<int64_t>(1, rows32 * 32) * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
      sorted_codes_kernel<<<(unsigned)ceil_div(nu, 256), 256, 0, st>>>(
          perm, len, V->U.slice_base, V->U.codes, nbase, nu, ncodes);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaFree(nlen);
      cudaFree(nbase);
      cudaFree(ncodes);
      free_pattern(new Pattern(N));   // releases N's device arrays
      return fail(rc ? rc : check_cuda(e, "work-sorted node blocks"));
    }
    cudaFree(V->U.slice_len);
    cudaFree(V->U.slice_base);
    cudaFree(V->U.codes);
    V->U.slice_len = nlen;
    V->U.slice_base = nbase;
    V->U.codes = ncodes;
    V->U.ncodes = rows32 * 32;
  }
  e = cudaMemsetAsync(flag, 0, sizeof(int32_t), st);
  if (e == cudaSuccess && nu > 0) {
    vec_block_pos_kernel<<<(unsigned)ceil_div(nu, 256), 256, 0, st>>>(
        perm, V->U.row, V->U.pos, N.indices, nu, V->U.nd, dim, P.indptr, P.indices, V->vpos,
        V->vposT, V->vmask, flag);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  free_pattern(new Pattern(N));   // releases N's device arrays
  if (e != cudaSuccess) return fail(check_cuda(e, "vec_block_pos_kernel"));
  if (h) {
    set_error(FEM_ERR_UNSUPPORTED, "one-pass node-block sum: the CSR pattern is not block-symmetric");
    return fail(FEM_ERR_UNSUPPORTED);
  }
  // the node-level CSR positions, rows and transposes are build-time only
  cudaFree(V->U.pos);
  cudaFree(V->U.tpos);
  cudaFree(V->U.row);
  V->U.pos = V->U.tpos = V->U.row = nullptr;
  return 0;
}

int64_t vec_window_rows(const VecUpper& V) { return V.block_rows * V.dim; }

// Slices per ticket of the scalar (1 x 1 block) sums, and the resident
// waves of work from which the node-block sums take their slices from a
// ticket.
constexpr int kScalarChunk = 4;
constexpr int kTicketWaves = 8;

int vec_upper_sum(const VecUpper& V, const double* E, bool mass, double* vals, cudaStream_t st,
                  int64_t row0, int64_t row1, bool coop) {
  if (V.U.nupper == 0) return 0;
  const int64_t nnodes = (int64_t)V.U.dpos_h.size() - 1;
  // node rows [n0, n1) of DOF rows [row0, row1) (multiples of dim; window
  // boundaries of the work-sorted layout, or the last row)
  int64_t n0 = row0 < 0 ? 0 : row0 / V.dim;
  int64_t n1 = (row1 < 0 || row1 / V.dim > nnodes) ? nnodes : row1 / V.dim;
  if (n1 <= n0) return 0;
  if ((n0 % V.block_rows) || ((n1 % V.block_rows) && n1 != nnodes)) {
    set_error(FEM_ERR_ARGUMENT, "vector one-pass rows [%lld, %lld) off the %lld-row blocks",
              (long long)row0, (long long)row1, (long long)(V.block_rows * V.dim));
    return FEM_ERR_ARGUMENT;
  }
  // the node rows' blocks: one range of the row-block layout
  const int64_t ranges[2][2] = {
      {(int64_t)V.U.dpos_h[n0] + V.U.opos_h[n0], (int64_t)V.U.dpos_h[n1] + V.U.opos_h[n1]},
      {0, 0}};
  const int threads = 128;
  for (int k = 0; k < 2; ++k) {
    const int64_t ua = ranges[k][0], ub = ranges[k][1];
    if (ub <= ua) continue;
    const int64_t nsl = ((ub + 31) >> 5) - (ua >> 5);
    // lane per block: a warp per slice of 32 blocks; cooperative: 32 / D^2 blocks per warp
    const int64_t nwarp = (coop && V.dim > 1) ? ceil_div(ub - ua, 32 / (V.dim * V.dim)) : nsl;
    // (lane per block and the scalar forms: one resident wave taking slices
    // from a ticket -- vector TetP2 elasticity on 384k cells 1.43 against
    // 1.62 ms, scalar TetP2 on 1.3M cells 0.83 against 0.91 ms; the vector
    // cooperative form: a grid of 32 blocks per SM, the block scheduler
    // evening out the slices' uneven work)
    const int64_t work = ceil_div(nwarp, threads / 32);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(work, (int64_t)num_sms() * 32));
    auto launch_coop = [&](auto kern) {
      kern<<<grid, threads, 0, st>>>(ua, ub, V.U.nupper, V.U.nd, V.nelems, V.ns, V.U.slice_len,
                                     V.U.slice_base, V.U.codes, V.vpos, V.vposT, V.vmask,
                                     static_cast<const VecTerm*>(V.terms), V.count, V.mm, E, vals);
    };
    auto launch = [&](auto kern) {
      kern<<<grid, threads, 0, st>>>(ua, ub, V.U.nupper, V.U.nd, V.nelems, V.ns, V.U.slice_len,
                                     V.U.slice_base, V.U.codes, V.vpos, V.vposT, V.vmask,
                                     static_cast<const VecTerm*>(V.terms), V.count, V.mm, E, vals,
                                     nullptr, 1);
    };
    // the slices' ticket: the word after the pair values in the caller's
    // staging (nelems x nbfun^2 doubles, always longer than the pair values'
    // nelems x vec_pair_stride), so concurrent calls with their own staging
    // never share it and nothing is allocated
    int32_t* ticket =
        reinterpret_cast<int32_t*>(const_cast<double*>(E) + V.nelems * vec_pair_stride(V.sdim, V.dim));
    // (the ticket pays where the slices' cells do not fit L2 at once; work
    // of at most kTicketWaves resident waves -- a mesh of up to about 200k
    // TriP2 cells -- keeps the oversubscribed grid, which the block
    // scheduler balances: 512 per-mesh TriP2 launches 21.0 ms that way,
    // 23.4 ms with the ticket from one wave up)
    auto launch_dyn = [&](auto kern, int chunk) -> int {
      const int g = resident_grid(kern, threads, 0, work);
      if (work <= (int64_t)g * kTicketWaves) {
        launch(kern);
        const cudaError_t le = cudaGetLastError();
        return le == cudaSuccess ? 0 : check_cuda(le, "vec_upper_kernel");
      }
      cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(int32_t), st);
      if (e == cudaSuccess) {
        kern<<<g, threads, 0, st>>>(ua, ub, V.U.nupper, V.U.nd, V.nelems, V.ns, V.U.slice_len,
                                    V.U.slice_base, V.U.codes, V.vpos, V.vposT, V.vmask,
                                    static_cast<const VecTerm*>(V.terms), V.count, V.mm, E, vals,
                                    ticket, chunk);
        e = cudaGetLastError();
      }
      return e == cudaSuccess ? 0 : check_cuda(e, "vec_upper_kernel");
    };
    int rc = 0;
    if (V.dim == 1) {
      // scalar bases: one entry per node block
      // (coop: the flattened form, one FMA per step)
      // (four slices per ticket: a scalar entry's slice is little work, and
      // one ticket per slice serialised the ~8M slices of 512 TriP2 meshes
      // on the counter)
      if (V.sdim == 3) {
        if (coop) {
          if (mass) rc = launch_dyn(vec_upper_kernel<3, 1, true, true, true>, kScalarChunk);
          else rc = launch_dyn(vec_upper_kernel<3, 1, false, true, true>, kScalarChunk);
        } else {
          if (mass) rc = launch_dyn(vec_upper_kernel<3, 1, true, false, true>, kScalarChunk);
          else rc = launch_dyn(vec_upper_kernel<3, 1, false, false, true>, kScalarChunk);
        }
      } else {
        if (coop) {
          if (mass) rc = launch_dyn(vec_upper_kernel<2, 1, true, true, true>, kScalarChunk);
          else rc = launch_dyn(vec_upper_kernel<2, 1, false, true, true>, kScalarChunk);
        } else {
          if (mass) rc = launch_dyn(vec_upper_kernel<2, 1, true, false, true>, kScalarChunk);
          else rc = launch_dyn(vec_upper_kernel<2, 1, false, false, true>, kScalarChunk);
        }
      }
    } else if (coop) {
      if (V.dim == 3) {
        if (mass) launch_coop(vec_upper_coop_kernel<3, true>);
        else launch_coop(vec_upper_coop_kernel<3, false>);
      } else {
        if (mass) launch_coop(vec_upper_coop_kernel<2, true>);
        else launch_coop(vec_upper_coop_kernel<2, false>);
      }
    } else if (V.dim == 3) {
      if (mass) rc = launch_dyn(vec_upper_kernel<3, 3, true, false, true>, 1);
      else rc = launch_dyn(vec_upper_kernel<3, 3, false, false, true>, 1);
    } else {
      if (mass) rc = launch_dyn(vec_upper_kernel<2, 2, true, false, true>, 1);
      else rc = launch_dyn(vec_upper_kernel<2, 2, false, false, true>, 1);
    }
    if (rc) return rc;
    FEM_LAUNCH_CHECK("vec_upper_kernel");
  }
  return 0;
}

}  // namespace fem
