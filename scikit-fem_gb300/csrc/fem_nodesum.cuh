// The one-pass node-block sum's shared pieces: the reference-tensor term
// records and the per-lane walk of one CSR entry (1 x 1 node block, scalar
// TriP2 / TetP2 bases), used by the sum kernel (fem_vecsum.cu) and by the
// batched persistent kernel's row-block units (fem_batched.cu).
#pragma once

#include "fem_common.cuh"

namespace fem {

constexpr int kMaxTerms = 4;
// vmask bit of a node block off the diagonal (its transpose is written too)
constexpr unsigned kOffDiagBit = 1u << 15;
// node pairs of the largest element (10 scalar functions)
constexpr int kMaxNodePairs = 100;

struct VecTerm {
  int32_t k;    // pair index of (min(p,q), max(p,q)) in row-major upper order
  int32_t tr;   // 1: the term reads E_qp transposed (p > q)
  double c;
};

// One lane of a warp walking the contribution list of its CSR entry u (a
// slot of the lists' slice layout; inr false: a lane of the neighbouring
// range, which takes part in the warp's votes with an empty list and writes
// nothing): per contribution (cell e, local pair ij), ascending e, the
// pair's reference-tensor terms c * E[e][k] (at most kMaxTerms, predicated)
// and, with MASS, its mass term E[e][NP] * mm[ij]; then the entry and its
// transpose are written through the entry's presence mask.  terms / count /
// mm are the element's tables (shared memory).  COHERENT: E was written in
// the same launch (loads through L2, not the read-only path).
template <int S, bool MASS, bool COHERENT>
__device__ __forceinline__ void scalar_entry_sum(
    bool inr, int64_t u, int len, const uint32_t* __restrict__ cp,
    int64_t nelems, int npairs, const VecTerm* terms, const int32_t* count, const double* mm,
    const int32_t* __restrict__ vpos, const int32_t* __restrict__ vposT,
    const uint16_t* __restrict__ vmask, const double* __restrict__ E,
    double* __restrict__ vals) {
  constexpr int NP = (S + 1) * (S + 2) / 2;
  constexpr int R = NP + 1;
  auto ldE = [&](const double* p) { return COHERENT ? __ldcg(p) : __ldg(p); };
  double acc = 0.0;
  uint32_t cur = len > 0 ? __ldg(cp) : 0xFFFFFFFFu;
  uint32_t nxt = len > 1 ? __ldg(cp + 32) : 0xFFFFFFFFu;
  int p = 0, nt = 0, ij = 0;
  bool valid = false;
  const double* Eb = E;
  auto decode = [&]() {
    const int64_t e = cur >> 7;
    ij = (int)(cur & 127u);
    valid = e < nelems && ij < npairs;   // never false for lists built by build_vec_upper
    nt = valid ? count[ij] : 0;
    Eb = E + (valid ? e : 0) * R;
  };
  bool live = cur != 0xFFFFFFFFu;
  if (live) decode();
  while (__any_sync(0xffffffffu, live)) {
    if (live) {
#pragma unroll
      for (int t = 0; t < kMaxTerms; ++t)
        if (t < nt) {
          const VecTerm tm = terms[ij * kMaxTerms + t];
          acc = __fma_rn(tm.c, ldE(Eb + tm.k), acc);
        }
      if (MASS && valid) acc = __fma_rn(ldE(Eb + NP), mm[ij], acc);
      ++p;
      cur = nxt;
      nxt = p + 1 < len ? __ldg(cp + (int64_t)(p + 1) * 32) : 0xFFFFFFFFu;   // one code ahead
      live = cur != 0xFFFFFFFFu;
      if (live) decode();
    }
  }
  if (inr) {
    const unsigned mk = vmask[u];
    if (mk & 1u) {
      vals[vpos[u]] = acc;
      if (mk & kOffDiagBit) vals[vposT[u]] = acc;
    }
  }
}

}  // namespace fem
