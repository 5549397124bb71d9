// Exact-zero mask of the pattern build: the reference's arithmetic, replayed.
//
// eliminate_zeros (coo_data.py:34-35) drops every local entry the reference
// computes as exactly 0.0.  For entries whose true value is far from zero
// any accurate evaluation agrees; for mathematically-zero entries the
// reference's result is rounding noise that lands on 0.0 or not depending
// on the exact sequence of floating-point operations.  This kernel replays
// that sequence for such entries -- only for them: candidates are entries
// whose accurately computed value is below 1e-9 of the element's largest
// entry -- so the CSR pattern matches the reference's bit for bit:
//
//   quadrature   the reference's own nodes and weights (fem_refquad.cuh)
//   lbasis       element_tri_p1.py:18-33, element_tri_p2.py:22-48,
//                element_tet_p1.py:19-45, element_tet_p2.py:26-103,
//                element_hex1.py:23-69, with their operation order
//   mapping      mapping_affine.py:55-131 (A, detA, invA = cofactor / detA),
//                mapping_isoparametric.py:112-226 (J accumulated node by
//                node from 0, detDF, invDF = cofactor / detDF)
//   gbasis       element_h1.py:17: grad_j = sum_i invDF[i][j] dphi[i], in i
//                order; ElementVector zero-pads the other components
//   form         the traced program (tracer.trace_tape) in the form's own
//                operation order
//   dx, sum      |detDF| * W, form * dx, then numpy's pairwise sum over the
//                quadrature points (bilinear_form.py:150-151)
//
// Every operation is a separately rounded IEEE double operation: this file
// is compiled with -fmad=false.

#include "fem_common.cuh"
#include "fem_refquad.cuh"

#include "fem_faithful_core.cuh"
#include "fem_program_kernel.cuh"
#include "fem_jit.h"

#include <type_traits>
#include <vector>

namespace fem_faithful {

__device__ bool rule_for(int refdim, bool hex, int nq, Rule& r) {
  if (hex) {
    if (nq != 64) return false;
    r = {c_rq_hex6_X, c_rq_hex6_W, 64};
    return true;
  }
  if (refdim == 2) {
    if (nq == 3) { r = {c_rq_tri2_X, c_rq_tri2_W, 3}; return true; }
    if (nq == 6) { r = {c_rq_tri4_X, c_rq_tri4_W, 6}; return true; }
    return false;
  }
  if (nq == 4) { r = {c_rq_tet2_X, c_rq_tet2_W, 4}; return true; }
  if (nq == 11) { r = {c_rq_tet4_X, c_rq_tet4_W, 11}; return true; }
  return false;
}

template <int D>
__global__ void mask_kernel(FemMesh m, FemBasis b, FemProgram prog, int nq, double tau,
                            double* __restrict__ local, int32_t* __restrict__ status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  Rule rule;
  if (prog.qX && prog.qW) {
    rule = {prog.qX, prog.qW, prog.nq};
  } else if (!rule_for(D, b.family == FEM_HEX_1, nq, rule)) {
    atomicOr(status, 1 << FEM_ERR_UNSUPPORTED);
    return;
  }
  const int NB = b.nbfun;
  double* Ke = local + e * (int64_t)NB * NB;
  double scale = 0.0;
  for (int k = 0; k < NB * NB; ++k) scale = fmax(scale, fabs(Ke[k]));
  double R[kMaxProgram];
  double vals[kMaxPoints];
  for (int i = 0; i < NB; ++i) {      // test function (row)
    for (int j = 0; j < NB; ++j) {    // trial function (column)
      const double v = Ke[i * NB + j];
      if (fabs(v) > tau * scale) continue;
      const double s = replay_entry<D>(m, b, prog, rule, e, i, j, R, vals);
      // the buffer only feeds the mask: mark exact zeros / noise nonzeros
      Ke[i * NB + j] = (s == 0.0) ? 0.0 : (v != 0.0 ? v : 1e-300);
    }
  }
}

// ------------------------------------------------------------ generic forms
template <int D, int MODE, bool FACET, bool VEC, bool VECU>
__global__ void program_kernel(FemMesh m, FemBasis b, FemBasis bu, FemFacets fc, FemProgram prog,
                               Rule rule, GenericLayout s, int64_t ncells,
                               double* __restrict__ out, int32_t* __restrict__ status) {
  program_body<D, MODE, FACET, VEC, VECU>(m, b, bu, fc, prog, rule, s, ncells, out, status);
}

// Basis.interpolate: a block takes CPB cells (or facets); stage 0 stages
// each cell's affine map and DOF values in shared memory, stage 1 gives one
// (cell, point) pair per thread: quantity k of the field,
// out[(k * ncells + e) * nq + q] = 0*(w0 phi_0) + sum_i w_i phi_i in
// local-function order (abstract_basis.py:295-304).  FACET: at the facet
// points, with the basis of the cell f2t[side].
template <int D, bool FACET, bool VEC>
__global__ void interpolate_kernel(FemMesh m, FemBasis b, FemFacets fc, Rule rule, int64_t ncells,
                                   int cpb, const double* __restrict__ w, double* __restrict__ out,
                                   int32_t* __restrict__ status) {
  extern __shared__ double ism[];
  constexpr bool vec = VEC;
  const bool hex = b.family == FEM_HEX_1;
  const bool maps = !FACET && !hex;
  const int nb = b.nbfun;
  constexpr int NQ = D + D * D;
  // P1 on affine cells: each function's quantities at the cell's first
  // point are staged; the other points take their derivative part
  const bool p1 = maps && point_free_gradients(b.family);
  const int per = kCell + nb + (p1 ? nb * NQ : 0);  // per cell: map, DOF values, quantities
  const int64_t e0 = (int64_t)blockIdx.x * cpb;
  for (int k = threadIdx.x; k < cpb; k += blockDim.x) {
    const int64_t e = e0 + k;
    if (e >= ncells) continue;
    double* S = ism + (size_t)k * per;
    const int64_t ec = FACET ? (int64_t)fc.tind[e] : e;   // the cell whose DOFs are read
    if (ec < 0 || ec >= m.nelems) {
      if (status) atomicOr(status, 1 << FEM_ERR_ARGUMENT);
      for (int i = 0; i < nb; ++i) S[kCell + i] = 0.0;
      continue;
    }
    if (maps) {
      CellGeo cg;
      cell_geometry<D>(m, e, false, cg);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          S[i * 3 + j] = cg.inv[i][j];
          S[10 + i * 3 + j] = cg.A[i][j];
        }
      S[9] = cg.det;
      for (int i = 0; i < 3; ++i) S[19 + i] = cg.x0[i];
    }
    for (int i = 0; i < nb; ++i) S[kCell + i] = w[b.element_dofs[(int64_t)i * m.nelems + ec]];
    if (p1) {
      PointGeo g0;
      double Y0[3];
      geometry_at<D, FACET>(m, b, fc, rule, ProgFlags(), e, 0, Y0, g0, S);
      for (int i = 0; i < nb; ++i)
        quantities<D>(b.family, VEC, i, Y0[0], Y0[1], Y0[2], g0.inv, S + kCell + nb + i * NQ);
    }
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int k = t / rule.nq, q = t - k * rule.nq;
  const int64_t e = e0 + k;
  if (k >= cpb || e >= ncells) return;
  const double* S = ism + (size_t)k * per;
  if (FACET) {
    const int64_t ec = fc.tind[e];
    if (ec < 0 || ec >= m.nelems) return;
  }
  PointGeo g;
  double Y[3];
  if (!geometry_at<D, FACET>(m, b, fc, rule, ProgFlags(), e, q, Y, g, maps ? S : nullptr)) {
    if (status) atomicOr(status, 1 << FEM_ERR_ARGUMENT);
    return;
  }
  constexpr int nquant = VEC ? D + D * D : 1 + D;
  double acc[NQ], qq[NQ];
  auto quant = [&](int i) {
    if (p1) quantities_values<D>(b.family, vec, i, Y[0], Y[1], Y[2], S + kCell + nb + i * NQ, qq);
    else quantities<D>(b.family, vec, i, Y[0], Y[1], Y[2], g.inv, qq);
  };
  const double w0 = S[kCell];
  quant(0);   // function 0: the start 0*(w0 q0) and the first term
#pragma unroll
  for (int a = 0; a < nquant; ++a) acc[a] = 0.0 * (w0 * qq[a]);
#pragma unroll
  for (int a = 0; a < nquant; ++a) acc[a] = acc[a] + w0 * qq[a];
  for (int i = 1; i < nb; ++i) {
    const double wi = S[kCell + i];
    quant(i);
#pragma unroll
    for (int a = 0; a < nquant; ++a) acc[a] = acc[a] + wi * qq[a];
  }
#pragma unroll
  for (int a = 0; a < nquant; ++a) out[((int64_t)a * ncells + e) * rule.nq + q] = acc[a];
}

// ------------------------------------------------------ Hex1 facet geometry
__global__ void hex_facet_newton_count(FemMesh m, FemFacets fc, Rule rule, int which,
                                       int32_t* __restrict__ kmax) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= fc.nfacets) return;
  atomicMax(kmax + which, hex_facet_newton_iters(m, fc, f, which, rule.X, rule.nq));
}

__global__ void hex_facet_geometry_kernel(FemMesh m, FemFacets fc, Rule rule,
                                          const int32_t* __restrict__ kmax,
                                          double* __restrict__ geo, int32_t* __restrict__ status) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= fc.nfacets * rule.nq) return;
  const int64_t f = t / rule.nq;
  const int q = (int)(t - f * rule.nq);
  const int st = hex_facet_point(m, fc, f, q, rule.X, rule.nq, kmax[0], kmax[1],
                                 geo + (size_t)t * kGeo);
  if (st) atomicOr(status, st);
}

// numpy's pairwise sum of n doubles (np.sum of a contiguous vector): the
// leaves (<= 128 values) in parallel, the combination tree by one thread.
__global__ void pairwise_leaves_kernel(const double* __restrict__ x, int64_t n,
                                       const int64_t* __restrict__ leaf_off,
                                       const int32_t* __restrict__ leaf_len, int64_t nleaves,
                                       double* __restrict__ leaf_sum) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nleaves) leaf_sum[k] = np_pairwise_sum(x + leaf_off[k], leaf_len[k]);
}

__global__ void pairwise_tree_kernel(const double* __restrict__ leaf_sum, int64_t n,
                                     double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  if (n == 0) {
    *out = 0.0;
    return;
  }
  // the same split recursion as np_pairwise_sum_any, consuming leaves in order
  struct Frame { int64_t n; int state; double left; };
  Frame st[64];
  int sp = 0;
  st[0] = {n, 0, 0.0};
  int64_t leaf = 0;
  double ret = 0.0;
  while (sp >= 0) {
    Frame& f = st[sp];
    if (f.n <= 128) {
      ret = leaf_sum[leaf++];
      --sp;
      continue;
    }
    int64_t n2 = f.n / 2;
    n2 -= n2 % 8;
    if (f.state == 0) {
      f.state = 1;
      st[sp + 1] = {n2, 0, 0.0};
      ++sp;
    } else if (f.state == 1) {
      f.left = ret;
      f.state = 2;
      st[sp + 1] = {f.n - n2, 0, 0.0};
      ++sp;
    } else {
      ret = f.left + ret;
      --sp;
    }
  }
  *out = ret;
}

}  // namespace fem_faithful
namespace fem {

int check_instructions(const FemInstr* h, int ninstr, int ncoef, int dim, bool vec);

// Host-side check of a form program before any kernel interprets it: every
// operand names an earlier register, a basis quantity, a coefficient slot
// or a coordinate that exists.
int check_program(const FemProgram& prog, int dim, bool vec, bool need_rule,
                  bool instructions = true) {
  using namespace fem_faithful;
  if (prog.ninstr <= 0 || prog.ninstr > kMaxProgram || prog.out < 0 ||
      prog.out >= prog.ninstr || prog.ncoef < 0 || prog.ncoef > kMaxCoef || !prog.ins ||
      prog.nq <= 0 || prog.nq > kMaxPoints) {
    set_error(FEM_ERR_UNSUPPORTED,
              "form program of %d instructions, %d coefficients, %d points (limits %d, %d, %d)",
              prog.ninstr, prog.ncoef, prog.nq, kMaxProgram, kMaxCoef, kMaxPoints);
    return FEM_ERR_UNSUPPORTED;
  }
  if (need_rule && (!prog.qX || !prog.qW)) {
    set_error(FEM_ERR_ARGUMENT, "form program without quadrature points (qX, qW)");
    return FEM_ERR_ARGUMENT;
  }
  for (int c = 0; c < prog.ncoef; ++c)
    if (prog.coef_stride[c] != 0 && prog.coef_stride[c] != prog.nq) {
      set_error(FEM_ERR_ARGUMENT, "coefficient slot %d: stride %d (0 or %d)", c,
                prog.coef_stride[c], prog.nq);
      return FEM_ERR_ARGUMENT;
    }
  // a compiled program's operands were checked when it was compiled
  if (!instructions) return 0;
  FemInstr h[kMaxProgram];
  FEM_TRY_CUDA(cudaMemcpy(h, prog.ins, prog.ninstr * sizeof(FemInstr), cudaMemcpyDefault));
  return check_instructions(h, prog.ninstr, prog.ncoef, dim, vec);
}

// Operand checks of a program held in host memory.
int check_instructions(const FemInstr* h, int ninstr, int ncoef, int dim, bool vec) {
  using namespace fem_faithful;
  const int nquant = vec ? dim + dim * dim : 1 + dim;
  for (int k = 0; k < ninstr; ++k) {
    const FemInstr& I = h[k];
    bool ok = true;
    switch (I.op) {
      case OP_CONST: case OP_H: break;
      case OP_U: case OP_V: ok = I.a >= 0 && I.a < nquant; break;
      case OP_COEF: ok = I.a >= 0 && I.a < ncoef; break;
      case OP_X: case OP_N: ok = I.a >= 0 && I.a < dim; break;
      case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_POW:
        ok = I.a >= 0 && I.a < k && I.b >= 0 && I.b < k; break;
      case OP_NEG: case OP_SQRT: case OP_EXP: case OP_LOG: case OP_SIN: case OP_COS:
      case OP_TAN: case OP_TANH: case OP_ARCTAN: case OP_ABS:
        ok = I.a >= 0 && I.a < k; break;
      default: ok = false;
    }
    if (!ok) {
      set_error(FEM_ERR_ARGUMENT, "form program instruction %d (op %d, a %d, b %d) is invalid", k,
                I.op, I.a, I.b);
      return FEM_ERR_ARGUMENT;
    }
  }
  return 0;
}

int faithful_mask(const FemMesh& m, const FemBasis& b, const FemProgram& prog, int nq, double* local,
                  int32_t* status, cudaStream_t st) {
  int rc = check_program(prog, m.dim, b.vector != 0, false);
  if (rc) return rc;
  if (m.nelems == 0) return 0;
  const unsigned grid = (unsigned)ceil_div(m.nelems, 64);
  if (m.dim == 2)
    fem_faithful::mask_kernel<2><<<grid, 64, 0, st>>>(m, b, prog, nq, 1e-9, local, status);
  else
    fem_faithful::mask_kernel<3><<<grid, 64, 0, st>>>(m, b, prog, nq, 1e-9, local, status);
  FEM_LAUNCH_CHECK("faithful mask kernel");
  return 0;
}

static bool facets_ok(const FemMesh& m, const FemBasis& b, const FemFacets* fc) {
  if (!fc) return true;
  if (b.family == FEM_HEX_1 && !fc->geo) {
    set_error(FEM_ERR_ARGUMENT, "Hex1 facets need their geometry (fem_facet_geometry)");
    return false;
  }
  if (fc->nfacets < 0 || (fc->nfacets > 0 && (!fc->fverts || !fc->tind || !fc->tind_n ||
                                               !fc->lfacet_n))) {
    set_error(FEM_ERR_ARGUMENT, "invalid facet arrays");
    return false;
  }
  (void)m;
  return true;
}

// mode 0: local matrices, 1: local vectors, 2: per-cell functional values;
// fc non-null: over the facets of a FacetBasis
int program_eval(int mode, const FemMesh& m, const FemBasis& b, const FemFacets* fc,
                 const FemProgram& prog, double* out, int32_t* status, cudaStream_t st,
                 const FemBasis* bu) {
  if (!facets_ok(m, b, fc)) return FEM_ERR_ARGUMENT;
  int rc = check_program(prog, m.dim, b.vector != 0 || (bu && bu->vector != 0), true,
                         prog.compiled == nullptr);
  if (rc) return rc;
  const int64_t ncells = fc ? fc->nfacets : m.nelems;
  if (ncells == 0) return 0;
  const int nb = b.nbfun;
  const bool mixed = bu && mode == 0;
  const FemBasis& ub = mixed ? *bu : b;
  if (mixed && fc) {
    set_error(FEM_ERR_UNSUPPORTED, "different trial and test bases on facets are not supported");
    return FEM_ERR_UNSUPPORTED;
  }
  if (mixed && prog.compiled && prog.compiled->vector_u != (ub.vector ? 1 : 0)) {
    set_error(FEM_ERR_ARGUMENT, "compiled program is for another trial basis");
    return FEM_ERR_ARGUMENT;
  }
  const int L = mode == 0 ? nb * ub.nbfun : (mode == 1 ? nb : 1);
  const int nq = prog.nq;
  fem_faithful::GenericLayout s;
  s.L = L;
  s.nq = nq;
  s.nb = nb;
  s.nquant = b.vector ? m.dim + m.dim * m.dim : 1 + m.dim;
  s.cells = !fc && b.family != FEM_HEX_1;
  s.quants = mode != 2;   // a functional reads no basis function
  s.npoint = prog.compiled ? prog.compiled->npoint : 0;
  s.mixed = mixed;
  s.nbu = ub.nbfun;
  s.nquantu = ub.vector ? m.dim + m.dim * m.dim : 1 + m.dim;
  s.uv = prog.compiled && prog.compiled->uv;
  s.nuval = prog.compiled ? prog.compiled->nuval : 0;
  s.nvval = prog.compiled ? prog.compiled->nvval : 0;
  auto bytes = [&](int epb) {
    fem_faithful::GenericLayout t = s;
    t.epb = epb;
    return t.total() * sizeof(double);
  };
  s.entry_loop = false;
  if (bytes(1) > 96 * 1024) {
    // no per-(entry, point) value stage; a compiled program evaluates its
    // trial-only and test-only parts per entry (in registers)
    s.entry_loop = true;
    s.uv = false;
  }
  // blocks of 128 threads holding at most ~44 KB: five blocks per SM, so
  // that the stage barriers of one block are covered by the others
  int epb = std::max(1, std::min(32, 1024 / (L * nq)));
  while (epb > 1 && bytes(epb) > 44 * 1024) --epb;
  s.epb = epb;
  const size_t smem = bytes(epb);
  if (smem > 200 * 1024) {
    set_error(FEM_ERR_CAPACITY, "%d local entries x %d points do not fit one block", L, nq);
    return FEM_ERR_CAPACITY;
  }
  const fem_faithful::Rule rule{prog.qX, prog.qW, nq};
  const FemFacets F = fc ? *fc : FemFacets{};
  const unsigned grid = (unsigned)ceil_div(ncells, epb);
  const int threads = 128;
  if (prog.compiled) {
    const FemCompiled* k = prog.compiled;
    if (k->dim != m.dim || k->mode != mode || k->facet != (fc ? 1 : 0)) {
      set_error(FEM_ERR_ARGUMENT, "compiled program is for dim %d mode %d facet %d", k->dim,
                k->mode, k->facet);
      return FEM_ERR_ARGUMENT;
    }
    FemMesh mm = m;
    FemBasis bb = b;
    FemBasis bbu = ub;
    FemFacets ff = F;
    FemProgram pp = prog;
    fem_faithful::Rule rr = rule;
    fem_faithful::GenericLayout ss = s;
    int64_t nc = ncells;
    double* o = out;
    int32_t* stp = status;
    void* args[] = {&mm, &bb, &bbu, &ff, &pp, &rr, &ss, &nc, &o, &stp};
    return jit_launch(k, dim3(grid), dim3(threads), smem, st, args);
  }
  auto go = [&](auto kern) -> int {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return check_cuda(e, "program kernel smem");
    }
    kern<<<grid, threads, smem, st>>>(m, b, ub, F, prog, rule, s, ncells, out, status);
    return 0;
  };
  using namespace fem_faithful;
  // <dim, mode, facet, vector> instantiations
  auto pick = [&](auto facet_tag, auto vec_tag) -> int {
    constexpr bool FC = decltype(facet_tag)::value, VC = decltype(vec_tag)::value;
    if (m.dim == 2)
      return mode == 0 ? go(program_kernel<2, 0, FC, VC, VC>)
                       : mode == 1 ? go(program_kernel<2, 1, FC, VC, VC>)
                                   : go(program_kernel<2, 2, FC, VC, VC>);
    return mode == 0 ? go(program_kernel<3, 0, FC, VC, VC>)
                     : mode == 1 ? go(program_kernel<3, 1, FC, VC, VC>)
                                 : go(program_kernel<3, 2, FC, VC, VC>);
  };
  // different trial and test bases (bilinear forms on cells)
  auto pick_mixed = [&](auto vv, auto vu) -> int {
    constexpr bool V = decltype(vv)::value, U = decltype(vu)::value;
    return m.dim == 2 ? go(program_kernel<2, 0, false, V, U>) : go(program_kernel<3, 0, false, V, U>);
  };
  using T = std::true_type;
  using Fl = std::false_type;
  if (mixed)
    rc = b.vector ? (ub.vector ? pick_mixed(T{}, T{}) : pick_mixed(T{}, Fl{}))
                  : (ub.vector ? pick_mixed(Fl{}, T{}) : pick_mixed(Fl{}, Fl{}));
  else if (fc) rc = b.vector ? pick(T{}, T{}) : pick(T{}, Fl{});
  else rc = b.vector ? pick(Fl{}, T{}) : pick(Fl{}, Fl{});
  if (rc) return rc;
  FEM_LAUNCH_CHECK("program kernel");
  return 0;
}

int interpolate(const FemMesh& m, const FemBasis& b, const FemFacets* fc, int nq, const double* X,
                const double* w, double* out, int32_t* status, cudaStream_t st) {
  if (nq <= 0 || nq > fem_faithful::kMaxPoints || !X || !w || !out || (fc && !status)) {
    set_error(FEM_ERR_ARGUMENT, "interpolate: %d points, X/w/out must be device arrays", nq);
    return FEM_ERR_ARGUMENT;
  }
  if (!facets_ok(m, b, fc)) return FEM_ERR_ARGUMENT;
  const int64_t ncells = fc ? fc->nfacets : m.nelems;
  if (ncells == 0) return 0;
  const fem_faithful::Rule rule{X, nullptr, nq};
  const FemFacets F = fc ? *fc : FemFacets{};
  // one (cell, point) pair per thread: blocks of cpb cells x nq points
  const int cpb = std::max(1, 128 / nq);
  const int threads = cpb * nq;
  // per cell: the affine map, the DOF values and, P1 on affine cells, every
  // function's quantities at the first point (interpolate_kernel)
  const bool p1 = !fc && b.family != FEM_HEX_1 && fem_faithful::point_free_gradients(b.family);
  const int nqmax = m.dim + m.dim * m.dim;
  const size_t smem = (size_t)cpb * (fem_faithful::kCell + b.nbfun + (p1 ? b.nbfun * nqmax : 0)) *
                      sizeof(double);
  const unsigned grid = (unsigned)ceil_div(ncells, cpb);
  using namespace fem_faithful;
  auto go = [&](auto kern) {
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grid, threads, smem, st>>>(m, b, F, rule, ncells, cpb, w, out, status);
  };
  const bool v = b.vector != 0;
  if (m.dim == 2) {
    if (fc) v ? go(interpolate_kernel<2, true, true>) : go(interpolate_kernel<2, true, false>);
    else v ? go(interpolate_kernel<2, false, true>) : go(interpolate_kernel<2, false, false>);
  } else {
    if (fc) v ? go(interpolate_kernel<3, true, true>) : go(interpolate_kernel<3, true, false>);
    else v ? go(interpolate_kernel<3, false, true>) : go(interpolate_kernel<3, false, false>);
  }
  FEM_LAUNCH_CHECK("interpolate kernel");
  return 0;
}

int facet_geometry(const FemMesh& m, const FemBasis& b, const FemFacets& fc, int nq,
                   const double* X, double* geo, int32_t* status, cudaStream_t st) {
  if (b.family != FEM_HEX_1) {
    set_error(FEM_ERR_ARGUMENT, "facet geometry is precomputed for Hex1 meshes only");
    return FEM_ERR_ARGUMENT;
  }
  if (nq <= 0 || nq > fem_faithful::kMaxPoints || !X || !geo || !status || fc.nfacets < 0 ||
      (fc.nfacets > 0 && (!fc.fverts || !fc.tind || !fc.tind_n || !fc.lfacet_n))) {
    set_error(FEM_ERR_ARGUMENT, "invalid facet geometry arguments");
    return FEM_ERR_ARGUMENT;
  }
  if (fc.nfacets == 0) return 0;
  int32_t* kmax = nullptr;
  FEM_TRY_CUDA(cudaMallocAsync(&kmax, 2 * sizeof(int32_t), st));
  FEM_TRY_CUDA(cudaMemsetAsync(kmax, 0, 2 * sizeof(int32_t), st));
  const fem_faithful::Rule rule{X, nullptr, nq};
  const unsigned g1 = (unsigned)ceil_div(fc.nfacets, 64);
  fem_faithful::hex_facet_newton_count<<<g1, 64, 0, st>>>(m, fc, rule, 0, kmax);
  fem_faithful::hex_facet_newton_count<<<g1, 64, 0, st>>>(m, fc, rule, 1, kmax);
  const unsigned g2 = (unsigned)ceil_div(fc.nfacets * (int64_t)nq, 128);
  fem_faithful::hex_facet_geometry_kernel<<<g2, 128, 0, st>>>(m, fc, rule, kmax, geo, status);
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(kmax, st);
  if (e != cudaSuccess) return check_cuda(e, "hex facet geometry kernels");
  return 0;
}

int sum_pairwise(const double* x, int64_t n, double* out, cudaStream_t st) {
  // leaves of numpy's split recursion, in order
  std::vector<int64_t> off;
  std::vector<int32_t> len;
  struct Seg { int64_t o, n; };
  std::vector<Seg> stack{{0, n}};
  while (!stack.empty()) {
    Seg s = stack.back();
    stack.pop_back();
    if (s.n <= 128) {
      if (n > 0) {
        off.push_back(s.o);
        len.push_back((int32_t)s.n);
      }
      continue;
    }
    int64_t n2 = s.n / 2;
    n2 -= n2 % 8;
    stack.push_back({s.o + n2, s.n - n2});  // right after left
    stack.push_back({s.o, n2});
  }
  const int64_t nl = (int64_t)off.size();
  int64_t* d_off = nullptr;
  int32_t* d_len = nullptr;
  double* d_sum = nullptr;
  const size_t bytes = std::max<int64_t>(1, nl) * (sizeof(int64_t) + sizeof(int32_t) + sizeof(double));
  char* blob = nullptr;
  FEM_TRY_CUDA(cudaMallocAsync(&blob, bytes, st));
  d_off = reinterpret_cast<int64_t*>(blob);
  d_sum = reinterpret_cast<double*>(blob + std::max<int64_t>(1, nl) * sizeof(int64_t));
  d_len = reinterpret_cast<int32_t*>(blob + std::max<int64_t>(1, nl) * 2 * sizeof(int64_t));
  if (nl > 0) {
    FEM_TRY_CUDA(cudaMemcpyAsync(d_off, off.data(), nl * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    FEM_TRY_CUDA(cudaMemcpyAsync(d_len, len.data(), nl * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    fem_faithful::pairwise_leaves_kernel<<<(unsigned)ceil_div(nl, 128), 128, 0, st>>>(
        x, n, d_off, d_len, nl, d_sum);
    FEM_LAUNCH_CHECK("pairwise leaves kernel");
  }
  fem_faithful::pairwise_tree_kernel<<<1, 32, 0, st>>>(d_sum, n, out);
  FEM_LAUNCH_CHECK("pairwise tree kernel");
  // the host vectors must outlive the asynchronous copies
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  cudaFreeAsync(blob, st);
  return 0;
}

}  // namespace fem
