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
  if (!rule_for(D, b.family == FEM_HEX_1, nq, rule)) {
    atomicOr(status, 1 << FEM_ERR_UNSUPPORTED);
    return;
  }
  const int NB = b.nbfun;
  double* Ke = local + e * (int64_t)NB * NB;
  double scale = 0.0;
  for (int k = 0; k < NB * NB; ++k) scale = fmax(scale, fabs(Ke[k]));
  double coef[8];
  for (int c = 0; c < prog.ncoef && c < 8; ++c) coef[c] = prog.coef[c] ? prog.coef[c][e] : 0.0;
  double R[kMaxProgram];
  double vals[64];
  for (int i = 0; i < NB; ++i) {      // test function (row)
    for (int j = 0; j < NB; ++j) {    // trial function (column)
      const double v = Ke[i * NB + j];
      if (fabs(v) > tau * scale) continue;
      const double s = replay_entry<D>(m, b, prog, rule, e, i, j, coef, R, vals);
      // the buffer only feeds the mask: mark exact zeros / noise nonzeros
      Ke[i * NB + j] = (s == 0.0) ? 0.0 : (v != 0.0 ? v : 1e-300);
    }
  }
}

}  // namespace fem_faithful
namespace fem {
int faithful_mask(const FemMesh& m, const FemBasis& b, const FemProgram& prog, int nq, double* local,
                  int32_t* status, cudaStream_t st) {
  if (prog.ninstr <= 0 || prog.ninstr > fem_faithful::kMaxProgram || prog.out < 0 ||
      prog.out >= prog.ninstr || prog.ncoef > 8) {
    set_error(FEM_ERR_UNSUPPORTED, "form program of %d instructions (limit %d)", prog.ninstr,
              fem_faithful::kMaxProgram);
    return FEM_ERR_UNSUPPORTED;
  }
  if (m.nelems == 0) return 0;
  const unsigned grid = (unsigned)ceil_div(m.nelems, 64);
  if (m.dim == 2)
    fem_faithful::mask_kernel<2><<<grid, 64, 0, st>>>(m, b, prog, nq, 1e-9, local, status);
  else
    fem_faithful::mask_kernel<3><<<grid, 64, 0, st>>>(m, b, prog, nq, 1e-9, local, status);
  FEM_LAUNCH_CHECK("faithful mask kernel");
  return 0;
}
}  // namespace fem
