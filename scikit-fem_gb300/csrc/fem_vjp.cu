// Adjoint (vector-Jacobian product) kernels.
//
// scikit-fem has no derivative of an assembled operator with respect to its
// coefficients or the mesh (skfem/autodiff differentiates a nonlinear form
// with respect to the solution only, skfem/autodiff/__init__.py:124-213).
// For J = w^T K(coef, X) u (and J = w^T b(coef, X)) these kernels return
//   dJ/dcoef[e]  for every per-element coefficient channel, and
//   dJ/dX        for the node coordinates (the shape derivative through
//                detDF and invDF),
// recomputing the cell geometry instead of storing anything per quadrature
// point.  Per-element vertex gradients go to a scratch array and are then
// summed per vertex in a fixed order (vertex incidence), without atomics.
//
// Affine simplices (closed form): with g_a = grad(lambda_a), V = |T|,
//   E_diff = V sum_ab Q_ab g_a.g_b,  Q_ab = sum_ij w_i u_j BB[i][j][a][b]
//   dV = V g_n . dx_n,   dg_a = -sum_n (g_a . dx_n) g_n
// give  dE_diff/dx_n = V (S g_n - sum_a [(Q + Q^T) G]_an g_a),  S = sum Q.G,
//       dE_mass/dx_n = V mu g_n,  mu = sum_ij w_i u_j MM[i][j].
// Trilinear hexahedra (per quadrature point q, G = J^{-1}, a = grad_ref w_h,
// b = grad_ref u_h, E_q = c |det J| (G^T a).(G^T b)):
//   dE_q/dJ = c |det J| [ (G^T a . G^T b) G^T - (G^T a)(G G^T b)^T - (G^T b)(G G^T a)^T ]
//   dE/dx_n[k] = sum_q sum_m dE_q/dJ[k][m] * d_m phi_n(q).
// On parallelepipeds every integrand is a polynomial of degree <= 3 per axis
// and the 2x2x2 Gauss rule is exact; other cells use the 4x4x4 rule of the
// forward kernel.

#include "fem_common.cuh"
#include "fem_tables.cuh"

namespace fem {
int build_incidence(const int32_t* dofs, int64_t nelems, int nb, int64_t nrows, Pattern* P,
                    cudaStream_t st);
}

namespace fem_vjp {

using fem::coef_at;

template <int D, int ORDER>
struct Traits;
template <> struct Traits<2, 1> { static constexpr int NB = 3; static constexpr double FACT = 2.0; };
template <> struct Traits<2, 2> { static constexpr int NB = 6; static constexpr double FACT = 2.0; };
template <> struct Traits<3, 1> { static constexpr int NB = 4; static constexpr double FACT = 6.0; };
template <> struct Traits<3, 2> { static constexpr int NB = 10; static constexpr double FACT = 6.0; };

// physical barycentric gradients g[a] and |T|
template <int D>
__device__ __forceinline__ void simplex_grads(const FemMesh& m, int64_t e, double g[D + 1][D],
                                              double& vol) {
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
  double det, c[D + 1][D];
  if constexpr (D == 2) {
    det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    c[1][0] = A[1][1];
    c[1][1] = -A[0][1];
    c[2][0] = -A[1][0];
    c[2][1] = A[0][0];
  } else {
    c[1][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    c[2][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    c[3][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    c[1][1] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
    c[2][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
    c[3][1] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
    c[1][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
    c[2][2] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
    c[3][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    det = A[0][0] * c[1][0] + A[0][1] * c[2][0] + A[0][2] * c[3][0];
  }
  const double inv = 1.0 / det;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    double s = 0.0;
#pragma unroll
    for (int a = 1; a <= D; ++a) {
      g[a][k] = c[a][k] * inv;
      s += g[a][k];
    }
    g[0][k] = -s;
  }
  vol = fabs(det) / Traits<D, 1>::FACT;
}

template <int D, int ORDER>
__global__ void simplex_bilinear_vjp_kernel(FemMesh m, FemBasis b, FemBilinear f,
                                            const double* __restrict__ w,
                                            const double* __restrict__ u,
                                            double* __restrict__ dcd, double* __restrict__ dcm,
                                            double* __restrict__ scratch) {
  constexpr int NB = Traits<D, ORDER>::NB;
  constexpr int NV = D + 1;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  double wl[NB], ul[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int64_t dof = b.element_dofs[i * m.nelems + e];
    wl[i] = w[dof];
    ul[i] = u[dof];
  }
  double g[NV][D], V;
  simplex_grads<D>(m, e, g, V);
  double Q[NV][NV];
#pragma unroll
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int c = 0; c < NV; ++c) Q[a][c] = 0.0;
  double mu = 0.0;
#define W(i) wl[i]
#define U(i) ul[i]
#define QQ(a, c) Q[a][c]
  if constexpr (D == 2 && ORDER == 1) { TRI1_QACC(W, U, QQ); TRI1_MACC(W, U, mu); }
  if constexpr (D == 2 && ORDER == 2) { TRI2_QACC(W, U, QQ); TRI2_MACC(W, U, mu); }
  if constexpr (D == 3 && ORDER == 1) { TET1_QACC(W, U, QQ); TET1_MACC(W, U, mu); }
  if constexpr (D == 3 && ORDER == 2) { TET2_QACC(W, U, QQ); TET2_MACC(W, U, mu); }
#undef W
#undef U
#undef QQ
  double G[NV][NV];
#pragma unroll
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int c = a; c < NV; ++c) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) s += g[a][k] * g[c][k];
      G[a][c] = s;
      G[c][a] = s;
    }
  double S = 0.0;
#pragma unroll
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int c = 0; c < NV; ++c) S += Q[a][c] * G[a][c];
  const double kd = coef_at(f.diff, e), km = coef_at(f.mass, e);
  if (dcd) dcd[e] = f.diff.scale * V * S;
  if (dcm) dcm[e] = f.mass.scale * V * mu;
  // P = (Q + Q^T) G
#pragma unroll
  for (int n = 0; n < NV; ++n) {
    double grad[D];
#pragma unroll
    for (int k = 0; k < D; ++k) grad[k] = (kd * S + km * mu) * g[n][k];
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      double P = 0.0;
#pragma unroll
      for (int c = 0; c < NV; ++c) P += (Q[a][c] + Q[c][a]) * G[c][n];
      P *= kd;
#pragma unroll
      for (int k = 0; k < D; ++k) grad[k] -= P * g[a][k];
    }
#pragma unroll
    for (int k = 0; k < D; ++k) scratch[(e * NV + n) * D + k] = V * grad[k];
  }
}

template <int D, int ORDER>
__global__ void simplex_linear_vjp_kernel(FemMesh m, FemBasis b, FemLinear f,
                                          const double* __restrict__ w, double* __restrict__ dl,
                                          double* __restrict__ scratch) {
  constexpr int NB = Traits<D, ORDER>::NB;
  constexpr int NV = D + 1;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  double wl[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) wl[i] = w[b.element_dofs[i * m.nelems + e]];
  double g[NV][D], V;
  simplex_grads<D>(m, e, g, V);
  double lw = 0.0;
#define W(i) wl[i]
  if constexpr (D == 2 && ORDER == 1) { TRI1_LACC(W, lw); }
  if constexpr (D == 2 && ORDER == 2) { TRI2_LACC(W, lw); }
  if constexpr (D == 3 && ORDER == 1) { TET1_LACC(W, lw); }
  if constexpr (D == 3 && ORDER == 2) { TET2_LACC(W, lw); }
#undef W
  const double fe = coef_at(f.load, e);
  if (dl) dl[e] = f.load.scale * V * lw;
#pragma unroll
  for (int n = 0; n < NV; ++n)
#pragma unroll
    for (int k = 0; k < D; ++k) scratch[(e * NV + n) * D + k] = fe * V * lw * g[n][k];
}

// ----------------------------------------------------------- hexahedron
__device__ __forceinline__ void hex_shape(double x, double y, double z, double phi[8],
                                          double dphi[8][3]) {
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int cx = c_hex_corner[n][0], cy = c_hex_corner[n][1], cz = c_hex_corner[n][2];
    const double fx = cx ? x : 1.0 - x, fy = cy ? y : 1.0 - y, fz = cz ? z : 1.0 - z;
    phi[n] = fx * fy * fz;
    dphi[n][0] = (cx ? 1.0 : -1.0) * (fy * fz);
    dphi[n][1] = (cy ? 1.0 : -1.0) * (fx * fz);
    dphi[n][2] = (cz ? 1.0 : -1.0) * (fx * fy);
  }
}

__device__ __forceinline__ double adj3(const double J[3][3], double ad[3][3]) {
  ad[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  ad[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  ad[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  ad[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  ad[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  ad[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  ad[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  ad[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  ad[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  return J[0][0] * ad[0][0] + J[0][1] * ad[1][0] + J[0][2] * ad[2][0];
}

// mode 0: bilinear (diff, mass); mode 1: linear (load * v)
template <int MODE>
__global__ void hex_vjp_kernel(FemMesh m, FemBasis b, FemCoef cd, FemCoef cm,
                               const double* __restrict__ w, const double* __restrict__ u,
                               double* __restrict__ dcd, double* __restrict__ dcm,
                               double* __restrict__ scratch, int32_t* __restrict__ status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.nelems) return;
  double x[8][3], wl[8], ul[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int64_t v = m.t[n * m.nelems + e];
#pragma unroll
    for (int k = 0; k < 3; ++k) x[n][k] = m.p[k * m.nverts + v];
    const int64_t dof = b.element_dofs[n * m.nelems + e];
    wl[n] = w[dof];
    ul[n] = MODE == 0 ? u[dof] : 0.0;
  }
  // parallelepiped test (as the forward kernel)
  bool affine = true;
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double v = x[7][k];
      if (c_hex_corner[n][0]) v = v + (x[4][k] - x[7][k]);
      if (c_hex_corner[n][1]) v = v + (x[5][k] - x[7][k]);
      if (c_hex_corner[n][2]) v = v + (x[6][k] - x[7][k]);
      affine = affine && (v == x[n][k]);
    }
  const int nq = affine ? 2 : 4;
  const double kd = coef_at(cd, e), km = MODE == 0 ? coef_at(cm, e) : 0.0;
  double Ed = 0.0, Em = 0.0;
  double gx[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int k = 0; k < 3; ++k) gx[n][k] = 0.0;
  for (int q = 0; q < nq * nq * nq; ++q) {
    const int qx = q % nq, qy = (q / nq) % nq, qz = q / (nq * nq);
    const double* xs = affine ? c_gl2_x : c_gl4_x;
    const double* ws = affine ? c_gl2_w : c_gl4_w;
    double phi[8], dphi[8][3];
    hex_shape(xs[qx], xs[qy], xs[qz], phi, dphi);
    const double wq = ws[qx] * ws[qy] * ws[qz];
    double J[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double s = 0.0;
#pragma unroll
        for (int n = 0; n < 8; ++n) s += x[n][a] * dphi[n][c];
        J[a][c] = s;
      }
    double ad[3][3];
    const double det = adj3(J, ad);
    if (det == 0.0) {
      if (status) atomicOr(status, 1 << FEM_ERR_ZERO_JACOBIAN);
      continue;
    }
    const double inv = 1.0 / det, adet = fabs(det);
    double Gm[3][3];  // G = J^{-1}
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) Gm[a][c] = ad[a][c] * inv;
    double ar[3] = {0, 0, 0}, br[3] = {0, 0, 0}, wv = 0.0, uv = 0.0;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      wv += wl[n] * phi[n];
      uv += ul[n] * phi[n];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ar[k] += wl[n] * dphi[n][k];
        br[k] += ul[n] * dphi[n][k];
      }
    }
    double D[3][3];  // dE_q / dJ
    if (MODE == 0) {
      double ga[3], gb[3];  // G^T a, G^T b
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ga[k] = Gm[0][k] * ar[0] + Gm[1][k] * ar[1] + Gm[2][k] * ar[2];
        gb[k] = Gm[0][k] * br[0] + Gm[1][k] * br[1] + Gm[2][k] * br[2];
      }
      double Ga[3], Gb[3];  // G (G^T a), G (G^T b)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Ga[k] = Gm[k][0] * ga[0] + Gm[k][1] * ga[1] + Gm[k][2] * ga[2];
        Gb[k] = Gm[k][0] * gb[0] + Gm[k][1] * gb[1] + Gm[k][2] * gb[2];
      }
      const double s = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
      const double cdf = wq * adet;
      Ed += cdf * s;
      Em += cdf * wv * uv;
      const double c0 = cdf * (kd * s + km * wv * uv);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          D[a][c] = c0 * Gm[c][a] - kd * cdf * (ga[a] * Gb[c] + gb[a] * Ga[c]);
    } else {
      const double cdf = wq * adet;
      Ed += cdf * wv;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) D[a][c] = kd * cdf * wv * Gm[c][a];
    }
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int a = 0; a < 3; ++a)
        gx[n][a] += D[a][0] * dphi[n][0] + D[a][1] * dphi[n][1] + D[a][2] * dphi[n][2];
  }
  if (dcd) dcd[e] = cd.scale * Ed;
  if (MODE == 0 && dcm) dcm[e] = cm.scale * Em;
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int a = 0; a < 3; ++a) scratch[(e * 8 + n) * 3 + a] = gx[n][a];
}

// dX[a][v] = sum over the vertex's incidence (fixed order) of scratch rows
__global__ void vertex_gather_kernel(const int32_t* __restrict__ inc_ptr,
                                     const int32_t* __restrict__ inc, int64_t nverts, int dim,
                                     const double* __restrict__ scratch, double* __restrict__ dX) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nverts) return;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int32_t q = inc_ptr[v]; q < inc_ptr[v + 1]; ++q) {
    const int64_t code = inc[q];
    for (int a = 0; a < dim; ++a) acc[a] += scratch[code * dim + a];
  }
  for (int a = 0; a < dim; ++a) dX[a * nverts + v] = acc[a];
}

}  // namespace fem_vjp

struct FemPattern;
namespace fem {
// accessors implemented in fem_abi.cu
const Pattern* pattern_of(const FemPattern* h);
int new_pattern_handle(Pattern* P, FemPattern** out);
void set_error(int code, const char* fmt, ...);
}  // namespace fem

namespace {

int gather(const FemMesh* m, const FemPattern* vinc, const double* scratch, double* dX,
           cudaStream_t st) {
  if (!dX) return 0;
  const fem::Pattern* P = fem::pattern_of(vinc);
  if (!P || P->nrows != m->nverts || P->nelems != m->nelems || P->nbfun_v != m->nloc) {
    fem::set_error(FEM_ERR_ARGUMENT, "vertex incidence does not belong to this mesh");
    return FEM_ERR_ARGUMENT;
  }
  if (m->nverts == 0) return 0;
  fem_vjp::vertex_gather_kernel<<<(unsigned)fem::ceil_div(m->nverts, 256), 256, 0, st>>>(
      P->inc_ptr, P->inc, m->nverts, m->dim, scratch, dX);
  FEM_LAUNCH_CHECK("vertex_gather_kernel");
  return 0;
}

int check_basis(const FemMesh* m, const FemBasis* b) {
  if (!m || !b) {
    fem::set_error(FEM_ERR_ARGUMENT, "null mesh or basis");
    return FEM_ERR_ARGUMENT;
  }
  if (b->vector) {
    fem::set_error(FEM_ERR_UNSUPPORTED, "the adjoint is implemented for scalar bases");
    return FEM_ERR_UNSUPPORTED;
  }
  if (fem::basis_dim(b->family) != m->dim) {
    fem::set_error(FEM_ERR_ARGUMENT, "Incompatible Mesh and Element.");
    return FEM_ERR_ARGUMENT;
  }
  return 0;
}

}  // namespace

extern "C" {

int fem_vertex_incidence_build(const FemMesh* mesh, FemPattern** out, fem_stream_t stream) {
  if (!mesh || !out) {
    fem::set_error(FEM_ERR_ARGUMENT, "null mesh or output");
    return FEM_ERR_ARGUMENT;
  }
  fem::Pattern* P = new fem::Pattern();
  int rc = fem::build_incidence(mesh->t, mesh->nelems, mesh->nloc, mesh->nverts, P,
                                (cudaStream_t)stream);
  if (rc) {
    delete P;
    return rc;
  }
  return fem::new_pattern_handle(P, out);
}

int fem_bilinear_vjp(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                     const FemPattern* vertex_incidence, const double* w, const double* u,
                     double* dcoef_diff, double* dcoef_mass, double* dX, double* elem_scratch,
                     fem_stream_t stream) {
  int rc = check_basis(mesh, basis);
  if (rc) return rc;
  if (!form || !w || !u || (dX && !elem_scratch)) {
    fem::set_error(FEM_ERR_ARGUMENT, "null form, vectors or scratch");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (mesh->nelems == 0) return 0;
  double* scratch = elem_scratch;
  const unsigned grid = (unsigned)fem::ceil_div(mesh->nelems, 128);
  switch (basis->family) {
    case FEM_TRI_P1:
      fem_vjp::simplex_bilinear_vjp_kernel<2, 1><<<grid, 128, 0, st>>>(
          *mesh, *basis, *form, w, u, dcoef_diff, dcoef_mass, scratch);
      break;
    case FEM_TRI_P2:
      fem_vjp::simplex_bilinear_vjp_kernel<2, 2><<<grid, 128, 0, st>>>(
          *mesh, *basis, *form, w, u, dcoef_diff, dcoef_mass, scratch);
      break;
    case FEM_TET_P1:
      fem_vjp::simplex_bilinear_vjp_kernel<3, 1><<<grid, 128, 0, st>>>(
          *mesh, *basis, *form, w, u, dcoef_diff, dcoef_mass, scratch);
      break;
    case FEM_TET_P2:
      fem_vjp::simplex_bilinear_vjp_kernel<3, 2><<<grid, 128, 0, st>>>(
          *mesh, *basis, *form, w, u, dcoef_diff, dcoef_mass, scratch);
      break;
    case FEM_HEX_1:
      fem_vjp::hex_vjp_kernel<0><<<grid, 128, 0, st>>>(*mesh, *basis, form->diff, form->mass, w,
                                                      u, dcoef_diff, dcoef_mass, scratch, nullptr);
      break;
    default:
      fem::set_error(FEM_ERR_UNSUPPORTED, "unsupported family %d", basis->family);
      return FEM_ERR_UNSUPPORTED;
  }
  FEM_LAUNCH_CHECK("bilinear vjp kernel");
  return gather(mesh, vertex_incidence, scratch, dX, st);
}

int fem_linear_vjp(const FemMesh* mesh, const FemBasis* basis, const FemLinear* form,
                   const FemPattern* vertex_incidence, const double* w, double* dload, double* dX,
                   double* elem_scratch, fem_stream_t stream) {
  int rc = check_basis(mesh, basis);
  if (rc) return rc;
  if (!form || !w || (dX && !elem_scratch)) {
    fem::set_error(FEM_ERR_ARGUMENT, "null form, vector or scratch");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (mesh->nelems == 0) return 0;
  const unsigned grid = (unsigned)fem::ceil_div(mesh->nelems, 128);
  switch (basis->family) {
    case FEM_TRI_P1:
      fem_vjp::simplex_linear_vjp_kernel<2, 1><<<grid, 128, 0, st>>>(*mesh, *basis, *form, w, dload,
                                                                     elem_scratch);
      break;
    case FEM_TRI_P2:
      fem_vjp::simplex_linear_vjp_kernel<2, 2><<<grid, 128, 0, st>>>(*mesh, *basis, *form, w, dload,
                                                                     elem_scratch);
      break;
    case FEM_TET_P1:
      fem_vjp::simplex_linear_vjp_kernel<3, 1><<<grid, 128, 0, st>>>(*mesh, *basis, *form, w, dload,
                                                                     elem_scratch);
      break;
    case FEM_TET_P2:
      fem_vjp::simplex_linear_vjp_kernel<3, 2><<<grid, 128, 0, st>>>(*mesh, *basis, *form, w, dload,
                                                                     elem_scratch);
      break;
    case FEM_HEX_1:
      fem_vjp::hex_vjp_kernel<1><<<grid, 128, 0, st>>>(*mesh, *basis, form->load, FemCoef{0.0, nullptr},
                                                      w, nullptr, dload, nullptr, elem_scratch,
                                                      nullptr);
      break;
    default:
      fem::set_error(FEM_ERR_UNSUPPORTED, "unsupported family %d", basis->family);
      return FEM_ERR_UNSUPPORTED;
  }
  FEM_LAUNCH_CHECK("linear vjp kernel");
  return gather(mesh, vertex_incidence, elem_scratch, dX, st);
}

}  // extern "C"
