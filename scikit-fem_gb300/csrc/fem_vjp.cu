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
using fem::hex_corner;

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
  vol = fem::abs_bits(det) / Traits<D, 1>::FACT;
}

// local DOF of the P2 edge function between vertices a != c (element_tri_p2.py:
// edges 01, 12, 02; element_tet_p2.py: 01, 12, 02, 03, 13, 23)
template <int D>
__device__ __forceinline__ constexpr int edge_dof(int a, int c) {
  const int lo = a < c ? a : c, hi = a < c ? c : a;
  if (D == 2) return lo == 0 ? (hi == 1 ? 3 : 5) : 4;
  if (lo == 0) return hi == 1 ? 4 : (hi == 2 ? 6 : 7);
  if (lo == 1) return hi == 2 ? 5 : 8;
  return 9;
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
  const bool need_mass = f.mass.scale != 0.0 || dcm != nullptr;
#define W(i) wl[i]
#define U(i) ul[i]
#define QQ(a, c) Q[a][c]
  if constexpr (ORDER == 1) {
    // P1: grad phi_a = grad lambda_a, so Q_ab = w_a u_b
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int c = 0; c < NV; ++c) Q[a][c] = wl[a] * ul[c];
    if (need_mass) {
      if constexpr (D == 2) { TRI1_MACC(W, U, mu); } else { TET1_MACC(W, U, mu); }
    }
  } else {
    // P2 in barycentric form: sum_i w_i p_ia = sum_c alpha_ac lambda_c with
    // alpha_aa = 3 w_a, alpha_ac = 4 w_(edge a-c) - w_a, and
    // (1/|T|) int lambda_c lambda_d = (1 + delta_cd) kappa, kappa = 1/((d+1)(d+2)),
    // so Q = kappa (alpha beta^T + (alpha 1)(beta 1)^T).
    constexpr double kappa = 1.0 / ((D + 1) * (D + 2));
    double al[NV][NV], be[NV][NV], ra[NV], rb[NV];
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      ra[a] = 0.0;
      rb[a] = 0.0;
#pragma unroll
      for (int c = 0; c < NV; ++c) {
        if (a == c) {
          al[a][c] = 3.0 * wl[a];
          be[a][c] = 3.0 * ul[a];
        } else {
          const int ed = edge_dof<D>(a, c);
          al[a][c] = 4.0 * wl[ed] - wl[a];
          be[a][c] = 4.0 * ul[ed] - ul[a];
        }
        ra[a] += al[a][c];
        rb[a] += be[a][c];
      }
    }
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int c = 0; c < NV; ++c) {
        double v = ra[a] * rb[c];
#pragma unroll
        for (int k = 0; k < NV; ++k) v += al[a][k] * be[c][k];
        Q[a][c] = kappa * v;
      }
    if (need_mass) {
      if constexpr (D == 2) { TRI2_MACC(W, U, mu); } else { TET2_MACC(W, U, mu); }
    }
  }
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
  // P = (Q + Q^T) G -- the vertex gradients, only when dX was asked for
  // (scratch null: the coefficient gradients alone)
  if (!scratch) return;
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
  if (!scratch) return;
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
    const int cx = hex_corner(n, 0), cy = hex_corner(n, 1), cz = hex_corner(n, 2);
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

// Parallelepiped cells (constant J): the 2x2x2 Gauss rule is exact for
// every adjoint integrand, and the trilinear tensor structure makes all
// quadrature-point values sum-factorisable.  Corner (cx,cy,cz) of the
// reference cube carries nodal value V[cx][cy][cz]; B[c][q] = f_c(g_q) with
// f_0(t) = 1 - t, f_1(t) = t at the two Gauss points.
//   grad_ref v at (qx,qy,qz):  d_x v = sum_{cy,cz} (V[1][cy][cz] - V[0][cy][cz]) B[cy][qy] B[cz][qz], ...
// With G = J^-1, M' = G G^T, c = w_q |det J| and a, b the reference
// gradients of w_h, u_h, the per-point stress-like matrix is
//   Z_q = c [ (kd a.M'b + km w_h u_h) I - kd (a (M'b)^T + b (M'a)^T) ]
// and dE/dx_n = G^T R_n,  R_n[r] = sum_q sum_m Z_q[r][m] d_m phi_n(q), which
// is again a tensor-product contraction.
template <int MODE>
__device__ __forceinline__ void hex_vjp_affine(const double x[8][3], const double wl[8],
                                               const double ul[8], double kd, double km,
                                               double& Ed, double& Em, double gx[8][3],
                                               int32_t* status) {
  double J[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    J[k][0] = x[4][k] - x[7][k];
    J[k][1] = x[5][k] - x[7][k];
    J[k][2] = x[6][k] - x[7][k];
  }
  double ad[3][3];
  const double det = adj3(J, ad);
  if (fem::zero_bits(det)) {
    if (status) atomicOr(status, 1 << FEM_ERR_ZERO_JACOBIAN);
    return;
  }
  const double inv = 1.0 / det, adet = fem::abs_bits(det);
  double Gm[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) Gm[a][c] = ad[a][c] * inv;
  double Mp[3][3];  // G G^T
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = a; c < 3; ++c) {
      const double v = Gm[a][0] * Gm[c][0] + Gm[a][1] * Gm[c][1] + Gm[a][2] * Gm[c][2];
      Mp[a][c] = v;
      Mp[c][a] = v;
    }
  // nodal values on the corner grid V[cx][cy][cz]
  double W[2][2][2], U[2][2][2];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    W[hex_corner(n, 0)][hex_corner(n, 1)][hex_corner(n, 2)] = wl[n];
    U[hex_corner(n, 0)][hex_corner(n, 1)][hex_corner(n, 2)] = ul[n];
  }
  const double g0 = c_gl2_x[0], g1 = c_gl2_x[1];
  const double B[2][2] = {{1.0 - g0, 1.0 - g1}, {g0, g1}};
  // BB[i][j][qa][qb] = B[i][qa] * B[j][qb], shared by every transform below
  double BB[2][2][2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int qa = 0; qa < 2; ++qa)
#pragma unroll
        for (int qb = 0; qb < 2; ++qb) BB[i][j][qa][qb] = B[i][qa] * B[j][qb];
  // Reference gradients at the 8 points, stored compactly: d_x v depends on
  // (qy, qz) only, d_y v on (qx, qz), d_z v on (qx, qy).
  auto grad4 = [&](const double V[2][2][2], double gx_[2][2], double gy_[2][2],
                   double gz_[2][2]) {
    double Dx[2][2], Dy[2][2], Dz[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        Dx[i][j] = V[1][i][j] - V[0][i][j];  // (cy, cz)
        Dy[i][j] = V[i][1][j] - V[i][0][j];  // (cx, cz)
        Dz[i][j] = V[i][j][1] - V[i][j][0];  // (cx, cy)
      }
#pragma unroll
    for (int qa = 0; qa < 2; ++qa)
#pragma unroll
      for (int qb = 0; qb < 2; ++qb) {
        double tx = 0.0, ty = 0.0, tz = 0.0;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const double f = BB[i][j][qa][qb];
            tx += f * Dx[i][j];
            ty += f * Dy[i][j];
            tz += f * Dz[i][j];
          }
        gx_[qa][qb] = tx;
        gy_[qa][qb] = ty;
        gz_[qa][qb] = tz;
      }
  };
  double wx[2][2], wy[2][2], wz[2][2], ux[2][2], uy[2][2], uz[2][2];
  grad4(W, wx, wy, wz);
  if (MODE == 0) grad4(U, ux, uy, uz);
  // values at the 8 points (mass / load terms)
  double Wv[2][2][2], Uv[2][2][2];
  auto value8 = [&](const double V[2][2][2], double out[2][2][2]) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          double acc = 0.0;
#pragma unroll
          for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
              for (int k = 0; k < 2; ++k) acc += V[i][j][k] * (B[i][q] * B[j][r] * B[k][t]);
          out[q][r][t] = acc;
        }
  };
  const bool need_vals = (MODE == 1) || (km != 0.0);
  if (need_vals) {
    value8(W, Wv);
    if (MODE == 0) value8(U, Uv);
  }
  const double c = 0.125 * adet;  // Gauss weights (1/2)^3
  // Partial sums of Z_q over the quadrature index of each derivative
  // direction: Sx[r][qy][qz] = sum_qx Z_q[r][x], Sy[r][qx][qz], Sz[r][qx][qy].
  double Sx[3][2][2], Sy[3][2][2], Sz[3][2][2];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) Sx[r][i][j] = Sy[r][i][j] = Sz[r][i][j] = 0.0;
#pragma unroll
  for (int qx = 0; qx < 2; ++qx)
#pragma unroll
    for (int qy = 0; qy < 2; ++qy)
#pragma unroll
      for (int qz = 0; qz < 2; ++qz) {
        double Z[3][3];
        if (MODE == 0) {
          const double a[3] = {wx[qy][qz], wy[qx][qz], wz[qx][qy]};
          const double b[3] = {ux[qy][qz], uy[qx][qz], uz[qx][qy]};
          double ap[3], bp[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            ap[k] = Mp[k][0] * a[0] + Mp[k][1] * a[1] + Mp[k][2] * a[2];
            bp[k] = Mp[k][0] * b[0] + Mp[k][1] * b[1] + Mp[k][2] * b[2];
          }
          const double s = a[0] * bp[0] + a[1] * bp[1] + a[2] * bp[2];
          const double wu = need_vals ? Wv[qx][qy][qz] * Uv[qx][qy][qz] : 0.0;
          Ed += c * s;
          Em += c * wu;
          const double P = c * (kd * s + km * wu);
          const double ck = c * kd;
          // Z_q = P I - ck (a bp^T + b ap^T), added straight into the partial sums
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            ap[k] *= ck;
            bp[k] *= ck;
          }
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            Sx[r][qy][qz] = Sx[r][qy][qz] - a[r] * bp[0] - b[r] * ap[0];
            Sy[r][qx][qz] = Sy[r][qx][qz] - a[r] * bp[1] - b[r] * ap[1];
            Sz[r][qx][qy] = Sz[r][qx][qy] - a[r] * bp[2] - b[r] * ap[2];
          }
          Sx[0][qy][qz] += P;
          Sy[1][qx][qz] += P;
          Sz[2][qx][qy] += P;
          continue;
        } else {
          const double wv = Wv[qx][qy][qz];
          Ed += c * wv;
          const double P = c * kd * wv;
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int mm = 0; mm < 3; ++mm) Z[r][mm] = (r == mm ? P : 0.0);
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          Sx[r][qy][qz] += Z[r][0];
          Sy[r][qx][qz] += Z[r][1];
          Sz[r][qx][qy] += Z[r][2];
        }
      }
  // R_n[r] = sum_m sum_q Z_q[r][m] d_m phi_n(q): transposed interpolation of
  // the partial sums, sign by the node's corner in the derivative direction.
  double R[2][2][2][3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    double Hx[2][2], Hy[2][2], Hz[2][2];
#pragma unroll
    for (int ca = 0; ca < 2; ++ca)
#pragma unroll
      for (int cb = 0; cb < 2; ++cb) {
        double hx = 0.0, hy = 0.0, hz = 0.0;
#pragma unroll
        for (int qa = 0; qa < 2; ++qa)
#pragma unroll
          for (int qb = 0; qb < 2; ++qb) {
            const double f = BB[ca][cb][qa][qb];
            hx += f * Sx[r][qa][qb];
            hy += f * Sy[r][qa][qb];
            hz += f * Sz[r][qa][qb];
          }
        Hx[ca][cb] = hx;
        Hy[ca][cb] = hy;
        Hz[ca][cb] = hz;
      }
#pragma unroll
    for (int cx = 0; cx < 2; ++cx)
#pragma unroll
      for (int cy = 0; cy < 2; ++cy)
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
          R[cx][cy][cz][r] = (cx ? Hx[cy][cz] : -Hx[cy][cz]) + (cy ? Hy[cx][cz] : -Hy[cx][cz]) +
                             (cz ? Hz[cx][cy] : -Hz[cx][cy]);
  }
  // dE/dx_n = G^T R_n
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const double* Rn = R[hex_corner(n, 0)][hex_corner(n, 1)][hex_corner(n, 2)];
#pragma unroll
    for (int k = 0; k < 3; ++k) gx[n][k] = Gm[0][k] * Rn[0] + Gm[1][k] * Rn[1] + Gm[2][k] * Rn[2];
  }
}

// Non-parallelepiped cells: the 4x4x4 isoparametric rule (kept out of line
// so that its registers do not load the common parallelepiped path).
// tab: the reference element's values [64][8], gradients [64][8][3] and the
// points' weights [64] (shared memory, filled once per block).
template <int MODE>
__device__ __noinline__ void hex_vjp_general(const FemMesh m, const FemBasis b, const FemCoef cd,
                                             const FemCoef cm, const double* __restrict__ w,
                                             const double* __restrict__ u, double* dcd,
                                             double* dcm, double* scratch, int32_t* status,
                                             int64_t e, const double* tab) {
  const int nq = 4;
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
  const double kd = coef_at(cd, e), km = MODE == 0 ? coef_at(cm, e) : 0.0;
  double Ed = 0.0, Em = 0.0;
  double gx[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int k = 0; k < 3; ++k) gx[n][k] = 0.0;
  // the mass channel's terms only when it is present or its gradient is asked for
  const bool mass = MODE == 0 && (dcm != nullptr || !fem::zero_bits(km));
  for (int q = 0; q < nq * nq * nq; ++q) {
    const double* phi = tab + q * 8;
    const double (*dphi)[3] = reinterpret_cast<const double (*)[3]>(tab + 64 * 8 + q * 24);
    const double wq = tab[64 * 32 + q];
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
    if (fem::zero_bits(det)) {
      if (status) atomicOr(status, 1 << FEM_ERR_ZERO_JACOBIAN);
      continue;
    }
    const double inv = 1.0 / det, adet = fem::abs_bits(det);
    double Gm[3][3];  // G = J^{-1}
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) Gm[a][c] = ad[a][c] * inv;
    double ar[3] = {0, 0, 0}, br[3] = {0, 0, 0}, wv = 0.0, uv = 0.0;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      if (mass || MODE == 1) wv += wl[n] * phi[n];
      if (mass) uv += ul[n] * phi[n];
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
      double c0;
      if (mass) {
        Em += cdf * wv * uv;
        c0 = cdf * (kd * s + km * wv * uv);
      } else {
        c0 = cdf * (kd * s);
      }
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
  if (!scratch) return;   // no dX asked for: the coefficient gradients alone
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int a = 0; a < 3; ++a) scratch[(e * 8 + n) * 3 + a] = gx[n][a];
}

// mode 0: bilinear (diff, mass); mode 1: linear (load * v)
template <int MODE>
__global__ void hex_vjp_kernel(FemMesh m, FemBasis b, FemCoef cd, FemCoef cm,
                               const double* __restrict__ w, const double* __restrict__ u,
                               double* __restrict__ dcd, double* __restrict__ dcm,
                               double* __restrict__ scratch, int32_t* __restrict__ status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = e < m.nelems;
  double x[8][3], wl[8], ul[8];
  bool affine = true;
  if (live) {
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
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double v = x[7][k];
        if (hex_corner(n, 0)) v = v + (x[4][k] - x[7][k]);
        if (hex_corner(n, 1)) v = v + (x[5][k] - x[7][k]);
        if (hex_corner(n, 2)) v = v + (x[6][k] - x[7][k]);
        affine = affine && (v == x[n][k]);
      }
  }
  // the reference element at the 64 points, once per block that holds a
  // general cell (their 4x4x4 rule)
  __shared__ double tab[64 * 33];
  if (__syncthreads_or(affine ? 0 : 1)) {
    for (int q = threadIdx.x; q < 64; q += blockDim.x) {
      const int qx = q & 3, qy = (q >> 2) & 3, qz = q >> 4;
      double phi[8], dphi[8][3];
      hex_shape(c_gl4_x[qx], c_gl4_x[qy], c_gl4_x[qz], phi, dphi);
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        tab[q * 8 + n] = phi[n];
#pragma unroll
        for (int k = 0; k < 3; ++k) tab[64 * 8 + (q * 8 + n) * 3 + k] = dphi[n][k];
      }
      tab[64 * 32 + q] = c_gl4_w[qx] * c_gl4_w[qy] * c_gl4_w[qz];
    }
    __syncthreads();
  }
  if (!live) return;
  const double kd = coef_at(cd, e), km = MODE == 0 ? coef_at(cm, e) : 0.0;
  double Ed = 0.0, Em = 0.0;
  double gx[8][3];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int k = 0; k < 3; ++k) gx[n][k] = 0.0;
  if (!affine) {
    hex_vjp_general<MODE>(m, b, cd, cm, w, u, dcd, dcm, scratch, status, e, tab);
    return;
  }
  hex_vjp_affine<MODE>(x, wl, ul, kd, km, Ed, Em, gx, status);
  if (dcd) dcd[e] = cd.scale * Ed;
  if (MODE == 0 && dcm) dcm[e] = cm.scale * Em;
  if (!scratch) return;   // no dX asked for: the coefficient gradients alone
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
