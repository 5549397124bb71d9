// Host/device core of the exact-zero mask (see fem_faithful.cu): the
// reference's basis expressions, mapping formulas, quadrature sum and the
// form-program interpreter, in separately rounded IEEE double arithmetic.
// Compile with -fmad=false (device) and without FMA contraction (host).
#pragma once

#ifndef __CUDACC_RTC__
#include <cmath>
#include <stdint.h>
#endif

#include "../../include/skfem_gb300.h"

#ifdef __CUDACC__
#define FEM_HD __host__ __device__ inline
#else
#define FEM_HD inline
#endif

namespace fem_faithful {

constexpr int kMaxProgram = 512;
constexpr int kMaxCoef = 16;
constexpr int kMaxPoints = 128;

using Instr = FemInstr;

// Program operations.  CONST..NEG, X, H, SQRT and ABS are correctly rounded
// (bitwise the reference's); EXP..ARCTAN and POW call the CUDA / C math
// library, whose last bits may differ from numpy's.
enum {
  OP_CONST = 0, OP_U, OP_V, OP_COEF, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_X, OP_H,
  OP_SQRT, OP_EXP, OP_LOG, OP_SIN, OP_COS, OP_TAN, OP_TANH, OP_ARCTAN, OP_ABS, OP_POW, OP_N
};

// ----------------------------------------------------------- reference bases
FEM_HD void lbasis(int family, int i, double x, double y, double z, double& phi,
                       double d[3]) {
  d[0] = d[1] = d[2] = 0.0;
  switch (family) {
    case FEM_TRI_P1:
      if (i == 0) { phi = (1. - x) - y; d[0] = -1. + 0. * x; d[1] = -1. + 0. * x; }
      else if (i == 1) { phi = x; d[0] = 1. + 0. * x; d[1] = 0. * x; }
      else { phi = y; d[0] = 0. * x; d[1] = 1. + 0. * x; }
      return;
    case FEM_TET_P1:
      if (i == 0) { phi = ((1 - x) - y) - z; d[0] = d[1] = d[2] = -1 + 0 * x; }
      else if (i == 1) { phi = x; d[0] = 1 + 0 * x; d[1] = 0 * x; d[2] = 0 * x; }
      else if (i == 2) { phi = y; d[0] = 0 * x; d[1] = 1 + 0 * x; d[2] = 0 * x; }
      else { phi = z; d[0] = 0 * x; d[1] = 0 * x; d[2] = 1 + 0 * x; }
      return;
    case FEM_TRI_P2:
      switch (i) {
        case 0:
          phi = ((((1. - 3. * x) - 3. * y) + 2. * (x * x)) + (4. * x) * y) + 2. * (y * y);
          d[0] = (-3 + 4. * x) + 4. * y;
          d[1] = (-3 + 4. * x) + 4. * y;
          return;
        case 1: phi = 2. * (x * x) - x; d[0] = 4. * x - 1; d[1] = 0. * x; return;
        case 2: phi = 2. * (y * y) - y; d[0] = 0. * x; d[1] = 4. * y - 1; return;
        case 3:
          phi = (4. * x - 4. * (x * x)) - (4. * x) * y;
          d[0] = (4 - 8. * x) - 4. * y;
          d[1] = -4. * x;
          return;
        case 4: phi = (4. * x) * y; d[0] = 4. * y; d[1] = 4. * x; return;
        default:
          phi = (4. * y - (4. * x) * y) - 4. * (y * y);
          d[0] = -4. * y;
          d[1] = (4 - 4. * x) - 8. * y;
          return;
      }
    case FEM_TET_P2:
      switch (i) {
        case 0: {
          phi = ((((((((1. - 3. * x) + 2. * (x * x)) - 3. * y) + (4. * x) * y) + 2. * (y * y)) -
                   3. * z) + (4. * x) * z) + (4. * y) * z) + 2. * (z * z);
          const double g = ((-3. + 4. * x) + 4. * y) + 4. * z;
          d[0] = d[1] = d[2] = g;
          return;
        }
        case 1: phi = -1. * x + 2. * (x * x); d[0] = -1 + 4 * x; d[1] = 0 * x; d[2] = 0 * x; return;
        case 2: phi = -1. * y + 2. * (y * y); d[0] = 0 * x; d[1] = -1. + 4. * y; d[2] = 0 * x; return;
        case 3: phi = -1. * z + 2. * (z * z); d[0] = 0 * x; d[1] = 0 * x; d[2] = -1. + 4. * z; return;
        case 4:
          phi = ((4. * x - 4. * (x * x)) - (4. * x) * y) - (4 * x) * z;
          d[0] = ((4. - 8. * x) - 4. * y) - 4. * z;
          d[1] = -4. * x;
          d[2] = -4. * x;
          return;
        case 5: phi = (4. * x) * y; d[0] = 4. * y; d[1] = 4. * x; d[2] = 0 * x; return;
        case 6:
          phi = (((0. + 4. * y) - (4. * x) * y) - 4. * (y * y)) - (4. * y) * z;
          d[0] = -4. * y;
          d[1] = ((4. - 4. * x) - 8. * y) - 4. * z;
          d[2] = -4. * y;
          return;
        case 7:
          phi = (((0. + 4. * z) - (4. * x) * z) - (4. * y) * z) - 4. * (z * z);
          d[0] = -4. * z;
          d[1] = -4. * z;
          d[2] = ((4. - 4. * x) - 4. * y) - 8. * z;
          return;
        case 8: phi = 0. + (4. * x) * z; d[0] = 4. * z; d[1] = 0 * x; d[2] = 4 * x; return;
        default: phi = 0. + (4. * y) * z; d[0] = 0 * x; d[1] = 4 * z; d[2] = 4 * y; return;
      }
    case FEM_HEX_1:
      switch (i) {
        case 0: phi = (x * y) * z; d[0] = y * z; d[1] = x * z; d[2] = x * y; return;
        case 1: phi = (x * y) * (1 - z); d[0] = y * (1 - z); d[1] = x * (1 - z); d[2] = (-x) * y; return;
        case 2: phi = (x * (1 - y)) * z; d[0] = (1 - y) * z; d[1] = (-x) * z; d[2] = x * (1 - y); return;
        case 3: phi = ((1 - x) * y) * z; d[0] = (-y) * z; d[1] = (1 - x) * z; d[2] = (1 - x) * y; return;
        case 4:
          phi = (x * (1 - y)) * (1 - z);
          d[0] = (1 - y) * (1 - z); d[1] = (-x) * (1 - z); d[2] = (-x) * (1 - y);
          return;
        case 5:
          phi = ((1 - x) * y) * (1 - z);
          d[0] = (-y) * (1 - z); d[1] = (1 - x) * (1 - z); d[2] = (-(1 - x)) * y;
          return;
        case 6:
          phi = ((1 - x) * (1 - y)) * z;
          d[0] = (-(1 - y)) * z; d[1] = (-(1 - x)) * z; d[2] = (1 - x) * (1 - y);
          return;
        default:
          phi = ((1 - x) * (1 - y)) * (1 - z);
          d[0] = (-(1 - y)) * (1 - z); d[1] = (-(1 - x)) * (1 - z); d[2] = (-(1 - x)) * (1 - y);
          return;
      }
    default:
      phi = 0.0;
      return;
  }
}

// ------------------------------------------------------ reference quadrature
struct Rule {
  const double* X;  // (dim, nq) row-major
  const double* W;
  int nq;
};

// numpy's pairwise summation for n <= 128 (as measured on the reference's
// platform: sequential below 8 terms, else eight accumulators)
FEM_HD double np_pairwise_sum(const double* a, int n) {
  if (n < 8) {
    double res = -0.0;
    for (int i = 0; i < n; ++i) res = res + a[i];
    return res;
  }
  double r[8];
  for (int j = 0; j < 8; ++j) r[j] = a[j];
  int i = 8;
  for (; i < n - (n % 8); i += 8)
    for (int j = 0; j < 8; ++j) r[j] = r[j] + a[i + j];
  double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
  for (; i < n; ++i) res = res + a[i];
  return res;
}

// ---------------------------------------------------------------- mappings
template <int D>
FEM_HD void affine_inverse(const FemMesh& m, int64_t e, double inv[3][3], double& det,
                           double A[3][3], double x0[3]) {
  for (int i = 0; i < D; ++i) x0[i] = m.p[i * m.nverts + m.t[e]];
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j)
      A[i][j] = m.p[i * m.nverts + m.t[(j + 1) * m.nelems + e]] - m.p[i * m.nverts + m.t[e]];
  if (D == 2) {
    det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    inv[0][0] = A[1][1] / det;
    inv[0][1] = (-A[0][1]) / det;
    inv[1][0] = (-A[1][0]) / det;
    inv[1][1] = A[0][0] / det;
  } else {
    det = (A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
           A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0])) +
          A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    inv[0][0] = ((-A[1][2]) * A[2][1] + A[1][1] * A[2][2]) / det;
    inv[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
    inv[2][0] = ((-A[1][1]) * A[2][0] + A[1][0] * A[2][1]) / det;
    inv[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
    inv[1][1] = ((-A[0][2]) * A[2][0] + A[0][0] * A[2][2]) / det;
    inv[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
    inv[0][2] = ((-A[0][2]) * A[1][1] + A[0][1] * A[1][2]) / det;
    inv[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
    inv[2][2] = ((-A[0][1]) * A[1][0] + A[0][0] * A[1][1]) / det;
  }
}

FEM_HD void hex_inverse(const FemMesh& m, int64_t e, double x, double y, double z,
                            double inv[3][3], double& det) {
  double J[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J[i][j] = 0.0;
  for (int itr = 0; itr < 8; ++itr) {
    double phi, d[3];
    lbasis(FEM_HEX_1, itr, x, y, z, phi, d);
    const int64_t v = m.t[itr * m.nelems + e];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) J[i][j] = J[i][j] + m.p[i * m.nverts + v] * d[j];
  }
  det = (J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0])) +
        J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  inv[0][0] = ((-J[1][2]) * J[2][1] + J[1][1] * J[2][2]) / det;
  inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  inv[2][0] = ((-J[1][1]) * J[2][0] + J[1][0] * J[2][1]) / det;
  inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  inv[1][1] = ((-J[0][2]) * J[2][0] + J[0][0] * J[2][2]) / det;
  inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  inv[0][2] = ((-J[0][2]) * J[1][1] + J[0][1] * J[1][2]) / det;
  inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  inv[2][2] = ((-J[0][1]) * J[1][0] + J[0][0] * J[1][1]) / det;
}

// quantities of local function `fn` at a point: q[c] values, q[ncomp + c*D + k] derivatives
template <int D>
FEM_HD void quantities(int family, bool vec, int fn, double x, double y, double z,
                           const double inv[3][3], double* q) {
  const int sfn = vec ? fn / D : fn;
  const int comp = vec ? fn % D : 0;
  const int ncomp = vec ? D : 1;
  double phi, d[3];
  lbasis(family, sfn, x, y, z, phi, d);
  double g[3];
  for (int j = 0; j < D; ++j) {
    double s = 0.0;
    for (int i = 0; i < D; ++i) s = s + inv[i][j] * d[i];
    g[j] = s;
  }
  for (int c = 0; c < ncomp; ++c) {
    q[c] = (c == comp) ? phi : 0.0;
    for (int k = 0; k < D; ++k) q[ncomp + c * D + k] = (c == comp) ? g[k] : 0.0;
  }
}

// P1 families: the reference gradients are constant (lbasis writes them as
// c + 0*x), so on an affine cell every quantity's derivative part is the
// same at every point -- computed once and reused, the same numbers.
FEM_HD bool point_free_gradients(int family) {
  return family == FEM_TRI_P1 || family == FEM_TET_P1;
}

// quantities() with the derivative part taken from qg (the quantities of the
// same function at another point of the same affine cell, P1 families) and
// the values evaluated here.
template <int D>
FEM_HD void quantities_values(int family, bool vec, int fn, double x, double y, double z,
                              const double* qg, double* q) {
  const int sfn = vec ? fn / D : fn;
  const int comp = vec ? fn % D : 0;
  const int ncomp = vec ? D : 1;
  double phi, d[3];
  lbasis(family, sfn, x, y, z, phi, d);
  for (int c = 0; c < ncomp; ++c) {
    q[c] = (c == comp) ? phi : 0.0;
    for (int k = 0; k < D; ++k) q[ncomp + c * D + k] = qg[ncomp + c * D + k];
  }
}

FEM_HD double run(const Instr* ins, int n, int out, const double* qu, const double* qv,
                      const double* coef, const double* qx, double* R) {
  for (int k = 0; k < n; ++k) {
    const Instr I = ins[k];
    double r = 0.0;
    switch (I.op) {
      case OP_CONST: r = I.imm; break;
      case OP_U: r = qu[I.a]; break;
      case OP_V: r = qv[I.a]; break;
      case OP_COEF: r = coef[I.a]; break;
      case OP_ADD: r = R[I.a] + R[I.b]; break;
      case OP_SUB: r = R[I.a] - R[I.b]; break;
      case OP_MUL: r = R[I.a] * R[I.b]; break;
      case OP_DIV: r = R[I.a] / R[I.b]; break;
      case OP_NEG: r = -R[I.a]; break;
      case OP_X: r = qx[I.a]; break;
      case OP_H: r = qx[3]; break;
      case OP_SQRT: r = sqrt(R[I.a]); break;
      case OP_EXP: r = exp(R[I.a]); break;
      case OP_LOG: r = log(R[I.a]); break;
      case OP_SIN: r = sin(R[I.a]); break;
      case OP_COS: r = cos(R[I.a]); break;
      case OP_TAN: r = tan(R[I.a]); break;
      case OP_TANH: r = tanh(R[I.a]); break;
      case OP_ARCTAN: r = atan(R[I.a]); break;
      case OP_ABS: r = fabs(R[I.a]); break;
      case OP_POW: r = pow(R[I.a], R[I.b]); break;
      case OP_N: r = qx[4 + I.a]; break;
      default: break;
    }
    R[k] = r;
  }
  return R[out];
}

// Global coordinates of a reference point: MappingAffine.F
// (mapping_affine.py:183-193: sum_j A[i][j] X_j in j order, then + b_i) or
// MappingIsoparametric.Fmap (mapping_isoparametric.py:50-58: sum over nodes
// of p_i(node) phi_node(X) from 0).
template <int D>
FEM_HD void global_coords(const FemMesh& m, int64_t e, bool hex, const double A[3][3],
                          const double x0[3], double x, double y, double z, double* qx) {
  const double X[3] = {x, y, z};
  if (!hex) {
    for (int i = 0; i < D; ++i) {
      double s = 0.0;
      for (int j = 0; j < D; ++j) s = s + A[i][j] * X[j];
      qx[i] = s + x0[i];
    }
    return;
  }
  for (int i = 0; i < 3; ++i) qx[i] = 0.0;
  for (int itr = 0; itr < 8; ++itr) {
    double phi, d[3];
    lbasis(FEM_HEX_1, itr, x, y, z, phi, d);
    const int64_t v = m.t[itr * m.nelems + e];
    for (int i = 0; i < 3; ++i) qx[i] = qx[i] + m.p[i * m.nverts + v] * phi;
  }
}

// What a program reads besides the basis functions.
struct ProgFlags {
  bool x = false, h = false;
};
FEM_HD ProgFlags prog_flags(const FemProgram& p) {
  ProgFlags f;
  for (int k = 0; k < p.ninstr; ++k) {
    f.x = f.x || p.ins[k].op == OP_X;
    f.h = f.h || p.ins[k].op == OP_H;
  }
  return f;
}

// Geometry of one quadrature point: invDF, detDF, global coordinates
// (qx[0..2]) and the mesh parameter h = |detDF|**(1/dim) (qx[3],
// cell_basis.py:136-141; numpy evaluates **0.5 as sqrt).
struct PointGeo {
  double inv[3][3];
  double det;     // detDF (cells) or detDG (facets): dx = |det| * W
  double qx[7];   // x, y, z, h, n_x, n_y, n_z
};

struct CellGeo {  // the affine map of a simplex (unused for Hex1)
  double inv[3][3], det, A[3][3], x0[3];
};

template <int D>
FEM_HD void cell_geometry(const FemMesh& m, int64_t e, bool hex, CellGeo& c) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c.inv[i][j] = c.A[i][j] = 0.0;
  c.x0[0] = c.x0[1] = c.x0[2] = 0.0;
  c.det = 0.0;
  if (!hex) affine_inverse<D>(m, e, c.inv, c.det, c.A, c.x0);
}

template <int D>
FEM_HD void point_geometry(const FemMesh& m, int64_t e, bool hex, const CellGeo& c,
                           ProgFlags f, double x, double y, double z, PointGeo& g) {
  if (hex) {
    hex_inverse(m, e, x, y, z, g.inv, g.det);
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) g.inv[i][j] = c.inv[i][j];
    g.det = c.det;
  }
  for (int k = 0; k < 7; ++k) g.qx[k] = 0.0;
  if (f.x) global_coords<D>(m, e, hex, c.A, c.x0, x, y, z, g.qx);
  if (f.h) g.qx[3] = D == 2 ? sqrt(fabs(g.det)) : pow(fabs(g.det), 1.0 / 3.0);
}

// ------------------------------------------------------------------ facets
// Outward normals of the reference cell's facets (refdom.py:60-62, 107-110).
FEM_HD void ref_normal(int D, int lf, double N[3], bool hex = false) {
  N[0] = N[1] = N[2] = 0.0;
  if (hex) {   // refdom.py:182-187
    const double T[6][3] = {{1.0, 0.0, 0.0},  {0.0, 0.0, 1.0},  {0.0, 1.0, 0.0},
                            {0.0, -1.0, 0.0}, {0.0, 0.0, -1.0}, {-1.0, 0.0, 0.0}};
    for (int i = 0; i < 3; ++i) N[i] = T[lf][i];
    return;
  }
  if (D == 2) {
    const double T[3][2] = {{0.0, -1.0}, {1.0, 1.0}, {-1.0, 0.0}};
    N[0] = T[lf][0];
    N[1] = T[lf][1];
  } else {
    const double T[4][3] = {{0.0, 0.0, -1.0}, {0.0, -1.0, 0.0}, {-1.0, 0.0, 0.0},
                            {1.0, 1.0, 1.0}};
    for (int i = 0; i < 3; ++i) N[i] = T[lf][i];
  }
}

// FacetBasis geometry at facet reference point Xf (facet_basis.py:84-106,
// affine simplices): the facet map G (mapping_affine.py:154-181, 234-245)
// x = B Xf + c with B's columns p[facet[j+1]] - p[facet[0]], its measure
// detDG (:166-180, 247-253), the cell's reference point Y = invA (x - b)
// (invF, :195-203), the normal invA_n^T N_ref / |.| of the cell f2t[0]
// (:255-281) and h = |detDG|**(1/(dim-1)) (facet_basis.py:129-135; numpy
// evaluates **1.0 as a copy and **0.5 as sqrt).  Returns false for a facet
// whose cell indices are out of range.
template <int D>
FEM_HD bool facet_point(const FemMesh& m, const FemFacets& fc, int64_t f, const double* Xf,
                        double Y[3], PointGeo& g) {
  const int64_t nf = fc.nfacets;
  const int64_t e = fc.tind[f], en = fc.tind_n[f];
  const int lf = fc.lfacet_n[f];
  if (e < 0 || e >= m.nelems || en < 0 || en >= m.nelems || lf < 0 || lf > D) return false;
  double cc[3], B[3][2];
  for (int i = 0; i < D; ++i) {
    cc[i] = m.p[i * m.nverts + fc.fverts[f]];
    for (int j = 0; j < D - 1; ++j)
      B[i][j] = m.p[i * m.nverts + fc.fverts[(j + 1) * nf + f]] - m.p[i * m.nverts + fc.fverts[f]];
  }
  double x[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < D; ++i) {
    double s = 0.0;
    for (int j = 0; j < D - 1; ++j) s = s + B[i][j] * Xf[j];
    x[i] = s + cc[i];
  }
  double detB;
  if (D == 2) {
    detB = sqrt(B[0][0] * B[0][0] + B[1][0] * B[1][0]);
  } else {
    const double a = B[1][0] * B[2][1] - B[2][0] * B[1][1];
    const double b = (-B[0][0]) * B[2][1] + B[2][0] * B[0][1];
    const double c = B[0][0] * B[1][1] - B[1][0] * B[0][1];
    detB = sqrt((a * a + b * b) + c * c);
  }
  double inv[3][3], det, A[3][3], x0[3];
  affine_inverse<D>(m, e, inv, det, A, x0);
  double y[3];
  for (int i = 0; i < D; ++i) y[i] = x[i] - x0[i];
  for (int i = 0; i < 3; ++i) Y[i] = 0.0;
  for (int i = 0; i < D; ++i) {
    double s = 0.0;
    for (int j = 0; j < D; ++j) s = s + inv[i][j] * y[j];
    Y[i] = s;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) g.inv[i][j] = inv[i][j];
  g.det = detB;
  for (int k = 0; k < 7; ++k) g.qx[k] = 0.0;
  for (int i = 0; i < D; ++i) g.qx[i] = x[i];
  g.qx[3] = D == 2 ? detB : sqrt(detB);
  double invn[3][3], detn, An[3][3], xn[3], N[3], n[3];
  affine_inverse<D>(m, en, invn, detn, An, xn);
  ref_normal(D, lf, N);
  for (int j = 0; j < D; ++j) {
    double s = 0.0;
    for (int i = 0; i < D; ++i) s = s + invn[i][j] * N[i];
    n[j] = s;
  }
  double len2 = n[0] * n[0];
  for (int j = 1; j < D; ++j) len2 = len2 + n[j] * n[j];
  const double rl = 1.0 / sqrt(len2);
  for (int j = 0; j < D; ++j) g.qx[4 + j] = n[j] * rl;
  return true;
}

// ---------------------------------------------------------- Hex1 facets
// ElementQuad1.lbasis (element_quad1.py:24-38), the facets' bilinear map.
FEM_HD void quad1_lbasis(int i, double x, double y, double& phi, double d[2]) {
  switch (i) {
    case 0: phi = (1.0 - x) * (1.0 - y); d[0] = -1.0 + y; d[1] = -1.0 + x; break;
    case 1: phi = x * (1.0 - y); d[0] = 1.0 - y; d[1] = -x; break;
    case 2: phi = x * y; d[0] = y; d[1] = x; break;
    default: phi = (1.0 - x) * y; d[0] = -y; d[1] = 1.0 - x; break;
  }
}

// G(X) and detDG of a quadrilateral facet (mapping_isoparametric.py:60-110,
// 137-155): node sums from 0 in facet-vertex order.
FEM_HD void quad_facet_map(const FemMesh& m, const FemFacets& fc, int64_t f, double u, double v,
                           double x[3], double& detB) {
  double J[3][2];
  for (int i = 0; i < 3; ++i) {
    x[i] = 0.0;
    J[i][0] = J[i][1] = 0.0;
  }
  for (int itr = 0; itr < 4; ++itr) {
    double phi, d[2];
    quad1_lbasis(itr, u, v, phi, d);
    const int64_t vtx = fc.fverts[itr * fc.nfacets + f];
    for (int i = 0; i < 3; ++i) {
      const double pv = m.p[i * m.nverts + vtx];
      x[i] = x[i] + pv * phi;
      J[i][0] = J[i][0] + pv * d[0];
      J[i][1] = J[i][1] + pv * d[1];
    }
  }
  const double a = J[1][0] * J[2][1] - J[2][0] * J[1][1];
  const double b = (-J[0][0]) * J[2][1] + J[2][0] * J[0][1];
  const double c = J[0][0] * J[1][1] - J[1][0] * J[0][1];
  detB = sqrt((a * a + b * b) + c * c);
}

// One step of MappingIsoparametric.invF's Newton iteration (:157-168) for
// cell e at the global point x; returns sum_i |dX_i| (the per-point term of
// its stopping norm).
FEM_HD double newton_step(const FemMesh& m, int64_t e, const double x[3], double X[3]) {
  double F[3], inv[3][3], det;
  const double unusedA[3][3] = {}, unusedx0[3] = {};   // affine map: not used for Hex1
  global_coords<3>(m, e, true, unusedA, unusedx0, X[0], X[1], X[2], F);
  hex_inverse(m, e, X[0], X[1], X[2], inv, det);
  double r[3], dX[3];
  for (int j = 0; j < 3; ++j) r[j] = x[j] - F[j];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s = s + inv[i][j] * r[j];
    dX[i] = s;
  }
  for (int i = 0; i < 3; ++i) {
    const double t = X[i] + dX[i];
    X[i] = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);   // np.clip
  }
  return (fabs(dX[0]) + fabs(dX[1])) + fabs(dX[2]);
}

// First pass of the Hex1 facet geometry: the first Newton iteration at
// which facet f's stopping norm (max over its points of sum_i |dX_i|) is
// below 1e-12 for the cell f2t[side] (which = 0) or f2t[0] (which = 1); 51
// if none of the 50 does.  invF stops for all facets at once, so the
// maximum over facets is every facet's iteration count.
FEM_HD int hex_facet_newton_iters(const FemMesh& m, const FemFacets& fc, int64_t f, int which,
                                  const double* X, int nq) {
  const int64_t e = which ? fc.tind_n[f] : fc.tind[f];
  if (e < 0 || e >= m.nelems || nq > kMaxPoints) return 0;
  double xs[kMaxPoints][3], Xs[kMaxPoints][3];
  for (int q = 0; q < nq; ++q) {
    double detB;
    quad_facet_map(m, fc, f, X[q], X[nq + q], xs[q], detB);
    Xs[q][0] = Xs[q][1] = Xs[q][2] = 0.5;
  }
  for (int it = 1; it <= 50; ++it) {
    double norm = 0.0;
    for (int q = 0; q < nq; ++q) {
      const double s = newton_step(m, e, xs[q], Xs[q]);
      if (s > norm || s != s) norm = s;   // np.max, NaN propagating
    }
    if (norm < 1e-12) return it;
  }
  return 51;
}

// Second pass: point q of facet f with the common iteration counts ks
// (cells f2t[side]) and kn (cells f2t[0]); writes the 20 doubles of the
// generic kernels' point geometry (invDF, detDG, x, h, n, reference point)
// and returns a status word.
FEM_HD int hex_facet_point(const FemMesh& m, const FemFacets& fc, int64_t f, int q,
                           const double* X, int nq, int ks, int kn, double* G) {
  const int64_t e = fc.tind[f], en = fc.tind_n[f];
  const int lf = fc.lfacet_n[f];
  if (e < 0 || e >= m.nelems || en < 0 || en >= m.nelems || lf < 0 || lf > 5) {
    for (int i = 0; i < 20; ++i) G[i] = 0.0;
    return 1 << FEM_ERR_ARGUMENT;
  }
  int st = 0;
  if (ks > 50 || kn > 50) st |= 1 << FEM_ERR_NEWTON;
  double x[3], detB;
  quad_facet_map(m, fc, f, X[q], X[nq + q], x, detB);
  double Y[3] = {0.5, 0.5, 0.5}, Y0[3] = {0.5, 0.5, 0.5};
  for (int it = 0; it < ks && it < 50; ++it) newton_step(m, e, x, Y);
  for (int it = 0; it < kn && it < 50; ++it) newton_step(m, en, x, Y0);
  double inv[3][3], det, invn[3][3], detn;
  hex_inverse(m, e, Y[0], Y[1], Y[2], inv, det);
  hex_inverse(m, en, Y0[0], Y0[1], Y0[2], invn, detn);
  if (det == 0.0 || detn == 0.0) st |= 1 << FEM_ERR_ZERO_JACOBIAN;
  double N[3], n[3];
  ref_normal(3, lf, N, true);
  for (int j = 0; j < 3; ++j) {
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s = s + invn[i][j] * N[i];
    n[j] = s;
  }
  const double rl = 1.0 / sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) G[i * 3 + j] = inv[i][j];
  G[9] = detB;
  for (int i = 0; i < 3; ++i) G[10 + i] = x[i];
  G[13] = sqrt(detB);
  for (int j = 0; j < 3; ++j) G[14 + j] = n[j] * rl;
  for (int i = 0; i < 3; ++i) G[17 + i] = Y[i];
  return st;
}

// form(u_j, v_i, w) * dx at quadrature point q (bilinear_form.py:150-151,
// linear_form.py:48-49, functional.py:19-24): dx = |detDF| * W[q]
// (cell_basis.py:104-105).  Coefficient slot c holds one value per element
// (stride 0) or per quadrature point (stride nq).
// The form at one point: the program interpreter, or (kernels compiled
// from a traced program) the program's own straight-line code.
#ifndef FEM_FORM_EVAL
#define FEM_FORM_EVAL(prog, qu, qv, cq, qx, R) \
  run((prog).ins, (prog).ninstr, (prog).out, qu, qv, cq, qx, R)
#endif

// ... with the trial (qu) and test (qv) quantities already evaluated
FEM_HD double point_value_q(const FemProgram& prog, int64_t e, int q, const double* qu,
                            const double* qv, const PointGeo& g, double wq, double* R) {
  double cq[kMaxCoef];
  for (int c = 0; c < prog.ncoef && c < kMaxCoef; ++c)
    cq[c] = prog.coef[c] ? prog.coef[c][prog.coef_stride[c] ? e * prog.coef_stride[c] + q : e]
                         : 0.0;
  const double f = FEM_FORM_EVAL(prog, qu, qv, cq, g.qx, R);
  return f * (fabs(g.det) * wq);
}

template <int D>
FEM_HD double point_value(const FemBasis& b, const FemProgram& prog, int64_t e, int q, int i,
                          int j, double x, double y, double z, const PointGeo& g, double wq,
                          double* R) {
  const bool vec = b.vector != 0;
  double qu[D + D * D], qv[D + D * D];
  quantities<D>(b.family, vec, j, x, y, z, g.inv, qu);
  quantities<D>(b.family, vec, i, x, y, z, g.inv, qv);
  return point_value_q(prog, e, q, qu, qv, g, wq, R);
}

// The replayed value of local entry (row i, column j) of element e: the
// reference's value bit for bit (for the correctly rounded operations).
template <int D>
FEM_HD double replay_entry(const FemMesh& m, const FemBasis& b, const FemProgram& prog,
                           const Rule& rule, int64_t e, int i, int j, double* R,
                           double* scratch) {
  double own[kMaxPoints];
  double* vals = scratch ? scratch : own;
  const bool hex = b.family == FEM_HEX_1;
  const ProgFlags f = prog_flags(prog);
  CellGeo c;
  cell_geometry<D>(m, e, hex, c);
  for (int q = 0; q < rule.nq; ++q) {
    const double x = rule.X[q];
    const double y = rule.X[rule.nq + q];
    const double z = D == 3 ? rule.X[2 * rule.nq + q] : 0.0;
    PointGeo g;
    point_geometry<D>(m, e, hex, c, f, x, y, z, g);
    vals[q] = point_value<D>(b, prog, e, q, i, j, x, y, z, g, rule.W[q], R);
  }
  return np_pairwise_sum(vals, rule.nq);
}

// numpy's pairwise summation of a contiguous array of any length
// (PW_BLOCKSIZE 128 leaves, split at n/2 rounded down to a multiple of 8).
FEM_HD double np_pairwise_sum_any(const double* a, int64_t n) {
  // explicit stack instead of recursion: depth <= 64
  struct Frame { int64_t off, n; int state; double left; };
  Frame st[64];
  int sp = 0;
  st[0] = {0, n, 0, 0.0};
  double ret = 0.0;
  while (sp >= 0) {
    Frame& f = st[sp];
    if (f.n <= 128) {
      ret = np_pairwise_sum(a + f.off, (int)f.n);
      --sp;
      continue;
    }
    int64_t n2 = f.n / 2;
    n2 -= n2 % 8;
    if (f.state == 0) {
      f.state = 1;
      st[sp + 1] = {f.off, n2, 0, 0.0};
      ++sp;
    } else if (f.state == 1) {
      f.left = ret;
      f.state = 2;
      st[sp + 1] = {f.off + n2, f.n - n2, 0, 0.0};
      ++sp;
    } else {
      ret = f.left + ret;
      --sp;
    }
  }
  return ret;
}

}  // namespace fem_faithful
