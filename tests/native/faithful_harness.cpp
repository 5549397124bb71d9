// Host build of the exact-zero replay core (test infrastructure): replays
// local entries on the CPU so that the transcription of the reference's
// arithmetic can be checked bit for bit against the oracle without a GPU.
// Build: g++ -O2 -ffp-contract=off -shared -fPIC faithful_harness.cpp
#include "../../scikit-fem_gb300/csrc/fem_faithful_core.cuh"

extern "C" int faithful_replay_host(const FemMesh* m, const FemBasis* b, const FemProgram* prog,
                                    const double* X, const double* W, int nq, double* out) {
  // out[(e * nb + i) * nb + j] = replayed entry (row i, column j)
  using namespace fem_faithful;
  const Rule rule{X, W, nq};
  const int nb = b->nbfun;
  double R[kMaxProgram];
  double vals[kMaxPoints];
  if (prog->ninstr > kMaxProgram || nq > kMaxPoints) return 1;
  for (int64_t e = 0; e < m->nelems; ++e) {
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        const double s = m->dim == 2
            ? replay_entry<2>(*m, *b, *prog, rule, e, i, j, R, vals)
            : replay_entry<3>(*m, *b, *prog, rule, e, i, j, R, vals);
        out[(e * nb + i) * nb + j] = s;
      }
  }
  return 0;
}

// The generic kernels' arithmetic on the host: mode 0 local matrices
// out[(e*nb + i)*nb + j], 1 local vectors out[e*nb + i], 2 per-cell values.
// prog->qX / qW are host arrays here.
extern "C" int faithful_program_host(int mode, const FemMesh* m, const FemBasis* b,
                                     const FemProgram* prog, double* out) {
  using namespace fem_faithful;
  const int nq = prog->nq;
  if (prog->ninstr > kMaxProgram || nq > kMaxPoints) return 1;
  const Rule rule{prog->qX, prog->qW, nq};
  const int nb = b->nbfun;
  const int L = mode == 0 ? nb * nb : (mode == 1 ? nb : 1);
  double R[kMaxProgram];
  for (int64_t e = 0; e < m->nelems; ++e)
    for (int r = 0; r < L; ++r) {
      const int i = mode == 0 ? r / nb : (mode == 1 ? r : 0);
      const int j = mode == 0 ? r % nb : 0;
      out[e * L + r] = m->dim == 2 ? replay_entry<2>(*m, *b, *prog, rule, e, i, j, R, nullptr)
                                   : replay_entry<3>(*m, *b, *prog, rule, e, i, j, R, nullptr);
    }
  return 0;
}

template <int D>
static void interp_host(const FemMesh& m, const FemBasis& b, int nq, const double* X,
                        const double* w, double* out) {
  using namespace fem_faithful;
  const bool hex = b.family == FEM_HEX_1, vec = b.vector != 0;
  const int nquant = vec ? D + D * D : 1 + D;
  for (int64_t e = 0; e < m.nelems; ++e) {
    CellGeo c;
    cell_geometry<D>(m, e, hex, c);
    for (int q = 0; q < nq; ++q) {
      const double x = X[q], y = X[nq + q], z = D == 3 ? X[2 * nq + q] : 0.0;
      PointGeo g;
      point_geometry<D>(m, e, hex, c, ProgFlags(), x, y, z, g);
      double acc[D + D * D], qq[D + D * D];
      const double w0 = w[b.element_dofs[e]];
      quantities<D>(b.family, vec, 0, x, y, z, g.inv, qq);
      for (int k = 0; k < nquant; ++k) acc[k] = 0.0 * (w0 * qq[k]);
      for (int i = 0; i < b.nbfun; ++i) {
        const double wi = w[b.element_dofs[(int64_t)i * m.nelems + e]];
        quantities<D>(b.family, vec, i, x, y, z, g.inv, qq);
        for (int k = 0; k < nquant; ++k) acc[k] = acc[k] + wi * qq[k];
      }
      for (int k = 0; k < nquant; ++k) out[((int64_t)k * m.nelems + e) * nq + q] = acc[k];
    }
  }
}

extern "C" int faithful_interpolate_host(const FemMesh* m, const FemBasis* b, int nq,
                                         const double* X, const double* w, double* out) {
  if (m->dim == 2) interp_host<2>(*m, *b, nq, X, w, out);
  else interp_host<3>(*m, *b, nq, X, w, out);
  return 0;
}

extern "C" double faithful_sum_host(const double* x, int64_t n) {
  return n == 0 ? 0.0 : fem_faithful::np_pairwise_sum_any(x, n);
}

// Global coordinates and mesh parameter at every point:
// out[(k*nelems + e)*nq + q], k = 0..2 coordinates, 3 h.
extern "C" int faithful_points_host(const FemMesh* m, const FemBasis* b, int nq, const double* X,
                                    double* out) {
  using namespace fem_faithful;
  const bool hex = b->family == FEM_HEX_1;
  ProgFlags f;
  f.x = f.h = true;
  for (int64_t e = 0; e < m->nelems; ++e) {
    CellGeo c;
    PointGeo g;
    if (m->dim == 2) cell_geometry<2>(*m, e, hex, c);
    else cell_geometry<3>(*m, e, hex, c);
    for (int q = 0; q < nq; ++q) {
      const double x = X[q], y = X[nq + q], z = m->dim == 3 ? X[2 * nq + q] : 0.0;
      if (m->dim == 2) point_geometry<2>(*m, e, hex, c, f, x, y, z, g);
      else point_geometry<3>(*m, e, hex, c, f, x, y, z, g);
      for (int k = 0; k < 4; ++k) out[((int64_t)k * m->nelems + e) * nq + q] = g.qx[k];
    }
  }
  return 0;
}

// Point geometry of a facet: precomputed (Hex1, fc.geo) or facet_point.
template <int D>
static bool facet_geo(const FemMesh& m, const FemFacets& fc, int64_t f, int q, const double* X,
                      int nq, double Y[3], fem_faithful::PointGeo& g) {
  if (fc.geo) {
    const double* G = fc.geo + ((size_t)f * nq + q) * 20;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) g.inv[i][j] = G[i * 3 + j];
    g.det = G[9];
    for (int i = 0; i < 7; ++i) g.qx[i] = G[10 + i];
    for (int i = 0; i < 3; ++i) Y[i] = G[17 + i];
    return true;
  }
  double Xf[2] = {X[q], D == 3 ? X[nq + q] : 0.0};
  return fem_faithful::facet_point<D>(m, fc, f, Xf, Y, g);
}

// Hex1 facet geometry (both passes) on the host.
extern "C" int faithful_hex_facet_geometry_host(const FemMesh* m, const FemFacets* fc, int nq,
                                                const double* X, double* geo) {
  using namespace fem_faithful;
  int k[2] = {0, 0};
  for (int which = 0; which < 2; ++which)
    for (int64_t f = 0; f < fc->nfacets; ++f) {
      const int it = hex_facet_newton_iters(*m, *fc, f, which, X, nq);
      if (it > k[which]) k[which] = it;
    }
  int st = 0;
  for (int64_t f = 0; f < fc->nfacets; ++f)
    for (int q = 0; q < nq; ++q)
      st |= hex_facet_point(*m, *fc, f, q, X, nq, k[0], k[1], geo + ((size_t)f * nq + q) * 20);
  return st;
}

// FacetBasis versions: the facet-point geometry (facet_point) and the same
// per-entry replay; prog->qX is the facet rule (dim-1, nq).
template <int D>
static double facet_entry(const FemMesh& m, const FemBasis& b, const FemFacets& fc,
                          const FemProgram& prog, int64_t f, int i, int j, double* R) {
  using namespace fem_faithful;
  double vals[kMaxPoints];
  const int nq = prog.nq;
  for (int q = 0; q < nq; ++q) {
    double Y[3];
    PointGeo g;
    facet_geo<D>(m, fc, f, q, prog.qX, nq, Y, g);
    vals[q] = point_value<D>(b, prog, f, q, i, j, Y[0], Y[1], Y[2], g, prog.qW[q], R);
  }
  return np_pairwise_sum(vals, nq);
}

extern "C" int faithful_facet_program_host(int mode, const FemMesh* m, const FemBasis* b,
                                           const FemFacets* fc, const FemProgram* prog,
                                           double* out) {
  using namespace fem_faithful;
  if (prog->ninstr > kMaxProgram || prog->nq > kMaxPoints) return 1;
  const int nb = b->nbfun;
  const int L = mode == 0 ? nb * nb : (mode == 1 ? nb : 1);
  double R[kMaxProgram];
  for (int64_t f = 0; f < fc->nfacets; ++f)
    for (int r = 0; r < L; ++r) {
      const int i = mode == 0 ? r / nb : (mode == 1 ? r : 0);
      const int j = mode == 0 ? r % nb : 0;
      out[f * L + r] = m->dim == 2 ? facet_entry<2>(*m, *b, *fc, *prog, f, i, j, R)
                                   : facet_entry<3>(*m, *b, *fc, *prog, f, i, j, R);
    }
  return 0;
}

// x (dim), h, n (dim) at every facet point: out[(k*nfacets + f)*nq + q], k < 7
extern "C" int faithful_facet_points_host(const FemMesh* m, const FemFacets* fc, int nq,
                                          const double* X, double* out) {
  using namespace fem_faithful;
  for (int64_t f = 0; f < fc->nfacets; ++f)
    for (int q = 0; q < nq; ++q) {
      double Y[3];
      PointGeo g;
      const bool ok = m->dim == 2 ? facet_geo<2>(*m, *fc, f, q, X, nq, Y, g)
                                  : facet_geo<3>(*m, *fc, f, q, X, nq, Y, g);
      if (!ok) return 1;
      for (int k = 0; k < 7; ++k) out[((int64_t)k * fc->nfacets + f) * nq + q] = g.qx[k];
    }
  return 0;
}

template <int D>
static void facet_interp_host(const FemMesh& m, const FemBasis& b, const FemFacets& fc, int nq,
                              const double* X, const double* w, double* out) {
  using namespace fem_faithful;
  const bool vec = b.vector != 0;
  const int nquant = vec ? D + D * D : 1 + D;
  for (int64_t f = 0; f < fc.nfacets; ++f) {
    const int64_t ec = fc.tind[f];
    for (int q = 0; q < nq; ++q) {
      double Y[3];
      PointGeo g;
      facet_geo<D>(m, fc, f, q, X, nq, Y, g);
      double acc[D + D * D], qq[D + D * D];
      const double w0 = w[b.element_dofs[ec]];
      quantities<D>(b.family, vec, 0, Y[0], Y[1], Y[2], g.inv, qq);
      for (int k = 0; k < nquant; ++k) acc[k] = 0.0 * (w0 * qq[k]);
      for (int i = 0; i < b.nbfun; ++i) {
        const double wi = w[b.element_dofs[(int64_t)i * m.nelems + ec]];
        quantities<D>(b.family, vec, i, Y[0], Y[1], Y[2], g.inv, qq);
        for (int k = 0; k < nquant; ++k) acc[k] = acc[k] + wi * qq[k];
      }
      for (int k = 0; k < nquant; ++k) out[((int64_t)k * fc.nfacets + f) * nq + q] = acc[k];
    }
  }
}

extern "C" int faithful_facet_interpolate_host(const FemMesh* m, const FemBasis* b,
                                               const FemFacets* fc, int nq, const double* X,
                                               const double* w, double* out) {
  if (m->dim == 2) facet_interp_host<2>(*m, *b, *fc, nq, X, w, out);
  else facet_interp_host<3>(*m, *b, *fc, nq, X, w, out);
  return 0;
}
