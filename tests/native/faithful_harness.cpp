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
