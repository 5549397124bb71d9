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
  double vals[64];
  if (prog->ninstr > kMaxProgram || nq > 64) return 1;
  for (int64_t e = 0; e < m->nelems; ++e) {
    double coef[8];
    for (int c = 0; c < prog->ncoef && c < 8; ++c) coef[c] = prog->coef[c] ? prog->coef[c][e] : 0.0;
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        const double s = m->dim == 2
            ? replay_entry<2>(*m, *b, *prog, rule, e, i, j, coef, R, vals)
            : replay_entry<3>(*m, *b, *prog, rule, e, i, j, coef, R, vals);
        out[(e * nb + i) * nb + j] = s;
      }
  }
  return 0;
}
