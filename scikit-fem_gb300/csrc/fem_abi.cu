// extern "C" entry points of libskfem_gb300 (declared in include/skfem_gb300.h).

#include <map>
#include <mutex>
#include <tuple>
#include <string>

#include "fem_common.cuh"

#include <algorithm>
#include <vector>

namespace fem_fast {
int local_matrices(const FemMesh&, const FemBasis&, const FemBilinear&, double*, int32_t*,
                   cudaStream_t);
// cells [ebeg, eend) only (eend < 0: to the last cell); with a cell list,
// the cells cells[ebeg .. eend-1]; upper: vector bases write only the
// blocks on and above the block diagonal (Pattern::staging_sym)
int local_matrices_checked(const FemMesh&, const FemBasis&, const FemBilinear&, double*,
                           const uint8_t*, int32_t*, cudaStream_t, int64_t ebeg = 0,
                           int64_t eend = -1, const int32_t* cells = nullptr, int upper = 0,
                           const double* geo = nullptr);
// per-cell geometry cache of the scalar simplex kernels: doubles per cell
// (0: none for this family) and the kernel that fills it
int geometry_count(const FemMesh&, const FemBasis&);
int geometry_cache(const FemMesh&, const FemBasis&, double* geo, cudaStream_t);
// the channel kernels' coefficient checks alone (status null: none)
int coef_checks(const FemBilinear& f, const uint8_t* ref_bits, int32_t* status, cudaStream_t st,
                int64_t ebeg, int64_t eend, const int32_t* cells);
int local_vectors(const FemMesh&, const FemBasis&, const FemLinear&, double*, int32_t*,
                  cudaStream_t);
// the vector channel forms' per-cell pair blocks (fem::vec_pair_stride doubles per
// cell) of the cells [ebeg, eend) (of the list cells, when given); with a
// status word also the coefficient checks (ref_bits: the pattern's zero bits)
int vector_pair_blocks(const FemMesh&, const FemBasis&, const FemBilinear&, double*, cudaStream_t,
                       int64_t ebeg = 0, int64_t eend = -1, const int32_t* cells = nullptr,
                       const uint8_t* ref_bits = nullptr, int32_t* status = nullptr);
// the same for scalar TriP2 / TetP2 bases (geo: the pattern's geometry cache
// of this mesh, or null)
int scalar_pair_values(const FemMesh&, const FemBasis&, const FemBilinear&, const double* geo,
                       double*, cudaStream_t, int64_t ebeg = 0, int64_t eend = -1,
                       const int32_t* cells = nullptr, const uint8_t* ref_bits = nullptr,
                       int32_t* status = nullptr);
}  // namespace fem_fast
namespace fem_exact {
int local_matrices(const FemMesh&, const FemBasis&, const FemBilinear&, double*, int32_t*,
                   cudaStream_t);
}  // namespace fem_exact

namespace fem {
int vector_sum(const Pattern& P, const double* local, double* b, cudaStream_t st);
int program_eval(int mode, const FemMesh& m, const FemBasis& b, const FemFacets* fc,
                 const FemProgram& prog, double* out, int32_t* status, cudaStream_t st,
                 const FemBasis* bu);
int interpolate(const FemMesh& m, const FemBasis& b, const FemFacets* fc, int nq, const double* X,
                const double* w, double* out, int32_t* status, cudaStream_t st);
int sum_pairwise(const double* x, int64_t n, double* out, cudaStream_t st);
int facet_geometry(const FemMesh& m, const FemBasis& b, const FemFacets& fc, int nq,
                   const double* X, double* geo, int32_t* status, cudaStream_t st);
int faithful_mask(const FemMesh& m, const FemBasis& b, const FemProgram& prog, int nq, double* local,
                  int32_t* status, cudaStream_t st);

namespace {
thread_local std::string g_err;
}

void set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = std::string("[") + std::to_string(code) + "] " + buf;
}

int resident_blocks_per_sm(const void* kern, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t, int>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const auto key = std::make_tuple(kern, threads, smem, dev);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) !=
          cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = per_sm;
  return per_sm;
}

int check_cuda(cudaError_t err, const char* what) {
  set_error(FEM_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(err), cudaGetErrorName(err));
  return FEM_ERR_CUDA;
}

int basis_nb_scalar(int family) {
  switch (family) {
    case FEM_TRI_P1: return 3;
    case FEM_TRI_P2: return 6;
    case FEM_TET_P1: return 4;
    case FEM_TET_P2: return 10;
    case FEM_HEX_1: return 8;
    default: return 0;
  }
}

int basis_dim(int family) {
  switch (family) {
    case FEM_TRI_P1:
    case FEM_TRI_P2: return 2;
    case FEM_TET_P1:
    case FEM_TET_P2:
    case FEM_HEX_1: return 3;
    default: return 0;
  }
}

// Per-element zero bits of the form's coefficients (bit k: channel k is 0).
__global__ void coef_zero_bits_kernel(FemBilinear f, int64_t n, const uint8_t* __restrict__ ref,
                                      uint8_t* __restrict__ out, int32_t* __restrict__ status) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const FemCoef* c[5] = {&f.diff, &f.mass, &f.lam, &f.lap, &f.tr};
  uint8_t bits = 0;
#pragma unroll
  for (int k = 0; k < 5; ++k)
    if (coef_zero(*c[k], e)) bits |= (uint8_t)(1u << k);
  if (out) out[e] = bits;
  if (ref && ref[e] != bits) atomicOr(status, 1 << FEM_ERR_STALE_PATTERN);
}

namespace {
std::mutex g_tuning_mu;
Tuning g_tuning[8];
}

Tuning tuning_for(int family) {
  std::lock_guard<std::mutex> lock(g_tuning_mu);
  return (family >= 0 && family < 8) ? g_tuning[family] : Tuning();
}

}  // namespace fem

struct FemPattern {
  fem::Pattern P;
  uint8_t* coef_bits = nullptr;  // nelems, or null when built without a form
  std::vector<int32_t> host_indptr;  // host copy of indptr (row ranges of fem_assemble_to_host)
  int family = 0, vector = 0;
  // Plan of fem_assemble_to_host_pipelined, built once per chunk count:
  // the cells sorted by their smallest DOF (device), the chunks' bounds in
  // that order, and the rows complete after each chunk.
  mutable std::mutex plan_mu;
  mutable int plan_nchunks = 0;
  mutable int32_t* plan_cells = nullptr;
  mutable std::vector<int64_t> plan_bounds;   // plan_nchunks + 1 positions
  mutable std::vector<int64_t> plan_rows;     // plan_nchunks: rows [0, plan_rows[c]) final
  // Per-cell geometry of the scalar simplex kernels (fem_pattern_cache_geometry),
  // computed from the coordinates at geo_p; used only for meshes whose p is
  // that same pointer.
  double* geo = nullptr;
  const double* geo_p = nullptr;
  // Fused assembly cache of scalar simplex bases, built with geo (same
  // validity): the geometry-only stiffness rows in incidence order (ninc x
  // nbfun) and the CSR values of the unit-coefficient mass matrix (nnz).
  double* stiff = nullptr;
  double* mass1 = nullptr;
  // The coefficient-update cache above is built only on request
  // (fem_pattern_cache_coefficient_update), then refreshed with geo.
  bool fused_wanted = false;
  // One-pass P1 assembly from geo (scalar TriP1 / TetP1, built with geo):
  // each row's binary point of the fixed-point mass sums; mbase_ok false
  // when some cell's |det| lies outside the range it covers.
  int16_t* mbase = nullptr;
  bool mbase_ok = false;
  // The one-pass P1 sum's upper-gather lists (pattern-only; built with the
  // first geometry cache of a scalar TriP1 / TetP1 pattern).
  fem::UpperLists upper;
  bool upper_ok = false, upper_tried = false;
  // The one-pass node-block sum's lists (simplex ElementVector bases, scalar
  // TriP2 / TetP2 bases; pattern-only, built with the first
  // fem_pattern_cache_geometry call).
  fem::VecUpper vec;
  bool vec_ok = false, vec_tried = false;
};

namespace {
// The pattern's geometry cache when it was computed from this mesh's
// coordinate array, else null (the kernels then compute the geometry).
const double* cached_geometry(const FemPattern* pat, const FemMesh* mesh) {
  return (pat->geo && pat->geo_p == mesh->p) ? pat->geo : nullptr;
}

// The fused assembly of one call: K = diff * sum_e k_e S_e + mass * M from
// the pattern's cache, for scalar forms whose mass coefficient is one
// constant (the stiffness coefficient may vary per cell).
struct FusedSum {
  const double* stiff;   // null: the stiffness coefficient is exactly 0
  FemCoef diff;
  const double* mass1;
  double mscale;
};

// The one-pass P1 assembly of one call: scalar TriP1 / TetP1 forms
// k_e dot(grad u, grad v) + m_e u v over the geometry cache, when the
// pattern holds the cache of this mesh's coordinates.
bool geometry_sum(const FemPattern* pat, const FemMesh* mesh, const FemBasis* basis,
                  const FemBilinear* form) {
  if (basis->vector || !cached_geometry(pat, mesh)) return false;
  if (basis->family != FEM_TRI_P1 && basis->family != FEM_TET_P1) return false;
  if (pat->P.nbfun_u != pat->P.nbfun_v) return false;
  return form->mass.field ? true : (pat->mbase && pat->mbase_ok);
}

// The one-pass node-block sum applies: simplex ElementVector bases and
// scalar TriP2 / TetP2 bases whose pattern holds its lists, unless the
// family's tuning selects the two-pass path (fem_set_onepass variant 0).
bool vector_onepass(const FemPattern* pat, const FemMesh* mesh, const FemBasis* basis) {
  if (!pat->vec_ok || pat->vec.sdim != mesh->dim) return false;
  if (pat->vec.dim != (basis->vector ? mesh->dim : 1)) return false;
  if (pat->P.nbfun_u != pat->P.nbfun_v || pat->P.nbfun_v != basis->nbfun) return false;
  return fem::tuning_for(basis->family).onepass >= 1;
}

// The per-cell pair values the one-pass node-block sum reads, cells
// [ebeg, eend) (of the list cells, when given), into the staging; with a
// status word the same kernel runs the coefficient checks (as the two-pass
// local kernel does).
int node_pair_values(const FemPattern* pat, const FemMesh* mesh, const FemBasis* basis,
                     const FemBilinear* form, double* staging, int32_t* status, cudaStream_t st,
                     int64_t ebeg = 0, int64_t eend = -1, const int32_t* cells = nullptr) {
  const uint8_t* ref = status ? pat->coef_bits : nullptr;
  if (basis->vector)
    return fem_fast::vector_pair_blocks(*mesh, *basis, *form, staging, st, ebeg, eend, cells,
                                        ref, status);
  return fem_fast::scalar_pair_values(*mesh, *basis, *form, cached_geometry(pat, mesh), staging,
                                      st, ebeg, eend, cells, ref, status);
}

bool fused_sum(const FemPattern* pat, const FemMesh* mesh, const FemBasis* basis,
               const FemBilinear* form, FusedSum* fs) {
  if (!pat->stiff || !pat->mass1 || !cached_geometry(pat, mesh) || basis->vector ||
      form->mass.field)
    return false;
  const bool no_stiffness = !form->diff.field && form->diff.scale == 0.0;
  fs->stiff = no_stiffness ? nullptr : pat->stiff;
  fs->diff = form->diff;
  fs->mass1 = pat->mass1;
  fs->mscale = form->mass.scale;
  return true;
}

void drop_fused(FemPattern* pat) {
  cudaFree(pat->stiff);
  cudaFree(pat->mass1);
  pat->stiff = nullptr;
  pat->mass1 = nullptr;
}

// The rows' fixed-point binary points of the one-pass P1 assembly, from the
// geometry cache just queued (scalar TriP1 / TetP1 patterns).  Without room
// for them the calls run the local kernel and the staging sum.
int cache_mass_base(FemPattern* pat, const FemMesh* mesh, const FemBasis* basis, cudaStream_t st) {
  const fem::Pattern& P = pat->P;
  pat->mbase_ok = false;
  if (basis->vector || (basis->family != FEM_TRI_P1 && basis->family != FEM_TET_P1) ||
      !P.has_matrix || P.nbfun_u != P.nbfun_v)
    return 0;
  if (!pat->mbase) {
    cudaError_t e = cudaMalloc(&pat->mbase, std::max<int64_t>(1, P.nrows) * sizeof(int16_t));
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      pat->mbase = nullptr;
      return 0;
    }
    if (e != cudaSuccess) {
      pat->mbase = nullptr;
      return fem::check_cuda(e, "cudaMalloc(row mass base)");
    }
  }
  const int ng = (mesh->dim + 1) * (mesh->dim + 2) / 2;
  int shmax = 0;
  bool ok = false;
  int rc = fem::row_mass_base(P, pat->geo + (int64_t)ng * mesh->nelems, pat->mbase, &shmax, &ok, st);
  if (rc) return rc;
  pat->mbase_ok = ok;
  if (!pat->upper_tried) {
    // the upper-gather form of the one-pass sum: an optimisation, left out
    // (with its error cleared) when the pattern is not symmetric or there
    // is no room for its lists
    pat->upper_tried = true;
    rc = fem::build_upper_lists(P, &pat->upper, st, false, fem::kUpperBlockRows);
    pat->upper_ok = rc == 0;
    if (rc) {
      cudaGetLastError();
      fem::set_error(FEM_OK, "");
    }
  }
  return 0;
}

// Builds the fused cache from the geometry cache just queued: the local
// kernels with unit stiffness (then unit mass) coefficients, the first
// gathered into incidence order, the second summed into CSR values.
// Without room for it the cache is left out (the calls run the local
// kernel and the staging sum).
int cache_fused(FemPattern* pat, const FemMesh* mesh, const FemBasis* basis, cudaStream_t st) {
  const fem::Pattern& P = pat->P;
  if (basis->vector || !P.has_matrix || P.nbfun_u != P.nbfun_v) return 0;
  const int64_t nl = P.ninc * (int64_t)P.nbfun_u;
  auto room = [&](double** ptr, int64_t n, const char* what) -> int {
    if (*ptr) return 0;
    cudaError_t e = cudaMalloc(ptr, std::max<int64_t>(1, n) * sizeof(double));
    if (e == cudaSuccess) return 0;
    *ptr = nullptr;
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      return -1;
    }
    return fem::check_cuda(e, what);
  };
  int rc = room(&pat->stiff, nl, "cudaMalloc(stiffness cache)");
  if (!rc) rc = room(&pat->mass1, P.nnz, "cudaMalloc(mass cache)");
  double* tmp = nullptr;
  if (!rc) {
    cudaError_t e = cudaMallocAsync(&tmp, std::max<int64_t>(1, nl) * sizeof(double), st);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      tmp = nullptr;
      rc = -1;
    } else if (e != cudaSuccess) {
      tmp = nullptr;
      rc = fem::check_cuda(e, "cudaMallocAsync(fused cache scratch)");
    }
  }
  if (!rc && mesh->nelems > 0) {
    FemBilinear unit{};
    unit.diff.scale = 1.0;
    rc = fem_fast::local_matrices_checked(*mesh, *basis, unit, tmp, nullptr, nullptr, st, 0, -1,
                                          nullptr, 0, pat->geo);
    if (!rc) rc = fem::incidence_rows(P, tmp, pat->stiff, st);
    FemBilinear mass{};
    mass.mass.scale = 1.0;
    if (!rc) rc = fem_fast::local_matrices_checked(*mesh, *basis, mass, tmp, nullptr, nullptr, st,
                                                   0, -1, nullptr, 0, pat->geo);
    fem::Pattern Q = P;
    Q.sum_unroll = fem::tuning_for(pat->family).sum_unroll;
    if (!rc) rc = fem::csr_sum(Q, tmp, pat->mass1, st);
  }
  if (tmp) cudaFreeAsync(tmp, st);
  if (rc) drop_fused(pat);
  return rc < 0 ? 0 : rc;
}
}  // namespace

using fem::set_error;

namespace fem {
const Pattern* pattern_of(const FemPattern* h) { return h ? &h->P : nullptr; }
const uint8_t* pattern_coef_bits(const FemPattern* h) { return h ? h->coef_bits : nullptr; }
// the pattern's one-pass node-block lists (null: none built)
const VecUpper* pattern_node_lists(const FemPattern* h) {
  return (h && h->vec_ok) ? &h->vec : nullptr;
}
int coef_check(const FemBilinear& f, int64_t n, const uint8_t* ref, int32_t* status,
               cudaStream_t st) {
  coef_zero_bits_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(f, n, ref, nullptr, status);
  FEM_LAUNCH_CHECK("coef_zero_bits_kernel");
  return 0;
}
int new_pattern_handle(Pattern* P, FemPattern** out) {
  FemPattern* H = new FemPattern();
  H->P = *P;
  delete P;
  *out = H;
  return 0;
}
}  // namespace fem

static int host_row_pointer(FemPattern* H, cudaStream_t st) {
  H->host_indptr.resize(H->P.nrows + 1);
  FEM_TRY_CUDA(cudaMemcpyAsync(H->host_indptr.data(), H->P.indptr,
                               (H->P.nrows + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  return 0;
}

// generic: the entry point runs the generic kernels, which also take
// ElementVector(ElementHex1); the channel kernels do not.
static int validate(const FemMesh* m, const FemBasis* b, bool generic = false) {
  if (!m || !b) {
    set_error(FEM_ERR_ARGUMENT, "null mesh or basis");
    return FEM_ERR_ARGUMENT;
  }
  const int nbs = fem::basis_nb_scalar(b->family);
  if (nbs == 0) {
    set_error(FEM_ERR_UNSUPPORTED, "unknown element family %d", b->family);
    return FEM_ERR_UNSUPPORTED;
  }
  const int dim = fem::basis_dim(b->family);
  if (m->dim != dim) {
    set_error(FEM_ERR_ARGUMENT, "Incompatible Mesh and Element: mesh dim %d, element dim %d",
              m->dim, dim);
    return FEM_ERR_ARGUMENT;
  }
  const int nloc = b->family == FEM_HEX_1 ? 8 : dim + 1;
  if (m->nloc != nloc) {
    set_error(FEM_ERR_ARGUMENT, "Incompatible Mesh and Element: %d vertices per cell, expected %d",
              m->nloc, nloc);
    return FEM_ERR_ARGUMENT;
  }
  const int nb = b->vector ? nbs * dim : nbs;
  if (b->nbfun != nb) {
    set_error(FEM_ERR_ARGUMENT, "nbfun %d does not match the family (%d)", b->nbfun, nb);
    return FEM_ERR_ARGUMENT;
  }
  if (m->nelems < 0 || m->nverts < 0 || (m->nelems > 0 && (!m->p || !m->t || !b->element_dofs))) {
    set_error(FEM_ERR_ARGUMENT, "invalid mesh arrays");
    return FEM_ERR_ARGUMENT;
  }
  if (b->vector && b->family == FEM_HEX_1 && !generic) {
    set_error(FEM_ERR_UNSUPPORTED, "ElementVector(ElementHex1) runs on the generic kernels only");
    return FEM_ERR_UNSUPPORTED;
  }
  return 0;
}

namespace fem {
// The host-side argument checks of the channel entry points (fem_assemble's),
// for the entry points in other translation units.
int validate_mesh_basis(const FemMesh* m, const FemBasis* b) { return validate(m, b); }
// The pattern's per-cell geometry cache when it was built from this mesh's
// coordinates, else null.
const double* pattern_geometry(const FemPattern* h, const FemMesh* m) {
  return (h && m) ? cached_geometry(h, m) : nullptr;
}
}  // namespace fem

static int read_status(int32_t* dstatus, cudaStream_t st) {
  int32_t h = 0;
  FEM_TRY_CUDA(cudaMemcpyAsync(&h, dstatus, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  FEM_TRY_CUDA(cudaStreamSynchronize(st));
  if (h & (1 << FEM_ERR_ZERO_JACOBIAN)) {
    set_error(FEM_ERR_ZERO_JACOBIAN, "Zero Jacobian determinant");
    return FEM_ERR_ZERO_JACOBIAN;
  }
  if (h & (1 << FEM_ERR_UNSUPPORTED)) {
    set_error(FEM_ERR_UNSUPPORTED, "the exact-zero mask has no reference rule for this basis's "
              "quadrature");
    return FEM_ERR_UNSUPPORTED;
  }
  return 0;
}

// interpolation with a status word of its own (invalid facet cells)
static int interp_with_status(const FemMesh* mesh, const FemBasis* basis, const FemFacets* facets,
                              int32_t nq, const double* X, const double* w, double* out,
                              fem_stream_t stream) {
  cudaStream_t st = (cudaStream_t)stream;
  int32_t* dstatus = nullptr;
  FEM_TRY_CUDA(cudaMallocAsync(&dstatus, sizeof(int32_t), st));
  cudaMemsetAsync(dstatus, 0, sizeof(int32_t), st);
  int rc = fem::interpolate(*mesh, *basis, facets, nq, X, w, out, dstatus, st);
  int32_t h = 0;
  if (!rc) {
    cudaMemcpyAsync(&h, dstatus, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fem::check_cuda(e, "interpolate");
  }
  cudaFreeAsync(dstatus, st);
  if (!rc && h) {
    set_error(FEM_ERR_ARGUMENT, "facet with a cell index out of range");
    rc = FEM_ERR_ARGUMENT;
  }
  return rc;
}

extern "C" {

const char* fem_last_error(void) { return fem::g_err.c_str(); }

const char* fem_version(void) { return "skfem_gb300 0.1 (sm_103a)"; }

int fem_set_onepass(int family, int variant) {
  if (family < 1 || family > 5 || variant < 0 || variant > 2) {
    set_error(FEM_ERR_ARGUMENT, "family %d / one-pass variant %d out of range", family, variant);
    return FEM_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(fem::g_tuning_mu);
  fem::g_tuning[family].onepass = variant;
  return 0;
}

int fem_set_local_tma(int family, int on) {
  if (family < 1 || family > 5 || (on != 0 && on != 1)) {
    set_error(FEM_ERR_ARGUMENT, "family %d / local TMA flag %d out of range", family, on);
    return FEM_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(fem::g_tuning_mu);
  fem::g_tuning[family].local_tma = on;
  return 0;
}

int fem_set_tuning(int family, int local_block, int persistent, int sum_unroll, int sum_cols) {
  if (family < 1 || family > 5 || (local_block != 64 && local_block != 128 && local_block != 256) ||
      persistent < 0 || (sum_unroll != 4 && sum_unroll != 8 && sum_unroll != 16) ||
      (sum_cols != 1 && sum_cols != 2)) {
    set_error(FEM_ERR_ARGUMENT,
              "invalid tuning (family %d, block %d, persistent %d, unroll %d, columns %d)", family,
              local_block, persistent, sum_unroll, sum_cols);
    return FEM_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(fem::g_tuning_mu);
  fem::g_tuning[family].local_block = local_block;
  fem::g_tuning[family].persistent = persistent;
  fem::g_tuning[family].sum_unroll = sum_unroll;
  fem::g_tuning[family].sum_cols = sum_cols;
  return 0;
}

int fem_local_matrices(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                       double* local, fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!form || !local) {
    set_error(FEM_ERR_ARGUMENT, "null form or output");
    return FEM_ERR_ARGUMENT;
  }
  return fem_fast::local_matrices(*mesh, *basis, *form, local, nullptr, (cudaStream_t)stream);
}

int fem_local_vectors(const FemMesh* mesh, const FemBasis* basis, const FemLinear* form,
                      double* local, fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!form || !local) {
    set_error(FEM_ERR_ARGUMENT, "null form or output");
    return FEM_ERR_ARGUMENT;
  }
  return fem_fast::local_vectors(*mesh, *basis, *form, local, nullptr, (cudaStream_t)stream);
}

int fem_pattern_build(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                      const FemProgram* program, FemPattern** out, fem_stream_t stream) {
  int rc = validate(mesh, basis, form == nullptr);   // incidence only: any basis
  if (rc) return rc;
  if (!out) {
    set_error(FEM_ERR_ARGUMENT, "null output handle");
    return FEM_ERR_ARGUMENT;
  }
  *out = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  FemPattern* H = new FemPattern();
  H->family = basis->family;
  H->vector = basis->vector;
  auto fail = [&](int code) {
    fem::free_pattern(new fem::Pattern(H->P));  // releases device arrays
    cudaFree(H->coef_bits);
    delete H;
    return code;
  };
  rc = fem::build_incidence(basis->element_dofs, mesh->nelems, basis->nbfun, basis->ndofs, &H->P, st);
  if (rc) return fail(rc);
  if (form) {
    const int nb = basis->nbfun;
    const int64_t L = (int64_t)nb * nb;
    double* local = nullptr;
    int32_t* dstatus = nullptr;
    cudaError_t e1 = cudaMallocAsync(&local, std::max<int64_t>(1, mesh->nelems * L) * sizeof(double), st);
    if (e1 != cudaSuccess) return fail(fem::check_cuda(e1, "cudaMallocAsync(local)"));
    e1 = cudaMallocAsync(&dstatus, sizeof(int32_t), st);
    if (e1 != cudaSuccess) return fail(fem::check_cuda(e1, "cudaMallocAsync(status)"));
    cudaMemsetAsync(dstatus, 0, sizeof(int32_t), st);
    rc = fem_exact::local_matrices(*mesh, *basis, *form, local, dstatus, st);
    if (!rc && program) rc = fem::faithful_mask(*mesh, *basis, *program, program->nq, local, dstatus, st);
    if (!rc) rc = read_status(dstatus, st);
    if (!rc) rc = fem::build_csr(basis->element_dofs, nb, basis->ndofs, local, &H->P, st);
    // the vector channel forms are symmetric: their local kernels write the
    // blocks on and above the block diagonal only, the sum mirrors the rest
    if (!rc && basis->vector) H->P.staging_sym = mesh->dim;
    if (!rc) rc = host_row_pointer(H, st);
    if (!rc && mesh->nelems > 0) {
      cudaError_t e2 = cudaMallocAsync(&H->coef_bits, mesh->nelems, st);
      if (e2 != cudaSuccess) rc = fem::check_cuda(e2, "cudaMallocAsync(coef_bits)");
      else {
        fem::coef_zero_bits_kernel<<<(unsigned)fem::ceil_div(mesh->nelems, 256), 256, 0, st>>>(
            *form, mesh->nelems, nullptr, H->coef_bits, nullptr);
        cudaError_t e3 = cudaGetLastError();
        if (e3 != cudaSuccess) rc = fem::check_cuda(e3, "coef_zero_bits_kernel");
      }
    }
    cudaFreeAsync(local, st);
    cudaFreeAsync(dstatus, st);
    cudaError_t e4 = cudaStreamSynchronize(st);
    if (!rc && e4 != cudaSuccess) rc = fem::check_cuda(e4, "pattern build");
    if (rc) return fail(rc);
  }
  *out = H;
  return 0;
}

int fem_pattern_info(const FemPattern* pat, int64_t* nnz, int64_t* nrows, int64_t* staging_bytes) {
  if (!pat) {
    set_error(FEM_ERR_ARGUMENT, "null pattern");
    return FEM_ERR_ARGUMENT;
  }
  if (nnz) *nnz = pat->P.nnz;
  if (nrows) *nrows = pat->P.nrows;
  if (staging_bytes)
    *staging_bytes = pat->P.nelems * (int64_t)pat->P.nbfun_v * std::max(1, pat->P.nbfun_u) *
                     (int64_t)sizeof(double);
  return 0;
}

int fem_pattern_export(const FemPattern* pat, int32_t* indptr, int32_t* indices,
                       fem_stream_t stream) {
  if (!pat || !pat->P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern has no CSR structure");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (indptr)
    FEM_TRY_CUDA(cudaMemcpyAsync(indptr, pat->P.indptr, (pat->P.nrows + 1) * sizeof(int32_t),
                                 cudaMemcpyDeviceToDevice, st));
  if (indices && pat->P.nnz > 0)
    FEM_TRY_CUDA(cudaMemcpyAsync(indices, pat->P.indices, pat->P.nnz * sizeof(int32_t),
                                 cudaMemcpyDeviceToDevice, st));
  return 0;
}

void fem_pattern_destroy(FemPattern* pat) {
  if (!pat) return;
  fem::free_pattern(new fem::Pattern(pat->P));
  cudaFree(pat->coef_bits);
  cudaFree(pat->plan_cells);
  cudaFree(pat->geo);
  cudaFree(pat->mbase);
  fem::free_upper_lists(&pat->upper);
  fem::free_vec_upper(&pat->vec);
  drop_fused(pat);
  delete pat;
}

int fem_pattern_cache_geometry(FemPattern* pat, const FemMesh* mesh, const FemBasis* basis,
                               fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!pat || pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int fam = basis->family;
  const bool node_blocks =
      basis->vector ? (fam == FEM_TRI_P1 || fam == FEM_TRI_P2 || fam == FEM_TET_P1 ||
                       fam == FEM_TET_P2)
                    : (fam == FEM_TRI_P2 || fam == FEM_TET_P2);
  if (node_blocks && !pat->vec_tried) {
    // the one-pass node-block sum's lists (pattern-only): an optimisation,
    // left out (with its error cleared) when the pattern does not allow it
    // or there is no room for them
    pat->vec_tried = true;
    pat->vec_ok = false;
    if (fem::basis_dim(fam) == mesh->dim) {
      rc = fem::build_vec_upper(pat->P, basis->element_dofs, fam, basis->vector ? mesh->dim : 1,
                                &pat->vec, st);
      pat->vec_ok = rc == 0;
      if (rc) {
        cudaGetLastError();
        fem::set_error(FEM_OK, "");
      }
    }
  }
  const int ng = fem_fast::geometry_count(*mesh, *basis);
  if (ng == 0) return 0;  // families without a cache compute their geometry per call
  if (!pat->geo) {
    cudaError_t e = cudaMalloc(&pat->geo, std::max<int64_t>(1, mesh->nelems) * ng * sizeof(double));
    if (e == cudaErrorMemoryAllocation) {
      // the cache is an optimisation: without room for it the kernels
      // compute the geometry per call
      cudaGetLastError();
      pat->geo = nullptr;
      pat->geo_p = nullptr;
      return 0;
    }
    if (e != cudaSuccess) {
      pat->geo = nullptr;
      return fem::check_cuda(e, "cudaMalloc(geometry cache)");
    }
  }
  pat->geo_p = nullptr;  // not valid until the kernels below have been queued
  rc = fem_fast::geometry_cache(*mesh, *basis, pat->geo, st);
  if (rc) return rc;
  rc = cache_mass_base(pat, mesh, basis, st);
  if (rc) return rc;
  if (pat->fused_wanted) {
    rc = cache_fused(pat, mesh, basis, st);
    if (rc) return rc;
  }
  pat->geo_p = mesh->p;
  return 0;
}

int fem_pattern_cache_coefficient_update(FemPattern* pat, const FemMesh* mesh,
                                         const FemBasis* basis, fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!pat || pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  if (!cached_geometry(pat, mesh)) {
    set_error(FEM_ERR_ARGUMENT, "the coefficient-update cache needs the pattern's geometry cache "
              "of this mesh's coordinates (fem_pattern_cache_geometry)");
    return FEM_ERR_ARGUMENT;
  }
  pat->fused_wanted = true;
  return cache_fused(pat, mesh, basis, (cudaStream_t)stream);
}

void fem_pattern_drop_coefficient_update(FemPattern* pat) {
  if (!pat) return;
  pat->fused_wanted = false;
  drop_fused(pat);
}

void fem_pattern_drop_geometry(FemPattern* pat) {
  if (!pat) return;
  cudaFree(pat->geo);
  pat->geo = nullptr;
  pat->geo_p = nullptr;
  drop_fused(pat);
}

int fem_assemble(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                 const FemPattern* pat, double* staging, double* csr_values, int32_t* status,
                 fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  // an empty pattern (no cells, or only exact zeros) takes no value buffer
  if (!form || !pat || !staging || (!csr_values && pat->P.nnz > 0)) {
    set_error(FEM_ERR_ARGUMENT, "null form, pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  if (pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun || !pat->P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  FusedSum fs;
  if (fused_sum(pat, mesh, basis, form, &fs)) {
    // the coefficient checks, then one fused sum over the cached matrices
    rc = fem_fast::coef_checks(*form, pat->coef_bits, status, st, 0, mesh->nelems, nullptr);
    if (rc) return rc;
    fem::Pattern P = pat->P;
    const fem::Tuning t = fem::tuning_for(basis->family);
    P.sum_unroll = t.sum_unroll;
    P.sum_cols = t.sum_cols;
    return fem::csr_sum_scaled(P, fs.stiff, fs.diff, fs.mass1, fs.mscale, csr_values, st);
  }
  if (geometry_sum(pat, mesh, basis, form)) {
    // the coefficient checks, then the one-pass P1 assembly over the
    // cached geometry (the form contracted per cell row as the rows sum);
    // the plain upper form checks the coefficients itself where it can
    fem::Pattern P = pat->P;
    const fem::Tuning t = fem::tuning_for(basis->family);
    P.sum_unroll = t.sum_unroll;
    const bool upper = t.onepass >= 1 && pat->upper_ok;
    const bool folded = upper && status && pat->coef_bits &&
                        fem::upper_p1_checks(form->diff, form->mass, t.onepass == 2);
    if (!folded) {
      rc = fem_fast::coef_checks(*form, pat->coef_bits, status, st, 0, mesh->nelems, nullptr);
      if (rc) return rc;
    }
    if (upper) {
      // the zero bits of the channels without a field (as coef_fields_kernel)
      int const_bits = form->diff.scale == 0.0 ? 1 : 0;
      const FemCoef* rest[4] = {&form->mass, &form->lam, &form->lap, &form->tr};
      for (int k = 0; k < 4; ++k)
        if (!rest[k]->field && rest[k]->scale == 0.0) const_bits |= 1 << (k + 1);
      return fem::csr_sum_upper_p1(P, pat->upper, mesh->dim, pat->geo, form->diff, form->mass,
                                   pat->mbase, csr_values, st, 0, -1, status, t.onepass == 2,
                                   folded ? pat->coef_bits : nullptr, const_bits);
    }
    return fem::csr_sum_geometry_p1(P, mesh->dim, pat->geo, form->diff, form->mass, pat->mbase,
                                    csr_values, st);
  }
  if (vector_onepass(pat, mesh, basis)) {
    // the cells' pair values (in the staging) with the coefficient checks,
    // then the one-pass sum contracting and summing the node blocks
    rc = node_pair_values(pat, mesh, basis, form, staging, status, st);
    if (rc) return rc;
    const bool mass = form->mass.field || form->mass.scale != 0.0;
    return fem::vec_upper_sum(pat->vec, staging, mass, csr_values, st, 0, -1,
                              fem::tuning_for(basis->family).onepass == 2);
  }
  // the local kernel also compares each element's coefficient zero bits
  // with the pattern's (FEM_ERR_STALE_PATTERN)
  rc = fem_fast::local_matrices_checked(*mesh, *basis, *form, staging,
                                        status ? pat->coef_bits : nullptr, status, st, 0, -1,
                                        nullptr, pat->P.staging_sym > 0,
                                        cached_geometry(pat, mesh));
  if (rc) return rc;
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(basis->family).sum_unroll;
  return fem::csr_sum(P, staging, csr_values, st, 0, -1, nullptr, P.staging_sym);
}

int fem_assemble_local(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                       const FemPattern* pat, double* staging, int32_t* status, int64_t cell_begin,
                       int64_t cell_end, fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!form || !pat || !staging) {
    set_error(FEM_ERR_ARGUMENT, "null form, pattern or staging");
    return FEM_ERR_ARGUMENT;
  }
  if (pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun || !pat->P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  if (cell_begin < 0 || cell_end > mesh->nelems || cell_end < cell_begin) {
    set_error(FEM_ERR_ARGUMENT, "cell range [%lld, %lld) outside [0, %lld)",
              (long long)cell_begin, (long long)cell_end, (long long)mesh->nelems);
    return FEM_ERR_ARGUMENT;
  }
  if (cell_end == cell_begin) return 0;
  return fem_fast::local_matrices_checked(*mesh, *basis, *form, staging,
                                          status ? pat->coef_bits : nullptr, status,
                                          (cudaStream_t)stream, cell_begin, cell_end, nullptr,
                                          pat->P.staging_sym > 0, cached_geometry(pat, mesh));
}

namespace {
// Row bounds of nchunks ranges of about equal nnz, cut with the pattern's
// host copy of indptr; every range non-empty in rows.
std::vector<int64_t> row_ranges(const std::vector<int32_t>& ip, int64_t nrows, int64_t nnz,
                                int nchunks) {
  std::vector<int64_t> b{0};
  int64_t row = 0;
  for (int c = 0; c < nchunks && row < nrows; ++c) {
    const int64_t target = nnz * (c + 1) / nchunks;
    int64_t row1 = c == nchunks - 1
        ? nrows
        : (int64_t)(std::upper_bound(ip.begin() + row, ip.end(), (int32_t)target) - ip.begin()) - 1;
    if (row1 <= row) row1 = std::min<int64_t>(nrows, row + 1);
    b.push_back(row1);
    row = row1;
  }
  return b;
}

// Sums rows [row0, row1) -- from the staging, or fused from the pattern's
// cache when fs is given -- and queues their values' copy to the host on cs
// behind the sum.
// The one-pass P1 assembly's inputs for sum_rows_to_host.
struct GeometrySum {
  int dim;
  const double* geo;
  FemCoef diff, mass;
  const int16_t* mbase;
  const fem::UpperLists* upper;   // null: the row kernel
  int32_t* status;                 // the staged upper form's wait errors
  bool tma;                        // stage the upper lists' codes with TMA
};

// The one-pass vector sum's inputs for sum_rows_to_host (its pair blocks
// are in the staging).
struct VecSum {
  const fem::VecUpper* vec;
  bool mass;
  bool coop;   // the cooperative form (fem_set_onepass variant 2)
};

int sum_rows_to_host(const fem::Pattern& P, const std::vector<int32_t>& ip, const double* staging,
                     double* csr_values, double* host_values, int64_t row0, int64_t row1,
                     cudaStream_t st, cudaStream_t cs, const FusedSum* fs = nullptr,
                     const GeometrySum* gs = nullptr, const VecSum* vs = nullptr) {
  int rc = vs ? fem::vec_upper_sum(*vs->vec, staging, vs->mass, csr_values, st, row0, row1,
                                   vs->coop)
           : fs ? fem::csr_sum_scaled(P, fs->stiff, fs->diff, fs->mass1, fs->mscale, csr_values, st,
                                    row0, row1)
           : gs ? (gs->upper ? fem::csr_sum_upper_p1(P, *gs->upper, gs->dim, gs->geo, gs->diff,
                                                      gs->mass, gs->mbase, csr_values, st, row0,
                                                      row1, gs->status, gs->tma)
                             : fem::csr_sum_geometry_p1(P, gs->dim, gs->geo, gs->diff, gs->mass,
                                                        gs->mbase, csr_values, st, row0, row1))
                : fem::csr_sum(P, staging, csr_values, st, row0, row1, nullptr, P.staging_sym);
  if (rc) return rc;
  const int64_t a = ip[row0], b = ip[row1];
  if (b > a) {
    cudaEvent_t ev;
    FEM_TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev, 0);
    cudaEventDestroy(ev);
    if (e != cudaSuccess) return fem::check_cuda(e, "sum -> copy event");
    FEM_TRY_CUDA(cudaMemcpyAsync(host_values + a, csr_values + a, (b - a) * sizeof(double),
                                 cudaMemcpyDeviceToHost, cs));
  }
  return 0;
}
}  // namespace

int fem_csr_sum_to_host(const FemPattern* pat, const double* staging, double* csr_values,
                        double* host_values, int32_t nchunks, fem_stream_t stream,
                        fem_stream_t copy_stream) {
  if (!pat || !staging || !csr_values || !host_values || nchunks < 1 || nchunks > 64) {
    set_error(FEM_ERR_ARGUMENT, "null pattern or buffer, or chunks outside 1..64");
    return FEM_ERR_ARGUMENT;
  }
  if (!pat->P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern has no CSR structure");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream, cs = (cudaStream_t)copy_stream;
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(pat->family).sum_unroll;
  // row ranges of about equal nnz, cut with the pattern's host copy of indptr
  const std::vector<int32_t>& ip = pat->host_indptr;
  if ((int64_t)ip.size() != P.nrows + 1) {
    set_error(FEM_ERR_ARGUMENT, "pattern has no host row pointer");
    return FEM_ERR_ARGUMENT;
  }
  const std::vector<int64_t> b = row_ranges(ip, P.nrows, P.nnz, nchunks);
  for (size_t k = 0; k + 1 < b.size(); ++k) {
    int rc = sum_rows_to_host(P, ip, staging, csr_values, host_values, b[k], b[k + 1], st, cs);
    if (rc) return rc;
  }
  return 0;
}

namespace {
// Smallest DOF of each cell (the sort key of the pipeline plan).
// A DOF outside [0, nrows) sets *bad and the cell is left out (the plan
// is then refused).
__global__ void cell_min_dof_kernel(const int32_t* __restrict__ dofs, int64_t nelems, int nb,
                                    int64_t nrows, int32_t* __restrict__ key,
                                    int32_t* __restrict__ hist, int32_t* __restrict__ bad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelems) return;
  int32_t k = dofs[e];
  for (int i = 1; i < nb; ++i) k = min(k, dofs[(int64_t)i * nelems + e]);
  if (k < 0 || k >= nrows) {
    atomicOr(bad, 1);
    key[e] = -1;
    return;
  }
  key[e] = k;
  atomicAdd(hist + k, 1);
}

// Chunk of each cell: chunk c takes the keys [kb[c], kb[c+1]).
__global__ void cell_chunk_kernel(const int32_t* __restrict__ key, int64_t nelems,
                                  const int32_t* __restrict__ kb, int nchunks,
                                  int32_t* __restrict__ chunk) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelems) return;
  const int32_t k = key[e];
  int lo = 0, hi = nchunks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (kb[mid] <= k) lo = mid;
    else hi = mid - 1;
  }
  chunk[e] = lo;
}

__global__ void chunk_flag_kernel(const int32_t* __restrict__ chunk, int64_t nelems, int c,
                                  int32_t* __restrict__ flag) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nelems) flag[e] = chunk[e] == c ? 1 : 0;
  else if (e == nelems) flag[e] = 0;
}

// Stable compaction: the cells of chunk c, ascending.
__global__ void chunk_scatter_kernel(const int32_t* __restrict__ chunk, int64_t nelems, int c,
                                     const int32_t* __restrict__ pos, int32_t* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nelems && chunk[e] == c) out[pos[e]] = (int32_t)e;
}

// Builds pat's pipeline plan for nchunks chunks (synchronous, once): the
// cells are split by their smallest DOF at key bounds chosen for chunks of
// about equal size, and each chunk lists its cells in ascending order (so
// that its coefficient rows, geometry and staging rows are read and
// written in runs).
int pipeline_plan(const FemPattern* pat, const FemBasis& b, int64_t nelems, int nchunks,
                  cudaStream_t st) {
  std::lock_guard<std::mutex> lock(pat->plan_mu);
  if (pat->plan_nchunks == nchunks && pat->plan_cells) return 0;
  const int64_t nrows = pat->P.nrows;
  int32_t *key = nullptr, *hist = nullptr, *cum = nullptr, *chunk = nullptr, *flag = nullptr,
          *pos = nullptr, *kb = nullptr, *cells = nullptr;
  int32_t bad_h = 0;
  auto cleanup = [&]() {
    for (int32_t* q : {key, hist, cum, chunk, flag, pos, kb}) cudaFreeAsync(q, st);
  };
  const int64_t ne1 = std::max<int64_t>(1, nelems);
  cudaError_t e = cudaMallocAsync(&key, ne1 * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&hist, (nrows + 2) * 4, st);  // + the bad flag
  if (e == cudaSuccess) e = cudaMallocAsync(&cum, (nrows + 1) * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&chunk, ne1 * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&flag, (ne1 + 1) * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&pos, (ne1 + 1) * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&kb, (nchunks + 1) * 4, st);
  if (e == cudaSuccess) e = cudaMalloc(&cells, ne1 * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, (nrows + 2) * 4, st);
  if (e != cudaSuccess) {
    cleanup();
    cudaFree(cells);
    return fem::check_cuda(e, "pipeline plan buffers");
  }
  const unsigned grid = (unsigned)fem::ceil_div(ne1 + 1, 256);
  std::vector<int64_t> bounds(nchunks + 1, 0);
  std::vector<int32_t> kbh(nchunks + 1, (int32_t)nrows);
  int rc = 0;
  if (nelems > 0) {
    int32_t* bad = hist + nrows + 1;
    cell_min_dof_kernel<<<grid, 256, 0, st>>>(b.element_dofs, nelems, b.nbfun, nrows, key, hist,
                                              bad);
    e = cudaMemcpyAsync(&bad_h, bad, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = fem::check_cuda(e, "pipeline plan keys");
    else if (bad_h) {
      fem::set_error(FEM_ERR_ARGUMENT, "element DOFs outside the pattern's %lld rows",
                     (long long)nrows);
      rc = FEM_ERR_ARGUMENT;
    }
    // cum[k] = cells whose key is below k; chunk c takes the keys from the
    // first k with cum[k] >= c * nelems / nchunks
    std::vector<int32_t> cumh(nrows + 1);
    if (!rc) rc = fem::exclusive_scan_i32(hist, cum, nrows, nullptr, st);
    if (!rc) {
      e = cudaMemcpyAsync(cumh.data(), cum, (nrows + 1) * 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) rc = fem::check_cuda(e, "pipeline plan histogram");
    }
    if (!rc) {
      kbh[0] = 0;
      for (int k = 1; k < nchunks; ++k) {
        const int64_t target = nelems * k / nchunks;
        kbh[k] = (int32_t)(std::lower_bound(cumh.begin(), cumh.end(), (int32_t)target) -
                           cumh.begin());
        kbh[k] = std::min<int32_t>(std::max(kbh[k], kbh[k - 1]), (int32_t)nrows);
      }
      kbh[nchunks] = (int32_t)nrows;
      for (int k = 0; k < nchunks; ++k) bounds[k] = cumh[kbh[k]];
      bounds[nchunks] = nelems;
      e = cudaMemcpyAsync(kb, kbh.data(), (nchunks + 1) * 4, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) {
        cell_chunk_kernel<<<grid, 256, 0, st>>>(key, nelems, kb, nchunks, chunk);
        e = cudaGetLastError();
      }
      for (int c = 0; c < nchunks && e == cudaSuccess && !rc; ++c) {
        if (bounds[c + 1] == bounds[c]) continue;
        chunk_flag_kernel<<<grid, 256, 0, st>>>(chunk, nelems, c, flag);
        rc = fem::exclusive_scan_i32(flag, pos, nelems, nullptr, st);
        if (!rc) {
          chunk_scatter_kernel<<<grid, 256, 0, st>>>(chunk, nelems, c, pos, cells + bounds[c]);
          e = cudaGetLastError();
        }
      }
      // kbh stays alive until the stream has read it
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (!rc && e != cudaSuccess) rc = fem::check_cuda(e, "pipeline plan");
    }
  }
  cleanup();
  if (rc) {
    cudaFree(cells);
    return rc;
  }
  cudaFree(pat->plan_cells);
  pat->plan_cells = cells;
  pat->plan_bounds = bounds;
  // rows below the first key of chunk c+1 are final once chunks 0..c are done
  pat->plan_rows.assign(nchunks, nrows);
  for (int k = 0; k + 1 < nchunks; ++k) pat->plan_rows[k] = std::min<int64_t>(kbh[k + 1], nrows);
  pat->plan_nchunks = nchunks;
  return 0;
}

// Copies the host rows of the cells cells[a .. b) (stride doubles each)
// into the device array, reading host memory directly (the device's
// pageable-memory access); 16-byte loads when the layout allows them.  The
// copy is bound by the host link's latency, not by the SMs: a small grid
// keeps kGatherUnroll independent loads in flight per thread and leaves
// the SMs to the local kernels that run beside it.
constexpr int kGatherUnroll = 4;

__global__ void gather_host_rows_kernel(FemHostRows r, const int32_t* __restrict__ cells,
                                        int64_t a, int64_t b, int wide) {
  const int64_t stride = r.stride > 1 ? r.stride : 1;
  const int64_t per = wide ? stride / 2 : stride;  // loads per row
  const int64_t n = (b - a) * per;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t g0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g0 < n;
       g0 += nt * kGatherUnroll) {
    int64_t off[kGatherUnroll];
#pragma unroll
    for (int u = 0; u < kGatherUnroll; ++u) {
      const int64_t g = g0 + u * nt;
      off[u] = -1;
      if (g < n) {
        const int64_t i = g / per, q = g - i * per;
        off[u] = (int64_t)__ldg(cells + a + i) * per + q;  // in load units
      }
    }
    if (wide) {
      double2 v[kGatherUnroll];
#pragma unroll
      for (int u = 0; u < kGatherUnroll; ++u)
        if (off[u] >= 0) v[u] = reinterpret_cast<const double2*>(r.host)[off[u]];
#pragma unroll
      for (int u = 0; u < kGatherUnroll; ++u)
        if (off[u] >= 0) reinterpret_cast<double2*>(r.dev)[off[u]] = v[u];
    } else {
      double v[kGatherUnroll];
#pragma unroll
      for (int u = 0; u < kGatherUnroll; ++u)
        if (off[u] >= 0) v[u] = r.host[off[u]];
#pragma unroll
      for (int u = 0; u < kGatherUnroll; ++u)
        if (off[u] >= 0) r.dev[off[u]] = v[u];
    }
  }
}
}  // namespace

int fem_host_memory_access(int32_t* supported) {
  if (!supported) {
    set_error(FEM_ERR_ARGUMENT, "null output");
    return FEM_ERR_ARGUMENT;
  }
  int dev = 0, v = 0;
  FEM_TRY_CUDA(cudaGetDevice(&dev));
  FEM_TRY_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev));
  *supported = v ? 1 : 0;
  return 0;
}

int fem_assemble_to_host_pipelined(const FemMesh* mesh, const FemBasis* basis,
                                   const FemBilinear* form, const FemPattern* pat,
                                   double* staging, double* csr_values, double* host_values,
                                   int32_t* status, const FemHostRows* rows, int32_t nfields,
                                   int32_t nchunks, fem_stream_t stream,
                                   fem_stream_t upload_stream, fem_stream_t copy_stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!form || !pat || !staging || !csr_values || !host_values || nchunks < 1 ||
      nchunks > 256 || nfields < 0 || nfields > 16 || (nfields > 0 && !rows)) {
    set_error(FEM_ERR_ARGUMENT, "null argument, chunks outside 1..256 or fields outside 0..16");
    return FEM_ERR_ARGUMENT;
  }
  if (pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun || !pat->P.has_matrix ||
      pat->P.nrows != basis->ndofs || (int64_t)pat->host_indptr.size() != pat->P.nrows + 1) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  for (int k = 0; k < nfields; ++k)
    if (!rows[k].host || !rows[k].dev || rows[k].stride < 0) {
      set_error(FEM_ERR_ARGUMENT, "host rows %d: null pointer or negative stride", k);
      return FEM_ERR_ARGUMENT;
    }
  if (nfields > 0) {
    int32_t ok = 0;
    if ((rc = fem_host_memory_access(&ok))) return rc;
    if (!ok) {
      set_error(FEM_ERR_UNSUPPORTED, "kernels on this device cannot read pageable host memory "
                "(upload the coefficients first, then pass no host rows)");
      return FEM_ERR_UNSUPPORTED;
    }
  }
  cudaStream_t st = (cudaStream_t)stream, up = (cudaStream_t)upload_stream,
               cs = (cudaStream_t)copy_stream;
  const int64_t ne = mesh->nelems;
  if ((rc = pipeline_plan(pat, *basis, ne, nchunks, st))) return rc;
  fem::Pattern P = pat->P;
  const fem::Tuning tune = fem::tuning_for(pat->family);
  P.sum_unroll = tune.sum_unroll;
  P.sum_cols = tune.sum_cols;
  const std::vector<int64_t>& cb = pat->plan_bounds;
  const std::vector<int64_t>& done = pat->plan_rows;
  const int32_t* cells = pat->plan_cells;
  FusedSum fs;
  const bool fused = fused_sum(pat, mesh, basis, form, &fs);
  GeometrySum gs{mesh->dim, pat->geo, form->diff, form->mass, pat->mbase,
                 (tune.onepass >= 1 && pat->upper_ok) ? &pat->upper : nullptr, status,
                 tune.onepass == 2};
  const bool onepass = !fused && geometry_sum(pat, mesh, basis, form);
  const bool vec1 = !fused && !onepass && vector_onepass(pat, mesh, basis);
  const VecSum vs{&pat->vec, form->mass.field || form->mass.scale != 0.0, tune.onepass == 2};
  std::vector<cudaEvent_t> evs;
  auto event = [&](cudaEvent_t* ev) -> cudaError_t {
    cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e == cudaSuccess) evs.push_back(*ev);
    return e;
  };
  auto release = [&]() {
    for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
  };
  // the coefficient rows of every chunk, queued on the upload stream
  std::vector<cudaEvent_t> ready(nchunks, nullptr);
  if (nfields > 0) {
    cudaEvent_t start;
    cudaError_t e = event(&start);
    if (e == cudaSuccess) e = cudaEventRecord(start, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(up, start, 0);
    for (int c = 0; c < nchunks && e == cudaSuccess; ++c) {
      const int64_t n = cb[c + 1] - cb[c];
      for (int k = 0; k < nfields && n > 0; ++k) {
        const int64_t s = rows[k].stride > 1 ? rows[k].stride : 1;
        const int wide = (s % 2 == 0) && ((uintptr_t)rows[k].host % 16 == 0) &&
                         ((uintptr_t)rows[k].dev % 16 == 0);
        const int64_t work = n * (wide ? s / 2 : s);
        const unsigned grid = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>(fem::ceil_div(work, 256 * kGatherUnroll),
                                 (int64_t)fem::num_sms() / 2));
        gather_host_rows_kernel<<<grid, 256, 0, up>>>(rows[k], cells, cb[c], cb[c + 1], wide);
      }
      e = cudaGetLastError();
      if (e == cudaSuccess) e = event(&ready[c]);
      if (e == cudaSuccess) e = cudaEventRecord(ready[c], up);
    }
    if (e != cudaSuccess) {
      release();
      return fem::check_cuda(e, "host row gather");
    }
  }
  int64_t row = 0;
  for (int c = 0; c < nchunks; ++c) {
    if (ready[c]) {
      cudaError_t e = cudaStreamWaitEvent(st, ready[c], 0);
      if (e != cudaSuccess) {
        release();
        return fem::check_cuda(e, "wait for host rows");
      }
    }
    if (cb[c + 1] > cb[c]) {
      rc = vec1 ? node_pair_values(pat, mesh, basis, form, staging, status, st, cb[c],
                                   cb[c + 1], cells)
           : (fused || onepass)
               ? fem_fast::coef_checks(*form, pat->coef_bits, status, st, cb[c], cb[c + 1], cells)
               : fem_fast::local_matrices_checked(*mesh, *basis, *form, staging,
                                                    status ? pat->coef_bits : nullptr, status, st,
                                                    cb[c], cb[c + 1], cells,
                                                    pat->P.staging_sym > 0,
                                                    cached_geometry(pat, mesh));
      if (rc) {
        release();
        return rc;
      }
    }
    // rows below the smallest DOF of the next chunk's first cell are final
    // (the one-pass vector sum: down to a window of its node blocks)
    int64_t row1 = done[c];
    if (vec1 && row1 < P.nrows) {
      const int64_t w = fem::vec_window_rows(pat->vec);
      row1 = row1 / w * w;
    }
    if (onepass && gs.upper && gs.upper->block_rows > 0 && row1 < P.nrows)
      row1 = row1 / gs.upper->block_rows * gs.upper->block_rows;
    if (row1 > row) {
      rc = sum_rows_to_host(P, pat->host_indptr, staging, csr_values, host_values, row, row1, st,
                            cs, fused ? &fs : nullptr, onepass ? &gs : nullptr,
                            vec1 ? &vs : nullptr);
      if (rc) {
        release();
        return rc;
      }
      row = row1;
    }
  }
  release();
  return 0;
}

int fem_assemble_to_host(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                         const FemPattern* pat, double* staging, double* csr_values,
                         double* host_values, int32_t* status, int32_t nchunks,
                         fem_stream_t stream, fem_stream_t copy_stream) {
  if (!mesh) {
    set_error(FEM_ERR_ARGUMENT, "null mesh");
    return FEM_ERR_ARGUMENT;
  }
  int rc = fem_assemble_local(mesh, basis, form, pat, staging, status, 0, mesh->nelems, stream);
  if (rc) return rc;
  return fem_csr_sum_to_host(pat, staging, csr_values, host_values, nchunks, stream, copy_stream);
}

int fem_csr_sum(const FemPattern* pat, const double* local, double* csr_values, int32_t* status,
                fem_stream_t stream) {
  (void)status;
  if (pat && pat->P.nnz == 0) return 0;   // nothing to sum: buffers may be null
  if (!pat || !local || !csr_values) {
    set_error(FEM_ERR_ARGUMENT, "null pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(pat->family).sum_unroll;
  return fem::csr_sum(P, local, csr_values, (cudaStream_t)stream);
}

int fem_csr_sum_staged(const FemPattern* pat, const double* staging, double* csr_values,
                       fem_stream_t stream) {
  if (pat && pat->P.nnz == 0) return 0;
  if (!pat || !staging || !csr_values) {
    set_error(FEM_ERR_ARGUMENT, "null pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(pat->family).sum_unroll;
  return fem::csr_sum(P, staging, csr_values, (cudaStream_t)stream, 0, -1, nullptr, P.staging_sym);
}

int fem_vector_sum(const FemPattern* pat, const double* local, double* b, fem_stream_t stream) {
  if (!pat || !local || !b) {
    set_error(FEM_ERR_ARGUMENT, "null pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  return fem::vector_sum(pat->P, local, b, (cudaStream_t)stream);
}

int fem_assemble_vector(const FemMesh* mesh, const FemBasis* basis, const FemLinear* form,
                        const FemPattern* pat, double* staging, double* b, fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!form || !pat || !staging || !b) {
    set_error(FEM_ERR_ARGUMENT, "null form, pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  if (pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  rc = fem_fast::local_vectors(*mesh, *basis, *form, staging, nullptr, st);
  if (rc) return rc;
  return fem::vector_sum(pat->P, staging, b, st);
}

static int program_entry(int mode, const FemMesh* mesh, const FemBasis* basis,
                         const FemFacets* facets, const FemProgram* program, double* out,
                         int32_t* status, fem_stream_t stream) {
  int rc = validate(mesh, basis, true);
  if (rc) return rc;
  if (!program || !out || !status) {
    set_error(FEM_ERR_ARGUMENT, "null program, output or status");
    return FEM_ERR_ARGUMENT;
  }
  return fem::program_eval(mode, *mesh, *basis, facets, *program, out, status,
                           (cudaStream_t)stream, nullptr);
}

int fem_program_local_matrices_mixed(const FemMesh* mesh, const FemBasis* vbasis,
                                     const FemBasis* ubasis, const FemProgram* program,
                                     double* local, int32_t* status, fem_stream_t stream) {
  int rc = validate(mesh, vbasis, true);
  if (!rc) rc = validate(mesh, ubasis, true);
  if (rc) return rc;
  if (!program || !local || !status) {
    set_error(FEM_ERR_ARGUMENT, "null program, output or status");
    return FEM_ERR_ARGUMENT;
  }
  return fem::program_eval(0, *mesh, *vbasis, nullptr, *program, local, status,
                           (cudaStream_t)stream, ubasis);
}

int fem_pattern_build_local_mixed(const FemMesh* mesh, const FemBasis* vbasis,
                                  const FemBasis* ubasis, const double* local, FemPattern** out,
                                  fem_stream_t stream) {
  int rc = validate(mesh, vbasis, true);
  if (!rc) rc = validate(mesh, ubasis, true);
  if (rc) return rc;
  if (!out || (!local && mesh->nelems > 0)) {
    set_error(FEM_ERR_ARGUMENT, "null local matrices or output handle");
    return FEM_ERR_ARGUMENT;
  }
  *out = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  FemPattern* H = new FemPattern();
  H->family = vbasis->family;
  H->vector = vbasis->vector;
  rc = fem::build_incidence(vbasis->element_dofs, mesh->nelems, vbasis->nbfun, vbasis->ndofs,
                            &H->P, st);
  if (!rc) rc = fem::build_csr(ubasis->element_dofs, ubasis->nbfun, ubasis->ndofs, local, &H->P, st);
  if (!rc) rc = host_row_pointer(H, st);
  if (rc) {
    fem::free_pattern(new fem::Pattern(H->P));
    delete H;
    return rc;
  }
  *out = H;
  return 0;
}

namespace {
__global__ void index_range_kernel(const int32_t* __restrict__ idx, int64_t n, int64_t hi,
                                   int32_t* __restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (idx[i] < 0 || idx[i] >= hi) atomicOr(bad, 1);
}
}  // namespace

int fem_coo_pattern_build(const int32_t* rows, const int32_t* cols, const double* data,
                          int64_t n, int64_t nrows, int64_t ncols, FemPattern** out,
                          fem_stream_t stream) {
  if (!out || n < 0 || nrows < 0 || ncols < 0 || (n > 0 && (!rows || !cols || !data))) {
    set_error(FEM_ERR_ARGUMENT, "null COO arrays or output handle, or a negative size");
    return FEM_ERR_ARGUMENT;
  }
  *out = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  if (n > 0) {
    fem::AsyncScratch scratch(st);
    int32_t* bad = nullptr;
    FEM_TRY_CUDA(scratch.alloc(&bad, sizeof(int32_t)));
    FEM_TRY_CUDA(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
    const unsigned grid = (unsigned)std::min<int64_t>(fem::ceil_div(n, 256), fem::num_sms() * 8);
    index_range_kernel<<<grid, 256, 0, st>>>(cols, n, ncols, bad);
    FEM_LAUNCH_CHECK("index_range_kernel");
    int32_t h = 0;
    FEM_TRY_CUDA(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, st));
    FEM_TRY_CUDA(cudaStreamSynchronize(st));
    if (h) {
      set_error(FEM_ERR_ARGUMENT, "a COO column index lies outside [0, %lld)", (long long)ncols);
      return FEM_ERR_ARGUMENT;
    }
  }
  FemPattern* H = new FemPattern();
  // each COO entry is a 1 x 1 "cell": its row the test DOF, its column the
  // trial DOF, its value the local entry (exact zeros create no CSR entry)
  int rc = fem::build_incidence(rows, n, 1, nrows, &H->P, st);
  if (!rc) rc = fem::build_csr(cols, 1, ncols, data, &H->P, st);
  if (!rc) rc = host_row_pointer(H, st);
  if (rc) {
    fem::free_pattern(new fem::Pattern(H->P));
    delete H;
    return rc;
  }
  *out = H;
  return 0;
}

int fem_program_local_matrices(const FemMesh* mesh, const FemBasis* basis,
                               const FemProgram* program, double* local, int32_t* status,
                               fem_stream_t stream) {
  return program_entry(0, mesh, basis, nullptr, program, local, status, stream);
}

int fem_program_local_vectors(const FemMesh* mesh, const FemBasis* basis,
                              const FemProgram* program, double* local, int32_t* status,
                              fem_stream_t stream) {
  return program_entry(1, mesh, basis, nullptr, program, local, status, stream);
}

int fem_program_elemental(const FemMesh* mesh, const FemBasis* basis, const FemProgram* program,
                          double* out, int32_t* status, fem_stream_t stream) {
  return program_entry(2, mesh, basis, nullptr, program, out, status, stream);
}

static int facets_given(const FemFacets* facets) {
  if (!facets) {
    set_error(FEM_ERR_ARGUMENT, "null facets");
    return FEM_ERR_ARGUMENT;
  }
  return 0;
}

int fem_facet_program_local_matrices(const FemMesh* mesh, const FemBasis* basis,
                                     const FemFacets* facets, const FemProgram* program,
                                     double* local, int32_t* status, fem_stream_t stream) {
  if (int rc = facets_given(facets)) return rc;
  return program_entry(0, mesh, basis, facets, program, local, status, stream);
}

int fem_facet_program_local_vectors(const FemMesh* mesh, const FemBasis* basis,
                                    const FemFacets* facets, const FemProgram* program,
                                    double* local, int32_t* status, fem_stream_t stream) {
  if (int rc = facets_given(facets)) return rc;
  return program_entry(1, mesh, basis, facets, program, local, status, stream);
}

int fem_facet_program_elemental(const FemMesh* mesh, const FemBasis* basis,
                                const FemFacets* facets, const FemProgram* program, double* out,
                                int32_t* status, fem_stream_t stream) {
  if (int rc = facets_given(facets)) return rc;
  return program_entry(2, mesh, basis, facets, program, out, status, stream);
}

int fem_facet_interpolate(const FemMesh* mesh, const FemBasis* basis, const FemFacets* facets,
                          int32_t nq, const double* X, const double* w, double* out,
                          fem_stream_t stream) {
  int rc = validate(mesh, basis, true);
  if (rc) return rc;
  if ((rc = facets_given(facets))) return rc;
  return interp_with_status(mesh, basis, facets, nq, X, w, out, stream);
}

int fem_pattern_build_local(const FemMesh* mesh, const FemBasis* basis, const double* local,
                            FemPattern** out, fem_stream_t stream) {
  int rc = validate(mesh, basis, true);
  if (rc) return rc;
  if (!out || (!local && mesh->nelems > 0)) {
    set_error(FEM_ERR_ARGUMENT, "null local matrices or output handle");
    return FEM_ERR_ARGUMENT;
  }
  *out = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  FemPattern* H = new FemPattern();
  H->family = basis->family;
  H->vector = basis->vector;
  rc = fem::build_incidence(basis->element_dofs, mesh->nelems, basis->nbfun, basis->ndofs, &H->P, st);
  if (!rc) rc = fem::build_csr(basis->element_dofs, basis->nbfun, basis->ndofs, local, &H->P, st);
  if (!rc) rc = host_row_pointer(H, st);
  if (rc) {
    fem::free_pattern(new fem::Pattern(H->P));
    delete H;
    return rc;
  }
  *out = H;
  return 0;
}

int fem_csr_sum_checked(const FemPattern* pat, const double* local, double* csr_values,
                        int32_t* status, fem_stream_t stream) {
  if (!pat || (!local && pat->P.nelems > 0) || (!csr_values && pat->P.nnz > 0) || !status) {
    set_error(FEM_ERR_ARGUMENT, "null pattern, buffer or status");
    return FEM_ERR_ARGUMENT;
  }
  if (!pat->P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern has no CSR structure");
    return FEM_ERR_ARGUMENT;
  }
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(pat->family).sum_unroll;
  return fem::csr_sum(P, local, csr_values, (cudaStream_t)stream, 0, -1, status);
}

int fem_interpolate(const FemMesh* mesh, const FemBasis* basis, int32_t nq, const double* X,
                    const double* w, double* out, fem_stream_t stream) {
  int rc = validate(mesh, basis, true);
  if (rc) return rc;
  return fem::interpolate(*mesh, *basis, nullptr, nq, X, w, out, nullptr, (cudaStream_t)stream);
}

int fem_facet_geometry(const FemMesh* mesh, const FemBasis* basis, const FemFacets* facets,
                       int32_t nq, const double* X, double* geo, int32_t* status,
                       fem_stream_t stream) {
  int rc = validate(mesh, basis, true);
  if (rc) return rc;
  if ((rc = facets_given(facets))) return rc;
  return fem::facet_geometry(*mesh, *basis, *facets, nq, X, geo, status, (cudaStream_t)stream);
}

int fem_sum_pairwise(const double* x, int64_t n, double* out, fem_stream_t stream) {
  if ((!x && n > 0) || !out || n < 0) {
    set_error(FEM_ERR_ARGUMENT, "null input or output");
    return FEM_ERR_ARGUMENT;
  }
  return fem::sum_pairwise(x, n, out, (cudaStream_t)stream);
}

}  // extern "C"
