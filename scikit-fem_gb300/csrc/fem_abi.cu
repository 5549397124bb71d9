// extern "C" entry points of libskfem_gb300 (declared in include/skfem_gb300.h).

#include <mutex>
#include <string>

#include "fem_common.cuh"

#include <algorithm>
#include <vector>

namespace fem_fast {
int local_matrices(const FemMesh&, const FemBasis&, const FemBilinear&, double*, int32_t*,
                   cudaStream_t);
// cells [ebeg, eend) only (eend < 0: to the last cell)
int local_matrices_checked(const FemMesh&, const FemBasis&, const FemBilinear&, double*,
                           const uint8_t*, int32_t*, cudaStream_t, int64_t ebeg = 0,
                           int64_t eend = -1);
int local_vectors(const FemMesh&, const FemBasis&, const FemLinear&, double*, int32_t*,
                  cudaStream_t);
}  // namespace fem_fast
namespace fem_exact {
int local_matrices(const FemMesh&, const FemBasis&, const FemBilinear&, double*, int32_t*,
                   cudaStream_t);
}  // namespace fem_exact

namespace fem {
int build_incidence(const int32_t* dofs, int64_t nelems, int nb, int64_t nrows, Pattern* P,
                    cudaStream_t st);
int build_csr(const int32_t* udofs, int nu, int64_t ncols, const double* local, Pattern* P,
              cudaStream_t st);
int vector_sum(const Pattern& P, const double* local, double* b, cudaStream_t st);
void free_pattern(Pattern* P);
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
};

using fem::set_error;

namespace fem {
const Pattern* pattern_of(const FemPattern* h) { return h ? &h->P : nullptr; }
const uint8_t* pattern_coef_bits(const FemPattern* h) { return h ? h->coef_bits : nullptr; }
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

int fem_set_tuning(int family, int local_block, int persistent, int sum_unroll) {
  if (family < 1 || family > 5 || (local_block != 64 && local_block != 128 && local_block != 256) ||
      persistent < 0 || (sum_unroll != 4 && sum_unroll != 8 && sum_unroll != 16)) {
    set_error(FEM_ERR_ARGUMENT, "invalid tuning (family %d, block %d, persistent %d, unroll %d)",
              family, local_block, persistent, sum_unroll);
    return FEM_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(fem::g_tuning_mu);
  fem::g_tuning[family].local_block = local_block;
  fem::g_tuning[family].persistent = persistent;
  fem::g_tuning[family].sum_unroll = sum_unroll;
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
  delete pat;
}

int fem_assemble(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                 const FemPattern* pat, double* staging, double* csr_values, int32_t* status,
                 fem_stream_t stream) {
  int rc = validate(mesh, basis);
  if (rc) return rc;
  if (!form || !pat || !staging || !csr_values) {
    set_error(FEM_ERR_ARGUMENT, "null form, pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  if (pat->P.nelems != mesh->nelems || pat->P.nbfun_v != basis->nbfun || !pat->P.has_matrix) {
    set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  cudaStream_t st = (cudaStream_t)stream;
  // the local kernel also compares each element's coefficient zero bits
  // with the pattern's (FEM_ERR_STALE_PATTERN)
  rc = fem_fast::local_matrices_checked(*mesh, *basis, *form, staging,
                                        status ? pat->coef_bits : nullptr, status, st);
  if (rc) return rc;
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(basis->family).sum_unroll;
  return fem::csr_sum(P, staging, csr_values, st);
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
                                          (cudaStream_t)stream, cell_begin, cell_end);
}

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
  int64_t row = 0;
  for (int c = 0; c < nchunks && row < P.nrows; ++c) {
    const int64_t target = (int64_t)P.nnz * (c + 1) / nchunks;
    int64_t row1 = c == nchunks - 1
        ? P.nrows
        : (int64_t)(std::upper_bound(ip.begin() + row, ip.end(), (int32_t)target) - ip.begin()) - 1;
    if (row1 <= row) row1 = std::min<int64_t>(P.nrows, row + 1);
    int rc = fem::csr_sum(P, staging, csr_values, st, row, row1);
    if (rc) return rc;
    const int64_t a = ip[row], b = ip[row1];
    if (b > a) {
      cudaEvent_t ev;
      FEM_TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      FEM_TRY_CUDA(cudaEventRecord(ev, st));
      FEM_TRY_CUDA(cudaStreamWaitEvent(cs, ev, 0));
      cudaEventDestroy(ev);
      FEM_TRY_CUDA(cudaMemcpyAsync(host_values + a, csr_values + a, (b - a) * sizeof(double),
                                   cudaMemcpyDeviceToHost, cs));
    }
    row = row1;
  }
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
  if (!pat || !local || !csr_values) {
    set_error(FEM_ERR_ARGUMENT, "null pattern or buffer");
    return FEM_ERR_ARGUMENT;
  }
  fem::Pattern P = pat->P;
  P.sum_unroll = fem::tuning_for(pat->family).sum_unroll;
  return fem::csr_sum(P, local, csr_values, (cudaStream_t)stream);
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
  if (!pat || !local || !csr_values || !status) {
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
