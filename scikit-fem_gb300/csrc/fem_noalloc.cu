// fem_assemble_noalloc: fem_assemble for callers that cannot allocate.
//
// Some callers can hand this library their input and output buffers but
// cannot give it scratch memory: a solver or simulation framework that has
// reserved the GPU's memory up front behind its own allocator (so a
// cudaMalloc from a third-party library would fail or break its budget),
// or an application that forbids device allocations after start-up.  For
// them this entry point runs the same two kernels as fem_assemble -- the
// fused local-matrix kernel and the fixed-order segmented sum -- but keeps
// the local-matrix staging in a file-scope device array instead of a
// caller-provided buffer.  It calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// The array is kNoAllocScratchBytes (64 MiB) per GPU; every GPU that loads
// this library holds it until the process exits.  An assembly needs
// nelems * nbfun^2 * 8 bytes of it (TetP1: 128 B per cell, so at most
// 524,288 cells; Hex1 512 B; scalar TetP2 800 B; vector TetP2 7,200 B) and
// larger meshes are rejected with FEM_ERR_CAPACITY.
//
// Calls share the array.  Nothing in it has to start at zero (the local
// kernel writes every entry the sum reads), but two calls whose kernels
// overlap on the GPU -- on different streams, or from different host
// threads -- race on it; callers serialise them.
//
// Loading: with CUDA's lazy module loading the module that holds the array
// is loaded on a device by this entry point's first call there (the symbol
// lookup below), which is also when its 64 MiB are taken.  A caller whose
// allocator reserves the device's memory makes one warm-up call at
// start-up, before that reservation and before any stream capture.  The
// device address is cached per device ordinal, for the runtime's primary
// context of that device (the context the CUDA runtime and torch use).

#include <mutex>

#include "fem_common.cuh"

namespace fem_fast {
int local_matrices_checked(const FemMesh&, const FemBasis&, const FemBilinear&, double*,
                           const uint8_t*, int32_t*, cudaStream_t, int64_t ebeg, int64_t eend,
                           const int32_t* cells, int upper, const double* geo);
}
namespace fem {
const Pattern* pattern_of(const FemPattern* h);
const uint8_t* pattern_coef_bits(const FemPattern* h);
int validate_mesh_basis(const FemMesh* m, const FemBasis* b);
const double* pattern_geometry(const FemPattern* h, const FemMesh* m);
}  // namespace fem

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

// In host code this name is only a host-side stand-in for the device
// array: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchBytes / sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up
// once per device (with that device current) and cached.
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return fem::check_cuda(err, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    fem::set_error(FEM_ERR_ARGUMENT, "device ordinal %d out of range", dev);
    return FEM_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    double* p = nullptr;
    err = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (err != cudaSuccess) return fem::check_cuda(err, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return 0;
}

}  // namespace

// The two-pass path of fem_assemble -- the local kernel (on the pattern's
// per-cell geometry cache when the mesh's coordinates are the cached ones)
// into the full local-matrix layout, then the fixed-order sum -- with the
// staging in the static array.  status (device int32, may be NULL): with it
// the local kernel also runs fem_assemble's coefficient checks and reports
// FEM_ERR_STALE_PATTERN / FEM_ERR_VARYING there; with NULL no check runs, so
// a coefficient whose zero structure changed since the pattern was built
// goes unreported (the values are then those of the old pattern).
extern "C" int fem_assemble_noalloc(const FemMesh* mesh, const FemBasis* basis,
                                    const FemBilinear* form, const FemPattern* pat,
                                    double* csr_values, int32_t* status, fem_stream_t stream) {
  int rc = fem::validate_mesh_basis(mesh, basis);
  if (rc) return rc;
  if (!form || !pat) {
    fem::set_error(FEM_ERR_ARGUMENT, "null form or pattern");
    return FEM_ERR_ARGUMENT;
  }
  const fem::Pattern* P = fem::pattern_of(pat);
  if (!P->has_matrix || P->nelems != mesh->nelems || P->nbfun_v != basis->nbfun) {
    fem::set_error(FEM_ERR_ARGUMENT, "pattern does not belong to this mesh / basis");
    return FEM_ERR_ARGUMENT;
  }
  // an empty pattern (no cells, or only exact zeros) takes no value buffer
  if (!csr_values && P->nnz > 0) {
    fem::set_error(FEM_ERR_ARGUMENT, "null output");
    return FEM_ERR_ARGUMENT;
  }
  const int64_t need = mesh->nelems * (int64_t)basis->nbfun * basis->nbfun * (int64_t)sizeof(double);
  if (need > (int64_t)kNoAllocScratchBytes) {
    fem::set_error(FEM_ERR_CAPACITY,
                   "fem_assemble_noalloc: %lld cells x %d x %d local matrices need %lld bytes of "
                   "scratch; its static scratch holds %lld bytes (use fem_assemble with a "
                   "caller-provided staging buffer)",
                   (long long)mesh->nelems, basis->nbfun, basis->nbfun, (long long)need,
                   (long long)kNoAllocScratchBytes);
    return FEM_ERR_CAPACITY;
  }
  if (mesh->nelems == 0) return 0;
  double* scratch = nullptr;
  rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  rc = fem_fast::local_matrices_checked(*mesh, *basis, *form, scratch,
                                        status ? fem::pattern_coef_bits(pat) : nullptr, status, st,
                                        0, -1, nullptr, 0, fem::pattern_geometry(pat, mesh));
  if (rc) return rc;
  return fem::csr_sum(*P, scratch, csr_values, st);
}
