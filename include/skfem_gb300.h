/*
 * skfem_gb300 -- C ABI of the GB300 (sm_103a) cell-assembly library.
 *
 * The library replaces the numerical core of scikit-fem's cell assembly:
 *
 *   CellBasis.__init__ / MappingAffine / MappingIsoparametric /
 *   ElementH1.gbasis / ElementVector.gbasis      (skfem/assembly/basis/cell_basis.py:42-106,
 *                                                 skfem/mapping/mapping_affine.py:55-232,
 *                                                 skfem/mapping/mapping_isoparametric.py:112-226,
 *                                                 skfem/element/element_h1.py:10-24,
 *                                                 skfem/element/element_vector.py:36-48)
 *   BilinearForm._assemble / LinearForm._assemble (skfem/assembly/form/bilinear_form.py:58-128,
 *                                                 skfem/assembly/form/linear_form.py:18-49)
 *   COOData._assemble_scipy_csr / COOData.toarray (skfem/assembly/form/coo_data.py:27-36, 102-108)
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer owned by the caller (torch
 *     tensors on the Python side).  The library never frees caller memory.
 *   - FemPattern objects are allocated by fem_pattern_build and released
 *     with fem_pattern_destroy.
 *   - Every entry point is stream-ordered on the given stream and returns 0
 *     on success or a FemStatus code; fem_last_error() gives a thread-local
 *     message describing the last failure on the calling thread.
 *   - Values are float64, indices int32, exactly as the reference
 *     (skfem/assembly/dofs.py:270, skfem/mesh/mesh.py:558-559).
 *   - Layouts follow the reference: p is (dim, nverts) C-contiguous
 *     (Mesh.p), element_dofs is (nbfun, nelems) C-contiguous
 *     (Dofs.element_dofs).
 */
#ifndef SKFEM_GB300_H
#define SKFEM_GB300_H

#ifndef __CUDACC_RTC__
#include <stdint.h>
#else
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef short int16_t;
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* fem_stream_t; /* == cudaStream_t */

/* Status codes. */
enum FemStatus {
  FEM_OK = 0,
  FEM_ERR_ARGUMENT = 1,      /* invalid argument (raised as ValueError by the Python layer) */
  FEM_ERR_UNSUPPORTED = 2,   /* family / form combination not implemented (NotImplementedError) */
  FEM_ERR_CUDA = 3,          /* CUDA runtime error */
  FEM_ERR_ZERO_JACOBIAN = 4, /* isoparametric detDF == 0 (mapping_isoparametric.py:195-196) */
  FEM_ERR_STALE_PATTERN = 5, /* exact-zero structure of the local matrices changed: rebuild */
  FEM_ERR_CAPACITY = 6,      /* a CSR row exceeds the per-row working-set limit */
  FEM_ERR_VARYING = 7,       /* a strided coefficient is not constant over a cell's
                                points (status word only): use the generic kernels */
  FEM_ERR_NEWTON = 8,        /* the inverse isoparametric map did not converge
                                (status word only, fem_facet_geometry) */
  FEM_ERR_TIMEOUT = 9        /* a bounded wait inside a persistent kernel ran out; that
                                launch's results are not valid (status word only) */
};

/* Element families (the reference classes they stand for). */
enum FemFamily {
  FEM_TRI_P1 = 1, /* ElementTriP1  (element_tri_p1.py:18-33)  */
  FEM_TRI_P2 = 2, /* ElementTriP2  (element_tri_p2.py:22-48)  */
  FEM_TET_P1 = 3, /* ElementTetP1  (element_tet_p1.py:19-45)  */
  FEM_TET_P2 = 4, /* ElementTetP2  (element_tet_p2.py:26-103) */
  FEM_HEX_1 = 5   /* ElementHex1   (element_hex1.py:23-69), isoparametric */
};

/* Mesh geometry (Mesh.p / Mesh.t, skfem/mesh/mesh.py:42-44, 544-591). */
typedef struct FemMesh {
  int32_t dim;      /* 2 or 3 */
  int32_t nloc;     /* vertices per element: 3, 4 or 8 */
  int64_t nverts;   /* columns of p */
  int64_t nelems;   /* columns of t */
  const double* p;  /* (dim, nverts) */
  const int32_t* t; /* (nloc, nelems) */
} FemMesh;

/* Global numbering of one basis (Dofs, skfem/assembly/dofs.py:264-334). */
typedef struct FemBasis {
  int32_t family;              /* FemFamily */
  int32_t vector;              /* 1 for ElementVector(family), 0 for scalar */
  int32_t nbfun;               /* local functions (vector: dim * scalar) */
  int32_t pad_;
  int64_t ndofs;               /* N */
  const int32_t* element_dofs; /* (nbfun, nelems) */
} FemBasis;

/* A per-element coefficient: scale * field[e], or scale when field == NULL. */
typedef struct FemCoef {
  double scale;
  const double* field;
  int64_t stride;   /* 0 or 1: field[e]; > 1: field[e * stride], a (nelems, stride)
                       per-point array whose rows the local kernels of
                       fem_assemble check are constant (FEM_ERR_VARYING in the
                       status word otherwise) */
} FemCoef;

/*
 * Bilinear forms the kernels evaluate (integrand, summed over terms whose
 * coefficient scale is nonzero):
 *   scalar bases:  diff * dot(grad u, grad v) + mass * u * v
 *   vector bases:  lam  * div u * div v                       (a_{bk,al} = d_bk d_al)
 *                + lap  * ddot(grad u, grad v)                (d_ab d_kl)
 *                + tr   * ddot(grad u, transpose(grad v))     (d_bl d_ka)
 *                + mass * dot(u, v)
 * linear_elasticity(L, M) (skfem/models/elasticity.py:44-53) is
 * lam = L, lap = M, tr = M.
 */
typedef struct FemBilinear {
  FemCoef diff, mass;
  FemCoef lam, lap, tr;
} FemBilinear;

/* Linear form: load * v (scalar) or dot(load_vec, v) with load_vec = (load, load, ...) off. */
typedef struct FemLinear {
  FemCoef load;
} FemLinear;

/*
 * The form as a straight-line program in the reference's own operation
 * order, for the exact-zero mask of the pattern build (see
 * fem_pattern_build).  Instruction k computes register k:
 *   op 0 CONST imm | 1 U a (trial quantity a) | 2 V a (test quantity a) |
 *   3 COEF a (coefficient slot a at the point) | 4 ADD a b | 5 SUB a b |
 *   6 MUL a b | 7 DIV a b | 8 NEG a | 9 X a (global coordinate a at the
 *   point, MappingAffine.F / MappingIsoparametric.F arithmetic) | 10 H (mesh
 *   parameter |detDF|**(1/dim)) | 11 SQRT a | 12 EXP a | 13 LOG a | 14 SIN a |
 *   15 COS a | 16 TAN a | 17 TANH a | 18 ARCTAN a | 19 ABS a | 20 POW a b |
 *   21 N a (component a of the unit outward normal, facet programs).
 *   Operands a, b of arithmetic ops name earlier instructions.  Ops 12-18 and
 *   20 use the CUDA math library (last-bit differences from numpy possible);
 *   all others are correctly rounded and reproduce the reference bit for bit.
 * Quantity c is the value of component c, ncomp + c*dim + k the derivative
 * k of component c (ncomp = dim for vector bases, 1 for scalar ones).
 */
typedef struct FemInstr {
  int32_t op, a, b, pad_;
  double imm;
} FemInstr;

typedef struct FemProgram {
  int32_t ninstr;         /* <= 512 */
  int32_t out;            /* register holding the integrand */
  int32_t ncoef;          /* <= 16 */
  int32_t nq;             /* quadrature points of the basis (<= 128) */
  const FemInstr* ins;    /* device array of ninstr instructions */
  const double* coef[16]; /* coefficient slots (device): one value per element
                             (stride 0) or per quadrature point (stride nq) */
  int32_t coef_stride[16];
  const double* qX;       /* the basis's reference points (dim, nq), device; */
  const double* qW;       /* and weights (nq); required by fem_program_*     */
  const struct FemCompiled* compiled;  /* optional: this program compiled by
                                          fem_program_compile (same dim, mode,
                                          facet use); null: interpreted */
} FemProgram;

/*
 * Compile a form program (ins: HOST array of ninstr instructions, as traced)
 * into a kernel for dim, the test (vector) and trial (vector_u) bases' vector
 * flags, mode (0 local matrices, 1 local vectors, 2 per-cell values) and
 * facet (0 cells, 1 FacetBasis facets): NVRTC, sm_103a,
 * -fmad=false, the program as straight-line code -- the interpreter's
 * operations in the same order, so results are bitwise the interpreter's.
 * Returns FEM_ERR_UNSUPPORTED when libnvrtc is unavailable.  Release with
 * fem_program_release.
 */
typedef struct FemCompiled FemCompiled;
int fem_program_compile(const FemInstr* ins, int32_t ninstr, int32_t out, int32_t ncoef,
                        int32_t dim, int32_t vector, int32_t vector_u, int32_t mode,
                        int32_t facet, FemCompiled** compiled);
void fem_program_release(FemCompiled* compiled);
/* The complete source fem_program_compile compiles for these arguments (its
 * headers: fem_faithful_core.cuh, fem_program_kernel.cuh and this file, by
 * name); *needed receives its length + 1.  Host-only, no GPU needed. */
int fem_program_source(const FemInstr* ins, int32_t ninstr, int32_t out, int32_t ncoef,
                       int32_t dim, int32_t vector, int32_t vector_u, int32_t mode, int32_t facet,
                       char* buf, int64_t size, int64_t* needed);

/* Opaque one-time structure: row incidence, CSR pattern, local-to-slot map. */
typedef struct FemPattern FemPattern;
typedef struct FemBatchPlan FemBatchPlan;

/* Last error message of the calling thread ("" if none). */
const char* fem_last_error(void);

/* Library version string. */
const char* fem_version(void);

/*
 * Launch parameters of one element family, set by the autotuner
 * (skfem_gb300.autotune): cells per CTA of the local kernel (64, 128, 256),
 * persistent grid (0: one CTA per tile; k > 0: at most k CTAs per SM,
 * grid-stride), incidence entries loaded together by the segmented sum
 * (4, 8, 16) and columns per lane of the fused sum (1, or 2 for bases
 * with 4, 6 or 10 local functions: each lane then takes two columns of an
 * incidence entry).  This table is the library's one piece of process-wide
 * configuration besides the thread-local error message: one entry per
 * family, written by this call (normally once, at set-up) and read under a
 * lock when a later call launches its kernels.  It chooses launch shapes
 * only -- every setting gives the same values bit for bit -- so calls that
 * race with a retune still return the same results; a caller that needs
 * fixed launch shapes per pattern sets the table once before its first
 * assembly.
 */
int fem_set_tuning(int family, int local_block, int persistent, int sum_unroll, int sum_cols);

/*
 * The one-pass TriP1 / TetP1 sum's variant, in the same table: 0 two lanes
 * per CSR row adding (cell, local row) contributions into shared-memory
 * slots; 1 (the default) one lane per CSR entry on or above the diagonal
 * walking that entry's contribution list in registers and writing the
 * entry and its transpose; 2 variant 1 with each warp's next list codes
 * brought into shared memory by the TMA bulk-copy engine (double-buffered
 * on mbarriers; used when the call passes a status word, which receives
 * FEM_ERR_TIMEOUT if a bounded wait runs out).  All add every entry's
 * contributions in the same order: the values are the same bit for bit
 * (up to the fixed-point mass sums' truncation on meshes whose cells around
 * a vertex differ in size by more than a factor 8, a few ulps).
 * For ElementVector bases of the same families (vector channel forms):
 * 0 the two-pass path (local matrices into the staging, then the
 * segmented sum); 1 (the default) the one-pass vector sum, one lane per
 * D x D node block of the CSR accumulating its cells' reference-tensor
 * terms from their pair blocks (computed into the staging first); 2 the
 * same with the D*D lanes of a block cooperating on its entries.  Variants
 * 1 and 2 are bitwise equal; the two-pass path agrees within 1e-14 of
 * max|K|.
 * For scalar TriP2 / TetP2 bases (k dot(grad u, grad v) + m u v): 0 the
 * two-pass path; 1 (the default) the same one-pass sum with 1 x 1 blocks,
 * one lane per CSR entry on or above the diagonal (per cell the scaled
 * Gram entries times k, and the mass scale, computed into the staging
 * first); 2 the same with one FMA per step of the lane's loop.  Variants
 * 1 and 2 are bitwise equal; the two-pass path agrees within 1e-14 of
 * max|K|.
 */
int fem_set_onepass(int family, int variant);

/*
 * The local-matrix kernel of the scalar simplex families on the pattern's
 * geometry cache (the two-pass path), in the same table: on = 1 brings each
 * tile's geometry -- a (cache entries) x (cells per block) box of the SoA
 * cache -- into shared memory with one 2-D TMA tensor copy
 * (cp.async.bulk.tensor) instead of per-thread coalesced loads.  Used when
 * the call passes a status word (FEM_ERR_TIMEOUT if its bounded wait runs
 * out), without a cell list, on a mesh with an even number of cells (the
 * tensor map's row stride); otherwise the loads.  Same values bit for bit.
 */
int fem_set_local_tma(int family, int on);

/*
 * Local (element) matrices: local[(e * nbfun + i) * nbfun + j] = K_e[i][j],
 * i = test function (row), j = trial function (column), the same entry as
 * the reference's data[j, i, e] (bilinear_form.py:90-98).
 */
int fem_local_matrices(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                       double* local, fem_stream_t stream);

/* Local load vectors: local[e * nbfun + i] (linear_form.py:40-44). */
int fem_local_vectors(const FemMesh* mesh, const FemBasis* basis, const FemLinear* form,
                      double* local, fem_stream_t stream);

/*
 * One-time pattern build (replaces coo_matrix(...).eliminate_zeros().tocsr(),
 * coo_data.py:34-36).  The local matrices of `form` are evaluated once with
 * separately rounded products and sums (no fused multiply-add, as numpy
 * evaluates the reference's forms); local entries that come out exactly
 * +-0.0 create no CSR entry, as eliminate_zeros drops them before the
 * duplicates are summed.  With `program` (may be NULL), the entries whose
 * value is rounding noise of a mathematically-zero integral -- below 1e-9
 * of their element's largest entry -- are re-evaluated with the reference's
 * exact sequence of operations (its quadrature nodes, basis expressions,
 * mapping formulas, the form's operation order, numpy's pairwise sum), so
 * that the pattern keeps exactly the entries the reference keeps.  The
 * pattern also records which per-element
 * coefficients were exactly zero, so that fem_assemble can report when the
 * zero structure changes.  form == NULL builds only the row incidence
 * (enough for load vectors).  Synchronises `stream`.
 */
int fem_pattern_build(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                      const FemProgram* program, FemPattern** out, fem_stream_t stream);

/*
 * Per-cell geometry cache (CellBasis keeps its mapping the same way,
 * cell_basis.py:101-105): for scalar TriP1/P2 and TetP1/P2 bases, the
 * coefficient-free part of the local kernel -- the Gram matrix of the
 * barycentric gradients scaled by 1/(d! |det DF|), and |det DF|: 7 (2D) or
 * 11 (3D) doubles per cell -- computed from mesh->p and kept in the pattern.
 * fem_assemble, fem_assemble_local and fem_assemble_to_host_pipelined then
 * read it instead of the coordinates whenever the mesh they are given has
 * the same p pointer; after changing the coordinates in place, call this
 * again (or fem_pattern_drop_geometry).  For scalar TriP1 / TetP1 bases the
 * call also records, per row, the binary point of the one-pass assembly's
 * fixed-point mass sums (from the cells' |det|, 2 bytes per row): with it
 * fem_assemble and fem_assemble_to_host_pipelined assemble
 * k_e dot(grad u, grad v) + m u v in one pass over the rows, contracting
 * the form per cell row from the cached geometry as they sum.  When the
 * pattern holds a coefficient-update cache (below) the call refreshes it.
 * Other families, or no device memory left for a cache: that cache is
 * left out, returns 0 (the kernels then compute the geometry per call, or
 * run the local kernel and the staging sum).
 * Stream-ordered; not concurrently with assembly calls on the pattern.
 */
int fem_pattern_cache_geometry(FemPattern* pat, const FemMesh* mesh, const FemBasis* basis,
                               fem_stream_t stream);
void fem_pattern_drop_geometry(FemPattern* pat);

/*
 * Opt-in coefficient-update cache of a scalar simplex pattern -- no
 * counterpart in the reference, which contracts the form on every call.
 * For callers that re-assemble one form with new per-cell stiffness
 * coefficients many times (optimisation loops): every cell's
 * unit-coefficient stiffness rows in the sum's incidence order (nelems *
 * nbfun^2 doubles) and the CSR values of the unit-coefficient mass matrix
 * (nnz doubles); fem_assemble then takes forms whose mass coefficient is
 * one constant as diff * sum_e k_e S_e + mass * M in one fused sum.  Needs
 * the pattern's geometry cache of this mesh's coordinates; refreshed with
 * it; fem_pattern_drop_coefficient_update releases it.  No room: returns 0
 * without the cache.
 */
int fem_pattern_cache_coefficient_update(FemPattern* pat, const FemMesh* mesh,
                                         const FemBasis* basis, fem_stream_t stream);
void fem_pattern_drop_coefficient_update(FemPattern* pat);

/* Sizes: nnz of the CSR pattern, number of rows (N), and the bytes of the
 * local-matrix staging buffer fem_assemble needs.  The staging holds the
 * local matrices cell after cell in the pattern's layout: full for scalar
 * bases; for vector bases (symmetric channel forms) only the dim x dim
 * blocks on and above the block diagonal are written, and the sums of
 * fem_assemble, fem_csr_sum_staged, fem_csr_sum_to_host and
 * fem_assemble_to_host_pipelined read the others at their transposed
 * positions.  fem_local_matrices always writes full matrices, and
 * fem_csr_sum takes full matrices. */
int fem_pattern_info(const FemPattern* pat, int64_t* nnz, int64_t* nrows, int64_t* staging_bytes);

/* Copy the CSR structure out: indptr (nrows+1), indices (nnz), both int32. */
int fem_pattern_export(const FemPattern* pat, int32_t* indptr, int32_t* indices, fem_stream_t stream);

void fem_pattern_destroy(FemPattern* pat);

/*
 * Steady-state assembly into an existing pattern: local matrices into
 * `staging` (fem_pattern_info bytes), then a fixed-order, atomic-free
 * segmented sum into csr_values (nnz).  Scalar TriP1 / TetP1 bases whose
 * pattern holds the geometry cache of this mesh's coordinates
 * (fem_pattern_cache_geometry) take one pass instead: the coefficient
 * checks, then each CSR row sums k_e * G_e[il][j] (FP64, ascending cell
 * order) and |det_e| (exact fixed point, or m_e |det_e| in FP64 for a
 * per-cell mass field) over its cells straight from the cached geometry
 * (staging untouched).  When the pattern holds a coefficient-update cache
 * (fem_pattern_cache_coefficient_update) and the form's mass coefficient
 * is one constant, one fused sum diff * sum_e k_e S_e + mass * M runs
 * instead.  Both group the additions differently from the two-pass path,
 * so the values may differ from its in the last bits (within 1e-14 of
 * max|K|), and are bitwise the same on every call and through
 * fem_assemble_to_host_pipelined.  status (device int32, may be NULL)
 * receives FEM_ERR_STALE_PATTERN when the exact-zero structure of the local
 * matrices may have changed: some per-element coefficient became exactly
 * zero or stopped being zero since the pattern was built.  The caller then
 * rebuilds the pattern and assembles again.
 */
int fem_assemble(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                 const FemPattern* pat, double* staging, double* csr_values, int32_t* status,
                 fem_stream_t stream);

/*
 * fem_assemble without any device allocation or scratch argument -- no
 * counterpart in the reference.  For callers that can pass inputs and
 * outputs but cannot allocate GPU memory (a framework that owns the
 * device's memory behind its own allocator, or an application that forbids
 * allocations after start-up).  The local-matrix staging lives in a 64 MiB
 * file-scope device array that every GPU loading the library keeps until
 * exit; meshes needing more (nelems * nbfun^2 * 8 bytes: TetP1 up to
 * 524,288 cells) are rejected with FEM_ERR_CAPACITY.  The first call on a
 * device loads the module holding the array (CUDA's lazy loading: that is
 * when the 64 MiB are taken) and looks up its device address for the
 * runtime's primary context; a caller whose allocator reserves the device's
 * memory makes one warm-up call at start-up, before that reservation and
 * before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race.  Arguments are checked as fem_assemble checks them; status
 * (may be NULL) receives the same coefficient checks, and with NULL none
 * runs (a stale pattern then goes unreported).
 */
int fem_assemble_noalloc(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                         const FemPattern* pat, double* csr_values, int32_t* status,
                         fem_stream_t stream);

/* Segmented sum only (local matrices already in `local`). */
/*
 * fem_assemble with the result streamed to the host: the local kernel, then
 * the segmented sum in nchunks row ranges of about equal nnz, each range's
 * values copied into host_values (pinned host memory, nnz doubles) on
 * copy_stream as soon as it is summed, overlapping the copy with the next
 * range's sum.  csr_values is the device buffer the sum writes first.  The
 * caller synchronises copy_stream (and reads status) before using
 * host_values.
 */
int fem_assemble_to_host(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                         const FemPattern* pat, double* staging, double* csr_values,
                         double* host_values, int32_t* status, int32_t nchunks,
                         fem_stream_t stream, fem_stream_t copy_stream);

/* The two halves of fem_assemble_to_host, for callers that pipeline the
 * coefficients' upload with the local kernel: local matrices of the cells
 * [cell_begin, cell_end) into staging in the pattern's layout (with the
 * coefficient and stale-pattern checks of fem_assemble), then the
 * row-range sum streamed to host_values. */
int fem_assemble_local(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                       const FemPattern* pat, double* staging, int32_t* status, int64_t cell_begin,
                       int64_t cell_end, fem_stream_t stream);
int fem_csr_sum_to_host(const FemPattern* pat, const double* staging, double* csr_values,
                        double* host_values, int32_t nchunks, fem_stream_t stream,
                        fem_stream_t copy_stream);

/* Rows of one strided host coefficient: row e (max(stride, 1) doubles) at
 * host + e * stride, copied to dev + e * stride. */
typedef struct FemHostRows {
  const double* host; /* pageable host memory */
  double* dev;
  int64_t stride;
} FemHostRows;

/* *supported = 1 when kernels on the current device can read pageable host
 * memory (cudaDevAttrPageableMemoryAccess) -- the condition for passing
 * host rows to fem_assemble_to_host_pipelined. */
int fem_host_memory_access(int32_t* supported);

/*
 * fem_assemble_to_host pipelined by data dependence.  The cells are taken
 * in order of their smallest DOF, in nchunks chunks of about equal size;
 * once every cell whose smallest DOF is below m has its local matrix, the
 * rows [0, m) are final.  Per chunk: the host rows of its cells' strided
 * coefficients (nfields of them, 0..16) are copied to their device arrays
 * on upload_stream by a kernel that reads the host memory directly; the
 * chunk's local kernel runs on stream after them; the rows it completes
 * are summed and their values copied to host_values (pinned, nnz doubles)
 * on copy_stream behind the sum.  The upload, the local kernels and the
 * copy of the values back overlap on any mesh, and the call returns
 * without waiting for any of it (the caller synchronises copy_stream and
 * reads status).  Results are the same, bit for bit, as fem_assemble.
 * The cell order and the chunks' row bounds are computed once per pattern
 * and chunk count (synchronous, on first use).  Host rows need
 * fem_host_memory_access (FEM_ERR_UNSUPPORTED otherwise).
 */
int fem_assemble_to_host_pipelined(const FemMesh* mesh, const FemBasis* basis,
                                   const FemBilinear* form, const FemPattern* pat,
                                   double* staging, double* csr_values, double* host_values,
                                   int32_t* status, const FemHostRows* rows, int32_t nfields,
                                   int32_t nchunks, fem_stream_t stream,
                                   fem_stream_t upload_stream, fem_stream_t copy_stream);

/* Segmented sum of full local matrices, cell after cell (nelems x nbfun x
 * nbfun, e.g. from fem_local_matrices), into CSR values. */
int fem_csr_sum(const FemPattern* pat, const double* local, double* csr_values, int32_t* status,
                fem_stream_t stream);
/* The two-pass sum: staging as fem_assemble_local wrote it, in the
 * pattern's layout, into CSR values on the device (fem_assemble's sum when
 * it does not take the fused path). */
int fem_csr_sum_staged(const FemPattern* pat, const double* staging, double* csr_values,
                       fem_stream_t stream);

/* Load vector b (nrows) from local vectors (incidence order, no atomics). */
int fem_vector_sum(const FemPattern* pat, const double* local, double* b, fem_stream_t stream);

/* Load vector end to end: local vectors into staging (nelems*nbfun doubles) then b. */
int fem_assemble_vector(const FemMesh* mesh, const FemBasis* basis, const FemLinear* form,
                        const FemPattern* pat, double* staging, double* b, fem_stream_t stream);

/*
 * Adjoint (no counterpart in the reference, which differentiates only with
 * respect to the solution field, skfem/autodiff/__init__.py:124-213).
 * For J = w^T K(coef, X) u with K from a bilinear form whose terms are
 * linear in per-element fields:
 *   dcoef_diff[e] = d J / d field_diff[e]  (may be NULL), likewise dcoef_mass,
 *   dX (dim, nverts) = d J / d p            (may be NULL), accumulated per
 *   vertex in a fixed order (no atomics).
 * Geometry is recomputed in the adjoint; nothing per quadrature point is stored.
 * elem_scratch: nelems * nloc * dim doubles (per-element vertex gradients).
 */
int fem_bilinear_vjp(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                     const FemPattern* vertex_incidence, const double* w, const double* u,
                     double* dcoef_diff, double* dcoef_mass, double* dX, double* elem_scratch,
                     fem_stream_t stream);

/* J = w^T b(coef, X): dload[e] and dX (same conventions). */
int fem_linear_vjp(const FemMesh* mesh, const FemBasis* basis, const FemLinear* form,
                   const FemPattern* vertex_incidence, const double* w, double* dload, double* dX,
                   double* elem_scratch, fem_stream_t stream);

/*
 * Dirichlet condensation of a device CSR matrix (skfem/utils.py:462-600,
 * condense): A_II = A[I][:, I] and b_I = b[I] - A[I][:, D] x[D].  map[r] is
 * the position of DOF r among the kept DOFs I (ascending) or -1.  Phase 1
 * writes out_indptr (nkeep+1) and *out_nnz (synchronises `stream`);
 * phase 2 fills indices, values and, when out_b is given, the right-hand
 * side (b and x may be NULL: zero).
 */
/* enforce (skfem/utils.py:327-400) on a device CSR, in place: rows[0..nd)
 * (sorted, unique, < nrows) are zeroed with diag on their diagonal -- the
 * entries stay in the pattern as stored zeros, as scipy keeps them -- and,
 * if b is given, b[r] = x[r] (0 without x).  *missing (device) is
 * incremented for every such row that has no diagonal entry. */
int fem_enforce(const int32_t* indptr, const int32_t* indices, double* vals, int64_t nrows,
                const int32_t* rows, int64_t nd, double diag, double* b, const double* x,
                int32_t* missing, fem_stream_t stream);

int fem_condense_pattern(const int32_t* indptr, const int32_t* indices, int64_t nrows,
                         const int32_t* map, int64_t nkeep, int32_t* out_indptr, int64_t* out_nnz,
                         fem_stream_t stream);
int fem_condense_values(const int32_t* indptr, const int32_t* indices, const double* vals,
                        int64_t nrows, const int32_t* map, const double* b, const double* x,
                        const int32_t* out_indptr, int32_t* out_indices, double* out_vals,
                        double* out_b, fem_stream_t stream);

/*
 * Generic forms.  Any form the tracer records as a FemProgram -- anisotropic
 * or advection-type terms, coefficients varying inside cells, interpolated
 * DOF-vector coefficients, quadrature-point coordinates -- is evaluated per
 * quadrature point with the reference's own arithmetic (the replay of
 * fem_pattern_build): the local entries are the reference's bit for bit.
 * fem_program_local_matrices: local[(e*nbfun + i)*nbfun + j] (test i, trial j);
 * fem_program_local_vectors: local[e*nbfun + i] (linear forms: trial-free program);
 * fem_program_elemental: out[e] = integral over element e (Functional).
 */
int fem_program_local_matrices(const FemMesh* mesh, const FemBasis* basis,
                               const FemProgram* program, double* local, int32_t* status,
                               fem_stream_t stream);
/* Local matrices of a bilinear form with different trial (ubasis) and test
 * (vbasis) bases on the same cells and points (BilinearForm.assemble(ubasis,
 * vbasis), bilinear_form.py:58-128): local[(e*nv + i)*nu + j]. */
int fem_program_local_matrices_mixed(const FemMesh* mesh, const FemBasis* vbasis,
                                     const FemBasis* ubasis, const FemProgram* program,
                                     double* local, int32_t* status, fem_stream_t stream);
/* Pattern of the (ndofs_v x ndofs_u) matrix of such local matrices. */
int fem_pattern_build_local_mixed(const FemMesh* mesh, const FemBasis* vbasis,
                                  const FemBasis* ubasis, const double* local, FemPattern** out,
                                  fem_stream_t stream);

/*
 * CSR pattern of a general COO matrix (replaces COOData._assemble_scipy_csr,
 * coo_data.py:27-36, for COOData built or combined by the caller): n
 * entries (rows[k], cols[k], data[k]) of an nrows x ncols matrix; entries
 * whose value is exactly +-0.0 create no CSR entry (eliminate_zeros), the
 * others are summed per (row, column) by fem_csr_sum(pat, data, values)
 * in ascending entry order.  Rows outside [0, nrows) or columns outside
 * [0, ncols) are refused (FEM_ERR_ARGUMENT); a row gathering more than
 * 8,192 entries returns FEM_ERR_CAPACITY.  The pattern is released with
 * fem_pattern_destroy.
 */
int fem_coo_pattern_build(const int32_t* rows, const int32_t* cols, const double* data,
                          int64_t n, int64_t nrows, int64_t ncols, FemPattern** out,
                          fem_stream_t stream);
int fem_program_local_vectors(const FemMesh* mesh, const FemBasis* basis,
                              const FemProgram* program, double* local, int32_t* status,
                              fem_stream_t stream);
int fem_program_elemental(const FemMesh* mesh, const FemBasis* basis, const FemProgram* program,
                          double* out, int32_t* status, fem_stream_t stream);

/* Pattern (incidence + CSR + slot map) whose eliminate_zeros mask is the
 * given local matrices' exact zeros (local from fem_program_local_matrices). */
int fem_pattern_build_local(const FemMesh* mesh, const FemBasis* basis, const double* local,
                            FemPattern** out, fem_stream_t stream);

/* Segmented sum that also verifies the zero structure: status receives
 * FEM_ERR_STALE_PATTERN if a nonzero local entry has no CSR slot or a CSR
 * entry has no nonzero contribution (exact zero masks, generic forms). */
int fem_csr_sum_checked(const FemPattern* pat, const double* local, double* csr_values,
                        int32_t* status, fem_stream_t stream);

/*
 * Basis.interpolate (skfem/assembly/basis/abstract_basis.py:271-322): the
 * DOF vector w (device, ndofs) at the nq reference points X (device, (dim,
 * nq)) of every element, with the reference's arithmetic (sum over local
 * functions in order).  out (device) holds nquant x nelems x nq doubles,
 * quantity-major: scalar bases value, d/dx_0 .. d/dx_{dim-1} (nquant =
 * 1 + dim); vector bases the dim components, then grad[c][k] at
 * dim + c*dim + k (nquant = dim + dim*dim).
 */
int fem_interpolate(const FemMesh* mesh, const FemBasis* basis, int32_t nq, const double* X,
                    const double* w, double* out, fem_stream_t stream);

/* np.sum of a contiguous device vector of n doubles in numpy's pairwise
 * order (leaves of <= 128 values, split at n/2 rounded down to a multiple
 * of 8); *out (device) receives the sum (Functional.assemble). */
int fem_sum_pairwise(const double* x, int64_t n, double* out, fem_stream_t stream);

/*
 * FacetBasis (skfem/assembly/basis/facet_basis.py:21-110) on affine simplex
 * meshes: the facets integrated over, each with the cell whose basis is
 * traced (f2t[side]) and the cell that orients the normal (f2t[0]).  The
 * program's qX / qW are the facet rule (dim-1, nq); its X / H / N ops read
 * the facet point's coordinates, |detDG|**(1/(dim-1)) and the unit outward
 * normal.  Outputs are per facet, laid out as the cell versions'.
 */
typedef struct FemFacets {
  int64_t nfacets;
  const int32_t* fverts;    /* (nfv, nfacets): the facets' vertices (Mesh.facets columns);
                               nfv = dim for simplices, 4 for Hex1 quadrilaterals */
  const int32_t* tind;      /* (nfacets) */
  const int32_t* tind_n;    /* (nfacets) */
  const int32_t* lfacet_n;  /* (nfacets): row of t2f holding the facet in tind_n */
  const double* geo;        /* Hex1: (nfacets, nq, 20) point geometry from
                               fem_facet_geometry; null for simplices */
} FemFacets;

/*
 * Hex1 FacetBasis geometry, once per basis: facet map G and detDG of the
 * bilinear quadrilateral facet (ElementQuad1 node sums, mapping_isoparametric.py
 * :60-110, 137-155), the cells' reference points by the reference's Newton
 * iteration invF (:157-168: X = 0.5, dX = invDF (x - F(X)), X = clip(X + dX,
 * 0, 1), stopped at the first iteration at which every facet's max over
 * points of sum |dX_i| is below 1e-12 -- a count common to all facets, found
 * by a first pass), and the normals invDF(Y0)^T N_ref / |.| of the cells
 * f2t[0].  geo (device, nfacets * nq * 20 doubles) per point: invDF (9,
 * row-major), detDG, x (3), h, n (3), reference point (3).  status receives
 * 1 << FEM_ERR_NEWTON when the iteration does not converge in 50 steps.
 */
int fem_facet_geometry(const FemMesh* mesh, const FemBasis* basis, const FemFacets* facets,
                       int32_t nq, const double* X, double* geo, int32_t* status,
                       fem_stream_t stream);

int fem_facet_program_local_matrices(const FemMesh* mesh, const FemBasis* basis,
                                     const FemFacets* facets, const FemProgram* program,
                                     double* local, int32_t* status, fem_stream_t stream);
int fem_facet_program_local_vectors(const FemMesh* mesh, const FemBasis* basis,
                                    const FemFacets* facets, const FemProgram* program,
                                    double* local, int32_t* status, fem_stream_t stream);
int fem_facet_program_elemental(const FemMesh* mesh, const FemBasis* basis,
                                const FemFacets* facets, const FemProgram* program, double* out,
                                int32_t* status, fem_stream_t stream);
/* FacetBasis.interpolate: as fem_interpolate at the facet points X (dim-1, nq). */
int fem_facet_interpolate(const FemMesh* mesh, const FemBasis* basis, const FemFacets* facets,
                          int32_t nq, const double* X, const double* w, double* out,
                          fem_stream_t stream);

/* Vertex incidence of the mesh (rows = vertices), used by the adjoint's
 * fixed-order gather of per-element coordinate gradients. */
int fem_vertex_incidence_build(const FemMesh* mesh, FemPattern** out, fem_stream_t stream);

/*
 * Batched assembly in one persistent launch -- no counterpart in the
 * reference, which assembles one mesh per BilinearForm.assemble call
 * (bilinear_form.py:130-148).  The meshes form one block-diagonal union
 * (FemMesh / FemBasis of the union, each mesh's cells, vertices and DOFs
 * offset, its own numbering kept inside its block).
 *
 * fem_batch_plan_build: the device work queue of the union, from the
 * meshes' cell offsets and row (DOF) offsets (nmeshes + 1 each, host
 * arrays): per mesh, units of 128 cells and units of rows_per_unit rows,
 * every mesh's cell units queued before its row units.  Released with
 * fem_batch_plan_destroy; fem_batch_plan_info gives the number of units
 * and of int32 counters a launch needs.
 *
 * fem_batched_assemble_vjp: one launch (after a memset of `counters`,
 * 1 + nmeshes int32) whose blocks take units in queue order from an atomic
 * ticket: a cell unit writes its cells' local matrices (k_e S_e + m_e M_e
 * from the pattern's geometry cache, required) into the staging and, when
 * w and u are given, dJ/dk_e = w_e^T S_e u_e and dJ/dm_e = w_e^T M_e u_e of
 * J = w^T K u (the scales of the form's channels applied) into
 * dcoef_diff / dcoef_mass (either may be NULL); a row unit waits (bounded)
 * until its mesh's cell units are done, then sums its rows in the fixed
 * order of fem_assemble's staging sum -- the CSR values equal the split
 * entry points' (fem_assemble_local + fem_csr_sum_staged) bit for bit for
 * TriP1, TriP2 and TetP1, within a few ulps for TetP2 (whose longer tensor
 * sums the compiler may contract differently).  Scalar simplex bases
 * (TriP1/P2, TetP1/P2)
 * and forms k dot(grad u, grad v) + m u v.  status (device int32)
 * receives the coefficient checks' bits and FEM_ERR_TIMEOUT if a wait ran
 * out.  Capturable in a CUDA graph (memset + kernel).
 * Scalar TriP2 / TetP2 patterns holding the one-pass node-block lists
 * (fem_pattern_cache_geometry builds them), unless fem_set_onepass selects
 * the two-pass path for the family: the launch runs the batched form of
 * fem_assemble's one-pass sum instead -- cell units write each cell's pair
 * values (and the same dJ/dk_e, dJ/dm_e), row-block units (the lists' slots
 * of one block of rows) wait (bounded) for the cell units of every mesh
 * their rows belong to and sum one CSR entry per lane; the CSR values then
 * equal fem_assemble's bit for bit.  Its queue is built from the pattern's
 * lists on the first such call (not during a stream capture: run the call
 * once before capturing it); fem_batch_plan_info then reports its units.
 */
int fem_batch_plan_build(const int64_t* cell_offsets, const int64_t* row_offsets,
                         int32_t nmeshes, int32_t rows_per_unit, FemBatchPlan** out);
void fem_batch_plan_destroy(FemBatchPlan* plan);
int fem_batch_plan_info(const FemBatchPlan* plan, int64_t* nunits, int64_t* ncounters);
int fem_batched_assemble_vjp(const FemMesh* mesh, const FemBasis* basis, const FemBilinear* form,
                             const FemPattern* pat, const FemBatchPlan* plan, double* staging,
                             double* csr_values, const double* w, const double* u,
                             double* dcoef_diff, double* dcoef_mass, int32_t* counters,
                             int32_t* status, fem_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SKFEM_GB300_H */
