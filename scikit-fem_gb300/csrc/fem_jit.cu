// Run-time compilation of traced form programs with NVRTC (sm_103a,
// -fmad=false).  The generated source is the generic-form kernel body
// (fem_program_kernel.cuh) with FEM_FORM_EVAL bound to the program written
// out as one statement per instruction -- the same operations in the same
// order as the interpreter, so results are bitwise the interpreter's.
// libnvrtc is opened on first use; without it compilation reports
// FEM_ERR_UNSUPPORTED and callers keep the interpreter.

#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fem_common.cuh"
#include "fem_faithful_core.cuh"
#include "fem_jit.h"

// header texts embedded at build time (generated by skfem_gb300/_build.py)
#include "fem_jit_sources.inc"

namespace {

struct Nvrtc {
  bool tried = false, ok = false;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

std::mutex g_mu;
Nvrtc g_nvrtc;

bool load_nvrtc() {
  if (g_nvrtc.tried) return g_nvrtc.ok;
  g_nvrtc.tried = true;
  const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  void* h = nullptr;
  for (const char* n : names)
    if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) return false;
  g_nvrtc.create = (decltype(g_nvrtc.create))dlsym(h, "nvrtcCreateProgram");
  g_nvrtc.compile = (decltype(g_nvrtc.compile))dlsym(h, "nvrtcCompileProgram");
  g_nvrtc.log_size = (decltype(g_nvrtc.log_size))dlsym(h, "nvrtcGetProgramLogSize");
  g_nvrtc.log = (decltype(g_nvrtc.log))dlsym(h, "nvrtcGetProgramLog");
  g_nvrtc.cubin_size = (decltype(g_nvrtc.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
  g_nvrtc.cubin = (decltype(g_nvrtc.cubin))dlsym(h, "nvrtcGetCUBIN");
  g_nvrtc.destroy = (decltype(g_nvrtc.destroy))dlsym(h, "nvrtcDestroyProgram");
  g_nvrtc.ok = g_nvrtc.create && g_nvrtc.compile && g_nvrtc.log_size && g_nvrtc.log &&
               g_nvrtc.cubin_size && g_nvrtc.cubin && g_nvrtc.destroy;
  return g_nvrtc.ok;
}

std::string dbl(double v) {
  uint64_t bits;
  std::memcpy(&bits, &v, sizeof bits);
  char buf[64];
  std::snprintf(buf, sizeof buf, "__longlong_as_double(0x%016llxLL)", (unsigned long long)bits);
  return buf;
}

// Right-hand side of instruction k.
std::string rhs_of(const FemInstr& I) {
  std::string rhs;
  auto r = [](int i) { return "r" + std::to_string(i); };
  switch (I.op) {
      case fem_faithful::OP_CONST: rhs = dbl(I.imm); break;
      case fem_faithful::OP_U: rhs = "qu[" + std::to_string(I.a) + "]"; break;
      case fem_faithful::OP_V: rhs = "qv[" + std::to_string(I.a) + "]"; break;
      case fem_faithful::OP_COEF: rhs = "cq[" + std::to_string(I.a) + "]"; break;
      case fem_faithful::OP_ADD: rhs = r(I.a) + " + " + r(I.b); break;
      case fem_faithful::OP_SUB: rhs = r(I.a) + " - " + r(I.b); break;
      case fem_faithful::OP_MUL: rhs = r(I.a) + " * " + r(I.b); break;
      case fem_faithful::OP_DIV: rhs = r(I.a) + " / " + r(I.b); break;
      case fem_faithful::OP_NEG: rhs = "-" + r(I.a); break;
      case fem_faithful::OP_X: rhs = "qx[" + std::to_string(I.a) + "]"; break;
      case fem_faithful::OP_H: rhs = "qx[3]"; break;
      case fem_faithful::OP_SQRT: rhs = "sqrt(" + r(I.a) + ")"; break;
      case fem_faithful::OP_EXP: rhs = "exp(" + r(I.a) + ")"; break;
      case fem_faithful::OP_LOG: rhs = "log(" + r(I.a) + ")"; break;
      case fem_faithful::OP_SIN: rhs = "sin(" + r(I.a) + ")"; break;
      case fem_faithful::OP_COS: rhs = "cos(" + r(I.a) + ")"; break;
      case fem_faithful::OP_TAN: rhs = "tan(" + r(I.a) + ")"; break;
      case fem_faithful::OP_TANH: rhs = "tanh(" + r(I.a) + ")"; break;
      case fem_faithful::OP_ARCTAN: rhs = "atan(" + r(I.a) + ")"; break;
      case fem_faithful::OP_ABS: rhs = "fabs(" + r(I.a) + ")"; break;
      case fem_faithful::OP_POW: rhs = "pow(" + r(I.a) + ", " + r(I.b) + ")"; break;
      case fem_faithful::OP_N: rhs = "qx[" + std::to_string(4 + I.a) + "]"; break;
      default: rhs = "0.0";
  }
  return rhs;
}

bool binary(int op) {
  using namespace fem_faithful;
  return op == OP_ADD || op == OP_SUB || op == OP_MUL || op == OP_DIV || op == OP_POW;
}
bool unary(int op) {
  using namespace fem_faithful;
  return op == OP_NEG || op == OP_SQRT || op == OP_EXP || op == OP_LOG || op == OP_SIN ||
         op == OP_COS || op == OP_TAN || op == OP_TANH || op == OP_ARCTAN || op == OP_ABS;
}

// Bilinear programs split four ways by what an instruction depends on: jit_point
// (neither u nor v: once per point, the values needed later in P), jit_u (the
// trial function only: once per point and trial function, into U), jit_v
// (the test function only: once per point and test function, into V) and
// jit_form_uv (the rest, reading P, U and V).  Every instruction keeps its
// operands and so its value, bit for bit; only where it is evaluated moves.
std::string program_source_uv(const FemInstr* ins, int n, int out, int* npoint, int* nuval,
                              int* nvval) {
  std::string s;
  char line[256];
  // dep bit 1: trial quantity, bit 2: test quantity
  std::vector<int> dep(n, 0);
  for (int k = 0; k < n; ++k) {
    const FemInstr& I = ins[k];
    if (I.op == fem_faithful::OP_U) dep[k] = 1;
    else if (I.op == fem_faithful::OP_V) dep[k] = 2;
    else if (binary(I.op)) dep[k] = dep[I.a] | dep[I.b];
    else if (unary(I.op)) dep[k] = dep[I.a];
  }
  // an instruction's value is stored when an instruction of another class
  // (or the output, evaluated in jit_form_uv) reads it
  std::vector<char> need(n, 0);
  auto use = [&](int k, int operand) {
    if (dep[operand] != dep[k]) need[operand] = 1;
  };
  for (int k = 0; k < n; ++k) {
    const FemInstr& I = ins[k];
    if (binary(I.op)) {
      use(k, I.a);
      use(k, I.b);
    } else if (unary(I.op)) {
      use(k, I.a);
    }
  }
  if (dep[out] != 3) need[out] = 1;
  std::vector<int> slot(n, -1);
  int cnt[4] = {0, 0, 0, 0};
  for (int k = 0; k < n; ++k)
    if (need[k]) slot[k] = cnt[dep[k]]++;
  *npoint = cnt[0];
  *nuval = cnt[1];
  *nvval = cnt[2];
  const char* store[3] = {"P", "U", "V"};
  auto operand_load = [&](int k, int cls, std::string& body) {
    // the operands of class-cls instructions that live in another class's slots
    std::vector<char> loaded(n, 0);
    for (int i = 0; i < n; ++i) {
      if (dep[i] != cls) continue;
      const FemInstr& I = ins[i];
      int ops[2] = {-1, -1};
      if (binary(I.op)) {
        ops[0] = I.a;
        ops[1] = I.b;
      } else if (unary(I.op)) {
        ops[0] = I.a;
      }
      for (int o : ops)
        if (o >= 0 && dep[o] != cls && !loaded[o]) {
          loaded[o] = 1;
          std::snprintf(line, sizeof line, "  const double r%d = %s[%d];\n", o, store[dep[o]],
                        slot[o]);
          body += line;
        }
    }
    (void)k;
  };
  auto emit_class = [&](int cls, std::string& body) {
    operand_load(0, cls, body);
    for (int k = 0; k < n; ++k) {
      if (dep[k] != cls) continue;
      std::snprintf(line, sizeof line, "  const double r%d = ", k);
      body += line + rhs_of(ins[k]) + ";\n";
    }
  };
  std::snprintf(line, sizeof line, "#define FEM_JIT_NUVAL %d\n#define FEM_JIT_NVVAL %d\n",
                std::max(1, cnt[1]), std::max(1, cnt[2]));
  s += line;
  s += "__device__ __forceinline__ void jit_point(const double* cq, const double* qx, "
       "double* P) {\n";
  emit_class(0, s);
  for (int k = 0; k < n; ++k)
    if (dep[k] == 0 && slot[k] >= 0) {
      std::snprintf(line, sizeof line, "  P[%d] = r%d;\n", slot[k], k);
      s += line;
    }
  s += "}\n";
  const char* fn[3] = {"", "jit_u(const double* qu, const double* P, double* U)",
                       "jit_v(const double* qv, const double* P, double* V)"};
  for (int cls = 1; cls <= 2; ++cls) {
    s += std::string("__device__ __forceinline__ void ") + fn[cls] + " {\n";
    emit_class(cls, s);
    for (int k = 0; k < n; ++k)
      if (dep[k] == cls && slot[k] >= 0) {
        std::snprintf(line, sizeof line, "  %s[%d] = r%d;\n", store[cls], slot[k], k);
        s += line;
      }
    s += "  (void)P;\n}\n";
  }
  s += "__device__ __forceinline__ double jit_form_uv(const double* P, const double* U, "
       "const double* V) {\n";
  emit_class(3, s);
  if (dep[out] != 3) {
    std::snprintf(line, sizeof line, "  const double r%d = %s[%d];\n", out, store[dep[out]],
                  slot[out]);
    s += line;
  }
  s += "  (void)P; (void)U; (void)V;\n  return r" + std::to_string(out) + ";\n}\n";
  return s;
}

// The program as straight-line code; the caller has validated operands.
// hoist: split it into jit_point (instructions that depend on neither u
// nor v, once per point, their values needed later stored in P) and
// jit_form_hoisted (the rest, reading P); *npoint receives |P|.
std::string program_source(const FemInstr* ins, int n, int out, bool hoist, int* npoint) {
  std::string s;
  char line[256];
  *npoint = 0;
  if (!hoist) {
    s += "__device__ __forceinline__ double jit_form(const double* qu, const double* qv, "
         "const double* cq, const double* qx) {\n";
    for (int k = 0; k < n; ++k) {
      std::snprintf(line, sizeof line, "  const double r%d = ", k);
      s += line + rhs_of(ins[k]) + ";\n";
    }
    s += "  return r" + std::to_string(out) + ";\n}\n";
    return s;
  }
  std::vector<char> dep(n, 0), need(n, 0);
  for (int k = 0; k < n; ++k) {
    const FemInstr& I = ins[k];
    if (I.op == fem_faithful::OP_U || I.op == fem_faithful::OP_V) dep[k] = 1;
    else if (binary(I.op)) dep[k] = dep[I.a] | dep[I.b];
    else if (unary(I.op)) dep[k] = dep[I.a];
  }
  for (int k = 0; k < n; ++k) {
    const FemInstr& I = ins[k];
    if (!dep[k]) continue;
    if (binary(I.op)) {
      if (!dep[I.a]) need[I.a] = 1;
      if (!dep[I.b]) need[I.b] = 1;
    } else if (unary(I.op) && !dep[I.a]) {
      need[I.a] = 1;
    }
  }
  if (!dep[out]) need[out] = 1;
  std::vector<int> slot(n, -1);
  for (int k = 0; k < n; ++k)
    if (need[k]) slot[k] = (*npoint)++;
  s += "__device__ __forceinline__ void jit_point(const double* cq, const double* qx, "
       "double* P) {\n";
  for (int k = 0; k < n; ++k) {
    if (dep[k]) continue;
    std::snprintf(line, sizeof line, "  const double r%d = ", k);
    s += line + rhs_of(ins[k]) + ";\n";
  }
  for (int k = 0; k < n; ++k)
    if (slot[k] >= 0) {
      std::snprintf(line, sizeof line, "  P[%d] = r%d;\n", slot[k], k);
      s += line;
    }
  s += "}\n__device__ __forceinline__ double jit_form_hoisted(const double* qu, "
       "const double* qv, const double* P) {\n";
  for (int k = 0; k < n; ++k) {
    if (slot[k] >= 0) {
      std::snprintf(line, sizeof line, "  const double r%d = P[%d];\n", k, slot[k]);
      s += line;
    } else if (dep[k]) {
      std::snprintf(line, sizeof line, "  const double r%d = ", k);
      s += line + rhs_of(ins[k]) + ";\n";
    }
  }
  s += "  return r" + std::to_string(out) + ";\n}\n";
  return s;
}

// The complete source compiled for a program (headers by name).
int kernel_source(const FemInstr* ins, int ninstr, int out, int ncoef, int dim, int vector,
                  int vector_u, int mode, int facet, std::string& src, int* npoint,
                  int* nuval, int* nvval);

}  // namespace

namespace fem {
int check_instructions(const FemInstr* h, int ninstr, int ncoef, int dim, bool vec);

int jit_launch(const FemCompiled* k, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
               void** args) {
  if (smem > k->smem_limit) {
    FEM_TRY_CUDA(cudaFuncSetAttribute((const void*)k->kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const_cast<FemCompiled*>(k)->smem_limit = smem;
  }
  FEM_TRY_CUDA(cudaLaunchKernel((const void*)k->kernel, grid, block, args, smem, st));
  return 0;
}
}  // namespace fem

namespace {
int kernel_source(const FemInstr* ins, int ninstr, int out, int ncoef, int dim, int vector,
                  int vector_u, int mode, int facet, std::string& src, int* npoint,
                  int* nuval, int* nvval) {
  using fem::set_error;
  *nuval = *nvval = 0;
  if (!ins || (dim != 2 && dim != 3) || mode < 0 || mode > 2 || ninstr <= 0 ||
      ninstr > fem_faithful::kMaxProgram || out < 0 || out >= ninstr || ncoef < 0 ||
      ncoef > fem_faithful::kMaxCoef) {
    set_error(FEM_ERR_ARGUMENT, "form program: invalid arguments");
    return FEM_ERR_ARGUMENT;
  }
  // operand checks (the same as the interpreter's; trial quantities of a
  // vector trial basis may index further)
  if (int rc = fem::check_instructions(ins, ninstr, ncoef, dim, vector != 0 || vector_u != 0))
    return rc;
  src.clear();
  // bilinear and linear forms evaluate each point's u/v-free part once;
  // a functional has one entry per cell and runs the program whole
  const bool hoist = mode != 2;
  if (mode == 0) {
    // bilinear: trial-only and test-only parts once per point and function
    const std::string body = program_source_uv(ins, ninstr, out, npoint, nuval, nvval);
    src += "#define FEM_JIT_HOIST 1\n#define FEM_JIT_HOIST_UV 1\n"
           "#include \"fem_faithful_core.cuh\"\n";
    src += "namespace fem_faithful {\n" + body + "}\n";
    src += "#include \"fem_program_kernel.cuh\"\n";
  } else {
  const std::string body = program_source(ins, ninstr, out, hoist, npoint);
  if (hoist) {
    src += "#define FEM_JIT_HOIST 1\n#include \"fem_faithful_core.cuh\"\n";
    src += "namespace fem_faithful {\n" + body + "}\n";
    src += "#include \"fem_program_kernel.cuh\"\n";
  } else {
    src += "namespace fem_faithful {\n__device__ __forceinline__ double jit_form(const double*, "
           "const double*, const double*, const double*);\n}\n";
    src += "#define FEM_FORM_EVAL(prog, qu, qv, cq, qx, R) jit_form(qu, qv, cq, qx)\n";
    src += "#include \"fem_faithful_core.cuh\"\n#include \"fem_program_kernel.cuh\"\n";
    src += "namespace fem_faithful {\n" + body + "}\n";
  }
  }
  char tail[512];
  std::snprintf(tail, sizeof tail,
                "extern \"C\" __global__ void fem_jit_program(FemMesh m, FemBasis b, FemBasis bu, "
                "FemFacets fc, FemProgram prog, fem_faithful::Rule rule, "
                "fem_faithful::GenericLayout s, int64_t ncells, double* out, int32_t* status) {\n"
                "  fem_faithful::program_body<%d, %d, %s, %s, %s>(m, b, bu, fc, prog, rule, s, "
                "ncells, out, status);\n}\n",
                dim, mode, facet ? "true" : "false", vector ? "true" : "false",
                (mode == 0 ? vector_u : vector) ? "true" : "false");
  src += tail;
  return 0;
}
}  // namespace

extern "C" {

int fem_program_source(const FemInstr* ins, int32_t ninstr, int32_t out, int32_t ncoef,
                       int32_t dim, int32_t vector, int32_t vector_u, int32_t mode, int32_t facet,
                       char* buf, int64_t size, int64_t* needed) {
  std::string src;
  int npoint = 0, nuval = 0, nvval = 0;
  if (int rc = kernel_source(ins, ninstr, out, ncoef, dim, vector, vector_u, mode, facet, src,
                             &npoint, &nuval, &nvval))
    return rc;
  if (needed) *needed = (int64_t)src.size() + 1;
  if (buf && size > 0) {
    const size_t n = std::min<size_t>(src.size(), (size_t)size - 1);
    std::memcpy(buf, src.data(), n);
    buf[n] = '\0';
  }
  return 0;
}

int fem_program_compile(const FemInstr* ins, int32_t ninstr, int32_t out, int32_t ncoef,
                        int32_t dim, int32_t vector, int32_t vector_u, int32_t mode,
                        int32_t facet, FemCompiled** compiled) {
  using fem::set_error;
  if (!compiled) {
    set_error(FEM_ERR_ARGUMENT, "fem_program_compile: null output");
    return FEM_ERR_ARGUMENT;
  }
  *compiled = nullptr;
  std::string src;
  int npoint = 0, nuval = 0, nvval = 0;
  if (int rc = kernel_source(ins, ninstr, out, ncoef, dim, vector, vector_u, mode, facet, src,
                             &npoint, &nuval, &nvval))
    return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!load_nvrtc()) {
    set_error(FEM_ERR_UNSUPPORTED, "libnvrtc is not available: programs are interpreted");
    return FEM_ERR_UNSUPPORTED;
  }
  const char* hdr_src[] = {kJitCoreSrc, kJitKernelSrc, kJitAbiSrc};
  const char* hdr_names[] = {"fem_faithful_core.cuh", "fem_program_kernel.cuh",
                             "../../include/skfem_gb300.h"};
  nvrtcProgram prog;
  if (g_nvrtc.create(&prog, src.c_str(), "fem_jit_program.cu", 3, hdr_src, hdr_names) !=
      NVRTC_SUCCESS) {
    set_error(FEM_ERR_UNSUPPORTED, "nvrtcCreateProgram failed");
    return FEM_ERR_UNSUPPORTED;
  }
  // -default-device: the ABI header's prototypes become (unused) device declarations
  const char* opts[] = {"--gpu-architecture=sm_103a", "-fmad=false", "--std=c++17",
                        "-default-device"};
  const nvrtcResult cr = g_nvrtc.compile(prog, 4, opts);
  if (cr != NVRTC_SUCCESS) {
    size_t n = 0;
    g_nvrtc.log_size(prog, &n);
    std::string log(n, '\0');
    g_nvrtc.log(prog, &log[0]);
    g_nvrtc.destroy(&prog);
    set_error(FEM_ERR_UNSUPPORTED, "form program compilation failed: %.900s", log.c_str());
    return FEM_ERR_UNSUPPORTED;
  }
  size_t nb = 0;
  g_nvrtc.cubin_size(prog, &nb);
  std::vector<char> cubin(nb);
  g_nvrtc.cubin(prog, cubin.data());
  g_nvrtc.destroy(&prog);
  FemCompiled* k = new FemCompiled();
  k->dim = dim;
  k->mode = mode;
  k->facet = facet ? 1 : 0;
  k->npoint = npoint;
  k->nuval = mode == 0 ? nuval : 0;
  k->nvval = mode == 0 ? nvval : 0;
  k->uv = mode == 0;
  k->vector_u = mode == 0 ? (vector_u ? 1 : 0) : (vector ? 1 : 0);
  cudaError_t e = cudaLibraryLoadData(&k->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&k->kernel, k->lib, "fem_jit_program");
  if (e != cudaSuccess) {
    if (k->lib) cudaLibraryUnload(k->lib);
    delete k;
    return fem::check_cuda(e, "loading the compiled form program");
  }
  *compiled = k;
  return 0;
}

void fem_program_release(FemCompiled* compiled) {
  if (!compiled) return;
  if (compiled->lib) cudaLibraryUnload(compiled->lib);
  delete compiled;
}

}  // extern "C"
