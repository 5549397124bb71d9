// Run-time compiled form programs (fem_jit.cu): the traced program as
// straight-line CUDA inside the generic-form kernel body, so that its
// registers live in registers instead of the interpreter's local-memory file.
#pragma once

#include <cuda_runtime.h>

#include "../../include/skfem_gb300.h"

struct FemCompiled {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
  int dim = 0, mode = 0, facet = 0;
  int npoint = 0;                  // per-point hoisted values (GenericLayout::npoint)
  int uv = 0;                      // bilinear: trial-only / test-only values hoisted
  int nuval = 0, nvval = 0;        // ... per point and function (GenericLayout::nuval/nvval)
  int vector_u = 0;                // the trial basis's vector flag (bilinear forms)
  size_t smem_limit = 48 * 1024;   // dynamic shared memory the kernel is enabled for
};

namespace fem {
// Launch a compiled program kernel with program_kernel's arguments.
int jit_launch(const FemCompiled* k, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
               void** args);
}  // namespace fem
