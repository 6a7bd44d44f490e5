// jit.h — plan specialiser: generated straight-line pass kernels (NVRTC).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"

namespace tcg {

struct Program;

// Compiled kernels of one program direction (one kernel per pass).
struct JitKernels {
  cudaLibrary_t lib = nullptr;
  std::vector<cudaKernel_t> fn;
  std::vector<size_t> smem;     // dynamic shared memory per pass kernel
  std::vector<int> nthreads;
  std::map<int, bool> attr_set;  // device -> attributes raised
  bool failed = false;
  std::string log;
};

// Source of the specialised kernels of `P` for `mode` (exposed for tests).
std::string jit_source(const Program& P, int mode, int R);

// Compile (or fetch from the cubin cache) and load; returns false if NVRTC is
// unavailable or compilation failed (the caller keeps the generic kernels).
bool jit_build(const Program& P, int mode, int R, JitKernels* out);

cudaError_t jit_launch(JitKernels* jk, int pass, const KParams_Host& kp, uint32_t ntiles, int64_t batch,
                       int n, cudaStream_t st);

// 0: never, 1: always, 2: after a plan direction ran twice (default)
int jit_policy();

}  // namespace tcg
