// swap_prof.h -- RAII scope that brackets one launcher call (kernels: how
// many kernels it launches) with CUDA events on the launching stream when
// profiling is enabled on the context.
#pragma once

#include <cuda_runtime.h>

struct swap_ctx;

class ProfScope {
 public:
  ProfScope(swap_ctx* c, const char* name, cudaStream_t st, int kernels = 1);
  ~ProfScope();
  ProfScope(const ProfScope&) = delete;
  ProfScope& operator=(const ProfScope&) = delete;

 private:
  swap_ctx* c_;
  cudaStream_t st_;
  int idx_ = -1;
  int kernels_ = 1;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
};

void swap_prof_collect(swap_ctx* c);
