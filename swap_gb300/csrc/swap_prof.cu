// swap_prof.cu -- per-kernel CUDA-event timing for the fused paths.
#include "swap_ctx.h"
#include "swap_prof.h"

void swap_ctx::prof_free() {
  for (auto& p : prof_pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  prof_pending.clear();
  for (cudaEvent_t e : prof_pool) cudaEventDestroy(e);
  prof_pool.clear();
}

static cudaEvent_t take_event(swap_ctx* c) {
  if (!c->prof_pool.empty()) {
    cudaEvent_t e = c->prof_pool.back();
    c->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(swap_ctx* c, const char* name, cudaStream_t st, int kernels)
    : c_(c), st_(st), kernels_(kernels) {
  if (!c_ || !c_->prof_on) {
    c_ = nullptr;
    return;
  }
  idx_ = -1;
  for (std::size_t i = 0; i < c_->prof.size(); ++i)
    if (c_->prof[i].name == name) idx_ = (int)i;
  if (idx_ < 0) {
    c_->prof.push_back(ProfEntry{name, 0.0, 0});
    idx_ = (int)c_->prof.size() - 1;
  }
  a_ = take_event(c_);
  b_ = take_event(c_);
  cudaEventRecord(a_, st_);
}

ProfScope::~ProfScope() {
  if (!c_) return;
  cudaEventRecord(b_, st_);
  c_->prof_pending.push_back({idx_, kernels_, a_, b_});
  if (c_->prof_pending.size() > 4096) swap_prof_collect(c_);
}

void swap_prof_collect(swap_ctx* c) {
  for (auto& p : c->prof_pending) {
    cudaEventSynchronize(p.b);
    float ms = 0;
    cudaEventElapsedTime(&ms, p.a, p.b);
    c->prof[(std::size_t)p.idx].ms += ms;
    c->prof[(std::size_t)p.idx].launches += p.kernels;
    c->prof_pool.push_back(p.a);
    c->prof_pool.push_back(p.b);
  }
  c->prof_pending.clear();
}

extern "C" int swap_profile_enable(swap_ctx* c, int on) {
  if (!c) return SWAP_EINVAL;
  c->prof_on = on != 0;
  return SWAP_OK;
}

extern "C" int swap_profile_reset(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  swap_prof_collect(c);
  c->prof.clear();
  return SWAP_OK;
}

extern "C" int swap_profile_read(swap_ctx* c, int32_t max, const char** names, double* total_ms, int64_t* launches,
                                 int32_t* n) {
  if (!c || !n) return SWAP_EINVAL;
  swap_prof_collect(c);
  const int32_t k = (int32_t)c->prof.size() < max ? (int32_t)c->prof.size() : max;
  for (int32_t i = 0; i < k; ++i) {
    if (names) names[i] = c->prof[(std::size_t)i].name;
    if (total_ms) total_ms[i] = c->prof[(std::size_t)i].ms;
    if (launches) launches[i] = c->prof[(std::size_t)i].launches;
  }
  *n = (int32_t)c->prof.size();
  return SWAP_OK;
}
