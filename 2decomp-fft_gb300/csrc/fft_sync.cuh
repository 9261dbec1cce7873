// Bounded wait used by the kernels whose CTAs depend on one another (the
// fused x/y kernel and the batch kernel): one thread polls a completion
// counter until it reaches `need`; after `limit` polls it records `code` in
// the error word and returns, so a wait that cannot end never holds the GPU.
#pragma once

#include <cuda/atomic>

namespace gbfft {
namespace dev {

__device__ __forceinline__ bool bounded_wait(int* counter, int need, long long limit, int* error_word,
                                             int code) {
  cuda::atomic_ref<int, cuda::thread_scope_device> done(*counter);
  long long polls = 0;
  while (done.load(cuda::memory_order_acquire) < need) {
    if (++polls > limit) {
      atomicExch(error_word, code);
      return false;
    }
    __nanosleep(64);
  }
  return true;
}

}  // namespace dev
}  // namespace gbfft
