// gridsync.cuh -- grid-wide barrier for cooperatively launched kernels (all
// CTAs resident): arrive on a counter, wait on a generation word.  The wait is
// bounded: after BARRIER_SPIN_LIMIT polls it raises err = 2 and returns false,
// and every CTA that sees a raised flag leaves its wait too, so a kernel whose
// barrier fails ends instead of hanging.  Words: count, gen, err (zeroed
// before the launch, on separate 64-byte lines); on a timeout err[1..3] hold
// the arrivals counted, the CTA that gave up and the barrier generation.
#pragma once

namespace mq {

constexpr long long BARRIER_SPIN_LIMIT = 20000000;  // ~ seconds of polling

struct GridSync {
  unsigned *count;
  unsigned *gen;
  int *err;
};

__device__ __forceinline__ bool grid_barrier(const GridSync &gs, unsigned nblocks) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *genv = gs.gen;
    const unsigned g = *genv;
    __threadfence();
    if (atomicAdd(gs.count, 1u) == nblocks - 1) {
      *gs.count = 0;
      __threadfence();
      atomicAdd(gs.gen, 1u);
    } else {
      long long it = 0;
      while (*genv == g) {
        if (++it > BARRIER_SPIN_LIMIT) {
          // record where the wait gave up: arrivals seen, this CTA, generation
          gs.err[1] = (int)*(volatile unsigned *)gs.count;
          gs.err[2] = (int)blockIdx.x;
          gs.err[3] = (int)g;
          atomicExch(gs.err, 2);
          break;
        }
        if (*(volatile int *)gs.err) break;
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int *)gs.err == 0;
}

}  // namespace mq
