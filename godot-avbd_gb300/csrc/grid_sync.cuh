// Bounded grid barrier for kernels launched cooperatively (all blocks co-resident).
//
// Every wait has an iteration limit: a block that waits too long raises `timeoutBit` in *errors
// and returns false, and every other waiter gives up as soon as it sees that bit, so a kernel
// never hangs the GPU; the host reports the flag as a timeout status.
#pragma once

#include <cuda_runtime.h>

namespace avbdg {

constexpr long long kBarrierSpinLimit = 4000000; // ~0.4 s of 100 ns sleeps

// bar[0] = arrivals, bar[1] = generation; zero both before the launch.
__device__ inline bool gridBarrier(unsigned *bar, int *errors, int timeoutBit) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned *vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            bar[0] = 0;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            volatile int *verr = errors;
            while (*vgen == gen) {
                if (++spins > kBarrierSpinLimit || (*verr & timeoutBit)) {
                    atomicOr(errors, timeoutBit);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

} // namespace avbdg
