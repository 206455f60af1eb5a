// Grid-wide barrier for the cooperative sweeps (every block of the launch resident at once).
#pragma once

#include "engine.cuh"

namespace avbdg {

__device__ __forceinline__ unsigned ldAcquireU32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void stReleaseU32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// d.gridBar[0] counts arrivals, d.gridBar[1] is the generation. The last block to arrive clears the
// count and advances the generation; the others wait for it, bounded by d.waitLimit (on running out
// they set kErrBarrierTimeout and the barrier returns false; every block then leaves the kernel,
// and the step reports the timeout). The arrival count must be zero when the launch starts (the
// launchers clear it). Writes before the barrier are visible to every block after it.
// `participants`: the blocks that take part (blocks 0 .. participants-1; the others have left the
// kernel and never call it); the whole grid by default.
__device__ __forceinline__ bool gridSync(const Dev &d, unsigned participants = 0) {
    __shared__ int ok;
    __syncthreads();
    const unsigned blocks = participants ? participants : gridDim.x;
    if (blocks == 1)
        return true; // one block: the block barrier orders its own global writes
    if (threadIdx.x == 0) {
        ok = 1;
        volatile int *errors = d.ctr + C_ERRORS;
        const unsigned gen = ldAcquireU32(d.gridBar + 1);
        __threadfence(); // this block's writes before its arrival
        if (atomicAdd(d.gridBar, 1u) + 1u == blocks) {
            d.gridBar[0] = 0;
            __threadfence();
            stReleaseU32(d.gridBar + 1, gen + 1u);
        } else {
            long long spins = 0;
            while (ldAcquireU32(d.gridBar + 1) == gen) {
                if (++spins > d.waitLimit || (*errors & kErrBarrierTimeout)) {
                    atomicOr(d.ctr + C_ERRORS, kErrBarrierTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

} // namespace avbdg
