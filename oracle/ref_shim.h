/*
 * TEST INFRASTRUCTURE ONLY.  Lets the reference's CUDA kernel sources compile
 * as host C++ so the oracle can be checked against the reference's own code:
 * the CUDA qualifiers are defined away and the thread indices become globals
 * that a driver loop sets (the technique of the reference's
 * crates/fritillaria-cuda/tests/harness/frame_host.cpp:19-32).
 */
#pragma once
struct RefDim3 {
    unsigned int x, y, z;
};
extern thread_local RefDim3 blockIdx, threadIdx, blockDim, gridDim;
#define __global__
#define __device__
#define __constant__
#define __forceinline__ inline
#define __shared__ static
#define __launch_bounds__(...)
static inline unsigned int atomicAdd(unsigned int *p, unsigned int v)
{
    unsigned int o = *p;
    *p += v;
    return o;
}
