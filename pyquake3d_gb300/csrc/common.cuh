// Shared helpers of the pq3d library: error recording, CUDA checks, the
// device-side bounded grid barrier and small math helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "pq3d.h"

namespace pq3d {

// Records `msg` as the calling host thread's last error and returns `code`.
int set_error(int code, const char *fmt, ...);
void clear_error();

#define PQ3D_CUDA_TRY(call)                                                              \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ::pq3d::set_error(PQ3D_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,  \
                                     #call, cudaGetErrorString(e_));                      \
    } while (0)

#define PQ3D_REQUIRE(cond, ...)                                                          \
    do {                                                                                 \
        if (!(cond)) return ::pq3d::set_error(PQ3D_ERR_ARG, __VA_ARGS__);                \
    } while (0)

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Iteration cap of every device-side spin wait (each iteration sleeps ~1 us,
// so a wait gives up after roughly two seconds).
constexpr unsigned kSpinLimit = 1u << 21;

// Grid-wide barrier for a cooperative launch.  Every block calls it with the
// same sequence; `count` and `gen` live in device memory and start at 0.
// Returns false when the wait hit `limit` iterations (kSpinLimit unless a
// self-test lowers it; the caller then records PQ3D_ERR_TIMEOUT and leaves).
__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned *gen, unsigned nblocks,
                                             unsigned limit = kSpinLimit)
{
    __shared__ bool ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = true;
        unsigned my_gen = *((volatile unsigned *)gen);
        __threadfence();
        unsigned arrived = atomicAdd(count, 1u) + 1u;
        if (arrived == nblocks) {
            *((volatile unsigned *)count) = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            unsigned it = 0;
            while (*((volatile unsigned *)gen) == my_gen) {
                if (++it > limit) { ok = false; break; }
                __nanosleep(1000);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok;
}

}  // namespace pq3d
