/*
 * Compatibility header force-included (nvcc -include) into every translation
 * unit of the reference's CUDA pipeline when oracle/build_ref.py compiles it.
 * TEST INFRASTRUCTURE ONLY: the reference build is the parity oracle and the
 * timed reference arm; nothing of the product includes this file.
 *
 * The reference sources compile unmodified with it.  It supplies the two
 * things they assume from the toolchain they were written for:
 *
 *  1. OctreeApi/OctreeLibrary/include/time_tracker.cuh:139,145 declare
 *     time_point<steady_clock> but initialise it from
 *     high_resolution_clock::now().  On libstdc++ high_resolution_clock is an
 *     alias of system_clock, so the two types differ.  Every standard header
 *     that names steady_clock is included here first; after that the token
 *     steady_clock is mapped to system_clock, which is what
 *     high_resolution_clock is on this library.
 *
 *  2. kernel/fp_subsample_evaluation.cuh:58, rp_subsample_evaluation.cuh:76 and
 *     kernel_inter_cell_filtering.cuh:85 call atomicAdd on uint64_t*.  On LP64
 *     Linux uint64_t is unsigned long, for which CUDA declares no overload.
 *     The overload below forwards to the unsigned long long one (same width).
 */
#pragma once

#include <chrono>
#include <condition_variable>
#include <future>
#include <mutex>
#include <shared_mutex>
#include <thread>

#include <spdlog/spdlog.h>

#define steady_clock system_clock

#ifdef __CUDACC__
#include <cuda_runtime.h>
static_assert(sizeof(unsigned long) == sizeof(unsigned long long), "LP64 expected");
__device__ __forceinline__ unsigned long atomicAdd(unsigned long* address, unsigned long value)
{
    return static_cast<unsigned long>(
            atomicAdd(reinterpret_cast<unsigned long long*>(address), static_cast<unsigned long long>(value)));
}
#endif
