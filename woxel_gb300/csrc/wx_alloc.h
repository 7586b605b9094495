// wx_alloc.h — the library's device and page-locked host allocations.
//
// Every cudaMalloc / cudaMallocHost of the library goes through these, so that
// tests can make them fail (wx_inject_alloc_failures): while injected failures
// remain, an allocation returns cudaErrorMemoryAllocation without calling CUDA,
// exactly as an exhausted device would, and the caller's error path runs.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace wx {

bool take_injected_alloc_failure();  // true (and one fewer remaining) while failures are injected

template <class T>
inline cudaError_t dev_alloc(T **p, size_t bytes) {
    if (take_injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return cudaMalloc(reinterpret_cast<void **>(p), bytes);
}

template <class T>
inline cudaError_t pinned_alloc(T **p, size_t bytes) {
    if (take_injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return cudaMallocHost(reinterpret_cast<void **>(p), bytes);
}

}  // namespace wx
