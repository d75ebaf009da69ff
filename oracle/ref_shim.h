// ref_shim.h -- stand-ins that let the reference's own headers (helper_math.h,
// tensors.h, AMR.h, BSSN.h, SimpleWave.h) compile unmodified with gcc/nvcc on Linux.
//
// TEST INFRASTRUCTURE ONLY.  Part of the oracle: this file is used to build the
// reference-build library under oracle/_ref and is never linked into the product.
//
// The reference's CUDA_memory.h (smart buffers) and image_process.h (PNG output)
// contain MSVC-only constructs (std::exception("msg"), members of a dependent
// base used without this->).  Neither is part of the per-timestep arithmetic, so
// their include guards are pre-defined here and minimal replacements with the
// same member names are supplied instead:
//   smart_cpu_buffer<T>      (AdaptiveMesh/CUDA_memory.h:49-87)
//   smart_gpu_buffer<T>      (AdaptiveMesh/CUDA_memory.h:89-134)
//   smart_gpu_cpu_buffer<T>  (AdaptiveMesh/CUDA_memory.h:136-196)
//   cuda_sync()              (AdaptiveMesh/CUDA_memory.h:213-220)
// Unlike the reference, the host half of a smart_gpu_cpu_buffer is always
// allocated, so the reference's host-side octree logic runs on a machine without
// a GPU (the device half then stays unallocated and copies report an error).
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <string>
#include <iostream>
#include <vector>
#include <stdexcept>
#include <algorithm>
#include <sys/types.h>
#include <cuda_runtime.h>
#include <device_launch_parameters.h>

// helper_math.h declares `typedef unsigned long long ulong;`, which collides with
// glibc's `ulong`.  Every system header is already included above, so renaming
// the identifier from here on only touches the reference's own declarations.
#define ulong amr_ref_ulong

#define CUDA_MEM_H
#define IMAGE_PROCESSING_H

#if defined(__CUDACC__)
#define ALIGN_BYTES(n) __align__(n)
#else
#define ALIGN_BYTES(n) __attribute__((aligned(n)))
#endif

template <class T>
struct smart_cpu_buffer {
    size_t dedicated_len = 0;
    T* cpu_buffer_ptr = nullptr;
    bool created = false;
    smart_cpu_buffer() = default;
    // value-initialised (the reference leaves e.g. the root's lifetime counter uninitialised)
    explicit smart_cpu_buffer(size_t n) : dedicated_len(n), cpu_buffer_ptr(new T[n]()), created(true) {}
    size_t total_size() const { return dedicated_len * sizeof(T); }
    void destroy() { if (created) delete[] cpu_buffer_ptr; created = false; }
};

template <class T>
struct smart_gpu_buffer {
    size_t dedicated_len = 0;
    T* gpu_buffer_ptr = nullptr;
    bool created = false;
    smart_gpu_buffer() = default;
    explicit smart_gpu_buffer(size_t n) : dedicated_len(n) {
        if (cudaMalloc((void**)&gpu_buffer_ptr, n * sizeof(T)) == cudaSuccess) {
            created = true;
            cudaMemset(gpu_buffer_ptr, 0, n * sizeof(T));
        } else {
            gpu_buffer_ptr = nullptr;
            cudaGetLastError();
        }
    }
    size_t total_size() const { return dedicated_len * sizeof(T); }
    virtual void destroy() { if (created) cudaFree(gpu_buffer_ptr); created = false; }
    virtual ~smart_gpu_buffer() {}
};

template <class T>
struct smart_gpu_cpu_buffer : smart_gpu_buffer<T> {
    T* cpu_buffer_ptr = nullptr;
    smart_gpu_cpu_buffer() = default;
    explicit smart_gpu_cpu_buffer(size_t n) : smart_gpu_buffer<T>(n), cpu_buffer_ptr(new T[n]()) {}
    cudaError_t copy_to_cpu() {
        if (!this->created) return cudaErrorInvalidValue;
        return cudaMemcpy(cpu_buffer_ptr, this->gpu_buffer_ptr, this->dedicated_len * sizeof(T), cudaMemcpyDeviceToHost);
    }
    cudaError_t copy_to_gpu() {
        if (!this->created) return cudaErrorInvalidValue;
        return cudaMemcpy(this->gpu_buffer_ptr, cpu_buffer_ptr, this->dedicated_len * sizeof(T), cudaMemcpyHostToDevice);
    }
    void destroy() override {
        if (this->created) cudaFree(this->gpu_buffer_ptr);
        delete[] cpu_buffer_ptr;
        cpu_buffer_ptr = nullptr;
        this->created = false;
    }
};

static cudaError_t cuda_sync() {
    cudaError_t st = cudaDeviceSynchronize();
    if (st != cudaSuccess) fprintf(stderr, "cudaDeviceSynchronize returned error code %d\n", (int)st);
    return st;
}
