// Shared helpers of the srf_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

#include "../../include/srf_gb300.h"

namespace srf {

// Device-side error flag: kernels set bits here instead of trapping.
enum : int {
    kFlagRange = 1,      // an index check failed; the access was skipped
    kFlagTimeout = 2,    // a bounded wait gave up
};

void set_cuda_error(cudaError_t e);
// Device address of the error flag on the current device (NULL if unavailable).
int* device_flag();
__device__ __forceinline__ void raise_flag(int* flag, int bits) {
    if (flag) atomicOr(flag, bits);
}

// Counts kernel launches issued by this library (every launch site calls
// launch_status() once); read through srf_launch_count().
void count_launch();

inline int launch_status() {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    return SRF_OK;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline unsigned grid_1d(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return static_cast<unsigned>(g);
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Workspace carving: 256-byte aligned sub-buffers from one caller allocation.
struct Carver {
    char* base;
    size_t used = 0;
    size_t cap;
    Carver(void* b, size_t c) : base(static_cast<char*>(b)), cap(c) {}
    template <class T>
    T* take(size_t count) {
        used = (used + 255) & ~size_t(255);
        T* p = reinterpret_cast<T*>(base ? base + used : nullptr);
        used += count * sizeof(T);
        return p;
    }
    bool ok() const { return used <= cap; }
};

__device__ __forceinline__ float relu_f(float x) { return x > 0.f ? x : 0.f; }
__device__ __forceinline__ float sigmoid_f(float x) { return 1.f / (1.f + expf(-x)); }

// MassConcentrationLoss06's bins over a ray of s samples: bin b covers samples
// [start[b], start[b + 1]).
struct BinLayout {
    int nb;
    int start[65];
};

// torch.linspace(0, B - 1, S % B) (CPU/CUDA formula: start + step i below the
// halfway point, end - step (steps - 1 - i) above it, in float), truncated: the
// bins that take one extra sample (MassConcentrationLoss06.py:69-72).
inline bool bin_layout(int s, int nb, BinLayout* bl) {
    if (nb < 1 || nb > 64 || s < nb) return false;
    bool bigger[64] = {};
    const int per = s / nb, rem = s % nb;
    if (rem == 1) {
        bigger[0] = true;
    } else if (rem > 1) {
        const float start = 0.f, end = float(nb - 1);
        const float step = (end - start) / float(rem - 1);
        for (int i = 0; i < rem; ++i) {
            float v = i < rem / 2 ? start + step * float(i) : end - step * float(rem - 1 - i);
            int k = int(v);
            if (k < 0 || k >= nb) return false;
            bigger[k] = true;
        }
    }
    bl->nb = nb;
    bl->start[0] = 0;
    for (int b = 0; b < nb; ++b) bl->start[b + 1] = bl->start[b] + per + (bigger[b] ? 1 : 0);
    return bl->start[nb] == s;
}

}  // namespace srf
