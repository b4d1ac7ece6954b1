// Shared device/host helpers of libnce_gb300: error reporting, Philox4x32-10, index draws.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "nce_gb300.h"

namespace nce {

// last error of the calling host thread
std::string &last_error();
int fail(int code, const char *fmt, ...);

// Raise (never lower) a kernel's dynamic shared-memory limit on the current device, under a process-wide lock.
// The attribute belongs to the function, not to the launch, so host threads that launch one kernel with different
// sizes (the job server's CE and NeuralCE threads share the exchange kernel) must not undo each other's setting.
cudaError_t raise_smem_limit(const void *func, size_t bytes);

// Scratch of one call, allocated and released in the order of its stream: calls on one model handle may run on
// several streams at once (a job's admission and another job's re-anchor), so no per-handle scratch is shared.
struct StreamScratch {
    void *p = nullptr; cudaStream_t s = nullptr;
    cudaError_t alloc(size_t bytes, cudaStream_t st) { s = st; return cudaMallocAsync(&p, bytes, st); }
    ~StreamScratch() { if (p) cudaFreeAsync(p, s); }
};

// device error flags of a model handle without clearing them (the job server checks them when a job ends), and
// the text of a flag word
int ce_error_peek(nce_ce_handle h, int32_t *flags);
int nce_error_peek(nce_nce_handle h, int32_t *flags);
const char *ce_error_text(int32_t flags);
const char *nce_error_text(int32_t flags);

// shapes of a model handle, for the job server's memory accounting
int ce_model_dims(nce_ce_handle h, int64_t *N, int32_t *n_cols, int32_t *mo, int32_t *binary);
int nce_model_dims(nce_nce_handle h, int64_t *N, int32_t *C0, int32_t *D, int32_t *depth);

#define NCE_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return ::nce::fail(NCE_ERR_CUDA, "%s failed: %s (%s:%d)", #call, \
                                                   cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define NCE_CHECK(cond, ...)                                                                  \
    do {                                                                                      \
        if (!(cond)) return ::nce::fail(NCE_ERR_INVALID, __VA_ARGS__);                        \
    } while (0)

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds, multipliers 0xD2511F53 / 0xCD9E8D57,
// Weyl key increments 0x9E3779B9 / 0xBB67AE85.
struct u32x4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ u32x4 philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                     uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return {c0, c1, c2, c3};
}

// index in [0, n) from 32 random bits (multiply-high)
__host__ __device__ __forceinline__ uint32_t draw_index(uint32_t x, uint32_t n) {
    return (uint32_t)(((uint64_t)x * (uint64_t)n) >> 32);
}

// uniform in (0, 1] from 53 random bits
__host__ __device__ __forceinline__ double draw_u01(uint32_t hi, uint32_t lo) {
    uint64_t m = ((uint64_t)hi << 21) | (uint64_t)(lo >> 11);
    return (double)(m + 1ull) * 1.1102230246251565404236316680908203125e-16;  // 2^-53
}

}  // namespace nce
