// Library-wide C ABI entry points: version, error text, host Philox.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "common.cuh"

namespace nce {

std::string &last_error() {
    static thread_local std::string msg;
    return msg;
}

int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    last_error() = buf;
    return code;
}

cudaError_t raise_smem_limit(const void *func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> limit;     // (device, kernel) -> attribute set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t &cur = limit[{dev, func}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

}  // namespace nce

extern "C" {

int nce_version(void) { return 10000; }

int nce_last_error(char *buf, size_t len) {
    const std::string &m = nce::last_error();
    if (buf && len) {
        size_t n = m.size() < len - 1 ? m.size() : len - 1;
        std::memcpy(buf, m.data(), n);
        buf[n] = 0;
    }
    return (int)m.size();
}

void nce_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    nce::u32x4 r = nce::philox4x32(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

}  // extern "C"
