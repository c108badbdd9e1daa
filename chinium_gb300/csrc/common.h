// Shared host-side helpers: status codes, the thread-local error message and
// CUDA error checks.  Every C-ABI entry point converts exceptions into a
// negative status and records the message for xc_last_error().
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/chinium_xc.h"

namespace cgb {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define CGB_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            throw ::cgb::Error(XC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CGB_CHECK(cond, code, msg)                         \
    do {                                                   \
        if (!(cond)) throw ::cgb::Error((code), (msg));    \
    } while (0)

// Runs f, mapping exceptions to status codes.
template <class F>
int guard(F&& f) {
    try {
        f();
        return XC_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return XC_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return XC_ERR_INTERNAL;
    }
}

// Device buffer owned by the library (RAII).
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            reset();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && p) return;
        reset();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error(XC_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
        }
        n = count;
    }
    void upload(const T* h, size_t count, cudaStream_t s = 0) {
        alloc(count);
        if (count) CGB_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void zero(cudaStream_t s = 0) {
        if (n) CGB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

}  // namespace cgb
