// host_common.h -- error reporting shared by the C-ABI entry points.
//
// Every entry point returns a sad_status_t.  On failure the message is kept in a
// thread-local buffer readable through sad_last_error().  Launch errors are
// collected with cudaGetLastError() right after each launch, so a bad launch
// configuration is reported by the call that made it.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/sad_gb300.h"

namespace sad {

// NVTX range in the library's own "sad_gb300" domain for the lifetime of the object: the
// stages of a fit (init, candidate refresh, gradients, tau diffusion and Adam, prune,
// densify, graph replays), a render from sites and executor requests, so profilers
// (nsys, ncu --nvtx) attribute the kernels to the step that launched them.  Header-only
// NVTX3: without an attached tool each range costs a few nanoseconds.
inline nvtxDomainHandle_t nvtx_domain() {
    static nvtxDomainHandle_t d = nvtxDomainCreateA("sad_gb300");
    return d;
}

struct NvtxRange {
    explicit NvtxRange(const char* name) {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(nvtx_domain(), &a);
    }
    ~NvtxRange() { nvtxDomainRangePop(nvtx_domain()); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

void set_error(const char* fmt, ...);
void clear_error();

inline sad_status_t fail(sad_status_t code, const char* msg) {
    set_error("%s", msg);
    return code;
}

inline sad_status_t check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SAD_ERR_OUT_OF_MEMORY : SAD_ERR_CUDA;
    }
    return SAD_OK;
}

inline sad_status_t check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SAD_ERR_OUT_OF_MEMORY : SAD_ERR_CUDA;
    }
    return SAD_OK;
}

inline cudaStream_t as_stream(sad_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// Largest image (or candidate field) the kernels address: a pixel's RGB offset, 3 * pixel,
// is a 32-bit int, so at most floor((2^31 - 1) / 3) pixels (e.g. 26,754 x 26,754).  Larger
// sizes are rejected as invalid arguments instead of overflowing an index.
constexpr long long kMaxPixels = 715827882;
inline bool image_size_ok(int w, int h) {
    return w > 0 && h > 0 && static_cast<long long>(w) * h <= kMaxPixels;
}

inline unsigned blocks_for(size_t n, unsigned threads) {
    return static_cast<unsigned>((n + threads - 1) / threads);
}

// Counts kernel launches issued by this library (read by the benchmark to report how
// many of its own kernels ran in a timed region).
void note_launches(uint64_t n);
void unnote_launches(uint64_t n);

}  // namespace sad

#define SAD_REQUIRE(cond, msg)                                      \
    do {                                                            \
        if (!(cond)) return ::sad::fail(SAD_ERR_INVALID_ARGUMENT, msg); \
    } while (0)

#define SAD_TRY(expr)                        \
    do {                                     \
        sad_status_t st_ = (expr);           \
        if (st_ != SAD_OK) return st_;       \
    } while (0)
