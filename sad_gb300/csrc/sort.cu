// sort.cu -- stable LSD radix sort of (key, value) u32 pairs and a u32 exclusive scan.
//
// Semantics of backends/cuda/src/radix_sort.cu:279-336: 8-bit digits, ascending, stable;
// 2 passes (the low 16 key bits) when max_key_exclusive <= 65536, else 4 passes; the
// result lands back in the input buffer.
//
// Per pass, three launches:
//   1. tile histograms: 2048 pairs per CTA; lanes holding the same digit are merged with
//      __match_any_sync so each warp adds one count per distinct digit;
//   2. one CTA scans the digit-major [256][tiles] histogram into global offsets;
//   3. scatter: each CTA re-reads its tile in 8 rounds of 256; within a round a lane's
//      rank is (same-digit lanes below it in its warp) + (same-digit elements of lower
//      warps this round) + (same-digit elements of earlier rounds), which keeps the sort
//      stable without the reference's O(n) per-thread rank loop.
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

namespace sad {

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;  // 2048 pairs per CTA

static inline uint32_t sort_tiles(uint32_t count) { return (count + kSortTile - 1) / kSortTile; }

size_t radix_sort_temp_bytes(uint32_t count) {
    size_t pairs = (static_cast<size_t>(count) * 8 + 255) & ~size_t(255);
    size_t hist = static_cast<size_t>(256) * sort_tiles(count) * 4;
    return pairs + ((hist + 255) & ~size_t(255)) + 256;
}

__global__ void __launch_bounds__(kSortThreads) sort_hist_kernel(const uint2* __restrict__ in,
                                                                 uint32_t* __restrict__ hist,
                                                                 uint32_t count, uint32_t shift,
                                                                 uint32_t tiles) {
    pdl_wait();
    __shared__ uint32_t bins[256];
    int tid = threadIdx.x;
    bins[tid] = 0;
    __syncthreads();
    uint32_t base = blockIdx.x * kSortTile;
    uint32_t lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        uint32_t e = base + r * kSortThreads + tid;
        bool ok = e < count;
        uint32_t d = ok ? (__ldg(&in[e].x) >> shift) & 0xffu : 0x100u + lane_id();
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        if (ok && (peers & lt) == 0u) atomicAdd(&bins[d], __popc(peers));
    }
    __syncthreads();
    hist[static_cast<size_t>(tid) * tiles + blockIdx.x] = bins[tid];
}

// Exclusive scan of `count` u32 in place by one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) scan_single_kernel(uint32_t* __restrict__ data,
                                                           uint32_t count,
                                                           uint32_t* __restrict__ total) {
    pdl_wait();
    __shared__ uint32_t warp_sums[32];
    int tid = threadIdx.x;
    uint32_t per = (count + 1023) / 1024;
    uint32_t b = tid * per, e = min(b + per, count);
    uint32_t local = 0;
    for (uint32_t i = b; i < e; ++i) local += data[i];
    // block exclusive scan of `local`
    uint32_t v = local;
    int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t run = v - local + (warp > 0 ? warp_sums[warp - 1] : 0u);
    for (uint32_t i = b; i < e; ++i) {
        uint32_t x = data[i];
        data[i] = run;
        run += x;
    }
    if (total && tid == 1023) *total = run;
}

__global__ void __launch_bounds__(kSortThreads) sort_scatter_kernel(const uint2* __restrict__ in,
                                                                    uint2* __restrict__ out,
                                                                    const uint32_t* __restrict__ offs,
                                                                    uint32_t count, uint32_t shift,
                                                                    uint32_t tiles) {
    pdl_wait();
    __shared__ uint32_t base[256];
    __shared__ uint32_t warp_cnt[kSortThreads / 32][256];
    int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = offs[static_cast<size_t>(tid) * tiles + blockIdx.x];
    uint32_t lt = lanemask_lt();
    uint32_t tile0 = blockIdx.x * kSortTile;
#pragma unroll 1
    for (int r = 0; r < kSortRounds; ++r) {
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) warp_cnt[w][tid] = 0;
        __syncthreads();
        uint32_t e = tile0 + r * kSortThreads + tid;
        bool ok = e < count;
        uint2 kv = ok ? in[e] : make_uint2(0u, 0u);
        uint32_t d = ok ? (kv.x >> shift) & 0xffu : 0x100u + lane;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        if (ok && rank == 0u) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = base[tid];
#pragma unroll
            for (int w = 0; w < kSortThreads / 32; ++w) {
                uint32_t c = warp_cnt[w][tid];
                warp_cnt[w][tid] = acc;
                acc += c;
            }
            base[tid] = acc;
        }
        __syncthreads();
        if (ok) out[warp_cnt[warp][d] + rank] = kv;
        __syncthreads();
    }
}

void launch_scan_single(uint32_t* data, uint32_t count, uint32_t* total, cudaStream_t st) {
    launch_pdl(scan_single_kernel, dim3(1), dim3(1024), 0, st, data, count, total);
    note_launches(1);
}

void launch_radix_sort(uint32_t* pairs, uint32_t count, uint32_t max_key_exclusive, void* temp,
                       cudaStream_t st) {
    if (count <= 1) return;
    uint32_t tiles = sort_tiles(count);
    char* t = static_cast<char*>(temp);
    uint2* scratch = reinterpret_cast<uint2*>(t);
    size_t pairs_bytes = (static_cast<size_t>(count) * 8 + 255) & ~size_t(255);
    uint32_t* hist = reinterpret_cast<uint32_t*>(t + pairs_bytes);
    int passes = max_key_exclusive <= 65536u ? 2 : 4;
    uint2* a = reinterpret_cast<uint2*>(pairs);
    uint2* b = scratch;
    for (int pass = 0; pass < passes; ++pass) {
        uint32_t shift = static_cast<uint32_t>(pass) * 8u;
        launch_pdl(sort_hist_kernel, dim3(tiles), dim3(kSortThreads), 0, st, a, hist, count, shift, tiles);
        launch_pdl(scan_single_kernel, dim3(1), dim3(1024), 0, st, hist, 256u * tiles, nullptr);
        launch_pdl(sort_scatter_kernel, dim3(tiles), dim3(kSortThreads), 0, st, a, b, hist, count, shift, tiles);
        uint2* tmp = a;
        a = b;
        b = tmp;
    }
    note_launches(3ull * passes);
}

}  // namespace sad

using namespace sad;

extern "C" size_t sad_radix_sort_temp_bytes(uint32_t count) { return radix_sort_temp_bytes(count); }

extern "C" sad_status_t sad_radix_sort_pairs(uint32_t* pairs, uint32_t count,
                                             uint32_t max_key_exclusive, void* temp,
                                             size_t temp_bytes, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count == 0 || pairs, "sad_radix_sort_pairs: null pairs");
    SAD_REQUIRE(count <= 1 || temp, "sad_radix_sort_pairs: null temp");
    SAD_REQUIRE(count <= 1 || temp_bytes >= radix_sort_temp_bytes(count),
                "sad_radix_sort_pairs: temp smaller than sad_radix_sort_temp_bytes(count)");
    SAD_REQUIRE((reinterpret_cast<uintptr_t>(pairs) & 7u) == 0, "sad_radix_sort_pairs: pairs must be 8-byte aligned");
    SAD_REQUIRE((reinterpret_cast<uintptr_t>(temp) & 15u) == 0, "sad_radix_sort_pairs: temp must be 16-byte aligned");
    launch_radix_sort(pairs, count, max_key_exclusive, temp, as_stream(stream));
    return check_launch("sad_radix_sort_pairs");
}

// ---------------------------------------------------------------------------
// Allocation-free entry point: the sort's scratch is a fixed file-scope device array,
// sized for SAD_NOALLOC_SORT_MAX_PAIRS pairs.  Every call looks its address up with
// cudaGetSymbolAddress on the current device (a host-side lookup, so a context that was
// torn down and re-created never leaves a stale address behind); host code never uses the
// symbol itself as a device address.  The first call on a device may load the module, so
// it should come before any stream capture.  Nothing in the scratch has to start at zero:
// each pass writes the histograms and the ping-pong buffer before reading them.  The
// scratch is shared: calls that overlap on one device (other streams or host threads) race
// on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace sad {

constexpr uint32_t kNoAllocMaxPairs = SAD_NOALLOC_SORT_MAX_PAIRS;
constexpr size_t kNoAllocScratchBytes =
    ((static_cast<size_t>(kNoAllocMaxPairs) * 8 + 255) & ~size_t(255)) +
    ((static_cast<size_t>(256) * ((kNoAllocMaxPairs + kSortTile - 1) / kSortTile) * 4 + 255) & ~size_t(255)) +
    256;

static __device__ __align__(256) unsigned char g_noalloc_sort_scratch[kNoAllocScratchBytes];

static sad_status_t noalloc_scratch(void** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
    if (e != cudaSuccess) return check_cuda(e, "sad_radix_sort_pairs_noalloc: cudaGetSymbolAddress");
    *out = p;
    return SAD_OK;
}

}  // namespace sad

extern "C" sad_status_t sad_radix_sort_pairs_noalloc(uint32_t* pairs, uint32_t count,
                                                     uint32_t max_key_exclusive, sad_stream_t stream) {
    clear_error();
    SAD_REQUIRE(count == 0 || pairs, "sad_radix_sort_pairs_noalloc: null pairs");
    SAD_REQUIRE(count <= kNoAllocMaxPairs,
                "sad_radix_sort_pairs_noalloc: count exceeds the fixed scratch of "
                "SAD_NOALLOC_SORT_MAX_PAIRS (262144) pairs; use sad_radix_sort_pairs");
    SAD_REQUIRE((reinterpret_cast<uintptr_t>(pairs) & 7u) == 0,
                "sad_radix_sort_pairs_noalloc: pairs must be 8-byte aligned");
    if (count <= 1) return SAD_OK;
    void* scratch = nullptr;
    SAD_TRY(noalloc_scratch(&scratch));
    launch_radix_sort(pairs, count, max_key_exclusive, scratch, as_stream(stream));
    return check_launch("sad_radix_sort_pairs_noalloc");
}
