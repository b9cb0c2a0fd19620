// sort.cu -- stable LSD radix sort of (key, value) u32 pairs and a u32 exclusive scan.
//
// Semantics of backends/cuda/src/radix_sort.cu:279-336: 8-bit digits, ascending, stable;
// 2 passes (the low 16 key bits) when max_key_exclusive <= 65536, else 4 passes; the
// result lands back in the input buffer.
//
// A onesweep sort (a published single-pass scheme: one histogram read of the keys, then
// one kernel per digit pass whose tiles find their output offsets by decoupled look-back):
//   1. upsweep: the global digit histogram of every pass, from one read of the keys;
//   2. per pass, one kernel: each CTA claims the next 2048-pair tile (a counter, so tiles
//      are claimed in launch order), counts its digits, publishes that count for its
//      tile, walks back over the earlier tiles' published counts / inclusive prefixes
//      until it reaches a prefix, publishes its own inclusive prefix, and scatters.
//      Within a tile a pair's rank is (same-digit lanes below it in its warp) + (same-digit
//      pairs of lower warps this round) + (same-digit pairs of earlier rounds), which
//      keeps the sort stable.
// A tile only ever waits for tiles claimed before it, by CTAs that publish their count
// before they wait themselves, so every wait ends; each still has an iteration limit,
// past which it records an error word in the control block and goes on.
#include "common.cuh"
#include "host_common.h"
#include "kernels.h"

namespace sad {

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;  // 2048 pairs per CTA
constexpr int kSortMaxPasses = 4;
constexpr uint32_t kTileFlagA = 1u << 30;  // the tile's own digit count is published
constexpr uint32_t kTileFlagP = 2u << 30;  // its inclusive prefix (all earlier tiles) is
constexpr uint32_t kTileValue = kTileFlagA - 1u;
constexpr int kLookbackSpinLimit = 1 << 24;

constexpr uint32_t sort_tiles(uint32_t count) { return (count + kSortTile - 1) / kSortTile; }
constexpr size_t a256c(size_t x) { return (x + 255) & ~size_t(255); }

// Scratch layout: the ping-pong pairs, then the control block (zeroed per sort): the
// per-pass digit histograms [4][256], the tile counters [4], the error word, and the
// tile status words [4][tiles][256].
constexpr size_t sort_ctrl_bytes(uint32_t count) {
    return a256c((kSortMaxPasses * 256 + kSortMaxPasses + 1) * sizeof(uint32_t)) +
           a256c(static_cast<size_t>(kSortMaxPasses) * sort_tiles(count) * 256 * sizeof(uint32_t));
}
constexpr size_t sort_temp_bytes(uint32_t count) {
    return a256c(static_cast<size_t>(count) * 8) + sort_ctrl_bytes(count) + 256;
}

size_t radix_sort_temp_bytes(uint32_t count) { return sort_temp_bytes(count); }

struct SortCtrl {
    uint32_t* hist;      // [4][256] digit counts of each pass over all pairs
    uint32_t* tile_ctr;  // [4] next tile to claim, per pass
    uint32_t* error;     // nonzero: a look-back wait hit its limit
    uint32_t* status;    // [4][tiles_max][256] flag | count per tile and digit
};

static SortCtrl sort_ctrl_at(char* ctrl, uint32_t max_count) {
    SortCtrl c;
    uint32_t* w = reinterpret_cast<uint32_t*>(ctrl);
    c.hist = w;
    c.tile_ctr = w + kSortMaxPasses * 256;
    c.error = c.tile_ctr + kSortMaxPasses;
    c.status = reinterpret_cast<uint32_t*>(ctrl + a256c((kSortMaxPasses * 256 + kSortMaxPasses + 1) * 4));
    (void)max_count;
    return c;
}

__device__ __forceinline__ uint32_t sort_count(uint32_t max_count, const uint32_t* dev_count) {
    return dev_count ? min(*dev_count, max_count) : max_count;
}

__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}
__device__ __forceinline__ void st_volatile_u32(uint32_t* p, uint32_t v) {
    *reinterpret_cast<volatile uint32_t*>(p) = v;
}

// 1. digit histograms of every pass (grid-stride over the tiles)
__global__ void __launch_bounds__(kSortThreads) sort_upsweep_kernel(const uint2* __restrict__ in,
                                                                    uint32_t max_count,
                                                                    const uint32_t* __restrict__ dev_count,
                                                                    SortCtrl c, int passes) {
    __shared__ uint32_t h[kSortMaxPasses][256];
    const int tid = threadIdx.x;
    const uint32_t count = sort_count(max_count, dev_count);
#pragma unroll
    for (int p = 0; p < kSortMaxPasses; ++p) h[p][tid] = 0;
    __syncthreads();
    const uint32_t lt = lanemask_lt();
    for (uint32_t base = blockIdx.x * kSortTile; base < count; base += gridDim.x * kSortTile) {
#pragma unroll 2
        for (int r = 0; r < kSortRounds; ++r) {
            const uint32_t e = base + r * kSortThreads + tid;
            const bool ok = e < count;
            const uint32_t key = ok ? __ldg(&in[e].x) : 0u;
#pragma unroll
            for (int p = 0; p < kSortMaxPasses; ++p) {
                if (p >= passes) break;
                const uint32_t d = ok ? (key >> (8 * p)) & 0xffu : 0x100u + lane_id();
                const uint32_t peers = __match_any_sync(0xffffffffu, d);
                if (ok && (peers & lt) == 0u) atomicAdd(&h[p][d], __popc(peers));
            }
        }
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p)
        if (h[p][tid]) atomicAdd(&c.hist[p * 256 + tid], h[p][tid]);
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* warp_sums) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    uint32_t before = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w)
        if (w < warp) before += warp_sums[w];
    return before + x - v;
}

// 2. one digit pass
__global__ void __launch_bounds__(kSortThreads) sort_onesweep_kernel(const uint2* __restrict__ in,
                                                                     uint2* __restrict__ out,
                                                                     uint32_t max_count,
                                                                     const uint32_t* __restrict__ dev_count,
                                                                     SortCtrl c, uint32_t pass,
                                                                     uint32_t tiles_max) {
    pdl_wait();
    __shared__ uint32_t s_tile;
    __shared__ uint32_t bins[256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t warp_sums[kSortThreads / 32];
    __shared__ uint32_t warp_cnt[kSortThreads / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t count = sort_count(max_count, dev_count);
    const uint32_t tiles = sort_tiles(count);
    if (tid == 0) s_tile = atomicAdd(&c.tile_ctr[pass], 1u);
    bins[tid] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= tiles) return;
    const uint32_t shift = 8u * pass;
    const uint32_t tile0 = tile * kSortTile;
    const uint32_t lt = lanemask_lt();

    uint2 kv[kSortRounds];
    uint32_t dg[kSortRounds];
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const uint32_t e = tile0 + r * kSortThreads + tid;
        const bool ok = e < count;
        kv[r] = ok ? in[e] : make_uint2(0u, 0u);
        dg[r] = ok ? (kv[r].x >> shift) & 0xffu : 0x100u + lane;
    }
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        const uint32_t peers = __match_any_sync(0xffffffffu, dg[r]);
        if (dg[r] < 256u && (peers & lt) == 0u) atomicAdd(&bins[dg[r]], __popc(peers));
    }
    __syncthreads();

    // publish this tile's count per digit, then look back for the exclusive prefix
    const uint32_t cnt = bins[tid];
    uint32_t* status = c.status + static_cast<size_t>(pass) * tiles_max * 256;
    uint32_t excl = 0;
    if (tile == 0) {
        st_volatile_u32(status + tid, kTileFlagP | cnt);
    } else {
        st_volatile_u32(status + static_cast<size_t>(tile) * 256 + tid, kTileFlagA | cnt);
        int look = static_cast<int>(tile) - 1;
        int spins = 0;
        while (look >= 0) {
            const uint32_t v = ld_volatile_u32(status + static_cast<size_t>(look) * 256 + tid);
            const uint32_t flag = v & ~kTileValue;
            if (flag == 0u) {
                if (++spins > kLookbackSpinLimit) {
                    atomicExch(c.error, 1u);
                    break;
                }
                continue;
            }
            excl += v & kTileValue;
            if (flag == kTileFlagP) break;
            --look;
        }
        st_volatile_u32(status + static_cast<size_t>(tile) * 256 + tid, kTileFlagP | (excl + cnt));
    }
    base[tid] = block_exclusive_scan_256(c.hist[pass * 256 + tid], warp_sums) + excl;
    __syncthreads();

#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) warp_cnt[w][tid] = 0;
        __syncthreads();
        const uint32_t d = dg[r];
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt);
        if (d < 256u && rank == 0u) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = base[tid];
#pragma unroll
            for (int w = 0; w < kSortThreads / 32; ++w) {
                const uint32_t k = warp_cnt[w][tid];
                warp_cnt[w][tid] = acc;
                acc += k;
            }
            base[tid] = acc;
        }
        __syncthreads();
        const uint32_t pos = warp_cnt[warp][d & 0xffu] + rank;
        // pos < count always holds unless a look-back gave up (error word set); the check
        // keeps that case from writing outside the buffer
        if (d < 256u && pos < count) out[pos] = kv[r];
        __syncthreads();  // warp_cnt is cleared again by the next round
    }
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

void launch_scan_single(uint32_t* data, uint32_t count, uint32_t* total, cudaStream_t st) {
    launch_pdl(scan_single_kernel, dim3(1), dim3(1024), 0, st, data, count, total);
    note_launches(1);
}

// Sort of max_count pairs, or of *dev_count pairs (at most max_count) when dev_count is
// given; temp holds sort_temp_bytes(max_count).
void launch_radix_sort_dev(uint32_t* pairs, uint32_t max_count, const uint32_t* dev_count,
                           uint32_t max_key_exclusive, void* temp, cudaStream_t st) {
    if (max_count <= 1) return;
    const uint32_t tiles = sort_tiles(max_count);
    char* t = static_cast<char*>(temp);
    uint2* scratch = reinterpret_cast<uint2*>(t);
    char* ctrl = t + a256c(static_cast<size_t>(max_count) * 8);
    SortCtrl c = sort_ctrl_at(ctrl, max_count);
    const int passes = max_key_exclusive <= 65536u ? 2 : 4;
    cudaMemsetAsync(ctrl, 0, sort_ctrl_bytes(max_count), st);
    uint2* a = reinterpret_cast<uint2*>(pairs);
    uint2* b = scratch;
    const uint32_t up_blocks = std::min<uint32_t>(tiles, 152u * 2u);
    sort_upsweep_kernel<<<up_blocks, kSortThreads, 0, st>>>(a, max_count, dev_count, c, passes);
    for (int pass = 0; pass < passes; ++pass) {
        launch_pdl(sort_onesweep_kernel, dim3(tiles), dim3(kSortThreads), 0, st, a, b, max_count, dev_count, c,
                   static_cast<uint32_t>(pass), tiles);
        uint2* tmp = a;
        a = b;
        b = tmp;
    }
    note_launches(1ull + passes);
}

void launch_radix_sort(uint32_t* pairs, uint32_t count, uint32_t max_key_exclusive, void* temp,
                       cudaStream_t st) {
    launch_radix_sort_dev(pairs, count, nullptr, max_key_exclusive, temp, st);
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
// the sort clears its control block itself (a memset on the stream) and writes the
// ping-pong buffer before reading it.  The scratch is shared: calls that overlap on one device (other streams or host threads) race
// on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
namespace sad {

constexpr uint32_t kNoAllocMaxPairs = SAD_NOALLOC_SORT_MAX_PAIRS;
constexpr size_t kNoAllocScratchBytes = sort_temp_bytes(kNoAllocMaxPairs);

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
