// accum.cuh -- per-tile accumulation of per-site values (gradients, removal deltas).
//
// The reference accumulates every (pixel, candidate) contribution with one shared-memory
// atomic per value into a 256-slot hash per 16x16 tile, falling back to global atomics
// (backends/cuda/src/gradients.cu:422-485).  Neighbouring pixels share most of their
// candidates, so those shared atomics collide on the same address.
//
// Here each warp first merges the contributions of its lanes that carry the same site:
// __match_any_sync groups the lanes by key and a segmented tree reduction over
// shuffles (log2 of the largest group rounds) leaves each group's sum in its lowest
// lane.  Only those leaders touch the shared hash, so the shared atomics of a warp go
// to distinct slots.  Keys that do not fit the table within kMaxProbe probes go straight
// to global memory through the caller's fallback.
#pragma once

#include "common.cuh"

namespace sad {

template <int NV, int SLOTS>
struct TileTable {
    static_assert((SLOTS & (SLOTS - 1)) == 0, "SLOTS must be a power of two");
    static constexpr int kMaxProbe = 16;
    uint32_t keys[SLOTS];
    float vals[NV][SLOTS];

    __device__ __forceinline__ void init(int tid, int nthreads) {
        for (int i = tid; i < SLOTS; i += nthreads) {
            keys[i] = kEmpty;
#pragma unroll
            for (int k = 0; k < NV; ++k) vals[k][i] = 0.0f;
        }
    }

    __device__ __forceinline__ static uint32_t home(uint32_t key) {
        return (key * 2654435761u) & (SLOTS - 1);
    }

    // Add v to the slot of `key`; returns false when the table is full along the probe run.
    __device__ __forceinline__ bool add(uint32_t key, const float (&v)[NV]) {
        uint32_t h = home(key);
#pragma unroll 1
        for (int p = 0; p < kMaxProbe; ++p) {
            uint32_t s = (h + p) & (SLOTS - 1);
            uint32_t old = atomicCAS(&keys[s], kEmpty, key);
            if (old == kEmpty || old == key) {
#pragma unroll
                for (int k = 0; k < NV; ++k) atomicAdd(&vals[k][s], v[k]);
                return true;
            }
        }
        return false;
    }
};

// Segmented sum over the lanes of a warp that hold the same key.  Must be called by all
// 32 lanes.  On return the lowest lane of every key group holds the group's sums and
// `leader` is true there.
template <int NV>
__device__ __forceinline__ bool warp_merge_by_key(uint32_t key, float (&v)[NV]) {
    const uint32_t full = 0xffffffffu;
    uint32_t lane = lane_id();
    uint32_t lt = lanemask_lt();
    uint32_t peers = __match_any_sync(full, key);
    bool leader = (peers & lt) == 0u;
    uint32_t rank = __popc(peers & lt);
    uint32_t above = peers & ~(lt | (1u << lane));
    // Round r: every lane adds the value of its next remaining higher peer; the lanes
    // of odd rank are then absorbed and drop out of all peer sets.
    while (__any_sync(full, above != 0u)) {
        int next = __ffs(above) - 1;
        int src = next < 0 ? static_cast<int>(lane) : next;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            float t = __shfl_sync(full, v[k], src);
            if (next >= 0) v[k] += t;
        }
        uint32_t absorbed = __ballot_sync(full, (rank & 1u) != 0u);
        above &= ~absorbed;
        rank >>= 1;
    }
    return leader;
}

}  // namespace sad
