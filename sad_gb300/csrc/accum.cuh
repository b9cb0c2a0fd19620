// accum.cuh -- per-tile accumulation of per-site values (gradients, removal deltas,
// statistics).
//
// The reference accumulates every (pixel, candidate) contribution with one shared-memory
// float atomic per value into a 256-slot hash per 16x16 tile, falling back to global
// atomics (backends/cuda/src/gradients.cu:422-485).  Neighbouring pixels share most of
// their candidates, often in the same slot order, so a warp's 32 lanes hit the same
// address and the atomics serialise.
//
// Here a tile table is filled in two steps:
//   1. registration: for each candidate slot, __match_any_sync groups the warp's lanes by
//      site; the group's lowest lane inserts the key (CAS probe) and broadcasts the table
//      slot, so each key costs one CAS per warp;
//   2. accumulation: every lane adds its values to the registered slot directly, visiting
//      its 8 candidates in a lane-rotated order so lanes with identical lists hit
//      different slots at the same instruction.
// Values are accumulated either as float (API calls, which add into caller buffers like
// the reference) or as fixed point (the trainer): integer addition is associative, so
// per-site sums -- and with them whole fits -- are bitwise reproducible.  Keys that do not
// fit within kMaxProbe probes go to global memory through the caller's fallback, which
// adds the same integers.
#pragma once

#include "common.cuh"

namespace sad {

// Fixed point with 24 fractional bits in 64-bit global records (range +-5.5e11 per site).
// The resolution, 6e-8 per pixel term, is far below what Adam resolves: gradients are
// divided by the pixel count and compared with eps = 1e-8.
constexpr int kFixFracBits = 24;
constexpr float kFixScale = 16777216.0f;                  // 2^24
constexpr float kFixInvScale = 5.9604644775390625e-08f;  // 2^-24
// Per tile, a fixed-point sum is kept as two 32-bit words (hi * 2^20 + lo): shared
// memory has native 32-bit integer atomics but no native 64-bit add.  Exact while a tile's
// sum of one value stays below 2^27 in magnitude (and each term below 2^27).
constexpr int kSplitLoBits = 20;

__device__ __forceinline__ long long to_fix(float v) { return __float2ll_rn(v * kFixScale); }
__host__ __device__ __forceinline__ float from_fix(long long v) {
#ifdef __CUDA_ARCH__
    return __ll2float_rn(v) * kFixInvScale;
#else
    return static_cast<float>(v) * kFixInvScale;
#endif
}

__device__ __forceinline__ void fix_add_global(long long* p, long long v) {
    atomicAdd(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(v));
}

// Split of to_fix(v) = h * 2^20 + l with |l| <= 2^19, in FP32 and INT32 arithmetic (a float
// -> 64-bit integer conversion runs on the FP64 pipe).  With y = v * 2^4 (exact), adding
// 1.5 * 2^23 rounds y to the nearest integer yr in the low mantissa bits; r = y - yr is exact
// and |r| <= 1/2, and rounding r * 2^20 the same way gives l.  h * 2^20 + l is then
// round-half-even(v * 2^24), the integer to_fix() gives for the global path.  h is 0 for
// |v| < 2^-5.  |v| < 2^18 takes this path; larger terms (to 2^27) split exactly via F2I.
__device__ __forceinline__ void split_fix(float v, int& h, int& l) {
    const float kMagic = 12582912.0f;  // 1.5 * 2^23
    const int kMagicBits = 0x4B400000;
    constexpr float kY = static_cast<float>(1 << (kFixFracBits - kSplitLoBits));
    if (fabsf(v) < 262144.0f) {
        float y = v * kY;
        float ym = y + kMagic;
        float r = y - (ym - kMagic);
        h = __float_as_int(ym) - kMagicBits;
        l = __float_as_int(fmaf(r, 1048576.0f, kMagic)) - kMagicBits;
    } else {
        float y = v * kY;  // at most one fractional bit; split it off
        float yf = truncf(y);
        h = __float2int_rz(yf);
        l = __float2int_rn((y - yf) * 1048576.0f);
    }
}

// Keys a 16x16 tile's accumulation table holds when its registration is precomputed (the
// registration depends only on the candidate field, which changes once per VPT refresh);
// a tile of the 1024^2 workload holds 20-100 distinct sites, more keys go to global memory.
constexpr int kTileKeys = 256;

// Accumulation modes of a tile table.
struct AccFloat {};  // float shared atomics (order-dependent rounding, like the reference)
struct AccSplit {};  // exact fixed point (hi, lo) words: bitwise reproducible sums

// Key -> dense index map of one tile.  Keys live in an open-addressing hash; each newly
// claimed key gets the next dense index, so the value arrays are packed: keys registered
// together sit in consecutive (bank-distinct) words, and the flush visits only used
// entries.
template <int SLOTS>
struct KeyTable {
    static_assert((SLOTS & (SLOTS - 1)) == 0, "SLOTS must be a power of two");
    static constexpr int kMaxProbe = 16;
    static constexpr int kSpinLimit = 1 << 20;
    uint32_t keys[SLOTS];
    int dense[SLOTS];      // dense index of hash slot s, -1 until its claimer publishes it
    uint32_t dkey[SLOTS];  // key of dense index d
    int count;

    __device__ __forceinline__ void init_keys(int tid, int nthreads) {
        for (int i = tid; i < SLOTS; i += nthreads) {
            keys[i] = kEmpty;
            dense[i] = -1;
        }
        if (tid == 0) count = 0;
    }

    // Dense index of `key` (inserting it), or -1 when the probe run is full.  A thread that
    // finds the key claimed by another warp waits (bounded) for its index; past the bound
    // it reports -1 and the caller takes the global path.
    __device__ __forceinline__ int insert(uint32_t key) {
        uint32_t h = (key * 2654435761u) & (SLOTS - 1);
#pragma unroll 1
        for (int p = 0; p < kMaxProbe; ++p) {
            uint32_t s = (h + p) & (SLOTS - 1);
            uint32_t old = atomicCAS(&keys[s], kEmpty, key);
            if (old == kEmpty) {
                int d = atomicAdd(&count, 1);
                dkey[d] = key;
                __threadfence_block();
                atomicExch(&dense[s], d);
                return d;
            }
            if (old == key) {
                volatile int* ds = &dense[s];
#pragma unroll 1
                for (int it = 0; it < kSpinLimit; ++it) {
                    int d = *ds;
                    if (d >= 0) return d;
                }
                return -1;
            }
        }
        return -1;
    }

    __device__ __forceinline__ int size() const { return count; }
    __device__ __forceinline__ uint32_t key_at(int d) const { return dkey[d]; }
};

// Values of a tile table: NV values per dense index.
template <int NV, int N, class Mode>
struct TileValues;

template <int NV, int N>
struct TileValues<NV, N, AccFloat> {
    float vals[NV][N];

    __device__ __forceinline__ void zero(int d) {
#pragma unroll
        for (int k = 0; k < NV; ++k) vals[k][d] = 0.0f;
    }
    __device__ __forceinline__ void add(int d, const float (&v)[NV]) {
#pragma unroll
        for (int k = 0; k < NV; ++k) atomicAdd(&vals[k][d], v[k]);
    }
    __device__ __forceinline__ float value(int k, int d) const { return vals[k][d]; }
    __device__ __forceinline__ long long fixed(int k, int d) const { return to_fix(vals[k][d]); }
};

// Fixed-point words: x = to_fix(v) = hi * 2^20 + lo with |lo| <= 2^19, so the lo sum of
// up to 2^11 terms fits an int32 and hi (zero for |v| < 2^-5, then skipped) wraps modulo
// 2^32, which the recombination absorbs while the tile's total stays below 2^27.
template <int NV, int N>
struct TileValues<NV, N, AccSplit> {
    int hi[NV][N];
    int lo[NV][N];

    __device__ __forceinline__ void zero(int d) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            hi[k][d] = 0;
            lo[k][d] = 0;
        }
    }
    __device__ __forceinline__ void add(int d, const float (&v)[NV]) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            int h, l;
            split_fix(v[k], h, l);
            atomicAdd(&lo[k][d], l);
            if (h != 0) atomicAdd(&hi[k][d], h);
        }
    }
    // For tables where each pixel adds at most once per entry (at most 256 adds per tile
    // entry): a candidate whose values are all below 1/4 in magnitude adds each as one
    // word, round(v * 2^24) with |.| <= 2^22, from one fused multiply-add (adding 1.5 * 2^23
    // rounds to an integer in the low mantissa bits) -- exactly to_fix(v); 256 such words
    // stay below 2^30.  Larger values take the split.
    __device__ __forceinline__ void add_unique(int d, const float (&v)[NV]) {
        float m = 0.0f;
#pragma unroll
        for (int k = 0; k < NV; ++k) m = fmaxf(m, fabsf(v[k]));
        if (m < 0.25f) {
#pragma unroll
            for (int k = 0; k < NV; ++k)
                atomicAdd(&lo[k][d], __float_as_int(fmaf(v[k], kFixScale, 12582912.0f)) - 0x4B400000);
        } else {
            add(d, v);
        }
    }
    __device__ __forceinline__ long long fixed(int k, int d) const {
        return static_cast<long long>(hi[k][d]) * (1ll << kSplitLoBits) + static_cast<long long>(lo[k][d]);
    }
};

// Fixed-point lo words of a precomputed tile table, privatised per lane group so that lanes
// adding to the same entry at the same instruction mostly hit different words (such
// same-address lanes serialise; with an 8-site nearest list per pixel, a warp's 32 lanes
// reach only 10-20 distinct sites per step).  The words form four banks-apart blocks of
// kNarrowKeys entries, used in one of two ways chosen per tile from its key count:
//   narrow (at most kNarrowKeys entries): block = the pixel's row in its 8x4 warp patch, so
//     each entry has four copies;
//   wide (up to kTileKeys entries): block = 2 * (entry / kNarrowKeys) + row parity, so each
//     entry has two copies.
// Both address a word as block * kStride + value * kNarrowKeys + entry % kNarrowKeys, so
// one accumulation loop serves both.  Adds follow TileValues<.., AccSplit>::add_unique (at
// most one add per pixel and entry: a copy sums at most 128 single-word terms of |x| <=
// 2^22); the hi words (rare) are shared.
constexpr int kNarrowKeys = kTileKeys / 2;

template <int NV>
struct TileWords {
    static constexpr int kStride = NV * kNarrowKeys + 8;  // blocks 8 banks apart
    int lo[4 * kStride];
    int hi[NV][kTileKeys];

    // the row bits of a lane in pixel row `row` (0-3) of its warp patch, and the block of
    // entry d for those bits (a narrow tile's entries are all below kNarrowKeys)
    static __device__ __forceinline__ int row_bits(int row, bool wide) { return row & (wide ? 1 : 3); }
    static __device__ __forceinline__ int block_of(int d, int rbits) { return ((d / kNarrowKeys) << 1) | rbits; }
    __device__ __forceinline__ int* word(int block, int d) { return lo + block * kStride + d % kNarrowKeys; }
    __device__ __forceinline__ const int* word(int block, int d) const {
        return lo + block * kStride + d % kNarrowKeys;
    }

    __device__ __forceinline__ void zero(int d, bool wide) {
        const int b0 = wide ? (d / kNarrowKeys) << 1 : 0, nb = wide ? 2 : 4;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            hi[k][d] = 0;
            for (int b = b0; b < b0 + nb; ++b) word(b, d)[k * kNarrowKeys] = 0;
        }
    }
    __device__ __forceinline__ void add_unique(int d, int block, const float (&v)[NV]) {
        int* lc = word(block, d);
        float m = 0.0f;
#pragma unroll
        for (int k = 0; k < NV; ++k) m = fmaxf(m, fabsf(v[k]));
        if (m < 0.25f) {
#pragma unroll
            for (int k = 0; k < NV; ++k)
                atomicAdd(lc + k * kNarrowKeys, __float_as_int(fmaf(v[k], kFixScale, 12582912.0f)) - 0x4B400000);
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                int h, l;
                split_fix(v[k], h, l);
                atomicAdd(lc + k * kNarrowKeys, l);
                if (h != 0) atomicAdd(&hi[k][d], h);
            }
        }
    }
    __device__ __forceinline__ long long fixed(int k, int d, bool wide) const {
        const int b0 = wide ? (d / kNarrowKeys) << 1 : 0, nb = wide ? 2 : 4;
        long long x = static_cast<long long>(hi[k][d]) * (1ll << kSplitLoBits);
        for (int b = b0; b < b0 + nb; ++b) x += static_cast<long long>(word(b, d)[k * kNarrowKeys]);
        return x;
    }
};

// A third shape, for tiles of at most kLaneKeys entries (late in a fit most tiles hold
// 10-30): one word per (entry, value, warp lane), shared by the block's eight warps, laid
// over the same shared memory as TileWords.  The adds of one instruction then land in 32
// banks, one per lane, and every lane may walk its candidates in the same order, which
// makes the staged site records' loads broadcasts: in a late-fit ncu capture the L1/shared
// pipe fell from 77% to 59% of its peak.  A word sums at most 8 terms (one pixel per warp; a
// pixel adds to an entry once) of |x| < 2^22, so an entry's 32 lane words sum to less than
// 2^30; a term of |v| >= 1/4 adds its low part here and its high part straight to the
// site's global record (an exact integer add, like the flush).
constexpr int kLaneKeys = 24;

template <int NV>
struct LaneWords {
    int w[kLaneKeys][NV][32];

    // zero the first `used` entries with the block's 256 threads
    __device__ __forceinline__ void zero(int used, int tid) {
        int4* p = reinterpret_cast<int4*>(&w[0][0][0]);
        const int n = used * NV * 8;
        for (int i = tid; i < n; i += 256) p[i] = make_int4(0, 0, 0, 0);
    }
    // lane `lane`'s terms for entry d (fix12: the [N][12] global records, dkey: the tile's
    // keys by entry, for the high parts of large terms)
    __device__ __forceinline__ void add(int d, int lane, const float (&v)[NV], long long* fix12,
                                        const uint32_t* dkey) {
        int* lw = &w[d][0][lane];
        float m = 0.0f;
#pragma unroll
        for (int k = 0; k < NV; ++k) m = fmaxf(m, fabsf(v[k]));
        if (m < 0.25f) {
#pragma unroll
            for (int k = 0; k < NV; ++k)
                atomicAdd(lw + 32 * k, __float_as_int(fmaf(v[k], kFixScale, 12582912.0f)) - 0x4B400000);
        } else {
            long long* rec = fix12 + static_cast<size_t>(dkey[d]) * 12;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                int h, l;
                split_fix(v[k], h, l);
                atomicAdd(lw + 32 * k, l);
                if (h != 0) fix_add_global(rec + k, static_cast<long long>(h) * (1ll << kSplitLoBits));
            }
        }
    }
    // the block's flush: thread t sums the 32 lane words of (entry, value) pairs t, t + 256,
    // ... in a bank-skewed order (lane l reads bank (j + l) & 31 at step j, so a warp's
    // reads never conflict) and adds each nonzero sum to the site's global record
    __device__ __forceinline__ void flush(int used, int tid, long long* fix12, const uint32_t* dkey) const {
        const int lane = tid & 31, pairs = used * NV;
        for (int q = tid; q < pairs; q += 256) {
            const int* wq = &w[0][0][0] + q * 32;
            int x = 0;
#pragma unroll 8
            for (int j = 0; j < 32; ++j) x += wq[(j + lane) & 31];
            if (x != 0) {
                const int d = q / NV, k = q - d * NV;
                fix_add_global(fix12 + static_cast<size_t>(dkey[d]) * 12 + k, x);
            }
        }
    }
};

// Keys and values of one tile (keys registered in the kernel).
template <int NV, int SLOTS, class Mode>
struct TileTable : KeyTable<SLOTS>, TileValues<NV, SLOTS, Mode> {
    __device__ __forceinline__ void init(int tid, int nthreads) {
        this->init_keys(tid, nthreads);
        for (int i = tid; i < SLOTS; i += nthreads) this->zero(i);
    }
};

// The table lives in dynamic shared memory (the 64-bit variants exceed the 48 KB static
// limit); launches pass sizeof(Table) and opt in through allow_dynamic_smem().
template <class Table>
__device__ __forceinline__ Table& shared_table() {
    extern __shared__ __align__(16) unsigned char sad_dyn_smem[];
    return *reinterpret_cast<Table*>(sad_dyn_smem);
}

// Step 1 for one candidate slot: all 32 lanes call it (key = kEmpty for none); returns the
// dense table index of the lane's key (-1: no key or table full).
template <class Table>
__device__ __forceinline__ int register_key(Table& table, uint32_t key) {
    const uint32_t full = 0xffffffffu;
    uint32_t peers = __match_any_sync(full, key);
    int leader = __ffs(peers) - 1;
    int slot = -1;
    if (static_cast<int>(lane_id()) == leader && key != kEmpty) slot = table.insert(key);
    slot = __shfl_sync(full, slot, leader);
    return key == kEmpty ? -1 : slot;
}

// Rotate an 8-entry register array left by r (0..7) with a 3-stage select network, so
// element j of the result is element (j + r) & 7 of the input (static indices only).
template <class T>
__device__ __forceinline__ void rotate8(T (&a)[8], uint32_t r) {
#pragma unroll
    for (int b = 1; b <= 4; b <<= 1) {
        bool on = (r & b) != 0;
        T t[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) t[j] = on ? a[(j + b) & 7] : a[j];
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = t[j];
    }
}

// Shift an 8-entry register array down by one (element 7 keeps its value).
template <class T>
__device__ __forceinline__ void shift8(T (&a)[8]) {
#pragma unroll
    for (int j = 0; j < 7; ++j) a[j] = a[j + 1];
}

__device__ __forceinline__ uint32_t rotate_mask8(uint32_t m, uint32_t r) {
    return ((m >> r) | (m << (8 - r))) & 0xffu;
}

// Per-lane rotation for 8x4 warp patches (lane = x + 8y): lanes that share a rotation
// are spread apart, so lanes with similar candidate lists visit different sites per step.
__device__ __forceinline__ uint32_t lane_rotation() {
    uint32_t l = lane_id();
    return ((l & 7u) * 5u + (l >> 3) * 2u) & 7u;
}

// Registration of one pixel's candidate list into its tile's table (all 32 lanes of the
// warp call it); writes the packed 8 x u16 table indices (0xFFFF: none) to the slot map and
// returns how many of them name an entry at or past kNarrowKeys (a far entry: keys are
// claimed nearest candidate first, so those are the tile's far, low-weight candidates).
template <class Table, class Map>
__device__ __forceinline__ int register_tile_pixel(Table& table, const uint32_t (&ids)[8],
                                                   uint32_t n, int x, int y, int w, bool inside,
                                                   const Map& map) {
    uint32_t packed[4] = {0u, 0u, 0u, 0u};
    int far = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        int slot = register_key(table, ids[i] < n ? ids[i] : kEmpty);
        // a repeated id in the list takes the global path, so a pixel adds at most once
        // to each table entry (TileValues::add_unique)
        bool repeat = false;
#pragma unroll
        for (int j = 0; j < i; ++j) repeat |= ids[j] == ids[i];
        uint32_t sidx = (slot < 0 || slot >= kTileKeys || repeat) ? 0xFFFFu : static_cast<uint32_t>(slot);
        far += (sidx != 0xFFFFu && sidx >= static_cast<uint32_t>(kNarrowKeys)) ? 1 : 0;
        packed[i >> 1] |= sidx << (16 * (i & 1));
    }
    if (inside)
        map.slot_map[static_cast<size_t>(y) * w + x] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    return inside ? far : 0;
}

// A tile's word-table shape (TileWords): wide when more than `rule` of its (pixel,
// candidate) references name far entries, narrow (far entries take the global path)
// otherwise.  Narrow gives the hot entries four copies instead of two, wide keeps the far
// entries in shared memory; which costs less depends on the image and the phase of the
// fit, so the trainer tunes the rule while it runs (every rule gives the same sums).  The
// default: wide when the far entries carry more than an eighth of the 2048 references.
constexpr int kWideFarRefs = 256;
// tile_count word: keys in use, plus this flag for a wide tile
constexpr int kTileWideFlag = 1 << 30;

// After the tile's registrations (and a barrier): its key list, and its key count with the
// shape flag (far_refs: the tile's summed register_tile_pixel results).
template <class Table, class Map>
__device__ __forceinline__ void write_tile_keys(const Table& table, int tid, int tile, int far_refs,
                                                int rule, const Map& map) {
    const int used = min(table.size(), kTileKeys);
    for (int d = tid; d < used; d += 256)
        map.tile_keys[static_cast<size_t>(tile) * kTileKeys + d] = table.key_at(d);
    if (tid == 0) map.tile_count[tile] = used | (far_refs > rule ? kTileWideFlag : 0);
}

#ifdef __CUDACC__
// Opt a kernel into `bytes` of dynamic shared memory when that and its static shared
// memory exceed the default 48 KB per block (a no-op below that).
template <class Kernel>
inline cudaError_t allow_dynamic_smem(Kernel kernel, size_t bytes) {
    cudaFuncAttributes a{};
    cudaError_t e = cudaFuncGetAttributes(&a, kernel);
    if (e != cudaSuccess) return e;
    if (bytes + a.sharedSizeBytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(bytes));
}
#endif

}  // namespace sad
