// Stable least-significant-digit radix sort and exclusive prefix sum for the broad phase (the cell
// keys of the spheres, the pair keys of a full run, the hi-id keys of the incidence lists).
//
// Sort: 8-bit digits, one pass per digit of the key's [beginBit, endBit) range. A pass is three
// launches: per-tile digit counts (tiles of 4096 keys, counts stored digit-major), their exclusive
// prefix sum (which is the output start of every (digit, tile) group), and the scatter, in which
// each warp ranks its 512 keys of the tile in order (32 at a time, grouped by __match_any_sync)
// against per-warp digit counters in shared memory, so that keys of equal digit keep their input
// order (the pass is stable, and so the sort).
// Scan: tiles of 4096 values scanned by a block each, the tile totals scanned by one block, the
// totals added back.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace wg {
namespace rsort {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;
constexpr int kRadix = 256;
constexpr int kWarps = kThreads / 32;

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int kSumsPerThread = 16;  // the tile totals one block scans: 16384 tiles, 67 M values

template <class K>
__device__ __forceinline__ unsigned digitOf(K k, int shift, unsigned mask) {
    return (unsigned)(k >> shift) & mask;
}

// digit counts of one tile, digit-major: hist[d * nTiles + tile]
template <class K>
__global__ void __launch_bounds__(kThreads) k_rs_hist(const K* __restrict__ keys, int64_t n, int shift, unsigned mask,
                                                      int32_t* __restrict__ hist, int nTiles) {
    __shared__ int32_t cnt[kRadix];
    for (int d = threadIdx.x; d < kRadix; d += kThreads) cnt[d] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int r = 0; r < kItems; r++) {
        const int64_t i = t0 + (int64_t)r * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[digitOf(keys[i], shift, mask)], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kThreads) hist[(int64_t)d * nTiles + blockIdx.x] = cnt[d];
}

// stable scatter of one tile to the start offsets off[d * nTiles + tile]. Warp w of the block owns
// the w-th run of kItems * 32 keys of the tile: it counts its digits (a round of 32 keys at a
// time, equal digits grouped by __match_any_sync, the group's first lane adding the group size to
// the warp's counter), the block turns the counters into output starts (warps in order within
// every digit), and the warp writes its keys in order, each at its counter plus its rank in its
// round's group. Keys keep their order: tile, warp, round and lane order is input order.
template <class K, class V>
__global__ void __launch_bounds__(kThreads) k_rs_scatter(const K* __restrict__ kin, const V* __restrict__ vin, K* __restrict__ kout,
                                                         V* __restrict__ vout, int64_t n, int shift, unsigned mask,
                                                         const int32_t* __restrict__ off, int nTiles) {
    __shared__ int32_t cnt[kWarps][kRadix];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < kRadix; d += kThreads)
        for (int w = 0; w < kWarps; w++) cnt[w][d] = 0;
    __syncthreads();
    const int64_t s0 = (int64_t)blockIdx.x * kTile + (int64_t)warp * (kItems * 32);
    const unsigned below = (1u << lane) - 1u;
    K k[kItems];
    V v[kItems];
    unsigned dg[kItems];
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        const int64_t i = s0 + r * 32 + lane;
        const bool valid = i < n;
        k[r] = valid ? kin[i] : K(0);
        v[r] = (valid && vin) ? vin[i] : V(0);
        dg[r] = valid ? digitOf(k[r], shift, mask) : 0xffffffffu;  // past the end: a group of their own
        const unsigned peers = __match_any_sync(0xffffffffu, dg[r]);
        if (valid && (peers & below) == 0) cnt[warp][dg[r]] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kThreads) {
        int run = off[(int64_t)d * nTiles + blockIdx.x];
        for (int w = 0; w < kWarps; w++) {
            const int c = cnt[w][d];
            cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        const bool valid = s0 + r * 32 + lane < n;
        const unsigned peers = __match_any_sync(0xffffffffu, dg[r]);
        const int rank = __popc(peers & below);
        if (valid) {
            const int32_t pos = cnt[warp][dg[r]] + rank;
            kout[pos] = k[r];
            if (vout) vout[pos] = v[r];
        }
        __syncwarp();
        if (valid && rank == 0) cnt[warp][dg[r]] += __popc(peers);
        __syncwarp();
    }
}

// exclusive scan of a block's kScanTile values (in place allowed); tot[blockIdx.x] = their sum
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t* in, int32_t* out, int64_t n, int32_t* __restrict__ tot) {
    __shared__ int32_t wsum[kScanThreads / 32];
    const int64_t i0 = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
        v[q] = (i0 + q < n) ? in[i0 + q] : 0;
        s += v[q];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int32_t w = lane < kScanThreads / 32 ? wsum[lane] : 0;
        int32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kScanThreads / 32) wsum[lane] = wi - w;  // exclusive over the warps
        if (lane == 31) tot[blockIdx.x] = wi;
    }
    __syncthreads();
    int32_t run = wsum[warp] + incl - s;
#pragma unroll
    for (int q = 0; q < kScanItems; q++) {
        if (i0 + q < n) out[i0 + q] = run;
        run += v[q];
    }
}

// exclusive scan of nb tile totals by one block (nb <= kScanThreads * kSumsPerThread)
__global__ void __launch_bounds__(kScanThreads) k_scan_totals(int32_t* __restrict__ tot, int nb) {
    __shared__ int32_t wsum[kScanThreads / 32];
    const int j0 = threadIdx.x * kSumsPerThread;
    int32_t s = 0;
    for (int q = 0; q < kSumsPerThread; q++)
        if (j0 + q < nb) s += tot[j0 + q];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int32_t w = lane < kScanThreads / 32 ? wsum[lane] : 0;
        int32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kScanThreads / 32) wsum[lane] = wi - w;
    }
    __syncthreads();
    int32_t run = wsum[warp] + incl - s;
    for (int q = 0; q < kSumsPerThread; q++)
        if (j0 + q < nb) {
            const int32_t t = tot[j0 + q];
            tot[j0 + q] = run;
            run += t;
        }
}

__global__ void k_scan_add(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ tot) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tot[i / kScanTile];
}

// scratch (int32 words) of an exclusive scan of n values
inline int64_t scanScratch(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

// exclusive prefix sum of n int32 values (in == out allowed); false if n is beyond its range
inline bool exclusiveScan(const int32_t* in, int32_t* out, int64_t n, int32_t* scratch, cudaStream_t st) {
    if (n <= 0) return true;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb > (int64_t)kScanThreads * kSumsPerThread) return false;
    k_scan_tiles<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, scratch);
    if (nb > 1) {
        k_scan_totals<<<1, kScanThreads, 0, st>>>(scratch, (int)nb);
        k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, scratch);
    }
    return true;
}

// scratch (int32 words) of a sort of n keys
inline int64_t sortScratch(int64_t n) {
    const int64_t nTiles = (n + kTile - 1) / kTile;
    const int64_t h = (int64_t)kRadix * nTiles;
    return h + scanScratch(h);
}

// Stable sort of the n keys kin (and values vin, if not null) by bits [beginBit, endBit) into
// kout (vout). kin and vin are overwritten (they are the other buffer of the passes). Returns
// false if n or the bit range is outside what it handles.
template <class K, class V>
inline bool sortPairs(K* kin, K* kout, V* vin, V* vout, int64_t n, int beginBit, int endBit, int32_t* scratch, cudaStream_t st) {
    if (n <= 0) return true;
    if (n >= (int64_t(1) << 31) - kTile || beginBit < 0 || endBit > (int)(8 * sizeof(K)) || endBit < beginBit) return false;
    const int nTiles = (int)((n + kTile - 1) / kTile);
    int32_t* hist = scratch;
    int32_t* sc = scratch + (int64_t)kRadix * nTiles;
    const int passes = (endBit - beginBit + 7) / 8;
    if (passes == 0) {
        cudaMemcpyAsync(kout, kin, sizeof(K) * n, cudaMemcpyDeviceToDevice, st);
        if (vin) cudaMemcpyAsync(vout, vin, sizeof(V) * n, cudaMemcpyDeviceToDevice, st);
        return true;
    }
    for (int p = 0; p < passes; p++) {
        const int shift = beginBit + 8 * p;
        const int bits = endBit - shift < 8 ? endBit - shift : 8;
        const unsigned mask = (1u << bits) - 1u;
        K* ks = (p % 2 == 0) ? kin : kout;
        K* kd = (p % 2 == 0) ? kout : kin;
        V* vs = vin ? ((p % 2 == 0) ? vin : vout) : nullptr;
        V* vd = vin ? ((p % 2 == 0) ? vout : vin) : nullptr;
        k_rs_hist<K><<<nTiles, kThreads, 0, st>>>(ks, n, shift, mask, hist, nTiles);
        if (!exclusiveScan(hist, hist, (int64_t)kRadix * nTiles, sc, st)) return false;
        k_rs_scatter<K, V><<<nTiles, kThreads, 0, st>>>(ks, vs, kd, vd, n, shift, mask, hist, nTiles);
    }
    if (passes % 2 == 0) {  // the last pass wrote kin
        cudaMemcpyAsync(kout, kin, sizeof(K) * n, cudaMemcpyDeviceToDevice, st);
        if (vin) cudaMemcpyAsync(vout, vin, sizeof(V) * n, cudaMemcpyDeviceToDevice, st);
    }
    return true;
}

}  // namespace rsort
}  // namespace wg
