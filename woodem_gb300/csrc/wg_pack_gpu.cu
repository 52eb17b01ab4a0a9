// Random sequential insertion of non-overlapping spheres on the device (scene generation).
//
// The device counterpart of wg_pack_rsa (wg_pack.cpp), which plays the role of
// SpherePack::makeCloud (lib/sphere-pack/SpherePack.hpp:75) for the regions of the benchmark
// scenes. The host version places sphere i (in the given order) at the first of up to
// max_attempts uniform candidate centres that overlaps no sphere placed before it. Here the
// spheres are inserted in rounds over a window of the lowest-indexed unplaced spheres (1/64 of
// the spheres, at least 256 and at most 32768):
//   1. every sphere of the window draws its next candidate centre (a counter-based hash of the
//      seed, the sphere index and the attempt number, so the result does not depend on the
//      launch shape) and tests it against the spheres placed in earlier rounds;
//   2. a candidate that is clear of them is accepted unless it overlaps the clear candidate of
//      a lower-indexed sphere of the same round;
//   3. accepted spheres join the placed set; the others draw again in the next round.
// Accepted spheres never overlap, and every sphere still gets max_attempts candidates. The
// order of acceptance follows the index order only within a window (a sphere may be placed a
// round before a lower-indexed one), so the packing is not the host version's sphere for
// sphere; its statistics (count, solid fraction, uniformity) are those of sequential insertion.
// As in the host version, the result is the prefix of spheres before the first one that found
// no place; spheres after it that were placed are dropped.
//
// Neighbour search: a uniform grid of edge 2 r_max over the region; placed spheres and the
// clear candidates of a round are kept in per-cell linked lists (a head per cell, a next link
// per sphere, pushed with atomicExch). The order of a list depends on the atomics, but every
// test is over the whole list, so the result does not.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct PackGrid {
    double lo[3], L[3], cw[3];
    int nc[3];
    int kind;  // 0 box, 1 cylinder along x, 2 periodic box
    double cyl[4];
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// the k-th uniform double in [0, 1) of attempt a of sphere i
__device__ __forceinline__ double uni(uint64_t seed, int64_t i, int64_t a, int k) {
    const uint64_t h = mix64(seed ^ mix64((uint64_t)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) ^
                             mix64((uint64_t)a * 0xD1B54A32D192ED03ull + (uint64_t)k * 0x8CB92BA72F3D8DD7ull + 1));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ int cellOf(const PackGrid& G, const double c[3], int ci[3]) {
    for (int k = 0; k < 3; k++) {
        int q = (int)floor((c[k] - G.lo[k]) / G.cw[k]);
        ci[k] = q < 0 ? 0 : (q >= G.nc[k] ? G.nc[k] - 1 : q);
    }
    return (ci[2] * G.nc[1] + ci[1]) * G.nc[0] + ci[0];
}

// whether centre c of radius r overlaps a sphere of the lists `head`/`next` in the 27 cells
// around ci (only entries below `below` count when below >= 0)
__device__ bool clashList(const PackGrid& G, const double c[3], double r, const int ci[3], const int32_t* __restrict__ head,
                          const int32_t* __restrict__ next, const double* __restrict__ pos, const double* __restrict__ radii,
                          int64_t below) {
    const bool peri = G.kind == 2;
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int q[3] = {ci[0] + dx, ci[1] + dy, ci[2] + dz};
                bool skip = false;
                for (int k = 0; k < 3; k++)
                    if (q[k] < 0 || q[k] >= G.nc[k]) {
                        if (!peri) skip = true;
                        else q[k] = (q[k] + G.nc[k]) % G.nc[k];
                    }
                if (skip) continue;
                for (int32_t j = head[(q[2] * G.nc[1] + q[1]) * G.nc[0] + q[0]]; j >= 0; j = next[j]) {
                    if (below >= 0 && j >= below) continue;
                    double d2 = 0;
                    for (int k = 0; k < 3; k++) {
                        double d = c[k] - pos[3 * (int64_t)j + k];
                        if (peri) d -= G.L[k] * rint(d / G.L[k]);
                        d2 += d * d;
                    }
                    const double rr = r + radii[j];
                    if (d2 < rr * rr) return true;
                }
            }
    return false;
}

// round step 1: candidates of the unplaced spheres in [w0, w1), tested against the placed set;
// clear ones are pushed on the round lists
__global__ void k_rsa_draw(PackGrid G, int64_t w0, int64_t w1, const double* __restrict__ radii, uint64_t seed,
                           const int32_t* __restrict__ state, const int64_t* __restrict__ attempt, double* __restrict__ cand,
                           int32_t* __restrict__ clear, const int32_t* __restrict__ headP, const int32_t* __restrict__ nextP,
                           const double* __restrict__ pos, int32_t* __restrict__ headR, int32_t* __restrict__ nextR) {
    const int64_t i = w0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w1) return;
    clear[i] = 0;
    if (state[i] != 0) return;  // placed or failed
    const double r = radii[i];
    const int64_t a = attempt[i];
    double c[3];
    const bool peri = G.kind == 2;
    for (int k = 0; k < 3; k++) {
        const double m = peri ? 0. : r;
        c[k] = G.lo[k] + m + uni(seed, i, a, k) * (G.L[k] - 2 * m);
    }
    for (int k = 0; k < 3; k++) cand[3 * i + k] = c[k];
    if (G.kind == 1) {
        const double dy = c[1] - G.cyl[0], dz = c[2] - G.cyl[1];
        if (sqrt(dy * dy + dz * dz) > G.cyl[2] - r) return;
        if (c[2] + r > G.cyl[3]) return;
    }
    int ci[3];
    const int cell = cellOf(G, c, ci);
    if (clashList(G, c, r, ci, headP, nextP, pos, radii, -1)) return;
    clear[i] = 1;
    nextR[i] = atomicExch(headR + cell, (int32_t)i);
}

// round step 2: a clear candidate is accepted unless it overlaps the clear candidate of a
// lower-indexed sphere; rejected and unclear ones move to their next attempt
__global__ void k_rsa_resolve(PackGrid G, int64_t w0, int64_t w1, const double* __restrict__ radii, int64_t maxAttempts,
                              int32_t* __restrict__ state, int64_t* __restrict__ attempt, const double* __restrict__ cand,
                              const int32_t* __restrict__ clear, const int32_t* __restrict__ headR, const int32_t* __restrict__ nextR,
                              int32_t* __restrict__ accepted) {
    const int64_t i = w0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w1) return;
    accepted[i] = 0;
    if (state[i] != 0) return;
    bool ok = false;
    if (clear[i]) {
        const double c[3] = {cand[3 * i], cand[3 * i + 1], cand[3 * i + 2]};
        int ci[3];
        cellOf(G, c, ci);
        ok = !clashList(G, c, radii[i], ci, headR, nextR, cand, radii, i);
    }
    if (ok) {
        accepted[i] = 1;
        return;
    }
    const int64_t a = attempt[i] + 1;
    attempt[i] = a;
    if (a >= maxAttempts) state[i] = 2;  // no place found
}

// round step 3: accepted spheres join the placed set (their round-list links are dead after
// the round; the placed set keeps its own links)
__global__ void k_rsa_commit(PackGrid G, int64_t w0, int64_t w1, int32_t* __restrict__ state, const double* __restrict__ cand,
                             const int32_t* __restrict__ clear, const int32_t* __restrict__ accepted, double* __restrict__ pos,
                             int32_t* __restrict__ headP, int32_t* __restrict__ nextP, int32_t* __restrict__ headR) {
    const int64_t i = w0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w1 || !clear[i]) return;
    const double c[3] = {cand[3 * i], cand[3 * i + 1], cand[3 * i + 2]};
    int ci[3];
    const int cell = cellOf(G, c, ci);
    headR[cell] = -1;  // the round lists end with the round (every clear candidate clears its cell)
    if (!accepted[i]) return;
    for (int k = 0; k < 3; k++) pos[3 * i + k] = c[k];
    nextP[i] = atomicExch(headP + cell, (int32_t)i);
    state[i] = 1;
}

// stream-ordered scratch (no device-wide synchronisation when it is freed, so that a packer
// running beside simulations on other streams does not wait for their work)
struct Scratch {
    cudaStream_t st = nullptr;
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFreeAsync(p, st);
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    }
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (cudaMallocAsync(&p, sizeof(T) * count, st) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T*)p;
    }
};

}  // namespace

extern "C" {

/* The device packer; arguments and result as wg_pack_rsa (wg_pack.cpp). Negative result: a CUDA
   error (-1) or an argument error (-2). */
int64_t wg_pack_rsa_device(int64_t n, const double* radii, const double* lo, const double* hi, int32_t region_kind,
                           const double* params, uint64_t seed, int64_t max_attempts, double* centers) {
    if (n <= 0) return 0;
    if (!radii || !lo || !hi || !centers || region_kind < 0 || region_kind > 2 || max_attempts < 1 || n >= (int64_t(1) << 31) - 1)
        return -2;
    if (region_kind == 1 && !params) return -2;
    double rmax = 0;
    for (int64_t i = 0; i < n; i++) {
        if (!(radii[i] > 0) || !std::isfinite(radii[i])) return -2;
        rmax = std::fmax(rmax, radii[i]);
    }
    PackGrid G{};
    G.kind = region_kind;
    const double cs = 2 * rmax;
    int64_t ncell = 1;
    for (int k = 0; k < 3; k++) {
        G.lo[k] = lo[k];
        G.L[k] = hi[k] - lo[k];
        if (!(G.L[k] > 0) || !std::isfinite(G.L[k])) return -2;
        const int64_t q = std::max<int64_t>(1, (int64_t)std::floor(G.L[k] / cs));
        if (q > (1 << 20)) return -2;
        G.nc[k] = (int)q;
        G.cw[k] = G.L[k] / (double)q;
        ncell *= q;
    }
    if (ncell > (int64_t(1) << 30)) return -2;
    if (region_kind == 1)
        for (int k = 0; k < 4; k++) G.cyl[k] = params[k];
    // device arrays, on a stream of the call's own
    Scratch X;
    if (cudaStreamCreateWithFlags(&X.st, cudaStreamNonBlocking) != cudaSuccess) {
        X.st = nullptr;
        return -1;
    }
    cudaStream_t st = X.st;
    double* dRad = X.get<double>(n);
    double* dPos = X.get<double>(3 * n);
    double* dCand = X.get<double>(3 * n);
    int32_t* dState = X.get<int32_t>(n);
    int64_t* dAtt = X.get<int64_t>(n);
    int32_t* dClear = X.get<int32_t>(n);
    int32_t* dAcc = X.get<int32_t>(n);
    int32_t* dHeadP = X.get<int32_t>(ncell);
    int32_t* dNextP = X.get<int32_t>(n);
    int32_t* dHeadR = X.get<int32_t>(ncell);
    int32_t* dNextR = X.get<int32_t>(n);
    if (!dRad || !dPos || !dCand || !dState || !dAtt || !dClear || !dAcc || !dHeadP || !dNextP || !dHeadR || !dNextR) return -1;
    bool ok = cudaMemcpyAsync(dRad, radii, sizeof(double) * n, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemsetAsync(dState, 0, sizeof(int32_t) * n, st) == cudaSuccess &&
              cudaMemsetAsync(dAtt, 0, sizeof(int64_t) * n, st) == cudaSuccess &&
              cudaMemsetAsync(dHeadP, 0xff, sizeof(int32_t) * ncell, st) == cudaSuccess &&
              cudaMemsetAsync(dHeadR, 0xff, sizeof(int32_t) * ncell, st) == cudaSuccess;
    if (!ok) return -1;
    // the window: the unplaced spheres of [w0, w1), w1 - w0 at most W, a small fraction of the
    // spheres so that the window holds spheres of similar rank (the insertion order puts the
    // largest first: a window of all spheres would let small ones fill the gaps the large ones
    // need); after every few rounds the state of the window comes back to the host, which moves w0
    // past the placed prefix and stops at the first sphere that found no place
    const int64_t W = std::min<int64_t>(32768, std::max<int64_t>(256, n / 64));
    const int kRoundsPerCheck = 16;
    std::vector<int32_t> hState((size_t)std::min<int64_t>(n, W));
    int64_t w0 = 0, prefix = n;
    while (w0 < n) {
        const int64_t w1 = std::min<int64_t>(n, w0 + W);
        const unsigned g = (unsigned)((w1 - w0 + 255) / 256);
        for (int round = 0; round < kRoundsPerCheck; round++) {
            k_rsa_draw<<<g, 256, 0, st>>>(G, w0, w1, dRad, seed, dState, dAtt, dCand, dClear, dHeadP, dNextP, dPos, dHeadR, dNextR);
            k_rsa_resolve<<<g, 256, 0, st>>>(G, w0, w1, dRad, max_attempts, dState, dAtt, dCand, dClear, dHeadR, dNextR, dAcc);
            k_rsa_commit<<<g, 256, 0, st>>>(G, w0, w1, dState, dCand, dClear, dAcc, dPos, dHeadP, dNextP, dHeadR);
        }
        if (cudaMemcpyAsync(hState.data(), dState + w0, sizeof(int32_t) * (w1 - w0), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return -1;
        int64_t k = 0;
        while (k < w1 - w0 && hState[(size_t)k] == 1) k++;
        if (k < w1 - w0 && hState[(size_t)k] == 2) {
            prefix = w0 + k;
            break;
        }
        w0 += k;
    }
    if (prefix > 0 && (cudaMemcpyAsync(centers, dPos, sizeof(double) * 3 * prefix, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                       cudaStreamSynchronize(st) != cudaSuccess))
        return -1;
    if (cudaGetLastError() != cudaSuccess) return -1;
    return prefix;
}

}  // extern "C"
