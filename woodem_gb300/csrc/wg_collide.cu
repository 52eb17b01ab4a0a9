// Broad phase: the full run of InsertionSortCollider (pkg/dem/InsertionSortCollider.cpp:445-646).
//
// The reference maintains three insertion-sorted bound arrays; every min/max inversion
// creates a potential contact when the closed 3-axis AABB test passes (:52-58, :63-98) or
// removes a non-real contact when the boxes separate. After each full run its contact set
// is therefore
//     { (i,j) : closed AABB overlap of i and j, Collider::mayCollide(i,j) }  U  { real contacts },
// and pending (law-removed) contacts survive only while their boxes overlap
// (ContactContainer::removePending, ContactContainer.hpp:78-93). This file computes exactly
// that set on the GPU:
//   1. Bo1 functors + verlet enlargement per particle            (k_aabb)
//   2. spheres bucketed into a uniform grid whose cell is at least the largest sphere box,
//      keyed by the cell of the box minimum and radix-sorted      (k_cellkey + cub radix sort)
//   3. half-shell sweep over the sorted cells: every candidate pair is tested once with the
//      reference's closed-interval comparisons                   (k_pairs_ss)
//   4. facets query the cells their box covers; walls (infinite boxes) test every sphere
//   5. the new pair keys are radix-sorted and merged with the real contacts of the previous
//      set, carrying their persistent state                      (k_mark_orphans .. k_gather)
//   6. CSR incidence for the deterministic force sum              (k_lo_start, hi sort, k_hi_start)
#include <cub/cub.cuh>


#include <algorithm>
#include <cmath>

#include "wg_internal.h"
#include "wg_math.cuh"
#include "wg_ends.cuh"
#include "wg_geom.cuh"

namespace wg {

struct CollideWork {
    // sphere and "large" (non-sphere) id lists, built at upload
    int32_t* sphereIds = nullptr;
    int nSph = 0;
    int32_t* largeIds = nullptr;   // facets with finite boxes (cell query)
    int nLarge = 0;
    int32_t* globalIds = nullptr;  // walls and oversized boxes (tested against every sphere)
    int nGlobal = 0;
    bool largeLargePossible = false;
    std::vector<int32_t> hLarge, hGlobal;
    // grid scratch
    uint32_t* cellKey = nullptr;
    uint32_t* cellKeySorted = nullptr;
    int32_t* cellVal = nullptr;
    int32_t* sid = nullptr;       // sorted sphere ids
    double4_32a* smn = nullptr;
    double4_32a* smx = nullptr;
    uint32_t* smask = nullptr;
    float4* smnf = nullptr;       // box min rounded down, mask in w
    float4* smxf = nullptr;       // box max rounded up, particle id in w
    int32_t* newLo = nullptr;     // first index of each lo id in the sorted new pairs (merge)
    int32_t* oldLo = nullptr;     // the same in the previous contact keys
    int64_t newLoCap = 0, oldLoCap = 0;
    float4* smnfi = nullptr;      // box min rounded up (inward)
    float4* smxfi = nullptr;      // box max rounded down (inward)
    int32_t* cellOff = nullptr;
    int64_t cellOffCap = 0;
    double* red = nullptr;        // reduction partials
    double* hRed = nullptr;       // pinned
    std::vector<int32_t> hChunk;      // grid-reduction chunks of sphereIds (never across scenes)
    std::vector<int32_t> hSceneChunk; // chunks of scene k: [hSceneChunk[k], hSceneChunk[k+1])
    std::vector<int64_t> hSceneSph;   // spheres of scene k: sphereIds[hSceneSph[k] .. hSceneSph[k+1])
    int32_t* dChunk = nullptr;
    Grid* dGrids = nullptr;
    bool chunksDirty = true;
    int32_t* gStart = nullptr;        // walls of scene k in globalIds (batches)
    // pairs
    uint64_t* pairs = nullptr;
    uint64_t* pairsSorted = nullptr;
    int64_t pairCap = 0;
    int32_t* pairCd = nullptr;        // periodic: cell distance of each new pair
    int32_t* pairCdSorted = nullptr;
    int64_t pairCdCap = 0;
    int32_t* newCd = nullptr;         // periodic: cell distance per merged contact
    int64_t newCdCap = 0;
    unsigned long long* counter = nullptr;
    unsigned long long* hCounter = nullptr;
    // merge scratch
    int32_t* orph = nullptr;      // flags then exclusive scan
    uint64_t* orphKey = nullptr;
    int32_t* orphSrc = nullptr;
    int32_t* src = nullptr;
    int64_t mergeCap = 0, orphCap = 0, srcCap = 0;
    int32_t* act = nullptr;       // exclusive scan of the active contacts
    int32_t* actSS = nullptr;     // exclusive scan of the active sphere-sphere contacts
    uint32_t* hiKeys = nullptr;
    uint32_t* hiKeysSorted = nullptr;
    int32_t* hiVals = nullptr;
    int64_t hiCap = 0;
    int32_t* heavyCount = nullptr;
    int32_t* hHeavy = nullptr;
    void* cubTmp = nullptr;
    size_t cubBytes = 0;
};

static const int BS = 256;

// ---------------------------------------------------------------- Bo1 functors + verlet
// Bo1_Sphere_Aabb::go pkg/dem/Sphere.cpp:50-79, Bo1_Wall_Aabb::go pkg/dem/Wall.cpp:24-33,
// Bo1_Facet_Aabb::go pkg/dem/Facet.cpp:177-200; enlargement by verletDist and nodeLastPos
// bookkeeping of updateBboxes_doFullRun pkg/dem/InsertionSortCollider.cpp:386-414.
__global__ void k_aabb(DevNodes N, DevParticles P, const ScenePar* __restrict__ spp, int* __restrict__ dErr) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    const ScenePar& sp = spp[sceneOfP(P, p)];
    const int sh = P.shape[p];
    D3 mn, mx;
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    if (sh == WG_SHAPE_SPHERE) {
        const double4_32a pr = N.posr[p];
        const double f = (sp.bo1DistFactor > 0 ? sp.bo1DistFactor : 1.) * pr.w;
        D3 h{f, f, f};
        const D3 pos{pr.x, pr.y, pr.z};
        if (!sp.periodic) {
            mn = pos - h;
            mx = pos + h;
        } else {
            if (sp.hasShear) {
                const D3 perp = h;
                for (int ax = 0; ax < 3; ax++) {
                    const int ax1 = (ax + 1) % 3, ax2 = (ax + 2) % 3;
                    setComp(h, ax1, comp(h, ax1) + .5 * comp(perp, ax1) * (1 / sp.cellCos[ax] - 1));
                    setComp(h, ax2, comp(h, ax2) + .5 * comp(perp, ax2) * (1 / sp.cellCos[ax] - 1));
                }
            }
            DM3 U;
            for (int k = 0; k < 9; k++) U.m[k] = sp.unshear[k];
            const D3 u = mul(U, pos);
            mn = u - h;
            mx = u + h;
        }
        N.lastPos[p] = make_double4_32a(pr.x, pr.y, pr.z, 0.);
        if (N.lh) {
            N.lh[p] = N.mir[p].ph;
            N.ll[p] = N.mir[p].pl;
        }
    } else if (sh == WG_SHAPE_WALL) {
        const int ax = P.aux[p].x;
        const double4_32a pr = N.posr[p];
        mn = D3{-inf, -inf, -inf};
        mx = D3{inf, inf, inf};
        setComp(mn, ax, comp(D3{pr.x, pr.y, pr.z}, ax));
        setComp(mx, ax, comp(D3{pr.x, pr.y, pr.z}, ax));
        N.lastPos[p] = make_double4_32a(pr.x, pr.y, pr.z, 0.);
        if (N.lh) {
            N.lh[p] = N.mir[p].ph;
            N.ll[p] = N.mir[p].pl;
        }
    } else {
        const int4 fn = P.aux[p];
        const double ht = P.facet[p].w;
        const D3 htv{ht, ht, ht};
        const int nn[3] = {fn.x, fn.y, fn.z};
        for (int k = 0; k < 3; k++) {
            const double4_32a pr = N.posr[nn[k]];
            D3 v{pr.x, pr.y, pr.z};
            if (sp.periodic) {
                DM3 U;
                for (int q = 0; q < 9; q++) U.m[q] = sp.unshear[q];
                v = mul(U, v);
            }
            const D3 a = v - htv, b = v + htv;
            if (k == 0) {
                mn = a;
                mx = b;
            } else {
                mn = D3{smin(mn.x, a.x), smin(mn.y, a.y), smin(mn.z, a.z)};
                mx = D3{smax(mx.x, b.x), smax(mx.y, b.y), smax(mx.z, b.z)};
            }
            N.lastPos[nn[k]] = make_double4_32a(pr.x, pr.y, pr.z, 0.);
            if (N.lh) {
                N.lh[nn[k]] = N.mir[nn[k]].ph;
                N.ll[nn[k]] = N.mir[nn[k]].pl;
            }
        }
        N.lastPos[p] = N.posr[p];
        if (N.lh) {
            N.lh[p] = N.mir[p].ph;
            N.ll[p] = N.mir[p].pl;
        }
    }
    if (sp.verletDist > 0) {
        const D3 vd{sp.verletDist, sp.verletDist, sp.verletDist};
        mx = mx + vd;
        mn = mn - vd;
    }
    // a NaN coordinate would silently drop the particle from every pair test: stop the run instead
    if (isnan(mn.x) || isnan(mn.y) || isnan(mn.z) || isnan(mx.x) || isnan(mx.y) || isnan(mx.z)) atomicCAS(dErr, 0, 102);
    P.mn[p] = make_double4_32a(mn.x, mn.y, mn.z, 0.);
    P.mx[p] = make_double4_32a(mx.x, mx.y, mx.z, 0.);
}

// ---------------------------------------------------------------- grid bounds over spheres
// partial[b] = {min mn.x, min mn.y, min mn.z, max mn.x, max mn.y, max mn.z, max extent} over the
// spheres ids[chunk[b] .. chunk[b+1]) (chunks never span two scenes of a batch)
__global__ void k_grid_reduce(DevParticles P, const int32_t* __restrict__ ids, const int32_t* __restrict__ chunk,
                              double* __restrict__ partial) {
    __shared__ double s[7][BS];
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    double v[7] = {inf, inf, inf, -inf, -inf, -inf, 0.};
    for (int i = chunk[blockIdx.x] + threadIdx.x; i < chunk[blockIdx.x + 1]; i += blockDim.x) {
        const int p = ids[i];
        const double4_32a a = P.mn[p], b = P.mx[p];
        v[0] = fmin(v[0], a.x); v[1] = fmin(v[1], a.y); v[2] = fmin(v[2], a.z);
        v[3] = fmax(v[3], a.x); v[4] = fmax(v[4], a.y); v[5] = fmax(v[5], a.z);
        v[6] = fmax(v[6], fmax(fmax(b.x - a.x, b.y - a.y), b.z - a.z));
    }
    for (int q = 0; q < 7; q++) s[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            for (int q = 0; q < 3; q++) s[q][threadIdx.x] = fmin(s[q][threadIdx.x], s[q][threadIdx.x + st]);
            for (int q = 3; q < 7; q++) s[q][threadIdx.x] = fmax(s[q][threadIdx.x], s[q][threadIdx.x + st]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 7; q++) partial[blockIdx.x * 7 + q] = s[q][0];
}

__device__ __forceinline__ int cellCoord(double v, double o, double h, int n) {
    double c = floor((v - o) / h);
    int ci = (int)c;
    return ci < 0 ? 0 : (ci >= n ? n - 1 : ci);
}

__global__ void k_cellkey(DevParticles P, const int32_t* __restrict__ ids, int n, const Grid* __restrict__ Gs,
                          uint32_t* __restrict__ key, int32_t* __restrict__ val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = ids[i];
    const Grid G = Gs[sceneOfP(P, p)];
    const double4_32a a = P.mn[p];
    const int cx = cellCoord(a.x, G.ox, G.h, G.nx), cy = cellCoord(a.y, G.oy, G.h, G.ny), cz = cellCoord(a.z, G.oz, G.h, G.nz);
    key[i] = (uint32_t)(G.base + ((int64_t)cz * G.ny + cy) * G.nx + cx);
    val[i] = p;
}

__device__ __forceinline__ int64_t lowerBound32(const uint32_t* a, int64_t n, uint32_t k) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t m = (lo + hi) >> 1;
        if (a[m] < k) lo = m + 1; else hi = m;
    }
    return lo;
}
__device__ __forceinline__ int64_t lowerBound64(const uint64_t* a, int64_t n, uint64_t k) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t m = (lo + hi) >> 1;
        if (a[m] < k) lo = m + 1; else hi = m;
    }
    return lo;
}

// cellOff[k] = number of sorted spheres with cell key < k, k in [0, ncell]
__global__ void k_cell_off(const uint32_t* __restrict__ skey, int n, int64_t ncell, int32_t* __restrict__ off) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k > ncell) return;
    off[k] = (int32_t)lowerBound32(skey, n, (uint32_t)k);
}

__global__ void k_gather_sorted(DevParticles P, const int32_t* __restrict__ sid, int n, double4_32a* __restrict__ smn,
                                double4_32a* __restrict__ smx, uint32_t* __restrict__ smask, float4* __restrict__ smnf,
                                float4* __restrict__ smxf, float4* __restrict__ smnfi, float4* __restrict__ smxfi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = sid[i];
    const double4_32a a = P.mn[p], b = P.mx[p];
    const uint32_t m = P.mask[p];
    smn[i] = a;
    smx[i] = b;
    smask[i] = m;
    smnf[i] = make_float4(__double2float_rd(a.x), __double2float_rd(a.y), __double2float_rd(a.z), __uint_as_float(m));
    smxf[i] = make_float4(__double2float_ru(b.x), __double2float_ru(b.y), __double2float_ru(b.z), __int_as_float(p));
    smnfi[i] = make_float4(__double2float_ru(a.x), __double2float_ru(a.y), __double2float_ru(a.z), 0.f);
    smxfi[i] = make_float4(__double2float_rd(b.x), __double2float_rd(b.y), __double2float_rd(b.z), 0.f);
}

// Collider::mayCollide pkg/dem/Collision.cpp:19-41 for particles that share no nodes
__device__ __forceinline__ bool maskOk(uint32_t a, uint32_t b, uint32_t lone) { return (a & b) != 0 && (a & b & lone) == 0; }

__device__ __forceinline__ void emitPair(int a, int b, uint64_t* pairs, int64_t cap, unsigned long long* counter) {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const unsigned long long idx = atomicAdd(counter, 1ull);
    if ((int64_t)idx < cap) pairs[idx] = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
}

// Outward-rounded FP32 boxes overlap whenever the FP64 boxes do, so the FP32 test rejects most
// candidates exactly; inward-rounded boxes (min up, max down) overlap only if the FP64 boxes do,
// so they accept most of the rest exactly, and the FP64 test (InsertionSortCollider::spatialOverlap)
// decides the cases where a bound lies within one FP32 rounding of the other.
__device__ __forceinline__ bool overlapF(const float4& mn1, const float4& mx1, const float4& mn2, const float4& mx2) {
    return (mn1.x <= mx2.x) && (mx1.x >= mn2.x) && (mn1.y <= mx2.y) && (mx1.y >= mn2.y) && (mn1.z <= mx2.z) && (mx1.z >= mn2.z);
}
// the FP64 closed overlap of sorted boxes i and j whose outward-rounded boxes overlap
__device__ __forceinline__ bool overlapSorted(int i, int j, const double4_32a* __restrict__ smn, const double4_32a* __restrict__ smx,
                                              const float4* __restrict__ smnfi, const float4* __restrict__ smxfi) {
    if (overlapF(smnfi[i], smxfi[i], smnfi[j], smxfi[j])) return true;
    return overlap3(smn[i], smx[i], smn[j], smx[j]);
}

// Pairs found by the lanes of a warp are written with one atomic per warp: each lane keeps up to
// kPairBuf pairs in registers, the warp reserves room for all of them at once (the single counter
// would otherwise serialise millions of atomics in L2), and a lane whose buffer fills flushes it
// the same way. Must be called by all lanes of the warp together.
constexpr int kPairBuf = 8;
__device__ __forceinline__ void flushPairs(uint64_t (&buf)[kPairBuf], int& nb, uint64_t* pairs, int64_t cap,
                                           unsigned long long* counter) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int incl = nb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(counter, (unsigned long long)total);
    base = __shfl_sync(FULL, base, 31);
    const unsigned long long at = base + (unsigned long long)(incl - nb);
#pragma unroll
    for (int q = 0; q < kPairBuf; q++)
        if (q < nb && (int64_t)(at + q) < cap) pairs[at + q] = buf[q];
    nb = 0;
}
__device__ __forceinline__ uint64_t pairKey(int a, int b) {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    return ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
}

// Appends key to the lane's pair buffer (register-resident: the slot is chosen by unrolled
// comparisons, never by a runtime index).
__device__ __forceinline__ void pushPair(uint64_t (&buf)[kPairBuf], int& nb, uint64_t key) {
#pragma unroll
    for (int q = 0; q < kPairBuf; q++)
        if (q == nb) buf[q] = key;
    nb++;
}

// Half-shell sweep: particle i tests the rest of its own cell, the next cell in x, and the
// three-cell x-runs of the rows (dy,dz) in {(1,0),(-1,1),(0,1),(1,1)}; each pair is met once.
// The candidate ranges of a lane are walked as one sequence, kSweepBatch candidates at a time
// (their boxes are loaded together), so that the warp can flush together.
constexpr int kSweepBatch = 2;
__global__ void __launch_bounds__(256, 4) k_pairs_ss(const uint32_t* __restrict__ skey, const double4_32a* __restrict__ smn,
                           const double4_32a* __restrict__ smx, const float4* __restrict__ smnf, const float4* __restrict__ smxf,
                           const float4* __restrict__ smnfi, const float4* __restrict__ smxfi,
                           int n, const Grid* __restrict__ Gs, const int32_t* __restrict__ pscene, const int32_t* __restrict__ off,
                           uint32_t lone, uint64_t* __restrict__ pairs, int64_t cap, unsigned long long* __restrict__ counter) {
    const unsigned FULL = 0xffffffffu;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    // the five ranges [b_r, b_r + len_r) of sorted indices, as starts and cumulative lengths
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0, total = 0;
    float4 fn1 = make_float4(0.f, 0.f, 0.f, 0.f), fx1 = fn1;
    uint32_t m1 = 0;
    int pi = 0;
    if (valid) {
        fn1 = smnf[i];
        fx1 = smxf[i];
        m1 = __float_as_uint(fn1.w);
        pi = __float_as_int(fx1.w);
        const Grid G = Gs[pscene ? pscene[pi] : 0];
        const uint32_t k = (uint32_t)((int64_t)skey[i] - G.base);
        const int cx = (int)(k % (uint32_t)G.nx);
        const int cy = (int)((k / (uint32_t)G.nx) % (uint32_t)G.ny);
        const int cz = (int)(k / ((uint32_t)G.nx * (uint32_t)G.ny));
        const int cx1 = cx + 1 < G.nx ? cx + 1 : cx;
        const int x0 = cx > 0 ? cx - 1 : 0;
        int rb[4], re[4];
        const int DY[4] = {1, -1, 0, 1}, DZ[4] = {0, 1, 1, 1};
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int y = cy + DY[r], z = cz + DZ[r];
            rb[r] = re[r] = 0;
            if (y < 0 || y >= G.ny || z >= G.nz) continue;
            const int64_t rowBase = G.base + ((int64_t)z * G.ny + y) * G.nx;
            rb[r] = off[rowBase + x0];
            re[r] = off[rowBase + cx1 + 1];
        }
        b0 = i + 1;
        c1 = off[G.base + ((int64_t)cz * G.ny + cy) * G.nx + cx1 + 1] - b0;
        b1 = rb[0];
        c2 = c1 + (re[0] - rb[0]);
        b2 = rb[1];
        c3 = c2 + (re[1] - rb[1]);
        b3 = rb[2];
        c4 = c3 + (re[2] - rb[2]);
        b4 = rb[3];
        total = c4 + (re[3] - rb[3]);
    }
    uint64_t buf[kPairBuf];
    int nb = 0;
    for (int v0 = 0; __any_sync(FULL, v0 < total); v0 += kSweepBatch) {
        int jj[kSweepBatch];
        float4 a[kSweepBatch], c[kSweepBatch];
#pragma unroll
        for (int u = 0; u < kSweepBatch; u++) {
            const int v = v0 + u;
            jj[u] = v >= total ? -1
                               : (v < c1 ? b0 + v : (v < c2 ? b1 + (v - c1) : (v < c3 ? b2 + (v - c2) : (v < c4 ? b3 + (v - c3) : b4 + (v - c4)))));
            if (jj[u] >= 0) {
                a[u] = smnf[jj[u]];
                c[u] = smxf[jj[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < kSweepBatch; u++)
            if (jj[u] >= 0 && overlapF(fn1, fx1, a[u], c[u]) && maskOk(m1, __float_as_uint(a[u].w), lone) &&
                overlapSorted(i, jj[u], smn, smx, smnfi, smxfi))
                pushPair(buf, nb, pairKey(pi, __float_as_int(c[u].w)));
        if (__any_sync(FULL, nb > kPairBuf - kSweepBatch)) flushPairs(buf, nb, pairs, cap, counter);
    }
    flushPairs(buf, nb, pairs, cap, counter);
}

// A facet (finite box) against the spheres of the cells its box can reach: a sphere j that
// overlaps it has mn_j in [mn_f - h, mx_f] on every axis. One warp per facet; its lanes split
// each x-run of cells.
__global__ void k_pairs_local(DevParticles P, const int32_t* __restrict__ lids, int nl, const double4_32a* __restrict__ smn,
                              const double4_32a* __restrict__ smx, const float4* __restrict__ smnf, const float4* __restrict__ smxf,
                              const float4* __restrict__ smnfi, const float4* __restrict__ smxfi, const Grid* __restrict__ Gs, const int32_t* __restrict__ off, uint32_t lone, uint64_t* __restrict__ pairs,
                              int64_t cap, unsigned long long* __restrict__ counter) {
    const unsigned FULL = 0xffffffffu;
    const int t = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= nl) return;  // warp-uniform
    const int p = lids[t];
    const Grid G = Gs[sceneOfP(P, p)];
    const double4_32a mn1 = P.mn[p], mx1 = P.mx[p];
    const float4 fn1 = make_float4(__double2float_rd(mn1.x), __double2float_rd(mn1.y), __double2float_rd(mn1.z), 0.f);
    const float4 fx1 = make_float4(__double2float_ru(mx1.x), __double2float_ru(mx1.y), __double2float_ru(mx1.z), 0.f);
    const float4 fni1 = make_float4(__double2float_ru(mn1.x), __double2float_ru(mn1.y), __double2float_ru(mn1.z), 0.f);
    const float4 fxi1 = make_float4(__double2float_rd(mx1.x), __double2float_rd(mx1.y), __double2float_rd(mx1.z), 0.f);
    const uint32_t m1 = P.mask[p];
    const int x0 = cellCoord(mn1.x - G.h, G.ox, G.h, G.nx), x1 = cellCoord(mx1.x, G.ox, G.h, G.nx);
    const int y0 = cellCoord(mn1.y - G.h, G.oy, G.h, G.ny), y1 = cellCoord(mx1.y, G.oy, G.h, G.ny);
    const int z0 = cellCoord(mn1.z - G.h, G.oz, G.h, G.nz), z1 = cellCoord(mx1.z, G.oz, G.h, G.nz);
    uint64_t buf[kPairBuf];
    int nb = 0;
    for (int z = z0; z <= z1; z++)
        for (int y = y0; y <= y1; y++) {
            const int64_t rowBase = G.base + ((int64_t)z * G.ny + y) * G.nx;
            const int beg = off[rowBase + x0], end = off[rowBase + x1 + 1];
            for (int j0 = beg; j0 < end; j0 += 32) {
                const int j = j0 + lane;
                if (j < end) {
                    const float4 fn2 = smnf[j], fx2 = smxf[j];
                    const int q = __float_as_int(fx2.w);
                    if (q != p && overlapF(fn1, fx1, fn2, fx2) && maskOk(m1, __float_as_uint(fn2.w), lone) &&
                        (overlapF(fni1, fxi1, smnfi[j], smxfi[j]) || overlap3(mn1, mx1, smn[j], smx[j])))
                        pushPair(buf, nb, pairKey(p, q));
                }
                if (__any_sync(FULL, nb == kPairBuf)) flushPairs(buf, nb, pairs, cap, counter);
            }
        }
    flushPairs(buf, nb, pairs, cap, counter);
}

// ---------------------------------------------------------------- periodic cell
__global__ void k_cellkey_peri(DevParticles P, const int32_t* __restrict__ ids, int n, Grid G, const ScenePar* __restrict__ spp,
                               uint32_t* __restrict__ key, int32_t* __restrict__ val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ScenePar& sp = *spp;
    const int p = ids[i];
    const double4_32a a = P.mn[p];
    const double w[3] = {cellWrapRelD(a.x, 0., sp.cellSize[0]), cellWrapRelD(a.y, 0., sp.cellSize[1]),
                         cellWrapRelD(a.z, 0., sp.cellSize[2])};
    const int nn[3] = {G.nx, G.ny, G.nz};
    int c[3];
    for (int k = 0; k < 3; k++) {
        const int ci = (int)floor(w[k] / (sp.cellSize[k] / nn[k]));
        c[k] = ci < 0 ? 0 : (ci >= nn[k] ? nn[k] - 1 : ci);
    }
    key[i] = (uint32_t)(((int64_t)c[2] * G.ny + c[1]) * G.nx + c[0]);
    val[i] = p;
}
// Pairs emitted with their cell distance (periods of the lo particle minus those of the hi one).
__device__ __forceinline__ void flushPairsCd(uint64_t (&buf)[kPairBuf], int32_t (&cbuf)[kPairBuf], int& nb, uint64_t* pairs,
                                             int32_t* cds, int64_t cap, unsigned long long* counter) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int incl = nb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(counter, (unsigned long long)total);
    base = __shfl_sync(FULL, base, 31);
    const unsigned long long at = base + (unsigned long long)(incl - nb);
#pragma unroll
    for (int q = 0; q < kPairBuf; q++)
        if (q < nb && (int64_t)(at + q) < cap) {
            pairs[at + q] = buf[q];
            cds[at + q] = cbuf[q];
        }
    nb = 0;
}
// Periodic sweep: particle i tests the spheres of higher id in the (up to 27, wrapped, distinct)
// cells around its own with the periodic overlap test; each pair is met once, from its lo id.
__global__ void k_pairs_ss_peri(const uint32_t* __restrict__ skey, const int32_t* __restrict__ sid, const double4_32a* __restrict__ smn,
                                const double4_32a* __restrict__ smx, const uint32_t* __restrict__ smask, int n, Grid G,
                                const int32_t* __restrict__ off, uint32_t lone, const ScenePar* __restrict__ spp,
                                uint64_t* __restrict__ pairs, int32_t* __restrict__ cds, int64_t cap,
                                unsigned long long* __restrict__ counter, int* __restrict__ dErr) {
    const unsigned FULL = 0xffffffffu;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const ScenePar& sp = *spp;
    int cx = 0, cy = 0, cz = 0, pi = 0;
    uint32_t m1 = 0;
    double4_32a mn1 = make_double4_32a(0., 0., 0., 0.), mx1 = mn1;
    if (valid) {
        const uint32_t k = skey[i];
        cx = (int)(k % (uint32_t)G.nx);
        cy = (int)((k / (uint32_t)G.nx) % (uint32_t)G.ny);
        cz = (int)(k / ((uint32_t)G.nx * (uint32_t)G.ny));
        pi = sid[i];
        m1 = smask[i];
        mn1 = smn[i];
        mx1 = smx[i];
    }
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    // distinct wrapped offsets per axis
    const int ox = nx >= 3 ? 3 : nx, oy = ny >= 3 ? 3 : ny, oz = nz >= 3 ? 3 : nz;
    uint64_t buf[kPairBuf];
    int32_t cbuf[kPairBuf];
    int nb = 0;
    for (int q = 0; q < ox * oy * oz; q++) {
        const int dx = q % ox - (ox == 3 ? 1 : 0), dy = (q / ox) % oy - (oy == 3 ? 1 : 0), dz = q / (ox * oy) - (oz == 3 ? 1 : 0);
        const int x = ((cx + dx) % nx + nx) % nx, y = ((cy + dy) % ny + ny) % ny, z = ((cz + dz) % nz + nz) % nz;
        const int64_t cell = ((int64_t)z * ny + y) * nx + x;
        const int beg = valid ? off[cell] : 0, end = valid ? off[cell + 1] : 0;
        int j = beg;
        for (;;) {
            const bool has = j < end;
            if (!__any_sync(FULL, has)) break;
            if (has) {
                const int pj = sid[j];
                if (pj > pi && maskOk(m1, smask[j], lone)) {
                    int per[3];
                    const int r = overlapPeri(mn1, mx1, smn[j], smx[j], sp.cellSize, per);
                    if (r < 0) atomicCAS(dErr, 0, 103);
                    else if (r > 0) {
                        const uint64_t key = pairKey(pi, pj);
                        const int32_t cd = packCellDist(per[0], per[1], per[2]);
#pragma unroll
                        for (int q = 0; q < kPairBuf; q++)
                            if (q == nb) {
                                buf[q] = key;
                                cbuf[q] = cd;
                            }
                        nb++;
                    }
                }
                j++;
            }
            if (__any_sync(FULL, nb == kPairBuf)) flushPairsCd(buf, cbuf, nb, pairs, cds, cap, counter);
        }
    }
    flushPairsCd(buf, cbuf, nb, pairs, cds, cap, counter);
}
// Walls against every sphere with the periodic overlap test (pair oriented lo, hi).
__global__ void k_pairs_global_peri(DevParticles P, const int32_t* __restrict__ gids, int ng, const int32_t* __restrict__ sph, int ns,
                                    uint32_t lone, const ScenePar* __restrict__ spp, uint64_t* __restrict__ pairs,
                                    int32_t* __restrict__ cds, int64_t cap, unsigned long long* __restrict__ counter,
                                    int* __restrict__ dErr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns) return;
    const int s = sph[i];
    for (int g = 0; g < ng; g++) {
        const int w = gids[g];
        if (w == s || !maskOk(P.mask[s], P.mask[w], lone)) continue;
        const int lo = s < w ? s : w, hi = s < w ? w : s;
        int per[3];
        const int r = overlapPeri(P.mn[lo], P.mx[lo], P.mn[hi], P.mx[hi], spp->cellSize, per);
        if (r < 0) atomicCAS(dErr, 0, 103);
        else if (r > 0) {
            const unsigned long long idx = atomicAdd(counter, 1ull);
            if ((int64_t)idx < cap) {
                pairs[idx] = pairKey(lo, hi);
                cds[idx] = packCellDist(per[0], per[1], per[2]);
            }
        }
    }
}

// Walls (and any box too large for the grid) against every sphere.
// gids are grouped by scene: the walls of scene k are gids[gStart[k] .. gStart[k+1]) (gStart null:
// one scene, all of gids)
__global__ void k_pairs_global(DevParticles P, const int32_t* __restrict__ gids, int ng, const int32_t* __restrict__ gStart,
                               const int32_t* __restrict__ sph, int ns, uint32_t lone, uint64_t* __restrict__ pairs, int64_t cap,
                               unsigned long long* __restrict__ counter) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns) return;
    const int s = sph[i];
    const double4_32a mn1 = P.mn[s], mx1 = P.mx[s];
    const uint32_t m1 = P.mask[s];
    const int sc = sceneOfP(P, s);
    const int g0 = gStart ? gStart[sc] : 0, g1 = gStart ? gStart[sc + 1] : ng;
    for (int g = g0; g < g1; g++) {
        const int w = gids[g];
        if (w == s) continue;
        if (overlap3(mn1, mx1, P.mn[w], P.mx[w]) && maskOk(m1, P.mask[w], lone)) emitPair(s, w, pairs, cap, counter);
    }
}

// Pairs among non-spheres (only launched when their masks allow contact at all).
__global__ void k_pairs_large_large(DevParticles P, const int32_t* __restrict__ ids, int n, uint32_t lone,
                                    uint64_t* __restrict__ pairs, int64_t cap, unsigned long long* __restrict__ counter) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * n) return;
    const int a = (int)(t / n), b = (int)(t % n);
    if (b <= a) return;
    const int pa = ids[a], pb = ids[b];
    if (sceneOfP(P, pa) != sceneOfP(P, pb)) return;  // the scenes of a batch never interact
    // facets sharing a node may not collide (Collision.cpp:27-31)
    if (P.shape[pa] == WG_SHAPE_FACET && P.shape[pb] == WG_SHAPE_FACET) {
        const int4 x = P.aux[pa], y = P.aux[pb];
        const int xa[3] = {x.x, x.y, x.z}, ya[3] = {y.x, y.y, y.z};
        for (int u = 0; u < 3; u++)
            for (int v = 0; v < 3; v++)
                if (xa[u] == ya[v]) return;
    }
    if (overlap3(P.mn[pa], P.mx[pa], P.mn[pb], P.mx[pb]) && maskOk(P.mask[pa], P.mask[pb], lone)) emitPair(pa, pb, pairs, cap, counter);
}

// ---------------------------------------------------------------- merge with previous contacts
// a contact of a particle that was (re)loaded or parked since the last full run does not survive
__device__ __forceinline__ bool freshPair(const uint8_t* fresh, uint64_t k) {
    return fresh && (fresh[(int)(k >> 32)] || fresh[(int)(k & 0xffffffffu)]);
}
// start[p] = first index of key array (sorted ascending, key = lo << 32 | hi) whose lo is >= p,
// for p in [0, nPar]; one thread per index fills the ids between its lo and its predecessor's.
__global__ void k_lo_bounds(const uint64_t* __restrict__ key, int64_t n, int nPar, int32_t* __restrict__ start) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    const int cur = (i < n) ? (int)(key[i] >> 32) : nPar;
    const int prev = (i > 0) ? (int)(key[i - 1] >> 32) : -1;
    for (int q = prev + 1; q <= cur && q <= nPar; q++) start[q] = (int32_t)i;
}
// position of k in the sorted key array, searched within the range of its lo id (a few entries
// for a sphere, thousands for a wall), or -1
__device__ __forceinline__ int64_t findInRange(const uint64_t* __restrict__ key, const int32_t* __restrict__ start, uint64_t k) {
    const int lo = (int)(k >> 32);
    int64_t a = start[lo], b = start[lo + 1];
    while (a < b) {
        const int64_t m = (a + b) >> 1;
        if (key[m] < k) a = m + 1;
        else b = m;
    }
    return (a < start[lo + 1] && key[a] == k) ? a : -1;
}
// pair keys (lo << 32 | hi) to (lo << bits | hi) for the sort, and back
__global__ void k_pack_keys(uint64_t* __restrict__ k, int64_t n, int bits) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) k[i] = ((k[i] >> 32) << bits) | (k[i] & 0xffffffffu);
}
__global__ void k_unpack_keys(uint64_t* __restrict__ k, int64_t n, int bits) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) k[i] = ((k[i] >> bits) << 32) | (k[i] & ((1ull << bits) - 1));
}
__global__ void k_mark_orphans(DevContacts C, const uint64_t* __restrict__ nk, const int32_t* __restrict__ newLo,
                               int32_t* __restrict__ orph, const uint8_t* __restrict__ fresh) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= C.n) return;
    int32_t o = 0;
    if ((C.flags[j] & C_REAL) && !freshPair(fresh, C.key[j])) o = findInRange(nk, newLo, C.key[j]) < 0 ? 1 : 0;
    orph[j] = o;
}
__global__ void k_compact_orphans(DevContacts C, const int32_t* __restrict__ orphFlag, const int32_t* __restrict__ orphScan,
                                  uint64_t* __restrict__ okey, int32_t* __restrict__ osrc) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= C.n) return;
    if (orphFlag[j]) {
        const int32_t o = orphScan[j];
        okey[o] = C.key[j];
        osrc[o] = (int32_t)j;
    }
}
__global__ void k_place_new(const uint64_t* __restrict__ nk, int64_t nn, const uint64_t* __restrict__ okey, int64_t no,
                            const uint64_t* __restrict__ oldKey, const int32_t* __restrict__ oldLo, uint64_t* __restrict__ outKey,
                            int32_t* __restrict__ src, const int32_t* __restrict__ nkCd, int32_t* __restrict__ outCd,
                            const uint8_t* __restrict__ fresh) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const uint64_t k = nk[i];
    const int64_t out = i + lowerBound64(okey, no, k);
    const int64_t pos = oldLo ? findInRange(oldKey, oldLo, k) : -1;
    outKey[out] = k;
    src[out] = (pos >= 0 && !freshPair(fresh, k)) ? (int32_t)pos : -1;
    if (nkCd) outCd[out] = nkCd[i];
}
__global__ void k_place_orph(const uint64_t* __restrict__ nk, int64_t nn, const uint64_t* __restrict__ okey,
                             const int32_t* __restrict__ osrc, int64_t no, uint64_t* __restrict__ outKey, int32_t* __restrict__ src) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const uint64_t k = okey[o];
    const int64_t out = o + lowerBound64(nk, nn, k);
    outKey[out] = k;
    src[out] = osrc[o];
}
// carry persistent state of surviving contacts; new contacts get their functor type and orientation
// (CGeomDispatcher functor order: Facet/Wall first, ContactLoop.cpp:145-152)
__global__ void k_gather(DevContacts Cold, DevContacts Cnew, const int32_t* __restrict__ src, DevParticles P,
                         const long long* __restrict__ dStep, const int32_t* __restrict__ newCd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Cnew.n) return;
    const int32_t s0 = src[i];
    // a contact removed since the last full run comes back as a new one
    const int32_t s = (s0 >= 0 && (Cold.flags[s0] & C_REMOVED)) ? -1 : s0;
    // FP32-force mode carries the state of real contacts only (a contact that is not real has no
    // state any kernel reads; the listing reports zeros for it)
    const bool fp32 = Cnew.fcol[0] != nullptr;
    if (s >= 0) {
        const uint32_t fo = Cold.flags[s];
        Cnew.flags[i] = fo & ~(C_PENDING | C_DORMANT);
        Cnew.step0[i] = Cold.step0[s];
        Cnew.cdist[i] = Cold.cdist[s];
        if (!fp32 || (fo & C_REAL)) {
#pragma unroll
            for (int q = 0; q < CC_NCOL; q++)
                if (Cnew.col[q]) Cnew.col[q][i] = Cold.col[q][s];
#pragma unroll
            for (int q = 0; q < CF_NCOL; q++)
                if (Cnew.fcol[q]) Cnew.fcol[q][i] = Cold.fcol[q][s];
        }
    } else {
        const uint64_t k = Cnew.key[i];
        const int lo = (int)(k >> 32), hi = (int)(k & 0xffffffffu);
        const int tl = P.shape[lo], th = P.shape[hi];
        uint32_t fl = 0, ty = CT_NONE;
        const int a = (tl == WG_SHAPE_SPHERE) ? th : tl;
        const bool sphLo = (tl == WG_SHAPE_SPHERE), sphHi = (th == WG_SHAPE_SPHERE);
        if (sphLo && sphHi) ty = CT_SS;
        else if (sphLo || sphHi) {
            if (a == WG_SHAPE_FACET) ty = CT_FS;
            else if (a == WG_SHAPE_WALL) ty = CT_WS;
            if (sphLo) fl |= C_SWAP;  // the non-sphere (hi) becomes pA
        }
        fl |= ty << 2;
        Cnew.flags[i] = fl;
        Cnew.step0[i] = (int32_t)(*dStep);
        Cnew.cdist[i] = newCd ? newCd[i] : packCellDist(0, 0, 0);
        if (!fp32) {
#pragma unroll
            for (int q = 0; q < CC_NCOL; q++)
                if (Cnew.col[q]) Cnew.col[q][i] = 0.;
        }
    }
}

// Dormant contacts. Between two full runs no node moves farther than verletDist from the position
// it had at the first of them (the verlet test of Leapfrog triggers the next full run before that),
// so a pair that is not real and whose surfaces are more than 2*verletDist apart now cannot touch
// before the next full run: the geometry functor would reject it at every step until then. Such
// contacts stay in the container (they are potential contacts of the reference) but the contact
// kernels skip them. The bounds are taken with a relative margin of 1e-9, and only for aperiodic
// scenes (a periodic cell moves the images of the particles by itself).
// The FP64 tests of k_dormant (sphere-sphere without mirrors, wall-sphere, facet-sphere), out of
// line: inlined, they become predicated FP64 instructions in the warps of mirror-tested pairs.
__device__ __noinline__ bool dormantFarFP64(const DevNodes& N, const DevParticles& P, const ScenePar* __restrict__ spp, int scene,
                                            uint32_t ty, int A, int B) {
    const ScenePar& sp = spp[scene];
    const double m2 = 2 * sp.verletDist;
    bool far;
    const double4_32a pb = N.posr[B];
    if (ty == CT_SS) {
        const double4_32a pa = N.posr[A];
        const double dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
        const double reach = (fabs(sp.ssDistFactor) * (pa.w + pb.w) + m2) * (1 + 1e-9);
        far = dx * dx + dy * dy + dz * dz > reach * reach;
    } else if (ty == CT_WS) {
        const int4 ax = P.aux[A];
        const double4_32a pw = N.posr[A];
        const double d = (ax.x == 0 ? pb.x - pw.x : (ax.x == 1 ? pb.y - pw.y : pb.z - pw.z));
        far = fabs(d) > (pb.w + m2) * (1 + 1e-9);
    } else {
        // distance from the sphere centre to the triangle: to its plane when the projection falls
        // inside, else to the nearest edge; it bounds from below the distance the functor tests
        // (Facet.cpp:247-259), and every point of the triangle moves at most verletDist since its
        // vertices do
        const int4 nd = P.aux[A];
        const D3 p0 = ld3(N.posr[nd.x]), p1 = ld3(N.posr[nd.y]), p2 = ld3(N.posr[nd.z]);
        const D3 sC = ld3(pb);
        const D3 nn = cross(p1 - p0, p2 - p0);
        const double nl = sqrt(sqn(nn));
        far = false;
        if (nl > 0) {
            const D3 fN = nn / nl;
            const double planeDist = dot(sC - p0, fN);
            const D3 fC = sC - planeDist * fN;
            const bool inside = dot(cross(p1 - p0, nn), fC - p0) <= 0 && dot(cross(p2 - p1, nn), fC - p1) <= 0 &&
                                dot(cross(p0 - p2, nn), fC - p2) <= 0;
            double d2;
            if (inside) d2 = planeDist * planeDist;
            else {
                d2 = sqn(sC - closestSegmentPt(sC, p0, p1));
                d2 = fmin(d2, sqn(sC - closestSegmentPt(sC, p1, p2)));
                d2 = fmin(d2, sqn(sC - closestSegmentPt(sC, p2, p0)));
            }
            const double reach = (pb.w + P.facet[A].w + m2) * (1 + 1e-9);
            far = d2 > reach * reach;
        }
    }
    return far;
}
__global__ void k_dormant(DevContacts C, DevNodes N, DevParticles P, const ScenePar* __restrict__ spp) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C.n) return;
    const uint32_t fl = C.flags[c];
    if (fl & C_REAL) return;
    const uint32_t ty = ctype(fl);
    if (ty == CT_NONE) return;
    const uint64_t key = C.key[c];
    const int lo = (int)(key >> 32), hi = (int)(key & 0xffffffffu);
    const int A = (fl & C_SWAP) ? hi : lo, B = (fl & C_SWAP) ? lo : hi;
    const int scene = sceneOfP(P, B);
    bool far;
    if (ty == CT_SS && N.mir) {
        // FP32-force mode: the double-float mirrors of the positions, FP32 arithmetic; the
        // relative position carries ~47 bits and the squares and sums ~2^-22 relative error
        const ScenePar& sp = spp[scene];
        const float4 ha = N.mir[A].ph, la = N.mir[A].pl, hb = N.mir[B].ph, lb = N.mir[B].pl;
        float sx, tx, sy, ty_, sz, tz;
        dfDiff(ha.x, la.x, hb.x, lb.x, sx, tx);
        dfDiff(ha.y, la.y, hb.y, lb.y, sy, ty_);
        dfDiff(ha.z, la.z, hb.z, lb.z, sz, tz);
        const float dx = sx + tx, dy = sy + ty_, dz = sz + tz;
        const float reach = (sp.ssDfAbsF * (ha.w + hb.w) + sp.reach2F) * (1.f + 1e-5f);
        far = dx * dx + dy * dy + dz * dz > reach * reach;
    } else far = dormantFarFP64(N, P, spp, scene, ty, A, B);
    if (far) C.flags[c] = fl | C_DORMANT;
}

// ---------------------------------------------------------------- CSR incidence
// Only active contacts (a functor applies and the pair is not dormant) own end slots; act is
// their exclusive scan over the key-sorted contacts, act[n] = number of active contacts.
__device__ __forceinline__ bool activeContact(uint32_t fl) { return ctype(fl) != CT_NONE && !(fl & C_DORMANT); }
__global__ void k_active(const uint32_t* __restrict__ flags, int64_t n, int32_t* __restrict__ act, int32_t* __restrict__ actSS) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const uint32_t fl = flags[c];
    const bool a = activeContact(fl);
    act[c] = a ? 1 : 0;
    actSS[c] = (a && ctype(fl) == CT_SS) ? 1 : 0;
}
// loStart[p] = active contacts with lo < p
__global__ void k_lo_start(const uint64_t* __restrict__ key, int64_t n, int nPar, const int32_t* __restrict__ act,
                           int32_t* __restrict__ loStart) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > nPar) return;
    loStart[p] = act[lowerBound64(key, n, (uint64_t)(uint32_t)p << 32)];
}
// hi id of the active contacts, nPar for the others (sorted past every particle)
__global__ void k_hi_keys(const uint64_t* __restrict__ key, const uint32_t* __restrict__ flags, int64_t n, uint32_t nPar,
                          uint32_t* __restrict__ hk, int32_t* __restrict__ hv) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    hk[c] = activeContact(flags[c]) ? (uint32_t)(key[c] & 0xffffffffu) : nPar;
    hv[c] = (int32_t)c;
}
__global__ void k_hi_start(const uint32_t* __restrict__ hks, int64_t n, int nPar, int32_t* __restrict__ hiStart) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > nPar) return;
    hiStart[p] = (int32_t)lowerBound32(hks, n, (uint32_t)p);
}
// end slots: active contact c with hi==p sits at loStart[p] + (its index k in hiList); with lo==p
// at hiStart[p+1] + act[c] (see DevIncidence); inactive contacts have no slot (-1)
// The work list holds the active contacts other than sphere-sphere first, then the sphere-sphere
// ones, each group in ascending contact order (actSS: exclusive scan of the active sphere-sphere
// contacts; nOther = active contacts that are not sphere-sphere).
__global__ void k_slots(const uint64_t* __restrict__ key, const uint32_t* __restrict__ flags, int64_t n, int64_t nAct,
                        const int32_t* __restrict__ act, const int32_t* __restrict__ actSS, int64_t nOther, DevIncidence I) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (k < nAct) {
        const int32_t ch = I.hiList[k];
        const int hiP = (int)(key[ch] & 0xffffffffu);
        I.slotHi[ch] = I.loStart[hiP] + (int32_t)k;
    }
    if (activeContact(flags[k])) {
        const int loP = (int)(key[k] >> 32);
        I.slotLo[k] = I.hiStart[loP + 1] + act[k];
        const uint32_t fl = flags[k];
        const int hiP = (int)(key[k] & 0xffffffffu);
        const int64_t w = (ctype(fl) == CT_SS) ? nOther + actSS[k] : act[k] - actSS[k];
        I.work[w] = (fl & C_SWAP) ? make_int4((int)k, hiP, loP, (int)(fl & 0xeu)) : make_int4((int)k, loP, hiP, (int)(fl & 0xeu));
    } else {
        I.slotLo[k] = -1;
        I.slotHi[k] = -1;
    }
}

// Particles summed by the block tree; the ones whose node has a free DOF are also summed before
// every Leapfrog (the others only when the forces are reported).
__global__ void k_heavy(DevIncidence I, DevParticles P, const uint32_t* __restrict__ nodeFlags, int threshold,
                        int32_t* __restrict__ count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.n) return;
    if (P.shape[p] == WG_SHAPE_FACET) return;
    const int d = (I.hiStart[p + 1] - I.hiStart[p]) + (I.loStart[p + 1] - I.loStart[p]);
    if (d > threshold) {
        const int q = atomicAdd(count, 1);
        I.heavy[q] = p;
        if ((nodeFlags[p] & F_DOF_ALL) != F_DOF_ALL) I.heavyFree[atomicAdd(count + 1, 1)] = p;
    }
}

// ---------------------------------------------------------------- host orchestration
static int ensureCub(Sim& S, size_t bytes) {
    CollideWork& W = *S.cw;
    if (bytes <= W.cubBytes) return 0;
    if (W.cubTmp) S.dfree(W.cubTmp);
    W.cubBytes = bytes * 3 / 2 + 1024;
    W.cubTmp = S.dalloc(W.cubBytes);
    return W.cubTmp ? 0 : S.fail(WG_ERR_CUDA, "out of device memory (collider scratch)");
}

template <class T>
static T* grow(Sim& S, T* p, int64_t& cap, int64_t need) {
    if (need <= cap && p) return p;
    if (p) S.dfree(p);
    cap = std::max<int64_t>(need, cap * 3 / 2 + 1024);
    return (T*)S.dalloc(sizeof(T) * cap);
}

static int buildLists(Sim& S) {
    CollideWork& W = *S.cw;
    std::vector<int32_t> sph, large, glob;
    for (int64_t p = 0; p < S.nPar; p++) {
        if (!S.hParked.empty() && S.hParked[p]) continue;  // empty part of a serving slot
        if (S.hShape[p] == WG_SHAPE_SPHERE) sph.push_back((int32_t)p);
        else if (S.hShape[p] == WG_SHAPE_WALL) glob.push_back((int32_t)p);
        else large.push_back((int32_t)p);
    }
    W.nSph = (int)sph.size();
    // per-scene sphere ranges and grid-reduction chunks (particles of a batch are grouped by scene)
    const int K = S.nScenes;
    W.hSceneSph.assign(K + 1, 0);
    for (int32_t p : sph) W.hSceneSph[(S.hSceneOfPar.empty() ? 0 : S.hSceneOfPar[p]) + 1]++;
    for (int k = 0; k < K; k++) W.hSceneSph[k + 1] += W.hSceneSph[k];
    W.chunksDirty = true;
    W.hChunk.assign(1, 0);
    W.hSceneChunk.assign(1, 0);
    const int64_t CH = 4096;
    for (int k = 0; k < K; k++) {
        for (int64_t b = W.hSceneSph[k]; b < W.hSceneSph[k + 1]; b += CH) W.hChunk.push_back((int32_t)std::min(b + CH, W.hSceneSph[k + 1]));
        W.hSceneChunk.push_back((int32_t)W.hChunk.size() - 1);
    }
    W.hLarge = large;
    W.hGlobal = glob;
    // capacity for every particle: the lists are rebuilt when serving slots change
    if (!W.sphereIds) {
        W.sphereIds = (int32_t*)S.dalloc(sizeof(int32_t) * std::max<int64_t>(1, S.nPar));
        W.largeIds = (int32_t*)S.dalloc(sizeof(int32_t) * std::max<int64_t>(1, S.nPar));
        W.globalIds = (int32_t*)S.dalloc(sizeof(int32_t) * std::max<int64_t>(1, S.nPar));
        W.gStart = (int32_t*)S.dalloc(sizeof(int32_t) * (S.nScenes + 1));
        if (!W.sphereIds || !W.largeIds || !W.globalIds || !W.gStart) return S.fail(WG_ERR_CUDA, "out of device memory");
    }
    W.nLarge = W.nGlobal = 0;
    if (!sph.empty()) WG_CUDA_TRY(cudaMemcpyAsync(W.sphereIds, sph.data(), sizeof(int32_t) * sph.size(), cudaMemcpyHostToDevice, S.stream));
    // non-sphere pairs are possible only if some pair of them shares a mask bit outside loneMask
    bool ll = false;
    std::vector<int32_t> nonSph(large);
    nonSph.insert(nonSph.end(), glob.begin(), glob.end());
    {
        uint32_t seen = 0;  // OR of masks
        // exact test on distinct mask values
        std::vector<uint32_t> masks;
        for (int32_t p : nonSph) masks.push_back(S.hMask[p]);
        std::sort(masks.begin(), masks.end());
        masks.erase(std::unique(masks.begin(), masks.end()), masks.end());
        for (size_t a = 0; a < masks.size() && !ll; a++)
            for (size_t b = a; b < masks.size() && !ll; b++)
                if ((masks[a] & masks[b]) != 0 && (masks[a] & masks[b] & S.cfg.lone_mask) == 0) ll = true;
        (void)seen;
    }
    W.largeLargePossible = ll && nonSph.size() > 1;
    return 0;
}

int collide_full_run(Sim& S) {
    cudaStream_t st = S.stream;
    // the contact arrays take back the packed sphere-sphere state before they are merged
    {
        int r = S.syncContacts(false);  // the merge below is queued on the same stream
        if (r) return r;
        S.K.n = 0;
    }
    if (!S.cw) {
        S.cw = new CollideWork();
        S.listsDirty = true;
    }
    if (S.listsDirty) {
        int r = buildLists(S);
        if (r) return r;
        S.listsDirty = false;
    }
    CollideWork& W = *S.cw;
    const uint32_t lone = S.cfg.lone_mask;
    if (S.cfg.periodic && S.hPar.hasShear && !W.hGlobal.empty())
        return S.fail(WG_ERR_UNSUPPORTED, "Walls not supported in skewed (Scene.cell.trsf is not diagonal) periodic boundary conditions.");
    // 1. boxes
    if (S.nPar > 0) k_aabb<<<(unsigned)((S.nPar + BS - 1) / BS), BS, 0, st>>>(S.N, S.P, S.dPar, S.dFlags + 1);
    // lastPos for node slots not owned by a particle box computation (dummy slots) stays stale:
    // they never move (blocked, zero velocity) and are never tested against a stale reference.
    // 2. grid over spheres, one per scene of a batch (keys of scene k start at its grid's base)
    const int K = S.nScenes;
    std::vector<Grid> hG(K, Grid{0, 0, 0, 1, 1, 1, 1, 1, 0});
    Grid G = hG[0];
    const int ns = W.nSph;
    if (ns > 0) {
        const int nb = (int)W.hChunk.size() - 1;
        if (!W.dGrids) {
            // capacity for the most chunks the particles can form (one per scene plus one per 4096 spheres)
            const int cap = (int)(S.nPar / 4096 + S.nScenes + 2);
            W.red = (double*)S.dalloc(sizeof(double) * 7 * cap);
            W.dChunk = (int32_t*)S.dalloc(sizeof(int32_t) * (cap + 1));
            WG_CUDA_TRY(cudaMallocHost(&W.hRed, sizeof(double) * 7 * cap));
            W.dGrids = (Grid*)S.dalloc(sizeof(Grid) * K);
            if (!W.dGrids || !W.dChunk) return S.fail(WG_ERR_CUDA, "out of device memory (grid)");
        }
        if (W.chunksDirty) {
            WG_CUDA_TRY(cudaMemcpyAsync(W.dChunk, W.hChunk.data(), sizeof(int32_t) * (nb + 1), cudaMemcpyHostToDevice, S.stream));
            W.chunksDirty = false;
        }
        k_grid_reduce<<<nb, BS, 0, st>>>(S.P, W.sphereIds, W.dChunk, W.red);
        WG_CUDA_TRY(cudaMemcpyAsync(W.hRed, W.red, sizeof(double) * 7 * nb, cudaMemcpyDeviceToHost, st));
        WG_CUDA_TRY(cudaStreamSynchronize(st));
        int64_t base = 0;
        for (int k = 0; k < K; k++) {
            double v[7] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.};
            for (int b = W.hSceneChunk[k]; b < W.hSceneChunk[k + 1]; b++) {
                for (int q = 0; q < 3; q++) v[q] = std::min(v[q], W.hRed[7 * b + q]);
                for (int q = 3; q < 7; q++) v[q] = std::max(v[q], W.hRed[7 * b + q]);
            }
            Grid& g = hG[k];
            g.base = base;
            if (W.hSceneChunk[k] == W.hSceneChunk[k + 1]) continue;  // a scene without spheres
            if (!(std::isfinite(v[0]) && std::isfinite(v[3]) && std::isfinite(v[6])))
                return S.fail(WG_ERR_NAN, "InsertionSortCollider: non-finite sphere bounding box (NaN or infinite position)");
            const int64_t nsk = W.hSceneSph[k + 1] - W.hSceneSph[k];
            // cell edge slightly above the largest sphere box, so boxes that overlap sit in adjacent cells
            double h = v[6] * (1 + 1e-9) + 1e-300;
            double ext[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
            int64_t dims[3];
            for (;;) {
                if (S.cfg.periodic)  // the periodic cell [0, size) per axis (unsheared coordinates)
                    for (int q = 0; q < 3; q++) dims[q] = std::max<int64_t>(1, (int64_t)std::floor(S.hPar.cellSize[q] / h));
                else
                    for (int q = 0; q < 3; q++) dims[q] = (int64_t)std::floor(ext[q] / h) + 1;
                int64_t nc = dims[0] * dims[1] * dims[2];
                if (nc <= std::max<int64_t>(8 * nsk, K > 1 ? 64 : (1 << 16)) && nc < (int64_t(1) << 31)) break;
                h *= 1.25;
            }
            g.ox = v[0]; g.oy = v[1]; g.oz = v[2]; g.h = h;
            g.nx = (int32_t)dims[0]; g.ny = (int32_t)dims[1]; g.nz = (int32_t)dims[2];
            g.ncell = dims[0] * dims[1] * dims[2];
            base += g.ncell;
        }
        if (base >= (int64_t(1) << 32) - 1) return S.fail(WG_ERR_CAPACITY, "too many broad-phase cells in the batch");
        const int64_t ncellAll = base;
        G = hG[0];
        WG_CUDA_TRY(cudaMemcpyAsync(W.dGrids, hG.data(), sizeof(Grid) * K, cudaMemcpyHostToDevice, st));
        // sort spheres by cell
        if (!W.cellKey) {
            const int64_t cap = S.nPar;  // every particle could be an active sphere
            W.cellKey = (uint32_t*)S.dalloc(sizeof(uint32_t) * cap);
            W.cellKeySorted = (uint32_t*)S.dalloc(sizeof(uint32_t) * cap);
            W.cellVal = (int32_t*)S.dalloc(sizeof(int32_t) * cap);
            W.sid = (int32_t*)S.dalloc(sizeof(int32_t) * cap);
            W.smn = (double4_32a*)S.dalloc(sizeof(double4_32a) * cap);
            W.smx = (double4_32a*)S.dalloc(sizeof(double4_32a) * cap);
            W.smask = (uint32_t*)S.dalloc(sizeof(uint32_t) * cap);
            W.smnf = (float4*)S.dalloc(sizeof(float4) * cap);
            W.smxf = (float4*)S.dalloc(sizeof(float4) * cap);
            W.smnfi = (float4*)S.dalloc(sizeof(float4) * cap);
            W.smxfi = (float4*)S.dalloc(sizeof(float4) * cap);
            if (!W.smask || !W.smxf || !W.smxfi) return S.fail(WG_ERR_CUDA, "out of device memory (grid)");
        }
        W.cellOff = grow(S, W.cellOff, W.cellOffCap, ncellAll + 1);
        if (S.cfg.periodic) k_cellkey_peri<<<(ns + BS - 1) / BS, BS, 0, st>>>(S.P, W.sphereIds, ns, G, S.dPar, W.cellKey, W.cellVal);
        else k_cellkey<<<(ns + BS - 1) / BS, BS, 0, st>>>(S.P, W.sphereIds, ns, W.dGrids, W.cellKey, W.cellVal);
        int endBit = 1;
        while ((int64_t(1) << endBit) < ncellAll) endBit++;
        size_t tb = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tb, W.cellKey, W.cellKeySorted, W.cellVal, W.sid, ns, 0, endBit, st);
        if (ensureCub(S, tb)) return WG_ERR_CUDA;
        tb = W.cubBytes;
        WG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(W.cubTmp, tb, W.cellKey, W.cellKeySorted, W.cellVal, W.sid, ns, 0, endBit, st));
        k_cell_off<<<(unsigned)((ncellAll + 1 + BS - 1) / BS), BS, 0, st>>>(W.cellKeySorted, ns, ncellAll, W.cellOff);
        k_gather_sorted<<<(ns + BS - 1) / BS, BS, 0, st>>>(S.P, W.sid, ns, W.smn, W.smx, W.smask, W.smnf, W.smxf, W.smnfi, W.smxfi);
    }
    // lists of large particles: facets with boxes spanning a few cells use the grid, the rest are global
    {
        // decide on the host from the facet sizes measured at the previous full run would need a copy;
        // facet boxes are static in the supported scenes, so classify them once by size here
        if (W.nLarge == 0 && W.nGlobal == 0 && (!W.hLarge.empty() || !W.hGlobal.empty())) {
            std::vector<double4_32a> mn(S.nPar), mx(S.nPar);
            WG_CUDA_TRY(cudaMemcpyAsync(mn.data(), S.P.mn, sizeof(double4_32a) * S.nPar, cudaMemcpyDeviceToHost, st));
            WG_CUDA_TRY(cudaMemcpyAsync(mx.data(), S.P.mx, sizeof(double4_32a) * S.nPar, cudaMemcpyDeviceToHost, st));
            WG_CUDA_TRY(cudaStreamSynchronize(st));
            std::vector<int32_t> loc, glo = W.hGlobal;
            for (int32_t p : W.hLarge) {
                double e = std::max({mx[p].x - mn[p].x, mx[p].y - mn[p].y, mx[p].z - mn[p].z});
                const double hk = hG[S.hSceneOfPar.empty() ? 0 : S.hSceneOfPar[p]].h;
                if (ns > 0 && std::isfinite(e) && e <= 8 * hk) loc.push_back(p);
                else glo.push_back(p);
            }
            std::sort(glo.begin(), glo.end());  // grouped by scene (particles of a batch are)
            W.nLarge = (int)loc.size();
            W.nGlobal = (int)glo.size();
            if (W.nLarge) WG_CUDA_TRY(cudaMemcpyAsync(W.largeIds, loc.data(), sizeof(int32_t) * loc.size(), cudaMemcpyHostToDevice, S.stream));
            if (W.nGlobal) WG_CUDA_TRY(cudaMemcpyAsync(W.globalIds, glo.data(), sizeof(int32_t) * glo.size(), cudaMemcpyHostToDevice, S.stream));
            if (K > 1) {
                std::vector<int32_t> gs(K + 1, 0);
                for (int32_t p : glo) gs[S.hSceneOfPar[p] + 1]++;
                for (int k = 0; k < K; k++) gs[k + 1] += gs[k];
                WG_CUDA_TRY(cudaMemcpyAsync(W.gStart, gs.data(), sizeof(int32_t) * (K + 1), cudaMemcpyHostToDevice, S.stream));
            }
        }
    }
    // 3-4. pair generation with a capacity retry
    if (!W.counter) {
        W.counter = (unsigned long long*)S.dalloc(sizeof(unsigned long long) * 2);
        WG_CUDA_TRY(cudaMallocHost(&W.hCounter, sizeof(unsigned long long) * 2));
    }
    if (W.pairCap == 0) {
        int64_t c0 = std::max<int64_t>(1 << 16, 8 * S.nPar);
        W.pairs = grow(S, W.pairs, W.pairCap, c0);
        int64_t cap2 = 0;
        W.pairsSorted = grow(S, W.pairsSorted, cap2, W.pairCap);
    }
    const bool peri = S.cfg.periodic != 0;
    int64_t nNew = 0;
    for (int attempt = 0; attempt < 3; attempt++) {
        WG_CUDA_TRY(cudaMemsetAsync(W.counter, 0, sizeof(unsigned long long), st));
        if (peri) {
            if (W.pairCdCap < W.pairCap) {
                int64_t c2 = W.pairCdCap;
                W.pairCd = grow(S, W.pairCd, W.pairCdCap, W.pairCap);
                W.pairCdSorted = grow(S, W.pairCdSorted, c2, W.pairCap);
                if (!W.pairCd || !W.pairCdSorted) return S.fail(WG_ERR_CUDA, "out of device memory (pairs)");
            }
            if (ns > 0)
                k_pairs_ss_peri<<<(ns + BS - 1) / BS, BS, 0, st>>>(W.cellKeySorted, W.sid, W.smn, W.smx, W.smask, ns, G, W.cellOff, lone,
                                                                 S.dPar, W.pairs, W.pairCd, W.pairCap, W.counter, S.dFlags + FL_ERR);
            if (ns > 0 && W.nGlobal > 0)
                k_pairs_global_peri<<<(ns + BS - 1) / BS, BS, 0, st>>>(S.P, W.globalIds, W.nGlobal, W.sphereIds, ns, lone, S.dPar,
                                                                     W.pairs, W.pairCd, W.pairCap, W.counter, S.dFlags + FL_ERR);
        } else if (ns > 0) {
            k_pairs_ss<<<(ns + BS - 1) / BS, BS, 0, st>>>(W.cellKeySorted, W.smn, W.smx, W.smnf, W.smxf, W.smnfi, W.smxfi, ns, W.dGrids,
                                                        S.P.scene,
                                                        W.cellOff, lone, W.pairs, W.pairCap, W.counter);
            if (W.nLarge > 0)
                k_pairs_local<<<(unsigned)(((int64_t)W.nLarge * 32 + BS - 1) / BS), BS, 0, st>>>(
                    S.P, W.largeIds, W.nLarge, W.smn, W.smx, W.smnf, W.smxf, W.smnfi, W.smxfi, W.dGrids, W.cellOff, lone, W.pairs,
                    W.pairCap, W.counter);
            if (W.nGlobal > 0)
                k_pairs_global<<<(ns + BS - 1) / BS, BS, 0, st>>>(S.P, W.globalIds, W.nGlobal, K > 1 ? W.gStart : nullptr, W.sphereIds, ns, lone,
                                                                W.pairs, W.pairCap, W.counter);
        }
        if (W.largeLargePossible && !peri) {
            // all non-spheres against each other
            int nn = W.nLarge + W.nGlobal;
            std::vector<int32_t> all;
            (void)all;
            int32_t* ids = W.globalIds;
            if (W.nLarge > 0) {
                // concatenate: globalIds has room for every non-sphere
                WG_CUDA_TRY(cudaMemcpyAsync(W.globalIds + W.nGlobal, W.largeIds, sizeof(int32_t) * W.nLarge, cudaMemcpyDeviceToDevice, st));
            }
            int64_t tot = (int64_t)nn * nn;
            k_pairs_large_large<<<(unsigned)((tot + BS - 1) / BS), BS, 0, st>>>(S.P, ids, nn, lone, W.pairs, W.pairCap, W.counter);
        }
        WG_CUDA_TRY(cudaMemcpyAsync(W.hCounter, W.counter, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        WG_CUDA_TRY(cudaStreamSynchronize(st));
        nNew = (int64_t)W.hCounter[0];
        if (nNew <= W.pairCap) break;
        int64_t cap2 = W.pairCap;
        W.pairs = grow(S, W.pairs, W.pairCap, nNew + nNew / 4);
        W.pairsSorted = grow(S, W.pairsSorted, cap2, W.pairCap);
        if (!W.pairs || !W.pairsSorted) return S.fail(WG_ERR_CUDA, "out of device memory (pairs)");
    }
    // sort new pair keys
    int idBits = 1;
    while ((int64_t(1) << idBits) < S.nPar) idBits++;
    if (nNew > 0 && peri) {
        size_t tb = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tb, W.pairs, W.pairsSorted, W.pairCd, W.pairCdSorted, nNew, 0, 32 + idBits, st);
        if (ensureCub(S, tb)) return WG_ERR_CUDA;
        tb = W.cubBytes;
        WG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(W.cubTmp, tb, W.pairs, W.pairsSorted, W.pairCd, W.pairCdSorted, nNew, 0,
                                                    32 + idBits, st));
    } else if (nNew > 0) {
        // ids take idBits each: sort (lo << idBits | hi), the same order in fewer radix passes
        const unsigned pb = (unsigned)((nNew + BS - 1) / BS);
        k_pack_keys<<<pb, BS, 0, st>>>(W.pairs, nNew, idBits);
        size_t tb = 0;
        cub::DeviceRadixSort::SortKeys(nullptr, tb, W.pairs, W.pairsSorted, nNew, 0, 2 * idBits, st);
        if (ensureCub(S, tb)) return WG_ERR_CUDA;
        tb = W.cubBytes;
        WG_CUDA_TRY(cub::DeviceRadixSort::SortKeys(W.cubTmp, tb, W.pairs, W.pairsSorted, nNew, 0, 2 * idBits, st));
        k_unpack_keys<<<pb, BS, 0, st>>>(W.pairsSorted, nNew, idBits);
    }
    // 5. merge with the previous contact set
    const int64_t nOld = S.C.n;
    W.orph = grow(S, W.orph, W.mergeCap, std::max<int64_t>(nOld, 1) * 2 + 2);
    int64_t capTmp = 0;
    if (!W.orphKey || W.mergeCap > 0) {
        // orphKey/orphSrc sized like orph
        static int64_t dummy;
        (void)dummy;
    }
    int64_t nOrph = 0;
    // the first index of every lo id in the new pairs and in the old contacts
    W.newLo = grow(S, W.newLo, W.newLoCap, S.nPar + 2);
    W.oldLo = grow(S, W.oldLo, W.oldLoCap, S.nPar + 2);
    if (!W.newLo || !W.oldLo) return S.fail(WG_ERR_CUDA, "out of device memory (merge)");
    k_lo_bounds<<<(unsigned)((nNew + 1 + BS - 1) / BS), BS, 0, st>>>(W.pairsSorted, nNew, (int)S.nPar, W.newLo);
    k_lo_bounds<<<(unsigned)((nOld + 1 + BS - 1) / BS), BS, 0, st>>>(S.C.key, nOld, (int)S.nPar, W.oldLo);
    if (nOld > 0) {
        int32_t* flagsArr = W.orph;
        int32_t* scanArr = W.orph + (std::max<int64_t>(nOld, 1) + 1);
        k_mark_orphans<<<(unsigned)((nOld + BS - 1) / BS), BS, 0, st>>>(S.C, W.pairsSorted, W.newLo, flagsArr, S.P.fresh);
        size_t tb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb, flagsArr, scanArr, (int)nOld, st);
        if (ensureCub(S, tb)) return WG_ERR_CUDA;
        tb = W.cubBytes;
        WG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(W.cubTmp, tb, flagsArr, scanArr, (int)nOld, st));
        int32_t last[2];
        WG_CUDA_TRY(cudaMemcpyAsync(&last[0], flagsArr + nOld - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        WG_CUDA_TRY(cudaMemcpyAsync(&last[1], scanArr + nOld - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        WG_CUDA_TRY(cudaStreamSynchronize(st));
        nOrph = (int64_t)last[0] + last[1];
        if (nOrph > 0) {
            if (nOrph > W.orphCap) {
                int64_t c1 = W.orphCap, c2 = W.orphCap;
                W.orphKey = grow(S, W.orphKey, c1, nOrph);
                W.orphSrc = grow(S, W.orphSrc, c2, nOrph);
                W.orphCap = c1;
                if (!W.orphKey || !W.orphSrc) return S.fail(WG_ERR_CUDA, "out of device memory (merge)");
            }
            k_compact_orphans<<<(unsigned)((nOld + BS - 1) / BS), BS, 0, st>>>(S.C, flagsArr, scanArr, W.orphKey, W.orphSrc);
        }
    }
    (void)capTmp;
    const int64_t nOut = nNew + nOrph;
    int r = S.ensureContactCapacity(nOut);
    if (r) return r;
    W.src = grow(S, W.src, W.srcCap, std::max<int64_t>(nOut, 1));
    if (!W.src) return S.fail(WG_ERR_CUDA, "out of device memory (merge)");
    S.Cb.n = nOut;
    if (peri) {
        W.newCd = grow(S, W.newCd, W.newCdCap, std::max<int64_t>(nOut, 1));
        if (!W.newCd) return S.fail(WG_ERR_CUDA, "out of device memory (merge)");
    }
    if (nNew > 0)
        k_place_new<<<(unsigned)((nNew + BS - 1) / BS), BS, 0, st>>>(W.pairsSorted, nNew, W.orphKey, nOrph, S.C.key,
                                                                    nOld > 0 ? W.oldLo : nullptr, S.Cb.key, W.src,
                                                                    peri ? W.pairCdSorted : nullptr, W.newCd, S.P.fresh);
    if (nOrph > 0)
        k_place_orph<<<(unsigned)((nOrph + BS - 1) / BS), BS, 0, st>>>(W.pairsSorted, nNew, W.orphKey, W.orphSrc, nOrph, S.Cb.key,
                                                                      W.src);
    if (nOut > 0) k_gather<<<(unsigned)((nOut + BS - 1) / BS), BS, 0, st>>>(S.C, S.Cb, W.src, S.P, S.dStep, peri ? W.newCd : nullptr);
    std::swap(S.C, S.Cb);
    if (nOut > 0 && !S.cfg.periodic)
        k_dormant<<<(unsigned)((nOut + BS - 1) / BS), BS, 0, st>>>(S.C, S.N, S.P, S.dPar);
    // 6. CSR incidence over the active contacts
    const int64_t n = S.C.n;
    if (W.hiCap < std::max<int64_t>(n, 1)) {
        if (W.hiKeys) {
            S.dfree(W.hiKeys); S.dfree(W.hiKeysSorted); S.dfree(W.hiVals); S.dfree(S.I.hiList);
            S.dfree(S.I.slotLo); S.dfree(S.I.slotHi); S.dfree(W.act); S.dfree(W.actSS); S.dfree(S.I.work);
        }
        W.hiCap = std::max<int64_t>(n, 1) * 3 / 2 + 1024;
        W.hiKeys = (uint32_t*)S.dalloc(sizeof(uint32_t) * W.hiCap);
        W.hiKeysSorted = (uint32_t*)S.dalloc(sizeof(uint32_t) * W.hiCap);
        W.hiVals = (int32_t*)S.dalloc(sizeof(int32_t) * W.hiCap);
        S.I.hiList = (int32_t*)S.dalloc(sizeof(int32_t) * W.hiCap);
        S.I.slotLo = (int32_t*)S.dalloc(sizeof(int32_t) * W.hiCap);
        S.I.slotHi = (int32_t*)S.dalloc(sizeof(int32_t) * W.hiCap);
        W.act = (int32_t*)S.dalloc(sizeof(int32_t) * (W.hiCap + 1));
        W.actSS = (int32_t*)S.dalloc(sizeof(int32_t) * (W.hiCap + 1));
        S.I.work = (int4*)S.dalloc(sizeof(int4) * W.hiCap);
        if (!S.I.slotHi || !W.act || !S.I.work) return S.fail(WG_ERR_CUDA, "out of device memory (incidence)");
    }
    int64_t nAct = 0, nSS = 0;
    {
        WG_CUDA_TRY(cudaMemsetAsync(W.act, 0, sizeof(int32_t) * (n + 1), st));
        WG_CUDA_TRY(cudaMemsetAsync(W.actSS, 0, sizeof(int32_t) * (n + 1), st));
        if (n > 0) {
            k_active<<<(unsigned)((n + BS - 1) / BS), BS, 0, st>>>(S.C.flags, n, W.act, W.actSS);
            size_t tb = 0;
            cub::DeviceScan::ExclusiveSum(nullptr, tb, W.act, W.act, (int)(n + 1), st);
            if (ensureCub(S, tb)) return WG_ERR_CUDA;
            tb = W.cubBytes;
            WG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(W.cubTmp, tb, W.act, W.act, (int)(n + 1), st));
            tb = W.cubBytes;
            WG_CUDA_TRY(cub::DeviceScan::ExclusiveSum(W.cubTmp, tb, W.actSS, W.actSS, (int)(n + 1), st));
        }
        int32_t h[2] = {0, 0};
        WG_CUDA_TRY(cudaMemcpyAsync(&h[0], W.act + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        WG_CUDA_TRY(cudaMemcpyAsync(&h[1], W.actSS + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        WG_CUDA_TRY(cudaStreamSynchronize(st));
        nAct = h[0];
        nSS = h[1];
    }
    k_lo_start<<<(unsigned)((S.nPar + 1 + BS - 1) / BS), BS, 0, st>>>(S.C.key, n, (int)S.nPar, W.act, S.I.loStart);
    if (S.I.endCap < 2 * std::max<int64_t>(nAct, 1)) {
        if (S.I.endA) { S.dfree(S.I.endA); S.dfree(S.I.endB); }
        if (S.I.endAf) { S.dfree(S.I.endAf); S.dfree(S.I.endBf); }
        S.I.endA = nullptr; S.I.endB = nullptr; S.I.endAf = nullptr; S.I.endBf = nullptr;
        S.I.endCap = 2 * std::max<int64_t>(nAct, 1) * 3 / 2 + 2048;
        if (S.prec == WG_PREC_FP32) {
            S.I.endAf = (float4*)S.dalloc(sizeof(float4) * S.I.endCap);
            S.I.endBf = (float2*)S.dalloc(sizeof(float2) * S.I.endCap);
            if (!S.I.endAf || !S.I.endBf) return S.fail(WG_ERR_CUDA, "out of device memory (contact ends)");
        } else {
            S.I.endA = (double4_32a*)S.dalloc(sizeof(double4_32a) * S.I.endCap);
            S.I.endB = (double2*)S.dalloc(sizeof(double2) * S.I.endCap);
            if (!S.I.endA || !S.I.endB) return S.fail(WG_ERR_CUDA, "out of device memory (contact ends)");
        }
    }
    int hiBits = 1;  // bits of the largest hi key, nPar
    while ((int64_t(1) << hiBits) <= S.nPar) hiBits++;
    if (n > 0) {
        k_hi_keys<<<(unsigned)((n + BS - 1) / BS), BS, 0, st>>>(S.C.key, S.C.flags, n, (uint32_t)S.nPar, W.hiKeys, W.hiVals);
        size_t tb = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tb, W.hiKeys, W.hiKeysSorted, W.hiVals, S.I.hiList, n, 0, hiBits, st);
        if (ensureCub(S, tb)) return WG_ERR_CUDA;
        tb = W.cubBytes;
        WG_CUDA_TRY(cub::DeviceRadixSort::SortPairs(W.cubTmp, tb, W.hiKeys, W.hiKeysSorted, W.hiVals, S.I.hiList, n, 0, hiBits, st));
    }
    k_hi_start<<<(unsigned)((S.nPar + 1 + BS - 1) / BS), BS, 0, st>>>(W.hiKeysSorted, n, (int)S.nPar, S.I.hiStart);
    if (n > 0) k_slots<<<(unsigned)((n + BS - 1) / BS), BS, 0, st>>>(S.C.key, S.C.flags, n, nAct, W.act, W.actSS, nAct - nSS, S.I);
    S.I.nAct = nAct;
    S.nMixed = nAct - nSS;
    // every end starts without a contribution; the contact kernel fills the real ones this step
    const int64_t ne = 2 * std::max<int64_t>(nAct, 1);
    if (S.prec == WG_PREC_FP32) {
        WG_CUDA_TRY(cudaMemsetAsync(S.I.endAf, 0, sizeof(float4) * ne, st));
        WG_CUDA_TRY(cudaMemsetAsync(S.I.endBf, 0, sizeof(float2) * ne, st));
    } else {
        WG_CUDA_TRY(cudaMemsetAsync(S.I.endA, 0, sizeof(double4_32a) * ne, st));
        WG_CUDA_TRY(cudaMemsetAsync(S.I.endB, 0, sizeof(double2) * ne, st));
    }
    // FP32-force mode, aperiodic scenes: the sphere-sphere contacts' state in work-list order
    if (S.prec == WG_PREC_FP32 && !S.cfg.periodic && nSS > 0) {
        DevPackedSS& K = S.K;
        if (K.cap < nSS) {
            S.dfree(K.item); S.dfree(K.flags);
            for (int q = 0; q < CF_NCOL; q++) S.dfree(K.col[q]);
            S.dfree(K.ft[0]); S.dfree(K.ft[1]);
            K = DevPackedSS{};
            K.cap = nSS * 5 / 4 + 4096;
            K.item = (int4*)S.dalloc(sizeof(int4) * K.cap);
            K.flags = (uint32_t*)S.dalloc(sizeof(uint32_t) * K.cap);
            bool ok = K.item && K.flags;
            for (int q = 0; q < CF_NCOL; q++) {
                K.col[q] = (float*)S.dalloc(sizeof(float) * K.cap);
                ok = ok && K.col[q];
            }
            // the IdealElPl shear force (a serving slot may take a job with that law at any time)
            K.ft[0] = (double*)S.dalloc(sizeof(double) * K.cap);
            K.ft[1] = (double*)S.dalloc(sizeof(double) * K.cap);
            ok = ok && K.ft[0] && K.ft[1];
            if (!ok) {
                K.cap = 0;
                return S.fail(WG_ERR_CUDA, "out of device memory (packed contacts)");
            }
        }
        K.n = nSS;
        bool law0 = S.cfg.law == 0;
        for (const wg_config& c : S.cfgs) law0 = law0 || c.law == 0;
        K.ftLive = law0;
        launch_pack_ss(st, S.C, S.I, S.P, K, S.nMixed);
    }
    S.packDirty = false;
    // heavy particles
    if (!W.heavyCount) {
        W.heavyCount = (int32_t*)S.dalloc(sizeof(int32_t) * 3);
        WG_CUDA_TRY(cudaMallocHost(&W.hHeavy, sizeof(int32_t) * 3));
    }
    WG_CUDA_TRY(cudaMemsetAsync(W.heavyCount, 0, sizeof(int32_t) * 3, st));
    k_heavy<<<(unsigned)((S.nPar + BS - 1) / BS), BS, 0, st>>>(S.I, S.P, S.N.flags, kHeavyThreshold, W.heavyCount);
    WG_CUDA_TRY(cudaMemcpyAsync(W.hHeavy, W.heavyCount, sizeof(int32_t) * 3, cudaMemcpyDeviceToHost, st));
    WG_CUDA_TRY(cudaStreamSynchronize(st));
    S.I.nHeavy = S.cfg.apply_forces ? W.hHeavy[0] : 0;
    S.I.nHeavyFree = S.cfg.apply_forces ? W.hHeavy[1] : 0;
    if (S.P.fresh) WG_CUDA_TRY(cudaMemsetAsync(S.P.fresh, 0, S.nPar, st));
    WG_CUDA_TRY(cudaGetLastError());
    S.nFullRuns++;
    return 0;
}

void collide_free(Sim& S) {
    if (!S.cw) return;
    if (S.cw->hRed) cudaFreeHost(S.cw->hRed);
    if (S.cw->hCounter) cudaFreeHost(S.cw->hCounter);
    if (S.cw->hHeavy) cudaFreeHost(S.cw->hHeavy);
    delete S.cw;
    S.cw = nullptr;
}

}  // namespace wg
