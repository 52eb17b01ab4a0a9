// Per-particle force/torque sum over the end slots of the contact incidence (DevIncidence),
// shared by the Leapfrog kernels (which fuse the sum into the integration) and by the
// reporting kernels that write DemData.force/torque.
//
// A warp handles 32 consecutive particles, whose end slots form one contiguous run of the end
// arrays. The warp stages that run through shared memory in chunks with coalesced loads; each
// lane then adds its own particle's slots in slot order (ascending id of the other particle),
// so every lane's sum is the serial sum of the reference's deterministic pass
// (pkg/dem/ContactLoop.cpp:250-257): F = m*g, then each end in order, T = 0, then each end.
// Lanes that take no part (facets, particles past the end, particles whose degree exceeds
// kHeavyThreshold and which are summed by the block tree instead) are left out of the staged
// range, so a wall with thousands of contacts does not stall the warp of its neighbours.
#pragma once
#include "wg_internal.h"
#include "wg_math.cuh"

namespace wg {

template <typename EA, typename EB, int CH>
struct EndStage {
    EA a[CH];
    EB b[CH];
};

// FP64 accumulation (FP64 ends): F and T start from the reset value and take each end in turn.
struct SumD {
    D3 F, T;
    __device__ __forceinline__ void add(const double4_32a& x, const double2& y) {
        F = F + D3{x.x, x.y, x.z};
        T = T + D3{x.w, y.x, y.y};
    }
};

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest FP32; the intrinsics are never
// contracted or reassociated).
__device__ __forceinline__ void twoSum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hB + lB) - (hA + lA) as s + t with |t| << |s|: s + e = hB - hA exactly, t = e + (lB - lA).
__device__ __forceinline__ void dfDiff(float hA, float lA, float hB, float lB, float& s, float& t) {
    float e;
    twoSum(hB, -hA, s, e);
    t = e + (lB - lA);
}
// (s + t)^2 as p + c: p = fl(s*s), c = the FMA residual of s*s plus t*(2s + t).
__device__ __forceinline__ void dfSquare(float s, float t, float& p, float& c) {
    p = s * s;
    c = fmaf(s, s, -p) + t * (2.f * s + t);
}

// Compensated accumulation of FP32 ends (FP32-force mode): each component is carried as an
// unevaluated FP32 pair hi + lo with the rounding error of every addition captured exactly by
// TwoSum, which keeps ~48 significant bits, and is converted to FP64 once per particle. On
// GB300 the FP64 pipe issues at 1/64 of the FP32 rate, and a per-end FP64 add (with the
// conversion of each addend) would cost more than the whole contact evaluation.
struct DF6 {
    float h[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, l[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    __device__ __forceinline__ void add1(int k, float v) {
        float s, e;
        twoSum(h[k], v, s, e);
        h[k] = s;
        l[k] = __fadd_rn(l[k], e);
    }
    __device__ __forceinline__ void add(const float4& x, const float2& y) {
        add1(0, x.x); add1(1, x.y); add1(2, x.z);
        add1(3, x.w); add1(4, y.x); add1(5, y.y);
    }
    // start the force from m*g, both given as double-float pairs: the exact product of the high
    // parts (FMA residual) plus the cross terms
    __device__ __forceinline__ void initGravity(float mh, float ml, const float* gh, const float* gl) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float p = mh * gh[k];
            h[k] = p;
            l[k] = fmaf(mh, gh[k], -p) + (mh * gl[k] + ml * gh[k]);
        }
    }
    __device__ __forceinline__ double val(int k) const { return (double)h[k] + (double)l[k]; }
    __device__ __forceinline__ float net(int k) const { return __fadd_rn(h[k], l[k]); }
};

// Asynchronous global -> shared copy of one element of 8, 16 or 32 bytes (cp.async: the copies of
// a lane are in flight together and hold no registers).
template <int BYTES>
__device__ __forceinline__ void cpAsync(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (BYTES == 8) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    } else if constexpr (BYTES == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
    } else {
        static_assert(BYTES == 32, "8, 16 or 32 bytes");
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d + 16u), "l"((const char*)src + 16) : "memory");
    }
}
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Adds the end slots [e0, e1) of every lane with take==true to acc. Must be called by all
// 32 lanes of the warp (warp-uniform control flow inside). Each chunk of the warp's run of slots
// is copied to shared memory with cp.async, all of a lane's copies in flight at once.
template <typename EA, typename EB, int CH, typename Acc>
__device__ __forceinline__ void warpSumEnds(const EA* __restrict__ endA, const EB* __restrict__ endB, bool take, int e0, int e1,
                                            EndStage<EA, EB, CH>& st, Acc& acc) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    if (!take) { e0 = 0; e1 = 0; }
    const unsigned skip = __ballot_sync(FULL, !take || e1 <= e0);
    int g = 0;
    while (g < 32) {
        const unsigned cand = ~skip & (FULL << g);
        if (!cand) break;
        const int s = __ffs(cand) - 1;                       // first lane of a group of takers
        const unsigned after = skip & (FULL << s);
        const int e = after ? __ffs(after) - 1 : 32;         // one past its last lane
        const int lo = __shfl_sync(FULL, e0, s), hi = __shfl_sync(FULL, e1, e - 1);
        for (int base = lo; base < hi; base += CH) {
            const int cnt = min(CH, hi - base);
#pragma unroll
            for (int u = 0; u < CH / 32; u++) {
                const int q = lane + 32 * u;
                if (q < cnt) {
                    cpAsync<sizeof(EA)>(&st.a[q], &endA[base + q]);
                    cpAsync<sizeof(EB)>(&st.b[q], &endB[base + q]);
                }
            }
            cpAsyncWaitAll();
            __syncwarp();
            if (lane >= s && lane < e) {
                const int a = max(e0, base), b = min(e1, base + cnt);
                for (int q = a; q < b; q++) acc.add(st.a[q - base], st.b[q - base]);
            }
            __syncwarp();
        }
        g = e;
    }
}

// Degree of particle p in the incidence and the first of its end slots.
__device__ __forceinline__ void endRange(const DevIncidence& I, int p, int& e0, int& e1) {
    e0 = I.hiStart[p] + I.loStart[p];
    e1 = I.hiStart[p + 1] + I.loStart[p + 1];
}

// Step-loop guard: a kernel of a step does nothing once a full collider run is pending, an
// error was raised, or an earlier step halted the queued steps.
__device__ __forceinline__ bool halted(const int* f) { return f[FL_HALT] != 0 || f[FL_ERR] != 0; }

}  // namespace wg
