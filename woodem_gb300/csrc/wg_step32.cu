// FP32-force mode: contact geometry and force laws in FP32; FP64 kept for the steps where
// FP32 would lose the result -- the relative position of the two particles and the normal
// overlap (a difference of nearly equal lengths), the relative velocity, the incremental
// shear force of IdealElPl, the Leapfrog position/velocity update and the per-particle force
// sum. The physics and its order of evaluation are those of the FP64 path (wg_step.cu), with
// the sphere-sphere branch vectors written relative to the particle centres:
//   contact point - x_A = (r1 + uN/2) n,   contact point - x_B' = -(r2 + uN/2) n
// which is Cg2_Sphere_Sphere_L6Geom's contPt = x1 + (r1 + uN/2) n (pkg/dem/Sphere.cpp:103), so the
// mid-step branches of L6Geom.cpp:156-160 need only the previous normal and uN.
//
// Compiled with --fmad=true (results are compared to the FP64 oracle within a tolerance).
#include <algorithm>
#include <mutex>

#include "wg_ends.cuh"
#include "wg_energy.cuh"
#include "wg_geom.cuh"

namespace wg {

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 toF(D3 a) { return F3{(float)a.x, (float)a.y, (float)a.z}; }
// x truncated toward zero to FP32 with 32-bit integer operations on its words (no FP64-pipe
// conversion on any path): |x| below the FP32 normal range gives a signed zero, finite |x| from
// 2^128 up the largest FP32 of its sign; infinities and NaN stay what they are.
__device__ __forceinline__ float d2fT(double x) {
    const unsigned top = (unsigned)__double2hiint(x), bot = (unsigned)__double2loint(x);
    const unsigned sign = top & 0x80000000u;
    const int e = (int)((top >> 20) & 0x7ffu);
    if (e < 897) return __uint_as_float(sign);
    if (e > 1150) {
        if (e < 2047) return __uint_as_float(sign | 0x7F7FFFFFu);
        return __uint_as_float(sign | 0x7F800000u | ((((top & 0xFFFFFu) | bot) != 0) ? 0x400000u : 0u));
    }
    return __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((top & 0xFFFFFu) << 3) | (bot >> 29));
}
__device__ __forceinline__ F3 toFt(D3 a) { return F3{d2fT(a.x), d2fT(a.y), d2fT(a.z)}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator-(F3 a) { return F3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 fcross(F3 a, F3 b) { return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
// x = h + l from the bits of x with 32-bit integer operations on its two words, on every path:
// FP64 arithmetic and conversions issue at 1/64 of the FP32 rate on GB300, and the compiler
// turns a rarely taken branch into predicated instructions that occupy the FP64 pipe in every
// warp. h is x truncated to 24 significant bits, l the remaining 29 mantissa bits truncated to
// 24, so |x - (h + l)| < 2^-47 |x|. Below 2^-74 (zero included) l is dropped (h = x truncated,
// or a signed zero under the FP32 normal range: an absolute error below 2^-97); from 2^127 up h
// is the signed infinity (NaN stays NaN) and l zero.
__device__ __forceinline__ void splitDF(double x, float& h, float& l) {
    const unsigned top = (unsigned)__double2hiint(x), bot = (unsigned)__double2loint(x);
    const unsigned sign = top & 0x80000000u;
    const int e = (int)((top >> 20) & 0x7ffu);
    if (e < 949) {
        h = __uint_as_float(e >= 897 ? (sign | ((unsigned)(e - 896) << 23) | ((top & 0xFFFFFu) << 3) | (bot >> 29)) : sign);
        l = 0.f;
        return;
    }
    if (e > 1150) {
        const bool nan = e == 2047 && ((top & 0xFFFFFu) | bot) != 0;
        h = __uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u));
        l = 0.f;
        return;
    }
    // the 52 mantissa bits are (top & 0xfffff):bot; h keeps the upper 23
    h = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | ((top & 0xFFFFFu) << 3) | (bot >> 29));
    const unsigned r = bot & 0x1FFFFFFFu;
    if (r == 0) {
        l = 0.f;
        return;
    }
    const int p = 31 - __clz((int)r);  // r = 1.f * 2^p, 0 <= p <= 28
    const unsigned frac = (p >= 23) ? (r >> (p - 23)) : (r << (23 - p));
    l = __uint_as_float(sign | ((unsigned)(p + e - 948) << 23) | (frac & 0x7FFFFFu));
}
// (double)f from the bits of f with 32-bit integer operations (exact for normal numbers,
// infinities and NaN; FP32 subnormals, below 1.2e-38, become zero).
__device__ __forceinline__ double f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned sign = u & 0x80000000u;
    if (e == 0) return __hiloint2double((int)sign, 0);
    const unsigned mant = u & 0x7fffffu;
    const unsigned ed = (e == 0xffu) ? 0x7ffu : e + 896u;
    return __hiloint2double((int)(sign | (ed << 20) | (mant >> 3)), (int)(mant << 29));
}
// x rounded toward zero to FP32 (the h of splitDF)
__device__ __forceinline__ float truncF(double x) {
    float h, l;
    splitDF(x, h, l);
    return h;
}
__device__ __forceinline__ F3 fnormalized(F3 a) {
    const float z = fdot(a, a);
    return z > 0.f ? a * rsqrtf(z) : a;
}

// ---------------------------------------------------------------------------------- Leapfrog
__device__ __forceinline__ float fsgn(float s) { return s < 0.f ? -1.f : (s > 0.f ? 1.f : 0.f); }

// Leapfrog::run (pkg/dem/Leapfrog.cpp:103-255), FP32-force mode. The force and torque of the step
// (m*g plus the compensated sum of the particle's FP32 end slots) give the accelerations in FP32;
// the velocity, angular velocity and position are accumulated in FP64:
//   vel += fl64(dt*a),  angVel += fl64(dt*alpha),  pos += vel*dt.
// The orientation, which no force of the supported shapes depends on, is advanced in FP32.
// Writes the double-float mirrors of position and velocity used by the contact kernel.
// The node state is loaded before the end-slot sum so that its loads overlap the staging.
// m*g written as the force of a node no contact sum rebuilds (facet vertices): kept out of line so
// that its FP64 arithmetic is a branch, not predicated instructions in every warp
__device__ __noinline__ void resetNodeForce(DevNodes N, int i, float mh, float ml, bool gravity, const ScenePar* __restrict__ spp,
                                            int scene) {
    const ScenePar& sp = spp[scene];
    D3 G{0, 0, 0};
    if (gravity) G = ((double)mh + (double)ml) * D3{sp.g[0], sp.g[1], sp.g[2]};
    N.force[i] = make_double4_32a(G.x, G.y, G.z, 0.);
    N.torque[i] = make_double4_32a(0., 0., 0., 0.);
}

// PERI: the scene is periodic (homothetic corrections of Leapfrog.cpp:103-255 with the cell's
// velocity gradient); the aperiodic instantiation carries none of that FP64 code.
// ENERGY: Scene.trackEnergy; each node writes its step's energy terms (Leapfrog.cpp:52-97, in FP64
// from this step's force and torque) into E, as the FP64 Leapfrog does.
template <bool PERI, bool ENERGY>
__global__ void __launch_bounds__(256) k_leapfrog32(DevNodes N, DevParticles P, DevIncidence I, const NodeConst32* __restrict__ ncs,
                                                    const ScenePar* __restrict__ spp, int* __restrict__ dFlags, int fromEnds,
                                                    const long long* __restrict__ dStepC, EnergyCols E) {
    __shared__ EndStage<float4, float2, kLeapfrogChunk32> stage[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < N.n;
    // every load of the node is issued before the step guard (nothing is written before it), so
    // that they are in flight together
    const int ii = valid ? i : 0;
    const NodeConst32 nc = ncs[ii];
    const double4_32a pr = N.posr[ii], v4 = N.vel[ii], w4 = N.angv[ii];
    const float4 lh = N.lh[ii], ll = N.ll[ii], o = N.orif[ii];
    const int pi = ii < P.n ? ii : 0;
    const bool freshLd = N.fresh && N.fresh[ii];
    int hs0 = 0, hs1 = 0, ls0 = 0, ls1 = 0;
    if (fromEnds) {
        hs0 = I.hiStart[pi];
        hs1 = I.hiStart[pi + 1];
        ls0 = I.loStart[pi];
        ls1 = I.loStart[pi + 1];
    }
    const long long stepAbs = *dStepC;
    const int scene = valid ? sceneOfN(N, i) : 0;
    if (halted(dFlags)) return;
    const ScenePar& sp = spp[scene];
    const uint32_t flags = nc.flags;
    // DemData.force/torque of this step
    const bool uni = valid && (nc.kind & NK_SUMMED);
    // a scene past its last step (serving slot) is frozen; a node just (re)loaded takes its stored force
    const bool frozen = valid && (stepAbs - sp.stepBase) >= sp.stepEnd;
    const bool fresh = valid && freshLd;
    int e0 = 0, e1 = 0;
    bool take = false, summed = false;
    DF6 acc;
    if (fromEnds && uni && !fresh && !frozen) {
        if (sp.hasGravity && !(flags & F_GRAVITY_SKIP)) acc.initGravity(nc.mh, nc.ml, sp.gH, sp.gL);
        summed = true;
        if (sp.applyForces) {
            e0 = hs0 + ls0;
            e1 = hs1 + ls1;
            take = (e1 - e0) <= kHeavyThreshold;
            summed = take;
        }
    }
    warpSumEnds(I.endAf, I.endBf, take, e0, e1, stage[threadIdx.x >> 5], acc);
    if (!valid || (flags & F_CLUMPED) || frozen) return;
    if (fresh) N.fresh[i] = 0;
    F3 f, t;
    if (summed) {
        f = F3{acc.net(0), acc.net(1), acc.net(2)};
        t = F3{acc.net(3), acc.net(4), acc.net(5)};
    } else {  // the stored value: first step after the host wrote the state, or a heavy particle
        f = toFt(ld3(N.force[i]));
        t = toFt(ld3(N.torque[i]));
    }
    const double dt = sp.dt;
    const float dtf = sp.dtF;
    const bool damp = (sp.dampingF != 0.f && !(flags & F_DAMPING_SKIP));
    D3 pos = ld3(pr);
    D3 vel = ld3(v4);
    D3 angVel = ld3(w4);
    const bool blockedAll = (flags & F_DOF_ALL) == F_DOF_ALL;
    const int homoDeform = PERI ? sp.homoDeform : -1;
    F3 la{0.f, 0.f, 0.f}, aaE{0.f, 0.f, 0.f};
    D3 pvfE = vel, pvaE = angVel;
    if constexpr (ENERGY) {
        if (sp.trackEnergy) {
            const D3 fd{(double)f.x, (double)f.y, (double)f.z}, td{(double)t.x, (double)t.y, (double)t.z};
            const double mass = (double)nc.mh + (double)nc.ml;
            if (damp && !(flags & F_ENERGY_SKIP)) E.col[EN_NODE_DAMP * E.cap + i] = energyDamp(vel, fd, angVel, td, sp.damping, dt);
            if (sp.hasGravity && !(flags & F_GRAVITY_SKIP)) {
                E.col[EN_NODE_GRAV * E.cap + i] = energyGrav(D3{sp.g[0], sp.g[1], sp.g[2]}, vel, mass, dt, flags);
                E.col[EN_NODE_NGRAV * E.cap + i] = 1.;
            }
            if (PERI) {
                if (homoDeform == 2 || homoDeform == 3) pvfE = vel - mul(*(const DM3*)sp.gradV, pos);
                else if (homoDeform == 4) pvfE = vel - mul(*(const DM3*)sp.gradV, pos - (dt / 2) * vel);
                if (homoDeform == 4) pvaE = angVel - D3{sp.spinVec[0], sp.spinVec[1], sp.spinVec[2]};
            }
        }
    }
    if (!blockedAll) {
        la = F3{(flags & 1u) ? 0.f : f.x * nc.invMass, (flags & 2u) ? 0.f : f.y * nc.invMass, (flags & 4u) ? 0.f : f.z * nc.invMass};
        F3 pvf{0.f, 0.f, 0.f}, pva{0.f, 0.f, 0.f};
        if (damp) {
            // nonviscDamp2nd (Leapfrog.cpp:32-34) on the fluctuation velocity (Cell.cpp:36-57)
            D3 v = vel, w = angVel;
            if (PERI) {
                if (homoDeform == 2 || homoDeform == 3) v = vel - mul(*(const DM3*)sp.gradV, pos);
                else if (homoDeform == 4) v = vel - mul(*(const DM3*)sp.gradV, pos - (dt / 2) * vel);
                if (homoDeform == 4) w = angVel - D3{sp.spinVec[0], sp.spinVec[1], sp.spinVec[2]};
            }
            pvf = toFt(v);
            pva = toFt(w);
            const float d = sp.dampingF;
            la.x *= 1.f - d * fsgn(f.x * (pvf.x + 0.5f * dtf * la.x));
            la.y *= 1.f - d * fsgn(f.y * (pvf.y + 0.5f * dtf * la.y));
            la.z *= 1.f - d * fsgn(f.z * (pvf.z + 0.5f * dtf * la.z));
        }
        if (PERI && homoDeform == 4)
            vel = mul(*(const DM3*)sp.ImLL4hInv, (mul(*(const DM3*)sp.LmL, pos) + mul(*(const DM3*)sp.IpLL4h, vel)) +
                                                   D3{(double)la.x, (double)la.y, (double)la.z} * dt);
        else
            vel = vel + D3{f2d(dtf * la.x), f2d(dtf * la.y), f2d(dtf * la.z)};
        if (nc.invI[0] != 0.f || nc.invI[1] != 0.f || nc.invI[2] != 0.f) {
            F3 aa{(flags & 8u) ? 0.f : t.x * nc.invI[0], (flags & 16u) ? 0.f : t.y * nc.invI[1], (flags & 32u) ? 0.f : t.z * nc.invI[2]};
            if (damp) {
                const float d = sp.dampingF;
                aa.x *= 1.f - d * fsgn(t.x * (pva.x + 0.5f * dtf * aa.x));
                aa.y *= 1.f - d * fsgn(t.y * (pva.y + 0.5f * dtf * aa.y));
                aa.z *= 1.f - d * fsgn(t.z * (pva.z + 0.5f * dtf * aa.z));
            }
            angVel = angVel + D3{f2d(dtf * aa.x), f2d(dtf * aa.y), f2d(dtf * aa.z)};
            if constexpr (ENERGY) aaE = aa;
            if (PERI && homoDeform == 4) angVel = angVel - D3{sp.deltaSpinVec[0], sp.deltaSpinVec[1], sp.deltaSpinVec[2]};
        }
    } else {
        if (PERI && homoDeform == 4) vel = mul(*(const DM3*)sp.ImLL4hInv, mul(*(const DM3*)sp.LmL, pos) + mul(*(const DM3*)sp.IpLL4h, vel));
    }
    if (PERI && homoDeform >= 0 && homoDeform != 4) {
        const D3 lad{(double)la.x, (double)la.y, (double)la.z};
        if (homoDeform == 2 || homoDeform == 3) {
            if (homoDeform == 3) vel = vel + mul(*(const DM3*)sp.midGradV, vel - (dt / 2.) * lad) * dt;
            vel = vel + mul(*(const DM3*)sp.dGradV, pos);
        } else if (homoDeform == 1) {
            pos = pos + mul(*(const DM3*)sp.nextGradV, pos) * dt;
        }
    }
    if constexpr (ENERGY) {
        if (sp.trackEnergy && !(flags & F_ENERGY_SKIP)) {
            const double4_32a mi = N.minert[i];
            const double2 ek = energyKin(pvfE, pvaE, D3{(double)la.x, (double)la.y, (double)la.z},
                                         D3{(double)aaE.x, (double)aaE.y, (double)aaE.z}, (double)nc.mh + (double)nc.ml,
                                         D3{mi.x, mi.y, mi.z}, dt);
            if (sp.kinSplit) {
                E.col[EN_NODE_K0 * E.cap + i] = ek.x;
                E.col[EN_NODE_K1 * E.cap + i] = ek.y;
            } else
                E.col[EN_NODE_K0 * E.cap + i] = ek.x + ek.y;
            E.col[EN_NODE_NKIN * E.cap + i] = 1.;
        }
    }
    pos = pos + vel * dt;
    N.posr[i] = make_double4_32a(pos.x, pos.y, pos.z, pr.w);
    N.vel[i] = make_double4_32a(vel.x, vel.y, vel.z, 0.);
    N.angv[i] = make_double4_32a(angVel.x, angVel.y, angVel.z, 0.);
    const F3 w{truncF(angVel.x), truncF(angVel.y), truncF(angVel.z)};
    {
        // double-float mirrors read by the sphere-sphere contact geometry
        Mirror m;
        splitDF(pos.x, m.ph.x, m.pl.x);
        splitDF(pos.y, m.ph.y, m.pl.y);
        splitDF(pos.z, m.ph.z, m.pl.z);
        splitDF(pr.w, m.ph.w, m.pl.w);  // the radius
        // verlet test (InsertionSortCollider.cpp:339-350): displacement since the last full run
        // from the double-float mirrors, in FP32
        const float dx = (m.ph.x - lh.x) + (m.pl.x - ll.x), dy = (m.ph.y - lh.y) + (m.pl.y - ll.y),
                    dz = (m.ph.z - lh.z) + (m.pl.z - ll.z);
        if (dx * dx + dy * dy + dz * dz > sp.maxD2F) atomicOr(dFlags + FL_FULL, 1);
        splitDF(vel.x, m.vh.x, m.vl.x);
        splitDF(vel.y, m.vh.y, m.vl.y);
        splitDF(vel.z, m.vh.z, m.vl.z);
        m.vh.w = w.x;
        m.vl.w = w.y;
        N.mir[i] = m;
        N.wz[i] = w.z;
    }
    const float ang = sqrtf(fdot(w, w));
    if (ang > 0.f) {
        // leapfrogSphericalRotate (Leapfrog.cpp:280-288) in FP32
        float s, c;
        sincosf(0.5f * ang * dtf, &s, &c);
        const F3 ax = w * (1.f / ang);
        const float qw = c, qx = s * ax.x, qy = s * ax.y, qz = s * ax.z;
        const float ow = o.x, ox = o.y, oy = o.z, oz = o.w;
        float rw = qw * ow - qx * ox - qy * oy - qz * oz;
        float rx = qw * ox + qx * ow + qy * oz - qz * oy;
        float ry = qw * oy + qy * ow + qz * ox - qx * oz;
        float rz = qw * oz + qz * ow + qx * oy - qy * ox;
        const float inv = rsqrtf(rw * rw + rx * rx + ry * ry + rz * rz);
        N.orif[i] = make_float4(rw * inv, rx * inv, ry * inv, rz * inv);
    }
    // force reset of nodes whose force is not rebuilt by the contact sum (facet vertices)
    if (sp.reset && !uni) resetNodeForce(N, i, nc.mh, nc.ml, sp.hasGravity && !(flags & F_GRAVITY_SKIP), spp, scene);
}

void launch_leapfrog32(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const NodeConst32* nc,
                       const ScenePar* sp, int* dFlags, int fromEnds, const long long* dStep, bool periodic, const EnergyCols* energy) {
    if (N.n == 0) return;
    const unsigned g = (N.n + 255) / 256;
    const EnergyCols E = energy ? *energy : EnergyCols{};
    if (energy) {
        if (periodic) k_leapfrog32<true, true><<<g, 256, 0, st>>>(N, P, I, nc, sp, dFlags, fromEnds, dStep, E);
        else k_leapfrog32<false, true><<<g, 256, 0, st>>>(N, P, I, nc, sp, dFlags, fromEnds, dStep, E);
    } else {
        if (periodic) k_leapfrog32<true, false><<<g, 256, 0, st>>>(N, P, I, nc, sp, dFlags, fromEnds, dStep, E);
        else k_leapfrog32<false, false><<<g, 256, 0, st>>>(N, P, I, nc, sp, dFlags, fromEnds, dStep, E);
    }
}

// ---------------------------------------------------------------------------------- ContactLoop
struct Frame {
    F3 c0, c1, c2;
};

// L6Geom update of the frame (pkg/dem/L6Geom.cpp:80-137) for approxMask==0; returns the
// mid-step frame in m and writes the current frame to f.
__device__ __forceinline__ void frameUpdate(F3 prevN, F3 prevC1, F3 n, F3 w1, F3 w2, float dt, bool renorm, Frame& f, Frame& m) {
    const F3 normRotVec = fcross(prevN, n);
    F3 midN = 0.5f * (prevN + n);
    const float mn2 = fdot(midN, midN);
    midN = (mn2 == 0.f) ? n : midN * rsqrtf(mn2);
    const F3 twist = midN * (dt * 0.5f * fdot(midN, w1 + w2));
    const F3 rt = normRotVec + twist;
    m.c0 = midN;
    m.c1 = prevC1 - 0.5f * fcross(prevC1, rt);
    m.c2 = fcross(m.c0, m.c1);
    f.c0 = n;
    f.c1 = prevC1 - fcross(m.c1, rt);
    if (renorm) {
        f.c0 = fnormalized(f.c0);
        f.c1 = f.c1 - f.c0 * fdot(f.c1, f.c0);
        f.c1 = fnormalized(f.c1);
    }
    f.c2 = fcross(f.c0, f.c1);
}
// L6Geom::setInitialLocalCoords, pkg/dem/L6Geom.cpp:27-38
__device__ __forceinline__ void frameInit(F3 n, Frame& f) {
    const F3 ref = (fabsf(n.y) < fabsf(n.z)) ? F3{0, 1, 0} : F3{0, 0, 1};
    F3 y = fcross(n, ref);
    y = fnormalized(y - n * fdot(y, n));
    f.c0 = n;
    f.c1 = y;
    f.c2 = fcross(n, y);
}

// ---- double-float arithmetic for the sphere-sphere geometry (FP32 pipe only)
// Sphere-sphere overlap test and normal overlap without FP64 arithmetic. Positions, velocities
// and radii are read from the double-float mirrors written by Leapfrog (x = hi + lo, both FP32,
// |x - (hi + lo)| <= 2^-48 |x|), so the relative position carries ~47 bits and
//   num = |dx|^2 - (r1 + r2)^2
// is formed with error-free products and sums: its error is ~2^-46 |dx|^2, i.e. about
// 1e-9 relative for an overlap of 1e-3 radius, far below the FP32 rounding of the force.
// uN = num / (|dx| + r1 + r2) is then the overlap of Cg2_Sphere_Sphere_L6Geom
// (pkg/dem/Sphere.cpp:97-101) without the cancellation of |dx| - (r1 + r2).
struct SSGeo {
    F3 n, dv, w1, w2;
    float uN, r1, r2;
};
__device__ __forceinline__ bool geomSS32(const Mirror& ma, const Mirror& mb, float wza, float wzb, float dfAbs, bool real, SSGeo& g) {
    const float4 ha = ma.ph, la = ma.pl, hb = mb.ph, lb = mb.pl;
    float sx, tx, sy, ty, sz, tz;
    dfDiff(ha.x, la.x, hb.x, lb.x, sx, tx);
    dfDiff(ha.y, la.y, hb.y, lb.y, sy, ty);
    dfDiff(ha.z, la.z, hb.z, lb.z, sz, tz);
    float px, cx, py, cy, pz, cz;
    dfSquare(sx, tx, px, cx);
    dfSquare(sy, ty, py, cy);
    dfSquare(sz, tz, pz, cz);
    float Rs, Re;
    twoSum(ha.w, hb.w, Rs, Re);
    const float Rt = Re + (la.w + lb.w);
    float a1, e1, a2, e2;
    twoSum(px, py, a1, e1);
    twoSum(a1, pz, a2, e2);
    const float csum = (e1 + e2) + (cx + cy + cz);
    // creation test of Sphere.cpp:94-96 against (|distFactor| (r1 + r2))^2
    float Ds = Rs, Dt = Rt;
    if (dfAbs != 1.f) {
        float pe;
        Ds = dfAbs * Rs;
        pe = fmaf(dfAbs, Rs, -Ds);
        Dt = pe + dfAbs * Rt;
    }
    float Dp, Dc;
    dfSquare(Ds, Dt, Dp, Dc);
    float b3, e3;
    twoSum(a2, -Dp, b3, e3);
    const float unDist = b3 + (e3 + (csum - Dc));
    if (unDist > 0.f && !real) return false;
    float num = unDist;
    if (dfAbs != 1.f) {
        float Rp, Rc;
        dfSquare(Rs, Rt, Rp, Rc);
        twoSum(a2, -Rp, b3, e3);
        num = b3 + (e3 + (csum - Rc));
    }
    const F3 dx{sx + tx, sy + ty, sz + tz};
    const float dist = sqrtf(a2 + csum);
    const float R = Rs + Rt;
    g.uN = num / (dist + R);
    g.n = dx * (1.f / dist);
    g.r1 = ha.w + la.w;
    g.r2 = hb.w + lb.w;
    const float4 vha = ma.vh, vla = ma.vl, vhb = mb.vh, vlb = mb.vl;
    float s, t;
    dfDiff(vha.x, vla.x, vhb.x, vlb.x, s, t);
    g.dv.x = s + t;
    dfDiff(vha.y, vla.y, vhb.y, vlb.y, s, t);
    g.dv.y = s + t;
    dfDiff(vha.z, vla.z, vhb.z, vlb.z, s, t);
    g.dv.z = s + t;
    g.w1 = F3{vha.w, vla.w, wza};
    g.w2 = F3{vhb.w, vlb.w, wzb};
    return true;
}

// L6Geom::trsf renormalisation step (L6Geom.cpp:129-135): every trsfRenorm-th step
__device__ __forceinline__ bool renormStep(long long step, int every) {
    if (every <= 0) return false;
    if (step >= 0 && step < 0x7fffffffLL) return ((unsigned)step % (unsigned)every) == 0u;
    return (step % every) == 0;
}

// Cp2_FrictMat_FrictPhys / Cp2_FrictMat_HertzPhys on contact creation (FrictMat.cpp:20-44,
// Hertz.cpp:9-50), evaluated in FP64 from the FP32 geometry; ma/mb: the two nodes' mass. Out of
// line: its FP64 arithmetic runs only in warps that create a contact (rare paths of FP64 code
// inlined into a kernel become predicated instructions that occupy the FP64 pipe in every warp).
struct Phys4 {
    float p0, p1, p2, p3;
};
__device__ __noinline__ Phys4 physCreateFP64(const ScenePar* __restrict__ spp, int scene, float r1, float r2, float uN,
                                             double4_32a m1, double4_32a m2, double ma, double mb) {
    const ScenePar& sp = spp[scene];
    float ph0, ph1, ph2, ph3;
    double lens0 = fabs((double)r1) + (double)uN / 2, lens1 = fabs((double)r2) + (double)uN / 2;
    if (lens0 < 0) lens0 = lens1;
    if (lens1 < 0) lens1 = lens0;
    const double rr = (r1 > 0 && r2 > 0) ? fmin((double)r1, (double)r2) : (r1 > 0 ? (double)r1 : (double)r2);
    const double contA = 3.14159265358979323846 * (rr * rr);
    ph3 = 0.f;
    if (sp.phys == 0) {
        const double kn = 1 / (1 / (m1.y * contA / lens0) + 1 / (m2.y * contA / lens1));
        ph0 = (float)kn;
        ph1 = (float)(.5 * (m1.w + m2.w) * kn);
        ph2 = (float)fmin(m1.z, m2.z);
    } else {
        const double nu = sp.hzPoisson;
        const double K = (4 / 3.) / ((1 - nu * nu) / m1.y + (1 - nu * nu) / m2.y);
        const double R = 1. / (1. / lens0 + 1. / lens1);
        const double kn0 = K * sqrt(R);
        const double G = .5 * (m1.y / (2 * (1 + nu)) + m2.y / (2 * (1 + nu)));
        ph0 = (float)kn0;
        ph1 = (float)(2 * sqrt(4 * R) * G / (2 - nu));
        ph2 = (float)fmin(m1.z, m2.z);
        if (sp.hzViscOn) {
            const double mbar = (ma <= 0 && mb > 0) ? mb : ((ma > 0 && mb <= 0) ? ma : (ma * mb) / (ma + mb));
            ph3 = (float)fmax(0., sp.hzViscConst * sqrt(mbar * kn0));
        }
    }
    return Phys4{ph0, ph1, ph2, ph3};
}
__device__ __forceinline__ void physCreate(const ScenePar* __restrict__ spp, int scene, float r1, float r2, float uN, const double4_32a& m1,
                                           const double4_32a& m2, double ma, double mb, float& ph0, float& ph1, float& ph2,
                                           float& ph3) {
    const Phys4 q = physCreateFP64(spp, scene, r1, r2, uN, m1, m2, ma, mb);
    ph0 = q.p0;
    ph1 = q.p1;
    ph2 = q.p2;
    ph3 = q.p3;
}

// Energies of one contact in one step (Scene.trackEnergy: EnergyTracker adds of IdealElPl.cpp:25-37,
// 58-90 and Hertz.cpp:154-179), in FP64 from the FP32 quantities of the law, written to the contact's
// entry of the per-step energy columns (zeroed before the step) as the FP64 contact kernel does.
struct EnergyTerms {
    double elast = 0, plast = 0, broken = 0, viscN = 0, viscT = 0, nElast = 0, nBroken = 0;
    // IdealElPl: the elastic potential of a contact that breaks (noSlip), lost
    __device__ __noinline__ void brokenElPl(float kn, float kt, float uN, double b1, double b2) {
        const double bf = (double)kn * (double)uN;
        broken = .5 * ((bf * bf) / (double)kn + (b1 * b1 + b2 * b2) / (double)kt);
        nBroken = 1;
    }
    // IdealElPl: dissipation of the Coulomb slip, from the trial shear force (squared norm q)
    __device__ __noinline__ void plastElPl(float kt, double maxFt, double q) {
        plast = kt != 0.f ? (maxFt * (sqrt(q) - maxFt)) / (double)kt : 0.;
    }
    __device__ __noinline__ void elastElPl(float kn, float kt, float fn, float ft1, float ft2) {
        const double n = fn, a = ft1, b = ft2;
        elast = 0.5 * ((n * n) / (double)kn + (kt != 0.f ? (a * a + b * b) / (double)kt : 0.));
        if (isnan(elast)) elast = 0.;
        nElast = 1;
    }
    // Hertz: slip dissipation from the trial shear force (squared norm q), tangent stiffness kt
    __device__ __noinline__ void plastHertz(float q, float maxFt, float kt) {
        const double fN = sqrt((double)q), m = maxFt;
        plast = ((.5 * (fN - m) + m) * (fN - m)) / (double)kt;
    }
    // Hertz: kn0 (2/5) (-uN)^(5/2) + |Ft|^2 / (2 kt), su = sqrt(-uN)
    __device__ __noinline__ void elastHertz(float kn0, float su, float ft1, float ft2, float kt) {
        const double s = su, a = ft1, b = ft2;
        elast = ((double)kn0 * (2 / 5.)) * ((((s * s) * s) * s) * s) + (0.5 * (a * a + b * b)) / (double)kt;
        nElast = 1;
    }
    __device__ __forceinline__ void store(const EnergyCols& E, int64_t rk) const {
        const int64_t cp = E.cap;
        E.col[EN_CON_ELAST * cp + rk] = elast;
        E.col[EN_CON_PLAST * cp + rk] = plast;
        E.col[EN_CON_BROKEN * cp + rk] = broken;
        E.col[EN_CON_VISCN * cp + rk] = viscN;
        E.col[EN_CON_VISCT * cp + rk] = viscT;
        E.col[EN_CON_NELAST * cp + rk] = nElast;
        E.col[EN_CON_NBROKEN * cp + rk] = nBroken;
    }
};

// The values one sphere-sphere contact is evaluated from: its packed item, flags, state and the
// two particles' mirror records.
struct SSIn {
    int4 it;
    uint32_t pf;
    float st[CF_NCOL];
    double ft1o, ft2o;
    Mirror ma, mb;
    float wza, wzb;
};

// k_step_advance folded into the last kernel(s) of a step: every block of the `total` blocks of
// those kernels calls this at its end; the last one to finish advances the step counter (unless
// the queued steps were halted) and resets the ticket. total <= 0: nothing.
__device__ __forceinline__ void stepTicket(int* dFlags, long long* dStep, int total) {
    if (total <= 0) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(dFlags + FL_TICKET, 1) == total - 1) {
            dFlags[FL_TICKET] = 0;
            if (!halted(dFlags)) *dStep += 1;
        }
    }
}

// One sphere-sphere contact of an aperiodic scene (packed position j): Cg2_Sphere_Sphere_L6Geom,
// Cp2 on creation, Law2, the two end slots and the packed state. FP32 arithmetic throughout
// except the IdealElPl shear accumulation (FP64) and contact creation.
template <bool ENERGY>
__device__ __forceinline__ void ssContact(const SSIn& x, int64_t j, const DevNodes& N, const DevParticles& P, const DevContacts& C,
                                          const DevIncidence& I, const DevPackedSS& K, const double4_32a* __restrict__ mats,
                                          const ScenePar* __restrict__ spp, long long stepAbs, int* dFlags, int64_t nm,
                                          const EnergyCols& E) {
    const int4 it = x.it;
    const uint32_t pf = x.pf;
    const float* st = x.st;
    double ft1o = x.ft1o, ft2o = x.ft2o;
    int* dErr = dFlags + FL_ERR;
    const int A = it.x, B = it.y;
    const ScenePar& sp = spp[pf >> 8];
    const long long step = stepAbs - sp.stepBase;
    if (step >= sp.stepEnd) return;  // frozen scene (serving slot past its last step)
    const uint32_t fl0 = pf & 0xffu, hiBits = pf & ~0xffu;
    uint32_t fl = fl0;
    if (fl & C_REMOVED) return;
    if ((fl & C_PENDING) && !pendingStays(P, A, B, false, nullptr, dErr)) {
        K.flags[j] = ((fl & ~C_PENDING) | C_REMOVED) | hiBits;
        return;
    }
    fl &= ~C_PENDING;
    const bool real = fl & C_REAL;
    SSGeo g;
    if (!geomSS32(x.ma, x.mb, x.wza, x.wzb, sp.ssDfAbsF, real, g)) {
        if (fl != fl0) K.flags[j] = fl | hiBits;
        return;
    }
    const float dtf = sp.dtF;
    const F3 n = g.n;
    const float uN = g.uN, r1 = g.r1, r2 = g.r2;
    // contPt = x1 + (r1 + uN/2) n (Sphere.cpp:103), written relative to both centres
    const F3 armA = (r1 + 0.5f * uN) * n;
    const F3 armB = -(r2 + 0.5f * uN) * n;
    Frame f, m;
    F3 lvel{0, 0, 0};
    float ph0, ph1, ph2, ph3;
    if (!real) {
        frameInit(n, f);
        physCreate(spp, (int)(pf >> 8), r1, r2, uN, mats[P.mat[A]], mats[P.mat[B]], N.minert[A].w, N.minert[B].w, ph0, ph1, ph2, ph3);
        K.col[CF_P0][j] = ph0;
        K.col[CF_P1][j] = ph1;
        K.col[CF_P2][j] = ph2;
        K.col[CF_P3][j] = ph3;
        C.step0[I.work[nm + j].x] = (int32_t)step;
        ft1o = 0.;
        ft2o = 0.;
        if (sp.law == 0) {
            K.ft[0][j] = 0.;
            K.ft[1][j] = 0.;
        }
    } else {
        const F3 pn{st[CF_T0X], st[CF_T0Y], st[CF_T0Z]};
        const F3 pc1{st[CF_T1X], st[CF_T1Y], st[CF_T1Z]};
        const float up = st[CF_UN];
        // mid-step branch vectors (L6Geom.cpp:156-160)
        const F3 c1x = 0.5f * ((r1 + 0.5f * up) * pn + armA);
        const F3 c2x = 0.5f * (-(r2 + 0.5f * up) * pn + armB);
        frameUpdate(pn, pc1, n, g.w1, g.w2, dtf, renormStep(step, sp.trsfRenorm), f, m);
        const F3 relVel = (g.dv + fcross(g.w2, c2x)) - fcross(g.w1, c1x);
        lvel = F3{fdot(m.c0, relVel), fdot(m.c1, relVel), fdot(m.c2, relVel)};
        ph0 = st[CF_P0];
        ph1 = st[CF_P1];
        ph2 = st[CF_P2];
        ph3 = st[CF_P3];
    }
    float fn, ft1 = 0.f, ft2 = 0.f;
    bool keep = true;
    EnergyTerms en;
    if (sp.law == 0) {
        // Law2_L6Geom_FrictPhys_IdealElPl (IdealElPl.cpp:18-81), shear force accumulated in FP64
        if (uN > 0 && !sp.noBreak) {
            keep = false;
            if constexpr (ENERGY)
                if (sp.noSlip) en.brokenElPl(ph0, ph1, uN, ft1o + (double)(dtf * ph1 * lvel.y), ft2o + (double)(dtf * ph1 * lvel.z));
        } else {
            fn = ph0 * uN;
            if (sp.noFrict || ph2 == 0.f) {
                K.ft[0][j] = 0.;
                K.ft[1][j] = 0.;
            } else {
                double t1 = ft1o, t2 = ft2o;
                t1 += (double)(dtf * ph1 * lvel.y);
                t2 += (double)(dtf * ph1 * lvel.z);
                const double maxFt = (double)(fabsf(fn) * ph2);
                const double q = t1 * t1 + t2 * t2;
                if (q > maxFt * maxFt && !sp.noSlip) {
                    if constexpr (ENERGY) en.plastElPl(ph1, maxFt, q);
                    const double ratio = (q > 0) ? maxFt * rsqrt(q) : 0.;
                    t1 *= ratio;
                    t2 *= ratio;
                }
                K.ft[0][j] = t1;
                K.ft[1][j] = t2;
                ft1 = (float)t1;
                ft2 = (float)t2;
                if (isnan(fn) || isnan(t1) || isnan(t2)) atomicCAS(dErr, 0, 101);
            }
            if constexpr (ENERGY) en.elastElPl(ph0, ph1, fn, ft1, ft2);
        }
    } else {
        // Law2_L6Geom_HertzPhys_DMT, DMT branch (Hertz.cpp:58-87,143-172)
        if (uN > 0) keep = false;
        else {
            const float su = sqrtf(-uN);
            const float Fne = -ph0 * (su * su * su);
            const float eta = (ph3 > 0.f) ? ph3 * sqrtf(su) : 0.f;
            float Fnv = eta * lvel.x;
            if (sp.noAttraction && Fne + Fnv > 0.f) Fnv = -Fne;
            fn = Fne + Fnv;  // the adhesion term 4 pi R gamma is zero (gamma = 0 is required in this mode)
            if constexpr (ENERGY) en.viscN = ((double)Fnv * (double)lvel.x) * (double)dtf;
            const float kt = ph1 * su;
            ft1 = dtf * kt * lvel.y;
            ft2 = dtf * kt * lvel.z;
            const float maxFt = fmaxf(0.f, fn) * ph2;
            const float q = ft1 * ft1 + ft2 * ft2;
            if (q > maxFt * maxFt) {
                if constexpr (ENERGY) en.plastHertz(q, maxFt, kt);
                const float ratio = maxFt * rsqrtf(q);
                ft1 *= ratio;
                ft2 *= ratio;
            } else {
                ft1 += eta * lvel.y;
                ft2 += eta * lvel.z;
                if constexpr (ENERGY) en.viscT = ((double)eta * ((double)lvel.y * lvel.y + (double)lvel.z * lvel.z)) * (double)dtf;
            }
            if constexpr (ENERGY)
                if (uN < 0.f) en.elastHertz(ph0, su, ft1, ft2, kt);
        }
    }
    if constexpr (ENERGY) en.store(E, nm + j);
    if (!keep) {
        K.flags[j] = ((fl & ~C_REAL) | C_PENDING) | hiBits;
        if (real) {
            I.endAf[it.z] = make_float4(0.f, 0.f, 0.f, 0.f);
            I.endBf[it.z] = make_float2(0.f, 0.f);
            I.endAf[it.w] = make_float4(0.f, 0.f, 0.f, 0.f);
            I.endBf[it.w] = make_float2(0.f, 0.f);
        }
        return;
    }
    // force on pA in global coordinates: trsf * (Fn, Ft1, Ft2); torques about the nodes
    const F3 F = fn * f.c0 + ft1 * f.c1 + ft2 * f.c2;
    const F3 TA = fcross(armA, F), TB = fcross(armB, -F);
    I.endAf[it.z] = make_float4(F.x, F.y, F.z, TA.x);
    I.endBf[it.z] = make_float2(TA.y, TA.z);
    I.endAf[it.w] = make_float4(-F.x, -F.y, -F.z, TB.x);
    I.endBf[it.w] = make_float2(TB.y, TB.z);
    K.col[CF_T0X][j] = f.c0.x;
    K.col[CF_T0Y][j] = f.c0.y;
    K.col[CF_T0Z][j] = f.c0.z;
    K.col[CF_T1X][j] = f.c1.x;
    K.col[CF_T1Y][j] = f.c1.y;
    K.col[CF_T1Z][j] = f.c1.z;
    K.col[CF_UN][j] = uN;
    if ((fl | C_REAL) != fl0) K.flags[j] = (fl | C_REAL) | hiBits;
}

// Sphere-sphere contacts of aperiodic scenes (work items [nMixed, nAct)), one per thread: item,
// flags and state are read at the contact's position in the work list (coalesced), the two
// particles' mirror records are gathered; every load is issued before the step guard and the
// branches, so a contact waits for two memory round trips.
template <int MINB, bool ENERGY>
__global__ void __launch_bounds__(256, MINB) k_contact_ss32(DevNodes N, DevParticles P, DevContacts C, DevIncidence I, DevPackedSS K,
                                                            const double4_32a* __restrict__ mats, const ScenePar* __restrict__ spp,
                                                            const long long* __restrict__ dStep, int* __restrict__ dFlags, int64_t nm,
                                                            int haltBlock, int loadFt, EnergyCols E) {
    const int64_t j0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = j0 < K.n;
    const int64_t j = in ? j0 : 0;
    SSIn x;
    x.it = K.item[j];
    x.pf = K.flags[j];
#pragma unroll
    for (int q = 0; q < CF_NCOL; q++) x.st[q] = K.col[q][j];
    x.ft1o = 0.;
    x.ft2o = 0.;
    if (loadFt) {  // some scene uses IdealElPl
        x.ft1o = K.ft[0][j];
        x.ft2o = K.ft[1][j];
    }
    x.ma = N.mir[x.it.x];
    x.mb = N.mir[x.it.y];
    x.wza = N.wz[x.it.x];
    x.wzb = N.wz[x.it.y];
    const long long stepAbs = *dStep;
    if (dFlags[FL_FULL] || halted(dFlags)) {
        if (haltBlock && blockIdx.x == 0 && threadIdx.x == 0) dFlags[FL_HALT] = 1;
        return;
    }
    if (!in) return;
    ssContact<ENERGY>(x, j, N, P, C, I, K, mats, spp, stepAbs, dFlags, nm, E);
}

// The same contacts through a resident grid, each thread walking the range with the grid's
// stride: the next contact's packed item is loaded while the current contact's state and mirror
// records are in flight, so each contact waits for one memory round trip instead of two.
template <int MINB, bool ENERGY>
__global__ void __launch_bounds__(256, MINB) k_contact_ss32p(DevNodes N, DevParticles P, DevContacts C, DevIncidence I, DevPackedSS K,
                                                             const double4_32a* __restrict__ mats, const ScenePar* __restrict__ spp,
                                                             long long* __restrict__ dStep, int* __restrict__ dFlags, int64_t nm,
                                                             int haltBlock, int loadFt, int ticketTotal, EnergyCols E) {
    const long long stepAbs = *dStep;
    if (dFlags[FL_FULL] || halted(dFlags)) {  // the same for every thread of the grid
        if (haltBlock && blockIdx.x == 0 && threadIdx.x == 0) dFlags[FL_HALT] = 1;
        return;
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int4 next = j < K.n ? K.item[j] : make_int4(0, 0, 0, 0);
    for (; j < K.n; j += stride) {
        SSIn x;
        x.it = next;
        if (j + stride < K.n) next = K.item[j + stride];
        x.pf = K.flags[j];
#pragma unroll
        for (int q = 0; q < CF_NCOL; q++) x.st[q] = K.col[q][j];
        x.ft1o = 0.;
        x.ft2o = 0.;
        if (loadFt) {
            x.ft1o = K.ft[0][j];
            x.ft2o = K.ft[1][j];
        }
        x.ma = N.mir[x.it.x];
        x.mb = N.mir[x.it.y];
        x.wza = N.wz[x.it.x];
        x.wzb = N.wz[x.it.y];
        ssContact<ENERGY>(x, j, N, P, C, I, K, mats, spp, stepAbs, dFlags, nm, E);
    }
    stepTicket(dFlags, dStep, ticketTotal);
}

__global__ void k_pack_ss(DevContacts C, DevIncidence I, DevParticles P, DevPackedSS K, int64_t nm, int copyFt) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= K.n) return;
    const int4 wk = I.work[nm + j];
    const int64_t c = wk.x;
    const uint32_t fl = C.flags[c];
    const int32_t sl = I.slotLo[c], sh = I.slotHi[c];
    const bool swap = fl & C_SWAP;
    K.item[j] = make_int4(wk.y, wk.z, swap ? sh : sl, swap ? sl : sh);
    K.flags[j] = fl | ((uint32_t)sceneOfP(P, wk.z) << 8);
#pragma unroll
    for (int q = 0; q < CF_NCOL; q++) K.col[q][j] = C.fcol[q][c];
    if (copyFt) {
        K.ft[0][j] = C.col[CC_FT1][c];
        K.ft[1][j] = C.col[CC_FT2][c];
    }
}

__global__ void k_unpack_ss(DevContacts C, DevIncidence I, DevPackedSS K, int64_t nm, int copyFt) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= K.n) return;
    const int64_t c = I.work[nm + j].x;
    C.flags[c] = K.flags[j] & 0xffu;
#pragma unroll
    for (int q = 0; q < CF_NCOL; q++) C.fcol[q][c] = K.col[q][j];
    if (copyFt) {
        C.col[CC_FT1][c] = K.ft[0][j];
        C.col[CC_FT2][c] = K.ft[1][j];
    }
}

void launch_pack_ss(cudaStream_t st, const DevContacts& C, const DevIncidence& I, const DevParticles& P, const DevPackedSS& K,
                    int64_t nMixed) {
    if (K.n > 0) k_pack_ss<<<(unsigned)((K.n + 255) / 256), 256, 0, st>>>(C, I, P, K, nMixed, K.ftLive ? 1 : 0);
}
void launch_unpack_ss(cudaStream_t st, const DevContacts& C, const DevIncidence& I, const DevPackedSS& K, int64_t nMixed) {
    if (K.n > 0) k_unpack_ss<<<(unsigned)((K.n + 255) / 256), 256, 0, st>>>(C, I, K, nMixed, K.ftLive ? 1 : 0);
}

// FacetPrep of every facet (Facet.cpp:240-246: normal; CompUtils.cpp:92-110: the barycentric
// matrix), from the vertex positions of this step; a facet whose vertices are where they were
// when its record was made keeps it (the record starts as NaN, which equals nothing).
__global__ void k_facet_prep(DevNodes N, DevParticles P, const int* __restrict__ dFlags) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= P.nFacets || (dFlags && halted(dFlags))) return;
    const int4 fn = P.aux[P.facetIds[f]];
    const D3 p0 = ld3(N.posr[fn.x]), p1 = ld3(N.posr[fn.y]), p2 = ld3(N.posr[fn.z]);
    {
        const FacetPrep& F = P.prep[f];
        const double4_32a o0 = F.p0, o1 = F.p1, o2 = F.p2;
        if (o0.x == p0.x && o0.y == p0.y && o0.z == p0.z && o1.x == p1.x && o1.y == p1.y && o1.z == p1.z && o2.x == p2.x &&
            o2.y == p2.y && o2.z == p2.z)
            return;
    }
    const D3 nn = cross(p1 - p0, p2 - p0);
    const D3 fNormal = normalized(nn);
    const D3 e0 = cross(p1 - p0, nn), e1 = cross(p2 - p1, nn), e2 = cross(p0 - p2, nn);
    const D3 vB = p1 - p0, vC = p2 - p0;
    const double m00 = dot(vB, vB), m01 = dot(vC, vB), m10 = dot(vB, vC), m11 = dot(vC, vC);
    const double det = m00 * m11 - m10 * m01;
    const double invdet = 1. / det;
    FacetPrep& F = P.prep[f];
    F.p0 = make_double4_32a(p0.x, p0.y, p0.z, m11 * invdet);
    F.p1 = make_double4_32a(p1.x, p1.y, p1.z, -m01 * invdet);
    F.p2 = make_double4_32a(p2.x, p2.y, p2.z, -m10 * invdet);
    F.n = make_double4_32a(fNormal.x, fNormal.y, fNormal.z, m00 * invdet);
    F.e0 = make_double4_32a(e0.x, e0.y, e0.z, 0.);
    F.e1 = make_double4_32a(e1.x, e1.y, e1.z, 0.);
    F.e2 = make_double4_32a(e2.x, e2.y, e2.z, 0.);
}
void launch_facet_prep(cudaStream_t st, const DevNodes& N, const DevParticles& P, const int* dFlags) {
    if (P.nFacets > 0 && P.prep) k_facet_prep<<<(P.nFacets + 63) / 64, 64, 0, st>>>(N, P, dFlags);
}

// rare paths of the facet geometry, out of line (see physCreateFP64)
__device__ __noinline__ D3 closestSegmentPtOut(D3 P, D3 A, D3 B) { return closestSegmentPt(P, A, B); }
__device__ __noinline__ D3 normalPartOut(D3 v, D3 n) { return dot(v, n) * n; }
// Facet::interpolatePtLinAngVel (Facet.cpp:158-174): the barycentric interpolation of the vertex
// velocities at contPt and the angular velocity they imply, for facets whose vertices move (a
// drum's facets are static and move the spheres by fakeVel only: there both are zero)
__device__ __noinline__ void facetVelOut(D3 contPt, D3 p0, D3 p1, D3 p2, double4_32a q0, double4_32a q1, double4_32a q2,
                                         double4_32a qn, D3 v0, D3 v1, D3 v2, D3& linVel, D3& angVel) {
    const D3 vX = contPt - p0;
    const double b0 = dot(vX, p1 - p0), b1 = dot(vX, p2 - p0);
    const double u = q0.w * b0 + q1.w * b1, v = q2.w * b0 + qn.w * b1;
    const double a0 = (1 - u) - v;
    linVel = (a0 * v0 + u * v1) + v * v2;
    angVel = (cross(p0 - contPt, v0) + cross(p1 - contPt, v1)) + cross(p2 - contPt, v2);
}

// Cg2_Facet_Sphere_L6Geom::go (Facet.cpp:235-288, Facet::interpolatePtLinAngVel :158-174) in FP64
// from the facet's FacetPrep of this step: the per-contact part of the functor (plane distance,
// region tests, closest point, barycentric velocity).
template <bool PERI>
__device__ __forceinline__ bool geomFS32(const DevNodes& N, const DevParticles& P, int A, int B, D3 shift2, bool real, Geo& g, int* dErr) {
    const int4 fn = P.aux[A];
    const FacetPrep& F = P.prep[fn.w];
    const double4_32a fd = P.facet[A];
    const double halfThick = fd.w;
    const D3 fakeVel{fd.x, fd.y, fd.z};
    const double4_32a ps = N.posr[B];
    const double4_32a q0 = F.p0, q1 = F.p1, q2 = F.p2, qn = F.n;
    const double radius = ps.w;
    const D3 sC = PERI ? ld3(ps) + shift2 : ld3(ps);
    const D3 p0 = ld3(q0), p1 = ld3(q1), p2 = ld3(q2);
    const D3 fNormal = ld3(qn);
    const double planeDist = dot(sC - p0, fNormal);
    if (fabs(planeDist) > (radius + halfThick) && !real) return false;
    const D3 fC = sC - planeDist * fNormal;
    const double l0 = dot(ld3(F.e0), fC - p0);
    const double l1 = dot(ld3(F.e1), fC - p1);
    const double l2 = dot(ld3(F.e2), fC - p2);
    const int w = (l0 > 0 ? 1 : 0) + (l1 > 0 ? 2 : 0) + (l2 > 0 ? 4 : 0);
    D3 contPt;
    switch (w) {
        case 0: contPt = fC; break;
        case 1: contPt = closestSegmentPtOut(fC, p0, p1); break;
        case 2: contPt = closestSegmentPtOut(fC, p1, p2); break;
        case 4: contPt = closestSegmentPtOut(fC, p2, p0); break;
        case 3: contPt = p1; break;
        case 5: contPt = p0; break;
        case 6: contPt = p2; break;
        default: atomicCAS(dErr, 0, 100); return false;  // "Impossible sphere-facet intersection"
    }
    D3 normal = sC - contPt;
    const double rh = radius + halfThick;
    const double d2 = sqn(normal);
    if (d2 > rh * rh && !real) return false;
    const double dist = sqrt(d2);
    normal = normal * (1. / dist);
    if (halfThick > 0) contPt = contPt + normal * halfThick;
    g.uN = (dist - radius) - halfThick;
    // the facet node velocities interpolated at contPt (zero for static vertices)
    const D3 v0 = ld3(N.vel[fn.x]), v1 = ld3(N.vel[fn.y]), v2 = ld3(N.vel[fn.z]);
    D3 linVel{0, 0, 0}, angVel{0, 0, 0};
    if (!isZero(v0) || !isZero(v1) || !isZero(v2)) facetVelOut(contPt, p0, p1, p2, q0, q1, q2, qn, v0, v1, v2, linVel, angVel);
    if (!isZero(fakeVel)) {
        if (!isnan(fakeVel.x)) linVel = linVel + fakeVel;
        else linVel = normalPartOut(linVel, fNormal);
    }
    g.normal = normal;
    g.contPt = contPt;
    g.pos1 = contPt;
    g.vel1 = linVel;
    g.angVel1 = angVel;
    g.pos2 = sC;
    g.vel2 = ld3(N.vel[B]);
    g.angVel2 = ld3(N.angv[B]);
    g.r1 = smax(halfThick, radius);
    g.r2 = radius;
    return true;
}

// Work items [c0, c1): facet and wall contacts, and every contact of a periodic scene (cell shifts,
// FP64 geometry of the shifted pairs); the state is read and written in the contact arrays.
template <bool PERI, bool ENERGY>
__device__ __forceinline__ void mixedContact(int64_t rk, const DevNodes& N, const DevParticles& P, const DevContacts& C,
                                             const DevIncidence& I, const double4_32a* __restrict__ mats,
                                             const ScenePar* __restrict__ spp, const long long* __restrict__ dStep, int* dFlags,
                                             const EnergyCols& E) {
    int* dErr = dFlags + FL_ERR;
    // work item: contact index, pA, pB and the static flag bits (type, swap) fixed at the full run
    const int4 wk = I.work[rk];
    const int64_t c = wk.x;
    const int A = wk.y, B = wk.z;
    const ScenePar& sp = spp[sceneOfP(P, B)];
    if (*dStep - sp.stepBase >= sp.stepEnd) return;  // frozen scene (serving slot past its last step)
    uint32_t fl = C.flags[c];
    if (fl & C_REMOVED) return;
    if ((fl & C_PENDING) && !pendingStays(P, A, B, PERI && sp.periodic, sp.cellSize, dErr)) {
        C.flags[c] = (fl & ~C_PENDING) | C_REMOVED;
        return;
    }
    fl &= ~C_PENDING;
    const uint32_t ty = ctype((uint32_t)wk.w);
    const bool real = fl & C_REAL;
    const long long step = *dStep - sp.stepBase;
    const float dtf = sp.dtF;
    bool shifted = false;
    D3 shift2{0, 0, 0}, shiftVel2{0, 0, 0};
    if (PERI && sp.periodic) {
        int a, b, cc;
        unpackCellDist(C.cdist[c], a, b, cc);
        if (fl & C_SWAP) { a = -a; b = -b; cc = -cc; }
        shifted = (a | b | cc) != 0;
        if (shifted) {
            const D3 cd{(double)a, (double)b, (double)cc};
            shift2 = mul(*(const DM3*)sp.hSize, cd);
            shiftVel2 = mul(*(const DM3*)sp.shiftVelMat, cd);
        }
    }
    // n: normal; armA/armB: contact point minus the nodes of pA/pB (torque arms, Contact.cpp:32);
    // c1x/c2x: mid-step branch vectors of L6Geom.cpp:156-160; dv: relative velocity of the centres
    F3 n, armA, armB, c1x, c2x, dv, w1, w2;
    float uN, r1, r2;
    if (PERI && ty == CT_SS && !shifted) {
        SSGeo g;
        if (!geomSS32(N.mir[A], N.mir[B], N.wz[A], N.wz[B], sp.ssDfAbsF, real, g)) {
            C.flags[c] = fl;
            return;
        }
        n = g.n;
        uN = g.uN;
        r1 = g.r1;
        r2 = g.r2;
        dv = g.dv;
        w1 = g.w1;
        w2 = g.w2;
    } else if (PERI && ty == CT_SS) {
        // a pair across the periodic boundary: FP64 relative position with the cell shift
        const double4_32a pa = N.posr[A], pb = N.posr[B];
        const D3 dx = (ld3(pb) + shift2) - ld3(pa);
        const double d2 = sqn(dx);
        const double R = pa.w + pb.w;
        const double dfr = fabs(sp.ssDistFactor) * R;
        if (d2 - dfr * dfr > 0 && !real) {
            C.flags[c] = fl;
            return;
        }
        const float distf = sqrtf((float)d2);
        uN = (float)(d2 - R * R) / (distf + (float)R);
        n = toF(dx) * (1.f / distf);
        r1 = (float)pa.w;
        r2 = (float)pb.w;
        dv = toF((ld3(N.vel[B]) + shiftVel2) - ld3(N.vel[A]));
        w1 = toF(ld3(N.angv[A]));
        w2 = toF(ld3(N.angv[B]));
    }
    if (PERI && ty == CT_SS) {
        // contPt = x1 + (r1 + uN/2) n (Sphere.cpp:103), written relative to both centres
        armA = (r1 + 0.5f * uN) * n;
        armB = -(r2 + 0.5f * uN) * n;
        if (real) {
            const F3 pn{C.fcol[CF_T0X][c], C.fcol[CF_T0Y][c], C.fcol[CF_T0Z][c]};
            const float up = C.fcol[CF_UN][c];
            c1x = 0.5f * ((r1 + 0.5f * up) * pn + armA);
            c2x = 0.5f * (-(r2 + 0.5f * up) * pn + armB);
        }
    } else {
        Geo g;
        bool touch;
        if (ty == CT_WS) touch = geomWS(N, P, real ? (double)C.fcol[CF_T0X + P.aux[A].x][c] : 0., A, B, shift2, real, g);
        else touch = geomFS32<PERI>(N, P, A, B, shift2, real, g, dErr);
        if (!touch) {
            C.flags[c] = fl;
            return;
        }
        n = toFt(g.normal);
        uN = d2fT(g.uN);
        r1 = d2fT(g.r1);
        r2 = d2fT(g.r2);
        // walls are uninodal (their node is pos1); facets take no force here
        armA = (ty == CT_WS) ? toFt(g.contPt - g.pos1) : F3{0.f, 0.f, 0.f};
        armB = toFt(g.contPt - g.pos2);
        const D3 vel2 = PERI ? g.vel2 + shiftVel2 : g.vel2;
        if (real) {
            // mid-step branch vectors (L6Geom.cpp:156-160): (prevCp + contPt)/2 - (pos - dt/2 vel),
            // from the FP64 differences of nearby points (a few mm) rounded to FP32
            const D3 prevCp{C.col[CC_CPX][c], C.col[CC_CPY][c], C.col[CC_CPZ][c]};
            const float hdt = 0.5f * dtf;
            c1x = 0.5f * (toFt(prevCp - g.pos1) + toFt(g.contPt - g.pos1)) + hdt * toFt(g.vel1);
            c2x = 0.5f * (toFt(prevCp - g.pos2) + armB) + hdt * toFt(vel2);
        }
        dv = toFt(vel2 - g.vel1);
        w1 = toFt(g.angVel1);
        w2 = toFt(g.angVel2);
        C.col[CC_CPX][c] = g.contPt.x;
        C.col[CC_CPY][c] = g.contPt.y;
        C.col[CC_CPZ][c] = g.contPt.z;
    }
    Frame f, m;
    F3 lvel{0, 0, 0};
    float ph0, ph1, ph2, ph3 = 0.f;
    if (!real) {
        frameInit(n, f);
        const double ma = N.minert[P.shape[A] == WG_SHAPE_FACET ? P.aux[A].x : A].w, mb = N.minert[B].w;
        physCreate(spp, sceneOfP(P, B), r1, r2, uN, mats[P.mat[A]], mats[P.mat[B]], ma, mb, ph0, ph1, ph2, ph3);
        C.fcol[CF_P0][c] = ph0;
        C.fcol[CF_P1][c] = ph1;
        C.fcol[CF_P2][c] = ph2;
        C.fcol[CF_P3][c] = ph3;
        C.step0[c] = (int32_t)step;
        if (sp.law == 0) {
            C.col[CC_FT1][c] = 0.;
            C.col[CC_FT2][c] = 0.;
        }
    } else {
        const F3 pn{C.fcol[CF_T0X][c], C.fcol[CF_T0Y][c], C.fcol[CF_T0Z][c]};
        const F3 pc1{C.fcol[CF_T1X][c], C.fcol[CF_T1Y][c], C.fcol[CF_T1Z][c]};
        frameUpdate(pn, pc1, n, w1, w2, dtf, renormStep(step, sp.trsfRenorm), f, m);
        const F3 relVel = (dv + fcross(w2, c2x)) - fcross(w1, c1x);
        lvel = F3{fdot(m.c0, relVel), fdot(m.c1, relVel), fdot(m.c2, relVel)};
        ph0 = C.fcol[CF_P0][c];
        ph1 = C.fcol[CF_P1][c];
        ph2 = C.fcol[CF_P2][c];
        ph3 = C.fcol[CF_P3][c];
    }
    float fn, ft1 = 0.f, ft2 = 0.f;
    bool keep = true;
    EnergyTerms en;
    if (sp.law == 0) {
        // Law2_L6Geom_FrictPhys_IdealElPl (IdealElPl.cpp:18-81), shear force accumulated in FP64
        if (uN > 0 && !sp.noBreak) {
            keep = false;
            if constexpr (ENERGY)
                if (sp.noSlip)
                    en.brokenElPl(ph0, ph1, uN, (real ? C.col[CC_FT1][c] : 0.) + (double)(dtf * ph1 * lvel.y),
                                  (real ? C.col[CC_FT2][c] : 0.) + (double)(dtf * ph1 * lvel.z));
        } else {
            fn = ph0 * uN;
            if (sp.noFrict || ph2 == 0.f) {
                if (real) { C.col[CC_FT1][c] = 0.; C.col[CC_FT2][c] = 0.; }
            } else {
                double t1 = real ? C.col[CC_FT1][c] : 0., t2 = real ? C.col[CC_FT2][c] : 0.;
                t1 += (double)(dtf * ph1 * lvel.y);
                t2 += (double)(dtf * ph1 * lvel.z);
                const double maxFt = (double)(fabsf(fn) * ph2);
                const double q = t1 * t1 + t2 * t2;
                if (q > maxFt * maxFt && !sp.noSlip) {
                    if constexpr (ENERGY) en.plastElPl(ph1, maxFt, q);
                    const double ratio = (q > 0) ? maxFt * rsqrt(q) : 0.;
                    t1 *= ratio;
                    t2 *= ratio;
                }
                C.col[CC_FT1][c] = t1;
                C.col[CC_FT2][c] = t2;
                ft1 = (float)t1;
                ft2 = (float)t2;
                if (isnan(fn) || isnan(t1) || isnan(t2)) atomicCAS(dErr, 0, 101);
            }
            if constexpr (ENERGY) en.elastElPl(ph0, ph1, fn, ft1, ft2);
        }
    } else {
        // Law2_L6Geom_HertzPhys_DMT, DMT branch (Hertz.cpp:58-87,143-172)
        if (uN > 0) keep = false;
        else {
            const float su = sqrtf(-uN);
            const float Fne = -ph0 * (su * su * su);
            const float eta = (ph3 > 0.f) ? ph3 * sqrtf(su) : 0.f;
            float Fnv = eta * lvel.x;
            if (sp.noAttraction && Fne + Fnv > 0.f) Fnv = -Fne;
            fn = Fne + Fnv;  // the adhesion term 4 pi R gamma is zero (gamma = 0 is required in this mode)
            if constexpr (ENERGY) en.viscN = ((double)Fnv * (double)lvel.x) * (double)dtf;
            const float kt = ph1 * su;
            ft1 = dtf * kt * lvel.y;
            ft2 = dtf * kt * lvel.z;
            const float maxFt = fmaxf(0.f, fn) * ph2;
            const float q = ft1 * ft1 + ft2 * ft2;
            if (q > maxFt * maxFt) {
                if constexpr (ENERGY) en.plastHertz(q, maxFt, kt);
                const float ratio = maxFt * rsqrtf(q);
                ft1 *= ratio;
                ft2 *= ratio;
            } else {
                ft1 += eta * lvel.y;
                ft2 += eta * lvel.z;
                if constexpr (ENERGY) en.viscT = ((double)eta * ((double)lvel.y * lvel.y + (double)lvel.z * lvel.z)) * (double)dtf;
            }
            if constexpr (ENERGY)
                if (uN < 0.f) en.elastHertz(ph0, su, ft1, ft2, kt);
        }
    }
    if constexpr (ENERGY) en.store(E, rk);
    const bool aIsLo = !(fl & C_SWAP);
    if (!keep) {
        C.flags[c] = (fl & ~C_REAL) | C_PENDING;
        if (real) {
            const int32_t sl = I.slotLo[c], sh = I.slotHi[c];
            I.endAf[sl] = make_float4(0.f, 0.f, 0.f, 0.f);
            I.endBf[sl] = make_float2(0.f, 0.f);
            I.endAf[sh] = make_float4(0.f, 0.f, 0.f, 0.f);
            I.endBf[sh] = make_float2(0.f, 0.f);
        }
        return;
    }
    // force on pA in global coordinates: trsf * (Fn, Ft1, Ft2); torques about the nodes
    const F3 F = fn * f.c0 + ft1 * f.c1 + ft2 * f.c2;
    const F3 TA = fcross(armA, F), TB = fcross(armB, -F);
    {
        const int sA = aIsLo ? I.slotLo[c] : I.slotHi[c], sB = aIsLo ? I.slotHi[c] : I.slotLo[c];
        if (ty != CT_FS) {
            I.endAf[sA] = make_float4(F.x, F.y, F.z, TA.x);
            I.endBf[sA] = make_float2(TA.y, TA.z);
        }
        I.endAf[sB] = make_float4(-F.x, -F.y, -F.z, TB.x);
        I.endBf[sB] = make_float2(TB.y, TB.z);
    }
    C.fcol[CF_T0X][c] = f.c0.x;
    C.fcol[CF_T0Y][c] = f.c0.y;
    C.fcol[CF_T0Z][c] = f.c0.z;
    C.fcol[CF_T1X][c] = f.c1.x;
    C.fcol[CF_T1Y][c] = f.c1.y;
    C.fcol[CF_T1Z][c] = f.c1.z;
    C.fcol[CF_UN][c] = uN;
    C.flags[c] = fl | C_REAL;
}

// One thread per work item of [c0, c1), looping over the range with the grid's stride (the
// launch sizes the grid so that its blocks leave room for the sphere-sphere kernel beside it).
template <bool PERI, bool ENERGY>
__global__ void __launch_bounds__(128, 4) k_contact_fp32(DevNodes N, DevParticles P, DevContacts C, DevIncidence I,
                                                       const double4_32a* __restrict__ mats, const ScenePar* __restrict__ spp,
                                                       long long* __restrict__ dStep, int* __restrict__ dFlags, int64_t c0,
                                                       int64_t c1, int haltBlock, int ticketTotal, EnergyCols E) {
    if (dFlags[FL_FULL] || halted(dFlags)) {  // the same for every thread of the grid
        if (haltBlock && blockIdx.x == 0 && threadIdx.x == 0) dFlags[FL_HALT] = 1;
        return;
    }
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t rk = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; rk < c1; rk += stride)
        mixedContact<PERI, ENERGY>(rk, N, P, C, I, mats, spp, dStep, dFlags, E);
    stepTicket(dFlags, dStep, ticketTotal);
}

// minimum resident blocks per SM the one-contact-per-thread kernel is compiled for (register budget)
constexpr int kSSMinBlocks = 3;

// streaming multiprocessors of the current device
static int smCount() {
    static std::mutex mu;
    static int n[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    std::lock_guard<std::mutex> lk(mu);
    if (!n[dev] && (cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n[dev] < 1)) n[dev] = 1;
    return n[dev];
}

// sphere-sphere range: block > 0 one contact per thread with that many threads per block;
// block < 0 the resident-grid kernel with prefetch (256 threads per block)
// Returns true when the launch also advances the step counter (advance requested and possible).
// grid of the resident sphere-sphere kernel (block < 0), or 0 for the one-contact-per-thread kernel
static int ssGrid(const DevPackedSS& K, int block, int blocksPerSM) {
    return block < 0 ? (int)std::min<int64_t>((K.n + 255) / 256, (int64_t)blocksPerSM * smCount()) : 0;
}
template <bool ENERGY>
static void launchSS(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C, const DevIncidence& I,
                     const DevPackedSS& K, const double4_32a* mats, const ScenePar* sp, long long* dStep, int* dFlags, int64_t nm,
                     int halt, int loadFt, int block, int grid, int ticketTotal, const EnergyCols& E) {
    if (block < 0) {
        k_contact_ss32p<kSSMinBlocks, ENERGY><<<(unsigned)grid, 256, 0, st>>>(N, P, C, I, K, mats, sp, dStep, dFlags, nm, halt, loadFt,
                                                                              ticketTotal, E);
        return;
    }
    k_contact_ss32<kSSMinBlocks, ENERGY><<<(unsigned)((K.n + block - 1) / block), (unsigned)block, 0, st>>>(
        N, P, C, I, K, mats, sp, dStep, dFlags, nm, halt, loadFt, E);
}

template <bool ENERGY>
static bool contactsFP32(cudaStream_t st, const SideStream& side, const DevNodes& N, const DevParticles& P, const DevContacts& C,
                         const DevIncidence& I, const DevPackedSS& K, const double4_32a* mats, const ScenePar* sp,
                         long long* dStep, int* dFlags, int64_t nMixed, bool periodic, bool anyLaw0, bool prepFacets,
                         int block, const EnergyCols& E) {
    const int64_t nm = periodic ? I.nAct : std::min<int64_t>(nMixed, I.nAct);
    const int64_t ns = periodic ? 0 : K.n;
    if (ns > 0 && nm > 0 && side.st) {
        // the mixed range (facets and walls, FP64 geometry) beside the sphere-sphere range: one block
        // of 128 threads per SM, and two resident sphere-sphere blocks per SM beside it; the
        // sphere-sphere launch raises FL_HALT when a full run is due; the last block of either
        // advances the step counter
        const int gM = (int)std::min<int64_t>((nm + 127) / 128, smCount());
        const int gS = ssGrid(K, block, kSSMinBlocks - 1);
        const int total = gS > 0 ? gM + gS : 0;
        cudaEventRecord(side.fork, st);
        cudaStreamWaitEvent(side.st, side.fork, 0);
        if (prepFacets) launch_facet_prep(side.st, N, P, dFlags);
        k_contact_fp32<false, ENERGY><<<(unsigned)gM, 128, 0, side.st>>>(N, P, C, I, mats, sp, dStep, dFlags, 0, nm, 0, total, E);
        launchSS<ENERGY>(st, N, P, C, I, K, mats, sp, dStep, dFlags, nm, 1, anyLaw0, block, gS, total, E);
        cudaEventRecord(side.join, side.st);
        cudaStreamWaitEvent(st, side.join, 0);
        return total > 0;
    }
    // the first launch also raises FL_HALT when a full run is due (it always runs); the last
    // kernel of the step advances the step counter
    if (nm > 0 && prepFacets) launch_facet_prep(st, N, P, dFlags);
    const int gS = ns > 0 ? ssGrid(K, block, kSSMinBlocks) : 0;
    const int gM = (int)std::max<int64_t>(1, std::min<int64_t>((nm + 127) / 128, 4 * smCount()));
    const int totalM = ns > 0 ? 0 : gM;
    if (periodic) k_contact_fp32<true, ENERGY><<<(unsigned)gM, 128, 0, st>>>(N, P, C, I, mats, sp, dStep, dFlags, 0, nm, 1, totalM, E);
    else k_contact_fp32<false, ENERGY><<<(unsigned)gM, 128, 0, st>>>(N, P, C, I, mats, sp, dStep, dFlags, 0, nm, 1, totalM, E);
    if (ns > 0) launchSS<ENERGY>(st, N, P, C, I, K, mats, sp, dStep, dFlags, nm, 0, anyLaw0, block, gS, gS, E);
    return totalM > 0 || gS > 0;
}

bool launch_contact_fp32(cudaStream_t st, const SideStream& side, const DevNodes& N, const DevParticles& P, const DevContacts& C,
                         const DevIncidence& I, const DevPackedSS& K, const double4_32a* mats, const ScenePar* sp,
                         long long* dStep, int* dFlags, int64_t nMixed, bool periodic, bool anyLaw0, bool prepFacets,
                         int block, const EnergyCols* energy) {
    if (energy)
        return contactsFP32<true>(st, side, N, P, C, I, K, mats, sp, dStep, dFlags, nMixed, periodic, anyLaw0, prepFacets, block,
                                  *energy);
    return contactsFP32<false>(st, side, N, P, C, I, K, mats, sp, dStep, dFlags, nMixed, periodic, anyLaw0, prepFacets, block,
                               EnergyCols{});
}

// ---------------------------------------------------------------------------------- force sum
// DemData.force/torque for reporting after a run: the sum of k_leapfrog32 (m*g and the
// particle's FP32 end slots, compensated, in slot order) converted to FP64, for every particle
// whose degree is at most kHeavyThreshold. Its FP32 rounding is the force k_leapfrog32 uses.
__global__ void __launch_bounds__(256) k_forces32(DevNodes N, DevParticles P, DevIncidence I, const NodeConst32* __restrict__ ncs,
                                                  const ScenePar* __restrict__ spp) {
    __shared__ EndStage<float4, float2, 128> stage[8];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const ScenePar& sp = spp[p < P.n ? sceneOfP(P, p) : 0];
    const bool uni = p < P.n && P.shape[p] != WG_SHAPE_FACET;
    int e0 = 0, e1 = 0;
    bool take = false;
    DF6 acc;
    if (uni) {
        const NodeConst32 nc = ncs[p];
        if (sp.hasGravity && !(nc.flags & F_GRAVITY_SKIP)) acc.initGravity(nc.mh, nc.ml, sp.gH, sp.gL);
        if (sp.applyForces) {
            endRange(I, p, e0, e1);
            take = (e1 - e0) <= kHeavyThreshold;
        }
    }
    warpSumEnds(I.endAf, I.endBf, take, e0, e1, stage[threadIdx.x >> 5], acc);
    if (uni && (take || !sp.applyForces)) {
        N.force[p] = make_double4_32a(acc.val(0), acc.val(1), acc.val(2), 0.);
        N.torque[p] = make_double4_32a(acc.val(3), acc.val(4), acc.val(5), 0.);
    }
}

__global__ void k_forces32_heavy(DevNodes N, DevIncidence I, const int32_t* __restrict__ list, const ScenePar* __restrict__ spp,
                                 const int* __restrict__ dFlags) {
    if (dFlags && halted(dFlags)) return;
    const int p = list[blockIdx.x];
    const ScenePar& sp = spp[sceneOfN(N, p)];
    int e0, e1;
    endRange(I, p, e0, e1);
    D3 F{0, 0, 0}, T{0, 0, 0};
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const float4 a = I.endAf[e];
        const float2 b = I.endBf[e];
        F = F + D3{(double)a.x, (double)a.y, (double)a.z};
        T = T + D3{(double)a.w, (double)b.x, (double)b.y};
    }
    __shared__ double sh[6][256];
    sh[0][threadIdx.x] = F.x; sh[1][threadIdx.x] = F.y; sh[2][threadIdx.x] = F.z;
    sh[3][threadIdx.x] = T.x; sh[4][threadIdx.x] = T.y; sh[5][threadIdx.x] = T.z;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 6; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const uint32_t flags = N.flags[p];
        const double mass = N.minert[p].w;
        D3 G{0, 0, 0};
        if (sp.hasGravity && !(flags & F_GRAVITY_SKIP)) G = mass * D3{sp.g[0], sp.g[1], sp.g[2]};
        N.force[p] = make_double4_32a(G.x + sh[0][0], G.y + sh[1][0], G.z + sh[2][0], 0.);
        N.torque[p] = make_double4_32a(sh[3][0], sh[4][0], sh[5][0], 0.);
    }
}

void launch_forces32(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const NodeConst32* nc,
                     const ScenePar* sp, const int* dFlags, bool perStep) {
    if (P.n == 0) return;
    if (perStep) {
        if (I.nHeavyFree > 0) k_forces32_heavy<<<I.nHeavyFree, 256, 0, st>>>(N, I, I.heavyFree, sp, dFlags);
        return;
    }
    k_forces32<<<(P.n + 255) / 256, 256, 0, st>>>(N, P, I, nc, sp);
    if (I.nHeavy > 0) k_forces32_heavy<<<I.nHeavy, 256, 0, st>>>(N, I, I.heavy, sp, nullptr);
}

}  // namespace wg
