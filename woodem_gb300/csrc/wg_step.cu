// Per-step kernels of the FP64 path: Leapfrog, the fused ContactLoop functors and the
// deterministic per-particle force/torque sum.
//
// Compiled with --fmad=false: every floating-point result is the correctly rounded
// value of the operation sequence written here, which is the operation sequence of
// the reference expression cited beside it.
#include <algorithm>

#include "wg_ends.cuh"
#include "wg_energy.cuh"
#include "wg_geom.cuh"

namespace wg {
__device__ __forceinline__ double4_32a st4(D3 a, double w) { return make_double4_32a(a.x, a.y, a.z, w); }
__device__ __forceinline__ DM3 ldm(const double* m) {
    DM3 r;
#pragma unroll
    for (int i = 0; i < 9; i++) r.m[i] = m[i];
    return r;
}
__device__ __forceinline__ double sgn(double s) { return s < 0 ? -1 : (s > 0 ? 1 : 0); }

// ---------------------------------------------------------------------------------- Leapfrog
// Leapfrog::run pkg/dem/Leapfrog.cpp:103-255 (spherical integrator; clumps and impose are
// outside the path), nonviscDamp2nd :32-34, computeAccel/AngAccel :36-47,
// applyPeriodicCorrections :258-272, leapfrogTranslate :275-278, leapfrogSphericalRotate :280-288,
// and the verlet-distance test of InsertionSortCollider::updateBboxes_doFullRun
// pkg/dem/InsertionSortCollider.cpp:339-350 on the new positions.
//
// Paths that few nodes take (partly blocked DOFs, damping, the force reset of facet vertices)
// are out-of-line functions: inlined, the compiler turns them into predicated FP64 instructions,
// which occupy the FP64 pipe (1/64 of the FP32 rate on GB300) in every warp. The operations, and
// so the results, are the same either way. PERI: the periodic corrections (Cell velocity gradient).
__device__ __noinline__ D3 linAccelPartial(D3 f, double mass, uint32_t flags) {
    D3 a{0, 0, 0};
    if (!(flags & 1u)) a.x = 0. + f.x / mass;
    if (!(flags & 2u)) a.y = 0. + f.y / mass;
    if (!(flags & 4u)) a.z = 0. + f.z / mass;
    return a;
}
__device__ __noinline__ D3 angAccelPartial(D3 t, D3 inertia, uint32_t flags) {
    D3 a{0, 0, 0};
    if (!(flags & 8u)) a.x = 0. + t.x / inertia.x;
    if (!(flags & 16u)) a.y = 0. + t.y / inertia.y;
    if (!(flags & 32u)) a.z = 0. + t.z / inertia.z;
    return a;
}
// nonviscDamp2nd (Leapfrog.cpp:32-34) of an acceleration a under force (or torque) f, with the
// fluctuation velocity v
__device__ __noinline__ D3 dampAccel(D3 a, D3 f, D3 v, double damping, double dt) {
    a.x = a.x * (1 - damping * sgn(f.x * (v.x + (0.5 * dt) * a.x)));
    a.y = a.y * (1 - damping * sgn(f.y * (v.y + (0.5 * dt) * a.y)));
    a.z = a.z * (1 - damping * sgn(f.z * (v.z + (0.5 * dt) * a.z)));
    return a;
}
// Leapfrog(reset=True) for nodes whose force is not rebuilt by the contact sum (facet vertices):
// force = mass*gravity, torque = 0 (Leapfrog.cpp:240-245)
__device__ __noinline__ void resetForce(DevNodes N, int i, double mass, bool gravity, const ScenePar* __restrict__ spp, int scene) {
    const ScenePar& sp = spp[scene];
    D3 G{0, 0, 0};
    if (gravity) G = mass * D3{sp.g[0], sp.g[1], sp.g[2]};
    N.force[i] = st4(G, 0.);
    N.torque[i] = make_double4_32a(0., 0., 0., 0.);
}
template <bool PERI, bool ENERGY>
__global__ void __launch_bounds__(256) k_leapfrog(DevNodes N, DevParticles P, DevIncidence I, const ScenePar* __restrict__ spp,
                                                  int* __restrict__ dFlags, int fromEnds, const long long* __restrict__ dStepC,
                                                  EnergyCols E) {
    __shared__ EndStage<double4_32a, double2, 32> stage[8];
    if (halted(dFlags)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < N.n;
    const ScenePar& sp = spp[valid ? sceneOfN(N, i) : 0];
    const int nPar = P.n;
    const uint32_t flags = valid ? N.flags[i] : 0u;
    const double4_32a mi = valid ? N.minert[i] : make_double4_32a(0., 0., 0., 0.);
    const double mass = mi.w;
    // DemData.force/torque of this step: m*g plus the end slots written by the last contact
    // loop (the force reset of Leapfrog.cpp:240-245 followed by the deterministic sum of
    // ContactLoop.cpp:250-257), or the stored value
    const bool uni = valid && i < nPar && P.shape[i] != WG_SHAPE_FACET;
    // a scene past its last step (serving slot) is frozen; a node just (re)loaded takes its stored force
    const bool frozen = valid && (*dStepC - sp.stepBase) >= sp.stepEnd;
    const bool fresh = valid && N.fresh && N.fresh[i];
    int e0 = 0, e1 = 0;
    bool take = false;
    D3 f{0, 0, 0}, t{0, 0, 0};
    if (fromEnds && uni && !fresh && !frozen) {
        if (sp.hasGravity && !(flags & F_GRAVITY_SKIP)) f = mass * D3{sp.g[0], sp.g[1], sp.g[2]};
        if (sp.applyForces) {
            endRange(I, i, e0, e1);
            take = (e1 - e0) <= kHeavyThreshold;
            if (!take) {  // summed by the block tree before this kernel
                f = ld3(N.force[i]);
                t = ld3(N.torque[i]);
            }
        }
    } else if (valid) {
        f = ld3(N.force[i]);
        t = ld3(N.torque[i]);
    }
    SumD acc{f, t};
    warpSumEnds(I.endA, I.endB, take, e0, e1, stage[threadIdx.x >> 5], acc);
    f = acc.F;
    t = acc.T;
    if (!valid || (flags & F_CLUMPED) || frozen) return;
    if (fresh) N.fresh[i] = 0;
    const double dt = sp.dt;
    const double damping = sp.damping;
    const bool damp = (damping != 0. && !(flags & F_DAMPING_SKIP));
    const double4_32a pr = N.posr[i];
    D3 pos = ld3(pr);
    D3 vel = ld3(N.vel[i]);
    D3 angVel = ld3(N.angv[i]);
    const D3 inertia{mi.x, mi.y, mi.z};
    const bool blockedAll = (flags & F_DOF_ALL) == F_DOF_ALL;
    const int homoDeform = PERI ? sp.homoDeform : -1;
    D3 linAccel{0, 0, 0};
    D3 angAccelE{0, 0, 0}, pvfE = vel, pvaE = angVel;
    if constexpr (ENERGY) {
        if (sp.trackEnergy) {
            if (damp && !(flags & F_ENERGY_SKIP)) E.col[EN_NODE_DAMP * E.cap + i] = energyDamp(vel, f, angVel, t, damping, dt);
            if (sp.hasGravity && !(flags & F_GRAVITY_SKIP)) {
                E.col[EN_NODE_GRAV * E.cap + i] = energyGrav(D3{sp.g[0], sp.g[1], sp.g[2]}, vel, mass, dt, flags);
                E.col[EN_NODE_NGRAV * E.cap + i] = 1.;
            }
            // fluctuation velocities of the previous half step; a fully blocked node has none in the
            // reference (it reads vectors it never set), here its velocities stand in
            if (PERI) {
                if (homoDeform == 2 || homoDeform == 3) pvfE = vel - mul(ldm(sp.gradV), pos);
                else if (homoDeform == 4) pvfE = vel - mul(ldm(sp.gradV), pos - (dt / 2) * vel);
                if (homoDeform == 4) pvaE = angVel - D3{sp.spinVec[0], sp.spinVec[1], sp.spinVec[2]};
            }
        }
    }
    if (!blockedAll) {
        if ((flags & F_DOF_ALL) == 0) linAccel = f / mass;
        else linAccel = linAccelPartial(f, mass, flags);
        D3 pvf = vel, pva = angVel;
        if (PERI) {
            // Cell::pprevFluctVel / pprevFluctAngVel, core/Cell.cpp:36-57
            if (homoDeform == 2 || homoDeform == 3) pvf = vel - mul(ldm(sp.gradV), pos);
            else if (homoDeform == 4) pvf = vel - mul(ldm(sp.gradV), pos - (dt / 2) * vel);
            if (homoDeform == 4) pva = angVel - D3{sp.spinVec[0], sp.spinVec[1], sp.spinVec[2]};
        }
        if (damp) linAccel = dampAccel(linAccel, f, pvf, damping, dt);
        if (PERI && homoDeform == 4)
            vel = mul(ldm(sp.ImLL4hInv), (mul(ldm(sp.LmL), pos) + mul(ldm(sp.IpLL4h), vel)) + linAccel * dt);
        else
            vel = vel + dt * linAccel;
        if (!isZero(inertia)) {
            D3 angAccel{0, 0, 0};
            if ((flags & F_DOF_ALL) == 0) angAccel = D3{t.x / inertia.x, t.y / inertia.y, t.z / inertia.z};
            else angAccel = angAccelPartial(t, inertia, flags);
            if (damp) angAccel = dampAccel(angAccel, t, pva, damping, dt);
            angVel = angVel + dt * angAccel;
            if constexpr (ENERGY) angAccelE = angAccel;
            if (PERI && homoDeform == 4) angVel = angVel - D3{sp.deltaSpinVec[0], sp.deltaSpinVec[1], sp.deltaSpinVec[2]};
        }
    } else {
        if (PERI && homoDeform == 4) vel = mul(ldm(sp.ImLL4hInv), mul(ldm(sp.LmL), pos) + mul(ldm(sp.IpLL4h), vel));
    }
    if (PERI && homoDeform >= 0 && homoDeform != 4) {
        if (homoDeform == 2 || homoDeform == 3) {
            if (homoDeform == 3) vel = vel + mul(ldm(sp.midGradV), vel - (dt / 2.) * linAccel) * dt;
            vel = vel + mul(ldm(sp.dGradV), pos);
        } else if (homoDeform == 1) {
            pos = pos + mul(ldm(sp.nextGradV), pos) * dt;
        }
    }
    if constexpr (ENERGY) {
        if (sp.trackEnergy && !(flags & F_ENERGY_SKIP)) {
            const double2 ek = energyKin(pvfE, pvaE, linAccel, angAccelE, mass, inertia, dt);
            if (sp.kinSplit) {
                E.col[EN_NODE_K0 * E.cap + i] = ek.x;
                E.col[EN_NODE_K1 * E.cap + i] = ek.y;
            } else
                E.col[EN_NODE_K0 * E.cap + i] = ek.x + ek.y;
            E.col[EN_NODE_NKIN * E.cap + i] = 1.;
        }
    }
    pos = pos + vel * dt;
    const double4_32a o4 = N.ori[i];
    DQ ori{o4.x, o4.y, o4.z, o4.w};
    if (!isZero(angVel)) {
        const double angle = sqrt(sqn(angVel));
        const D3 axis = angVel / angle;
        const double ha = 0.5 * (angle * dt);
        double s, c;
        sincos(ha, &s, &c);
        const DQ q{c, s * axis.x, s * axis.y, s * axis.z};
        ori = qmul(q, ori);
    }
    ori = qnormalized(ori);
    N.posr[i] = st4(pos, pr.w);
    N.vel[i] = st4(vel, 0.);
    N.angv[i] = st4(angVel, 0.);
    N.ori[i] = make_double4_32a(ori.w, ori.x, ori.y, ori.z);
    if (sp.reset && !uni) resetForce(N, i, mass, sp.hasGravity && !(flags & F_GRAVITY_SKIP), spp, valid ? sceneOfN(N, i) : 0);
    // verlet test (d2 + moveDueToRot2 > maxD2 with no rotation term for spheres, walls, facets)
    const D3 lp = ld3(N.lastPos[i]);
    const double d2 = sqn(lp - pos);
    if (d2 + 0. > sp.maxD2) atomicOr(dFlags + FL_FULL, 1);
}

void launch_leapfrog(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const ScenePar* sp,
                     int* dFlags, int fromEnds, const long long* dStep, bool periodic, const EnergyCols* energy) {
    if (N.n == 0) return;
    const unsigned g = (N.n + 255) / 256;
    const EnergyCols E = energy ? *energy : EnergyCols{};
    if (energy) {
        if (periodic) k_leapfrog<true, true><<<g, 256, 0, st>>>(N, P, I, sp, dFlags, fromEnds, dStep, E);
        else k_leapfrog<false, true><<<g, 256, 0, st>>>(N, P, I, sp, dFlags, fromEnds, dStep, E);
    } else {
        if (periodic) k_leapfrog<true, false><<<g, 256, 0, st>>>(N, P, I, sp, dFlags, fromEnds, dStep, E);
        else k_leapfrog<false, false><<<g, 256, 0, st>>>(N, P, I, sp, dFlags, fromEnds, dStep, E);
    }
}

// ---------------------------------------------------------------------------------- ContactLoop
// Fused ContactLoop body (pkg/dem/ContactLoop.cpp:135-224) for one contact:
// Cg2 (above) -> Cg2_Any_Any_L6Geom__Base::handleSpheresLikeContact (pkg/dem/L6Geom.cpp:51-217)
// -> Cp2 on creation (FrictMat.cpp:20-44 / Hertz.cpp:9-50) -> Law2 (IdealElPl.cpp:12-122 /
// Hertz.cpp:58-182) -> global force on pA (Contact::getForceTorqueBranch, Contact.cpp:24-34).
// Clear the end slots of a contact that stops being real (its last contribution must vanish).
__device__ __forceinline__ void clearEnds(const DevIncidence& I, int64_t c) {
    const double4_32a z = make_double4_32a(0., 0., 0., 0.);
    const double2 z2 = make_double2(0., 0.);
    const int32_t sl = I.slotLo[c], sh = I.slotHi[c];
    I.endA[sl] = z;
    I.endB[sl] = z2;
    I.endA[sh] = z;
    I.endB[sh] = z2;
}

// A contact that becomes real: L6Geom::setInitialLocalCoords (pkg/dem/L6Geom.cpp:27-38, :53-71)
// and Cp2 (FrictMat.cpp:20-44 / Hertz.cpp:9-50). Out of line (see k_leapfrog).
struct NewContact {
    D3 c0, c1, c2;
    double ph[5];
};
__device__ __noinline__ NewContact newContact(D3 normal, double r1, double r2, double uN, double4_32a m1, double4_32a m2, double ma,
                                              double mb, const ScenePar* __restrict__ spp, int scene) {
    const ScenePar& sp = spp[scene];
    D3 c0, c1, c2;
    double ph0, ph1, ph2, ph3 = 0, ph4 = 0;
    const D3 locX = normal;
    const D3 ref = (fabs(locX.y) < fabs(locX.z)) ? D3{0, 1, 0} : D3{0, 0, 1};
    D3 locY = cross(locX, ref);
    locY = locY - locX * dot(locY, locX);
    locY = normalized(locY);
    c0 = locX;
    c1 = locY;
    c2 = cross(locX, locY);
    double lens0 = fabs(r1) + uN / 2, lens1 = fabs(r2) + uN / 2;
    if (lens0 < 0) lens0 = lens1;
    if (lens1 < 0) lens1 = lens0;
    const double rr = (r1 > 0 && r2 > 0) ? smin(r1, r2) : (r1 > 0 ? r1 : r2);
    const double contA = 3.14159265358979323846 * (rr * rr);
    // m1, m2: the materials' density young tanPhi ktDivKn; ma, mb: the nodes' masses
    if (sp.phys == 0) {
        // Cp2_FrictMat_FrictPhys::updateFrictPhys, pkg/dem/FrictMat.cpp:20-44
        ph0 = 1 / (1 / (m1.y * contA / lens0) + 1 / (m2.y * contA / lens1));
        ph1 = .5 * (m1.w + m2.w) * ph0;
        ph2 = smin(m1.z, m2.z);
    } else {
        // Cp2_FrictMat_HertzPhys::go, pkg/dem/Hertz.cpp:9-50 (kn0 = K*sqrt(R) is stored)
        const double nu1 = sp.hzPoisson, nu2 = sp.hzPoisson;
        const double E1 = m1.y, E2 = m2.y;
        const double K = (4 / 3.) * 1. / ((1 - nu1 * nu1) / E1 + (1 - nu2 * nu2) / E2);
        const double R = 1. / (1. / lens0 + 1. / lens1);
        const double kn0 = K * sqrt(R);
        const double G1 = E1 / (2 * (1 + nu1)), G2 = E2 / (2 * (1 + nu2));
        const double G = .5 * (G1 + G2);
        const double nu = .5 * (nu1 + nu2);
        ph0 = kn0;
        ph1 = 2 * sqrt(4 * R) * G / (2 - nu);
        ph2 = smin(m1.z, m2.z);
        ph4 = R;
        if (sp.hzViscOn) {
            const double mbar = (ma <= 0 && mb > 0) ? mb : ((ma > 0 && mb <= 0) ? ma : (ma * mb) / (ma + mb));
            ph3 = smax(0., sp.hzViscConst * sqrt(mbar * kn0));
        } else ph3 = 0.0;
    }
    NewContact r;
    r.c0 = c0;
    r.c1 = c1;
    r.c2 = c2;
    r.ph[0] = ph0;
    r.ph[1] = ph1;
    r.ph[2] = ph2;
    r.ph[3] = ph3;
    r.ph[4] = ph4;
    return r;
}
// L6Geom renormalisation of the frame every trsfRenorm steps (L6Geom.cpp:129-135). Out of line.
struct Frame3 {
    D3 c0, c1, c2;
};
__device__ __noinline__ Frame3 renormFrame(D3 c0, D3 c1) {
    Frame3 f;
    f.c0 = normalized(c0);
    c1 = c1 - f.c0 * dot(c1, f.c0);
    f.c1 = normalized(c1);
    f.c2 = cross(f.c0, f.c1);
    return f;
}
// Coulomb cap of the shear force: IdealElPl.cpp:57-63 (zeroIfNull) and Hertz.cpp:160-165. Out of line.
__device__ __noinline__ double2 capShear(double ft1, double ft2, double maxFt, bool zeroIfNull) {
    const double FtNorm = sqrt(ft1 * ft1 + ft2 * ft2);
    double ratio = maxFt / FtNorm;
    if (zeroIfNull && FtNorm == 0.) ratio = 0.;
    return make_double2(ft1 * ratio, ft2 * ratio);
}

template <bool PERI, bool ENERGY>
__global__ void __launch_bounds__(128) k_contact_fp64(DevNodes N, DevParticles P, DevContacts C, DevIncidence I,
                                                     const double4_32a* __restrict__ mats, const ScenePar* __restrict__ spp,
                                                     const long long* __restrict__ dStep, int* __restrict__ dFlags,
                                                     EnergyCols E) {
    if (dFlags[FL_FULL] || halted(dFlags)) {
        // the collider runs before this step's contacts; the steps queued after it wait
        if (blockIdx.x == 0 && threadIdx.x == 0) dFlags[FL_HALT] = 1;
        return;
    }
    int* dErr = dFlags + FL_ERR;
    const int64_t rk = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (rk >= I.nAct) return;
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
    const double dt = sp.dt;
    D3 shift2{0, 0, 0}, shiftVel2{0, 0, 0};
    if (PERI) {
        int a, b, cc;
        unpackCellDist(C.cdist[c], a, b, cc);
        if (fl & C_SWAP) { a = -a; b = -b; cc = -cc; }
        const D3 cd{(double)a, (double)b, (double)cc};
        shift2 = mul(ldm(sp.hSize), cd);
        shiftVel2 = mul(ldm(sp.shiftVelMat), cd);
    }
    Geo g;
    bool touch;
    if (ty == CT_SS) touch = geomSS(N, A, B, shift2, real, sp.ssDistFactor, g);
    else if (ty == CT_WS) touch = geomWS(N, P, real ? C.col[CC_T0X + P.aux[A].x][c] : 0., A, B, shift2, real, g);
    else touch = geomFS(N, P, A, B, shift2, real, g, dErr);
    if (!touch) {
        C.flags[c] = fl;
        return;
    }
    D3 c0, c1, c2;
    D3 lvel{0, 0, 0};
    double ph0, ph1, ph2, ph3 = 0, ph4 = 0;
    double fn, ft1 = 0, ft2 = 0;
    if (!real) {
        // new geometry: L6Geom::setInitialLocalCoords pkg/dem/L6Geom.cpp:27-38 and :53-71, Cp2
        const double ma = N.minert[P.shape[A] == WG_SHAPE_FACET ? P.aux[A].x : A].w, mb = N.minert[B].w;
        const NewContact nc = newContact(g.normal, g.r1, g.r2, g.uN, mats[P.mat[A]], mats[P.mat[B]], ma, mb, spp, sceneOfP(P, B));
        c0 = nc.c0;
        c1 = nc.c1;
        c2 = nc.c2;
        ph0 = nc.ph[0];
        ph1 = nc.ph[1];
        ph2 = nc.ph[2];
        ph3 = nc.ph[3];
        ph4 = nc.ph[4];
        C.col[CC_P0][c] = ph0;
        C.col[CC_P1][c] = ph1;
        C.col[CC_P2][c] = ph2;
        C.col[CC_P3][c] = ph3;
        C.col[CC_P4][c] = ph4;
        C.col[CC_UN0][c] = g.uN;  // uN of the first step, which fixes L6Geom.lens (DynDt)
        C.step0[c] = (int32_t)step;
    } else {
        // existing geometry: update branch, pkg/dem/L6Geom.cpp:79-216
        const int am = sp.approxMask;
        const D3 currNormal = g.normal;
        const D3 prevNormal{C.col[CC_T0X][c], C.col[CC_T0Y][c], C.col[CC_T0Z][c]};
        const D3 prevC1{C.col[CC_T1X][c], C.col[CC_T1Y][c], C.col[CC_T1Z][c]};
        const D3 prevContPt{C.col[CC_CPX][c], C.col[CC_CPY][c], C.col[CC_CPZ][c]};
        const D3 normRotVec = cross(prevNormal, currNormal);
        D3 midNormal = (am & 1) ? prevNormal : .5 * (prevNormal + currNormal);
        if (sqrt(sqn(midNormal)) == 0) midNormal = currNormal;
        else if (!(am & 2) && !(am & 1)) midNormal = normalized(midNormal);
        const D3 normTwistVec = ((midNormal * dt) * .5) * dot(midNormal, g.angVel1 + g.angVel2);
        const D3 rt = normRotVec + normTwistVec;
        D3 m0, m1v;
        if (am & 4) {
            m0 = prevNormal;
            m1v = prevC1;
        } else {
            m0 = midNormal;
            m1v = prevC1 - cross(prevC1, rt) / 2.;
        }
        const D3 m2v = cross(m0, m1v);
        c0 = currNormal;
        c1 = prevC1 - cross(m1v, rt);
        c2 = cross(c0, c1);
        if (sp.trsfRenorm > 0 && (step % sp.trsfRenorm) == 0) {
            const Frame3 f = renormFrame(c0, c1);
            c0 = f.c0;
            c1 = f.c1;
            c2 = f.c2;
        }
        D3 midContPt, midPos1, midPos2;
        if (am & 8) {
            midContPt = g.contPt;
            midPos1 = g.pos1;
            midPos2 = g.pos2;
        } else {
            midContPt = .5 * (prevContPt + g.contPt);
            midPos1 = g.pos1 - (dt / 2.) * g.vel1;
            midPos2 = g.pos2 - (dt / 2.) * (g.vel2 + shiftVel2);
        }
        const D3 c1x = (sp.noRatch && g.r1 > 0) ? g.r1 * midNormal : midContPt - midPos1;
        const D3 c2x = (sp.noRatch && g.r2 > 0) ? (-g.r2) * midNormal : midContPt - midPos2;
        const D3 relVel = ((g.vel2 + shiftVel2) + cross(g.angVel2, c2x)) - (g.vel1 + cross(g.angVel1, c1x));
        lvel = D3{dot(m0, relVel), dot(m1v, relVel), dot(m2v, relVel)};
        ph0 = C.col[CC_P0][c];
        ph1 = C.col[CC_P1][c];
        ph2 = C.col[CC_P2][c];
        ph3 = C.col[CC_P3][c];
        ph4 = C.col[CC_P4][c];
        ft1 = C.col[CC_FT1][c];
        ft2 = C.col[CC_FT2][c];
    }
    const double uN = g.uN;
    bool keep = true;
    // energies of this contact in this step (EnergyTracker adds, IdealElPl.cpp:25-37,58-90,
    // Hertz.cpp:154-179)
    double eElast = 0, ePlast = 0, eBroken = 0, eViscN = 0, eViscT = 0, nElast = 0, nBroken = 0;
    if (sp.law == 0) {
        // Law2_L6Geom_FrictPhys_IdealElPl::go, pkg/dem/IdealElPl.cpp:18-81 (kn kt tanPhi = ph0 ph1 ph2)
        if (uN > 0 && !sp.noBreak) {
            keep = false;
            if (ENERGY && sp.noSlip) {
                // the broken contact's current elastic potential is lost
                const double bf = ph0 * uN, b1 = ft1 + (dt * ph1) * lvel.y, b2 = ft2 + (dt * ph1) * lvel.z;
                eBroken = .5 * ((bf * bf) / ph0 + (b1 * b1 + b2 * b2) / ph1);
                nBroken = 1;
            }
        } else {
            fn = ph0 * uN;
            if (sp.noFrict || ph2 == 0.) {
                ft1 = 0;
                ft2 = 0;
            } else {
                ft1 = ft1 + (dt * ph1) * lvel.y;
                ft2 = ft2 + (dt * ph1) * lvel.z;
                const double maxFt = fabs(fn) * ph2;
                if ((ft1 * ft1 + ft2 * ft2) > maxFt * maxFt && !sp.noSlip) {
                    if (ENERGY) ePlast = (ph1 != 0. ? (maxFt * (sqrt(ft1 * ft1 + ft2 * ft2) - maxFt)) / ph1 : 0.);
                    const double2 q = capShear(ft1, ft2, maxFt, true);
                    ft1 = q.x;
                    ft2 = q.y;
                }
                if (isnan(fn) || isnan(ft1) || isnan(ft2)) atomicCAS(dErr, 0, 101);  // "NaN force in contact"
            }
            if (ENERGY) {
                eElast = 0.5 * ((fn * fn) / ph0 + (ph1 != 0. ? (ft1 * ft1 + ft2 * ft2) / ph1 : 0.));
                if (isnan(eElast)) eElast = 0.;
                nElast = 1;
            }
        }
    } else {
        // Law2_L6Geom_HertzPhys_DMT::go, DMT branch, pkg/dem/Hertz.cpp:58-87,143-172 (kn0 kt0 tanPhi alpha_sqrtMK R)
        if (uN > 0) keep = false;
        else {
            const double su = sqrt(-uN);
            const double Fne = -ph0 * (su * su * su);
            const double Fna = 4 * 3.14159265358979323846 * ph4 * sp.hzGamma;
            const double eta = (ph3 > 0 ? ph3 * sqrt(sqrt(smax(-uN, 0.))) : 0.);
            double Fnv = eta * lvel.x;
            if (sp.noAttraction && Fne + Fnv > 0) Fnv = -Fne;
            fn = (Fne + Fna) + Fnv;
            if (ENERGY) eViscN = (Fnv * lvel.x) * dt;
            const double kt = ph1 * sqrt(uN < 0 ? -uN : 0);
            ft1 = (dt * kt) * lvel.y;
            ft2 = (dt * kt) * lvel.z;
            const double maxFt = smax(0., fn) * ph2;
            if ((ft1 * ft1 + ft2 * ft2) > maxFt * maxFt) {
                if (ENERGY) {
                    const double fN = sqrt(ft1 * ft1 + ft2 * ft2);
                    ePlast = ((.5 * (fN - maxFt) + maxFt) * (fN - maxFt)) / kt;
                }
                const double2 q = capShear(ft1, ft2, maxFt, false);
                ft1 = q.x;
                ft2 = q.y;
            } else {
                ft1 = ft1 + eta * lvel.y;
                ft2 = ft2 + eta * lvel.z;
                if (ENERGY) eViscT = (eta * (lvel.y * lvel.y + lvel.z * lvel.z)) * dt;
            }
            if (ENERGY && uN < 0) {
                // normalElasticEnergy(kn0, -uN) = kn0*(2/5)*(-uN)^(5/2) (Hertz.hpp:48), pow(sqrt(x),5) as s^5
                eElast = (ph0 * (2 / 5.)) * ((((su * su) * su) * su) * su) + (0.5 * (ft1 * ft1 + ft2 * ft2)) / kt;
                nElast = 1;
            }
        }
    }
    if constexpr (ENERGY) {
        const int64_t cp = E.cap;
        E.col[EN_CON_ELAST * cp + rk] = eElast;
        E.col[EN_CON_PLAST * cp + rk] = ePlast;
        E.col[EN_CON_BROKEN * cp + rk] = eBroken;
        E.col[EN_CON_VISCN * cp + rk] = eViscN;
        E.col[EN_CON_VISCT * cp + rk] = eViscT;
        E.col[EN_CON_NELAST * cp + rk] = nElast;
        E.col[EN_CON_NBROKEN * cp + rk] = nBroken;
    }
    if (!keep) {
        // ContactContainer::requestRemoval: geom and phys reset, contact pending for the collider
        C.flags[c] = (fl & ~C_REAL) | C_PENDING;
        if (real) clearEnds(I, c);
        return;
    }
    const DQ ori = quatFromCols(c0, c1, c2);
    const D3 Fg = qrot(ori, D3{fn, ft1, ft2});
    // Contact::getForceTorqueBranch + applyForceUninodal (Contact.cpp:24-34, ContactLoop.cpp:261-267):
    // F = ori*force*sign, torque = xc x F + T with xc = contact point - (node + shift for pB)
    {
        const bool aIsLo = !(fl & C_SWAP);
        if (ty != CT_FS) {  // facets are multinodal: no force is applied to them here
            const D3 FA = Fg * 1.0;
            const D3 xcA = g.contPt - ld3(N.posr[A]);
            const D3 TA = cross(xcA, FA) + D3{0, 0, 0};
            const int sA = aIsLo ? I.slotLo[c] : I.slotHi[c];
            I.endA[sA] = make_double4_32a(FA.x, FA.y, FA.z, TA.x);
            I.endB[sA] = make_double2(TA.y, TA.z);
        }
        const D3 FB = Fg * -1.0;
        const D3 xcB = g.contPt - (ld3(N.posr[B]) + (PERI ? shift2 : D3{0, 0, 0}));
        const D3 TB = cross(xcB, FB) + D3{0, 0, 0};
        const int sB = aIsLo ? I.slotHi[c] : I.slotLo[c];
        I.endA[sB] = make_double4_32a(FB.x, FB.y, FB.z, TB.x);
        I.endB[sB] = make_double2(TB.y, TB.z);
    }
    C.col[CC_T0X][c] = c0.x;
    C.col[CC_T0Y][c] = c0.y;
    C.col[CC_T0Z][c] = c0.z;
    C.col[CC_T1X][c] = c1.x;
    C.col[CC_T1Y][c] = c1.y;
    C.col[CC_T1Z][c] = c1.z;
    C.col[CC_CPX][c] = g.contPt.x;
    C.col[CC_CPY][c] = g.contPt.y;
    C.col[CC_CPZ][c] = g.contPt.z;
    C.col[CC_FN][c] = fn;
    C.col[CC_FT1][c] = ft1;
    C.col[CC_FT2][c] = ft2;
    C.flags[c] = fl | C_REAL;
}

void launch_contact_fp64(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C, const DevIncidence& I,
                         const double4_32a* mats, const ScenePar* sp, const long long* dStep, int* dFlags, bool periodic, int block,
                         const EnergyCols* energy) {
    const int bs = block;
    // launched even without contacts: it raises FL_HALT when a full run is due
    const unsigned g = (unsigned)std::max<int64_t>(1, (I.nAct + bs - 1) / bs);
    const EnergyCols E = energy ? *energy : EnergyCols{};
    if (energy) {
        if (periodic) k_contact_fp64<true, true><<<g, bs, 0, st>>>(N, P, C, I, mats, sp, dStep, dFlags, E);
        else k_contact_fp64<false, true><<<g, bs, 0, st>>>(N, P, C, I, mats, sp, dStep, dFlags, E);
    } else {
        if (periodic) k_contact_fp64<true, false><<<g, bs, 0, st>>>(N, P, C, I, mats, sp, dStep, dFlags, E);
        else k_contact_fp64<false, false><<<g, bs, 0, st>>>(N, P, C, I, mats, sp, dStep, dFlags, E);
    }
}

// ---------------------------------------------------------------------------------- energy sums
// The step's contributions of every node or active contact (columns of E), summed per column in
// a fixed order (grid-stride per thread, a shared-memory tree per block, then the blocks in order)
// and added to Scene.energy: the resettable entries take the step's sum, the others accumulate.
// An entry exists once a contribution was added (a zero one for the entries that a zero creates).
// Nothing is added for a step whose kernels did not run (halted; for contacts also a step waiting
// for the collider, whose contact loop runs after it).
constexpr int kEnergyBlocks = 256;
__global__ void __launch_bounds__(256) k_energy_partial(EnergyCols E, int ncol, int64_t n, double* __restrict__ partial,
                                                        const int* __restrict__ dFlags) {
    __shared__ double sm[256];
    if (halted(dFlags)) return;
    for (int c = 0; c < ncol; c++) {
        double a = 0;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            a = a + E.col[c * E.cap + i];
        sm[threadIdx.x] = a;
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if (threadIdx.x < w) sm[threadIdx.x] = sm[threadIdx.x] + sm[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = sm[0];
        __syncthreads();
    }
}
// which = 0: node columns, 1: contact columns
__global__ void k_energy_final(const double* __restrict__ partial, int nb, int which, double* __restrict__ energy,
                               int32_t* __restrict__ created, const int* __restrict__ dFlags, int kinSplit) {
    if (threadIdx.x != 0 || halted(dFlags) || (which == 1 && dFlags[FL_FULL])) return;
    auto sum = [&](int c) {
        double a = 0;
        for (int b = 0; b < nb; b++) a = a + partial[c * nb + b];
        return a;
    };
    if (which == 0) {
        const double k0 = sum(EN_NODE_K0), k1 = sum(EN_NODE_K1), gr = sum(EN_NODE_GRAV), dm = sum(EN_NODE_DAMP);
        const bool kin = sum(EN_NODE_NKIN) > 0, grav = sum(EN_NODE_NGRAV) > 0;
        if (kinSplit) {
            energy[EN_KINTRANS] = k0;
            energy[EN_KINROT] = k1;
            if (kin) created[EN_KINTRANS] = created[EN_KINROT] = 1;
        } else {
            energy[EN_KINETIC] = k0;
            if (kin) created[EN_KINETIC] = 1;
        }
        energy[EN_GRAV] += gr;
        if (grav) created[EN_GRAV] = 1;
        energy[EN_DAMP] += dm;
        if (dm != 0) created[EN_DAMP] = 1;
    } else {
        const double el = sum(EN_CON_ELAST), pl = sum(EN_CON_PLAST), br = sum(EN_CON_BROKEN), vn = sum(EN_CON_VISCN),
                     vt = sum(EN_CON_VISCT);
        energy[EN_ELAST] = el;
        if (sum(EN_CON_NELAST) > 0) created[EN_ELAST] = 1;
        energy[EN_PLAST] += pl;
        if (pl != 0) created[EN_PLAST] = 1;
        energy[EN_BROKEN] += br;
        if (sum(EN_CON_NBROKEN) > 0) created[EN_BROKEN] = 1;
        energy[EN_VISCN] += vn;
        if (vn != 0) created[EN_VISCN] = 1;
        energy[EN_VISCT] += vt;
        if (vt != 0) created[EN_VISCT] = 1;
    }
}
// ContactLoop::run, pkg/dem/ContactLoop.cpp:236-246: stress = sum / volume, then
// dW = -tr(gradV * (stress + prevStress)/2) * dt * midVol, midVol the mean of this step's and the
// previous step's cell volume (this step's at first); prev takes this step's stress and volume.
__global__ void k_energy_gradv(const double* __restrict__ sum9, const ScenePar* __restrict__ sp, double* __restrict__ prev,
                               double* __restrict__ energy, int32_t* __restrict__ created, const int* __restrict__ dFlags) {
    if (threadIdx.x != 0 || halted(dFlags) || dFlags[FL_FULL]) return;
    const double* a = sp->hSize;
    const double vol = (a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6])) + a[2] * (a[3] * a[7] - a[4] * a[6]);
    double st[9], mid[9];
    for (int q = 0; q < 9; q++) {
        st[q] = sum9[q] / vol;
        mid[q] = .5 * (st[q] + prev[q]);
    }
    const double pv = prev[9];
    const double midVol = !isnan(pv) ? .5 * (pv + vol) : vol;
    const double* g = sp->gradV;
    double tr = 0;
    for (int i = 0; i < 3; i++) tr = tr + ((g[3 * i] * mid[i] + g[3 * i + 1] * mid[3 + i]) + g[3 * i + 2] * mid[6 + i]);
    const double dW = ((-tr) * sp->dt) * midVol;
    energy[EN_GRADV] += dW;
    if (dW != 0) created[EN_GRADV] = 1;
    for (int q = 0; q < 9; q++) prev[q] = st[q];
    prev[9] = vol;
}
void launch_energy_gradv(cudaStream_t st, const double* sum9, const ScenePar* sp, double* prev, double* energy, int32_t* created,
                         const int* dFlags) {
    k_energy_gradv<<<1, 32, 0, st>>>(sum9, sp, prev, energy, created, dFlags);
}

void launch_energy_sum(cudaStream_t st, const EnergyCols& E, int which, int64_t n, double* partial, double* energy, int32_t* created,
                       const int* dFlags, bool kinSplit) {
    const int ncol = which == 0 ? (int)EN_NODE_NCOL : (int)EN_CON_NCOL;
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(kEnergyBlocks, (n + 255) / 256));
    k_energy_partial<<<nb, 256, 0, st>>>(E, ncol, n, partial, dFlags);
    k_energy_final<<<1, 32, 0, st>>>(partial, nb, which, energy, created, dFlags, kinSplit ? 1 : 0);
}

// ---------------------------------------------------------------------------------- force sum
// DemData.force/torque for reporting after a run: the sum of the Leapfrog kernel (m*g, then every
// end slot of the particle in slot order) written to the node, for every particle whose degree
// is at most kHeavyThreshold.
__global__ void __launch_bounds__(256) k_forces(DevNodes N, DevParticles P, DevIncidence I, const ScenePar* __restrict__ spp) {
    __shared__ EndStage<double4_32a, double2, 32> stage[8];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const ScenePar& sp = spp[p < P.n ? sceneOfP(P, p) : 0];
    const bool uni = p < P.n && P.shape[p] != WG_SHAPE_FACET;
    int e0 = 0, e1 = 0;
    bool take = false;
    D3 F{0, 0, 0}, T{0, 0, 0};
    if (uni) {
        const uint32_t flags = N.flags[p];
        const double mass = N.minert[p].w;
        if (sp.hasGravity && !(flags & F_GRAVITY_SKIP)) F = mass * D3{sp.g[0], sp.g[1], sp.g[2]};
        if (sp.applyForces) {
            endRange(I, p, e0, e1);
            take = (e1 - e0) <= kHeavyThreshold;
        }
    }
    SumD acc{F, T};
    warpSumEnds(I.endA, I.endB, take, e0, e1, stage[threadIdx.x >> 5], acc);
    if (uni && (take || !sp.applyForces)) {
        N.force[p] = st4(acc.F, 0.);
        N.torque[p] = st4(acc.T, 0.);
    }
}

// Particles with many end slots (walls, crowded spheres): one warp each, lane q < 6 adds
// component q of the particle's slots one after the other in slot order, starting from m*g
// (force) or 0 (torque): the order of the reference's deterministic pass, the same as the
// Leapfrog kernel's sum for the other particles, so FP64 results stay bitwise. Six dependent
// chains per particle; only particles with a free DOF take this path every step.
__global__ void __launch_bounds__(128) k_forces_heavy(DevNodes N, DevIncidence I, const int32_t* __restrict__ list, int n,
                                                      const ScenePar* __restrict__ spp, const int* __restrict__ dFlags) {
    if (dFlags && halted(dFlags)) return;
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (w >= n || lane >= 6) return;
    const int p = list[w];
    const ScenePar& sp = spp[sceneOfN(N, p)];
    int e0, e1;
    endRange(I, p, e0, e1);
    double acc = 0;
    if (lane < 3 && sp.hasGravity && !(N.flags[p] & F_GRAVITY_SKIP)) acc = N.minert[p].w * sp.g[lane];
    const double* a = reinterpret_cast<const double*>(I.endA);
    const double* b = reinterpret_cast<const double*>(I.endB);
    for (int e = e0; e < e1; e++) acc = acc + (lane < 4 ? a[4 * (int64_t)e + lane] : b[2 * (int64_t)e + (lane - 4)]);
    double* f = reinterpret_cast<double*>(N.force + p);
    double* t = reinterpret_cast<double*>(N.torque + p);
    if (lane < 3) f[lane] = acc;
    else t[lane - 3] = acc;
    if (lane == 0) f[3] = 0.;
    if (lane == 3) t[3] = 0.;
}

// ContactLoop.stress for periodic scenes (ContactLoop.cpp:211-247): sum over real contacts of
// F_A (x) (x_B + shift - x_A), divided by the cell volume on the host. Per-block partial sums in a
// fixed tree, then one block adds the partials in block order.
__global__ void k_stress_partial(DevNodes N, DevParticles P, DevContacts C, DevIncidence I, const ScenePar* __restrict__ spp,
                                 double* __restrict__ partial) {
    __shared__ double sh[9][256];
    const int64_t rk = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (rk < I.nAct) {
        const int4 wk = I.work[rk];
        const int64_t c = wk.x;
        const uint32_t fl = C.flags[c];
        if (fl & C_REAL) {
            const int A = wk.y, B = wk.z;
            const bool aIsLo = !(fl & C_SWAP);
            const int sA = aIsLo ? I.slotLo[c] : I.slotHi[c];
            D3 F;
            if (I.endA) F = D3{I.endA[sA].x, I.endA[sA].y, I.endA[sA].z};
            else F = D3{(double)I.endAf[sA].x, (double)I.endAf[sA].y, (double)I.endAf[sA].z};
            const int nA = (P.shape[A] == WG_SHAPE_FACET) ? P.aux[A].x : A;
            D3 branch = D3{N.posr[B].x, N.posr[B].y, N.posr[B].z} - D3{N.posr[nA].x, N.posr[nA].y, N.posr[nA].z};
            int a, b, cc;
            unpackCellDist(C.cdist[c], a, b, cc);
            if (fl & C_SWAP) { a = -a; b = -b; cc = -cc; }
            if (a != 0 || b != 0 || cc != 0) branch = branch + mul(ldm(spp->hSize), D3{(double)a, (double)b, (double)cc});
            const double Fa[3] = {F.x, F.y, F.z}, Ba[3] = {branch.x, branch.y, branch.z};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) v[3 * i + j] = Fa[i] * Ba[j];
        }
    }
    for (int q = 0; q < 9; q++) sh[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 9; q++) sh[q][threadIdx.x] = sh[q][threadIdx.x] + sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 9; q++) partial[9 * blockIdx.x + q] = sh[q][0];
}
__global__ void k_stress_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    if (threadIdx.x >= 9) return;
    double acc = 0;
    for (int b = 0; b < nb; b++) acc = acc + partial[9 * b + threadIdx.x];
    out[threadIdx.x] = acc;
}
int launch_stress(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C, const DevIncidence& I,
                  const ScenePar* sp, double* scratch, int64_t scratchDoubles, double* out) {
    const int64_t nb = std::max<int64_t>(1, (I.nAct + 255) / 256);
    if (9 * nb > scratchDoubles) return -1;
    k_stress_partial<<<(unsigned)nb, 256, 0, st>>>(N, P, C, I, sp, scratch);
    k_stress_final<<<1, 32, 0, st>>>(scratch, (int)nb, out);
    return 0;
}

// ---------------------------------------------------------------------------------- DynDt
// DynDt::nodalStiffAdd (pkg/dem/DynDt.cpp:17-38), the part of one contact: each real contact
// writes into the end slot of each of its particles the contact's additions to that node's
// translational and rotational stiffness,
//   ktrans += n²(kn - kt) + kt,   krot += lens[ix]²·kt·(n²y + n²z, n²z + n²x, n²x + n²y),
// n = the L6Geom node orientation (Quaternionr(trsf), L6Geom.cpp:216) applied to the x axis, ix
// the particle's index in the contact. kn and kt are those the last law call left in the phys:
// FrictPhys keeps them constant; the Hertz law sets kn = 3/2·kn0·sqrt(-uN) and
// kt = kt0·sqrt(max(-uN, 0)) (Hertz.cpp:69,157) from the uN of the step, which the geometry
// functor recomputes here from the unchanged positions. lens are |r| + uN/2 of the contact's first
// step (L6Geom.cpp:63-66). Facets are left out (their nodes must be fully blocked). The slots
// are zeroed beforehand, so non-real contacts add nothing.
// F32: the contact state of the FP32-force mode (trsf columns and phys constants in FP32, written
// back from the packed sphere-sphere state before the call); n is trsf column 0 itself, and the
// lens are |r| + uN/2 of the current step (that mode keeps no uN of the first step: the
// difference is uN0/2 - uN/2, below 1e-4 of the radius for the overlaps of a stable contact).
template <bool PERI, bool F32>
__global__ void __launch_bounds__(128) k_dyndt_ends(DevNodes N, DevParticles P, DevContacts C, DevIncidence I,
                                                    const ScenePar* __restrict__ spp, double4_32a* __restrict__ kA,
                                                    double2* __restrict__ kB, int* __restrict__ dErr) {
    const int64_t rk = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (rk >= I.nAct) return;
    const int4 wk = I.work[rk];
    const int64_t c = wk.x;
    const int A = wk.y, B = wk.z;
    const uint32_t fl = C.flags[c];
    if (!(fl & C_REAL)) return;
    const ScenePar& sp = spp[sceneOfP(P, B)];
    const uint32_t ty = ctype((uint32_t)wk.w);
    D3 shift2{0, 0, 0};
    if (PERI) {
        int a, b, cc;
        unpackCellDist(C.cdist[c], a, b, cc);
        if (fl & C_SWAP) { a = -a; b = -b; cc = -cc; }
        shift2 = mul(ldm(sp.hSize), D3{(double)a, (double)b, (double)cc});
    }
    Geo g;
    const double wallSense = ty == CT_WS ? (F32 ? (double)C.fcol[CF_T0X + P.aux[A].x][c] : C.col[CC_T0X + P.aux[A].x][c]) : 0.;
    if (ty == CT_SS) geomSS(N, A, B, shift2, true, sp.ssDistFactor, g);
    else if (ty == CT_WS) geomWS(N, P, wallSense, A, B, shift2, true, g);
    else geomFS(N, P, A, B, shift2, true, g, dErr);
    D3 n;
    double p0, p1, uN0;
    if (F32) {
        n = D3{(double)C.fcol[CF_T0X][c], (double)C.fcol[CF_T0Y][c], (double)C.fcol[CF_T0Z][c]};
        p0 = C.fcol[CF_P0][c];
        p1 = C.fcol[CF_P1][c];
        uN0 = g.uN;
    } else {
        const D3 c0{C.col[CC_T0X][c], C.col[CC_T0Y][c], C.col[CC_T0Z][c]};
        const D3 c1{C.col[CC_T1X][c], C.col[CC_T1Y][c], C.col[CC_T1Z][c]};
        n = qrot(quatFromCols(c0, c1, cross(c0, c1)), D3{1., 0., 0.});
        p0 = C.col[CC_P0][c];
        p1 = C.col[CC_P1][c];
        uN0 = C.col[CC_UN0][c];
    }
    const D3 n2{n.x * n.x, n.y * n.y, n.z * n.z};
    double kn, kt;
    if (sp.law == 0) {
        kn = p0;
        kt = p1;
    } else {
        kn = (3 / 2.) * p0 * sqrt(-g.uN);
        kt = p1 * sqrt(g.uN < 0 ? -g.uN : 0);
    }
    double l0 = fabs(g.r1) + uN0 / 2, l1 = fabs(g.r2) + uN0 / 2;
    if (l0 < 0) l0 = l1;
    if (l1 < 0) l1 = l0;
    const D3 kTr{n2.x * (kn - kt) + kt, n2.y * (kn - kt) + kt, n2.z * (kn - kt) + kt};
    const D3 rv{n2.y + n2.z, n2.z + n2.x, n2.x + n2.y};
    const bool aIsLo = !(fl & C_SWAP);
    if (ty != CT_FS) {
        const double s0 = (l0 * l0) * kt;
        const int sA = aIsLo ? I.slotLo[c] : I.slotHi[c];
        kA[sA] = make_double4_32a(kTr.x, kTr.y, kTr.z, s0 * rv.x);
        kB[sA] = make_double2(s0 * rv.y, s0 * rv.z);
    }
    const double s1 = (l1 * l1) * kt;
    const int sB = aIsLo ? I.slotHi[c] : I.slotLo[c];
    kA[sB] = make_double4_32a(kTr.x, kTr.y, kTr.z, s1 * rv.x);
    kB[sB] = make_double2(s1 * rv.y, s1 * rv.z);
}

// DynDt::nodalCritDtSq (pkg/dem/DynDt.cpp:42-63) of the node of each sphere and wall: the sums
// over the particle's end slots in slot order (ascending id of the other particle, the order of
// Particle.contacts), then 2·min(m/|ktrans_i|, I_i/|krot_i|) over the free, stiff axes; fully
// blocked nodes are always stable. The minimum over nodes (critDt_stiffness, :66-76) goes to
// *out as the bits of a non-negative double.
// perScene: out[scene of the node] instead of *out (a batch of scenes, each with its own DynDt).
__global__ void __launch_bounds__(256) k_dyndt_nodes(DevNodes N, DevParticles P, DevIncidence I, const double4_32a* __restrict__ kA,
                                                     const double2* __restrict__ kB, unsigned long long* __restrict__ out,
                                                     int perScene) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const double kInf = __longlong_as_double(0x7ff0000000000000LL);
    double v = kInf;
    if (p < P.n && P.shape[p] != WG_SHAPE_FACET) {
        const uint32_t fl = N.flags[p];
        if ((fl & F_DOF_ALL) != F_DOF_ALL) {
            int e0, e1;
            endRange(I, p, e0, e1);
            D3 kt{0., 0., 0.}, kr{0., 0., 0.};
            for (int e = e0; e < e1; e++) {
                const double4_32a a = kA[e];
                const double2 b = kB[e];
                kt = kt + D3{a.x, a.y, a.z};
                kr = kr + D3{a.w, b.x, b.y};
            }
            const double4_32a mi = N.minert[p];
            const double m = mi.w, in[3] = {mi.x, mi.y, mi.z}, t[3] = {kt.x, kt.y, kt.z}, r[3] = {kr.x, kr.y, kr.z};
            double ret = kInf;
            for (int i = 0; i < 3; i++)
                if (t[i] != 0 && m > 0. && !(fl & (1u << i))) {
                    const double q = m / fabs(t[i]);
                    ret = q < ret ? q : ret;
                }
            for (int i = 0; i < 3; i++)
                if (r[i] != 0 && in[i] > 0. && !(fl & (8u << i))) {
                    const double q = in[i] / fabs(r[i]);
                    ret = q < ret ? q : ret;
                }
            v = 2 * ret;
        }
    }
    if (perScene) {  // uniform over the grid
        if (v < kInf) atomicMin(out + sceneOfP(P, p), (unsigned long long)__double_as_longlong(v));
        return;
    }
    // block minimum, then one atomic per block (non-negative doubles order like their bit patterns)
    __shared__ double sm[256];
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const double o = sm[threadIdx.x + w];
            if (o < sm[threadIdx.x]) sm[threadIdx.x] = o;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicMin(out, (unsigned long long)__double_as_longlong(sm[0]));
}

void launch_dyndt(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C, const DevIncidence& I,
                  const ScenePar* sp, double4_32a* kA, double2* kB, unsigned long long* out, int* dErr, bool periodic, bool fp32,
                  bool perScene) {
    if (I.nAct > 0) {
        const unsigned g = (unsigned)((I.nAct + 127) / 128);
        if (fp32) {
            if (periodic) k_dyndt_ends<true, true><<<g, 128, 0, st>>>(N, P, C, I, sp, kA, kB, dErr);
            else k_dyndt_ends<false, true><<<g, 128, 0, st>>>(N, P, C, I, sp, kA, kB, dErr);
        } else {
            if (periodic) k_dyndt_ends<true, false><<<g, 128, 0, st>>>(N, P, C, I, sp, kA, kB, dErr);
            else k_dyndt_ends<false, false><<<g, 128, 0, st>>>(N, P, C, I, sp, kA, kB, dErr);
        }
    }
    if (P.n > 0) k_dyndt_nodes<<<(P.n + 255) / 256, 256, 0, st>>>(N, P, I, kA, kB, out, perScene ? 1 : 0);
}

// Scene::doOneStep's step counter (core/Scene.cpp:386), advanced only by a step that completed.
__global__ void k_step_advance(long long* dStep, const int* __restrict__ dFlags) {
    if (dFlags[FL_FULL] || halted(dFlags)) return;
    *dStep += 1;
}

void launch_forces(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const ScenePar* sp,
                   const int* dFlags, bool perStep) {
    if (P.n == 0) return;
    if (perStep) {
        if (I.nHeavyFree > 0) k_forces_heavy<<<(I.nHeavyFree + 3) / 4, 128, 0, st>>>(N, I, I.heavyFree, I.nHeavyFree, sp, dFlags);
        return;
    }
    k_forces<<<(P.n + 255) / 256, 256, 0, st>>>(N, P, I, sp);
    if (I.nHeavy > 0) k_forces_heavy<<<(I.nHeavy + 3) / 4, 128, 0, st>>>(N, I, I.heavy, I.nHeavy, sp, nullptr);
}

void launch_advance(cudaStream_t st, long long* dStep, const int* dFlags) { k_step_advance<<<1, 1, 0, st>>>(dStep, dFlags); }

}  // namespace wg
