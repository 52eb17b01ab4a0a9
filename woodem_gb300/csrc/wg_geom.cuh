// Cg2 geometry functors in FP64 (shared by the FP64 and FP32 contact kernels).
// Every expression keeps the operand order of the reference expression it restates.
#pragma once
#include "wg_internal.h"
#include "wg_math.cuh"

namespace wg {

__device__ __forceinline__ D3 ld3(const double4_32a& v) { return D3{v.x, v.y, v.z}; }

struct Geo {
    D3 pos1, vel1, angVel1, pos2, vel2, angVel2, normal, contPt;
    double uN, r1, r2;
};

// closed-interval 3-axis overlap, InsertionSortCollider::spatialOverlap :52-58
__device__ __forceinline__ bool overlap3(const double4_32a& mn1, const double4_32a& mx1, const double4_32a& mn2, const double4_32a& mx2) {
    return (mn1.x <= mx2.x) && (mx1.x >= mn2.x) && (mn1.y <= mx2.y) && (mx1.y >= mn2.y) && (mn1.z <= mx2.z) && (mx1.z >= mn2.z);
}
// cellWrap / cellWrapRel, pkg/dem/InsertionSortCollider.cpp:650-660
// (rounded intrinsics: no contraction in the translation units compiled with --fmad=true)
__device__ __forceinline__ double cellWrapD(double x, double x0, double x1, int& period) {
    const double xNorm = __ddiv_rn(__dsub_rn(x, x0), __dsub_rn(x1, x0));
    period = (int)floor(xNorm);
    return __dadd_rn(x0, __dmul_rn(__dsub_rn(xNorm, (double)period), __dsub_rn(x1, x0)));
}
__device__ __forceinline__ double cellWrapRelD(double x, double x0, double x1) {
    const double xNorm = __ddiv_rn(__dsub_rn(x, x0), __dsub_rn(x1, x0));
    return __dmul_rn(__dsub_rn(xNorm, floor(xNorm)), __dsub_rn(x1, x0));
}
// InsertionSortCollider::spatialOverlapPeri, pkg/dem/InsertionSortCollider.cpp:903-957, for the
// pair (id1, id2); periods[] = pmn1 - pmn2 per axis. Returns 1 on overlap, 0 without, -1 when a
// box spans more than one period ("Particle larger than half of the cell size").
__device__ __forceinline__ int overlapPeri(const double4_32a& mn1, const double4_32a& mx1, const double4_32a& mn2,
                                          const double4_32a& mx2, const double* size, int periods[3]) {
    const double m1a[3] = {mn1.x, mn1.y, mn1.z}, x1a[3] = {mx1.x, mx1.y, mx1.z};
    const double m2a[3] = {mn2.x, mn2.y, mn2.z}, x2a[3] = {mx2.x, mx2.y, mx2.z};
    int res = 1;
    for (int axis = 0; axis < 3; axis++) {
        const double dim = size[axis];
        const double m1 = m1a[axis], m2 = m2a[axis];
        if (isinf(m1) || isinf(m2)) {
            periods[axis] = 0;
            continue;
        }
        const double wMn = (cellWrapRelD(m1, m2, m2 + dim) < cellWrapRelD(m2, m1, m1 + dim)) ? m2 : m1;
        int pmn1, pmx1, pmn2, pmx2;
        const double a1 = cellWrapD(m1, wMn, wMn + dim, pmn1), b1 = cellWrapD(x1a[axis], wMn, wMn + dim, pmx1);
        const double a2 = cellWrapD(m2, wMn, wMn + dim, pmn2), b2 = cellWrapD(x2a[axis], wMn, wMn + dim, pmx2);
        if ((pmn1 != pmx1) || (pmn2 != pmx2)) return -1;
        periods[axis] = pmn1 - pmn2;
        if (!(a1 <= b2 && b1 >= a2)) res = 0;
    }
    return res;
}
// ContactContainer::removePending (pkg/dem/ContactContainer.hpp:78-93 with
// InsertionSortCollider::shouldBeRemoved, InsertionSortCollider.hpp:209-214): a contact that the
// law removed in the last step leaves the container at the next collider run unless the boxes of
// its particles (those of the last full run) still overlap.
__device__ __forceinline__ bool pendingStays(const DevParticles& P, int A, int B, bool periodic, const double* cellSize, int* dErr) {
    const int lo = A < B ? A : B, hi = A < B ? B : A;
    if (!periodic) return overlap3(P.mn[lo], P.mx[lo], P.mn[hi], P.mx[hi]);
    int per[3];
    const int r = overlapPeri(P.mn[lo], P.mx[lo], P.mn[hi], P.mx[hi], cellSize, per);
    if (r < 0) atomicCAS(dErr, 0, 103);
    return r > 0;
}
// Cg2_Sphere_Sphere_L6Geom::go, pkg/dem/Sphere.cpp:88-109
__device__ __forceinline__ bool geomSS(const DevNodes& N, int A, int B, D3 shift2, bool real, double ssDf, Geo& g) {
    const double4_32a pa = N.posr[A], pb = N.posr[B];
    const double r1 = pa.w, r2 = pb.w;
    const D3 p1 = ld3(pa), p2 = ld3(pb);
    const D3 relPos = (p2 + shift2) - p1;
    const double dfr = fabs(ssDf) * (r1 + r2);
    const double unDistSq = sqn(relPos) - dfr * dfr;
    if (unDistSq > 0 && !real) return false;
    const double dist = sqrt(sqn(relPos));
    g.uN = dist - (r1 + r2);
    g.normal = relPos / dist;
    g.contPt = p1 + (r1 + 0.5 * g.uN) * g.normal;
    g.pos1 = p1;
    g.vel1 = ld3(N.vel[A]);
    g.angVel1 = ld3(N.angv[A]);
    g.pos2 = p2 + shift2;
    g.vel2 = ld3(N.vel[B]);
    g.angVel2 = ld3(N.angv[B]);
    g.r1 = r1;
    g.r2 = r2;
    return true;
}

// Cg2_Wall_Sphere_L6Geom::go, pkg/dem/Wall.cpp:45-79
// prevNormalAx: component `axis` of the previous contact normal (trsf column 0), used by
// sense==0 walls with an existing geometry.
__device__ __forceinline__ bool geomWS(const DevNodes& N, const DevParticles& P, double prevNormalAx, int A, int B, D3 shift2,
                                       bool real, Geo& g) {
    const int4 aux = P.aux[A];
    const int ax = aux.x, sense = aux.y;
    const double4_32a pw = N.posr[A], ps = N.posr[B];
    const double radius = ps.w;
    const D3 wallPos = ld3(pw);
    const D3 spherePos = ld3(ps) + shift2;
    const double dist = comp(spherePos, ax) - comp(wallPos, ax);
    if (!real && fabs(dist) > radius) return false;
    D3 contPt = spherePos;
    setComp(contPt, ax, comp(wallPos, ax));
    D3 normal{0, 0, 0};
    if (sense == 0) {
        if (!real) setComp(normal, ax, dist > 0 ? 1. : -1.);
        else setComp(normal, ax, prevNormalAx);
    } else setComp(normal, ax, sense == 1 ? 1. : -1);
    g.uN = comp(normal, ax) * dist - radius;
    g.normal = normal;
    g.contPt = contPt;
    g.pos1 = wallPos;
    g.vel1 = ld3(N.vel[A]);
    g.angVel1 = ld3(N.angv[A]);
    g.pos2 = spherePos;
    g.vel2 = ld3(N.vel[B]);
    g.angVel2 = ld3(N.angv[B]);
    g.r1 = -radius;
    g.r2 = radius;
    return true;
}

// CompUtils::closestSegmentPt, lib/base/CompUtils.cpp:57-63
__device__ __forceinline__ D3 closestSegmentPt(D3 P, D3 A, D3 B) {
    const D3 BA = B - A;
    if (sqn(BA) == 0.) return A;
    const double u = (dot(P, BA) - dot(A, BA)) / sqn(BA);
    return A + smin(1., smax(0., u)) * BA;
}

// Cg2_Facet_Sphere_L6Geom::go, pkg/dem/Facet.cpp:235-288 with Facet::interpolatePtLinAngVel :158-174
// and CompUtils::triangleBarycentrics lib/base/CompUtils.cpp:92-110
__device__ __forceinline__ bool geomFS(const DevNodes& N, const DevParticles& P, int A, int B, D3 shift2, bool real, Geo& g,
                                       int* dErr) {
    const int4 fn = P.aux[A];
    const double4_32a fd = P.facet[A];
    const double halfThick = fd.w;
    const D3 fakeVel{fd.x, fd.y, fd.z};
    const double4_32a ps = N.posr[B];
    const double radius = ps.w;
    const D3 sC = ld3(ps) + shift2;
    const D3 p0 = ld3(N.posr[fn.x]), p1 = ld3(N.posr[fn.y]), p2 = ld3(N.posr[fn.z]);
    const D3 nn = cross(p1 - p0, p2 - p0);
    const D3 fNormal = normalized(nn);
    const double planeDist = dot(sC - p0, fNormal);
    if (fabs(planeDist) > (radius + halfThick) && !real) return false;
    const D3 fC = sC - planeDist * fNormal;
    const double l0 = dot(cross(p1 - p0, nn), fC - p0);
    const double l1 = dot(cross(p2 - p1, nn), fC - p1);
    const double l2 = dot(cross(p0 - p2, nn), fC - p2);
    const int w = (l0 > 0 ? 1 : 0) + (l1 > 0 ? 2 : 0) + (l2 > 0 ? 4 : 0);
    D3 contPt;
    switch (w) {
        case 0: contPt = fC; break;
        case 1: contPt = closestSegmentPt(fC, p0, p1); break;
        case 2: contPt = closestSegmentPt(fC, p1, p2); break;
        case 4: contPt = closestSegmentPt(fC, p2, p0); break;
        case 3: contPt = p1; break;
        case 5: contPt = p0; break;
        case 6: contPt = p2; break;
        default: atomicCAS(dErr, 0, 100); return false;  // "Impossible sphere-facet intersection"
    }
    D3 normal = sC - contPt;
    const double rh = radius + halfThick;
    if (sqn(normal) > rh * rh && !real) return false;
    const double dist = sqrt(sqn(normal));
    normal = normal / dist;
    if (halfThick > 0) contPt = contPt + normal * halfThick;
    g.uN = (dist - radius) - halfThick;
    // barycentric interpolation of the facet node velocities at contPt
    const D3 vB = p1 - p0, vC = p2 - p0, vX = contPt - p0;
    const double m00 = dot(vB, vB), m01 = dot(vC, vB), m10 = dot(vB, vC), m11 = dot(vC, vC);
    const double det = m00 * m11 - m10 * m01;
    const double invdet = 1. / det;
    const double i00 = m11 * invdet, i10 = -m10 * invdet, i01 = -m01 * invdet, i11 = m00 * invdet;
    const double b0 = dot(vX, vB), b1 = dot(vX, vC);
    const double u = i00 * b0 + i01 * b1, v = i10 * b0 + i11 * b1;
    const double a0 = (1 - u) - v;
    const D3 v0 = ld3(N.vel[fn.x]), v1 = ld3(N.vel[fn.y]), v2 = ld3(N.vel[fn.z]);
    D3 linVel = (a0 * v0 + u * v1) + v * v2;
    const D3 angVel = (cross(p0 - contPt, v0) + cross(p1 - contPt, v1)) + cross(p2 - contPt, v2);
    if (!isZero(fakeVel)) {
        if (!isnan(fakeVel.x)) linVel = linVel + fakeVel;
        else linVel = dot(linVel, fNormal) * fNormal;
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


}  // namespace wg
