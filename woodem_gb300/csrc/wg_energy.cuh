// Energy terms of Leapfrog (Scene.trackEnergy, pkg/dem/Leapfrog.cpp:52-97), shared by the FP64
// and the FP32-force Leapfrog kernels. Out of line: their FP64 arithmetic runs only in the energy
// variants of those kernels.
#pragma once
#include "wg_internal.h"
#include "wg_math.cuh"

namespace wg {

// Leapfrog::doDampingDissipation (Leapfrog.cpp:52-63): |v|.|F|*damping*dt + |w|.|T|*damping*dt
// with the velocities of the previous half step and this step's force and torque.
static __device__ __noinline__ double energyDamp(D3 v, D3 f, D3 w, D3 t, double damping, double dt) {
    const double a = (fabs(v.x) * fabs(f.x) + fabs(v.y) * fabs(f.y)) + fabs(v.z) * fabs(f.z);
    const double b = (fabs(w.x) * fabs(t.x) + fabs(w.y) * fabs(t.y)) + fabs(w.z) * fabs(t.z);
    return ((a * damping) * dt) + ((b * damping) * dt);
}
// Leapfrog::doGravityWork (Leapfrog.cpp:66-73): -g.v*m*dt over the free translations.
static __device__ __noinline__ double energyGrav(D3 g, D3 v, double mass, double dt, uint32_t flags) {
    if ((flags & F_DOF_ALL) == 0) return ((-dot(g, v)) * mass) * dt;
    double gr = 0;
    if (!(flags & 1u)) gr = gr - ((g.x * v.x) * mass) * dt;
    if (!(flags & 2u)) gr = gr - ((g.y * v.y) * mass) * dt;
    if (!(flags & 4u)) gr = gr - ((g.z * v.z) * mass) * dt;
    return gr;
}
// Leapfrog::doKineticEnergy (Leapfrog.cpp:75-97), spherical nodes: on-step fluctuation
// velocities v + dt/2 a; returns (Etrans, Erot).
static __device__ __noinline__ double2 energyKin(D3 pvf, D3 pva, D3 la, D3 aa, double mass, D3 inertia, double dt) {
    const D3 cv = pvf + (.5 * dt) * la, cw = pva + (.5 * dt) * aa;
    const double et = (.5 * mass) * sqn(cv);
    double er = 0.5 * ((cw.x * (inertia.x * cw.x) + cw.y * (inertia.y * cw.y)) + cw.z * (inertia.z * cw.z));
    const double imax = smax(smax(inertia.x, inertia.y), inertia.z);
    if (isnan(er) || isinf(imax)) er = 0;
    return make_double2(et, er);
}
}  // namespace wg
