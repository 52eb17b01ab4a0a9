// Host side of the GB300 DEM hot path: scene upload, the per-step loop of
// Scene::doOneStep (core/Scene.cpp:319-389) for the engine list
// [Leapfrog(reset=True), InsertionSortCollider, ContactLoop], and the C ABI of include/woo_gpu.h.
#include <cuda_profiler_api.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "wg_internal.h"
#include "wg_math.cuh"

namespace wg {
// Scene.nextDt of a configuration: a positive finite value (0 and NaN: none)
static double validNextDt(const wg_config& c) {
    return (c.next_dt > 0 && std::isfinite(c.next_dt)) ? c.next_dt : std::numeric_limits<double>::quiet_NaN();
}
}  // namespace wg
namespace wg {

void collide_free(Sim& S);

static thread_local std::string g_createError;

void* Sim::dalloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    allocs.push_back(p);
    return p;
}
void Sim::dfree(void* p) {
    if (!p) return;
    auto it = std::find(allocs.begin(), allocs.end(), p);
    if (it != allocs.end()) allocs.erase(it);
    cudaFree(p);
}
Sim::~Sim() {
    if (stream) cudaStreamSynchronize(stream);
    collide_free(*this);
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (hFlags) cudaFreeHost(hFlags);
    for (int i = 0; i < 8; i++)
        if (ev[i]) cudaEventDestroy(ev[i]);
    for (cudaEvent_t e : evPool) cudaEventDestroy(e);
    if (graphExec) cudaGraphExecDestroy(graphExec);
    if (side.st) cudaStreamSynchronize(side.st);
    if (side.fork) cudaEventDestroy(side.fork);
    if (side.join) cudaEventDestroy(side.join);
    if (side.st) cudaStreamDestroy(side.st);
    if (earlySt) {
        cudaStreamSynchronize(earlySt);
        cudaStreamDestroy(earlySt);
    }
    if (earlyFork) cudaEventDestroy(earlyFork);
    if (stream) cudaStreamDestroy(stream);
}

// ------------------------------------------------------------------ periodic cell (host)
// Cell::integrateAndUpdate / setNextGradV, core/Cell.cpp:60-120, with 3x3 algebra in the same
// operation order as the oracle so that the matrices handed to the kernels agree bitwise.
struct HM {
    double m[3][3];
};
static HM hI() { HM r{}; r.m[0][0] = r.m[1][1] = r.m[2][2] = 1; return r; }
static bool isIdentity(const HM& a) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (a.m[i][j] != (i == j ? 1. : 0.)) return false;
    return true;
}
static HM hmul(const HM& A, const HM& B) {
    HM r{};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = (A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j]) + A.m[i][2] * B.m[2][j];
    return r;
}
static HM hadd(const HM& A, const HM& B) { HM r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] + B.m[i][j]; return r; }
static HM hsub(const HM& A, const HM& B) { HM r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] - B.m[i][j]; return r; }
static HM hscale(const HM& A, double s) { HM r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] * s; return r; }
static HM hdiv(const HM& A, double s) { HM r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] / s; return r; }
static HM htr(const HM& A) { HM r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[j][i]; return r; }
static double hcof(const HM& a, int i, int j) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    return a.m[i1][j1] * a.m[i2][j2] - a.m[i1][j2] * a.m[i2][j1];
}
static HM hinv(const HM& a) {
    double c00 = hcof(a, 0, 0), c10 = hcof(a, 1, 0), c20 = hcof(a, 2, 0);
    double det = (c00 * a.m[0][0] + c10 * a.m[1][0]) + c20 * a.m[2][0];
    double invdet = 1.0 / det;
    HM r;
    r.m[0][0] = c00 * invdet; r.m[0][1] = c10 * invdet; r.m[0][2] = c20 * invdet;
    r.m[1][0] = hcof(a, 0, 1) * invdet; r.m[1][1] = hcof(a, 1, 1) * invdet; r.m[1][2] = hcof(a, 2, 1) * invdet;
    r.m[2][0] = hcof(a, 0, 2) * invdet; r.m[2][1] = hcof(a, 1, 2) * invdet; r.m[2][2] = hcof(a, 2, 2) * invdet;
    return r;
}
static double hdet(const HM& a) {
    return (a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) - a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0])) +
           a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}
static void hlevi(const HM& m, double out[3]) { out[0] = m.m[1][2] - m.m[2][1]; out[1] = m.m[2][0] - m.m[0][2]; out[2] = m.m[0][1] - m.m[1][0]; }
static HM fromRow(const double* a) { HM r; for (int i = 0; i < 9; i++) r.m[i / 3][i % 3] = a[i]; return r; }
static void toRow(const HM& m, double* a) { for (int i = 0; i < 9; i++) a[i] = m.m[i / 3][i % 3]; }

struct HostCell {
    HM trsf, hSize, pprevHsize, gradV, nextGradV;
    double spinVec[3] = {0, 0, 0};
    int homoDeform = 4;
    HM invTrsf, shearTrsf, unshearTrsf;
    double size[3], cosv[3];
    bool hasShear = false;
    void integrateAndUpdate(double dt) {
        HM trsfInc = hscale(gradV, dt);
        trsf = hadd(trsf, hmul(trsfInc, trsf));
        invTrsf = hinv(trsf);
        HM prevHsize = hSize;
        if (homoDeform == 4) {
            HM a = hinv(hsub(hI(), hdiv(hscale(gradV, dt), 2.)));
            HM b = hadd(hI(), hdiv(hscale(gradV, dt), 2.));
            hSize = hmul(hmul(a, b), hSize);
        } else hSize = hadd(hSize, hmul(trsfInc, hSize));
        pprevHsize = hscale(hadd(prevHsize, hSize), .5);
        HM Hnorm;
        for (int i = 0; i < 3; i++) {
            D3 base{hSize.m[0][i], hSize.m[1][i], hSize.m[2][i]};
            size[i] = std::sqrt(sqn(base));
            base = base / size[i];
            Hnorm.m[0][i] = base.x; Hnorm.m[1][i] = base.y; Hnorm.m[2][i] = base.z;
        }
        for (int i = 0; i < 3; i++) {
            int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            cosv[i] = sqn(cross(D3{Hnorm.m[0][i1], Hnorm.m[1][i1], Hnorm.m[2][i1]}, D3{Hnorm.m[0][i2], Hnorm.m[1][i2], Hnorm.m[2][i2]}));
        }
        shearTrsf = Hnorm;
        unshearTrsf = hinv(shearTrsf);
        hasShear = (hSize.m[0][1] != 0 || hSize.m[0][2] != 0 || hSize.m[1][0] != 0 || hSize.m[1][2] != 0 || hSize.m[2][0] != 0 ||
                    hSize.m[2][1] != 0);
    }
    void setNextGradV() {
        gradV = nextGradV;
        HM W = hscale(hsub(gradV, htr(gradV)), .5);
        double lv[3];
        hlevi(W, lv);
        for (int i = 0; i < 3; i++) spinVec[i] = .5 * lv[i];
    }
};

struct SimEx : Sim {
    HostCell cell;
    // api <-> slot staging for state transfer
    int32_t* dApiMap = nullptr;   // api node -> slot (-1: not used by any particle)
    double* dStage = nullptr;     // 19 doubles per api node
    std::vector<double> hApiStage; // last uploaded api state (for unmapped nodes)
    std::vector<int32_t> hApiMap;
};

// The six per-node arrays of wg_put_state / wg_get_nodes in the device staging buffer (pos 3,
// ori 4, vel 3, angVel 3, force 3, torque 3 doubles per API node).
struct StateArrays {
    double *pos, *ori, *vel, *av, *f, *t;
};
__host__ __device__ inline StateArrays stagedArrays(double* st, int64_t na) {
    return StateArrays{st, st + 3 * na, st + 7 * na, st + 10 * na, st + 13 * na, st + 16 * na};
}
__global__ void k_put_state(DevNodes N, const int32_t* __restrict__ map, int64_t na, StateArrays A) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= na) return;
    const int s = map[a];
    if (s < 0) return;
    const double* pos = A.pos;
    const double* ori = A.ori;
    const double* vel = A.vel;
    const double* av = A.av;
    const double* f = A.f;
    const double* t = A.t;
    const double r = N.posr[s].w;
    N.posr[s] = make_double4_32a(pos[3 * a], pos[3 * a + 1], pos[3 * a + 2], r);
    N.ori[s] = make_double4_32a(ori[4 * a], ori[4 * a + 1], ori[4 * a + 2], ori[4 * a + 3]);
    if (N.orif) N.orif[s] = make_float4((float)ori[4 * a], (float)ori[4 * a + 1], (float)ori[4 * a + 2], (float)ori[4 * a + 3]);
    if (N.mir) {
        // the double-float mirrors of the FP32-force mode follow the written state
        auto split = [](double x, float& h, float& l) {
            h = __double2float_rn(x);
            l = __double2float_rn(x - (double)h);
        };
        float4 h, l;
        const float2 rs = N.rsplit[s];
        split(pos[3 * a], h.x, l.x);
        split(pos[3 * a + 1], h.y, l.y);
        split(pos[3 * a + 2], h.z, l.z);
        h.w = rs.x;
        l.w = rs.y;
        Mirror m;
        m.ph = h;
        m.pl = l;
        split(vel[3 * a], h.x, l.x);
        split(vel[3 * a + 1], h.y, l.y);
        split(vel[3 * a + 2], h.z, l.z);
        h.w = (float)av[3 * a];
        l.w = (float)av[3 * a + 1];
        m.vh = h;
        m.vl = l;
        N.mir[s] = m;
        N.wz[s] = (float)av[3 * a + 2];
    }
    N.vel[s] = make_double4_32a(vel[3 * a], vel[3 * a + 1], vel[3 * a + 2], 0.);
    N.angv[s] = make_double4_32a(av[3 * a], av[3 * a + 1], av[3 * a + 2], 0.);
    N.force[s] = make_double4_32a(f[3 * a], f[3 * a + 1], f[3 * a + 2], 0.);
    N.torque[s] = make_double4_32a(t[3 * a], t[3 * a + 1], t[3 * a + 2], 0.);
}
// part 0: the whole state; 1: position, orientation, velocity, angular velocity; 2: force, torque
__global__ void k_get_state(DevNodes N, const int32_t* __restrict__ map, int64_t na, StateArrays A, int part = 0) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= na) return;
    const int s = map[a];
    if (s < 0) return;
    if (part != 2) {
        double* pos = A.pos;
        double* ori = A.ori;
        double* vel = A.vel;
        double* av = A.av;
        const double4_32a p = N.posr[s], v = N.vel[s], w = N.angv[s];
        double4_32a o;
        if (N.orif) {
            const float4 q = N.orif[s];
            o = make_double4_32a(q.x, q.y, q.z, q.w);
        } else o = N.ori[s];
        pos[3 * a] = p.x; pos[3 * a + 1] = p.y; pos[3 * a + 2] = p.z;
        ori[4 * a] = o.x; ori[4 * a + 1] = o.y; ori[4 * a + 2] = o.z; ori[4 * a + 3] = o.w;
        vel[3 * a] = v.x; vel[3 * a + 1] = v.y; vel[3 * a + 2] = v.z;
        av[3 * a] = w.x; av[3 * a + 1] = w.y; av[3 * a + 2] = w.z;
    }
    if (part != 1) {
        double* f = A.f;
        double* t = A.t;
        const double4_32a ff = N.force[s], tt = N.torque[s];
        f[3 * a] = ff.x; f[3 * a + 1] = ff.y; f[3 * a + 2] = ff.z;
        t[3 * a] = tt.x; t[3 * a + 1] = tt.y; t[3 * a + 2] = tt.z;
    }
}

// Copies between the staging buffer (pos 3, ori 4, vel 3, angVel 3, force 3, torque 3 doubles
// per API node, array after array) and the caller's arrays q0..q1-1: arrays that follow each
// other in host memory as they do in the staging buffer go as one copy. Null arrays are skipped.
static cudaError_t copyState(double* stage, int64_t na, double* const host[6], int q0, int q1, bool toDevice, cudaStream_t st) {
    const int64_t off[6] = {0, 3, 7, 10, 13, 16}, w[6] = {3, 4, 3, 3, 3, 3};
    for (int q = q0; q < q1;) {
        if (!host[q]) {
            q++;
            continue;
        }
        int e = q + 1;
        while (e < q1 && host[e] && host[e] == host[e - 1] + w[e - 1] * na) e++;
        const size_t bytes = sizeof(double) * (size_t)(off[e - 1] + w[e - 1] - off[q]) * (size_t)na;
        const cudaError_t r = toDevice ? cudaMemcpyAsync(stage + off[q] * na, host[q], bytes, cudaMemcpyHostToDevice, st)
                                       : cudaMemcpyAsync(host[q], stage + off[q] * na, bytes, cudaMemcpyDeviceToHost, st);
        if (r != cudaSuccess) return r;
        q = e;
    }
    return cudaSuccess;
}

// The early part of wg_run_host's copy-out (see Sim::earlyOut), issued right after the run's
// last Leapfrog is queued: the early stream waits for it, converts the kinematic state into the
// staging buffer and copies it to the caller's arrays. The contact loop that follows reads that
// state and writes none of it.
int Sim::issueEarlyGet() {
    Sim& S = *this;
    SimEx& X = static_cast<SimEx&>(*this);
    if (!earlySt) {
        WG_CUDA_TRY(cudaStreamCreateWithFlags(&earlySt, cudaStreamNonBlocking));
        WG_CUDA_TRY(cudaEventCreateWithFlags(&earlyFork, cudaEventDisableTiming));
    }
    const int64_t na = nApiNodes;
    WG_CUDA_TRY(cudaEventRecord(earlyFork, stream));
    WG_CUDA_TRY(cudaStreamWaitEvent(earlySt, earlyFork, 0));
    k_get_state<<<(unsigned)((na + 255) / 256), 256, 0, earlySt>>>(N, X.dApiMap, na, stagedArrays(X.dStage, na), 1);
    double* const host[6] = {earlyOut[0], earlyOut[1], earlyOut[2], earlyOut[3], nullptr, nullptr};
    WG_CUDA_TRY(copyState(X.dStage, na, host, 0, 4, false, earlySt));
    earlyIssued = true;
    return 0;
}

int Sim::ensureContactCapacity(int64_t need) {
    Sim& S = *this;
    if (need <= cCap && C.key) return 0;
    int64_t cap = std::max<int64_t>(need + need / 2, std::max<int64_t>(1024, 2 * cCap));
    DevContacts nc{}, nb{};
    // FP64 plain: every FP64 column. FP32-force: the FP32 columns plus the FP64 shear force
    // (IdealElPl) and contact point (facet and wall contacts).
    auto needD = [&](int q) { return prec == WG_PREC_FP64 || q == CC_FT1 || q == CC_FT2 || q == CC_CPX || q == CC_CPY || q == CC_CPZ; };
    for (DevContacts* d : {&nc, &nb}) {
        d->key = (uint64_t*)dalloc(sizeof(uint64_t) * cap);
        d->flags = (uint32_t*)dalloc(sizeof(uint32_t) * cap);
        d->step0 = (int32_t*)dalloc(sizeof(int32_t) * cap);
        d->cdist = (int32_t*)dalloc(sizeof(int32_t) * cap);
        if (!d->cdist) return fail(WG_ERR_CUDA, "out of device memory (contacts)");
        for (int q = 0; q < CC_NCOL; q++) {
            d->col[q] = needD(q) ? (double*)dalloc(sizeof(double) * cap) : nullptr;
            if (needD(q) && !d->col[q]) return fail(WG_ERR_CUDA, "out of device memory (contacts)");
        }
        for (int q = 0; q < CF_NCOL; q++) {
            d->fcol[q] = (prec == WG_PREC_FP32) ? (float*)dalloc(sizeof(float) * cap) : nullptr;
            if (prec == WG_PREC_FP32 && !d->fcol[q]) return fail(WG_ERR_CUDA, "out of device memory (contacts)");
        }
    }
    if (C.key && C.n > 0) {
        WG_CUDA_TRY(cudaMemcpyAsync(nc.key, C.key, sizeof(uint64_t) * C.n, cudaMemcpyDeviceToDevice, stream));
        WG_CUDA_TRY(cudaMemcpyAsync(nc.flags, C.flags, sizeof(uint32_t) * C.n, cudaMemcpyDeviceToDevice, stream));
        WG_CUDA_TRY(cudaMemcpyAsync(nc.step0, C.step0, sizeof(int32_t) * C.n, cudaMemcpyDeviceToDevice, stream));
        WG_CUDA_TRY(cudaMemcpyAsync(nc.cdist, C.cdist, sizeof(int32_t) * C.n, cudaMemcpyDeviceToDevice, stream));
        for (int q = 0; q < CC_NCOL; q++)
            if (nc.col[q]) WG_CUDA_TRY(cudaMemcpyAsync(nc.col[q], C.col[q], sizeof(double) * C.n, cudaMemcpyDeviceToDevice, stream));
        for (int q = 0; q < CF_NCOL; q++)
            if (nc.fcol[q]) WG_CUDA_TRY(cudaMemcpyAsync(nc.fcol[q], C.fcol[q], sizeof(float) * C.n, cudaMemcpyDeviceToDevice, stream));
    }
    WG_CUDA_TRY(cudaStreamSynchronize(stream));
    nc.n = C.n;
    for (DevContacts* d : {&C, &Cb}) {
        if (!d->key) continue;
        dfree(d->key); dfree(d->flags); dfree(d->step0); dfree(d->cdist);
        for (int q = 0; q < CC_NCOL; q++) dfree(d->col[q]);
        for (int q = 0; q < CF_NCOL; q++) dfree(d->fcol[q]);
    }
    C = nc;
    Cb = nb;
    cCap = cap;
    return 0;
}

int Sim::prepareParams() {
    if (nScenes <= 1) {
        // a single scene is also a batch of one (serving slots address it as scene 0)
        int r = prepareParamsFor(cfg, 0, nPar, hPar);
        hPars.assign(1, hPar);
        cfgs.assign(1, cfg);
        sceneStart = {0, nPar};
        sceneTime0.assign(1, 0.0);
        return r;
    }
    hPars.resize(nScenes);
    for (int k = 0; k < nScenes; k++) prepareParamsFor(cfgs[k], sceneStart[k], sceneStart[k + 1], hPars[k]);
    hPar = hPars[0];
    return 0;
}

// ScenePar of one scene (configuration cfg, particles [p0, p1))
int Sim::prepareParamsFor(const wg_config& cfg, int64_t p0, int64_t p1, ScenePar& p) {
    Sim& S = *this;
    SimEx& X = static_cast<SimEx&>(*this);
    std::memset(&p, 0, sizeof(p));
    p.stepBase = 0;
    p.stepEnd = (long long)1 << 62;
    p.dt = cfg.dt;
    p.trackEnergy = cfg.track_energy != 0;
    p.kinSplit = cfg.kin_split != 0;
    for (int i = 0; i < 3; i++) p.g[i] = cfg.gravity[i];
    p.hasGravity = (cfg.gravity[0] != 0 || cfg.gravity[1] != 0 || cfg.gravity[2] != 0);
    p.damping = cfg.damping;
    p.ssDistFactor = cfg.cg2_ss_dist_factor;
    p.dtF = (float)cfg.dt;
    p.ssDfAbsF = (float)std::fabs(cfg.cg2_ss_dist_factor);
    p.dampingF = (float)cfg.damping;
    for (int i = 0; i < 3; i++) {
        p.gH[i] = (float)cfg.gravity[i];
        p.gL[i] = (float)(cfg.gravity[i] - (double)p.gH[i]);
    }
    p.bo1DistFactor = cfg.bo1_sphere_dist_factor;
    p.law = cfg.law;
    p.phys = cfg.phys;
    p.reset = cfg.reset;
    p.applyForces = cfg.apply_forces;
    p.trsfRenorm = cfg.trsf_renorm;
    p.approxMask = cfg.approx_mask;
    p.noRatch = cfg.no_ratch;
    p.noSlip = cfg.no_slip;
    p.noBreak = cfg.no_break;
    p.noFrict = cfg.no_frict;
    p.noAttraction = cfg.hz_no_attraction;
    p.hzGamma = cfg.hz_gamma;
    p.hzPoisson = cfg.hz_poisson;
    p.hzViscOn = (cfg.hz_en > 0 && cfg.hz_en < 1.);
    if (p.hzViscOn) {
        // Cp2_FrictMat_HertzPhys::go, pkg/dem/Hertz.cpp:43 (constant per functor)
        const double PI = 3.14159265358979323846;
        double sqrt5 = std::sqrt(5.);
        double le = std::log(cfg.hz_en);
        p.hzViscConst = -sqrt5 * le / (std::sqrt(le * le + PI * PI));
    }
    p.periodic = cfg.periodic;
    p.homoDeform = cfg.homo_deform;
    p.evalStress = cfg.eval_stress;
    p.loneMask = cfg.lone_mask;
    // InsertionSortCollider.verletDist < 0: |verletDist| * min sphere radius
    // (InsertionSortCollider.cpp:290-298)
    double vd = cfg.verlet_dist;
    if (vd < 0) {
        double minR = std::numeric_limits<double>::infinity();
        // radius of spheres is in posr.w; read back from the host description
        for (int64_t i = p0; i < p1; i++)
            if (hShape[i] == WG_SHAPE_SPHERE) minR = std::min(minR, hRadius[i]);
        vd = std::isinf(minR) ? 0 : std::abs(vd) * minR;
    }
    p.verletDist = vd;
    p.maxD2 = vd * vd;
    // FP32 verlet test: a hair below maxD2 so that rounding can only trigger a full run early
    p.maxD2F = (float)(p.maxD2 * (1 - 1e-6));
    p.reach2F = (float)(2 * p.verletDist);
    (void)X;
    (void)S;
    return 0;
}

static void fillCellPar(SimEx& X) {
    ScenePar& p = X.hPar;
    HostCell& c = X.cell;
    toRow(c.hSize, p.hSize);
    toRow(c.pprevHsize, p.pprevHsize);
    toRow(c.gradV, p.gradV);
    toRow(c.nextGradV, p.nextGradV);
    toRow(hsub(c.nextGradV, c.gradV), p.dGradV);
    toRow(hscale(hadd(c.gradV, c.nextGradV), .5), p.midGradV);
    // Cell::intrShiftVel, core/Cell.cpp:28-34
    if (c.homoDeform == 4) toRow(hmul(c.gradV, c.pprevHsize), p.shiftVelMat);
    else if (c.homoDeform == 2 || c.homoDeform == 3) toRow(hmul(c.gradV, c.hSize), p.shiftVelMat);
    else toRow(HM{}, p.shiftVelMat);
    toRow(c.unshearTrsf, p.unshear);
    for (int i = 0; i < 3; i++) { p.cellSize[i] = c.size[i]; p.spinVec[i] = c.spinVec[i]; }
    p.hasShear = c.hasShear;
    // Leapfrog::run, pkg/dem/Leapfrog.cpp:118-126
    const double dt = X.cfg.dt;
    const HM& pprevL = c.gradV;
    const HM& nnextL = c.nextGradV;
    HM q = hdiv(hscale(hadd(nnextL, pprevL), dt), 4.);
    toRow(hinv(hsub(hI(), q)), p.ImLL4hInv);
    toRow(hadd(hI(), q), p.IpLL4h);
    toRow(hsub(nnextL, pprevL), p.LmL);
    double a[3], b[3];
    hlevi(hscale(hsub(pprevL, htr(pprevL)), .5), a);
    hlevi(hscale(hsub(nnextL, htr(nnextL)), .5), b);
    for (int i = 0; i < 3; i++) p.deltaSpinVec[i] = -.5 * a[i] + .5 * b[i];
    // skew cosines for Cell::shearAlignedExtents (core/Cell.cpp:68-78)
    for (int i = 0; i < 3; i++) p.cellCos[i] = c.cosv[i];
}

int Sim::upload() {
    Sim& S = *this;
    SimEx& X = static_cast<SimEx&>(*this);
    if (!haveCfg) return fail(WG_ERR_STATE, "wg_set_config must be called before running");
    if (nPar == 0) return fail(WG_ERR_STATE, "no particles");
    if (nScenes > 1 && (int64_t)sceneStart.size() == nScenes + 1 && sceneStart[nScenes] != nPar)
        return fail(WG_ERR_ARG, "the scenes of the batch do not cover the particles");
    for (int k = 0; k < nScenes; k++) {
        const wg_config& c = nScenes > 1 ? cfgs[k] : cfg;
        if (!c.reset) return fail(WG_ERR_UNSUPPORTED, "Leapfrog.reset=False: the GPU path integrates the engine list [Leapfrog(reset=True), InsertionSortCollider, ContactLoop]");
        if (!((c.phys == 0 && c.law == 0) || (c.phys == 1 && c.law == 1)))
            return fail(WG_ERR_UNSUPPORTED, "unsupported Cp2/Law2 combination (FrictPhys+IdealElPl or HertzPhys+HertzPhys_DMT)");
        if (c.law == 1 && c.hz_alpha != 0) return fail(WG_ERR_UNSUPPORTED, "Law2_L6Geom_HertzPhys_DMT with Cp2_FrictMat_HertzPhys.alpha!=0 (Schwarz model) is not supported");
        if (c.precision != WG_PREC_FP64 && c.precision != WG_PREC_FP32) return fail(WG_ERR_ARG, "unknown precision mode");
        if (c.precision != cfg.precision) return fail(WG_ERR_UNSUPPORTED, "the scenes of a batch share one precision mode");
        if (c.precision == WG_PREC_FP32 && c.law == 1 && c.hz_gamma != 0)
            return fail(WG_ERR_UNSUPPORTED, "FP32-force mode: Cp2_FrictMat_HertzPhys.gamma (DMT adhesion) must be 0; use precision fp64");
        if (nScenes > 1 && c.periodic) return fail(WG_ERR_UNSUPPORTED, "periodic scenes run one per simulation, not in a batch");
        if (nScenes > 1 && (c.lone_mask != cfg.lone_mask || c.apply_forces != cfg.apply_forces))
            return fail(WG_ERR_UNSUPPORTED, "the scenes of a batch share loneMask and ContactLoop.applyForces");
    }
    prec = cfg.precision;
    if (cfg.periodic)
        for (int64_t i = 0; i < nPar; i++)
            if (hShape[i] == WG_SHAPE_FACET)
                return fail(WG_ERR_UNSUPPORTED, "facets in a periodic cell are outside the GPU path");
    for (int64_t i = 0; i < nPar; i++) {
        if (hMat[i] < 0 || hMat[i] >= (int)hDensity.size()) return fail(WG_ERR_ARG, "particle material index out of range");
    }
    // node slots
    std::vector<int32_t> map(nApiNodes, -1);
    int64_t nExtra = 0;
    for (int64_t p = 0; p < nPar; p++) {
        const int sh = hShape[p];
        if (sh == WG_SHAPE_SPHERE || sh == WG_SHAPE_WALL) {
            int32_t a = hNodes3[3 * p];
            if (a < 0 || a >= nApiNodes) return fail(WG_ERR_ARG, "particle node index out of range");
            if (map[a] >= 0) return fail(WG_ERR_UNSUPPORTED, "a node shared between particles (clumps, meshes with spheres) is outside the GPU path");
            map[a] = (int32_t)p;
        }
    }
    for (int64_t p = 0; p < nPar; p++) {
        if (hShape[p] != WG_SHAPE_FACET) continue;
        for (int k = 0; k < 3; k++) {
            int32_t a = hNodes3[3 * p + k];
            if (a < 0 || a >= nApiNodes) return fail(WG_ERR_ARG, "facet node index out of range");
            if (map[a] >= 0 && map[a] < nPar) return fail(WG_ERR_UNSUPPORTED, "facet shares a node with a sphere or wall");
            if (map[a] < 0) map[a] = (int32_t)(nPar + nExtra++);
        }
    }
    const int64_t nSlots = nPar + nExtra;
    std::vector<double4_32a> posr(nSlots), vel(nSlots), angv(nSlots), ori(nSlots), force(nSlots), torque(nSlots), minert(nSlots);
    std::vector<uint32_t> flags(nSlots, F_DOF_ALL);
    for (int64_t s = 0; s < nSlots; s++) {
        posr[s] = vel[s] = angv[s] = force[s] = torque[s] = minert[s] = make_double4_32a(0, 0, 0, 0);
        ori[s] = make_double4_32a(1, 0, 0, 0);
    }
    const double* st = hApi.data();
    const int64_t na = nApiNodes;
    for (int64_t a = 0; a < na; a++) {
        int32_t s = map[a];
        if (s < 0) continue;
        posr[s] = make_double4_32a(st[3 * a], st[3 * a + 1], st[3 * a + 2], 0.);
        ori[s] = make_double4_32a(st[3 * na + 4 * a], st[3 * na + 4 * a + 1], st[3 * na + 4 * a + 2], st[3 * na + 4 * a + 3]);
        vel[s] = make_double4_32a(st[7 * na + 3 * a], st[7 * na + 3 * a + 1], st[7 * na + 3 * a + 2], 0);
        angv[s] = make_double4_32a(st[10 * na + 3 * a], st[10 * na + 3 * a + 1], st[10 * na + 3 * a + 2], 0);
        force[s] = make_double4_32a(st[13 * na + 3 * a], st[13 * na + 3 * a + 1], st[13 * na + 3 * a + 2], 0);
        torque[s] = make_double4_32a(st[16 * na + 3 * a], st[16 * na + 3 * a + 1], st[16 * na + 3 * a + 2], 0);
        minert[s] = make_double4_32a(hInertia[3 * a], hInertia[3 * a + 1], hInertia[3 * a + 2], hMass[a]);
        flags[s] = hFlagsApi[a];
    }
    std::vector<int32_t> shape(nPar), mat(nPar);
    std::vector<int4> aux(nPar);
    std::vector<double4_32a> facet(nPar);
    std::vector<uint32_t> mask(nPar);
    nSpheres = 0;
    std::vector<int32_t> facetIds;
    for (int64_t p = 0; p < nPar; p++) {
        shape[p] = hShape[p];
        mat[p] = hMat[p];
        mask[p] = hMask[p];
        aux[p] = make_int4(0, 0, 0, 0);
        facet[p] = make_double4_32a(0, 0, 0, 0);
        if (hShape[p] == WG_SHAPE_SPHERE) {
            posr[p].w = hRadius[p];
            nSpheres++;
        } else if (hShape[p] == WG_SHAPE_WALL) {
            if (hAxis[p] < 0 || hAxis[p] > 2) return fail(WG_ERR_ARG, "Wall.axis must be 0, 1 or 2");
            aux[p] = make_int4(hAxis[p], hSense[p], 0, 0);
        } else if (hShape[p] == WG_SHAPE_FACET) {
            aux[p] = make_int4(map[hNodes3[3 * p]], map[hNodes3[3 * p + 1]], map[hNodes3[3 * p + 2]], (int)facetIds.size());
            facetIds.push_back((int32_t)p);
            facet[p] = make_double4_32a(hFakeVel[3 * p], hFakeVel[3 * p + 1], hFakeVel[3 * p + 2], hHalfThick[p]);
        } else return fail(WG_ERR_UNSUPPORTED, "unknown shape code");
    }
    WG_CUDA_TRY(cudaSetDevice(device));
    N.n = (int32_t)nSlots;
    N.posr = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.vel = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.angv = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.ori = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.force = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.torque = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.minert = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.lastPos = (double4_32a*)dalloc(sizeof(double4_32a) * nSlots);
    N.flags = (uint32_t*)dalloc(sizeof(uint32_t) * nSlots);
    P.n = (int32_t)nPar;
    P.shape = (int32_t*)dalloc(sizeof(int32_t) * nPar);
    P.aux = (int4*)dalloc(sizeof(int4) * nPar);
    P.facet = (double4_32a*)dalloc(sizeof(double4_32a) * nPar);
    P.mat = (int32_t*)dalloc(sizeof(int32_t) * nPar);
    P.mask = (uint32_t*)dalloc(sizeof(uint32_t) * nPar);
    P.mn = (double4_32a*)dalloc(sizeof(double4_32a) * nPar);
    P.mx = (double4_32a*)dalloc(sizeof(double4_32a) * nPar);
    I.loStart = (int32_t*)dalloc(sizeof(int32_t) * (nPar + 1));
    I.hiStart = (int32_t*)dalloc(sizeof(int32_t) * (nPar + 1));
    I.heavy = (int32_t*)dalloc(sizeof(int32_t) * 2 * std::max<int64_t>(1, nPar));
    I.heavyFree = I.heavy + std::max<int64_t>(1, nPar);
    dMats = (double4_32a*)dalloc(sizeof(double4_32a) * std::max<size_t>(1, hDensity.size()));
    dPar = (ScenePar*)dalloc(sizeof(ScenePar) * nScenes);
    if (nScenes > 1) {
        // scene of each particle and node slot
        hSceneOfPar.assign(nPar, 0);
        std::vector<int32_t> nsc(nSlots, 0);
        for (int k = 0; k < nScenes; k++)
            for (int64_t p = sceneStart[k]; p < sceneStart[k + 1]; p++) {
                hSceneOfPar[p] = k;
                if (hShape[p] == WG_SHAPE_FACET) {
                    for (int q = 0; q < 3; q++) nsc[map[hNodes3[3 * p + q]]] = k;
                } else nsc[p] = k;
            }
        P.scene = (int32_t*)dalloc(sizeof(int32_t) * nPar);
        N.scene = (int32_t*)dalloc(sizeof(int32_t) * nSlots);
        if (!N.scene) return fail(WG_ERR_CUDA, "out of device memory (scene)");
        WG_CUDA_TRY(cudaMemcpyAsync(P.scene, hSceneOfPar.data(), sizeof(int32_t) * nPar, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(N.scene, nsc.data(), sizeof(int32_t) * nSlots, cudaMemcpyHostToDevice, S.stream));
    }
    dStep = (long long*)dalloc(sizeof(long long));
    dFlags = (int*)dalloc(sizeof(int) * FL_WORDS);
    X.dApiMap = (int32_t*)dalloc(sizeof(int32_t) * std::max<int64_t>(1, na));
    X.dStage = (double*)dalloc(sizeof(double) * 19 * std::max<int64_t>(1, na));
    if (!X.dStage) return fail(WG_ERR_CUDA, "out of device memory (scene)");
    WG_CUDA_TRY(cudaMallocHost(&hFlags, sizeof(int) * 4 + sizeof(long long)));
    std::vector<double4_32a> mats(hDensity.size());
    for (size_t m = 0; m < hDensity.size(); m++) mats[m] = make_double4_32a(hDensity[m], hYoung[m], hTanPhi[m], hKtDivKn[m]);
    WG_CUDA_TRY(cudaMemcpyAsync(N.posr, posr.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.vel, vel.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.angv, angv.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.ori, ori.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.force, force.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.torque, torque.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.minert, minert.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.lastPos, posr.data(), sizeof(double4_32a) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(N.flags, flags.data(), sizeof(uint32_t) * nSlots, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(P.shape, shape.data(), sizeof(int32_t) * nPar, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(P.aux, aux.data(), sizeof(int4) * nPar, cudaMemcpyHostToDevice, S.stream));
    P.nFacets = (int32_t)facetIds.size();
    P.facetIds = nullptr;
    P.prep = nullptr;
    if (P.nFacets > 0) {
        P.facetIds = (int32_t*)dalloc(sizeof(int32_t) * P.nFacets);
        if (!P.facetIds) return fail(WG_ERR_CUDA, "out of device memory (facets)");
        WG_CUDA_TRY(cudaMemcpyAsync(P.facetIds, facetIds.data(), sizeof(int32_t) * P.nFacets, cudaMemcpyHostToDevice, S.stream));
        if (prec == WG_PREC_FP32) {
            P.prep = (FacetPrep*)dalloc(sizeof(FacetPrep) * P.nFacets);
            if (!P.prep) return fail(WG_ERR_CUDA, "out of device memory (facets)");
            WG_CUDA_TRY(cudaMemsetAsync(P.prep, 0xff, sizeof(FacetPrep) * P.nFacets, S.stream));  // NaN: made at the first step
        }
    }
    // facets whose vertices are all fully blocked and at rest never move: their FacetPrep records
    // are made once (here and when the host writes the state) instead of at every step
    facetsStatic = P.nFacets > 0;
    for (int64_t p = 0; p < nPar && facetsStatic; p++) {
        if (hShape[p] != WG_SHAPE_FACET) continue;
        for (int k = 0; k < 3; k++) {
            const int32_t v = map[hNodes3[3 * p + k]];
            if ((flags[v] & F_DOF_ALL) != F_DOF_ALL || vel[v].x != 0 || vel[v].y != 0 || vel[v].z != 0) facetsStatic = false;
        }
    }
    WG_CUDA_TRY(cudaMemcpyAsync(P.facet, facet.data(), sizeof(double4_32a) * nPar, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(P.mat, mat.data(), sizeof(int32_t) * nPar, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(P.mask, mask.data(), sizeof(uint32_t) * nPar, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(dMats, mats.data(), sizeof(double4_32a) * mats.size(), cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(X.dApiMap, map.data(), sizeof(int32_t) * na, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(X.dStage, hApi.data(), sizeof(double) * 19 * na, cudaMemcpyHostToDevice, S.stream));
    X.hApiMap = map;
    if (prec == WG_PREC_FP32) {
        std::vector<NodeConst32> nc(nSlots);
        for (int64_t q = 0; q < nSlots; q++) {
            const double4_32a m = minert[q];
            nc[q].invMass = m.w != 0 ? (float)(1. / m.w) : 0.f;
            nc[q].invI[0] = m.x != 0 ? (float)(1. / m.x) : 0.f;
            nc[q].invI[1] = m.y != 0 ? (float)(1. / m.y) : 0.f;
            nc[q].invI[2] = m.z != 0 ? (float)(1. / m.z) : 0.f;
            nc[q].mh = (float)m.w;
            nc[q].ml = (float)(m.w - (double)nc[q].mh);
            nc[q].flags = flags[q];
            nc[q].kind = (q < nPar && shape[q] != WG_SHAPE_FACET) ? NK_SUMMED : 0u;
        }
        std::vector<float4> orf(nSlots);
        std::vector<float2> rsp(nSlots);
        for (int64_t q = 0; q < nSlots; q++) {
            orf[q] = make_float4((float)ori[q].x, (float)ori[q].y, (float)ori[q].z, (float)ori[q].w);
            const float rh = (float)posr[q].w;
            rsp[q] = make_float2(rh, (float)(posr[q].w - (double)rh));
        }
        dNodeC = (NodeConst32*)dalloc(sizeof(NodeConst32) * nSlots);
        N.mir = (Mirror*)dalloc(sizeof(Mirror) * nSlots);
        N.wz = (float*)dalloc(sizeof(float) * nSlots);
        N.orif = (float4*)dalloc(sizeof(float4) * nSlots);
        N.rsplit = (float2*)dalloc(sizeof(float2) * nSlots);
        N.lh = (float4*)dalloc(sizeof(float4) * nSlots);
        N.ll = (float4*)dalloc(sizeof(float4) * nSlots);
        if (!N.ll) return fail(WG_ERR_CUDA, "out of device memory (scene)");
        if (!dNodeC || !N.mir || !N.wz || !N.orif || !N.rsplit) return fail(WG_ERR_CUDA, "out of device memory (scene)");
        WG_CUDA_TRY(cudaMemcpyAsync(N.orif, orf.data(), sizeof(float4) * nSlots, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(N.rsplit, rsp.data(), sizeof(float2) * nSlots, cudaMemcpyHostToDevice, S.stream));
        // double-float mirrors of the initial state (x = hi + lo)
        std::vector<float4> hph(nSlots), hpl(nSlots), hvh(nSlots), hvl(nSlots);
        std::vector<float> hwz(nSlots);
        auto split = [](double x, float& h, float& l) {
            h = (float)x;
            l = (float)(x - (double)h);
        };
        for (int64_t q = 0; q < nSlots; q++) {
            split(posr[q].x, hph[q].x, hpl[q].x);
            split(posr[q].y, hph[q].y, hpl[q].y);
            split(posr[q].z, hph[q].z, hpl[q].z);
            split(posr[q].w, hph[q].w, hpl[q].w);
            split(vel[q].x, hvh[q].x, hvl[q].x);
            split(vel[q].y, hvh[q].y, hvl[q].y);
            split(vel[q].z, hvh[q].z, hvl[q].z);
            hvh[q].w = (float)angv[q].x;
            hvl[q].w = (float)angv[q].y;
            hwz[q] = (float)angv[q].z;
        }
        std::vector<Mirror> hm(nSlots);
        for (int64_t q = 0; q < nSlots; q++) hm[q] = Mirror{hph[q], hpl[q], hvh[q], hvl[q]};
        WG_CUDA_TRY(cudaMemcpyAsync(N.mir, hm.data(), sizeof(Mirror) * nSlots, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(N.wz, hwz.data(), sizeof(float) * nSlots, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(N.lh, hph.data(), sizeof(float4) * nSlots, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(N.ll, hpl.data(), sizeof(float4) * nSlots, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(dNodeC, nc.data(), sizeof(NodeConst32) * nSlots, cudaMemcpyHostToDevice, S.stream));
    }
    launch_facet_prep(stream, N, P, nullptr);
    long long st0 = cfg.step;
    step = cfg.step;
    WG_CUDA_TRY(cudaMemcpyAsync(dStep, &st0, sizeof(long long), cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemsetAsync(dFlags, 0, sizeof(int) * FL_WORDS, S.stream));
    int r = ensureContactCapacity(std::max<int64_t>(1024, 4 * nPar));
    if (r) return r;
    C.n = 0;
    K.n = 0;
    packDirty = false;
    if (cfg.periodic) {
        X.cell.trsf = fromRow(cfg.cell_trsf);
        X.cell.hSize = fromRow(cfg.cell_hsize);
        X.cell.pprevHsize = X.cell.hSize;
        X.cell.gradV = fromRow(cfg.cell_gradv);
        X.cell.nextGradV = fromRow(cfg.cell_next_gradv);
        X.cell.homoDeform = cfg.homo_deform;
        HM W = hscale(hsub(X.cell.gradV, htr(X.cell.gradV)), .5);
        double lv[3];
        hlevi(W, lv);
        for (int i = 0; i < 3; i++) X.cell.spinVec[i] = .5 * lv[i];
        X.cell.integrateAndUpdate(0);
    }
    prepareParams();
    if (cfg.periodic) fillCellPar(X);
    if (nScenes > 1) {
        for (int k = 0; k < nScenes; k++) hPars[k].stepBase = (long long)cfg.step - (long long)cfgs[k].step;
        WG_CUDA_TRY(cudaMemcpyAsync(dPar, hPars.data(), sizeof(ScenePar) * nScenes, cudaMemcpyHostToDevice, S.stream));
    } else
        WG_CUDA_TRY(cudaMemcpyAsync(dPar, &hPar, sizeof(ScenePar), cudaMemcpyHostToDevice, S.stream));
    uploaded = true;
    initialized = false;
    return 0;
}

int Sim::checkErr() {
    Sim& S = *this;
    WG_CUDA_TRY(cudaMemcpyAsync(hFlags, dFlags, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
    WG_CUDA_TRY(cudaStreamSynchronize(stream));
    if (hFlags[1] == 101) return fail(WG_ERR_NAN, "NaN force in contact (message above)?!");
    if (hFlags[1] == 102) return fail(WG_ERR_NAN, "InsertionSortCollider: NaN in a particle bounding box (NaN position)");
    if (hFlags[1] == 103) return fail(WG_ERR_PERIODIC, "InsertionSortCollider: Particle larger than half of the cell size encountered.");
    if (hFlags[1] == 100) return fail(WG_ERR_ARG, "Cg2_Facet_Sphere_L3Geom: Impossible sphere-facet intersection (all points are outside the edges). (please report bug)");
    if (hFlags[1] != 0) return fail(WG_ERR_STATE, "device error code " + std::to_string(hFlags[1]));
    return 0;
}

// Clears the step-loop flags (an error code is kept) and optionally requests a full collider run.
__global__ void k_set_flags(int* f, int full) {
    f[FL_FULL] = full;
    f[FL_HALT] = 0;
}

// Scene::doOneStep (core/Scene.cpp:319-389) for n steps. Steps are queued on the stream in
// chunks without waiting for the verlet test of each one: every per-step kernel checks the
// device flag words, and once Leapfrog of step s finds a node past verletDist, the contact
// kernel of step s raises FL_HALT and everything queued after it does nothing. The host then
// reads the step counter, runs the collider for step s, finishes its contact loop and goes on.
int Sim::syncContacts(bool hostWait) {
    Sim& S = *this;
    if (packDirty && K.n > 0) {
        WG_CUDA_TRY(cudaSetDevice(device));
        launch_unpack_ss(stream, C, I, K, nMixed);
        WG_CUDA_TRY(cudaGetLastError());
        if (hostWait) WG_CUDA_TRY(cudaStreamSynchronize(stream));
    }
    packDirty = false;
    return 0;
}

// Scratch of the per-step energy contributions, grown to the nodes and active contacts (called
// outside stream capture: at the start of each chunk and after each full collider run).
int Sim::ensureEnergyCapacity() {
    Sim& S = *this;
    if (!dEnergy) {
        dEnergy = (double*)dalloc(sizeof(double) * WG_ENERGY_N);
        dECreated = (int32_t*)dalloc(sizeof(int32_t) * WG_ENERGY_N);
        dEPartial = (double*)dalloc(sizeof(double) * EN_CON_NCOL * 256);
        dEPrev = (double*)dalloc(sizeof(double) * 10);
        if (!dEnergy || !dECreated || !dEPartial || !dEPrev) return fail(WG_ERR_CUDA, "out of device memory (energy)");
        WG_CUDA_TRY(cudaMemsetAsync(dEnergy, 0, sizeof(double) * WG_ENERGY_N, S.stream));
        WG_CUDA_TRY(cudaMemsetAsync(dECreated, 0, sizeof(int32_t) * WG_ENERGY_N, S.stream));
        // ContactLoop.prevStress = 0, prevVol = NaN (ContactLoop.hpp:119-123)
        double prev[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, std::numeric_limits<double>::quiet_NaN()};
        WG_CUDA_TRY(cudaMemcpyAsync(dEPrev, prev, sizeof(prev), cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaStreamSynchronize(S.stream));
    }
    if (cfg.periodic && cfg.eval_stress) {
        const int64_t need = 9 * (std::max<int64_t>(1, (I.nAct + 255) / 256) + 1);
        if (stressCap < need) {
            if (dStress) dfree(dStress);
            stressCap = need + need / 2;
            dStress = (double*)dalloc(sizeof(double) * stressCap);
            if (!dStress) return fail(WG_ERR_CUDA, "out of device memory (stress)");
            if (graphExec) {
                cudaGraphExecDestroy(graphExec);
                graphExec = nullptr;
            }
        }
    }
    if (eNode.cap < N.n) {
        if (eNode.col) dfree(eNode.col);
        eNode.cap = std::max<int64_t>(N.n, 1);
        eNode.col = (double*)dalloc(sizeof(double) * EN_NODE_NCOL * eNode.cap);
        if (!eNode.col) return fail(WG_ERR_CUDA, "out of device memory (energy)");
    }
    if (eCon.cap < I.nAct || !eCon.col) {
        if (eCon.col) dfree(eCon.col);
        eCon.cap = std::max<int64_t>(I.nAct + I.nAct / 2, 1024);
        eCon.col = (double*)dalloc(sizeof(double) * EN_CON_NCOL * eCon.cap);
        if (!eCon.col) return fail(WG_ERR_CUDA, "out of device memory (energy)");
        if (graphExec) {  // captured with the old scratch
            cudaGraphExecDestroy(graphExec);
            graphExec = nullptr;
        }
    }
    return 0;
}

// Scene.dt of the steps from the next one on (core/Scene.cpp:389): the scene parameters the
// kernels read, and the cell integration of periodic runs (which takes cfg.dt)
// DynDt's engine state from the scene configuration (the counters carried over from the host)
DynDtState dynDtFromConfig(const wg_config& c) {
    DynDtState d;
    d.on = c.dyndt != 0;
    d.dryRun = c.dyndt_dry_run != 0;
    d.stepModulo = c.dyndt_step_modulo != 0;
    d.initRun = c.dyndt_init_run != 0;
    d.stepPeriod = c.dyndt_step_period;
    d.nDo = c.dyndt_n_do;
    d.nDone = c.dyndt_n_done;
    d.stepLast = c.dyndt_step_last;
    d.stepPrev = c.dyndt_step_prev;
    d.virtPeriod = c.dyndt_virt_period;
    d.virtLast = c.dyndt_virt_last;
    d.virtPrev = c.dyndt_virt_prev;
    d.maxRelInc = c.dyndt_max_rel_inc;
    d.dtSafety = c.dt_safety;
    return d;
}

// Scene.dt of scene k of a batch (or slot) from the next step on
int Sim::applyDtScene(int k, double ndt) {
    Sim& S = *this;
    cfgs[k].dt = ndt;
    hPars[k].dt = ndt;
    hPars[k].dtF = (float)ndt;
    if (k == 0) {
        cfg.dt = ndt;
        hPar = hPars[0];
    }
    WG_CUDA_TRY(cudaMemcpyAsync(dPar + k, &hPars[k], sizeof(ScenePar), cudaMemcpyHostToDevice, stream));
    return 0;
}

// DynDt::run (pkg/dem/DynDt.cpp:93-113) for the scenes of a batch whose DynDt is due after the
// contact loop of device step deviceStep: one stiffness pass over all scenes, the critical
// timestep of each scene (the minimum over its own nodes), then each due scene's rule.
int Sim::runDynDtScenes(const std::vector<char>& due, long long deviceStep) {
    Sim& S = *this;
    if (I.endCap > kCap || !dCritB) {
        if (I.endCap > kCap) {
            if (dKA) dfree(dKA);
            if (dKB) dfree(dKB);
            kCap = std::max<int64_t>(I.endCap, 1);
            dKA = (double4_32a*)dalloc(sizeof(double4_32a) * kCap);
            dKB = (double2*)dalloc(sizeof(double2) * kCap);
        }
        if (!dCritB) dCritB = (unsigned long long*)dalloc(sizeof(unsigned long long) * nScenes);
        if (!dKA || !dKB || !dCritB) return fail(WG_ERR_CUDA, "out of device memory (DynDt)");
    }
    const double inf = std::numeric_limits<double>::infinity();
    unsigned long long bits;
    std::memcpy(&bits, &inf, sizeof bits);
    std::vector<unsigned long long> crit(nScenes, bits);
    WG_CUDA_TRY(cudaMemsetAsync(dKA, 0, sizeof(double4_32a) * kCap, stream));
    WG_CUDA_TRY(cudaMemsetAsync(dKB, 0, sizeof(double2) * kCap, stream));
    WG_CUDA_TRY(cudaMemcpyAsync(dCritB, crit.data(), sizeof(unsigned long long) * nScenes, cudaMemcpyHostToDevice, stream));
    const bool fp32 = prec == WG_PREC_FP32;
    if (fp32) {
        int r = syncContacts();
        if (r) return r;
    }
    launch_dyndt(stream, N, P, C, I, dPar, dKA, dKB, dCritB, dFlags + FL_ERR, cfg.periodic != 0, fp32, true);
    WG_CUDA_TRY(cudaGetLastError());
    WG_CUDA_TRY(cudaMemcpyAsync(crit.data(), dCritB, sizeof(unsigned long long) * nScenes, cudaMemcpyDeviceToHost, stream));
    WG_CUDA_TRY(cudaStreamSynchronize(stream));
    for (int k = 0; k < nScenes; k++) {
        if (!due[k]) continue;
        DynDtState& d = bdd[k];
        double minSq;
        std::memcpy(&minSq, &crit[k], sizeof minSq);
        const double crDt = std::sqrt(minSq);
        d.critDt = crDt;
        d.nEvals++;
        if (std::isinf(crDt)) continue;
        const int64_t nSteps = sceneStep(k, deviceStep) - d.stepPrev;
        const double maxNewDt = hPars[k].dt * std::pow(1. + d.maxRelInc, (double)nSteps);
        const double a = crDt * d.dtSafety;
        const double ndt = maxNewDt < a ? maxNewDt : a;
        if (!d.dryRun) {
            if (ndt != hPars[k].dt) {
                d.dynDt = std::numeric_limits<double>::quiet_NaN();
                bNextDt[k] = ndt;
            }
        } else
            d.dynDt = ndt;
    }
    return 0;
}

int Sim::applyDt(double ndt) {
    Sim& S = *this;
    cfg.dt = ndt;
    hPar.dt = ndt;
    hPar.dtF = (float)ndt;
    if (!hPars.empty()) {
        hPars[0].dt = ndt;
        hPars[0].dtF = (float)ndt;
    }
    if (!cfg.periodic) WG_CUDA_TRY(cudaMemcpyAsync(dPar, &hPar, sizeof(ScenePar), cudaMemcpyHostToDevice, stream));
    return 0;
}

// DynDt::run (pkg/dem/DynDt.cpp:93-113) after the contact loop of step stepNow: the critical
// timestep from the contact stiffnesses (critDt_stiffness, :66-76, on the device), then
// nextDt = min(crDt*dtSafety, dt*(1+maxRelInc)^(steps since the previous run)).
int Sim::runDynDt(int64_t stepNow) {
    Sim& S = *this;
    if (I.endCap > kCap || !dCrit) {
        if (dKA) dfree(dKA);
        if (dKB) dfree(dKB);
        kCap = std::max<int64_t>(I.endCap, 1);
        dKA = (double4_32a*)dalloc(sizeof(double4_32a) * kCap);
        dKB = (double2*)dalloc(sizeof(double2) * kCap);
        if (!dCrit) dCrit = (unsigned long long*)dalloc(sizeof(unsigned long long));
        if (!dKA || !dKB || !dCrit) return fail(WG_ERR_CUDA, "out of device memory (DynDt)");
    }
    const double inf = std::numeric_limits<double>::infinity();
    unsigned long long bits;
    std::memcpy(&bits, &inf, sizeof bits);
    WG_CUDA_TRY(cudaMemsetAsync(dKA, 0, sizeof(double4_32a) * kCap, stream));
    WG_CUDA_TRY(cudaMemsetAsync(dKB, 0, sizeof(double2) * kCap, stream));
    WG_CUDA_TRY(cudaMemcpyAsync(dCrit, &bits, sizeof bits, cudaMemcpyHostToDevice, stream));
    const bool fp32 = prec == WG_PREC_FP32;
    if (fp32) {
        int r = syncContacts();  // the packed sphere-sphere state back into the contact arrays
        if (r) return r;
    }
    launch_dyndt(stream, N, P, C, I, dPar, dKA, dKB, dCrit, dFlags + FL_ERR, cfg.periodic != 0, fp32);
    WG_CUDA_TRY(cudaGetLastError());
    WG_CUDA_TRY(cudaMemcpyAsync(&bits, dCrit, sizeof bits, cudaMemcpyDeviceToHost, stream));
    WG_CUDA_TRY(cudaStreamSynchronize(stream));
    double minSq;
    std::memcpy(&minSq, &bits, sizeof minSq);
    const double crDt = std::sqrt(minSq);
    dd.critDt = crDt;
    dd.nEvals++;
    if (std::isinf(crDt)) return 0;  // no timestep computed, the current value stays
    const int64_t nSteps = stepNow - dd.stepPrev;
    const double maxNewDt = cfg.dt * std::pow(1. + dd.maxRelInc, (double)nSteps);
    const double a = crDt * dd.dtSafety;
    const double ndt = maxNewDt < a ? maxNewDt : a;  // std::min(a, maxNewDt)
    if (!dd.dryRun) {
        if (ndt != cfg.dt) {
            dd.dynDt = std::numeric_limits<double>::quiet_NaN();
            nextDt = ndt;
        }
    } else
        dd.dynDt = ndt;
    return 0;
}

int Sim::run(int64_t n) {
    Sim& S = *this;
    SimEx& X = static_cast<SimEx&>(*this);
    if (!uploaded) {
        int r = upload();
        if (r) return r;
    }
    WG_CUDA_TRY(cudaSetDevice(device));
    double ph[4] = {0, 0, 0, 0};
    int64_t launches = 0;
    bool anyZeroVd = hPar.verletDist == 0;
    for (const ScenePar& q : hPars) anyZeroVd = anyZeroVd || q.verletDist == 0;
    const int64_t maxChunk = anyZeroVd ? 1 : std::max<int64_t>(1, std::min<int64_t>(chunkSteps, 1024));
    // periodic cells: the cell of each queued step is integrated on the host ahead of the chunk (it
    // depends on the velocity gradient only) and its parameters uploaded as one record per step
    std::vector<HostCell> cellInt, cellEnd;
    std::vector<ScenePar> parSeq;
    if (cfg.periodic) {
        if (parSeqCap < maxChunk) {
            if (dParSeq) dfree(dParSeq);
            dParSeq = (ScenePar*)dalloc(sizeof(ScenePar) * maxChunk);
            if (!dParSeq) return fail(WG_ERR_CUDA, "out of device memory (cell parameters)");
            parSeqCap = maxChunk;
        }
        cellInt.resize(maxChunk);
        cellEnd.resize(maxChunk);
        parSeq.resize(maxChunk);
    }
    if ((int64_t)evPool.size() < 3 * maxChunk + 2) {
        for (int64_t q = (int64_t)evPool.size(); q < 3 * maxChunk + 2; q++) {
            cudaEvent_t e;
            WG_CUDA_TRY(cudaEventCreate(&e));
            evPool.push_back(e);
        }
    }
    cudaEvent_t* E = evPool.data();
    long long* hStepPin = (long long*)(hFlags + 4);
    const bool fp32 = prec == WG_PREC_FP32;
    bool anyLaw0 = cfg.law == 0;
    for (const wg_config& c : cfgs) anyLaw0 = anyLaw0 || c.law == 0;
    auto stepLeapfrog = [&](int fromEndsArg, ScenePar* sp) {
        if (fromEndsArg) {
            if (fp32) launch_forces32(stream, N, P, I, dNodeC, sp, dFlags, true);
            else launch_forces(stream, N, P, I, sp, dFlags, true);
            launches += I.nHeavyFree > 0;
        }
        if (fp32 && trackE) {
            cudaMemsetAsync(eNode.col, 0, sizeof(double) * EN_NODE_NCOL * eNode.cap, stream);
            launch_leapfrog32(stream, N, P, I, dNodeC, sp, dFlags, fromEndsArg, dStep, cfg.periodic != 0, &eNode);
            launch_energy_sum(stream, eNode, 0, N.n, dEPartial, dEnergy, dECreated, dFlags, cfg.kin_split != 0);
            launches += 2;
        } else if (fp32)
            launch_leapfrog32(stream, N, P, I, dNodeC, sp, dFlags, fromEndsArg, dStep, cfg.periodic != 0);
        else if (trackE) {
            cudaMemsetAsync(eNode.col, 0, sizeof(double) * EN_NODE_NCOL * eNode.cap, stream);
            launch_leapfrog(stream, N, P, I, sp, dFlags, fromEndsArg, dStep, cfg.periodic != 0, &eNode);
            launch_energy_sum(stream, eNode, 0, N.n, dEPartial, dEnergy, dECreated, dFlags, cfg.kin_split != 0);
            launches += 2;
        } else
            launch_leapfrog(stream, N, P, I, sp, dFlags, fromEndsArg, dStep, cfg.periodic != 0);
        launches++;
    };
    auto stepContact = [&](ScenePar* sp) {
        bool advanced = false;  // the last contact kernel advanced the step counter itself
        if (fp32 && trackE) {
            // the energy sums after the contact kernels read the step counter those advance: they
            // run with the step advance at the end instead
            cudaMemsetAsync(eCon.col, 0, sizeof(double) * EN_CON_NCOL * eCon.cap, stream);
            launch_contact_fp32(stream, SideStream{}, N, P, C, I, K, dMats, sp, dStep, dFlags, nMixed, cfg.periodic != 0, anyLaw0,
                                !facetsStatic, 128, &eCon);
            launch_energy_sum(stream, eCon, 1, I.nAct, dEPartial, dEnergy, dECreated, dFlags, false);
            launches += 2;
            if (cfg.periodic && cfg.eval_stress) {
                launch_stress(stream, N, P, C, I, sp, dStress + 9, stressCap - 9, dStress);
                launch_energy_gradv(stream, dStress, sp, dEPrev, dEnergy, dECreated, dFlags);
                launches += 3;
            }
        } else if (fp32)
            advanced = launch_contact_fp32(stream, concurrentContacts ? side : SideStream{}, N, P, C, I, K, dMats, sp, dStep, dFlags,
                                           nMixed, cfg.periodic != 0, anyLaw0, !facetsStatic, contactBlock != 0 ? contactBlock : -256);
        else if (trackE) {
            cudaMemsetAsync(eCon.col, 0, sizeof(double) * EN_CON_NCOL * eCon.cap, stream);
            launch_contact_fp64(stream, N, P, C, I, dMats, sp, dStep, dFlags, cfg.periodic != 0,
                                (contactBlock > 0 && contactBlock <= 128) ? contactBlock : 128, &eCon);
            launch_energy_sum(stream, eCon, 1, I.nAct, dEPartial, dEnergy, dECreated, dFlags, false);
            launches += 2;
            if (cfg.periodic && cfg.eval_stress) {
                // the stress of every step, for the gradV work (capacity ensured with the energy scratch)
                launch_stress(stream, N, P, C, I, sp, dStress + 9, stressCap - 9, dStress);
                launch_energy_gradv(stream, dStress, sp, dEPrev, dEnergy, dECreated, dFlags);
                launches += 3;
            }
        } else
            launch_contact_fp64(stream, N, P, C, I, dMats, sp, dStep, dFlags, cfg.periodic != 0,
                                (contactBlock > 0 && contactBlock <= 128) ? contactBlock : 128);  // launch bounds 128
        if (!advanced) launch_advance(stream, dStep, dFlags);
        launches += advanced ? 1 : 2;
    };
    WG_CUDA_TRY(cudaMemsetAsync(dFlags, 0, sizeof(int) * FL_WORDS, stream));
    WG_CUDA_TRY(cudaEventRecord(ev[6], stream));
    int64_t done = 0;
    while (done < n) {
        // the sphere-sphere kernel updates the packed state from here on
        if (K.n > 0) packDirty = true;
        if (trackE) {
            int r = ensureEnergyCapacity();
            if (r) return r;
        }
        int64_t k = std::min<int64_t>(n - done, maxChunk);
        // dt may change after a step (Scene.nextDt, DynDt): such a step ends its chunk
        if (std::isfinite(nextDt)) k = 1;
        // wg_run_host's early copy-out: the run's last step gets a chunk of its own, whose first
        // Leapfrog always runs (a halt only stops the steps after a full-run request)
        if (earlyWanted && !earlyIssued && done < n - 1) k = std::min<int64_t>(k, n - 1 - done);
        if (batchDyn) {
            // the same for every scene of a batch, with the scene's own step, time and dt
            for (int q = 0; q < nScenes; q++) {
                if (std::isfinite(bNextDt[q])) k = 1;
                if (!bdd[q].on) continue;
                DynDtState t = bdd[q];
                double tv = bTime[q];
                for (int64_t j = 0; j < k; j++) {
                    if (sceneFrozen(q, step + j)) break;
                    if (t.activated(sceneStep(q, step + j), tv)) {
                        k = j + 1;
                        break;
                    }
                    tv += hPars[q].dt;
                }
            }
        }
        if (dd.on) {
            DynDtState t = dd;
            double tv = timeAbs;
            for (int64_t j = 0; j < k; j++) {
                if (t.activated(step + j, tv)) {
                    k = j + 1;
                    break;
                }
                tv += cfg.dt;
            }
        }
        const bool needFull = !initialized || anyZeroVd || forceFull;
        k_set_flags<<<1, 1, 0, stream>>>(dFlags, needFull ? 1 : 0);
        if (cfg.periodic) {
            // Cell::integrateAndUpdate then setNextGradV for every queued step (Scene::doOneStep)
            for (int64_t j = 0; j < k; j++) {
                X.cell.integrateAndUpdate(cfg.dt);
                fillCellPar(X);
                parSeq[j] = hPar;
                // Leapfrog's reallyTrackEnergy (Leapfrog.cpp:104): not in the first step of a
                // periodic scene unless gradV is the identity
                parSeq[j].trackEnergy = cfg.track_energy && (step + j > 0 || isIdentity(X.cell.gradV));
                cellInt[j] = X.cell;
                X.cell.setNextGradV();
                cellEnd[j] = X.cell;
            }
            WG_CUDA_TRY(cudaMemcpyAsync(dParSeq, parSeq.data(), sizeof(ScenePar) * k, cudaMemcpyHostToDevice, stream));
        }
        auto spOf = [&](int64_t j) { return cfg.periodic ? dParSeq + j : dPar; };
        const int64_t s0 = step;
        // a chunk that starts from the end slots and is not due for a full run is replayed as a
        // CUDA graph (re-captured after every full run, whose contact arrays it refers to)
        const bool lastEarly = earlyWanted && !earlyIssued && done + k == n && k == 1;
        const bool graphChunk = useGraph && fromEnds && !needFull && k == maxChunk && !cfg.periodic && !lastEarly;
        if (graphChunk) {
            if (!graphExec || graphSteps != k || graphEpoch != nFullRuns) {
                if (graphExec) cudaGraphExecDestroy(graphExec);
                graphExec = nullptr;
                cudaGraph_t g = nullptr;
                WG_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                const int64_t l0 = launches;
                for (int64_t j = 0; j < k; j++) {
                    stepLeapfrog(1, dPar);
                    stepContact(dPar);
                }
                graphLaunches = launches - l0;
                launches = l0;
                WG_CUDA_TRY(cudaStreamEndCapture(stream, &g));
                WG_CUDA_TRY(cudaGraphInstantiate(&graphExec, g, 0));
                cudaGraphDestroy(g);
                graphSteps = k;
                graphEpoch = nFullRuns;
            }
            WG_CUDA_TRY(cudaEventRecord(E[0], stream));
            WG_CUDA_TRY(cudaGraphLaunch(graphExec, stream));
            WG_CUDA_TRY(cudaEventRecord(E[1], stream));
            launches += graphLaunches;
        } else {
            for (int64_t j = 0; j < k; j++) {
                WG_CUDA_TRY(cudaEventRecord(E[3 * j], stream));
                stepLeapfrog(j == 0 ? (fromEnds ? 1 : 0) : 1, spOf(j));
                WG_CUDA_TRY(cudaEventRecord(E[3 * j + 1], stream));
                if (lastEarly) {
                    int r = issueEarlyGet();
                    if (r) return r;
                }
                stepContact(spOf(j));
                WG_CUDA_TRY(cudaEventRecord(E[3 * j + 2], stream));
            }
        }
        WG_CUDA_TRY(cudaGetLastError());
        WG_CUDA_TRY(cudaMemcpyAsync(hFlags, dFlags, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
        WG_CUDA_TRY(cudaMemcpyAsync(hStepPin, dStep, sizeof(long long), cudaMemcpyDeviceToHost, stream));
        WG_CUDA_TRY(cudaStreamSynchronize(stream));
        if (hFlags[FL_ERR]) break;
        int64_t ds = (int64_t)*hStepPin - s0;
        if (ds < 0 || ds > k) return fail(WG_ERR_STATE, "device step counter out of sequence");
        float a;
        if (graphChunk) {
            cudaEventElapsedTime(&a, E[0], E[1]);
            ph[2] += a;  // whole steps replayed as a graph
        } else
            for (int64_t j = 0; j < ds; j++) {
                cudaEventElapsedTime(&a, E[3 * j], E[3 * j + 1]); ph[0] += a;
                cudaEventElapsedTime(&a, E[3 * j + 1], E[3 * j + 2]); ph[1] += a;
            }
        if (ds < k || hFlags[FL_FULL]) {
            // Leapfrog of step s0+ds ran, its contact loop waits for the collider
            if (!hFlags[FL_FULL]) return fail(WG_ERR_STATE, "queued steps halted without a collider request");
            if (!graphChunk) {
                cudaEventElapsedTime(&a, E[3 * ds], E[3 * ds + 1]);
                ph[0] += a;
            }
            if (cfg.periodic) {
                // the cell of step s0+ds, for the collider and that step's contact loop
                X.cell = cellInt[ds];
                hPar = parSeq[ds];
                WG_CUDA_TRY(cudaMemcpyAsync(dPar, &hPar, sizeof(ScenePar), cudaMemcpyHostToDevice, stream));
            }
            WG_CUDA_TRY(cudaEventRecord(E[3 * maxChunk], stream));
            int r = collide_full_run(*this);
            if (r) return r;
            if (trackE) {
                r = ensureEnergyCapacity();
                if (r) return r;
            }
            initialized = true;
            forceFull = false;
            launches += 12;
            WG_CUDA_TRY(cudaEventRecord(E[3 * maxChunk + 1], stream));
            k_set_flags<<<1, 1, 0, stream>>>(dFlags, 0);
            if (K.n > 0) packDirty = true;
            WG_CUDA_TRY(cudaEventRecord(E[0], stream));
            stepContact(dPar);
            WG_CUDA_TRY(cudaEventRecord(E[1], stream));
            WG_CUDA_TRY(cudaMemcpyAsync(hFlags, dFlags, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
            WG_CUDA_TRY(cudaStreamSynchronize(stream));
            cudaEventElapsedTime(&a, E[3 * maxChunk], E[3 * maxChunk + 1]); ph[3] += a;
            cudaEventElapsedTime(&a, E[0], E[1]); ph[1] += a;
            if (hFlags[FL_ERR]) {
                for (int64_t j = 0; j < ds; j++) {
                    if (dd.on) dd.activated(step + j, timeAbs);
                    time += cfg.dt;
                    timeAbs += cfg.dt;
                }
                step += ds;
                break;
            }
            ds += 1;
        }
        fromEnds = true;
        if (cfg.periodic && ds > 0) {
            // the cell after the last step done; dPar holds that step's parameters (stress, listing)
            X.cell = cellEnd[ds - 1];
            hPar = parSeq[ds - 1];
            WG_CUDA_TRY(cudaMemcpyAsync(dPar, &hPar, sizeof(ScenePar), cudaMemcpyHostToDevice, stream));
        }
        // Scene::doOneStep epilogue for each step done (core/Scene.cpp:384-389): the engines' turn
        // for DynDt (activation counters; it runs after ContactLoop of the chunk's last step, which
        // the chunk was cut at), then step++, time += dt, dt = nextDt
        bool dynDtNow = false;
        for (int64_t j = 0; j < ds; j++) {
            if (dd.on && dd.activated(step + j, timeAbs)) {
                if (j != ds - 1) return fail(WG_ERR_STATE, "DynDt activation inside a chunk");
                dynDtNow = true;
            }
            if (j < ds - 1) {
                time += cfg.dt;
                timeAbs += cfg.dt;
            }
        }
        step += ds;
        done += ds;
        if (nScenes > 1 && ds > 0) {
            // each scene of the batch: its DynDt turn (the chunk ends at any scene's activation),
            // time += its dt for each step it did (not frozen), then its dt = nextDt
            std::vector<char> due(nScenes, 0);
            bool anyDue = false;
            for (int q = 0; q < nScenes; q++) {
                for (int64_t j = 0; j < ds; j++) {
                    const long long sd = step - ds + j;
                    if (sceneFrozen(q, sd)) break;
                    if (bdd[q].on && bdd[q].activated(sceneStep(q, sd), bTime[q])) {
                        if (j != ds - 1) return fail(WG_ERR_STATE, "DynDt activation inside a chunk");
                        due[q] = 1;
                        anyDue = true;
                    }
                    bTime[q] += hPars[q].dt;
                }
            }
            if (anyDue) {
                int r = runDynDtScenes(due, step - 1);
                if (r) return r;
            }
            for (int q = 0; q < nScenes; q++)
                if (std::isfinite(bNextDt[q])) {
                    int r = applyDtScene(q, bNextDt[q]);
                    if (r) return r;
                    bNextDt[q] = std::numeric_limits<double>::quiet_NaN();
                }
        }
        if (ds > 0) {
            if (dynDtNow) {
                int r = runDynDt(step - 1);
                if (r) return r;
            }
            time += cfg.dt;
            timeAbs += cfg.dt;
            if (std::isfinite(nextDt)) {
                int r = applyDt(nextDt);
                if (r) return r;
                nextDt = std::numeric_limits<double>::quiet_NaN();
            }
        }
    }
    // ContactLoop.stress of the last step (periodic cells with evalStress)
    if (cfg.periodic && cfg.eval_stress && fromEnds && done > 0) {
        const int64_t need = 9 * (std::max<int64_t>(1, (I.nAct + 255) / 256) + 1);
        if (stressCap < need) {
            if (dStress) dfree(dStress);
            stressCap = need + need / 2;
            dStress = (double*)dalloc(sizeof(double) * stressCap);
            if (!dStress) return fail(WG_ERR_CUDA, "out of device memory (stress)");
        }
        int r = syncContacts();
        if (r) return r;
        if (launch_stress(stream, N, P, C, I, dPar, dStress + 9, stressCap - 9, dStress))
            return fail(WG_ERR_STATE, "stress scratch too small");
        double sum[9];
        WG_CUDA_TRY(cudaMemcpyAsync(sum, dStress, sizeof(double) * 9, cudaMemcpyDeviceToHost, stream));
        WG_CUDA_TRY(cudaStreamSynchronize(stream));
        const double det = hdet(X.cell.hSize);
        for (int q = 0; q < 9; q++) stress[q] = sum[q] / det;
    }
    // DemData.force/torque of the last contact loop, for the host and for the next run
    if (fromEnds) {
        if (fp32) launch_forces32(stream, N, P, I, dNodeC, dPar, nullptr, false);
        else launch_forces(stream, N, P, I, dPar, nullptr, false);
        launches += 1 + (I.nHeavy > 0);
    }
    WG_CUDA_TRY(cudaEventRecord(ev[7], stream));
    WG_CUDA_TRY(cudaEventSynchronize(ev[7]));
    WG_CUDA_TRY(cudaGetLastError());
    float tot = 0;
    cudaEventElapsedTime(&tot, ev[6], ev[7]);
    lastTotalMs = tot;
    for (int q = 0; q < 4; q++) phaseMs[q] = ph[q];
    lastLaunches = launches;
    return checkErr();
}

}  // namespace wg

using namespace wg;

extern "C" {

int wg_create(wg_scene** out, int device) {
    if (!out) return WG_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        g_createError = "no CUDA device available";
        return WG_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) {
        g_createError = "CUDA device index out of range";
        return WG_ERR_ARG;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        g_createError = "cudaSetDevice failed";
        return WG_ERR_CUDA;
    }
    SimEx* s = new SimEx();
    s->device = device;
    for (int i = 0; i < 8; i++) s->ev[i] = nullptr;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->side.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->side.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->side.join, cudaEventDisableTiming) != cudaSuccess) {
        g_createError = "cudaStreamCreate failed";
        delete s;
        return WG_ERR_CUDA;
    }
    for (int i = 0; i < 8; i++) cudaEventCreate(&s->ev[i]);
    std::memset(&s->cfg, 0, sizeof(s->cfg));
    *out = reinterpret_cast<wg_scene*>(static_cast<Sim*>(s));
    return WG_OK;
}

void wg_destroy(wg_scene* s) { delete static_cast<SimEx*>(reinterpret_cast<Sim*>(s)); }

const char* wg_last_error(const wg_scene* s) {
    if (!s) return g_createError.c_str();
    return reinterpret_cast<const Sim*>(s)->err.c_str();
}

static Sim* SIM(wg_scene* s) { return reinterpret_cast<Sim*>(s); }

int wg_set_config(wg_scene* s, const wg_config* c) {
    if (!s || !c) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (S.uploaded) return S.fail(WG_ERR_STATE, "configuration is fixed once the scene runs; create a new scene");
    if (!(c->dt > 0) || !std::isfinite(c->dt)) return S.fail(WG_ERR_ARG, "Scene.dt must be positive and finite");
    if (c->dyndt && !(c->dyndt_max_rel_inc > 0 && 1. + c->dyndt_max_rel_inc != 1.))
        return S.fail(WG_ERR_ARG, "DynDt: maxRelInc too small (1.0+maxRelInc==1.0)");  // DynDt::postLoad, DynDt.cpp:12-14
    S.cfg = *c;
    S.haveCfg = true;
    S.dd = dynDtFromConfig(*c);
    S.nextDt = validNextDt(*c);
    S.timeAbs = c->time;
    S.trackE = c->track_energy != 0;
    return WG_OK;
}

int wg_set_scenes(wg_scene* s, int32_t n_scenes, const wg_config* cfgs, const int64_t* particle_start) {
    if (!s || n_scenes < 1 || !cfgs || !particle_start) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (S.uploaded) return S.fail(WG_ERR_STATE, "scenes are fixed once the simulation runs; create a new one");
    if (particle_start[0] != 0) return S.fail(WG_ERR_ARG, "particle_start[0] must be 0");
    for (int k = 0; k < n_scenes; k++) {
        if (particle_start[k + 1] < particle_start[k]) return S.fail(WG_ERR_ARG, "particle_start must be non-decreasing");
        if (!(cfgs[k].dt > 0) || !std::isfinite(cfgs[k].dt)) return S.fail(WG_ERR_ARG, "Scene.dt must be positive and finite");
        if (cfgs[k].track_energy)
            return S.fail(WG_ERR_UNSUPPORTED, "energy tracking is not supported in a batch of scenes");
        if (cfgs[k].dyndt && !(cfgs[k].dyndt_max_rel_inc > 0 && 1. + cfgs[k].dyndt_max_rel_inc != 1.))
            return S.fail(WG_ERR_ARG, "DynDt: maxRelInc too small (1.0+maxRelInc==1.0)");
    }
    S.nScenes = n_scenes;
    S.cfgs.assign(cfgs, cfgs + n_scenes);
    S.sceneStart.assign(particle_start, particle_start + n_scenes + 1);
    S.sceneTime0.assign(n_scenes, 0.0);
    S.bdd.assign(n_scenes, DynDtState{});
    S.bTime.assign(n_scenes, 0.0);
    S.bNextDt.assign(n_scenes, std::numeric_limits<double>::quiet_NaN());
    S.batchDyn = false;
    for (int k = 0; k < n_scenes; k++) {
        S.bdd[k] = dynDtFromConfig(cfgs[k]);
        S.bTime[k] = cfgs[k].time;
        S.bNextDt[k] = validNextDt(cfgs[k]);
        S.batchDyn = S.batchDyn || S.bdd[k].on || std::isfinite(S.bNextDt[k]);
    }
    S.cfg = cfgs[0];
    S.haveCfg = true;
    return WG_OK;
}

// ------------------------------------------------------------------ serving slots
namespace wg {
// Writes particles [p0, p0 + cap) of a slot (uninodal: node slot = particle): the first n from the
// job's arrays, the rest parked (blocked, at rest, left out of the collider).
static int writeSlot(Sim& S, int64_t p0, int64_t cap, int64_t n, const double* pos, const double* ori, const double* vel,
                     const double* angv, const double* mass, const double* inertia, const uint32_t* flags, const int32_t* shape,
                     const double* radius, const int32_t* axis, const int32_t* sense, const int32_t* mat, int32_t matBase,
                     const uint32_t* mask) {
    std::vector<double4_32a> posr(cap), v4(cap), w4(cap), o4(cap), zero(cap), mi(cap);
    std::vector<uint32_t> fl(cap), mk(cap);
    std::vector<int32_t> sh(cap), mt(cap);
    std::vector<int4> aux(cap);
    std::vector<double4_32a> fac(cap);
    for (int64_t q = 0; q < cap; q++) {
        const int64_t p = p0 + q;
        zero[q] = make_double4_32a(0, 0, 0, 0);
        fac[q] = zero[q];
        aux[q] = make_int4(0, 0, 0, 0);
        if (q < n) {
            sh[q] = shape[q];
            const double r = shape[q] == WG_SHAPE_SPHERE ? radius[q] : 0.;
            posr[q] = make_double4_32a(pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], r);
            v4[q] = make_double4_32a(vel[3 * q], vel[3 * q + 1], vel[3 * q + 2], 0);
            w4[q] = make_double4_32a(angv[3 * q], angv[3 * q + 1], angv[3 * q + 2], 0);
            o4[q] = make_double4_32a(ori[4 * q], ori[4 * q + 1], ori[4 * q + 2], ori[4 * q + 3]);
            mi[q] = make_double4_32a(inertia[3 * q], inertia[3 * q + 1], inertia[3 * q + 2], mass[q]);
            fl[q] = flags[q];
            mt[q] = matBase + mat[q];
            mk[q] = mask[q];
            if (shape[q] == WG_SHAPE_WALL) aux[q] = make_int4(axis[q], sense[q], 0, 0);
        } else {
            sh[q] = WG_SHAPE_SPHERE;
            posr[q] = make_double4_32a(0, 0, 0, 0);
            v4[q] = w4[q] = zero[q];
            o4[q] = make_double4_32a(1, 0, 0, 0);
            mi[q] = make_double4_32a(1, 1, 1, 1);
            fl[q] = F_DOF_ALL;
            mt[q] = matBase;
            mk[q] = 0;
        }
        S.hShape[p] = sh[q];
        S.hRadius[p] = posr[q].w;
        S.hAxis[p] = aux[q].x;
        S.hSense[p] = aux[q].y;
        S.hMat[p] = mt[q];
        S.hMask[p] = mk[q];
        S.hParked[p] = q < n ? 0 : 1;
    }
    auto put = [&](void* dst, const void* src, size_t bytes) -> int {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, S.stream) == cudaSuccess ? 0 : -1;
    };
    const size_t d4 = sizeof(double4_32a);
    if (put(S.N.posr + p0, posr.data(), d4 * cap) || put(S.N.vel + p0, v4.data(), d4 * cap) || put(S.N.angv + p0, w4.data(), d4 * cap) ||
        put(S.N.ori + p0, o4.data(), d4 * cap) || put(S.N.force + p0, zero.data(), d4 * cap) || put(S.N.torque + p0, zero.data(), d4 * cap) ||
        put(S.N.minert + p0, mi.data(), d4 * cap) || put(S.N.lastPos + p0, posr.data(), d4 * cap) ||
        put(S.N.flags + p0, fl.data(), sizeof(uint32_t) * cap) || put(S.P.shape + p0, sh.data(), sizeof(int32_t) * cap) ||
        put(S.P.aux + p0, aux.data(), sizeof(int4) * cap) || put(S.P.facet + p0, fac.data(), d4 * cap) ||
        put(S.P.mat + p0, mt.data(), sizeof(int32_t) * cap) || put(S.P.mask + p0, mk.data(), sizeof(uint32_t) * cap))
        return S.fail(WG_ERR_CUDA, "slot upload failed");
    if (S.prec == WG_PREC_FP32) {
        std::vector<NodeConst32> nc(cap);
        std::vector<float4> ph(cap), pl(cap), vh(cap), vl(cap), of(cap);
        std::vector<float> wz(cap);
        std::vector<float2> rs(cap);
        auto split = [](double x, float& h, float& l) {
            h = (float)x;
            l = (float)(x - (double)h);
        };
        for (int64_t q = 0; q < cap; q++) {
            const double4_32a m = mi[q];
            nc[q].invMass = m.w != 0 ? (float)(1. / m.w) : 0.f;
            nc[q].invI[0] = m.x != 0 ? (float)(1. / m.x) : 0.f;
            nc[q].invI[1] = m.y != 0 ? (float)(1. / m.y) : 0.f;
            nc[q].invI[2] = m.z != 0 ? (float)(1. / m.z) : 0.f;
            nc[q].mh = (float)m.w;
            nc[q].ml = (float)(m.w - (double)nc[q].mh);
            nc[q].flags = fl[q];
            nc[q].kind = sh[q] != WG_SHAPE_FACET ? NK_SUMMED : 0u;
            split(posr[q].x, ph[q].x, pl[q].x);
            split(posr[q].y, ph[q].y, pl[q].y);
            split(posr[q].z, ph[q].z, pl[q].z);
            split(posr[q].w, ph[q].w, pl[q].w);
            split(v4[q].x, vh[q].x, vl[q].x);
            split(v4[q].y, vh[q].y, vl[q].y);
            split(v4[q].z, vh[q].z, vl[q].z);
            vh[q].w = (float)w4[q].x;
            vl[q].w = (float)w4[q].y;
            wz[q] = (float)w4[q].z;
            of[q] = make_float4((float)o4[q].x, (float)o4[q].y, (float)o4[q].z, (float)o4[q].w);
            rs[q] = make_float2(ph[q].w, pl[q].w);
        }
        std::vector<Mirror> mr(cap);
        for (int64_t q = 0; q < cap; q++) mr[q] = Mirror{ph[q], pl[q], vh[q], vl[q]};
        if (put(S.dNodeC + p0, nc.data(), sizeof(NodeConst32) * cap) || put(S.N.mir + p0, mr.data(), sizeof(Mirror) * cap) ||
            put(S.N.wz + p0, wz.data(), sizeof(float) * cap) ||
            put(S.N.orif + p0, of.data(), sizeof(float4) * cap) || put(S.N.rsplit + p0, rs.data(), sizeof(float2) * cap) ||
            put(S.N.lh + p0, ph.data(), sizeof(float4) * cap) || put(S.N.ll + p0, pl.data(), sizeof(float4) * cap))
            return S.fail(WG_ERR_CUDA, "slot upload failed");
    }
    // the slot's contacts end at the next full run; its nodes take their stored force first
    if (cudaMemsetAsync(S.P.fresh + p0, 1, cap, S.stream) != cudaSuccess || cudaMemsetAsync(S.N.fresh + p0, 1, cap, S.stream) != cudaSuccess)
        return S.fail(WG_ERR_CUDA, "slot upload failed");
    if (cudaStreamSynchronize(S.stream) != cudaSuccess) return S.fail(WG_ERR_CUDA, "slot upload failed");
    S.listsDirty = true;
    S.forceFull = true;
    return 0;
}

static int slotCheck(Sim& S, int32_t k) {
    if (S.nScenes < 1 || k < 0 || k >= S.nScenes || (int64_t)S.sceneStart.size() != S.nScenes + 1)
        return S.fail(WG_ERR_ARG, "slot index out of range");
    if (!S.uploaded) {
        int r = S.upload();
        if (r) return r;
    }
    if (S.cfg.periodic) return S.fail(WG_ERR_UNSUPPORTED, "serving slots hold aperiodic scenes");
    for (int64_t p = S.sceneStart[k]; p < S.sceneStart[k + 1]; p++)
        if (S.hShape[p] == WG_SHAPE_FACET) return S.fail(WG_ERR_UNSUPPORTED, "serving slots hold spheres and walls");
    if (!S.P.fresh) {
        S.P.fresh = (uint8_t*)S.dalloc(S.nPar);
        S.N.fresh = (uint8_t*)S.dalloc(S.N.n);
        if (!S.N.fresh) return S.fail(WG_ERR_CUDA, "out of device memory (slots)");
        WG_CUDA_TRY(cudaMemsetAsync(S.P.fresh, 0, S.nPar, S.stream));
        WG_CUDA_TRY(cudaMemsetAsync(S.N.fresh, 0, S.N.n, S.stream));
    }
    if (S.hParked.empty()) S.hParked.assign(S.nPar, 0);
    return 0;
}
}  // namespace wg

int wg_slot_load(wg_scene* s, int32_t k, const wg_config* c, int64_t n, const double* pos, const double* ori, const double* vel,
                 const double* ang_vel, const double* mass, const double* inertia, const uint32_t* flags, const int32_t* shape,
                 const double* radius, const int32_t* wall_axis, const int32_t* wall_sense, const int32_t* mat, const uint32_t* mask,
                 int32_t n_mat, const double* density, const double* young, const double* tan_phi, const double* kt_div_kn,
                 int64_t n_steps) {
    if (!s || !c || n < 0 || n_steps < 0 || n_mat < 1) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    int r = slotCheck(S, k);
    if (r) return r;
    if (c->track_energy) return S.fail(WG_ERR_UNSUPPORTED, "energy tracking is not supported in serving slots");
    if (c->dyndt && !(c->dyndt_max_rel_inc > 0 && 1. + c->dyndt_max_rel_inc != 1.))
        return S.fail(WG_ERR_ARG, "DynDt: maxRelInc too small (1.0+maxRelInc==1.0)");
    const int64_t p0 = S.sceneStart[k], cap = S.sceneStart[k + 1] - p0;
    if (n > cap) return S.fail(WG_ERR_CAPACITY, "job larger than the slot");
    const int32_t matCap = (int32_t)(S.hDensity.size() / S.nScenes);
    if (n_mat > matCap) return S.fail(WG_ERR_CAPACITY, "job has more materials than the slot");
    if (c->precision != S.cfg.precision || c->periodic || c->lone_mask != S.cfg.lone_mask || c->apply_forces != S.cfg.apply_forces ||
        !c->reset || !((c->phys == 0 && c->law == 0) || (c->phys == 1 && c->law == 1)) || (c->law == 1 && c->hz_alpha != 0) ||
        !(c->dt > 0))
        return S.fail(WG_ERR_UNSUPPORTED, "job configuration does not fit the serving batch");
    for (int64_t q = 0; q < n; q++) {
        if (shape[q] != WG_SHAPE_SPHERE && shape[q] != WG_SHAPE_WALL) return S.fail(WG_ERR_UNSUPPORTED, "serving slots hold spheres and walls");
        if (mat[q] < 0 || mat[q] >= n_mat) return S.fail(WG_ERR_ARG, "particle material index out of range");
    }
    WG_CUDA_TRY(cudaSetDevice(S.device));
    const int32_t matBase = k * matCap;
    std::vector<double4_32a> mats(n_mat);
    for (int m = 0; m < n_mat; m++) {
        mats[m] = make_double4_32a(density[m], young[m], tan_phi[m], kt_div_kn[m]);
        S.hDensity[matBase + m] = density[m];
        S.hYoung[matBase + m] = young[m];
        S.hTanPhi[matBase + m] = tan_phi[m];
        S.hKtDivKn[matBase + m] = kt_div_kn[m];
    }
    WG_CUDA_TRY(cudaMemcpyAsync(S.dMats + matBase, mats.data(), sizeof(double4_32a) * n_mat, cudaMemcpyHostToDevice, S.stream));
    r = writeSlot(S, p0, cap, n, pos, ori, vel, ang_vel, mass, inertia, flags, shape, radius, wall_axis, wall_sense, mat, matBase, mask);
    if (r) return r;
    S.cfgs[k] = *c;
    S.prepareParamsFor(*c, p0, p0 + n, S.hPars[k]);
    S.hPars[k].stepBase = (long long)S.step - (long long)c->step;
    S.hPars[k].stepEnd = (long long)c->step + (long long)n_steps;
    S.sceneTime0[k] = 0.;
    S.bdd[k] = dynDtFromConfig(*c);
    S.bTime[k] = c->time;
    S.bNextDt[k] = validNextDt(*c);
    S.batchDyn = S.batchDyn || S.bdd[k].on || std::isfinite(S.bNextDt[k]);
    if (k == 0) S.hPar = S.hPars[0];
    WG_CUDA_TRY(cudaMemcpyAsync(S.dPar + k, &S.hPars[k], sizeof(ScenePar), cudaMemcpyHostToDevice, S.stream));
    return WG_OK;
}

int wg_slot_clear(wg_scene* s, int32_t k) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    int r = slotCheck(S, k);
    if (r) return r;
    const int64_t p0 = S.sceneStart[k], cap = S.sceneStart[k + 1] - p0;
    for (int64_t p = p0; p < p0 + cap; p++) S.hParked[p] = 1;
    WG_CUDA_TRY(cudaMemsetAsync(S.P.fresh + p0, 1, cap, S.stream));
    S.hPars[k].stepEnd = -((long long)1 << 62);  // frozen
    S.bdd[k].on = false;
    S.bNextDt[k] = std::numeric_limits<double>::quiet_NaN();
    if (k == 0) S.hPar = S.hPars[0];
    WG_CUDA_TRY(cudaMemcpyAsync(S.dPar + k, &S.hPars[k], sizeof(ScenePar), cudaMemcpyHostToDevice, S.stream));
    S.listsDirty = true;
    S.forceFull = true;
    return WG_OK;
}

int wg_slot_status(wg_scene* s, int32_t k, int64_t* steps_done, int64_t* steps_end) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (k < 0 || k >= S.nScenes || (int64_t)S.hPars.size() != S.nScenes) return S.fail(WG_ERR_ARG, "slot index out of range");
    const ScenePar& q = S.hPars[k];
    const long long done = (long long)S.step - q.stepBase;
    if (steps_done) *steps_done = std::min<long long>(done, std::max<long long>(q.stepEnd, 0));
    if (steps_end) *steps_end = q.stepEnd;
    return WG_OK;
}

int wg_get_slot_nodes(wg_scene* s, int32_t k, int64_t n, double* pos, double* ori, double* vel, double* ang_vel, double* force,
                      double* torque) {
    if (!s || n < 0) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (k < 0 || k >= S.nScenes || !S.uploaded) return S.fail(WG_ERR_ARG, "slot index out of range");
    const int64_t p0 = S.sceneStart[k];
    if (n > S.sceneStart[k + 1] - p0) return S.fail(WG_ERR_ARG, "more nodes than the slot holds");
    WG_CUDA_TRY(cudaStreamSynchronize(S.stream));
    std::vector<double4_32a> a(n);
    auto get = [&](const double4_32a* src, double* dst, int w) -> int {
        if (!dst) return 0;
        if (cudaMemcpyAsync(a.data(), src + p0, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, S.stream) != cudaSuccess) return -1;
        for (int64_t q = 0; q < n; q++) {
            const double v[4] = {a[q].x, a[q].y, a[q].z, a[q].w};
            for (int j = 0; j < w; j++) dst[w * q + j] = v[j];
        }
        return 0;
    };
    if (get(S.N.posr, pos, 3) || get(S.N.vel, vel, 3) || get(S.N.angv, ang_vel, 3) || get(S.N.force, force, 3) ||
        get(S.N.torque, torque, 3))
        return S.fail(WG_ERR_CUDA, "slot download failed");
    if (ori) {
        if (S.N.orif) {
            std::vector<float4> f(n);
            WG_CUDA_TRY(cudaMemcpyAsync(f.data(), S.N.orif + p0, sizeof(float4) * n, cudaMemcpyDeviceToHost, S.stream));
            for (int64_t q = 0; q < n; q++) {
                ori[4 * q] = f[q].x; ori[4 * q + 1] = f[q].y; ori[4 * q + 2] = f[q].z; ori[4 * q + 3] = f[q].w;
            }
        } else if (get(S.N.ori, ori, 4))
            return S.fail(WG_ERR_CUDA, "slot download failed");
    }
    return WG_OK;
}

int wg_set_launch(wg_scene* s, int32_t contact_block, int32_t chunk_steps, int32_t launch_flags) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (contact_block != 0 && contact_block != 64 && contact_block != 128 && contact_block != 256 && contact_block != -256)
        return S.fail(WG_ERR_ARG, "contact_block must be 0, 64, 128, 256 or -256");
    if (chunk_steps < 1 || chunk_steps > 1024) return S.fail(WG_ERR_ARG, "chunk_steps must be in [1, 1024]");
    S.contactBlock = contact_block;
    S.chunkSteps = chunk_steps;
    if (launch_flags & ~(WG_LAUNCH_GRAPH | WG_LAUNCH_SERIAL)) return S.fail(WG_ERR_ARG, "unknown launch flag");
    S.useGraph = (launch_flags & WG_LAUNCH_GRAPH) != 0;
    S.concurrentContacts = (launch_flags & WG_LAUNCH_SERIAL) == 0;
    return WG_OK;
}

int wg_get_scene_stats(wg_scene* s, int32_t k, wg_stats* o) {
    if (!s || !o) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (k < 0 || k >= S.nScenes) return S.fail(WG_ERR_ARG, "scene index out of range");
    int r = S.syncContacts();
    if (r) return r;
    std::memset(o, 0, sizeof(*o));
    const wg_config& c = S.nScenes > 1 ? S.cfgs[k] : S.cfg;
    const int64_t done = S.step - S.cfg.step;
    o->step = c.step + done;
    o->time = S.nScenes > 1 ? S.bTime[k] : S.time;
    o->n_full_runs = S.nFullRuns;
    o->verlet_dist = S.nScenes > 1 && S.uploaded ? S.hPars[k].verletDist : S.hPar.verletDist;
    if (S.uploaded && S.C.n > 0) {
        const int64_t n = S.C.n;
        std::vector<uint32_t> fl(n);
        std::vector<uint64_t> key(n);
        WG_CUDA_TRY(cudaMemcpyAsync(fl.data(), S.C.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(key.data(), S.C.key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, S.stream));
        const int64_t p0 = S.nScenes > 1 ? S.sceneStart[k] : 0, p1 = S.nScenes > 1 ? S.sceneStart[k + 1] : S.nPar;
        for (int64_t c2 = 0; c2 < n; c2++) {
            const int64_t lo = (int64_t)(key[c2] >> 32);
            if (lo < p0 || lo >= p1 || (fl[c2] & C_REMOVED)) continue;
            o->n_contacts++;
            if (fl[c2] & C_REAL) o->n_real++;
        }
    }
    return WG_OK;
}

int wg_set_materials(wg_scene* s, int32_t n, const double* density, const double* young, const double* tan_phi,
                     const double* kt_div_kn) {
    if (!s || n < 0 || (n > 0 && (!density || !young || !tan_phi || !kt_div_kn))) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (S.uploaded) return S.fail(WG_ERR_STATE, "materials are fixed once the scene runs");
    S.hDensity.assign(density, density + n);
    S.hYoung.assign(young, young + n);
    S.hTanPhi.assign(tan_phi, tan_phi + n);
    S.hKtDivKn.assign(kt_div_kn, kt_div_kn + n);
    return WG_OK;
}

int wg_set_nodes(wg_scene* s, int64_t n, const double* pos, const double* ori, const double* vel, const double* ang_vel,
                 const double* force, const double* torque, const double* mass, const double* inertia, const uint32_t* flags) {
    if (!s || n < 0 || (n > 0 && (!pos || !ori || !vel || !ang_vel || !force || !torque || !mass || !inertia || !flags))) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (S.uploaded) return S.fail(WG_ERR_STATE, "use wg_put_state to change the state of a running scene");
    S.nApiNodes = n;
    S.hApi.resize(19 * n);
    std::memcpy(S.hApi.data(), pos, sizeof(double) * 3 * n);
    std::memcpy(S.hApi.data() + 3 * n, ori, sizeof(double) * 4 * n);
    std::memcpy(S.hApi.data() + 7 * n, vel, sizeof(double) * 3 * n);
    std::memcpy(S.hApi.data() + 10 * n, ang_vel, sizeof(double) * 3 * n);
    std::memcpy(S.hApi.data() + 13 * n, force, sizeof(double) * 3 * n);
    std::memcpy(S.hApi.data() + 16 * n, torque, sizeof(double) * 3 * n);
    S.hMass.assign(mass, mass + n);
    S.hInertia.assign(inertia, inertia + 3 * n);
    S.hFlagsApi.assign(flags, flags + n);
    return WG_OK;
}

int wg_set_particles(wg_scene* s, int64_t n, const int32_t* shape, const int32_t* nodes3, const double* radius,
                     const int32_t* wall_axis, const int32_t* wall_sense, const double* half_thick, const double* fake_vel,
                     const int32_t* mat, const uint32_t* mask) {
    if (!s || n < 0 || (n > 0 && (!shape || !nodes3 || !radius || !wall_axis || !wall_sense || !half_thick || !fake_vel || !mat || !mask)))
        return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (S.uploaded) return S.fail(WG_ERR_STATE, "particles are fixed once the scene runs; create a new scene");
    if (n >= (int64_t(1) << 31) - 2) return S.fail(WG_ERR_ARG, "too many particles");
    S.nPar = n;
    S.hShape.assign(shape, shape + n);
    S.hNodes3.assign(nodes3, nodes3 + 3 * n);
    S.hRadius.assign(radius, radius + n);
    S.hAxis.assign(wall_axis, wall_axis + n);
    S.hSense.assign(wall_sense, wall_sense + n);
    S.hHalfThick.assign(half_thick, half_thick + n);
    S.hFakeVel.assign(fake_vel, fake_vel + 3 * n);
    S.hMat.assign(mat, mat + n);
    S.hMask.assign(mask, mask + n);
    return WG_OK;
}

int wg_run(wg_scene* s, int64_t n_steps) {
    if (!s || n_steps < 0) return WG_ERR_ARG;
    return SIM(s)->run(n_steps);
}

int wg_collide_only(wg_scene* s) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.uploaded) {
        int r = S.upload();
        if (r) return r;
    }
    int r = collide_full_run(S);
    if (r) return r;
    S.initialized = true;
    S.fromEnds = false;  // the new incidence starts empty; the next step takes the stored forces
    WG_CUDA_TRY(cudaStreamSynchronize(S.stream));
    return WG_OK;
}

int wg_put_state(wg_scene* s, const double* pos, const double* ori, const double* vel, const double* ang_vel, const double* force,
                 const double* torque) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    SimEx& X = static_cast<SimEx&>(S);
    if (!S.uploaded) {
        // before the first run the description itself is replaced
        const int64_t n = S.nApiNodes;
        if (pos) std::memcpy(S.hApi.data(), pos, sizeof(double) * 3 * n);
        if (ori) std::memcpy(S.hApi.data() + 3 * n, ori, sizeof(double) * 4 * n);
        if (vel) std::memcpy(S.hApi.data() + 7 * n, vel, sizeof(double) * 3 * n);
        if (ang_vel) std::memcpy(S.hApi.data() + 10 * n, ang_vel, sizeof(double) * 3 * n);
        if (force) std::memcpy(S.hApi.data() + 13 * n, force, sizeof(double) * 3 * n);
        if (torque) std::memcpy(S.hApi.data() + 16 * n, torque, sizeof(double) * 3 * n);
        return WG_OK;
    }
    const int64_t na = S.nApiNodes;
    // staged: copies by the copy engines (they move page-locked arrays faster than kernels
    // reading host memory directly; one stream already fills the host link), one per run of
    // arrays adjacent in host memory, then the conversion into the node slots
    if (!(pos && ori && vel && ang_vel && force && torque)) {
        // fill missing components from the current device state
        k_get_state<<<(unsigned)((na + 255) / 256), 256, 0, S.stream>>>(S.N, X.dApiMap, na, stagedArrays(X.dStage, na));
    }
    {
        double* const host[6] = {const_cast<double*>(pos), const_cast<double*>(ori), const_cast<double*>(vel),
                                 const_cast<double*>(ang_vel), const_cast<double*>(force), const_cast<double*>(torque)};
        WG_CUDA_TRY(copyState(X.dStage, na, host, 0, 6, true, S.stream));
    }
    k_put_state<<<(unsigned)((na + 255) / 256), 256, 0, S.stream>>>(S.N, X.dApiMap, na, stagedArrays(X.dStage, na));
    S.fromEnds = false;  // the next step starts from the forces written here
    if (vel) S.facetsStatic = false;  // facet vertices may have been given a velocity
    launch_facet_prep(S.stream, S.N, S.P, nullptr);
    WG_CUDA_TRY(cudaGetLastError());
    WG_CUDA_TRY(cudaStreamSynchronize(S.stream));
    return WG_OK;
}

int wg_get_nodes(wg_scene* s, double* pos, double* ori, double* vel, double* ang_vel, double* force, double* torque) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    SimEx& X = static_cast<SimEx&>(S);
    const int64_t na = S.nApiNodes;
    double* dst[6] = {pos, ori, vel, ang_vel, force, torque};
    const int64_t off[6] = {0, 3, 7, 10, 13, 16}, w[6] = {3, 4, 3, 3, 3, 3};
    if (!S.uploaded) {
        for (int q = 0; q < 6; q++)
            if (dst[q]) std::memcpy(dst[q], S.hApi.data() + off[q] * na, sizeof(double) * w[q] * na);
        return WG_OK;
    }
    const int part = (pos || ori || vel || ang_vel) ? ((force || torque) ? 0 : 1) : 2;
    k_get_state<<<(unsigned)((na + 255) / 256), 256, 0, S.stream>>>(S.N, X.dApiMap, na, stagedArrays(X.dStage, na), part);
    WG_CUDA_TRY(copyState(X.dStage, na, dst, 0, 6, false, S.stream));
    WG_CUDA_TRY(cudaGetLastError());
    WG_CUDA_TRY(cudaStreamSynchronize(S.stream));
    return WG_OK;
}

namespace {
bool pageLocked(const void* p) {
    cudaPointerAttributes a;
    if (!p) return true;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}
}  // namespace

int wg_run_host(wg_scene* s, int64_t n_steps, double* pos, double* ori, double* vel, double* ang_vel, double* force, double* torque) {
    int r = wg_put_state(s, pos, ori, vel, ang_vel, force, torque);
    if (r) return r;
    Sim& S = *SIM(s);
    // with page-locked arrays the kinematic state leaves during the last contact loop (an async
    // copy into pageable memory would hold the host until it is done)
    if (n_steps < 1 || !(pageLocked(pos) && pageLocked(ori) && pageLocked(vel) && pageLocked(ang_vel))) {
        r = wg_run(s, n_steps);
        if (r) return r;
        return wg_get_nodes(s, pos, ori, vel, ang_vel, force, torque);
    }
    double* early[4] = {pos, ori, vel, ang_vel};
    for (int q = 0; q < 4; q++) S.earlyOut[q] = early[q];
    S.earlyWanted = true;
    S.earlyIssued = false;
    r = wg_run(s, n_steps);
    const bool issued = S.earlyIssued;
    S.earlyWanted = false;
    S.earlyIssued = false;
    for (int q = 0; q < 4; q++) S.earlyOut[q] = nullptr;
    // the caller's arrays are not touched after return: the early copies end here, failed run or not
    const cudaError_t e = issued ? cudaStreamSynchronize(S.earlySt) : cudaSuccess;
    if (r) return r;
    if (e != cudaSuccess) return S.fail(WG_ERR_CUDA, cudaGetErrorString(e));
    if (!issued) return wg_get_nodes(s, pos, ori, vel, ang_vel, force, torque);
    return wg_get_nodes(s, nullptr, nullptr, nullptr, nullptr, force, torque);
}

int wg_set_dt(wg_scene* s, double dt, double next_dt) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.haveCfg) return S.fail(WG_ERR_STATE, "wg_set_config must be called first");
    if (S.nScenes > 1) return S.fail(WG_ERR_UNSUPPORTED, "the scenes of a batch keep their dt");
    if (!(dt > 0) || !std::isfinite(dt)) return S.fail(WG_ERR_ARG, "Scene.dt must be positive and finite");
    if (dt != S.cfg.dt) {
        if (S.uploaded) {
            int r = S.applyDt(dt);
            if (r) return r;
        } else
            S.cfg.dt = dt;
    }
    S.nextDt = (next_dt > 0 && std::isfinite(next_dt)) ? next_dt : std::numeric_limits<double>::quiet_NaN();
    return WG_OK;
}

int wg_get_energy(wg_scene* s, double* values, int32_t* created) {
    if (!s || !values || !created) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.dEnergy) {
        for (int k = 0; k < WG_ENERGY_N; k++) {
            values[k] = 0;
            created[k] = 0;
        }
        return WG_OK;
    }
    WG_CUDA_TRY(cudaSetDevice(S.device));
    WG_CUDA_TRY(cudaMemcpyAsync(values, S.dEnergy, sizeof(double) * WG_ENERGY_N, cudaMemcpyDeviceToHost, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(created, S.dECreated, sizeof(int32_t) * WG_ENERGY_N, cudaMemcpyDeviceToHost, S.stream));
    WG_CUDA_TRY(cudaStreamSynchronize(S.stream));  // the destination may be page-locked
    return WG_OK;
}

int wg_set_energy(wg_scene* s, const double* values, const int32_t* created) {
    if (!s || !values || !created) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.haveCfg) return S.fail(WG_ERR_STATE, "wg_set_config must be called first");
    if (!S.trackE) return S.fail(WG_ERR_STATE, "the scene does not track energy");
    WG_CUDA_TRY(cudaSetDevice(S.device));
    if (!S.dEnergy) {
        int r = S.ensureEnergyCapacity();
        if (r) return r;
    }
    WG_CUDA_TRY(cudaMemcpyAsync(S.dEnergy, values, sizeof(double) * WG_ENERGY_N, cudaMemcpyHostToDevice, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(S.dECreated, created, sizeof(int32_t) * WG_ENERGY_N, cudaMemcpyHostToDevice, S.stream));
    return WG_OK;
}

int wg_get_dyndt(wg_scene* s, wg_dyndt_state* o) {
    if (!s || !o) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.haveCfg) return S.fail(WG_ERR_STATE, "wg_set_config must be called first");
    o->dt = S.cfg.dt;
    o->next_dt = S.nextDt;
    o->dyndt_dt = S.dd.dynDt;
    o->crit_dt = S.dd.critDt;
    o->n_done = S.dd.nDone;
    o->step_last = S.dd.stepLast;
    o->step_prev = S.dd.stepPrev;
    o->n_evals = S.dd.nEvals;
    o->virt_last = S.dd.virtLast;
    o->virt_prev = S.dd.virtPrev;
    return WG_OK;
}

int wg_get_scene_dyndt(wg_scene* s, int32_t k, wg_dyndt_state* o) {
    if (!s || !o) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (S.nScenes <= 1) return k == 0 ? wg_get_dyndt(s, o) : S.fail(WG_ERR_ARG, "scene index out of range");
    if (k < 0 || k >= S.nScenes || (int64_t)S.bdd.size() != S.nScenes) return S.fail(WG_ERR_ARG, "scene index out of range");
    const DynDtState& d = S.bdd[k];
    o->dt = S.cfgs[k].dt;
    o->next_dt = S.bNextDt[k];
    o->dyndt_dt = d.dynDt;
    o->crit_dt = d.critDt;
    o->n_done = d.nDone;
    o->step_last = d.stepLast;
    o->step_prev = d.stepPrev;
    o->n_evals = d.nEvals;
    o->virt_last = d.virtLast;
    o->virt_prev = d.virtPrev;
    return WG_OK;
}

int wg_get_stats(wg_scene* s, wg_stats* o) {
    if (!s || !o) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    int r = S.syncContacts();
    if (r) return r;
    std::memset(o, 0, sizeof(*o));
    o->step = S.step;
    o->time = S.time;
    o->n_full_runs = S.nFullRuns;
    o->n_contacts = S.uploaded ? S.C.n : 0;
    o->verlet_dist = S.hPar.verletDist;
    for (int q = 0; q < 9; q++) o->stress[q] = S.stress[q];
    if (S.uploaded && S.C.n > 0) {
        std::vector<uint32_t> fl(S.C.n);
        WG_CUDA_TRY(cudaMemcpyAsync(fl.data(), S.C.flags, sizeof(uint32_t) * S.C.n, cudaMemcpyDeviceToHost, S.stream));
        int64_t r = 0;
        for (uint32_t f : fl) r += (f & C_REAL) ? 1 : 0;
        o->n_real = r;
    }
    return WG_OK;
}

int wg_set_next_gradv(wg_scene* s, const double* g) {
    if (!s || !g) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    SimEx& X = static_cast<SimEx&>(S);
    for (int i = 0; i < 9; i++) S.cfg.cell_next_gradv[i] = g[i];
    if (S.uploaded) X.cell.nextGradV = fromRow(g);
    return WG_OK;
}

int wg_get_cell(wg_scene* s, double* hsize, double* trsf, double* gradv) {
    if (!s) return WG_ERR_ARG;
    SimEx& X = static_cast<SimEx&>(*SIM(s));
    if (!X.uploaded) {
        if (hsize) std::memcpy(hsize, X.cfg.cell_hsize, sizeof(double) * 9);
        if (trsf) std::memcpy(trsf, X.cfg.cell_trsf, sizeof(double) * 9);
        if (gradv) std::memcpy(gradv, X.cfg.cell_gradv, sizeof(double) * 9);
        return WG_OK;
    }
    if (hsize) toRow(X.cell.hSize, hsize);
    if (trsf) toRow(X.cell.trsf, trsf);
    if (gradv) toRow(X.cell.gradV, gradv);
    return WG_OK;
}

// Contacts listed the way the reference's container holds them after a step.
static int collectContacts(Sim& S, std::vector<int64_t>& keep, std::vector<uint64_t>& key, std::vector<uint32_t>& fl,
                           std::vector<int32_t>& cd, std::vector<std::vector<double>>& cols) {
    int r = S.syncContacts();
    if (r) return r;
    const int64_t n = S.C.n;
    key.resize(n); fl.resize(n); cd.resize(n);
    cols.assign(CC_NCOL + 3, std::vector<double>(n, 0.));  // + global force on pA
    if (n > 0) {
        // global force on pA from the end slots (pB's slot negated where pA is a facet)
        std::vector<int32_t> sLo(n), sHi(n);
        WG_CUDA_TRY(cudaMemcpyAsync(sLo.data(), S.I.slotLo, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(sHi.data(), S.I.slotHi, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        std::vector<uint32_t> flc(n);
        std::vector<uint64_t> kc(n);
        WG_CUDA_TRY(cudaMemcpyAsync(flc.data(), S.C.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(kc.data(), S.C.key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, S.stream));
        const int64_t ne = 2 * std::max<int64_t>(S.I.nAct, 1);
        std::vector<double> ef(4 * ne);
        if (S.prec == WG_PREC_FP32) {
            std::vector<float> tmp(4 * ne);
            WG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), S.I.endAf, sizeof(float4) * ne, cudaMemcpyDeviceToHost, S.stream));
            for (int64_t q = 0; q < 4 * ne; q++) ef[q] = tmp[q];
        } else {
            WG_CUDA_TRY(cudaMemcpyAsync(ef.data(), S.I.endA, sizeof(double4_32a) * ne, cudaMemcpyDeviceToHost, S.stream));
        }
        for (int64_t c = 0; c < n; c++) {
            const bool aIsLo = !(flc[c] & C_SWAP);
            const bool facetA = ctype(flc[c]) == CT_FS;
            const int32_t slot = facetA ? (aIsLo ? sHi[c] : sLo[c]) : (aIsLo ? sLo[c] : sHi[c]);
            const double sg = facetA ? -1.0 : 1.0;
            if (slot >= 0)
                for (int k = 0; k < 3; k++) cols[CC_NCOL + k][c] = sg * ef[4 * slot + k] + 0.0;
        }
    }
    if (n > 0) {
        WG_CUDA_TRY(cudaMemcpyAsync(key.data(), S.C.key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(fl.data(), S.C.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(cd.data(), S.C.cdist, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        if (S.prec == WG_PREC_FP64) {
            for (int q = 0; q < CC_NCOL; q++) WG_CUDA_TRY(cudaMemcpyAsync(cols[q].data(), S.C.col[q], sizeof(double) * n, cudaMemcpyDeviceToHost, S.stream));
        } else {
            // FP32-force mode: map the FP32 columns onto the FP64 listing layout
            std::vector<std::vector<float>> fc(CF_NCOL, std::vector<float>(n));
            for (int q = 0; q < CF_NCOL; q++) WG_CUDA_TRY(cudaMemcpyAsync(fc[q].data(), S.C.fcol[q], sizeof(float) * n, cudaMemcpyDeviceToHost, S.stream));
            std::vector<double> cp[3];
            for (int k = 0; k < 3; k++) {
                cp[k].resize(n);
                WG_CUDA_TRY(cudaMemcpyAsync(cp[k].data(), S.C.col[CC_CPX + k], sizeof(double) * n, cudaMemcpyDeviceToHost, S.stream));
            }
            std::vector<double4_32a> pos(S.nPar);
            WG_CUDA_TRY(cudaMemcpyAsync(pos.data(), S.N.posr, sizeof(double4_32a) * S.nPar, cudaMemcpyDeviceToHost, S.stream));
            for (int64_t c = 0; c < n; c++) {
                const int map[] = {CF_T0X, CF_T0Y, CF_T0Z, CF_T1X, CF_T1Y, CF_T1Z};
                for (int q = 0; q < 6; q++) cols[CC_T0X + q][c] = fc[map[q]][c];
                // phys.force (local) = trsf^T * (global force on pA), trsf = (c0, c1, c0 x c1)
                const double t0[3] = {fc[CF_T0X][c], fc[CF_T0Y][c], fc[CF_T0Z][c]};
                const double t1[3] = {fc[CF_T1X][c], fc[CF_T1Y][c], fc[CF_T1Z][c]};
                const double t2[3] = {t0[1] * t1[2] - t0[2] * t1[1], t0[2] * t1[0] - t0[0] * t1[2], t0[0] * t1[1] - t0[1] * t1[0]};
                const double F[3] = {cols[CC_NCOL][c], cols[CC_NCOL + 1][c], cols[CC_NCOL + 2][c]};
                cols[CC_FN][c] = t0[0] * F[0] + t0[1] * F[1] + t0[2] * F[2];
                cols[CC_FT1][c] = t1[0] * F[0] + t1[1] * F[1] + t1[2] * F[2];
                cols[CC_FT2][c] = t2[0] * F[0] + t2[1] * F[1] + t2[2] * F[2];
                if (ctype(fl[c]) == CT_SS) {
                    // contact point = x_A + (r_A + uN/2) n (Sphere.cpp:103)
                    const int a = (fl[c] & C_SWAP) ? (int)(key[c] & 0xffffffffu) : (int)(key[c] >> 32);
                    const double s = pos[a].w + 0.5 * (double)fc[CF_UN][c];
                    cols[CC_CPX][c] = pos[a].x + s * fc[CF_T0X][c];
                    cols[CC_CPY][c] = pos[a].y + s * fc[CF_T0Y][c];
                    cols[CC_CPZ][c] = pos[a].z + s * fc[CF_T0Z][c];
                } else {
                    for (int k = 0; k < 3; k++) cols[CC_CPX + k][c] = cp[k][c];
                }
                if (!(fl[c] & C_REAL))  // no geometry nor phys: the state arrays hold nothing for it
                    for (int q : {CC_T0X, CC_T0Y, CC_T0Z, CC_T1X, CC_T1Y, CC_T1Z, CC_FN, CC_FT1, CC_FT2, CC_CPX, CC_CPY, CC_CPZ})
                        cols[q][c] = 0.;
            }
        }
    }
    // every contact but those removed by the collider since the last full run (pending contacts
    // whose boxes stopped overlapping)
    keep.clear();
    for (int64_t c = 0; c < n; c++)
        if (!(fl[c] & C_REMOVED)) keep.push_back(c);
    return 0;
}

// the FP64 columns of the contact state in a snapshot: all in FP64 mode; in FP32-force mode
// those the mode keeps in FP64 (contact point, IdealElPl shear force), then the FP32 columns
static std::vector<int> snapshotCols64(const Sim& S) {
    std::vector<int> q;
    for (int c = 0; c < CC_NCOL; c++)
        if (S.C.col[c]) q.push_back(c);
    return q;
}
int32_t wg_contact_state_cols(wg_scene* s) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.haveCfg) return S.fail(WG_ERR_STATE, "wg_set_config must be called first");
    if (S.cfg.precision == WG_PREC_FP64) return CC_NCOL;
    return 5 + CF_NCOL;  // CC_FT1, CC_FT2, CC_CPX, CC_CPY, CC_CPZ and the FP32 columns
}

int wg_get_contact_state(wg_scene* s, int64_t cap, int64_t* n_out, uint64_t* key, uint32_t* flags, int32_t* step0, int32_t* cell_dist,
                         double* cols) {
    if (!s || !n_out) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    *n_out = 0;
    if (!S.uploaded) return WG_OK;
    int r = S.syncContacts();
    if (r) return r;
    WG_CUDA_TRY(cudaSetDevice(S.device));
    const int64_t n = S.C.n;
    std::vector<uint64_t> k(n);
    std::vector<uint32_t> f(n);
    std::vector<int32_t> s0(n), cd(n);
    if (n > 0) {
        WG_CUDA_TRY(cudaMemcpyAsync(k.data(), S.C.key, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(f.data(), S.C.flags, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(s0.data(), S.C.step0, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(cd.data(), S.C.cdist, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, S.stream));
    }
    std::vector<int64_t> keep;
    for (int64_t c = 0; c < n; c++)
        if (!(f[c] & C_REMOVED)) keep.push_back(c);
    *n_out = (int64_t)keep.size();
    if (cap < (int64_t)keep.size()) return keep.empty() ? WG_OK : WG_ERR_CAPACITY;
    if (keep.empty()) return WG_OK;
    if (!key || !flags || !step0 || !cell_dist || !cols) return WG_ERR_ARG;
    const std::vector<int> q64 = snapshotCols64(S);
    const int ncols = wg_contact_state_cols(s);
    std::vector<double> v(n);
    std::vector<float> vf(n);
    int col = 0;
    for (int q : q64) {
        WG_CUDA_TRY(cudaMemcpyAsync(v.data(), S.C.col[q], sizeof(double) * n, cudaMemcpyDeviceToHost, S.stream));
        for (size_t i = 0; i < keep.size(); i++) cols[(int64_t)i * ncols + col] = v[keep[i]];
        col++;
    }
    if (S.prec == WG_PREC_FP32)
        for (int q = 0; q < CF_NCOL; q++) {
            WG_CUDA_TRY(cudaMemcpyAsync(vf.data(), S.C.fcol[q], sizeof(float) * n, cudaMemcpyDeviceToHost, S.stream));
            for (size_t i = 0; i < keep.size(); i++) cols[(int64_t)i * ncols + col] = (double)vf[keep[i]];
            col++;
        }
    for (size_t i = 0; i < keep.size(); i++) {
        key[i] = k[keep[i]];
        flags[i] = f[keep[i]] & ~(uint32_t)C_DORMANT;
        step0[i] = s0[keep[i]];
        cell_dist[i] = cd[keep[i]];
    }
    return WG_OK;
}

int wg_set_contact_state(wg_scene* s, int64_t n, const uint64_t* key, const uint32_t* flags, const int32_t* step0,
                         const int32_t* cell_dist, const double* cols, int32_t ncols) {
    if (!s || n < 0 || (n > 0 && (!key || !flags || !step0 || !cell_dist || !cols))) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (ncols != wg_contact_state_cols(s)) return S.fail(WG_ERR_ARG, "contact state has a different column count (precision mode)");
    if (S.nScenes > 1) return S.fail(WG_ERR_UNSUPPORTED, "contact snapshots are per scene, not per batch");
    WG_CUDA_TRY(cudaSetDevice(S.device));
    if (!S.uploaded) {
        int r = S.upload();
        if (r) return r;
    }
    // the keys name existing particles, ascending; the type bits agree with the shapes
    for (int64_t i = 0; i < n; i++) {
        const int64_t lo = (int64_t)(key[i] >> 32), hi = (int64_t)(key[i] & 0xffffffffu);
        if (lo >= hi || hi >= S.nPar || (i > 0 && key[i] <= key[i - 1])) return S.fail(WG_ERR_ARG, "contact keys out of order or range");
        const bool sl = S.hShape[lo] == WG_SHAPE_SPHERE, sh = S.hShape[hi] == WG_SHAPE_SPHERE;
        const int32_t other = sl ? S.hShape[hi] : S.hShape[lo];
        const uint32_t ty = (sl && sh) ? CT_SS : ((sl || sh) ? (other == WG_SHAPE_FACET ? CT_FS : CT_WS) : CT_NONE);
        if (ctype(flags[i]) != ty || (flags[i] & C_REMOVED)) return S.fail(WG_ERR_ARG, "contact flags do not match the particles");
    }
    int r = S.ensureContactCapacity(std::max<int64_t>(n, 1));
    if (r) return r;
    if (n > 0) {
        std::vector<uint32_t> f(n);
        for (int64_t i = 0; i < n; i++) f[i] = flags[i] & ~(uint32_t)C_DORMANT;
        WG_CUDA_TRY(cudaMemcpyAsync(S.C.key, key, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(S.C.flags, f.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(S.C.step0, step0, sizeof(int32_t) * n, cudaMemcpyHostToDevice, S.stream));
        WG_CUDA_TRY(cudaMemcpyAsync(S.C.cdist, cell_dist, sizeof(int32_t) * n, cudaMemcpyHostToDevice, S.stream));
        const std::vector<int> q64 = snapshotCols64(S);
        std::vector<double> v(n);
        std::vector<float> vf(n);
        int col = 0;
        for (int q : q64) {
            for (int64_t i = 0; i < n; i++) v[i] = cols[i * ncols + col];
            WG_CUDA_TRY(cudaMemcpyAsync(S.C.col[q], v.data(), sizeof(double) * n, cudaMemcpyHostToDevice, S.stream));
            col++;
        }
        if (S.prec == WG_PREC_FP32)
            for (int q = 0; q < CF_NCOL; q++) {
                for (int64_t i = 0; i < n; i++) vf[i] = (float)cols[i * ncols + col];
                WG_CUDA_TRY(cudaMemcpyAsync(S.C.fcol[q], vf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, S.stream));
                col++;
            }
    }
    S.C.n = n;
    S.K.n = 0;
    S.packDirty = false;
    S.fromEnds = false;    // the first step takes the node forces as written by the host
    S.forceFull = true;    // and starts with a full run that merges these contacts
    return WG_OK;
}

int64_t wg_num_contacts(wg_scene* s) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.uploaded) return 0;
    std::vector<int64_t> keep;
    std::vector<uint64_t> key;
    std::vector<uint32_t> fl;
    std::vector<int32_t> cd;
    std::vector<std::vector<double>> cols;
    int r = collectContacts(S, keep, key, fl, cd, cols);
    if (r) return r;
    return (int64_t)keep.size();
}

int wg_get_contacts(wg_scene* s, int32_t* id_lo, int32_t* id_hi, int32_t* id_a, int32_t* real, int32_t* cell_dist, double* fglob,
                    double* local, double* cpt, double* trsf) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.uploaded) return WG_OK;
    std::vector<int64_t> keep;
    std::vector<uint64_t> key;
    std::vector<uint32_t> fl;
    std::vector<int32_t> cd;
    std::vector<std::vector<double>> cols;
    int r = collectContacts(S, keep, key, fl, cd, cols);
    if (r) return r;
    for (size_t i = 0; i < keep.size(); i++) {
        const int64_t c = keep[i];
        const int lo = (int)(key[c] >> 32), hi = (int)(key[c] & 0xffffffffu);
        const bool isReal = fl[c] & C_REAL;
        if (id_lo) id_lo[i] = lo;
        if (id_hi) id_hi[i] = hi;
        if (id_a) id_a[i] = (fl[c] & C_SWAP) ? hi : lo;
        if (real) real[i] = isReal ? 1 : 0;
        int a, b, cc;
        unpackCellDist(cd[c], a, b, cc);
        if (cell_dist) { cell_dist[3 * i] = a; cell_dist[3 * i + 1] = b; cell_dist[3 * i + 2] = cc; }
        for (int k = 0; k < 3; k++) {
            if (fglob) fglob[3 * i + k] = isReal ? cols[CC_NCOL + k][c] : 0.;
            if (local) local[3 * i + k] = isReal ? cols[CC_FN + k][c] : 0.;
            if (cpt) cpt[3 * i + k] = isReal ? cols[CC_CPX + k][c] : 0.;
        }
        if (trsf) {
            D3 c0{cols[CC_T0X][c], cols[CC_T0Y][c], cols[CC_T0Z][c]}, c1{cols[CC_T1X][c], cols[CC_T1Y][c], cols[CC_T1Z][c]};
            D3 c2 = cross(c0, c1);
            const D3 cc3[3] = {c0, c1, c2};
            for (int row = 0; row < 3; row++)
                for (int col = 0; col < 3; col++) trsf[9 * i + 3 * row + col] = isReal ? comp(cc3[col], row) : 0.;
        }
    }
    return WG_OK;
}

int wg_get_aabbs(wg_scene* s, double* mn, double* mx) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (!S.uploaded) return S.fail(WG_ERR_STATE, "no boxes before the first run");
    std::vector<double4_32a> a(S.nPar), b(S.nPar);
    WG_CUDA_TRY(cudaMemcpyAsync(a.data(), S.P.mn, sizeof(double4_32a) * S.nPar, cudaMemcpyDeviceToHost, S.stream));
    WG_CUDA_TRY(cudaMemcpyAsync(b.data(), S.P.mx, sizeof(double4_32a) * S.nPar, cudaMemcpyDeviceToHost, S.stream));
    for (int64_t i = 0; i < S.nPar; i++) {
        mn[3 * i] = a[i].x; mn[3 * i + 1] = a[i].y; mn[3 * i + 2] = a[i].z;
        mx[3 * i] = b[i].x; mx[3 * i + 1] = b[i].y; mx[3 * i + 2] = b[i].z;
    }
    return WG_OK;
}

int wg_profiler(int on) {
    cudaError_t e = on ? cudaProfilerStart() : cudaProfilerStop();
    return e == cudaSuccess ? WG_OK : WG_ERR_CUDA;
}

void* wg_host_alloc(int64_t bytes) {
    void* p = nullptr;
    if (bytes <= 0 || cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
void wg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

int wg_get_timing(wg_scene* s, double* total_ms, double* phase_ms4, int64_t* launches) {
    if (!s) return WG_ERR_ARG;
    Sim& S = *SIM(s);
    if (total_ms) *total_ms = S.lastTotalMs;
    if (phase_ms4)
        for (int q = 0; q < 4; q++) phase_ms4[q] = S.phaseMs[q];
    if (launches) *launches = S.lastLaunches;
    return WG_OK;
}

}  // extern "C"
