// Internal declarations of the GB300 DEM hot path: device data layout, kernel
// launchers and the host-side simulation object behind the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <limits>
#include <string>
#include <vector>

#include "../../include/woo_gpu.h"

namespace wg {

// DemData flag bits (pkg/dem/Particle.hpp:179-186)
enum : uint32_t {
    F_DOF_ALL = 63u, F_DOF_RXRYRZ = 56u, F_CLUMPED = 64u, F_CLUMP = 128u, F_ENERGY_SKIP = 256u, F_GRAVITY_SKIP = 512u,
    F_DAMPING_SKIP = 2048u
};
// Energy tracking (Scene.trackEnergy, core/EnergyTracker.hpp): the slots of Scene.energy, in the
// order of WG_ENERGY_NAMES (include/woo_gpu.h). kinetic/kinTrans/kinRot/elast are reset every step.
enum { EN_KINETIC, EN_KINTRANS, EN_KINROT, EN_GRAV, EN_DAMP, EN_ELAST, EN_PLAST, EN_BROKEN, EN_VISCN, EN_VISCT, EN_GRADV, EN_N };
static_assert(EN_N == WG_ENERGY_N, "energy slots");
// One step's contributions of each node / active contact, SoA columns of `cap` doubles each: the
// values and, for the entries a zero addition creates, the number of additions.
enum { EN_NODE_K0, EN_NODE_K1, EN_NODE_GRAV, EN_NODE_DAMP, EN_NODE_NKIN, EN_NODE_NGRAV, EN_NODE_NCOL };
enum { EN_CON_ELAST, EN_CON_PLAST, EN_CON_BROKEN, EN_CON_VISCN, EN_CON_VISCT, EN_CON_NELAST, EN_CON_NBROKEN, EN_CON_NCOL };
struct EnergyCols {
    double* col = nullptr;  // EN_*_NCOL columns of cap entries
    int64_t cap = 0;
};
// contact flag bits
enum : uint32_t {
    C_REAL = 1u,     // geom && phys exist
    C_SWAP = 2u,     // pA is the hi id (functor order Facet/Wall first)
    C_PENDING = 16u, // law requested removal in the last ContactLoop
    C_DORMANT = 32u, // not real and too far apart to touch before the next full collider run
    C_REMOVED = 64u  // pending contact whose boxes no longer overlapped at the next collider run
};
enum { CT_SS = 0, CT_FS = 1, CT_WS = 2, CT_NONE = 3 };
__host__ __device__ inline uint32_t ctype(uint32_t fl) { return (fl >> 2) & 3u; }

// Per-scene constants read by the kernels (one entry per scene in the batch).
struct ScenePar {
    double dt;
    double g[3];
    double damping;
    double verletDist;
    double maxD2;
    double ssDistFactor;
    double bo1DistFactor;
    double hzViscConst;   // -sqrt(5)*log(en)/sqrt(log(en)^2+pi^2), Hertz.cpp:43
    double hzGamma;
    double hzPoisson;
    int32_t law, phys, reset, applyForces;
    int32_t trsfRenorm, approxMask, noRatch, noSlip, noBreak, noFrict, noAttraction, hzViscOn;
    int32_t periodic, homoDeform, hasGravity, evalStress;
    int32_t trackEnergy, kinSplit;   // Leapfrog energies this step (reallyTrackEnergy), Leapfrog.kinSplit
    uint32_t loneMask;
    float dtF, ssDfAbsF;  // FP32 copies read by the FP32-force kernels
    float gH[3], gL[3];   // gravity as double-float pairs (g = gH + gL)
    float dampingF, maxD2F;
    float reach2F;        // 2*verletDist in FP32 (dormant-contact test of the FP32-force mode)
    long long stepBase;   // Scene.step of this scene = device step counter - stepBase
    long long stepEnd;    // the scene is frozen once Scene.step reaches stepEnd (serving slots)
    // periodic cell, integrated on the host each step (core/Cell.cpp:81-120)
    double hSize[9], pprevHsize[9], gradV[9], nextGradV[9], dGradV[9], midGradV[9], shiftVelMat[9];
    double ImLL4hInv[9], IpLL4h[9], LmL[9], unshear[9];
    double deltaSpinVec[3], spinVec[3], cellSize[3], cellCos[3];
    int32_t hasShear, _pad2;
};

// Double-float mirror of a node: ph/pl = position and radius, vh/vl = velocity with angVel.x/.y
// in w (x = hi + lo).
struct __align__(64) Mirror {
    float4 ph, pl, vh, vl;
};
// Node-slot arrays (uninodal particle p owns slot p; facet vertices follow the particles).
struct DevNodes {
    int32_t n;
    double4_32a* posr;    // x y z radius
    double4_32a* vel;     // vx vy vz 0
    double4_32a* angv;    // wx wy wz 0
    double4_32a* ori;     // w x y z
    double4_32a* force;   // fx fy fz 0
    double4_32a* torque;  // tx ty tz 0
    double4_32a* minert;  // ix iy iz mass
    double4_32a* lastPos; // verlet reference position
    uint32_t* flags;
    // FP32-force mode: double-float mirrors written by Leapfrog for the sphere-sphere contacts
    // (x = hi + lo), one 64-byte record per node so that a contact gathers two adjacent sectors
    // per particle; wz = angVel.z
    Mirror* mir;
    float* wz;
    float4* orif;   // FP32-force mode: the orientation (w x y z), in place of ori
    float2* rsplit; // FP32-force mode: the radius as a double-float pair (constant)
    float4 *lh, *ll; // FP32-force mode: the position mirror at the last full run (verlet reference)
    int32_t* scene;  // batch of scenes: scene of each node slot (null: one scene)
    uint8_t* fresh;  // serving slots: node (re)loaded since its last step; Leapfrog takes its stored force
};
// FP32-force mode: the quantities of Cg2_Facet_Sphere_L6Geom that depend only on a facet's
// vertices (Facet.cpp:240-246 and the barycentric matrix of CompUtils::triangleBarycentrics),
// evaluated once per step for every facet instead of once per contact.
struct FacetPrep {
    double4_32a p0, p1, p2;  // vertices; w: the inverse barycentric matrix i00, i01, i10
    double4_32a n;           // unit normal; w: i11
    double4_32a e0, e1, e2;  // edge normals in the plane: (p1-p0) x nn, (p2-p1) x nn, (p0-p2) x nn
};
struct DevParticles {
    int32_t n;
    int32_t* shape;   // WG_SHAPE_*
    int4* aux;        // facet: node slots n0 n1 n2 and the facet's ordinal; wall: axis sense
    int32_t nFacets;
    int32_t* facetIds;  // particle id of each facet ordinal
    FacetPrep* prep;    // FP32-force mode: per facet ordinal
    double4_32a* facet;   // fakeVel xyz, halfThick
    int32_t* mat;
    uint32_t* mask;
    double4_32a* mn;      // Aabb.min (verletDist included)
    double4_32a* mx;      // Aabb.max
    int32_t* scene;       // batch of scenes: scene of each particle (null: one scene)
    uint8_t* fresh;       // serving slots: particle (re)loaded or parked since the last full run; its
                          // contacts do not survive that run
};
// the parameters of the scene a node or particle belongs to
__device__ __forceinline__ int sceneOfP(const DevParticles& P, int p) { return P.scene ? P.scene[p] : 0; }
__device__ __forceinline__ int sceneOfN(const DevNodes& N, int i) { return N.scene ? N.scene[i] : 0; }
enum {
    CC_T0X, CC_T0Y, CC_T0Z, CC_T1X, CC_T1Y, CC_T1Z,  // L6Geom.trsf columns 0 and 1 (column 2 = c0 x c1)
    CC_CPX, CC_CPY, CC_CPZ,                          // L6Geom node position (contact point)
    CC_P0, CC_P1, CC_P2, CC_P3, CC_P4,               // FrictPhys kn kt tanPhi | HertzPhys kn0 kt0 tanPhi alpha_sqrtMK R
    CC_FN, CC_FT1, CC_FT2,                           // phys.force (local)
    CC_UN0,                                          // L6Geom.uN of the contact's first step (L6Geom.lens)
    CC_NCOL
};
// FP32-force mode columns (the FP64 columns CC_FT1/CC_FT2 keep the IdealElPl shear force and
// CC_CPX..Z the contact point of facet and wall contacts in that mode)
enum {
    CF_T0X, CF_T0Y, CF_T0Z, CF_T1X, CF_T1Y, CF_T1Z,  // trsf columns 0 and 1
    CF_UN,                                           // L6Geom.uN of the last step
    CF_P0, CF_P1, CF_P2, CF_P3,                      // FrictPhys kn kt tanPhi | HertzPhys kn0 kt0 tanPhi alpha_sqrtMK
    CF_NCOL
};
struct DevContacts {
    int64_t n;
    uint64_t* key;    // (lo<<32)|hi, sorted ascending
    uint32_t* flags;
    int32_t* step0;   // Contact.stepCreated
    int32_t* cdist;   // Contact.cellDist for (lo,hi), packed 3x10 bits
    double* col[CC_NCOL];   // columns not used by the precision mode are null
    float* fcol[CF_NCOL];
};
// CSR incidence for the deterministic per-particle force sum.
// Particle p owns the end slots [hiStart[p]+loStart[p], hiStart[p+1]+loStart[p+1]): first its
// contacts with lower-id partners (ascending), then those with higher-id partners (ascending),
// i.e. the order in which the reference's deterministic pass over key-sorted contacts adds them
// (ContactLoop.cpp:250-257). The contact kernel stores each end's force and torque in its slot
// (zero while the contact is not real); the force sum reads each particle's slots as one
// contiguous run.
struct DevIncidence {
    int32_t* loStart;  // nPar+1: contacts with lo==p are [loStart[p], loStart[p+1])
    int32_t* hiStart;  // nPar+1: hiList[hiStart[p] .. hiStart[p+1]) are contacts with hi==p, ascending
    int32_t* hiList;
    int4* work;        // active contacts (contact, pA, pB, type|swap flag bits): those that are not
                       // sphere-sphere first, then the sphere-sphere ones, each in ascending order
    int64_t nAct;
    int32_t* slotLo;   // per contact: end slot of its lo particle (-1: no slot, the contact is inactive)
    int32_t* slotHi;   // per contact: end slot of its hi particle
    double4_32a* endA; // FP64 mode: (Fx, Fy, Fz, Tx) on the particle, torque about its node
    double2* endB;     // FP64 mode: (Ty, Tz)
    float4* endAf;     // FP32-force mode: the same in FP32
    float2* endBf;
    int64_t endCap;
    int32_t* heavy;      // [0, nHeavy): particles whose degree exceeds kHeavyThreshold
    int32_t* heavyFree;  // [0, nHeavyFree): those of them whose node has a free DOF
    int32_t nHeavy, nHeavyFree;
};
// FP32-force mode per-node constants, one 32-byte record read by Leapfrog instead of the
// inertia/mass and flag arrays: 1/m and 1/I per axis in FP32, the mass as a double-float pair
// (mass = mh + ml), the DemData flags.
struct NodeConst32 {
    float invMass;
    float invI[3];
    float mh, ml;
    uint32_t flags;
    uint32_t kind;  // NK_SUMMED: the node of a particle whose force is the sum of its end slots (not a facet)
};
enum : uint32_t { NK_SUMMED = 1u };
// Particles with more end slots than this are summed by a block tree instead of one lane.
constexpr int kHeavyThreshold = 64;
// End slots a warp of the FP32 Leapfrog stages per chunk (32 particles of ~6 contacts each fit
// one chunk; 8 warps x 256 x 24 bytes = 48 KB of shared memory per block).
constexpr int kLeapfrogChunk32 = 256;

// FP32-force mode, aperiodic scenes: the state of the active sphere-sphere contacts (work items
// [nMixed, nAct)) held in work-list order, so that the per-step kernel loads and stores it
// coalesced, with the particle ids and end slots beside it. Filled from the contact arrays at
// each full collider run and written back before the next one and before the host reads the
// contacts; the contact arrays hold the state of those contacts only after such a write-back.
struct DevPackedSS {
    int64_t n = 0, cap = 0;
    int4* item = nullptr;      // (pA, pB, end slot of pA, end slot of pB)
    uint32_t* flags = nullptr; // contact flags | scene << 8
    float* col[CF_NCOL] = {};
    double* ft[2] = {};        // IdealElPl shear force
    bool ftLive = false;       // ft is copied (some scene used IdealElPl at the last full run); it is
                               // read only for contacts of scenes with that law
};
// Step-loop flag words (device int[FL_WORDS]).
enum { FL_FULL = 0,   // set by Leapfrog: a node moved farther than verletDist, a full collider run is due
       FL_ERR = 1,    // error code raised by a kernel
       FL_HALT = 2,   // set by the contact kernel of a step that found FL_FULL: later queued steps do nothing
       FL_TICKET = 3, // blocks of the last contact kernel of a step that have finished (the last advances the step)
       FL_WORDS = 4 };

__host__ __device__ inline int32_t packCellDist(int a, int b, int c) {
    return (int32_t)(((uint32_t)(a + 512) & 1023u) | (((uint32_t)(b + 512) & 1023u) << 10) | (((uint32_t)(c + 512) & 1023u) << 20));
}
__host__ __device__ inline void unpackCellDist(int32_t p, int& a, int& b, int& c) {
    a = (int)(p & 1023) - 512;
    b = (int)((p >> 10) & 1023) - 512;
    c = (int)((p >> 20) & 1023) - 512;
}

// ------------------------------------------------------------------ launchers (wg_step.cu)
// One step is: [heavy sums] -> Leapfrog (with the force sum of the other particles fused in)
// -> (collider full run, host-driven) -> contact kernel -> step counter. Every per-step kernel
// takes the flag words and does nothing once FL_HALT or FL_ERR is set, so the host can queue
// several steps without waiting for each verlet test.
// fromEnds = 0: take DemData.force/torque as stored (first step after the host wrote the state).
void launch_leapfrog(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const ScenePar* sp,
                     int* dFlags, int fromEnds, const long long* dStep, bool periodic, const EnergyCols* energy = nullptr);
void launch_contact_fp64(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C,
                         const DevIncidence& I, const double4_32a* mats, const ScenePar* sp, const long long* dStep, int* dFlags,
                         bool periodic, int block = 128, const EnergyCols* energy = nullptr);
// perStep: only the heavy particles with a free DOF (guarded by the flags), before Leapfrog;
// otherwise every particle's DemData.force/torque (reporting at the end of a run).
void launch_forces(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const ScenePar* sp,
                   const int* dFlags, bool perStep);
void launch_advance(cudaStream_t st, long long* dStep, const int* dFlags);
// Adds one step's node (which = 0) or contact (which = 1) contributions in E to the energy slots;
// partial holds EN_CON_NCOL * 256 doubles.
// ContactLoop's gradV work of a periodic step from the step's stress sum (out of launch_stress);
// prev holds the previous stress (9) and cell volume (NaN at first).
void launch_energy_gradv(cudaStream_t st, const double* sum9, const ScenePar* sp, double* prev, double* energy, int32_t* created,
                         const int* dFlags);
void launch_energy_sum(cudaStream_t st, const EnergyCols& E, int which, int64_t n, double* partial, double* energy, int32_t* created,
                       const int* dFlags, bool kinSplit);
// DynDt: per-end stiffness of the real contacts into kA/kB (zeroed by the caller, I.endCap
// entries), then the minimum over nodes of the squared critical timestep into *out (initialised
// by the caller to the bits of +Inf). FP64 contact arrays, or with fp32 the FP32-force mode's
// (the packed sphere-sphere state written back first).
// perScene: out holds one value per scene of a batch (the minimum over that scene's nodes).
void launch_dyndt(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C, const DevIncidence& I,
                  const ScenePar* sp, double4_32a* kA, double2* kB, unsigned long long* out, int* dErr, bool periodic,
                  bool fp32 = false, bool perScene = false);
// sum over real contacts of F_A (x) branch into out[9] (not divided by the volume); scratch holds
// 9 doubles per 256 active contacts; returns -1 when it is too small
int launch_stress(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevContacts& C, const DevIncidence& I,
                  const ScenePar* sp, double* scratch, int64_t scratchDoubles, double* out);
// FP32-force mode (wg_step32.cu)
void launch_leapfrog32(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const NodeConst32* nc,
                       const ScenePar* sp, int* dFlags, int fromEnds, const long long* dStep, bool periodic,
                       const EnergyCols* energy = nullptr);
// The kernels walk the active contacts I.work[0, I.nAct). Items [0, nMixed) are facet and wall
// contacts; [nMixed, I.nAct) join two spheres and, in an aperiodic scene, go to a
// sphere-sphere-only kernel.
// With a side stream the mixed range runs beside the sphere-sphere range (joined on st).
struct SideStream {
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
// Returns true when the sphere-sphere kernel, last of the step, also advanced the step counter.
bool launch_contact_fp32(cudaStream_t st, const SideStream& side, const DevNodes& N, const DevParticles& P, const DevContacts& C,
                         const DevIncidence& I, const DevPackedSS& K, const double4_32a* mats, const ScenePar* sp,
                         long long* dStep, int* dFlags, int64_t nMixed, bool periodic, bool anyLaw0, bool prepFacets,
                         int block = 256, const EnergyCols* energy = nullptr);
// copy the packed sphere-sphere state from (pack) / back to (unpack) the contact arrays
void launch_pack_ss(cudaStream_t st, const DevContacts& C, const DevIncidence& I, const DevParticles& P, const DevPackedSS& K,
                    int64_t nMixed);
void launch_unpack_ss(cudaStream_t st, const DevContacts& C, const DevIncidence& I, const DevPackedSS& K, int64_t nMixed);
void launch_forces32(cudaStream_t st, const DevNodes& N, const DevParticles& P, const DevIncidence& I, const NodeConst32* nc,
                     const ScenePar* sp, const int* dFlags, bool perStep);
// FP32-force mode: P.prep from the current vertex positions (before the contact kernels of a step;
// dFlags null: unconditionally)
void launch_facet_prep(cudaStream_t st, const DevNodes& N, const DevParticles& P, const int* dFlags);

// ------------------------------------------------------------------ broad phase (wg_collide.cu)
struct Grid {
    double ox, oy, oz, h;
    int32_t nx, ny, nz;
    int64_t ncell;
    int64_t base;  // first cell key of this grid (a batch of scenes has one grid per scene)
};
struct CollideWork;  // scratch owned by the simulation
struct Sim;
int collide_full_run(Sim& S);

// DynDt after ContactLoop (pkg/dem/DynDt.hpp:19-23) with the counters of its PeriodicEngine.
struct DynDtState;
DynDtState dynDtFromConfig(const wg_config& c);
struct DynDtState {
    bool on = false, dryRun = false, stepModulo = true, initRun = true;
    int64_t stepPeriod = 0, nDo = -1, nDone = 0, stepLast = -1, stepPrev = -1, nEvals = 0;
    double virtPeriod = 0, virtLast = 0, virtPrev = 0, maxRelInc = 1e-4, dtSafety = 0.9;
    double dynDt = std::numeric_limits<double>::quiet_NaN();   // DynDt.dt (dry run)
    double critDt = std::numeric_limits<double>::infinity();    // last critical timestep
    // PeriodicEngine::isActivated (core/Engine.cpp:169-194) by step count and simulation time
    bool activated(int64_t stepNow, double virtNow) {
        const bool initNow = stepLast < 0;
        if (initNow) { virtLast = virtNow; stepLast = stepNow; }
        if ((nDo < 0 || nDone < nDo) &&
            ((virtPeriod > 0 && virtNow - virtLast >= virtPeriod) ||
             (stepPeriod > 0 && ((stepNow - stepLast >= stepPeriod) || (stepModulo && stepNow % stepPeriod == 0))))) {
            virtPrev = virtLast; virtLast = virtNow;
            stepPrev = stepLast; stepLast = stepNow;
            if (initNow && !initRun) return false;
            nDone++;
            return true;
        }
        return false;
    }
};

// ------------------------------------------------------------------ host simulation object
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct Sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    SideStream side;
    std::string err;
    wg_config cfg{};
    bool haveCfg = false;
    // host copies of the description
    std::vector<double> hDensity, hYoung, hTanPhi, hKtDivKn;
    int64_t nApiNodes = 0, nPar = 0;
    std::vector<int32_t> apiNodeToSlot;  // api node index -> slot
    std::vector<double> hApi;            // 19 doubles per api node: pos ori vel angVel force torque
    std::vector<double> hMass, hInertia;
    std::vector<uint32_t> hFlagsApi;
    std::vector<int32_t> hShape;
    std::vector<int32_t> hNodes3;
    std::vector<double> hRadius, hHalfThick, hFakeVel;
    std::vector<int32_t> hAxis, hSense, hMat;
    std::vector<uint32_t> hMask;
    int nSpheres = 0;
    // device state
    DevNodes N{};
    DevParticles P{};
    DevContacts C{}, Cb{};  // current and spare (merge target)
    DevIncidence I{};
    int64_t cCap = 0;
    int64_t nMixed = 0;   // work items [0, nMixed) are not sphere-sphere (see launch_contact_fp32)
    DevPackedSS K{};      // FP32-force mode: packed state of the active sphere-sphere contacts
    bool packDirty = false;  // K changed since it was last written back to the contact arrays
    double4_32a* dMats = nullptr;
    NodeConst32* dNodeC = nullptr;  // per node slot (FP32-force mode)
    int prec = 0;                  // WG_PREC_*
    ScenePar hPar{};
    ScenePar* dPar = nullptr;  // one per scene
    ScenePar* dParSeq = nullptr;  // periodic cell: the parameters of each step of a queued chunk
    int64_t parSeqCap = 0;
    // batch of independent scenes: scene k owns particles [sceneStart[k], sceneStart[k+1])
    int nScenes = 1;
    std::vector<wg_config> cfgs;
    std::vector<int64_t> sceneStart;
    std::vector<int32_t> hSceneOfPar;  // empty for one scene
    std::vector<ScenePar> hPars;
    std::vector<double> sceneTime0;    // Scene.time of each scene at upload
    std::vector<uint8_t> hParked;      // serving slots: particle holds no job (left out of the collider)
    bool listsDirty = true;            // particle lists of the collider to be rebuilt at the next full run
    bool forceFull = false;            // next step starts with a full collider run
    long long* dStep = nullptr;
    int* dFlags = nullptr;   // [0] full run requested, [1] error code
    int* hFlags = nullptr;   // pinned mirror
    std::vector<void*> allocs;
    CollideWork* cw = nullptr;
    bool uploaded = false, initialized = false;
    int64_t step = 0;
    double time = 0;
    int64_t nFullRuns = 0;
    bool fromEnds = false;   // the end slots hold the forces of the last contact loop
    // launch shape (wg_set_launch): threads per block of the contact kernels, steps queued per host
    // check, and whether a chunk of steps is replayed as a CUDA graph
    int contactBlock = 0;    // 0: default (FP32: the resident-grid sphere-sphere kernel; FP64: 128)
    int chunkSteps = 32;
    bool useGraph = false;
    bool concurrentContacts = true;   // facet/wall contacts beside, not before, the sphere-sphere ones
    bool facetsStatic = false;        // every facet vertex is fully blocked and at rest: FacetPrep is made once
    cudaGraphExec_t graphExec = nullptr;
    int64_t graphSteps = 0;  // steps in the captured chunk, 0: none valid
    int64_t graphEpoch = -1; // nFullRuns when it was captured
    int64_t graphLaunches = 0;
    double* dStress = nullptr;       // 9 doubles + per-block partials
    int64_t stressCap = 0;
    double stress[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // ContactLoop.stress of the last step
    // DynDt (one scene, FP64 mode): engine state, Scene.nextDt, Scene.time since the scene's
    // time 0 (for virtPeriod), and the scratch of the stiffness evaluation
    DynDtState dd;
    double nextDt = std::numeric_limits<double>::quiet_NaN();
    double timeAbs = 0;
    double4_32a* dKA = nullptr;
    double2* dKB = nullptr;
    int64_t kCap = 0;
    unsigned long long* dCrit = nullptr;
    // batch of scenes or serving slots (nScenes > 1) with DynDt or Scene.nextDt: per scene the
    // engine state, Scene.time (accumulated with the scene's own dt) and Scene.nextDt
    bool batchDyn = false;
    std::vector<DynDtState> bdd;
    std::vector<double> bTime, bNextDt;
    unsigned long long* dCritB = nullptr;  // one critical timestep (squared, as bits) per scene
    long long sceneStep(int k, long long deviceStep) const { return deviceStep - hPars[k].stepBase; }
    bool sceneFrozen(int k, long long deviceStep) const { return sceneStep(k, deviceStep) >= hPars[k].stepEnd; }
    int runDynDtScenes(const std::vector<char>& due, long long deviceStep);
    int applyDtScene(int k, double dt);
    // energy tracking (one scene, FP64 mode): Scene.energy on the device and the per-step scratch
    bool trackE = false;
    EnergyCols eNode, eCon;
    double* dEnergy = nullptr;      // WG_ENERGY_N values
    int32_t* dECreated = nullptr;   // WG_ENERGY_N flags
    double* dEPartial = nullptr;    // EN_CON_NCOL * 256 block partials
    double* dEPrev = nullptr;       // periodic gradV work: previous stress (9) and volume
    int ensureEnergyCapacity();
    // timing
    std::vector<cudaEvent_t> evPool;  // per queued step: before Leapfrog, before contacts, after
    cudaEvent_t ev[8];
    double lastTotalMs = 0, phaseMs[4] = {0, 0, 0, 0};
    int64_t lastLaunches = 0;
    // wg_run_host: the node state the last Leapfrog of a run leaves (position, orientation,
    // velocity, angular velocity) is copied to the caller's page-locked arrays on a stream of its
    // own while that step's contact loop runs; earlyOut are those arrays (null: not wanted)
    cudaStream_t earlySt = nullptr;
    cudaEvent_t earlyFork = nullptr;
    double* earlyOut[4] = {nullptr, nullptr, nullptr, nullptr};
    bool earlyWanted = false, earlyIssued = false;
    int issueEarlyGet();

    ~Sim();
    void* dalloc(size_t bytes);
    void dfree(void* p);
    int fail(int code, const std::string& m) { err = m; return code; }
    int upload();
    int prepareParams();
    int prepareParamsFor(const wg_config& c, int64_t p0, int64_t p1, ScenePar& out);
    int run(int64_t n);
    int applyDt(double dt);
    int runDynDt(int64_t stepNow);
    int checkErr();
    int ensureContactCapacity(int64_t need);
    // write the packed sphere-sphere state back to the contact arrays if needed; hostWait: also wait
    // for it (the host reads the arrays next), else it is only queued on the simulation stream
    int syncContacts(bool hostWait = true);
};

#define WG_CUDA_TRY(expr)                                                                  \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess) return S.fail(WG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

}  // namespace wg
