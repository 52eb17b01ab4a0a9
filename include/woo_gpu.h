/*
 * woo_gpu.h -- C ABI of the GB300 DEM hot path (libwoogpu.so).
 *
 * One call of wg_run(scene, n) performs n steps of the reference's engine list
 *     Leapfrog(reset=True) -> InsertionSortCollider -> ContactLoop
 * on the GPU. It replaces, per step:
 *   - Scene::doOneStep                    core/Scene.cpp:319-389 (engine sequencing, cell update)
 *   - Leapfrog::run                       pkg/dem/Leapfrog.cpp:103-255
 *   - InsertionSortCollider::run          pkg/dem/InsertionSortCollider.cpp:445-646
 *   - ContactLoop::run                    pkg/dem/ContactLoop.cpp:93-259 with the functors
 *       Cg2_Sphere_Sphere_L6Geom          pkg/dem/Sphere.cpp:88-109
 *       Cg2_Facet_Sphere_L6Geom           pkg/dem/Facet.cpp:235-288
 *       Cg2_Wall_Sphere_L6Geom            pkg/dem/Wall.cpp:45-79
 *       Cp2_FrictMat_FrictPhys            pkg/dem/FrictMat.cpp:13-44
 *       Cp2_FrictMat_HertzPhys            pkg/dem/Hertz.cpp:9-50
 *       Law2_L6Geom_FrictPhys_IdealElPl   pkg/dem/IdealElPl.cpp:12-122
 *       Law2_L6Geom_HertzPhys_DMT         pkg/dem/Hertz.cpp:58-182
 *
 * Conventions: plain host pointers and sizes, no CUDA or framework types. Every
 * function returns WG_OK (0) or a negative WG_ERR_* code; wg_last_error() gives
 * the message (the reference's exception text where one exists). Arrays are
 * row-major: 3 doubles per vector, 4 per quaternion (w,x,y,z).
 */
#ifndef WOO_GPU_H
#define WOO_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define WG_OK 0
#define WG_ERR_ARG (-1)          /* invalid argument / std::invalid_argument */
#define WG_ERR_CUDA (-2)         /* CUDA runtime failure */
#define WG_ERR_NAN (-3)          /* NaN force, IdealElPl.cpp:76-80 */
#define WG_ERR_UNSUPPORTED (-4)  /* engine/functor/attribute outside the GPU path */
#define WG_ERR_CAPACITY (-5)     /* a fixed-size buffer is too small */
#define WG_ERR_PERIODIC (-6)     /* particle spans over half the cell, InsertionSortCollider.cpp:945-949 */
#define WG_ERR_STATE (-7)        /* call sequence error (e.g. run before particles are set) */

enum { WG_SHAPE_SPHERE = 0, WG_SHAPE_WALL = 1, WG_SHAPE_FACET = 2 };
enum { WG_PREC_FP64 = 0, WG_PREC_FP32 = 1 };

/* Engine and functor attributes read by the hot path. Field names follow the
   reference attributes; see the comments for the owning class. */
typedef struct wg_config {
    double dt;                  /* Scene.dt */
    double gravity[3];          /* DemField.gravity */
    uint32_t lone_mask;         /* DemField.loneMask */
    int32_t deterministic;      /* Scene.deterministic (the GPU path is always deterministic) */
    int64_t step;               /* Scene.step at upload */
    double damping;             /* Leapfrog.damping */
    int32_t reset;              /* Leapfrog.reset (must be 1) */
    int32_t _pad0;
    double verlet_dist;         /* InsertionSortCollider.verletDist (<0: relative to min sphere radius) */
    double bo1_sphere_dist_factor; /* Bo1_Sphere_Aabb.distFactor */
    int32_t sort_axis;          /* InsertionSortCollider.sortAxis (no effect on the pair set) */
    int32_t apply_forces;       /* ContactLoop.applyForces */
    double cg2_ss_dist_factor;  /* Cg2_Sphere_Sphere_L6Geom.distFactor */
    int32_t trsf_renorm;        /* Cg2_Any_Any_L6Geom__Base.trsfRenorm */
    int32_t approx_mask;        /* Cg2_Any_Any_L6Geom__Base.approxMask */
    int32_t no_ratch;           /* Cg2_Any_Any_L6Geom__Base.noRatch */
    int32_t phys;               /* 0 Cp2_FrictMat_FrictPhys, 1 Cp2_FrictMat_HertzPhys */
    int32_t law;                /* 0 Law2_L6Geom_FrictPhys_IdealElPl, 1 Law2_L6Geom_HertzPhys_DMT */
    int32_t no_slip;            /* IdealElPl.noSlip */
    int32_t no_break;           /* IdealElPl.noBreak */
    int32_t no_frict;           /* IdealElPl.noFrict */
    double hz_poisson;          /* Cp2_FrictMat_HertzPhys.poisson */
    double hz_gamma;            /* Cp2_FrictMat_HertzPhys.gamma */
    double hz_en;               /* Cp2_FrictMat_HertzPhys.en */
    double hz_alpha;            /* Cp2_FrictMat_HertzPhys.alpha (must be 0: DMT branch) */
    int32_t hz_no_attraction;   /* Law2_L6Geom_HertzPhys_DMT.noAttraction */
    int32_t periodic;           /* Scene.periodic */
    int32_t homo_deform;        /* Cell.homoDeform */
    int32_t eval_stress;        /* ContactLoop.evalStress */
    double cell_hsize[9];       /* Cell.hSize, row-major */
    double cell_trsf[9];        /* Cell.trsf */
    double cell_gradv[9];       /* Cell.gradV */
    double cell_next_gradv[9];  /* Cell.nextGradV */
    int32_t precision;          /* WG_PREC_FP64 (plain) or WG_PREC_FP32 (FP32 contact math, FP64 accumulation) */
    int32_t _pad1;
    /* DynDt (pkg/dem/DynDt.hpp:19-23) as the engine after ContactLoop, with the activation of a
       PeriodicEngine (core/Engine.cpp:169-194) by step count and/or simulation time. dyndt = 0: no
       DynDt. The *_last/*_prev/n_done fields are the engine's counters at upload (stepLast < 0:
       never evaluated); wg_get_dyndt returns their current values. */
    int32_t dyndt;              /* 1: DynDt in the engine list */
    int32_t dyndt_dry_run;      /* DynDt.dryRun */
    int32_t dyndt_step_modulo;  /* PeriodicEngine.stepModulo */
    int32_t dyndt_init_run;     /* PeriodicEngine.initRun */
    int64_t dyndt_step_period;  /* PeriodicEngine.stepPeriod (<= 0: off) */
    int64_t dyndt_n_do;         /* PeriodicEngine.nDo (< 0: unlimited) */
    int64_t dyndt_n_done;       /* PeriodicEngine.nDone */
    int64_t dyndt_step_last;    /* PeriodicEngine.stepLast */
    int64_t dyndt_step_prev;    /* PeriodicEngine.stepPrev */
    double dyndt_virt_period;   /* PeriodicEngine.virtPeriod (<= 0: off) */
    double dyndt_virt_last;     /* PeriodicEngine.virtLast */
    double dyndt_virt_prev;     /* PeriodicEngine.virtPrev */
    double dyndt_max_rel_inc;   /* DynDt.maxRelInc */
    double dt_safety;           /* Scene.dtSafety */
    double next_dt;             /* Scene.nextDt (0 or NaN: none), taken as dt after the next step */
    double time;                /* Scene.time at upload */
    int32_t track_energy;       /* Scene.trackEnergy (FP64 mode, one scene) */
    int32_t kin_split;          /* Leapfrog.kinSplit */
} wg_config;

/* Scene.energy entries (EnergyTracker, core/EnergyTracker.hpp), in this order: the Leapfrog
   energies (Leapfrog.cpp:52-97), those of the contact laws (IdealElPl.cpp:25-90,
   Hertz.cpp:150-179) and the work of the periodic cell's velocity gradient on the contacts
   (ContactLoop.cpp:236-246, with ContactLoop.evalStress). kinetic, kinTrans, kinRot and elast
   hold the last step's value, the others accumulate. */
#define WG_ENERGY_N 11
#define WG_ENERGY_NAMES {"kinetic", "kinTrans", "kinRot", "grav", "nonviscDamp", "elast", "plast", "broken", "viscN", "viscT", "gradV"}

/* DynDt state after a run: Scene.dt and nextDt, the engine's counters and DynDt.dt (the dry-run
   value), and the last critical timestep computed (Inf: no stiff contact). */
typedef struct wg_dyndt_state {
    double dt, next_dt, dyndt_dt, crit_dt;
    int64_t n_done, step_last, step_prev, n_evals;
    double virt_last, virt_prev;
} wg_dyndt_state;

typedef struct wg_stats {
    int64_t step;               /* Scene.step */
    int64_t n_full_runs;        /* InsertionSortCollider.nFullRuns */
    int64_t n_contacts;         /* len(S.dem.con): potential + real */
    int64_t n_real;             /* S.dem.con.countReal() */
    double time;                /* Scene.time */
    double verlet_dist;         /* resolved InsertionSortCollider.verletDist */
    double stress[9];           /* ContactLoop.stress (periodic, evalStress) */
} wg_stats;

typedef struct wg_scene wg_scene;

/* Create an empty scene on CUDA device `device`. */
int wg_create(wg_scene** out, int device);
void wg_destroy(wg_scene* s);
/* Message of the last error on this scene (or of the last failed wg_create when s is NULL). */
const char* wg_last_error(const wg_scene* s);

/* Scene description. Nodes carry Node.pos/ori and DemData (pkg/dem/Particle.hpp:169-274);
   particles carry shape, material index and mask (pkg/dem/Particle.hpp:26-123).
   nodes3: 3 node indices per particle (-1 unused); wall_axis/wall_sense: Wall.axis/sense;
   half_thick/fake_vel: Facet.halfThick/fakeVel; radius: Sphere.radius. */
int wg_set_config(wg_scene* s, const wg_config* c);
/* Batch of independent scenes in one simulation (no counterpart in the reference, where each
   Scene is its own object; a batch runs many Scene.run loops at once). Scene k owns the particles
   [particle_start[k], particle_start[k+1]) (and the nodes they use) and has its own configuration
   cfgs[k] (dt, gravity, damping, verletDist, laws, Scene.step); particles of different scenes never
   interact. All scenes share the precision mode, loneMask and applyForces; periodic scenes are not
   batched. Replaces wg_set_config; call before the first run. */
int wg_set_scenes(wg_scene* s, int32_t n_scenes, const wg_config* cfgs, const int64_t* particle_start);
/* Launch shape (no counterpart in the reference): threads per block of the contact kernels
   (0 = default, 64, 128, 256; -256: the FP32 sphere-sphere contacts through a resident grid whose
   threads prefetch their next contact), steps
   queued per host check of the collider request (1..1024), and flags: WG_LAUNCH_GRAPH replays each
   such chunk of steps as one CUDA graph, WG_LAUNCH_SERIAL runs the facet/wall contacts before the
   sphere-sphere ones instead of beside them on a second stream. Results do not depend on these;
   only the speed does. */
#define WG_LAUNCH_GRAPH 1
#define WG_LAUNCH_SERIAL 2
int wg_set_launch(wg_scene* s, int32_t contact_block, int32_t chunk_steps, int32_t launch_flags);
/* Serving slots (no counterpart in the reference): the scenes of a batch (wg_set_scenes) are slots
   whose particle ranges bound the jobs they can hold. wg_slot_load puts a job (an aperiodic scene
   of n spheres and walls, its configuration, its n_mat materials indexed 0..n_mat-1, its step
   count) into slot k in place of whatever the slot held: the other slots keep running and keep
   their contacts; the job runs n_steps steps from the next one on and then stays frozen.
   wg_slot_clear empties slot k. wg_slot_status reports the steps a slot's job has done.
   wg_get_slot_nodes copies the state of the first n nodes of slot k. */
int wg_slot_load(wg_scene* s, int32_t k, const wg_config* cfg, int64_t n, const double* pos, const double* ori,
                 const double* vel, const double* ang_vel, const double* mass, const double* inertia,
                 const uint32_t* flags, const int32_t* shape, const double* radius, const int32_t* wall_axis,
                 const int32_t* wall_sense, const int32_t* mat, const uint32_t* mask, int32_t n_mat,
                 const double* density, const double* young, const double* tan_phi, const double* kt_div_kn,
                 int64_t n_steps);
int wg_slot_clear(wg_scene* s, int32_t k);
int wg_slot_status(wg_scene* s, int32_t k, int64_t* steps_done, int64_t* steps_end);
int wg_get_slot_nodes(wg_scene* s, int32_t k, int64_t n, double* pos, double* ori, double* vel, double* ang_vel,
                      double* force, double* torque);
/* Scene.step, Scene.time and the contacts (counted by their lower particle id) of scene k. */
int wg_get_scene_stats(wg_scene* s, int32_t k, wg_stats* out);
int wg_set_materials(wg_scene* s, int32_t n, const double* density, const double* young,
                     const double* tan_phi, const double* kt_div_kn);
int wg_set_nodes(wg_scene* s, int64_t n, const double* pos, const double* ori, const double* vel,
                 const double* ang_vel, const double* force, const double* torque,
                 const double* mass, const double* inertia, const uint32_t* flags);
int wg_set_particles(wg_scene* s, int64_t n, const int32_t* shape, const int32_t* nodes3,
                     const double* radius, const int32_t* wall_axis, const int32_t* wall_sense,
                     const double* half_thick, const double* fake_vel, const int32_t* mat,
                     const uint32_t* mask);

/* Advance n steps with device-resident state. */
int wg_run(wg_scene* s, int64_t n_steps);
/* Same step loop driven from host buffers (the reference keeps state in host objects):
   copies the node state in from host memory, runs n steps, copies it back out. */
int wg_run_host(wg_scene* s, int64_t n_steps, double* pos, double* ori, double* vel, double* ang_vel,
                double* force, double* torque);
/* Replace the dynamic node state (pos, ori, vel, angVel, force, torque) keeping contacts. */
int wg_put_state(wg_scene* s, const double* pos, const double* ori, const double* vel,
                 const double* ang_vel, const double* force, const double* torque);
int wg_get_nodes(wg_scene* s, double* pos, double* ori, double* vel, double* ang_vel,
                 double* force, double* torque);
int wg_get_stats(wg_scene* s, wg_stats* out);
/* Scene.dt/nextDt and the DynDt counters after the last run (DynDt::run, pkg/dem/DynDt.cpp:93-113;
   PeriodicEngine::isActivated, core/Engine.cpp:169-194). */
int wg_get_dyndt(wg_scene* s, wg_dyndt_state* out);
/* The same for scene k of a batch (wg_set_scenes) or serving slot k: each scene of a batch keeps
   its own DynDt counters, Scene.dt, Scene.nextDt and Scene.time (no counterpart in the reference:
   a reference scene is one process, pkg/dem/DynDt.cpp:93-113 per scene). */
int wg_get_scene_dyndt(wg_scene* s, int32_t k, wg_dyndt_state* out);
/* Scene.dt and Scene.nextDt set between runs (0 or NaN next_dt: none); one scene only. */
int wg_set_dt(wg_scene* s, double dt, double next_dt);
/* Scene.energy: the WG_ENERGY_N values and whether each entry exists (created by an addition);
   wg_set_energy replaces them (EnergyTracker.clear or a checkpoint). */
int wg_get_energy(wg_scene* s, double* values, int32_t* created);
int wg_set_energy(wg_scene* s, const double* values, const int32_t* created);
/* Set Cell.nextGradV (row-major) between runs (periodic scenes). */
int wg_set_next_gradv(wg_scene* s, const double* next_gradv);
int wg_get_cell(wg_scene* s, double* hsize, double* trsf, double* gradv);

/* Contacts as (lo id, hi id) rows in key order. id_a: Contact.pA; real: geom&&phys;
   cell_dist: Contact.cellDist for the (lo,hi) orientation; fglob: force on pA in
   global coordinates; local: phys.force; cpt: geom.node.pos; trsf: L6Geom.trsf. */
int64_t wg_num_contacts(wg_scene* s);
/* Contact container snapshot for checkpoint/resume (the reference serializes the
   ContactContainer with the Scene, lib/object/ObjectIO.hpp:28-90): every contact the collider
   keeps, in key order, with its key (lo << 32 | hi), flags, creation step, packed cell distance
   and the persistent state as `wg_contact_state_cols` doubles per contact (row-major; the
   columns depend on the precision mode). wg_get_contact_state with cap < the count returns
   WG_ERR_CAPACITY and the count in *n_out. wg_set_contact_state replaces the container of an
   uploaded (or not yet run) scene; its next step starts with a collider full run, which keeps
   the state of the real contacts, so a run resumed from wg_put_state + wg_set_contact_state
   continues as the saved one would have (FP64 mode: bitwise). No counterpart in the reference's
   C++ interface. */
int32_t wg_contact_state_cols(wg_scene* s);
int wg_get_contact_state(wg_scene* s, int64_t cap, int64_t* n_out, uint64_t* key, uint32_t* flags, int32_t* step0, int32_t* cell_dist,
                         double* cols);
int wg_set_contact_state(wg_scene* s, int64_t n, const uint64_t* key, const uint32_t* flags, const int32_t* step0,
                         const int32_t* cell_dist, const double* cols, int32_t ncols);
int wg_get_contacts(wg_scene* s, int32_t* id_lo, int32_t* id_hi, int32_t* id_a, int32_t* real,
                    int32_t* cell_dist, double* fglob, double* local, double* cpt, double* trsf);
/* Aabb.min/max per particle from the last full run (verletDist included), 3 doubles each. */
int wg_get_aabbs(wg_scene* s, double* mn, double* mx);
/* Run only the broad phase on the current positions (full run), no stepping. */
int wg_collide_only(wg_scene* s);

/* Mark the region a profiler started with "profile from start off" captures (1 = start, 0 = stop). */
int wg_profiler(int on);

/* Page-locked host memory for wg_run_host buffers (cudaMallocHost); NULL on failure. */
void* wg_host_alloc(int64_t bytes);
void wg_host_free(void* p);

/* Timing of the last wg_run, measured with CUDA events on the simulation stream:
   total milliseconds from the first to the last kernel of the run, the milliseconds spent
   in each kernel class (0 leapfrog, 1 contact, 2 reduce, 3 collider full runs), and the
   number of kernel launches. */
int wg_get_timing(wg_scene* s, double* total_ms, double* phase_ms4, int64_t* launches);

/* Allocation-free broad phase (no counterpart in the reference): for callers that must not
   allocate device memory -- a process whose device memory belongs to another runtime's pool
   (which forbids raw cudaMalloc/cudaFree), or a loop that cannot take the device-wide
   synchronisation of cudaMalloc/cudaFree.
   Given n sphere boxes in host memory (mn, mx: 3 doubles each; mask: Particle.mask) it
   returns in host memory the overlapping pairs -- closed 3-axis box overlap and the mask test
   of Collider::mayCollide with lone_mask -- sorted by (id_lo, id_hi), *n_pairs of them.
   All device scratch is one static __device__ array (about 13 MB, held by every GPU that
   loads the library until the process exits); n above 32768 or more than 262144 pairs is
   rejected with WG_ERR_CAPACITY, as is a pair count above cap (*n_pairs is still set to the
   true count); a NaN or infinite box coordinate is rejected with WG_ERR_ARG.
   The first call on a device resolves the scratch address (cudaGetSymbolAddress, with that
   device current) and should come before any stream capture; the address is kept for the
   life of the process, so the call must not be used after a cudaDeviceReset. Calls share the
   scratch: calls that overlap on the GPU (concurrent host threads on one device) race. It
   runs on the current device and the legacy default stream and returns after the result is
   in host memory. */
int wg_broadphase_noalloc(int32_t n, const double* mn, const double* mx, const uint32_t* mask, uint32_t lone_mask,
                          int64_t cap, int32_t* id_lo, int32_t* id_hi, int64_t* n_pairs);
/* Message of the last failed wg_broadphase_noalloc call on this thread. */
const char* wg_broadphase_noalloc_error(void);

/* Scene generation (host only): seeded random sequential insertion of n non-overlapping
   spheres, the role of SpherePack::makeCloud (lib/sphere-pack/SpherePack.hpp:75).
   region_kind 0: box lo..hi; 1: x-axis cylinder through (params[0],params[1]) of radius
   params[2], clipped at z <= params[3]; 2: periodic box lo..hi. Returns the number placed. */
int64_t wg_pack_rsa(int64_t n, const double* radii, const double* lo, const double* hi, int32_t region_kind,
                    const double* params, uint64_t seed, int64_t max_attempts, double* centers);
/* The same insertion on the current device, in rounds over a window of the lowest-indexed
   unplaced spheres: every sphere of the window draws a candidate (a hash of seed, index and
   attempt), a candidate clear of the placed spheres is accepted unless it overlaps the clear
   candidate of a lower-indexed sphere of its round, the others draw again. Arguments and result
   as wg_pack_rsa (the prefix of spheres before the first that found no place in max_attempts);
   the packing is a sequential insertion of its own, not wg_pack_rsa's sphere for sphere.
   -1: CUDA error, -2: invalid argument. */
int64_t wg_pack_rsa_device(int64_t n, const double* radii, const double* lo, const double* hi, int32_t region_kind,
                           const double* params, uint64_t seed, int64_t max_attempts, double* centers);

#ifdef __cplusplus
}
#endif
#endif
