/*
 * CPU oracle for the Woo DEM hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is the oracle: a plain C++17/OpenMP FP64 restatement of the
 * reference's per-step loop (Leapfrog -> InsertionSortCollider -> ContactLoop
 * with the Cg2/Cp2/Law2 functors). Only the test-suite, the smoke check and the
 * CPU-baseline leg of the benchmark load it. The product library never links,
 * loads or calls it.
 *
 * The reference (Woo, C++11 + Eigen3 + Boost) cannot be compiled in this
 * environment (no Eigen, no Boost), so this is a restatement written from the
 * reference sources; every function in woo_oracle.cpp cites the reference
 * file:line it follows.
 *
 * Parity pinning: the reference ships no golden vectors for this path. The
 * oracle is pinned against the reference's own known-answer tests
 * (py/tests/hertz.py, py/tests/pbc.py, the py/utils.py pWaveDt doctest) and the
 * analytic cases derived from the cited formulas (tests/test_oracle_kat.py).
 * Many-body per-step results are "parity unpinned" at the Eigen boundary: the
 * restatement performs the same operations in the same order as the reference
 * expressions, but no reference output exists to compare against bit-for-bit.
 */
#ifndef WOO_ORACLE_H
#define WOO_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Mirror of the fields of the reference's engine/functor attributes that the
   hot path reads. Layout identical to wg_config in include/woo_gpu.h so the
   tests can fill both from one description. */
typedef struct wo_config {
    double dt;
    double gravity[3];
    uint32_t lone_mask;
    int32_t deterministic;      /* 1: canonical linView order + serial force application */
    int64_t step;
    /* Leapfrog */
    double damping;
    int32_t reset;
    int32_t _pad0;
    /* InsertionSortCollider / Bo1_Sphere_Aabb */
    double verlet_dist;
    double bo1_sphere_dist_factor;
    int32_t sort_axis;
    /* ContactLoop */
    int32_t apply_forces;
    double cg2_ss_dist_factor;
    int32_t trsf_renorm;
    int32_t approx_mask;
    int32_t no_ratch;
    int32_t phys;               /* 0 Cp2_FrictMat_FrictPhys, 1 Cp2_FrictMat_HertzPhys */
    int32_t law;                /* 0 Law2_L6Geom_FrictPhys_IdealElPl, 1 Law2_L6Geom_HertzPhys_DMT */
    int32_t no_slip;
    int32_t no_break;
    int32_t no_frict;
    double hz_poisson;
    double hz_gamma;
    double hz_en;
    double hz_alpha;
    int32_t hz_no_attraction;
    /* periodic cell */
    int32_t periodic;
    int32_t homo_deform;
    int32_t eval_stress;
    double cell_hsize[9];       /* row-major 3x3 */
    double cell_trsf[9];
    double cell_gradv[9];
    double cell_next_gradv[9];
    int32_t precision;          /* ignored by the oracle (always FP64) */
    int32_t _pad1;
    /* DynDt engine after ContactLoop (pkg/dem/DynDt.hpp:19-23) and its PeriodicEngine counters */
    int32_t dyndt;
    int32_t dyndt_dry_run;
    int32_t dyndt_step_modulo;
    int32_t dyndt_init_run;
    int64_t dyndt_step_period;
    int64_t dyndt_n_do;
    int64_t dyndt_n_done;
    int64_t dyndt_step_last;
    int64_t dyndt_step_prev;
    double dyndt_virt_period;
    double dyndt_virt_last;
    double dyndt_virt_prev;
    double dyndt_max_rel_inc;
    double dt_safety;           /* Scene.dtSafety */
    double next_dt;             /* Scene.nextDt (NaN: none) */
    double time;                /* Scene.time at the start */
    int32_t track_energy;       /* Scene.trackEnergy */
    int32_t kin_split;          /* Leapfrog.kinSplit */
} wo_config;

typedef struct wo_dyndt_state {
    double dt, next_dt, dyndt_dt, crit_dt;
    int64_t n_done, step_last, step_prev, n_evals;
    double virt_last, virt_prev;
} wo_dyndt_state;

typedef struct wo_stats {
    int64_t step;
    int64_t n_full_runs;
    int64_t n_contacts;
    int64_t n_real;
    double time;
    double verlet_dist;
    double stress[9];
} wo_stats;

void* wo_create(void);
void wo_destroy(void* s);
const char* wo_last_error(void* s);
int wo_set_threads(void* s, int n);
int wo_set_config(void* s, const wo_config* c);
int wo_set_materials(void* s, int32_t n, const double* density, const double* young,
                     const double* tan_phi, const double* kt_div_kn);
int wo_set_nodes(void* s, int64_t n, const double* pos, const double* ori, const double* vel,
                 const double* ang_vel, const double* force, const double* torque,
                 const double* mass, const double* inertia, const uint32_t* flags);
int wo_set_particles(void* s, int64_t n, const int32_t* shape, const int32_t* nodes3,
                     const double* radius, const int32_t* wall_axis, const int32_t* wall_sense,
                     const double* half_thick, const double* fake_vel, const int32_t* mat,
                     const uint32_t* mask);
int wo_run(void* s, int64_t n_steps);
int wo_get_nodes(void* s, double* pos, double* ori, double* vel, double* ang_vel,
                 double* force, double* torque);
int wo_get_stats(void* s, wo_stats* out);
int wo_get_dyndt(void* s, wo_dyndt_state* out);
/* Scene.energy in the order kinetic, kinTrans, kinRot, grav, nonviscDamp, elast, plast, broken,
   viscN, viscT, gradV, and whether each entry exists */
int wo_get_energy(void* s, double* values, int32_t* created);
int64_t wo_num_contacts(void* s);
/* Contacts as (lo id, hi id) pairs plus state. Arrays sized n = wo_num_contacts.
   real: 1 if geom&&phys. fglob: global force on particle A (3/contact, zeros if
   not real). local: phys.force in the contact frame. cpt: contact point. */
int wo_get_contacts(void* s, int32_t* id_lo, int32_t* id_hi, int32_t* id_a, int32_t* real,
                    int32_t* cell_dist, double* fglob, double* local, double* cpt, double* trsf);
/* Run only the broad phase (full run) on the current positions, without stepping. */
int wo_collide_only(void* s);
/* periodic cell: hSize, trsf, gradV (row-major 3x3) */
int wo_get_cell(void* s, double* hsize, double* trsf, double* gradv);
/* Per-particle force/torque as applied by the last ContactLoop (the node arrays). */
int wo_kinetic_energy(void* s, double* ek);
/* Aabb.min/max of every particle as computed at the last full run (verletDist included). */
int wo_get_aabbs(void* s, double* mn, double* mx);

#ifdef __cplusplus
}
#endif
#endif
