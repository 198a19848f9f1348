/*
 * posidonius_gb300.h -- C ABI of the GB300-native WHFast + tidal-effects path.
 *
 * The reference (Posidonius, Rust) has no C FFI: its surface is the JSON case
 * format, the `posidonius start|resume` flow and the Rust entry points
 * `Universe::new`, `WHFast::new`, the `Integrator` trait and the `Universe`
 * methods.  Every entry point below replaces one of those; the comment of each
 * cites the reference item it stands for (paths inside the posidonius project).
 *
 * Conventions
 *  - Plain pointers and sizes only; no C++ or torch types cross this boundary.
 *  - Every function returns a POSI_* status code (0 = success); physics events
 *    that make the reference `panic!` are reported as codes instead.
 *  - The library owns all device memory; the caller owns handles and must
 *    release them with the matching destroy call.  One CUDA stream per handle;
 *    calls on one handle are not thread-safe.
 *  - All arithmetic is IEEE FP64.
 */
#ifndef POSIDONIUS_GB300_H
#define POSIDONIUS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum posi_status {
    POSI_OK = 0,
    POSI_COMPLETED = 1,          /* src/integrator/whfast.rs:300-301 Err("Simulation completed") */
    POSI_ERR_ARG = -1,           /* bad argument / null pointer */
    POSI_ERR_IO = -2,            /* file missing or unreadable (src/integrator/output.rs:178-203) */
    POSI_ERR_PARSE = -3,         /* malformed JSON case */
    POSI_ERR_UNSUPPORTED = -4,   /* case uses an effect outside this path (Kaula, creep,
                                    dynamic tides, non-WHFast integrator, ...) */
    POSI_ERR_CUDA = -5,          /* CUDA runtime error or no device */
    POSI_ERR_PHYSICS = -6,       /* a system hit a reference panic (see posi_system_status) */
    POSI_ERR_STATE = -7          /* call not valid in this state (e.g. initialise a resumed run) */
};

/* Per-system status word (sys_i64[POSI_SI_STATUS]).  The low byte holds the
 * fatal event that froze the system; higher bits are sticky warnings. */
enum posi_system_status {
    POSI_SYS_OK = 0,
    POSI_SYS_ROCHE = 1,          /* src/particles/universe.rs:225-228 destroyed by close encounter */
    POSI_SYS_COLLISION = 2,      /* src/particles/universe.rs:230-233 radii overlap */
    POSI_SYS_EJECTED = 3,        /* src/particles/universe.rs:234-237 beyond MAX_DISTANCE */
    POSI_SYS_ZERO_INERTIA = 4,   /* src/particles/common.rs:5-7 moment of inertia is zero */
    POSI_SYS_BISECTION_LIMIT = 5,/* Kepler bisection did not close (src/integrator/whfast.rs:792-805) */
    POSI_SYS_COMPLETED = 6,      /* time limit reached; the system is frozen */
    POSI_SYS_FATAL_MASK = 0xff,
    POSI_SYS_WARN_NONCONVERGED = 1 << 8,  /* src/integrator/whfast.rs:389-391 */
    POSI_SYS_WARN_TIMESTEP = 1 << 9       /* src/integrator/whfast.rs:702-707 */
};

/* ---- flat system layout ---------------------------------------------------
 * One system = sys_i64[POSI_SI_COUNT] + sys_f64[POSI_SF_COUNT]
 *            + nmax bodies of body_i64[POSI_BI_COUNT] + body_f64[POSI_BF_COUNT].
 * Host arrays are row-major: system s, body b, field f lives at
 * body_f64[(s*nmax + b)*POSI_BF_COUNT + f].  Bodies keep the reference's
 * particle order (the host may sit at any index).
 */
enum posi_coords { POSI_JACOBI = 0, POSI_DEMOCRATIC_HELIOCENTRIC = 1, POSI_WHDS = 2 };
/* Integrator of a system (src/integrator/mod.rs): WHFast (src/integrator/whfast.rs)
 * or IAS15 (src/integrator/ias15.rs).  A batch holds systems of one integrator.
 * For IAS15, sys_f64[POSI_SF_DT] is the adaptive Ias15.time_step and
 * POSI_SF_HALF_DT, POSI_SI_COORDS and the WHFast error fields are unused. */
enum posi_integrator { POSI_INTEGRATOR_WHFAST = 0, POSI_INTEGRATOR_IAS15 = 1 };
enum posi_effect_kind { POSI_EFFECT_DISABLED = 0, POSI_EFFECT_CENTRAL = 1, POSI_EFFECT_ORBITING = 2 };
/* GeneralRelativityImplementation (src/effects/general_relativity.rs) */
enum posi_gr_impl { POSI_GR_KIDDER1995 = 0, POSI_GR_ANDERSON1975 = 1, POSI_GR_NEWHALL1983 = 2 };
enum posi_evolution {
    POSI_EVO_NON_EVOLVING = 0,
    POSI_EVO_LECONTE2011 = 1,
    POSI_EVO_BARAFFE1998 = 2,
    POSI_EVO_BARAFFE2015 = 3,
    POSI_EVO_LECONTE_CHABRIER2013 = 4,    /* LeconteChabrier2013(false) */
    POSI_EVO_BOLMONT_MATHIS2016 = 5,      /* dynamical tides (a tidal host only); its */
    POSI_EVO_GALLET_BOLMONT2017 = 6       /* table's 4th column holds inverse_tidal_q_factor */
};

enum posi_sys_i64_field {
    POSI_SI_N = 0,               /* Universe::n_particles */
    POSI_SI_HOST,                /* Hosts.index.most_massive (also tides/flattening/GR host) */
    POSI_SI_COORDS,              /* WHFast.alternative_coordinates_type */
    POSI_SI_TIDES,               /* ConsiderEffects.tides */
    POSI_SI_FLAT,                /* ConsiderEffects.rotational_flattening */
    POSI_SI_GR,                  /* ConsiderEffects.general_relativity */
    POSI_SI_EVOLUTION,           /* ConsiderEffects.evolution */
    POSI_SI_ITERATION,           /* WHFast.current_iteration */
    POSI_SI_N_HIST,              /* WHFast.n_historic_snapshots */
    POSI_SI_TIMESTEP_WARNING,    /* WHFast.timestep_warning */
    POSI_SI_STATUS,              /* posi_system_status word */
    POSI_SI_FAIL_STEP,           /* iteration at which a fatal event froze the system */
    POSI_SI_FAIL_PAIR,           /* i*1024 + j of the offending pair */
    POSI_SI_LAST_MIDPOINT_ITERS, /* midpoint iterations of the last half kick */
    POSI_SI_GR_IMPL,             /* Universe.general_relativity_implementation (posi_gr_impl) */
    POSI_SI_WIND,                /* ConsiderEffects.wind */
    POSI_SI_DISK,                /* ConsiderEffects.disk */
    POSI_SI_INTEGRATOR,          /* posi_integrator: the case document's integrator */
    POSI_SI_IAS_MAX_EXCEEDED,    /* Ias15.integrator_iterations_max_exceeded */
    POSI_SI_COUNT
};

enum posi_sys_f64_field {
    POSI_SF_DT = 0,              /* WHFast.time_step */
    POSI_SF_HALF_DT,             /* WHFast.half_time_step */
    POSI_SF_TIME,                /* WHFast.current_time */
    POSI_SF_TIME_LIMIT,          /* Universe.time_limit */
    POSI_SF_LAST_HIST,           /* WHFast.last_historic_snapshot_time */
    POSI_SF_HIST_PERIOD,         /* WHFast.historic_snapshot_period */
    POSI_SF_LAST_REC,            /* WHFast.last_recovery_snapshot_time */
    POSI_SF_REC_PERIOD,          /* WHFast.recovery_snapshot_period */
    POSI_SF_INITIAL_TIME,        /* Universe.initial_time */
    POSI_SF_IAS_DT_LAST,         /* Ias15.time_step_last_success */
    POSI_SF_COUNT
};

enum posi_body_i64_field {
    POSI_BI_TIDES_KIND = 0,      /* TidesEffect: posi_effect_kind (ConstantTimeLag model) */
    POSI_BI_FLAT_KIND,           /* RotationalFlatteningEffect: posi_effect_kind (OblateSpheroid) */
    POSI_BI_GR_KIND,             /* GeneralRelativityEffect: posi_effect_kind */
    POSI_BI_EVO_TYPE,            /* posi_evolution */
    POSI_BI_EVO_OFFSET,          /* offset of this body's tables in `tables` */
    POSI_BI_EVO_LEN,             /* rows per table (time, radius, rg2, love: 4*len doubles) */
    POSI_BI_EVO_LEFT,            /* Evolver.left_index */
    POSI_BI_WIND_KIND,           /* WindEffect: 1 Interaction, 0 Disabled */
    POSI_BI_DISK_KIND,           /* DiskEffect: posi_effect_kind */
    POSI_BI_COUNT
};

enum posi_body_f64_field {
    POSI_BF_MASS = 0, POSI_BF_MASS_G, POSI_BF_RADIUS, POSI_BF_RG2, POSI_BF_MOI,
    POSI_BF_PX, POSI_BF_PY, POSI_BF_PZ,          /* inertial_position */
    POSI_BF_VX, POSI_BF_VY, POSI_BF_VZ,          /* inertial_velocity */
    POSI_BF_AX, POSI_BF_AY, POSI_BF_AZ,          /* inertial_acceleration (Newtonian) */
    POSI_BF_LX, POSI_BF_LY, POSI_BF_LZ,          /* angular_momentum */
    POSI_BF_SX, POSI_BF_SY, POSI_BF_SZ,          /* spin */
    POSI_BF_NSV2,                                /* norm_spin_vector_2 */
    POSI_BF_EVX, POSI_BF_EVY, POSI_BF_EVZ,       /* WHFast.inertial_velocity_errors */
    POSI_BF_ELX, POSI_BF_ELY, POSI_BF_ELZ,       /* WHFast.particle_angular_momentum_errors */
    POSI_BF_SIGMA,                               /* tides scaled_dissipation_factor */
    POSI_BF_K2,                                  /* tides (ConstantTimeLag) love_number */
    POSI_BF_K2F,                                 /* flattening (OblateSpheroid) love_number */
    POSI_BF_ADDAX, POSI_BF_ADDAY, POSI_BF_ADDAZ, /* inertial_additional_acceleration */
    POSI_BF_DLX, POSI_BF_DLY, POSI_BF_DLZ,       /* dangular_momentum_dt */
    POSI_BF_DENERGY_DT,                          /* tides denergy_dt (history output) */
    POSI_BF_LAG_ANGLE,                           /* tides lag_angle (history output) */
    /* tidal internals of the last evaluation (TidesParticleInternalParameters and
     * coordinates, src/effects/tides/common.rs:35-79), read by the historic
     * snapshot's dE/dt (src/effects/tides/common.rs:263-279) */
    POSI_BF_TD_DIST, POSI_BF_TD_VR, POSI_BF_TD_ORTHO, POSI_BF_TD_DPM,
    POSI_BF_TD_PX, POSI_BF_TD_PY, POSI_BF_TD_PZ,
    POSI_BF_TD_VX, POSI_BF_TD_VY, POSI_BF_TD_VZ,
    POSI_BF_TD_LX, POSI_BF_TD_LY, POSI_BF_TD_LZ,
    /* wind (src/effects/wind.rs:6-15): input k_factor, rotation_saturation,
     * internal rotation_saturation_2 */
    POSI_BF_WIND_K, POSI_BF_WIND_RSAT, POSI_BF_WIND_RSAT2,
    /* ConstantTimeLag input dissipation_factor and dissipation_factor_scale
     * (src/effects/tides/constant_time_lag.rs:13-19), read by the dynamical
     * tide of a BolmontMathis2016 / GalletBolmont2017 host */
    POSI_BF_DISS_FACTOR, POSI_BF_DISS_SCALE,
    /* DiskProperties of a disk host (src/effects/disk.rs:6-14) */
    POSI_BF_DISK_INNER, POSI_BF_DISK_OUTER, POSI_BF_DISK_LIFETIME, POSI_BF_DISK_ALPHA,
    POSI_BF_DISK_SIGMA0, POSI_BF_DISK_MU,
    POSI_BF_DISK_MTS,                            /* disk migration_timescale of the last evaluation (history output) */
    POSI_BF_COUNT
};

/* IAS15 per-body state (src/integrator/ias15.rs:28-224, the fields that carry
 * over from one step to the next), body_ias[(s*nmax + b)*POSI_IAS_COUNT + f]:
 * the Gauss-Radau coefficients b_0..b_6, their predictions e_0..e_6, the
 * last accepted br_0..br_6 and er_0..er_6, the same four sets for the spin
 * angular momentum (sb, se, sbr, ser), and the compensated-summation terms
 * csx, csv, css.  Set k of a field block holds its three components at
 * block + 3*k + {0, 1, 2}. */
enum posi_ias15_field {
    POSI_IAS_B = 0, POSI_IAS_E = 21, POSI_IAS_BR = 42, POSI_IAS_ER = 63,
    POSI_IAS_SB = 84, POSI_IAS_SE = 105, POSI_IAS_SBR = 126, POSI_IAS_SER = 147,
    POSI_IAS_CSX = 168, POSI_IAS_CSV = 171, POSI_IAS_CSS = 174,
    POSI_IAS_COUNT = 177
};

/* Largest body count of the batched kernels. */
#define POSI_MAX_BODIES 32

/* Arithmetic modes.  EXACT keeps the reference's operation order with no FMA
 * contraction and reproduces the Rust FP64 results bit for bit; FAST lets the
 * compiler contract FMAs and shares reciprocals (<= 1e-12 relative per step). */
enum posi_mode { POSI_MODE_EXACT = 0, POSI_MODE_FAST = 1 };

/* Thread mappings of the batched kernel (bodies per lane group). */
enum posi_mapping {
    POSI_MAP_AUTO = 0,           /* autotuned per body-count bucket */
    POSI_MAP_THREAD = 1,         /* one thread per system: not built, refused with POSI_ERR_UNSUPPORTED */
    POSI_MAP_LANES2 = 2,         /* 2 lanes per system (one body per lane) */
    POSI_MAP_LANES4 = 4,         /* 4 lanes per system */
    POSI_MAP_LANES8 = 8,
    POSI_MAP_LANES16 = 16,
    POSI_MAP_WARP = 32           /* one warp per system */
};

typedef struct posi_handle posi_handle;
typedef struct posi_batch posi_batch;

/* ---- library ----------------------------------------------------------- */
const char* posi_version(void);
const char* posi_status_string(int status);
/* Human-readable detail of the last failing call on this thread. */
const char* posi_last_error(void);
/* Number of CUDA devices visible (0 when none); never allocates. */
int posi_device_count(void);

/* ---- case files ---------------------------------------------------------- */

/* src/integrator/output.rs:205-241 deserialize_json_snapshot, without the GPU:
 * parse a WHFast JSON case into the flat layout.  Call once with null arrays
 * to learn *n and *n_tables, then with buffers of POSI_SI_COUNT,
 * POSI_SF_COUNT, n*POSI_BI_COUNT, n*POSI_BF_COUNT, n_tables and n*n elements. */
int posi_read_case(const char* path, int64_t* n, int64_t* n_tables, int64_t* sys_i64, double* sys_f64,
                   int64_t* body_i64, double* body_f64, double* tables, double* roche);

/* IAS15 cases: the per-body Gauss-Radau state of the case (n*POSI_IAS_COUNT
 * doubles, posi_ias15_field layout).  POSI_ERR_STATE for a WHFast case. */
int posi_read_case_ias15(const char* path, double* body_ias);

/* ---- single system (the drop-in path: one system, one launch per step) -- */

/* src/integrator/output.rs:178-279 restore_snapshot + deserialize_json_snapshot
 * / deserialize_bin_snapshot: read a WHFast or Ias15 case or recovery
 * snapshot -- JSON when the path's extension is "json", bincode otherwise
 * (WHFast tried first, then Ias15), as the reference decides. */
posi_handle* posi_universe_from_json(const char* path, int mode, int* status);

/* src/particles/universe.rs:73-175 Universe::new + src/integrator/whfast.rs:143-165
 * WHFast::new, from one system in the flat layout (nmax = n).  roche: n*n
 * Roche radii of a resumed state (Universe.roche_radiuses), or NULL for zeros
 * (a new run computes them in posi_initialize_physical_values). */
posi_handle* posi_universe_from_arrays(const int64_t* sys_i64, const double* sys_f64,
                                       const int64_t* body_i64, const double* body_f64,
                                       const double* tables, int64_t n_tables, const double* roche,
                                       int mode, int* status);

void posi_destroy(posi_handle* h);

/* src/integrator/mod.rs:16-27 Integrator::get_n_particles / get_current_time /
 * get_n_historic_snapshots. */
int posi_get_n_particles(const posi_handle* h, int64_t* n);
int posi_get_current_time(const posi_handle* h, double* t);
int posi_get_n_historic_snapshots(const posi_handle* h, int64_t* n);

/* src/integrator/whfast.rs:187-224 set_time_limit / set_snapshot_periods
 * (non-positive values keep the current setting). */
int posi_set_time_limit(posi_handle* h, double time_limit);
int posi_set_snapshot_periods(posi_handle* h, double historic_period, double recovery_period);

/* src/integrator/whfast.rs:226-233 initialize_physical_values
 * (+ src/particles/universe.rs:177-196 calculate_roche_radiuses). */
int posi_initialize_physical_values(posi_handle* h);

/* src/integrator/whfast.rs:235-305 (src/integrator/ias15.rs:420-463 for an
 * IAS15 case) Integrator::iterate, n_steps times (one kernel launch per step).  Returns POSI_COMPLETED after the step that makes
 * current_time + time_step exceed time_limit, like Err("Simulation completed").
 * *steps_done receives the steps performed; *recovery_trigger is set when the
 * last step reported a recovery-snapshot trigger (Ok(true)). */
int posi_iterate(posi_handle* h, int64_t n_steps, int64_t* steps_done, int* recovery_trigger);

/* src/particles/universe.rs:198-303 gravity_calculate_acceleration
 * (ignore_terms: 0 None, 1 WHFastOne, 2 WHFastTwo). */
int posi_gravity_calculate_acceleration(posi_handle* h, int ignore_terms);

/* src/particles/universe.rs:318-351 inertial_to_heliocentric followed by
 * src/particles/universe.rs:428-538 calculate_additional_effects. */
int posi_calculate_additional_effects(posi_handle* h, double current_time, int evolution,
                                      int dangular_momentum_dt, int accelerations);

/* Copy the state to/from the host in the flat layout (nmax = n); roche (n*n)
 * may be NULL. */
int posi_get_state(const posi_handle* h, int64_t* sys_i64, double* sys_f64,
                   int64_t* body_i64, double* body_f64, double* roche);
int posi_set_state(posi_handle* h, const int64_t* sys_i64, const double* sys_f64,
                   const int64_t* body_i64, const double* body_f64);

/* IAS15 systems: copy the per-body Gauss-Radau state (n*POSI_IAS_COUNT) to or
 * from the host; POSI_ERR_STATE for a WHFast system. */
int posi_get_ias15(const posi_handle* h, double* body_ias);
int posi_set_ias15(posi_handle* h, const double* body_ias);

/* src/integrator/output.rs:63-89 get_universe_history_writer: open the
 * historic-snapshot file (created if absent), fail with POSI_ERR_STATE when it
 * is shorter than expected_bytes (n_historic_snapshots * 156 * n_particles),
 * and truncate it to expected_bytes.  From then on posi_iterate appends one
 * 156-byte bincode record per body at every historic trigger
 * (src/integrator/output.rs:91-135). */
int posi_open_history(posi_handle* h, const char* path, int64_t expected_bytes);
int posi_close_history(posi_handle* h);

/* src/integrator/whfast.rs:307-316 + src/integrator/output.rs:28-54
 * write_recovery_snapshot: set last_recovery_snapshot_time, flush the history,
 * rename an existing file to <stem>.<YYYYMMDD>T<AM|PM>.bin and write the
 * case document with the current state: pretty JSON for a ".json" path,
 * bincode (bincode 1.3 layout of the WHFast / Ias15 struct) for any other
 * (the handle must come from posi_universe_from_json). */
int posi_write_recovery_snapshot(posi_handle* h, const char* path);

/* src/integrator/output.rs:43-51, 186-191: convert a case or recovery
 * snapshot between its JSON and bincode forms, each path's form chosen by
 * its extension as the reference chooses it (no device needed). */
int posi_convert_snapshot(const char* src, const char* dst);

/* ---- batched ensembles (many independent systems, one persistent kernel) -- */

/* nmax >= every system's n, nmax <= POSI_MAX_BODIES.  The arrays are copied to
 * the device; roche is n_systems*nmax*nmax or NULL; mapping selects the
 * thread layout (POSI_MAP_AUTO = autotuned). */
posi_batch* posi_batch_create(int64_t n_systems, int64_t nmax,
                              const int64_t* sys_i64, const double* sys_f64,
                              const int64_t* body_i64, const double* body_f64,
                              const double* tables, int64_t n_tables, const double* roche,
                              int mode, int mapping, int* status);
void posi_batch_destroy(posi_batch* b);

/* initialize_physical_values for every system (whfast.rs:226-233). */
int posi_batch_initialize_physical_values(posi_batch* b);

/* Advance every live system by n_steps WHFast steps, steps_per_launch steps per
 * persistent-kernel launch; the launches are captured once in a CUDA graph and
 * replayed.  Systems that complete or hit a fatal event are frozen.  When a
 * lane mapping leaves between one and two warps of systems per SMSP, a launch
 * runs as a balanced schedule of sub-launches (warps alone on an SMSP take
 * more steps, and the systems rotate), with the same results bit for bit. */
int posi_batch_iterate(posi_batch* b, int64_t n_steps, int64_t steps_per_launch);
/* Balanced schedules on (1, the default) or off (0).  No reference
 * counterpart: a scheduling switch of this implementation. */
int posi_batch_set_balanced(posi_batch* b, int on);

/* Host <-> device copies of the whole ensemble (flat layout). */
int posi_batch_get_state(const posi_batch* b, int64_t* sys_i64, double* sys_f64,
                         int64_t* body_i64, double* body_f64, double* roche);
int posi_batch_set_state(posi_batch* b, const int64_t* sys_i64, const double* sys_f64,
                         const int64_t* body_i64, const double* body_f64);

/* IAS15 batches: the per-body Gauss-Radau state, [n_systems][nmax]
 * [POSI_IAS_COUNT] (zeros after posi_batch_create); POSI_ERR_STATE for a
 * WHFast batch.  A batch holds systems of one integrator (sys_i64
 * [POSI_SI_INTEGRATOR]); an IAS15 batch advances by IAS15 steps in
 * posi_batch_iterate (adaptive per system, the smallest lane group that holds
 * the system, no balanced schedules, no autotuning). */
int posi_batch_get_ias15(const posi_batch* b, double* body_ias);
int posi_batch_set_ias15(posi_batch* b, const double* body_ias);

/* Size of the ensemble. */
int posi_batch_size(const posi_batch* b, int64_t* n_systems, int64_t* nmax);

/* Mapping chosen for systems with n bodies (after autotuning), or -1. */
int posi_batch_mapping_for(const posi_batch* b, int64_t n);

/* Autotuner of the batched kernel (no reference counterpart: the reference
 * integrates one system per process).  For every body count present, each
 * admissible lane mapping (2..32 lanes per system, one body per lane) runs
 * probe_steps steps on the systems of that count, timed with CUDA events; the
 * state is restored after every trial.  A batch of one body count keeps the
 * fastest mapping.  When several counts together hold at least one warp per
 * SMSP at their smallest lane groups (their launches share the GPU), each
 * keeps the mapping of least SMSP time: probe time x min(warps, SMSPs) /
 * SMSPs, since a bucket probed alone on fewer warps than SMSPs takes its
 * longest lane's time whatever its lane group, while side by side its warps
 * hold SMSPs the other buckets could use.
 * lanes_by_n (optional, POSI_MAX_BODIES + 1 entries) receives the choice per
 * body count (0 where no system has that count).  Results do not depend on
 * the mapping: every mapping computes the same bits. */
int posi_batch_autotune(posi_batch* b, int64_t probe_steps, int32_t* lanes_by_n);

/* The last autotune's probe times for systems of n bodies: ms_by_lanes[k]
 * (6 entries) is the timed probe of 2^k lanes per system (k = 0: one thread
 * per system, never probed since it is not built), -1 where that mapping was
 * not admissible or not tried.  POSI_ERR_STATE when no system of n bodies
 * was tuned. */
int posi_batch_autotune_report(const posi_batch* b, int64_t n, double* ms_by_lanes);

/* Device time of the last posi_batch_iterate in milliseconds (CUDA events on
 * the batch's stream) and the number of kernel launches it made. */
int posi_batch_last_timing(const posi_batch* b, double* ms, int64_t* launches);

/* ---- diagnostics ------------------------------------------------------- */

/* FP64 rate of the device: `blocks` x `threads` threads, each running eight
 * independent DFMA chains for `iters` iterations.  Reports the kernel time and
 * the rate in TFLOP/s (a DFMA counts 2 flops).  Roofline denominator of the
 * FP64-bound kernels. */
int posi_fp64_probe(int blocks, int threads, int iters, double* ms, double* tflops);

/* ---- adjoint (reverse mode) of the batched WHFast step ----------------------
 * No reference counterpart: the reference has no derivatives.  Gradients of a
 * function of the state after n_steps steps with respect to the state at the
 * start (positions, velocities, spin angular momenta, spins) and to every
 * body's tidal dissipation factor (scaled_dissipation_factor) and Love number.
 * Supported: Jacobi coordinates, non-evolving bodies, up to 8 bodies per system.
 * The forward run stores the batch state every checkpoint_every steps; the
 * backward run re-integrates each chunk from a copy of its checkpoint
 * (recording its steps) and sweeps it in reverse, the re-integration of one
 * chunk overlapping the reverse sweep of the next on a second stream when a
 * second tape fits (2 x checkpoint_every x 209 doubles per body slot); it
 * leaves the batch state as the forward run ended it.  Derivatives are those of the computed map (the midpoint loop is
 * reversed with its iteration counts, the Kepler root is differentiated
 * implicitly). */
typedef struct posi_adjoint posi_adjoint;
posi_adjoint* posi_adjoint_create(posi_batch* b, int64_t n_steps, int64_t checkpoint_every, int* status);
void posi_adjoint_destroy(posi_adjoint* a);
/* Run the n_steps forward steps of the batch from its current state, keeping
 * the checkpoints; the batch ends at the final state. */
int posi_adjoint_forward(posi_adjoint* a);
/* Per-system flags of posi_adjoint_backward: the system's gradients are not
 * meaningful when any is set. */
enum posi_adjoint_flag {
    POSI_ADJ_KEPLER = 1,        /* a Kepler root did not converge */
    POSI_ADJ_ZERO_INERTIA = 2,  /* a body has no moment of inertia */
    POSI_ADJ_FROZEN = 4,        /* the forward run froze the system (collision, Roche limit, ejection) */
    POSI_ADJ_UNSUPPORTED = 8    /* not Jacobi, evolving bodies, or too many bodies (posi_adjoint_vjp_static) */
};
/* lam_final: [n_systems][nmax][12] adjoints of the final (r, v, L, S); out:
 * lam_initial (same layout, may be NULL), grad [n_systems][nmax][2] (d/d
 * sigma, d/d k2; may be NULL) and system_flags [n_systems] (may be NULL).
 * Host or device pointers (unified addressing). */
int posi_adjoint_backward(posi_adjoint* a, const double* lam_final, double* lam_initial, double* grad,
                          int32_t* system_flags);
/* Allocation-free adjoint of a short run.  No counterpart in the reference.
 * For callers that may not allocate device memory -- an application whose
 * device memory belongs to its own pool or arena (a framework's caching
 * allocator that has reserved the GPU, an embedded solver with a fixed
 * budget), or a latency-sensitive loop where a cudaMalloc, which can
 * synchronise the device, is not acceptable.  It calls no cudaMalloc,
 * cudaFree or allocating library routine: the step records live in a
 * file-scope device array of 48 MiB, enough for 48 MiB / (209 * 8 bytes) =
 * 30,102 body-steps (n_steps * n_systems * nmax, less 4 bytes per system for
 * the system list); larger requests fail with POSI_ERR_ARG and a message
 * giving the limit (the bound is checked by division, so that no request
 * size can wrap it).
 * Same computation as one chunk of posi_adjoint_backward: from the state in
 * the device arrays (the library's field-major layout: sys_i64
 * [POSI_SI_COUNT][n_systems], sys_f64 [POSI_SF_COUNT][n_systems], body_i64
 * [POSI_BI_COUNT][n_systems * nmax], body_f64 [POSI_BF_COUNT][n_systems *
 * nmax]), re-integrate n_steps steps, recording them, and sweep them in
 * reverse.  d_lam [12][n_systems * nmax] holds the adjoints of the final
 * (r, v, L, S) on entry and those of the initial state on return; d_grad
 * [2][n_systems * nmax] (d/d sigma, d/d k2) is added to; d_flags
 * [n_systems] receives posi_adjoint_flag bits (cleared first).  A system
 * the adjoint does not support (POSI_ADJ_UNSUPPORTED: not Jacobi, evolving
 * bodies, Anderson / Newhall GR, wind, disk, IAS15, or a body count outside
 * 1..nmax) is left out of the run: its d_lam and d_grad entries are not
 * touched.  All pointers
 * are device pointers; the work is queued on `stream` (a cudaStream_t, or
 * NULL) and the outputs are ready when the stream reaches it.
 * The first call on a device takes the array's address
 * (cudaGetSymbolAddress) and sets the kernels' shared-memory attributes
 * (under a lock, so host threads making their first calls at once are
 * safe): make that first call before any stream capture.  Every call on a device
 * shares the one array: calls whose work overlaps on the GPU (other streams,
 * other host threads) race on it and must be serialised by the caller. */
int posi_adjoint_vjp_static(int64_t n_systems, int64_t nmax, const int64_t* d_sys_i64, const double* d_sys_f64,
                            const int64_t* d_body_i64, const double* d_body_f64, int64_t n_steps, double* d_lam,
                            double* d_grad, int32_t* d_flags, void* stream);

/* CUDA-event times of the last forward and backward runs, and the backward
 * run's split into chunk re-integration (record) and reverse sweeps (sums
 * over the chunks; the two overlap, so they may add up to more than the
 * backward time). */
int posi_adjoint_last_timing(const posi_adjoint* a, double* forward_ms, double* backward_ms, double* record_ms,
                             double* reverse_ms);

/* ---- one system of many bodies ---------------------------------------------
 * src/particles/universe.rs:198-303 and src/integrator/whfast.rs:235-305 for a
 * single system beyond the batched kernels' 32 bodies (a star, tidally active
 * planets and hundreds or thousands of small massive bodies): one cooperative
 * grid, thread per body, the O(N^2) pair loop spread over the whole GPU.
 * Democratic-heliocentric, Jacobi or WHDS coordinates (the reference's
 * sequential Jacobi recurrences run as grid-wide prefix scans), non-evolving
 * bodies, the host the most massive body; FAST arithmetic.  State arrays as posi_universe_from_arrays
 * (one system of n bodies, row-major).  A physical event freezes the system
 * (posi_large_iterate returns POSI_ERR_PHYSICS; sys_i64[POSI_SI_FAIL_PAIR] =
 * i * n + j of the first failing pair). */
typedef struct posi_large posi_large;
posi_large* posi_large_create(int64_t n, const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                              const double* body_f64, int* status);
void posi_large_destroy(posi_large* L);
int posi_large_set_state(posi_large* L, const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                         const double* body_f64);
int posi_large_get_state(const posi_large* L, int64_t* sys_i64, double* sys_f64, int64_t* body_i64,
                         double* body_f64);
int posi_large_initialize_physical_values(posi_large* L);
/* n_steps steps in one launch (fewer when the run completes or freezes). */
int posi_large_iterate(posi_large* L, int64_t n_steps);
/* Forward-mode derivatives (no reference counterpart: the reference computes
 * no derivatives).  Integrates n_steps like posi_large_iterate while carrying
 * the tangents of every body's state along n_dirs directions (1 to 4).
 * tangents[d][i][12] (host memory; r, v, L, S of body i), in and out: on
 * entry the tangent of the state along direction d (zeros for a pure
 * parameter derivative), on return the tangent after the steps.  Direction d
 * also perturbs, at unit rate, the parameter seed_param[d] of body
 * seed_body[d]: POSI_SEED_SIGMA (dissipation factor) or POSI_SEED_K2 (Love
 * number k2); seed_body[d] = -1 perturbs no parameter.  The primal state
 * advances exactly as posi_large_iterate advances it.  Democratic-heliocentric
 * systems only (POSI_ERR_UNSUPPORTED for Jacobi and WHDS). */
enum posi_seed_param { POSI_SEED_SIGMA = 0, POSI_SEED_K2 = 1 };
int posi_large_iterate_tangent(posi_large* L, int64_t n_steps, int32_t n_dirs, const int32_t* seed_body,
                               const int32_t* seed_param, double* tangents);
int posi_large_last_timing(const posi_large* L, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* POSIDONIUS_GB300_H */
