/*
 * redgb.h -- C ABI of libredgb, the GB300-native (sm_103a) implementation of
 * the integration hot path of suliaron/red.cuda.
 *
 * red has no plugin or FFI layer: its hot path sits behind the in-process
 * C++ seam formed by pp_disk (src/red.cuda/pp_disk.h) and the integrator
 * classes (src/red.cuda/integrator.h, int_rungekutta4.h, int_rungekutta8.h),
 * driven by run_simulation (src/red.cuda/main.cu:403-640).  Each entry point
 * below names the member function it replaces.  All functions return an int
 * status (RED_OK = 0); red_last_error() gives the message of the last failure
 * on the calling thread.  Records are laid out exactly as red.type/red_type.h
 * lays them out on LP64, so red's arrays can be passed without conversion.
 *
 * A handle holds one or more independent systems ("disks"), each with its
 * own bodies, time, step size and counters.  One system reproduces red; many
 * systems form a batched ensemble integrated by the same kernels.
 */
#ifndef REDGB_H
#define REDGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- records (red.type/red_type.h) ------------------------------------- */
typedef struct { double x, y, z, w; } red_var4_t;                       /* var4_t, red_type.h:206-212 */
typedef struct { double mass, radius, density, cd; } red_param_t;       /* pp_disk_t::param_t, red_type.h:347-353 */
typedef struct { int32_t id, body_type, mig_type; double mig_stop_at; } red_body_metadata_t; /* red_type.h:356-362 */

typedef struct {                                                        /* analytic_gas_disk_params_t, red_type.h:464-485 */
    double rho[2], sch[2], eta[2], tau[2], mfp[2], temp[2];
    double c_vth;
    int32_t gas_decrease;
    double t0, t1, e_folding_time;
    double alpha, mean_molecular_weight, particle_diameter;
} red_gas_params_t;

typedef struct {                                                        /* pp_disk_t::event_data_t, red_type.h:415-461 */
    int32_t event_name;
    double t, d;
    int32_t id0; uint32_t idx0; red_param_t p0; red_var4_t r0, v0;
    int32_t id1; uint32_t idx1; red_param_t p1; red_var4_t r1, v1;
    int32_t id2; uint32_t idx2; red_param_t p2; red_var4_t r2, v2;
    red_param_t ps; red_var4_t rs, vs;
} red_event_t;

typedef struct { red_var4_t R, V, C; double E; } red_integral_t;       /* pp_disk_t::integral_t, red_type.h:375-381 */

/* ---- enumerations (values as in red_type.h) ----------------------------- */
enum { RED_BODY_STAR = 0, RED_BODY_GIANTPLANET, RED_BODY_ROCKYPLANET, RED_BODY_PROTOPLANET,
       RED_BODY_SUPERPLANETESIMAL, RED_BODY_PLANETESIMAL, RED_BODY_TESTPARTICLE, RED_BODY_N };
enum { RED_INTEGRATOR_EULER = 0, RED_INTEGRATOR_RUNGEKUTTA2 = 1, RED_INTEGRATOR_RUNGEKUTTA4 = 2,
       RED_INTEGRATOR_RUNGEKUTTAFEHLBERG78 = 4 };
enum { RED_EVENT_NONE = 0, RED_EVENT_HIT_CENTRUM, RED_EVENT_EJECTION, RED_EVENT_COLLISION };
enum { RED_THRESHOLD_HIT_CENTRUM_DISTANCE = 0, RED_THRESHOLD_EJECTION_DISTANCE,
       RED_THRESHOLD_RADII_ENHANCE_FACTOR, RED_THRESHOLD_N };

/* Arithmetic of the pairwise gravity (the rest of the path is FP64 always). */
enum {
    RED_PREC_MIXED = 0,      /* central-star term FP64; body-body pairs in FP32 on double-single
                                coordinates, tile sums folded into double-single accumulators */
    RED_PREC_FP64 = 1,       /* every pair FP64, tiled and split over sources */
    RED_PREC_FP64_EXACT = 2, /* red's FP64 kernel arithmetic in red's order, no FMA: bit-identical
                                to red's calc_grav_accel_naive (pp_disk.cu:373-416) */
    RED_PREC_FP32 = 3        /* as MIXED, body-body pairs on plain FP32 coordinates */
};

/* Status codes. */
enum {
    RED_OK = 0,
    RED_ERR_ARG = 1,              /* bad argument (red: throw std::string) */
    RED_ERR_CUDA = 2,             /* CUDA runtime error */
    RED_ERR_EVENT_OVERFLOW = 3,   /* more events than the event buffer holds */
    RED_ERR_TIMEOUT = 4,          /* a bounded device wait gave up */
    RED_ERR_NONFINITE = 5,        /* NaN / Inf in the state or the error estimate */
    RED_ERR_NOT_IMPLEMENTED = 6,  /* integrator or option red does not provide on this path */
    RED_ERR_SUPERPLANETESIMAL = 7,/* merge with a super-planetesimal (pp_disk.cu:1333-1337) */
    RED_ERR_NO_DEVICE = 8
};

typedef struct {
    int32_t integrator;          /* RED_INTEGRATOR_EULER, _RUNGEKUTTA2, _RUNGEKUTTA4 or _RUNGEKUTTAFEHLBERG78
                                    (options.cpp:297-326) */
    int32_t adaptive;            /* integrator ctor argument (int_rungekutta4.cu:101, int_rungekutta8.cu:405);
                                    Euler and RK2 are fixed-step, as red's constructors make them */
    double tolerance;
    int32_t error_check_for_tp;  /* integrator::error_check_for_tp (integrator.h:33) */
    int32_t precision;           /* RED_PREC_* */
    int32_t stage_exact;         /* stage sums in red's order without FMA (bit-identical): implied by
                                    RED_PREC_FP64_EXACT, refused (RED_ERR_ARG) with the other modes */
    double threshold[RED_THRESHOLD_N]; /* parameter::threshold (parameter.cpp:214-237) */
    double output_interval;      /* dt_next is clamped to it after every step (main.cu:535-538); 0 = off */
    double length;               /* per-system integration length, code units (main.cu:471); 0 = unbounded */
    int32_t gas_disk;            /* 0 none, 1 analytic (GAS_DISK_MODEL_ANALYTIC); 2 (FARGO) is refused with
                                    RED_ERR_NOT_IMPLEMENTED: red's fargo_gas_disk cannot be constructed */
    red_gas_params_t gas;        /* after analytic_gas_disk::calc and transform_time */
    uint32_t event_capacity;     /* device event buffer, records; 0 = max(1024, total bodies) */
    int32_t device;              /* CUDA device ordinal */
    void* stream;                /* cudaStream_t to launch on; NULL = the handle creates its own */
} red_config_t;

typedef struct {
    double t, dt_try, dt_did, dt_next;
    uint64_t n_tried, n_passed, n_failed;   /* integrator::get_n_*_step (integrator.cu:277-290) */
    uint32_t playing[RED_BODY_N], inactive[RED_BODY_N], removed[RED_BODY_N]; /* n_objects_t */
    uint32_t n_total;              /* bodies stored (n_objects_t::get_n_total_playing) */
    int32_t active;                /* still integrating (length not reached, > 1 active body) */
    int32_t halted;                /* events detected and not yet handled */
    int32_t status;                /* RED_OK or the error that stopped this system */
    uint32_t n_collision[3], n_ejection[3], n_hit_centrum[3], n_event[3]; /* pp_disk.h:195-198 */
} red_system_info_t;

typedef struct red_sim red_sim;

/* Creates a handle for n_systems systems.  playing holds 7 counts per system
 * (n_objects_t::playing, red_type.h:545-566); the body arrays of all systems
 * are concatenated, each system's bodies sorted by type as red requires
 * (star, giant, rocky, proto | super-pl, pl | test particle).  t0 and dt0 give
 * each system's time and first step size (pp_disk::t, pp_disk::dt).
 * Replaces: pp_disk::pp_disk + copy_to_device (pp_disk.cu:1546-1575, 1667-1684)
 * and options::create_integrator (options.cpp:297-326). */
int red_create(const red_config_t* cfg, uint32_t n_systems, const uint32_t* playing,
               const red_var4_t* r, const red_var4_t* v, const red_param_t* p,
               const red_body_metadata_t* md, const double* t0, const double* dt0, red_sim** out);
/* Replaces: pp_disk::~pp_disk, integrator::~integrator. */
int red_destroy(red_sim* sim);

/* One integrator step of every active system, retrying rejected tries until
 * each has accepted one (blocking).  dt_did receives the accepted step of
 * system 0.  Replaces: integrator::step (int_rungekutta4.cu:173-249,
 * int_rungekutta8.cu:635-716) including pp_disk::swap. */
int red_step(red_sim* sim, double* dt_did);

/* Enqueues n tries on the stream without waiting: every active system whose
 * events are handled makes one try; accepted systems advance, rejected ones
 * retry on the next try with the smaller step.  After each accepted try the
 * collision and ejection checks run on the device; a system with events halts
 * until red_handle_events.  Device-side equivalent of run_simulation's loop
 * body (main.cu:470-569). */
int red_launch_tries(red_sim* sim, uint32_t n);
/* Waits for the stream; n_active / n_halted count the systems still
 * integrating / waiting for event handling. */
int red_synchronize(red_sim* sim, uint32_t* n_active, uint32_t* n_halted);
/* Handles the pending events of every halted system as red does: collisions
 * (pp_disk::handle_collision, pp_disk.cu:1220-1248) first, then ejections and
 * hits of the centre (pp_disk::handle_ejection_hit_centrum, pp_disk.cu:1290-1326),
 * and compacts a system after 16 events (main.cu:582-607).  The handled records
 * are copied to out (up to cap); *n_out receives their number. */
int red_handle_events(red_sim* sim, red_event_t* out, uint32_t cap, uint32_t* n_out);

/* Collision detection on the current state of every system, without merging.
 * Events are returned in red's CPU loop order (i ascending, then j).
 * Replaces: pp_disk::check_for_collision (pp_disk.cu:1080-1094, 1203-1218). */
int red_check_for_collision(red_sim* sim, red_event_t* out, uint32_t cap, uint32_t* n_out);
/* Replaces: pp_disk::check_for_ejection_hit_centrum (pp_disk.cu:1064-1078, 1186-1201). */
int red_check_for_ejection_hit_centrum(red_sim* sim, red_event_t* out, uint32_t cap, uint32_t* n_out);

/* Derivatives of the current state of system sys at time t: i = 0 gives the
 * velocities, i = 1 gravity plus drag.  Replaces: pp_disk::calc_dydx
 * (pp_disk.cu:1450-1502). */
int red_calc_dydx(red_sim* sim, uint32_t sys, int32_t i, double t, red_var4_t* dy);

/* Integrals of system sys, as pp_disk::calc_integral (pp_disk.cu:1504-1516):
 * barycentre, its velocity, angular momentum and energy over all active pairs. */
int red_calc_integral(red_sim* sim, uint32_t sys, red_integral_t* out);
/* Energy and angular momentum of red's own dynamics: the potential runs over
 * the pairs that interact (both massive, not both planetesimals).  out[4] =
 * {E, C.x, C.y, C.z}.  No counterpart in red (its energy counts
 * planetesimal-planetesimal pairs, tools.cpp:591-620). */
int red_calc_energy_interacting(red_sim* sim, uint32_t sys, double out[4]);

/* Host copies of / updates to system sys (replaces pp_disk::copy_to_host /
 * copy_to_device, pp_disk.cu:1667-1699).  Arrays hold info.n_total records. */
int red_get_state(red_sim* sim, uint32_t sys, red_var4_t* r, red_var4_t* v, red_param_t* p,
                  red_body_metadata_t* md);
int red_set_state(red_sim* sim, uint32_t sys, const red_var4_t* r, const red_var4_t* v,
                  const red_param_t* p, const red_body_metadata_t* md);
/* The same for the systems [sys0, sys0 + count) at once: each array holds the
 * systems' records one system after the other (the sum of their n_total).  One
 * kernel and one synchronisation move an ensemble's state (no counterpart in
 * red, which holds one system per process).  Null arrays are skipped; pinned
 * (page-locked) arrays are read or written by the device directly. */
int red_get_states(red_sim* sim, uint32_t sys0, uint32_t count, red_var4_t* r, red_var4_t* v, red_param_t* p,
                   red_body_metadata_t* md);
int red_set_states(red_sim* sim, uint32_t sys0, uint32_t count, const red_var4_t* r, const red_var4_t* v,
                   const red_param_t* p, const red_body_metadata_t* md);
int red_get_system_info(red_sim* sim, uint32_t sys, red_system_info_t* info);
/* Sets dt_next of system sys (integrator::set_dt_next, integrator.h:24). */
int red_set_dt_next(red_sim* sim, uint32_t sys, double dt_next);

/* Removes inactive bodies of every system (pp_disk::rebuild_vectors,
 * pp_disk.cu:1370-1430). */
int red_rebuild_vectors(red_sim* sim);

/* Times candidate launch plans (threads per sink group; source chunks from
 * the planner's heuristic with or without the thread-block-cluster reduction,
 * or fixed chunk sizes) by integrating real tries of the captured graph from
 * a snapshot of the current state, keeps the fastest plan and restores the
 * state, so the systems are left exactly where they were (red's own n_tpb
 * search: pp_disk::benchmark, pp_disk.cu:553-611).  The red-exact mode has a
 * single plan and is left as it is. */
int red_autotune(red_sim* sim);
/* The plan in use and what the last red_autotune measured (no counterpart in
 * red, whose launch parameter is the single n_tpb, pp_disk.h:32-33). */
typedef struct {
    int32_t chunk;                /* sources per chunk (0: the planner's heuristic) */
    int32_t lanes_cap;            /* largest threads per sink group */
    int32_t cluster;              /* chunk sums reduced within thread-block clusters */
    int32_t packed;               /* 2-sink tiles on the packed FP32-pair instance */
    int32_t n_items;              /* stage-kernel CTAs of one launch */
    int32_t candidates;           /* plans timed by the last red_autotune (0: none) */
    float ms_per_try;             /* its best try time */
    float ms_per_try_default;     /* its try time of the heuristic plan */
} red_plan_info_t;
int red_get_plan_info(red_sim* sim, red_plan_info_t* out);

/* Runs one try launch by launch (outside the graph) with a CUDA event after
 * every kernel: ms[k] is the duration of launch k and kind[k] its kernel
 * (0 stage, 1 control, 2 finish, 3 collision, 4 ejection / hit-centrum, 5 the
 * learned proposer's two kernels, timed together).  The
 * try is a real one: the systems advance.  No counterpart in red; it stands in
 * for the per-launch cudaEvent timing of pp_disk::benchmark_calc_grav_accel
 * (pp_disk.cu:613-632). */
int red_profile_try(red_sim* sim, float* ms, int32_t* kind, uint32_t cap, uint32_t* n_out);

/* Directed gravity interactions per force evaluation, summed over systems. */
uint64_t red_interactions_per_eval(red_sim* sim);
/* Kernel launches made by the library since creation (for launch accounting). */
uint64_t red_kernel_launches(red_sim* sim);
uint32_t red_n_systems(red_sim* sim);
/* Records in system sys's arrays (n_total of red_get_system_info), from host
   bookkeeping: no device synchronisation.  0 for a bad handle or index. */
uint32_t red_n_bodies(red_sim* sim, uint32_t sys);

/* ---- initial conditions of disk ensembles -------------------------------
 * red.cuda.initial's disk recipe (populate_disk, red.cuda.initial/main.cu:251-314;
 * calculate_phase, main.cu:317-342; distribution.cpp:11-204) on the GPU, one
 * thread per body: a star, n_pp protoplanets and n_pl planetesimals per
 * system, sorted by type.  Orbital elements: protoplanet semi-major axes
 * pp_a0 * f^k (f for pp_hill mutual Hill radii, pp_hill > 0) or pp_a0 + k pp_da;
 * planetesimal a uniform (pl_a_log = 0) or log-uniform in [pl_a_min, pl_a_max];
 * e and i Rayleigh (sigma_*), e capped at e_max; peri, node, mean anomaly
 * uniform in [0, 2 pi).  Planetesimal masses m_j = pl_mass_total a_j^pl_mass_exp
 * / sum_j a_j^pl_mass_exp.  Kepler -> Cartesian with mu = K^2 (m_star + m)
 * (tools.cpp:789-828), the system moved to its barycentre (tools.cpp:413-434),
 * velocities divided by K (red.cuda.initial/main.cu:1666-1670).  Random
 * numbers: Philox4x32-10 (Salmon et al., SC'11), key = seed, counter = (body,
 * draw), so every body's draws are independent of the launch shape.  Output:
 * red's records for all systems, concatenated (1 + n_pp + n_pl each), and 7
 * playing counts per system. */
typedef struct {
    uint32_t n_pp, n_pl;
    double m_star, star_radius;                /* M_sun, AU */
    double pp_mass, pp_a0, pp_da, pp_hill;
    double pl_a_min, pl_a_max;
    int32_t pl_a_log, pad;
    double pl_mass_total, pl_mass_exp;
    double sigma_e_pp, sigma_i_pp, sigma_e, sigma_i, e_max;
    double density;                            /* g/cm^3, protoplanets and planetesimals */
    double cd;                                 /* planetesimals */
    uint64_t seed;
} red_disk_spec_t;
int red_populate_disks(const red_disk_spec_t* specs, uint32_t n_systems, int32_t device, uint32_t* playing,
                       red_var4_t* r, red_var4_t* v, red_param_t* p, red_body_metadata_t* md);

/* ---- allocation-free gravity ---------------------------------------------
 * No counterpart in red.  For callers that cannot call cudaMalloc (device
 * memory owned by another pool, real-time loops that must not enter the
 * allocator): gravity plus analytic drag of one system, as red_calc_dydx with
 * i = 1, from device buffers the caller owns, launched on the caller's
 * stream.  Temporaries live in a fixed 4 MiB __device__ array inside the
 * library, held by every GPU that loads it until exit; calls share it, so
 * calls that overlap on the GPU race and must be ordered by the caller.  The
 * first call on a device does a one-time set-up (it looks up the device
 * address of the array).  The call writes no constant memory, so simulations created earlier keep
 * their integrator coefficients.  Every system of up to
 * RED_NOALLOC_MAX_BODIES bodies fits, whatever its body classes (a plan that
 * would need more partial-sum records than the array holds falls back to
 * unchunked source lists); larger systems are rejected with RED_ERR_ARG.
 * The caller's current device is the same after the call as before it. */
#define RED_NOALLOC_MAX_BODIES 32768
typedef struct {
    uint32_t playing[RED_BODY_N];  /* bodies per type; bodies sorted by type */
    const double* r;               /* device: x, y, z per body (3 N doubles) */
    const double* v;               /* device: velocities (3 N), needed with gas drag */
    const double* mass;            /* device: N doubles */
    const double* radius;          /* device: N doubles (may be NULL without gas drag) */
    const double* density;         /* device: N doubles (gas drag) */
    const double* cd;              /* device: N doubles (gas drag) */
    const int32_t* id;             /* device: N body ids (id < 0: inactive) */
    double* accel;                 /* device: output accelerations (3 N doubles) */
    int32_t precision;             /* RED_PREC_* */
    int32_t gas_disk;              /* 0 none, 1 analytic */
    red_gas_params_t gas;
    double t;                      /* time of the evaluation (gas density factor) */
    int32_t device;                /* CUDA device ordinal */
    void* stream;                  /* cudaStream_t; NULL = legacy default stream */
} red_accel_args_t;
int red_calc_accel_noalloc(const red_accel_args_t* args);

/* ---- Learned step proposer ---------------------------------------------
 * A BF16 MLP (12 -> 64 -> 64 -> 1, SiLU, FP32 accumulation) proposes each
 * system's next step from features of its accepted state (log|dt|, log of
 * the error / tol, log of the smallest protoplanet-body distance in Hill
 * radii, log max|a|, max |v|/v_kep, log N, mean / rms / max of e and i).  The
 * embedded error estimate judges every try as before; a rejected proposal is
 * retried with the classical controller's step (int_rungekutta8.cu:690-716).
 * red.cuda has no learned component: these entry points have no counterpart
 * in the reference.  Parameters are flat: W1[64][12], b1[64], W2[64][64],
 * b2[64], w3[64], b3. */
#define RED_MLP_NFEAT 12
typedef struct {
    float x_mean[RED_MLP_NFEAT], x_std[RED_MLP_NFEAT];   /* feature normalisation */
    float y_mean, y_std;                                  /* of the target log|dt| */
} red_mlp_norm_t;
uint32_t red_mlp_param_count(void);
/* Device buffers: w_bf16 (param_count BF16), x (n x 12 raw features) -> out
 * (n predicted log|dt|). */
int red_mlp_predict(const void* w_bf16, const red_mlp_norm_t* norm, const float* x, float* out, uint32_t n,
                    void* stream);
/* Gradient of sum_r (y_r - t_r)^2 / (2 n) over n rows of normalised features xn
 * (n x 12) and targets tn, into grad (param_count floats) and loss (1 float);
 * device buffers, deterministic (fixed-order reduction). */
int red_mlp_grad(const void* w_bf16, const float* xn, const float* tn, uint32_t n, float* grad, float* loss,
                 void* stream);
/* One Adam step on FP32 master weights (device); refreshes the BF16 copy. */
int red_mlp_adam(float* master, void* w_bf16, float* m, float* v, const float* grad, uint32_t step, float lr,
                 float beta1, float beta2, float eps, void* stream);
/* Enables the proposals (host copy of the BF16 weights).  The proposed step is
 * safety * exp(prediction), its ratio to the last accepted step clamped to
 * [ratio_lo, ratio_hi], then to the output interval.  Adaptive runs only. */
int red_set_step_proposer(red_sim* sim, const uint16_t* w_bf16, const red_mlp_norm_t* norm, double safety,
                          double ratio_lo, double ratio_hi);
int red_clear_step_proposer(red_sim* sim);
/* Logs (features of an accepted state, log|dt| of the next accepted step,
 * log(err / tol) of that step) records, 14 floats each, into a device buffer
 * of `capacity` records (0 stops). */
int red_log_features(red_sim* sim, uint32_t capacity);
int red_get_feature_log(red_sim* sim, float* out, uint32_t cap, uint32_t* n_out, int32_t reset);

const char* red_last_error(void);
const char* red_version(void);

#ifdef __cplusplus
}
#endif
#endif
