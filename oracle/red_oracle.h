/*
 * red_oracle.h -- CPU restatement of red.cuda's integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * library is compared against.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it.  The product path
 * (libredgb) never links or calls it.
 *
 * Every routine restates one function of the reference (suliaron/red.cuda) and
 * cites it as path:line.  Arithmetic follows the reference's expression order
 * term by term; build with -ffp-contract=off so that no multiply-add is fused,
 * which mirrors the reference's own -fmad=false build (Makefile:17).  The
 * result is bit-identical to the reference's CPU code where that code exists
 * (pinned by tests/golden/, generated from the reference's own sources by
 * oracle/ref_harness.cu) and, for the GPU-only parts (planetesimal gravity,
 * the GPU collision loop), restates the GPU kernels sequentially.
 */
#ifndef RED_ORACLE_H
#define RED_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* --- types: same field order and sizes as red.type/red_type.h ------------ */

/* var4_t, red_type.h:206-212 */
typedef struct { double x, y, z, w; } orc_var4;
/* pp_disk_t::param_t, red_type.h:347-353 */
typedef struct { double mass, radius, density, cd; } orc_param;
/* pp_disk_t::body_metadata_t, red_type.h:356-362 (24 bytes on LP64) */
typedef struct { int32_t id, body_type, mig_type; double mig_stop_at; } orc_bmd;

/* analytic_gas_disk_params_t, red_type.h:464-485 */
typedef struct {
    double rho[2], sch[2], eta[2], tau[2], mfp[2], temp[2];
    double c_vth;
    int32_t gas_decrease;
    double t0, t1, e_folding_time;
    double alpha, mean_molecular_weight, particle_diameter;
} orc_gas;

/* pp_disk_t::event_data_t, red_type.h:415-461 */
typedef struct {
    int32_t event_name;
    double t, d;
    int32_t id0; uint32_t idx0; orc_param p0; orc_var4 r0, v0;
    int32_t id1; uint32_t idx1; orc_param p1; orc_var4 r1, v1;
    int32_t id2; uint32_t idx2; orc_param p2; orc_var4 r2, v2;
    orc_param ps; orc_var4 rs, vs;
} orc_event;

/* body types, red_type.h:169-179 */
enum { ORC_STAR = 0, ORC_GIANT, ORC_ROCKY, ORC_PROTO, ORC_SUPERPL, ORC_PL, ORC_TP, ORC_NTYPE };
/* integrator types, red_type.h:136-143 */
enum { ORC_EULER = 0, ORC_RK2 = 1, ORC_RK4 = 2, ORC_RKF78 = 4 };
/* event names, red_type.h:145-152 */
enum { ORC_EV_NONE = 0, ORC_EV_HIT_CENTRUM, ORC_EV_EJECTION, ORC_EV_COLLISION };
/* semantics of the force / collision loops */
enum { ORC_SEM_GPU = 0, ORC_SEM_CPU = 1 };

/* Error codes. */
enum { ORC_OK = 0, ORC_ERR_NOT_IMPLEMENTED = 1, ORC_ERR_ARG = 2, ORC_ERR_OVERFLOW = 3,
       ORC_ERR_SUPERPLANETESIMAL = 4 };

/* --- body classes: n_objects_t, red_type.h:580-700 ---------------------- */
uint32_t orc_n_SI(const uint32_t playing[7]);
uint32_t orc_n_NSI(const uint32_t playing[7]);
uint32_t orc_n_NI(const uint32_t playing[7]);
uint32_t orc_n_massive(const uint32_t playing[7]);
uint32_t orc_n_total(const uint32_t playing[7]);
/* out = {sink.x, sink.y, source.x, source.y}; which: 0 SI, 1 NSI, 2 NI, 3 GD */
void orc_bound(const uint32_t playing[7], int which, uint32_t out[4]);

/* --- right-hand side ------------------------------------------------------ */
/* Gravity.  sem = ORC_SEM_GPU restates kernel_pp_disk::calc_grav_accel_naive
 * (pp_disk.cu:373-416) over the SI, NSI and NI bounds as gpu_calc_grav_accel
 * launches it (pp_disk.cu:1014-1045).  sem = ORC_SEM_CPU restates
 * cpu_calc_grav_accel (pp_disk.cu:984-1012) and returns
 * ORC_ERR_NOT_IMPLEMENTED when planetesimals are present, as red does.
 * nthreads > 1 parallelises the GPU-semantics loop over sinks (OpenMP). */
int orc_grav_accel(int sem, const uint32_t playing[7], const orc_bmd* md, const orc_param* p,
                   const orc_var4* r, orc_var4* a, int nthreads);
/* Analytic gas drag on the NSI bodies: calc_drag_accel_NSI (pp_disk.cu:485-521),
 * added to a. */
void orc_drag_accel(double t, const orc_gas* gas, const uint32_t playing[7], const orc_param* p,
                    const orc_var4* r, const orc_var4* v, orc_var4* a);
/* pp_disk::calc_dydx (pp_disk.cu:1450-1502): i == 0 copies v, i == 1 is gravity + drag. */
int orc_calc_dydx(int sem, int i, double t, const uint32_t playing[7], const orc_bmd* md,
                  const orc_param* p, const orc_gas* gas, const orc_var4* r, const orc_var4* v,
                  orc_var4* dy, int nthreads);

/* --- integrators ------------------------------------------------------------ */
typedef struct {
    int32_t type;              /* ORC_EULER, ORC_RK2 (fixed step), ORC_RK4 or ORC_RKF78 */
    int32_t adaptive;
    int32_t error_check_for_tp;
    int32_t sem;               /* ORC_SEM_GPU or ORC_SEM_CPU */
    double tolerance;
    double dt_try, dt_did, dt_next;
    uint64_t n_tried, n_passed, n_failed;
    int32_t nthreads;
} orc_integrator;

/* One call of rungekutta4::step (int_rungekutta4.cu:173-249) or
 * rungekutta8::step (int_rungekutta8.cu:635-716) followed by pp_disk::swap:
 * r, v are replaced by y_{n+1} and *t advances by dt_did. */
int orc_step(orc_integrator* ig, double* t, const uint32_t playing[7], const orc_bmd* md,
             const orc_param* p, const orc_gas* gas, orc_var4* r, orc_var4* v);

/* --- events ----------------------------------------------------------------- */
/* sem GPU: kernel_pp_disk::check_for_collision (pp_disk.cu:320-371), events in
 * (i, j) loop order.  sem CPU: pp_disk::cpu_check_for_collision (pp_disk.cu:1143-1184). */
int orc_check_collision(int sem, double t, double factor, uint32_t n_total, const orc_bmd* md,
                        const orc_param* p, const orc_var4* r, const orc_var4* v,
                        orc_event* ev, uint32_t cap, uint32_t* n_ev);
/* The same test with the i loop spread over nthreads (OpenMP). */
int orc_check_collision_mt(int sem, double t, double factor, uint32_t n_total, const orc_bmd* md,
                           const orc_param* p, const orc_var4* r, const orc_var4* v,
                           orc_event* ev, uint32_t cap, uint32_t* n_ev, int nthreads);
/* check_for_ejection_hit_centrum (pp_disk.cu:283-318 / 1096-1127). */
int orc_check_ejection_hit_centrum(double t, double ejection, double hit_centrum, uint32_t n_total,
                                   const orc_bmd* md, const orc_param* p, const orc_var4* r,
                                   const orc_var4* v, orc_event* ev, uint32_t cap, uint32_t* n_ev);
/* pp_disk::populate_sp_events (pp_disk.cu:1250-1288); returns the unique count,
 * written to the front of ev. */
uint32_t orc_populate_sp_events(orc_event* ev, uint32_t n_ev);
/* pp_disk::handle_collision (pp_disk.cu:1220-1248): dedup, merge each pair
 * (handle_collision_pair, pp_disk.cu:1328-1368), flip the merger's id and count
 * it in inactive[].  ev is rewritten with the merged records; *n_ev becomes the
 * unique count. */
int orc_handle_collision(orc_event* ev, uint32_t* n_ev, orc_var4* r, orc_var4* v, orc_param* p,
                         orc_bmd* md, uint32_t inactive[7]);
/* pp_disk::handle_ejection_hit_centrum (pp_disk.cu:1290-1326). */
int orc_handle_ejection_hit_centrum(orc_event* ev, uint32_t n_ev, orc_var4* r, orc_var4* v,
                                    orc_param* p, orc_bmd* md, uint32_t inactive[7]);
/* pp_disk::rebuild_vectors (pp_disk.cu:1370-1430) + n_objects::update
 * (red_type.h:568-578).  Returns the new total. */
uint32_t orc_rebuild_vectors(uint32_t n_total, orc_var4* r, orc_var4* v, orc_param* p, orc_bmd* md,
                             uint32_t playing[7], uint32_t inactive[7], uint32_t removed[7],
                             int32_t* perm_out);

/* --- merge formulas, tools.cpp:455-507 ------------------------------------- */
double orc_calc_radius(double m, double density);
double orc_calc_density(double m, double R);
double orc_calc_mass(double R, double density);
void orc_calc_position_after_collision(double m1, double m2, const orc_var4* r1, const orc_var4* r2, orc_var4* r);
void orc_calc_velocity_after_collision(double m1, double m2, const orc_var4* v1, const orc_var4* v2, orc_var4* v);
void orc_calc_physical_properties(const orc_param* p1, const orc_param* p2, orc_param* p);

/* --- integrals -------------------------------------------------------------- */
/* pp_disk::calc_integral (pp_disk.cu:1504-1516) with tools::get_total_mass,
 * calc_bc, calc_angular_momentum, calc_total_energy (tools.cpp:365-410, 545-620).
 * out = {R.x,R.y,R.z, V.x,V.y,V.z, C.x,C.y,C.z, E} */
void orc_calc_integral(uint32_t n, const orc_bmd* md, const orc_param* p, const orc_var4* r,
                       const orc_var4* v, double out[10]);
/* Energy of red's own dynamics: the potential runs over the pairs that interact
 * (both massive, not both planetesimals), the kinetic term over massive bodies.
 * out = {E, C.x, C.y, C.z}. */
void orc_calc_energy_interacting(const uint32_t playing[7], const orc_bmd* md, const orc_param* p,
                                 const orc_var4* r, const orc_var4* v, double out[4], int nthreads);

/* Interactions per gravity evaluation (directed pairs). */
uint64_t orc_interactions_per_eval(const uint32_t playing[7]);

#ifdef __cplusplus
}
#endif
#endif
