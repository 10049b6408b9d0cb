/*
 * red_oracle.c -- CPU restatement of red.cuda's hot path (test infrastructure).
 *
 * This file is the checker, not the product: only tests/, __graft_entry__.smoke()
 * and the CPU legs of bench.py load it.  See red_oracle.h for the contract.
 * Build with -O2 -ffp-contract=off (mirrors the reference's -fmad=false).
 *
 * Citations are path:line in suliaron/red.cuda; pp_disk.cu means
 * src/red.cuda/pp_disk.cu, tools.cpp means src/red.cuda.utility/tools.cpp.
 */
#include "red_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQR(x) ((x) * (x))
#define CUBE(x) ((x) * (x) * (x))
#define GAS_REDUCTION_THRESHOLD 1.0e-6 /* pp_disk.cu:21 */
#define GAS_INNER_EDGE 0.1             /* pp_disk.cu:22 */

/* ------------------------------------------------------------------------- */
/* body classes, red_type.h:580-700                                           */
/* ------------------------------------------------------------------------- */
uint32_t orc_n_SI(const uint32_t pl[7]) { return pl[ORC_STAR] + pl[ORC_GIANT] + pl[ORC_ROCKY] + pl[ORC_PROTO]; }
uint32_t orc_n_NSI(const uint32_t pl[7]) { return pl[ORC_SUPERPL] + pl[ORC_PL]; }
uint32_t orc_n_NI(const uint32_t pl[7]) { return pl[ORC_TP]; }
uint32_t orc_n_massive(const uint32_t pl[7]) { return orc_n_SI(pl) + orc_n_NSI(pl); }
uint32_t orc_n_total(const uint32_t pl[7])
{
    uint32_t n = 0;
    for (int i = 0; i < ORC_NTYPE; i++) n += pl[i];
    return n;
}

/* get_bound_SI / NSI / NI / GD, red_type.h:670-700 */
void orc_bound(const uint32_t pl[7], int which, uint32_t out[4])
{
    const uint32_t nsi = orc_n_SI(pl), nnsi = orc_n_NSI(pl), nm = orc_n_massive(pl), nni = orc_n_NI(pl);
    switch (which) {
    case 0: out[0] = 0;   out[1] = nsi;       out[2] = 0; out[3] = nm;  break;
    case 1: out[0] = nsi; out[1] = nsi + nnsi; out[2] = 0; out[3] = nsi; break;
    case 2: out[0] = nm;  out[1] = nm + nni;  out[2] = 0; out[3] = nm;  break;
    default: out[0] = nsi; out[1] = nsi + nnsi; out[2] = 0; out[3] = 0; break;
    }
}

uint64_t orc_interactions_per_eval(const uint32_t pl[7])
{
    const uint64_t nsi = orc_n_SI(pl), nnsi = orc_n_NSI(pl), nm = orc_n_massive(pl), nni = orc_n_NI(pl);
    return (nsi ? nsi * (nm - 1) : 0) + nnsi * nsi + nni * nm;
}

/* ------------------------------------------------------------------------- */
/* gravity                                                                    */
/* ------------------------------------------------------------------------- */

/* One sink of kernel_pp_disk::calc_grav_accel_naive, pp_disk.cu:383-415:
 * a_i = sum_j m_j d / |d|^3 over the source range, j != i, id_j >= 0; the
 * sink is zeroed first and left at zero when id_i <= 0. */
static void grav_sink_naive(uint32_t i, const uint32_t b[4], const orc_bmd* md, const orc_param* p,
                            const orc_var4* r, orc_var4* a)
{
    a[i].x = a[i].y = a[i].z = a[i].w = 0.0;
    if (!(0 < md[i].id)) return;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (uint32_t j = b[2]; j < b[3]; j++) {
        if (i == j || 0 > md[j].id) continue;
        const double dx = r[j].x - r[i].x;
        const double dy = r[j].y - r[i].y;
        const double dz = r[j].z - r[i].z;
        double w = SQR(dx) + SQR(dy) + SQR(dz);
        const double d = sqrt(w);
        w = p[j].mass / (d * w);
        ax += w * dx;
        ay += w * dy;
        az += w * dz;
    }
    a[i].x = ax; a[i].y = ay; a[i].z = az;
}

/* pp_disk::cpu_calc_grav_accel_SI, pp_disk.cu:822-865: symmetric j > i loop
 * that also accumulates onto a[j] (including NSI j). */
static void grav_cpu_SI(const uint32_t b[4], const orc_bmd* md, const orc_param* p,
                        const orc_var4* r, orc_var4* a)
{
    for (uint32_t i = b[0]; i < b[1]; i++) {
        if (!(0 < md[i].id)) continue;
        for (uint32_t j = i + 1; j < b[3]; j++) {
            if (0 > md[j].id) continue;
            const double dx = r[j].x - r[i].x;
            const double dy = r[j].y - r[i].y;
            const double dz = r[j].z - r[i].z;
            double w = SQR(dx) + SQR(dy) + SQR(dz);
            const double d = sqrt(w);
            const double r_3 = 1.0 / (d * w);
            w = p[j].mass * r_3;
            a[i].x += w * dx;
            a[i].y += w * dy;
            a[i].z += w * dz;
            w = p[i].mass * r_3;
            a[j].x -= w * dx;
            a[j].y -= w * dy;
            a[j].z -= w * dz;
        }
    }
}

/* pp_disk::cpu_calc_grav_accel_NI, pp_disk.cu:933-967 */
static void grav_cpu_NI(const uint32_t b[4], const orc_bmd* md, const orc_param* p,
                        const orc_var4* r, orc_var4* a)
{
    for (uint32_t i = b[0]; i < b[1]; i++) {
        if (!(0 < md[i].id)) continue;
        for (uint32_t j = b[2]; j < b[3]; j++) {
            if (i == j || 0 > md[j].id) continue;
            const double dx = r[j].x - r[i].x;
            const double dy = r[j].y - r[i].y;
            const double dz = r[j].z - r[i].z;
            double w = SQR(dx) + SQR(dy) + SQR(dz);
            const double d = sqrt(w);
            const double r_3 = 1.0 / (d * w);
            w = p[j].mass * r_3;
            a[i].x += w * dx;
            a[i].y += w * dy;
            a[i].z += w * dz;
        }
    }
}

int orc_grav_accel(int sem, const uint32_t pl[7], const orc_bmd* md, const orc_param* p,
                   const orc_var4* r, orc_var4* a, int nthreads)
{
    uint32_t b[4];
    if (sem == ORC_SEM_CPU) {
        /* pp_disk::cpu_calc_grav_accel, pp_disk.cu:984-1012 */
        const uint32_t n = orc_n_total(pl);
        memset(a, 0, n * sizeof(orc_var4));
        if (orc_n_SI(pl)) { orc_bound(pl, 0, b); grav_cpu_SI(b, md, p, r, a); }
        if (orc_n_NSI(pl)) return ORC_ERR_NOT_IMPLEMENTED; /* pp_disk.cu:974-982 */
        if (orc_n_NI(pl)) { orc_bound(pl, 2, b); grav_cpu_NI(b, md, p, r, a); }
        return ORC_OK;
    }
    /* pp_disk::gpu_calc_grav_accel, pp_disk.cu:1014-1045: three launches, SI, NSI, NI */
    for (int which = 0; which < 3; which++) {
        orc_bound(pl, which, b);
        if (b[1] <= b[0]) continue;
        const int64_t lo = b[0], hi = b[1];
        (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1) if (nthreads > 1)
#endif
        for (int64_t i = lo; i < hi; i++) grav_sink_naive((uint32_t)i, b, md, p, r, a);
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* analytic gas drag, pp_disk.cu:59-155 and 485-521                           */
/* ------------------------------------------------------------------------- */
static double reduction_factor(int gas_decrease, double t0, double t1, double e_folding_time, double t)
{ /* pp_disk.cu:59-84 */
    switch (gas_decrease) {
    case 0: return 1.0;
    case 1:
        if (t <= t0) return 1.0;
        else if (t0 < t && t <= t1 && t0 != t1) return 1.0 - (t - t0) / (t1 - t0);
        else return 0.0;
    case 2: return exp(-(t - t0) / e_folding_time);
    default: return 1.0;
    }
}

static double get_density(const double sch[2], const double rho[2], const orc_var4* rv)
{ /* pp_disk.cu:86-105 */
    double density = 0.0;
    const double r = sqrt(SQR(rv->x) + SQR(rv->y));
    const double h = sch[0] * pow(r, sch[1]);
    const double arg = SQR(rv->z / h);
    if (GAS_INNER_EDGE < r) {
        density = rho[0] * pow(r, rho[1]) * exp(-arg);
    } else {
        const double a = rho[0] * pow(GAS_INNER_EDGE, rho[1] - 4.0);
        density = a * SQR(SQR(r)) * exp(-arg);
    }
    return density;
}

static orc_var4 circular_velocity(double mu, const orc_var4* rv)
{ /* pp_disk.cu:107-142 */
    orc_var4 res = {0.0, 0.0, 0.0, 0.0};
    const double r = sqrt(SQR(rv->x) + SQR(rv->y));
    const double vc = sqrt(mu / r);
    double p = 0.0;
    if (rv->x == 0.0 && rv->y == 0.0) {
        return res;
    } else if (rv->y == 0.0) {
        res.y = rv->x > 0.0 ? vc : -vc;
    } else if (rv->x == 0.0) {
        res.x = rv->y > 0.0 ? -vc : vc;
    } else if (rv->x >= rv->y) {
        p = rv->y / rv->x;
        res.y = rv->x >= 0 ? vc / sqrt(1.0 + SQR(p)) : -vc / sqrt(1.0 + SQR(p));
        res.x = -res.y * p;
    } else {
        p = rv->x / rv->y;
        res.x = rv->y >= 0 ? -vc / sqrt(1.0 + SQR(p)) : vc / sqrt(1.0 + SQR(p));
        res.y = -res.x * p;
    }
    return res;
}

static orc_var4 get_velocity(double mu, const double eta[2], const orc_var4* rv)
{ /* pp_disk.cu:144-155 */
    orc_var4 vg = circular_velocity(mu, rv);
    const double r = sqrt(SQR(rv->x) + SQR(rv->y));
    const double v = sqrt(1.0 - 2.0 * eta[0] * pow(r, eta[1]));
    vg.x *= v;
    vg.y *= v;
    return vg;
}

void orc_drag_accel(double t, const orc_gas* g, const uint32_t pl[7], const orc_param* p,
                    const orc_var4* r, const orc_var4* v, orc_var4* a)
{
    if (!g || orc_n_NSI(pl) == 0) return;
    const double decr = reduction_factor(g->gas_decrease, g->t0, g->t1, g->e_folding_time, t);
    if (GAS_REDUCTION_THRESHOLD > decr) return;
    uint32_t b[4];
    orc_bound(pl, 3, b);
    const double m_star = p[0].mass;
    for (uint32_t i = b[0]; i < b[1]; i++) {
        const orc_var4 vg = get_velocity(m_star, g->eta, &r[i]);
        const double ux = vg.x - v[i].x, uy = vg.y - v[i].y, uz = vg.z - v[i].z;
        const double u_n = sqrt(SQR(ux) + SQR(uy) + SQR(uz));
        const double dens = get_density(g->sch, g->rho, &r[i]);
        const double f = decr * (3.0 * p[i].cd * dens * u_n) / (8.0 * p[i].radius * p[i].density);
        a[i].x += f * ux;
        a[i].y += f * uy;
        a[i].z += f * uz;
    }
}

int orc_calc_dydx(int sem, int i, double t, const uint32_t pl[7], const orc_bmd* md,
                  const orc_param* p, const orc_gas* gas, const orc_var4* r, const orc_var4* v,
                  orc_var4* dy, int nthreads)
{ /* pp_disk::calc_dydx, pp_disk.cu:1450-1502 */
    const uint32_t n = orc_n_total(pl);
    if (i == 0) {
        memcpy(dy, v, n * sizeof(orc_var4));
        return ORC_OK;
    }
    int rc = orc_grav_accel(sem, pl, md, p, r, dy, nthreads);
    if (rc) return rc;
    if (gas) orc_drag_accel(t, gas, pl, p, r, v, dy);
    return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* integrators                                                                */
/* ------------------------------------------------------------------------- */

/* The flat vectors the stage kernels work on are the 4*N doubles of var4_t
 * arrays; red integrates the .w lane too (always 0). */

/* RK4 tableau, int_rungekutta4.cu:26-31 */
#define RK4_LAMBDA (1.0 / 10.0)
static const double rk4_a[] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0, 1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
static const double rk4_b[] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0 - RK4_LAMBDA, RK4_LAMBDA};
static const double rk4_c[] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0, 1.0};

/* RKF7(8) tableau, int_rungekutta8.cu:26-48 */
#define RK8_LAMBDA (41.0 / 840.0)
static const double rk8_c[] = {0.0, 2.0 / 27.0, 1.0 / 9.0, 1.0 / 6.0, 5.0 / 12.0, 1.0 / 2.0, 5.0 / 6.0,
                               1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0, 1.0, 0.0, 1.0};
static const double rk8_a[] = {
    0.0,
    2.0 / 27.0,
    1.0 / 36.0, 1.0 / 12.0,
    1.0 / 24.0, 0.0, 1.0 / 8.0,
    5.0 / 12.0, 0.0, -25.0 / 16.0, 25.0 / 16.0,
    1.0 / 20.0, 0.0, 0.0, 1.0 / 4.0, 1.0 / 5.0,
    -25.0 / 108.0, 0.0, 0.0, 125.0 / 108.0, -65.0 / 27.0, 125.0 / 54.0,
    31.0 / 300.0, 0.0, 0.0, 0.0, 61.0 / 225.0, -2.0 / 9.0, 13.0 / 900.0,
    2.0, 0.0, 0.0, -53.0 / 6.0, 704.0 / 45.0, -107.0 / 9.0, 67.0 / 90.0, 3.0,
    -91.0 / 108.0, 0.0, 0.0, 23.0 / 108.0, -976.0 / 135.0, 311.0 / 54.0, -19.0 / 60.0, 17.0 / 6.0, -1.0 / 12.0,
    2383.0 / 4100.0, 0.0, 0.0, -341.0 / 164.0, 4496.0 / 1025.0, -301.0 / 82.0, 2133.0 / 4100.0, 45.0 / 82.0, 45.0 / 164.0, 18.0 / 41.0,
    3.0 / 205.0, 0.0, 0.0, 0.0, 0.0, -6.0 / 41.0, -3.0 / 205.0, -3.0 / 41.0, 3.0 / 41.0, 6.0 / 41.0, 0.0,
    -1777.0 / 4100.0, 0.0, 0.0, -341.0 / 164.0, 4496.0 / 1025.0, -289.0 / 82.0, 2193.0 / 4100.0, 51.0 / 82.0, 33.0 / 164.0, 12.0 / 41.0, 0.0, 1.0};
static const double rk8_b[] = {41.0 / 840.0, 0.0, 0.0, 0.0, 0.0, 34.0 / 105.0, 9.0 / 35.0, 9.0 / 35.0,
                               9.0 / 280.0, 9.0 / 280.0, 41.0 / 840.0};

/* Nonzero terms of each RKF78 stage, in the order red's stage kernels add them
 * (rk8_kernel::calc_ytemp_for_f1..f12, int_rungekutta8.cu:80-246; the flat
 * tableau offset of row r is 1 + r(r-1)/2, int_rungekutta8.cu:431-580). */
static const int rk8_nnz[13] = {0, 1, 2, 2, 3, 3, 4, 4, 6, 7, 8, 6, 9};
static const int rk8_src[13][9] = {
    {0}, {0}, {0, 1}, {0, 2}, {0, 2, 3}, {0, 3, 4}, {0, 3, 4, 5}, {0, 4, 5, 6},
    {0, 3, 4, 5, 6, 7}, {0, 3, 4, 5, 6, 7, 8}, {0, 3, 4, 5, 6, 7, 8, 9},
    {0, 5, 6, 7, 8, 9}, {0, 3, 4, 5, 6, 7, 8, 9, 11}};

static double max_abs_err(uint32_t n_var, const double* er, const double* ev)
{ /* integrator::get_max_error, integrator.cu:222-268 (CPU branch) */
    double mr = 0.0, mv = 0.0;
    for (uint32_t i = 0; i < n_var; i++) {
        if (mr < er[i]) mr = er[i];
        if (mv < ev[i]) mv = ev[i];
    }
    return mr > mv ? mr : mv;
}

typedef struct {
    uint32_t n;
    orc_var4 *yr_t, *yv_t;  /* ytemp */
    orc_var4 *fr[13], *fv[13];
    orc_var4 *outr, *outv;  /* yout */
    double *er, *ev;
} orc_work;

static int work_alloc(orc_work* w, uint32_t n, int n_stage)
{
    memset(w, 0, sizeof(*w));
    w->n = n;
    const size_t sz = (size_t)(n ? n : 1) * sizeof(orc_var4);
    w->yr_t = calloc(1, sz); w->yv_t = calloc(1, sz);
    w->outr = calloc(1, sz); w->outv = calloc(1, sz);
    for (int s = 0; s < n_stage; s++) { w->fr[s] = calloc(1, sz); w->fv[s] = calloc(1, sz); }
    w->er = calloc((size_t)(n ? n : 1) * 4, sizeof(double));
    w->ev = calloc((size_t)(n ? n : 1) * 4, sizeof(double));
    return (w->yr_t && w->yv_t && w->outr && w->outv && w->er && w->ev) ? ORC_OK : ORC_ERR_ARG;
}

static void work_free(orc_work* w)
{
    free(w->yr_t); free(w->yv_t); free(w->outr); free(w->outv); free(w->er); free(w->ev);
    for (int s = 0; s < 13; s++) { free(w->fr[s]); free(w->fv[s]); }
}

static int dydx_both(const orc_integrator* ig, double tt, const uint32_t pl[7], const orc_bmd* md,
                     const orc_param* p, const orc_gas* gas, const orc_var4* r, const orc_var4* v,
                     orc_var4* fr, orc_var4* fv)
{
    int rc = orc_calc_dydx(ig->sem, 0, tt, pl, md, p, gas, r, v, fr, ig->nthreads);
    if (rc) return rc;
    return orc_calc_dydx(ig->sem, 1, tt, pl, md, p, gas, r, v, fv, ig->nthreads);
}

/* rungekutta4::step, int_rungekutta4.cu:173-249 */
static int step_rk4(orc_integrator* ig, double* t, const uint32_t pl[7], const orc_bmd* md,
                    const orc_param* p, const orc_gas* gas, orc_var4* r, orc_var4* v, orc_work* w)
{
    const uint32_t n_body = orc_n_total(pl);
    const uint32_t n_var = 4 * n_body;
    const int order = 4;
    int rc;
    ig->dt_try = ig->dt_next;
    rc = dydx_both(ig, *t + rk4_c[0] * ig->dt_try, pl, md, p, gas, r, v, w->fr[0], w->fv[0]);
    if (rc) return rc;
    double max_err = 0.0;
    int iter = 0;
    do {
        ig->dt_did = ig->dt_try;
        for (int stage = 1; stage < order; stage++) {
            const double tt = *t + rk4_c[stage] * ig->dt_try;
            /* rungekutta4::calc_ytemp_for_fr -> rk4_kernel::sum_vector, int_rungekutta4.cu:36-47, 111-129 */
            const double bf = rk4_a[stage] * ig->dt_try;
            const double *yr = (const double*)r, *yv = (const double*)v;
            const double *fr = (const double*)w->fr[stage - 1], *fv = (const double*)w->fv[stage - 1];
            double *tr = (double*)w->yr_t, *tv = (double*)w->yv_t;
            for (uint32_t k = 0; k < n_var; k++) {
                tr[k] = yr[k] + bf * fr[k];
                tv[k] = yv[k] + bf * fv[k];
            }
            rc = dydx_both(ig, tt, pl, md, p, gas, w->yr_t, w->yv_t, w->fr[stage], w->fv[stage]);
            if (rc) return rc;
        }
        /* rk4_kernel::calc_y_np1, int_rungekutta4.cu:49-60, 131-152 */
        const double b0 = rk4_b[0] * ig->dt_try, b1 = rk4_b[1] * ig->dt_try;
        for (int half = 0; half < 2; half++) {
            const double* y = (const double*)(half ? v : r);
            const double* f1 = (const double*)(half ? w->fv[0] : w->fr[0]);
            const double* f2 = (const double*)(half ? w->fv[1] : w->fr[1]);
            const double* f3 = (const double*)(half ? w->fv[2] : w->fr[2]);
            const double* f4 = (const double*)(half ? w->fv[3] : w->fr[3]);
            double* o = (double*)(half ? w->outv : w->outr);
            for (uint32_t k = 0; k < n_var; k++) o[k] = y[k] + b0 * (f1[k] + f4[k]) + b1 * (f2[k] + f3[k]);
        }
        if (ig->adaptive) {
            const int stage = 4;
            rc = dydx_both(ig, *t + rk4_c[stage] * ig->dt_try, pl, md, p, gas, w->outr, w->outv,
                           w->fr[stage], w->fv[stage]);
            if (rc) return rc;
            const uint32_t nv = 4 * (ig->error_check_for_tp ? n_body : orc_n_massive(pl));
            /* rk4_kernel::calc_error, int_rungekutta4.cu:62-73 */
            for (uint32_t k = 0; k < nv; k++) {
                w->er[k] = fabs(((const double*)w->fr[3])[k] - ((const double*)w->fr[4])[k]);
                w->ev[k] = fabs(((const double*)w->fv[3])[k] - ((const double*)w->fv[4])[k]);
            }
            max_err = fabs(RK4_LAMBDA * ig->dt_try * max_abs_err(nv, w->er, w->ev));
            if (0.0 < max_err) ig->dt_next = ig->dt_try *= 0.9 * pow(ig->tolerance / max_err, 1.0 / (order));
            else ig->dt_next = ig->dt_try *= 2.0;
        }
        iter++;
    } while (ig->adaptive && max_err > ig->tolerance);
    /* integrator::update_counters, integrator.cu:270-275 */
    ig->n_tried += iter; ig->n_failed += iter - 1; ig->n_passed++;
    *t += ig->dt_did;
    memcpy(r, w->outr, n_body * sizeof(orc_var4));
    memcpy(v, w->outv, n_body * sizeof(orc_var4));
    return ORC_OK;
}

/* euler::step, int_euler.cu:73-105: f0 = f(t, y); y_{n+1} = y + dt_try f0
   (euler::cpu_sum_vector, :34-40); the step size stays the constructor's
   dt_try, and dt_next = dt_try after the step */
static int step_euler(orc_integrator* ig, double* t, const uint32_t pl[7], const orc_bmd* md,
                      const orc_param* p, const orc_gas* gas, orc_var4* r, orc_var4* v, orc_work* w)
{
    const uint32_t n_body = orc_n_total(pl);
    const uint32_t n_var = 4 * n_body;
    int rc = dydx_both(ig, *t, pl, md, p, gas, r, v, w->fr[0], w->fv[0]);
    if (rc) return rc;
    const double bf = ig->dt_try;
    for (int half = 0; half < 2; half++) {
        const double* y = (const double*)(half ? v : r);
        const double* f = (const double*)(half ? w->fv[0] : w->fr[0]);
        double* o = (double*)(half ? w->outv : w->outr);
        for (uint32_t k = 0; k < n_var; k++) o[k] = y[k] + bf * f[k];
    }
    ig->dt_did = ig->dt_try;
    ig->dt_next = ig->dt_try;
    ig->n_tried += 1; ig->n_passed++;   /* update_counters(1), integrator.cu:270-275 */
    *t += ig->dt_did;
    memcpy(r, w->outr, n_body * sizeof(orc_var4));
    memcpy(v, w->outv, n_body * sizeof(orc_var4));
    return ORC_OK;
}

/* rungekutta2::step, int_rungekutta2.cu:91-131, with a = {0, 1/2}, b = {0, 1},
   c = {0, 1/2} (:12-14): f1 = f(t, y); ytemp = y + (a1 dt) f1
   (calc_ytemp_for_fr, :47-64); f2 = f(t + c1 dt, ytemp); y_{n+1} = y + (b1 dt) f2
   (calc_y_np1, :66-83); fixed step as in euler::step */
static const double rk2_a[2] = {0.0, 1.0 / 2.0}, rk2_b[2] = {0.0, 1.0}, rk2_c[2] = {0.0, 1.0 / 2.0};
static int step_rk2(orc_integrator* ig, double* t, const uint32_t pl[7], const orc_bmd* md,
                    const orc_param* p, const orc_gas* gas, orc_var4* r, orc_var4* v, orc_work* w)
{
    const uint32_t n_body = orc_n_total(pl);
    const uint32_t n_var = 4 * n_body;
    int rc = dydx_both(ig, *t + rk2_c[0] * ig->dt_try, pl, md, p, gas, r, v, w->fr[0], w->fv[0]);
    if (rc) return rc;
    const double af = rk2_a[1] * ig->dt_try;
    for (int half = 0; half < 2; half++) {
        const double* y = (const double*)(half ? v : r);
        const double* f = (const double*)(half ? w->fv[0] : w->fr[0]);
        double* o = (double*)(half ? w->yv_t : w->yr_t);
        for (uint32_t k = 0; k < n_var; k++) o[k] = y[k] + af * f[k];
    }
    rc = dydx_both(ig, *t + rk2_c[1] * ig->dt_try, pl, md, p, gas, w->yr_t, w->yv_t, w->fr[1], w->fv[1]);
    if (rc) return rc;
    const double bf = rk2_b[1] * ig->dt_try;
    for (int half = 0; half < 2; half++) {
        const double* y = (const double*)(half ? v : r);
        const double* f = (const double*)(half ? w->fv[1] : w->fr[1]);
        double* o = (double*)(half ? w->outv : w->outr);
        for (uint32_t k = 0; k < n_var; k++) o[k] = y[k] + bf * f[k];
    }
    ig->dt_did = ig->dt_try;
    ig->dt_next = ig->dt_try;
    ig->n_tried += 1; ig->n_passed++;
    *t += ig->dt_did;
    memcpy(r, w->outr, n_body * sizeof(orc_var4));
    memcpy(v, w->outv, n_body * sizeof(orc_var4));
    return ORC_OK;
}

/* ytemp = y_n + dt*(sum_s a_rs f_s) in red's term order */
static void rk8_stage_combine(int rs, double dt, uint32_t n_var, const double* y, double* const* f, double* out)
{
    const int nnz = rk8_nnz[rs];
    const int off = 1 + rs * (rs - 1) / 2;
    for (uint32_t k = 0; k < n_var; k++) {
        double acc = rk8_a[off + rk8_src[rs][0]] * f[rk8_src[rs][0]][k];
        for (int q = 1; q < nnz; q++) acc = acc + rk8_a[off + rk8_src[rs][q]] * f[rk8_src[rs][q]][k];
        out[k] = y[k] + dt * acc;
    }
}

/* rungekutta8::step, int_rungekutta8.cu:635-716 */
static int step_rk8(orc_integrator* ig, double* t, const uint32_t pl[7], const orc_bmd* md,
                    const orc_param* p, const orc_gas* gas, orc_var4* r, orc_var4* v, orc_work* w)
{
    const uint32_t n_body = orc_n_total(pl);
    const uint32_t n_var = 4 * n_body;
    const int order = 7;
    const int n_stage = ig->adaptive ? 13 : 11;
    int rc;
    double *fr[13], *fv[13];
    for (int s = 0; s < 13; s++) { fr[s] = (double*)w->fr[s]; fv[s] = (double*)w->fv[s]; }
    ig->dt_try = ig->dt_next;
    rc = dydx_both(ig, *t + rk8_c[0] * ig->dt_try, pl, md, p, gas, r, v, w->fr[0], w->fv[0]);
    if (rc) return rc;
    double max_err = 0.0;
    int iter = 0;
    do {
        ig->dt_did = ig->dt_try;
        for (int rs = 1; rs <= 10; rs++) {
            rk8_stage_combine(rs, ig->dt_try, n_var, (const double*)r, fr, (double*)w->yr_t);
            rk8_stage_combine(rs, ig->dt_try, n_var, (const double*)v, fv, (double*)w->yv_t);
            rc = dydx_both(ig, *t + rk8_c[rs] * ig->dt_try, pl, md, p, gas, w->yr_t, w->yv_t, w->fr[rs], w->fv[rs]);
            if (rc) return rc;
        }
        /* rk8_kernel::calc_y_np1, int_rungekutta8.cu:262-274 */
        const double dt = ig->dt_try;
        const double b0 = rk8_b[0], b5 = rk8_b[5], b6 = rk8_b[6], b8 = rk8_b[8], b10 = rk8_b[10];
        for (int half = 0; half < 2; half++) {
            double* const* f = half ? fv : fr;
            const double* y = (const double*)(half ? v : r);
            double* o = (double*)(half ? w->outv : w->outr);
            for (uint32_t k = 0; k < n_var; k++)
                o[k] = y[k] + dt * (b0 * f[0][k] + b5 * f[5][k] + b6 * (f[6][k] + f[7][k]) + b8 * (f[8][k] + f[9][k]) + b10 * f[10][k]);
        }
        if (ig->adaptive) {
            for (int rs = 11; rs < n_stage; rs++) {
                rk8_stage_combine(rs, ig->dt_try, n_var, (const double*)r, fr, (double*)w->yr_t);
                rk8_stage_combine(rs, ig->dt_try, n_var, (const double*)v, fv, (double*)w->yv_t);
                rc = dydx_both(ig, *t + rk8_c[rs] * ig->dt_try, pl, md, p, gas, w->yr_t, w->yv_t, w->fr[rs], w->fv[rs]);
                if (rc) return rc;
            }
            const uint32_t nv = 4 * (ig->error_check_for_tp ? n_body : orc_n_massive(pl));
            /* rk8_kernel::calc_error, int_rungekutta8.cu:248-260 */
            for (uint32_t k = 0; k < nv; k++) {
                w->er[k] = fabs(fr[0][k] + fr[10][k] - fr[11][k] - fr[12][k]);
                w->ev[k] = fabs(fv[0][k] + fv[10][k] - fv[11][k] - fv[12][k]);
            }
            max_err = fabs(RK8_LAMBDA * ig->dt_try * max_abs_err(nv, w->er, w->ev));
            if (0.0 < max_err) ig->dt_next = ig->dt_try *= 0.9 * pow(ig->tolerance / max_err, 1.0 / (order));
            else ig->dt_next = ig->dt_try *= 2.0;
        }
        iter++;
    } while (ig->adaptive && max_err > ig->tolerance);
    ig->n_tried += iter; ig->n_failed += iter - 1; ig->n_passed++;
    *t += ig->dt_did;
    memcpy(r, w->outr, n_body * sizeof(orc_var4));
    memcpy(v, w->outv, n_body * sizeof(orc_var4));
    return ORC_OK;
}

int orc_step(orc_integrator* ig, double* t, const uint32_t pl[7], const orc_bmd* md,
             const orc_param* p, const orc_gas* gas, orc_var4* r, orc_var4* v)
{
    orc_work w;
    int rc;
    const uint32_t n = orc_n_total(pl);
    if (ig->type == ORC_RK4) {
        if ((rc = work_alloc(&w, n, ig->adaptive ? 5 : 4))) { work_free(&w); return rc; }
        rc = step_rk4(ig, t, pl, md, p, gas, r, v, &w);
    } else if (ig->type == ORC_RKF78) {
        if ((rc = work_alloc(&w, n, ig->adaptive ? 13 : 11))) { work_free(&w); return rc; }
        rc = step_rk8(ig, t, pl, md, p, gas, r, v, &w);
    } else if (ig->type == ORC_EULER) {
        if ((rc = work_alloc(&w, n, 1))) { work_free(&w); return rc; }
        rc = step_euler(ig, t, pl, md, p, gas, r, v, &w);
    } else if (ig->type == ORC_RK2) {
        if ((rc = work_alloc(&w, n, 2))) { work_free(&w); return rc; }
        rc = step_rk2(ig, t, pl, md, p, gas, r, v, &w);
    } else {
        return ORC_ERR_NOT_IMPLEMENTED;
    }
    work_free(&w);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* events                                                                     */
/* ------------------------------------------------------------------------- */

/* pp_disk_utility::store_event_data, pp_disk.cu:190-253 (without the printf) */
static void store_event_data(int name, double t, double d, uint32_t idx1, uint32_t idx2,
                             const orc_param* p, const orc_var4* r, const orc_var4* v,
                             const orc_bmd* md, orc_event* e)
{
    memset(e, 0, sizeof(*e));
    e->event_name = name;
    e->d = d;
    e->t = t;
    e->id0 = md[0].id; e->id1 = md[idx1].id; e->id2 = md[idx2].id;
    e->idx0 = 0; e->idx1 = idx1; e->idx2 = idx2;
    e->r0 = r[0]; e->v0 = v[0];
    e->r1 = r[idx1]; e->v1 = v[idx1];
    e->r2 = r[idx2]; e->v2 = v[idx2];
    e->p0 = p[0];
    if (ORC_EV_EJECTION == name) {
        e->p1 = p[idx1];
        e->p2 = p[idx2];
        e->rs = e->r1;
        e->vs = e->v1;
        e->ps = e->p1;
    }
}

int orc_check_collision(int sem, double t, double factor, uint32_t n, const orc_bmd* md,
                        const orc_param* p, const orc_var4* r, const orc_var4* v,
                        orc_event* ev, uint32_t cap, uint32_t* n_ev)
{
    const double f = SQR(factor);
    uint32_t k = 0;
    int rc = ORC_OK;
    for (uint32_t i = 0; i < n; i++) {
        if (sem == ORC_SEM_GPU) {
            if (!(0 < md[i].id)) continue;                                 /* pp_disk.cu:336 */
        } else {
            if (!(0 < md[i].id && ORC_STAR != md[i].body_type)) continue; /* pp_disk.cu:1149 */
        }
        for (uint32_t j = i + 1; j < n; j++) {
            if (sem == ORC_SEM_GPU) {
                if (0 > md[j].id) continue;                                /* pp_disk.cu:342 */
            } else {
                if (0 > md[j].id && ORC_STAR != md[j].body_type) continue; /* pp_disk.cu:1155 */
            }
            const double dx = r[j].x - r[i].x;
            const double dy = r[j].y - r[i].y;
            const double dz = r[j].z - r[i].z;
            const double w = SQR(dx) + SQR(dy) + SQR(dz);
            if (w < f * SQR((p[i].radius + p[j].radius))) {
                uint32_t surv = i, merg = j;
                if (p[merg].mass > p[surv].mass) { uint32_t x = surv; surv = merg; merg = x; }
                if (k < cap) store_event_data(ORC_EV_COLLISION, t, sqrt(w), surv, merg, p, r, v, md, &ev[k]);
                else rc = ORC_ERR_OVERFLOW;
                k++;
            }
        }
    }
    *n_ev = k;
    return rc;
}

/* orc_check_collision with the i loop split over nthreads (OpenMP); the events
 * come out in the same (i, j) order as the sequential loop. */
int orc_check_collision_mt(int sem, double t, double factor, uint32_t n, const orc_bmd* md,
                           const orc_param* p, const orc_var4* r, const orc_var4* v,
                           orc_event* ev, uint32_t cap, uint32_t* n_ev, int nthreads)
{
    if (nthreads <= 1) return orc_check_collision(sem, t, factor, n, md, p, r, v, ev, cap, n_ev);
    const double f = SQR(factor);
    /* pass 1: events per i (count only) */
    uint32_t* cnt = calloc(n ? n : 1, sizeof(uint32_t));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        if (sem == ORC_SEM_GPU ? !(0 < md[i].id) : !(0 < md[i].id && ORC_STAR != md[i].body_type)) continue;
        uint32_t c = 0;
        for (uint32_t j = i + 1; j < n; j++) {
            if (sem == ORC_SEM_GPU ? (0 > md[j].id) : (0 > md[j].id && ORC_STAR != md[j].body_type)) continue;
            const double dx = r[j].x - r[i].x;
            const double dy = r[j].y - r[i].y;
            const double dz = r[j].z - r[i].z;
            const double w = SQR(dx) + SQR(dy) + SQR(dz);
            if (w < f * SQR((p[i].radius + p[j].radius))) c++;
        }
        cnt[i] = c;
    }
    uint32_t total = 0;
    for (uint32_t i = 0; i < n; i++) total += cnt[i];
    free(cnt);
    if (total == 0) { *n_ev = 0; return ORC_OK; }
    /* events exist (rare): the sequential loop writes them in order */
    return orc_check_collision(sem, t, factor, n, md, p, r, v, ev, cap, n_ev);
}

int orc_check_ejection_hit_centrum(double t, double ejection, double hit_centrum, uint32_t n,
                                   const orc_bmd* md, const orc_param* p, const orc_var4* r,
                                   const orc_var4* v, orc_event* ev, uint32_t cap, uint32_t* n_ev)
{ /* kernel_pp_disk::check_for_ejection_hit_centrum, pp_disk.cu:283-318 */
    const double ed2 = (0.0 < ejection ? SQR(ejection) : DBL_MAX);
    const double hcd2 = SQR(hit_centrum);
    uint32_t k = 0;
    int rc = ORC_OK;
    for (uint32_t i = 0; i < n; i++) {
        if (!(md[i].id > 0 && md[i].body_type != ORC_STAR)) continue;
        const double r2 = SQR(r[i].x) + SQR(r[i].y) + SQR(r[i].z);
        if (ed2 < r2) {
            if (k < cap) store_event_data(ORC_EV_EJECTION, t, sqrt(r2), 0, i, p, r, v, md, &ev[k]);
            else rc = ORC_ERR_OVERFLOW;
            k++;
        }
        if (hcd2 > r2) {
            if (k < cap) store_event_data(ORC_EV_HIT_CENTRUM, t, sqrt(r2), 0, i, p, r, v, md, &ev[k]);
            else rc = ORC_ERR_OVERFLOW;
            k++;
        }
    }
    *n_ev = k;
    return rc;
}

uint32_t orc_populate_sp_events(orc_event* ev, uint32_t n_ev)
{ /* pp_disk::populate_sp_events, pp_disk.cu:1250-1288 */
    if (n_ev == 0) return 0;
    char* processed = calloc(n_ev, 1);
    orc_event* sp = malloc(n_ev * sizeof(orc_event));
    uint32_t n = 0;
    for (uint32_t k = 0; k < n_ev; k++) {
        if (processed[k]) continue;
        processed[k] = 1;
        sp[n] = ev[k];
        for (uint32_t i = k + 1; i < n_ev; i++) {
            if (sp[n].id1 == ev[i].id1 && sp[n].id2 == ev[i].id2) {
                processed[i] = 1;
                if (sp[n].t > ev[i].t) sp[n] = ev[i];
            }
        }
        n++;
    }
    memcpy(ev, sp, n * sizeof(orc_event));
    free(sp);
    free(processed);
    return n;
}

/* tools.cpp:455-460 */
double orc_calc_radius(double m, double density)
{
    static const double four_pi_over_three = 4.188790204786391;
    return pow(1.0 / four_pi_over_three * m / density, 1.0 / 3.0);
}
/* tools.cpp:462-472 */
double orc_calc_density(double m, double R)
{
    static const double four_pi_over_three = 4.188790204786391;
    if (R == 0.0) return 0.0;
    return m / (four_pi_over_three * CUBE(R));
}
/* tools.cpp:474-479 */
double orc_calc_mass(double R, double density)
{
    static const double four_pi_over_three = 4.188790204786391;
    return four_pi_over_three * CUBE(R) * density;
}
/* tools.cpp:480-487 */
void orc_calc_position_after_collision(double m1, double m2, const orc_var4* r1, const orc_var4* r2, orc_var4* r)
{
    const double M = m1 + m2;
    r->x = (m1 * r1->x + m2 * r2->x) / M;
    r->y = (m1 * r1->y + m2 * r2->y) / M;
    r->z = (m1 * r1->z + m2 * r2->z) / M;
}
/* tools.cpp:489-496 */
void orc_calc_velocity_after_collision(double m1, double m2, const orc_var4* v1, const orc_var4* v2, orc_var4* v)
{
    const double M = m1 + m2;
    v->x = (m1 * v1->x + m2 * v2->x) / M;
    v->y = (m1 * v1->y + m2 * v2->y) / M;
    v->z = (m1 * v1->z + m2 * v2->z) / M;
}
/* tools.cpp:498-507 */
void orc_calc_physical_properties(const orc_param* p1, const orc_param* p2, orc_param* p)
{
    const double volume = 4.188790204786391 * (CUBE(p1->radius) + CUBE(p2->radius));
    p->mass = p1->mass + p2->mass;
    p->density = p->mass / volume;
    p->radius = orc_calc_radius(p->mass, p->density);
    p->cd = p1->cd;
}

/* pp_disk::handle_collision_pair, pp_disk.cu:1328-1368 */
static int handle_collision_pair(orc_event* c, orc_var4* r, orc_var4* v, orc_param* p, const orc_bmd* md)
{
    const uint32_t s = c->idx1, m = c->idx2;
    if (ORC_SUPERPL == md[m].body_type) return ORC_ERR_SUPERPLANETESIMAL;
    c->p1 = p[s];
    c->p2 = p[m];
    orc_calc_position_after_collision(c->p1.mass, c->p2.mass, &c->r1, &c->r2, &c->rs);
    orc_calc_velocity_after_collision(c->p1.mass, c->p2.mass, &c->v1, &c->v2, &c->vs);
    r[s] = c->rs;
    v[s] = c->vs;
    orc_calc_physical_properties(&c->p1, &c->p2, &c->ps);
    p[s] = c->ps;
    return ORC_OK;
}

int orc_handle_collision(orc_event* ev, uint32_t* n_ev, orc_var4* r, orc_var4* v, orc_param* p,
                         orc_bmd* md, uint32_t inactive[7])
{ /* pp_disk::handle_collision, pp_disk.cu:1220-1248 */
    const uint32_t n = orc_populate_sp_events(ev, *n_ev);
    *n_ev = n;
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t ictv = ev[i].idx2;
        int rc = handle_collision_pair(&ev[i], r, v, p, md);
        if (rc) return rc;
        md[ictv].id *= -1;
        inactive[md[ictv].body_type]++;
    }
    return ORC_OK;
}

int orc_handle_ejection_hit_centrum(orc_event* ev, uint32_t n_ev, orc_var4* r, orc_var4* v,
                                    orc_param* p, orc_bmd* md, uint32_t inactive[7])
{ /* pp_disk::handle_ejection_hit_centrum, pp_disk.cu:1290-1326 */
    for (uint32_t i = 0; i < n_ev; i++) {
        const uint32_t ictv = ev[i].idx2;
        if (ORC_EV_EJECTION != ev[i].event_name) {
            int rc = handle_collision_pair(&ev[i], r, v, p, md);
            if (rc) return rc;
        }
        md[ictv].id *= -1;
        inactive[md[ictv].body_type]++;
    }
    return ORC_OK;
}

uint32_t orc_rebuild_vectors(uint32_t n_total, orc_var4* r, orc_var4* v, orc_param* p, orc_bmd* md,
                             uint32_t playing[7], uint32_t inactive[7], uint32_t removed[7],
                             int32_t* perm_out)
{ /* pp_disk::rebuild_vectors, pp_disk.cu:1370-1430 */
    uint32_t n_active = 0;
    for (int i = 0; i < ORC_NTYPE; i++) n_active += playing[i] - inactive[i];
    uint32_t k = 0;
    for (uint32_t i = 0; i < n_total; i++) {
        if (0 < md[i].id && n_active > k) {
            r[k] = r[i]; v[k] = v[i]; p[k] = p[i]; md[k] = md[i];
            if (perm_out) perm_out[k] = (int32_t)i;
            k++;
        }
    }
    /* n_objects::update, red_type.h:568-578 */
    for (int i = 0; i < ORC_NTYPE; i++) {
        playing[i] -= inactive[i];
        removed[i] += inactive[i];
        inactive[i] = 0;
    }
    return k;
}

/* ------------------------------------------------------------------------- */
/* integrals                                                                  */
/* ------------------------------------------------------------------------- */
void orc_calc_integral(uint32_t n, const orc_bmd* md, const orc_param* p, const orc_var4* r,
                       const orc_var4* v, double out[10])
{
    /* tools::get_total_mass, tools.cpp:367-380 */
    double M0 = 0.0;
    for (int j = (int)n - 1; j >= 0; j--) {
        if (0 > md[j].id) continue;
        M0 += p[j].mass;
    }
    /* tools::calc_bc, tools.cpp:384-410 */
    double R[3] = {0, 0, 0}, V[3] = {0, 0, 0};
    for (int j = (int)n - 1; j >= 0; j--) {
        if (0 > md[j].id) continue;
        const double m = p[j].mass;
        R[0] += m * r[j].x; R[1] += m * r[j].y; R[2] += m * r[j].z;
        V[0] += m * v[j].x; V[1] += m * v[j].y; V[2] += m * v[j].z;
    }
    R[0] /= M0; R[1] /= M0; R[2] /= M0;
    V[0] /= M0; V[1] /= M0; V[2] /= M0;
    /* tools::calc_angular_momentum, tools.cpp:545-565 */
    double C[3] = {0, 0, 0};
    for (uint32_t i = 0; i < n; i++) {
        if (0 > md[i].id) continue;
        double cx = r[i].y * v[i].z - r[i].z * v[i].y;
        double cy = r[i].z * v[i].x - r[i].x * v[i].z;
        double cz = r[i].x * v[i].y - r[i].y * v[i].x;
        cx *= p[i].mass; cy *= p[i].mass; cz *= p[i].mass;
        C[0] += cx; C[1] += cy; C[2] += cz;
    }
    /* tools::calc_kinetic_energy / calc_potential_energy, tools.cpp:591-694 */
    double T = 0.0;
    for (uint32_t i = 0; i < n; i++) {
        if (0 > md[i].id) continue;
        T += p[i].mass * (SQR(v[i].x) + SQR(v[i].y) + SQR(v[i].z));
    }
    T = T / 2.0;
    double U = 0.0;
    for (uint32_t i = 0; i < n; i++) {
        if (0 > md[i].id) continue;
        for (uint32_t j = 0; j < n; j++) {
            if (i == j) continue;
            if (0 > md[j].id) continue;
            const double rij = sqrt(SQR(r[j].x - r[i].x) + SQR(r[j].y - r[i].y) + SQR(r[j].z - r[i].z));
            U += p[i].mass * p[j].mass / rij;
        }
    }
    U = U / 2.0;
    out[0] = R[0]; out[1] = R[1]; out[2] = R[2];
    out[3] = V[0]; out[4] = V[1]; out[5] = V[2];
    out[6] = C[0]; out[7] = C[1]; out[8] = C[2];
    out[9] = T - U;
}

void orc_calc_energy_interacting(const uint32_t pl[7], const orc_bmd* md, const orc_param* p,
                                 const orc_var4* r, const orc_var4* v, double out[4], int nthreads)
{
    const uint32_t nsi = orc_n_SI(pl), nm = orc_n_massive(pl);
    double T = 0.0, C[3] = {0, 0, 0};
    for (uint32_t i = 0; i < nm; i++) {
        if (0 > md[i].id) continue;
        T += p[i].mass * (SQR(v[i].x) + SQR(v[i].y) + SQR(v[i].z));
        C[0] += p[i].mass * (r[i].y * v[i].z - r[i].z * v[i].y);
        C[1] += p[i].mass * (r[i].z * v[i].x - r[i].x * v[i].z);
        C[2] += p[i].mass * (r[i].x * v[i].y - r[i].y * v[i].x);
    }
    double U = 0.0;
    (void)nthreads;
    /* pairs (i < j) with i in SI; NSI-NSI pairs do not interact in red */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : U) num_threads(nthreads > 0 ? nthreads : 1) if (nthreads > 1)
#endif
    for (int64_t ii = 0; ii < (int64_t)nsi; ii++) {
        const uint32_t i = (uint32_t)ii;
        if (0 > md[i].id) continue;
        double u = 0.0;
        for (uint32_t j = i + 1; j < nm; j++) {
            if (0 > md[j].id) continue;
            const double rij = sqrt(SQR(r[j].x - r[i].x) + SQR(r[j].y - r[i].y) + SQR(r[j].z - r[i].z));
            u += p[i].mass * p[j].mass / rij;
        }
        U += u;
    }
    out[0] = T / 2.0 - U;
    out[1] = C[0]; out[2] = C[1]; out[3] = C[2];
}
