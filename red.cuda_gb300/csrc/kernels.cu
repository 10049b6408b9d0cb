// kernels.cu -- the sm_103a kernels of libredgb.
//
//   (k_stage, one Runge-Kutta stage, is in stage.cuh / stage_*.cu)
//   k_prep      positions of stage 0 from y (FP32 double-single copies)
//   k_control   per-system error -> accept / reject -> new step size
//   k_finish    y_{n+1} for accepted systems, positions of the next stage 0,
//               the small bodies into the collision check's spatial hash
//   k_collide   the collision check after a try: tile pairs of the large
//               bodies (FP32 prefilter + red's FP64 test) and hash queries
//   k_collision, k_grid_insert, k_grid_query   the same, for the explicit check
//   k_ejhc      ejection / hit-centrum test
//   k_potential per-body potential sums for the integrals
#include <algorithm>
#include <cfloat>
#include <cstdio>

#include "common.cuh"

namespace redgb {

namespace {
thread_local bool t_pdl = false;
}
void set_pdl(bool on) { t_pdl = on; }
bool pdl_on() { return t_pdl; }

// ---------------------------------------------------------------------------
// per-body kernels
// ---------------------------------------------------------------------------
// FP32 copies of y_r for stage 0 (buffer 0), and the mass / radius words of
// both stage buffers: the stage kernels write only x, y, z, so the .w words
// set here hold until the next host update of the bodies.
__global__ void __launch_bounds__(kSegment) k_prep(const Segment* segs, const SysInfo* sinfo, const DevSys* sys,
                                                   const double* y_r, const double* mass, const double* radius,
                                                   const int* id, float4* hi, float4* lo, float4* hi1, float4* lo1,
                                                   int all)
{
    const Segment sg = segs[blockIdx.x];
    if (!all && !runnable(sys[sg.sys])) return;
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1) return;
    const double m_eff = id[i] >= 0 ? mass[i] : 0.0;
    write_pos(hi, lo, i, y_r[3 * i], y_r[3 * i + 1], y_r[3 * i + 2], m_eff, radius[i]);
    reinterpret_cast<float*>(hi1 + i)[3] = __double2float_rn(m_eff);
    reinterpret_cast<float*>(lo1 + i)[3] = __double2float_rn(radius[i]);
}

// One thread per system: integrator::step's accept / reject logic
// (int_rungekutta8.cu:690-716, int_rungekutta4.cu:226-248), the counters
// (integrator.cu:270-275) and run_simulation's dt_next clamp and loop bound
// (main.cu:471, 535-538).
__global__ void k_control(const ControlParams P)
{
    pdl_wait();
    pdl_trigger();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.n_sys) return;
    DevSys& S = P.sys[s];
    S.accepted = 0;
    if (!runnable(S)) return;
    const double dt = S.dt_try;
    double dt_new = dt;
    S.iter++;
    if (P.adaptive) {
        const double err = __longlong_as_double((long long)S.err_bits);
        S.err_bits = 0ull;
        const double max_err = fabs(P.lambda * dt * err);
        S.err_last = max_err;
        if (max_err != max_err) {
            S.status = 5;   // RED_ERR_NONFINITE
            S.halted = 1;
            S.active = 0;
            return;
        }
        // the red-exact mode takes the nearest double of the power, as the C
        // library's pow of red's host controller does (crmath.cuh)
        if (0.0 < max_err)
            dt_new = dt * (0.9 * (P.exact ? crmath::cr_pow(P.tolerance / max_err, 1.0 / (double)P.order)
                                          : pow(P.tolerance / max_err, 1.0 / (double)P.order)));
        else dt_new = dt * 2.0;
        if (max_err > P.tolerance) {
            S.dt_try = dt_new;
            S.dt_next = dt_new;
            return;
        }
    }
    S.dt_did = dt;
    S.dt_next = dt_new;
    S.t += dt;
    S.n_tried += (unsigned long long)S.iter;
    S.n_failed += (unsigned long long)(S.iter - 1);
    S.n_passed += 1ull;
    S.iter = 0;
    S.accepted = 1;
    if (S.quota > 0) S.quota--;
    if (P.output_interval != 0.0 && fabs(P.output_interval) < fabs(S.dt_next))
        S.dt_next = 0.0 < dt ? P.output_interval : -P.output_interval;
    // euler::step / rungekutta2::step take dt_try, never dt_next (int_euler.cu:73-105)
    if (!P.keep_dt) S.dt_try = S.dt_next;
    if (P.length != 0.0 && fabs(S.t - S.t_start) > fabs(P.length)) S.active = 0;
}

// Spatial-hash broad phase for the small bodies.  Cell coordinates are
// clamped so that far-away bodies share border cells (tested exactly, never
// missed).
__device__ __forceinline__ int cell_coord(double x, double inv_h)
{
    const double lim = 1.0e9;
    return (int)floor(fmin(fmax(x * inv_h, -lim), lim));
}
__device__ __forceinline__ int4 cell_of(double x, double y, double z, double inv_h)
{
    return make_int4(cell_coord(x, inv_h), cell_coord(y, inv_h), cell_coord(z, inv_h), 0);
}

__device__ __forceinline__ int bucket_of(int cx, int cy, int cz, int mask)
{
    const unsigned h = ((unsigned)cx * 73856093u) ^ ((unsigned)cy * 19349663u) ^ ((unsigned)cz * 83492791u);
    return (int)(h & (unsigned)mask);
}

// Inserts small body i at position (x, y, z) into its system's hash table.
__device__ __forceinline__ void grid_insert_one(const GridInfo& g, int4* cell, int* next, int* head, int i, double x,
                                                double y, double z)
{
    const int4 c = cell_of(x, y, z, g.inv_h);
    cell[i] = c;
    next[i] = atomicExch(&head[g.toff + bucket_of(c.x, c.y, c.z, g.mask)], i);
}

// y_{n+1} of the accepted systems and the positions of the next stage 0.  One
// thread per component: element e of a segment of kFinishBodies bodies is
// component e % 3 of body e / 3, contiguous in memory, so every FP64 warp
// instruction runs on full warps (the FP64 pipe charges a warp instruction the
// same for any number of active lanes).  The threads then form the hash-cell
// coordinate of their component, and one thread per small body inserts it
// into the collision check's spatial hash.
template <bool EXACT>
__global__ void __launch_bounds__(3 * kFinishBodies) k_finish(const FinishParams P)
{
    pdl_wait();
    pdl_trigger();
    __shared__ int cellc[3 * kFinishBodies];
    const Segment sg = P.segs[blockIdx.x];
    DevSys* S = P.sys + sg.sys;
    if (S->halted) return;
    const bool acc = S->accepted;
    if (!acc && !runnable(*S)) return;   // uniform over the CTA
    const int e = threadIdx.x;
    const int nb = sg.b1 - sg.b0;
    const bool live = e < 3 * nb;
    const int i = sg.b0 + e / 3;
    const int c = e % 3;
    const int x = 3 * sg.b0 + e;
    double r = 0.0;
    if (live) {
        if (acc) {
            const double dt = S->dt_did;
            double v;
            if (P.scheme == SCHEME_RKF78) {
                r = rk8_ynp1<EXACT>(P.y_r[x], dt, P.Kr, x);
                v = rk8_ynp1<EXACT>(P.y_v[x], dt, P.Kv, x);
            } else if (P.scheme == SCHEME_EULER) {
                // euler::calc_y_np1 -> sum_vector, int_euler.cu:19-31, 54-71: y + dt f0
                r = madd<EXACT>(P.y_r[x], dt, P.Kr[0][x]);
                v = madd<EXACT>(P.y_v[x], dt, P.Kv[0][x]);
            } else if (P.scheme == SCHEME_RK2) {
                // rungekutta2::calc_y_np1, int_rungekutta2.cu:66-83: y + (b_1 dt) f2
                const double bf = mul<EXACT>(c_tb.b2[1], dt);
                r = madd<EXACT>(P.y_r[x], bf, P.Kr[1][x]);
                v = madd<EXACT>(P.y_v[x], bf, P.Kv[1][x]);
            } else if (P.commit_from_stage4) {
                r = P.t_r0[x];
                v = P.Kr[4][x];
            } else {
                const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
                r = rk4_ynp1<EXACT>(P.y_r[x], b0, b1, P.Kr[0][x], P.Kr[1][x], P.Kr[2][x], P.Kr[3][x]);
                v = rk4_ynp1<EXACT>(P.y_v[x], b0, b1, P.Kv[0][x], P.Kv[1][x], P.Kv[2][x], P.Kv[3][x]);
            }
            P.y_r[x] = r;
            P.y_v[x] = v;
            // finiteness from the exponent bits (integer pipe, not the FP64 pipe)
            const long long br = __double_as_longlong(r), bv = __double_as_longlong(v);
            if (((br >> 52) & 0x7ff) == 0x7ff || ((bv >> 52) & 0x7ff) == 0x7ff) S->status = 5;   // RED_ERR_NONFINITE
        } else {
            r = P.y_r[x];
        }
        // x, y, z of the FP32 copies; k_prep holds the .w words (mass, radius)
        write_pos_c(P.pos_hi0, P.pos_lo0, i, c, r);
    }
    if (P.head && acc) {   // uniform over the CTA
        const GridInfo g = P.grid[sg.sys];
        if (!g.enabled) return;
        if (live) cellc[e] = cell_coord(r, g.inv_h);
        __syncthreads();
        const int small0 = P.sinfo[sg.sys].off + P.sinfo[sg.sys].n_SI;
        if (e < nb && sg.b0 + e >= small0) {
            const int b = sg.b0 + e;
            const int4 cl = make_int4(cellc[3 * e], cellc[3 * e + 1], cellc[3 * e + 2], 0);
            P.cell[b] = cl;
            P.next[b] = atomicExch(&P.head[g.toff + bucket_of(cl.x, cl.y, cl.z, g.mask)], b);
        }
    }
}

// ---------------------------------------------------------------------------
// collision detection: kernel_pp_disk::check_for_collision (pp_disk.cu:320-371)
// over tile pairs; an FP32 double-single prefilter with a safety margin picks
// the candidates, red's FP64 test (no FMA) decides.
// ---------------------------------------------------------------------------
// After a try the check runs for the systems that just accepted one (a halted
// system makes no tries, so it never has `accepted` set); the explicit check
// runs for every system.  `halted` is not consulted: the first kernel of the
// check may set it.
__device__ __forceinline__ bool coll_runs(const CollParams& P, const DevSys& S)
{
    return !P.only_accepted || S.accepted;
}

// red's test for one pair i < j, bit for bit (pp_disk.cu:336-357), and the event.
__device__ __forceinline__ void collide_exact(const CollParams& P, DevSys* S, int sys, int i, int jx, double f)
{
    if (!(0 < P.id[i]) || 0 > P.id[jx]) return;
    const double ddx = __dsub_rn(P.y_r[3 * jx], P.y_r[3 * i]);
    const double ddy = __dsub_rn(P.y_r[3 * jx + 1], P.y_r[3 * i + 1]);
    const double ddz = __dsub_rn(P.y_r[3 * jx + 2], P.y_r[3 * i + 2]);
    const double w = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
    const double rs = __dadd_rn(P.radius[i], P.radius[jx]);
    if (!(w < __dmul_rn(f, __dmul_rn(rs, rs)))) return;
    int surv = i, merg = jx;
    if (P.mass[merg] > P.mass[surv]) {
        surv = jx;
        merg = i;
    }
    const unsigned kk = atomicAdd(P.n_events, 1u);
    if (kk < P.capacity) {
        DevEvent ev;
        ev.sys = sys;
        ev.name = 3;   // RED_EVENT_COLLISION
        ev.i = i;
        ev.j = jx;
        ev.surv = surv;
        ev.merg = merg;
        ev.d = __dsqrt_rn(w);
        P.events[kk] = ev;
    }
    if (P.mark) {
        atomicAdd(&S->n_coll, 1);
        S->halted = 1;
    }
}

// Brute-force tile pairs: the large bodies (SI class) against every later body.
// One thread per later body j; the i tile (the SI bodies) sits in shared
// memory.  FP32 double-single prefilter with a safety margin, red's FP64
// test decides.
__device__ __forceinline__ void coll_pairs(const CollParams& P, int item)
{
    __shared__ float4 shi[kTile], slo[kTile];
    const PairItem it = P.items[item];
    DevSys* S = P.sys + it.sys;
    if (!coll_runs(P, *S)) return;
    const SysInfo si = P.sinfo[it.sys];
    const int end = si.off + si.n;
    const int ni = min(kTile, it.i1 - it.i0);
    if (threadIdx.x < ni) {
        shi[threadIdx.x] = P.pos_hi[it.i0 + threadIdx.x];
        slo[threadIdx.x] = P.pos_lo[it.i0 + threadIdx.x];
    }
    __syncthreads();
    const int j = it.j0 + threadIdx.x;
    if (j >= end) return;
    const float4 H = P.pos_hi[j], Lo = P.pos_lo[j];
    const float fac = (float)P.factor;
    const double f = P.factor * P.factor;
    const int nii = min(ni, j - it.i0);   // i < j
    for (int ii = 0; ii < nii; ii++) {
        const float4 h = shi[ii], l = slo[ii];
        const float dx = (H.x - h.x) + (Lo.x - l.x);
        const float dy = (H.y - h.y) + (Lo.y - l.y);
        const float dz = (H.z - h.z) + (Lo.z - l.z);
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float th = fac * (Lo.w + l.w);
        if (!(d2 <= 1.0001f * th * th + 1.0e-30f)) continue;
        collide_exact(P, S, it.sys, it.i0 + ii, j, f);
    }
}

__global__ void __launch_bounds__(kTile) k_collision(const CollParams P)
{
    pdl_wait();
    pdl_trigger();
    coll_pairs(P, blockIdx.x);
}



__global__ void __launch_bounds__(kSegment) k_grid_insert(const CollParams P)
{
    pdl_wait();
    pdl_trigger();
    const Segment sg = P.segs[blockIdx.x];
    const DevSys& S = P.sys[sg.sys];
    const GridInfo g = P.grid[sg.sys];
    if (!g.enabled || !coll_runs(P, S)) return;
    const SysInfo si = P.sinfo[sg.sys];
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1 || i < si.off + si.n_SI) return;
    grid_insert_one(g, P.cell, P.next, P.head, i, P.y_r[3 * i], P.y_r[3 * i + 1], P.y_r[3 * i + 2]);
}

// Half of the neighbourhood: the own cell (pairs with j > i) and the 13 cells
// of the forward half-space, so that every unordered pair of small bodies in
// neighbouring cells is seen once; the pair is tested as (min, max) like red's
// i < j loop.  The 14 bucket lists are walked side by side: each round loads
// the current element of every list at once, so a thread needs as many
// dependent memory round trips as its longest list, not their sum.
__device__ __forceinline__ void grid_query(const CollParams& P, int seg, int local)
{
    const Segment sg = P.segs[seg];
    DevSys* S = P.sys + sg.sys;
    const GridInfo g = P.grid[sg.sys];
    if (!g.enabled || !coll_runs(P, *S)) return;
    const SysInfo si = P.sinfo[sg.sys];
    const int i = sg.b0 + local;
    if (i >= sg.b1 || i < si.off + si.n_SI) return;
    const double f = P.factor * P.factor;
    const int4 c = P.cell[i];
    constexpr int kNb = 14;
    int cur[kNb];
    int4 nb[kNb];
    int q = 0;
#pragma unroll
    for (int dz = 0; dz <= 1; dz++)
#pragma unroll
        for (int dy = -1; dy <= 1; dy++)
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) {
                const bool fwd = dz > 0 || (dz == 0 && (dy > 0 || (dy == 0 && dx >= 0)));
                if (!fwd) continue;
                nb[q] = make_int4(c.x + dx, c.y + dy, c.z + dz, 0);
                cur[q] = __ldcg(P.head + g.toff + bucket_of(nb[q].x, nb[q].y, nb[q].z, g.mask));
                q++;
            }
    // a list is at most as long as the system's small-body count: the bound ends every walk
    const int bound = si.n - si.n_SI;
    bool any = true;
    for (int round = 0; any && round <= bound; round++) {
        int4 cj[kNb];
        int nx[kNb];
#pragma unroll
        for (int b = 0; b < kNb; b++) {
            if (cur[b] >= 0) {
                cj[b] = P.cell[cur[b]];
                nx[b] = __ldcg(P.next + cur[b]);
            }
        }
        any = false;
#pragma unroll
        for (int b = 0; b < kNb; b++) {
            if (cur[b] >= 0) {
                const int j = cur[b];
                if (cj[b].x == nb[b].x && cj[b].y == nb[b].y && cj[b].z == nb[b].z && (b != 0 || j > i))
                    collide_exact(P, S, sg.sys, min(i, j), max(i, j), f);
                cur[b] = nx[b];
                any = any || nx[b] >= 0;
            }
        }
    }
}

__global__ void __launch_bounds__(kSegment) k_grid_query(const CollParams P)
{
    pdl_wait();
    pdl_trigger();
    grid_query(P, blockIdx.x, threadIdx.x);
}

// The collision check after a try in one launch: CTAs [0, n_pairs) test the
// tile pairs of the large bodies, the others run the hash-grid query for half
// a segment each (the bodies were inserted by k_finish).
static_assert(kSegment == 2 * kTile, "k_collide runs half a segment per CTA");
__global__ void __launch_bounds__(kTile) k_collide(const CollParams P, int n_pairs)
{
    pdl_wait();
    pdl_trigger();
    if ((int)blockIdx.x < n_pairs) {
        coll_pairs(P, blockIdx.x);
        return;
    }
    const int q = (int)blockIdx.x - n_pairs;
    grid_query(P, q / 2, (q % 2) * kTile + (int)threadIdx.x);
}

// kernel_pp_disk::check_for_ejection_hit_centrum (pp_disk.cu:283-318)
__global__ void __launch_bounds__(kSegment) k_ejhc(const EjhcParams P)
{
    pdl_wait();
    pdl_trigger();
    const Segment sg = P.segs[blockIdx.x];
    DevSys* S = P.sys + sg.sys;
    if (P.only_accepted && !S->accepted) return;
    if (S->halted && P.only_accepted) return;
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1) return;
    const double ed2 = 0.0 < P.ejection ? P.ejection * P.ejection : DBL_MAX;
    const double hcd2 = P.hit_centrum * P.hit_centrum;
    if (!(P.id[i] > 0 && P.btype[i] != 0)) return;
    const double x = P.y_r[3 * i], y = P.y_r[3 * i + 1], z = P.y_r[3 * i + 2];
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    const int star = P.sinfo[sg.sys].off;
    for (int which = 0; which < 2; which++) {
        const bool hit = which == 0 ? (ed2 < r2) : (hcd2 > r2);
        if (!hit) continue;
        const unsigned kk = atomicAdd(P.n_events, 1u);
        if (kk < P.capacity) {
            DevEvent ev;
            ev.sys = sg.sys;
            ev.name = which == 0 ? 2 : 1;   // RED_EVENT_EJECTION : RED_EVENT_HIT_CENTRUM
            ev.i = star;
            ev.j = i;
            ev.surv = star;
            ev.merg = i;
            ev.d = __dsqrt_rn(r2);
            P.events[kk] = ev;
        }
        if (P.mark) {
            atomicAdd(&S->n_ejhc, 1);
            S->halted = 1;
        }
    }
}

// Per-body potential sums in FP64: u_i = m_i * sum_j m_j / r_ij over the
// partners of i (all other active bodies, or the interacting partners j > i).
__global__ void __launch_bounds__(kSegment) k_potential(const Segment* segs, const SysInfo* sinfo,
                                                        const double* y_r, const double* mass, const int* id,
                                                        int sys_filter, int interacting, double* u)
{
    const Segment sg = segs[blockIdx.x];
    if (sg.sys != sys_filter) return;
    const SysInfo si = sinfo[sg.sys];
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1) return;
    double acc = 0.0;
    if (id[i] >= 0) {
        const double xi = y_r[3 * i], yi = y_r[3 * i + 1], zi = y_r[3 * i + 2];
        int j0 = si.off, j1 = si.off + si.n;
        if (interacting) {
            // each interacting pair once: from its SI member i towards j > i among the massive bodies
            const int rel = i - si.off;
            j0 = i + 1;
            j1 = rel < si.n_SI ? si.off + si.n_massive : j0;
        }
        for (int j = j0; j < j1; j++) {
            if (j == i || id[j] < 0) continue;
            const double dx = y_r[3 * j] - xi, dy = y_r[3 * j + 1] - yi, dz = y_r[3 * j + 2] - zi;
            acc += mass[j] / sqrt(dx * dx + dy * dy + dz * dz);
        }
        acc *= mass[i];
    }
    u[i] = acc;
}

// ---------------------------------------------------------------------------
// host transfers: one system's bodies between the device's structure of
// arrays and the caller's records (var4_t r, v; param_t p: 4n doubles each,
// one array per segment) and ib = [id, type] x n
// ---------------------------------------------------------------------------
__global__ void k_pack_state(int o, int n, const double* y_r, const double* y_v, const double* mass,
                             const double* radius, const double* density, const double* cd, const int* id,
                             const int* btype, StateSegs dst, int* ib)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        ib[2 * k] = id[o + k];
        ib[2 * k + 1] = btype[o + k];
    }
    if (k >= 12LL * n) return;
    const int seg = (int)(k / (4LL * n));
    double* out = dst.seg[seg];
    if (!out) return;
    const int w = (int)(k - seg * 4LL * n);
    const int i = o + w / 4, c = w % 4;
    double v;
    if (seg == 0) v = c < 3 ? y_r[3 * i + c] : 0.0;
    else if (seg == 1) v = c < 3 ? y_v[3 * i + c] : 0.0;
    else v = c == 0 ? mass[i] : (c == 1 ? radius[i] : (c == 2 ? density[i] : cd[i]));
    out[w] = v;
}

// Inverse of k_pack_state for the parts named in `what` (1 r, 2 v, 4 p, 8 id).
// New positions also go to the FP32 copies of stage 0 (x, y, z; the .w words
// follow mass and radius and are set by k_prep).
__global__ void k_unpack_state(int o, int n, int what, StateSegs src, const int* ib, double* y_r, double* y_v,
                               double* mass, double* radius, double* density, double* cd, int* id, float4* hi0,
                               float4* lo0)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && (what & 8)) id[o + k] = ib[2 * k];
    if (k >= 12LL * n) return;
    const int seg = (int)(k / (4LL * n));
    if (!(what & (1 << seg)) || !src.seg[seg]) return;
    const int w = (int)(k - seg * 4LL * n);
    const int i = o + w / 4, c = w % 4;
    const double v = src.seg[seg][w];
    if (seg == 0) {
        if (c < 3) y_r[3 * i + c] = v;
        write_pos_c(hi0, lo0, i, c, v);
    }
    else if (seg == 1) { if (c < 3) y_v[3 * i + c] = v; }
    else if (c == 0) mass[i] = v;
    else if (c == 1) radius[i] = v;
    else if (c == 2) density[i] = v;
    else cd[i] = v;
}

// Sets the try quota of every system (red_step: 1 accepted step, then -1 = none).
__global__ void k_set_quota(DevSys* sys, int n_sys, int q)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n_sys) sys[s].quota = q;
}

// Empties the partial-record slots of the stage kernel's chunk reduction.
__global__ void k_fill_records(unsigned long long* recs, size_t n)
{
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        recs[k] = kRecEmpty;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_set_quota(DevSys* sys, int n_sys, int q, cudaStream_t s)
{
    if (n_sys > 0) k_set_quota<<<(unsigned)((n_sys + 127) / 128), 128, 0, s>>>(sys, n_sys, q);
}

void fill_records_empty(void* recs, size_t n, cudaStream_t s)
{
    if (n == 0) return;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4 * 152);
    k_fill_records<<<blocks, 256, 0, s>>>(static_cast<unsigned long long*>(recs), n);
}

void set_tableau(const Tableau& tb, cudaStream_t s)
{
    cudaMemcpyToSymbolAsync(c_tb, &tb, sizeof(Tableau), 0, cudaMemcpyHostToDevice, s);
    set_tableau_mixed(tb, s);
    set_tableau_fp32(tb, s);
    set_tableau_fp64(tb, s);
    set_tableau_exact(tb, s);
}

// Variant of k_stage: the shape of the combination its epilogue forms.
int stage_variant(const StageParams& P)
{
    if (P.standalone) return 0;
    if (P.err_after) return P.scheme == SCHEME_RKF78 ? 15 : 16;
    if (P.next < 0) return 0;
    if (P.scheme == SCHEME_RKF78) return P.next;   // next = stage + 1 in [1, 12]
    return P.ynp1_to_out ? 14 : 13;
}

void launch_stage(const StageParams& P, int n_items, int mode, cudaStream_t s)
{
    if (n_items <= 0) return;
    const int v = stage_variant(P);
    switch (mode) {
    case MODE_MIXED: launch_stage_mixed(P, n_items, v, s); break;
    case MODE_FP64: launch_stage_fp64(P, n_items, v, s); break;
    case MODE_FP64_EXACT: launch_stage_exact(P, n_items, v, s); break;
    default: launch_stage_fp32(P, n_items, v, s); break;
    }
}

int stage_active_clusters(int mode)
{
    if (mode == MODE_MIXED) return active_clusters_mixed();
    if (mode == MODE_FP32) return active_clusters_fp32();
    return 0;
}

void launch_prep(const Segment* segs, int n_segs, const SysInfo* sinfo, const DevSys* sys, const double* y_r,
                 const double* mass, const double* radius, const int* id, float4* hi, float4* lo, float4* hi1,
                 float4* lo1, int all, cudaStream_t s)
{
    if (n_segs > 0) k_prep<<<n_segs, kSegment, 0, s>>>(segs, sinfo, sys, y_r, mass, radius, id, hi, lo, hi1, lo1, all);
}

void launch_control(const ControlParams& P, cudaStream_t s)
{
    launch_k(k_control, (unsigned)((P.n_sys + 127) / 128), 128u, s, P);
}

void launch_finish(const FinishParams& P, int n_segs, cudaStream_t s)
{
    if (n_segs <= 0) return;
    if (P.stage_exact) launch_k(k_finish<true>, (unsigned)n_segs, 3u * kFinishBodies, s, P);
    else launch_k(k_finish<false>, (unsigned)n_segs, 3u * kFinishBodies, s, P);
}

// The explicit collision check (red_check_for_collision) on the current state.
void launch_collision(const CollParams& P, int n_items, int n_segs, bool use_grid, size_t table_size,
                      cudaStream_t s)
{
    if (n_items > 0) launch_k(k_collision, (unsigned)n_items, (unsigned)kTile, s, P);
    if (use_grid && n_segs > 0) {
        cudaMemsetAsync(P.head, 0xff, table_size * sizeof(int), s);
        launch_k(k_grid_insert, (unsigned)n_segs, (unsigned)kSegment, s, P);
        launch_k(k_grid_query, (unsigned)n_segs, (unsigned)kSegment, s, P);
    }
}

// The collision check after a try (k_collide): the bodies are in the hash
// already (k_finish), the pair tiles and the queries run in one launch.
void launch_collide(const CollParams& P, int n_items, int n_segs, bool use_grid, cudaStream_t s)
{
    const int nq = use_grid ? 2 * n_segs : 0;
    if (n_items + nq > 0) launch_k(k_collide, (unsigned)(n_items + nq), (unsigned)kTile, s, P, n_items);
}

void launch_pack_state(int o, int n, const double* y_r, const double* y_v, const double* mass, const double* radius,
                       const double* density, const double* cd, const int* id, const int* btype, StateSegs dst,
                       int* ib, cudaStream_t s)
{
    if (n <= 0) return;
    const long long tot = 12LL * n;
    k_pack_state<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(o, n, y_r, y_v, mass, radius, density, cd, id, btype,
                                                               dst, ib);
}

void launch_unpack_state(int o, int n, int what, StateSegs src, const int* ib, double* y_r, double* y_v,
                         double* mass, double* radius, double* density, double* cd, int* id, float4* hi0,
                         float4* lo0, cudaStream_t s)
{
    if (n <= 0) return;
    const long long tot = 12LL * n;
    k_unpack_state<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(o, n, what, src, ib, y_r, y_v, mass, radius,
                                                                 density, cd, id, hi0, lo0);
}

void launch_ejhc(const EjhcParams& P, int n_segs, cudaStream_t s)
{
    if (n_segs > 0) launch_k(k_ejhc, (unsigned)n_segs, (unsigned)kSegment, s, P);
}

void launch_potential(const Segment* segs, int n_segs, const SysInfo* sinfo, const double* y_r,
                      const double* mass, const int* id, int sys_filter, int interacting, double* u,
                      cudaStream_t s)
{
    if (n_segs > 0) k_potential<<<n_segs, kSegment, 0, s>>>(segs, sinfo, y_r, mass, id, sys_filter, interacting, u);
}

}  // namespace redgb
