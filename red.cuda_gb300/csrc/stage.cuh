// stage.cuh -- the Runge-Kutta stage kernel of libredgb.
//
// One launch evaluates stage s of every system: the gravity of each sink
// against its chunk of sources (shared-memory tiles), the reduction of the
// source chunks of a sink tile (two-level, by the CTAs that finish last), and
// an element-wise FP64 epilogue: central-star term, gas drag, K storage, the
// combination that gives the positions of the next stage (or the error norm
// after the last stage).
//
// The kernel is instantiated per arithmetic mode and per "variant" V, the
// shape of the next-stage combination:
//   V = 0        no combination (standalone evaluation, last stage of a try)
//   V = 1 .. 12  RKF7(8) stage V: y + dt * sum_q a_{V,q} K_q
//   V = 13       RK4 stage s + 1: y + (a_{s+1} dt) K_s
//   V = 14       RK4 y_{n+1} as the input of the adaptive stage 4
//   V = 15       RKF7(8) error norm after stage 12
//   V = 16       RK4 error norm after stage 4
// With V known at compile time the operands of the combination are loaded
// into registers at the start of the kernel, overlapping the gravity loop.
// Each mode lives in its own translation unit (stage_*.cu).
#pragma once
#include "common.cuh"

namespace redgb {

constexpr int kStarBatch = 4;   // star factors formed per pass of the epilogue
constexpr int kBatch = 16;      // partial records loaded per batch by the reducing CTA

struct SmemStage {
    union {
        struct { float4 hi[kTile]; float4 lo[kTile]; } f;
        struct { D4 d[kTile]; int id[kTile]; } d;
    } src;
    double acc[3 * kTile];          // per (sink, component) gravity sums
    double sc[kTile][3];            // drag factor and gas velocity per sink
    double fs[kTile][kStarBatch];   // star factors per sink
    int flag;
};

template <int MODE>
__device__ __forceinline__ void load_sources(SmemStage& sm, const StageParams& P, int j0, int nj)
{
    const int t = threadIdx.x;
    if (t < nj) {
        const int j = j0 + t;
        if (MODE == MODE_MIXED || MODE == MODE_FP32) {
            sm.src.f.hi[t] = P.pos_hi_in[j];
            if (MODE == MODE_MIXED) sm.src.f.lo[t] = P.pos_lo_in[j];
        } else {
            const int idj = P.id[j];
            const double m = P.mass[j];
            sm.src.d.d[t] = D4{P.r_in[3 * j], P.r_in[3 * j + 1], P.r_in[3 * j + 2],
                                (MODE == MODE_FP64 && idj < 0) ? 0.0 : m};
            sm.src.d.id[t] = idj;
        }
    }
}

// Sum over the `lanes` threads of a sink (aligned groups inside a warp).
__device__ __forceinline__ double group_sum(double v, int lanes)
{
    for (int o = 1; o < lanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum of the partial records [c0, c1) of one element (3 doubles per sink record,
// element t of the tile at offset t), in order, loads issued in one batch per
// kBatch records.
__device__ __forceinline__ double sum_records(const double* base, long long stride, int c0, int c1)
{
    double a = 0.0;
    for (int b = c0; b < c1; b += kBatch) {
        double pv[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; u++) pv[u] = (b + u < c1) ? __ldcg(base + (b + u) * stride) : 0.0;
#pragma unroll
        for (int u = 0; u < kBatch; u++) a += pv[u];
    }
    return a;
}

// ---------------------------------------------------------------------------
// k_stage
//
// Thread layout of the gravity loop: each sink is served by `lanes`
// consecutive threads of one warp (lanes in {4, 8, 16, 32}); the lanes split
// the sources of every shared-memory tile and combine their partial sums with
// a butterfly of shuffles (every lane ends with the same bits).  The epilogue
// is element-wise: thread t < 3 nsink owns component x = 3 sink0 + t, which is
// contiguous in HBM, so every FP64 instruction runs in full warps.
//
// Memory round trips on the critical path: the work item; then, in one batch,
// the system state, the first source tile, the sink's operands for the
// epilogue and the star / drag inputs; then one trip per further source tile
// (prefetched into registers while the previous tile is in use); then, for a
// chunked tile, the partial records of the reduction.
// ---------------------------------------------------------------------------
template <int MODE, bool EXACT, int V>
__global__ void __launch_bounds__(kTile) k_stage(const StageParams P)
{
    constexpr bool kF32 = (MODE == MODE_MIXED || MODE == MODE_FP32);
    constexpr bool kRkf = (V >= 1 && V <= 12);
    __shared__ SmemStage sm;
    const GravItem it = P.items[blockIdx.x];
    const int s = P.stage;
    DevSys* S = P.sys + it.sys;
    double tsys = 0.0, dt = 0.0;
    if (!P.standalone) {
        const int act = S->active, hal = S->halted, quo = S->quota;
        tsys = S->t;
        dt = S->dt_try;
        if (!(act && !hal && quo != 0)) return;   // uniform over the CTA
    }

    const int L = it.lanes;
    const int t = threadIdx.x;
    const int k = t / L;                          // sink slot of the gravity loop
    const int lane = t % L;
    const bool has = k < it.nsink;
    const int i = it.sink0 + (has ? k : 0);       // inactive slots shadow sink 0 (results unused)
    const int gbase = (t & 31) & ~(L - 1);        // first lane of the sink's group in the warp

    // ---- batch of independent loads ----
    // first source tile, in registers until stored to shared memory
    float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th;
    D4 td{0.0, 0.0, 0.0, 0.0};
    int tid = 0;
    auto fetch = [&](int j0) {
        const int nj = min(kTile, it.src1 - j0);
        if (t < nj) {
            const int j = j0 + t;
            if (kF32) {
                th = P.pos_hi_in[j];
                if (MODE == MODE_MIXED) tl = P.pos_lo_in[j];
            } else {
                tid = P.id[j];
                const double m = P.mass[j];
                td = D4{P.r_in[3 * j], P.r_in[3 * j + 1], P.r_in[3 * j + 2], (MODE == MODE_FP64 && tid < 0) ? 0.0 : m};
            }
        }
    };
    auto stash = [&]() {
        if (kF32) {
            sm.src.f.hi[t] = th;
            if (MODE == MODE_MIXED) sm.src.f.lo[t] = tl;
        } else {
            sm.src.d.d[t] = td;
            sm.src.d.id[t] = tid;
        }
    };
    if (it.src0 < it.src1) fetch(it.src0);

    // the sink of the gravity loop
    float4 H = make_float4(0.f, 0.f, 0.f, 0.f), Lo = H;
    double xi = 0.0, yi = 0.0, zi = 0.0;
    if (kF32) {
        H = P.pos_hi_in[i];
        if (MODE == MODE_MIXED) Lo = P.pos_lo_in[i];
    } else {
        xi = P.r_in[3 * i];
        yi = P.r_in[3 * i + 1];
        zi = P.r_in[3 * i + 2];
    }

    // the element of the epilogue
    const int nel = 3 * it.nsink;
    const bool elem = t < nel;
    const int ke = elem ? t / 3 : 0;
    const int ce = elem ? t % 3 : 0;
    const int ie = it.sink0 + ke;
    const int x = 3 * ie + ce;
    const int idi = P.id[ie];
    const double rc = P.r_in[x];
    const bool drag_on = P.gas.enabled && it.cls == CLS_NSI;
    const bool need_vs = drag_on || (!P.standalone && V != 0);
    const double vs = need_vs ? P.Kr[s][x] : 0.0;    // stage velocity of the element
    double yr = 0.0, yv = 0.0;
    double kr[9], kv[9];
#pragma unroll
    for (int q = 0; q < 9; q++) kr[q] = kv[q] = 0.0;
    if constexpr (kRkf) {
        yr = P.y_r[x];
        yv = P.y_v[x];
#pragma unroll
        for (int q = 0; q < kNnz[V]; q++) {
            kr[q] = P.Kr[kSrc[V][q]][x];
            if (kSrc[V][q] != V - 1) kv[q] = P.Kv[kSrc[V][q]][x];
        }
    } else if constexpr (V == 13) {
        yr = P.y_r[x];
        yv = P.y_v[x];
    } else if constexpr (V == 14) {
        yr = P.y_r[x];
        yv = P.y_v[x];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            kr[q] = P.Kr[q][x];
            kv[q] = P.Kv[q][x];
        }
    } else if constexpr (V == 15) {
        kr[0] = P.Kr[0][x]; kr[1] = P.Kr[10][x]; kr[2] = P.Kr[11][x];
        kv[0] = P.Kv[0][x]; kv[1] = P.Kv[10][x]; kv[2] = P.Kv[11][x];
    } else if constexpr (V == 16) {
        kr[0] = P.Kr[3][x];
        kv[0] = P.Kv[3][x];
    }
    double m_i = 0.0, rad_i = 0.0;
    if (V != 0 && V <= 14 && ce == 0) {
        m_i = P.mass[ie];
        rad_i = P.radius[ie];
    }

    // ---- drag factor and star factors: scalars per sink, thread t < nsink ----
    const bool star_term = kF32 && it.nstar > 0;
    double decr = 0.0;
    if (drag_on) {
        const double ts = P.standalone ? P.t_standalone
                                       : tsys + (P.scheme == SCHEME_RKF78 ? c_tb.c[s] : c_tb.c4[s]) * dt;
        decr = gas_reduction_factor(P.gas, ts);
    }
    const bool drag_act = drag_on && !(1.0e-6 > decr);
    const bool sink_thread = t < it.nsink;
    const int ib = it.sink0 + (sink_thread ? t : 0);
    double bx = 0.0, by = 0.0, bz = 0.0;
    if (star_term || drag_act) {
        bx = P.r_in[3 * ib];
        by = P.r_in[3 * ib + 1];
        bz = P.r_in[3 * ib + 2];
    }
    if (drag_act && sink_thread) {
        double f, gx, gy;
        drag_factor(P.gas, decr, P.mass[it.soff], bx, by, bz, P.Kr[s][3 * ib], P.Kr[s][3 * ib + 1],
                    P.Kr[s][3 * ib + 2], P.cd[ib], P.radius[ib], P.density[ib], f, gx, gy);
        sm.sc[t][0] = f;
        sm.sc[t][1] = gx;
        sm.sc[t][2] = gy;
    }
    // central-star term in FP64: m_j d / |d|^3 with |d|^-1 from rsqrt, the factor
    // per (sink, star) formed by one thread per sink
    auto star_factors = [&](int b0, int nst) {
        if (sink_thread) {
#pragma unroll
            for (int q = 0; q < kStarBatch; q++) {
                if (q < nst) {
                    const int j = it.soff + b0 + q;
                    const double dx = P.r_in[3 * j] - bx, dy = P.r_in[3 * j + 1] - by, dz = P.r_in[3 * j + 2] - bz;
                    const double w = fma(dz, dz, fma(dy, dy, dx * dx));
                    const double ri = rsqrt(w);
                    sm.fs[t][q] = (j == ib || P.id[j] < 0) ? 0.0 : P.mass[j] * (ri * ri) * ri;
                }
            }
        }
    };
    double sp[kStarBatch];
    const int nst0 = star_term ? min(kStarBatch, it.nstar) : 0;
#pragma unroll
    for (int q = 0; q < kStarBatch; q++) sp[q] = q < nst0 ? P.r_in[3 * (it.soff + q) + ce] : 0.0;
    if (star_term) star_factors(0, nst0);
    if (it.src0 < it.src1) stash();
    __syncthreads();
    double sc_sum = 0.0;
    if (star_term) {
#pragma unroll
        for (int q = 0; q < kStarBatch; q++)
            if (q < nst0) sc_sum = fma(sm.fs[ke][q], sp[q] - rc, sc_sum);
        for (int b0 = kStarBatch; b0 < it.nstar; b0 += kStarBatch) {   // more than kStarBatch stars
            const int nst = min(kStarBatch, it.nstar - b0);
            __syncthreads();
            star_factors(b0, nst);
            __syncthreads();
            for (int q = 0; q < nst; q++) sc_sum = fma(sm.fs[ke][q], P.r_in[3 * (it.soff + b0 + q) + ce] - rc, sc_sum);
        }
    }

    // ---- gravity of the chunk's sources; the next tile is fetched while the
    // current one is in use ----
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (kF32) {
        float sxh = 0.f, sxl = 0.f, syh = 0.f, syl = 0.f, szh = 0.f, szl = 0.f;
        for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
            const int nj = min(kTile, it.src1 - j0);
            const bool more = j0 + kTile < it.src1;
            if (more) fetch(j0 + kTile);
            if (has) {
                float tx = 0.f, ty = 0.f, tz = 0.f;
#pragma unroll 4
                for (int jj = lane; jj < nj; jj += L) {
                    const float4 h = sm.src.f.hi[jj];
                    float dx, dy, dz;
                    if (MODE == MODE_MIXED) {
                        const float4 l = sm.src.f.lo[jj];
                        dx = (h.x - H.x) + (l.x - Lo.x);
                        dy = (h.y - H.y) + (l.y - Lo.y);
                        dz = (h.z - H.z) + (l.z - Lo.z);
                    } else {
                        dx = h.x - H.x;
                        dy = h.y - H.y;
                        dz = h.z - H.z;
                    }
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, kEps2)));
                    const float ri = rsqrtf(r2);
                    const float ri2 = ri * ri;
                    const float sc = h.w * ri * ri2;
                    tx = fmaf(sc, dx, tx);
                    ty = fmaf(sc, dy, ty);
                    tz = fmaf(sc, dz, tz);
                }
                ds_add(sxh, sxl, tx);
                ds_add(syh, syl, ty);
                ds_add(szh, szl, tz);
            }
            if (more) {
                __syncthreads();
                stash();
                __syncthreads();
            }
        }
        // lanes -> one double-single sum (TwoSum in FP32, a fixed butterfly), then lane c
        // converts component c to FP64
        for (int o = 1; o < L; o <<= 1) {
            ds_merge(sxh, sxl, __shfl_xor_sync(0xffffffffu, sxh, o), __shfl_xor_sync(0xffffffffu, sxl, o));
            ds_merge(syh, syl, __shfl_xor_sync(0xffffffffu, syh, o), __shfl_xor_sync(0xffffffffu, syl, o));
            ds_merge(szh, szl, __shfl_xor_sync(0xffffffffu, szh, o), __shfl_xor_sync(0xffffffffu, szl, o));
        }
        const int cl = lane < 3 ? lane : 0;
        const float hh = cl == 0 ? sxh : (cl == 1 ? syh : szh);
        const float ll = cl == 0 ? sxl : (cl == 1 ? syl : szl);
        const double v = lane < 3 ? (double)hh + (double)ll : 0.0;
        ax = ay = az = v;   // lane c holds component c in all three
    } else {
        for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
            const int nj = min(kTile, it.src1 - j0);
            const bool more = j0 + kTile < it.src1;
            if (more) fetch(j0 + kTile);
            if (has) {
                if (MODE == MODE_FP64_EXACT) {
                    // calc_grav_accel_naive, pp_disk.cu:389-413, bit for bit: lane 0 alone,
                    // sources in index order
                    if (lane == 0) {
                        for (int jj = 0; jj < nj; jj++) {
                            const D4 q = sm.src.d.d[jj];
                            if (j0 + jj == i || 0 > sm.src.d.id[jj]) continue;
                            const double dx = __dsub_rn(q.x, xi), dy = __dsub_rn(q.y, yi), dz = __dsub_rn(q.z, zi);
                            double w = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                            const double d = __dsqrt_rn(w);
                            w = __ddiv_rn(q.w, __dmul_rn(d, w));
                            ax = __dadd_rn(ax, __dmul_rn(w, dx));
                            ay = __dadd_rn(ay, __dmul_rn(w, dy));
                            az = __dadd_rn(az, __dmul_rn(w, dz));
                        }
                    }
                } else {
                    for (int jj = lane; jj < nj; jj += L) {
                        const D4 q = sm.src.d.d[jj];
                        const double dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
                        const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
                        double ri = rsqrt(r2);
                        ri = r2 > 0.0 ? ri : 0.0;
                        const double sc = q.w * ri * ri * ri;
                        ax = fma(sc, dx, ax);
                        ay = fma(sc, dy, ay);
                        az = fma(sc, dz, az);
                    }
                }
            }
            if (more) {
                __syncthreads();
                stash();
                __syncthreads();
            }
        }
        if (MODE == MODE_FP64_EXACT) {
            ax = __shfl_sync(0xffffffffu, ax, gbase);
            ay = __shfl_sync(0xffffffffu, ay, gbase);
            az = __shfl_sync(0xffffffffu, az, gbase);
        } else {
            ax = group_sum(ax, L);
            ay = group_sum(ay, L);
            az = group_sum(az, L);
        }
    }
    // lane c of each sink holds component c
    const double mine = lane == 0 ? ax : (lane == 1 ? ay : az);

    // ---- source chunks of one sink tile -> the CTA that finishes last sums them,
    // every thread of it on a contiguous range of chunks, in a fixed order ----
    double a = 0.0;
    if (it.nchunk > 1) {
        if (has && lane < 3) {
            double* p = P.partial + 3 * ((long long)it.part_off + (long long)it.chunk * it.nsink) + 3 * k + lane;
            *p = mine;
        }
        __threadfence();
        __syncthreads();
        if (t == 0) {
            const unsigned prev = atomicAdd(&P.tile_cnt[it.tile], 1u);
            sm.flag = (prev == (unsigned)(it.nchunk - 1));
        }
        __syncthreads();
        if (!sm.flag) return;   // uniform
        __threadfence();
        const int nsplit = kTile / nel;
        const int sp_i = t / nel;
        const int e = t - sp_i * nel;
        double part = 0.0;
        if (sp_i < nsplit) {
            const int c0 = (int)((long long)sp_i * it.nchunk / nsplit);
            const int c1 = (int)((long long)(sp_i + 1) * it.nchunk / nsplit);
            part = sum_records(P.partial + 3 * (long long)it.part_off + e, 3LL * it.nsink, c0, c1);
        }
        sm.acc[t] = part;
        __syncthreads();
        if (elem)
            for (int q = 0; q < nsplit; q++) a += sm.acc[q * nel + t];
        if (t == 0) P.tile_cnt[it.tile] = 0u;
    } else {
        if (has && lane < 3) sm.acc[3 * k + lane] = mine;
        __syncthreads();
        if (elem) a = sm.acc[t];
    }
    if (!elem) return;

    // ---- element-wise FP64 epilogue ----
    if (star_term) a = sc_sum + a;
    if (!(idi > 0)) a = 0.0;   // calc_grav_accel_naive zeroes inactive sinks (pp_disk.cu:386-388)
    if (drag_act) {
        const double g = ce == 0 ? sm.sc[ke][1] : (ce == 1 ? sm.sc[ke][2] : 0.0);
        a += sm.sc[ke][0] * (g - vs);
    }
    P.Kv[s][x] = a;

    if constexpr (V >= 1 && V <= 14) {
        double orr, ovv;
        if constexpr (kRkf) {
            // ytemp of stage V: y + dt * sum_q a_{V,q} K_q, terms in red's order
            // (rk8_kernel::calc_ytemp_for_f1..f12, int_rungekutta8.cu:80-246)
            constexpr int off = 1 + V * (V - 1) / 2;
            if (kSrc[V][0] == V - 1) kv[0] = a;
            double ar = mul<EXACT>(c_tb.a[off + kSrc[V][0]], kr[0]);
            double av = mul<EXACT>(c_tb.a[off + kSrc[V][0]], kv[0]);
#pragma unroll
            for (int q = 1; q < kNnz[V]; q++) {
                const double aq = c_tb.a[off + kSrc[V][q]];
                const double kvq = (kSrc[V][q] == V - 1) ? a : kv[q];
                ar = madd<EXACT>(ar, aq, kr[q]);
                av = madd<EXACT>(av, aq, kvq);
            }
            orr = madd<EXACT>(yr, dt, ar);
            ovv = madd<EXACT>(yv, dt, av);
        } else if constexpr (V == 13) {
            // rk4_kernel::sum_vector, int_rungekutta4.cu:36-47: y + (a dt) K_s
            const double bf = mul<EXACT>(c_tb.a4[s + 1], dt);
            orr = madd<EXACT>(yr, bf, vs);
            ovv = madd<EXACT>(yv, bf, a);
        } else {
            // RK4 y_{n+1} as the positions of the adaptive stage 4
            const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
            orr = rk4_ynp1<EXACT>(yr, b0, b1, kr[0], kr[1], kr[2], vs);
            ovv = rk4_ynp1<EXACT>(yv, b0, b1, kv[0], kv[1], kv[2], a);
        }
        P.r_out[x] = orr;
        P.Kr[P.next][x] = ovv;
        write_pos_c(P.pos_hi_out, P.pos_lo_out, ie, ce, orr);
        if (ce == 0) {
            reinterpret_cast<float*>(P.pos_hi_out + ie)[3] = __double2float_rn(idi >= 0 ? m_i : 0.0);
            reinterpret_cast<float*>(P.pos_lo_out + ie)[3] = __double2float_rn(rad_i);
        }
    } else if constexpr (V == 15 || V == 16) {
        double e = 0.0;
        if (ie - it.soff < it.nerr) {
            double er, ev;
            if constexpr (V == 15) {
                // rk8_kernel::calc_error, int_rungekutta8.cu:248-260
                er = fabs(sub<EXACT>(sub<EXACT>(add<EXACT>(kr[0], kr[1]), kr[2]), vs));
                ev = fabs(sub<EXACT>(sub<EXACT>(add<EXACT>(kv[0], kv[1]), kv[2]), a));
            } else {
                // rk4_kernel::calc_error, int_rungekutta4.cu:62-73
                er = fabs(kr[0] - vs);
                ev = fabs(kv[0] - a);
            }
            e = fmax(er, ev);
            if (er != er || ev != ev) e = __longlong_as_double(0x7ff8000000000000ll);
        }
        // max over the active lanes of the warp, one atomic per warp (non-negative
        // doubles order as their bits; high words first, then low words)
        const unsigned long long b = (unsigned long long)__double_as_longlong(e);
        const unsigned m = __activemask();
        const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
        const unsigned mh = __reduce_max_sync(m, hi);
        const unsigned m2 = __ballot_sync(m, hi == mh);
        if (hi == mh) {
            const unsigned ml = __reduce_max_sync(m2, lo);
            const unsigned long long w = ((unsigned long long)mh << 32) | ml;
            if ((t & 31) == __ffs(m2) - 1 && w) atomicMax(&S->err_bits, w);
        }
    }
}

// Launches the variant of k_stage that P asks for (stage_variant).
template <int MODE, bool EXACT>
void launch_stage_variant(const StageParams& P, int n, int v, cudaStream_t s)
{
    switch (v) {
    case 1: k_stage<MODE, EXACT, 1><<<n, kTile, 0, s>>>(P); break;
    case 2: k_stage<MODE, EXACT, 2><<<n, kTile, 0, s>>>(P); break;
    case 3: k_stage<MODE, EXACT, 3><<<n, kTile, 0, s>>>(P); break;
    case 4: k_stage<MODE, EXACT, 4><<<n, kTile, 0, s>>>(P); break;
    case 5: k_stage<MODE, EXACT, 5><<<n, kTile, 0, s>>>(P); break;
    case 6: k_stage<MODE, EXACT, 6><<<n, kTile, 0, s>>>(P); break;
    case 7: k_stage<MODE, EXACT, 7><<<n, kTile, 0, s>>>(P); break;
    case 8: k_stage<MODE, EXACT, 8><<<n, kTile, 0, s>>>(P); break;
    case 9: k_stage<MODE, EXACT, 9><<<n, kTile, 0, s>>>(P); break;
    case 10: k_stage<MODE, EXACT, 10><<<n, kTile, 0, s>>>(P); break;
    case 11: k_stage<MODE, EXACT, 11><<<n, kTile, 0, s>>>(P); break;
    case 12: k_stage<MODE, EXACT, 12><<<n, kTile, 0, s>>>(P); break;
    case 13: k_stage<MODE, EXACT, 13><<<n, kTile, 0, s>>>(P); break;
    case 14: k_stage<MODE, EXACT, 14><<<n, kTile, 0, s>>>(P); break;
    case 15: k_stage<MODE, EXACT, 15><<<n, kTile, 0, s>>>(P); break;
    case 16: k_stage<MODE, EXACT, 16><<<n, kTile, 0, s>>>(P); break;
    default: k_stage<MODE, EXACT, 0><<<n, kTile, 0, s>>>(P); break;
    }
}

}  // namespace redgb
