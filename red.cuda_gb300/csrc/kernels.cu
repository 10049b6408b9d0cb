// kernels.cu -- the sm_103a kernels of libredgb.
//
//   k_stage     one Runge-Kutta stage: gravity of every sink against its
//               source chunk (shared-memory tiles), cross-CTA reduction of
//               source chunks, then a fused per-body epilogue: central-star
//               term, gas drag, K storage, the next stage's combination
//               y + dt * sum a_rs K_s (or the error norm on the last stage)
//   k_prep      positions of stage 0 from y (FP32 double-single copies)
//   k_control   per-system error -> accept / reject -> new step size
//   k_finish    y_{n+1} for accepted systems, positions of the next stage 0
//   k_collision pairwise overlap test, FP32 prefilter + red's FP64 test
//   k_ejhc      ejection / hit-centrum test
//   k_potential per-body potential sums for the integrals
#include <cfloat>
#include <cstdio>

#include "redgb_dev.cuh"

namespace redgb {

__constant__ Tableau c_tb;

// Squared softening added to r^2 in the FP32 loops only, so that the self pair
// (r = 0 exactly) contributes 0 * finite instead of 0 * inf.  For any real pair
// (r >= 1e-6 AU) it changes the force by < 1e-11 relative, far below FP32
// rounding.  The FP64 paths use no softening, as red.
constexpr float kEps2 = 1.0e-24f;

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// Folds the FP32 tile sum t into the double-single accumulator (hi, lo).
__device__ __forceinline__ void ds_add(float& hi, float& lo, float t)
{
    float s, e;
    two_sum(hi, t, s, e);
    hi = s;
    lo += e;
}

// (ah, al) += (bh, bl) for double-single values (TwoSum on the high words,
// low words added; Dekker 1971 / Knuth TwoSum).
__device__ __forceinline__ void ds_merge(float& ah, float& al, float bh, float bl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    ah = s;
    al = al + bl + e;
}

__device__ __forceinline__ void split_ds(double x, float& h, float& l)
{
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
}

__device__ __forceinline__ void write_pos(float4* hi, float4* lo, int i, double x, double y, double z,
                                          double m_eff, double radius)
{
    float4 H, L;
    split_ds(x, H.x, L.x);
    split_ds(y, H.y, L.y);
    split_ds(z, H.z, L.z);
    H.w = __double2float_rn(m_eff);
    L.w = __double2float_rn(radius);
    hi[i] = H;
    lo[i] = L;
}

// Multiply / add that either follows red's -fmad=false arithmetic (EXACT)
// or lets the compiler fuse.
template <bool EXACT> __device__ __forceinline__ double mul(double a, double b)
{
    return EXACT ? __dmul_rn(a, b) : a * b;
}
template <bool EXACT> __device__ __forceinline__ double add(double a, double b)
{
    return EXACT ? __dadd_rn(a, b) : a + b;
}
template <bool EXACT> __device__ __forceinline__ double sub(double a, double b)
{
    return EXACT ? __dsub_rn(a, b) : a - b;
}
// a + b * c
template <bool EXACT> __device__ __forceinline__ double madd(double a, double b, double c)
{
    return EXACT ? __dadd_rn(a, __dmul_rn(b, c)) : fma(b, c, a);
}

// ---------------------------------------------------------------------------
// analytic gas disk, pp_disk.cu:59-155 and 485-521
// ---------------------------------------------------------------------------
__device__ double gas_reduction_factor(const GasDev& g, double t)
{
    switch (g.gas_decrease) {
    case 0: return 1.0;
    case 1:
        if (t <= g.t0) return 1.0;
        else if (g.t0 < t && t <= g.t1 && g.t0 != g.t1) return 1.0 - (t - g.t0) / (g.t1 - g.t0);
        else return 0.0;
    case 2: return exp(-(t - g.t0) / g.e_folding_time);
    default: return 1.0;
    }
}

// Drag factor f and gas velocity (gx, gy, 0) at (r, v): the acceleration is
// f (v_gas - v) (calc_drag_accel_NSI, pp_disk.cu:485-521).
__device__ void drag_factor(const GasDev& g, double decr, double m_star, double rx, double ry, double rz, double vx,
                            double vy, double vz, double cd, double radius, double density, double& f, double& gx,
                            double& gy)
{
    // gas velocity: circular velocity scaled by sqrt(1 - 2 eta r^p) (pp_disk.cu:107-155)
    const double r = sqrt(rx * rx + ry * ry);
    const double vc = sqrt(m_star / r);
    gx = 0.0;
    gy = 0.0;
    if (rx == 0.0 && ry == 0.0) {
    } else if (ry == 0.0) {
        gy = rx > 0.0 ? vc : -vc;
    } else if (rx == 0.0) {
        gx = ry > 0.0 ? -vc : vc;
    } else if (rx >= ry) {
        const double p = ry / rx;
        gy = rx >= 0 ? vc / sqrt(1.0 + p * p) : -vc / sqrt(1.0 + p * p);
        gx = -gy * p;
    } else {
        const double p = rx / ry;
        gx = ry >= 0 ? -vc / sqrt(1.0 + p * p) : vc / sqrt(1.0 + p * p);
        gy = -gx * p;
    }
    const double fv = sqrt(1.0 - 2.0 * g.eta[0] * pow(r, g.eta[1]));
    gx *= fv;
    gy *= fv;
    // gas density (pp_disk.cu:86-105)
    const double h = g.sch[0] * pow(r, g.sch[1]);
    const double arg = (rz / h) * (rz / h);
    double dens;
    if (0.1 < r) {
        dens = g.rho[0] * pow(r, g.rho[1]) * exp(-arg);
    } else {
        const double a = g.rho[0] * pow(0.1, g.rho[1] - 4.0);
        dens = a * (r * r) * (r * r) * exp(-arg);
    }
    const double ux = gx - vx, uy = gy - vy, uz = 0.0 - vz;
    const double un = sqrt(ux * ux + uy * uy + uz * uz);
    f = decr * (3.0 * cd * dens * un) / (8.0 * radius * density);
}

struct alignas(32) D4 {
    double x, y, z, w;
};

// Nonzero terms of each RKF7(8) stage row in the order red's stage kernels
// add them (rk8_kernel::calc_ytemp_for_f1..f12, int_rungekutta8.cu:80-246).
// Compile-time copies of Tableau::nnz / src so that the combination unrolls.
__device__ constexpr int kNnz[13] = {0, 1, 2, 2, 3, 3, 4, 4, 6, 7, 8, 6, 9};
__device__ constexpr int kSrc[13][9] = {
    {0}, {0}, {0, 1}, {0, 2}, {0, 2, 3}, {0, 3, 4}, {0, 3, 4, 5}, {0, 4, 5, 6},
    {0, 3, 4, 5, 6, 7}, {0, 3, 4, 5, 6, 7, 8}, {0, 3, 4, 5, 6, 7, 8, 9},
    {0, 5, 6, 7, 8, 9}, {0, 3, 4, 5, 6, 7, 8, 9, 11}};

// Component x (= 3 i + c) of the ytemp of RKF7(8) stage NX:
// y + dt * sum_q a_{NX,q} K_q, terms in red's order; loads issued first.
template <int NX, bool EXACT>
__device__ __forceinline__ void combine_rkf78(const StageParams& P, double dt, int x, double& out_r, double& out_v)
{
    constexpr int nnz = kNnz[NX];
    constexpr int off = 1 + NX * (NX - 1) / 2;
    double kr[nnz], kv[nnz];
#pragma unroll
    for (int q = 0; q < nnz; q++) {
        kr[q] = P.Kr[kSrc[NX][q]][x];
        kv[q] = P.Kv[kSrc[NX][q]][x];
    }
    double ar = mul<EXACT>(c_tb.a[off + kSrc[NX][0]], kr[0]);
    double av = mul<EXACT>(c_tb.a[off + kSrc[NX][0]], kv[0]);
#pragma unroll
    for (int q = 1; q < nnz; q++) {
        const double aq = c_tb.a[off + kSrc[NX][q]];
        ar = madd<EXACT>(ar, aq, kr[q]);
        av = madd<EXACT>(av, aq, kv[q]);
    }
    out_r = madd<EXACT>(P.y_r[x], dt, ar);
    out_v = madd<EXACT>(P.y_v[x], dt, av);
}

// Component x of the ytemp of stage nx (RKF78: y + dt*sum a K in red's term
// order; RK4: y + (a dt) K, rk4_kernel::sum_vector, int_rungekutta4.cu:36-47).
template <bool EXACT>
__device__ __forceinline__ void combine(const StageParams& P, int scheme, int nx, double dt, int x, double& out_r,
                                        double& out_v)
{
    if (scheme == SCHEME_RKF78) {
        switch (nx) {
        case 1: combine_rkf78<1, EXACT>(P, dt, x, out_r, out_v); break;
        case 2: combine_rkf78<2, EXACT>(P, dt, x, out_r, out_v); break;
        case 3: combine_rkf78<3, EXACT>(P, dt, x, out_r, out_v); break;
        case 4: combine_rkf78<4, EXACT>(P, dt, x, out_r, out_v); break;
        case 5: combine_rkf78<5, EXACT>(P, dt, x, out_r, out_v); break;
        case 6: combine_rkf78<6, EXACT>(P, dt, x, out_r, out_v); break;
        case 7: combine_rkf78<7, EXACT>(P, dt, x, out_r, out_v); break;
        case 8: combine_rkf78<8, EXACT>(P, dt, x, out_r, out_v); break;
        case 9: combine_rkf78<9, EXACT>(P, dt, x, out_r, out_v); break;
        case 10: combine_rkf78<10, EXACT>(P, dt, x, out_r, out_v); break;
        case 11: combine_rkf78<11, EXACT>(P, dt, x, out_r, out_v); break;
        default: combine_rkf78<12, EXACT>(P, dt, x, out_r, out_v); break;
        }
    } else {
        const double bf = mul<EXACT>(c_tb.a4[nx], dt);
        out_r = madd<EXACT>(P.y_r[x], bf, P.Kr[nx - 1][x]);
        out_v = madd<EXACT>(P.y_v[x], bf, P.Kv[nx - 1][x]);
    }
}

// RK4 y_{n+1} = y + b0 (f1 + f4) + b1 (f2 + f3), b = (1/6, 1/3) * dt
// (rk4_kernel::calc_y_np1, int_rungekutta4.cu:49-60)
template <bool EXACT>
__device__ __forceinline__ double rk4_ynp1(double y, double b0, double b1, double k0, double k1, double k2,
                                           double k3)
{
    return add<EXACT>(madd<EXACT>(y, b0, add<EXACT>(k0, k3)), mul<EXACT>(b1, add<EXACT>(k1, k2)));
}

// RKF78 y_{n+1} = y + dt (b0 f0 + b5 f5 + b6 (f6 + f7) + b8 (f8 + f9) + b10 f10)
// (rk8_kernel::calc_y_np1, int_rungekutta8.cu:262-274)
template <bool EXACT>
__device__ __forceinline__ double rk8_ynp1(double y, double dt, const double* const* K, int idx)
{
    double acc = mul<EXACT>(c_tb.b[0], K[0][idx]);
    acc = madd<EXACT>(acc, c_tb.b[5], K[5][idx]);
    acc = madd<EXACT>(acc, c_tb.b[6], add<EXACT>(K[6][idx], K[7][idx]));
    acc = madd<EXACT>(acc, c_tb.b[8], add<EXACT>(K[8][idx], K[9][idx]));
    acc = madd<EXACT>(acc, c_tb.b[10], K[10][idx]);
    return madd<EXACT>(y, dt, acc);
}

// Writes one component of a stage position: the hi / lo words of coordinate c
// (c < 3), or the mass of the source and the radius (c == 3).
__device__ __forceinline__ void write_pos_c(float4* hi, float4* lo, int i, int c, double v)
{
    float* H = reinterpret_cast<float*>(hi + i);
    float* L = reinterpret_cast<float*>(lo + i);
    if (c < 3) {
        float h, l;
        split_ds(v, h, l);
        H[c] = h;
        L[c] = l;
    }
}

// ---------------------------------------------------------------------------
// stage kernel
//
// Thread layout: each sink is served by `lanes` consecutive threads of one
// warp (lanes in {4, 8, 16, 32}).  The lanes split the sources of every
// shared-memory tile; their partial sums are combined with a butterfly of
// shuffles (IEEE addition is commutative, so every lane ends with the same
// bits).  In the epilogue lanes 0, 1, 2 own the x, y, z components and lane 3
// computes the scalar parts (star term factor, drag factor) and broadcasts them.
// ---------------------------------------------------------------------------
constexpr int kStarBatch = 4;   // star factors formed per pass of the epilogue

struct SmemStage {
    union {
        struct { float4 hi[kTile]; float4 lo[kTile]; } f;
        struct { D4 d[kTile]; int id[kTile]; } d;
    } src;
    double acc[3 * kTile];          // per (sink, component) gravity sums
    double sc[kTile][3];            // drag factor and gas velocity per sink
    double fs[kTile][kStarBatch];   // star factors per sink
    int last;
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

template <int MODE, bool EXACT>
__global__ void __launch_bounds__(kTile) k_stage(const StageParams P)
{
    __shared__ SmemStage sm;
    const GravItem it = P.items[blockIdx.x];
    DevSys* S = P.sys + it.sys;
    if (!P.standalone && !runnable(*S)) return;   // uniform over the CTA

    const int L = it.lanes;
    const int k = threadIdx.x / L;                // sink slot
    const int lane = threadIdx.x % L;
    const bool has = k < it.nsink;
    const int i = it.sink0 + (has ? k : 0);       // inactive slots shadow sink 0 (results unused)
    const int gbase = (threadIdx.x & 31) & ~(L - 1);   // first lane of the group in the warp

    double ax = 0.0, ay = 0.0, az = 0.0;

    if (MODE == MODE_MIXED || MODE == MODE_FP32) {
        const float4 H = P.pos_hi_in[i];
        float4 Lo = make_float4(0.f, 0.f, 0.f, 0.f);
        if (MODE == MODE_MIXED) Lo = P.pos_lo_in[i];
        float sxh = 0.f, sxl = 0.f, syh = 0.f, syl = 0.f, szh = 0.f, szl = 0.f;
        for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
            const int nj = min(kTile, it.src1 - j0);
            __syncthreads();
            load_sources<MODE>(sm, P, j0, nj);
            __syncthreads();
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
        }
        // lanes -> one double-single sum (TwoSum in FP32, a fixed butterfly), then lane c
        // converts component c to FP64 (FP64 work is scarce on this part)
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
        const double xi = P.r_in[3 * i], yi = P.r_in[3 * i + 1], zi = P.r_in[3 * i + 2];
        for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
            const int nj = min(kTile, it.src1 - j0);
            __syncthreads();
            load_sources<MODE>(sm, P, j0, nj);
            __syncthreads();
            if (!has) continue;
            if (MODE == MODE_FP64_EXACT) {
                // calc_grav_accel_naive, pp_disk.cu:389-413, bit for bit: lane 0 alone,
                // sources in index order
                if (lane != 0) continue;
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
    }

    // FP64 modes: lanes of one sink -> one sum, the same bits on every lane
    if (MODE == MODE_FP64_EXACT) {
        ax = __shfl_sync(0xffffffffu, ax, gbase);
        ay = __shfl_sync(0xffffffffu, ay, gbase);
        az = __shfl_sync(0xffffffffu, az, gbase);
    } else if (MODE == MODE_FP64) {
        ax = group_sum(ax, L);
        ay = group_sum(ay, L);
        az = group_sum(az, L);
    }
    // lane c of each sink holds component c (FP32 modes: ax = ay = az = component c)
    const double mine = lane == 0 ? ax : (lane == 1 ? ay : az);

    // ---- from here on the CTA works element-wise: thread t < 3 nsink owns
    // component x = 3 sink0 + t (contiguous in HBM), so every FP64 instruction
    // runs in full warps; scalars per sink are formed by thread t < nsink ----
    const int nel = 3 * it.nsink;
    const int t = threadIdx.x;
    const bool elem = t < nel;
    const int ke = elem ? t / 3 : 0;          // sink slot of the element
    const int ce = elem ? t % 3 : 0;          // component of the element
    const int ie = it.sink0 + ke;
    const int x = 3 * ie + ce;

    double a = 0.0;
    if (it.nchunk > 1) {
        // source chunks of one sink tile -> the CTA that finishes last reduces them
        if (has && lane < 3) {
            double* p = P.partial + 3 * ((long long)it.part_off + (long long)it.chunk * it.nsink) + 3 * k + lane;
            *p = mine;
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned prev = atomicAdd(&P.tile_cnt[it.tile], 1u);
            sm.last = (prev == (unsigned)(it.nchunk - 1));
        }
        __syncthreads();
        if (!sm.last) return;   // uniform
        __threadfence();
        if (elem) {
            // chunks in order, loads issued in batches of B
            constexpr int B = 8;
            const double* base = P.partial + 3 * (long long)it.part_off + t;
            const long long stride = 3LL * it.nsink;
            for (int c0 = 0; c0 < it.nchunk; c0 += B) {
                double pv[B];
#pragma unroll
                for (int u = 0; u < B; u++) pv[u] = (c0 + u < it.nchunk) ? __ldcg(base + (c0 + u) * stride) : 0.0;
#pragma unroll
                for (int u = 0; u < B; u++) a += pv[u];
            }
        }
        if (threadIdx.x == 0) P.tile_cnt[it.tile] = 0u;
    } else {
        if (has && lane < 3) sm.acc[3 * k + lane] = mine;
        __syncthreads();
        if (elem) a = sm.acc[t];
    }

    const SysInfo si = P.sinfo[it.sys];
    const int s = P.stage;
    const double dt = S->dt_try;
    const bool drag_on = P.gas.enabled && it.cls == CLS_NSI;
    double decr = 0.0;
    if (drag_on) {
        const double ts = P.standalone ? P.t_standalone
                                       : S->t + (P.scheme == SCHEME_RKF78 ? c_tb.c[s] : c_tb.c4[s]) * dt;
        decr = gas_reduction_factor(P.gas, ts);
    }
    const bool drag_act = drag_on && !(1.0e-6 > decr);
    const bool star_term = (MODE == MODE_MIXED || MODE == MODE_FP32) && si.n_star > 0;

    // scalars, one thread per sink: drag factor and gas velocity
    if (drag_act && t < it.nsink) {
        const int i = it.sink0 + t;
        double f, gx, gy;
        drag_factor(P.gas, decr, P.mass[si.off], P.r_in[3 * i], P.r_in[3 * i + 1], P.r_in[3 * i + 2],
                    P.Kr[s][3 * i], P.Kr[s][3 * i + 1], P.Kr[s][3 * i + 2], P.cd[i], P.radius[i], P.density[i], f,
                    gx, gy);
        sm.sc[t][0] = f;
        sm.sc[t][1] = gx;
        sm.sc[t][2] = gy;
    }
    const double rc = elem ? P.r_in[x] : 0.0;
    double sc_sum = 0.0;
    if (star_term) {
        // central-star term in FP64, m_j d / |d|^3 with |d|^-1 from rsqrt; the
        // factor per (sink, star) is formed by one thread per sink
        for (int j0 = si.off; j0 < si.off + si.n_star; j0 += kStarBatch) {
            const int nst = min(kStarBatch, si.off + si.n_star - j0);
            __syncthreads();
            if (t < it.nsink) {
                const int i = it.sink0 + t;
                const double xi = P.r_in[3 * i], yi = P.r_in[3 * i + 1], zi = P.r_in[3 * i + 2];
                for (int q = 0; q < nst; q++) {
                    const int j = j0 + q;
                    const double dx = P.r_in[3 * j] - xi, dy = P.r_in[3 * j + 1] - yi, dz = P.r_in[3 * j + 2] - zi;
                    const double w = fma(dz, dz, fma(dy, dy, dx * dx));
                    const double ri = rsqrt(w);
                    sm.fs[t][q] = (j == i || P.id[j] < 0) ? 0.0 : P.mass[j] * (ri * ri) * ri;
                }
            }
            __syncthreads();
            if (elem)
                for (int q = 0; q < nst; q++) sc_sum = fma(sm.fs[ke][q], P.r_in[3 * (j0 + q) + ce] - rc, sc_sum);
        }
    } else {
        __syncthreads();
    }
    if (!elem) return;
    if (star_term) a = sc_sum + a;
    const int idi = P.id[ie];
    if (!(idi > 0)) a = 0.0;   // calc_grav_accel_naive zeroes inactive sinks (pp_disk.cu:386-388)
    if (drag_act) {
        const double g = ce == 0 ? sm.sc[ke][1] : (ce == 1 ? sm.sc[ke][2] : 0.0);
        a += sm.sc[ke][0] * (g - P.Kr[s][x]);
    }
    P.Kv[s][x] = a;
    if (P.standalone) return;

    if (P.next >= 0) {
        double orr, ovv;
        if (P.ynp1_to_out) {
            const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
            orr = rk4_ynp1<EXACT>(P.y_r[x], b0, b1, P.Kr[0][x], P.Kr[1][x], P.Kr[2][x], P.Kr[3][x]);
            ovv = rk4_ynp1<EXACT>(P.y_v[x], b0, b1, P.Kv[0][x], P.Kv[1][x], P.Kv[2][x], P.Kv[3][x]);
        } else {
            combine<EXACT>(P, P.scheme, P.next, dt, x, orr, ovv);
        }
        P.r_out[x] = orr;
        P.Kr[P.next][x] = ovv;
        write_pos_c(P.pos_hi_out, P.pos_lo_out, ie, ce, orr);
        if (ce == 0) {
            reinterpret_cast<float*>(P.pos_hi_out + ie)[3] = __double2float_rn(idi >= 0 ? P.mass[ie] : 0.0);
            reinterpret_cast<float*>(P.pos_lo_out + ie)[3] = __double2float_rn(P.radius[ie]);
        }
    }
    if (P.err_after) {
        double e = 0.0;
        if (ie - si.off < si.n_err) {
            double er, ev;
            if (P.scheme == SCHEME_RKF78) {
                // rk8_kernel::calc_error, int_rungekutta8.cu:248-260
                er = fabs(sub<EXACT>(sub<EXACT>(add<EXACT>(P.Kr[0][x], P.Kr[10][x]), P.Kr[11][x]), P.Kr[12][x]));
                ev = fabs(sub<EXACT>(sub<EXACT>(add<EXACT>(P.Kv[0][x], P.Kv[10][x]), P.Kv[11][x]), P.Kv[12][x]));
            } else {
                // rk4_kernel::calc_error, int_rungekutta4.cu:62-73
                er = fabs(P.Kr[3][x] - P.Kr[4][x]);
                ev = fabs(P.Kv[3][x] - P.Kv[4][x]);
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
            if ((threadIdx.x & 31) == __ffs(m2) - 1 && w) atomicMax(&S->err_bits, w);
        }
    }
}

// ---------------------------------------------------------------------------
// per-body kernels
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSegment) k_prep(const Segment* segs, const SysInfo* sinfo, const DevSys* sys,
                                                   const double* y_r, const double* mass, const double* radius,
                                                   const int* id, float4* hi, float4* lo, int all)
{
    const Segment sg = segs[blockIdx.x];
    if (!all && !runnable(sys[sg.sys])) return;
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1) return;
    write_pos(hi, lo, i, y_r[3 * i], y_r[3 * i + 1], y_r[3 * i + 2], id[i] >= 0 ? mass[i] : 0.0, radius[i]);
}

// One thread per system: integrator::step's accept / reject logic
// (int_rungekutta8.cu:690-716, int_rungekutta4.cu:226-248), the counters
// (integrator.cu:270-275) and run_simulation's dt_next clamp and loop bound
// (main.cu:471, 535-538).
__global__ void k_control(const ControlParams P)
{
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
        if (max_err != max_err) {
            S.status = 5;   // RED_ERR_NONFINITE
            S.halted = 1;
            S.active = 0;
            return;
        }
        if (0.0 < max_err) dt_new = dt * (0.9 * pow(P.tolerance / max_err, 1.0 / (double)P.order));
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
    S.dt_try = S.dt_next;
    if (P.length != 0.0 && fabs(S.t - S.t_start) > fabs(P.length)) S.active = 0;
}

// y_{n+1} of the accepted systems and the positions of the next stage 0.  Four
// threads per body: lanes 0..2 the x, y, z components, lane 3 the mass / radius
// words of the FP32 copies.  Segments of kFinishBodies bodies.
template <bool EXACT>
__global__ void __launch_bounds__(4 * kFinishBodies) k_finish(const FinishParams P)
{
    const Segment sg = P.segs[blockIdx.x];
    DevSys* S = P.sys + sg.sys;
    if (S->halted) return;
    const int i = sg.b0 + threadIdx.x / 4;
    const int c = threadIdx.x % 4;
    const bool acc = S->accepted;
    if (!acc && !runnable(*S)) return;
    if (i >= sg.b1) return;
    if (c == 3) {
        reinterpret_cast<float*>(P.pos_hi0 + i)[3] = __double2float_rn(P.id[i] >= 0 ? P.mass[i] : 0.0);
        reinterpret_cast<float*>(P.pos_lo0 + i)[3] = __double2float_rn(P.radius[i]);
        return;
    }
    const int x = 3 * i + c;
    double r;
    if (acc) {
        const double dt = S->dt_did;
        double v;
        if (P.scheme == SCHEME_RKF78) {
            r = rk8_ynp1<EXACT>(P.y_r[x], dt, P.Kr, x);
            v = rk8_ynp1<EXACT>(P.y_v[x], dt, P.Kv, x);
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
        if (!(isfinite(r) && isfinite(v))) S->status = 5;   // RED_ERR_NONFINITE
    } else {
        r = P.y_r[x];
    }
    write_pos_c(P.pos_hi0, P.pos_lo0, i, c, r);
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
__global__ void __launch_bounds__(kTile) k_collision(const CollParams P)
{
    __shared__ float4 shi[kTile], slo[kTile];
    const PairItem it = P.items[blockIdx.x];
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

// Spatial-hash broad phase for the small bodies.  Cell coordinates are
// clamped so that far-away bodies share border cells (tested exactly, never
// missed).
__device__ __forceinline__ int4 cell_of(double x, double y, double z, double inv_h)
{
    const double lim = 1.0e9;
    int4 c;
    c.x = (int)floor(fmin(fmax(x * inv_h, -lim), lim));
    c.y = (int)floor(fmin(fmax(y * inv_h, -lim), lim));
    c.z = (int)floor(fmin(fmax(z * inv_h, -lim), lim));
    c.w = 0;
    return c;
}

__device__ __forceinline__ int bucket_of(int cx, int cy, int cz, int mask)
{
    const unsigned h = ((unsigned)cx * 73856093u) ^ ((unsigned)cy * 19349663u) ^ ((unsigned)cz * 83492791u);
    return (int)(h & (unsigned)mask);
}

__global__ void __launch_bounds__(kSegment) k_grid_insert(const CollParams P)
{
    const Segment sg = P.segs[blockIdx.x];
    const DevSys& S = P.sys[sg.sys];
    const GridInfo g = P.grid[sg.sys];
    if (!g.enabled || !coll_runs(P, S)) return;
    const SysInfo si = P.sinfo[sg.sys];
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1 || i < si.off + si.n_SI) return;
    const int4 c = cell_of(P.y_r[3 * i], P.y_r[3 * i + 1], P.y_r[3 * i + 2], g.inv_h);
    P.cell[i] = c;
    P.next[i] = atomicExch(&P.head[g.toff + bucket_of(c.x, c.y, c.z, g.mask)], i);
}

// Half of the neighbourhood: the own cell (pairs with j > i) and the 13 cells
// of the forward half-space, so that every unordered pair of small bodies in
// neighbouring cells is seen once; the pair is tested as (min, max) like red's
// i < j loop.  The 14 bucket heads are loaded before any list is walked.
__global__ void __launch_bounds__(kSegment) k_grid_query(const CollParams P)
{
    const Segment sg = P.segs[blockIdx.x];
    DevSys* S = P.sys + sg.sys;
    const GridInfo g = P.grid[sg.sys];
    if (!g.enabled || !coll_runs(P, *S)) return;
    const SysInfo si = P.sinfo[sg.sys];
    const int i = sg.b0 + threadIdx.x;
    if (i >= sg.b1 || i < si.off + si.n_SI) return;
    const double f = P.factor * P.factor;
    const int4 c = P.cell[i];
    int head[14];
    int4 nb[14];
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
                head[q] = __ldcg(P.head + g.toff + bucket_of(nb[q].x, nb[q].y, nb[q].z, g.mask));
                q++;
            }
#pragma unroll
    for (int b = 0; b < 14; b++) {
        int j = head[b];
        while (j >= 0) {
            const int4 cj = P.cell[j];
            if (cj.x == nb[b].x && cj.y == nb[b].y && cj.z == nb[b].z && (b != 0 || j > i))
                collide_exact(P, S, sg.sys, min(i, j), max(i, j), f);
            j = __ldcg(P.next + j);
        }
    }
}

// kernel_pp_disk::check_for_ejection_hit_centrum (pp_disk.cu:283-318)
__global__ void __launch_bounds__(kSegment) k_ejhc(const EjhcParams P)
{
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
// launchers
// ---------------------------------------------------------------------------
void set_tableau(const Tableau& tb, cudaStream_t s)
{
    cudaMemcpyToSymbolAsync(c_tb, &tb, sizeof(Tableau), 0, cudaMemcpyHostToDevice, s);
}

template <int MODE>
static void launch_stage_mode(const StageParams& P, int n, int exact, cudaStream_t s)
{
    if (exact) k_stage<MODE, true><<<n, kTile, 0, s>>>(P);
    else k_stage<MODE, false><<<n, kTile, 0, s>>>(P);
}

void launch_stage(const StageParams& P, int n_items, int mode, int stage_exact, cudaStream_t s)
{
    if (n_items <= 0) return;
    switch (mode) {
    case MODE_MIXED: launch_stage_mode<MODE_MIXED>(P, n_items, stage_exact, s); break;
    case MODE_FP64: launch_stage_mode<MODE_FP64>(P, n_items, stage_exact, s); break;
    case MODE_FP64_EXACT: launch_stage_mode<MODE_FP64_EXACT>(P, n_items, stage_exact, s); break;
    default: launch_stage_mode<MODE_FP32>(P, n_items, stage_exact, s); break;
    }
}

void launch_prep(const Segment* segs, int n_segs, const SysInfo* sinfo, const DevSys* sys, const double* y_r,
                 const double* mass, const double* radius, const int* id, float4* hi, float4* lo, int all,
                 cudaStream_t s)
{
    if (n_segs > 0) k_prep<<<n_segs, kSegment, 0, s>>>(segs, sinfo, sys, y_r, mass, radius, id, hi, lo, all);
}

void launch_control(const ControlParams& P, cudaStream_t s)
{
    k_control<<<(P.n_sys + 127) / 128, 128, 0, s>>>(P);
}

void launch_finish(const FinishParams& P, int n_segs, cudaStream_t s)
{
    if (n_segs <= 0) return;
    if (P.stage_exact) k_finish<true><<<n_segs, 4 * kFinishBodies, 0, s>>>(P);
    else k_finish<false><<<n_segs, 4 * kFinishBodies, 0, s>>>(P);
}

void launch_collision(const CollParams& P, int n_items, int n_segs, bool use_grid, size_t table_size,
                      cudaStream_t s)
{
    if (n_items > 0) k_collision<<<n_items, kTile, 0, s>>>(P);
    if (use_grid && n_segs > 0) {
        cudaMemsetAsync(P.head, 0xff, table_size * sizeof(int), s);
        k_grid_insert<<<n_segs, kSegment, 0, s>>>(P);
        k_grid_query<<<n_segs, kSegment, 0, s>>>(P);
    }
}

void launch_ejhc(const EjhcParams& P, int n_segs, cudaStream_t s)
{
    if (n_segs > 0) k_ejhc<<<n_segs, kSegment, 0, s>>>(P);
}

void launch_potential(const Segment* segs, int n_segs, const SysInfo* sinfo, const double* y_r,
                      const double* mass, const int* id, int sys_filter, int interacting, double* u,
                      cudaStream_t s)
{
    if (n_segs > 0) k_potential<<<n_segs, kSegment, 0, s>>>(segs, sinfo, y_r, mass, id, sys_filter, interacting, u);
}

}  // namespace redgb
