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

__device__ void drag_accel(const GasDev& g, double decr, double m_star, double rx, double ry, double rz,
                           double vx, double vy, double vz, double cd, double radius, double density,
                           double& ax, double& ay, double& az)
{
    // gas velocity: circular velocity scaled by sqrt(1 - 2 eta r^p) (pp_disk.cu:107-155)
    const double r = sqrt(rx * rx + ry * ry);
    const double vc = sqrt(m_star / r);
    double gx = 0.0, gy = 0.0;
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
    const double f = decr * (3.0 * cd * dens * un) / (8.0 * radius * density);
    ax += f * ux;
    ay += f * uy;
    az += f * uz;
}

// ---------------------------------------------------------------------------
// stage kernel
// ---------------------------------------------------------------------------
struct alignas(32) D4 {
    double x, y, z, w;
};

struct SmemStage {
    union {
        struct { float4 hi[kTile]; float4 lo[kTile]; } f;
        struct { D4 d[kTile]; int id[kTile]; } d;
    } src;
    double red[kTile][3];
    unsigned long long emax[kTile / 32];
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

// Stage combination for body i: ytemp of stage `nx` (RKF78: y + dt*sum a K,
// red's term order; RK4: y + (a dt) K).
template <bool EXACT>
__device__ __forceinline__ void combine(const StageParams& P, int scheme, int nx, double dt, int i,
                                        double out_r[3], double out_v[3])
{
    if (scheme == SCHEME_RKF78) {
        const int nnz = c_tb.nnz[nx];
        const int off = 1 + nx * (nx - 1) / 2;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            int q0 = c_tb.src[nx][0];
            double ar = mul<EXACT>(c_tb.a[off + q0], P.Kr[q0][3 * i + c]);
            double av = mul<EXACT>(c_tb.a[off + q0], P.Kv[q0][3 * i + c]);
            for (int q = 1; q < nnz; q++) {
                const int sq = c_tb.src[nx][q];
                const double aq = c_tb.a[off + sq];
                ar = madd<EXACT>(ar, aq, P.Kr[sq][3 * i + c]);
                av = madd<EXACT>(av, aq, P.Kv[sq][3 * i + c]);
            }
            out_r[c] = madd<EXACT>(P.y_r[3 * i + c], dt, ar);
            out_v[c] = madd<EXACT>(P.y_v[3 * i + c], dt, av);
        }
    } else {
        // rk4_kernel::sum_vector: y + (a[r] * dt) * f_{r-1} (int_rungekutta4.cu:36-47, 111-129)
        const double bf = mul<EXACT>(c_tb.a4[nx], dt);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            out_r[c] = madd<EXACT>(P.y_r[3 * i + c], bf, P.Kr[nx - 1][3 * i + c]);
            out_v[c] = madd<EXACT>(P.y_v[3 * i + c], bf, P.Kv[nx - 1][3 * i + c]);
        }
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

template <int MODE, bool EXACT>
__device__ __forceinline__ double stage_epilogue(const StageParams& P, const GravItem& it, DevSys* S, int i,
                                                 double ax, double ay, double az)
{
    const SysInfo si = P.sinfo[it.sys];
    const int s = P.stage;
    const double rx = P.r_in[3 * i], ry = P.r_in[3 * i + 1], rz = P.r_in[3 * i + 2];
    const int idi = P.id[i];
    if (idi > 0) {
        if (MODE == MODE_MIXED || MODE == MODE_FP32) {
            // central-star term in FP64 with red's pair formula (pp_disk.cu:399-413)
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int j = si.off; j < si.off + si.n_star; j++) {
                if (j == i || P.id[j] < 0) continue;
                const double dx = P.r_in[3 * j] - rx, dy = P.r_in[3 * j + 1] - ry, dz = P.r_in[3 * j + 2] - rz;
                const double w = dx * dx + dy * dy + dz * dz;
                const double d = sqrt(w);
                const double f = P.mass[j] / (d * w);
                sx += f * dx;
                sy += f * dy;
                sz += f * dz;
            }
            ax = sx + ax;
            ay = sy + ay;
            az = sz + az;
        }
    } else {
        ax = ay = az = 0.0;   // calc_grav_accel_naive zeroes inactive sinks (pp_disk.cu:386-388)
    }
    const double dt = S->dt_try;
    if (P.gas.enabled && it.cls == CLS_NSI) {
        const double ts = P.standalone ? P.t_standalone
                                       : S->t + (P.scheme == SCHEME_RKF78 ? c_tb.c[s] : c_tb.c4[s]) * dt;
        const double decr = gas_reduction_factor(P.gas, ts);
        if (!(1.0e-6 > decr)) {
            drag_accel(P.gas, decr, P.mass[si.off], rx, ry, rz, P.Kr[s][3 * i], P.Kr[s][3 * i + 1],
                       P.Kr[s][3 * i + 2], P.cd[i], P.radius[i], P.density[i], ax, ay, az);
        }
    }
    P.Kv[s][3 * i] = ax;
    P.Kv[s][3 * i + 1] = ay;
    P.Kv[s][3 * i + 2] = az;
    if (P.standalone) return 0.0;

    if (P.next >= 0) {
        double orr[3], ovv[3];
        if (P.ynp1_to_out) {
            const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int x = 3 * i + c;
                orr[c] = rk4_ynp1<EXACT>(P.y_r[x], b0, b1, P.Kr[0][x], P.Kr[1][x], P.Kr[2][x], P.Kr[3][x]);
                ovv[c] = rk4_ynp1<EXACT>(P.y_v[x], b0, b1, P.Kv[0][x], P.Kv[1][x], P.Kv[2][x], P.Kv[3][x]);
            }
        } else {
            combine<EXACT>(P, P.scheme, P.next, dt, i, orr, ovv);
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            P.r_out[3 * i + c] = orr[c];
            P.Kr[P.next][3 * i + c] = ovv[c];
        }
        write_pos(P.pos_hi_out, P.pos_lo_out, i, orr[0], orr[1], orr[2], idi >= 0 ? P.mass[i] : 0.0, P.radius[i]);
    }
    double e = 0.0;
    if (P.err_after && i - si.off < si.n_err) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int x = 3 * i + c;
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
            e = fmax(e, fmax(er, ev));
            if (er != er || ev != ev) e = __longlong_as_double(0x7ff8000000000000ll);
        }
    }
    return e;
}

template <int MODE, bool EXACT>
__global__ void __launch_bounds__(kTile) k_stage(const StageParams P)
{
    __shared__ SmemStage sm;
    const GravItem it = P.items[blockIdx.x];
    DevSys* S = P.sys + it.sys;
    if (!P.standalone && !runnable(*S)) return;   // uniform over the CTA

    // lanes threads per sink: thread t works on sink t % nsink over the sources
    // j = sub_lane, sub_lane + lanes, ... of every tile
    const int L = it.lanes;
    const int SP = it.nsink;
    const int k = threadIdx.x % SP;
    const int sub_lane = threadIdx.x / SP;
    const bool has = sub_lane < L;
    const int i = it.sink0 + k;

    double ax = 0.0, ay = 0.0, az = 0.0;

    if (MODE == MODE_MIXED || MODE == MODE_FP32) {
        float4 H = make_float4(0.f, 0.f, 0.f, 0.f), Lo = make_float4(0.f, 0.f, 0.f, 0.f);
        if (has) {
            H = P.pos_hi_in[i];
            if (MODE == MODE_MIXED) Lo = P.pos_lo_in[i];
        }
        float sxh = 0.f, sxl = 0.f, syh = 0.f, syl = 0.f, szh = 0.f, szl = 0.f;
        for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
            const int nj = min(kTile, it.src1 - j0);
            __syncthreads();
            load_sources<MODE>(sm, P, j0, nj);
            __syncthreads();
            if (has) {
                float tx = 0.f, ty = 0.f, tz = 0.f;
#pragma unroll 4
                for (int jj = sub_lane; jj < nj; jj += L) {
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
        ax = (double)sxh + (double)sxl;
        ay = (double)syh + (double)syl;
        az = (double)szh + (double)szl;
    } else {
        double xi = 0.0, yi = 0.0, zi = 0.0;
        if (has) {
            xi = P.r_in[3 * i];
            yi = P.r_in[3 * i + 1];
            zi = P.r_in[3 * i + 2];
        }
        for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
            const int nj = min(kTile, it.src1 - j0);
            __syncthreads();
            load_sources<MODE>(sm, P, j0, nj);
            __syncthreads();
            if (has) {
                for (int jj = sub_lane; jj < nj; jj += L) {
                    const D4 q = sm.src.d.d[jj];
                    if (MODE == MODE_FP64_EXACT) {
                        // calc_grav_accel_naive, pp_disk.cu:389-413, bit for bit
                        if (j0 + jj == i || 0 > sm.src.d.id[jj]) continue;
                        const double dx = __dsub_rn(q.x, xi), dy = __dsub_rn(q.y, yi), dz = __dsub_rn(q.z, zi);
                        double w = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                        const double d = __dsqrt_rn(w);
                        w = __ddiv_rn(q.w, __dmul_rn(d, w));
                        ax = __dadd_rn(ax, __dmul_rn(w, dx));
                        ay = __dadd_rn(ay, __dmul_rn(w, dy));
                        az = __dadd_rn(az, __dmul_rn(w, dz));
                    } else {
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
    }

    // lanes of one sink -> one sum, fixed order
    if (L > 1) {
        __syncthreads();
        sm.red[threadIdx.x][0] = ax;
        sm.red[threadIdx.x][1] = ay;
        sm.red[threadIdx.x][2] = az;
        __syncthreads();
        if (sub_lane == 0) {
            for (int q = 1; q < L; q++) {
                ax += sm.red[k + q * SP][0];
                ay += sm.red[k + q * SP][1];
                az += sm.red[k + q * SP][2];
            }
        }
    }
    const bool owner = (sub_lane == 0) && has;

    // source chunks of one sink tile -> the CTA that finishes last reduces them
    if (it.nchunk > 1) {
        if (owner) {
            double* p = P.partial + 3 * ((long long)it.part_off + (long long)it.chunk * it.nsink + k);
            p[0] = ax;
            p[1] = ay;
            p[2] = az;
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
        // the lanes of each sink split the chunks (c = sub_lane, sub_lane + L, ...);
        // loads are issued in batches so that they overlap, sums run in a fixed order
        ax = ay = az = 0.0;
        if (has) {
            constexpr int B = 8;
            for (int c0 = sub_lane; c0 < it.nchunk; c0 += B * L) {
                double px[B], py[B], pz[B];
#pragma unroll
                for (int u = 0; u < B; u++) {
                    const int c = c0 + u * L;
                    if (c < it.nchunk) {
                        const double* p = P.partial + 3 * ((long long)it.part_off + (long long)c * it.nsink + k);
                        px[u] = __ldcg(p);
                        py[u] = __ldcg(p + 1);
                        pz[u] = __ldcg(p + 2);
                    } else {
                        px[u] = py[u] = pz[u] = 0.0;
                    }
                }
#pragma unroll
                for (int u = 0; u < B; u++) {
                    ax += px[u];
                    ay += py[u];
                    az += pz[u];
                }
            }
        }
        if (L > 1) {
            __syncthreads();
            sm.red[threadIdx.x][0] = ax;
            sm.red[threadIdx.x][1] = ay;
            sm.red[threadIdx.x][2] = az;
            __syncthreads();
            if (sub_lane == 0) {
                for (int q = 1; q < L; q++) {
                    ax += sm.red[k + q * SP][0];
                    ay += sm.red[k + q * SP][1];
                    az += sm.red[k + q * SP][2];
                }
            }
        }
        if (threadIdx.x == 0) P.tile_cnt[it.tile] = 0u;
    }

    double e = 0.0;
    if (owner) e = stage_epilogue<MODE, EXACT>(P, it, S, i, ax, ay, az);

    if (P.err_after) {
        // CTA max of the error, one atomic per CTA (non-negative doubles order as their bits)
        unsigned long long b = (unsigned long long)__double_as_longlong(e);
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(0xffffffffu, b, o);
            b = ob > b ? ob : b;
        }
        if ((threadIdx.x & 31) == 0) sm.emax[threadIdx.x >> 5] = b;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long m = 0;
            for (int w = 0; w < kTile / 32; w++) m = sm.emax[w] > m ? sm.emax[w] : m;
            if (m) atomicMax(&S->err_bits, m);
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

template <bool EXACT>
__global__ void __launch_bounds__(kSegment) k_finish(const FinishParams P)
{
    const Segment sg = P.segs[blockIdx.x];
    DevSys* S = P.sys + sg.sys;
    if (S->halted) return;
    const int i = sg.b0 + threadIdx.x;
    const bool acc = S->accepted;
    if (!acc && !runnable(*S)) return;
    if (i >= sg.b1) return;
    double r[3], v[3];
    if (acc) {
        const double dt = S->dt_did;
        if (P.scheme == SCHEME_RKF78) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                r[c] = rk8_ynp1<EXACT>(P.y_r[3 * i + c], dt, P.Kr, 3 * i + c);
                v[c] = rk8_ynp1<EXACT>(P.y_v[3 * i + c], dt, P.Kv, 3 * i + c);
            }
        } else if (P.commit_from_stage4) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                r[c] = P.t_r0[3 * i + c];
                v[c] = P.Kr[4][3 * i + c];
            }
        } else {
            const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int x = 3 * i + c;
                r[c] = rk4_ynp1<EXACT>(P.y_r[x], b0, b1, P.Kr[0][x], P.Kr[1][x], P.Kr[2][x], P.Kr[3][x]);
                v[c] = rk4_ynp1<EXACT>(P.y_v[x], b0, b1, P.Kv[0][x], P.Kv[1][x], P.Kv[2][x], P.Kv[3][x]);
            }
        }
        bool fin = true;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            P.y_r[3 * i + c] = r[c];
            P.y_v[3 * i + c] = v[c];
            fin = fin && isfinite(r[c]) && isfinite(v[c]);
        }
        if (!fin) S->status = 5;
    } else {
#pragma unroll
        for (int c = 0; c < 3; c++) r[c] = P.y_r[3 * i + c];
    }
    write_pos(P.pos_hi0, P.pos_lo0, i, r[0], r[1], r[2], P.id[i] >= 0 ? P.mass[i] : 0.0, P.radius[i]);
}

// ---------------------------------------------------------------------------
// collision detection: kernel_pp_disk::check_for_collision (pp_disk.cu:320-371)
// over tile pairs; an FP32 double-single prefilter with a safety margin picks
// the candidates, red's FP64 test (no FMA) decides.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) k_collision(const CollParams P)
{
    __shared__ float4 shi[kTile], slo[kTile];
    const PairItem it = P.items[blockIdx.x];
    DevSys* S = P.sys + it.sys;
    if (S->halted) return;
    if (P.only_accepted && !S->accepted) return;
    const SysInfo si = P.sinfo[it.sys];
    const int end = si.off + si.n;
    const int i = it.i0 + threadIdx.x;
    const int j = it.j0 + threadIdx.x;
    if (j < end) {
        shi[threadIdx.x] = P.pos_hi[j];
        slo[threadIdx.x] = P.pos_lo[j];
    }
    __syncthreads();
    if (i >= end) return;
    const float4 H = P.pos_hi[i], Lo = P.pos_lo[i];
    const int nj = min(kTile, end - it.j0);
    const float fac = (float)P.factor;
    const double f = P.factor * P.factor;
    for (int jj = 0; jj < nj; jj++) {
        const int jx = it.j0 + jj;
        if (jx <= i) continue;
        const float4 h = shi[jj], l = slo[jj];
        const float dx = (h.x - H.x) + (l.x - Lo.x);
        const float dy = (h.y - H.y) + (l.y - Lo.y);
        const float dz = (h.z - H.z) + (l.z - Lo.z);
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float th = fac * (Lo.w + l.w);
        if (!(d2 <= 1.0001f * th * th + 1.0e-30f)) continue;
        // red's test, bit for bit (pp_disk.cu:336-357)
        if (!(0 < P.id[i]) || 0 > P.id[jx]) continue;
        const double ddx = __dsub_rn(P.y_r[3 * jx], P.y_r[3 * i]);
        const double ddy = __dsub_rn(P.y_r[3 * jx + 1], P.y_r[3 * i + 1]);
        const double ddz = __dsub_rn(P.y_r[3 * jx + 2], P.y_r[3 * i + 2]);
        const double w = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
        const double rs = __dadd_rn(P.radius[i], P.radius[jx]);
        if (w < __dmul_rn(f, __dmul_rn(rs, rs))) {
            int surv = i, merg = jx;
            if (P.mass[merg] > P.mass[surv]) {
                surv = jx;
                merg = i;
            }
            const unsigned kk = atomicAdd(P.n_events, 1u);
            if (kk < P.capacity) {
                DevEvent ev;
                ev.sys = it.sys;
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
    if (P.stage_exact) k_finish<true><<<n_segs, kSegment, 0, s>>>(P);
    else k_finish<false><<<n_segs, kSegment, 0, s>>>(P);
}

void launch_collision(const CollParams& P, int n_items, cudaStream_t s)
{
    if (n_items > 0) k_collision<<<n_items, kTile, 0, s>>>(P);
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
