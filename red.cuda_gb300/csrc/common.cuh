// common.cuh -- device helpers shared by the kernels of libredgb: double-single
// arithmetic, red's multiply/add order switch, analytic gas drag, the RKF7(8)
// and RK4 stage combinations, the FP32 position copies.
#pragma once
#include <cfloat>
#include <cstdio>
#include <utility>

#include "crmath.cuh"
#include "redgb_dev.cuh"

namespace redgb {

// Integrator tableaux; every translation unit that includes this header has
// its own copy, loaded by its set_tableau_* function.
static __constant__ Tableau c_tb;

// Squared softening added to r^2 in the FP32 loops only, so that the self pair
// (r = 0 exactly) contributes 0 * finite instead of 0 * inf.  For any real pair
// (r >= 1e-6 AU) it changes the force by < 1e-11 relative, far below FP32
// rounding.  The FP64 paths use no softening, as red.
constexpr float kEps2 = 1.0e-24f;

// ---------------------------------------------------------------------------
// programmatic dependent launch
// ---------------------------------------------------------------------------
// Every kernel of a try calls pdl_wait() in each CTA before it reads what the
// previous kernel of the try wrote, and before it exits; then pdl_trigger().
// So a kernel completes only after its predecessor has completed, and the
// successor is scheduled only once every CTA of this kernel has passed its
// wait: whatever kernels before the predecessor wrote is complete when the
// successor starts.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// Launches kernel k in thread-block clusters of `cluster` CTAs when cluster >
// 1, and with the programmatic-stream-serialization attribute while pdl_on()
// holds on this thread.
template <typename... KArgs, typename... Args>
inline void launch_kx(void (*k)(KArgs...), unsigned grid, unsigned block, unsigned cluster, cudaStream_t s,
                      Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    int na = 0;
    if (pdl_on()) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        na++;
    }
    if (cluster > 1) {
        at[na].id = cudaLaunchAttributeClusterDimension;
        at[na].val.clusterDim.x = cluster;
        at[na].val.clusterDim.y = 1;
        at[na].val.clusterDim.z = 1;
        na++;
    }
    cfg.attrs = at;
    cfg.numAttrs = na;
    cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}
template <typename... KArgs, typename... Args>
inline void launch_k(void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args&&... args)
{
    launch_kx(k, grid, block, 1u, s, std::forward<Args>(args)...);
}

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

// Double-single numbers as float2 (x = hi, y = lo, hi + lo the value, |lo| <=
// ulp(hi)): Dekker (1971) and Knuth's TwoSum, the product's error term from
// fmaf.  About 48 significant bits.
__device__ __forceinline__ float2 dsn(float hi, float lo) { return make_float2(hi, lo); }
// a + b with |a| >= |b| (Dekker's Fast2Sum)
__device__ __forceinline__ float2 dsn_fast(float a, float b)
{
    const float s = a + b;
    return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 dsn_norm(float a, float b)
{
    float s, e;
    two_sum(a, b, s, e);
    return make_float2(s, e);
}
__device__ __forceinline__ float2 dsn_add(float2 a, float2 b)
{
    float s, e;
    two_sum(a.x, b.x, s, e);
    return dsn_fast(s, e + (a.y + b.y));
}
__device__ __forceinline__ float2 dsn_sub(float2 a, float2 b)
{
    float s, e;
    two_sum(a.x, -b.x, s, e);
    return dsn_fast(s, e + (a.y - b.y));
}
__device__ __forceinline__ float2 dsn_mul(float2 a, float2 b)
{
    const float p = a.x * b.x;
    const float e = fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.x, b.x, -p)));
    return dsn_fast(p, e);
}
__device__ __forceinline__ float2 dsn_sqr(float2 a)
{
    const float p = a.x * a.x;
    return dsn_fast(p, fmaf(a.x + a.x, a.y, fmaf(a.x, a.x, -p)));
}
// 1 / sqrt(x) for x > 0: the hardware estimate, one FP32 Newton step (to
// ~1 ulp of FP32), then one Newton step y + y (1 - x y^2) / 2 with the
// residual formed in double-single: relative error ~2e-14.
__device__ __forceinline__ float2 dsn_rsqrt(float2 x)
{
    float y = rsqrtf(x.x);
    y = y * fmaf(-0.5f * x.x, y * y, 1.5f);
    const float yy = y * y;
    const float2 t = dsn_mul(x, make_float2(yy, fmaf(y, y, -yy)));
    const float r = (1.0f - t.x) - t.y;
    return dsn_fast(y, 0.5f * y * r);
}

// x -> (h, l), h + l = x to 2^-48 relative: h is x truncated to 24 significant
// bits, l the remaining 29 bits rounded to 24.  Built from the bits with
// integer operations (GB300's FP64 pipe runs at 1/64 of FP32); values outside
// FP32's normal range (|x| < 2^-74 for l, zero, Inf, NaN) take the FP64 route.
__device__ __forceinline__ void split_ds(double x, float& h, float& l)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e >= 1023 - 74 + 23 && e <= 1023 + 127) {
        const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
        h = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
        const float m = __uint2float_rn((unsigned)(b & 0x1FFFFFFFull));        // the low 29 bits, rounded
        const float scale = __uint_as_float((unsigned)(e - 1075 + 127) << 23);  // 2^(e - 1023 - 52)
        l = __uint_as_float(__float_as_uint(m * scale) | sign);
    } else {
        h = __double2float_rn(x);
        l = __double2float_rn(x - (double)h);
    }
}

// Exact float -> double from the bits (zero and FP32 denormals give signed
// zero; Inf and NaN are kept).
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)sign);
    const unsigned long long ee = e == 0xFFu ? 0x7FFull : (unsigned long long)(e + 896u);
    return __longlong_as_double((long long)(sign | (ee << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}
__device__ __forceinline__ double dsn_to_double(float2 a) { return f2d_bits(a.x) + f2d_bits(a.y); }

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
// In the red-exact mode (EXACT) every operation is one rounding in red's
// order (no contraction into FMA) and exp / pow return the nearest double
// (crmath.cuh), as the C library's functions in red's CPU twin do.
template <bool EXACT> __device__ __forceinline__ double dexp(double x)
{
    return EXACT ? crmath::cr_exp(x) : exp(x);
}
template <bool EXACT> __device__ __forceinline__ double dpow(double x, double y)
{
    return EXACT ? crmath::cr_pow(x, y) : pow(x, y);
}
template <bool EXACT> __device__ __forceinline__ double ddiv(double a, double b)
{
    return EXACT ? __ddiv_rn(a, b) : a / b;
}
template <bool EXACT> __device__ __forceinline__ double dsqrt(double a)
{
    return EXACT ? __dsqrt_rn(a) : sqrt(a);
}

template <bool EXACT> static __device__ double gas_reduction_factor(const GasDev& g, double t)
{
    switch (g.gas_decrease) {
    case 0: return 1.0;
    case 1:
        if (t <= g.t0) return 1.0;
        else if (g.t0 < t && t <= g.t1 && g.t0 != g.t1) return 1.0 - (t - g.t0) / (g.t1 - g.t0);
        else return 0.0;
    case 2: return dexp<EXACT>(ddiv<EXACT>(-sub<EXACT>(t, g.t0), g.e_folding_time));
    default: return 1.0;
    }
}

// Drag factor f and gas velocity (gx, gy, 0) at (r, v): the acceleration is
// f (v_gas - v) (calc_drag_accel_NSI, pp_disk.cu:485-521).  red's FP64
// arithmetic, for the FP64 modes.
template <bool EXACT>
static __device__ void drag_factor(const GasDev& g, double decr, double m_star, double rx, double ry, double rz,
                                   double vx, double vy, double vz, double cd, double radius, double density,
                                   double& f, double& gx, double& gy)
{
    // gas velocity: circular velocity scaled by sqrt(1 - 2 eta r^p) (pp_disk.cu:107-155)
    const double r = dsqrt<EXACT>(add<EXACT>(mul<EXACT>(rx, rx), mul<EXACT>(ry, ry)));
    const double vc = dsqrt<EXACT>(ddiv<EXACT>(m_star, r));
    gx = 0.0;
    gy = 0.0;
    if (rx == 0.0 && ry == 0.0) {
    } else if (ry == 0.0) {
        gy = rx > 0.0 ? vc : -vc;
    } else if (rx == 0.0) {
        gx = ry > 0.0 ? -vc : vc;
    } else if (rx >= ry) {
        const double p = ddiv<EXACT>(ry, rx);
        const double q = dsqrt<EXACT>(add<EXACT>(1.0, mul<EXACT>(p, p)));
        gy = rx >= 0 ? ddiv<EXACT>(vc, q) : ddiv<EXACT>(-vc, q);
        gx = mul<EXACT>(-gy, p);
    } else {
        const double p = ddiv<EXACT>(rx, ry);
        const double q = dsqrt<EXACT>(add<EXACT>(1.0, mul<EXACT>(p, p)));
        gx = ry >= 0 ? ddiv<EXACT>(-vc, q) : ddiv<EXACT>(vc, q);
        gy = mul<EXACT>(-gx, p);
    }
    const double fv =
        dsqrt<EXACT>(sub<EXACT>(1.0, mul<EXACT>(mul<EXACT>(2.0, g.eta[0]), dpow<EXACT>(r, g.eta[1]))));
    gx = mul<EXACT>(gx, fv);
    gy = mul<EXACT>(gy, fv);
    // gas density (pp_disk.cu:86-105)
    const double h = mul<EXACT>(g.sch[0], dpow<EXACT>(r, g.sch[1]));
    const double zh = ddiv<EXACT>(rz, h);
    const double arg = mul<EXACT>(zh, zh);
    double dens;
    if (0.1 < r) {
        dens = mul<EXACT>(mul<EXACT>(g.rho[0], dpow<EXACT>(r, g.rho[1])), dexp<EXACT>(-arg));
    } else {
        const double a = mul<EXACT>(g.rho[0], dpow<EXACT>(0.1, sub<EXACT>(g.rho[1], 4.0)));
        const double r2 = mul<EXACT>(r, r);
        dens = mul<EXACT>(mul<EXACT>(a, mul<EXACT>(r2, r2)), dexp<EXACT>(-arg));
    }
    const double ux = sub<EXACT>(gx, vx), uy = sub<EXACT>(gy, vy), uz = sub<EXACT>(0.0, vz);
    const double un =
        dsqrt<EXACT>(add<EXACT>(add<EXACT>(mul<EXACT>(ux, ux), mul<EXACT>(uy, uy)), mul<EXACT>(uz, uz)));
    f = ddiv<EXACT>(mul<EXACT>(decr, mul<EXACT>(mul<EXACT>(mul<EXACT>(3.0, cd), dens), un)),
                    mul<EXACT>(mul<EXACT>(8.0, radius), density));
}

// The same drag for the FP32 modes, with the transcendental factors in FP32.
// GB300 runs FP64 at 1/64 of the FP32 rate: red's chain of one sink (three
// pow, an exp, five square roots, three divisions) held a warp for ~9 us of
// every tile.  The gas velocity stays FP64, as vc fv (-y, x) / r (the vector
// red's branches form), because v_gas - v cancels ~99.5 % of it; fv = 1 + d,
// d = -x / (1 + sqrt(1 - x)) for x = 2 eta r^p, keeps it to ~1e-10.  The
// factor f (gas density, |v_gas - v|, the body's cross-section) is FP32, a
// ~1e-6 relative error on a drag that is at most ~1e-5 of a body's
// acceleration in red's disks, below the modes' own FP32 pair error.
static __device__ void drag_factor_fast(const GasDev& g, double decr, double m_star, double rx, double ry, double rz,
                                        double vx, double vy, double vz, double cd, double radius, double density,
                                        double& f, double& gx, double& gy)
{
    const double r2 = rx * rx + ry * ry;   // 0 on the disk's axis: NaN drag, as red's pow(0, p < 0)
    const double ir = rsqrt(r2);
    const float r = (float)(r2 * ir);
    const float x = 2.0f * (float)g.eta[0] * powf(r, (float)g.eta[1]);
    const double fv = 1.0 + (double)(-x / (1.0f + sqrtf(1.0f - x)));
    const double s = sqrt(m_star * ir) * ir * fv;
    gx = -ry * s;
    gy = rx * s;
    const float h = (float)g.sch[0] * powf(r, (float)g.sch[1]);
    const float zh = (float)rz / h;
    const float arg = zh * zh;
    float dens;
    if (0.1f < r) {
        dens = (float)g.rho[0] * powf(r, (float)g.rho[1]) * expf(-arg);
    } else {
        const float a = (float)g.rho[0] * powf(0.1f, (float)g.rho[1] - 4.0f);
        dens = a * (r * r) * (r * r) * expf(-arg);
    }
    const double ux = gx - vx, uy = gy - vy, uz = -vz;
    const float un = sqrtf((float)(ux * ux + uy * uy + uz * uz));
    f = decr * (double)((3.0f * (float)cd * dens * un) / (8.0f * (float)radius * (float)density));
}

struct alignas(32) D4 {
    double x, y, z, w;
};

// Nonzero terms of each RKF7(8) stage row in the order red's stage kernels
// add them (rk8_kernel::calc_ytemp_for_f1..f12, int_rungekutta8.cu:80-246).
// Compile-time copy of Tableau::src (the source stages of each RKF7(8)
// combination, in red's term order), for the per-variant kernel instances.
__device__ constexpr int kSrc[13][9] = {
    {0}, {0}, {0, 1}, {0, 2}, {0, 2, 3}, {0, 3, 4}, {0, 3, 4, 5}, {0, 4, 5, 6},
    {0, 3, 4, 5, 6, 7}, {0, 3, 4, 5, 6, 7, 8}, {0, 3, 4, 5, 6, 7, 8, 9},
    {0, 5, 6, 7, 8, 9}, {0, 3, 4, 5, 6, 7, 8, 9, 11}};

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

}  // namespace redgb
