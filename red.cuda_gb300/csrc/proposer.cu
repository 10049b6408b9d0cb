// proposer.cu -- learned step-size proposals for the adaptive integrators.
//
// After every accepted step, a per-system feature vector is formed on the
// device from the new state.  A small MLP (12 -> 64 -> 64 -> 1, SiLU, BF16
// weights, FP32 accumulation) maps the normalised features to the log of the
// next step size.  The embedded error estimate still judges every try: a
// rejected proposal is retried with the classical controller's step, so only
// the number of rejected tries can change, never the accuracy test.
//
// Training runs on the GPU with the kernels below: a forward / backward pass
// over 16-row tiles writing per-tile gradients, a fixed-order reduction of the
// tiles (deterministic), and Adam on FP32 master weights that refreshes the
// BF16 copy used by inference.  The network is far too small for tensor cores
// to pay (a 16 x 64 x 64 tile per CTA): the kernels are latency-bound FMA code.
//
// Features (per system, from the accepted state; FP32 from the truncated FP64
// state -- they steer the step size only):
//   0 log|dt| of the accepted step      6 mean e      9 mean i
//   1 log(err / tol) of that step       7 rms e      10 rms i
//   2 log min over protoplanet-body pairs of distance / Hill radius
//   3 log max |a|                       8 max e      11 max i
//   4 max |v| / v_kep                   (e, i: osculating heliocentric elements
//   5 log N (active bodies)              of the active non-star bodies)
#include <cuda_bf16.h>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "proposer.cuh"
#include "redgb.h"

namespace redgb {

// FP64 -> FP32 by truncation of the bits (no FP64 instruction; within 1 ulp of
// FP32 of the rounded conversion).  Zero, denormals and values outside FP32's
// range are clamped.
__device__ __forceinline__ float d2f_trunc(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7F7FFFFFu);
    return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ float bf(const __nv_bfloat16* w, int i) { return __bfloat162float(w[i]); }

// partial q is combined by max (3, 6, 7, 8), min (9) or sum (the rest)
__device__ __forceinline__ float combine_part(int q, float a, float b)
{
    return (q == 3 || q == 6 || q == 7 || q == 8) ? fmaxf(a, b) : (q == 9 ? fminf(a, b) : a + b);
}

// ---------------------------------------------------------------------------
// features: per-segment partial sums, then per system in a fixed order
// ---------------------------------------------------------------------------
constexpr int kMaxHill = 64;   // protoplanet-class bodies tested for the Hill-radius feature

__global__ void __launch_bounds__(kSegment) k_feat_seg(const FeatParams P)
{
    __shared__ float hx[kMaxHill], hy[kMaxHill], hz[kMaxHill], hr[kMaxHill];
    __shared__ float red[kNPart][kSegment / 32];
    pdl_wait();
    pdl_trigger();
    const Segment sg = P.segs[blockIdx.x];
    const DevSys& S = P.sys[sg.sys];
    if (!S.accepted) return;   // uniform
    const SysInfo si = P.sinfo[sg.sys];
    const float mstar = si.n_star > 0 ? d2f_trunc(P.mass[si.off]) : 0.f;
    // the protoplanet-class bodies (SI bodies after the stars) and their Hill radii
    const int nh = min(kMaxHill, si.n_SI - si.n_star);
    for (int k = threadIdx.x; k < nh; k += blockDim.x) {
        const int i = si.off + si.n_star + k;
        const float4 p = P.pos[i];
        hx[k] = p.x;
        hy[k] = p.y;
        hz[k] = p.z;
        const float rr = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
        const float m = P.id[i] >= 0 ? d2f_trunc(P.mass[i]) : 0.f;
        hr[k] = (m > 0.f && mstar > 0.f) ? rr * cbrtf(m / (3.0f * mstar)) : 0.f;
    }
    __syncthreads();
    float part[kNPart];
#pragma unroll
    for (int q = 0; q < kNPart; q++) part[q] = q == 9 ? FLT_MAX : 0.f;
    const int j = sg.b0 + threadIdx.x;
    if (j < sg.b1 && j >= si.off + si.n_star && P.id[j] >= 0) {
        const float4 p = P.pos[j];
        const float vx = d2f_trunc(P.y_v[3 * j]), vy = d2f_trunc(P.y_v[3 * j + 1]), vz = d2f_trunc(P.y_v[3 * j + 2]);
        const float ax = d2f_trunc(P.acc[3 * j]), ay = d2f_trunc(P.acc[3 * j + 1]), az = d2f_trunc(P.acc[3 * j + 2]);
        const float mu = mstar + d2f_trunc(P.mass[j]);
        const float r = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
        const float v2 = vx * vx + vy * vy + vz * vz;
        // angular momentum h = r x v, eccentricity vector (v x h) / mu - r / |r|
        const float hxv = p.y * vz - p.z * vy, hyv = p.z * vx - p.x * vz, hzv = p.x * vy - p.y * vx;
        const float h = sqrtf(hxv * hxv + hyv * hyv + hzv * hzv);
        float e = 0.f, inc = 0.f, vr = 0.f;
        if (mu > 0.f && r > 0.f) {
            const float ex = (vy * hzv - vz * hyv) / mu - p.x / r;
            const float ey = (vz * hxv - vx * hzv) / mu - p.y / r;
            const float ez = (vx * hyv - vy * hxv) / mu - p.z / r;
            e = sqrtf(ex * ex + ey * ey + ez * ez);
            inc = h > 0.f ? acosf(fminf(1.f, fmaxf(-1.f, hzv / h))) : 0.f;
            vr = sqrtf(v2 * r / mu);
        }
        part[0] = 1.f;
        part[1] = e;
        part[2] = e * e;
        part[3] = e;
        part[4] = inc;
        part[5] = inc * inc;
        part[6] = inc;
        part[7] = vr;
        part[8] = sqrtf(ax * ax + ay * ay + az * az);
        const int self = j - (si.off + si.n_star);
        for (int k = 0; k < nh; k++) {
            if (k == self || !(hr[k] > 0.f)) continue;
            const float dx = p.x - hx[k], dy = p.y - hy[k], dz = p.z - hz[k];
            part[9] = fminf(part[9], sqrtf(dx * dx + dy * dy + dz * dz) / hr[k]);
        }
    }
    // block reduction in a fixed order: warp trees, then one thread per partial over the warps
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kNPart; q++) {
        float v = part[q];
        for (int o = 16; o > 0; o >>= 1) v = combine_part(q, v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[q][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < kNPart) {
        const int q = threadIdx.x;
        float v = red[q][0];
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) v = combine_part(q, v, red[q][k]);
        P.part[(size_t)blockIdx.x * kNPart + q] = v;
    }
}

// ---------------------------------------------------------------------------
// the MLP on one warp: hidden units lane and lane + 32 of both layers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float mlp_warp(const __nv_bfloat16* w, const float (&xn)[kFeat], int lane)
{
    float h1[2], h2[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int u = lane + 32 * q;
        float z = bf(w, oB1 + u);
#pragma unroll
        for (int c = 0; c < kFeat; c++) z = fmaf(bf(w, oW1 + u * kFeat + c), xn[c], z);
        h1[q] = silu(z);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int u = lane + 32 * q;
        float z = bf(w, oB2 + u);
#pragma unroll
        for (int k = 0; k < kHid; k++) z = fmaf(bf(w, oW2 + u * kHid + k), __shfl_sync(0xffffffffu, h1[k >> 5], k & 31), z);
        h2[q] = silu(z);
    }
    float y = fmaf(bf(w, oW3 + lane), h2[0], bf(w, oW3 + lane + 32) * h2[1]);
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
    return y + bf(w, oB3);
}

__device__ __forceinline__ void normalise(const MlpNorm& nm, const float (&f)[kFeat], float (&xn)[kFeat])
{
#pragma unroll
    for (int c = 0; c < kFeat; c++) xn[c] = (f[c] - nm.x_mean[c]) / nm.x_std[c];
}

// One warp per system that accepted its try: the features from the segment
// partials (fixed order), the log record, the proposal.
__global__ void k_propose(const ProposeParams P)
{
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= P.n_sys) return;
    DevSys& S = P.sys[s];
    if (!S.accepted) return;   // uniform over the warp
    float part[kNPart];
#pragma unroll
    for (int q = 0; q < kNPart; q++) part[q] = q == 9 ? FLT_MAX : 0.f;
    for (int k = lane; k < P.nseg[s]; k += 32) {
        const float* p = P.part + (size_t)(P.seg0[s] + k) * kNPart;
#pragma unroll
        for (int q = 0; q < kNPart; q++) part[q] = combine_part(q, part[q], p[q]);
    }
#pragma unroll
    for (int q = 0; q < kNPart; q++)
        for (int o = 16; o > 0; o >>= 1) part[q] = combine_part(q, part[q], __shfl_xor_sync(0xffffffffu, part[q], o));
    const double dt_did = S.dt_did;
    const float cnt = fmaxf(part[0], 1.f);
    float f[kFeat];
    f[0] = logf(fmaxf(d2f_trunc(fabs(dt_did)), 1e-30f));
    f[1] = logf(fmaxf(d2f_trunc(S.err_last / P.tolerance), 1e-30f));
    f[2] = part[9] < FLT_MAX ? logf(fmaxf(part[9], 1e-30f)) : 0.f;
    f[3] = logf(fmaxf(part[8], 1e-30f));
    f[4] = part[7];
    f[5] = logf(cnt);
    f[6] = part[1] / cnt;
    f[7] = sqrtf(part[2] / cnt);
    f[8] = part[3];
    f[9] = part[4] / cnt;
    f[10] = sqrtf(part[5] / cnt);
    f[11] = part[6];
    if (P.log && lane == 0) {
        if (P.has_prev[s]) {
            const unsigned k = atomicAdd(P.log_n, 1u);
            if (k < P.log_cap) {
                float* r = P.log_buf + (size_t)k * kLogRec;
                for (int c = 0; c < kFeat; c++) r[c] = P.feat_prev[s * kFeat + c];
                r[kFeat] = f[0];       // log|dt| of the step accepted after those features
                r[kFeat + 1] = f[1];   // log(err / tol) of that step
            }
        }
        for (int c = 0; c < kFeat; c++) P.feat_prev[s * kFeat + c] = f[c];
        P.has_prev[s] = 1;
    }
    if (!P.propose) return;
    float xn[kFeat];
    normalise(P.norm, f, xn);
    const float y = mlp_warp(P.w, xn, lane);
    if (lane != 0) return;
    const double log_dt = (double)y * P.norm.y_std + P.norm.y_mean;
    const double mag = fabs(dt_did);
    double ratio = exp(log_dt) * P.safety / mag;
    ratio = fmin(fmax(ratio, P.ratio_lo), P.ratio_hi);
    if (!(ratio == ratio)) return;   // keep the classical step
    double dt = (dt_did < 0.0 ? -mag : mag) * ratio;
    if (P.output_interval != 0.0 && fabs(P.output_interval) < fabs(dt))
        dt = 0.0 < dt ? fabs(P.output_interval) : -fabs(P.output_interval);
    S.dt_next = dt;
    S.dt_try = dt;
}

// Inference on rows of raw features (warp per row): out = predicted log|dt|.
__global__ void k_mlp_rows(const __nv_bfloat16* w, const MlpNorm nm, const float* x, float* out, int n)
{
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= n) return;
    float f[kFeat], xn[kFeat];
#pragma unroll
    for (int c = 0; c < kFeat; c++) f[c] = x[(size_t)r * kFeat + c];
    normalise(nm, f, xn);
    const float y = mlp_warp(w, xn, lane);
    if (lane == 0) out[r] = y * nm.y_std + nm.y_mean;
}

// ---------------------------------------------------------------------------
// training: loss = sum over rows of (y - t)^2 / (2 n), normalised inputs and
// targets.  CTA = kTrainRows rows, thread u = hidden unit u of both layers.
// Each CTA writes its gradient (kNParam floats) and loss; k_mlp_sum adds the
// CTAs in index order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kHid) k_mlp_train(const __nv_bfloat16* w, const float* xn, const float* tn, int n,
                                                   float* part)
{
    constexpr int R = kTrainRows;
    __shared__ float W1[kHid * kFeat], W2[kHid * kHid], w3[kHid];
    __shared__ float x[R][kFeat], h1[R][kHid], h2[R][kHid], dz2[R][kHid], yv[R], dy[R];
    const int u = threadIdx.x;
    const int r0 = blockIdx.x * R;
    for (int k = u; k < kHid * kFeat; k += kHid) W1[k] = bf(w, oW1 + k);
    for (int k = u; k < kHid * kHid; k += kHid) W2[k] = bf(w, oW2 + k);
    w3[u] = bf(w, oW3 + u);
    for (int k = u; k < R * kFeat; k += kHid) {
        const int r = k / kFeat, c = k % kFeat;
        x[r][c] = r0 + r < n ? xn[(size_t)(r0 + r) * kFeat + c] : 0.f;
    }
    __syncthreads();
    // forward
    float z1[R], z2[R];
    const float b1 = bf(w, oB1 + u), b2 = bf(w, oB2 + u);
#pragma unroll
    for (int r = 0; r < R; r++) {
        float z = b1;
#pragma unroll
        for (int c = 0; c < kFeat; c++) z = fmaf(W1[u * kFeat + c], x[r][c], z);
        z1[r] = z;
        h1[r][u] = silu(z);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; r++) {
        float z = b2;
        for (int k = 0; k < kHid; k++) z = fmaf(W2[u * kHid + k], h1[r][k], z);
        z2[r] = z;
        h2[r][u] = silu(z);
    }
    __syncthreads();
    if (u < R) {
        const int r = u;
        float y = bf(w, oB3);
        for (int k = 0; k < kHid; k++) y = fmaf(w3[k], h2[r][k], y);
        yv[r] = y;
        dy[r] = r0 + r < n ? (y - tn[r0 + r]) / (float)n : 0.f;
    }
    __syncthreads();
    float* g = part + (size_t)blockIdx.x * (kNParam + 1);
    // output layer
    {
        float gw3 = 0.f;
        for (int r = 0; r < R; r++) gw3 = fmaf(dy[r], h2[r][u], gw3);
        g[oW3 + u] = gw3;
        if (u == 0) {
            float gb3 = 0.f, loss = 0.f;
            for (int r = 0; r < R; r++) {
                gb3 += dy[r];
                if (r0 + r < n) {
                    const float e = yv[r] - tn[r0 + r];
                    loss += e * e / (2.0f * (float)n);
                }
            }
            g[oB3] = gb3;
            g[kNParam] = loss;
        }
    }
    // hidden layer 2
    float gb2 = 0.f;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const float d = dy[r] * w3[u] * silu_grad(z2[r]);
        dz2[r][u] = d;
        gb2 += d;
    }
    g[oB2 + u] = gb2;
    __syncthreads();
    for (int k = 0; k < kHid; k++) {
        float a = 0.f;
#pragma unroll
        for (int r = 0; r < R; r++) a = fmaf(dz2[r][u], h1[r][k], a);
        g[oW2 + u * kHid + k] = a;
    }
    // hidden layer 1: thread u is unit u of layer 1 (its z1 is in registers)
    float gb1 = 0.f, gw1[kFeat];
#pragma unroll
    for (int c = 0; c < kFeat; c++) gw1[c] = 0.f;
#pragma unroll
    for (int r = 0; r < R; r++) {
        float dh = 0.f;
        for (int k = 0; k < kHid; k++) dh = fmaf(W2[k * kHid + u], dz2[r][k], dh);
        const float d = dh * silu_grad(z1[r]);
        gb1 += d;
#pragma unroll
        for (int c = 0; c < kFeat; c++) gw1[c] = fmaf(d, x[r][c], gw1[c]);
    }
    g[oB1 + u] = gb1;
#pragma unroll
    for (int c = 0; c < kFeat; c++) g[oW1 + u * kFeat + c] = gw1[c];
}

// Sum of the CTAs' gradients and losses, in CTA order.
__global__ void k_mlp_sum(const float* part, int nblk, float* grad, float* loss)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kNParam) return;
    float a = 0.f;
    for (int b = 0; b < nblk; b++) a += part[(size_t)b * (kNParam + 1) + p];
    if (p < kNParam) grad[p] = a;
    else *loss = a;
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the BF16 copy.
__global__ void k_adam(float* master, __nv_bfloat16* w, float* m, float* v, const float* grad, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kNParam) return;
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.f - b1) * g;
    const float vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float x = master[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    master[p] = x;
    w[p] = __float2bfloat16_rn(x);
}

void launch_features(const FeatParams& F, int n_segs, cudaStream_t s)
{
    if (n_segs > 0) launch_k(k_feat_seg, (unsigned)n_segs, (unsigned)kSegment, s, F);
}

void launch_propose(const ProposeParams& P, cudaStream_t s)
{
    if (P.n_sys > 0) launch_k(k_propose, (unsigned)((P.n_sys + 3) / 4), 128u, s, P);
}

}  // namespace redgb

// ---------------------------------------------------------------------------
// C ABI: the network on its own (training and evaluation on device buffers)
// ---------------------------------------------------------------------------
using namespace redgb;

int redgb_set_error(int code, const char* msg);

static_assert(sizeof(red_mlp_norm_t) == sizeof(MlpNorm), "red_mlp_norm_t mirrors MlpNorm");

namespace {
std::mutex g_work_mu;
float* g_work = nullptr;   // per-CTA gradients of red_mlp_grad, grown as needed
size_t g_work_cap = 0;
int g_work_dev = -1;

int cuda_fail(cudaError_t e, const char* what)
{
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return redgb_set_error(RED_ERR_CUDA, buf);
}
}  // namespace

extern "C" {

uint32_t red_mlp_param_count(void) { return (uint32_t)kNParam; }

int red_mlp_predict(const void* w_bf16, const red_mlp_norm_t* norm, const float* x, float* out, uint32_t n,
                    void* stream)
{
    if (!w_bf16 || !norm || (n && (!x || !out))) return redgb_set_error(RED_ERR_ARG, "red_mlp_predict: null argument");
    if (n == 0) return RED_OK;
    MlpNorm nm;
    memcpy(&nm, norm, sizeof(nm));
    k_mlp_rows<<<(n + 3) / 4, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)w_bf16, nm, x, out, (int)n);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RED_OK : cuda_fail(e, "red_mlp_predict");
}

int red_mlp_grad(const void* w_bf16, const float* xn, const float* tn, uint32_t n, float* grad, float* loss,
                 void* stream)
{
    if (!w_bf16 || !xn || !tn || !grad || !loss || n == 0)
        return redgb_set_error(RED_ERR_ARG, "red_mlp_grad: bad argument");
    const int nblk = (int)((n + kTrainRows - 1) / kTrainRows);
    const size_t need = (size_t)nblk * (kNParam + 1);
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_work_mu);
    if (need > g_work_cap || dev != g_work_dev) {
        cudaStreamSynchronize((cudaStream_t)stream);
        if (g_work) cudaFree(g_work);
        g_work = nullptr;
        g_work_cap = 0;
        const cudaError_t e = cudaMalloc(&g_work, need * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(e, "red_mlp_grad: workspace");
        g_work_cap = need;
        g_work_dev = dev;
    }
    cudaStream_t s = (cudaStream_t)stream;
    k_mlp_train<<<nblk, kHid, 0, s>>>((const __nv_bfloat16*)w_bf16, xn, tn, (int)n, g_work);
    k_mlp_sum<<<(kNParam + 1 + 255) / 256, 256, 0, s>>>(g_work, nblk, grad, loss);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RED_OK : cuda_fail(e, "red_mlp_grad");
}

int red_mlp_adam(float* master, void* w_bf16, float* m, float* v, const float* grad, uint32_t step, float lr,
                 float beta1, float beta2, float eps, void* stream)
{
    if (!master || !w_bf16 || !m || !v || !grad || step == 0)
        return redgb_set_error(RED_ERR_ARG, "red_mlp_adam: bad argument");
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<(kNParam + 255) / 256, 256, 0, (cudaStream_t)stream>>>(master, (__nv_bfloat16*)w_bf16, m, v, grad, lr,
                                                                   beta1, beta2, eps, c1, c2);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RED_OK : cuda_fail(e, "red_mlp_adam");
}

}  // extern "C"
