// populate.cu -- initial conditions of disk ensembles on the GPU
// (red_populate_disks): red.cuda.initial's disk recipe, one thread per body.
//
//   k_pop_elements  orbital elements (Philox4x32-10 draws), planetesimal weights
//   k_pop_wsum      per system: the sum of the planetesimal weights (fixed order)
//   k_pop_phase     masses, Kepler -> Cartesian, radii, densities, metadata
//   k_pop_bary      per system: barycentre (fixed order), shift, velocities / K,
//                   red's records
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "redgb.h"

namespace redgb {

namespace {

constexpr double kK = 0.01720209895;                 // red_macro.h:13
constexpr double kK2 = 0.0002959122082855911025;     // red_macro.h:14
constexpr double kFourPiOverThree = 4.188790204786391;   // tools.cpp:457
constexpr double kTwoPi = 6.283185307179586;
constexpr double kPi = 3.1415926535897932384626;   // red_macro.h:16
constexpr int kPopBlock = 256;

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): ten rounds of two 32x32 -> 64-bit products on a
// 4-word counter, the 2-word key bumped by the Weyl constants between rounds.
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// A double in (0, 1] from two words: 53 bits of (hi, lo), plus one.
__device__ inline double u01(uint32_t hi, uint32_t lo)
{
    const uint64_t b = (((uint64_t)hi << 32) | lo) >> 11;
    return (double)(b + 1) * 1.1102230246251565e-16;   // 2^-53
}

// The six draws of body k of a system with this seed: counters (k, 0..2, 0, 0).
__device__ inline void draws6(uint64_t seed, uint32_t k, double u[6])
{
    for (int b = 0; b < 3; b++) {
        uint32_t c[4] = {k, (uint32_t)b, 0u, 0u};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        u[2 * b] = u01(c[0], c[1]);
        u[2 * b + 1] = u01(c[2], c[3]);
    }
}

struct PopParams {
    const red_disk_spec_t* spec;
    const int* off;          // first body of each system
    int n_sys;
    double rho_unit;         // g/cm^3 -> M_sun / AU^3
    double* el;              // 6 per body: a, e, i, peri, node, mean
    double* w;               // planetesimal weights a^pl_mass_exp
    double* wsum;            // per system
    double* st;              // 8 per body: rx, ry, rz, vx, vy, vz, mass, radius
    double* dens;
    double* cd;
    int* id;
    int* type;
    red_var4_t* r_out;
    red_var4_t* v_out;
    red_param_t* p_out;
    red_body_metadata_t* md_out;
};

__global__ void __launch_bounds__(kPopBlock) k_pop_elements(const PopParams P)
{
    const int s = blockIdx.y;
    const red_disk_spec_t S = P.spec[s];
    const int n = 1 + (int)S.n_pp + (int)S.n_pl;
    const int k = blockIdx.x * kPopBlock + threadIdx.x;
    if (k >= n) return;
    const int i = P.off[s] + k;
    double* e6 = P.el + 6 * (size_t)i;
    if (k == 0) {   // the star
        for (int q = 0; q < 6; q++) e6[q] = 0.0;
        P.w[i] = 0.0;
        return;
    }
    double u[6];
    draws6(S.seed, (uint32_t)k, u);
    const bool pp = k <= (int)S.n_pp;
    double a;
    if (pp) {
        const int j = k - 1;
        if (S.pp_hill > 0.0) {   // equal masses spaced pp_hill mutual Hill radii apart
            const double h = cbrt(2.0 * S.pp_mass / (3.0 * S.m_star));
            const double f = (1.0 + 0.5 * S.pp_hill * h) / (1.0 - 0.5 * S.pp_hill * h);
            a = S.pp_a0 * pow(f, (double)j);
        } else {
            a = S.pp_a0 + j * S.pp_da;
        }
        P.w[i] = 0.0;
    } else {
        a = S.pl_a_log ? exp(log(S.pl_a_min) + u[0] * (log(S.pl_a_max) - log(S.pl_a_min)))
                       : S.pl_a_min + u[0] * (S.pl_a_max - S.pl_a_min);
        P.w[i] = pow(a, S.pl_mass_exp);
    }
    // Rayleigh sigma sqrt(-2 ln u) (distribution.cpp:105-109), uniform angles
    const double se = pp ? S.sigma_e_pp : S.sigma_e, si = pp ? S.sigma_i_pp : S.sigma_i;
    e6[0] = a;
    e6[1] = fmin(se * sqrt(-2.0 * log(u[1])), S.e_max);
    e6[2] = si * sqrt(-2.0 * log(u[2]));
    e6[3] = kTwoPi * u[3];
    e6[4] = kTwoPi * u[4];
    e6[5] = kTwoPi * u[5];
}

// Fixed-order block sum of v over the threads of one CTA (kPopBlock threads).
__device__ inline double block_sum(double v, double* sh)
{
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int o = kPopBlock / 2; o > 0; o >>= 1) {
        if (t < o) sh[t] += sh[t + o];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kPopBlock) k_pop_wsum(const PopParams P)
{
    __shared__ double sh[kPopBlock];
    const int s = blockIdx.x;
    const red_disk_spec_t S = P.spec[s];
    const int n = 1 + (int)S.n_pp + (int)S.n_pl;
    double acc = 0.0;
    for (int k = threadIdx.x; k < n; k += kPopBlock) acc += P.w[P.off[s] + k];
    const double tot = block_sum(acc, sh);
    if (threadIdx.x == 0) P.wsum[s] = tot;
}

// tools::kepler_equation_solver as calc_phase calls it (tools.cpp:715-755,
// 789-795; tolerance 1e-8): Newton from red's starting value.  For a mean
// anomaly above pi red's solver ends with E = (mean - pi) + pi, the mean
// anomaly itself rather than the solution; that is kept, so that the disks
// follow red's generator (the point is still on the orbit, at another phase).
__device__ inline double kepler_E(double ecc, double mean)
{
    if (ecc == 0.0 || mean == 0.0 || mean == kPi) return mean;
    const bool s = kPi < mean;
    if (s) mean -= kPi;
    double E = mean + ecc * sin(mean) / (1.0 - sin(mean + ecc) + sin(mean));
    for (int it = 0; it < 34; it++) {
        const double E1 = E - (E - ecc * sin(E) - mean) / (1.0 - ecc * cos(E));
        const double err = fabs(E1 - E);
        E = E1;
        if (!(err > 1.0e-8)) break;
    }
    if (s) E += (mean - E) + kPi;
    return E;
}

__global__ void __launch_bounds__(kPopBlock) k_pop_phase(const PopParams P)
{
    const int s = blockIdx.y;
    const red_disk_spec_t S = P.spec[s];
    const int n = 1 + (int)S.n_pp + (int)S.n_pl;
    const int k = blockIdx.x * kPopBlock + threadIdx.x;
    if (k >= n) return;
    const int i = P.off[s] + k;
    const double rho = S.density * P.rho_unit;
    double* o = P.st + 8 * (size_t)i;
    P.id[i] = k + 1;
    if (k == 0) {
        for (int q = 0; q < 6; q++) o[q] = 0.0;
        o[6] = S.m_star;
        o[7] = S.star_radius;
        P.dens[i] = S.star_radius == 0.0 ? 0.0 : S.m_star / (kFourPiOverThree * S.star_radius * S.star_radius *
                                                             S.star_radius);
        P.cd[i] = 0.0;
        P.type[i] = RED_BODY_STAR;
        return;
    }
    const bool pp = k <= (int)S.n_pp;
    const double* e6 = P.el + 6 * (size_t)i;
    const double m = pp ? S.pp_mass : S.pl_mass_total * P.w[i] / P.wsum[s];
    // tools::calc_phase (tools.cpp:789-828), mu = K^2 (m_0 + m)
    const double mu = kK2 * (S.m_star + m);
    const double a = e6[0], ecc = e6[1], inc = e6[2], peri = e6[3], node = e6[4];
    const double E = kepler_E(ecc, e6[5]);
    const double nu = 2.0 * atan(sqrt((1.0 + ecc) / (1.0 - ecc)) * tan(0.5 * E));
    const double p = a * (1.0 - ecc * ecc);
    const double rr = p / (1.0 + ecc * cos(nu));
    const double ksi = rr * cos(nu), eta = rr * sin(nu);
    const double vk = -sqrt(mu / p) * sin(nu), ve = sqrt(mu / p) * (ecc + cos(nu));
    const double cw = cos(peri), sw = sin(peri), cO = cos(node), sO = sin(node), ci = cos(inc), sinc = sin(inc);
    const double Px = cw * cO - sw * sO * ci, Py = cw * sO + sw * cO * ci, Pz = sw * sinc;
    const double Qx = -sw * cO - cw * sO * ci, Qy = -sw * sO + cw * cO * ci, Qz = cw * sinc;
    o[0] = ksi * Px + eta * Qx;
    o[1] = ksi * Py + eta * Qy;
    o[2] = ksi * Pz + eta * Qz;
    o[3] = vk * Px + ve * Qx;
    o[4] = vk * Py + ve * Qy;
    o[5] = vk * Pz + ve * Qz;
    o[6] = m;
    o[7] = cbrt(m / (kFourPiOverThree * rho));   // tools::calc_radius (tools.cpp:455-460)
    P.dens[i] = rho;
    P.cd[i] = pp ? 0.0 : S.cd;
    P.type[i] = pp ? RED_BODY_PROTOPLANET : RED_BODY_PLANETESIMAL;
}

// tools::transform_to_bc (tools.cpp:413-434), then velocities in AU per code
// time unit (red.cuda.initial/main.cu:1666-1670), written as red's records.
__global__ void __launch_bounds__(kPopBlock) k_pop_bary(const PopParams P)
{
    __shared__ double sh[kPopBlock];
    const int s = blockIdx.x;
    const red_disk_spec_t S = P.spec[s];
    const int n = 1 + (int)S.n_pp + (int)S.n_pl;
    const int i0 = P.off[s];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int k = threadIdx.x; k < n; k += kPopBlock) {
        const double* o = P.st + 8 * (size_t)(i0 + k);
        acc[0] += o[6];
        for (int q = 0; q < 6; q++) acc[1 + q] += o[6] * o[q];
    }
    double tot[7];
    for (int q = 0; q < 7; q++) tot[q] = block_sum(acc[q], sh);
    for (int k = threadIdx.x; k < n; k += kPopBlock) {
        const int i = i0 + k;
        const double* o = P.st + 8 * (size_t)i;
        red_var4_t r, v;
        r.x = o[0] - tot[1] / tot[0];
        r.y = o[1] - tot[2] / tot[0];
        r.z = o[2] - tot[3] / tot[0];
        r.w = 0.0;
        v.x = (o[3] - tot[4] / tot[0]) / kK;
        v.y = (o[4] - tot[5] / tot[0]) / kK;
        v.z = (o[5] - tot[6] / tot[0]) / kK;
        v.w = 0.0;
        P.r_out[i] = r;
        P.v_out[i] = v;
        red_param_t pp;
        pp.mass = o[6];
        pp.radius = o[7];
        pp.density = P.dens[i];
        pp.cd = P.cd[i];
        P.p_out[i] = pp;
        red_body_metadata_t md;
        memset(&md, 0, sizeof(md));
        md.id = P.id[i];
        md.body_type = P.type[i];
        P.md_out[i] = md;
    }
}

}  // namespace
}  // namespace redgb

int redgb_set_error(int code, const char* msg);

int red_populate_disks(const red_disk_spec_t* specs, uint32_t n_systems, int32_t device, uint32_t* playing,
                       red_var4_t* r, red_var4_t* v, red_param_t* p, red_body_metadata_t* md)
{
    using namespace redgb;
    if (!specs || n_systems == 0 || n_systems > 65535 || !playing || !r || !v || !p || !md)
        return redgb_set_error(RED_ERR_ARG, "red_populate_disks: bad argument");
    std::vector<int> off(n_systems);
    size_t total = 0;
    int nmax = 0;
    for (uint32_t s = 0; s < n_systems; s++) {
        const red_disk_spec_t& S = specs[s];
        const double h = std::cbrt(2.0 * S.pp_mass / (3.0 * S.m_star));
        if (!(S.m_star > 0.0) || !(S.density > 0.0) || S.pp_mass < 0.0 || S.pl_mass_total < 0.0 ||
            !(S.e_max >= 0.0 && S.e_max < 1.0) || (S.n_pl > 0 && !(S.pl_a_max >= S.pl_a_min && S.pl_a_min > 0.0)) ||
            (S.n_pp > 0 && !(S.pp_a0 > 0.0)) || (S.pp_hill > 0.0 && !(0.5 * S.pp_hill * h < 1.0)) ||
            (uint64_t)S.n_pp + S.n_pl > (1u << 28))
            return redgb_set_error(RED_ERR_ARG, "red_populate_disks: bad disk specification");
        off[s] = (int)total;
        const int n = 1 + (int)S.n_pp + (int)S.n_pl;
        total += (size_t)n;
        nmax = std::max(nmax, n);
        uint32_t* pl = playing + 7 * (size_t)s;
        for (int q = 0; q < 7; q++) pl[q] = 0;
        pl[RED_BODY_STAR] = 1;
        pl[RED_BODY_PROTOPLANET] = S.n_pp;
        pl[RED_BODY_PLANETESIMAL] = S.n_pl;
    }
    if (total > (size_t)1 << 30) return redgb_set_error(RED_ERR_ARG, "red_populate_disks: too many bodies");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return redgb_set_error(RED_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return redgb_set_error(RED_ERR_ARG, "red_populate_disks: bad device");
    cudaError_t e = cudaSetDevice(device);
    // device buffers: specs, offsets, 6 + 1 + 8 + 2 doubles and 2 ints per body, the records
    red_disk_spec_t* d_spec = nullptr;
    int* d_off = nullptr;
    double* d_buf = nullptr;
    double* d_wsum = nullptr;
    int* d_int = nullptr;
    red_var4_t* d_r = nullptr;
    red_var4_t* d_v = nullptr;
    red_param_t* d_p = nullptr;
    red_body_metadata_t* d_md = nullptr;
    auto ok = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
        return e == cudaSuccess;
    };
    ok(cudaMalloc(&d_spec, n_systems * sizeof(red_disk_spec_t)));
    ok(cudaMalloc(&d_off, n_systems * sizeof(int)));
    ok(cudaMalloc(&d_buf, total * 17 * sizeof(double)));
    ok(cudaMalloc(&d_wsum, n_systems * sizeof(double)));
    ok(cudaMalloc(&d_int, total * 2 * sizeof(int)));
    ok(cudaMalloc(&d_r, total * sizeof(red_var4_t)));
    ok(cudaMalloc(&d_v, total * sizeof(red_var4_t)));
    ok(cudaMalloc(&d_p, total * sizeof(red_param_t)));
    ok(cudaMalloc(&d_md, total * sizeof(red_body_metadata_t)));
    if (e == cudaSuccess) {
        ok(cudaMemcpy(d_spec, specs, n_systems * sizeof(red_disk_spec_t), cudaMemcpyHostToDevice));
        ok(cudaMemcpy(d_off, off.data(), n_systems * sizeof(int), cudaMemcpyHostToDevice));
    }
    if (e == cudaSuccess) {
        PopParams P;
        memset(&P, 0, sizeof(P));
        P.spec = d_spec;
        P.off = d_off;
        P.n_sys = (int)n_systems;
        // g/cm^3 -> M_sun/AU^3 (red_constants.h:142-143, 162-167, 184)
        const double cm_au = 1.0e-2 / 1.495978707e11;
        P.rho_unit = (1.0 / (1.0e3 * 1.98911e30)) / (cm_au * cm_au * cm_au);
        P.el = d_buf;
        P.w = d_buf + 6 * total;
        P.st = d_buf + 7 * total;
        P.dens = d_buf + 15 * total;
        P.cd = d_buf + 16 * total;
        P.wsum = d_wsum;
        P.id = d_int;
        P.type = d_int + total;
        P.r_out = d_r;
        P.v_out = d_v;
        P.p_out = d_p;
        P.md_out = d_md;
        const dim3 grid((unsigned)((nmax + kPopBlock - 1) / kPopBlock), n_systems);
        k_pop_elements<<<grid, kPopBlock>>>(P);
        k_pop_wsum<<<n_systems, kPopBlock>>>(P);
        k_pop_phase<<<grid, kPopBlock>>>(P);
        k_pop_bary<<<n_systems, kPopBlock>>>(P);
        ok(cudaGetLastError());
        ok(cudaMemcpy(r, d_r, total * sizeof(red_var4_t), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(v, d_v, total * sizeof(red_var4_t), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(p, d_p, total * sizeof(red_param_t), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(md, d_md, total * sizeof(red_body_metadata_t), cudaMemcpyDeviceToHost));
    }
    cudaFree(d_spec);
    cudaFree(d_off);
    cudaFree(d_buf);
    cudaFree(d_wsum);
    cudaFree(d_int);
    cudaFree(d_r);
    cudaFree(d_v);
    cudaFree(d_p);
    cudaFree(d_md);
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof(msg), "red_populate_disks: CUDA error %s", cudaGetErrorString(e));
        return redgb_set_error(RED_ERR_CUDA, msg);
    }
    return RED_OK;
}
