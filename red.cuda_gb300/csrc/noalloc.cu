// noalloc.cu -- gravity (+ drag) of one system without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while another component
// owns the device memory through its own pool, real-time loops that must not
// enter the allocator, or hosts whose GPU memory is fully reserved up front.
// red_calc_accel_noalloc serves them: the caller passes device buffers for
// the inputs and the output, and every temporary the stage kernel needs (the
// FP32 copies of the positions, the launch plan, the per-chunk partial sums
// and their completion counters) lives in one file-scope __device__ array of
// kScratchBytes.  Every GPU that loads the library holds that array until the
// process exits.
//
// All calls share the array and it keeps the contents of the last call: the
// counters that must start at zero are cleared on every call, and two calls
// that overlap on the GPU (different streams, or different host threads)
// race on it -- callers must order them.
//
// The first call on a device looks up the device address of the array with
// cudaGetSymbolAddress (with that device current).  The entry point writes no
// constant memory: a standalone evaluation reads no integrator coefficients,
// and the tableau that live simulations loaded stays as it is.
//
// Every system of at most RED_NOALLOC_MAX_BODIES bodies fits: when the
// allocating path's launch plan (sources split into chunks whose partial sums
// need scratch records) does not fit the array, the plan falls back to one
// CTA per sink tile over the whole source list, which needs no partial
// records and at most n / 16 + 3 work items.
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "redgb.h"

using namespace redgb;

namespace {

constexpr size_t kScratchBytes = 4u << 20;          // 4 MiB
constexpr size_t kMaxItems = 8192;                   // stage-kernel CTAs
constexpr size_t kMaxTiles = 4096;                   // chunked sink tiles

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {nullptr};

// Layout of the scratch array (offsets in bytes, 256-aligned).
constexpr size_t kOffSys = 0;
constexpr size_t kOffSinfo = 128;
constexpr size_t kOffItems = 256;
constexpr size_t kOffTiles = kOffItems + kMaxItems * sizeof(GravItem);
constexpr size_t kOffPos = ((kOffTiles + kMaxTiles * sizeof(unsigned) + 255) / 256) * 256;
// then pos_hi (N float4), pos_lo (N float4), partial records (3 doubles each)

__global__ void k_noalloc_prep(int n, const double* r, const double* mass, const double* radius, const int* id,
                               float4* hi, float4* lo)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // the same double-single split as the allocating path (k_prep)
    redgb::write_pos(hi, lo, i, r[3 * i], r[3 * i + 1], r[3 * i + 2], id[i] >= 0 ? mass[i] : 0.0,
                     radius ? radius[i] : 0.0);
}

}  // namespace

// sets the message returned by red_last_error (sim.cu)
int redgb_set_error(int code, const char* msg);

namespace {
int fail(int code, const char* msg) { return redgb_set_error(code, msg); }
static_assert(sizeof(DevSys) <= 128 && sizeof(SysInfo) <= 128, "scratch header layout");
}  // namespace

extern "C" int red_calc_accel_noalloc(const red_accel_args_t* a)
{
    if (!a) return fail(RED_ERR_ARG, "null argument");
    uint32_t n = 0;
    for (int k = 0; k < 7; k++) n += a->playing[k];
    if (n == 0) return fail(RED_ERR_ARG, "no bodies");
    if (n > RED_NOALLOC_MAX_BODIES)
        return fail(RED_ERR_ARG, "red_calc_accel_noalloc: more bodies than RED_NOALLOC_MAX_BODIES");
    if (!a->r || !a->mass || !a->id || !a->accel) return fail(RED_ERR_ARG, "null device buffer");
    if (a->gas_disk == 2) return fail(RED_ERR_NOT_IMPLEMENTED, "the FARGO gas disk cannot be constructed in red either");
    if (a->gas_disk < 0 || a->gas_disk > 2) return fail(RED_ERR_ARG, "bad gas_disk");
    if (a->gas_disk && (!a->v || !a->radius || !a->density || !a->cd))
        return fail(RED_ERR_ARG, "gas drag needs v, radius, density and cd");
    if (a->precision < 0 || a->precision > 3) return fail(RED_ERR_ARG, "bad precision");
    if (a->device < 0 || a->device >= kMaxDevices) return fail(RED_ERR_ARG, "bad device");
    const size_t pos_bytes = (size_t)n * sizeof(float4);
    const size_t off_part = ((kOffPos + 2 * pos_bytes + 255) / 256) * 256;

    // the launch plan, on the host
    SysInfo si;
    memset(&si, 0, sizeof(si));
    si.off = 0;
    si.n = (int)n;
    si.n_star = (int)a->playing[0];
    si.n_SI = (int)(a->playing[0] + a->playing[1] + a->playing[2] + a->playing[3]);
    si.n_massive = si.n_SI + (int)(a->playing[4] + a->playing[5]);
    si.n_err = si.n_massive;
    std::vector<GravItem> items;
    size_t part = 0;
    int tiles = 0;
    auto fits = [&]() {
        return items.size() <= kMaxItems && (size_t)tiles <= kMaxTiles &&
               off_part + part * 3 * sizeof(double) <= kScratchBytes;
    };
    long long short_ctas = 0;
    const int tiles_all = count_sink_tiles(si, a->precision, 32, &short_ctas);
    plan_gravity_items(si, 0, a->precision, 0, 32, tiles_all, short_ctas <= 6 * 152, nullptr, items, part, tiles);
    if (!fits()) {
        // unchunked: one chunk spans all n bodies, and 8 lanes per sink group
        // give tiles of >= 16 sinks, so no partial records and few items
        items.clear();
        part = 0;
        tiles = 0;
        plan_gravity_items(si, 0, a->precision, (int)n, 8, tiles_all, false, nullptr, items, part, tiles);
    }
    if (!fits()) return fail(RED_ERR_ARG, "red_calc_accel_noalloc: the launch plan does not fit the scratch array");

    // the caller's current device is restored on every return path
    int prev_device = -1;
    if (cudaGetDevice(&prev_device) != cudaSuccess) return fail(RED_ERR_CUDA, "cudaGetDevice failed");
    struct DeviceGuard {
        int prev;
        ~DeviceGuard() { cudaSetDevice(prev); }
    } guard{prev_device};
    if (cudaSetDevice(a->device) != cudaSuccess) return fail(RED_ERR_CUDA, "cudaSetDevice failed");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_dev[a->device]) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess || !p) return fail(RED_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
            g_scratch_dev[a->device] = p;
        }
        base = g_scratch_dev[a->device];
    }
    cudaStream_t st = (cudaStream_t)a->stream;
    unsigned char* b = (unsigned char*)base;
    DevSys* d_sys = (DevSys*)(b + kOffSys);
    SysInfo* d_sinfo = (SysInfo*)(b + kOffSinfo);
    GravItem* d_items = (GravItem*)(b + kOffItems);
    unsigned* d_tiles = (unsigned*)(b + kOffTiles);
    float4* d_hi = (float4*)(b + kOffPos);
    float4* d_lo = (float4*)(b + kOffPos + pos_bytes);
    double* d_part = (double*)(b + off_part);

    if (cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(GravItem), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemsetAsync(d_tiles, 0, kMaxTiles * sizeof(unsigned), st) != cudaSuccess ||
        cudaMemsetAsync(d_sys, 0, sizeof(DevSys), st) != cudaSuccess ||
        cudaMemcpyAsync(d_sinfo, &si, sizeof(SysInfo), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return fail(RED_ERR_CUDA, "red_calc_accel_noalloc: staging the plan failed");
    k_noalloc_prep<<<(n + 255) / 256, 256, 0, st>>>((int)n, a->r, a->mass, a->radius, a->id, d_hi, d_lo);

    StageParams P;
    memset(&P, 0, sizeof(P));
    P.stage = 0;
    P.next = -1;
    P.scheme = SCHEME_RKF78;
    P.standalone = 1;
    P.t_standalone = a->t;
    P.items = d_items;
    P.sinfo = d_sinfo;
    P.sys = d_sys;
    P.pos_hi_in = d_hi;
    P.pos_lo_in = d_lo;
    P.r_in = a->r;
    P.y_r = a->r;
    P.y_v = a->v;
    P.Kr[0] = const_cast<double*>(a->v);
    P.Kv[0] = a->accel;
    P.mass = a->mass;
    P.radius = a->radius;
    P.density = a->density;
    P.cd = a->cd;
    P.id = a->id;
    P.partial = d_part;
    P.tile_cnt = d_tiles;
    P.gas.enabled = a->gas_disk == 1;
    for (int k = 0; k < 2; k++) {
        P.gas.rho[k] = a->gas.rho[k];
        P.gas.sch[k] = a->gas.sch[k];
        P.gas.eta[k] = a->gas.eta[k];
    }
    P.gas.t0 = a->gas.t0;
    P.gas.t1 = a->gas.t1;
    P.gas.e_folding_time = a->gas.e_folding_time;
    P.gas.gas_decrease = a->gas.gas_decrease;
    launch_stage(P, (int)items.size(), a->precision, st);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(RED_ERR_CUDA, cudaGetErrorString(e));
    return RED_OK;
}
