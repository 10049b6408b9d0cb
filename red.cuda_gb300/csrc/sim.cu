// sim.cu -- host layer of libredgb: the C++ mirror of red's pp_disk +
// integrator seam (src/red.cuda/pp_disk.h, integrator.h) over the device
// kernels, and the C ABI declared in include/redgb.h.
//
// One handle integrates n independent systems.  Device memory holds every
// system's bodies back to back; a host-built plan lists the CTAs of each
// kernel (gravity tiles, per-body segments, collision tile pairs).  One try of
// the integrator is a fixed sequence of launches, captured once into a CUDA
// graph and replayed; all accept / reject decisions are taken on the device,
// so the host only waits when it wants to look at the results or to handle
// collision / ejection events.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "redgb_dev.cuh"
#include "proposer.cuh"
#include "redgb.h"

using namespace redgb;

namespace {

thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

struct CudaError {
    cudaError_t e;
    const char* what;
    int line;
};

#define CK(call)                                                 \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) throw CudaError{e_, #call, __LINE__}; \
    } while (0)

struct ArgError {
    int code;
    std::string msg;
};

// Tableaux of red's integrators.
Tableau make_tableau()
{
    Tableau t;
    memset(&t, 0, sizeof(t));
    // int_rungekutta8.cu:26-48
    const double c[13] = {0.0, 2.0 / 27.0, 1.0 / 9.0, 1.0 / 6.0, 5.0 / 12.0, 1.0 / 2.0, 5.0 / 6.0,
                          1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0, 1.0, 0.0, 1.0};
    const double a[79] = {
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
        2383.0 / 4100.0, 0.0, 0.0, -341.0 / 164.0, 4496.0 / 1025.0, -301.0 / 82.0, 2133.0 / 4100.0, 45.0 / 82.0,
        45.0 / 164.0, 18.0 / 41.0,
        3.0 / 205.0, 0.0, 0.0, 0.0, 0.0, -6.0 / 41.0, -3.0 / 205.0, -3.0 / 41.0, 3.0 / 41.0, 6.0 / 41.0, 0.0,
        -1777.0 / 4100.0, 0.0, 0.0, -341.0 / 164.0, 4496.0 / 1025.0, -289.0 / 82.0, 2193.0 / 4100.0, 51.0 / 82.0,
        33.0 / 164.0, 12.0 / 41.0, 0.0, 1.0};
    const double b[11] = {41.0 / 840.0, 0.0, 0.0, 0.0, 0.0, 34.0 / 105.0, 9.0 / 35.0, 9.0 / 35.0,
                          9.0 / 280.0, 9.0 / 280.0, 41.0 / 840.0};
    memcpy(t.c, c, sizeof(c));
    memcpy(t.a, a, sizeof(a));
    memcpy(t.b, b, sizeof(b));
    // nonzero coefficients of each stage row in the order red's stage kernels
    // add them (rk8_kernel::calc_ytemp_for_f1..f12, int_rungekutta8.cu:80-246)
    for (int r = 1; r < 13; r++) {
        const int off = 1 + r * (r - 1) / 2;
        int n = 0;
        for (int q = 0; q < r; q++)
            if (a[off + q] != 0.0) t.src[r][n++] = q;
        t.nnz[r] = n;
    }
    // int_rungekutta4.cu:26-31
    const double lam = 1.0 / 10.0;
    const double a4[8] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0, 1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    const double b4[5] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0 - lam, lam};
    const double c4[5] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0, 1.0};
    memcpy(t.a4, a4, sizeof(a4));
    memcpy(t.b4, b4, sizeof(b4));
    memcpy(t.c4, c4, sizeof(c4));
    // int_rungekutta2.cu:12-14
    const double a2[2] = {0.0, 1.0 / 2.0}, b2[2] = {0.0, 1.0}, c2[2] = {0.0, 1.0 / 2.0};
    memcpy(t.a2, a2, sizeof(a2));
    memcpy(t.b2, b2, sizeof(b2));
    memcpy(t.c2, c2, sizeof(c2));
    return t;
}

template <class T> T* dalloc(size_t n)
{
    void* p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMalloc(&p, n * sizeof(T)));
    CK(cudaMemset(p, 0, n * sizeof(T)));
    return (T*)p;
}

struct SysHost {
    uint32_t off = 0, cap = 0, n = 0;
    uint32_t playing[7] = {0}, inactive[7] = {0}, removed[7] = {0};
    uint32_t n_collision[3] = {0}, n_ejection[3] = {0}, n_hit_centrum[3] = {0}, n_event[3] = {0};
    uint32_t n_SI() const { return playing[0] + playing[1] + playing[2] + playing[3]; }
    uint32_t n_NSI() const { return playing[4] + playing[5]; }
    uint32_t n_NI() const { return playing[6]; }
    uint32_t n_massive() const { return n_SI() + n_NSI(); }
    uint32_t n_active() const
    {
        uint32_t s = 0;
        for (int i = 0; i < 7; i++) s += playing[i] - inactive[i];
        return s;
    }
};

// Per-system host copy of the state, used by the event handling.
struct HostState {
    std::vector<red_var4_t> r, v;
    std::vector<red_param_t> p;
    std::vector<red_body_metadata_t> md;
};

}  // namespace


namespace redgb {
// CTAs of the stage kernel for one system: sink tiles of the SI, NSI and NI
// classes (red_type.h:670-692), each split into source chunks; appends to
// items and advances the partial-record and tile counters.
// The gravity classes of one system: sinks [s0, s1) against sources [j0, j1)
// (body indices relative to the system), red's interaction bounds
// (red_type.h:670-692); the FP32 modes take the stars out of the sources (their
// term is added in FP64 by the epilogue).
struct GravClass { int cls, s0, s1, j0, j1; };
static void gravity_classes(const SysInfo& si, int mode, GravClass out[3])
{
    const bool fp32 = (mode == MODE_MIXED || mode == MODE_FP32);
    const int src_start = fp32 ? si.n_star : 0;
    out[0] = {CLS_SI, 0, si.n_SI, src_start, si.n_massive};
    out[1] = {CLS_NSI, si.n_SI, si.n_massive, src_start, si.n_SI};
    out[2] = {CLS_NI, si.n_massive, si.n, src_start, si.n_massive};
}

// Threads per sink group and sinks per group of one class: a power of two in
// [4, 32] lanes.  Many sinks against more than 64 sources in the FP32 modes: 8
// lanes serving 2 sinks each (each source read feeds two interactions).  A
// short source list (a planetesimal class against a few protoplanets): 4 lanes
// per sink, two butterfly rounds instead of three.  Few sinks: more lanes, the
// more the longer the source list.
static void class_shape(int mode, int nsink_all, int nsrc, int lanes_cap, int& lanes, int& spt)
{
    const bool fp32 = (mode == MODE_MIXED || mode == MODE_FP32);
    lanes = 4;
    spt = 1;
    if (mode == MODE_FP64_EXACT) return;
    if (fp32 && nsink_all >= 32 && lanes_cap >= 8 && nsrc > 64) {
        lanes = 8;
        spt = 2;
        return;
    }
    while (lanes < 32 && lanes < lanes_cap && (2 * lanes * nsink_all <= kTile || 256 * 2 * lanes <= nsrc)) lanes *= 2;
}

int count_sink_tiles(const SysInfo& si, int mode, int lanes_cap, long long* short_ctas)
{
    GravClass cls[3];
    gravity_classes(si, mode, cls);
    int n = 0;
    for (const GravClass& q : cls) {
        const int nsink_all = q.s1 - q.s0;
        if (nsink_all <= 0) continue;
        const int nsrc = std::max(0, q.j1 - q.j0);
        int lanes, spt;
        class_shape(mode, nsink_all, nsrc, lanes_cap, lanes, spt);
        const int tile_sinks = kTile / lanes * spt;
        const int nt = (nsink_all + tile_sinks - 1) / tile_sinks;
        n += nt;
        if (short_ctas) *short_ctas += (long long)nt * std::max(1, (nsrc + 2 * kTile - 1) / (2 * kTile));
    }
    return n;
}

void plan_gravity_items(const SysInfo& si, int s, int mode, int chunk_override, int lanes_cap, int tiles_all,
                        bool short_chunks, const double* star_mass, std::vector<GravItem>& items, size_t& part,
                        int& tiles)
{
    // Two regimes.  When chunks of two source tiles keep the whole launch within
    // one wave (short_chunks), every chunk is two tiles, staged in shared memory
    // at once: the launch is as short as its slowest CTA.  Otherwise the launch
    // should hold several waves of CTAs (6 resident on each of GB300's 152 SMs);
    // tiles_all counts the sink tiles of every system in it.
    const int kTargetCtas = 8 * 6 * 152;
    GravClass cls[3];
    gravity_classes(si, mode, cls);
    for (const GravClass& q : cls) {
        const int nsink_all = q.s1 - q.s0;
        if (nsink_all <= 0) continue;
        const int nsrc = std::max(0, q.j1 - q.j0);
        int lanes, spt;
        class_shape(mode, nsink_all, nsrc, lanes_cap, lanes, spt);
        const int tile_sinks = kTile / lanes * spt;
        const int ntile = (nsink_all + tile_sinks - 1) / tile_sinks;
        for (int t = 0; t < ntile; t++) {
            const int s0 = q.s0 + t * tile_sinks;
            const int nsink = std::min(tile_sinks, q.s1 - s0);
            int chunk = std::max(nsrc, 1);
            if (mode != MODE_FP64_EXACT) {
                if (chunk_override > 0) {
                    chunk = chunk_override;
                } else {
                    // chunks of 2 to 4 source tiles, fewer when the launch already has enough
                    // CTAs; no CTA's gravity then runs much longer than the others'
                    const int want = std::max(1, kTargetCtas / std::max(1, tiles_all));
                    const int c = (nsrc + want - 1) / want;
                    chunk = short_chunks ? 2 * kTile
                                         : std::min(std::max((c + kTile / 2) / kTile * kTile, 2 * kTile), 16 * kTile);
                }
                // the reducing CTA reads at most 2 batches of records per thread
                const int nel = 3 * nsink;
                const int max_chunks = 2 * kBatchRecords * std::max(1, kTile / nel);
                if ((nsrc + chunk - 1) / chunk > max_chunks)
                    chunk = ((nsrc + max_chunks - 1) / max_chunks + kTile - 1) / kTile * kTile;
                chunk = std::max(chunk, 1);
            }
            const int nchunk = std::max(1, (nsrc + chunk - 1) / chunk);
            GravItem g;
            memset(&g, 0, sizeof(g));
            g.sys = (int)s;
            g.sink0 = si.off + s0;
            g.nsink = nsink;
            g.nchunk = nchunk;
            g.lanes = lanes;
            g.spt = spt;
            g.cls = q.cls;
            g.soff = si.off;
            g.nstar = si.n_star;
            g.nerr = si.n_err;
            if (star_mass && si.n_star > 0) {
                g.mstar_set = 1;
                g.mstar_hi = (float)*star_mass;
                g.mstar_lo = (float)(*star_mass - (double)g.mstar_hi);
            }
            g.tile = nchunk > 1 ? tiles++ : -1;
            g.part_off = (int)part;
            if (nchunk > 1) part += (size_t)nchunk * nsink;
            for (int c = 0; c < nchunk; c++) {
                g.chunk = c;
                g.src0 = si.off + q.j0 + c * chunk;
                g.src1 = si.off + std::min(q.j1, q.j0 + (c + 1) * chunk);
                if (nsrc == 0) g.src0 = g.src1 = si.off;
                items.push_back(g);
            }
        }
    }
}
// Items of a cluster launch (FP32 modes): a tile whose source list is longer
// than two tiles becomes kClusterChunks chunks, the CTAs of one cluster; the
// others are single items.  max_chunk is the longest chunk.
static void plan_cluster_items(const SysInfo& si, int s, int mode, int lanes_cap, const double* star_mass,
                               std::vector<GravItem>& groups, std::vector<GravItem>& singles, int& max_chunk)
{
    GravClass cls[3];
    gravity_classes(si, mode, cls);
    for (const GravClass& q : cls) {
        const int nsink_all = q.s1 - q.s0;
        if (nsink_all <= 0) continue;
        const int nsrc = std::max(0, q.j1 - q.j0);
        int lanes, spt;
        class_shape(mode, nsink_all, nsrc, lanes_cap, lanes, spt);
        const int tile_sinks = kTile / lanes * spt;
        const int ntile = (nsink_all + tile_sinks - 1) / tile_sinks;
        const int nchunk = nsrc > 2 * kTile ? kClusterChunks : 1;
        const int chunk = std::max(1, (nsrc + nchunk - 1) / nchunk);
        max_chunk = std::max(max_chunk, chunk);
        for (int t = 0; t < ntile; t++) {
            const int s0 = q.s0 + t * tile_sinks;
            GravItem g;
            memset(&g, 0, sizeof(g));
            g.sys = s;
            g.sink0 = si.off + s0;
            g.nsink = std::min(tile_sinks, q.s1 - s0);
            g.nchunk = nchunk;
            g.lanes = lanes;
            g.spt = spt;
            g.cls = q.cls;
            g.soff = si.off;
            g.nstar = si.n_star;
            g.nerr = si.n_err;
            if (star_mass && si.n_star > 0) {
                g.mstar_set = 1;
                g.mstar_hi = (float)*star_mass;
                g.mstar_lo = (float)(*star_mass - (double)g.mstar_hi);
            }
            g.tile = -1;
            for (int c = 0; c < nchunk; c++) {
                g.chunk = c;
                g.src0 = si.off + q.j0 + std::min(nsrc, c * chunk);
                g.src1 = si.off + q.j0 + std::min(nsrc, (c + 1) * chunk);
                (nchunk > 1 ? groups : singles).push_back(g);
            }
        }
    }
}

// The layout a cluster launch relies on: every chunked tile fills exactly one
// cluster (chunks 0 .. kClusterChunks - 1 at ranks 0 .. kClusterChunks - 1, one
// system), the other clusters hold single items (or padding, nsink = 0), and
// the item count is a multiple of the cluster size.
static void check_cluster_layout(const std::vector<GravItem>& items)
{
    if (items.size() % kClusterChunks) throw ArgError{RED_ERR_ARG, "internal error, cluster plan: ragged item count"};
    for (size_t b = 0; b < items.size(); b += kClusterChunks) {
        const GravItem& g0 = items[b];
        for (int r = 0; r < kClusterChunks; r++) {
            const GravItem& g = items[b + r];
            if (g0.nchunk > 1) {
                if (g.nchunk != kClusterChunks || g.chunk != r || g.sys != g0.sys || g.sink0 != g0.sink0 ||
                    g.nsink <= 0)
                    throw ArgError{RED_ERR_ARG, "internal error, cluster plan: a chunk group is split"};
            } else if (g.nchunk != 1) {
                throw ArgError{RED_ERR_ARG, "internal error, cluster plan: a chunk group is misaligned"};
            }
        }
    }
}
}  // namespace redgb

struct red_sim {
    red_config_t cfg;
    int mode = MODE_MIXED;
    int scheme = SCHEME_RKF78;
    int n_stage = 13;
    int order = 7;
    double lambda = 41.0 / 840.0;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint32_t n_sys = 0;
    uint32_t n_cap = 0;
    std::vector<SysHost> sh;
    std::vector<double> mig_stop_at;   // kept on the host (not used by the path)
    std::vector<int> mig_type;

    // device state
    double *y_r = nullptr, *y_v = nullptr, *tr[2] = {nullptr, nullptr};
    double* Kr[kMaxStages] = {nullptr};
    double* Kv[kMaxStages] = {nullptr};
    float4 *pos_hi[2] = {nullptr, nullptr}, *pos_lo[2] = {nullptr, nullptr};
    double *mass = nullptr, *radius = nullptr, *density = nullptr, *cd = nullptr;
    int *id = nullptr, *btype = nullptr;
    double* partial = nullptr;
    size_t partial_cap = 0;
    unsigned int* tile_cnt = nullptr;
    size_t tile_cap = 0;
    DevSys* d_sys = nullptr;
    SysInfo* d_sinfo = nullptr;
    GravItem* d_items = nullptr;
    // the work items of each system, items[item_begin[s], item_begin[s + 1]) (plans
    // without clusters), and a device list of the items of the systems that a
    // red_step retry still integrates
    std::vector<size_t> item_begin;
    std::vector<GravItem> sparse_items;
    GravItem* d_sparse_items = nullptr;
    size_t sparse_cap = 0;
    const GravItem* items_override = nullptr;   // enqueue_try: launch these instead of the plan's items
    int n_items_override = 0;
    size_t items_cap = 0;
    Segment* d_segs = nullptr;
    size_t segs_cap = 0;
    Segment* d_fsegs = nullptr;
    size_t fsegs_cap = 0;
    PairItem* d_pairs = nullptr;
    size_t pairs_cap = 0;
    GridInfo* d_grid = nullptr;
    int* d_head = nullptr;
    size_t head_cap = 0;
    size_t table_size = 0;
    int* d_next = nullptr;
    int4* d_cell = nullptr;
    bool use_grid = false;
    DevEvent* d_events = nullptr;
    unsigned int* d_nev = nullptr;
    uint32_t ev_cap = 0;
    double* d_u = nullptr;
    // host transfers: device records (k_pack_state layout) and a pinned host copy
    char* d_xfer = nullptr;
    char* h_xfer = nullptr;
    DevSys* h_sys = nullptr;   // page-locked copy of the system records (read_sys)
    size_t xfer_cap = 0;
    void ensure_xfer(size_t bytes);
    void pack_range_to_host(size_t o, size_t n);   // bodies [o, o + n) into h_xfer
    std::vector<double> grid_rmax;   // largest small-body radius the collision grid was planned for
    std::vector<double> star_mass;   // the first star's effective mass the plan was made with
    // learned step proposer (proposer.cu) and the feature log it is trained on
    bool prop_on = false, log_on = false;
    __nv_bfloat16* d_mlp_w = nullptr;
    MlpNorm mlp_norm{};
    double prop_safety = 1.0, prop_lo = 0.5, prop_hi = 2.0;
    float* d_fpart = nullptr;
    size_t fpart_cap = 0;
    int* d_seg0 = nullptr;
    int* d_nseg = nullptr;
    float* d_feat_prev = nullptr;
    int* d_has_prev = nullptr;
    float* d_log = nullptr;
    unsigned int* d_log_n = nullptr;
    uint32_t log_cap = 0;
    void enqueue_proposer(int& n);

    // plan
    std::vector<GravItem> items;
    std::vector<Segment> segs;
    std::vector<Segment> fsegs;   // kFinishBodies bodies each (k_finish)
    std::vector<PairItem> pairs;
    std::vector<SysInfo> sinfo;
    std::vector<GridInfo> grid;
    int chunk_override = 0;     // sources per chunk chosen by the autotuner (0 = heuristic)
    bool use_cluster = false;   // the plan's items are laid out for a cluster launch
    int lanes_cap = 32;         // upper bound on threads per sink (autotuner)
    bool allow_cluster = true;  // the planner may lay chunk groups out as clusters (autotuner)
    bool allow_packed = true;   // plans of 2-sink tiles may take the packed-pair instance (autotuner)
    bool use_packed = false;    // the plan's stage launches take the packed-pair instance
    red_plan_info_t plan_info{};   // what the last red_autotune measured

    cudaGraphExec_t graph = nullptr;
    int launches_per_try = 0;
    uint64_t launches = 0;
    std::vector<red_event_t> event_log;

    ~red_sim();
    void create(const red_config_t* c, uint32_t n_systems, const uint32_t* playing, const red_var4_t* r,
                const red_var4_t* v, const red_param_t* p, const red_body_metadata_t* md, const double* t0,
                const double* dt0);
    void build_plan();
    StageParams stage_params(int s, bool standalone);
    void enqueue_try(std::vector<int>* kinds = nullptr, std::vector<cudaEvent_t>* evs = nullptr);
    void capture();
    void launch_tries(uint32_t n);
    bool launch_sparse_try(const std::vector<DevSys>& ds);
    void read_sys(std::vector<DevSys>& out);
    void write_sys(const std::vector<DevSys>& in);
    void prep_positions();
    void get_host_state(uint32_t s, HostState& hs);
    void put_host_state(uint32_t s, const HostState& hs);
    void fill_event(uint32_t s, const HostState& hs, const DevEvent& de, double t, red_event_t& ev);
    uint32_t collect_events(std::vector<DevEvent>& ev);
    int handle_events(red_event_t* out, uint32_t cap, uint32_t* n_out);
    void rebuild_system(uint32_t s);
    void invalidate() { if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; } }
    bool has_ejhc() const
    {
        return cfg.threshold[RED_THRESHOLD_EJECTION_DISTANCE] > 0.0 ||
               cfg.threshold[RED_THRESHOLD_HIT_CENTRUM_DISTANCE] > 0.0;
    }
    bool ejhc_initial_done = false;
    // Ejection / hit-centrum check of every system's current state, halting the
    // systems with events (run_simulation checks before every step, main.cu:499-523).
    void ejhc_all()
    {
        EjhcParams E;
        memset(&E, 0, sizeof(E));
        E.segs = d_segs; E.sinfo = d_sinfo; E.sys = d_sys; E.y_r = y_r; E.id = id; E.btype = btype;
        E.ejection = cfg.threshold[RED_THRESHOLD_EJECTION_DISTANCE];
        E.hit_centrum = cfg.threshold[RED_THRESHOLD_HIT_CENTRUM_DISTANCE];
        E.only_accepted = 0;
        E.mark = 1;
        E.events = d_events; E.n_events = d_nev; E.capacity = ev_cap;
        launch_ejhc(E, (int)segs.size(), stream);
        CK(cudaGetLastError());
        launches++;
    }
    void fill_coll(CollParams& Q)
    {
        memset(&Q, 0, sizeof(Q));
        Q.items = d_pairs; Q.segs = d_segs; Q.grid = d_grid; Q.head = d_head; Q.next = d_next; Q.cell = d_cell;
        Q.sinfo = d_sinfo; Q.sys = d_sys;
        Q.pos_hi = pos_hi[0]; Q.pos_lo = pos_lo[0]; Q.y_r = y_r;
        Q.radius = radius; Q.mass = mass; Q.id = id;
        Q.factor = cfg.threshold[RED_THRESHOLD_RADII_ENHANCE_FACTOR];
        Q.events = d_events; Q.n_events = d_nev; Q.capacity = ev_cap;
    }
    uint64_t interactions_per_eval() const;
};

red_sim::~red_sim()
{
    invalidate();
    cudaFree(y_r); cudaFree(y_v); cudaFree(tr[0]); cudaFree(tr[1]);
    for (int s = 1; s < kMaxStages; s++) cudaFree(Kr[s]);
    for (int s = 0; s < kMaxStages; s++) cudaFree(Kv[s]);
    for (int k = 0; k < 2; k++) { cudaFree(pos_hi[k]); cudaFree(pos_lo[k]); }
    cudaFree(mass); cudaFree(radius); cudaFree(density); cudaFree(cd); cudaFree(id); cudaFree(btype);
    cudaFree(partial); cudaFree(tile_cnt); cudaFree(d_sys); cudaFree(d_sinfo); cudaFree(d_items); cudaFree(d_sparse_items);
    cudaFree(d_segs); cudaFree(d_pairs); cudaFree(d_events); cudaFree(d_nev); cudaFree(d_u);
    cudaFree(d_grid); cudaFree(d_head); cudaFree(d_next); cudaFree(d_cell); cudaFree(d_fsegs);
    cudaFree(d_xfer);
    if (h_xfer) cudaFreeHost(h_xfer);
    if (h_sys) cudaFreeHost(h_sys);
    cudaFree(d_mlp_w); cudaFree(d_fpart); cudaFree(d_seg0); cudaFree(d_nseg); cudaFree(d_feat_prev);
    cudaFree(d_has_prev); cudaFree(d_log); cudaFree(d_log_n);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

uint64_t red_sim::interactions_per_eval() const
{
    uint64_t n = 0;
    for (const SysHost& h : sh) {
        const uint64_t nsi = h.n_SI(), nnsi = h.n_NSI(), nm = h.n_massive(), nni = h.n_NI();
        n += (nsi ? nsi * (nm - 1) : 0) + nnsi * nsi + nni * nm;
    }
    return n;
}

void red_sim::create(const red_config_t* c, uint32_t n_systems, const uint32_t* playing, const red_var4_t* r,
                     const red_var4_t* v, const red_param_t* p, const red_body_metadata_t* md, const double* t0,
                     const double* dt0)
{
    cfg = *c;
    if (n_systems == 0) throw ArgError{RED_ERR_ARG, "n_systems must be positive"};
    if (cfg.integrator == RED_INTEGRATOR_RUNGEKUTTA4) {
        scheme = SCHEME_RK4;
        n_stage = cfg.adaptive ? 5 : 4;
        order = 4;
        lambda = 1.0 / 10.0;
    } else if (cfg.integrator == RED_INTEGRATOR_RUNGEKUTTAFEHLBERG78) {
        scheme = SCHEME_RKF78;
        n_stage = cfg.adaptive ? 13 : 11;
        order = 7;
        lambda = 41.0 / 840.0;
    } else if (cfg.integrator == RED_INTEGRATOR_EULER || cfg.integrator == RED_INTEGRATOR_RUNGEKUTTA2) {
        // euler / rungekutta2 (int_euler.cu:42-47, int_rungekutta2.cu:39-44) are
        // fixed-step only: their constructors pass adaptive = false
        const bool eu = cfg.integrator == RED_INTEGRATOR_EULER;
        scheme = eu ? SCHEME_EULER : SCHEME_RK2;
        n_stage = eu ? 1 : 2;
        order = eu ? 1 : 2;
        lambda = 0.0;
        cfg.adaptive = 0;
    } else {
        throw ArgError{RED_ERR_NOT_IMPLEMENTED, "integrator not on this path (EULER, RUNGEKUTTA2, RUNGEKUTTA4, "
                                                "RUNGEKUTTAFEHLBERG78 are)"};
    }
    if (cfg.precision < 0 || cfg.precision > 3) throw ArgError{RED_ERR_ARG, "bad precision"};
    // GAS_DISK_MODEL_FARGO: red's fargo_gas_disk constructor throws
    // (transform_time "not yet implemented", fargo_gas_disk.cu:35, 259-261)
    if (cfg.gas_disk == 2)
        throw ArgError{RED_ERR_NOT_IMPLEMENTED, "the FARGO gas disk cannot be constructed in red either"};
    if (cfg.gas_disk < 0 || cfg.gas_disk > 2) throw ArgError{RED_ERR_ARG, "bad gas_disk"};
    mode = cfg.precision;
    // FP64_EXACT combines the stages in red's order without FMA; the other
    // modes combine with FMA
    if (cfg.stage_exact && mode != MODE_FP64_EXACT)
        throw ArgError{RED_ERR_ARG, "stage_exact requires precision RED_PREC_FP64_EXACT"};
    if (mode == MODE_FP64_EXACT) cfg.stage_exact = 1;
    device = cfg.device;
    n_sys = n_systems;
    sh.resize(n_sys);
    uint32_t off = 0;
    for (uint32_t s = 0; s < n_sys; s++) {
        SysHost& h = sh[s];
        h.off = off;
        uint32_t n = 0;
        for (int k = 0; k < 7; k++) {
            h.playing[k] = playing[7 * s + k];
            n += h.playing[k];
        }
        if (n == 0) throw ArgError{RED_ERR_ARG, "system without bodies"};
        h.n = h.cap = n;
        // red requires bodies sorted by type (the bounds of red_type.h:670-700 assume it)
        uint32_t k = 0;
        for (int ty = 0; ty < 7; ty++) {
            for (uint32_t q = 0; q < h.playing[ty]; q++, k++) {
                if (md[off + k].body_type != ty)
                    throw ArgError{RED_ERR_ARG, "bodies must be sorted by type matching the counts (system " +
                                                    std::to_string(s) + ", body " + std::to_string(k) + ": type " +
                                                    std::to_string(md[off + k].body_type) + ", expected " +
                                                    std::to_string(ty) + ")"};
            }
        }
        off += n;
    }
    n_cap = off;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw ArgError{RED_ERR_NO_DEVICE, "no CUDA device"};
    CK(cudaSetDevice(device));
    if (cfg.stream) {
        stream = (cudaStream_t)cfg.stream;
    } else {
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
    }
    const size_t N = n_cap;
    // host -> packed xyz
    std::vector<double> hr(3 * N), hv(3 * N), hm(N), hR(N), hd(N), hc(N);
    std::vector<int> hid(N), hty(N);
    mig_stop_at.resize(N);
    mig_type.resize(N);
    for (size_t i = 0; i < N; i++) {
        hr[3 * i] = r[i].x; hr[3 * i + 1] = r[i].y; hr[3 * i + 2] = r[i].z;
        hv[3 * i] = v[i].x; hv[3 * i + 1] = v[i].y; hv[3 * i + 2] = v[i].z;
        hm[i] = p[i].mass; hR[i] = p[i].radius; hd[i] = p[i].density; hc[i] = p[i].cd;
        hid[i] = md[i].id; hty[i] = md[i].body_type;
        mig_stop_at[i] = md[i].mig_stop_at;
        mig_type[i] = md[i].mig_type;
    }
    y_r = dalloc<double>(3 * N);
    y_v = dalloc<double>(3 * N);
    tr[0] = dalloc<double>(3 * N);
    tr[1] = dalloc<double>(3 * N);
    Kr[0] = y_v;
    for (int s = 1; s < n_stage; s++) Kr[s] = dalloc<double>(3 * N);
    for (int s = 0; s < n_stage; s++) Kv[s] = dalloc<double>(3 * N);
    for (int k = 0; k < 2; k++) {
        pos_hi[k] = dalloc<float4>(N);
        pos_lo[k] = dalloc<float4>(N);
    }
    mass = dalloc<double>(N); radius = dalloc<double>(N); density = dalloc<double>(N); cd = dalloc<double>(N);
    id = dalloc<int>(N); btype = dalloc<int>(N);
    d_u = dalloc<double>(N);
    d_next = dalloc<int>(N);
    d_cell = dalloc<int4>(N);
    d_grid = dalloc<GridInfo>(n_sys);
    CK(cudaMemcpy(y_r, hr.data(), 3 * N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(y_v, hv.data(), 3 * N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(mass, hm.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(radius, hR.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(density, hd.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(cd, hc.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(id, hid.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(btype, hty.data(), N * sizeof(int), cudaMemcpyHostToDevice));

    std::vector<DevSys> ds(n_sys);
    for (uint32_t s = 0; s < n_sys; s++) {
        memset(&ds[s], 0, sizeof(DevSys));
        ds[s].t = ds[s].t_start = t0 ? t0[s] : 0.0;
        const double dt = dt0 ? dt0[s] : 0.0;
        ds[s].dt_try = ds[s].dt_next = dt;
        ds[s].active = sh[s].n_active() > 1 ? 1 : 0;   // run_simulation's loop bound (main.cu:471)
        ds[s].quota = -1;
    }
    d_sys = dalloc<DevSys>(n_sys);
    d_sinfo = dalloc<SysInfo>(n_sys);
    CK(cudaMemcpy(d_sys, ds.data(), n_sys * sizeof(DevSys), cudaMemcpyHostToDevice));
    ev_cap = cfg.event_capacity ? cfg.event_capacity : std::max<uint32_t>(1024u, n_cap);
    d_events = dalloc<DevEvent>(ev_cap);
    d_nev = dalloc<unsigned int>(1);
    Tableau tb = make_tableau();
    set_tableau(tb, stream);
    build_plan();
    prep_positions();
    CK(cudaStreamSynchronize(stream));
}

void red_sim::build_plan()
{
    invalidate();
    items.clear();
    segs.clear();
    fsegs.clear();
    pairs.clear();
    sinfo.assign(n_sys, SysInfo{});
    grid.assign(n_sys, GridInfo{});
    grid_rmax.assign(n_sys, 0.0);
    size_t table = 0;
    // radii, for the cell size of the collision grid
    std::vector<double> h_radius(n_cap), h_mass(n_cap);
    std::vector<int> h_id(n_cap);
    CK(cudaMemcpy(h_radius.data(), radius, n_cap * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h_mass.data(), mass, n_cap * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h_id.data(), id, n_cap * sizeof(int), cudaMemcpyDeviceToHost));
    star_mass.assign(n_sys, 0.0);
    size_t part = 0;
    int tiles = 0;
    for (uint32_t s = 0; s < n_sys; s++) {
        const SysHost& h = sh[s];
        SysInfo& si = sinfo[s];
        si.off = (int)h.off;
        si.n = (int)h.n;
        si.n_star = (int)h.playing[0];
        si.n_SI = (int)h.n_SI();
        si.n_massive = (int)h.n_massive();
        si.n_err = cfg.error_check_for_tp ? si.n : si.n_massive;
    }
    int tiles_all = 0;
    long long short_ctas = 0;
    for (uint32_t s = 0; s < n_sys; s++) tiles_all += count_sink_tiles(sinfo[s], mode, lanes_cap, &short_ctas);
    const bool short_chunks = short_ctas <= 6 * 152;   // one wave at 6 CTAs per SM
    item_begin.assign(n_sys + 1, 0);
    for (uint32_t s = 0; s < n_sys; s++) {
        const SysHost& h = sh[s];
        SysInfo& si = sinfo[s];
        (void)h;
        item_begin[s] = items.size();
        star_mass[s] = si.n_star > 0 && h_id[si.off] >= 0 ? h_mass[si.off] : 0.0;
        plan_gravity_items(si, (int)s, mode, chunk_override, lanes_cap, tiles_all, short_chunks, &star_mass[s], items,
                           part, tiles);
        for (int b = 0; b < si.n; b += kSegment) segs.push_back(Segment{(int)s, si.off + b, si.off + std::min(si.n, b + kSegment), 0});
        for (int b = 0; b < si.n; b += kFinishBodies)
            fsegs.push_back(Segment{(int)s, si.off + b, si.off + std::min(si.n, b + kFinishBodies), 0});
        // collision check: the SI bodies (large radii) by brute force against
        // every later body, the rest through the spatial hash grid
        const int T = (si.n + kTile - 1) / kTile;
        const int TI = (si.n_SI + kTile - 1) / kTile;
        for (int I = 0; I < TI; I++)
            for (int J = I; J < T; J++)
                pairs.push_back(PairItem{(int)s, si.off + I * kTile, si.off + J * kTile, si.off + si.n_SI});
        GridInfo& g = grid[s];
        memset(&g, 0, sizeof(g));
        const int n_small = si.n - si.n_SI;
        double rmax = 0.0;
        for (int k = si.n_SI; k < si.n; k++) rmax = std::max(rmax, h_radius[si.off + k]);
        grid_rmax[s] = rmax;
        const double factor = cfg.threshold[RED_THRESHOLD_RADII_ENHANCE_FACTOR];
        if (n_small > 1 && rmax > 0.0 && factor > 0.0) {
            // cell edge >= the largest collision distance f (R_i + R_j) of two small
            // bodies, widened a little so that rounding in x / h cannot split a pair
            // by more than one cell
            const double h = 2.0 * factor * rmax * (1.0 + 1.0e-6) + 1.0e-300;
            size_t m = 1024;
            while (m < 4 * (size_t)n_small) m <<= 1;
            g.inv_h = 1.0 / h;
            g.toff = (int)table;
            g.mask = (int)(m - 1);
            g.enabled = 1;
            table += m;
        }
    }
    // Cluster plan (FP32 modes): when every tile's chunks fit the two-tile
    // shared-memory buffer as kClusterChunks chunks and the whole launch, laid
    // out in clusters, is resident at once, a tile's chunks run as the CTAs of
    // one thread-block cluster and reduce through distributed shared memory:
    // no GPU-scope fence or global partial records on the critical path.
    // REDGB_CLUSTER=0 keeps the global reduction.
    if (!item_begin.empty()) item_begin[n_sys] = items.size();
    use_cluster = false;
    const char* cenv = getenv("REDGB_CLUSTER");
    if ((mode == MODE_MIXED || mode == MODE_FP32) && chunk_override == 0 && allow_cluster &&
        !(cenv && cenv[0] == '0')) {
        std::vector<GravItem> groups, singles;
        int max_chunk = 0;
        for (uint32_t s = 0; s < n_sys; s++)
            plan_cluster_items(sinfo[s], (int)s, mode, lanes_cap, &star_mass[s], groups, singles, max_chunk);
        if (!groups.empty() && max_chunk <= 2 * kTile) {
            GravItem pad;   // padding: nsink = 0, the CTA returns at once
            memset(&pad, 0, sizeof(pad));
            pad.nchunk = 1;
            pad.tile = -1;
            std::vector<GravItem> cl(groups);
            cl.insert(cl.end(), singles.begin(), singles.end());
            while (cl.size() % kClusterChunks) cl.push_back(pad);
            if ((int)(cl.size() / kClusterChunks) <= stage_active_clusters(mode)) {
                check_cluster_layout(cl);
                items.swap(cl);
                use_cluster = true;
                item_begin.clear();   // the cluster layout interleaves the systems' items
            }
        }
    }
    // A plan of many waves whose tiles mostly hold 2 sinks per thread (FP32
    // modes) takes the packed-pair stage instance.
    // REDGB_PACKED=0 keeps the scalar instance.
    use_packed = false;
    const char* penv = getenv("REDGB_PACKED");
    if ((mode == MODE_MIXED || mode == MODE_FP32) && allow_packed && !(penv && penv[0] == '0') && !use_cluster &&
        items.size() > (size_t)6 * 152) {
        size_t n2 = 0;
        for (const GravItem& g : items) n2 += g.spt == 2 ? 1 : 0;
        use_packed = 2 * n2 >= items.size();
    }
    auto upload = [&](auto& vec, auto*& dptr, size_t& cap) {
        using T = typename std::remove_reference<decltype(vec)>::type::value_type;
        if (vec.size() > cap) {
            cudaFree(dptr);
            cap = vec.size();
            dptr = dalloc<T>(cap);
        }
        if (!vec.empty()) CK(cudaMemcpy(dptr, vec.data(), vec.size() * sizeof(T), cudaMemcpyHostToDevice));
    };
    upload(items, d_items, items_cap);
    upload(segs, d_segs, segs_cap);
    upload(fsegs, d_fsegs, fsegs_cap);
    upload(pairs, d_pairs, pairs_cap);
    {
        // each system's range of per-body segments, for the proposer's features;
        // allocated here because the try is captured into a graph
        std::vector<int> seg0(n_sys, 0), nseg(n_sys, 0);
        for (size_t k = segs.size(); k-- > 0;) {
            seg0[segs[k].sys] = (int)k;
            nseg[segs[k].sys]++;
        }
        if (!d_seg0) {
            d_seg0 = dalloc<int>(n_sys);
            d_nseg = dalloc<int>(n_sys);
        }
        CK(cudaMemcpy(d_seg0, seg0.data(), n_sys * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_nseg, nseg.data(), n_sys * sizeof(int), cudaMemcpyHostToDevice));
        if (segs.size() > fpart_cap) {
            cudaFree(d_fpart);
            d_fpart = dalloc<float>(segs.size() * kNPart);
            fpart_cap = segs.size();
        }
    }
    CK(cudaMemcpy(d_sinfo, sinfo.data(), n_sys * sizeof(SysInfo), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_grid, grid.data(), n_sys * sizeof(GridInfo), cudaMemcpyHostToDevice));
    table_size = table;
    use_grid = table > 0;
    if (table > head_cap) {
        cudaFree(d_head);
        head_cap = table;
        d_head = dalloc<int>(head_cap);
    }
    if (part > partial_cap) {
        cudaFree(partial);
        partial_cap = part;
        partial = dalloc<double>(3 * part);
    }
    // The one-wave stage instance polls its partial records and needs their
    // slots empty; the many-wave instances leave theirs filled.
    fill_records_empty(partial, 3 * part, stream);
    if ((size_t)tiles > tile_cap) {
        cudaFree(tile_cnt);
        tile_cap = tiles;
        tile_cnt = dalloc<unsigned int>(tile_cap);
    }
}

StageParams red_sim::stage_params(int s, bool standalone)
{
    StageParams P;
    memset(&P, 0, sizeof(P));
    P.stage = s;
    P.scheme = scheme;
    P.standalone = standalone ? 1 : 0;
    if (!standalone) {
        if (scheme == SCHEME_RKF78) {
            P.next = (s + 1 < n_stage) ? s + 1 : -1;
        } else {
            P.next = (s + 1 < n_stage) ? s + 1 : -1;
            P.ynp1_to_out = (cfg.adaptive && s == 3) ? 1 : 0;
        }
        P.err_after = (cfg.adaptive && s == n_stage - 1) ? 1 : 0;
    } else {
        P.next = -1;
    }
    P.items = d_items;
    P.sinfo = d_sinfo;
    P.sys = d_sys;
    P.pos_hi_in = pos_hi[s & 1];
    P.pos_lo_in = pos_lo[s & 1];
    P.pos_hi_out = pos_hi[(s + 1) & 1];
    P.pos_lo_out = pos_lo[(s + 1) & 1];
    P.r_in = (s == 0) ? y_r : tr[s & 1];
    P.r_out = tr[(s + 1) & 1];
    P.y_r = y_r;
    P.y_v = y_v;
    for (int k = 0; k < kMaxStages; k++) {
        P.Kr[k] = Kr[k];
        P.Kv[k] = Kv[k];
    }
    P.mass = mass; P.radius = radius; P.density = density; P.cd = cd; P.id = id;
    P.partial = partial;
    P.tile_cnt = tile_cnt;
    P.cluster = use_cluster ? 1 : 0;
    P.one_wave = items.size() <= (size_t)6 * 152 ? 1 : 0;
    P.packed = use_packed ? 1 : 0;
    P.gas.enabled = cfg.gas_disk == 1;
    for (int k = 0; k < 2; k++) {
        P.gas.rho[k] = cfg.gas.rho[k];
        P.gas.sch[k] = cfg.gas.sch[k];
        P.gas.eta[k] = cfg.gas.eta[k];
    }
    P.gas.t0 = cfg.gas.t0;
    P.gas.t1 = cfg.gas.t1;
    P.gas.e_folding_time = cfg.gas.e_folding_time;
    P.gas.gas_decrease = cfg.gas.gas_decrease;
    return P;
}

void red_sim::prep_positions()
{
    launch_prep(d_segs, (int)segs.size(), d_sinfo, d_sys, y_r, mass, radius, id, pos_hi[0], pos_lo[0], pos_hi[1],
                pos_lo[1], 1, stream);
    CK(cudaGetLastError());
    launches++;
}

// One try of the integrator.  With kinds / evs set (profiling), an event is
// recorded after every launch and the kernel kind noted: 0 stage, 1 control,
// 2 finish, 3 collision, 4 ejection / hit-centrum, 5 learned proposer.
void red_sim::enqueue_try(std::vector<int>* kinds, std::vector<cudaEvent_t>* evs)
{
    int n = 0;
    auto mark = [&](int kind) {
        if (!kinds) return;
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        CK(cudaEventRecord(e, stream));
        kinds->push_back(kind);
        evs->push_back(e);
    };
    mark(-1);
    const bool coll = cfg.threshold[RED_THRESHOLD_RADII_ENHANCE_FACTOR] > 0.0;
    const bool hash = coll && use_grid && !segs.empty();   // the small bodies' spatial hash
    for (int s = 0; s < n_stage; s++) {
        StageParams P = stage_params(s, false);
        if (s == 0 && hash) {
            P.head = d_head;
            P.head_n = (long long)table_size;
        }
        if (items_override) P.items = items_override;
        launch_stage(P, items_override ? n_items_override : (int)items.size(), mode, stream);
        mark(0);
        n++;
    }
    ControlParams C;
    memset(&C, 0, sizeof(C));
    C.n_sys = (int)n_sys;
    C.scheme = scheme;
    C.adaptive = cfg.adaptive;
    C.order = order;
    C.keep_dt = (scheme == SCHEME_EULER || scheme == SCHEME_RK2) ? 1 : 0;
    C.exact = mode == MODE_FP64_EXACT ? 1 : 0;
    C.tolerance = cfg.tolerance;
    C.lambda = lambda;
    C.output_interval = cfg.output_interval;
    C.length = cfg.length;
    C.sys = d_sys;
    launch_control(C, stream);
    mark(1);
    n++;
    FinishParams F;
    memset(&F, 0, sizeof(F));
    F.scheme = scheme;
    F.adaptive = cfg.adaptive;
    F.commit_from_stage4 = (scheme == SCHEME_RK4 && cfg.adaptive) ? 1 : 0;
    F.stage_exact = cfg.stage_exact;
    F.segs = d_fsegs;
    F.sinfo = d_sinfo;
    F.sys = d_sys;
    F.y_r = y_r;
    F.y_v = y_v;
    for (int k = 0; k < kMaxStages; k++) {
        F.Kr[k] = Kr[k];
        F.Kv[k] = Kv[k];
    }
    F.t_r0 = tr[0];
    F.mass = mass;
    F.radius = radius;
    F.id = id;
    F.pos_hi0 = pos_hi[0];
    F.pos_lo0 = pos_lo[0];
    if (hash) {
        F.head = d_head;
        F.next = d_next;
        F.cell = d_cell;
        F.grid = d_grid;
    }
    launch_finish(F, (int)fsegs.size(), stream);
    mark(2);
    n++;
    if (prop_on || log_on) {
        enqueue_proposer(n);
        mark(5);
    }
    if (coll) {
        CollParams Q;
        memset(&Q, 0, sizeof(Q));
        fill_coll(Q);
        Q.only_accepted = 1;
        Q.mark = 1;
        launch_collide(Q, (int)pairs.size(), (int)segs.size(), hash, stream);
        mark(3);
        n += (!pairs.empty() || hash) ? 1 : 0;
    }
    if (cfg.threshold[RED_THRESHOLD_EJECTION_DISTANCE] > 0.0 || cfg.threshold[RED_THRESHOLD_HIT_CENTRUM_DISTANCE] > 0.0) {
        EjhcParams E;
        memset(&E, 0, sizeof(E));
        E.segs = d_segs; E.sinfo = d_sinfo; E.sys = d_sys; E.y_r = y_r; E.id = id; E.btype = btype;
        E.ejection = cfg.threshold[RED_THRESHOLD_EJECTION_DISTANCE];
        E.hit_centrum = cfg.threshold[RED_THRESHOLD_HIT_CENTRUM_DISTANCE];
        E.only_accepted = 1;
        E.mark = 1;
        E.events = d_events; E.n_events = d_nev; E.capacity = ev_cap;
        launch_ejhc(E, (int)segs.size(), stream);
        mark(4);
        n++;
    }
    launches_per_try = n;
}

// Features of the systems that accepted a try, the log record and the MLP's
// proposal for their next step (proposer.cu).
void red_sim::enqueue_proposer(int& n)
{
    FeatParams Fe;
    memset(&Fe, 0, sizeof(Fe));
    Fe.segs = d_segs; Fe.sinfo = d_sinfo; Fe.sys = d_sys; Fe.pos = pos_hi[0]; Fe.y_v = y_v; Fe.acc = Kv[0];
    Fe.mass = mass; Fe.id = id; Fe.part = d_fpart;
    launch_features(Fe, (int)segs.size(), stream);
    ProposeParams Pp;
    memset(&Pp, 0, sizeof(Pp));
    Pp.n_sys = (int)n_sys; Pp.sys = d_sys; Pp.seg0 = d_seg0; Pp.nseg = d_nseg; Pp.part = d_fpart;
    Pp.tolerance = cfg.tolerance > 0.0 ? cfg.tolerance : 1.0;
    Pp.propose = prop_on && cfg.adaptive ? 1 : 0;
    Pp.w = d_mlp_w; Pp.norm = mlp_norm;
    Pp.safety = prop_safety; Pp.ratio_lo = prop_lo; Pp.ratio_hi = prop_hi; Pp.output_interval = cfg.output_interval;
    Pp.log = log_on ? 1 : 0;
    Pp.feat_prev = d_feat_prev; Pp.has_prev = d_has_prev; Pp.log_buf = d_log; Pp.log_n = d_log_n; Pp.log_cap = log_cap;
    launch_propose(Pp, stream);
    CK(cudaGetLastError());
    n += 2;
}

void red_sim::capture()
{
    if (graph) return;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    // the kernels of the try are chained by programmatic dependent launch
    // (REDGB_PDL=0 captures plain launches)
    const char* pe = getenv("REDGB_PDL");
    set_pdl(!(pe && pe[0] == '0'));
    try {
        enqueue_try();
    } catch (...) {
        set_pdl(false);
        cudaStreamEndCapture(stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    set_pdl(false);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (e != cudaSuccess) throw CudaError{e, "cudaStreamEndCapture", __LINE__};
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        graph = nullptr;
        throw CudaError{e, "cudaGraphInstantiate", __LINE__};
    }
}

void red_sim::launch_tries(uint32_t n)
{
    if (has_ejhc() && !ejhc_initial_done) {
        ejhc_initial_done = true;
        ejhc_all();
    }
    capture();
    for (uint32_t k = 0; k < n; k++) {
        CK(cudaGraphLaunch(graph, stream));
        launches += (uint64_t)launches_per_try;
    }
}

// One try over the work items of the systems a red_step still waits for (ds:
// the system records after the previous try), launched directly instead of
// the try's graph, whose stage launches would start a CTA for every item of
// every system.  The same kernels and item records as the graph's, so the
// results are the same bits.  Returns false (nothing launched) when the plan
// interleaves the systems' items (cluster layout) or half the items or more
// are still pending.
bool red_sim::launch_sparse_try(const std::vector<DevSys>& ds)
{
    if (item_begin.size() != n_sys + 1 || !graph || ds.size() != n_sys) return false;
    sparse_items.clear();
    for (uint32_t s = 0; s < n_sys; s++) {
        const DevSys& d = ds[s];
        if (d.active && !d.halted && d.quota != 0)
            sparse_items.insert(sparse_items.end(), items.begin() + item_begin[s], items.begin() + item_begin[s + 1]);
    }
    if (sparse_items.empty() || 2 * sparse_items.size() > items.size()) return false;
    if (sparse_items.size() > sparse_cap) {
        cudaFree(d_sparse_items);
        d_sparse_items = nullptr;
        sparse_cap = 0;
        d_sparse_items = dalloc<GravItem>(sparse_items.size());
        sparse_cap = sparse_items.size();
    }
    // a pageable source: the copy has read it when the call returns
    CK(cudaMemcpyAsync(d_sparse_items, sparse_items.data(), sparse_items.size() * sizeof(GravItem),
                       cudaMemcpyHostToDevice, stream));
    const char* pe = getenv("REDGB_PDL");
    set_pdl(!(pe && pe[0] == '0'));
    items_override = d_sparse_items;
    n_items_override = (int)sparse_items.size();
    try {
        enqueue_try();
    } catch (...) {
        items_override = nullptr;
        set_pdl(false);
        throw;
    }
    items_override = nullptr;
    set_pdl(false);
    launches += (uint64_t)launches_per_try;
    return true;
}

void red_sim::read_sys(std::vector<DevSys>& out)
{
    // through page-locked memory: a DMA copy with no staging by the driver
    // (red_step reads the records after every try)
    if (!h_sys) CK(cudaMallocHost(&h_sys, n_sys * sizeof(DevSys)));
    CK(cudaMemcpyAsync(h_sys, d_sys, n_sys * sizeof(DevSys), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    out.assign(h_sys, h_sys + n_sys);
}

void red_sim::write_sys(const std::vector<DevSys>& in)
{
    CK(cudaMemcpyAsync(d_sys, in.data(), n_sys * sizeof(DevSys), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
}

void red_sim::get_host_state(uint32_t s, HostState& hs)
{
    const SysHost& h = sh[s];
    const size_t n = h.n, o = h.off;
    std::vector<double> hr(3 * n), hv(3 * n), hm(n), hR(n), hd(n), hc(n);
    std::vector<int> hid(n), hty(n);
    CK(cudaMemcpyAsync(hr.data(), y_r + 3 * o, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hv.data(), y_v + 3 * o, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hm.data(), mass + o, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hR.data(), radius + o, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hd.data(), density + o, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hc.data(), cd + o, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hid.data(), id + o, n * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(hty.data(), btype + o, n * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    hs.r.resize(n); hs.v.resize(n); hs.p.resize(n); hs.md.resize(n);
    for (size_t i = 0; i < n; i++) {
        hs.r[i] = red_var4_t{hr[3 * i], hr[3 * i + 1], hr[3 * i + 2], 0.0};
        hs.v[i] = red_var4_t{hv[3 * i], hv[3 * i + 1], hv[3 * i + 2], 0.0};
        hs.p[i] = red_param_t{hm[i], hR[i], hd[i], hc[i]};
        hs.md[i].id = hid[i];
        hs.md[i].body_type = hty[i];
        hs.md[i].mig_type = mig_type[o + i];
        hs.md[i].mig_stop_at = mig_stop_at[o + i];
    }
}

void red_sim::put_host_state(uint32_t s, const HostState& hs)
{
    const SysHost& h = sh[s];
    const size_t n = hs.r.size(), o = h.off;
    std::vector<double> hr(3 * n), hv(3 * n), hm(n), hR(n), hd(n), hc(n);
    std::vector<int> hid(n), hty(n);
    for (size_t i = 0; i < n; i++) {
        hr[3 * i] = hs.r[i].x; hr[3 * i + 1] = hs.r[i].y; hr[3 * i + 2] = hs.r[i].z;
        hv[3 * i] = hs.v[i].x; hv[3 * i + 1] = hs.v[i].y; hv[3 * i + 2] = hs.v[i].z;
        hm[i] = hs.p[i].mass; hR[i] = hs.p[i].radius; hd[i] = hs.p[i].density; hc[i] = hs.p[i].cd;
        hid[i] = hs.md[i].id; hty[i] = hs.md[i].body_type;
        mig_type[o + i] = hs.md[i].mig_type;
        mig_stop_at[o + i] = hs.md[i].mig_stop_at;
    }
    CK(cudaMemcpyAsync(y_r + 3 * o, hr.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(y_v + 3 * o, hv.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(mass + o, hm.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(radius + o, hR.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(density + o, hd.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(cd + o, hc.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(id + o, hid.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(btype + o, hty.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
}

// pp_disk_utility::store_event_data (pp_disk.cu:190-253) from a device record.
void red_sim::fill_event(uint32_t s, const HostState& hs, const DevEvent& de, double t, red_event_t& ev)
{
    const uint32_t o = sh[s].off;
    memset(&ev, 0, sizeof(ev));
    const uint32_t i1 = (uint32_t)de.surv - o, i2 = (uint32_t)de.merg - o;
    ev.event_name = de.name;
    ev.t = t;
    ev.d = de.d;
    ev.id0 = hs.md[0].id;
    ev.id1 = hs.md[i1].id;
    ev.id2 = hs.md[i2].id;
    ev.idx0 = 0;
    ev.idx1 = i1;
    ev.idx2 = i2;
    ev.r0 = hs.r[0]; ev.v0 = hs.v[0];
    ev.r1 = hs.r[i1]; ev.v1 = hs.v[i1];
    ev.r2 = hs.r[i2]; ev.v2 = hs.v[i2];
    ev.p0 = hs.p[0];
    if (de.name == RED_EVENT_EJECTION) {
        ev.p1 = hs.p[i1];
        ev.p2 = hs.p[i2];
        ev.rs = ev.r1;
        ev.vs = ev.v1;
        ev.ps = ev.p1;
    }
}

uint32_t red_sim::collect_events(std::vector<DevEvent>& ev)
{
    unsigned int n = 0;
    CK(cudaMemcpyAsync(&n, d_nev, sizeof(unsigned int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    const uint32_t m = std::min<uint32_t>(n, ev_cap);
    ev.resize(m);
    if (m) CK(cudaMemcpyAsync(ev.data(), d_events, m * sizeof(DevEvent), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemsetAsync(d_nev, 0, sizeof(unsigned int), stream));
    CK(cudaStreamSynchronize(stream));
    // red's CPU loop order: system, then i, then j
    std::sort(ev.begin(), ev.end(), [](const DevEvent& a, const DevEvent& b) {
        if (a.sys != b.sys) return a.sys < b.sys;
        if (a.i != b.i) return a.i < b.i;
        if (a.j != b.j) return a.j < b.j;
        return a.name > b.name;   // ejection before hit-centrum for the same body (pp_disk.cu:306-315)
    });
    return n;
}

namespace {
// tools.cpp:455-507
double calc_radius(double m, double density)
{
    static const double four_pi_over_three = 4.188790204786391;
    return pow(1.0 / four_pi_over_three * m / density, 1.0 / 3.0);
}

void merge_pair(red_event_t& c, HostState& hs)
{
    const uint32_t s = c.idx1, m = c.idx2;
    c.p1 = hs.p[s];
    c.p2 = hs.p[m];
    const double m1 = c.p1.mass, m2 = c.p2.mass;
    const double M = m1 + m2;
    c.rs.x = (m1 * c.r1.x + m2 * c.r2.x) / M;
    c.rs.y = (m1 * c.r1.y + m2 * c.r2.y) / M;
    c.rs.z = (m1 * c.r1.z + m2 * c.r2.z) / M;
    c.vs.x = (m1 * c.v1.x + m2 * c.v2.x) / M;
    c.vs.y = (m1 * c.v1.y + m2 * c.v2.y) / M;
    c.vs.z = (m1 * c.v1.z + m2 * c.v2.z) / M;
    hs.r[s] = c.rs;
    hs.v[s] = c.vs;
    const double volume = 4.188790204786391 * (c.p1.radius * c.p1.radius * c.p1.radius +
                                               c.p2.radius * c.p2.radius * c.p2.radius);
    c.ps.mass = c.p1.mass + c.p2.mass;
    c.ps.density = c.ps.mass / volume;
    c.ps.radius = calc_radius(c.ps.mass, c.ps.density);
    c.ps.cd = c.p1.cd;
    hs.p[s] = c.ps;
}

void bump(uint32_t* counter, uint32_t* n_event)
{
    for (int i = 0; i < 3; i++) {
        counter[i]++;
        n_event[i]++;
    }
}
}  // namespace

// Handles the events of the halted systems (pp_disk::handle_collision,
// pp_disk.cu:1220-1248; handle_ejection_hit_centrum, 1290-1326; rebuild after
// 16 events, main.cu:582-607).
int red_sim::handle_events(red_event_t* out, uint32_t cap, uint32_t* n_out)
{
    std::vector<DevSys> ds;
    read_sys(ds);
    std::vector<DevEvent> ev;
    const uint32_t n_raw = collect_events(ev);
    uint32_t n_written = 0;
    int rc = RED_OK;
    if (n_raw > ev_cap) rc = set_error(RED_ERR_EVENT_OVERFLOW, "%u events exceed the event buffer (%u)", n_raw, ev_cap);
    bool changed = false;
    size_t k = 0;
    for (uint32_t s = 0; s < n_sys; s++) {
        size_t k1 = k;
        while (k1 < ev.size() && ev[k1].sys == (int)s) k1++;
        if (!ds[s].halted) {
            k = k1;
            continue;
        }
        HostState hs;
        get_host_state(s, hs);
        SysHost& h = sh[s];
        // collisions first (main.cu:540-569), then ejection / hit-centrum
        std::vector<red_event_t> coll, ejhc;
        for (size_t q = k; q < k1; q++) {
            red_event_t e;
            fill_event(s, hs, ev[q], ds[s].t, e);
            if (ev[q].name == RED_EVENT_COLLISION) coll.push_back(e);
            else ejhc.push_back(e);
        }
        // populate_sp_events: one record per (id1, id2), the earliest (pp_disk.cu:1250-1288)
        std::vector<red_event_t> sp;
        std::vector<char> done(coll.size(), 0);
        for (size_t a = 0; a < coll.size(); a++) {
            if (done[a]) continue;
            done[a] = 1;
            red_event_t e = coll[a];
            for (size_t b = a + 1; b < coll.size(); b++) {
                if (e.id1 == coll[b].id1 && e.id2 == coll[b].id2) {
                    done[b] = 1;
                    if (e.t > coll[b].t) e = coll[b];
                }
            }
            sp.push_back(e);
        }
        for (red_event_t& e : sp) {
            if (hs.md[e.idx2].body_type == RED_BODY_SUPERPLANETESIMAL) {
                ds[s].status = RED_ERR_SUPERPLANETESIMAL;
                rc = set_error(RED_ERR_SUPERPLANETESIMAL, "collision between a massive body and a super-planetesimal");
                break;
            }
            merge_pair(e, hs);
            bump(h.n_collision, h.n_event);
            hs.md[e.idx2].id *= -1;
            h.inactive[hs.md[e.idx2].body_type]++;
            event_log.push_back(e);
            if (out && n_written < cap) out[n_written] = e;
            n_written++;
        }
        for (red_event_t& e : ejhc) {
            if (e.event_name == RED_EVENT_EJECTION) {
                bump(h.n_ejection, h.n_event);
            } else {
                merge_pair(e, hs);
                bump(h.n_hit_centrum, h.n_event);
            }
            hs.md[e.idx2].id *= -1;
            h.inactive[hs.md[e.idx2].body_type]++;
            event_log.push_back(e);
            if (out && n_written < cap) out[n_written] = e;
            n_written++;
        }
        put_host_state(s, hs);
        ds[s].halted = 0;
        ds[s].n_coll = 0;
        ds[s].n_ejhc = 0;
        if (ds[s].status) ds[s].active = 0;
        if (h.n_active() <= 1) ds[s].active = 0;   // main.cu:471
        changed = true;
        if (16 <= h.n_event[1]) {                    // EVENT_COUNTER_NAME_LAST_CLEAR, main.cu:582-585
            for (int c = 0; c < 3; c++) (void)c;
            h.n_event[1] = h.n_collision[1] = h.n_ejection[1] = h.n_hit_centrum[1] = 0;
            write_sys(ds);
            rebuild_system(s);
            read_sys(ds);
        }
        k = k1;
    }
    if (changed) {
        write_sys(ds);
        build_plan();
        prep_positions();
        CK(cudaStreamSynchronize(stream));
        // systems whose ejection check was skipped because of collisions get it now
        // (red checks at the start of the next loop iteration, main.cu:499-523)
        if (has_ejhc() && rc == RED_OK) {
            ejhc_all();
            std::vector<DevSys> d2;
            read_sys(d2);
            bool again = false;
            for (const DevSys& d : d2) again = again || d.halted;
            if (again) {
                uint32_t more = 0;
                const uint32_t room = (out && cap > n_written) ? cap - n_written : 0;
                rc = handle_events(out ? out + std::min(n_written, cap) : nullptr, room, &more);
                n_written += more;
            }
        }
    }
    if (n_out) *n_out = n_written;
    return rc;
}

// pp_disk::rebuild_vectors (pp_disk.cu:1370-1430) and n_objects::update
// (red_type.h:568-578) for one system; the slot keeps its capacity.
void red_sim::rebuild_system(uint32_t s)
{
    SysHost& h = sh[s];
    HostState hs, out;
    get_host_state(s, hs);
    const uint32_t n_active = h.n_active();
    for (uint32_t i = 0; i < h.n; i++) {
        if (0 < hs.md[i].id && n_active > out.r.size()) {
            out.r.push_back(hs.r[i]);
            out.v.push_back(hs.v[i]);
            out.p.push_back(hs.p[i]);
            out.md.push_back(hs.md[i]);
        }
    }
    if (out.r.size() != n_active)
        throw ArgError{RED_ERR_ARG, "Number of copied bodies does not equal to the number of active bodies."};
    for (int i = 0; i < 7; i++) {
        h.playing[i] -= h.inactive[i];
        h.removed[i] += h.inactive[i];
        h.inactive[i] = 0;
    }
    h.n = (uint32_t)out.r.size();
    if (h.n) put_host_state(s, out);
    invalidate();
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define GUARD_BEGIN try {
#define GUARD_END                                                                                        \
    }                                                                                                    \
    catch (const CudaError& e) {                                                                         \
        return set_error(RED_ERR_CUDA, "CUDA error %s (%s) at sim.cu:%d: %s", cudaGetErrorName(e.e),   \
                         cudaGetErrorString(e.e), e.line, e.what);                                     \
    }                                                                                                    \
    catch (const ArgError& e) {                                                                          \
        return set_error(e.code, "%s", e.msg.c_str());                                                   \
    }                                                                                                    \
    catch (const std::bad_alloc&) {                                                                      \
        return set_error(RED_ERR_ARG, "host allocation failed");                                         \
    }

int redgb_set_error(int code, const char* msg) { return set_error(code, "%s", msg); }

static int check_sim(red_sim* sim)
{
    if (!sim) return set_error(RED_ERR_ARG, "null handle");
    cudaSetDevice(sim->device);
    return RED_OK;
}

extern "C" {

const char* red_last_error(void) { return g_last_error.c_str(); }
const char* red_version(void) { return "redgb 0.1 (sm_103a)"; }

int red_create(const red_config_t* cfg, uint32_t n_systems, const uint32_t* playing, const red_var4_t* r,
               const red_var4_t* v, const red_param_t* p, const red_body_metadata_t* md, const double* t0,
               const double* dt0, red_sim** out)
{
    if (!cfg || !playing || !r || !v || !p || !md || !out) return set_error(RED_ERR_ARG, "null argument");
    *out = nullptr;
    red_sim* sim = new (std::nothrow) red_sim();
    if (!sim) return set_error(RED_ERR_ARG, "host allocation failed");
    try {
        sim->create(cfg, n_systems, playing, r, v, p, md, t0, dt0);
    } catch (const CudaError& e) {
        delete sim;
        return set_error(RED_ERR_CUDA, "CUDA error %s at sim.cu:%d: %s", cudaGetErrorString(e.e), e.line, e.what);
    } catch (const ArgError& e) {
        delete sim;
        return set_error(e.code, "%s", e.msg.c_str());
    }
    *out = sim;
    return RED_OK;
}

int red_destroy(red_sim* sim)
{
    if (!sim) return RED_OK;
    cudaSetDevice(sim->device);
    if (sim->stream) cudaStreamSynchronize(sim->stream);
    delete sim;
    return RED_OK;
}

int red_launch_tries(red_sim* sim, uint32_t n)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    sim->launch_tries(n);
    return RED_OK;
    GUARD_END
}

int red_synchronize(red_sim* sim, uint32_t* n_active, uint32_t* n_halted)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    std::vector<DevSys> ds;
    sim->read_sys(ds);
    uint32_t a = 0, h = 0;
    int status = RED_OK;
    for (const DevSys& d : ds) {
        a += d.active ? 1 : 0;
        h += d.halted ? 1 : 0;
        if (d.status && !status) status = d.status;
    }
    if (n_active) *n_active = a;
    if (n_halted) *n_halted = h;
    if (status) return set_error(status, "a system stopped with status %d (non-finite state or error estimate)", status);
    return RED_OK;
    GUARD_END
}

int red_step(red_sim* sim, double* dt_did)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    std::vector<DevSys> ds;
    // Each try is one graph launch, followed by one read of the system records
    // (the only host synchronisation).  Several systems get a quota of one
    // accepted step, so that those done wait for the others; a single system
    // just stops being launched once its try is accepted.
    const bool quota = sim->n_sys > 1;
    if (quota) {
        launch_set_quota(sim->d_sys, (int)sim->n_sys, 1, sim->stream);
        CK(cudaGetLastError());
        sim->launches++;
    }
    for (int guard = 0; guard < 100000; guard++) {
        // retries of an ensemble launch only the items of the systems still pending
        if (!(quota && guard > 0 && sim->launch_sparse_try(ds))) sim->launch_tries(1);
        sim->read_sys(ds);
        bool pending = false;
        for (const DevSys& d : ds) {
            if (d.status) {
                if (quota) launch_set_quota(sim->d_sys, (int)sim->n_sys, -1, sim->stream);
                CK(cudaStreamSynchronize(sim->stream));
                return set_error(d.status, "integration stopped: status %d", d.status);
            }
            if (d.active && !d.halted && (quota ? d.quota != 0 : !d.accepted)) pending = true;
        }
        if (!pending) break;
    }
    if (dt_did) *dt_did = ds[0].dt_did;
    if (quota) {
        launch_set_quota(sim->d_sys, (int)sim->n_sys, -1, sim->stream);
        CK(cudaGetLastError());
        sim->launches++;
    }
    return RED_OK;
    GUARD_END
}

int red_handle_events(red_sim* sim, red_event_t* out, uint32_t cap, uint32_t* n_out)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    return sim->handle_events(out, cap, n_out);
    GUARD_END
}

static int check_generic(red_sim* sim, int collision, red_event_t* out, uint32_t cap, uint32_t* n_out)
{
    CK(cudaStreamSynchronize(sim->stream));
    // the explicit check must not see events left by the device-side checks
    CK(cudaMemsetAsync(sim->d_nev, 0, sizeof(unsigned int), sim->stream));
    if (collision) {
        CollParams Q;
        memset(&Q, 0, sizeof(Q));
        sim->fill_coll(Q);
        Q.only_accepted = 0;
        Q.mark = 0;
        sim->prep_positions();
        launch_collision(Q, (int)sim->pairs.size(), (int)sim->segs.size(), sim->use_grid, sim->table_size,
                         sim->stream);
    } else {
        EjhcParams E;
        memset(&E, 0, sizeof(E));
        E.segs = sim->d_segs; E.sinfo = sim->d_sinfo; E.sys = sim->d_sys; E.y_r = sim->y_r;
        E.id = sim->id; E.btype = sim->btype;
        E.ejection = sim->cfg.threshold[RED_THRESHOLD_EJECTION_DISTANCE];
        E.hit_centrum = sim->cfg.threshold[RED_THRESHOLD_HIT_CENTRUM_DISTANCE];
        E.only_accepted = 0;
        E.mark = 0;
        E.events = sim->d_events; E.n_events = sim->d_nev; E.capacity = sim->ev_cap;
        launch_ejhc(E, (int)sim->segs.size(), sim->stream);
    }
    CK(cudaGetLastError());
    sim->launches++;
    std::vector<DevEvent> ev;
    const uint32_t n_raw = sim->collect_events(ev);
    std::vector<DevSys> ds;
    sim->read_sys(ds);
    uint32_t w = 0;
    uint32_t cur = UINT32_MAX;
    HostState hs;
    for (const DevEvent& de : ev) {
        if ((uint32_t)de.sys != cur) {
            cur = de.sys;
            sim->get_host_state(cur, hs);
        }
        if (out && w < cap) sim->fill_event(cur, hs, de, ds[cur].t, out[w]);
        w++;
    }
    if (n_out) *n_out = w;
    if (n_raw > sim->ev_cap)
        return set_error(RED_ERR_EVENT_OVERFLOW, "%u events exceed the event buffer (%u)", n_raw, sim->ev_cap);
    return RED_OK;
}

int red_check_for_collision(red_sim* sim, red_event_t* out, uint32_t cap, uint32_t* n_out)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    return check_generic(sim, 1, out, cap, n_out);
    GUARD_END
}

int red_check_for_ejection_hit_centrum(red_sim* sim, red_event_t* out, uint32_t cap, uint32_t* n_out)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    return check_generic(sim, 0, out, cap, n_out);
    GUARD_END
}

int red_calc_dydx(red_sim* sim, uint32_t sys, int32_t i, double t, red_var4_t* dy)
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys || !dy || (i != 0 && i != 1)) return set_error(RED_ERR_ARG, "bad argument");
    GUARD_BEGIN
    const SysHost& h = sim->sh[sys];
    std::vector<double> buf(3 * (size_t)h.n);
    CK(cudaStreamSynchronize(sim->stream));
    if (i == 1) {
        sim->prep_positions();
        StageParams P = sim->stage_params(0, true);
        P.t_standalone = t;
        // only this system's items
        std::vector<GravItem> mine;
        for (const GravItem& g : sim->items)
            if (g.sys == (int)sys) mine.push_back(g);
        GravItem* d = dalloc<GravItem>(mine.size());
        CK(cudaMemcpy(d, mine.data(), mine.size() * sizeof(GravItem), cudaMemcpyHostToDevice));
        P.items = d;
        launch_stage(P, (int)mine.size(), sim->mode, sim->stream);
        CK(cudaGetLastError());
        sim->launches++;
        CK(cudaMemcpyAsync(buf.data(), sim->Kv[0] + 3 * (size_t)h.off, buf.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, sim->stream));
        CK(cudaStreamSynchronize(sim->stream));
        cudaFree(d);
    } else {
        CK(cudaMemcpyAsync(buf.data(), sim->y_v + 3 * (size_t)h.off, buf.size() * sizeof(double),
                           cudaMemcpyDeviceToHost, sim->stream));
        CK(cudaStreamSynchronize(sim->stream));
    }
    for (uint32_t k = 0; k < h.n; k++) dy[k] = red_var4_t{buf[3 * k], buf[3 * k + 1], buf[3 * k + 2], 0.0};
    return RED_OK;
    GUARD_END
}

static int potential(red_sim* sim, uint32_t sys, int interacting, std::vector<double>& u)
{
    const SysHost& h = sim->sh[sys];
    launch_potential(sim->d_segs, (int)sim->segs.size(), sim->d_sinfo, sim->y_r, sim->mass, sim->id, (int)sys,
                     interacting, sim->d_u, sim->stream);
    CK(cudaGetLastError());
    sim->launches++;
    u.resize(h.n);
    CK(cudaMemcpyAsync(u.data(), sim->d_u + h.off, h.n * sizeof(double), cudaMemcpyDeviceToHost, sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    return RED_OK;
}

int red_calc_integral(red_sim* sim, uint32_t sys, red_integral_t* out)
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys || !out) return set_error(RED_ERR_ARG, "bad argument");
    GUARD_BEGIN
    CK(cudaStreamSynchronize(sim->stream));
    HostState hs;
    sim->get_host_state(sys, hs);
    const uint32_t n = (uint32_t)hs.r.size();
    // tools::get_total_mass, calc_bc, calc_angular_momentum, calc_kinetic_energy (tools.cpp:365-690)
    double M0 = 0.0, R[3] = {0, 0, 0}, V[3] = {0, 0, 0}, C[3] = {0, 0, 0}, T = 0.0;
    for (int j = (int)n - 1; j >= 0; j--) {
        if (0 > hs.md[j].id) continue;
        M0 += hs.p[j].mass;
    }
    for (int j = (int)n - 1; j >= 0; j--) {
        if (0 > hs.md[j].id) continue;
        const double m = hs.p[j].mass;
        R[0] += m * hs.r[j].x; R[1] += m * hs.r[j].y; R[2] += m * hs.r[j].z;
        V[0] += m * hs.v[j].x; V[1] += m * hs.v[j].y; V[2] += m * hs.v[j].z;
    }
    for (uint32_t i = 0; i < n; i++) {
        if (0 > hs.md[i].id) continue;
        const red_var4_t& r = hs.r[i];
        const red_var4_t& v = hs.v[i];
        const double m = hs.p[i].mass;
        C[0] += m * (r.y * v.z - r.z * v.y);
        C[1] += m * (r.z * v.x - r.x * v.z);
        C[2] += m * (r.x * v.y - r.y * v.x);
        T += m * (v.x * v.x + v.y * v.y + v.z * v.z);
    }
    std::vector<double> u;
    potential(sim, sys, 0, u);
    double U = 0.0;
    for (double x : u) U += x;
    out->R = red_var4_t{R[0] / M0, R[1] / M0, R[2] / M0, 0.0};
    out->V = red_var4_t{V[0] / M0, V[1] / M0, V[2] / M0, 0.0};
    out->C = red_var4_t{C[0], C[1], C[2], 0.0};
    out->E = T / 2.0 - U / 2.0;
    return RED_OK;
    GUARD_END
}

int red_calc_energy_interacting(red_sim* sim, uint32_t sys, double out[4])
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys || !out) return set_error(RED_ERR_ARG, "bad argument");
    GUARD_BEGIN
    CK(cudaStreamSynchronize(sim->stream));
    HostState hs;
    sim->get_host_state(sys, hs);
    const uint32_t nm = sim->sh[sys].n_massive();
    double T = 0.0, C[3] = {0, 0, 0};
    for (uint32_t i = 0; i < nm && i < hs.r.size(); i++) {
        if (0 > hs.md[i].id) continue;
        const red_var4_t& r = hs.r[i];
        const red_var4_t& v = hs.v[i];
        const double m = hs.p[i].mass;
        T += m * (v.x * v.x + v.y * v.y + v.z * v.z);
        C[0] += m * (r.y * v.z - r.z * v.y);
        C[1] += m * (r.z * v.x - r.x * v.z);
        C[2] += m * (r.x * v.y - r.y * v.x);
    }
    std::vector<double> u;
    potential(sim, sys, 1, u);
    double U = 0.0;
    for (double x : u) U += x;
    out[0] = T / 2.0 - U;
    out[1] = C[0];
    out[2] = C[1];
    out[3] = C[2];
    return RED_OK;
    GUARD_END
}

// Bytes of the transfer records of n bodies: r, v, p as 12 doubles, id and type as 2 ints.
static size_t xfer_bytes(size_t n) { return n * (12 * sizeof(double) + 2 * sizeof(int)); }
static_assert(sizeof(red_var4_t) == 4 * sizeof(double) && sizeof(red_param_t) == 4 * sizeof(double),
              "the state records are 4 doubles each");

// The device address of page-locked host memory (cudaHostAlloc / cudaHostRegister,
// mapped into the device's address space), or null for any other pointer.
static const void* device_view_of_host(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void red_sim::ensure_xfer(size_t bytes)
{
    if (bytes <= xfer_cap) return;
    cudaFree(d_xfer);
    if (h_xfer) cudaFreeHost(h_xfer);
    d_xfer = nullptr;
    h_xfer = nullptr;
    xfer_cap = 0;
    CK(cudaMalloc(&d_xfer, bytes));
    CK(cudaMallocHost(&h_xfer, bytes));
    xfer_cap = bytes;
}

// System s's records, packed on the device and copied into h_xfer in one transfer.
void red_sim::pack_range_to_host(size_t o, size_t n)
{
    ensure_xfer(xfer_bytes(n));
    double* rvp = (double*)d_xfer;
    int* ib = (int*)(d_xfer + 12 * n * sizeof(double));
    launch_pack_state((int)o, (int)n, y_r, y_v, mass, radius, density, cd, id, btype,
                      StateSegs{{rvp, rvp + 4 * n, rvp + 8 * n}}, ib, stream);
    CK(cudaGetLastError());
    launches++;
    CK(cudaMemcpyAsync(h_xfer, d_xfer, xfer_bytes(n), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
}

// Systems [s0, s0 + cnt) whose body ranges follow each other on the device
// (always, until a compaction leaves a system's tail unused).
static bool contiguous(const red_sim* sim, uint32_t s0, uint32_t cnt)
{
    for (uint32_t s = s0 + 1; s < s0 + cnt; s++)
        if (sim->sh[s].off != sim->sh[s - 1].off + sim->sh[s - 1].n) return false;
    return true;
}

static size_t bodies_in(const red_sim* sim, uint32_t s0, uint32_t cnt)
{
    size_t n = 0;
    for (uint32_t s = s0; s < s0 + cnt; s++) n += sim->sh[s].n;
    return n;
}

// The records of systems [s0, s0 + cnt), contiguous on the device, packed on
// the device into the caller's arrays: pinned (page-locked) arrays directly by
// the kernel over the host link, others through the device staging buffer and
// one copy each (no staging copy on the host).
static void get_state_range(red_sim* sim, uint32_t s0, uint32_t cnt, red_var4_t* r, red_var4_t* v, red_param_t* p,
                            red_body_metadata_t* md)
{
    const size_t o = sim->sh[s0].off;
    const size_t n = bodies_in(sim, s0, cnt);
    sim->ensure_xfer(xfer_bytes(n));
    double* d_rvp = (double*)sim->d_xfer;
    const size_t ib_off = 12 * n * sizeof(double);
    void* const out[3] = {r, v, p};
    StateSegs dst{{nullptr, nullptr, nullptr}};
    bool copy[3] = {false, false, false};
    for (int k = 0; k < 3; k++) {
        if (!out[k]) continue;
        dst.seg[k] = (double*)device_view_of_host(out[k]);
        if (!dst.seg[k]) {
            dst.seg[k] = d_rvp + 4 * n * k;
            copy[k] = true;
        }
    }
    launch_pack_state((int)o, (int)n, sim->y_r, sim->y_v, sim->mass, sim->radius, sim->density, sim->cd, sim->id,
                      sim->btype, dst, (int*)(sim->d_xfer + ib_off), sim->stream);
    CK(cudaGetLastError());
    sim->launches++;
    for (int k = 0; k < 3; k++)   // var4_t and param_t are both 4 doubles
        if (copy[k])
            CK(cudaMemcpyAsync(out[k], d_rvp + 4 * n * k, n * sizeof(red_var4_t), cudaMemcpyDeviceToHost,
                               sim->stream));
    if (md)
        CK(cudaMemcpyAsync(sim->h_xfer + ib_off, sim->d_xfer + ib_off, 2 * n * sizeof(int), cudaMemcpyDeviceToHost,
                           sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    const int* ib = (const int*)(sim->h_xfer + ib_off);
    if (md) {
        for (size_t i = 0; i < n; i++) {
            md[i].id = ib[2 * i];
            md[i].body_type = ib[2 * i + 1];
            md[i].mig_type = sim->mig_type[o + i];
            md[i].mig_stop_at = sim->mig_stop_at[o + i];
        }
    }
}

static void get_states(red_sim* sim, uint32_t s0, uint32_t cnt, red_var4_t* r, red_var4_t* v, red_param_t* p,
                       red_body_metadata_t* md)
{
    sim->ensure_xfer(xfer_bytes(bodies_in(sim, s0, cnt)));   // no reallocation between the ranges
    if (contiguous(sim, s0, cnt)) {
        get_state_range(sim, s0, cnt, r, v, p, md);
        return;
    }
    size_t a = 0;
    for (uint32_t s = s0; s < s0 + cnt; s++) {
        get_state_range(sim, s, 1, r ? r + a : nullptr, v ? v + a : nullptr, p ? p + a : nullptr,
                        md ? md + a : nullptr);
        a += sim->sh[s].n;
    }
}

int red_get_state(red_sim* sim, uint32_t sys, red_var4_t* r, red_var4_t* v, red_param_t* p,
                  red_body_metadata_t* md)
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys) return set_error(RED_ERR_ARG, "bad system index");
    GUARD_BEGIN
    get_states(sim, sys, 1, r, v, p, md);
    return RED_OK;
    GUARD_END
}

int red_get_states(red_sim* sim, uint32_t sys0, uint32_t count, red_var4_t* r, red_var4_t* v, red_param_t* p,
                   red_body_metadata_t* md)
{
    if (int rc = check_sim(sim)) return rc;
    if (count == 0 || sys0 >= sim->n_sys || count > sim->n_sys - sys0)
        return set_error(RED_ERR_ARG, "bad system range");
    GUARD_BEGIN
    get_states(sim, sys0, count, r, v, p, md);
    return RED_OK;
    GUARD_END
}

// The caller's records of systems [s0, s0 + cnt), contiguous on the device, to
// the device.  Pinned (page-locked) arrays are read by the unpacking kernel over
// the host link, others are copied to the device staging buffer first (no
// staging copy on the host); only the ids pass through the pinned staging
// buffer.  Returns whether the plan must be rebuilt.
static bool set_state_range(red_sim* sim, uint32_t s0, uint32_t cnt, const red_var4_t* r, const red_var4_t* v,
                            const red_param_t* p, const red_body_metadata_t* md)
{
    const size_t o = sim->sh[s0].off;
    const size_t n = bodies_in(sim, s0, cnt);
    sim->ensure_xfer(xfer_bytes(n));
    const size_t ib_off = 12 * n * sizeof(double);
    int* ib = (int*)(sim->h_xfer + ib_off);
    double* d_rvp = (double*)sim->d_xfer;
    const void* const in[3] = {r, v, p};
    StateSegs src{{nullptr, nullptr, nullptr}};
    int what = 0;
    for (int k = 0; k < 3; k++) {   // var4_t and param_t are both 4 doubles
        if (!in[k]) continue;
        what |= 1 << k;
        src.seg[k] = (double*)device_view_of_host(in[k]);
        if (!src.seg[k]) {
            src.seg[k] = d_rvp + 4 * n * k;
            CK(cudaMemcpyAsync(src.seg[k], in[k], n * sizeof(red_var4_t), cudaMemcpyHostToDevice, sim->stream));
        }
    }
    if (md) {
        for (size_t i = 0; i < n; i++) {
            ib[2 * i] = md[i].id;
            sim->mig_type[o + i] = md[i].mig_type;
            sim->mig_stop_at[o + i] = md[i].mig_stop_at;
        }
        CK(cudaMemcpyAsync(sim->d_xfer + ib_off, ib, 2 * n * sizeof(int), cudaMemcpyHostToDevice, sim->stream));
        what |= 8;
    }
    launch_unpack_state((int)o, (int)n, what, src, (const int*)(sim->d_xfer + ib_off), sim->y_r, sim->y_v,
                        sim->mass, sim->radius, sim->density, sim->cd, sim->id, sim->pos_hi[0], sim->pos_lo[0],
                        sim->stream);
    CK(cudaGetLastError());
    sim->launches++;
    bool replan = md != nullptr;   // ids decide which bodies act as sources
    if (p) {
        // the collision grid's cells must stay wider than the largest collision distance,
        // and the work items carry the first star's mass
        size_t a = 0;
        for (uint32_t s = s0; s < s0 + cnt; s++) {
            const SysHost& h = sim->sh[s];
            double rmax = 0.0;
            for (size_t k = h.n_SI(); k < h.n; k++) rmax = std::max(rmax, p[a + k].radius);
            if (rmax > sim->grid_rmax[s]) replan = true;
            if (h.playing[0] > 0 && p[a].mass != sim->star_mass[s]) replan = true;
            a += h.n;
        }
    }
    return replan;
}

// Body types are fixed by the class ranges: the new metadata of systems
// [s0, s0 + cnt) must keep the current ones (checked before anything is written).
static void check_body_types(red_sim* sim, uint32_t s0, uint32_t cnt, const red_body_metadata_t* md)
{
    size_t a = 0;
    for (uint32_t s = s0; s < s0 + cnt; s++) {
        const size_t n = sim->sh[s].n;
        sim->pack_range_to_host(sim->sh[s].off, n);
        const int* ib = (const int*)(sim->h_xfer + 12 * n * sizeof(double));
        for (size_t i = 0; i < n; i++)
            if (md[a + i].body_type != ib[2 * i + 1])
                throw ArgError{RED_ERR_ARG, "body types cannot change through red_set_state"};
        a += n;
    }
}

static void set_states(red_sim* sim, uint32_t s0, uint32_t cnt, const red_var4_t* r, const red_var4_t* v,
                       const red_param_t* p, const red_body_metadata_t* md)
{
    bool replan = false;
    sim->ensure_xfer(xfer_bytes(bodies_in(sim, s0, cnt)));   // no reallocation between the ranges
    if (md) check_body_types(sim, s0, cnt, md);
    if (contiguous(sim, s0, cnt)) {
        replan = set_state_range(sim, s0, cnt, r, v, p, md);
    } else {
        size_t a = 0;
        for (uint32_t s = s0; s < s0 + cnt; s++) {
            replan |= set_state_range(sim, s, 1, r ? r + a : nullptr, v ? v + a : nullptr, p ? p + a : nullptr,
                                      md ? md + a : nullptr);
            a += sim->sh[s].n;
        }
    }
    if (replan) {
        CK(cudaStreamSynchronize(sim->stream));
        sim->build_plan();
    }
    // new positions alone are already in the FP32 copies (k_unpack_state);
    // masses, radii and ids change their .w words
    if (p || md || replan) sim->prep_positions();
    // the unpacking kernel reads pinned caller arrays: done before they may be reused
    CK(cudaStreamSynchronize(sim->stream));
}

int red_set_state(red_sim* sim, uint32_t sys, const red_var4_t* r, const red_var4_t* v, const red_param_t* p,
                  const red_body_metadata_t* md)
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys) return set_error(RED_ERR_ARG, "bad system index");
    GUARD_BEGIN
    set_states(sim, sys, 1, r, v, p, md);
    return RED_OK;
    GUARD_END
}

int red_set_states(red_sim* sim, uint32_t sys0, uint32_t count, const red_var4_t* r, const red_var4_t* v,
                   const red_param_t* p, const red_body_metadata_t* md)
{
    if (int rc = check_sim(sim)) return rc;
    if (count == 0 || sys0 >= sim->n_sys || count > sim->n_sys - sys0)
        return set_error(RED_ERR_ARG, "bad system range");
    GUARD_BEGIN
    set_states(sim, sys0, count, r, v, p, md);
    return RED_OK;
    GUARD_END
}

int red_get_system_info(red_sim* sim, uint32_t sys, red_system_info_t* info)
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys || !info) return set_error(RED_ERR_ARG, "bad argument");
    GUARD_BEGIN
    std::vector<DevSys> ds;
    sim->read_sys(ds);
    const DevSys& d = ds[sys];
    const SysHost& h = sim->sh[sys];
    memset(info, 0, sizeof(*info));
    info->t = d.t;
    info->dt_try = d.dt_try;
    info->dt_did = d.dt_did;
    info->dt_next = d.dt_next;
    info->n_tried = d.n_tried;
    info->n_passed = d.n_passed;
    info->n_failed = d.n_failed;
    memcpy(info->playing, h.playing, sizeof(h.playing));
    memcpy(info->inactive, h.inactive, sizeof(h.inactive));
    memcpy(info->removed, h.removed, sizeof(h.removed));
    info->n_total = h.n;
    info->active = d.active;
    info->halted = d.halted;
    info->status = d.status;
    memcpy(info->n_collision, h.n_collision, sizeof(h.n_collision));
    memcpy(info->n_ejection, h.n_ejection, sizeof(h.n_ejection));
    memcpy(info->n_hit_centrum, h.n_hit_centrum, sizeof(h.n_hit_centrum));
    memcpy(info->n_event, h.n_event, sizeof(h.n_event));
    return RED_OK;
    GUARD_END
}

int red_set_dt_next(red_sim* sim, uint32_t sys, double dt_next)
{
    if (int rc = check_sim(sim)) return rc;
    if (sys >= sim->n_sys) return set_error(RED_ERR_ARG, "bad system index");
    GUARD_BEGIN
    std::vector<DevSys> ds;
    sim->read_sys(ds);
    ds[sys].dt_next = ds[sys].dt_try = dt_next;
    sim->write_sys(ds);
    return RED_OK;
    GUARD_END
}

int red_rebuild_vectors(red_sim* sim)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    CK(cudaStreamSynchronize(sim->stream));
    for (uint32_t s = 0; s < sim->n_sys; s++) sim->rebuild_system(s);
    sim->build_plan();
    sim->prep_positions();
    CK(cudaStreamSynchronize(sim->stream));
    return RED_OK;
    GUARD_END
}

int red_profile_try(red_sim* sim, float* ms, int32_t* kind, uint32_t cap, uint32_t* n_out)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    std::vector<int> kinds;
    std::vector<cudaEvent_t> evs;
    sim->enqueue_try(&kinds, &evs);
    CK(cudaGetLastError());
    sim->launches += (uint64_t)sim->launches_per_try;
    CK(cudaStreamSynchronize(sim->stream));
    uint32_t w = 0;
    for (size_t k = 1; k < evs.size(); k++) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, evs[k - 1], evs[k]));
        if (w < cap) {
            if (ms) ms[w] = t;
            if (kind) kind[w] = kinds[k];
        }
        w++;
    }
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    if (n_out) *n_out = w;
    return RED_OK;
    GUARD_END
}

uint64_t red_interactions_per_eval(red_sim* sim) { return sim ? sim->interactions_per_eval() : 0; }
uint64_t red_kernel_launches(red_sim* sim) { return sim ? sim->launches : 0; }
uint32_t red_n_systems(red_sim* sim) { return sim ? sim->n_sys : 0; }
uint32_t red_n_bodies(red_sim* sim, uint32_t sys) { return sim && sys < sim->n_sys ? sim->sh[sys].n : 0; }

int red_autotune(red_sim* sim)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    // Candidate plans: threads per sink group (lanes_cap), and source chunks
    // from the planner's heuristic (with or without the cluster reduction) or
    // fixed sizes.  Each candidate integrates real tries (the whole captured
    // graph) from a snapshot of the live state, which is restored afterwards:
    // the systems end exactly where they were.  red's own precedent times its
    // gravity kernel over thread-per-block counts (pp_disk.cu:553-611).
    CK(cudaStreamSynchronize(sim->stream));
    red_plan_info_t& info = sim->plan_info;
    info.candidates = 0;
    if (sim->mode == MODE_FP64_EXACT) {   // one lane per sink in red's order: nothing to choose
        info.chunk = sim->chunk_override;
        info.lanes_cap = sim->lanes_cap;
        info.cluster = sim->use_cluster ? 1 : 0;
        info.packed = sim->use_packed ? 1 : 0;
        info.n_items = (int32_t)sim->items.size();
        return RED_OK;
    }
    const size_t N = sim->n_cap;
    double* s_r = dalloc<double>(3 * N);
    double* s_v = dalloc<double>(3 * N);
    DevSys* s_sys = dalloc<DevSys>(sim->n_sys);
    unsigned int* s_nev = dalloc<unsigned int>(1);
    float* s_feat = nullptr;
    int* s_has = nullptr;
    unsigned int* s_logn = nullptr;
    cudaStream_t st = sim->stream;
    auto copy = [&](void* dst, const void* src, size_t bytes) {
        CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
    };
    auto swap_state = [&](bool save) {
        auto mv = [&](void* live, void* saved, size_t bytes) { save ? copy(saved, live, bytes) : copy(live, saved, bytes); };
        mv(sim->y_r, s_r, 3 * N * sizeof(double));
        mv(sim->y_v, s_v, 3 * N * sizeof(double));
        mv(sim->d_sys, s_sys, sim->n_sys * sizeof(DevSys));
        mv(sim->d_nev, s_nev, sizeof(unsigned int));
        if (s_feat) mv(sim->d_feat_prev, s_feat, (size_t)sim->n_sys * kFeat * sizeof(float));
        if (s_has) mv(sim->d_has_prev, s_has, sim->n_sys * sizeof(int));
        if (s_logn) mv(sim->d_log_n, s_logn, sizeof(unsigned int));
    };
    if (sim->d_feat_prev) s_feat = dalloc<float>((size_t)sim->n_sys * kFeat);
    if (sim->d_has_prev) s_has = dalloc<int>(sim->n_sys);
    if (sim->d_log_n) s_logn = dalloc<unsigned int>(1);
    swap_state(true);
    const bool ejhc_done = sim->ejhc_initial_done;   // the first try's ejection check is still owed
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    struct Cand { int chunk, lanes; bool cluster, packed; };
    std::vector<Cand> cands;
    for (int lanes : {32, 16, 8}) {
        cands.push_back({0, lanes, true, false});   // a cluster plan never takes the packed instance
        for (bool pk : {true, false}) {
            cands.push_back({0, lanes, false, pk});
            for (int c : {256, 512, 1024, 2048, 4096}) cands.push_back({c, lanes, false, pk});
        }
    }
    float best = 1e30f;
    Cand best_c = cands[0];
    int reps = 0;
    for (const Cand& c : cands) {
        sim->chunk_override = c.chunk;
        sim->lanes_cap = c.lanes;
        sim->allow_cluster = c.cluster;
        sim->allow_packed = c.packed;
        sim->build_plan();
        if (c.cluster && !sim->use_cluster && c.chunk == 0) continue;   // same plan as a later candidate
        if (c.packed && !sim->use_packed) continue;                       // the same as its unpacked twin
        sim->prep_positions();
        sim->launch_tries(2);                  // graph capture, warm caches
        if (reps == 0) {
            CK(cudaEventRecord(e0, st));
            sim->launch_tries(3);
            CK(cudaEventRecord(e1, st));
            CK(cudaEventSynchronize(e1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            reps = std::max(3, std::min(50, (int)ceil(2.0 / std::max(ms / 3.0f, 1e-3f))));
        }
        CK(cudaEventRecord(e0, st));
        sim->launch_tries((uint32_t)reps);
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ms /= (float)reps;
        if (info.candidates == 0) info.ms_per_try_default = ms;
        info.candidates++;
        if (ms < best) {
            best = ms;
            best_c = c;
        }
        swap_state(false);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sim->chunk_override = best_c.chunk;
    sim->lanes_cap = best_c.lanes;
    sim->allow_cluster = best_c.cluster;
    sim->allow_packed = best_c.packed;
    sim->build_plan();
    swap_state(false);
    sim->ejhc_initial_done = ejhc_done;
    sim->prep_positions();
    CK(cudaStreamSynchronize(st));
    cudaFree(s_r); cudaFree(s_v); cudaFree(s_sys); cudaFree(s_nev);
    cudaFree(s_feat); cudaFree(s_has); cudaFree(s_logn);
    info.chunk = sim->chunk_override;
    info.lanes_cap = sim->lanes_cap;
    info.cluster = sim->use_cluster ? 1 : 0;
    info.packed = sim->use_packed ? 1 : 0;
    info.n_items = (int32_t)sim->items.size();
    info.ms_per_try = best;
    return RED_OK;
    GUARD_END
}

int red_get_plan_info(red_sim* sim, red_plan_info_t* out)
{
    if (int rc = check_sim(sim)) return rc;
    if (!out) return set_error(RED_ERR_ARG, "null argument");
    red_plan_info_t i = sim->plan_info;
    i.chunk = sim->chunk_override;
    i.lanes_cap = sim->lanes_cap;
    i.cluster = sim->use_cluster ? 1 : 0;
    i.packed = sim->use_packed ? 1 : 0;
    i.n_items = (int32_t)sim->items.size();
    *out = i;
    return RED_OK;
}


int red_set_step_proposer(red_sim* sim, const uint16_t* w_bf16, const red_mlp_norm_t* norm, double safety,
                          double ratio_lo, double ratio_hi)
{
    if (int rc = check_sim(sim)) return rc;
    if (!w_bf16 || !norm || !(safety > 0.0) || !(ratio_lo > 0.0) || !(ratio_hi >= ratio_lo))
        return set_error(RED_ERR_ARG, "red_set_step_proposer: bad argument");
    for (int c = 0; c < kFeat; c++)
        if (!(norm->x_std[c] > 0.f)) return set_error(RED_ERR_ARG, "red_set_step_proposer: x_std must be positive");
    if (!(norm->y_std > 0.f)) return set_error(RED_ERR_ARG, "red_set_step_proposer: y_std must be positive");
    GUARD_BEGIN
    CK(cudaStreamSynchronize(sim->stream));
    if (!sim->d_mlp_w) sim->d_mlp_w = dalloc<__nv_bfloat16>(kNParam);
    CK(cudaMemcpyAsync(sim->d_mlp_w, w_bf16, kNParam * sizeof(uint16_t), cudaMemcpyHostToDevice, sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    memcpy(&sim->mlp_norm, norm, sizeof(MlpNorm));
    sim->prop_safety = safety;
    sim->prop_lo = ratio_lo;
    sim->prop_hi = ratio_hi;
    sim->prop_on = true;
    sim->invalidate();
    return RED_OK;
    GUARD_END
}

int red_clear_step_proposer(red_sim* sim)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    CK(cudaStreamSynchronize(sim->stream));
    sim->prop_on = false;
    sim->invalidate();
    return RED_OK;
    GUARD_END
}

int red_log_features(red_sim* sim, uint32_t capacity)
{
    if (int rc = check_sim(sim)) return rc;
    GUARD_BEGIN
    CK(cudaStreamSynchronize(sim->stream));
    cudaFree(sim->d_log);
    sim->d_log = nullptr;
    sim->log_cap = 0;
    sim->log_on = capacity > 0;
    if (sim->log_on) {
        sim->d_log = dalloc<float>((size_t)capacity * kLogRec);
        sim->log_cap = capacity;
        if (!sim->d_log_n) sim->d_log_n = dalloc<unsigned int>(1);
        if (!sim->d_feat_prev) {
            sim->d_feat_prev = dalloc<float>((size_t)sim->n_sys * kFeat);
            sim->d_has_prev = dalloc<int>(sim->n_sys);
        }
        CK(cudaMemsetAsync(sim->d_log_n, 0, sizeof(unsigned int), sim->stream));
        CK(cudaMemsetAsync(sim->d_has_prev, 0, sim->n_sys * sizeof(int), sim->stream));
        CK(cudaStreamSynchronize(sim->stream));
    }
    sim->invalidate();
    return RED_OK;
    GUARD_END
}

int red_get_feature_log(red_sim* sim, float* out, uint32_t cap, uint32_t* n_out, int32_t reset)
{
    if (int rc = check_sim(sim)) return rc;
    if (!n_out || (cap && !out)) return set_error(RED_ERR_ARG, "red_get_feature_log: bad argument");
    GUARD_BEGIN
    unsigned int count = 0;
    CK(cudaStreamSynchronize(sim->stream));
    if (sim->d_log_n) CK(cudaMemcpy(&count, sim->d_log_n, sizeof(count), cudaMemcpyDeviceToHost));
    const uint32_t n = std::min<uint32_t>(count, sim->log_cap);
    *n_out = n;
    const uint32_t k = std::min(n, cap);
    if (k) CK(cudaMemcpy(out, sim->d_log, (size_t)k * kLogRec * sizeof(float), cudaMemcpyDeviceToHost));
    if (reset && sim->d_log_n) CK(cudaMemset(sim->d_log_n, 0, sizeof(unsigned int)));
    return RED_OK;
    GUARD_END
}

}  // extern "C"
