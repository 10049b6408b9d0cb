// redgb_dev.cuh -- device-side layout shared by the kernels and the host layer.
//
// HBM layout (all systems concatenated; system s owns bodies [off, off+n)):
//   y_r, y_v        double[3N]   current positions / velocities, xyz packed per body
//   Kr[s], Kv[s]    double[3N]   stage derivatives: Kr[s] = stage velocity (the
//                                r-derivative), Kv[s] = acceleration; Kr[0] aliases y_v
//   tr[2]           double[3N]   FP64 stage positions, ping-pong by stage parity
//   pos_hi[2]       float4[N]    (x, y, z, mass) rounded to FP32, by stage parity
//   pos_lo[2]       float4[N]    (x - hi, y - hi, z - hi, radius), the low words of
//                                the double-single coordinates
//   mass, radius, density, cd    double[N], id / btype int32[N]
// The .w lane red integrates (always 0) is not stored.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace redgb {

constexpr int kTile = 128;          // sinks per CTA and sources per shared-memory tile
constexpr int kSegment = 256;       // bodies per CTA in the per-body kernels
constexpr int kFinishBodies = 64;   // bodies per CTA of k_finish (one thread per component)
constexpr int kClusterChunks = 16;  // source chunks of a tile in a cluster launch (one cluster)
constexpr int kMaxStages = 13;

enum Mode { MODE_MIXED = 0, MODE_FP64 = 1, MODE_FP64_EXACT = 2, MODE_FP32 = 3 };
enum Scheme { SCHEME_RK4 = 0, SCHEME_RKF78 = 1, SCHEME_EULER = 2, SCHEME_RK2 = 3 };
enum Cls { CLS_SI = 0, CLS_NSI = 1, CLS_NI = 2 };

// Per-system integrator state, device resident.  Mirrors integrator's
// dt_try / dt_did / dt_next and counters (integrator.h:37-52) and pp_disk::t.
struct DevSys {
    double t;
    double t_start;
    double dt_try;        // step of the try in flight
    double dt_did;        // last accepted step
    double dt_next;
    unsigned long long err_bits;   // max |error| of the try, as the bits of a non-negative double
    unsigned long long n_tried, n_passed, n_failed;
    int iter;             // tries made in the current step
    int accepted;         // the last try was accepted
    int active;           // integrating (length not reached)
    int halted;           // events found, waiting for the host
    int status;           // 0 or a RED_ERR_* code
    int n_coll;           // collision events found for this system in the last check
    int n_ejhc;           // ejection / hit-centrum events found in the last check
    int quota;            // accepted steps still allowed (-1: unlimited)
    int pad;
    double err_last;      // lambda dt |error| of the last try (0 for fixed steps)
};

__host__ __device__ inline bool runnable(const DevSys& S)
{
    return S.active && !S.halted && S.quota != 0;
}

// Static description of a system.
struct SysInfo {
    int off, n;           // body range
    int n_star;           // stars: bodies [off, off + n_star)
    int n_SI, n_massive;  // counts relative to off
    int n_err;            // bodies in the error norm (n_massive, or n with error_check_for_tp)
};

// One CTA of the stage kernel: a tile of sinks against one chunk of sources.
struct GravItem {
    int sys;
    int sink0, nsink;     // absolute first sink, count (<= kTile)
    int src0, src1;       // absolute source range of this chunk
    int chunk, nchunk;
    int tile;             // tile id: counter index when nchunk > 1
    int part_off;         // first partial record of the tile
    int lanes;            // threads per sink (4, 8, 16 or 32), lanes * nsink <= kTile
    int cls;
    int soff;             // first body of the system; its stars are [soff, soff + nstar)
    int nstar;
    int nerr;             // bodies [soff, soff + nerr) enter the error norm
    int spt;              // sinks per thread group (1, or 2 in the FP32 modes: lanes >= 8)
    int mstar_set;        // 1: mstar holds the mass of the system's first star (0 if inactive)
    float mstar_hi, mstar_lo;   // that mass, double-single
    int pad[2];
};

// Per-body kernels: one CTA per segment of one system.
struct Segment {
    int sys, b0, b1, pad;
};

// Tile pair of the brute-force collision check: i in [i0, min(i0 + kTile, i1)),
// j in the tile starting at j0, j > i (bodies of one system).
struct PairItem {
    int sys, i0, j0, i1;
};

// Spatial hash grid of one system's small bodies (the NSI and NI classes) for
// the collision check: cells of edge 1/inv_h >= the largest collision distance
// between two small bodies, buckets [toff, toff + mask + 1) of a global table.
struct GridInfo {
    double inv_h;
    int toff, mask;
    int enabled;
    int pad;
};

// Compact collision / ejection record written by the device.
struct DevEvent {
    int sys;
    int name;             // RED_EVENT_*
    int i, j;             // loop indices (i < j for collisions; 0, body for ejection)
    int surv, merg;       // idx1, idx2 of red's event record
    double d;
};

struct GasDev {
    double rho[2], sch[2], eta[2];
    double t0, t1, e_folding_time;
    int gas_decrease;
    int enabled;
};

struct Tableau {
    // RKF7(8), int_rungekutta8.cu:26-48
    double c[kMaxStages];
    double a[79];
    double b[11];
    int nnz[kMaxStages];
    int src[kMaxStages][9];
    // RK4, int_rungekutta4.cu:26-31
    double a4[8], b4[5], c4[5];
    // RK2, int_rungekutta2.cu:12-14 (Euler has no coefficients: y + dt f)
    double a2[2], b2[2], c2[2];
};

struct StageParams {
    int stage;            // stage s evaluated by this launch
    int next;             // stage whose positions the epilogue prepares, -1 for none
    int scheme;           // SCHEME_*
    int err_after;        // 1: this stage closes an adaptive try, epilogue adds the error norm
    int ynp1_to_out;      // RK4 adaptive: the epilogue of stage 3 writes y_{n+1} as stage 4's input
    int standalone;       // red_calc_dydx: only store Kv[stage]
    int nthreads_pad;
    double t_standalone;  // time of a standalone evaluation (drag)
    const GravItem* items;
    const SysInfo* sinfo;
    DevSys* sys;
    const float4* pos_hi_in;
    const float4* pos_lo_in;
    float4* pos_hi_out;
    float4* pos_lo_out;
    const double* r_in;   // FP64 positions of stage s
    double* r_out;        // FP64 positions of stage `next`
    const double* y_r;
    const double* y_v;
    double* Kr[kMaxStages];
    double* Kv[kMaxStages];
    const double* mass;
    const double* radius;
    const double* density;
    const double* cd;
    const int* id;
    double* partial;      // 3 doubles per record
    unsigned int* tile_cnt;
    GasDev gas;
    int* head;            // stage 0 sets the collision check's bucket heads to -1 (not null)
    long long head_n;
    int cluster;          // 1: launched in clusters of kClusterChunks CTAs (items laid out for it)
    int one_wave;         // 1: the launch is one wave (one kernel instance for every variant)
    int packed;           // 1: plans of many waves with 2-sink tiles take the packed-pair instance
};

struct FinishParams {
    int scheme, adaptive;
    int commit_from_stage4;   // RK4 adaptive: y_{n+1} lives in tr[0] / Kr[4]
    int stage_exact;
    const Segment* segs;
    const SysInfo* sinfo;
    DevSys* sys;
    double* y_r;
    double* y_v;
    const double* Kr[kMaxStages];
    const double* Kv[kMaxStages];
    const double* t_r0;       // tr[0]
    const double* mass;
    const double* radius;
    const int* id;
    float4* pos_hi0;
    float4* pos_lo0;
    // spatial hash of the collision check that follows (head not null): the
    // accepted systems' small bodies are inserted at their new positions
    int* head;
    int* next;
    int4* cell;
    const GridInfo* grid;
};

struct ControlParams {
    int n_sys;
    int scheme, adaptive, order;
    int keep_dt;          // Euler / RK2: every step takes the initial dt (the dt_next clamp does not feed back)
    int exact;            // red-exact mode: the step-size power rounded to the nearest double
    double tolerance, lambda;
    double output_interval, length;
    DevSys* sys;
};

struct CollParams {
    const PairItem* items;
    const Segment* segs;
    const GridInfo* grid;
    int* head;            // bucket heads (-1 = empty)
    int* next;            // per-body link of the bucket lists
    int4* cell;           // per-body cell coordinates
    const SysInfo* sinfo;
    DevSys* sys;
    const float4* pos_hi;
    const float4* pos_lo;
    const double* y_r;
    const double* radius;
    const double* mass;
    const int* id;
    double factor;        // radii enhance factor
    int only_accepted;    // run only for systems that just accepted a try
    int mark;             // 1: count the events in DevSys and halt the system
    DevEvent* events;
    unsigned int* n_events;
    unsigned int capacity;
};

struct EjhcParams {
    const Segment* segs;
    const SysInfo* sinfo;
    DevSys* sys;
    const double* y_r;
    const int* id;
    const int* btype;
    double ejection, hit_centrum;
    int only_accepted;
    int mark;
    DevEvent* events;
    unsigned int* n_events;
    unsigned int capacity;
};

constexpr int kBatchRecords = 16;   // partial records loaded per batch by the reducing CTA
// An empty partial-record slot (8 bytes) of the one-wave stage instance: a
// signalling-NaN pattern no arithmetic produces.  Slots are filled with it
// when a plan is built (fill_records_empty) and reset to it by the CTA that
// sums them.
constexpr unsigned long long kRecEmpty = 0x7ff0000000000001ull;

// Host-side plan of the stage kernel for one system (sim.cu).
// tiles_all: sink tiles of every system planned into the same launch (count_sink_tiles).
// short_ctas (optional) accumulates the CTAs the system would need with chunks of
// two source tiles; short_chunks selects those chunks for the plan.
int count_sink_tiles(const SysInfo& si, int mode, int lanes_cap, long long* short_ctas);
// star_mass: the effective mass of the system's first star (0 if its id < 0), or
// nullptr when the host does not hold it (the kernel then reads it).
void plan_gravity_items(const SysInfo& si, int sys, int mode, int chunk_override, int lanes_cap, int tiles_all,
                        bool short_chunks, const double* star_mass, std::vector<GravItem>& items, size_t& part,
                        int& tiles);

// Host-side launchers (kernels.cu, stage_*.cu).  The stage kernel's mode
// fixes the arithmetic of the stage combinations: FP64_EXACT combines in red's
// operation order without FMA, the other modes with FMA.
void set_tableau(const Tableau& tb, cudaStream_t s);
// Programmatic dependent launch of the kernels of a try (kernels.cu): while set
// on the calling thread, the launchers give each kernel the
// programmatic-stream-serialization attribute, so that it is scheduled while
// its predecessor runs and waits for it with griddepcontrol.wait.
void set_pdl(bool on);
bool pdl_on();
void launch_stage(const StageParams& P, int n_items, int mode, cudaStream_t s);
int stage_variant(const StageParams& P);
void set_tableau_mixed(const Tableau& tb, cudaStream_t s);
void set_tableau_fp32(const Tableau& tb, cudaStream_t s);
void set_tableau_fp64(const Tableau& tb, cudaStream_t s);
void set_tableau_exact(const Tableau& tb, cudaStream_t s);
void launch_stage_mixed(const StageParams& P, int n, int variant, cudaStream_t s);
// Clusters of kClusterChunks stage CTAs resident at once (FP32 modes; 0 for
// the others or when the query fails).
int active_clusters_mixed();
int active_clusters_fp32();
int stage_active_clusters(int mode);
void launch_stage_fp32(const StageParams& P, int n, int variant, cudaStream_t s);
void launch_stage_fp64(const StageParams& P, int n, int variant, cudaStream_t s);
void launch_stage_exact(const StageParams& P, int n, int variant, cudaStream_t s);
void launch_prep(const Segment* segs, int n_segs, const SysInfo* sinfo, const DevSys* sys, const double* y_r,
                 const double* mass, const double* radius, const int* id, float4* hi, float4* lo, float4* hi1,
                 float4* lo1, int all, cudaStream_t s);
void launch_control(const ControlParams& P, cudaStream_t s);
void launch_finish(const FinishParams& P, int n_segs, cudaStream_t s);
void launch_collision(const CollParams& P, int n_items, int n_segs, bool use_grid, size_t table_size,
                      cudaStream_t s);
void launch_collide(const CollParams& P, int n_items, int n_segs, bool use_grid, cudaStream_t s);
void launch_ejhc(const EjhcParams& P, int n_segs, cudaStream_t s);
void launch_set_quota(DevSys* sys, int n_sys, int q, cudaStream_t s);
// Sets n partial-record slots (8 bytes each) to kRecEmpty.
void fill_records_empty(void* recs, size_t n, cudaStream_t s);
// The three record arrays of red_get_state / red_set_state (r, v, p: 4 doubles
// per body each).  Each is the device staging buffer or, when the caller's
// array is pinned host memory, that array itself, read or written by the
// kernel over the host link; a null entry is skipped.
struct StateSegs {
    double* seg[3];
};
void launch_pack_state(int o, int n, const double* y_r, const double* y_v, const double* mass, const double* radius,
                       const double* density, const double* cd, const int* id, const int* btype, StateSegs dst,
                       int* ib, cudaStream_t s);
void launch_unpack_state(int o, int n, int what, StateSegs src, const int* ib, double* y_r, double* y_v,
                         double* mass, double* radius, double* density, double* cd, int* id, float4* hi0,
                         float4* lo0, cudaStream_t s);
void launch_potential(const Segment* segs, int n_segs, const SysInfo* sinfo, const double* y_r,
                      const double* mass, const int* id, int sys_filter, int interacting, double* u,
                      cudaStream_t s);

}  // namespace redgb
