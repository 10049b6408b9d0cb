// stage.cuh -- the Runge-Kutta stage kernel of libredgb.
//
// One launch evaluates stage s of every system: the gravity of each sink
// against its chunk of sources (shared-memory tiles), the reduction of the
// source chunks of a sink tile (two-level, by the CTAs that finish last), and
// an element-wise FP64 epilogue: central-star term, gas drag, K storage, the
// combination that gives the positions of the next stage (or the error norm
// after the last stage).
//
// The kernel is instantiated per arithmetic mode; the "variant" V, the shape
// of the next-stage combination, is a launch argument:
//   V = 0        no combination (standalone evaluation, last stage of a try)
//   V = 1 .. 12  RKF7(8) stage V: y + dt * sum_q a_{V,q} K_q
//   V = 13       RK4 stage s + 1: y + (a_{s+1} dt) K_s
//   V = 14       RK4 y_{n+1} as the input of the adaptive stage 4
//   V = 15       RKF7(8) error norm after stage 12
//   V = 16       RK4 error norm after stage 4
// The operands of the combination are copied into shared memory at the start
// of the kernel, overlapping the gravity loop.  One kernel body serves all
// stages, so after the first stage of a try its code is cached.  Each mode
// lives in its own translation unit (stage_*.cu).
#pragma once
#include "common.cuh"

namespace redgb {

constexpr int kStarBatch = 4;   // stars staged in shared memory (more are read from global memory)

struct SmemStage {
    union {
        struct { float4 hi[2 * kTile]; float4 lo[2 * kTile]; } f;   // up to two tiles staged at once
        struct { D4 d[kTile]; int id[kTile]; } d;
    } src;
    double acc[kTile];              // per (sink, component) gravity sums; per-thread record sums
    double sc[32][3];               // drag factor and gas velocity per sink
    float4 star_hi[kStarBatch], star_lo[kStarBatch];   // the stars' double-single positions
    float2 star_m[kStarBatch];      // the stars' masses, double-single (0 for inactive stars)
    union {                         // the tile's sinks (cp.async in the prologue)
        struct { float4 hi[32]; float4 lo[32]; } f;
        double d[3 * 32];
    } snk;
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

// Double-single sum of the float2 partial records [c0, c1) of one element (FP32
// modes), in order, loads issued in one batch per kBatchRecords records.
__device__ __forceinline__ float2 sum_records_ds(const float2* base, long long stride, int c0, int c1)
{
    float2 a = make_float2(0.f, 0.f);
    for (int b = c0; b < c1; b += kBatchRecords) {
        float2 pv[kBatchRecords];
#pragma unroll
        for (int u = 0; u < kBatchRecords; u++) pv[u] = (b + u < c1) ? __ldcg(base + (b + u) * stride) : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kBatchRecords; u++)
            if (b + u < c1) a = dsn_add(a, pv[u]);
    }
    return a;
}

// Sum of the partial records [c0, c1) of one element (3 doubles per sink record,
// element t of the tile at offset t), in order, loads issued in one batch per
// kBatchRecords records.
__device__ __forceinline__ double sum_records(const double* base, long long stride, int c0, int c1)
{
    double a = 0.0;
    for (int b = c0; b < c1; b += kBatchRecords) {
        double pv[kBatchRecords];
#pragma unroll
        for (int u = 0; u < kBatchRecords; u++) pv[u] = (b + u < c1) ? __ldcg(base + (b + u) * stride) : 0.0;
#pragma unroll
        for (int u = 0; u < kBatchRecords; u++)
            if (b + u < c1) a += pv[u];
    }
    return a;
}

// Polled partial records (the one-wave stage instance).  There the chunks of
// a tile store their records and advance the tile's counter with no fence, so
// each record carries its own readiness: its slot holds kRecEmpty
// (redgb_dev.cuh), a signalling-NaN bit pattern that no arithmetic produces
// (FP64 results carry the canonical quiet NaN; as a float2 it is a denormal
// beside a non-canonical NaN), until its chunk's store lands.  The CTA that
// takes the last count re-reads a record it finds empty, and resets every
// slot it read to kRecEmpty for the next launch.  Every store it waits for has
// been issued (the chunk's CTA passed a barrier after its stores, then
// counted), so the wait ends within the memory system's latency; it is bounded
// all the same: after kRecPollLimit reads of a batch its missing records count
// as NaN, the system's status is set to RED_ERR_TIMEOUT and the system is
// halted.  (The many-wave instances keep a release fence before the count and
// an acquire fence after the last one, and plain records: the fences' latency
// hides behind other CTAs there, and their reducing CTAs would otherwise meet
// stores in flight.)
constexpr unsigned long long kRecNaN = 0x7ff800007fc00000ull;   // NaN as a double and in both float halves
constexpr int kRecPollLimit = 1 << 20;

__device__ __forceinline__ void st_rec(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_rec(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];\n" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long rec_bits(float2 v)
{
    return ((unsigned long long)__float_as_uint(v.y) << 32) | __float_as_uint(v.x);
}
__device__ __forceinline__ unsigned long long rec_bits(double v) { return (unsigned long long)__double_as_longlong(v); }
__device__ __forceinline__ void rec_add(float2& a, unsigned long long b)
{
    a = dsn_add(a, make_float2(__uint_as_float((unsigned)b), __uint_as_float((unsigned)(b >> 32))));
}
__device__ __forceinline__ void rec_add(double& a, unsigned long long b) { a += __longlong_as_double((long long)b); }

// Re-reads the records [b, b1) until every chunk's store has landed, within
// one budget of kRecPollLimit reads for the whole batch.  Returns false if
// the budget runs out first.
__device__ __forceinline__ bool poll_records(const unsigned long long* base, long long stride, int b, int b1)
{
    int budget = kRecPollLimit;
    for (int c = b; c < b1; c++) {
        unsigned long long v = kRecEmpty;
        while (v == kRecEmpty && budget > 0) {
            v = ld_rec(base + c * stride);
            budget--;
        }
        if (v == kRecEmpty) return false;
    }
    return true;
}

// Sum of the polled records [c0, c1) of one element (element t of the tile at
// offset t, `stride` words per chunk), in chunk order: double-single for the
// float2 records of the FP32 modes, FP64 otherwise.  Loads are issued in
// batches of kBatchRecords; a batch with a record still empty waits for its
// records (poll_records) and is read again.  The slots are then emptied.
// Returns false if a record stayed empty (it then adds NaN).
template <typename T>
__device__ __forceinline__ bool sum_polled_records(unsigned long long* base, long long stride, int c0, int c1, T& sum)
{
    bool ok = true, again = false;
    for (int b = c0; b < c1;) {
        unsigned long long pv[kBatchRecords];
        bool empty = false;
#pragma unroll
        for (int u = 0; u < kBatchRecords; u++) {
            pv[u] = (b + u < c1) ? ld_rec(base + (b + u) * stride) : 0ull;
            empty |= pv[u] == kRecEmpty;
        }
        if (empty && !again) {   // rare: a store of this batch is still in flight; wait, then read it again
            ok = poll_records(base, stride, b, min(b + kBatchRecords, c1)) && ok;
            again = true;
            continue;
        }
        again = false;
        ok = ok && !empty;
#pragma unroll
        for (int u = 0; u < kBatchRecords; u++)
            if (b + u < c1) rec_add(sum, pv[u] == kRecEmpty ? kRecNaN : pv[u]);
        b += kBatchRecords;
    }
    for (int c = c0; c < c1; c++) st_rec(base + c * stride, kRecEmpty);   // empty again for the next launch
    return ok;
}

// 8-byte asynchronous copy global -> shared (cp.async, no register held while
// the copy is in flight), its commit and the wait for all of a thread's copies.
__device__ __forceinline__ void cp_async8(void* dst, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// Waits until at most the most recent group of the thread's copies is in flight.
__device__ __forceinline__ void cp_async_wait_prior() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Release / acquire at GPU scope (the writes of the whole CTA are ordered
// before it by the preceding barrier; fences are cumulative).
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;\n" ::: "memory"); }

// Operands of the epilogue of variant V, staged in shared memory by cp.async
// at the start of the kernel: slot [slot][t] belongs to element thread t.
constexpr int kMaxElem = 96;   // 3 * 32 sinks: the largest tile the planner makes
static_assert(kMaxElem < kTile, "thread kTile - 1 holds no element of the epilogue");
__host__ __device__ constexpr int var_nk(int v)
{
    return v == 1 ? 1 : v == 2 ? 2 : v == 3 ? 2 : v == 4 ? 3 : v == 5 ? 3 : v == 6 ? 4 : v == 7 ? 4 : v == 8 ? 6
         : v == 9 ? 7 : v == 10 ? 8 : v == 11 ? 6 : v == 12 ? 9 : (v == 14 || v == 15) ? 3 : v == 16 ? 1 : 0;
}
constexpr int kNkMax = 9;                  // the most K operands of a variant (RKF7(8) stage 12)
constexpr int kOpsMax = 3 + 2 * kNkMax;    // shared-memory operand slots
// The time offset c_s of stage s (RKF7(8), RK4, RK2; Euler evaluates at t).
__device__ __forceinline__ double stage_c(int scheme, int s)
{
    if (scheme == SCHEME_RKF78) return c_tb.c[s];
    if (scheme == SCHEME_RK4) return c_tb.c4[s];
    if (scheme == SCHEME_RK2) return c_tb.c2[s];
    return 0.0;
}

// Thread-block cluster helpers (a tile's source chunks as one cluster): the
// barrier in two halves (every thread of every CTA of the cluster arrives;
// release / acquire at cluster scope) and a read of another CTA's shared memory.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory"); }
__device__ __forceinline__ float2 ld_cluster_f2(const float2* local, unsigned rank)
{
    unsigned a = (unsigned)__cvta_generic_to_shared(local), r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(r) : "memory");
    return v;
}

// Operand slots of a variant: the stage velocity, y_r, y_v, then nk K_r and nk K_v.
constexpr int kOpVS = 0, kOpYR = 1, kOpYV = 2, kOpKR = 3;
// Source stages of the RKF7(8) combinations (Tableau::src), for runtime indexing.
static __constant__ int c_src[13][kNkMax] = {
    {0}, {0}, {0, 1}, {0, 2}, {0, 2, 3}, {0, 3, 4}, {0, 3, 4, 5}, {0, 4, 5, 6},
    {0, 3, 4, 5, 6, 7}, {0, 3, 4, 5, 6, 7, 8}, {0, 3, 4, 5, 6, 7, 8, 9},
    {0, 5, 6, 7, 8, 9}, {0, 3, 4, 5, 6, 7, 8, 9, 11}};
// Stage index of operand q of variant V: from the compile-time table when the
// kernel instance fixes the variant (VT >= 0), else from constant memory.
template <int VT>
__device__ __forceinline__ int op_src(int V, int q)
{
    if constexpr (VT >= 1 && VT <= 12) {
        return kSrc[VT][q];
    } else if constexpr (VT == 14) {
        return q;
    } else if constexpr (VT == 15) {
        return q == 0 ? 0 : (q == 1 ? 10 : 11);
    } else if constexpr (VT >= 0) {
        return 3;
    } else {
        if (V >= 1 && V <= 12) return c_src[V][q];
        if (V == 14) return q;
        if (V == 15) return q == 0 ? 0 : (q == 1 ? 10 : 11);
        return 3;
    }
}

// Gravity of the chunk's sources on SPT sinks per thread, FP32 modes.  The
// first tile is in shared memory; (th, tl) carry the prefetch of the next.
// On return thread lane l < 3 SPT of its sink group holds component l % 3 of
// sink slot (group * SPT + l / 3) in `mine`, a double-single sum.
template <int MODE, int SPT>
__device__ __forceinline__ void gravity_f32(SmemStage& sm, const StageParams& P, const GravItem& it, bool staged,
                                            float4& th, float4& tl, float2& mine, int& mine_k, bool& mine_ok)
{
    const int t = threadIdx.x;
    constexpr int LC = SPT == 2 ? 8 : 0;   // the planner pairs 2 sinks per thread with 8 lanes
    const int L = LC ? LC : it.lanes;
    const int grp = t / L, lane = t % L;
    float4 H[SPT], Lo[SPT];
#pragma unroll
    for (int q = 0; q < SPT; q++) {
        const int k = grp * SPT + q;
        const int ks = k < it.nsink ? k : 0;   // inactive slots shadow sink 0 (results unused)
        H[q] = sm.snk.f.hi[ks];
        Lo[q] = MODE == MODE_MIXED ? sm.snk.f.lo[ks] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float acc[SPT][6];
#pragma unroll
    for (int q = 0; q < SPT; q++)
#pragma unroll
        for (int c = 0; c < 6; c++) acc[q][c] = 0.f;
    for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
        const int nj = min(kTile, it.src1 - j0);
        const bool more = !staged && j0 + kTile < it.src1;
        const int base = staged ? j0 - it.src0 : 0;   // staged chunks hold all their tiles
        if (more && t < min(kTile, it.src1 - j0 - kTile)) {
            th = P.pos_hi_in[j0 + kTile + t];
            if (MODE == MODE_MIXED) tl = P.pos_lo_in[j0 + kTile + t];
        }
        float tx[SPT], ty[SPT], tz[SPT];
#pragma unroll
        for (int q = 0; q < SPT; q++) tx[q] = ty[q] = tz[q] = 0.f;
        auto source = [&](int jj) {
            const float4 h = sm.src.f.hi[base + jj];
            float4 l = make_float4(0.f, 0.f, 0.f, 0.f);
            if (MODE == MODE_MIXED) l = sm.src.f.lo[base + jj];
#pragma unroll
            for (int q = 0; q < SPT; q++) {
                float dx, dy, dz;
                if (MODE == MODE_MIXED) {
                    dx = (h.x - H[q].x) + (l.x - Lo[q].x);
                    dy = (h.y - H[q].y) + (l.y - Lo[q].y);
                    dz = (h.z - H[q].z) + (l.z - Lo[q].z);
                } else {
                    dx = h.x - H[q].x;
                    dy = h.y - H[q].y;
                    dz = h.z - H[q].z;
                }
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, kEps2)));
                const float ri = rsqrtf(r2);
                const float ri2 = ri * ri;
                const float sc = h.w * ri * ri2;
                tx[q] = fmaf(sc, dx, tx[q]);
                ty[q] = fmaf(sc, dy, ty[q]);
                tz[q] = fmaf(sc, dz, tz[q]);
            }
        };
        if (LC && nj == kTile) {
#pragma unroll 4
            for (int u = 0; u < kTile / (LC ? LC : 1); u++) source(lane + u * L);
        } else {
#pragma unroll 4
            for (int jj = lane; jj < nj; jj += L) source(jj);
        }
#pragma unroll
        for (int q = 0; q < SPT; q++) {
            ds_add(acc[q][0], acc[q][1], tx[q]);
            ds_add(acc[q][2], acc[q][3], ty[q]);
            ds_add(acc[q][4], acc[q][5], tz[q]);
        }
        if (more) {
            __syncthreads();
            sm.src.f.hi[t] = th;
            if (MODE == MODE_MIXED) sm.src.f.lo[t] = tl;
            __syncthreads();
        }
    }
    // lanes -> one double-single sum per (sink, component): TwoSum in FP32 over a
    // fixed butterfly, so every lane of the group ends with the same bits
    for (int o = 1; o < L; o <<= 1) {
#pragma unroll
        for (int q = 0; q < SPT; q++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float oh = __shfl_xor_sync(0xffffffffu, acc[q][2 * c], o);
                const float ol = __shfl_xor_sync(0xffffffffu, acc[q][2 * c + 1], o);
                ds_merge(acc[q][2 * c], acc[q][2 * c + 1], oh, ol);
            }
    }
    float hh = 0.f, ll = 0.f;
#pragma unroll
    for (int q = 0; q < SPT; q++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (lane == 3 * q + c) {
                hh = acc[q][2 * c];
                ll = acc[q][2 * c + 1];
            }
    mine = dsn_norm(hh, ll);
    mine_k = grp * SPT + lane / 3;
    mine_ok = lane < 3 * SPT && mine_k < it.nsink;
}

// The same gravity for tiles of 2 sinks per thread on 8 lanes, with packed
// FP32 pairs (add / mul / fma .f32x2: one instruction for two interactions).
// The lanes step over pairs of sources, held in shared memory as pair records:
//   A[p] = (x_2p, x_2p+1, y_2p, y_2p+1), B[p] = (z_2p, z_2p+1, m_2p, m_2p+1)
// and, for the double-single low parts, C[p] = (x, x', y, y') and D[p] = (z, z').
// A chunk of up to two tiles, staged at once as one float4 per source, is
// rewritten in place (pair_tiles); the tiles of a longer chunk go from the
// registers that prefetch them straight into the records of two alternating
// buffers (put_pair), one barrier per tile.
// An odd source count pads the last pair with a copy of its first source of
// mass 0 (its term is 0 * finite).  The sums are those of gravity_f32 in
// another grouping: each lane's tile sum is the sum of its two pair halves.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

template <int MODE>
__device__ __forceinline__ void pair_tiles(SmemStage& sm, int nsrc, int ntile)
{
    // tile tau (kTile sources at tau * kTile) -> its pair records, in place
    const int t = threadIdx.x;
    constexpr int kHalf = kTile / 2;
    const int tau = t / kHalf, lp = t % kHalf;
    const int b = tau * kTile;
    const int nt = min(kTile, nsrc - tau * kTile);
    const bool on = tau < ntile && 2 * lp < nt;
    float4 h0 = make_float4(0.f, 0.f, 0.f, 0.f), h1 = h0, l0 = h0, l1 = h0;
    if (on) {
        h0 = sm.src.f.hi[b + 2 * lp];
        if (MODE == MODE_MIXED) l0 = sm.src.f.lo[b + 2 * lp];
        if (2 * lp + 1 < nt) {
            h1 = sm.src.f.hi[b + 2 * lp + 1];
            if (MODE == MODE_MIXED) l1 = sm.src.f.lo[b + 2 * lp + 1];
        } else {
            h1 = make_float4(h0.x, h0.y, h0.z, 0.f);
            l1 = l0;
        }
    }
    __syncthreads();
    if (on) {
        sm.src.f.hi[b + lp] = make_float4(h0.x, h1.x, h0.y, h1.y);
        sm.src.f.hi[b + kHalf + lp] = make_float4(h0.z, h1.z, h0.w, h1.w);
        if (MODE == MODE_MIXED) {
            sm.src.f.lo[b + lp] = make_float4(l0.x, l1.x, l0.y, l1.y);
            sm.src.f.lo[b + kHalf + lp] = make_float4(l0.z, l1.z, 0.f, 0.f);
        }
    }
    __syncthreads();
}

// Source t of a streamed tile, from registers straight into pair buffer buf
// (sm.src.f.hi / .lo from buf * kTile): the records pair_tiles makes, with no
// staging pass.  A source beyond the chunk comes as zeros (mass 0).
template <int MODE>
__device__ __forceinline__ void put_pair(SmemStage& sm, int buf, int t, float4 h, float4 l)
{
    constexpr int kHalf = kTile / 2;
    float* A = reinterpret_cast<float*>(sm.src.f.hi + buf * kTile);
    float* B = A + 4 * kHalf;
    const int o = 4 * (t >> 1) + (t & 1);
    A[o] = h.x;
    A[o + 2] = h.y;
    B[o] = h.z;
    B[o + 2] = h.w;
    if (MODE == MODE_MIXED) {
        float* Cl = reinterpret_cast<float*>(sm.src.f.lo + buf * kTile);
        float* Dl = Cl + 4 * kHalf;
        Cl[o] = l.x;
        Cl[o + 2] = l.y;
        Dl[o] = l.z;
        Dl[o + 2] = 0.f;
    }
}

template <int MODE>
__device__ __forceinline__ void gravity_f32_pair(SmemStage& sm, const StageParams& P, const GravItem& it,
                                                 bool staged, float4& th, float4& tl, float2& mine, int& mine_k,
                                                 bool& mine_ok)
{
    constexpr int SPT = 2, L = 8, kHalf = kTile / 2;
    const int t = threadIdx.x;
    const int grp = t / L, lane = t % L;
    float2 nHx[SPT], nHy[SPT], nHz[SPT], nLx[SPT], nLy[SPT], nLz[SPT];
#pragma unroll
    for (int q = 0; q < SPT; q++) {
        const int k = grp * SPT + q;
        const int ks = k < it.nsink ? k : 0;   // inactive slots shadow sink 0 (results unused)
        const float4 H = sm.snk.f.hi[ks];
        const float4 Lo = MODE == MODE_MIXED ? sm.snk.f.lo[ks] : make_float4(0.f, 0.f, 0.f, 0.f);
        nHx[q] = f2(-H.x, -H.x);
        nHy[q] = f2(-H.y, -H.y);
        nHz[q] = f2(-H.z, -H.z);
        nLx[q] = f2(-Lo.x, -Lo.x);
        nLy[q] = f2(-Lo.y, -Lo.y);
        nLz[q] = f2(-Lo.z, -Lo.z);
    }
    float acc[SPT][6];
#pragma unroll
    for (int q = 0; q < SPT; q++)
#pragma unroll
        for (int c = 0; c < 6; c++) acc[q][c] = 0.f;
    if (staged) pair_tiles<MODE>(sm, it.src1 - it.src0, (it.src1 - it.src0 + kTile - 1) / kTile);
    int buf = 0;   // streamed chunks: the pair buffer of the current tile (the prologue filled buffer 0)
    for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
        const int nj = min(kTile, it.src1 - j0);
        const bool more = !staged && j0 + kTile < it.src1;
        const int nnext = more ? min(kTile, it.src1 - j0 - kTile) : 0;
        const int base = staged ? j0 - it.src0 : buf * kTile;   // staged chunks hold all their tiles
        if (t < nnext) {
            th = P.pos_hi_in[j0 + kTile + t];
            if (MODE == MODE_MIXED) tl = P.pos_lo_in[j0 + kTile + t];
        }
        const float4* A = sm.src.f.hi + base;
        const float4* B = A + kHalf;
        const float4* Cl = sm.src.f.lo + base;
        const float4* Dl = Cl + kHalf;
        float2 tx[SPT], ty[SPT], tz[SPT];
#pragma unroll
        for (int q = 0; q < SPT; q++) tx[q] = ty[q] = tz[q] = f2(0.f, 0.f);
        const int np = (nj + 1) >> 1;
        const float2 eps2 = f2(kEps2, kEps2);
#pragma unroll 4
        for (int pp = lane; pp < np; pp += L) {
            const float4 a = A[pp], bz = B[pp];
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f), d = c;
            if (MODE == MODE_MIXED) {
                c = Cl[pp];
                d = Dl[pp];
            }
#pragma unroll
            for (int q = 0; q < SPT; q++) {
                float2 dx = __fadd2_rn(f2(a.x, a.y), nHx[q]);
                float2 dy = __fadd2_rn(f2(a.z, a.w), nHy[q]);
                float2 dz = __fadd2_rn(f2(bz.x, bz.y), nHz[q]);
                if (MODE == MODE_MIXED) {
                    dx = __fadd2_rn(dx, __fadd2_rn(f2(c.x, c.y), nLx[q]));
                    dy = __fadd2_rn(dy, __fadd2_rn(f2(c.z, c.w), nLy[q]));
                    dz = __fadd2_rn(dz, __fadd2_rn(f2(d.x, d.y), nLz[q]));
                }
                float2 r2 = __ffma2_rn(dx, dx, eps2);
                r2 = __ffma2_rn(dy, dy, r2);
                r2 = __ffma2_rn(dz, dz, r2);
                const float2 ri = f2(rsqrtf(r2.x), rsqrtf(r2.y));
                const float2 sc = __fmul2_rn(__fmul2_rn(f2(bz.z, bz.w), ri), __fmul2_rn(ri, ri));
                tx[q] = __ffma2_rn(sc, dx, tx[q]);
                ty[q] = __ffma2_rn(sc, dy, ty[q]);
                tz[q] = __ffma2_rn(sc, dz, tz[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < SPT; q++) {
            ds_add(acc[q][0], acc[q][1], tx[q].x + tx[q].y);
            ds_add(acc[q][2], acc[q][3], ty[q].x + ty[q].y);
            ds_add(acc[q][4], acc[q][5], tz[q].x + tz[q].y);
        }
        if (more) {
            // the next tile goes into the other buffer, which every thread finished
            // reading before the barrier that ended the previous tile
            if (t >= nnext) th = tl = make_float4(0.f, 0.f, 0.f, 0.f);
            put_pair<MODE>(sm, buf ^ 1, t, th, tl);
            __syncthreads();
            buf ^= 1;
        }
    }
    for (int o = 1; o < L; o <<= 1) {
#pragma unroll
        for (int q = 0; q < SPT; q++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float oh = __shfl_xor_sync(0xffffffffu, acc[q][2 * c], o);
                const float ol = __shfl_xor_sync(0xffffffffu, acc[q][2 * c + 1], o);
                ds_merge(acc[q][2 * c], acc[q][2 * c + 1], oh, ol);
            }
    }
    float hh = 0.f, ll = 0.f;
#pragma unroll
    for (int q = 0; q < SPT; q++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (lane == 3 * q + c) {
                hh = acc[q][2 * c];
                ll = acc[q][2 * c + 1];
            }
    mine = dsn_norm(hh, ll);
    mine_k = grp * SPT + lane / 3;
    mine_ok = lane < 3 * SPT && mine_k < it.nsink;
}

// Gravity of the chunk's sources, FP64 modes (one sink per thread group).
template <int MODE>
__device__ __forceinline__ void gravity_f64(SmemStage& sm, const StageParams& P, const GravItem& it, D4& td, int& tid,
                                            double& mine, int& mine_k, bool& mine_ok)
{
    const int t = threadIdx.x;
    const int L = it.lanes;
    const int k = t / L, lane = t % L;
    const bool has = k < it.nsink;
    const int i = it.sink0 + (has ? k : 0);
    const int ks = has ? k : 0;
    const double xi = sm.snk.d[3 * ks], yi = sm.snk.d[3 * ks + 1], zi = sm.snk.d[3 * ks + 2];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int j0 = it.src0; j0 < it.src1; j0 += kTile) {
        const int nj = min(kTile, it.src1 - j0);
        const bool more = j0 + kTile < it.src1;
        if (more && t < min(kTile, it.src1 - j0 - kTile)) {
            const int j = j0 + kTile + t;
            tid = P.id[j];
            const double m = P.mass[j];
            td = D4{P.r_in[3 * j], P.r_in[3 * j + 1], P.r_in[3 * j + 2], (MODE == MODE_FP64 && tid < 0) ? 0.0 : m};
        }
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
            sm.src.d.d[t] = td;
            sm.src.d.id[t] = tid;
            __syncthreads();
        }
    }
    if (MODE == MODE_FP64_EXACT) {
        const int gbase = (t & 31) & ~(L - 1);
        ax = __shfl_sync(0xffffffffu, ax, gbase);
        ay = __shfl_sync(0xffffffffu, ay, gbase);
        az = __shfl_sync(0xffffffffu, az, gbase);
    } else {
        ax = group_sum(ax, L);
        ay = group_sum(ay, L);
        az = group_sum(az, L);
    }
    mine = lane == 0 ? ax : (lane == 1 ? ay : az);
    mine_k = k;
    mine_ok = has && lane < 3;
}

// ---------------------------------------------------------------------------
// k_stage
//
// Gravity: each group of `lanes` consecutive threads of a warp serves SPT
// sinks (SPT = 2 in the FP32 modes when the class has many sinks, so that
// every source read from shared memory feeds two interactions); the lanes
// split the sources of every tile.  Epilogue: element-wise, thread t < 3 nsink
// owns component x = 3 sink0 + t, which is contiguous in HBM, so every FP64
// instruction runs in full warps.
//
// Memory round trips on the critical path: the work item; then, in one batch,
// the system state, the first source tile, the sinks and the star / drag
// inputs; then one per further source tile (fetched while the previous one is
// in use); then, for a chunked tile, the partial records.  The epilogue's
// operands (y, the K vectors of the combination) are copied into shared
// memory by cp.async at the start, so they arrive during the gravity loop
// without holding registers.
// ---------------------------------------------------------------------------
// CL: the cluster-launch instance (FP32 modes), whose items are laid out in
// clusters of kClusterChunks CTAs.  VT >= 0 fixes the variant at compile time
// (one instance per variant, for launches of many waves); VT = -1 takes it from
// the launch argument, so that one kernel body serves all stages of a try and
// stays in the instruction caches (launches of one wave, where the cold start
// of each stage is on the critical path).  The per-variant instances run 7 CTAs
// per SM (72 registers, 27 KB of shared memory each): their launches are many
// waves of CTAs that each wait on a chain of memory round trips, and the seventh
// CTA hides more of it (512-disk ensemble stage -17 %, 65536-body gas-drag
// disk -13 %, all-pairs 16384-body disk -1.3 %; 8 CTAs at 64 registers spill
// and are slower).  The one-wave instance keeps 80 registers.
template <int MODE, bool EXACT, bool CL, int VT, bool PK = false>
__global__ void __launch_bounds__(kTile, PK ? 6 : (VT >= 0 ? 7 : 6)) k_stage(const StageParams P, const int Vrt)
{
    constexpr bool kF32 = (MODE == MODE_MIXED || MODE == MODE_FP32);
    const int V = VT >= 0 ? VT : Vrt;
    const bool kRkf = (V >= 1 && V <= 12);
    const int nk = var_nk(V);
    const int kOpKV = 3 + nk;
    constexpr int kUnroll = VT >= 0 ? kNkMax : 1;   // operand loops: unrolled when nk is a constant
    __shared__ SmemStage sm;
    __shared__ double ops[kOpsMax][kMaxElem];
    const GravItem it = P.items[blockIdx.x];
    const int s = P.stage;
    // Stage 0 follows the kernels that update the system records, y and the
    // stage-0 positions, and waits first.  A later stage reads before its wait
    // only what the previous stage does not write: the system record (written
    // after the last stage), y, ids, masses, K_q of stages <= s - 2 (the stage
    // velocity Kr[q] is written by stage q - 1, the acceleration Kv[q] by q).
    if (s == 0) {
        pdl_wait();
        if (P.head) {   // the collision check at the end of this try starts from an empty hash
            const long long nt = (long long)gridDim.x * blockDim.x;
            for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < P.head_n; k += nt) P.head[k] = -1;
        }
    }
    if (CL && it.nsink == 0) {   // padding of the last cluster
        pdl_wait();
        return;
    }
    DevSys* S = P.sys + it.sys;
    double tsys = 0.0, dt = 0.0;
    if (!P.standalone) {
        const int act = S->active, hal = S->halted, quo = S->quota;
        tsys = S->t;
        dt = S->dt_try;
        if (!(act && !hal && quo != 0)) {   // uniform over the CTA
            pdl_wait();
            return;
        }
    }
    const int t = threadIdx.x;

    // ---- the element of the epilogue; its operands go to shared memory ----
    const int nel = 3 * it.nsink;
    const bool elem = t < nel;
    const int ke = elem ? t / 3 : 0;
    const int ce = elem ? t % 3 : 0;
    const int ie = it.sink0 + ke;
    const int x = 3 * ie + ce;
    const int idi = P.id[ie];
    const bool drag_on = P.gas.enabled && it.cls == CLS_NSI;
    const bool need_vs = drag_on || V != 0;
    if (elem) {   // copy group 0: the operands older than the previous stage
        if (V >= 1 && V <= 14) {
            cp_async8(&ops[kOpYR][t], P.y_r + x);
            cp_async8(&ops[kOpYV][t], P.y_v + x);
        }
#pragma unroll kUnroll
        for (int q = 0; q < nk; q++) {
            const int src = op_src<VT>(V, q);
            if (src != s) cp_async8(&ops[kOpKR + q][t], P.Kr[src] + x);
            if (!(kRkf && src == V - 1) && src != s - 1) cp_async8(&ops[kOpKV + q][t], P.Kv[src] + x);
        }
    }
    cp_async_commit();
    // ---- the stars' masses for the central-star term (FP32 modes), double-single ----
    const bool star_term = kF32 && it.nstar > 0;
    const int nst0 = star_term ? min(kStarBatch, it.nstar) : 0;
    if (t < nst0) {
        if (t == 0 && it.mstar_set) {
            sm.star_m[0] = make_float2(it.mstar_hi, it.mstar_lo);
        } else {
            const int j = it.soff + t;
            const double m = P.id[j] < 0 ? 0.0 : P.mass[j];
            const float mh = __double2float_rn(m);
            sm.star_m[t] = make_float2(mh, __double2float_rn(m - (double)mh));
        }
    }

    pdl_wait();
    pdl_trigger();

    // ---- first source tile, into registers ----
    float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th;
    D4 td{0.0, 0.0, 0.0, 0.0};
    int tid = 0;
    // FP32 modes: chunks of up to two tiles go to shared memory by cp.async at once
    const bool staged = kF32 && it.src1 - it.src0 <= 2 * kTile;
    if (t < min(kTile, it.src1 - it.src0)) {
        const int j = it.src0 + t;
        if (kF32) {
            if (!staged) {
                th = P.pos_hi_in[j];
                if (MODE == MODE_MIXED) tl = P.pos_lo_in[j];
            }
        } else {
            tid = P.id[j];
            const double m = P.mass[j];
            td = D4{P.r_in[3 * j], P.r_in[3 * j + 1], P.r_in[3 * j + 2], (MODE == MODE_FP64 && tid < 0) ? 0.0 : m};
        }
    }
    // copy group A: the positions of this stage
    if (kF32) {
        if (t < it.nsink) {
            cp_async16(&sm.snk.f.hi[t], P.pos_hi_in + it.sink0 + t);
            cp_async16(&sm.snk.f.lo[t], P.pos_lo_in + it.sink0 + t);
        }
        if (t < min(kStarBatch, it.nstar)) {
            cp_async16(&sm.star_hi[t], P.pos_hi_in + it.soff + t);
            cp_async16(&sm.star_lo[t], P.pos_lo_in + it.soff + t);
        }
        if (staged) {
            for (int k = t; k < it.src1 - it.src0; k += kTile) {
                cp_async16(&sm.src.f.hi[k], P.pos_hi_in + it.src0 + k);
                if (MODE == MODE_MIXED) cp_async16(&sm.src.f.lo[k], P.pos_lo_in + it.src0 + k);
            }
        }
    } else if (t < nel) {
        cp_async8(&sm.snk.d[t], P.r_in + 3 * it.sink0 + t);
    }
    cp_async_commit();
    if (elem) {   // copy group B: the operands the previous stage wrote
        if (need_vs) cp_async8(&ops[kOpVS][t], P.Kr[s] + x);
#pragma unroll kUnroll
        for (int q = 0; q < nk; q++) {
            const int src = op_src<VT>(V, q);
            if (src == s) cp_async8(&ops[kOpKR + q][t], P.Kr[src] + x);
            if (!(kRkf && src == V - 1) && src == s - 1) cp_async8(&ops[kOpKV + q][t], P.Kv[src] + x);
        }
    }
    cp_async_commit();

    // ---- drag factor: scalars per sink, thread t < nsink (FP64, red's gas formulas) ----
    double decr = 0.0;
    if (drag_on) {
        const double ts = P.standalone ? P.t_standalone
                                       : tsys + stage_c(P.scheme, s) * dt;
        decr = gas_reduction_factor<EXACT>(P.gas, ts);
    }
    const bool drag_act = drag_on && !(1.0e-6 > decr);
    if (drag_act && t < it.nsink) {
        const int ib = it.sink0 + t;
        double f, gx, gy;
        const double* rb = P.r_in + 3 * ib;
        const double* vb = P.Kr[s] + 3 * ib;
        if constexpr (kF32)
            drag_factor_fast(P.gas, decr, P.mass[it.soff], rb[0], rb[1], rb[2], vb[0], vb[1], vb[2], P.cd[ib],
                             P.radius[ib], P.density[ib], f, gx, gy);
        else
            drag_factor<EXACT>(P.gas, decr, P.mass[it.soff], rb[0], rb[1], rb[2], vb[0], vb[1], vb[2], P.cd[ib],
                               P.radius[ib], P.density[ib], f, gx, gy);
        sm.sc[t][0] = f;
        sm.sc[t][1] = gx;
        sm.sc[t][2] = gy;
    }
    if (kF32) {
        if (!staged) {
            if (PK && it.spt == 2) {   // the packed-pair loop streams its tiles as pair records
                put_pair<MODE>(sm, 0, t, th, tl);
            } else {
                sm.src.f.hi[t] = th;
                if (MODE == MODE_MIXED) sm.src.f.lo[t] = tl;
            }
        }
    } else {
        sm.src.d.d[t] = td;
        sm.src.d.id[t] = tid;
    }
    cp_async_wait_prior();   // the sinks and stars; the epilogue's operands may still be in flight
    __syncthreads();

    // ---- gravity of the chunk's sources ----
    float2 mine_ds = make_float2(0.f, 0.f);   // FP32 modes: double-single sums
    double mine = 0.0;                        // FP64 modes
    int mine_k;
    bool mine_ok;
    if constexpr (kF32) {
        if (PK && it.spt == 2) gravity_f32_pair<MODE>(sm, P, it, staged, th, tl, mine_ds, mine_k, mine_ok);
        else if (!PK && it.spt == 2) gravity_f32<MODE, 2>(sm, P, it, staged, th, tl, mine_ds, mine_k, mine_ok);
        else gravity_f32<MODE, 1>(sm, P, it, staged, th, tl, mine_ds, mine_k, mine_ok);
    } else {
        gravity_f64<MODE>(sm, P, it, td, tid, mine, mine_k, mine_ok);
    }
    const int mine_c = (t % it.lanes) % 3;

    // ---- source chunks of one sink tile.  In a cluster launch (FP32 modes) the
    // tile's kClusterChunks chunks are the CTAs of one cluster: each leaves its
    // partial in its shared memory and chunk 0 sums them through distributed
    // shared memory, in chunk order.  Otherwise the CTA that counts last sums
    // the partial records in global memory, every thread of it on a contiguous
    // range of chunks, in a fixed order; the chunk counter is advanced by the
    // last thread, which holds no element (3 nsink <= 96 < kTile).  The
    // one-wave instance counts without fences and re-reads a record until it
    // has landed: its launch is the critical chain of a try, and a release
    // and an acquire fence cost ~1.2 us there.  The many-wave instances keep
    // the fences, whose latency other CTAs hide, so that their reducing CTA
    // never waits on a store in flight.  The element threads form the star
    // term meanwhile ----
    constexpr bool kFencedRecords = VT >= 0;
    float2 g_ds = make_float2(0.f, 0.f);   // gravity of the element, FP32 modes
    double a = 0.0;                         // gravity of the element, FP64 modes
    float2* acc2 = reinterpret_cast<float2*>(sm.acc);
    const bool in_cluster = CL && it.nchunk > 1;   // uniform over the cluster
    if (in_cluster) {
        if (mine_ok) acc2[3 * mine_k + mine_c] = mine_ds;
        cluster_arrive();
    } else if (it.nchunk > 1) {
        if (mine_ok) {
            const long long rec = 3 * ((long long)it.part_off + (long long)it.chunk * it.nsink) + 3 * mine_k + mine_c;
            if constexpr (!kFencedRecords) {
                st_rec(reinterpret_cast<unsigned long long*>(P.partial) + rec, kF32 ? rec_bits(mine_ds) : rec_bits(mine));
            } else {
                if (kF32) reinterpret_cast<float2*>(P.partial)[rec] = mine_ds;
                else P.partial[rec] = mine;
            }
        }
        __syncthreads();
        if (t == kTile - 1) {
            if (kFencedRecords) fence_acq_rel_gpu();   // release the CTA's partial records
            const unsigned prev = atomicAdd(&P.tile_cnt[it.tile], 1u);
            const bool last = prev == (unsigned)(it.nchunk - 1);
            if (kFencedRecords && last) fence_acq_rel_gpu();   // acquire the other chunks' records
            sm.flag = last;
        }
    }

    // ---- central-star term (FP32 modes), double-single: m_j d / |d|^3 per star,
    // each element thread forming the factor of its own sink; a sum of its own,
    // added to the gravity after the reduction ----
    float2 star_ds = make_float2(0.f, 0.f);
    if (star_term && elem) {
        const float4 H = sm.snk.f.hi[ke], Lo = sm.snk.f.lo[ke];
        auto star_one = [&](float4 S, float4 SL, float2 m) {
            const float2 dx = dsn_sub(dsn(S.x, SL.x), dsn(H.x, Lo.x));
            const float2 dy = dsn_sub(dsn(S.y, SL.y), dsn(H.y, Lo.y));
            const float2 dz = dsn_sub(dsn(S.z, SL.z), dsn(H.z, Lo.z));
            const float2 r2 = dsn_add(dsn_add(dsn_sqr(dx), dsn_sqr(dy)), dsn_sqr(dz));
            const float2 ri = dsn_rsqrt(r2);
            const float2 f = dsn_mul(m, dsn_mul(dsn_sqr(ri), ri));
            star_ds = dsn_add(star_ds, dsn_mul(f, ce == 0 ? dx : (ce == 1 ? dy : dz)));
        };
        for (int q = 0; q < nst0; q++)
            if (it.soff + q != ie) star_one(sm.star_hi[q], sm.star_lo[q], sm.star_m[q]);
        for (int j = it.soff + kStarBatch; j < it.soff + it.nstar; j++) {   // more than kStarBatch stars
            if (j == ie) continue;
            const double m = P.id[j] < 0 ? 0.0 : P.mass[j];
            const float mh = __double2float_rn(m);
            star_one(P.pos_hi_in[j], P.pos_lo_in[j], make_float2(mh, __double2float_rn(m - (double)mh)));
        }
    }

    if (in_cluster) {
        cluster_wait();   // every chunk's partial is in its CTA's shared memory
        if (it.chunk == 0 && elem) {
            for (int c0 = 0; c0 < kClusterChunks; c0 += 8) {   // loads in batches of 8, sums in chunk order
                float2 v[8];
#pragma unroll
                for (int c = 0; c < 8; c++) v[c] = ld_cluster_f2(acc2 + t, (unsigned)(c0 + c));
#pragma unroll
                for (int c = 0; c < 8; c++) g_ds = dsn_add(g_ds, v[c]);
            }
        }
        cluster_arrive();   // the other chunks keep their shared memory until chunk 0 has read it
        cluster_wait();
        if (it.chunk != 0) {
            cp_async_wait_all();
            return;
        }
    } else if (it.nchunk > 1) {
        __syncthreads();
        if (!sm.flag) {        // uniform
            cp_async_wait_all();   // no copy may land in shared memory after the CTA has gone
            return;
        }
        const int nsplit = kTile / nel;
        const int sp_i = t / nel;
        const int e = t - sp_i * nel;
        const int c0 = sp_i < nsplit ? sp_i * it.nchunk / nsplit : 0;
        const int c1 = sp_i < nsplit ? (sp_i + 1) * it.nchunk / nsplit : 0;
        if constexpr (kFencedRecords) {
            const long long base = 3 * (long long)it.part_off + e;
            if (kF32) acc2[t] = sum_records_ds(reinterpret_cast<const float2*>(P.partial) + base, 3LL * it.nsink, c0, c1);
            else sm.acc[t] = sum_records(P.partial + base, 3LL * it.nsink, c0, c1);
        } else {
            unsigned long long* recs = reinterpret_cast<unsigned long long*>(P.partial) + 3 * (long long)it.part_off + e;
            bool landed;
            if (kF32) {
                float2 sum = make_float2(0.f, 0.f);
                landed = sum_polled_records(recs, 3LL * it.nsink, c0, c1, sum);
                acc2[t] = sum;
            } else {
                double sum = 0.0;
                landed = sum_polled_records(recs, 3LL * it.nsink, c0, c1, sum);
                sm.acc[t] = sum;
            }
            if (!landed) {   // RED_ERR_TIMEOUT; the system stops (k_control then leaves it alone)
                S->status = 4;
                S->halted = 1;
            }
        }
        __syncthreads();
        if (elem) {
            for (int q = 0; q < nsplit; q++) {
                if (kF32) g_ds = dsn_add(g_ds, acc2[q * nel + t]);
                else a += sm.acc[q * nel + t];
            }
        }
        if (t == 0) P.tile_cnt[it.tile] = 0u;
    } else {
        if (mine_ok) {
            if (kF32) acc2[3 * mine_k + mine_c] = mine_ds;
            else sm.acc[3 * mine_k + mine_c] = mine;
        }
        __syncthreads();
        if (elem) {
            if (kF32) g_ds = acc2[t];
            else a = sm.acc[t];
        }
    }
    if (kF32) a = dsn_to_double(dsn_add(g_ds, star_ds));

    cp_async_wait_all();

    // ---- element-wise FP64 epilogue ----
    // The combinations of variants 1 .. 14 for element e: the positions
    // y_r + dt sum_q a_q K_r,q from the stage velocity vse, and the velocities
    // y_v + dt sum_q a_q K_v,q from the element's acceleration ae.
    auto comb_r = [&](int e, double vse) -> double {
        const double yr = ops[kOpYR][e];
        if (kRkf) {
            // ytemp of stage V: y + dt * sum_q a_{V,q} K_q, terms in red's order
            // (rk8_kernel::calc_ytemp_for_f1..f12, int_rungekutta8.cu:80-246)
            const int off = 1 + V * (V - 1) / 2;
            double ar = mul<EXACT>(c_tb.a[off + op_src<VT>(V, 0)], ops[kOpKR][e]);
#pragma unroll kUnroll
            for (int q = 1; q < nk; q++) ar = madd<EXACT>(ar, c_tb.a[off + op_src<VT>(V, q)], ops[kOpKR + q][e]);
            return madd<EXACT>(yr, dt, ar);
        } else if (V == 13) {
            // rk4_kernel::sum_vector, int_rungekutta4.cu:36-47: y + (a dt) K_s
            const double bf = mul<EXACT>(P.scheme == SCHEME_RK2 ? c_tb.a2[s + 1] : c_tb.a4[s + 1], dt);
            return madd<EXACT>(yr, bf, vse);
        } else {
            // RK4 y_{n+1} as the positions of the adaptive stage 4
            const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
            return rk4_ynp1<EXACT>(yr, b0, b1, ops[kOpKR][e], ops[kOpKR + 1][e], ops[kOpKR + 2][e], vse);
        }
    };
    auto comb_v = [&](int e, double ae) -> double {
        const double yv = ops[kOpYV][e];
        if (kRkf) {
            const int off = 1 + V * (V - 1) / 2;
            const int s0 = op_src<VT>(V, 0);
            double av = mul<EXACT>(c_tb.a[off + s0], (s0 == V - 1) ? ae : ops[kOpKV][e]);
#pragma unroll kUnroll
            for (int q = 1; q < nk; q++) {
                const int sq = op_src<VT>(V, q);
                av = madd<EXACT>(av, c_tb.a[off + sq], (sq == V - 1) ? ae : ops[kOpKV + q][e]);
            }
            return madd<EXACT>(yv, dt, av);
        } else if (V == 13) {
            const double bf = mul<EXACT>(P.scheme == SCHEME_RK2 ? c_tb.a2[s + 1] : c_tb.a4[s + 1], dt);
            return madd<EXACT>(yv, bf, ae);
        } else {
            const double b0 = mul<EXACT>(c_tb.b4[0], dt), b1 = mul<EXACT>(c_tb.b4[1], dt);
            return rk4_ynp1<EXACT>(yv, b0, b1, ops[kOpKV][e], ops[kOpKV + 1][e], ops[kOpKV + 2][e], ae);
        }
    };
    // The one-wave instance with at most kTile / 2 elements (the large-body
    // tiles, whose epilogue ends the launch) forms the position and velocity
    // combinations of an element on two threads, t and t + kTile / 2, in
    // different warps: each warp issues half the FP64 instructions.  The
    // acceleration passes through sm.acc, whose slot t only thread t has read.
    if constexpr (VT >= 0) {
        if (!elem) return;
    }
    const double vs = (elem && need_vs) ? ops[kOpVS][t] : 0.0;   // stage velocity of the element
    if (elem) {
        if (!(idi > 0)) a = 0.0;   // calc_grav_accel_naive zeroes inactive sinks (pp_disk.cu:386-388)
        if (drag_act) {
            const double g = ce == 0 ? sm.sc[ke][1] : (ce == 1 ? sm.sc[ke][2] : 0.0);
            a = add<EXACT>(a, mul<EXACT>(sm.sc[ke][0], sub<EXACT>(g, vs)));   // a[i] += f u (pp_disk.cu:516-518)
        }
        P.Kv[s][x] = a;
    }
    if (VT < 0 && V >= 1 && V <= 14 && 2 * nel <= kTile) {   // uniform over the CTA
        if (elem) sm.acc[t] = a;
        __syncthreads();   // the accelerations and every element's cp.async operands
        const bool vside = t >= kTile / 2;
        const int e = vside ? t - kTile / 2 : t;
        if (e >= nel) return;
        const int xe = 3 * it.sink0 + e;
        if (vside) {
            P.Kr[P.next][xe] = comb_v(e, sm.acc[e]);
        } else {
            const double orr = comb_r(e, need_vs ? ops[kOpVS][e] : 0.0);
            P.r_out[xe] = orr;
            write_pos_c(P.pos_hi_out, P.pos_lo_out, it.sink0 + e / 3, e % 3, orr);   // k_prep holds the .w words
        }
        return;
    }
    if (!elem) return;

    if (V >= 1 && V <= 14) {
        const double orr = comb_r(t, vs);
        P.r_out[x] = orr;
        P.Kr[P.next][x] = comb_v(t, a);
        write_pos_c(P.pos_hi_out, P.pos_lo_out, ie, ce, orr);   // x, y, z; k_prep holds the .w words
    } else if (V == 15 || V == 16) {
        double e = 0.0;
        if (ie - it.soff < it.nerr) {
            double er, ev;
            if (V == 15) {
                // rk8_kernel::calc_error, int_rungekutta8.cu:248-260
                er = fabs(sub<EXACT>(sub<EXACT>(add<EXACT>(ops[kOpKR][t], ops[kOpKR + 1][t]), ops[kOpKR + 2][t]), vs));
                ev = fabs(sub<EXACT>(sub<EXACT>(add<EXACT>(ops[kOpKV][t], ops[kOpKV + 1][t]), ops[kOpKV + 2][t]), a));
            } else {
                // rk4_kernel::calc_error, int_rungekutta4.cu:62-73
                er = fabs(ops[kOpKR][t] - vs);
                ev = fabs(ops[kOpKV][t] - a);
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

// Launches k_stage for variant v (stage_variant): one kernel per mode serves
// every stage of a try, so its code stays in the caches from stage to stage.
// Clusters of kClusterChunks CTAs are above the portable 8.
template <int MODE, bool EXACT>
void stage_attributes()
{
    static const bool done = [] {
        cudaFuncSetAttribute(k_stage<MODE, EXACT, true, -1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        return true;
    }();
    (void)done;
}

template <int MODE, bool EXACT, int VT>
void launch_fixed(const StageParams& P, int n, int v, cudaStream_t s)
{
    // plans of 2-sink tiles on 8 lanes (P.packed, FP32 modes): the packed-pair
    // instance, 6 CTAs per SM (its pair loop needs the registers of the seventh)
    if constexpr (MODE == MODE_MIXED || MODE == MODE_FP32) {
        if (P.packed) {
            launch_k(k_stage<MODE, EXACT, false, VT, true>, (unsigned)n, (unsigned)kTile, s, P, v);
            return;
        }
    }
    launch_k(k_stage<MODE, EXACT, false, VT>, (unsigned)n, (unsigned)kTile, s, P, v);
}

// A cluster plan takes the cluster instance, a plan of one wave the instance
// with the variant as an argument, a plan of many waves the variant's own.
template <int MODE, bool EXACT>
void launch_stage_variant(const StageParams& P, int n, int v, cudaStream_t s)
{
    if constexpr (MODE == MODE_MIXED || MODE == MODE_FP32) {
        if (P.cluster) {
            stage_attributes<MODE, EXACT>();
            launch_kx(k_stage<MODE, EXACT, true, -1>, (unsigned)n, (unsigned)kTile, (unsigned)kClusterChunks, s, P,
                      v);
            return;
        }
    }
    if (P.one_wave) {
        launch_k(k_stage<MODE, EXACT, false, -1>, (unsigned)n, (unsigned)kTile, s, P, v);
        return;
    }
    switch (v) {
    case 1: launch_fixed<MODE, EXACT, 1>(P, n, v, s); break;
    case 2: launch_fixed<MODE, EXACT, 2>(P, n, v, s); break;
    case 3: launch_fixed<MODE, EXACT, 3>(P, n, v, s); break;
    case 4: launch_fixed<MODE, EXACT, 4>(P, n, v, s); break;
    case 5: launch_fixed<MODE, EXACT, 5>(P, n, v, s); break;
    case 6: launch_fixed<MODE, EXACT, 6>(P, n, v, s); break;
    case 7: launch_fixed<MODE, EXACT, 7>(P, n, v, s); break;
    case 8: launch_fixed<MODE, EXACT, 8>(P, n, v, s); break;
    case 9: launch_fixed<MODE, EXACT, 9>(P, n, v, s); break;
    case 10: launch_fixed<MODE, EXACT, 10>(P, n, v, s); break;
    case 11: launch_fixed<MODE, EXACT, 11>(P, n, v, s); break;
    case 12: launch_fixed<MODE, EXACT, 12>(P, n, v, s); break;
    case 13: launch_fixed<MODE, EXACT, 13>(P, n, v, s); break;
    case 14: launch_fixed<MODE, EXACT, 14>(P, n, v, s); break;
    case 15: launch_fixed<MODE, EXACT, 15>(P, n, v, s); break;
    case 16: launch_fixed<MODE, EXACT, 16>(P, n, v, s); break;
    default: launch_fixed<MODE, EXACT, 0>(P, n, v, s); break;
    }
}

// Clusters of kClusterChunks stage CTAs that can be resident at once (FP32
// modes; 0 if the query fails).
template <int MODE, bool EXACT>
int stage_active_clusters()
{
    stage_attributes<MODE, EXACT>();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kClusterChunks);
    cfg.blockDim = dim3(kTile);
    cfg.dynamicSmemBytes = 0;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kClusterChunks;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_stage<MODE, EXACT, true, -1>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace redgb
