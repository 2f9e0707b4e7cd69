// Internal definitions shared by the CUDA translation units of libvvgpu.
//
// Device layout (structure of arrays, one context per Space):
//   vortices  x, y, g, ie (= TObj::_1_eps), vx, vy : double[n]; orig : int64[n]
//   segments  corner, r, dl, ie, g, fric, gsum     : double[m] (all bodies concatenated)
//   nodes     geom (x, y, h, w) : double4[nn]; vortex range vf/vl, segment range sf/sl,
//             first child ch1 (ch2 = ch1 + 1, -1 for a leaf), depth, path bits,
//             +/- centroids cm (px, py, pg, mx, my, mg)
//   leaves    in bottomNodes (depth-first) order, which is also increasing vortex index
//   near      per leaf, runs of consecutive leaves (each run is one contiguous vortex range)
//   far       per leaf, node ids in depth-first order
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vvgpu.h"
#include "stage.cuh"

namespace vvgpu {

constexpr double C_PI = 3.14159265358979323846;
constexpr double C_2PI = 2. * C_PI;
constexpr double C_1_2PI = 1. / (2. * C_PI);
constexpr double C_1_PI = 1. / C_PI;
constexpr int TREE_MAX_LIST_SIZE = 16;   // TSortedTree.cpp:10
constexpr double EXP_ARG_RESTRICTION = -8.;  // MDiffusiveFast.cpp:6
constexpr double REMOVE_EPS = 1e-10;         // MFlowmove.hpp:8
constexpr int MAX_DEPTH = 62;            // path bits are kept in an int64

struct CudaError {
    cudaError_t err;
    const char* what;
};

#define VV_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) throw ::vvgpu::CudaError{e_, #call};            \
    } while (0)

// Checks the last launch and counts it in the context (c must be in scope).
#define VV_LAUNCH_CHECK()                   \
    do {                                    \
        VV_CUDA(cudaGetLastError());        \
        ++c.launches;                       \
    } while (0)

struct ApiError {
    int code;
    std::string msg;
};

// Growable device array (capacity only grows; contents not preserved on growth unless asked).
template <class T>
struct DArr {
    T* p = nullptr;
    size_t cap = 0;
    DArr() = default;
    DArr(const DArr&) = delete;
    DArr& operator=(const DArr&) = delete;
    DArr(DArr&& o) noexcept : p(o.p), cap(o.cap) { o.p = nullptr; o.cap = 0; }
    DArr& operator=(DArr&& o) noexcept {
        if (this != &o) { release(); p = o.p; cap = o.cap; o.p = nullptr; o.cap = 0; }
        return *this;
    }
    ~DArr() { release(); }
    void reserve(size_t n, bool keep = false, size_t keep_n = 0, cudaStream_t s = 0) {
        if (n <= cap) return;
        size_t nc = cap ? cap : 256;
        while (nc < n) nc *= 2;
        T* q = nullptr;
        cudaError_t e = cudaMalloc(&q, nc * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw ApiError{VVGPU_ERR_NOMEM, "cudaMalloc failed"};
        }
        if (keep && p && keep_n) VV_CUDA(cudaMemcpyAsync(q, p, keep_n * sizeof(T), cudaMemcpyDeviceToDevice, s));
        if (p) {
            if (keep) VV_CUDA(cudaStreamSynchronize(s));
            cudaFree(p);
        }
        p = q;
        cap = nc;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// The smoothing of a sink scales with abs(src.g), written in MConvectiveFast.cpp:166 without
// std:: and without a global abs(double) in scope: C's int abs(int) runs on the circulation
// truncated to int, so sinks with |g| < 1 are unsmoothed.
__host__ __device__ __forceinline__ double sink_abs(double g) { return (double)abs((int)g); }

struct BodyHost {
    int64_t first, count;
    vvgpu_body_params p;
    double slen, area, cofm_x, cofm_y, moi_cofm;
    double friction_x = 0, friction_y = 0, friction_o = 0, nusselt = 0;  // TBody::friction, nusselt
};

struct Ctx {
    int device = 0;
    int precision = VVGPU_FP64;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // second stream for work that runs beside the main stream's kernels within one call
    // (forked and joined through the two events); created on first use
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // list download beside later calls (vvgpu_get_vortices_async): device snapshot of x, y,
    // g, ie, orig (5 n words), copy stream, snapshot-taken and copies-done events
    DArr<double> dl_snap;
    cudaStream_t dl_stream = nullptr;
    cudaEvent_t dl_ready = nullptr, dl_done = nullptr;
    bool dl_pending = false;
    std::string last_error;

    double re = 1.0 / 0.0, dt = 1.0, inf_vx = 0, inf_vy = 0, inf_g = 0, time = 0, grav_x = 0, grav_y = 0;

    // vortices
    int64_t n = 0;
    DArr<double> x, y, g, ie, vx, vy;
    DArr<int64_t> orig;
    int64_t next_orig = 0;
    // input check of the last vvgpu_set_vortices* (non-finite values), read on first use
    DArr<int32_t> in_bad;
    bool in_pending = false;
    // fixed-point rounds the epsilon/merge pass may take (vvgpu_set_eps_round_limit)
    int64_t eps_max_rounds = 4096;
    uint32_t wait_spins = STAGE_SPINS;  // polls of one shared-memory staging wait
    int32_t* h_pin = nullptr;           // 512 pinned host bytes for the small device reads of a step
    // kernel shapes of the FP32 pair passes (vvgpu_autotune_tiles): sources per staged tile
    // of the convective near field (256 by default), shape of the diffusive pass (1: 16
    // targets, 2: 8 per pass)
    int conv_tile = 256, diff_targets = 1;
    bool tune_pending = false;  // tune both at the next convective pass

    // segments (host copies of geometry are kept for body bookkeeping)
    int64_t m = 0;
    std::vector<double> h_cx, h_cy, h_rx, h_ry, h_dlx, h_dly, h_sie;
    std::vector<uint32_t> h_slip;
    std::vector<BodyHost> bodies;
    DArr<double> s_cx, s_cy, s_rx, s_ry, s_dlx, s_dly, s_ie, s_g, s_fric, s_gsum;
    DArr<double> s_cp, s_fr, s_nu;  // TAtt::Cp, Fr, Nu (Space::calc_forces accumulators)
    DArr<int64_t> f_fc;
    DArr<double> f_out;
    DArr<uint32_t> s_slip;
    std::vector<double> h_att;       // attached sheets: per segment speed x, y, o and axis x, y
    std::vector<int32_t> h_att_on;   // ... of a body whose speed_slae is not zero
    DArr<double> s_att;
    DArr<int32_t> s_att_on;
    bool segs_dirty = true;
    // sinks
    int64_t ns = 0;
    DArr<double> k_x, k_y, k_g;

    // tree
    bool built = false;
    bool lists_full = false;        // near runs of every leaf (else only of segment leaves)
    double far_criteria = 8, min_node = 0, max_node = 0;
    int64_t nnodes = 0, nleaves = 0, depth = 0;
    std::vector<int64_t> level_begin;
    DArr<double4> nd_geom;          // x, y, h, w
    DArr<int32_t> nd_vf, nd_vl, nd_sf, nd_sl, nd_ch1, nd_depth;
    DArr<int64_t> nd_path;
    DArr<double> nd_cm;             // 6 per node: px, py, pg, mx, my, mg
    DArr<unsigned long long> nd_bbox;  // 4 per node: encoded min x, min y, max x, max y
    DArr<double> nd_pivot;
    DArr<int32_t> nd_axis, nd_split, nd_nlow, nd_nlow_s, nd_lc, nd_dfs;
    DArr<int32_t> seg_node_of, seg_node_of2, flags, scan;
    DArr<int32_t> perm;              // tree build: source slot of each slot (keys move, payload follows once)
    DArr<int32_t> nd_cbase, nd_npair;  // tree build: node's first chunk, pairs swapped in its split
    DArr<int32_t> nd_parent, nd_arrive;  // tree build: parent node; children arrived (bottom-up pass)
    DArr<int32_t> lvl_cnt;           // tree build: per-level counts of warp-split nodes and of chunks
    DArr<int32_t> lvl_list;          // tree build: per-level list of warp-split nodes
    DArr<int32_t> chunk_node, chunk_cnt, chunk_pre;  // tree build: per-level chunks of the larger nodes
    DArr<int32_t> sel_pos, sel_list, lf_fallback;  // leaves walked one warp each
    int64_t n_sel = 0, n_fallback = 0;
    DArr<double> ptmp;               // tree build: payload staging for the final permutation
    DArr<int64_t> otmp;
    DArr<int32_t> tab_lh, tab_rl;
    DArr<int32_t> seg_order, seg_order2;
    DArr<int32_t> leaf_node;        // DFS order -> node id
    DArr<int32_t> lf_vf, lf_vl, lf_sf, lf_sl;
    DArr<double4> lf_geom;
    DArr<int32_t> near_off, far_off, near_cnt, far_cnt;
    DArr<int2> near_run;
    DArr<int32_t> far_node;         // far lists of flagged leaves only (see lists.cu)
    DArr<int32_t> lf_flag;          // leaf holds a segment centre
    DArr<int2> run_buf;             // warp walk: fixed-capacity near runs per leaf
    DArr<int32_t> lf_overflow;      // leaf had more runs than the buffer holds
    DArr<double4> lf_taylor;        // far-field expansion coefficients T1..T4 per leaf
    // far nodes of every leaf, kept by the warp walk when keep_far is set (learned far field)
    bool keep_far = false, far_kept = false;
    DArr<int32_t> far_buf, lf_far_cnt, lf_far_off, lf_far_node, lf_far_leaf;  // lf_far_leaf: the leaf's node id
    int64_t n_far_pairs = 0;
    // learned far field (learned_step.cu): per-node 64-byte input records, per-pair
    // corrections, corrected coefficients, the judge's samples and results
    DArr<uint4> ln_rec;
    DArr<double4> lf_taylor_l;
    DArr<float2> ln_pv;
    DArr<double> ln_v0, ln_judge;
    DArr<int32_t> ln_idx;
    uint64_t judge_calls = 0;
    int taylor_precision = 0;
    DArr<float4> nf_geo, nf_cm;     // per node, anchor frame: centre + (h+w); centroids
    DArr<float2> nf_k;              // per node anchor (FP32, exact)
    DArr<float2> nf_g;              // per node centroid circulations
    DArr<float4> nf_rec;            // per node packed walk record (4 x float4)
    int64_t n_near_runs = 0, n_far = 0;
    DArr<int32_t> leaf_of;          // vortex -> leaf (DFS index)

    // scratch for reductions / counters
    DArr<unsigned long long> counters;
    DArr<double> sum_part;          // partial sums of the deterministic reductions
    DArr<double> nd_mom;            // learned correction: per node complex moments M2..M4 of each sign
    bool mom_valid = false;
    DArr<int32_t> scan_tmp;

    // epsilon / merge (fixed-point rounds; [2] = double buffer)
    DArr<int32_t> e_partner[2], e_zb, e_changed;
    DArr<double> e_x0, e_y0, e_g0, e_ox[2], e_oy[2], e_og[2], e_oie[2];
    DArr<float4> e_rec0, e_recO[2];
    DArr<int32_t> e_vch, e_chg, e_nchg;  // per vortex: outcome changed; per leaf: changed near leaves
    DArr<float> e_sr1, e_sr2;            // per vortex: search radii^2 of its last evaluation
    DArr<float4> e_box_prev;             // per leaf: the last round's box
    DArr<float> e_rreg;                  // per leaf: largest search radius^2 of its members
    DArr<int32_t> e_lchg_pre;            // exclusive prefix sums of the changed-leaf flags
    DArr<int32_t> e_flag, e_pos, e_list; // targets to evaluate in a round (flags, offsets, list)
    // move_and_clean
    DArr<double> mv_bodies, mv_acc;      // per body inside-test geometry; bookkeeping sums
    DArr<int32_t> mv_dead, mv_dpos, mv_list;
    DArr<int2> mv_at;
    std::vector<int64_t> h_bfc;          // body first segments, then counts
    DArr<int64_t> e_bfc;
    DArr<float2> e_seg32;                // segment centres in FP32 relative to their body's anchor
    DArr<double2> e_banchor;
    DArr<float> e_brad;
    DArr<double> lf_mcs, lf_epr;
    DArr<int32_t> e_zb_prev, e_live, e_cand, e_ncand, e_dirty, e_lchanged;
    DArr<float> e_rlist, e_rnear;
    DArr<int32_t> e_ldisp;          // per leaf: largest merge displacement of its members (float bits)
    DArr<float> e_dloc;             // per leaf: bound on e_ldisp over its near leaves (as last computed)
    DArr<int32_t> e_chglist;        // the changed leaves in order (rank = e_lchg_pre)

    // local FP32 frames (frame.cuh)
    double frame_G = 1.0;
    DArr<float2> lf_anchor;
    DArr<float4> lf_box32;          // per leaf: min x, min y, max x, max y in its own frame
    DArr<float> lf_rn;              // per leaf: extent of its near region in its frame
    DArr<float4> src32;             // per vortex: x, y in own leaf frame, g, eps^2
    DArr<float2> src_k;             // per vortex: anchor of its leaf
    DArr<float> src_ie;             // per vortex: (float)_1_eps
    DArr<float4> src_a4;            // per vortex: anchor of its leaf (x, y, 0, 0), 16-byte records
    DArr<int2> run_js;              // per near run: first source slot, offset in its leaf's near sequence
    DArr<int32_t> np_nz, np_pre;    // near-pair count: non-zero vortices per leaf and their prefix
    DArr<int32_t> leaf_tot;         // per leaf: length of its near sequence
    DArr<float4> lf_dbox;           // per leaf (diffusive): box of non-zero vortices and segment centres

    // SLAE
    int64_t neq = 0;
    DArr<double> A, B, X, Acache, LU, inv;
    DArr<float> inv32;
    DArr<int32_t> piv;
    bool lu_valid = false;
    int lu_precision = 0;
    int64_t neq_cached = 0;
    std::vector<double> slae_sig;   // inputs of the matrix in A (A is reused while they are equal)
    uint64_t seg_version = 0;       // bumped whenever the segment geometry changes
    DArr<int32_t> sub_i32;          // subtree pass: roots, new-node counts, their prefix
    DArr<double4> sub_scratch;      // subtree pass: node records (two double4 per record)
    DArr<int32_t> slae_maps;        // column / row maps of the system
    DArr<double> slae_bodies;       // per-body row data
    DArr<double> slae_r, slae_sq;   // refinement residual and its squared terms
    DArr<float2> slae_vs;           // a vector split into FP32 pairs for the FP32 inverse
    vvgpu_stats stats{};
    // per-kernel device time (vvgpu_set_kernel_timing): event pairs recorded on the stream,
    // summed per slot when the host asks
    bool timing = false;
    std::vector<cudaEvent_t> ev_free;
    struct TimedLaunch { int slot; cudaEvent_t a, b; };
    std::vector<TimedLaunch> ev_rec;
    double t_ms[VVGPU_T_COUNT] = {};
    int64_t t_count[VVGPU_T_COUNT] = {};
    int64_t launches = 0;           // kernels launched by this context
    int64_t eps_evaluations = 0;    // target evaluations over the rounds of the last epsilon pass
    int64_t eps_records = 0;        // candidate records read by those evaluations' FP32 passes
    int64_t walk_loads = 0;         // node records loaded by the warps of the last full walk
    int64_t diff_sources = 0;       // sources in the candidate leaves of every diffusive target chunk
    bool count_pairs = true;        // count algorithmic near pairs before each convective pass

    cudaStream_t st() const { return stream; }
};

// Device time of the work queued on the context's stream while an instance lives, added to
// slot `slot` of the kernel timing (nothing is recorded while timing is off).
struct KernelTimer {
    Ctx& c;
    int slot;
    cudaEvent_t a = nullptr;
    KernelTimer(Ctx& cc, int sl) : c(cc), slot(sl) {
        if (!c.timing) return;
        a = take();
        if (a && cudaEventRecord(a, c.st()) != cudaSuccess) { c.ev_free.push_back(a); a = nullptr; }
    }
    ~KernelTimer() {
        if (!a) return;
        cudaEvent_t b = take();
        if (b && cudaEventRecord(b, c.st()) == cudaSuccess) c.ev_rec.push_back({slot, a, b});
        else {
            c.ev_free.push_back(a);
            if (b) c.ev_free.push_back(b);
        }
    }
    cudaEvent_t take() {
        if (!c.ev_free.empty()) {
            cudaEvent_t e = c.ev_free.back();
            c.ev_free.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
    }
};
// Folds the recorded event pairs into t_ms / t_count (synchronises on the last one).
void collect_kernel_timing(Ctx& c);

// The context's side stream (and its fork / join events), created on first use.
inline cudaStream_t side_stream(Ctx& c) {
    if (!c.side) {
        VV_CUDA(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
        VV_CUDA(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming));
        VV_CUDA(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming));
    }
    return c.side;
}

// ---- exact FP64 arithmetic (no FMA contraction: the reference is built without FMA) ----
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dabs2(double x, double y) { return dadd(dmul(x, x), dmul(y, y)); }
// std::max / std::min as libstdc++ defines them
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dsgn(double v) { return (v > 0) ? 1. : ((v < 0) ? -1. : 0.); }
// Compensated FP32 accumulation (Knuth's TwoSum): hi + lo carries the running sum.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float v) {
    float s = hi + v;
    float bp = s - hi;
    lo += (hi - (s - bp)) + (v - bp);
    hi = s;
}

// Order-preserving map double -> uint64 for atomicMin/atomicMax on doubles.
__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
    unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}
// x < p on the integer pipe (sm_103's FP64 pipe is narrow): order-preserving keys with -0
// folded onto +0, and NaN never below, as the IEEE comparison.  kp = lt_key_of(p), p not NaN.
__device__ __forceinline__ unsigned long long lt_key_of(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    if ((u << 1) == 0ull) u = 0ull;
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ bool lt_key(double x, unsigned long long kp) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return lt_key_of(x) < kp && (u & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull;
}
inline unsigned long long dkey_host(double v) {
    unsigned long long u;
    memcpy(&u, &v, 8);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Warp-cooperative iteration over the leaves of the near runs [r0, r1).  Every lane calls
// f(q, valid) the same number of times, so f may use warp votes; q is a near leaf when
// valid.  Runs are taken 32 at a time, their lengths prefix-summed across the lanes into s
// (32 entries of per-warp shared memory), and each lane finds its run by binary search: all
// lanes stay busy however short the runs are.  Leaves come in near-list order, 32 per call.
template <class F>
__device__ __forceinline__ void for_near_leaves(const int2* __restrict__ near_run, int32_t r0, int32_t r1, int2* s,
                                                F&& f) {
    const int lane = threadIdx.x & 31;
    for (int32_t rb = r0; rb < r1; rb += 32) {
        const int32_t rr = rb + lane;
        int32_t first = 0, len = 0;
        if (rr < r1) {
            const int2 run = near_run[rr];
            first = run.x;
            len = run.y - run.x;
        }
        int32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const int nrun = min(32, r1 - rb);
        __syncwarp();
        s[lane] = make_int2(incl - len, first);
        __syncwarp();
        for (int32_t kb = 0; kb < total; kb += 32) {
            const int32_t k = kb + lane;
            int lo = 0, hi = nrun - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s[mid].x <= k) lo = mid;
                else hi = mid - 1;
            }
            const int2 e = s[lo];
            f(e.y + (k - e.x), k < total);
        }
    }
    __syncwarp();
}

// Calls f(q, ok) for the near leaves of [r0, r1) that are in the ranked list `list` (for
// each leaf q of a run [x, y), the ones with pre[x] <= rank < pre[y], list[rank] = q), in
// the order of for_near_leaves; ok is false (and q = 0) for the padding lanes.
template <class F>
__device__ __forceinline__ void for_listed_near_leaves(const int2* __restrict__ near_run, int32_t r0, int32_t r1,
                                                       const int32_t* __restrict__ pre,
                                                       const int32_t* __restrict__ list, int2* s, F&& f) {
    const int lane = threadIdx.x & 31;
    for (int32_t rb = r0; rb < r1; rb += 32) {
        const int32_t rr = rb + lane;
        int32_t first = 0, len = 0;
        if (rr < r1) {
            const int2 run = near_run[rr];
            first = pre[run.x];
            len = pre[run.y] - first;
        }
        int32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const int nrun = min(32, r1 - rb);
        __syncwarp();
        s[lane] = make_int2(incl - len, first);
        __syncwarp();
        for (int32_t kb = 0; kb < total; kb += 32) {
            const int32_t k = kb + lane;
            int lo = 0, hi = nrun - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s[mid].x <= k) lo = mid;
                else hi = mid - 1;
            }
            const int2 e = s[lo];
            const bool ok = k < total;
            f(ok ? list[e.y + (k - e.x)] : 0, ok);
        }
    }
    __syncwarp();
}

inline unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return (unsigned)g;
}

// ---- scan.cu ----
// Exclusive prefix sum of n int32 values into out[0..n] (out[n] = total).
void exclusive_scan(Ctx& c, const int32_t* in, int32_t* out, int64_t n);
// Reads one int32 from device memory (synchronises the stream).
int32_t read_i32(Ctx& c, const int32_t* p);
// Host landing place of a small device read at byte `off` of the context's pinned block
// (bytes: 0 read_i32, 16 tree counts, 64 root box, 96 staging error, 104 diffusive
// counts, 120 near-pair count, 128 epsilon counters, 160 residual norms), or `fallback`
// without the block.
template <class T>
inline T* pinned_at(Ctx& c, size_t off, T* fallback) {
    return c.h_pin ? reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(c.h_pin) + off) : fallback;
}

// ---- per-module entry points (throw ApiError / CudaError) ----
void ensure_vortex_capacity(Ctx& c, int64_t n, bool keep);
// VVGPU_ERR_ARG if the last vortex list set holds a non-finite position or circulation or a
// NaN / negative inverse epsilon (reads the device flag once per list; synchronises).
void check_input(Ctx& c);
// Leaf anchors (frame.cuh) and per-leaf FP32 boxes of the current vortex positions.
void build_frames(Ctx& c);
void tree_build(Ctx& c, double far_criteria, double min_node, double max_node);
// Node frames plus the near runs and far lists of the leaves holding a segment centre
// (all the SLAE right-hand side reads).
void tree_lists(Ctx& c);
// Near runs and far-field coefficients of every leaf, built once per tree on first use.
void ensure_full_lists(Ctx& c);
// Compacts the far nodes the walk kept (keep_far) into lf_far_off / lf_far_node / lf_far_leaf.
void keep_far_lists(Ctx& c);
// Far lists by an exact FP64 walk (inspection): offsets, and the nodes when fill is set.
void tree_lists_exact(Ctx& c, std::vector<int32_t>& far_off, std::vector<int32_t>& far_node, bool fill);
void eps_pass(Ctx& c, int merge, int64_t* merged);
// the learned far field in the convective pass with its judge (learned_step.cu)
void convective_learned(Ctx& c, vvgpu_mlp& M, const vvgpu_judge_cfg* jc, vvgpu_judge_out* jo);
void convective(Ctx& c);
void autotune_tiles(Ctx& c, double* ms);
void velocity_points(Ctx& c, int64_t n, const double* px, const double* py, double* vx, double* vy);
void velocity_points_on_device(Ctx& c, int64_t n, const double* dpx, const double* dpy, double* dvx, double* dvy);
void direct_velocity(Ctx& c, int64_t n, const double* px, const double* py, double* vx, double* vy);
// velocity(p) at the vortices d_idx[0 .. nt) with the near/far split of far criterion fc on
// the built tree (the learned far field's judge); d_out: (vx, vy, valid) per target.
void judge_velocity(Ctx& c, int64_t nt, const int32_t* d_idx, double fc, double* d_out);
// Its vortex part by a warp-per-target level walk (lists.cu); out[3 q + 2] = -1 where the walk
// did not fit its buffers.
void judge_walk(Ctx& c, int64_t nt, const int32_t* d_idx, double fc, double* d_out);
// The same by one FP64 walk per target (any size).
void judge_velocity_exact(Ctx& c, int64_t nt, const int32_t* d_idx, double fc, double* d_out);
// TVec3D::iszero of every body's speed_slae (TVec3D.hpp:17), else VVGPU_ERR_UNSUPPORTED.
void check_bodies_at_rest(Ctx& c);
// grid fields (fields.cu)
void field_velocity(Ctx& c, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres, char mode,
                    char ref_frame, float* out);
void field_streamfunction(Ctx& c, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                          double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                          uint16_t* gap_yj, float* gap, int64_t* ngaps);
void field_vorticity(Ctx& c, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres, double eps_mult,
                     float* out);
void diffusive(Ctx& c);
void slae(Ctx& c, vvgpu_body_out* out);
void upload_segments(Ctx& c);
void vortex_shed(Ctx& c);
void move_and_clean(Ctx& c, int remove, int64_t* cleaned);
void calc_forces(Ctx& c, double* out4);
void zero_forces(Ctx& c);
double gsum(Ctx& c);

}  // namespace vvgpu

// The opaque handle of include/vvgpu.h.
struct vvgpu_ctx {
    vvgpu::Ctx c;
};
