// Near/far classification per leaf (snode::FindNearNodes, libvvhd/src/TSortedTree.cpp:199-217)
// fused with the far-field expansion of the convective velocity
// (MConvectiveFast::process_all_lists, libvvhd/src/MConvectiveFast.cpp:48-69).
//
// A leaf's depth-first walk decides "far" when |dc|^2 > farCriteria (h+w+h'+w')^2.  The
// test runs in FP32 on anchor-relative node centres (frame.cuh); only when the two sides are
// within a relative 2^-16 of each other is it repeated in FP64 with the reference's
// operation order, so every decision equals the reference's.
//
// Near leaves come out in depth-first order (increasing leaf index) and are stored as runs
// of consecutive leaves, i.e. contiguous vortex ranges.  Far nodes are not stored: the walk
// folds each far node's two monopoles straight into the leaf's expansion coefficients
// T1..T4 (the reference computes the same coefficients from the same centroids, which are
// fixed when the tree is built).  Far lists are kept only for leaves that hold a segment
// centre (the SLAE right-hand side reads them), and an exact walk rebuilds full lists on
// request for inspection.
#include <cfloat>

#include "frame.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr int LB = 128;

struct ListView {
    const double4* geom;     // exact node geometry
    const int32_t* ch1;
    const int32_t* dfs;
    const float4* nf_geo;    // x, y (anchor frame), h + w, 0
    const float2* nf_k;      // node anchors (FP32, exact)
    const float4* nf_cm;     // CMp x, y, CMm x, y (anchor frame)
    const float2* nf_g;      // CMp g, CMm g
    const double* cm;        // exact centroids (6 per node)
    const float4* rec;       // packed per-node record (4 x float4, see k_node_frames)
    double fc;
    float fcf;
    float Gf;
};

// Exact FP64 far test with the reference's operation order.
__device__ __forceinline__ bool far_exact(const double4& tg, const double4& me, double fc) {
    double dx = dsub(tg.x, me.x), dy = dsub(tg.y, me.y);
    double hp = dadd(dadd(dadd(tg.z, tg.w), me.z), me.w);
    return dabs2(dx, dy) > dmul(dmul(fc, hp), hp);
}

// FP32 filter, FP64 on the boundary; node data given.
__device__ __forceinline__ bool far_test_at(const ListView& v, float4 tg, float2 tk, int32_t t, int32_t meN, float4 mg,
                                            float2 mk) {
    float dx = (tk.x - mk.x) + (tg.x - mg.x);
    float dy = (tk.y - mk.y) + (tg.y - mg.y);
    float lhs = dx * dx + dy * dy;
    float hp = tg.z + mg.z;
    float rhs = v.fcf * hp * hp;
    if (isfinite(lhs) && isfinite(rhs)) {
        const float m = 1.52587890625e-05f;  // 2^-16
        if (lhs > rhs * (1.f + m) + 1e-37f) return true;
        if (lhs < rhs * (1.f - m) - 1e-37f) return false;
    }
    return far_exact(v.geom[t], v.geom[meN], v.fc);
}

__device__ __forceinline__ bool far_test(const ListView& v, int32_t t, int32_t meN, float4 mg, float2 mk) {
    return far_test_at(v, v.nf_geo[t], v.nf_k[t], t, meN, mg, mk);
}

// Packed node record: everything a walk reads about node t, in one 64-byte line.
//   r0 = centre x, y (anchor frame), h + w, first child (int bits, -1 for a leaf)
//   r1 = anchor x, y, depth-first leaf index (int bits, leaves only), 0
//   r2 = CMp x, y, CMm x, y (anchor frame)      r3 = CMp g, CMm g, 0, 0
struct NodeRec {
    float4 r0, r1, r2, r3;
};
__device__ __forceinline__ NodeRec load_rec(const float4* __restrict__ rec, int32_t t) {
    const float4* p = rec + 4 * (size_t)t;
    return NodeRec{p[0], p[1], p[2], p[3]};
}

__global__ void k_node_frames(int64_t nn, const double4* __restrict__ geom, const double* __restrict__ cm, double G,
                              const int32_t* __restrict__ ch1, const int32_t* __restrict__ dfs, float4* nf_geo,
                              float2* nf_k, float4* nf_cm, float2* nf_g, float4* rec) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nn) return;
    double4 gm = geom[k];
    double cx = isfinite(gm.x) ? gm.x : 0., cy = isfinite(gm.y) ? gm.y : 0.;
    float2 a = anchor_of(cx, cy, G);
    double ax = (double)a.x, ay = (double)a.y;
    const float4 g4 = make_float4((float)(gm.x - ax), (float)(gm.y - ay), (float)(gm.z + gm.w), 0.f);
    nf_geo[k] = g4;
    nf_k[k] = a;
    const double* c = cm + 6 * k;
    const float4 c4 = make_float4((float)(c[0] - ax), (float)(c[1] - ay), (float)(c[3] - ax), (float)(c[4] - ay));
    const float2 gg = make_float2((float)c[2], (float)c[5]);
    nf_cm[k] = c4;
    nf_g[k] = gg;
    const int32_t c1 = ch1[k];
    float4* r = rec + 4 * (size_t)k;
    r[0] = make_float4(g4.x, g4.y, g4.z, __int_as_float(c1));
    r[1] = make_float4(a.x, a.y, __int_as_float(c1 < 0 ? dfs[k] : -1), 0.f);
    r[2] = c4;
    r[3] = make_float4(gg.x, gg.y, 0.f, 0.f);
}

// Marks the leaves that hold a segment centre (stree::findNode, TSortedTree.cpp:284-303).
__global__ void k_flag_seg_leaves(int64_t m, const double* __restrict__ rx, const double* __restrict__ ry,
                                  const double4* __restrict__ geom, const int32_t* __restrict__ ch1,
                                  const int32_t* __restrict__ dfs, int32_t* flag) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    double px = rx[s], py = ry[s];
    int32_t k = 0;
    for (int it = 0; it <= MAX_DEPTH && ch1[k] >= 0; it++) {
        double4 gm = geom[k];
        if (gm.z < gm.w) k = (px < gm.x) ? ch1[k] : ch1[k] + 1;
        else k = (py < gm.y) ? ch1[k] : ch1[k] + 1;
    }
    flag[dfs[k]] = 1;
}

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Per-leaf walk (one thread per leaf) for selected leaves only (sel[L] != 0).
// PASS 0 counts, PASS 1 writes at the offsets.  Bit 1 of `what`: near runs (near_cnt /
// near_off / near_run); bit 2: far nodes (far_cnt / far_off / far_node).  Unselected leaves
// are not touched.  Used for the leaves the warp-per-leaf walk could not hold.
template <int PASS>
__global__ void __launch_bounds__(LB) k_walk(int64_t nl, ListView v, const int32_t* __restrict__ leaf_node,
                                             const int32_t* __restrict__ sel, int32_t* near_cnt, int32_t* far_cnt,
                                             const int32_t* __restrict__ near_off, const int32_t* __restrict__ far_off,
                                             int2* near_run, int32_t* far_node, int64_t nodes_bound, int32_t* err,
                                             int what) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    const bool want_near = what & 1, want_far = what & 2;
    if (!sel[L]) return;
    const int32_t meN = leaf_node[L];
    const float4 mg = v.nf_geo[meN];
    const float2 mk = v.nf_k[meN];
    int32_t stack[MAX_DEPTH + 2];
    int sp = 0;
    stack[sp++] = 0;
    int32_t nr = 0, nf = 0, last = -2, rfirst = -1;
    const int32_t nbase = (PASS && want_near) ? near_off[L] : 0;
    const int32_t fbase = (PASS && want_far) ? far_off[L] : 0;
    int64_t guard = 0;
    while (sp) {
        if (++guard > nodes_bound) { atomicExch(err, 2); break; }
        const int32_t t = stack[--sp];
        if (far_test(v, t, meN, mg, mk)) {
            if (PASS && want_far) far_node[fbase + nf] = t;
            nf++;
            continue;
        }
        const int32_t c1 = v.ch1[t];
        if (c1 >= 0) {
            if (sp + 2 > MAX_DEPTH + 2) { atomicExch(err, 2); break; }
            stack[sp++] = c1 + 1;
            stack[sp++] = c1;
            continue;
        }
        const int32_t q = v.dfs[t];
        if (q == last + 1) {
            last = q;
        } else {
            if (PASS && want_near && rfirst >= 0) near_run[nbase + nr - 1] = make_int2(rfirst, last + 1);
            rfirst = q;
            last = q;
            nr++;
        }
    }
    if (PASS && want_near && rfirst >= 0) near_run[nbase + nr - 1] = make_int2(rfirst, last + 1);
    if (PASS == 0 && want_near) near_cnt[L] = nr;
    if (PASS == 0 && want_far) far_cnt[L] = nf;
}

// Warp-per-leaf walk for a list of selected leaves: the warp expands the tree level by
// level (each lane tests one frontier node with the same far decision as every other walk),
// so a leaf's walk takes one step per level instead of one per visited node.  Near leaves
// are sorted (they come out level by level) and stored as runs; far nodes are stored in
// level order.  PASS 0 counts, PASS 1 writes at the offsets; bit 1 of `what`: near runs,
// bit 2: far nodes.  A leaf whose frontier or near set does not fit the shared buffers is
// flagged in `fallback` (PASS 0) and left to the per-thread walk.
constexpr int BW = 4;        // warps (leaves) per block
constexpr int FCAP = 1024;   // frontier capacity per warp
template <int PASS>
__global__ void __launch_bounds__(BW * 32) k_walk_bfs(int64_t nsel, const int32_t* __restrict__ list, ListView v,
                                                      const int32_t* __restrict__ leaf_node, int32_t* near_cnt,
                                                      int32_t* far_cnt, const int32_t* __restrict__ near_off,
                                                      const int32_t* __restrict__ far_off, int2* near_run,
                                                      int32_t* far_node, int what, int32_t* fallback,
                                                      int32_t* n_fallback) {
    __shared__ int32_t s_f[BW][2][FCAP];
    __shared__ int32_t s_near[BW][FCAP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t idx = (int64_t)blockIdx.x * BW + w;
    if (idx >= nsel) return;
    const int32_t L = list[idx];
    if (PASS == 1 && fallback[L]) return;
    const bool want_near = what & 1, want_far = what & 2;
    const int32_t meN = leaf_node[L];
    const float4 mg = v.nf_geo[meN];
    const float2 mk = v.nf_k[meN];
    const unsigned lt = (1u << lane) - 1;
    const int32_t fbase = (PASS && want_far) ? far_off[L] : 0;
    int cur = 0, ncur = 1, nnear = 0, nfar = 0;
    bool ovf = false;
    if (lane == 0) s_f[w][0][0] = 0;
    __syncwarp();
    for (int depth = 0; ncur > 0; depth++) {
        if (depth > MAX_DEPTH + 1) { ovf = true; break; }
        int nnext = 0;
        for (int base = 0; base < ncur; base += 32) {
            const int k = base + lane;
            int32_t t = -1, c1 = -1;
            bool far = false, inner = false, leaf = false;
            if (k < ncur) {
                t = s_f[w][cur][k];
                far = far_test(v, t, meN, mg, mk);
                if (!far) {
                    c1 = v.ch1[t];
                    inner = c1 >= 0;
                    leaf = !inner;
                }
            }
            unsigned m = __ballot_sync(0xffffffffu, far);
            if (far && PASS && want_far) far_node[fbase + nfar + __popc(m & lt)] = t;
            nfar += __popc(m);
            m = __ballot_sync(0xffffffffu, inner);
            if (inner) {
                const int pos = nnext + 2 * __popc(m & lt);
                if (pos + 1 < FCAP) { s_f[w][cur ^ 1][pos] = c1; s_f[w][cur ^ 1][pos + 1] = c1 + 1; }
            }
            nnext += 2 * __popc(m);
            m = __ballot_sync(0xffffffffu, leaf);
            if (leaf) {
                const int pos = nnear + __popc(m & lt);
                if (pos < FCAP) s_near[w][pos] = v.dfs[t];
            }
            nnear += __popc(m);
        }
        if (nnext > FCAP || nnear > FCAP) { ovf = true; break; }
        __syncwarp();
        cur ^= 1;
        ncur = nnext;
    }
    if (ovf) {
        if (PASS == 0 && lane == 0) { fallback[L] = 1; atomicAdd(n_fallback, 1); }
        return;
    }
    int32_t nr = 0, ne = 0;  // runs started, runs ended
    if (want_near) {
        // rank sort of the (distinct) near leaves into the free frontier buffer, then runs
        int32_t* srt = s_f[w][cur];
        __syncwarp();
        for (int e = lane; e < nnear; e += 32) {
            const int32_t x = s_near[w][e];
            int r = 0;
            for (int q = 0; q < nnear; q++) r += s_near[w][q] < x;
            srt[r] = x;
        }
        __syncwarp();
        const int32_t nbase = PASS ? near_off[L] : 0;
        int32_t* out = reinterpret_cast<int32_t*>(near_run);
        for (int base = 0; base < nnear; base += 32) {
            const int p = base + lane;
            bool st = false, en = false;
            int32_t x = 0;
            if (p < nnear) {
                x = srt[p];
                st = (p == 0) || (srt[p - 1] != x - 1);
                en = (p == nnear - 1) || (srt[p + 1] != x + 1);
            }
            const unsigned ms = __ballot_sync(0xffffffffu, st), me = __ballot_sync(0xffffffffu, en);
            if (PASS) {
                if (st) out[2 * (size_t)(nbase + nr + __popc(ms & lt))] = x;
                if (en) out[2 * (size_t)(nbase + ne + __popc(me & lt)) + 1] = x + 1;
            }
            nr += __popc(ms);
            ne += __popc(me);
        }
    }
    if (PASS == 0 && lane == 0) {
        if (want_near) near_cnt[L] = nr;
        if (want_far) far_cnt[L] = nfar;
    }
}

// The judge of the learned far field (learned_step.cu): the vortex part of velocity(p) at
// vortex idx[q] with the near/far split of the judge's far criterion (v.fc).  One warp per
// target walks the tree level by level as k_walk_bfs does (same far decisions), adding the
// far nodes' monopoles as it goes, then the lanes split the near leaves' vortices.  Pair
// terms in FP32 from FP64 offsets, compensated sums, partials by a fixed shuffle tree.
// out[3 q ..] = (vx, vy, 1) without the free-stream, sink and slip terms; (0, 0, 0) for a
// vortex with g = 0; out[3 q + 2] = -1 when the walk did not fit the shared buffers.
__global__ void __launch_bounds__(BW * 32) k_judge_bfs(int64_t nt, const int32_t* __restrict__ idx, ListView v,
                                                       const double* __restrict__ x, const double* __restrict__ y,
                                                       const double* __restrict__ g, const double* __restrict__ ie,
                                                       const int32_t* __restrict__ nvf, const int32_t* __restrict__ nvl,
                                                       double* out) {
    __shared__ int32_t s_f[BW][2][FCAP];
    __shared__ int32_t s_near[BW][FCAP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * BW + w;
    if (q >= nt) return;
    const int32_t i = idx[q];
    if (g[i] == 0.) {
        if (lane == 0) { out[3 * q] = 0.; out[3 * q + 1] = 0.; out[3 * q + 2] = 0.; }
        return;
    }
    const double px = x[i], py = y[i];
    int32_t meN = 0;
    for (int it = 0; it <= MAX_DEPTH && v.ch1[meN] >= 0; it++) {
        const double4 gm = v.geom[meN];
        if (gm.z < gm.w) meN = (px < gm.x) ? v.ch1[meN] : v.ch1[meN] + 1;
        else meN = (py < gm.y) ? v.ch1[meN] : v.ch1[meN] + 1;
    }
    const float4 mg = v.nf_geo[meN];
    const float2 mk = v.nf_k[meN];
    const unsigned lt = (1u << lane) - 1;
    float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
    auto pair = [&](double sx, double sy, float gs, float e2) {
        const float dx = (float)(px - sx), dy = (float)(py - sy);
        const float s = gs * rcp_approx(fmaf(dx, dx, fmaf(dy, dy, e2)));
        two_sum_acc(hx, lx, -dy * s);
        two_sum_acc(hy, ly, dx * s);
    };
    int cur = 0, ncur = 1, nnear = 0;
    bool ovf = false;
    if (lane == 0) s_f[w][0][0] = 0;
    __syncwarp();
    for (int depth = 0; ncur > 0; depth++) {
        if (depth > MAX_DEPTH + 1) { ovf = true; break; }
        int nnext = 0;
        for (int base = 0; base < ncur; base += 32) {
            const int k = base + lane;
            int32_t t = -1, c1 = -1;
            bool far = false, inner = false, leaf = false;
            if (k < ncur) {
                t = s_f[w][cur][k];
                far = far_test(v, t, meN, mg, mk);
                if (far) {  // far_nodes_influence (MConvectiveFast.cpp:139-151)
                    const double* c = v.cm + 6 * (size_t)t;
                    if (c[2] != 0.) pair(c[0], c[1], (float)c[2], 0.f);
                    if (c[5] != 0.) pair(c[3], c[4], (float)c[5], 0.f);
                } else {
                    c1 = v.ch1[t];
                    inner = c1 >= 0;
                    leaf = !inner;
                }
            }
            unsigned m = __ballot_sync(0xffffffffu, inner);
            if (inner) {
                const int pos = nnext + 2 * __popc(m & lt);
                if (pos + 1 < FCAP) { s_f[w][cur ^ 1][pos] = c1; s_f[w][cur ^ 1][pos + 1] = c1 + 1; }
            }
            nnext += 2 * __popc(m);
            m = __ballot_sync(0xffffffffu, leaf);
            if (leaf) {
                const int pos = nnear + __popc(m & lt);
                if (pos < FCAP) s_near[w][pos] = t;
            }
            nnear += __popc(m);
        }
        if (nnext > FCAP || nnear > FCAP) { ovf = true; break; }
        __syncwarp();
        cur ^= 1;
        ncur = nnext;
    }
    if (ovf) {
        if (lane == 0) out[3 * q + 2] = -1.;
        return;
    }
    __syncwarp();
    for (int e = lane; e < nnear; e += 32) {  // near_nodes_influence (MConvectiveFast.cpp:122-137)
        const int32_t t = s_near[w][e];
        for (int32_t j = nvf[t]; j < nvl[t]; j++) {
            const double gj = g[j];
            if (gj == 0.) continue;
            const float ep = rcp_approx((float)ie[j]);  // 1/_1_eps; _1_eps = 0 gives inf, s = 0
            pair(x[j], y[j], (float)gj, ep * ep);
        }
    }
    double sx = (double)hx + (double)lx, sy = (double)hy + (double)ly;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (lane == 0) {
        out[3 * q] = sx * C_1_2PI;
        out[3 * q + 1] = sy * C_1_2PI;
        out[3 * q + 2] = 1.;
    }
}

// Indices of the flagged leaves, in order.
__global__ void k_list_flags(int64_t nl, const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                             int32_t* list) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L < nl && flag[L]) list[pos[L]] = (int32_t)L;
}

// Far-field contribution of far node t to leaf (mg, mk | me), FP32 or FP64.
template <bool FP32>
struct Taylor {
    double d1 = 0, d2 = 0, d3 = 0, d4 = 0;
    float h1 = 0, l1 = 0, h2 = 0, l2 = 0, h3 = 0, l3 = 0, h4 = 0, l4 = 0;
    __device__ __forceinline__ void add(const ListView& v, int32_t t, float4 mg, float2 mk, const double4& me) {
        if (FP32) {
            const float2 tk = v.nf_k[t];
            const float sx = mk.x - tk.x, sy = mk.y - tk.y;
            const float4 c4 = v.nf_cm[t];
            const float2 gg = v.nf_g[t];
            float dpx = sx + (mg.x - c4.x), dpy = sy + (mg.y - c4.y);
            float dmx = sx + (mg.x - c4.z), dmy = sy + (mg.y - c4.w);
            float ap = dpx * dpx + dpy * dpy, am = dmx * dmx + dmy * dmy;
            float ip = rcp_approx(ap), im = rcp_approx(am);
            float fp1 = gg.x * ip, fm1 = gg.y * im;
            float fp2 = fp1 * ip, fm2 = fm1 * im;
            two_sum_acc(h1, l1, -(fp1 * dpy + fm1 * dmy));
            two_sum_acc(h2, l2, fp1 * dpx + fm1 * dmx);
            two_sum_acc(h3, l3, fp2 * dpy * dpx + fm2 * dmy * dmx);
            two_sum_acc(h4, l4, fp2 * (dpy * dpy - dpx * dpx) + fm2 * (dmy * dmy - dmx * dmx));
        } else {
            const double* c = v.cm + 6 * (size_t)t;
            double dpx = me.x - c[0], dpy = me.y - c[1], dmx = me.x - c[3], dmy = me.y - c[4];
            double ap = dpx * dpx + dpy * dpy, am = dmx * dmx + dmy * dmy;
            double fp1 = c[2] / ap, fm1 = c[5] / am;
            double fp2 = c[2] / (ap * ap), fm2 = c[5] / (am * am);
            d1 -= (fp1 * dpy + fm1 * dmy);
            d2 += (fp1 * dpx + fm1 * dmx);
            d3 += (fp2 * dpy * dpx + fm2 * dmy * dmx);
            d4 += (fp2 * (dpy * dpy - dpx * dpx) + fm2 * (dmy * dmy - dmx * dmx));
        }
    }
    // FP32 path with the node's record already loaded.
    __device__ __forceinline__ void add_rec(const NodeRec& n, float4 mg, float2 mk) {
        const float sx = mk.x - n.r1.x, sy = mk.y - n.r1.y;
        const float4 c4 = n.r2;
        const float gp = n.r3.x, gm = n.r3.y;
        float dpx = sx + (mg.x - c4.x), dpy = sy + (mg.y - c4.y);
        float dmx = sx + (mg.x - c4.z), dmy = sy + (mg.y - c4.w);
        float ap = dpx * dpx + dpy * dpy, am = dmx * dmx + dmy * dmy;
        float ip = rcp_approx(ap), im = rcp_approx(am);
        float fp1 = gp * ip, fm1 = gm * im;
        float fp2 = fp1 * ip, fm2 = fm1 * im;
        two_sum_acc(h1, l1, -(fp1 * dpy + fm1 * dmy));
        two_sum_acc(h2, l2, fp1 * dpx + fm1 * dmx);
        two_sum_acc(h3, l3, fp2 * dpy * dpx + fm2 * dmy * dmx);
        two_sum_acc(h4, l4, fp2 * (dpy * dpy - dpx * dpx) + fm2 * (dmy * dmy - dmx * dmx));
    }
    __device__ __forceinline__ double4 result() const {
        double a = d1, b = d2, cc = d3, d = d4;
        if (FP32) {
            a = (double)h1 + (double)l1; b = (double)h2 + (double)l2;
            cc = (double)h3 + (double)l3; d = (double)h4 + (double)l4;
        }
        return make_double4(a * C_1_2PI, b * C_1_2PI, cc * C_1_PI, d * C_1_2PI);
    }
};

constexpr int RUN_CAP = 64;   // near runs kept per leaf by the warp walk
constexpr int FAR_CAP = 2048; // far nodes kept per leaf by the warp walk (when asked to keep them)
// One warp per block and 32 blocks per SM (64 registers): a block ends with its warp, so
// the SM refills as walks of different lengths finish (measured 9.5 against 11.0 ms for
// four warps per block, 4M wake)
#ifndef VV_WALK_WARPS
#define VV_WALK_WARPS 1
#endif
#ifndef VV_WALK_MIN_BLOCKS
#define VV_WALK_MIN_BLOCKS 32
#endif
constexpr int WW = VV_WALK_WARPS;  // warps per block in the warp walk

// One warp walks the tree for 32 consecutive leaves at once (they are neighbours in space,
// so their walks share most nodes).  The stack holds (node, mask of lanes still walking
// below it); node data are broadcast loads.  Each lane keeps its own near runs (in depth-
// first order) and far-field coefficients.  Runs beyond RUN_CAP are counted, not stored.
// With far_buf set, each leaf's far nodes are also kept (walk order, at most far_cap of
// them; the count in far_cnt may exceed far_cap, and the caller then rebuilds that list).
template <bool FP32>
__global__ void __launch_bounds__(WW * 32, VV_WALK_MIN_BLOCKS) k_walk_warp(int64_t nl, ListView v, const int32_t* __restrict__ leaf_node,
                                                       int32_t* near_cnt, int2* run_buf, double4* taylor,
                                                       unsigned long long* far_total, int64_t nodes_bound,
                                                       int32_t* err, int32_t* far_buf, int32_t far_cap,
                                                       int32_t* far_cnt) {
    __shared__ int32_t s_node[WW][MAX_DEPTH + 2];
    __shared__ uint32_t s_mask[WW][MAX_DEPTH + 2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t L = ((int64_t)blockIdx.x * WW + w) * 32 + lane;
    const bool valid = L < nl;
    const uint32_t all = __ballot_sync(0xffffffffu, valid);
    if (!all) return;
    const int32_t meN = valid ? leaf_node[L] : 0;
    const float4 mg = v.nf_geo[meN];
    const float2 mk = v.nf_k[meN];
    const double4 me = v.geom[meN];
    Taylor<FP32> tay;
    int32_t nr = 0, last = -2, rfirst = -1, nfar = 0;
    int2* myruns = run_buf + (size_t)(valid ? L : 0) * RUN_CAP;
    // Each visit reads the node's packed record (one 64-byte line) for the far test, the
    // far field, the children and the leaf index.
    if (lane == 0) { s_node[w][0] = 0; s_mask[w][0] = all; }
    int sp = 1;
    __syncwarp();
    int64_t guard = 0;
    while (sp > 0) {
        if (++guard > nodes_bound) { if (lane == 0) atomicExch(err, 2); break; }
        sp--;
        const int32_t t = s_node[w][sp];
        const uint32_t mask = s_mask[w][sp];
        __syncwarp();
        const bool act = (mask >> lane) & 1u;
        const NodeRec cur = load_rec(v.rec, t);
        const bool far = act && far_test_at(v, cur.r0, make_float2(cur.r1.x, cur.r1.y), t, meN, mg, mk);
        if (far) {
            if (FP32) tay.add_rec(cur, mg, mk); else tay.add(v, t, mg, mk, me);
            if (far_buf && nfar < far_cap) far_buf[(size_t)L * far_cap + nfar] = t;
            nfar++;
        }
        const uint32_t rest = mask & ~__ballot_sync(0xffffffffu, far);
        if (rest) {
            const int32_t c1 = __float_as_int(cur.r0.w);
            if (c1 >= 0) {
                if (sp + 2 > MAX_DEPTH + 2) { if (lane == 0) atomicExch(err, 2); break; }
                if (lane == 0) {
                    s_node[w][sp] = c1 + 1; s_mask[w][sp] = rest;
                    s_node[w][sp + 1] = c1; s_mask[w][sp + 1] = rest;
                }
                sp += 2;
            } else if ((rest >> lane) & 1u) {
                const int32_t q = __float_as_int(cur.r1.z);
                if (q == last + 1) {
                    last = q;
                } else {
                    if (rfirst >= 0 && nr <= RUN_CAP) myruns[nr - 1] = make_int2(rfirst, last + 1);
                    rfirst = q;
                    last = q;
                    nr++;
                }
            }
        }
        __syncwarp();
    }
    if (valid) {
        if (rfirst >= 0 && nr <= RUN_CAP) myruns[nr - 1] = make_int2(rfirst, last + 1);
        near_cnt[L] = nr;
        taylor[L] = tay.result();
        if (far_cnt) far_cnt[L] = nfar;
    }
    unsigned long long f = warp_sum_u64(valid ? (unsigned long long)nfar : 0ull);
    if (lane == 0) {
        atomicAdd(far_total, f);
        atomicAdd(far_total + 8, (unsigned long long)guard);  // node records this warp loaded
    }
}

__global__ void k_count_over(int64_t nl, const int32_t* __restrict__ cnt, int32_t cap, int32_t* n_over) {
    const int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool o = L < nl && cnt[L] > cap;
    if (__any_sync(0xffffffffu, o) && (threadIdx.x & 31) == 0) atomicAdd(n_over, 1);
}

__global__ void k_runs_compact(int64_t nl, const int32_t* __restrict__ near_cnt, const int32_t* __restrict__ near_off,
                               const int2* __restrict__ run_buf, int2* near_run, int32_t* overflow,
                               int32_t* n_overflow) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    int32_t n = near_cnt[L];
    if (n > RUN_CAP) {
        overflow[L] = 1;
        atomicAdd(n_overflow, 1);
        return;
    }
    overflow[L] = 0;
    const int2* src = run_buf + (size_t)L * RUN_CAP;
    int2* dst = near_run + near_off[L];
    for (int32_t k = 0; k < n; k++) dst[k] = src[k];
}

// Exact walk writing every leaf's far list (inspection only).
template <bool FILL>
__global__ void k_walk_exact(int64_t nl, const int32_t* __restrict__ leaf_node, const double4* __restrict__ geom,
                             const int32_t* __restrict__ ch1, double fc, int32_t* far_cnt,
                             const int32_t* __restrict__ far_off, int32_t* far_node, int64_t nodes_bound,
                             int32_t* err) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    const double4 me = geom[leaf_node[L]];
    int32_t stack[MAX_DEPTH + 2];
    int sp = 0;
    stack[sp++] = 0;
    int32_t nf = 0;
    const int32_t fbase = FILL ? far_off[L] : 0;
    int64_t guard = 0;
    while (sp) {
        if (++guard > nodes_bound) { atomicExch(err, 2); break; }
        const int32_t t = stack[--sp];
        if (far_exact(geom[t], me, fc)) {
            if (FILL) far_node[fbase + nf] = t;
            nf++;
            continue;
        }
        const int32_t c1 = ch1[t];
        if (c1 >= 0) {
            if (sp + 2 > MAX_DEPTH + 2) { atomicExch(err, 2); break; }
            stack[sp++] = c1 + 1;
            stack[sp++] = c1;
        }
    }
    if (!FILL) far_cnt[L] = nf;
}

}  // namespace

namespace {
// Walks the leaves with sel[L] != 0: counts (count = true) into near_cnt / far_cnt, or
// writes at near_off / far_off.  Counting keeps the list of selected leaves and flags the
// leaves the warp-per-leaf walk could not hold; those take the per-thread walk.
void walk_selected(Ctx& c, const ListView& v, const int32_t* sel, int what, bool count) {
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves, nn = c.nnodes;
    int32_t* err = (int32_t*)c.counters.p + 1;
    int32_t* nfb = (int32_t*)(c.counters.p + 15);
    if (count || what == 1) {
        c.sel_pos.reserve(nl + 2);
        c.sel_list.reserve(nl + 1);
        exclusive_scan(c, sel, c.sel_pos.p, nl);
        c.n_sel = read_i32(c, c.sel_pos.p + nl);
        k_list_flags<<<grid_for(nl, 256), 256, 0, s>>>(nl, sel, c.sel_pos.p, c.sel_list.p);
        VV_LAUNCH_CHECK();
        c.lf_fallback.reserve(nl + 1);
        VV_CUDA(cudaMemsetAsync(c.lf_fallback.p, 0, (nl + 1) * 4, s));
        VV_CUDA(cudaMemsetAsync(nfb, 0, 4, s));
    }
    if (c.n_sel == 0) return;
    const unsigned g = grid_for(c.n_sel, BW);
    if (count || what == 1) {
        // the count pass (for `what == 1` the counts come from the warp walk; this pass only
        // finds the leaves that need the per-thread walk)
        k_walk_bfs<0><<<g, BW * 32, 0, s>>>(c.n_sel, c.sel_list.p, v, c.leaf_node.p,
                                            count ? c.near_cnt.p : nullptr, c.far_cnt.p, nullptr, nullptr,
                                            nullptr, nullptr, count ? what : 0, c.lf_fallback.p, nfb);
        VV_LAUNCH_CHECK();
        c.n_fallback = read_i32(c, nfb);
        if (count && c.n_fallback > 0) {
            k_walk<0><<<grid_for(nl, LB), LB, 0, s>>>(nl, v, c.leaf_node.p, c.lf_fallback.p, c.near_cnt.p,
                                                      c.far_cnt.p, nullptr, nullptr, nullptr, nullptr, nn, err, what);
            VV_LAUNCH_CHECK();
        }
    }
    if (!count) {
        k_walk_bfs<1><<<g, BW * 32, 0, s>>>(c.n_sel, c.sel_list.p, v, c.leaf_node.p, nullptr, nullptr, c.near_off.p,
                                            c.far_off.p, c.near_run.p, c.far_node.p, what, c.lf_fallback.p, nfb);
        VV_LAUNCH_CHECK();
        if (c.n_fallback > 0) {
            k_walk<1><<<grid_for(nl, LB), LB, 0, s>>>(nl, v, c.leaf_node.p, c.lf_fallback.p, nullptr, nullptr,
                                                      c.near_off.p, c.far_off.p, c.near_run.p, c.far_node.p, nn, err,
                                                      what);
            VV_LAUNCH_CHECK();
        }
    }
}

// Far nodes of every leaf, contiguous in leaf order: node ids and their leaf's node id.  One
// warp per leaf copies its walk buffer.
__global__ void k_far_compact(int64_t nl, const int32_t* __restrict__ far_cnt, const int32_t* __restrict__ far_off,
                              const int32_t* __restrict__ far_buf, int32_t far_cap,
                              const int32_t* __restrict__ leaf_node, int32_t* node, int32_t* leaf) {
    const int64_t L = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    const int32_t n = far_cnt[L], o = far_off[L], me = leaf_node[L];
    const int32_t* src = far_buf + (size_t)L * far_cap;
    for (int32_t k = lane; k < n; k += 32) {
        node[o + k] = src[k];
        leaf[o + k] = me;
    }
}

__global__ void k_far_leaf_of(int64_t nl, const int32_t* __restrict__ far_off, const int32_t* __restrict__ leaf_node,
                              int32_t* leaf) {
    const int64_t L = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    const int32_t me = leaf_node[L];
    for (int32_t k = far_off[L] + lane; k < far_off[L + 1]; k += 32) leaf[k] = me;
}

ListView list_view(Ctx& c) {
    return ListView{c.nd_geom.p, c.nd_ch1.p, c.nd_dfs.p, c.nf_geo.p, c.nf_k.p, c.nf_cm.p, c.nf_g.p, c.nd_cm.p,
                    c.nf_rec.p, c.far_criteria, (float)c.far_criteria, (float)c.frame_G};
}
}  // namespace

void tree_lists(Ctx& c) {
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves, nn = c.nnodes;
    int32_t* err = (int32_t*)c.counters.p + 1;
    VV_CUDA(cudaMemsetAsync(err, 0, 4, s));
    // frames of every node
    double4 rootl;
    double4* rp = pinned_at(c, 64, &rootl);
    VV_CUDA(cudaMemcpyAsync(rp, c.nd_geom.p, sizeof rootl, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    const double4 root = *rp;
    Frame fr = make_frame(std::fmax(std::fabs(root.x), std::fabs(root.y)) + std::fmax(root.z, root.w));
    c.frame_G = fr.G;
    c.nf_geo.reserve(nn); c.nf_k.reserve(nn); c.nf_cm.reserve(nn); c.nf_g.reserve(nn);
    c.nf_rec.reserve(4 * (size_t)nn);
    k_node_frames<<<grid_for(nn, 256), 256, 0, s>>>(nn, c.nd_geom.p, c.nd_cm.p, fr.G, c.nd_ch1.p, c.nd_dfs.p,
                                                    c.nf_geo.p, c.nf_k.p, c.nf_cm.p, c.nf_g.p, c.nf_rec.p);
    VV_LAUNCH_CHECK();
    c.lf_flag.reserve(nl + 1);
    VV_CUDA(cudaMemsetAsync(c.lf_flag.p, 0, (nl + 1) * 4, s));
    if (c.m > 0) {
        k_flag_seg_leaves<<<grid_for(c.m, 256), 256, 0, s>>>(c.m, c.s_rx.p, c.s_ry.p, c.nd_geom.p, c.nd_ch1.p,
                                                             c.nd_dfs.p, c.lf_flag.p);
        VV_LAUNCH_CHECK();
    }
    const ListView v = list_view(c);
    c.near_cnt.reserve(nl + 1); c.far_cnt.reserve(nl + 1);
    c.near_off.reserve(nl + 2); c.far_off.reserve(nl + 2);
    VV_CUDA(cudaMemsetAsync(c.near_cnt.p, 0, (nl + 1) * 4, s));
    VV_CUDA(cudaMemsetAsync(c.far_cnt.p, 0, (nl + 1) * 4, s));
    // near runs and far lists of the leaves that hold a segment centre
    walk_selected(c, v, c.lf_flag.p, 3, /*count=*/true);
    exclusive_scan(c, c.near_cnt.p, c.near_off.p, nl);
    exclusive_scan(c, c.far_cnt.p, c.far_off.p, nl);
    c.n_near_runs = read_i32(c, c.near_off.p + nl);
    c.n_far = read_i32(c, c.far_off.p + nl);
    c.near_run.reserve(c.n_near_runs + 1);
    c.far_node.reserve(c.n_far + 1);
    walk_selected(c, v, c.lf_flag.p, 3, /*count=*/false);
    if (read_i32(c, err)) throw ApiError{VVGPU_ERR_LIMIT, "tree traversal exceeded its bound"};
    c.lists_full = false;
    c.far_kept = false;
    c.stats.near_runs = c.n_near_runs;
    c.stats.far_pairs = 0;
}

// The far nodes the warp walk kept, compacted (lf_far_off / lf_far_node / lf_far_leaf).  A
// leaf with more than FAR_CAP far nodes makes every list come from the exact walk instead
// (the same nodes in the same depth-first order).
void keep_far_lists(Ctx& c) {
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves;
    c.lf_far_off.reserve(nl + 2);
    int32_t* n_over = (int32_t*)(c.counters.p + 17);
    VV_CUDA(cudaMemsetAsync(n_over, 0, 4, s));
    k_count_over<<<grid_for(nl, 256), 256, 0, s>>>(nl, c.lf_far_cnt.p, FAR_CAP, n_over);
    VV_LAUNCH_CHECK();
    if (read_i32(c, n_over) > 0) {
        std::vector<int32_t> off, node;
        tree_lists_exact(c, off, node, true);
        if ((int64_t)node.size() > 0x7fffffffLL) throw ApiError{VVGPU_ERR_LIMIT, "more than 2^31 far pairs"};
        c.n_far_pairs = (int64_t)node.size();
        c.lf_far_node.reserve(c.n_far_pairs + 1);
        c.lf_far_leaf.reserve(c.n_far_pairs + 1);
        VV_CUDA(cudaMemcpyAsync(c.lf_far_off.p, off.data(), (nl + 1) * 4, cudaMemcpyHostToDevice, s));
        if (c.n_far_pairs)
            VV_CUDA(cudaMemcpyAsync(c.lf_far_node.p, node.data(), c.n_far_pairs * 4, cudaMemcpyHostToDevice, s));
        k_far_leaf_of<<<grid_for(nl, 8), 256, 0, s>>>(nl, c.lf_far_off.p, c.leaf_node.p, c.lf_far_leaf.p);
        VV_LAUNCH_CHECK();
        VV_CUDA(cudaStreamSynchronize(s));
    } else {
        exclusive_scan(c, c.lf_far_cnt.p, c.lf_far_off.p, nl);
        c.n_far_pairs = (uint32_t)read_i32(c, c.lf_far_off.p + nl);
        c.lf_far_node.reserve(c.n_far_pairs + 1);
        c.lf_far_leaf.reserve(c.n_far_pairs + 1);
        k_far_compact<<<grid_for(nl, 8), 256, 0, s>>>(nl, c.lf_far_cnt.p, c.lf_far_off.p, c.far_buf.p, FAR_CAP,
                                                      c.leaf_node.p, c.lf_far_node.p, c.lf_far_leaf.p);
        VV_LAUNCH_CHECK();
    }
    c.far_kept = true;
}

void ensure_full_lists(Ctx& c) {
    if (c.lists_full) return;
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves, nn = c.nnodes;
    int32_t* err = (int32_t*)c.counters.p + 1;
    VV_CUDA(cudaMemsetAsync(err, 0, 4, s));
    const ListView v = list_view(c);
    c.lf_taylor.reserve(nl + 1);
    c.run_buf.reserve((size_t)nl * RUN_CAP + 1);
    c.lf_overflow.reserve(nl + 1);
    unsigned long long* far_total = c.counters.p + 10;  // and, at + 8, the walk's record loads
    VV_CUDA(cudaMemsetAsync(far_total, 0, 8, s));
    VV_CUDA(cudaMemsetAsync(far_total + 8, 0, 8, s));
    const bool fp32 = c.precision == VVGPU_FP32;
    const unsigned gw = grid_for((nl + 31) / 32, WW);
    {
        KernelTimer kt(c, VVGPU_T_WALK);
        int32_t* fb = nullptr;
        int32_t* fcnt = nullptr;
        if (c.keep_far) {
            c.far_buf.reserve((size_t)nl * FAR_CAP + 1);
            c.lf_far_cnt.reserve(nl + 1);
            fb = c.far_buf.p;
            fcnt = c.lf_far_cnt.p;
        }
        if (fp32) k_walk_warp<true><<<gw, WW * 32, 0, s>>>(nl, v, c.leaf_node.p, c.near_cnt.p, c.run_buf.p,
                                                            c.lf_taylor.p, far_total, nn, err, fb, FAR_CAP, fcnt);
        else k_walk_warp<false><<<gw, WW * 32, 0, s>>>(nl, v, c.leaf_node.p, c.near_cnt.p, c.run_buf.p,
                                                         c.lf_taylor.p, far_total, nn, err, fb, FAR_CAP, fcnt);
        VV_LAUNCH_CHECK();
    }
    exclusive_scan(c, c.near_cnt.p, c.near_off.p, nl);
    c.n_near_runs = read_i32(c, c.near_off.p + nl);
    c.near_run.reserve(c.n_near_runs + 1);
    int32_t* n_over = (int32_t*)(c.counters.p + 12);
    VV_CUDA(cudaMemsetAsync(n_over, 0, 4, s));
    k_runs_compact<<<grid_for(nl, 256), 256, 0, s>>>(nl, c.near_cnt.p, c.near_off.p, c.run_buf.p, c.near_run.p,
                                                     c.lf_overflow.p, n_over);
    VV_LAUNCH_CHECK();
    if (read_i32(c, err)) throw ApiError{VVGPU_ERR_LIMIT, "tree traversal exceeded its bound"};
    const int32_t nover = read_i32(c, n_over);
    if (nover > 0) {
        // leaves with more than RUN_CAP runs: write their runs with the warp-per-leaf walk
        walk_selected(c, v, c.lf_overflow.p, 1, /*count=*/false);
        if (read_i32(c, err)) throw ApiError{VVGPU_ERR_LIMIT, "tree traversal exceeded its bound"};
    }
    c.lists_full = true;
    c.stats.near_runs = c.n_near_runs;
    c.taylor_precision = c.precision;
    unsigned long long ft = 0, nv = 0;
    VV_CUDA(cudaMemcpyAsync(&ft, far_total, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaMemcpyAsync(&nv, far_total + 8, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    c.walk_loads = (int64_t)nv;
    c.stats.far_pairs = 2 * (int64_t)ft;  // two monopoles per far node
    if (c.keep_far) {
        if (ft > 0x7fffffffull) throw ApiError{VVGPU_ERR_LIMIT, "more than 2^31 far pairs to keep"};
        keep_far_lists(c);
    }
}

void judge_walk(Ctx& c, int64_t nt, const int32_t* d_idx, double fc, double* d_out) {
    if (nt <= 0) return;
    ListView v = list_view(c);
    v.fc = fc;
    v.fcf = (float)fc;
    k_judge_bfs<<<grid_for(nt, BW), BW * 32, 0, c.st()>>>(nt, d_idx, v, c.x.p, c.y.p, c.g.p, c.ie.p, c.nd_vf.p,
                                                            c.nd_vl.p, d_out);
    VV_LAUNCH_CHECK();
}

void tree_lists_exact(Ctx& c, std::vector<int32_t>& far_off, std::vector<int32_t>& far_node, bool fill) {
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves, nn = c.nnodes;
    int32_t* err = (int32_t*)c.counters.p + 1;
    VV_CUDA(cudaMemsetAsync(err, 0, 4, s));
    DArr<int32_t> cnt, off, fnode;
    cnt.reserve(nl + 1);
    off.reserve(nl + 2);
    k_walk_exact<false><<<grid_for(nl, LB), LB, 0, s>>>(nl, c.leaf_node.p, c.nd_geom.p, c.nd_ch1.p, c.far_criteria,
                                                        cnt.p, nullptr, nullptr, nn, err);
    VV_LAUNCH_CHECK();
    exclusive_scan(c, cnt.p, off.p, nl);
    int32_t tot = read_i32(c, off.p + nl);
    far_off.resize(nl + 1);
    if (!fill) {
        VV_CUDA(cudaMemcpyAsync(far_off.data(), off.p, (nl + 1) * 4, cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
        if (read_i32(c, err)) throw ApiError{VVGPU_ERR_LIMIT, "tree traversal exceeded its bound"};
        far_node.clear();
        return;
    }
    fnode.reserve(tot + 1);
    k_walk_exact<true><<<grid_for(nl, LB), LB, 0, s>>>(nl, c.leaf_node.p, c.nd_geom.p, c.nd_ch1.p, c.far_criteria,
                                                       nullptr, off.p, fnode.p, nn, err);
    VV_LAUNCH_CHECK();
    far_node.resize(tot);
    VV_CUDA(cudaMemcpyAsync(far_off.data(), off.p, (nl + 1) * 4, cudaMemcpyDeviceToHost, s));
    if (tot) VV_CUDA(cudaMemcpyAsync(far_node.data(), fnode.p, (size_t)tot * 4, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    if (read_i32(c, err)) throw ApiError{VVGPU_ERR_LIMIT, "tree traversal exceeded its bound"};
}

}  // namespace vvgpu
