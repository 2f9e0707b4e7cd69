// Epsilon / merge pass of libvvhd (MEpsilonFast, libvvhd/src/MEpsilonFast.cpp:11-253).
//
// The reference walks the vortices in list order; each one finds its two nearest non-zero
// neighbours among its leaf's near leaves, may absorb the nearest (MergeVortexes: move
// and add circulation, zero the neighbour) and then sets _1_eps.  Later vortices see those
// changes, so the pass is order dependent.
//
// Here every vortex i computes its outcome from the state "as of its turn": a vortex j is
// zero if some k < i absorbed it, and sits at its merged position with its merged
// circulation if j < i merged at its own turn.  Given guesses of all outcomes, every
// vortex evaluates in parallel; the outcome of i only depends on outcomes of k < i, so
// repeating until nothing changes converges to the unique fixed point, which is the
// sequential result, bit for bit.  Typical runs need 5-7 rounds.  After the first round a
// target is evaluated again only when its absorber changed or a vortex whose outcome
// changed lies (before or after the change) inside a region its last searches examined.
//
// Candidate leaves: for each target leaf L, R_L bounds every target's second-nearest
// distance from above (the farthest corner distance to a leaf that holds two live
// vortices, or three for L itself); only near leaves whose box comes within 3 R_L of L's
// box can hold a top-two candidate of the search or of the re-search from a merged
// position (see k_eps_cand).
//
// The two-nearest search filters candidates in FP32 in local frames (frame.cuh) with a
// rigorous margin and evaluates only the candidates inside the margin in FP64, with the
// reference's operation order and its tie rule (first in list order wins), so every
// decision equals the reference's.
#include <algorithm>
#include <cfloat>
#include <climits>

#include "frame.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr int EB = 128;
constexpr int32_t SKIPPED = -2;  // partner code: vortex not evaluated (g = 0 at its turn)
constexpr int CAND_CAP = 96;     // candidate leaves kept per target leaf
constexpr int CHG_CAP = 48;      // changed near leaves kept per target leaf

// MEpsilonFast::nearestBodySegment (MEpsilonFast.cpp:214-253) and the per-leaf merge
// criterion / epsilon floor (MEpsilonFast.cpp:25-47).
// Segment centres in FP32 relative to an exact per-body anchor (a float-representable
// point), and the largest coordinate, for the FP32 filter of the fallback scan below.
__global__ void k_seg_frame(int nbodies, const int64_t* __restrict__ body_first, const int64_t* __restrict__ body_count,
                            const double* __restrict__ rx, const double* __restrict__ ry, float2* seg32,
                            double2* banchor, float* brad) {
    __shared__ float s_r[EB / 32];
    const int b = blockIdx.x;
    if (b >= nbodies) return;
    const int64_t f = body_first[b], cnt = body_count[b];
    const double ax = cnt > 0 ? (double)(float)rx[f] : 0., ay = cnt > 0 ? (double)(float)ry[f] : 0.;
    float r = 0.f;
    for (int64_t k = threadIdx.x; k < cnt; k += blockDim.x) {
        const float sx = (float)(rx[f + k] - ax), sy = (float)(ry[f + k] - ay);
        seg32[f + k] = make_float2(sx, sy);
        r = fmaxf(r, fmaxf(fabsf(sx), fabsf(sy)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
    if ((threadIdx.x & 31) == 0) s_r[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) r = fmaxf(r, s_r[w]);
        banchor[b] = make_double2(ax, ay);
        brad[b] = r;
    }
}

__global__ void k_leaf_params(int64_t nl, const double4* __restrict__ lgeom, const int32_t* __restrict__ near_off,
                              const int2* __restrict__ near_run, const int32_t* __restrict__ lsf,
                              const int32_t* __restrict__ lsl, const int32_t* __restrict__ seg_order,
                              const double* __restrict__ rx, const double* __restrict__ ry,
                              const double* __restrict__ dlx, const double* __restrict__ dly,
                              const int64_t* __restrict__ body_first, const int64_t* __restrict__ body_count,
                              const float2* __restrict__ seg32, const double2* __restrict__ banchor,
                              const float* __restrict__ brad, int nbodies, int merge, double* mcs_out,
                              double* epr_out) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    double4 me = lgeom[L];
    const double px = me.x, py = me.y;
    int64_t att = -1;
    double res = DBL_MAX;
    for (int32_t r = near_off[L]; r < near_off[L + 1]; r++) {
        int2 run = near_run[r];
        int32_t q0 = lsf[run.x], q1 = lsl[run.y - 1];
        for (int32_t q = q0; q < q1; q++) {
            int32_t s = seg_order[q];
            double d = dabs2(dsub(px, rx[s]), dsub(py, ry[s]));
            if (d < res) { res = d; att = s; }
        }
    }
    if (att < 0) {
        // Every body's segments with the reference's skip rule.  Each comparison d < res is
        // decided in FP32 when the two values differ by more than their error bounds
        // (E <= 2^-19 R^2 with R bounding every coordinate involved), else in FP64 with the
        // reference's operation order; the FP64 res is formed only when needed.
        float resf = INFINITY, eres = 0.f;
        bool rese_ok = true;
        for (int b = 0; b < nbodies; b++) {
            const int64_t f = body_first[b], cnt = body_count[b];
            if (cnt <= 0) continue;
            const double2 A = banchor[b];
            const float pxg = (float)(px - A.x), pyg = (float)(py - A.y);
            const float R = brad[b] + fabsf(pxg) + fabsf(pyg);
            const float E = ldexpf(R * R, -19);
            // the decision bounds, formed when resf or E changes rather than per segment
            float lo = resf - (E + eres), hi = resf + (E + eres);
            for (int64_t k = 0; k < cnt; k++) {
                const int64_t s = f + k;
                const float2 sp = seg32[s];
                const float dx = pxg - sp.x, dy = pyg - sp.y;
                const float df = dx * dx + dy * dy;
                bool less, exact = false;
                if (att < 0) less = true;  // res = DBL_MAX: any finite distance is smaller
                else if (df < lo) less = true;
                else if (df > hi) less = false;
                else {
                    if (!rese_ok) { res = dabs2(dsub(px, rx[att]), dsub(py, ry[att])); rese_ok = true; }
                    const double d = dabs2(dsub(px, rx[s]), dsub(py, ry[s]));
                    less = d < res;
                    if (less) res = d;
                    exact = true;
                }
                if (less) {
                    resf = df; eres = E; att = s; rese_ok = exact;
                    lo = resf - (E + eres);
                    hi = resf + (E + eres);
                } else {
                    k += 9;  // MEpsilonFast.cpp:248
                }
            }
        }
    }
    double mcs, epr;
    if (merge) {
        mcs = (att >= 0) ? dmul(dmul(0.16, dabs2(dlx[att], dly[att])),
                                dadd(1., __dsqrt_rn(dabs2(dsub(px, rx[att]), dsub(py, ry[att])))))
                         : 0.;
    } else {
        mcs = __longlong_as_double(0x7ff8000000000000ll);  // quiet NaN: never merge
    }
    epr = (att >= 0) ? dmul(__dsqrt_rn(dabs2(dlx[att], dly[att])), (1.0 / 3.0)) : 0.;
    mcs_out[L] = mcs;
    epr_out[L] = epr;
}

__global__ void k_anchor(int64_t nl, const double4* __restrict__ lgeom, double G, float2* anchor) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    double4 me = lgeom[L];
    double cx = isfinite(me.x) ? me.x : 0., cy = isfinite(me.y) ? me.y : 0.;
    anchor[L] = anchor_of(cx, cy, G);
}

__device__ __forceinline__ float rel(double v, float a) { return (float)(v - (double)a); }

// Initial records: position in own leaf frame and the sign of g.
__global__ void k_rec0(int64_t n, const int32_t* __restrict__ leaf_of, const float2* __restrict__ anchor, double G,
                       const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ g,
                       float4* rec0, double* x0, double* y0, double* g0, int32_t* partner, int32_t* zb,
                       int32_t* zb_prev) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 a = anchor[leaf_of[i]];
    double xi = x[i], yi = y[i], gi = g[i];
    rec0[i] = make_float4(rel(xi, a.x), rel(yi, a.y), (float)dsgn(gi), 0.f);
    x0[i] = xi; y0[i] = yi; g0[i] = gi;
    partner[i] = -1;
    zb[i] = INT_MAX;
    zb_prev[i] = INT_MAX;
}

// Per-leaf FP32 box (own frame) over every position a non-zero member may have this round,
// and the number of members that are live for every target (never absorbed, non-zero).
// Also keeps the previous round's box, and the largest squared search radius any member's
// last evaluation used (rreg; -1 when no member searched).
__global__ void k_eps_box(int64_t nl, const int32_t* __restrict__ lvf, const int32_t* __restrict__ lvl,
                          const float4* __restrict__ rec0, const float4* __restrict__ recO,
                          const int32_t* __restrict__ partner, const int32_t* __restrict__ zb, float4* box,
                          float4* box_prev, int32_t* live, const float* __restrict__ sr1,
                          const float* __restrict__ sr2, float* rreg, int first_round, int32_t* changed) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L == 0) *changed = 0;  // the round's changed flag (read by the host after the last round)
    if (L >= nl) return;
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    int32_t nlive = 0;
    float rr = -1.f;
    if (!first_round)
        for (int32_t i = lvf[L]; i < lvl[L]; i++) rr = fmaxf(rr, fmaxf(sr1[i], sr2[i]));
    for (int32_t i = lvf[L]; i < lvl[L]; i++) {
        float4 r = rec0[i];
        if (r.z != 0.f) {
            mnx = fminf(mnx, r.x); mny = fminf(mny, r.y); mxx = fmaxf(mxx, r.x); mxy = fmaxf(mxy, r.y);
        }
        bool moved = partner[i] >= 0;
        if (moved) {
            float4 o = recO[i];
            mnx = fminf(mnx, o.x); mny = fminf(mny, o.y); mxx = fmaxf(mxx, o.x); mxy = fmaxf(mxy, o.y);
        }
        if (r.z != 0.f && zb[i] == INT_MAX && (!moved || recO[i].z != 0.f)) nlive++;
    }
    const float4 nb = make_float4(mnx, mny, mxx, mxy);
    box_prev[L] = first_round ? nb : box[L];
    box[L] = nb;
    live[L] = nlive;
    rreg[L] = first_round ? INFINITY : rr;
}

// Candidate leaves of every target leaf (one warp per target leaf).
//
// R_L bounds every target's second-nearest distance from above: the farthest-corner
// distance between L's box and a leaf holding two live vortices (three for L itself, which
// contains the target; then R_L is L's own diagonal).  The first search of a target needs
// only candidates within R_L of it.  The list keeps near leaves within 2 R_L of L's box and
// remembers that radius; in later rounds it stays valid while R_L (now) plus the largest
// merge displacement fits inside it (boxes only grow by merged positions), otherwise it is
// rebuilt.  The re-search after a merge (from a point up to R_L away) walks the whole near
// list instead.  The warp also collects the near leaves whose members' outcomes changed in
// the last round (L is dirty when there is one) and records the extents of the list and of
// the near region in L's frame.
__global__ void k_eps_cand(int64_t nl, const int32_t* __restrict__ near_off, const int2* __restrict__ near_run,
                           const float2* __restrict__ anchor, const float4* __restrict__ box,
                           const int32_t* __restrict__ live, float Gf, int32_t* cand, int32_t* ncand, float* rn,
                           float* rlist, float* rnear, const int32_t* __restrict__ leaf_changed, int32_t* dirty,
                           int32_t* chg, int32_t* nchg, const float4* __restrict__ box_prev,
                           const float* __restrict__ rreg, const int32_t* __restrict__ chg_pre, int first_round,
                           const int32_t* __restrict__ leaf_disp, const int32_t* __restrict__ chg_list,
                           float* dloc_store) {
    __shared__ int2 s_runs[EB / 32][32];
    const int wq = threadIdx.x >> 5;
    const int64_t L = (int64_t)blockIdx.x * (blockDim.x / 32) + wq;
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    const int32_t r0 = near_off[L], r1 = near_off[L + 1];
    if (!first_round) {
        // No near leaf changed in the last round (prefix sums of the changed flags over each
        // near run): the boxes the list was checked against are unchanged, so the list stays
        // valid and no target of L needs a new evaluation.
        bool any = false;
        for (int32_t r = r0 + lane; r < r1; r += 32) {
            const int2 run = near_run[r];
            any = any || chg_pre[run.y] != chg_pre[run.x];
        }
        if (!__any_sync(0xffffffffu, any)) {
            if (lane == 0) { dirty[L] = 0; nchg[L] = 0; }
            return;
        }
    }
    const float4 bL = box[L];
    const float2 aL = anchor[L];
    // upper bound on every target's second-nearest distance (squared)
    float R2 = INFINITY;
    if (bL.x <= bL.z) {
        if (live[L] >= 3) {
            const float ux = bL.z - bL.x, uy = bL.w - bL.y;
            R2 = ux * ux + uy * uy;
        } else {
            for_near_leaves(near_run, r0, r1, s_runs[wq], [&](int32_t q, bool ok) {
                if (!ok) return;
                const int need = (q == L) ? 3 : 2;
                if (live[q] < need) return;
                const float4 b = box[q];
                const float2 sh = frame_shift(anchor[q], aL, Gf);
                const float ux = fmaxf(fabsf(b.z + sh.x - bL.x), fabsf(bL.z - (b.x + sh.x)));
                const float uy = fmaxf(fabsf(b.w + sh.y - bL.y), fabsf(bL.w - (b.y + sh.y)));
                R2 = fminf(R2, ux * ux + uy * uy);
            });
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) R2 = fminf(R2, __shfl_xor_sync(0xffffffffu, R2, o));
        }
    }
    const float absm = ldexpf(fabsf(bL.x) + fabsf(bL.z) + fabsf(bL.y) + fabsf(bL.w) + Gf, -12);
    const int32_t nc_old = first_round ? -2 : ncand[L];
    const bool try_reuse = !first_round && nc_old >= 0 && isfinite(R2);
    // Near leaves whose members' outcomes changed in the last round and whose box (this or
    // the last round's, which hold every position those members had) comes within the
    // largest search radius of L's targets; each target then checks them against its own
    // search regions.  L itself always counts (a member's absorber may have changed).
    int32_t nch = 0;
    const float rr2 = first_round ? -1.f : rreg[L];
    const float rreach = isfinite(rr2) ? sqrtf(fmaxf(rr2, 0.f)) * (1.f + 1e-4f) : INFINITY;
    auto box_gap = [&](float4 b, float2 sh) {
        if (!(b.x <= b.z)) return INFINITY;
        const float dx = fmaxf(fmaxf(b.x + sh.x - bL.z, bL.x - (b.z + sh.x)), 0.f);
        const float dy = fmaxf(fmaxf(b.y + sh.y - bL.w, bL.y - (b.w + sh.y)), 0.f);
        const float slack = ldexpf(fabsf(b.x + sh.x) + fabsf(b.z + sh.x) + fabsf(b.y + sh.y) + fabsf(b.w + sh.y), -12);
        return sqrtf(dx * dx + dy * dy) - slack;
    };
    auto collect = [&](int32_t q, bool ok) {
        bool ch = ok && !first_round && leaf_changed[q];
        if (ch && q != L) {
            if (!(rr2 >= 0.f)) {
                ch = false;  // no member of L searched: only its own absorbers matter
            } else if (isfinite(rreach)) {
                const float2 sh = frame_shift(anchor[q], aL, Gf);
                const float gap = fminf(box_gap(box[q], sh), box_gap(box_prev[q], sh));
                ch = gap <= rreach + absm;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, ch);
        if (ch) {
            const int pos = nch + __popc(m & ((1u << lane) - 1));
            if (pos < CHG_CAP) chg[(size_t)L * CHG_CAP + pos] = q;
        }
        nch += __popc(m);
    };
    // The list stays valid while R_L (now) plus the largest merge displacement of the near
    // leaves' members fits inside the radius it was built with: a leaf left out had its box
    // farther than that radius, and a box only grows by its members' merged positions.
    // That displacement is bounded by the one last computed for L (dloc_store) and the
    // current one of the near leaves that changed since (an unchanged leaf's members have
    // the same merges, so the same displacement); only the changed leaves are visited.
    bool collected = false;
    if (try_reuse) {
        float dloc = 0.f;
        for_listed_near_leaves(near_run, r0, r1, chg_pre, chg_list, s_runs[wq], [&](int32_t q, bool ok) {
            collect(q, ok);
            if (ok) dloc = fmaxf(dloc, __int_as_float(leaf_disp[q]));
        });
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dloc = fmaxf(dloc, __shfl_xor_sync(0xffffffffu, dloc, o));
        dloc = fmaxf(dloc, dloc_store[L]);
        const float need_r = sqrtf(R2) * (1.f + 1e-4f) + dloc + absm;
        if (need_r <= rlist[L]) {
            if (lane == 0) {
                nchg[L] = (nch > CHG_CAP) ? -1 : nch;
                dirty[L] = nch > 0 ? 1 : 0;
                dloc_store[L] = dloc;
            }
            return;
        }
        collected = true;
    }
    // (re)build: near leaves within 2 R_L of L's box (FP32 with margins)
    const float lim = isfinite(R2) ? 2.f * sqrtf(R2) * (1.f + 1e-4f) + absm : INFINITY;
    float ext = 0.f, next = 0.f, dall = 0.f;
    int32_t cnt = 0;
    for_near_leaves(near_run, r0, r1, s_runs[wq], [&](int32_t q, bool ok) {
        bool hit = false;
        float e = 0.f;
        if (ok && !first_round) dall = fmaxf(dall, __int_as_float(leaf_disp[q]));  // nothing merges before the first epsilon round
        if (ok) {
            const float4 b = box[q];
            if (b.x <= b.z) {
                const float2 sh = frame_shift(anchor[q], aL, Gf);
                const float bx0 = b.x + sh.x, bx1 = b.z + sh.x, by0 = b.y + sh.y, by1 = b.w + sh.y;
                const float dx = fmaxf(fmaxf(bx0 - bL.z, bL.x - bx1), 0.f);
                const float dy = fmaxf(fmaxf(by0 - bL.w, bL.y - by1), 0.f);
                hit = !isfinite(lim) || (dx <= lim && dy <= lim && dx * dx + dy * dy <= lim * lim);
                e = fmaxf(fmaxf(fabsf(bx0), fabsf(bx1)), fmaxf(fabsf(by0), fabsf(by1)));
                next = fmaxf(next, e);
                if (!hit) e = 0.f;
            }
        }
        const unsigned mask = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int pos = cnt + __popc(mask & ((1u << lane) - 1));
            if (pos < CAND_CAP) cand[(size_t)L * CAND_CAP + pos] = q;
        }
        cnt += __popc(mask);
        ext = fmaxf(ext, e);
        if (!collected) collect(q, ok);
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ext = fmaxf(ext, __shfl_xor_sync(0xffffffffu, ext, o));
        next = fmaxf(next, __shfl_xor_sync(0xffffffffu, next, o));
        dall = fmaxf(dall, __shfl_xor_sync(0xffffffffu, dall, o));
    }
    if (lane == 0) {
        dloc_store[L] = dall;
        ncand[L] = (cnt > CAND_CAP) ? -1 : cnt;  // -1: use the whole near list
        rlist[L] = (cnt > CAND_CAP) ? -1.f : lim;
        // extents of the coordinates the searches form in L's frame
        const float own = fmaxf(fmaxf(fabsf(bL.x), fabsf(bL.z)), fmaxf(fabsf(bL.y), fabsf(bL.w)));
        rn[L] = fmaxf(ext, own + (isfinite(lim) ? lim : 0.f));
        if (first_round) rnear[L] = fmaxf(next, own);
        nchg[L] = (nch > CHG_CAP) ? -1 : nch;
        dirty[L] = (first_round || nch > 0) ? 1 : 0;
    }
}

struct Top2 {
    double r1, r2;
    int32_t l1, l2;
    float thr;  // FP32 squared radius in the leaf frame holding every candidate that can decide
    uint32_t nrec;  // candidate records read by the FP32 pass
};

__device__ __forceinline__ void top2_push(Top2& t, double d, int32_t j) {
    if (!(d < DBL_MAX)) return;  // the reference never registers DBL_MAX or NaN
    // lexicographic (distance, list position); list position = slot index
    if (d < t.r1 || (d == t.r1 && j < t.l1)) { t.r2 = t.r1; t.l2 = t.l1; t.r1 = d; t.l1 = j; }
    else if (d < t.r2 || (d == t.r2 && j < t.l2)) { t.r2 = d; t.l2 = j; }
}

struct EpsView {
    const int32_t* lvf; const int32_t* lvl;
    const float2* anchor; const float4* box; const float* rn; const float* rnear; const float* dmax;
    const int32_t* near_off; const int2* near_run;
    const int32_t* cand; const int32_t* ncand;
    const float4* rec0; const float4* recO;
    const double* x0; const double* y0; const double* g0;
    const int32_t* partner; const int32_t* zb;
    const double* ox; const double* oy; const double* og;
    double G; float Gf;
};

// Candidate state as of the turn of target i.
struct Cand {
    bool live;
    float4 rec;
};
// FIRST: the first round, where nobody is absorbed or merged yet (no state to look up).
template <bool FIRST>
__device__ __forceinline__ Cand cand_state(const EpsView& v, int32_t j, int32_t i, int32_t excl) {
    Cand c;
    c.live = false;
    if (j == i || j == excl) return c;
    if (FIRST) {
        c.rec = v.rec0[j];
        c.live = c.rec.z != 0.f;
        return c;
    }
    if (v.zb[j] < i) return c;
    bool moved = (j < i) && (v.partner[j] >= 0);
    c.rec = moved ? v.recO[j] : v.rec0[j];
    c.live = c.rec.z != 0.f;
    return c;
}
template <bool FIRST>
__device__ __forceinline__ void cand_exact(const EpsView& v, int32_t j, int32_t i, double& xj, double& yj, double& gj) {
    bool moved = !FIRST && (j < i) && (v.partner[j] >= 0);
    xj = moved ? v.ox[j] : v.x0[j];
    yj = moved ? v.oy[j] : v.y0[j];
    gj = moved ? v.og[j] : v.g0[j];
}

// FP32 squared distance of a candidate, formed the same way by every search kernel
__device__ __forceinline__ float cand_d2(float dx, float dy) { return __fmaf_rn(dx, dx, __fmul_rn(dy, dy)); }

__device__ __forceinline__ float thr_of(float t2, float D) {
    if (!(t2 < INFINITY)) return INFINITY;
    float r = sqrtf(t2) * (1.f + 1e-5f) + 2.f * D;
    return r * r * (1.f + 1e-6f);
}

__device__ __forceinline__ float box_lb(float4 b, float2 sh, float tx, float ty) {
    float bx0 = b.x + sh.x, bx1 = b.z + sh.x, by0 = b.y + sh.y, by1 = b.w + sh.y;
    float dx = fmaxf(fmaxf(bx0 - tx, tx - bx1), 0.f);
    float dy = fmaxf(fmaxf(by0 - ty, ty - by1), 0.f);
    return dx * dx + dy * dy;
}

// Candidates met by the FP32 pass whose distance was within the threshold at the time
// (the threshold only shrinks, so they include every candidate within the final one).
// When it overflows, the exact pass scans the candidate leaves again.
constexpr int NBUF = 12;
struct NearBuf {
    float d[NBUF];
    int32_t j[NBUF];
    int n = 0;
    bool ovf = false;
    uint32_t nrec = 0;  // records read by the FP32 pass (leaves its box test did not prune)
    __device__ __forceinline__ void push(float dd, int32_t jj, float thr) {
        if (n == NBUF) {  // drop what the threshold has excluded since
            int m = 0;
            for (int k = 0; k < NBUF; k++)
                if (d[k] <= thr) { d[m] = d[k]; j[m] = j[k]; m++; }
            n = m;
        }
        if (n < NBUF) { d[n] = dd; j[n] = jj; n++; }
        else ovf = true;
    }
};

// Visits leaf q's live candidates for target i (shared by both passes).
template <int PASS, bool FIRST>
__device__ __forceinline__ void scan_leaf(const EpsView& v, int32_t q, float2 aL, int32_t i, int32_t excl, float tx,
                                          float ty, double px, double py, float D, float& t1, float& t2,
                                          float& thr, Top2& best, NearBuf& buf) {
    float2 sh = frame_shift(v.anchor[q], aL, v.Gf);
    if (box_lb(v.box[q], sh, tx, ty) > thr) return;
    if (PASS == 0) buf.nrec += (uint32_t)(v.lvl[q] - v.lvf[q]);
    for (int32_t j = v.lvf[q]; j < v.lvl[q]; j++) {
        Cand c = cand_state<FIRST>(v, j, i, excl);
        if (!c.live) continue;
        float dx = tx - (c.rec.x + sh.x), dy = ty - (c.rec.y + sh.y);
        float d = cand_d2(dx, dy);
        if (PASS == 0) {
            if (d < t1) { t2 = t1; t1 = d; thr = thr_of(t2, D); }
            else if (d < t2) { t2 = d; thr = thr_of(t2, D); }
            if (d <= thr) buf.push(d, j, thr);
        } else if (d <= thr) {
            double xj, yj, gj;
            cand_exact<FIRST>(v, j, i, xj, yj, gj);
            top2_push(best, dabs2(dsub(px, xj), dsub(py, yj)), j);
        }
    }
}

// Two nearest live candidates of target i (at exact position px,py) among leaf L's
// candidate leaves, excluding slot excl.  Returns the exact FP64 top-2 of the reference.
template <bool FIRST>
__device__ Top2 two_nearest(const EpsView& v, int32_t L, int32_t i, int32_t excl, double px, double py,
                            bool use_list) {
    const float2 aL = v.anchor[L];
    const float tx = (float)(px - (double)aL.x), ty = (float)(py - (double)aL.y);
    const float ext = (use_list ? v.rn[L] : v.rnear[L]) + *v.dmax;
    const float D = ldexpf(ext + fabsf(tx) + fabsf(ty) + v.Gf, -17);
    float t1 = INFINITY, t2 = INFINITY, thr = INFINITY;
    Top2 best{DBL_MAX, DBL_MAX, INT_MAX, INT_MAX, INFINITY, 0};
    const int32_t nc = use_list ? v.ncand[L] : -1;
    NearBuf buf;
    // pass 0: FP32 second-smallest distance, buffering the candidates within the running
    // threshold; then the exact top-2 over the buffered candidates within the final margin
    // (pass 1 rescans the leaves only when the buffer overflowed)
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            thr = thr_of(t2, D);
            if (!buf.ovf) {
                for (int k = 0; k < buf.n; k++) {
                    if (!(buf.d[k] <= thr)) continue;
                    double xj, yj, gj;
                    cand_exact<FIRST>(v, buf.j[k], i, xj, yj, gj);
                    top2_push(best, dabs2(dsub(px, xj), dsub(py, yj)), buf.j[k]);
                }
                break;
            }
        }
        if (pass == 0) scan_leaf<0, FIRST>(v, L, aL, i, excl, tx, ty, px, py, D, t1, t2, thr, best, buf);
        else scan_leaf<1, FIRST>(v, L, aL, i, excl, tx, ty, px, py, D, t1, t2, thr, best, buf);
        if (nc >= 0) {
            const int32_t* cl = v.cand + (size_t)L * CAND_CAP;
            for (int32_t k = 0; k < nc; k++) {
                int32_t q = cl[k];
                if (q == L) continue;
                if (pass == 0) scan_leaf<0, FIRST>(v, q, aL, i, excl, tx, ty, px, py, D, t1, t2, thr, best, buf);
                else scan_leaf<1, FIRST>(v, q, aL, i, excl, tx, ty, px, py, D, t1, t2, thr, best, buf);
            }
        } else {
            for (int32_t r = v.near_off[L]; r < v.near_off[L + 1]; r++) {
                int2 run = v.near_run[r];
                for (int32_t q = run.x; q < run.y; q++) {
                    if (q == L) continue;
                    if (pass == 0) scan_leaf<0, FIRST>(v, q, aL, i, excl, tx, ty, px, py, D, t1, t2, thr, best, buf);
                    else scan_leaf<1, FIRST>(v, q, aL, i, excl, tx, ty, px, py, D, t1, t2, thr, best, buf);
                }
            }
        }
    }
    best.thr = thr;
    best.nrec = buf.nrec;
    return best;
}

// Warp-collective two_nearest for the rounds with few targets (their time is the longest
// single search).  The lanes split the candidate leaves (lane k takes every 32nd one, the
// target's own leaf included) and keep their own FP32 two smallest distances, pruning with
// their own threshold (never below the final one); the warp's two smallest give the final
// threshold, then each lane takes the exact FP64 top-2 of its candidates within it and the
// warp merges those in (distance, slot) order.  The two smallest FP32 distances, the final
// threshold and the exact (distance, slot) top-2 do not depend on the order in which the
// candidates are met, so the result is two_nearest's.  Every lane returns it.
__device__ __forceinline__ void min2_merge(float& t1, float& t2, float a1, float a2) {
    const float n1 = fminf(t1, a1);
    t2 = fminf(fmaxf(t1, a1), fminf(t2, a2));
    t1 = n1;
}
__device__ Top2 two_nearest_w(const EpsView& v, int32_t L, int32_t i, int32_t excl, double px, double py,
                              bool use_list, int2* s_runs) {
    const int lane = threadIdx.x & 31;
    const float2 aL = v.anchor[L];
    const float tx = (float)(px - (double)aL.x), ty = (float)(py - (double)aL.y);
    const float ext = (use_list ? v.rn[L] : v.rnear[L]) + *v.dmax;
    const float D = ldexpf(ext + fabsf(tx) + fabsf(ty) + v.Gf, -17);
    float t1 = INFINITY, t2 = INFINITY, thr = INFINITY;
    uint32_t nrec = 0;
    Top2 best{DBL_MAX, DBL_MAX, INT_MAX, INT_MAX, INFINITY, 0};
    const int32_t nc = use_list ? v.ncand[L] : -1;
    const int32_t* cl = v.cand + (size_t)L * CAND_CAP;
    {
        // starting threshold for the lanes' pruning: the warp's two smallest distances over
        // L's own members (not below the final threshold, which takes every candidate)
        float s1 = INFINITY, s2 = INFINITY;
        for (int32_t j = v.lvf[L] + lane; j < v.lvl[L]; j += 32) {
            Cand c = cand_state<false>(v, j, i, excl);
            if (!c.live) continue;
            const float d = cand_d2(tx - c.rec.x, ty - c.rec.y);
            if (d < s1) { s2 = s1; s1 = d; }
            else if (d < s2) s2 = d;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            min2_merge(s1, s2, __shfl_xor_sync(0xffffffffu, s1, o), __shfl_xor_sync(0xffffffffu, s2, o));
        thr = thr_of(s2, D);
    }
#pragma unroll 1
    for (int pass = 0; pass < 2; pass++) {
        auto visit = [&](int32_t q) {
            const float2 sh = frame_shift(v.anchor[q], aL, v.Gf);
            if (box_lb(v.box[q], sh, tx, ty) > thr) return;
            if (pass == 0) nrec += (uint32_t)(v.lvl[q] - v.lvf[q]);
            for (int32_t j = v.lvf[q]; j < v.lvl[q]; j++) {
                Cand c = cand_state<false>(v, j, i, excl);
                if (!c.live) continue;
                const float dx = tx - (c.rec.x + sh.x), dy = ty - (c.rec.y + sh.y);
                const float d = cand_d2(dx, dy);
                if (pass == 0) {
                    if (d < t1) { t2 = t1; t1 = d; thr = fminf(thr, thr_of(t2, D)); }
                    else if (d < t2) { t2 = d; thr = fminf(thr, thr_of(t2, D)); }
                } else if (d <= thr) {
                    double xj, yj, gj;
                    cand_exact<false>(v, j, i, xj, yj, gj);
                    top2_push(best, dabs2(dsub(px, xj), dsub(py, yj)), j);
                }
            }
        };
        if (lane == 0) visit(L);
        if (nc >= 0) {
            for (int32_t k = lane; k < nc; k += 32) {
                const int32_t q = cl[k];
                if (q != L) visit(q);
            }
        } else {
            for_near_leaves(v.near_run, v.near_off[L], v.near_off[L + 1], s_runs, [&](int32_t q, bool ok) {
                if (ok && q != L) visit(q);
            });
        }
        if (pass == 0) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                min2_merge(t1, t2, __shfl_xor_sync(0xffffffffu, t1, o), __shfl_xor_sync(0xffffffffu, t2, o));
            thr = thr_of(t2, D);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double r1 = __shfl_xor_sync(0xffffffffu, best.r1, o), r2 = __shfl_xor_sync(0xffffffffu, best.r2, o);
        const int32_t l1 = __shfl_xor_sync(0xffffffffu, best.l1, o), l2 = __shfl_xor_sync(0xffffffffu, best.l2, o);
        if (l1 != INT_MAX) top2_push(best, r1, l1);
        if (l2 != INT_MAX) top2_push(best, r2, l2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nrec += __shfl_xor_sync(0xffffffffu, nrec, o);
    best.thr = thr;
    best.nrec = nrec;
    return best;
}

// Inputs of the last round's evaluation of a target, to tell whether it must run again.
struct DirtyView {
    const int32_t* zb_prev;   // absorber table the last evaluation saw
    const int32_t* vch;       // vortex outcome changed in the last round
    const int32_t* chg; const int32_t* nchg;
    const float4* recO_old;   // merged records of the outcomes before the last round
    float* sr1; float* sr2;   // search radii^2 of the last evaluation (< 0: no search)
};

// True when target i's evaluation can differ from its last one: its absorber changed, or a
// vortex whose outcome changed had (or now has) a position inside one of the regions its
// last searches examined (the first search around its own position, the re-search around
// its merged position).  Positions and distances are formed exactly as the searches form
// them, so every candidate that could enter a top-2 is seen.
__device__ __forceinline__ bool touched(const EpsView& v, const DirtyView& d, int32_t L, int32_t i) {
    if (d.zb_prev[i] != v.zb[i]) return true;
    const float r1 = d.sr1[i], r2 = d.sr2[i];
    if (!(r1 >= 0.f) && !(r2 >= 0.f)) return false;  // skipped last time, for the same reason now
    const int32_t nch = d.nchg[L];
    if (nch < 0) return true;
    const float2 aL = v.anchor[L];
    const float4 me = v.rec0[i];
    const float4 mo = v.recO[i];
    const float r1m = r1 * (1.f + 1e-5f), r2m = r2 * (1.f + 1e-5f);
    for (int32_t k = 0; k < nch; k++) {
        const int32_t q = d.chg[(size_t)L * CHG_CAP + k];
        const float2 sh = frame_shift(v.anchor[q], aL, v.Gf);
        for (int32_t j = v.lvf[q]; j < v.lvl[q]; j++) {
            if (!d.vch[j] || j == i) continue;
#pragma unroll
            for (int w = 0; w < 3; w++) {
                const float4 p = (w == 0) ? v.rec0[j] : (w == 1 ? v.recO[j] : d.recO_old[j]);
                const float px = p.x + sh.x, py = p.y + sh.y;
                if (r1 >= 0.f) {
                    const float dx = me.x - px, dy = me.y - py;
                    if (!(dx * dx + dy * dy > r1m)) return true;
                }
                if (r2 >= 0.f) {
                    const float dx = mo.x - px, dy = mo.y - py;
                    if (!(dx * dx + dy * dy > r2m)) return true;
                }
            }
        }
    }
    return false;
}

// Rounds after the first: targets whose inputs did not change keep their outcome; the
// others are flagged for evaluation (compacted in index order, so that neighbouring targets
// stay together in a warp).
__global__ void k_eps_mark(int64_t n, EpsView v, DirtyView dv, const int32_t* __restrict__ leaf_of,
                           const int32_t* __restrict__ dirty, const double* __restrict__ oie_old,
                           int32_t* partner_new, double* ox_new, double* oy_new, double* og_new, double* oie_new,
                           int32_t* flag) {
    int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= n) return;
    const int32_t i = (int32_t)ii;
    const int32_t L = leaf_of[i];
    const bool keep = !dirty[L] || !touched(v, dv, L, i);
    flag[i] = keep ? 0 : 1;
    if (keep) {  // no input of this target changed
        partner_new[i] = v.partner[i];
        ox_new[i] = v.ox[i]; oy_new[i] = v.oy[i]; og_new[i] = v.og[i]; oie_new[i] = oie_old[i];
    }
}

__global__ void k_eps_compact(int64_t n, const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                              int32_t* list) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) list[pos[i]] = (int32_t)i;
}

// One target's evaluation: its two nearest live candidates, the merge decision
// (MEpsilonFast.cpp:128-173) and its new epsilon.  WARP: the searches are warp-collective
// (two_nearest_w; every lane computes the same outcome).
struct Outcome {
    int32_t partner;
    double px, py, gi, ie;
    float sr1, sr2;
    uint32_t nrec;
};
template <bool FIRST, bool WARP>
__device__ __forceinline__ Outcome eval_target(const EpsView& v, int32_t i, const int32_t* __restrict__ leaf_of,
                                               const double* __restrict__ mcs_l, const double* __restrict__ epr_l,
                                               const double* __restrict__ ie_in, int2* s_runs) {
    auto search = [&](int32_t L, int32_t excl, double x, double y, bool use_list) {
        if constexpr (WARP) return two_nearest_w(v, L, i, excl, x, y, use_list, s_runs);
        else return two_nearest<FIRST>(v, L, i, excl, x, y, use_list);
    };
    const int32_t L = leaf_of[i];
    const double gi0 = v.g0[i];
    Outcome o{SKIPPED, v.x0[i], v.y0[i], gi0, ie_in[i], -1.f, -1.f, 0u};
    if (gi0 != 0 && !(v.zb[i] < i)) {
        const double mcs = mcs_l[L];
        Top2 t = search(L, -1, o.px, o.py, true);
        o.sr1 = t.thr;
        o.nrec += t.nrec;
        double e;
        o.partner = -1;
        if (t.l1 == INT_MAX) e = DBL_MIN;
        else if (t.l2 == INT_MAX) e = __dsqrt_rn(t.r1);
        else if (isnan(mcs)) e = __dsqrt_rn(t.r2);
        else {
            double x1, y1, g1, x2, y2, g2;
            cand_exact<FIRST>(v, t.l1, i, x1, y1, g1);
            cand_exact<FIRST>(v, t.l2, i, x2, y2, g2);
            if ((t.r1 < mcs) || ((dsgn(g1) == dsgn(g2)) && (dsgn(g1) != dsgn(o.gi)))) {
                // MergeVortexes (MEpsilonFast.cpp:111-126)
                if (dsgn(o.gi) == dsgn(g1)) {
                    double sx = dadd(dmul(o.px, o.gi), dmul(x1, g1));
                    double sy = dadd(dmul(o.py, o.gi), dmul(y1, g1));
                    double inv = ddiv(1., dadd(o.gi, g1));
                    o.px = dmul(sx, inv);
                    o.py = dmul(sy, inv);
                } else if (fabs(o.gi) < fabs(g1)) {
                    o.px = x1;
                    o.py = y1;
                }
                o.gi = dadd(o.gi, g1);
                o.partner = t.l1;
                Top2 u = search(L, t.l1, o.px, o.py, false);
                o.sr2 = u.thr;
                o.nrec += u.nrec;
                if (u.l1 == INT_MAX) e = DBL_MIN;
                else if (u.l2 == INT_MAX) e = __dsqrt_rn(u.r1);
                else e = __dsqrt_rn(u.r2);
            } else {
                e = __dsqrt_rn(t.r2);
            }
        }
        o.ie = ddiv(1.0, smax(e, epr_l[L]));
    }
    return o;
}

// Whether an outcome differs from target i's last one; stores it and its search radii.
__device__ __forceinline__ bool store_outcome(const EpsView& v, DirtyView& dv, int32_t i, const Outcome& o,
                                              const double* __restrict__ oie_old, int32_t* partner_new,
                                              double* ox_new, double* oy_new, double* og_new, double* oie_new) {
    const bool ch = (o.partner != v.partner[i] && !(o.partner == SKIPPED && v.partner[i] == SKIPPED)) ||
                    (__double_as_longlong(o.px) != __double_as_longlong(v.ox[i])) ||
                    (__double_as_longlong(o.py) != __double_as_longlong(v.oy[i])) ||
                    (__double_as_longlong(o.gi) != __double_as_longlong(v.og[i])) ||
                    (__double_as_longlong(o.ie) != __double_as_longlong(oie_old[i]));
    partner_new[i] = o.partner;
    ox_new[i] = o.px; oy_new[i] = o.py; og_new[i] = o.gi; oie_new[i] = o.ie;
    dv.sr1[i] = o.sr1;
    dv.sr2[i] = o.sr2;
    return ch;
}

// Rounds with at most this many targets run one warp per target (k_eps_round_w): their time
// is the longest single search, which the warp splits 32 ways.
constexpr int64_t EPS_WARP_MAX = 8192;
constexpr unsigned EPS_WARP_GRID = 152u * 16u;  // blocks of EB / 32 warps: one pass at the limit

// Evaluates every target (FIRST: the first round) or the targets list[0 .. *count) when
// there are more than EPS_WARP_MAX of them, one thread per target.
template <bool FIRST>
__global__ void k_eps_round(int64_t n, EpsView v, DirtyView dv, const int32_t* __restrict__ list,
                            const int32_t* __restrict__ count, const int32_t* __restrict__ leaf_of,
                            const double* __restrict__ mcs_l, const double* __restrict__ epr_l,
                            const double* __restrict__ ie_in, const double* __restrict__ oie_old,
                            int32_t* partner_new, double* ox_new, double* oy_new, double* og_new, double* oie_new,
                            int32_t* changed, unsigned long long* evals, unsigned long long* nrec_total) {
    const int64_t cnt = FIRST ? n : (int64_t)*count;
    if (!FIRST && cnt <= EPS_WARP_MAX) return;  // k_eps_round_w's
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(evals, (unsigned long long)cnt);
    const int64_t k0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t kstep = FIRST ? cnt : (int64_t)gridDim.x * blockDim.x;  // FIRST: one target per thread
    for (int64_t kk = k0; kk < cnt; kk += kstep) {
        const int32_t i = FIRST ? (int32_t)kk : list[kk];
        const Outcome o = eval_target<FIRST, false>(v, i, leaf_of, mcs_l, epr_l, ie_in, nullptr);
        const bool ch = store_outcome(v, dv, i, o, oie_old, partner_new, ox_new, oy_new, og_new, oie_new);
        const unsigned am = __activemask();  // one store per warp to the shared flag
        if (__any_sync(am, ch) && (threadIdx.x & 31) == __ffs(am) - 1) *changed = 1;
        const unsigned wrec = __reduce_add_sync(am, o.nrec);
        if ((threadIdx.x & 31) == __ffs(am) - 1) atomicAdd(nrec_total, (unsigned long long)wrec);
    }
}

// The targets list[0 .. *count) of a round after the first when there are at most
// EPS_WARP_MAX of them: one warp per target, same outcomes as k_eps_round.
__global__ void __launch_bounds__(EB) k_eps_round_w(EpsView v, DirtyView dv, const int32_t* __restrict__ list,
                                                    const int32_t* __restrict__ count,
                                                    const int32_t* __restrict__ leaf_of,
                                                    const double* __restrict__ mcs_l,
                                                    const double* __restrict__ epr_l,
                                                    const double* __restrict__ ie_in,
                                                    const double* __restrict__ oie_old, int32_t* partner_new,
                                                    double* ox_new, double* oy_new, double* og_new,
                                                    double* oie_new, int32_t* changed, unsigned long long* evals,
                                                    unsigned long long* nrec_total) {
    __shared__ int2 s_runs[EB / 32][32];
    const int64_t cnt = *count;
    if (cnt > EPS_WARP_MAX) return;  // k_eps_round's
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(evals, (unsigned long long)cnt);
    const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t kk = (int64_t)blockIdx.x * (EB / 32) + wq; kk < cnt; kk += (int64_t)gridDim.x * (EB / 32)) {
        const int32_t i = list[kk];
        const Outcome o = eval_target<false, true>(v, i, leaf_of, mcs_l, epr_l, ie_in, s_runs[wq]);
        if (lane == 0) {
            if (store_outcome(v, dv, i, o, oie_old, partner_new, ox_new, oy_new, og_new, oie_new)) *changed = 1;
            atomicAdd(nrec_total, (unsigned long long)o.nrec);
        }
        __syncwarp();
    }
}

// The changed leaves in order: list[rank] = q for every q with changed[q] (rank = pre[q]).
__global__ void k_chg_list(int64_t nl, const int32_t* __restrict__ changed, const int32_t* __restrict__ pre,
                           int32_t* list) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nl && changed[q]) list[pre[q]] = (int32_t)q;
}

// Also clears the round's per-leaf displacement bounds and changed flags [0, nl] and the
// largest displacement, which k_zb_scatter and k_leaf_changed then fill.
__global__ void k_zb_reset(int64_t n, int64_t nl, const int32_t* __restrict__ zb, int32_t* zb_prev, int32_t* zb_new,
                           int32_t* dmax_bits, int32_t* leaf_disp, int32_t* leaf_changed) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { zb_prev[i] = zb[i]; zb_new[i] = INT_MAX; }
    if (i <= nl) { leaf_disp[i] = 0; leaf_changed[i] = 0; }
    if (i == 0) *dmax_bits = 0;
}

__global__ void k_zb_scatter(int64_t n, const int32_t* __restrict__ partner, const int32_t* __restrict__ leaf_of,
                             const float2* __restrict__ anchor, double G, const double* __restrict__ ox,
                             const double* __restrict__ oy, const double* __restrict__ og,
                             const double* __restrict__ x0, const double* __restrict__ y0, int32_t* zb, float4* recO,
                             int32_t* dmax_bits, int32_t* leaf_disp) {
    __shared__ int s_max[EB / 32];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int dbits = 0;  // displacement bits (non-negative floats order as integers)
    if (i < n) {
        const int32_t p = partner[i];
        if (p >= 0) {
            atomicMin(&zb[p], (int32_t)i);
            float2 a = anchor[leaf_of[i]];
            recO[i] = make_float4(rel(ox[i], a.x), rel(oy[i], a.y), (float)dsgn(og[i]), 0.f);
            // displacement of the merged position (rounded up), for the candidate-list check
            float d = (float)(fabs(ox[i] - x0[i]) + fabs(oy[i] - y0[i])) * (1.f + 1e-5f);
            dbits = __float_as_int(d);
            atomicMax(&leaf_disp[leaf_of[i]], dbits);  // per leaf, for the list check
        }
    }
    // the global maximum: one atomic per block (every merged vortex would hit one address)
    dbits = __reduce_max_sync(0xffffffffu, dbits);
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = dbits;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = 0;
        for (int w = 0; w < EB / 32; w++) m = max(m, s_max[w]);
        if (m > 0) atomicMax(dmax_bits, m);
    }
}

// Leaves whose members' state (as other vortices see it) changed in the last round.
__global__ void k_leaf_changed(int64_t n, const int32_t* __restrict__ leaf_of, const int32_t* __restrict__ p_old,
                               const int32_t* __restrict__ p_new, const double* __restrict__ x_old,
                               const double* __restrict__ x_new, const double* __restrict__ y_old,
                               const double* __restrict__ y_new, const double* __restrict__ g_old,
                               const double* __restrict__ g_new, const int32_t* __restrict__ zb_old,
                               const int32_t* __restrict__ zb_new, int32_t* leaf_changed, int32_t* vch) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t po = p_old[i] < 0 ? -1 : p_old[i], pn = p_new[i] < 0 ? -1 : p_new[i];
    bool ch = (po != pn) || (zb_old[i] != zb_new[i]);
    if (pn >= 0) {
        ch = ch || __double_as_longlong(x_old[i]) != __double_as_longlong(x_new[i]) ||
             __double_as_longlong(y_old[i]) != __double_as_longlong(y_new[i]) ||
             __double_as_longlong(g_old[i]) != __double_as_longlong(g_new[i]);
    }
    vch[i] = ch ? 1 : 0;
    if (ch) leaf_changed[leaf_of[i]] = 1;
}

__global__ void k_eps_final(int64_t n, const int32_t* __restrict__ partner, const int32_t* __restrict__ zb,
                            const double* __restrict__ ox, const double* __restrict__ oy,
                            const double* __restrict__ og, const double* __restrict__ oie, double* x, double* y,
                            double* g, double* ie, unsigned long long* merged) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t p = partner[i];
    if (p != SKIPPED) ie[i] = oie[i];
    if (p >= 0) {
        x[i] = ox[i]; y[i] = oy[i]; g[i] = og[i];
        const unsigned am = __activemask();  // one atomic per warp
        if ((threadIdx.x & 31) == __ffs(am) - 1) atomicAdd(merged, (unsigned long long)__popc(am));
    }
    if (zb[i] != INT_MAX) g[i] = 0.;
}

}  // namespace

void eps_pass(Ctx& c, int merge, int64_t* merged) {
    cudaStream_t s = c.st();
    const int64_t n = c.n, nl = c.nleaves;
    // per-leaf merge criterion and epsilon floor
    c.lf_mcs.reserve(nl + 1);
    c.lf_epr.reserve(nl + 1);
    const int nb = (int)c.bodies.size();
    c.h_bfc.assign(2 * (size_t)nb + 2, 0);
    for (int b = 0; b < nb; b++) { c.h_bfc[b] = c.bodies[b].first; c.h_bfc[nb + 1 + b] = c.bodies[b].count; }
    c.e_bfc.reserve(c.h_bfc.size());
    VV_CUDA(cudaMemcpyAsync(c.e_bfc.p, c.h_bfc.data(), c.h_bfc.size() * 8, cudaMemcpyHostToDevice, s));
    const int64_t* dbf = c.e_bfc.p;
    const int64_t* dbc = c.e_bfc.p + nb + 1;
    c.e_seg32.reserve(c.m + 1);
    c.e_banchor.reserve(nb + 1);
    c.e_brad.reserve(nb + 1);
    if (nb > 0) {
        k_seg_frame<<<nb, EB, 0, s>>>(nb, dbf, dbc, c.s_rx.p, c.s_ry.p, c.e_seg32.p, c.e_banchor.p, c.e_brad.p);
        VV_LAUNCH_CHECK();
    }
    if (nl > 0) {
        k_leaf_params<<<grid_for(nl, EB), EB, 0, s>>>(nl, c.lf_geom.p, c.near_off.p, c.near_run.p, c.lf_sf.p,
                                                      c.lf_sl.p, c.seg_order.p, c.s_rx.p, c.s_ry.p, c.s_dlx.p,
                                                      c.s_dly.p, dbf, dbc, c.e_seg32.p, c.e_banchor.p, c.e_brad.p,
                                                      nb, merge, c.lf_mcs.p, c.lf_epr.p);
        VV_LAUNCH_CHECK();
    }
    if (n == 0) {
        if (merged) *merged = 0;
        VV_CUDA(cudaStreamSynchronize(s));
        c.stats.merged = 0;
        c.stats.merge_rounds = 0;
        return;
    }
    // frames
    const Frame fr{c.frame_G, (float)c.frame_G};
    c.lf_anchor.reserve(nl + 1);
    c.lf_box32.reserve(nl + 1);
    c.lf_rn.reserve(nl + 1);
    c.e_live.reserve(nl + 1);
    c.e_cand.reserve((size_t)nl * CAND_CAP + 1);
    c.e_ncand.reserve(nl + 1);
    c.e_dirty.reserve(nl + 1);
    c.e_lchanged.reserve(nl + 1);
    k_anchor<<<grid_for(nl, EB), EB, 0, s>>>(nl, c.lf_geom.p, fr.G, c.lf_anchor.p);
    VV_LAUNCH_CHECK();
    c.e_rec0.reserve(n); c.e_recO[0].reserve(n); c.e_recO[1].reserve(n);
    c.e_vch.reserve(n); c.e_sr1.reserve(n); c.e_sr2.reserve(n);
    c.e_chg.reserve((size_t)nl * CHG_CAP + 1);
    c.e_nchg.reserve(nl + 1);
    c.e_box_prev.reserve(nl + 1);
    c.e_lchg_pre.reserve(nl + 2);
    c.e_flag.reserve(n + 1);
    c.e_pos.reserve(n + 2);
    c.e_list.reserve(n + 1);
    c.e_rreg.reserve(nl + 1);
    VV_CUDA(cudaMemsetAsync(c.e_recO[0].p, 0, n * sizeof(float4), s));
    VV_CUDA(cudaMemsetAsync(c.e_recO[1].p, 0, n * sizeof(float4), s));
    c.e_x0.reserve(n); c.e_y0.reserve(n); c.e_g0.reserve(n); c.e_zb.reserve(n); c.e_zb_prev.reserve(n);
    for (int k = 0; k < 2; k++) {
        c.e_partner[k].reserve(n); c.e_ox[k].reserve(n); c.e_oy[k].reserve(n); c.e_og[k].reserve(n);
        c.e_oie[k].reserve(n);
    }
    c.e_changed.reserve(4);
    k_rec0<<<grid_for(n, EB), EB, 0, s>>>(n, c.leaf_of.p, c.lf_anchor.p, fr.G, c.x.p, c.y.p, c.g.p, c.e_rec0.p,
                                          c.e_x0.p, c.e_y0.p, c.e_g0.p, c.e_partner[0].p, c.e_zb.p, c.e_zb_prev.p);
    VV_LAUNCH_CHECK();
    // round-0 guess: nobody merges; outcomes equal to the input state
    VV_CUDA(cudaMemcpyAsync(c.e_ox[0].p, c.x.p, n * 8, cudaMemcpyDeviceToDevice, s));
    VV_CUDA(cudaMemcpyAsync(c.e_oy[0].p, c.y.p, n * 8, cudaMemcpyDeviceToDevice, s));
    VV_CUDA(cudaMemcpyAsync(c.e_og[0].p, c.g.p, n * 8, cudaMemcpyDeviceToDevice, s));
    VV_CUDA(cudaMemcpyAsync(c.e_oie[0].p, c.ie.p, n * 8, cudaMemcpyDeviceToDevice, s));
    int cur = 0;
    int64_t rounds = 0;
    const int64_t max_rounds = c.eps_max_rounds;
    c.e_rlist.reserve(nl + 1);
    c.e_ldisp.reserve(nl + 1);
    c.e_dloc.reserve(nl + 1);
    c.e_chglist.reserve(nl + 1);
    c.e_rnear.reserve(nl + 1);
    int32_t* dmax_bits = (int32_t*)(c.counters.p + 13);
    VV_CUDA(cudaMemsetAsync(dmax_bits, 0, 4, s));
    VV_CUDA(cudaMemsetAsync(c.counters.p + 14, 0, 8, s));
    VV_CUDA(cudaMemsetAsync(c.counters.p + 16, 0, 8, s));
    // One round: evaluations from the current guesses (buffer cr) into the other buffer.
    auto enqueue_round = [&](bool first, int cr) {
        // boxes and candidate leaves from the current guesses
        k_eps_box<<<grid_for(nl, EB), EB, 0, s>>>(nl, c.lf_vf.p, c.lf_vl.p, c.e_rec0.p, c.e_recO[cr].p,
                                                  c.e_partner[cr].p, c.e_zb.p, c.lf_box32.p, c.e_box_prev.p,
                                                  c.e_live.p, c.e_sr1.p, c.e_sr2.p, c.e_rreg.p, first,
                                                  c.e_changed.p);
        VV_LAUNCH_CHECK();
        {
            KernelTimer kt(c, VVGPU_T_EPS_CAND);
            k_eps_cand<<<grid_for(nl, EB / 32), EB, 0, s>>>(nl, c.near_off.p, c.near_run.p, c.lf_anchor.p,
                                                           c.lf_box32.p, c.e_live.p, fr.Gf, c.e_cand.p, c.e_ncand.p,
                                                           c.lf_rn.p, c.e_rlist.p, c.e_rnear.p, c.e_lchanged.p,
                                                           c.e_dirty.p, c.e_chg.p, c.e_nchg.p, c.e_box_prev.p,
                                                           c.e_rreg.p, c.e_lchg_pre.p, first, c.e_ldisp.p,
                                                           c.e_chglist.p, c.e_dloc.p);
            VV_LAUNCH_CHECK();
        }
        EpsView v{c.lf_vf.p, c.lf_vl.p, c.lf_anchor.p, c.lf_box32.p, c.lf_rn.p, c.e_rnear.p,
                  (const float*)dmax_bits, c.near_off.p, c.near_run.p,
                  c.e_cand.p, c.e_ncand.p, c.e_rec0.p, c.e_recO[cr].p, c.e_x0.p, c.e_y0.p, c.e_g0.p,
                  c.e_partner[cr].p, c.e_zb.p, c.e_ox[cr].p, c.e_oy[cr].p, c.e_og[cr].p, fr.G, fr.Gf};
        const int nx = cr ^ 1;
        DirtyView dv{c.e_zb_prev.p, c.e_vch.p, c.e_chg.p, c.e_nchg.p, c.e_recO[nx].p, c.e_sr1.p, c.e_sr2.p};
        const int32_t* list = nullptr;
        if (!first) {
            k_eps_mark<<<grid_for(n, EB), EB, 0, s>>>(n, v, dv, c.leaf_of.p, c.e_dirty.p, c.e_oie[cr].p,
                                                      c.e_partner[nx].p, c.e_ox[nx].p, c.e_oy[nx].p, c.e_og[nx].p,
                                                      c.e_oie[nx].p, c.e_flag.p);
            VV_LAUNCH_CHECK();
            exclusive_scan(c, c.e_flag.p, c.e_pos.p, n);
            k_eps_compact<<<grid_for(n, EB), EB, 0, s>>>(n, c.e_flag.p, c.e_pos.p, c.e_list.p);
            VV_LAUNCH_CHECK();
            list = c.e_list.p;
        }
        {
            KernelTimer kt(c, VVGPU_T_EPS_ROUND);
            if (first)
                // one-warp blocks: a block holds no warp waiting for a slower one (5.49
                // against 5.54 ms for the rounds at 4M with four-warp blocks)
                k_eps_round<true><<<grid_for(n, 32), 32, 0, s>>>(
                    n, v, dv, nullptr, nullptr, c.leaf_of.p, c.lf_mcs.p, c.lf_epr.p, c.ie.p, c.e_oie[cr].p,
                    c.e_partner[nx].p, c.e_ox[nx].p, c.e_oy[nx].p, c.e_og[nx].p, c.e_oie[nx].p, c.e_changed.p,
                    c.counters.p + 14, c.counters.p + 16);
            else {
                // the round's target count is on the device: each kernel returns at once
                // unless the count is its own
                k_eps_round<false><<<std::min<unsigned>(grid_for(n, EB), 152u * 32u), EB, 0, s>>>(
                    n, v, dv, list, c.e_pos.p + n, c.leaf_of.p, c.lf_mcs.p, c.lf_epr.p, c.ie.p, c.e_oie[cr].p,
                    c.e_partner[nx].p, c.e_ox[nx].p, c.e_oy[nx].p, c.e_og[nx].p, c.e_oie[nx].p, c.e_changed.p,
                    c.counters.p + 14, c.counters.p + 16);
                VV_LAUNCH_CHECK();
                k_eps_round_w<<<EPS_WARP_GRID, EB, 0, s>>>(
                    v, dv, list, c.e_pos.p + n, c.leaf_of.p, c.lf_mcs.p, c.lf_epr.p, c.ie.p, c.e_oie[cr].p,
                    c.e_partner[nx].p, c.e_ox[nx].p, c.e_oy[nx].p, c.e_og[nx].p, c.e_oie[nx].p, c.e_changed.p,
                    c.counters.p + 14, c.counters.p + 16);
            }
            VV_LAUNCH_CHECK();
        }
        // new absorber table and merged records; leaves whose members changed
        k_zb_reset<<<grid_for(std::max<int64_t>(n, nl + 1), EB), EB, 0, s>>>(
            n, nl, c.e_zb.p, c.e_zb_prev.p, c.e_zb.p, dmax_bits, c.e_ldisp.p, c.e_lchanged.p);
        VV_LAUNCH_CHECK();
        k_zb_scatter<<<grid_for(n, EB), EB, 0, s>>>(n, c.e_partner[nx].p, c.leaf_of.p, c.lf_anchor.p, fr.G,
                                                    c.e_ox[nx].p, c.e_oy[nx].p, c.e_og[nx].p, c.e_x0.p, c.e_y0.p,
                                                    c.e_zb.p, c.e_recO[nx].p, dmax_bits, c.e_ldisp.p);
        VV_LAUNCH_CHECK();
        k_leaf_changed<<<grid_for(n, EB), EB, 0, s>>>(n, c.leaf_of.p, c.e_partner[cr].p, c.e_partner[nx].p,
                                                      c.e_ox[cr].p, c.e_ox[nx].p, c.e_oy[cr].p, c.e_oy[nx].p,
                                                      c.e_og[cr].p, c.e_og[nx].p, c.e_zb_prev.p, c.e_zb.p,
                                                      c.e_lchanged.p, c.e_vch.p);
        VV_LAUNCH_CHECK();
        exclusive_scan(c, c.e_lchanged.p, c.e_lchg_pre.p, nl);
        k_chg_list<<<grid_for(nl, EB), EB, 0, s>>>(nl, c.e_lchanged.p, c.e_lchg_pre.p, c.e_chglist.p);
        VV_LAUNCH_CHECK();
    };
    const auto timeout = [] { return ApiError{VVGPU_ERR_TIMEOUT, "epsilon/merge rounds did not converge"}; };
    rounds = 1;
    enqueue_round(true, 0);
    cur = 1;
    int32_t changed = read_i32(c, c.e_changed.p);
    if (changed && rounds >= max_rounds) throw timeout();
    if (changed) {
        for (;;) {
            rounds++;
            enqueue_round(false, cur);
            cur ^= 1;
            changed = read_i32(c, c.e_changed.p);
            if (!changed) break;
            if (rounds >= max_rounds) throw timeout();
        }
    }
    VV_CUDA(cudaMemsetAsync(c.counters.p, 0, 8, s));
    k_eps_final<<<grid_for(n, EB), EB, 0, s>>>(n, c.e_partner[cur].p, c.e_zb.p, c.e_ox[cur].p, c.e_oy[cur].p,
                                               c.e_og[cur].p, c.e_oie[cur].p, c.x.p, c.y.p, c.g.p, c.ie.p,
                                               c.counters.p);
    VV_LAUNCH_CHECK();
    unsigned long long hl[3] = {0, 0, 0};
    unsigned long long* h3 = pinned_at(c, 128, hl);
    VV_CUDA(cudaMemcpyAsync(h3, c.counters.p, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaMemcpyAsync(h3 + 1, c.counters.p + 14, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaMemcpyAsync(h3 + 2, c.counters.p + 16, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    const unsigned long long mcount = h3[0], nev = h3[1], nrec = h3[2];
    c.eps_evaluations = (int64_t)nev;
    c.eps_records = (int64_t)nrec;
    if (merged) *merged = (int64_t)mcount;
    c.stats.merged = (int64_t)mcount;
    c.stats.merge_rounds = rounds;
}

}  // namespace vvgpu
