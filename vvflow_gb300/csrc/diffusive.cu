// Diffusive velocity of the Viscous Vortex Domains method
// (MDiffusiveFast::process_vort_list, libvvhd/src/MDiffusiveFast.cpp:8-48).
//
// For every non-zero vortex: I1, I2 over same-sign vortices of the near leaves
// (vortex_influence, :94-105), I0, I3 over the near leaves' wall segments
// (segment_influence, :108-123, which also accumulates wall friction), then the clamps of
// :41-45.  Every pair with exp argument -|dr|/eps < -8 contributes exactly zero in the
// reference, so whole near leaves farther than 8 eps from all targets of a leaf are
// skipped: the warp tests boxes once per (target leaf, near leaf) in FP32 with a margin.
//
// One warp per target leaf in both paths.  FP64 path (k_diff64): eight target slots times
// four source lanes, every pair in double precision with the reference's formulas.  FP32
// path (k_diff32): only same-sign pairs contribute, so the candidate sources (staged in
// shared memory per batch) are split by sign, and each target, one per lane group of
// 32 / G lanes (G the power of two at or above the targets of the pass), strides over the
// sources of its own sign only; vortex pairs in local frames (frame.cuh) with
// FP32 exp/rsqrt; pairs whose cut-off or coincidence test falls within a rigorous bound of
// the FP32 error of its threshold are re-evaluated in FP64, so the set of contributing
// pairs is the reference's.  Wall segments are always FP64.  Friction goes to TAtt::fric
// with FP64 atomics.
#include <cfloat>

#include "frame.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

// warps per block: two (12 blocks per SM in the FP32 pass): 5.52 ms at 4M against 5.74 ms for
// four and 6.33 ms for one
constexpr int DW = 2;
// FP32 path: shared-memory source records per warp (256: 5.74 ms at 4M against 5.85 ms for
// 320) and sources staged per warp at a time
constexpr int SRC_CAP = 256;
constexpr int SRC_BATCH = SRC_CAP - 32;
// candidate leaves gathered per warp before their sources are staged (64: 5.74 ms at 4M
// against 5.80 ms for 48 and 5.86 ms for 96)
constexpr int HIT_CAP = 64;

// Box of non-zero vortices and segment centres of each leaf, FP32 in the leaf's own frame.
__global__ void k_dbox(int64_t nl, const int32_t* __restrict__ lvf, const int32_t* __restrict__ lvl,
                       const int32_t* __restrict__ lsf, const int32_t* __restrict__ lsl,
                       const int32_t* __restrict__ seg_order, const double* __restrict__ x,
                       const double* __restrict__ y, const double* __restrict__ g, const double* __restrict__ rx,
                       const double* __restrict__ ry, const float2* __restrict__ anchor, double G, float4* box) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    float2 k = anchor[L];
    double ax = (double)k.x, ay = (double)k.y;
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (int32_t i = lvf[L]; i < lvl[L]; i++) {
        if (g[i] == 0.) continue;
        float px = (float)(x[i] - ax), py = (float)(y[i] - ay);
        mnx = fminf(mnx, px); mny = fminf(mny, py); mxx = fmaxf(mxx, px); mxy = fmaxf(mxy, py);
    }
    for (int32_t q = lsf[L]; q < lsl[L]; q++) {
        int32_t s = seg_order[q];
        float px = (float)(rx[s] - ax), py = (float)(ry[s] - ay);
        mnx = fminf(mnx, px); mny = fminf(mny, py); mxx = fmaxf(mxx, px); mxy = fmaxf(mxy, py);
    }
    box[L] = make_float4(mnx, mny, mxx, mxy);
}

struct DiffArgs {
    int64_t nl;
    const int32_t* lvf; const int32_t* lvl; const int32_t* lsf; const int32_t* lsl;
    const int32_t* near_off; const int2* near_run; const int32_t* seg_order;
    const double* x; const double* y; const double* g; const double* ie;
    double* vx; double* vy;
    const double* rx; const double* ry; const double* dlx; const double* dly; double* fric;
    const float2* anchor; const float4* box; const float4* src32; const float2* src_k; const float* src_ie;
    double G; float Gf; double re;
    unsigned long long* cand;
};

// Per-pair vortex term in FP64 exactly as vortex_influence (MDiffusiveFast.cpp:94-105).
__device__ __forceinline__ void vortex_term64(double xi, double yi, double gi, double ie, double xj, double yj,
                                              double gj, double& s2x, double& s2y, double& s1) {
    if (dsgn(gi) != dsgn(gj)) return;
    double dx = xi - xj, dy = yi - yj;
    if (fabs(dx) + fabs(dy) < 1E-10) return;
    double drabs = sqrt(dx * dx + dy * dy);
    double ea = -drabs * ie;
    if (ea < EXP_ARG_RESTRICTION) return;
    double t = gj * exp(ea);
    double q = t / drabs;
    s2x += dx * q; s2y += dy * q;
    s1 += t;
}

// Compensated accumulation: TwoSum (Knuth) of h + v, the rounding error collected in l.
__device__ __forceinline__ void acc_add(float& h, float& l, float v) {
    const float s = h + v;
    const float bp = s - h;
    l += (h - (s - bp)) + (v - bp);
    h = s;
}

// Double-float addition (a_h, a_l) += (b_h, b_l): TwoSum of the heads, tails added to the
// error term, renormalised by Fast2Sum (Dekker).
__device__ __forceinline__ void ff_add(float& ah, float& al, float bh, float bl) {
    const float s = ah + bh;
    const float bp = s - ah;
    float e = (ah - (s - bp)) + (bh - bp);
    e += al + bl;
    ah = s + e;
    al = e - (ah - s);
}

// FP64 path.  Warp per target leaf.  Lane = target slot (lane & 7) x source lane
// (lane >> 3): eight targets per pass, the four source lanes split each candidate leaf's
// vortices.  Candidate leaves come from a lane-parallel box test against the targets' box
// grown by 8 eps.  Every pair in double precision with the reference's formulas.
__global__ void __launch_bounds__(DW * 32) k_diff64(DiffArgs a) {
    __shared__ int2 s_runs[DW][32];
    const int wq = threadIdx.x >> 5;
    const int64_t L = (int64_t)blockIdx.x * DW + wq;
    const int lane = threadIdx.x & 31;
    const int ts = lane & 7, sl = lane >> 3;
    if (L >= a.nl) return;
    const float2 kL = a.anchor[L];
    const double axL = (double)kL.x, ayL = (double)kL.y;
    const int32_t v0 = a.lvf[L], v1 = a.lvl[L];
    const int32_t r0 = a.near_off[L], r1 = a.near_off[L + 1];
    unsigned long long ncand = 0;
    for (int32_t c0 = v0; c0 < v1; c0 += 8) {
        const int32_t i = c0 + ts;
        const bool act = (i < v1) && (a.g[i] != 0.);
        double xi = 0, yi = 0, gi = 0, ie = 0;
        float txf = 0, tyf = 0, reach = 0.f;
        if (act) {
            xi = a.x[i]; yi = a.y[i]; gi = a.g[i]; ie = a.ie[i];
            txf = (float)(xi - axL); tyf = (float)(yi - ayL);
            reach = (float)(8.0 / ie) * (1.f + 1e-4f);
        }
        float bx0 = act ? txf : INFINITY, by0 = act ? tyf : INFINITY;
        float bx1 = act ? txf : -INFINITY, by1 = act ? tyf : -INFINITY;
        float rmax = reach;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
            by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
            bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
            by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
            rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        }
        if (!(bx0 <= bx1)) continue;  // no active target in this group (warp-uniform)
        const float pad = rmax + ldexpf(fabsf(bx0) + fabsf(bx1) + fabsf(by0) + fabsf(by1) + a.Gf, -16);
        double s2x = 0, s2y = 0, s3x = 0, s3y = 0, s1 = 0, s0 = 0;
        for_near_leaves(a.near_run, r0, r1, s_runs[wq], [&](int32_t q, bool ok) {
            bool hit = false;
            if (ok) {
                const float4 b = a.box[q];
                if (b.x <= b.z) {
                    const float2 sh = frame_shift(a.anchor[q], kL, a.Gf);
                    const float dx = fmaxf(fmaxf(b.x + sh.x - bx1, bx0 - (b.z + sh.x)), 0.f);
                    const float dy = fmaxf(fmaxf(b.y + sh.y - by1, by0 - (b.w + sh.y)), 0.f);
                    hit = dx <= pad && dy <= pad && (dx * dx + dy * dy) <= pad * pad;
                }
            }
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            while (mask) {
                const int32_t qq = __shfl_sync(0xffffffffu, q, __ffs(mask) - 1);
                mask &= mask - 1;
                const int32_t j0 = a.lvf[qq], j1 = a.lvl[qq];
                if (!act) continue;
                if (sl == 0) ncand += (unsigned long long)(j1 - j0);
                for (int32_t j = j0 + sl; j < j1; j += 4) {
                    const double gj = a.g[j];
                    if (gj == 0.) continue;
                    vortex_term64(xi, yi, gi, ie, a.x[j], a.y[j], gj, s2x, s2y, s1);
                }
                // wall segments of this near leaf (segment_influence), split over source lanes
                for (int32_t qs = a.lsf[qq] + sl; qs < a.lsl[qq]; qs += 4) {
                    const int32_t sgm = a.seg_order[qs];
                    const double dx = xi - a.rx[sgm], dy = yi - a.ry[sgm];
                    const double dr2 = dx * dx + dy * dy;
                    const double dr = sqrt(dr2);
                    const double ea = -dr * ie;
                    if (ea < EXP_ARG_RESTRICTION) continue;
                    const double ex = exp(ea);
                    const double dsx = -a.dly[sgm], dsy = a.dlx[sgm];
                    s3x += dsx * ex; s3y += dsy * ex;
                    s0 += (dr * ie + 1) / dr2 * (dx * dsx + dy * dsy) * ex;
                    atomicAdd(&a.fric[sgm], ie * ie * gi * ex * sqrt(dsx * dsx + dsy * dsy));
                }
            }
        });
        // combine the four source lanes of each target slot
#pragma unroll
        for (int o = 8; o < 32; o <<= 1) {
            s2x += __shfl_xor_sync(0xffffffffu, s2x, o);
            s2y += __shfl_xor_sync(0xffffffffu, s2y, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s3x += __shfl_xor_sync(0xffffffffu, s3x, o);
            s3y += __shfl_xor_sync(0xffffffffu, s3y, o);
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        }
        if (act && sl == 0) {
            if ((dsgn(s1) != dsgn(gi)) || (fabs(s1) < fabs(0.1 * gi))) s1 = 0.1 * gi;
            double f = ie / (a.re * s1);
            double vx = a.vx[i] + s2x * f, vy = a.vy[i] + s2y * f;
            if (s0 > C_PI) s0 = C_PI;
            f = ie * ie / (a.re * (C_2PI - s0));
            vx += s3x * f;
            vy += s3y * f;
            a.vx[i] = vx;
            a.vy[i] = vy;
        }
    }
    ncand = warp_sum_u64(ncand);
    if (lane == 0 && ncand) atomicAdd(a.cand, ncand);
}

// FP32 path.  Warp per target leaf.  Only same-sign pairs contribute (vortex_influence,
// MDiffusiveFast.cpp:97), so each staged batch of candidate sources (up to HIT_CAP candidate
// leaves, flattened) is split by sign: positive sources from the front of the warp's
// buffer, negative ones from the back, zero ones dropped.  A pass takes up to TMAX targets
// of the leaf (a window of TMAX vortices), positives first; G (the power of two at or above
// its active targets) lane groups of 32 / G lanes each hold one target and stride over the
// sources of that target's sign only, all lanes stepping the same count (the longer
// list's) so that the loop and the compensated folds every 32 steps are warp-uniform.
// Pair arithmetic is FP32 in local frames.  Pairs whose cut-off or coincidence test falls
// within the rigorous FP32 error bound of its threshold are marked in a per-window mask and
// evaluated in FP64 after the window, outside the arithmetic loop; they and the wall-segment
// terms go to per-lane accumulators that are reduced in a fixed order, so results are
// reproducible.
template <int TMAX>
__global__ void __launch_bounds__(DW * 32, 12) k_diff32(DiffArgs a) {
    __shared__ int2 s_runs[DW][32];
    __shared__ int4 s_hit[DW][HIT_CAP];     // flattened start, first vortex, shift x, shift y (bits)
    __shared__ float2 s_hitb[DW][HIT_CAP];  // error bound D of the leaf
    __shared__ float4 s_src[DW][SRC_CAP];   // x, y in L's frame, g, index (bits); + front, - back
    __shared__ int32_t s_hitq[DW][HIT_CAP]; // leaf
    __shared__ unsigned long long s_nsrc[DW];
    __shared__ double s_d64[DW][6][32];     // per lane FP64 s2x, s2y, s1, s3x, s3y, s0
    const int wq = threadIdx.x >> 5;
    const int64_t L = (int64_t)blockIdx.x * DW + wq;
    const int lane = threadIdx.x & 31;
    if (L >= a.nl) return;
    const float2 kL = a.anchor[L];
    const int32_t v0 = a.lvf[L], v1 = a.lvl[L];
    const int32_t r0 = a.near_off[L], r1 = a.near_off[L + 1];
    const float bandc = ldexpf(64.f, -19);
    double(&d64)[6][32] = s_d64[wq];
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long ncand = 0;
    if (lane == 0) s_nsrc[wq] = 0ull;
    for (int k = lane; k < SRC_CAP; k += 32) s_src[wq][k] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    for (int32_t c0 = v0; c0 < v1; c0 += TMAX) {
        // signs of the window's vortices from their bit patterns (g != 0: active)
        const int32_t wi = c0 + lane;
        const unsigned long long gw =
            (lane < TMAX && wi < v1) ? (unsigned long long)__double_as_longlong(a.g[wi]) : 0ull;
        const bool nzw = (gw << 1) != 0ull;
        const unsigned P = __ballot_sync(0xffffffffu, nzw && (gw >> 63) == 0ull);
        const unsigned N = __ballot_sync(0xffffffffu, nzw && (gw >> 63) != 0ull);
        const int nP = __popc(P), na = nP + __popc(N);
        if (na == 0) continue;  // warp-uniform
        const int lgg = na <= 1 ? 0 : 32 - __clz(na - 1);  // log2 G
        const int lgl = 5 - lgg;                           // log2 of the lanes per group
        const int LG = 1 << lgl;
        const int grp = lane >> lgl, sub = lane & (LG - 1);
        const bool act = grp < na;
        const bool neg = grp >= nP;
        int32_t i = -1;
        float tx = 0.f, ty = 0.f, ief = 0.f, ie2 = 0.f, b16 = 0.f, iefl = 0.f, reach = 0.f;
        if (act) {
            unsigned m = neg ? N : P;
            for (int t = neg ? nP : 0; t < grp; t++) m &= m - 1u;
            i = c0 + (__ffs(m) - 1);
            const float4 r4 = a.src32[i];
            tx = r4.x; ty = r4.y;
            ief = a.src_ie[i];
            ie2 = ief * ief;
            iefl = ief * 1.4426950408889634f;  // log2(e) / eps
            b16 = 16.f * ief * (1.f + 1e-3f);
            reach = (8.f / ief) * (1.f + 1e-4f);
        }
        float bx0 = act ? tx : INFINITY, by0 = act ? ty : INFINITY;
        float bx1 = act ? tx : -INFINITY, by1 = act ? ty : -INFINITY, rmax = reach;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
            by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
            bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
            by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
            rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        }
        const float pad = rmax + ldexpf(fabsf(bx0) + fabsf(bx1) + fabsf(by0) + fabsf(by1) + a.Gf, -16);
        const float tmax = fmaxf(fmaxf(fabsf(bx0), fabsf(bx1)), fmaxf(fabsf(by0), fabsf(by1)));
        float p2x = 0.f, p2y = 0.f, p1 = 0.f, h2x = 0.f, l2x = 0.f, h2y = 0.f, l2y = 0.f, h1 = 0.f, l1 = 0.f;
        bool used64 = false;
        int since = 0;  // this lane's sources in the plain partial sums
        int nh_acc = 0;
        int32_t tot_acc = 0;
        bool seg_acc = false;
        const bool want_p = nP > 0, want_n = nP < na;
        auto flush = [&]() {
            float Dm = 0.f;
            for (int h = 0; h < nh_acc; h++) Dm = fmaxf(Dm, s_hitb[wq][h].x);
            const float tiny = 2.f * Dm + 1e-9f, tiny2 = tiny * tiny;
            const float bndv = fmaf(b16, Dm, bandc);
            for (int32_t kb = 0; kb < tot_acc; kb += SRC_BATCH) {
                const int32_t nst = min(SRC_BATCH, tot_acc - kb);
                // stage the batch's sources (shifted into L's frame), split by sign
                int np_b = 0, nn_b = 0;
                for (int32_t k0 = 0; k0 < nst; k0 += 32) {
                    const int32_t k = k0 + lane;
                    bool sp = false, sn = false;
                    float4 rec = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (k < nst) {
                        const int32_t kk = kb + k;
                        int lo = 0, hi = nh_acc - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (s_hit[wq][mid].x <= kk) lo = mid;
                            else hi = mid - 1;
                        }
                        const int4 hc = s_hit[wq][lo];
                        const int32_t j = hc.y + (kk - hc.x);
                        const float4 s4 = a.src32[j];
                        rec = make_float4(s4.x + __int_as_float(hc.z), s4.y + __int_as_float(hc.w), s4.z,
                                          __int_as_float(j));
                        sp = want_p && s4.z > 0.f;
                        sn = want_n && s4.z < 0.f;
                    }
                    const unsigned bp = __ballot_sync(0xffffffffu, sp), bn = __ballot_sync(0xffffffffu, sn);
                    if (sp) s_src[wq][np_b + __popc(bp & lt)] = rec;
                    if (sn) s_src[wq][SRC_CAP - 1 - (nn_b + __popc(bn & lt))] = rec;
                    np_b += __popc(bp);
                    nn_b += __popc(bn);
                }
                __syncwarp();
                // Every lane steps through max(np_b, nn_b) / LG sources (warp-uniform trip
                // count and fold points); steps beyond the lane's own list read a finite record
                // (the buffer is zeroed at the start and a batch fills at most SRC_BATCH <=
                // SRC_CAP - 32 of it, so no index leaves the buffer) and add exactly zero.
                const int nmine = act ? (neg ? nn_b : np_b) : 0;
                const int steps = (max(np_b, nn_b) + LG - 1) >> lgl;
                const int stride = neg ? -LG : LG;
                const float4* p = s_src[wq] + (neg ? SRC_CAP - 1 - sub : sub);
                int rem = nmine - sub;  // > 0: the lane's current source is in its list
                for (int s0 = 0; s0 < steps;) {
                    // at most 32 - since steps before the next fold
                    const int cnt = min(32 - since, steps - s0);
                    unsigned bmask = 0;  // band pairs of this window (bit: step within it)
                    const float4* pw = p;
                    for (int st = 0; st < cnt; st++) {
                        const float4 sv = *p;
                        p += stride;
                        const bool ok = rem > 0;
                        rem -= LG;
                        const float dx = tx - sv.x, dy = ty - sv.y;
                        const float r2 = dx * dx + dy * dy;
                        const float du = r2 * ie2 - 64.f;  // (|dr| / eps)^2 - 64
                        const bool in = ok && du <= -bndv && r2 >= tiny2;
                        const float r2c = in ? r2 : 1.f;
                        const float rs = rsqrtf(r2c);
                        // exp(-|dr| / eps) as 2^(-|dr| (log2(e) / eps)), one MUFU ex2
                        float ex2v;
                        asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(ex2v) : "f"(-(r2c * rs) * iefl));
                        const float tv = in ? sv.z * ex2v : 0.f;
                        const float qv = tv * rs;
                        p2x = fmaf(dx, qv, p2x);
                        p2y = fmaf(dy, qv, p2y);
                        p1 += tv;
                        // the cut-off or coincidence test within the FP32 error bound
                        if (ok && (fabsf(du) < bndv || r2 < tiny2)) bmask |= 1u << st;
                    }
                    // the window's band pairs, in order: the reference's FP64 test and term
                    // (a target's pair with itself excluded)
                    while (bmask) {
                        const int st = __ffs(bmask) - 1;
                        bmask &= bmask - 1u;
                        const int32_t j = __float_as_int(pw[st * stride].w);
                        if (j == i) continue;
                        if (!used64) {
                            for (int w = 0; w < 6; w++) d64[w][lane] = 0.;
                            used64 = true;
                        }
                        vortex_term64(a.x[i], a.y[i], a.g[i], a.ie[i], a.x[j], a.y[j], a.g[j], d64[0][lane],
                                      d64[1][lane], d64[2][lane]);
                    }
                    s0 += cnt;
                    since += cnt;
                    if (since == 32) {
                        since = 0;
                        acc_add(h2x, l2x, p2x); p2x = 0.f;
                        acc_add(h2y, l2y, p2y); p2y = 0.f;
                        acc_add(h1, l1, p1); p1 = 0.f;
                    }
                }
                __syncwarp();
            }
            if (seg_acc) {
                // wall segments of the candidate leaves (segment_influence, MDiffusiveFast.cpp:108-123), FP64
                for (int h = 0; h < nh_acc; h++) {
                    const int32_t qq = s_hitq[wq][h];
                    const int32_t qs0 = a.lsf[qq], qs1 = a.lsl[qq];
                    if (qs0 >= qs1 || !act) continue;
                    if (!used64) {
                        for (int w = 0; w < 6; w++) d64[w][lane] = 0.;
                        used64 = true;
                    }
                    const double xi = a.x[i], yi = a.y[i], gi = a.g[i], ie = a.ie[i];
                    for (int32_t qs = qs0 + sub; qs < qs1; qs += LG) {
                        const int32_t sgm = a.seg_order[qs];
                        const double dx = xi - a.rx[sgm], dy = yi - a.ry[sgm];
                        const double dr2 = dx * dx + dy * dy;
                        const double dr = sqrt(dr2);
                        const double ea = -dr * ie;
                        if (ea < EXP_ARG_RESTRICTION) continue;
                        const double ex = exp(ea);
                        const double dsx = -a.dly[sgm], dsy = a.dlx[sgm];
                        d64[3][lane] += dsx * ex;
                        d64[4][lane] += dsy * ex;
                        d64[5][lane] += (dr * ie + 1) / dr2 * (dx * dsx + dy * dsy) * ex;
                        atomicAdd(&a.fric[sgm], ie * ie * gi * ex * sqrt(dsx * dsx + dsy * dsy));
                    }
                }
            }
            __syncwarp();
            nh_acc = 0;
            tot_acc = 0;
            seg_acc = false;
        };
        for_near_leaves(a.near_run, r0, r1, s_runs[wq], [&](int32_t q, bool ok) {
            bool hit = false;
            float4 b = make_float4(0.f, 0.f, -1.f, -1.f);
            float2 sh = make_float2(0.f, 0.f);
            if (ok) {
                b = a.box[q];
                if (b.x <= b.z) {
                    sh = frame_shift(a.anchor[q], kL, a.Gf);
                    const float dx = fmaxf(fmaxf(b.x + sh.x - bx1, bx0 - (b.z + sh.x)), 0.f);
                    const float dy = fmaxf(fmaxf(b.y + sh.y - by1, by0 - (b.w + sh.y)), 0.f);
                    hit = dx <= pad && dy <= pad && (dx * dx + dy * dy) <= pad * pad;
                }
            }
            const unsigned mask = __ballot_sync(0xffffffffu, hit);
            if (!mask) return;
            int32_t j0 = 0, len = 0, segs = 0;
            if (hit) {
                j0 = a.lvf[q];
                len = a.lvl[q] - j0;
                segs = a.lsl[q] - a.lsf[q];
            }
            int32_t incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
            const int nh = __popc(mask);
            const bool any_seg = __any_sync(0xffffffffu, segs > 0);
            __syncwarp();
            if (hit) {
                const int r = __popc(mask & lt);
                // Bound D on the FP32 error of |dr| for any pair of this leaf: each of dx, dy
                // carries at most 2^-24 (|t| + |s| + |s + sh| + |dx|) from the roundings of the
                // records, the shift and the subtraction (4x slack).
                const float s4max = fmaxf(fmaxf(fabsf(b.x), fabsf(b.z)), fmaxf(fabsf(b.y), fabsf(b.w)));
                const float spmax = fmaxf(fmaxf(fabsf(b.x + sh.x), fabsf(b.z + sh.x)),
                                          fmaxf(fabsf(b.y + sh.y), fabsf(b.w + sh.y)));
                const float D = ldexpf(2.f * tmax + s4max + 2.f * spmax, -21);
                s_hit[wq][nh_acc + r] = make_int4(tot_acc + incl - len, j0, __float_as_int(sh.x), __float_as_int(sh.y));
                s_hitb[wq][nh_acc + r] = make_float2(D, 0.f);
                s_hitq[wq][nh_acc + r] = q;
            }
            __syncwarp();
            if (lane == 0) {
                ncand += (unsigned long long)na * (unsigned long long)total;
                s_nsrc[wq] += (unsigned long long)total;
            }
            nh_acc += nh;
            tot_acc += total;
            seg_acc = seg_acc || any_seg;
            if (nh_acc > HIT_CAP - 32) flush();
        });
        if (nh_acc > 0) flush();
        // fold, then combine the LG lanes of each group as double-float pairs
        acc_add(h2x, l2x, p2x);
        acc_add(h2y, l2y, p2y);
        acc_add(h1, l1, p1);
        for (int o = LG >> 1; o > 0; o >>= 1) {
            ff_add(h2x, l2x, __shfl_xor_sync(0xffffffffu, h2x, o), __shfl_xor_sync(0xffffffffu, l2x, o));
            ff_add(h2y, l2y, __shfl_xor_sync(0xffffffffu, h2y, o), __shfl_xor_sync(0xffffffffu, l2y, o));
            ff_add(h1, l1, __shfl_xor_sync(0xffffffffu, h1, o), __shfl_xor_sync(0xffffffffu, l1, o));
        }
        const bool any64 = __any_sync(0xffffffffu, used64);
        if (any64) {
            if (!used64)
                for (int w = 0; w < 6; w++) d64[w][lane] = 0.;
            __syncwarp();
            // fixed-order sum over the LG lanes of each group into the group's first slot
            for (int w = sub; w < 6; w += LG) {
                double acc = 0.;
                for (int l2 = 0; l2 < LG; l2++) acc += d64[w][(grp << lgl) + l2];
                d64[w][grp << lgl] = acc;
            }
            __syncwarp();
        }
        if (act && sub == 0) {
            if (!any64) {
                // MDiffusiveFast.cpp:41-45 with no wall term (s0 = s3 = 0), in FP32
                const float gif = (float)a.g[i];
                float t1 = h1 + l1;
                if (((t1 > 0.f) - (t1 < 0.f)) != ((gif > 0.f) - (gif < 0.f)) || fabsf(t1) < fabsf(0.1f * gif))
                    t1 = 0.1f * gif;
                const float f = ief / ((float)a.re * t1);
                a.vx[i] = a.vx[i] + (double)((h2x + l2x) * f);
                a.vy[i] = a.vy[i] + (double)((h2y + l2y) * f);
            } else {
                const double gi = a.g[i], ie = a.ie[i];
                const int g0 = grp << lgl;
                double s2x = d64[0][g0] + ((double)h2x + (double)l2x);
                double s2y = d64[1][g0] + ((double)h2y + (double)l2y);
                double s1 = d64[2][g0] + ((double)h1 + (double)l1);
                double s0 = d64[5][g0];
                if ((dsgn(s1) != dsgn(gi)) || (fabs(s1) < fabs(0.1 * gi))) s1 = 0.1 * gi;
                double f = ie / (a.re * s1);
                double vx = a.vx[i] + s2x * f, vy = a.vy[i] + s2y * f;
                if (s0 > C_PI) s0 = C_PI;
                f = ie * ie / (a.re * (C_2PI - s0));
                vx += d64[3][g0] * f;
                vy += d64[4][g0] * f;
                a.vx[i] = vx;
                a.vy[i] = vy;
            }
        }
        __syncwarp();  // the group sums in d64 are read before the next pass clears them
    }
    ncand = warp_sum_u64(ncand);
    if (lane == 0 && ncand) atomicAdd(a.cand, ncand);
    if (lane == 0 && s_nsrc[wq]) atomicAdd(a.cand + 1, s_nsrc[wq]);
}

// Targets per pass: the context's choice (vvgpu_autotune_tiles; shape 1: up to 16, shape
// 2: up to 8).  Against the earlier mapping (eight targets per pass, four lanes each, every
// candidate source applied to every target and the opposite-sign pairs zeroed): 7.16 against
// 8.54 ms at 4M, with bit-identical epsilon and merges.

}  // namespace

void diffusive(Ctx& c) {
    if (c.n == 0 || c.nleaves == 0) return;
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves;
    build_frames(c);
    c.lf_dbox.reserve(nl + 1);
    k_dbox<<<grid_for(nl, 128), 128, 0, s>>>(nl, c.lf_vf.p, c.lf_vl.p, c.lf_sf.p, c.lf_sl.p, c.seg_order.p,
                                             c.x.p, c.y.p, c.g.p, c.s_rx.p, c.s_ry.p, c.lf_anchor.p, c.frame_G,
                                             c.lf_dbox.p);
    VV_LAUNCH_CHECK();
    DiffArgs a{};
    a.nl = nl;
    a.lvf = c.lf_vf.p; a.lvl = c.lf_vl.p; a.lsf = c.lf_sf.p; a.lsl = c.lf_sl.p;
    a.near_off = c.near_off.p; a.near_run = c.near_run.p; a.seg_order = c.seg_order.p;
    a.x = c.x.p; a.y = c.y.p; a.g = c.g.p; a.ie = c.ie.p; a.vx = c.vx.p; a.vy = c.vy.p;
    a.rx = c.s_rx.p; a.ry = c.s_ry.p; a.dlx = c.s_dlx.p; a.dly = c.s_dly.p; a.fric = c.s_fric.p;
    a.anchor = c.lf_anchor.p; a.box = c.lf_dbox.p; a.src32 = c.src32.p; a.src_k = c.src_k.p; a.src_ie = c.src_ie.p;
    a.G = c.frame_G; a.Gf = (float)c.frame_G; a.re = c.re;
    VV_CUDA(cudaMemsetAsync(c.counters.p + 2, 0, 16, s));  // candidate pairs, candidate sources
    a.cand = c.counters.p + 2;
    unsigned grid = grid_for(nl, DW);
    {
        KernelTimer kt(c, VVGPU_T_DIFFUSIVE);
        if (c.precision == VVGPU_FP64) k_diff64<<<grid, DW * 32, 0, s>>>(a);
        else if (c.diff_targets == 2) k_diff32<8><<<grid, DW * 32, 0, s>>>(a);
        else k_diff32<16><<<grid, DW * 32, 0, s>>>(a);
        VV_LAUNCH_CHECK();
    }
    unsigned long long candl[2] = {0, 0};
    unsigned long long* cand = pinned_at(c, 104, candl);
    VV_CUDA(cudaMemcpyAsync(cand, c.counters.p + 2, 16, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    c.stats.diff_candidates = (int64_t)cand[0];
    c.diff_sources = (int64_t)cand[1];
}

}  // namespace vvgpu
