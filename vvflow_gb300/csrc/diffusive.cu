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
// One warp per target leaf: eight target slots times four source lanes.  FP64 path: every
// pair in double precision
// with the reference's formulas.  FP32 path: vortex pairs in local frames (frame.cuh) with
// FP32 exp/sqrt; pairs whose cut-off or coincidence test falls within a rigorous bound of
// the FP32 error of its threshold are re-evaluated in FP64, so the set of contributing
// pairs is the reference's.
// Wall segments are always FP64.  Friction goes to TAtt::fric with FP64 atomics.
#include <cfloat>

#include "frame.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr int DW = 4;

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

// Warp per target leaf.  Lane = target slot (lane & 7) x source lane (lane >> 3): eight
// targets per pass, the four source lanes split each candidate leaf's vortices.  Candidate
// leaves come from a lane-parallel box test against the targets' box grown by 8 eps.
//
// FP32 path: targets come from the FP32 source records (own leaf frame), pair sums are
// double-float pairs, and the final update runs in FP32 plus one FP64 addition per
// coordinate.  FP64 (a narrow pipe on sm_103) is used only where a pair fell in the band
// around a threshold or the leaf sees wall segments; a warp that met either takes the FP64
// reduction and update for that group of targets.
template <bool FP32>
__global__ void __launch_bounds__(DW * 32) k_diff(DiffArgs a) {
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
        bool act = false;
        double xi = 0, yi = 0, gi = 0, ie = 0;
        float txf = 0, tyf = 0, ief = 0;
        bool pos = false;
        float reach = 0.f;
        if (FP32) {
            // g != 0 and its sign from the bit pattern (integer pipe)
            const unsigned long long gb = (i < v1) ? (unsigned long long)__double_as_longlong(a.g[i]) : 0ull;
            act = (gb << 1) != 0ull;
            if (act) {
                const float4 r4 = a.src32[i];
                txf = r4.x; tyf = r4.y;
                ief = a.src_ie[i];
                pos = (gb >> 63) == 0ull;
                reach = (8.f / ief) * (1.f + 1e-4f);
                xi = a.x[i]; yi = a.y[i]; gi = a.g[i]; ie = a.ie[i];
            }
        } else {
            act = (i < v1) && (a.g[i] != 0.);
            if (act) {
                xi = a.x[i]; yi = a.y[i]; gi = a.g[i]; ie = a.ie[i];
                txf = (float)(xi - axL); tyf = (float)(yi - ayL);
                pos = gi > 0;
                reach = (float)(8.0 / ie) * (1.f + 1e-4f);
            }
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
        const float tmax = fmaxf(fmaxf(fabsf(bx0), fabsf(bx1)), fmaxf(fabsf(by0), fabsf(by1)));
        double s2x = 0, s2y = 0, s3x = 0, s3y = 0, s1 = 0, s0 = 0;
        float f2x = 0, f2y = 0, f1 = 0, c2x = 0, c2y = 0, c1 = 0;
        bool used64 = false;  // this lane added an FP64 term
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
                if (FP32) {
                    const float2 sh = frame_shift(a.anchor[qq], kL, a.Gf);
                    // Bound D on the FP32 error of |dr| for any pair of this leaf: each of
                    // dx, dy carries at most 2^-24 (|t| + |s| + |s + sh| + |dx|) from the
                    // roundings of the records, the shift and the subtraction (4x slack).
                    // Pairs whose (|dr| / eps)^2 lies within the resulting band of the cut-off
                    // 64, or whose |dx| + |dy| may be below the coincidence limit, are
                    // evaluated in FP64.
                    const float4 sb = a.box[qq];
                    const float s4max = fmaxf(fmaxf(fabsf(sb.x), fabsf(sb.z)), fmaxf(fabsf(sb.y), fabsf(sb.w)));
                    const float spmax = fmaxf(fmaxf(fabsf(sb.x + sh.x), fabsf(sb.z + sh.x)),
                                              fmaxf(fabsf(sb.y + sh.y), fabsf(sb.w + sh.y)));
                    const float D = ldexpf(2.f * tmax + s4max + 2.f * spmax, -21);
                    const float band = 16.f * ief * D * (1.f + 1e-3f) + ldexpf(64.f, -19);
                    const float tiny = 2.f * D + 1e-9f;
                    float p2x = 0, p2y = 0, p1 = 0;
                    for (int32_t j = j0 + sl; j < j1; j += 4) {
                        const float4 s4 = a.src32[j];
                        if (s4.z == 0.f || ((s4.z > 0.f) != pos)) continue;
                        const float dx = txf - (s4.x + sh.x), dy = tyf - (s4.y + sh.y);
                        const float r2 = dx * dx + dy * dy;
                        const float u = r2 * ief * ief;  // (|dr| / eps)^2
                        if (fabsf(u - 64.f) < band || (fabsf(dx) + fabsf(dy)) < tiny) {
                            vortex_term64(xi, yi, gi, ie, a.x[j], a.y[j], a.g[j], s2x, s2y, s1);
                            used64 = true;
                            continue;
                        }
                        if (u > 64.f) continue;
                        const float rs = rsqrtf(r2);
                        const float t = s4.z * __expf(-(r2 * rs) * ief);
                        const float qv = t * rs;
                        p2x = fmaf(dx, qv, p2x);
                        p2y = fmaf(dy, qv, p2y);
                        p1 += t;
                    }
                    acc_add(f2x, c2x, p2x);
                    acc_add(f2y, c2y, p2y);
                    acc_add(f1, c1, p1);
                } else {
                    for (int32_t j = j0 + sl; j < j1; j += 4) {
                        const double gj = a.g[j];
                        if (gj == 0.) continue;
                        vortex_term64(xi, yi, gi, ie, a.x[j], a.y[j], gj, s2x, s2y, s1);
                    }
                }
                // wall segments of this near leaf (segment_influence), FP64, split over source lanes
                for (int32_t qs = a.lsf[qq] + sl; qs < a.lsl[qq]; qs += 4) {
                    const int32_t sgm = a.seg_order[qs];
                    const double dx = xi - a.rx[sgm], dy = yi - a.ry[sgm];
                    const double dr2 = dx * dx + dy * dy;
                    const double dr = sqrt(dr2);
                    const double ea = -dr * ie;
                    used64 = true;
                    if (ea < EXP_ARG_RESTRICTION) continue;
                    const double ex = exp(ea);
                    const double dsx = -a.dly[sgm], dsy = a.dlx[sgm];
                    s3x += dsx * ex; s3y += dsy * ex;
                    s0 += (dr * ie + 1) / dr2 * (dx * dsx + dy * dsy) * ex;
                    atomicAdd(&a.fric[sgm], ie * ie * gi * ex * sqrt(dsx * dsx + dsy * dsy));
                }
            }
        });
        if (FP32) {
            // combine the four source lanes of each target slot as double-float pairs
#pragma unroll
            for (int o = 8; o < 32; o <<= 1) {
                ff_add(f2x, c2x, __shfl_xor_sync(0xffffffffu, f2x, o), __shfl_xor_sync(0xffffffffu, c2x, o));
                ff_add(f2y, c2y, __shfl_xor_sync(0xffffffffu, f2y, o), __shfl_xor_sync(0xffffffffu, c2y, o));
                ff_add(f1, c1, __shfl_xor_sync(0xffffffffu, f1, o), __shfl_xor_sync(0xffffffffu, c1, o));
            }
            if (!__any_sync(0xffffffffu, used64)) {
                if (act && sl == 0) {
                    // MDiffusiveFast.cpp:41-45 with no wall term (s0 = s3 = 0), in FP32
                    const float gif = (float)gi;
                    float t1 = f1 + c1;
                    if (((t1 > 0.f) - (t1 < 0.f)) != ((gif > 0.f) - (gif < 0.f)) || fabsf(t1) < fabsf(0.1f * gif))
                        t1 = 0.1f * gif;
                    const float f = ief / ((float)a.re * t1);
                    a.vx[i] = a.vx[i] + (double)((f2x + c2x) * f);
                    a.vy[i] = a.vy[i] + (double)((f2y + c2y) * f);
                }
                continue;
            }
        }
        // combine the four source lanes of each target slot (FP64 terms)
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
            if (FP32) {  // the FP32 pair sums, already combined over the source lanes
                s2x += (double)f2x + (double)c2x;
                s2y += (double)f2y + (double)c2y;
                s1 += (double)f1 + (double)c1;
            }
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
    VV_CUDA(cudaMemsetAsync(c.counters.p + 2, 0, 8, s));
    a.cand = c.counters.p + 2;
    unsigned grid = grid_for(nl, DW);
    if (c.precision == VVGPU_FP32) k_diff<true><<<grid, DW * 32, 0, s>>>(a);
    else k_diff<false><<<grid, DW * 32, 0, s>>>(a);
    VV_LAUNCH_CHECK();
    unsigned long long cand = 0;
    VV_CUDA(cudaMemcpyAsync(&cand, c.counters.p + 2, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    c.stats.diff_candidates = (int64_t)cand;
}

}  // namespace vvgpu
