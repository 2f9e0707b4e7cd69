// Convective velocity (MConvectiveFast::process_all_lists, libvvhd/src/MConvectiveFast.cpp:36-114)
// and point queries (MConvectiveFast::velocity, :20-34).
//
// One warp per target leaf.  The leaf's targets are held in registers in chunks of TC; the
// 32 lanes stride over the leaf's near sources (each near run is one contiguous vortex
// range), so every source is loaded once per chunk and applied to all TC targets.  Lane
// partials are reduced with shuffles.  The far field (two monopoles per far node, expanded
// to first order about the leaf centre, :48-69 and :84-85) is computed by the same warp.
//
// FP64 path: Biot-Savart kernel rotl(dr) g / (|dr|^2 + eps^2) / 2pi in double precision,
// the reciprocal by Newton-Raphson iteration from the hardware approximation.
// FP32 path: sources in local frames (frame.cuh), staged through shared memory by bulk
// copies (stage.cuh), FP32 pair arithmetic, lane partials folded into a two-sum (Knuth's
// TwoSum) compensated pair every at most 32 sources, lane partials reduced as double-float
// pairs; FP64 (a narrow pipe on sm_103) only in the final per-target update.
#include <cfloat>

#include "frame.cuh"
#include "stage.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr int CW = 4;  // warps per block

// Reciprocal by Newton-Raphson refinement r <- r (2 - x r) of the PTX approximation.
__device__ __forceinline__ double rcp64(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    // x = +-0 or +-inf: the approximation is already the exact 1/x, and a Newton step
    // would turn it into NaN (0 * inf); the reference's 1/inf = 0 and g/0 = inf matter for
    // vortices whose epsilon is 0 (coincident vortices).  The approximation flushes
    // subnormal inputs and results to zero: a subnormal x (|x| < 2.2e-308, whose 1/x is
    // finite) or an x whose 1/x is subnormal takes the IEEE quotient instead.
    if (r == 0.0 || isinf(r)) return (x == 0.0 || isinf(x)) ? r : 1.0 / x;
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

__device__ __forceinline__ float rcp32(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bp = s - a;
    float ap = s - bp;
    e = (a - ap) + (b - bp);
}

// Double-float addition (a_h, a_l) += (b_h, b_l): TwoSum of the heads, the tails added to
// the error term, renormalised by Dekker's Fast2Sum.
__device__ __forceinline__ void ff_add(float& ah, float& al, float bh, float bl) {
    float s, e;
    two_sum(ah, bh, s, e);
    e += al + bl;
    ah = s + e;
    al = e - (ah - s);
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct ConvArgs {
    int64_t nl;
    const int32_t* lvf; const int32_t* lvl;
    const double4* lgeom;
    const int32_t* near_off; const int2* near_run;
    const double4* taylor;
    const double* cm;
    const double* x; const double* y; const double* g; const double* ie;
    double* vx; double* vy;
    // sinks and slip segments
    int64_t ns; const double* kx; const double* ky; const double* kg; double sink_e2;
    int64_t m; const double* srx; const double* sry; const double* sg; const double* sie; const uint32_t* slip;
    int any_slip;
    // attached sheets of moving bodies: per segment corner, dl, and (speed x, y, o, axis x,
    // y) of its body, flagged where the body's speed_slae is not zero
    int any_moving;
    const double* scx; const double* scy; const double* sdlx; const double* sdly;
    const double* att; const int32_t* att_on;
    double inf_vx, inf_vy;
    double fc; int64_t nnodes;
    // FP32 records
    const float4* src32; const float2* src_k; const float2* anchor; double G; float Gf;
    // FP32 near field: anchors of the sources' leaves as 16-byte records, and per near run
    // (first source slot, offset in the leaf's flattened near sequence), per leaf the
    // sequence's length; staging waits and their error flag
    const float4* src_a4; const int2* run_js; const int32_t* leaf_tot; int64_t nsrc;
    uint32_t spins; unsigned long long* err;
};

// (a + ib) / (c + id)
__device__ __forceinline__ void cdiv(double a, double b, double c, double d, double& re, double& im) {
    const double den = c * c + d * d;
    re = (a * c + b * d) / den;
    im = (b * c - a * d) / den;
}

// SegmentInfluence_linear_source (MConvectiveFast.cpp:440-457): a source sheet of strength
// q1 -> q2 along the segment centred at (rx, ry) with vector (dlx, dly), at (px, py):
// ((q2 - q1) - conj(q2 z1 - q1 z2) / conj(dz) log(conj(z2) / conj(z1))) / conj(dz) with
// z1, z2 the point's offsets from the segment's ends; FP64 with CUDA's log and atan2.
__device__ __forceinline__ void linear_source(double px, double py, double rx, double ry, double dlx, double dly,
                                              double q1, double q2, double& ox, double& oy) {
    const double z1x = px - (rx - dlx * 0.5), z1y = py - (ry - dly * 0.5);
    const double z2x = px - (rx + dlx * 0.5), z2y = py - (ry + dly * 0.5);
    double bx, by, wx, wy, nx, ny;
    cdiv(q2 * z1x - q1 * z2x, -(q2 * z1y - q1 * z2y), dlx, -dly, bx, by);
    cdiv(z2x, -z2y, z1x, -z1y, wx, wy);
    const double lx = log(hypot(wx, wy)), ly = atan2(wy, wx);
    nx = (q2 - q1) - (bx * lx - by * ly);
    ny = -(bx * ly + by * lx);
    cdiv(nx, ny, dlx, -dly, ox, oy);
}

// The attached vortex and source sheets of the moving bodies (body_list_influence,
// MConvectiveFast.cpp:185-210) at (px, py), before the 1/2pi: sheets of strength
// -Vs.dl and -rotl(Vs).dl with Vs the body's velocity at the segment (rotation about
// holder + dpos); linear sheets within |dl| of the segment centre, point singularities
// beyond.
__device__ __forceinline__ void attached_terms(const ConvArgs& a, double px, double py, double& rx, double& ry) {
    for (int64_t k = 0; k < a.m; k++) {
        if (!a.att_on[k]) continue;
        const double* w = a.att + 5 * k;
        const double vx = w[0], vy = w[1], vo = w[2], ax = w[3], ay = w[4];
        const double dlx = a.sdlx[k], dly = a.sdly[k];
        const double dx = px - a.srx[k], dy = py - a.sry[k];
        const double drabs2 = dx * dx + dy * dy;
        if (drabs2 < dlx * dlx + dly * dly) {
            const double c1x = a.scx[k] - ax, c1y = a.scy[k] - ay;
            const double w1x = vx - c1y * vo, w1y = vy + c1x * vo;
            const double c2x = (a.scx[k] + dlx) - ax, c2y = (a.scy[k] + dly) - ay;
            const double w2x = vx - c2y * vo, w2y = vy + c2x * vo;
            double ux, uy;
            linear_source(px, py, a.srx[k], a.sry[k], dlx, dly, -(w1x * dlx + w1y * dly), -(w2x * dlx + w2y * dly),
                          ux, uy);
            rx -= uy; ry += ux;  // rotl
            linear_source(px, py, a.srx[k], a.sry[k], dlx, dly, w1y * dlx - w1x * dly, w2y * dlx - w2x * dly, ux, uy);
            rx += ux; ry += uy;
        } else {
            const double cx = a.srx[k] - ax, cy = a.sry[k] - ay;
            const double wx = vx - cy * vo, wy = vy + cx * vo;
            const double g = -(wx * dlx + wy * dly), q = wy * dlx - wx * dly;
            const double inv = 1. / drabs2;
            rx += (dx * q - dy * g) * inv;
            ry += (dy * q + dx * g) * inv;
        }
    }
}

// sink_list_influence + body_list_influence (slip segments, attached sheets of moving
// bodies), FP64 (per target).
__device__ __forceinline__ void extra_terms(const ConvArgs& a, double px, double py, double& ox, double& oy) {
    double rx = 0, ry = 0;
    for (int64_t k = 0; k < a.ns; k++) {
        double dx = px - a.kx[k], dy = py - a.ky[k];
        double s = a.kg[k] / (dx * dx + dy * dy + a.sink_e2 * sink_abs(a.kg[k]));
        rx += dx * s; ry += dy * s;
    }
    double bx = 0, by = 0;
    if (a.any_slip) {
        for (int64_t k = 0; k < a.m; k++) {
            if (!a.slip[k]) continue;
            double dx = px - a.srx[k], dy = py - a.sry[k];
            double e = 1. / a.sie[k];
            double s = a.sg[k] / (dx * dx + dy * dy + e * e);
            bx -= dy * s; by += dx * s;
        }
    }
    if (a.any_moving) attached_terms(a, px, py, bx, by);
    ox = (rx + bx) * C_1_2PI;
    oy = (ry + by) * C_1_2PI;
}

template <int TC>
__global__ void __launch_bounds__(CW * 32) k_conv64(ConvArgs a) {
    const int64_t L = (int64_t)blockIdx.x * CW + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (L >= a.nl) return;
    const double4 me = a.lgeom[L];
    const double4 tc = a.taylor[L];
    const double t1 = tc.x, t2 = tc.y, t3 = tc.z, t4 = tc.w;
    const int32_t v0 = a.lvf[L], v1 = a.lvl[L];
    const int32_t r0 = a.near_off[L], r1 = a.near_off[L + 1];
    for (int32_t c0 = v0; c0 < v1; c0 += TC) {
        double tx[TC], ty[TC], ax[TC], ay[TC];
#pragma unroll
        for (int t = 0; t < TC; t++) {
            int32_t i = c0 + t;
            tx[t] = (i < v1) ? a.x[i] : 0.;
            ty[t] = (i < v1) ? a.y[i] : 0.;
            ax[t] = 0; ay[t] = 0;
        }
        for (int32_t r = r0; r < r1; r++) {
            int2 run = a.near_run[r];
            int32_t j0 = a.lvf[run.x], j1 = a.lvl[run.y - 1];
            for (int32_t j = j0 + lane; j < j1; j += 32) {
                double gj = a.g[j], iej = a.ie[j];
                if (gj == 0. || iej == 0.) continue;
                double e = rcp64(iej);
                double e2 = e * e;
                double xj = a.x[j], yj = a.y[j];
#pragma unroll
                for (int t = 0; t < TC; t++) {
                    double dx = tx[t] - xj, dy = ty[t] - yj;
                    double s = gj * rcp64(fma(dx, dx, fma(dy, dy, e2)));
                    ax[t] = fma(-dy, s, ax[t]);
                    ay[t] = fma(dx, s, ay[t]);
                }
            }
        }
#pragma unroll
        for (int t = 0; t < TC; t++) {
            ax[t] = warp_sum(ax[t]);
            ay[t] = warp_sum(ay[t]);
        }
#pragma unroll
        for (int t = 0; t < TC; t++) {
            int32_t i = c0 + t;
            if (lane == t && i < v1 && a.g[i] != 0.) {
                double ex, ey;
                extra_terms(a, tx[t], ty[t], ex, ey);
                double lx = tx[t] - me.x, ly = ty[t] - me.y;
                double vx = a.vx[i], vy = a.vy[i];
                vx += a.inf_vx; vy += a.inf_vy;
                vx += ax[t] * C_1_2PI; vy += ay[t] * C_1_2PI;
                vx += ex; vy += ey;
                vx += t1; vy += t2;
                vx += t3 * lx + t4 * ly;
                vy += t4 * lx + (-t3) * ly;
                a.vx[i] = vx; a.vy[i] = vy;
            }
        }
    }
}

// FP32 near field.  Eight targets per lane.  A leaf with at most 8 targets uses all 32
// lanes over its sources; with 9..16 targets each half-warp takes 8 targets and strides
// over the sources by 16 (larger leaves loop in groups of 16).  The leaf's near sources are
// one flattened sequence (its near runs in list order; run_js holds each run's first slot
// and offset).  The warp streams it through shared memory in tiles of CT sources, two
// buffers: for the next tile every lane whose run overlaps it issues one bulk copy of the
// piece's records and one of their anchors, completing on the buffer's mbarrier, while the
// lanes apply the current tile.  Each lane keeps plain FP32 partial sums over at most 32
// of its sources and then folds them into a TwoSum-compensated pair.
constexpr int TC32 = 8;
// CT: sources per staged tile (128, 192 or 256; the context's choice, vvgpu_autotune_tiles)
// Warps per block of k_conv32: one (16 blocks per SM), so that an SM takes a new leaf as
// soon as any warp's leaf is done (6.81 ms at 4M against 7.32 ms for two warps per block
// and 7.63 ms for four, where a block waited for its slowest leaf)
constexpr int CW32 = 1;
constexpr size_t conv32_smem(int ct) {
    return (size_t)CW32 * 2 * ct * 2 * sizeof(float4) + (size_t)CW32 * 2 * sizeof(uint64_t);
}

template <int CT>
__global__ void __launch_bounds__(CW32 * 32, 16) k_conv32(ConvArgs a) {
    extern __shared__ __align__(128) unsigned char conv_smem[];
    const int wq = threadIdx.x >> 5;
    const int64_t L = (int64_t)blockIdx.x * CW32 + wq;
    const int lane = threadIdx.x & 31;
    if (L >= a.nl) return;
    float4* const t_rec = reinterpret_cast<float4*>(conv_smem) + (size_t)wq * 2 * CT;           // [2][CT]
    float4* const t_anc = reinterpret_cast<float4*>(conv_smem) + (size_t)(CW32 + wq) * 2 * CT;    // [2][CT]
    uint64_t* const bar = reinterpret_cast<uint64_t*>(reinterpret_cast<float4*>(conv_smem) + (size_t)CW32 * 4 * CT) +
                          2 * wq;
    if (lane == 0) {
        stage_bar_init(&bar[0]);
        stage_bar_init(&bar[1]);
    }
    __syncwarp();
    const double4 me = a.lgeom[L];
    const double4 tc = a.taylor[L];
    const float2 kL = a.anchor[L];
    const int32_t v0 = a.lvf[L], v1 = a.lvl[L];
    const int32_t r0 = a.near_off[L], r1 = a.near_off[L + 1];
    const int32_t tot = a.leaf_tot[L];
    const int ntile = (tot + CT - 1) / CT;
    uint32_t parity = 0;  // bit b: parity of buffer b's next phase
    int ib = 0, cb = 0;   // buffer of the next tile issued / consumed
    int pending = 0;      // tiles issued and not yet consumed
    bool fail = false;
    // Issues tile t (sources [t CT, min((t+1) CT, tot))) into buffer ib.  rcur: the first
    // run that ends beyond the tile's start; on return, the first run ending beyond its end.
    auto issue = [&](int t, int32_t& rcur) {
        const int32_t kb = t * CT, ke = min(kb + CT, tot);
        const int b = ib;
        ib ^= 1;
        pending++;
        if (lane == 0) stage_expect(&bar[b], (uint32_t)(ke - kb) * 32u);
        __syncwarp();
        for (int32_t rb = rcur; rb < r1; rb += 32) {
            const int32_t r = rb + lane;
            int32_t j0 = 0, off = tot;
            if (r < r1) {
                const int2 js = a.run_js[r];
                j0 = js.x;
                off = js.y;
            }
            int32_t end = __shfl_down_sync(0xffffffffu, off, 1);
            if (lane == 31) end = (rb + 32 < r1) ? a.run_js[rb + 32].y : tot;
            if (r >= r1) end = tot;
            const int32_t lo = max(off, kb), hi = min(end, ke);
            if (r < r1 && hi > lo) {
                const int32_t j = j0 + (lo - off);
                // every piece lies inside the vortex arrays and the tile (else the wait runs out)
                if (j >= 0 && (int64_t)j + (hi - lo) <= a.nsrc && lo >= kb && hi <= kb + CT) {
                    stage_fence();
                    stage_copy(t_rec + b * CT + (lo - kb), a.src32 + j, (uint32_t)(hi - lo) * 16u, &bar[b]);
                    stage_copy(t_anc + b * CT + (lo - kb), a.src_a4 + j, (uint32_t)(hi - lo) * 16u, &bar[b]);
                }
            }
            const unsigned beyond = __ballot_sync(0xffffffffu, r < r1 && end > ke);
            if (beyond) {
                rcur = rb + __ffs(beyond) - 1;
                return;
            }
            rcur = rb + 32;
        }
    };
    for (int32_t c0 = v0; c0 < v1 && !fail; c0 += 2 * TC32) {
        const int32_t nt = min(v1 - c0, 2 * TC32);
        const bool split = nt > TC32;                 // two groups of 8 targets
        const int half = split ? (lane >> 4) : 0;
        const int sub = split ? (lane & 15) : lane;   // lane index within the source stride
        const int stride = split ? 16 : 32;
        const int32_t t0 = c0 + half * TC32;
        float tx[TC32], ty[TC32], hx[TC32], hy[TC32], lx[TC32], ly[TC32], px[TC32], py[TC32];
#pragma unroll
        for (int t = 0; t < TC32; t++) {
            const int32_t i = t0 + t;
            // a target's own source record is already in this leaf's frame
            const float4 r4 = (i < c0 + nt) ? a.src32[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            tx[t] = r4.x;
            ty[t] = r4.y;
            hx[t] = hy[t] = lx[t] = ly[t] = px[t] = py[t] = 0.f;
        }
        int since = 0;  // sources in the plain partial sums (at most, over the lanes)
        int32_t rcur = r0;
        if (ntile > 0) issue(0, rcur);
        for (int t = 0; t < ntile; t++) {
            if (t + 1 < ntile) issue(t + 1, rcur);
            const int b = cb;
            const bool ok = stage_wait(&bar[b], (parity >> b) & 1u, a.spins);
            if (!__all_sync(0xffffffffu, ok)) {
                fail = true;  // this tile stays pending: the drain below waits for it
                break;
            }
            cb ^= 1;
            parity ^= 1u << b;
            pending--;
            const int32_t ns = min(CT, tot - t * CT);
            const int per = (ns + stride - 1) / stride;  // sources of lane 0 in this tile
            if (since + per > 32) {
                since = 0;
#pragma unroll
                for (int tt = 0; tt < TC32; tt++) {
                    float sv, e;
                    two_sum(hx[tt], px[tt], sv, e); hx[tt] = sv; lx[tt] += e; px[tt] = 0.f;
                    two_sum(hy[tt], py[tt], sv, e); hy[tt] = sv; ly[tt] += e; py[tt] = 0.f;
                }
            }
            since += per;
            const float4* rt = t_rec + b * CT;
            const float4* at = t_anc + b * CT;
#pragma unroll 2
            for (int k = sub; k < ns; k += stride) {
                const float4 s4 = rt[k];
                const float4 k4 = at[k];
                const float sx = s4.x + (k4.x - kL.x);
                const float sy = s4.y + (k4.y - kL.y);
#pragma unroll
                for (int tt = 0; tt < TC32; tt++) {
                    const float dx = tx[tt] - sx, dy = ty[tt] - sy;
                    const float q = s4.z * rcp32(fmaf(dx, dx, fmaf(dy, dy, s4.w)));
                    px[tt] = fmaf(-dy, q, px[tt]);
                    py[tt] = fmaf(dx, q, py[tt]);
                }
            }
            __syncwarp();  // the buffer is free for the tile after next
        }
        if (fail) break;
        // Reduce-scatter of the 16 float-float partials (x and y of 8 targets) over the 16
        // lanes of each source stride: after the xor-8/4/2/1 steps lane k (= lane & 15)
        // holds value k, i.e. coordinate k >> 3 of target k & 7, summed over its 16 lanes.
        float vh[2 * TC32], vl[2 * TC32];
#pragma unroll
        for (int t = 0; t < TC32; t++) {
            float sv, e;
            two_sum(hx[t], px[t], sv, e); vh[t] = sv; vl[t] = lx[t] + e;
            two_sum(hy[t], py[t], sv, e); vh[t + TC32] = sv; vl[t + TC32] = ly[t] + e;
        }
#pragma unroll
        for (int m = TC32; m >= 1; m >>= 1) {
            const bool up = (lane & m) != 0;
#pragma unroll
            for (int k = 0; k < m; k++) {
                float kh = up ? vh[k + m] : vh[k], kl = up ? vl[k + m] : vl[k];
                const float sh = up ? vh[k] : vh[k + m], sl = up ? vl[k] : vl[k + m];
                ff_add(kh, kl, __shfl_xor_sync(0xffffffffu, sh, m), __shfl_xor_sync(0xffffffffu, sl, m));
                vh[k] = kh; vl[k] = kl;
            }
        }
        float rh = vh[0], rl = vl[0];
        if (!split) ff_add(rh, rl, __shfl_xor_sync(0xffffffffu, rh, 16), __shfl_xor_sync(0xffffffffu, rl, 16));
        // FP64 only from here on, once per (target, coordinate) and with all lanes converged.
        const int k = lane & 15;
        const int32_t i = t0 + (k & (TC32 - 1));
        if ((split || lane < 16) && i < c0 + nt && a.g[i] != 0.) {
            const double pxd = a.x[i], pyd = a.y[i];
            const double acc = ((double)rh + (double)rl) * C_1_2PI;
            double ex, ey;
            extra_terms(a, pxd, pyd, ex, ey);
            const double dlx = pxd - me.x, dly = pyd - me.y;
            if (k < TC32) {
                double vx = a.vx[i];
                vx += a.inf_vx;
                vx += acc;
                vx += ex;
                vx += tc.x;
                vx += tc.z * dlx + tc.w * dly;
                a.vx[i] = vx;
            } else {
                double vy = a.vy[i];
                vy += a.inf_vy;
                vy += acc;
                vy += ey;
                vy += tc.y;
                vy += tc.w * dlx + (-tc.z) * dly;
                a.vy[i] = vy;
            }
        }
    }
    if (fail) {
        // a staging wait ran out: drain the copies in flight (bounded), flag the error
        for (; pending > 0; pending--) {
            stage_wait(&bar[cb], (parity >> cb) & 1u, STAGE_SPINS);
            parity ^= 1u << cb;
            cb ^= 1;
        }
        if (lane == 0) atomicExch(a.err, 1ull);
    }
}

// Per near run of every leaf: its first source slot and its offset in the leaf's flattened
// near sequence (the runs in list order); per leaf the sequence's length.  One warp per leaf.
__global__ void k_run_table(int64_t nl, const int32_t* __restrict__ near_off, const int2* __restrict__ near_run,
                            const int32_t* __restrict__ lvf, const int32_t* __restrict__ lvl, int2* run_js,
                            int32_t* leaf_tot) {
    const int64_t L = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    const int32_t r0 = near_off[L], r1 = near_off[L + 1];
    int32_t base = 0;
    for (int32_t rb = r0; rb < r1; rb += 32) {
        const int32_t r = rb + lane;
        int32_t j0 = 0, len = 0;
        if (r < r1) {
            const int2 run = near_run[r];
            j0 = lvf[run.x];
            len = lvl[run.y - 1] - j0;
        }
        int32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (r < r1) run_js[r] = make_int2(j0, base + incl - len);
        base += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) leaf_tot[L] = base;
}

// FP32 source records: position in own leaf frame, g, eps^2 (eps = 1/_1_eps; a zero
// _1_eps or zero g gives a record that contributes exactly zero).
__global__ void k_src32(int64_t n, const int32_t* __restrict__ leaf_of, const float2* __restrict__ anchor, double G,
                        const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ g,
                        const double* __restrict__ ie, float4* src, float2* src_k, float* src_ie,
                        float4* src_a4) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 k = anchor[leaf_of[i]];
    // eps^2 = 1 / _1_eps^2 on the FP32 pipe (the record holds it in FP32; an FP64 division
    // per vortex costs more than the rest of this kernel on GB300's narrow FP64 pipe)
    const double iel = ie[i];
    const float ief = (float)iel;
    float gf = (float)g[i];
    float e2 = __frcp_rn(ief * ief);
    if (iel == 0.) { gf = 0.f; e2 = 1.f; }
    src[i] = make_float4((float)(x[i] - (double)k.x), (float)(y[i] - (double)k.y), gf, e2);
    src_k[i] = k;
    src_a4[i] = make_float4(k.x, k.y, 0.f, 0.f);
    src_ie[i] = (float)ie[i];
}

__global__ void k_anchor2(int64_t nl, const double4* __restrict__ lgeom, double G, float2* anchor) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    double4 me = lgeom[L];
    double cx = isfinite(me.x) ? me.x : 0., cy = isfinite(me.y) ? me.y : 0.;
    anchor[L] = anchor_of(cx, cy, G);
}

// stree::findNode (TSortedTree.cpp:284-303) + near/far (exact monopoles) + extra terms.
__global__ void k_points(int64_t np, const double* __restrict__ qx, const double* __restrict__ qy,
                         const double4* __restrict__ geom, const int32_t* __restrict__ ch1,
                         const int32_t* __restrict__ dfs, ConvArgs a, double* ovx, double* ovy) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    double px = qx[q], py = qy[q];
    int32_t k = 0;
    for (int it = 0; it <= MAX_DEPTH && ch1[k] >= 0; it++) {
        double4 gm = geom[k];
        if (gm.z < gm.w) k = (px < gm.x) ? ch1[k] : ch1[k] + 1;
        else k = (py < gm.y) ? ch1[k] : ch1[k] + 1;
    }
    int32_t L = dfs[k];
    double rx = 0, ry = 0;
    for (int32_t r = a.near_off[L]; r < a.near_off[L + 1]; r++) {
        int2 run = a.near_run[r];
        for (int32_t j = a.lvf[run.x]; j < a.lvl[run.y - 1]; j++) {
            if (a.g[j] == 0.) continue;
            double dx = px - a.x[j], dy = py - a.y[j];
            double e = 1. / a.ie[j];
            double s = a.g[j] / (dx * dx + dy * dy + e * e);
            rx -= dy * s; ry += dx * s;
        }
    }
    // far nodes of leaf k by the reference's walk (exact FP64 decisions)
    double fx = 0, fy = 0;
    {
        const double4 me = geom[k];
        int32_t stack[MAX_DEPTH + 2];
        int sp = 0;
        stack[sp++] = 0;
        int64_t guard = 0;
        while (sp && ++guard <= a.nnodes) {
            const int32_t t = stack[--sp];
            const double4 tg = geom[t];
            double ddx = dsub(tg.x, me.x), ddy = dsub(tg.y, me.y);
            double hp = dadd(dadd(dadd(tg.z, tg.w), me.z), me.w);
            if (dabs2(ddx, ddy) > dmul(dmul(a.fc, hp), hp)) {
                const double* c = a.cm + 6 * (size_t)t;
                double dx = px - c[0], dy = py - c[1];
                double s = c[2] / (dx * dx + dy * dy);
                fx -= dy * s; fy += dx * s;
                dx = px - c[3]; dy = py - c[4];
                s = c[5] / (dx * dx + dy * dy);
                fx -= dy * s; fy += dx * s;
                continue;
            }
            const int32_t c1 = ch1[t];
            if (c1 >= 0 && sp + 2 <= MAX_DEPTH + 2) {
                stack[sp++] = c1 + 1;
                stack[sp++] = c1;
            }
        }
    }
    double ex, ey;
    extra_terms(a, px, py, ex, ey);
    ovx[q] = rx * C_1_2PI + fx * C_1_2PI + ex + a.inf_vx;
    ovy[q] = ry * C_1_2PI + fy * C_1_2PI + ey + a.inf_vy;
}

// FP64 direct sum over every vortex (no tree), each source with its own epsilon (biot_savart,
// MConvectiveFast.cpp:116-120), plus the sink, slip-segment and free-stream terms of
// velocity(p): the tree's own approximation error is measured against it.  One block per
// target, fixed-order reduction.
constexpr int DIRECT_TB = 256;
__global__ void __launch_bounds__(DIRECT_TB) k_direct(int64_t n, const double* __restrict__ qx,
                                                     const double* __restrict__ qy, ConvArgs a, double* ovx,
                                                     double* ovy) {
    __shared__ double sh[2][DIRECT_TB / 32];
    const int64_t q = blockIdx.x;
    const double px = qx[q], py = qy[q];
    double rx = 0, ry = 0;
    for (int64_t j = threadIdx.x; j < n; j += DIRECT_TB) {
        const double gj = a.g[j];
        if (gj == 0.) continue;
        const double dx = px - a.x[j], dy = py - a.y[j];
        const double e = 1. / a.ie[j];
        const double s = gj / (dx * dx + dy * dy + e * e);
        rx -= dy * s;
        ry += dx * s;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rx += __shfl_xor_sync(0xffffffffu, rx, o);
        ry += __shfl_xor_sync(0xffffffffu, ry, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[0][w] = rx; sh[1][w] = ry; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sx = 0, sy = 0;
        for (int k = 0; k < DIRECT_TB / 32; k++) { sx += sh[0][k]; sy += sh[1][k]; }
        double ex, ey;
        extra_terms(a, px, py, ex, ey);
        ovx[q] = sx * C_1_2PI + ex + a.inf_vx;
        ovy[q] = sy * C_1_2PI + ey + a.inf_vy;
    }
}

// Algorithmic near-pair count: sum over leaves of (non-zero targets) x (non-zero sources
// in the near runs).
__global__ void k_leaf_nz(int64_t nl, const int32_t* __restrict__ lvf, const int32_t* __restrict__ lvl,
                          const double* __restrict__ g, int32_t* nz) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    int32_t k = 0;
    for (int32_t i = lvf[L]; i < lvl[L]; i++) k += (g[i] != 0.);
    nz[L] = k;
}

__global__ void k_near_pairs(int64_t nl, const int32_t* __restrict__ nz, const int32_t* __restrict__ pre,
                             const int32_t* __restrict__ near_off, const int2* __restrict__ near_run,
                             unsigned long long* out) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v = 0;
    if (L < nl && nz[L]) {
        int64_t src = 0;
        for (int32_t r = near_off[L]; r < near_off[L + 1]; r++) src += pre[near_run[r].y] - pre[near_run[r].x];
        v = (unsigned long long)nz[L] * (unsigned long long)src;
    }
    v = warp_sum_u64(v);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

// The judge of the learned far field: MConvectiveFast::velocity(p) (:20-34) at the positions
// of vortices idx[k], with the tree's near/far split redone at far criterion fc (the plain
// tree's) by the reference's depth-first walk with its exact FP64 test.
// Pass 1 (k_judge_walk<false>, one thread per target): counts each target's far nodes and
// near leaves; pass 2 (<true>): writes them at the scanned offsets.  Then k_judge_sum, one
// warp per target: the lanes split the far nodes' monopoles and the near leaves' vortices
// (FP64, reciprocal by Newton steps), partials reduced by a fixed shuffle tree.
// out[3 k ..] = (vx, vy, 1) for a vortex with g != 0, (0, 0, 0) otherwise (it takes no
// convective term).
template <bool FILL>
__global__ void k_judge_walk(int64_t nt, const int32_t* __restrict__ idx, const double* __restrict__ x,
                             const double* __restrict__ y, const double* __restrict__ g,
                             const double4* __restrict__ geom, const int32_t* __restrict__ ch1, double fc,
                             int64_t nnodes, int32_t* cnt, const int64_t* __restrict__ off, int32_t* list,
                             int32_t* err) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nt) return;
    const int32_t i = idx[q];
    int32_t nf = 0, nn = 0;
    if (g[i] != 0.) {
        const double px = x[i], py = y[i];
        int32_t k = 0;
        for (int it = 0; it <= MAX_DEPTH && ch1[k] >= 0; it++) {
            const double4 gm = geom[k];
            if (gm.z < gm.w) k = (px < gm.x) ? ch1[k] : ch1[k] + 1;
            else k = (py < gm.y) ? ch1[k] : ch1[k] + 1;
        }
        const double4 me = geom[k];
        // far nodes from the front of the target's range, near leaves from its back
        int32_t* fl = FILL ? list + off[q] : nullptr;
        int32_t* nl = FILL ? list + off[q + 1] : nullptr;
        int32_t stack[MAX_DEPTH + 2];
        int sp = 0;
        stack[sp++] = 0;
        int64_t guard = 0;
        while (sp) {
            if (++guard > nnodes) { atomicExch(err, 1); break; }
            const int32_t t = stack[--sp];
            const double4 tg = geom[t];
            const double ddx = dsub(tg.x, me.x), ddy = dsub(tg.y, me.y);
            const double hp = dadd(dadd(dadd(tg.z, tg.w), me.z), me.w);
            if (dabs2(ddx, ddy) > dmul(dmul(fc, hp), hp)) {
                if (FILL) fl[nf] = t;
                nf++;
                continue;
            }
            const int32_t c1 = ch1[t];
            if (c1 < 0) {
                nn++;
                if (FILL) nl[-nn] = t;
                continue;
            }
            if (sp + 2 > MAX_DEPTH + 2) { atomicExch(err, 1); break; }
            stack[sp++] = c1 + 1;
            stack[sp++] = c1;
        }
    }
    if (!FILL) {
        cnt[2 * q] = nf;
        cnt[2 * q + 1] = nn;
    }
}

__global__ void k_judge_sum(int64_t nt, const int32_t* __restrict__ idx, const int32_t* __restrict__ cnt,
                            const int64_t* __restrict__ off, const int32_t* __restrict__ list,
                            const int32_t* __restrict__ nvf, const int32_t* __restrict__ nvl, ConvArgs a,
                            double* out) {
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (q >= nt) return;
    const int32_t i = idx[q];
    if (a.g[i] == 0.) {
        if (lane == 0) { out[3 * q] = 0.; out[3 * q + 1] = 0.; out[3 * q + 2] = 0.; }
        return;
    }
    const double px = a.x[i], py = a.y[i];
    const int32_t nf = cnt[2 * q], nn = cnt[2 * q + 1];
    const int32_t* fl = list + off[q];
    const int32_t* nl = list + off[q + 1] - nn;
    double rx = 0, ry = 0;
    for (int32_t k = lane; k < nf; k += 32) {  // far_nodes_influence (:139-151)
        const double* c = a.cm + 6 * (size_t)fl[k];
#pragma unroll
        for (int sgn = 0; sgn < 2; sgn++) {
            const double gs = c[3 * sgn + 2];
            const double dx = px - c[3 * sgn], dy = py - c[3 * sgn + 1];
            const double s = gs * rcp64(dx * dx + dy * dy);
            rx -= dy * s; ry += dx * s;
        }
    }
    for (int32_t k = lane; k < nn; k += 32) {  // near_nodes_influence (:122-137)
        const int32_t t = nl[k];
        for (int32_t j = nvf[t]; j < nvl[t]; j++) {
            const double gj = a.g[j];
            if (gj == 0.) continue;
            const double dx = px - a.x[j], dy = py - a.y[j];
            const double e = rcp64(a.ie[j]);
            const double s = gj * rcp64(dx * dx + dy * dy + e * e);
            rx -= dy * s; ry += dx * s;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rx += __shfl_xor_sync(0xffffffffu, rx, o);
        ry += __shfl_xor_sync(0xffffffffu, ry, o);
    }
    if (lane == 0) {
        double ex, ey;
        extra_terms(a, px, py, ex, ey);
        out[3 * q] = rx * C_1_2PI + ex + a.inf_vx;
        out[3 * q + 1] = ry * C_1_2PI + ey + a.inf_vy;
        out[3 * q + 2] = 1.;
    }
}

// Free-stream, sink and slip-segment terms added to the judge's vortex part (lists.cu).
__global__ void k_judge_finish(int64_t nt, const int32_t* __restrict__ idx, ConvArgs a, double* out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nt || out[3 * q + 2] != 1.) return;
    const int32_t i = idx[q];
    double ex, ey;
    extra_terms(a, a.x[i], a.y[i], ex, ey);
    out[3 * q] += ex + a.inf_vx;
    out[3 * q + 1] += ey + a.inf_vy;
}

__global__ void k_pair_counts(int64_t nt, const int32_t* __restrict__ cnt, int32_t* tot) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nt) tot[q] = cnt[2 * q] + cnt[2 * q + 1];
}

__global__ void k_i32_prefix64(int64_t n, const int32_t* __restrict__ in, int64_t* out) {
    // one thread: n is the number of judged targets (thousands)
    if (blockIdx.x || threadIdx.x) return;
    int64_t s = 0;
    for (int64_t k = 0; k < n; k++) { out[k] = s; s += in[k]; }
    out[n] = s;
}

ConvArgs make_args(Ctx& c) {
    ConvArgs a{};
    a.nl = c.nleaves;
    a.lvf = c.lf_vf.p; a.lvl = c.lf_vl.p; a.lgeom = c.lf_geom.p;
    a.near_off = c.near_off.p; a.near_run = c.near_run.p;
    a.taylor = c.lf_taylor.p; a.cm = c.nd_cm.p;
    a.x = c.x.p; a.y = c.y.p; a.g = c.g.p; a.ie = c.ie.p; a.vx = c.vx.p; a.vy = c.vy.p;
    a.ns = c.ns; a.kx = c.k_x.p; a.ky = c.k_y.p; a.kg = c.k_g.p; a.sink_e2 = c.dt * C_1_PI;
    a.m = c.m; a.srx = c.s_rx.p; a.sry = c.s_ry.p; a.sg = c.s_g.p; a.sie = c.s_ie.p; a.slip = c.s_slip.p;
    a.any_slip = 0;
    for (auto s : c.h_slip) a.any_slip |= (s != 0);
    // moving bodies: per-segment speed and axis of the body (TBody::get_axis = holder + dpos)
    a.any_moving = 0;
    for (auto& b : c.bodies) {
        const vvgpu_body_params& p = b.p;
        if (!(std::fabs(p.speed_slae_x) + std::fabs(p.speed_slae_y) + std::fabs(p.speed_slae_o) < 1E-10))
            a.any_moving = 1;
    }
    if (a.any_moving) {
        c.h_att.assign(5 * (size_t)c.m, 0.);
        c.h_att_on.assign((size_t)c.m, 0);
        for (auto& b : c.bodies) {
            const vvgpu_body_params& p = b.p;
            if (std::fabs(p.speed_slae_x) + std::fabs(p.speed_slae_y) + std::fabs(p.speed_slae_o) < 1E-10) continue;
            for (int64_t k = b.first; k < b.first + b.count; k++) {
                double* w = c.h_att.data() + 5 * k;
                w[0] = p.speed_slae_x; w[1] = p.speed_slae_y; w[2] = p.speed_slae_o;
                w[3] = p.holder_x + p.dpos_x; w[4] = p.holder_y + p.dpos_y;
                c.h_att_on[k] = 1;
            }
        }
        c.s_att.reserve(5 * (size_t)c.m);
        c.s_att_on.reserve((size_t)c.m);
        VV_CUDA(cudaMemcpyAsync(c.s_att.p, c.h_att.data(), 5 * c.m * 8, cudaMemcpyHostToDevice, c.st()));
        VV_CUDA(cudaMemcpyAsync(c.s_att_on.p, c.h_att_on.data(), c.m * 4, cudaMemcpyHostToDevice, c.st()));
        a.scx = c.s_cx.p; a.scy = c.s_cy.p; a.sdlx = c.s_dlx.p; a.sdly = c.s_dly.p;
        a.att = c.s_att.p; a.att_on = c.s_att_on.p;
    }
    a.inf_vx = c.inf_vx; a.inf_vy = c.inf_vy;
    a.fc = c.far_criteria; a.nnodes = c.nnodes;
    return a;
}

}  // namespace

void check_bodies_at_rest(Ctx& c) {
    for (auto& b : c.bodies) {
        const vvgpu_body_params& p = b.p;
        if (!(std::fabs(p.speed_slae_x) + std::fabs(p.speed_slae_y) + std::fabs(p.speed_slae_o) < 1E-10))
            throw ApiError{VVGPU_ERR_UNSUPPORTED, "moving bodies (attached sheets) are not supported"};
    }
}

void build_frames(Ctx& c) {
    cudaStream_t s = c.st();
    const int64_t n = c.n, nl = c.nleaves;
    double4 rootl;
    double4* rp = pinned_at(c, 64, &rootl);
    VV_CUDA(cudaMemcpyAsync(rp, c.nd_geom.p, sizeof rootl, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    const double4 root = *rp;
    Frame fr = make_frame(std::fmax(std::fabs(root.x), std::fabs(root.y)) + std::fmax(root.z, root.w));
    c.frame_G = fr.G;
    c.lf_anchor.reserve(nl + 1);
    c.src32.reserve(n + 1);
    c.src_k.reserve(n + 1);
    c.src_ie.reserve(n + 1);
    c.src_a4.reserve(n + 1);
    if (nl) {
        k_anchor2<<<grid_for(nl, 128), 128, 0, s>>>(nl, c.lf_geom.p, fr.G, c.lf_anchor.p);
        VV_LAUNCH_CHECK();
    }
    if (n) {
        k_src32<<<grid_for(n, 256), 256, 0, s>>>(n, c.leaf_of.p, c.lf_anchor.p, fr.G, c.x.p, c.y.p, c.g.p, c.ie.p,
                                                 c.src32.p, c.src_k.p, c.src_ie.p, c.src_a4.p);
        VV_LAUNCH_CHECK();
    }
}

void count_near_pairs(Ctx& c) {
    cudaStream_t s = c.st();
    const int64_t nl = c.nleaves;
    DArr<int32_t>& nz = c.np_nz;  // context scratch: no device allocation per pass
    DArr<int32_t>& pre = c.np_pre;
    nz.reserve(nl + 1);
    pre.reserve(nl + 2);
    k_leaf_nz<<<grid_for(nl, 256), 256, 0, s>>>(nl, c.lf_vf.p, c.lf_vl.p, c.g.p, nz.p);
    VV_LAUNCH_CHECK();
    exclusive_scan(c, nz.p, pre.p, nl);
    unsigned long long* out = c.counters.p + 11;
    VV_CUDA(cudaMemsetAsync(out, 0, 8, s));
    k_near_pairs<<<grid_for(nl, 256), 256, 0, s>>>(nl, nz.p, pre.p, c.near_off.p, c.near_run.p, out);
    VV_LAUNCH_CHECK();
    unsigned long long vl = 0;
    unsigned long long* v = pinned_at(c, 120, &vl);
    VV_CUDA(cudaMemcpyAsync(v, out, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    c.stats.near_pairs = (int64_t)*v;
}

void convective(Ctx& c) {
    if (c.n == 0 || c.nleaves == 0) return;
    if (c.tune_pending) autotune_tiles(c, nullptr);  // the shapes of this and the later passes
    cudaStream_t s = c.st();
    if (c.count_pairs) count_near_pairs(c);
    ConvArgs a = make_args(c);
    unsigned grid = grid_for(c.nleaves, CW);
    if (c.precision == VVGPU_FP32) {
        build_frames(c);
        a.src32 = c.src32.p; a.src_k = c.src_k.p; a.anchor = c.lf_anchor.p; a.G = c.frame_G; a.Gf = (float)c.frame_G;
        const int64_t nr = c.n_near_runs;
        c.run_js.reserve(nr + 1);
        c.leaf_tot.reserve(c.nleaves + 1);
        k_run_table<<<grid_for(c.nleaves, 8), 256, 0, s>>>(c.nleaves, c.near_off.p, c.near_run.p, c.lf_vf.p,
                                                         c.lf_vl.p, c.run_js.p, c.leaf_tot.p);
        VV_LAUNCH_CHECK();
        a.src_a4 = c.src_a4.p; a.run_js = c.run_js.p; a.leaf_tot = c.leaf_tot.p; a.nsrc = c.n;
        a.spins = c.wait_spins;
        a.err = c.counters.p + 20;
        VV_CUDA(cudaMemsetAsync(a.err, 0, 8, s));
        auto launch = [&](auto kern, int ct) {
            VV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)conv32_smem(ct)));
            KernelTimer kt(c, VVGPU_T_CONVECTIVE);
            kern<<<grid_for(c.nleaves, CW32), CW32 * 32, conv32_smem(ct), s>>>(a);
            VV_LAUNCH_CHECK();
        };
        // default 256 sources per tile: 6.50 ms at 4M against 6.81 ms for 192 (one-warp blocks)
        if (c.conv_tile == 128) launch(k_conv32<128>, 128);
        else if (c.conv_tile == 192) launch(k_conv32<192>, 192);
        else launch(k_conv32<256>, 256);
        unsigned long long el = 0;
        unsigned long long* ep = pinned_at(c, 96, &el);
        VV_CUDA(cudaMemcpyAsync(ep, a.err, 8, cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
        if (*ep) throw ApiError{VVGPU_ERR_TIMEOUT, "near-field staging wait timed out"};
    } else {
        KernelTimer kt(c, VVGPU_T_CONVECTIVE);
        k_conv64<8><<<grid, CW * 32, 0, s>>>(a);
        VV_LAUNCH_CHECK();
    }
    VV_CUDA(cudaStreamSynchronize(s));
}

void velocity_points(Ctx& c, int64_t np, const double* px, const double* py, double* vx, double* vy) {
    if (np == 0) return;
    cudaStream_t s = c.st();
    DArr<double> q;
    q.reserve(4 * np);
    VV_CUDA(cudaMemcpyAsync(q.p, px, np * 8, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(q.p + np, py, np * 8, cudaMemcpyHostToDevice, s));
    ConvArgs a = make_args(c);
    k_points<<<grid_for(np, 128), 128, 0, s>>>(np, q.p, q.p + np, c.nd_geom.p, c.nd_ch1.p, c.nd_dfs.p, a,
                                              q.p + 2 * np, q.p + 3 * np);
    VV_LAUNCH_CHECK();
    VV_CUDA(cudaMemcpyAsync(vx, q.p + 2 * np, np * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaMemcpyAsync(vy, q.p + 3 * np, np * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
}

void direct_velocity(Ctx& c, int64_t np, const double* px, const double* py, double* vx, double* vy) {
    check_input(c);
    if (np == 0) return;
    upload_segments(c);
    cudaStream_t s = c.st();
    DArr<double> q;
    q.reserve(4 * np);
    VV_CUDA(cudaMemcpyAsync(q.p, px, np * 8, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(q.p + np, py, np * 8, cudaMemcpyHostToDevice, s));
    ConvArgs a = make_args(c);
    for (int64_t b = 0; b < np; b += 65535) {
        const int64_t cnt = std::min<int64_t>(65535, np - b);
        k_direct<<<(unsigned)cnt, DIRECT_TB, 0, s>>>(c.n, q.p + b, q.p + np + b, a, q.p + 2 * np + b,
                                                     q.p + 3 * np + b);
        VV_LAUNCH_CHECK();
    }
    VV_CUDA(cudaMemcpyAsync(vx, q.p + 2 * np, np * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaMemcpyAsync(vy, q.p + 3 * np, np * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
}

// The judged velocities: the warp walk, then the per-thread FP64 walk for the few targets
// whose level walk did not fit its buffers.
void judge_velocity(Ctx& c, int64_t nt, const int32_t* d_idx, double fc, double* d_out) {
    if (nt <= 0) return;
    cudaStream_t s = c.st();
    judge_walk(c, nt, d_idx, fc, d_out);
    ConvArgs a = make_args(c);
    k_judge_finish<<<grid_for(nt, 128), 128, 0, s>>>(nt, d_idx, a, d_out);
    VV_LAUNCH_CHECK();
    std::vector<double> h(3 * (size_t)nt);
    VV_CUDA(cudaMemcpyAsync(h.data(), d_out, 3 * nt * 8, cudaMemcpyDeviceToHost, s));
    std::vector<int32_t> hidx(nt);
    VV_CUDA(cudaMemcpyAsync(hidx.data(), d_idx, nt * 4, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    std::vector<int32_t> rest;
    std::vector<int64_t> where;
    for (int64_t q = 0; q < nt; q++)
        if (h[3 * q + 2] < 0.) { rest.push_back(hidx[q]); where.push_back(q); }
    if (rest.empty()) return;
    DArr<int32_t> ridx;
    DArr<double> rout;
    ridx.reserve(rest.size());
    rout.reserve(3 * rest.size());
    VV_CUDA(cudaMemcpyAsync(ridx.p, rest.data(), rest.size() * 4, cudaMemcpyHostToDevice, s));
    judge_velocity_exact(c, (int64_t)rest.size(), ridx.p, fc, rout.p);
    std::vector<double> hr(3 * rest.size());
    VV_CUDA(cudaMemcpyAsync(hr.data(), rout.p, hr.size() * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    for (size_t k = 0; k < rest.size(); k++)
        VV_CUDA(cudaMemcpyAsync(d_out + 3 * where[k], &hr[3 * k], 24, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaStreamSynchronize(s));
}

// Per-thread FP64 walks (k_judge_walk) and warp sums (k_judge_sum) at the vortices d_idx.
void judge_velocity_exact(Ctx& c, int64_t nt, const int32_t* d_idx, double fc, double* d_out) {
    if (nt <= 0) return;
    cudaStream_t s = c.st();
    ConvArgs a = make_args(c);
    DArr<int32_t> cnt, tot, err;
    DArr<int64_t> off;
    cnt.reserve(2 * nt);
    tot.reserve(nt);
    off.reserve(nt + 1);
    err.reserve(1);
    VV_CUDA(cudaMemsetAsync(err.p, 0, 4, s));
    k_judge_walk<false><<<grid_for(nt, 64), 64, 0, s>>>(nt, d_idx, c.x.p, c.y.p, c.g.p, c.nd_geom.p, c.nd_ch1.p, fc,
                                                        c.nnodes, cnt.p, nullptr, nullptr, err.p);
    VV_LAUNCH_CHECK();
    k_pair_counts<<<grid_for(nt, 256), 256, 0, s>>>(nt, cnt.p, tot.p);
    VV_LAUNCH_CHECK();
    k_i32_prefix64<<<1, 32, 0, s>>>(nt, tot.p, off.p);
    VV_LAUNCH_CHECK();
    int64_t total = 0;
    VV_CUDA(cudaMemcpyAsync(&total, off.p + nt, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    DArr<int32_t> list;
    list.reserve(total + 1);
    k_judge_walk<true><<<grid_for(nt, 64), 64, 0, s>>>(nt, d_idx, c.x.p, c.y.p, c.g.p, c.nd_geom.p, c.nd_ch1.p, fc,
                                                       c.nnodes, cnt.p, off.p, list.p, err.p);
    VV_LAUNCH_CHECK();
    k_judge_sum<<<grid_for(nt, 4), 128, 0, s>>>(nt, d_idx, cnt.p, off.p, list.p, c.nd_vf.p, c.nd_vl.p, a, d_out);
    VV_LAUNCH_CHECK();
    if (read_i32(c, err.p)) throw ApiError{VVGPU_ERR_LIMIT, "judge walk exceeded its bound"};
}

// Point velocities for points already in device memory: the same kernel as
// velocity_points, launched on caller-provided device buffers, allocating nothing.
void velocity_points_on_device(Ctx& c, int64_t np, const double* dpx, const double* dpy, double* dvx,
                               double* dvy) {
    if (np == 0) return;
    ConvArgs a = make_args(c);
    k_points<<<grid_for(np, 128), 128, 0, c.st()>>>(np, dpx, dpy, c.nd_geom.p, c.nd_ch1.p, c.nd_dfs.p, a, dvx, dvy);
    VV_LAUNCH_CHECK();
}

}  // namespace vvgpu
