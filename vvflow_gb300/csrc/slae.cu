// Body SLAE of libvvhd (MConvectiveFast::calc_circulation / fill_matrix,
// libvvhd/src/MConvectiveFast.cpp:235-273, 882-1017) for rigid bodies.
//
// Rows and columns follow the reference's equation numbering and solution-pointer map
// (MConvectiveFast.cpp:250-267, 896-975): per body [segments..., speed_slae x,y,o,
// force_hydro x,y,o, force_holder x,y,o].
//   * slip rows (fillSlipEquationForSegment, :459-482): one thread block per row; the
//     M cells are 2 pi Xi_gamma (:286-310) of every segment's corner, the right-hand side
//     is the free stream, sinks and NodeInfluence (:398-418) through the tree.
//   * special rows (InfSteady / Steady / Zero, :484-522) and the nine body rows (Speed,
//     Hydro, Newton, :533-862): one thread each.
// Solve: the inverse is computed on the GPU by in-place Gauss-Jordan elimination with
// partial pivoting and cached while the matrix bytes are unchanged (the reference caches
// its LAPACK inverse by a hash of the matrix, TMatrix.cpp:225-259).  FP64 mode inverts in
// FP64; FP32 mode inverts in FP32.  Either way x = inv b is refined with FP64 residuals
// r = b - A x until |r| / |b| < 1e-13 (at most 12 sweeps).
#include <cfloat>
#include <cstring>

#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

struct SegDev {
    const double* cx; const double* cy; const double* rx; const double* ry; const double* dlx; const double* dly;
};

__device__ __forceinline__ double xi_g_near(double px, double py, double pcx, double pcy, double dlx, double dly,
                                            double rd) {
    return ((pcx - px) * dlx + (pcy - py) * dly) / (rd * rd);
}
__device__ __forceinline__ double xi_g_dist(double px, double py, double p1x, double p1y, double p2x, double p2y) {
    double a = (px - p2x) * (px - p2x) + (py - p2y) * (py - p2y);
    double b = (px - p1x) * (px - p1x) + (py - p1y) * (py - p1y);
    return 0.5 * log(a / b);
}
// _2PI_Xi_g (MConvectiveFast.cpp:286-310)
__device__ double xi_g(const SegDev& S, double px, double py, int32_t s, double rd) {
    double cx = S.cx[s], cy = S.cy[s], dlx = S.dlx[s], dly = S.dly[s];
    double rd_sqr = rd * rd;
    double dr1 = (px - cx) * (px - cx) + (py - cy) * (py - cy);
    double ex = (px - cx) - dlx, ey = (py - cy) - dly;
    double dr2 = ex * ex + ey * ey;
    if (dr1 >= rd_sqr && dr2 >= rd_sqr) return 0.5 * log(dr2 / dr1);
    double rx = S.rx[s], ry = S.ry[s];
    if (dr1 <= rd_sqr && dr2 <= rd_sqr) return xi_g_near(px, py, rx, ry, dlx, dly, rd);
    double a0 = dlx * dlx + dly * dly;
    double b0 = (px - rx) * dlx + (py - ry) * dly;
    double d = sqrt(b0 * b0 - a0 * (((px - rx) * (px - rx) + (py - ry) * (py - ry)) - rd * rd));
    double k = (b0 + d) / a0;
    if ((k <= -0.5) || (k >= 0.5)) k = (b0 - d) / a0;
    double p3x = rx + dlx * k, p3y = ry + dly * k;
    if (dr1 < rd_sqr)
        return xi_g_near(px, py, (p3x + cx) * 0.5, (p3y + cy) * 0.5, p3x - cx, p3y - cy, rd) +
               xi_g_dist(px, py, p3x, p3y, cx + dlx, cy + dly);
    return xi_g_dist(px, py, cx, cy, p3x, p3y) +
           xi_g_near(px, py, ((cx + dlx) + p3x) * 0.5, ((cy + dly) + p3y) * 0.5, (cx + dlx) - p3x,
                     (cy + dly) - p3y, rd);
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; w++) t += sh[w];
    __syncthreads();
    return t;  // valid in thread 0
}

struct RowInfo {
    int32_t seg;     // global segment index of the row (slip rows)
    int32_t body;
};

struct FillArgs {
    int64_t n;       // system size
    double* A; double* B;
    SegDev S;
    const int32_t* slip_rows; int64_t nslip;  // row index of each slip row
    const int32_t* row_seg; const int32_t* row_body;
    const int32_t* col_seg0; const int32_t* body_first; const int32_t* body_count; int nbodies;
    // tree
    const double4* geom; const int32_t* ch1; const int32_t* dfs;
    const int32_t* lvf; const int32_t* lvl; const int32_t* near_off; const int2* near_run;
    const int32_t* far_off; const int32_t* far_node; const double* cm;
    const double* x; const double* y; const double* g; const double* ie;
    int64_t ns; const double* kx; const double* ky; const double* kg; double sink_e2;
    double inf_vx, inf_vy;
    bool rhs_only;
};

// 0.5 log(dr2 / dr1) in FP32 for a point clear of both smoothing discs; d = point - corner
// 1, dr2 - dr1 = |dl|^2 - 2 d.dl exactly, so a ratio near 1 goes through log1p of that
// difference instead of a cancelling quotient.
__device__ __forceinline__ float half_log_ratio(float dr1, float dr2, float dx, float dy, float dlx, float dly,
                                                float dl2) {
    const float q = dr2 / dr1;
    if (q > 0.5f && q < 2.f) return 0.5f * log1pf((dl2 - 2.f * (dx * dlx + dy * dly)) / dr1);
    return 0.5f * logf(q);
}

// One block per slip row: RHS through the tree, then (unless rhs_only) the M + 3 nb cells.
// F32: the RHS pairs clear of both smoothing discs (the reference's log branch, decided
// with a 1e-4 margin) and the far centroids run in FP32 with compensated sums; every other
// pair takes the FP64 formula.  The matrix cells are FP64 in both modes.
template <bool F32>
__global__ void k_slip_rows(FillArgs a) {
    __shared__ double sh[32];
    const int64_t ri = blockIdx.x;
    if (ri >= a.nslip) return;
    const int32_t row = a.slip_rows[ri];
    const int32_t s = a.row_seg[row];
    const int32_t bi = a.row_body[row];
    const double srx = a.S.rx[s], sry = a.S.ry[s], dlx = a.S.dlx[s], dly = a.S.dly[s];
    // findNode(seg.r)
    int32_t k = 0;
    for (int it = 0; it <= MAX_DEPTH && a.ch1[k] >= 0; it++) {
        double4 gm = a.geom[k];
        if (gm.z < gm.w) k = (srx < gm.x) ? a.ch1[k] : a.ch1[k] + 1;
        else k = (sry < gm.y) ? a.ch1[k] : a.ch1[k] + 1;
    }
    const int32_t L = a.dfs[k];
    double part = 0;
    const double c1x = a.S.cx[s], c1y = a.S.cy[s], c2x = c1x + dlx, c2y = c1y + dly;
    const float dlxf = (float)dlx, dlyf = (float)dly, dl2f = (float)(dlx * dlx + dly * dly);
    float ph = 0.f, pl = 0.f;
    for (int32_t r = a.near_off[L]; r < a.near_off[L + 1]; r++) {
        int2 run = a.near_run[r];
        for (int32_t j = a.lvf[run.x] + threadIdx.x; j < a.lvl[run.y - 1]; j += blockDim.x) {
            double gj = a.g[j];
            if (gj == 0.) continue;
            if (F32) {
                const double xj = a.x[j], yj = a.y[j], iej = a.ie[j];
                const float dx = (float)(xj - c1x), dy = (float)(yj - c1y);
                const float ex = dx - dlxf, ey = dy - dlyf;
                const float dr1 = dx * dx + dy * dy, dr2 = ex * ex + ey * ey;
                const float ie2 = (float)iej * (float)iej;
                if (dr1 * ie2 > 1.0001f && dr2 * ie2 > 1.0001f) {  // false for NaN
                    two_sum_acc(ph, pl, half_log_ratio(dr1, dr2, dx, dy, dlxf, dlyf, dl2f) * (float)gj);
                    continue;
                }
                part += xi_g(a.S, xj, yj, s, 1. / iej) * gj;
            } else {
                part += xi_g(a.S, a.x[j], a.y[j], s, 1. / a.ie[j]) * gj;
            }
        }
    }
    for (int32_t t = a.far_off[L] + threadIdx.x; t < a.far_off[L + 1]; t += blockDim.x) {
        const double* c = a.cm + 6 * (size_t)a.far_node[t];
        if (F32) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const double px = c[3 * h], py = c[3 * h + 1], g = c[3 * h + 2];
                const float dx = (float)(px - c1x), dy = (float)(py - c1y);
                const float ex = dx - dlxf, ey = dy - dlyf;
                const float dr1 = dx * dx + dy * dy, dr2 = ex * ex + ey * ey;
                if (dr1 > 1e-30f && dr2 > 1e-30f && dr1 < 1e30f && dr2 < 1e30f) {
                    // a finite log times g: an empty sign (g = 0) adds exactly 0
                    if (g != 0.) two_sum_acc(ph, pl, half_log_ratio(dr1, dr2, dx, dy, dlxf, dlyf, dl2f) * (float)g);
                } else {
                    part += xi_g_dist(px, py, c1x, c1y, c2x, c2y) * g;
                }
            }
        } else {
            part += xi_g_dist(c[0], c[1], c1x, c1y, c2x, c2y) * c[2];
            part += xi_g_dist(c[3], c[4], c1x, c1y, c2x, c2y) * c[5];
        }
    }
    if (F32) part += (double)ph + (double)pl;
    double node_inf = block_sum(part, sh);
    if (threadIdx.x == 0) {
        double rhs = (-a.inf_vy) * dlx + a.inf_vx * dly;
        double kxs = 0, kys = 0;
        for (int64_t q = 0; q < a.ns; q++) {
            double dx = srx - a.kx[q], dy = sry - a.ky[q];
            double f = a.kg[q] / (dx * dx + dy * dy + a.sink_e2 * sink_abs(a.kg[q]));
            kxs += dx * f; kys += dy * f;
        }
        kxs *= C_1_2PI; kys *= C_1_2PI;
        rhs += (-kys) * dlx + kxs * dly;
        rhs -= node_inf * C_1_2PI;
        a.B[row] = rhs;
    }
    if (a.rhs_only) return;
    double* Arow = a.A + (size_t)row * a.n;
    for (int bj = 0; bj < a.nbodies; bj++) {
        const int32_t f = a.body_first[bj], cnt = a.body_count[bj], c0 = a.col_seg0[bj];
        for (int32_t q = threadIdx.x; q < cnt; q += blockDim.x) {
            int32_t sj = f + q;
            double rd = sqrt(a.S.dlx[sj] * a.S.dlx[sj] + a.S.dly[sj] * a.S.dly[sj]) * 0.25;
            Arow[c0 + q] = xi_g(a.S, a.S.cx[sj], a.S.cy[sj], s, rd) * C_1_2PI;
        }
        if (threadIdx.x == 0) {
            double a1 = (bi == bj) ? C_2PI * dly : 0;
            double a2 = (bi == bj) ? -C_2PI * dlx : 0;
            Arow[c0 + cnt + 0] = a1 * C_1_2PI;
            Arow[c0 + cnt + 1] = a2 * C_1_2PI;
            Arow[c0 + cnt + 2] = 0.;
        }
    }
}

struct BodyDev {
    double area, cofx, cofy, axx, axy, moi, dens;
    double pvx, pvy, pvo, fpx, fpy, fpo, fdx, fdy, fdo, gdead;
    double spx, spy, spo;
    int32_t special, kutta;
};

// Special and body rows: one block per body; the threads fill the per-segment cells, thread
// 0 the scalar cells and right-hand sides.  inf_body is the body whose special segment
// carries the InfSteady row (the first non-Kutta body, MConvectiveFast.cpp:905-913).
__global__ void k_body_rows(int64_t n, double* A, double* B, const BodyDev* bd, int nb,
                            const int32_t* col_seg0, const int32_t* body_count, const double* cy_,
                            const double* cx_, const int32_t* body_first, double dt, double gsum, double inf_g,
                            double gx, double gy, int inf_body, bool rhs_only) {
    const int bi = blockIdx.x;
    if (bi >= nb) return;
    const double _1_dt = 1 / dt, _1_2dt = 0.5 / dt;
    const BodyDev& b = bd[bi];
    const int32_t c0 = col_seg0[bi], cnt = body_count[bi], f = body_first[bi];
    const int32_t e0 = c0 + cnt;
    const double area = b.area, rcx = b.cofx - b.axx, rcy = b.cofy - b.axy, moi = b.moi, dens = b.dens;
    // special segment row
    {
        const int32_t eq = c0 + b.special;
        double* Ar = A + (size_t)eq * n;
        if (b.kutta) {
            if (threadIdx.x == 0) { B[eq] = 0; if (!rhs_only) Ar[c0 + b.special] = 1; }
        } else if (bi == inf_body) {
            if (threadIdx.x == 0) B[eq] = -gsum - inf_g;
            if (!rhs_only)
                for (int bj = 0; bj < nb; bj++) {
                    for (int32_t q = threadIdx.x; q < body_count[bj]; q += blockDim.x) Ar[col_seg0[bj] + q] = 1;
                    if (threadIdx.x == 0) Ar[col_seg0[bj] + body_count[bj] + 2] = 2 * bd[bj].area;
                }
        } else {
            if (threadIdx.x == 0) {
                B[eq] = b.gdead + 2 * b.area * b.pvo;
                if (!rhs_only) Ar[c0 + cnt + 2] = 2 * b.area;
            }
            if (!rhs_only) for (int32_t q = threadIdx.x; q < cnt; q += blockDim.x) Ar[c0 + q] = 1;
        }
    }
    // per-segment cells of the Hydro rows (:551-552, :582-583, :612-613)
    if (!rhs_only)
        for (int32_t q = threadIdx.x; q < cnt; q += blockDim.x) {
            A[(size_t)(e0 + 3) * n + c0 + q] = _1_dt * (-cy_[f + q]);
            A[(size_t)(e0 + 4) * n + c0 + q] = _1_dt * (cx_[f + q]);
            const double dx = cx_[f + q] - b.axx, dy = cy_[f + q] - b.axy;
            A[(size_t)(e0 + 5) * n + c0 + q] = _1_2dt * (dx * dx + dy * dy);
        }
    if (threadIdx.x != 0) return;
    auto cell = [&](int32_t eq, int q, double v) { if (!rhs_only) A[(size_t)eq * n + e0 + q] = v; };
    // Speed rows (rigid bodies, :803-862)
    B[e0 + 0] = b.spx; cell(e0 + 0, 0, 1);
    B[e0 + 1] = b.spy; cell(e0 + 1, 1, 1);
    B[e0 + 2] = b.spo; cell(e0 + 2, 2, 1);
    // Hydro X/Y/O (:533-623)
    {
        const int32_t eq = e0 + 3;
        const double ty = b.cofy * 2 + rcy;
        B[eq] = area * _1_dt * b.pvx + area * _1_dt * (-ty) * b.pvo + (b.pvo * b.pvo) * area * rcx - b.fpx +
                b.fdx * _1_dt;
        cell(eq, 0, area * _1_dt); cell(eq, 1, 0); cell(eq, 2, area * _1_dt * (-2 * b.cofy - rcy)); cell(eq, 3, -1);
    }
    {
        const int32_t eq = e0 + 4;
        const double tx = b.cofx * 2 + rcx;
        B[eq] = area * _1_dt * b.pvy + area * _1_dt * tx * b.pvo + (b.pvo * b.pvo) * area * rcy - b.fpy +
                b.fdy * _1_dt;
        cell(eq, 0, 0); cell(eq, 1, area * _1_dt); cell(eq, 2, area * _1_dt * (2 * b.cofx + rcx)); cell(eq, 4, -1);
    }
    {
        const int32_t eq = e0 + 5;
        const double c = area * _1_dt;
        const double lx = (-rcy) * c, ly = rcx * c;
        B[eq] = (lx * b.pvx + ly * b.pvy) + 2 * moi * _1_dt * b.pvo - b.fpo + b.fdo * _1_2dt;
        cell(eq, 0, area * _1_dt * (-rcy)); cell(eq, 1, area * _1_dt * rcx); cell(eq, 2, 2 * moi * _1_dt);
        cell(eq, 5, -1);
    }
    // Newton X/Y/O (:634-739)
    {
        const int32_t eq = e0 + 6;
        B[eq] = -area * _1_dt * dens * b.pvx + area * _1_dt * dens * rcy * b.pvo -
                area * dens * rcx * (b.pvo * b.pvo) - (dens - 1.0) * gx * area;
        cell(eq, 0, -area * _1_dt * dens); cell(eq, 1, 0); cell(eq, 2, area * _1_dt * dens * rcy);
        cell(eq, 3, 1); cell(eq, 6, -1);
    }
    {
        const int32_t eq = e0 + 7;
        B[eq] = -area * _1_dt * dens * b.pvy - area * _1_dt * dens * rcx * b.pvo -
                area * dens * rcy * (b.pvo * b.pvo) - (dens - 1.0) * gy * area;
        cell(eq, 0, 0); cell(eq, 1, -area * _1_dt * dens); cell(eq, 2, -area * _1_dt * dens * rcx);
        cell(eq, 4, 1); cell(eq, 7, -1);
    }
    {
        const int32_t eq = e0 + 8;
        const double rlx = -rcy, rly = rcx;
        B[eq] = -area * _1_dt * dens * (rlx * b.pvx + rly * b.pvy) - moi * _1_dt * dens * b.pvo -
                (dens - 1.0) * (rlx * gx + rly * gy) * area;
        cell(eq, 0, +area * _1_dt * dens * rcy); cell(eq, 1, -area * _1_dt * dens * rcx);
        cell(eq, 2, -moi * _1_dt * dens); cell(eq, 5, 1); cell(eq, 8, -1);
    }
}

// ---- Gauss-Jordan inversion in place (row pivoting; columns unscrambled at the end) ----
// Step k eliminates column k from every other row with the pivot row as it stands
// (M[i][j] -= (M[i][k] / d) M[k][j]) and normalises the pivot row afterwards (at the start
// of step k + 1, or by k_gj_norm after the last step).  Rows that are equal stay equal
// under the same operations and the second of them becomes exactly zero, so an exactly
// singular system ends with a zero (or NaN) pivot, as in LAPACK's LU (dgetrf's info > 0,
// where the reference exits, TMatrix.cpp:195-213).

// Row r of M divided by its pivot d = dpiv[r] (the diagonal entry becomes 1 / d).
template <class T>
__device__ __forceinline__ void gj_normalise_row(int64_t n, int64_t r, T* M, const T* dpiv) {
    const T d = dpiv[r];
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        if (j == r) M[r * n + r] = (T)1 / d;
        else M[r * n + j] = M[r * n + j] / d;
    }
}

template <class T>
__global__ void k_gj_pivot(int64_t n, int64_t k, T* M, int32_t* perm, T* col, T* dpiv, int32_t* singular) {
    __shared__ double bv[1024];
    __shared__ int32_t bi[1024];
    if (k > 0) gj_normalise_row(n, k - 1, M, dpiv);
    __syncthreads();
    double best = -1;
    int32_t arg = -1;
    for (int64_t i = k + threadIdx.x; i < n; i += blockDim.x) {
        double v = fabs((double)M[i * n + k]);
        if (v > best) { best = v; arg = (int32_t)i; }
    }
    bv[threadIdx.x] = best;
    bi[threadIdx.x] = arg;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            double v2 = bv[threadIdx.x + o];
            int32_t i2 = bi[threadIdx.x + o];
            if (v2 > bv[threadIdx.x] || (v2 == bv[threadIdx.x] && i2 >= 0 && i2 < bi[threadIdx.x])) {
                bv[threadIdx.x] = v2;
                bi[threadIdx.x] = i2;
            }
        }
        __syncthreads();
    }
    const int32_t p = bi[0];
    if (bv[0] <= 0 || p < 0) {  // zero or NaN column: singular (the rest of the inverse is void)
        if (threadIdx.x == 0) { *singular = 1; perm[k] = (int32_t)k; dpiv[k] = (T)1; }
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) col[i] = 0;
        return;
    }
    if (threadIdx.x == 0) perm[k] = p;
    if (p != k)
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            T t = M[k * n + j];
            M[k * n + j] = M[(int64_t)p * n + j];
            M[(int64_t)p * n + j] = t;
        }
    __syncthreads();
    const T d = M[k * n + k];
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) col[i] = (i == k) ? (T)0 : M[i * n + k] / d;
    if (threadIdx.x == 0) dpiv[k] = d;
}

template <class T>
__global__ void k_gj_elim(int64_t n, int64_t k, T* M, const T* __restrict__ col) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i = blockIdx.y;
    if (j >= n || i == k) return;
    const T f = col[i];
    if (j == k) M[i * n + k] = -f;
    else M[i * n + j] -= f * M[k * n + j];
}

template <class T>
__global__ void k_gj_norm(int64_t n, int64_t r, T* M, const T* dpiv) {
    gj_normalise_row(n, r, M, dpiv);
}

template <class T>
__global__ void k_gj_colswap(int64_t n, T* M, const int32_t* perm, int64_t k) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t p = perm[k];
    if (p == k) return;
    T t = M[i * n + k];
    M[i * n + k] = M[i * n + p];
    M[i * n + p] = t;
}

template <class T>
void invert(Ctx& c, T* M, int64_t n, int32_t* singular) {
    cudaStream_t s = c.st();
    DArr<T> col, dpiv;
    col.reserve(n);
    dpiv.reserve(n);
    c.piv.reserve(n);
    for (int64_t k = 0; k < n; k++) {
        k_gj_pivot<T><<<1, 1024, 0, s>>>(n, k, M, c.piv.p, col.p, dpiv.p, singular);
        VV_LAUNCH_CHECK();
        dim3 grid(grid_for(n, 256), (unsigned)n);
        k_gj_elim<T><<<grid, 256, 0, s>>>(n, k, M, col.p);
        VV_LAUNCH_CHECK();
    }
    if (n > 0) {
        k_gj_norm<T><<<1, 1024, 0, s>>>(n, n - 1, M, dpiv.p);
        VV_LAUNCH_CHECK();
    }
    for (int64_t k = n - 1; k >= 0; k--) {
        k_gj_colswap<T><<<grid_for(n, 256), 256, 0, s>>>(n, M, c.piv.p, k);
        VV_LAUNCH_CHECK();
    }
    VV_CUDA(cudaStreamSynchronize(s));
}

__global__ void k_differs(int64_t n, const unsigned long long* __restrict__ a,
                          const unsigned long long* __restrict__ b, int32_t* diff) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && a[i] != b[i]) *diff = 1;
}

__global__ void k_to_f32(int64_t n, const double* a, float* b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// y = M v (+ y0): one warp per row, FP64 accumulation.
template <class T>
__global__ void k_gemv(int64_t n, const T* __restrict__ M, const double* __restrict__ v, double* y, bool add) {
    int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double acc = 0;
    const T* r = M + row * n;
    for (int64_t j = lane; j < n; j += 32) acc += (double)r[j] * v[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[row] = add ? y[row] + acc : acc;
}

// FP32 inverse times an FP64 vector on the FP32 pipe: the vector split once into FP32
// pairs (hi, lo), each product m hi with its exact rounding error (an FMA) and m lo,
// accumulated as a TwoSum pair per lane and reduced as double-float pairs: the accuracy of
// FP64 accumulation (about 2^-48) without its narrow pipe.  One warp per row.
__global__ void k_split_vec(int64_t n, const double* __restrict__ v, float2* vs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = v[i];
    const float hi = (float)x;
    vs[i] = make_float2(hi, (float)(x - (double)hi));
}
__global__ void k_gemv32(int64_t n, const float* __restrict__ M, const float2* __restrict__ vs, double* y,
                         bool add) {
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const float* r = M + row * n;
    float h = 0.f, l = 0.f;
    for (int64_t j = lane; j < n; j += 32) {
        const float m = r[j];
        const float2 v = vs[j];
        const float p = m * v.x;
        const float pe = fmaf(m, v.x, -p);  // m v.x - p exactly
        const float sm = h + p, bp = sm - h;
        l += ((h - (sm - bp)) + (p - bp)) + fmaf(m, v.y, pe);
        h = sm;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
        const float sm = h + oh, bp = sm - h;
        l = l + ol + ((h - (sm - bp)) + (oh - bp));
        h = sm;
    }
    if (lane == 0) {
        const double acc = (double)h + (double)l;
        y[row] = add ? y[row] + acc : acc;
    }
}

// r = b - A x; sq[row] = r^2, sq[n + row] = b^2 (summed deterministically afterwards)
__global__ void k_residual(int64_t n, const double* __restrict__ A, const double* __restrict__ x,
                           const double* __restrict__ b, double* r, double* sq) {
    int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0;
    const double* Ar = A + row * n;
    for (int64_t j = lane; j < n; j += 32) s += Ar[j] * x[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        double rr = b[row] - s;
        r[row] = rr;
        sq[row] = rr * rr;
        sq[n + row] = b[row] * b[row];
    }
}

// Deterministic sums (the same bits on every run, unlike atomics across blocks): SUM_BLOCKS
// fixed blocks reduce fixed grid-stride slices, then one block adds their partials.
constexpr int SUM_BLOCKS = 304;
__global__ void k_sum_stage1(int64_t n, const double* __restrict__ v, double* part) {
    __shared__ double sh[32];
    double t = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        t += v[i];
    t = block_sum(t, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}
__global__ void k_sum_stage2(int nparts, const double* __restrict__ part, double* out) {
    __shared__ double sh[32];
    double t = 0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) t += part[i];
    t = block_sum(t, sh);
    if (threadIdx.x == 0) *out = t;
}

__global__ void k_scatter_solution(int64_t nb, const int32_t* col_seg0, const int32_t* body_first,
                                   const int32_t* body_count, const double* X, double* sg) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int b = 0; b < nb; b++) {
        if (t < body_count[b]) sg[body_first[b] + t] = X[col_seg0[b] + t];
    }
}

}  // namespace

double gsum(Ctx& c) {
    cudaStream_t s = c.st();
    c.counters.reserve(24);
    double* out = (double*)(c.counters.p + 4);
    VV_CUDA(cudaMemsetAsync(out, 0, 8, s));
    if (c.n) {
        c.sum_part.reserve(SUM_BLOCKS);
        k_sum_stage1<<<SUM_BLOCKS, 256, 0, s>>>(c.n, c.g.p, c.sum_part.p);
        VV_LAUNCH_CHECK();
        k_sum_stage2<<<1, 256, 0, s>>>(SUM_BLOCKS, c.sum_part.p, out);
        VV_LAUNCH_CHECK();
    }
    double v = 0;
    VV_CUDA(cudaMemcpyAsync(&v, out, 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    return v;
}

void slae(Ctx& c, vvgpu_body_out* out) {
    const int nb = (int)c.bodies.size();
    for (auto& b : c.bodies) {
        auto rigid = [](double k) { return !(k >= 0 && std::isfinite(k)); };
        if (!rigid(b.p.kspring_x) || !rigid(b.p.kspring_y) || !rigid(b.p.kspring_o))
            throw ApiError{VVGPU_ERR_UNSUPPORTED, "spring-mounted bodies are not supported"};
        if (b.p.speed_o != 0) throw ApiError{VVGPU_ERR_UNSUPPORTED, "rotating bodies are not supported"};
        if (b.p.special_segment_no < 0 || b.p.special_segment_no >= b.count)
            throw ApiError{VVGPU_ERR_ARG, "special_segment_no out of range"};
    }
    if (nb == 0) return;
    cudaStream_t s = c.st();
    const int64_t n = c.m + 9 * (int64_t)nb;
    c.neq = n;
    const double gs = gsum(c);
    // host-side row/column maps
    std::vector<int32_t> col0(nb), bfirst(nb), bcount(nb), row_seg(n, -1), row_body(n, -1), slip_rows;
    std::vector<BodyDev> bd(nb);
    {
        int32_t cc = 0;
        for (int bi = 0; bi < nb; bi++) {
            const BodyHost& b = c.bodies[bi];
            col0[bi] = cc;
            bfirst[bi] = (int32_t)b.first;
            bcount[bi] = (int32_t)b.count;
            for (int32_t k = 0; k < b.count; k++) {
                row_seg[cc + k] = (int32_t)(b.first + k);
                row_body[cc + k] = bi;
                if (k != b.p.special_segment_no) slip_rows.push_back(cc + k);
            }
            cc += (int32_t)b.count + 9;
            BodyDev& d = bd[bi];
            d.area = b.area; d.cofx = b.cofm_x; d.cofy = b.cofm_y;
            d.axx = b.p.holder_x + b.p.dpos_x; d.axy = b.p.holder_y + b.p.dpos_y;
            double dx = d.axx - b.cofm_x, dy = d.axy - b.cofm_y;
            d.moi = b.moi_cofm + (dx * dx + dy * dy) * b.area;
            d.dens = b.p.density;
            d.pvx = b.p.speed_slae_prev_x; d.pvy = b.p.speed_slae_prev_y; d.pvo = b.p.speed_slae_prev_o;
            d.fpx = b.p.friction_prev_x; d.fpy = b.p.friction_prev_y; d.fpo = b.p.friction_prev_o;
            d.fdx = b.p.fdt_dead_x; d.fdy = b.p.fdt_dead_y; d.fdo = b.p.fdt_dead_o; d.gdead = b.p.g_dead;
            d.spx = b.p.speed_x; d.spy = b.p.speed_y; d.spo = b.p.speed_o;
            d.special = b.p.special_segment_no; d.kutta = b.p.bc_kutta;
        }
    }
    int inf_body = -1;
    for (int bi = 0; bi < nb; bi++)
        if (!c.bodies[bi].p.bc_kutta) { inf_body = bi; break; }
    // Everything the matrix cells depend on.  While it is unchanged and the inverse is
    // cached, only the right-hand side is filled (the reference likewise refills just its
    // right column once the body matrix and its inverse are in place,
    // MConvectiveFast.cpp:245-246).
    std::vector<double> sig{(double)n, (double)nb, (double)c.precision, c.dt, (double)inf_body,
                            (double)c.seg_version};
    for (int bi = 0; bi < nb; bi++) {
        const BodyDev& d = bd[bi];
        sig.insert(sig.end(), {(double)bfirst[bi], (double)bcount[bi], d.area, d.cofx, d.cofy, d.axx, d.axy, d.moi,
                               d.dens, (double)d.special, (double)d.kutta});
    }
    const bool rhs_only = c.lu_valid && c.lu_precision == c.precision && c.neq_cached == n &&
                          sig.size() == c.slae_sig.size() &&
                          std::memcmp(sig.data(), c.slae_sig.data(), sig.size() * sizeof(double)) == 0;
    const size_t nsl = slip_rows.size();
    c.slae_maps.reserve(3 * nb + 2 * n + nsl + 1);
    int32_t* d_col0 = c.slae_maps.p;
    int32_t* d_bfirst = d_col0 + nb;
    int32_t* d_bcount = d_bfirst + nb;
    int32_t* d_rowseg = d_bcount + nb;
    int32_t* d_rowbody = d_rowseg + n;
    int32_t* d_slip = d_rowbody + n;
    VV_CUDA(cudaMemcpyAsync(d_col0, col0.data(), nb * 4, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(d_bfirst, bfirst.data(), nb * 4, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(d_bcount, bcount.data(), nb * 4, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(d_rowseg, row_seg.data(), n * 4, cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(d_rowbody, row_body.data(), n * 4, cudaMemcpyHostToDevice, s));
    if (nsl) VV_CUDA(cudaMemcpyAsync(d_slip, slip_rows.data(), nsl * 4, cudaMemcpyHostToDevice, s));
    c.slae_bodies.reserve((nb * sizeof(BodyDev) + sizeof(double) - 1) / sizeof(double));
    BodyDev* dbd = reinterpret_cast<BodyDev*>(c.slae_bodies.p);
    VV_CUDA(cudaMemcpyAsync(dbd, bd.data(), nb * sizeof(BodyDev), cudaMemcpyHostToDevice, s));

    c.A.reserve(n * n);
    c.B.reserve(n);
    c.X.reserve(n);
    if (!rhs_only) VV_CUDA(cudaMemsetAsync(c.A.p, 0, n * n * sizeof(double), s));
    VV_CUDA(cudaMemsetAsync(c.B.p, 0, n * sizeof(double), s));
    FillArgs fa{};
    fa.n = n; fa.A = c.A.p; fa.B = c.B.p;
    fa.S = SegDev{c.s_cx.p, c.s_cy.p, c.s_rx.p, c.s_ry.p, c.s_dlx.p, c.s_dly.p};
    fa.slip_rows = d_slip; fa.nslip = (int64_t)nsl; fa.row_seg = d_rowseg; fa.row_body = d_rowbody;
    fa.col_seg0 = d_col0; fa.body_first = d_bfirst; fa.body_count = d_bcount; fa.nbodies = nb;
    fa.geom = c.nd_geom.p; fa.ch1 = c.nd_ch1.p; fa.dfs = c.nd_dfs.p;
    fa.lvf = c.lf_vf.p; fa.lvl = c.lf_vl.p; fa.near_off = c.near_off.p; fa.near_run = c.near_run.p;
    fa.far_off = c.far_off.p; fa.far_node = c.far_node.p; fa.cm = c.nd_cm.p;
    fa.x = c.x.p; fa.y = c.y.p; fa.g = c.g.p; fa.ie = c.ie.p;
    fa.ns = c.ns; fa.kx = c.k_x.p; fa.ky = c.k_y.p; fa.kg = c.k_g.p; fa.sink_e2 = c.dt * C_1_PI;
    fa.inf_vx = c.inf_vx; fa.inf_vy = c.inf_vy;
    fa.rhs_only = rhs_only;
    if (nsl) {
        if (c.precision == VVGPU_FP32) k_slip_rows<true><<<(unsigned)nsl, 256, 0, s>>>(fa);
        else k_slip_rows<false><<<(unsigned)nsl, 256, 0, s>>>(fa);
        VV_LAUNCH_CHECK();
    }
    k_body_rows<<<nb, 256, 0, s>>>(n, c.A.p, c.B.p, dbd, nb, d_col0, d_bcount, c.s_cy.p, c.s_cx.p, d_bfirst, c.dt,
                                   gs, c.inf_g, c.grav_x, c.grav_y, inf_body, rhs_only);
    VV_LAUNCH_CHECK();

    // reuse the cached inverse while the matrix bytes are unchanged
    bool same = rhs_only;
    int32_t* singular = (int32_t*)(c.counters.p + 6);
    if (!rhs_only && c.lu_valid && c.lu_precision == c.precision && c.neq_cached == n) {
        int32_t* diff = (int32_t*)(c.counters.p + 7);
        VV_CUDA(cudaMemsetAsync(diff, 0, 4, s));
        k_differs<<<grid_for(n * n, 256), 256, 0, s>>>(n * n, (const unsigned long long*)c.A.p,
                                                      (const unsigned long long*)c.Acache.p, diff);
        VV_LAUNCH_CHECK();
        same = read_i32(c, diff) == 0;
    }
    if (!same) {
        c.Acache.reserve(n * n);
        VV_CUDA(cudaMemcpyAsync(c.Acache.p, c.A.p, n * n * 8, cudaMemcpyDeviceToDevice, s));
        VV_CUDA(cudaMemsetAsync(singular, 0, 4, s));
        if (c.precision == VVGPU_FP32) {
            c.inv32.reserve(n * n);
            k_to_f32<<<grid_for(n * n, 256), 256, 0, s>>>(n * n, c.A.p, c.inv32.p);
            VV_LAUNCH_CHECK();
            invert<float>(c, c.inv32.p, n, singular);
        } else {
            c.inv.reserve(n * n);
            VV_CUDA(cudaMemcpyAsync(c.inv.p, c.A.p, n * n * 8, cudaMemcpyDeviceToDevice, s));
            invert<double>(c, c.inv.p, n, singular);
        }
        if (read_i32(c, singular)) {
            c.lu_valid = false;
            throw ApiError{VVGPU_ERR_SINGULAR, "singular SLAE"};
        }
        c.lu_valid = true;
        c.lu_precision = c.precision;
        c.neq_cached = n;
    }
    c.slae_sig = std::move(sig);
    // x = inv b, then FP64 iterative refinement
    c.slae_r.reserve(n);
    c.slae_sq.reserve(2 * (size_t)n);
    DArr<double>& r = c.slae_r;
    DArr<double>& sq = c.slae_sq;
    c.sum_part.reserve(2 * SUM_BLOCKS);
    double* acc = (double*)(c.counters.p + 8);
    const unsigned gg = grid_for(n, 8);
    c.slae_vs.reserve(n + 1);
    auto apply_inv = [&](const double* v, double* y, bool add) {
        if (c.lu_precision == VVGPU_FP32) {
            k_split_vec<<<grid_for(n, 256), 256, 0, s>>>(n, v, c.slae_vs.p);
            VV_LAUNCH_CHECK();
            k_gemv32<<<gg, 256, 0, s>>>(n, c.inv32.p, c.slae_vs.p, y, add);
        } else {
            k_gemv<double><<<gg, 256, 0, s>>>(n, c.inv.p, v, y, add);
        }
        VV_LAUNCH_CHECK();
    };
    apply_inv(c.B.p, c.X.p, false);
    // refine until |r|^2 <= 1e-26 |b|^2, or until a correction stops paying (the residual
    // falls by less than 4x: it has reached the rounding floor of its own FP64 evaluation)
    double r2_prev = INFINITY;
    for (int it = 0; it < 12; it++) {
        k_residual<<<gg, 256, 0, s>>>(n, c.A.p, c.X.p, c.B.p, r.p, sq.p);
        VV_LAUNCH_CHECK();
        for (int k = 0; k < 2; k++) {
            k_sum_stage1<<<SUM_BLOCKS, 256, 0, s>>>(n, sq.p + k * n, c.sum_part.p + k * SUM_BLOCKS);
            VV_LAUNCH_CHECK();
            k_sum_stage2<<<1, 256, 0, s>>>(SUM_BLOCKS, c.sum_part.p + k * SUM_BLOCKS, acc + k);
            VV_LAUNCH_CHECK();
        }
        double hl[2];
        double* h = pinned_at(c, 160, hl);
        VV_CUDA(cudaMemcpyAsync(h, acc, 16, cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
        if (!(h[0] > 1e-26 * h[1])) break;
        if (!(h[0] < 0.25 * r2_prev)) break;
        r2_prev = h[0];
        apply_inv(r.p, c.X.p, true);
    }
    int64_t maxcnt = 0;
    for (auto& b : c.bodies) maxcnt = std::max<int64_t>(maxcnt, b.count);
    k_scatter_solution<<<grid_for(maxcnt, 256), 256, 0, s>>>(nb, d_col0, d_bfirst, d_bcount, c.X.p, c.s_g.p);
    VV_LAUNCH_CHECK();
    std::vector<double> hx(n);
    VV_CUDA(cudaMemcpyAsync(hx.data(), c.X.p, n * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    for (int bi = 0; bi < nb; bi++) {
        const double* u = hx.data() + col0[bi] + c.bodies[bi].count;
        vvgpu_body_params& p = c.bodies[bi].p;
        p.speed_slae_x = u[0]; p.speed_slae_y = u[1]; p.speed_slae_o = u[2];
        if (out) {
            vvgpu_body_out& o = out[bi];
            o.speed_slae_x = u[0]; o.speed_slae_y = u[1]; o.speed_slae_o = u[2];
            o.force_hydro_x = u[3]; o.force_hydro_y = u[4]; o.force_hydro_o = u[5];
            o.force_holder_x = u[6]; o.force_holder_y = u[7]; o.force_holder_o = u[8];
        }
    }
}

}  // namespace vvgpu
