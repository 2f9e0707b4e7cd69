// Grid fields of libvvhd on the GPU: XVelocity (libvvhd/src/XVelocity.cpp:24-73),
// XStreamfunction (XStreamfunction.cpp:47-212) and XVorticity (XVorticity.cpp:26-94).
//
// The grid is xres x yres points p = (xmin, ymin) + dxdy (xi, yj) with xmin, ymin and dxdy
// rounded to float, as XField stores them (libvvhd/headers/XField.hpp:47); the result is
// float, row-major by yj as XField::map.  Each field builds its own tree over the space
// (the reference builds it on a private copy of Space), so the context's vortex list,
// epsilon and attached-segment sums are saved before and put back after; no tree may be
// built on entry and none is left.
//
// Work per grid point, all FP64 (the outputs are float, the decisions are bit-exact):
//   velocity        MConvectiveFast::velocity(p) (the point kernel of the convective pass);
//   streamfunction  sum over all segments and the far nodes' +/- centroids of -g log(r^2 + rd2),
//                   over the near leaves' vortices of -g log(r^2 + eps^2), sinks' q atan2;
//   vorticity       sum over the near leaves' vortices of g a exp(-a r^2) (cut at -6) plus
//                   the erf layer term of the nearest segment centre.
// Per-vortex smoothing comes from MEpsilonFast::eps2h (MEpsilonFast.cpp:66-92): the squared
// distance to the second nearest vortex over the vortex's near leaves (coincident points
// skipped, any circulation), one thread per vortex.
#include <cfloat>
#include <cmath>

#include "body_test.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr double C_1_4PI = 1. / (4. * C_PI);

struct Grid {
    double x0, y0, d;  // float-rounded origin and spacing
    int32_t xres, yres;
};

struct TreeView {
    const double4* geom;
    const int32_t* ch1;
    const int32_t* dfs;
    const int32_t* near_off;
    const int2* near_run;
    const int32_t* lvf;
    const int32_t* lvl;
    const int32_t* lsf;
    const int32_t* lsl;
    const int32_t* seg_order;
    const double* cm;
    double fc;
    int64_t nnodes;
};

TreeView tree_view(Ctx& c) {
    TreeView t;
    t.geom = c.nd_geom.p;
    t.ch1 = c.nd_ch1.p;
    t.dfs = c.nd_dfs.p;
    t.near_off = c.near_off.p;
    t.near_run = c.near_run.p;
    t.lvf = c.lf_vf.p;
    t.lvl = c.lf_vl.p;
    t.lsf = c.lf_sf.p;
    t.lsl = c.lf_sl.p;
    t.seg_order = c.seg_order.p;
    t.cm = c.nd_cm.p;
    t.fc = c.far_criteria;
    t.nnodes = c.nnodes;
    return t;
}

// XVelocity.cpp:59 / XStreamfunction.cpp:98 / XVorticity.cpp:70:
// p = TVec(xmin, ymin) + dxdy * TVec(xi, yj).
__device__ __forceinline__ void grid_point(const Grid& g, int64_t q, double& px, double& py) {
    const int32_t xi = (int32_t)(q % g.xres), yj = (int32_t)(q / g.xres);
    px = dadd(g.x0, dmul((double)xi, g.d));
    py = dadd(g.y0, dmul((double)yj, g.d));
}

// stree::findNode (TSortedTree.cpp:284-303): node id of the leaf that holds p.
__device__ __forceinline__ int32_t find_leaf_node(const TreeView& t, double px, double py) {
    int32_t k = 0;
    for (int it = 0; it <= MAX_DEPTH && t.ch1[k] >= 0; it++) {
        const double4 gm = t.geom[k];
        if (gm.z < gm.w) k = (px < gm.x) ? t.ch1[k] : t.ch1[k] + 1;
        else k = (py < gm.y) ? t.ch1[k] : t.ch1[k] + 1;
    }
    return k;
}

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }  // std::min

__global__ void k_grid(Grid g, int64_t np, double* px, double* py) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    grid_point(g, q, px[q], py[q]);
}

__global__ void k_vel_store(int64_t np, const double* __restrict__ v, double ref, float* out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    out[q] = (float)dsub(v[q], ref);
}

// Per vortex: eps2h, then the field's smoothing.  kind 0 (stream function):
// s0 = eps_mult^2 max(eps2h / 4, (0.2 dl)^2) (XStreamfunction.cpp:87-88); kind 1 (vorticity):
// s0 = 1 / (eps_mult^2 max(eps2h, (0.6 dl)^2)), s1 = s0 g (XVorticity.cpp:55-57).
__global__ void k_smoothing(int64_t n, TreeView t, const int32_t* __restrict__ leaf_of,
                            const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ g, int kind, double eps_mult, double dl, double* s0,
                            double* s1) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t L = leaf_of[i];
    const double px = x[i], py = y[i];
    double res1 = INFINITY, res2 = INFINITY;
    for (int32_t r = t.near_off[L]; r < t.near_off[L + 1]; r++) {
        const int2 run = t.near_run[r];
        for (int32_t j = t.lvf[run.x]; j < t.lvl[run.y - 1]; j++) {
            const double d = dabs2(dsub(px, x[j]), dsub(py, y[j]));
            if (!d) continue;
            else if (d < res1) { res2 = res1; res1 = d; }
            else if (d < res2) res2 = d;
        }
    }
    const double e2h = isfinite(res2) ? res2 : (isfinite(res1) ? res1 : -DBL_MAX);
    const double em2 = dmul(eps_mult, eps_mult);
    if (kind == 0) {
        const double fl = dmul(0.2, dl);
        s0[i] = dmul(em2, smax(dmul(e2h, 0.25), dmul(fl, fl)));
    } else {
        const double fl = dmul(0.6, dl);
        const double a = ddiv(1., dmul(em2, smax(e2h, dmul(fl, fl))));
        s0[i] = a;
        s1[i] = dmul(a, g[i]);
    }
}

// _4pi_psi_g (XStreamfunction.cpp:27-31): -g log(|dr|^2 + rd2).
__device__ __forceinline__ double psi_g(double dx, double dy, double rd2, double g) {
    return dmul(-g, log(dadd(dabs2(dx, dy), rd2)));
}

struct PsiArgs {
    Grid grid;
    TreeView t;
    int64_t m, ns;
    const double *srx, *sry, *sg;   // segment centres and circulations
    const double *kx, *ky, *kg;     // sinks
    const double *x, *y, *g, *e2;   // vortices and their eps^2
    double rd2, vfx, vfy;           // (0.2 dl)^2, V_inf - V_frame
};

// XStreamfunction::streamfunction(node, p, gap) (XStreamfunction.cpp:160-212), in its order:
// segments, sinks, far nodes (the reference's depth-first walk), near vortices.
__global__ void k_psi(int64_t np, PsiArgs a, float* out, double* gap) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    double px, py;
    grid_point(a.grid, q, px, py);
    double t4 = 0, t2 = 0, pgap = 0;
    for (int64_t s = 0; s < a.m; s++) t4 = dadd(t4, psi_g(dsub(px, a.srx[s]), dsub(py, a.sry[s]), a.rd2, a.sg[s]));
    for (int64_t s = 0; s < a.ns; s++) {
        t2 = dadd(t2, dmul(a.kg[s], atan2(dsub(py, a.ky[s]), dsub(px, a.kx[s]))));
        if (px < a.kx[s] && a.kx[s] <= dadd(px, a.grid.d) && py < a.ky[s] && a.ky[s] <= dadd(py, a.grid.d))
            pgap = dadd(pgap, a.kg[s]);
    }
    const TreeView& t = a.t;
    const int32_t k = find_leaf_node(t, px, py);
    {
        const double4 me = t.geom[k];
        int32_t stack[MAX_DEPTH + 2];
        int sp = 0;
        stack[sp++] = 0;
        int64_t guard = 0;
        while (sp && ++guard <= t.nnodes) {
            const int32_t u = stack[--sp];
            const double4 tg = t.geom[u];
            const double ddx = dsub(tg.x, me.x), ddy = dsub(tg.y, me.y);
            const double hp = dadd(dadd(dadd(tg.z, tg.w), me.z), me.w);
            if (dabs2(ddx, ddy) > dmul(dmul(t.fc, hp), hp)) {
                const double* c = t.cm + 6 * (size_t)u;
                t4 = dadd(t4, psi_g(dsub(px, c[0]), dsub(py, c[1]), a.rd2, c[2]));
                t4 = dadd(t4, psi_g(dsub(px, c[3]), dsub(py, c[4]), a.rd2, c[5]));
                continue;
            }
            const int32_t c1 = t.ch1[u];
            if (c1 >= 0 && sp + 2 <= MAX_DEPTH + 2) {
                stack[sp++] = c1 + 1;
                stack[sp++] = c1;
            }
        }
    }
    const int32_t L = t.dfs[k];
    for (int32_t r = t.near_off[L]; r < t.near_off[L + 1]; r++) {
        const int2 run = t.near_run[r];
        for (int32_t j = t.lvf[run.x]; j < t.lvl[run.y - 1]; j++)
            t4 = dadd(t4, psi_g(dsub(px, a.x[j]), dsub(py, a.y[j]), a.e2[j], a.g[j]));
    }
    // p * rotl(V) = p.x (-V.y) + p.y V.x
    const double res = dadd(dadd(dmul(t4, C_1_4PI), dmul(t2, C_1_2PI)), dadd(dmul(px, -a.vfy), dmul(py, a.vfx)));
    out[q] = (float)res;
    gap[q] = pgap;
}

struct VortArgs {
    Grid grid;
    TreeView t;
    const BodyTest* bodies;
    int nb;
    const double *cx, *cy, *srx, *sry;  // corners and segment centres
    const double *x, *y, *a, *ag;       // vortices: a = eps^-2, ag = a g
    double e2;                          // (dl eps_mult)^2
};

// XVorticity::vorticity (XVorticity.cpp:78-94) behind Space::point_is_in_body.
__global__ void k_vorticity(int64_t np, VortArgs v, float* out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    double px, py;
    grid_point(v.grid, q, px, py);
    for (int b = 0; b < v.nb; b++)
        if (point_invalid(v.bodies[b], v.cx, v.cy, v.srx, v.sry, px, py) >= 0) {
            out[q] = 0.f;
            return;
        }
    const TreeView& t = v.t;
    const int32_t L = t.dfs[find_leaf_node(t, px, py)];
    double res = 0;
    for (int32_t r = t.near_off[L]; r < t.near_off[L + 1]; r++) {
        const int2 run = t.near_run[r];
        for (int32_t j = t.lvf[run.x]; j < t.lvl[run.y - 1]; j++) {
            const double exparg = dmul(-dabs2(dsub(px, v.x[j]), dsub(py, v.y[j])), v.a[j]);
            res = dadd(res, (exparg > -6) ? dmul(v.ag[j], exp(exparg)) : 0.);
        }
    }
    res = dmul(res, C_1_PI);
    // MEpsilonFast::h2 (MEpsilonFast.cpp:94-107): nearest segment centre of the near leaves
    double h2 = INFINITY;
    for (int32_t r = t.near_off[L]; r < t.near_off[L + 1]; r++) {
        const int2 run = t.near_run[r];
        for (int32_t k = t.lsf[run.x]; k < t.lsl[run.y - 1]; k++) {
            const int32_t s = t.seg_order[k];
            h2 = smin(h2, dabs2(dsub(px, v.srx[s]), dsub(py, v.sry[s])));
        }
    }
    const double erfarg = ddiv(h2, v.e2);
    res = dadd(res, (erfarg < 3) ? dmul(0.5, dsub(1., erf(erfarg))) : 0.);
    out[q] = (float)res;
}

// Space::average_segment_length (TSpace.hpp:119-129): of the first body.
double average_segment_length(const Ctx& c) {
    if (c.bodies.empty()) return 0;
    const BodyHost& b = c.bodies[0];
    if (b.count <= 1) return 0;
    return b.slen / (double)(b.count - 1);
}

// XField::XField (XField.cpp:8-24) on the float members.
Grid make_grid(double xmin, double ymin, double dxdy, int32_t xres, int32_t yres) {
    const float fx = (float)xmin, fy = (float)ymin, fd = (float)dxdy;
    if (xres <= 1) throw ApiError{VVGPU_ERR_ARG, "XField(): xres must be > 1"};
    if (yres <= 1) throw ApiError{VVGPU_ERR_ARG, "XField(): yres must be > 1"};
    if (!std::isfinite(fd)) throw ApiError{VVGPU_ERR_ARG, "XField(): dxdy must be finite"};
    if (fd <= 0) throw ApiError{VVGPU_ERR_ARG, "XField(): dxdy must be positive"};
    return Grid{(double)fx, (double)fy, (double)fd, xres, yres};
}

void frame_speed(const Ctx& c, char ref_frame, double& vx, double& vy) {
    switch (ref_frame) {
    case 'o': vx = 0; vy = 0; return;
    case 'f': vx = c.inf_vx; vy = c.inf_vy; return;
    case 'b':
        if (c.bodies.empty()) throw ApiError{VVGPU_ERR_ARG, "ref_frame 'b' needs a body"};
        vx = c.bodies[0].p.speed_slae_x;
        vy = c.bodies[0].p.speed_slae_y;
        return;
    default: throw ApiError{VVGPU_ERR_ARG, "bad ref_frame"};
    }
}

// The private copy of the reference: what the field's tree build, epsilon and shed change.
struct Saved {
    int64_t n = 0;
    DArr<double> d;      // x, y, g, ie, vx, vy (n each), then gsum (m)
    DArr<int64_t> orig;
};

void save_state(Ctx& c, Saved& sv) {
    cudaStream_t s = c.st();
    const int64_t n = c.n, m = c.m;
    sv.n = n;
    sv.d.reserve(6 * (size_t)n + (size_t)m + 1);
    sv.orig.reserve((size_t)n + 1);
    double* src[6] = {c.x.p, c.y.p, c.g.p, c.ie.p, c.vx.p, c.vy.p};
    if (n > 0) {
        for (int k = 0; k < 6; k++)
            VV_CUDA(cudaMemcpyAsync(sv.d.p + k * n, src[k], n * 8, cudaMemcpyDeviceToDevice, s));
        VV_CUDA(cudaMemcpyAsync(sv.orig.p, c.orig.p, n * 8, cudaMemcpyDeviceToDevice, s));
    }
    if (m > 0) VV_CUDA(cudaMemcpyAsync(sv.d.p + 6 * n, c.s_gsum.p, m * 8, cudaMemcpyDeviceToDevice, s));
}

void restore_state(Ctx& c, Saved& sv) {
    cudaStream_t s = c.st();
    const int64_t n = sv.n, m = c.m;
    c.built = false;
    c.lists_full = false;
    c.far_kept = false;
    double* dst[6] = {c.x.p, c.y.p, c.g.p, c.ie.p, c.vx.p, c.vy.p};
    if (n > 0) {
        for (int k = 0; k < 6; k++)
            VV_CUDA(cudaMemcpyAsync(dst[k], sv.d.p + k * n, n * 8, cudaMemcpyDeviceToDevice, s));
        VV_CUDA(cudaMemcpyAsync(c.orig.p, sv.orig.p, n * 8, cudaMemcpyDeviceToDevice, s));
    }
    if (m > 0) VV_CUDA(cudaMemcpyAsync(c.s_gsum.p, sv.d.p + 6 * n, m * 8, cudaMemcpyDeviceToDevice, s));
    c.n = n;
    VV_CUDA(cudaStreamSynchronize(s));
}

// Runs body() on the private copy, then puts the context back even when body() throws.
template <class F>
void on_private_copy(Ctx& c, F&& body) {
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "grid fields build their own tree: destroy the tree first"};
    check_bodies_at_rest(c);
    upload_segments(c);
    Saved sv;
    save_state(c, sv);
    try {
        body();
    } catch (...) {
        restore_state(c, sv);
        throw;
    }
    restore_state(c, sv);
}

}  // namespace

void field_velocity(Ctx& c, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres, char mode,
                    char ref_frame, float* out) {
    const Grid grid = make_grid(xmin, ymin, dxdy, xres, yres);
    double rfx, rfy;
    frame_speed(c, ref_frame, rfx, rfy);
    if (mode != 'x' && mode != 'y') throw ApiError{VVGPU_ERR_ARG, "bad mode"};
    on_private_copy(c, [&] {
        const double dl = average_segment_length(c);
        tree_build(c, 8, dl * 20, 0.1);
        ensure_full_lists(c);
        int64_t merged = 0;
        eps_pass(c, 0, &merged);
        const int64_t np = (int64_t)xres * yres;
        cudaStream_t s = c.st();
        DArr<double> buf;
        buf.reserve(4 * (size_t)np);
        DArr<float> fo;
        fo.reserve((size_t)np);
        k_grid<<<grid_for(np, 256), 256, 0, s>>>(grid, np, buf.p, buf.p + np);
        VV_LAUNCH_CHECK();
        velocity_points_on_device(c, np, buf.p, buf.p + np, buf.p + 2 * np, buf.p + 3 * np);
        k_vel_store<<<grid_for(np, 256), 256, 0, s>>>(np, buf.p + (mode == 'x' ? 2 : 3) * np,
                                                      mode == 'x' ? rfx : rfy, fo.p);
        VV_LAUNCH_CHECK();
        VV_CUDA(cudaMemcpyAsync(out, fo.p, np * sizeof(float), cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
    });
}

void field_streamfunction(Ctx& c, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                          double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                          uint16_t* gap_yj, float* gap, int64_t* ngaps) {
    const Grid grid = make_grid(xmin, ymin, dxdy, xres, yres);
    if (eps_mult <= 0) throw ApiError{VVGPU_ERR_ARG, "XStreamfunction(): eps_mult must be positive"};
    double rfx, rfy;
    frame_speed(c, ref_frame, rfx, rfy);
    on_private_copy(c, [&] {
        const double dl = average_segment_length(c);
        tree_build(c, 8, dl > 0 ? dl * 10 : 0, dl > 0 ? dl * 20 : INFINITY);
        ensure_full_lists(c);
        cudaStream_t s = c.st();
        const int64_t n = c.n, np = (int64_t)xres * yres;
        DArr<double> e2;
        e2.reserve((size_t)n + 1);
        const TreeView t = tree_view(c);
        if (n > 0) {
            k_smoothing<<<grid_for(n, 128), 128, 0, s>>>(n, t, c.leaf_of.p, c.x.p, c.y.p, c.g.p, 0, eps_mult, dl,
                                                         e2.p, nullptr);
            VV_LAUNCH_CHECK();
        }
        PsiArgs a;
        a.grid = grid;
        a.t = t;
        a.m = c.m;
        a.ns = c.ns;
        a.srx = c.s_rx.p; a.sry = c.s_ry.p; a.sg = c.s_g.p;
        a.kx = c.k_x.p; a.ky = c.k_y.p; a.kg = c.k_g.p;
        a.x = c.x.p; a.y = c.y.p; a.g = c.g.p; a.e2 = e2.p;
        const double fl = 0.2 * dl;
        a.rd2 = fl * fl;
        a.vfx = c.inf_vx - rfx;
        a.vfy = c.inf_vy - rfy;
        DArr<float> fo;
        fo.reserve((size_t)np);
        DArr<double> dgap;
        dgap.reserve((size_t)np);
        k_psi<<<grid_for(np, 128), 128, 0, s>>>(np, a, fo.p, dgap.p);
        VV_LAUNCH_CHECK();
        VV_CUDA(cudaMemcpyAsync(out, fo.p, np * sizeof(float), cudaMemcpyDeviceToHost, s));
        std::vector<double> hgap(c.ns > 0 ? (size_t)np : 0);
        if (c.ns > 0) VV_CUDA(cudaMemcpyAsync(hgap.data(), dgap.p, np * 8, cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
        // cells holding a sink, in grid order (the reference collects them per thread)
        int64_t k = 0;
        for (size_t q = 0; q < hgap.size(); q++) {
            if (hgap[q] == 0.) continue;
            if (k < gap_cap) {
                gap_xi[k] = (uint16_t)(q % xres);
                gap_yj[k] = (uint16_t)(q / xres);
                gap[k] = (float)hgap[q];
            }
            k++;
        }
        if (ngaps) *ngaps = k;
    });
}

void field_vorticity(Ctx& c, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres, double eps_mult,
                     float* out) {
    const Grid grid = make_grid(xmin, ymin, dxdy, xres, yres);
    if (eps_mult <= 0) throw ApiError{VVGPU_ERR_ARG, "XVorticity(): eps_mult must be positive"};
    on_private_copy(c, [&] {
        const double dl = average_segment_length(c);
        vortex_shed(c);
        tree_build(c, 8, dl * 20, DBL_MAX);
        ensure_full_lists(c);
        cudaStream_t s = c.st();
        const int64_t n = c.n, np = (int64_t)xres * yres;
        DArr<double> sm;
        sm.reserve(2 * (size_t)n + 1);
        const TreeView t = tree_view(c);
        if (n > 0) {
            k_smoothing<<<grid_for(n, 128), 128, 0, s>>>(n, t, c.leaf_of.p, c.x.p, c.y.p, c.g.p, 1, eps_mult, dl,
                                                         sm.p, sm.p + n);
            VV_LAUNCH_CHECK();
        }
        const int nb = (int)c.bodies.size();
        std::vector<BodyTest> hb(nb + 1);
        for (int b = 0; b < nb; b++) hb[b] = body_test_of(c, c.bodies[b]);
        DArr<double> dbody;
        dbody.reserve(hb.size() * sizeof(BodyTest) / sizeof(double) + 1);
        VV_CUDA(cudaMemcpyAsync(dbody.p, hb.data(), hb.size() * sizeof(BodyTest), cudaMemcpyHostToDevice, s));
        VortArgs v;
        v.grid = grid;
        v.t = t;
        v.bodies = reinterpret_cast<const BodyTest*>(dbody.p);
        v.nb = nb;
        v.cx = c.s_cx.p; v.cy = c.s_cy.p; v.srx = c.s_rx.p; v.sry = c.s_ry.p;
        v.x = c.x.p; v.y = c.y.p; v.a = sm.p; v.ag = sm.p + n;
        const double de = dl * eps_mult;
        v.e2 = de * de;
        DArr<float> fo;
        fo.reserve((size_t)np);
        k_vorticity<<<grid_for(np, 128), 128, 0, s>>>(np, v, fo.p);
        VV_LAUNCH_CHECK();
        VV_CUDA(cudaMemcpyAsync(out, fo.p, np * sizeof(float), cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
    });
}

}  // namespace vvgpu
