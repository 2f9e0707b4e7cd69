// MFlowmove::move_and_clean (libvvhd/src/MFlowmove.cpp:11-215) on the GPU, for rigid bodies
// at rest (the configurations of this path): with no spring there is no collision, so the
// step is current_dt = dt, and the bodies do not move (their SLAE speed is zero up to the
// solver's round-off, below 1e-10, which is not applied).  What remains:
//   r += v dt for every vortex (:104);
//   erase |g| < 1e-10 (:110-114), then, with `remove`, erase the vortices that a body's
//   TBody::isPointInvalid reports (:121-143, TBody.cpp:217-280) with the dead-vortex
//   bookkeeping on the body (fdt_dead, g_dead) and on the nearest segment (gsum);
//   v = 0 (:192-197);
//   dead-segment bookkeeping for |g| < 1e-10 or slip segments (:199-214).
// Erasing keeps the list order (a stream compaction).  The FP64 bookkeeping sums are
// order dependent, so one thread applies them in the reference's order (the vortices in
// list order, then each body's segments); everything else is one thread per vortex.
#include <cfloat>

#include "body_test.cuh"
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

// Move, then classify: keep (1), erase as small (0, seg = -1), erase inside body b at
// segment seg (0, seg >= 0).
__global__ void k_move_classify(int64_t n, double dt, int remove, double* x, double* y, const double* __restrict__ vx,
                                const double* __restrict__ vy, const double* __restrict__ g, const BodyTest* bodies,
                                int nb, const double* __restrict__ cx, const double* __restrict__ cy,
                                const double* __restrict__ rx, const double* __restrict__ ry, int32_t* keep,
                                int32_t* dead, int2* dead_at) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = dadd(x[i], dmul(vx[i], dt)), py = dadd(y[i], dmul(vy[i], dt));
    x[i] = px;
    y[i] = py;
    int k = 1, d = 0;
    int2 at = make_int2(-1, -1);
    if (fabs(g[i]) < REMOVE_EPS) {
        k = 0;
    } else if (remove) {
        for (int b = 0; b < nb; b++) {
            const int64_t s = point_invalid(bodies[b], cx, cy, rx, ry, px, py);
            if (s >= 0) { k = 0; d = 1; at = make_int2(b, (int32_t)s); break; }
        }
    }
    keep[i] = k;
    dead[i] = d;
    dead_at[i] = at;
}

// Kept vortices to their new slots (staging), velocities reset.
__global__ void k_move_compact(int64_t n, const int32_t* __restrict__ keep, const int32_t* __restrict__ pos,
                               const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ g, const double* __restrict__ ie,
                               const int64_t* __restrict__ orig, double* tmp, int64_t* otmp, int64_t cap) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    const int64_t p = pos[i];
    tmp[p] = x[i];
    tmp[cap + p] = y[i];
    tmp[2 * cap + p] = g[i];
    tmp[3 * cap + p] = ie[i];
    otmp[p] = orig[i];
}

__global__ void k_move_store(int64_t n, const double* __restrict__ tmp, const int64_t* __restrict__ otmp, int64_t cap,
                             double* x, double* y, double* g, double* ie, double* vx, double* vy, int64_t* orig) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = tmp[i];
    y[i] = tmp[cap + i];
    g[i] = tmp[2 * cap + i];
    ie[i] = tmp[3 * cap + i];
    orig[i] = otmp[i];
    vx[i] = 0.;
    vy[i] = 0.;
}

__global__ void k_dead_list(int64_t n, const int32_t* __restrict__ dead, const int32_t* __restrict__ pos,
                            int32_t* list) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && dead[i]) list[pos[i]] = (int32_t)i;
}

// The order-dependent FP64 bookkeeping, one thread.  acc[4 b + 0..3] = fdt_dead x, y, o,
// g_dead of body b (in: current values, out: updated).
__global__ void k_move_bookkeep(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                const int2* __restrict__ dead_at, const double* __restrict__ x,
                                const double* __restrict__ y, const double* __restrict__ g,
                                const BodyTest* bodies, int nb, const double* __restrict__ cx,
                                const double* __restrict__ cy, const double* __restrict__ sg,
                                const uint32_t* __restrict__ slip, double* gsum, double* acc) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int32_t nd = *count;
    for (int32_t k = 0; k < nd; k++) {
        const int32_t i = list[k];
        const int2 at = dead_at[i];
        const BodyTest& b = bodies[at.x];
        const double gi = g[i], px = x[i], py = y[i];
        double* a = acc + 4 * at.x;
        a[0] = dadd(a[0], dmul(-py, gi));
        a[1] = dadd(a[1], dmul(px, gi));
        a[2] = dadd(a[2], dmul(dabs2(dsub(px, b.axx), dsub(py, b.axy)), gi));
        gsum[at.y] = dsub(gsum[at.y], gi);
        a[3] = dadd(a[3], gi);
    }
    for (int bi = 0; bi < nb; bi++) {
        const BodyTest& b = bodies[bi];
        double* a = acc + 4 * bi;
        for (int64_t q = 0; q < b.count; q++) {
            const int64_t s = b.first + q;
            const double gs = sg[s];
            if (fabs(gs) < REMOVE_EPS || slip[s]) {
                a[0] = dadd(a[0], dmul(-cy[s], gs));
                a[1] = dadd(a[1], dmul(cx[s], gs));
                a[2] = dadd(a[2], dmul(dabs2(dsub(cx[s], b.axx), dsub(cy[s], b.axy)), gs));
                gsum[s] = dsub(gsum[s], gs);
                a[3] = dadd(a[3], gs);
            }
        }
    }
}

}  // namespace

void move_and_clean(Ctx& c, int remove, int64_t* cleaned) {
    check_input(c);
    for (auto& b : c.bodies) {
        const vvgpu_body_params& p = b.p;
        auto rigid = [](double k) { return !(k >= 0 && std::isfinite(k)); };
        if (!rigid(p.kspring_x) || !rigid(p.kspring_y) || !rigid(p.kspring_o))
            throw ApiError{VVGPU_ERR_UNSUPPORTED, "spring-mounted bodies (collisions) are not supported"};
        // at rest: no prescribed motion, and a SLAE speed that is zero up to the solver's
        // round-off (the same test as the convective pass); such a body is not moved
        if (p.speed_x != 0 || p.speed_y != 0 || p.speed_o != 0 ||
            !(std::fabs(p.speed_slae_x) + std::fabs(p.speed_slae_y) + std::fabs(p.speed_slae_o) < 1E-10))
            throw ApiError{VVGPU_ERR_UNSUPPORTED, "moving bodies are not supported"};
    }
    upload_segments(c);
    cudaStream_t s = c.st();
    const int64_t n = c.n;
    const int nb = (int)c.bodies.size();
    // per-body inside-test geometry (TBody::doFillProperties, TBody.cpp:327-342)
    std::vector<BodyTest> hb(nb + 1);
    std::vector<double> hacc(4 * (size_t)nb + 4, 0.);
    for (int bi = 0; bi < nb; bi++) {
        const BodyHost& b = c.bodies[bi];
        const BodyTest mb = body_test_of(c, b);
        hb[bi] = mb;
        hacc[4 * bi + 0] = b.p.fdt_dead_x;
        hacc[4 * bi + 1] = b.p.fdt_dead_y;
        hacc[4 * bi + 2] = b.p.fdt_dead_o;
        hacc[4 * bi + 3] = b.p.g_dead;
    }
    c.mv_bodies.reserve(hb.size() * sizeof(BodyTest) / sizeof(double) + 1);
    c.mv_acc.reserve(hacc.size());
    VV_CUDA(cudaMemcpyAsync(c.mv_bodies.p, hb.data(), hb.size() * sizeof(BodyTest), cudaMemcpyHostToDevice, s));
    VV_CUDA(cudaMemcpyAsync(c.mv_acc.p, hacc.data(), hacc.size() * 8, cudaMemcpyHostToDevice, s));
    const BodyTest* dbodies = reinterpret_cast<const BodyTest*>(c.mv_bodies.p);
    int32_t new_n = 0, ndead = 0;
    if (n > 0) {
        c.flags.reserve(n + 1);
        c.scan.reserve(n + 2);
        c.mv_dead.reserve(n + 1);
        c.mv_dpos.reserve(n + 2);
        c.mv_list.reserve(n + 1);
        c.mv_at.reserve(n + 1);
        k_move_classify<<<grid_for(n, 256), 256, 0, s>>>(n, c.dt, remove, c.x.p, c.y.p, c.vx.p, c.vy.p, c.g.p, dbodies,
                                                         nb, c.s_cx.p, c.s_cy.p, c.s_rx.p, c.s_ry.p, c.flags.p,
                                                         c.mv_dead.p, c.mv_at.p);
        VV_LAUNCH_CHECK();
        exclusive_scan(c, c.flags.p, c.scan.p, n);
        exclusive_scan(c, c.mv_dead.p, c.mv_dpos.p, n);
        k_dead_list<<<grid_for(n, 256), 256, 0, s>>>(n, c.mv_dead.p, c.mv_dpos.p, c.mv_list.p);
        VV_LAUNCH_CHECK();
    }
    if (nb > 0 || n > 0) {
        // with no vortices the dead count reads the zeroed slot of an empty scan
        const int32_t* cnt = n > 0 ? c.mv_dpos.p + n : nullptr;
        if (cnt == nullptr) {
            c.mv_dpos.reserve(2);
            VV_CUDA(cudaMemsetAsync(c.mv_dpos.p, 0, 4, s));
            cnt = c.mv_dpos.p;
        }
        k_move_bookkeep<<<1, 32, 0, s>>>(c.mv_list.p, cnt, c.mv_at.p, c.x.p, c.y.p, c.g.p, dbodies, nb, c.s_cx.p,
                                         c.s_cy.p, c.s_g.p, c.s_slip.p, c.s_gsum.p, c.mv_acc.p);
        VV_LAUNCH_CHECK();
    }
    if (n > 0) {
        new_n = read_i32(c, c.scan.p + n);
        ndead = read_i32(c, c.mv_dpos.p + n);
        c.ptmp.reserve(4 * (size_t)n);
        c.otmp.reserve(n);
        k_move_compact<<<grid_for(n, 256), 256, 0, s>>>(n, c.flags.p, c.scan.p, c.x.p, c.y.p, c.g.p, c.ie.p, c.orig.p,
                                                        c.ptmp.p, c.otmp.p, n);
        VV_LAUNCH_CHECK();
        if (new_n > 0) {
            k_move_store<<<grid_for(new_n, 256), 256, 0, s>>>(new_n, c.ptmp.p, c.otmp.p, n, c.x.p, c.y.p, c.g.p, c.ie.p,
                                                              c.vx.p, c.vy.p, c.orig.p);
            VV_LAUNCH_CHECK();
        }
    }
    VV_CUDA(cudaMemcpyAsync(hacc.data(), c.mv_acc.p, hacc.size() * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    for (int bi = 0; bi < nb; bi++) {
        vvgpu_body_params& p = c.bodies[bi].p;
        p.fdt_dead_x = hacc[4 * bi + 0];
        p.fdt_dead_y = hacc[4 * bi + 1];
        p.fdt_dead_o = hacc[4 * bi + 2];
        p.g_dead = hacc[4 * bi + 3];
    }
    c.n = new_n;
    if (cleaned) *cleaned = ndead;
}

}  // namespace vvgpu
