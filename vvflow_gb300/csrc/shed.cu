// MFlowmove::vortex_shed (libvvhd/src/MFlowmove.cpp:217-235): every segment adds its
// circulation to gsum; every non-slip segment with |g| >= 1e-10 appends one vortex at
// corner + rotl(dl) * 1e-4 with that circulation, in segment order.
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

__global__ void k_shed_flags(int64_t m, const double* __restrict__ sg, const uint32_t* __restrict__ slip,
                             int32_t* flags, double* gsum) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    double g = sg[s];
    gsum[s] += g;
    flags[s] = (fabs(g) >= REMOVE_EPS && !slip[s]) ? 1 : 0;
}

__global__ void k_shed_append(int64_t m, int64_t n0, const int32_t* __restrict__ flags,
                              const int32_t* __restrict__ pos, const double* __restrict__ sg,
                              const double* __restrict__ cx, const double* __restrict__ cy,
                              const double* __restrict__ dlx, const double* __restrict__ dly, double* x, double* y,
                              double* g, double* ie, double* vx, double* vy, int64_t* orig) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m || !flags[s]) return;
    int64_t i = n0 + pos[s];
    x[i] = dadd(cx[s], dmul(-dly[s], 1e-4));  // corner + rotl(dl) * 1e-4, two roundings
    y[i] = dadd(cy[s], dmul(dlx[s], 1e-4));
    g[i] = sg[s];
    ie[i] = 0.;
    vx[i] = 0.;
    vy[i] = 0.;
    orig[i] = i;
}

}  // namespace

void vortex_shed(Ctx& c) {
    const int64_t m = c.m;
    if (m == 0) return;
    upload_segments(c);
    cudaStream_t s = c.st();
    c.flags.reserve(m + 1);
    c.scan.reserve(m + 2);
    k_shed_flags<<<grid_for(m, 256), 256, 0, s>>>(m, c.s_g.p, c.s_slip.p, c.flags.p, c.s_gsum.p);
    VV_LAUNCH_CHECK();
    exclusive_scan(c, c.flags.p, c.scan.p, m);
    int32_t add = read_i32(c, c.scan.p + m);
    if (add == 0) return;
    ensure_vortex_capacity(c, c.n + add, true);
    k_shed_append<<<grid_for(m, 256), 256, 0, s>>>(m, c.n, c.flags.p, c.scan.p, c.s_g.p, c.s_cx.p, c.s_cy.p,
                                                   c.s_dlx.p, c.s_dly.p, c.x.p, c.y.p, c.g.p, c.ie.p, c.vx.p,
                                                   c.vy.p, c.orig.p);
    VV_LAUNCH_CHECK();
    VV_CUDA(cudaStreamSynchronize(s));
    c.n += add;
}

}  // namespace vvgpu
