// Space::calc_forces (libvvhd/src/TSpace.cpp:94-117) and Space::zero_forces (:122-142) on
// the GPU, in FP64 with the reference's operation order: each body's prefix sum of the
// segments' gsum (TAtt::Cp), the friction integral and the per-segment accumulators are
// sequential sums over the body's segments, so one thread per body walks them in order.
// No heat here: TAtt::hsum = 0 and Space::pr = 0 (the reference's defaults) stay in the
// formulas so that Nu and nusselt come out as the reference's.
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

__global__ void k_calc_forces(int nb, const int64_t* __restrict__ first, const int64_t* __restrict__ count,
                              double dt, double re, double c_nyudt_pi, double c_nyu_pi,
                              const double* __restrict__ rx, const double* __restrict__ ry,
                              const double* __restrict__ dlx, const double* __restrict__ dly,
                              const double* __restrict__ fric, const double* __restrict__ gsum, double* cp,
                              double* fr, double* nu, double* out4) {
    const int b = blockIdx.x;
    if (b >= nb || threadIdx.x != 0) return;
    const double pr = 0., hsum = 0.;
    double tmp_gsum = 0., fx = 0., fy = 0., fo = 0., nus = 0.;
    for (int64_t k = 0; k < count[b]; k++) {
        const int64_t s = first[b] + k;
        const double dlabs = __dsqrt_rn(dabs2(dlx[s], dly[s]));
        tmp_gsum = dadd(tmp_gsum, gsum[s]);
        cp[s] = dadd(cp[s], tmp_gsum);
        fr[s] = dadd(fr[s], dmul(fric[s], c_nyudt_pi));
        nu[s] = dadd(nu[s], dmul(hsum, ddiv(dmul(re, pr), dlabs)));
        const double f = ddiv(dmul(fric[s], c_nyu_pi), dlabs);
        fx = dsub(fx, dmul(dlx[s], f));
        fy = dsub(fy, dmul(dly[s], f));
        fo = dsub(fo, dmul(dadd(dmul(-ry[s], dlx[s]), dmul(rx[s], dly[s])), f));
        nus = dadd(nus, dmul(hsum, dmul(re, pr)));
    }
    out4[4 * b + 0] = fx;
    out4[4 * b + 1] = fy;
    out4[4 * b + 2] = fo;
    out4[4 * b + 3] = ddiv(nus, dt);
}

}  // namespace

void calc_forces(Ctx& c, double* out4) {
    const int nb = (int)c.bodies.size();
    if (nb == 0) return;
    upload_segments(c);
    cudaStream_t s = c.st();
    std::vector<int64_t> fc(2 * (size_t)nb);
    for (int b = 0; b < nb; b++) { fc[b] = c.bodies[b].first; fc[nb + b] = c.bodies[b].count; }
    c.f_fc.reserve(fc.size());
    c.f_out.reserve(4 * (size_t)nb);
    VV_CUDA(cudaMemcpyAsync(c.f_fc.p, fc.data(), fc.size() * 8, cudaMemcpyHostToDevice, s));
    const double c_nyudt_pi = c.dt / (C_PI * c.re);
    const double c_nyu_pi = 1. / (C_PI * c.re);
    k_calc_forces<<<nb, 32, 0, s>>>(nb, c.f_fc.p, c.f_fc.p + nb, c.dt, c.re, c_nyudt_pi, c_nyu_pi, c.s_rx.p, c.s_ry.p,
                                    c.s_dlx.p, c.s_dly.p, c.s_fric.p, c.s_gsum.p, c.s_cp.p, c.s_fr.p, c.s_nu.p,
                                    c.f_out.p);
    VV_LAUNCH_CHECK();
    std::vector<double> h(4 * (size_t)nb);
    VV_CUDA(cudaMemcpyAsync(h.data(), c.f_out.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    for (int b = 0; b < nb; b++) {
        BodyHost& bh = c.bodies[b];
        bh.friction_x = h[4 * b + 0];
        bh.friction_y = h[4 * b + 1];
        bh.friction_o = h[4 * b + 2];
        bh.nusselt = h[4 * b + 3];
        if (out4) for (int k = 0; k < 4; k++) out4[4 * b + k] = h[4 * b + k];
    }
}

void zero_forces(Ctx& c) {
    cudaStream_t s = c.st();
    if (c.m) {
        VV_CUDA(cudaMemsetAsync(c.s_gsum.p, 0, c.m * sizeof(double), s));
        VV_CUDA(cudaMemsetAsync(c.s_fric.p, 0, c.m * sizeof(double), s));
    }
    for (auto& b : c.bodies) {
        b.p.friction_prev_x = b.friction_x;
        b.p.friction_prev_y = b.friction_y;
        b.p.friction_prev_o = b.friction_o;
        b.friction_x = b.friction_y = b.friction_o = 0.;
        b.p.fdt_dead_x = b.p.fdt_dead_y = b.p.fdt_dead_o = 0.;
        b.p.g_dead = 0.;
        b.nusselt = 0.;
    }
    VV_CUDA(cudaStreamSynchronize(s));
}

}  // namespace vvgpu
