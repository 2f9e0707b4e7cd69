// Kernel shapes of the FP32 pair passes, chosen per context by timing them on the
// context's own tree: the sources per staged tile of the convective near field (k_conv32:
// 128, 192 or 256; shared memory per one-warp block 8, 12 or 16 KB) and the targets per pass
// of the diffusive pass (k_diff32: shape 1 takes up to 16, shape 2 up to 8).  Each variant
// computes the same sums (in a different order of the FP32 partial sums), so the choice
// changes speed, not the method.  No
// counterpart in the reference, whose OpenMP loops have no tile shapes.
#include <cmath>

#include "vvgpu_internal.cuh"

namespace vvgpu {

// ms (may be null): convective at tiles 128, 192, 256, then diffusive at shapes 1 and 2
// (device time, the best of two runs each).  Velocities and friction are left as
// they were.
void autotune_tiles(Ctx& c, double* ms) {
    c.tune_pending = false;
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    if (c.precision != VVGPU_FP32) {  // the FP64 passes have one shape each
        if (ms)
            for (int k = 0; k < 5; k++) ms[k] = -1.;
        return;
    }
    ensure_full_lists(c);
    cudaStream_t s = c.st();
    const int64_t n = c.n, m = c.m;
    DArr<double> keep;
    keep.reserve(2 * (size_t)n + (size_t)m + 1);
    auto copy = [&](bool save) {
        double* k = keep.p;
        if (n) {
            VV_CUDA(cudaMemcpyAsync(save ? k : c.vx.p, save ? c.vx.p : k, n * 8, cudaMemcpyDeviceToDevice, s));
            VV_CUDA(cudaMemcpyAsync(save ? k + n : c.vy.p, save ? c.vy.p : k + n, n * 8, cudaMemcpyDeviceToDevice, s));
        }
        if (m) VV_CUDA(cudaMemcpyAsync(save ? k + 2 * n : c.s_fric.p, save ? c.s_fric.p : k + 2 * n, m * 8,
                                       cudaMemcpyDeviceToDevice, s));
    };
    copy(true);
    const bool timing = c.timing;
    c.timing = false;  // the trials stay out of the kernel-time sums
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    VV_CUDA(cudaEventCreate(&e0));
    VV_CUDA(cudaEventCreate(&e1));
    auto timed = [&](auto&& fn) {
        float best = INFINITY;
        for (int r = 0; r < 2; r++) {
            copy(false);
            VV_CUDA(cudaEventRecord(e0, s));
            fn();
            VV_CUDA(cudaEventRecord(e1, s));
            VV_CUDA(cudaEventSynchronize(e1));
            float t = 0.f;
            VV_CUDA(cudaEventElapsedTime(&t, e0, e1));
            best = std::fmin(best, t);
        }
        return (double)best;
    };
    try {
        const int tiles[3] = {128, 192, 256};
        double t[5];
        int bt = c.conv_tile, bd = c.diff_targets;
        double best = INFINITY;
        for (int k = 0; k < 3; k++) {
            c.conv_tile = tiles[k];
            t[k] = timed([&] { convective(c); });
            if (t[k] < best) { best = t[k]; bt = tiles[k]; }
        }
        best = INFINITY;
        for (int k = 0; k < 2; k++) {
            c.diff_targets = k + 1;
            t[3 + k] = timed([&] { diffusive(c); });
            if (t[3 + k] < best) { best = t[3 + k]; bd = k + 1; }
        }
        c.conv_tile = bt;
        c.diff_targets = bd;
        copy(false);
        if (ms)
            for (int k = 0; k < 5; k++) ms[k] = t[k];
    } catch (...) {
        copy(false);
        c.timing = timing;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    c.timing = timing;
    VV_CUDA(cudaStreamSynchronize(s));
    VV_CUDA(cudaEventDestroy(e0));
    VV_CUDA(cudaEventDestroy(e1));
}

}  // namespace vvgpu
