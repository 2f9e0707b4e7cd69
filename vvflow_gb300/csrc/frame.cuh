// Local FP32 frames for pairwise kernels.
//
// Every leaf gets an anchor point a = G * (kx, ky) on a power-of-two grid G.  A vortex is
// stored in FP32 relative to the anchor of its own leaf.  For a target leaf L and a source
// leaf q the shift between frames, G * (kq - kL), is exact in FP32 (an integer below 2^24
// times a power of two), so a source coordinate in the target's frame costs one rounded
// addition.  Positions of order 100 with spacings of order 1e-3 keep ~1e-7 relative
// precision in every pair displacement, where a global FP32 frame would keep ~1e-3.
#pragma once

#include <cmath>

#include "vvgpu_internal.cuh"

namespace vvgpu {

struct Frame {
    double G = 1.0;        // anchor grid spacing (power of two)
    float Gf = 1.0f;
};

// Chooses G so that |k| stays below 2^21 for the whole box of the root.
inline Frame make_frame(double extent) {
    Frame f;
    if (!(extent > 0) || !std::isfinite(extent)) extent = 1.0;
    int e = (int)std::ceil(std::log2(extent / (double)(1 << 20)));
    f.G = std::ldexp(1.0, e);
    f.Gf = (float)f.G;
    return f;
}

__device__ __forceinline__ int2 anchor_of(double cx, double cy, double G) {
    return make_int2((int)rint(cx / G), (int)rint(cy / G));
}

// Exact FP32 shift between two anchors.
__device__ __forceinline__ float2 frame_shift(int2 from, int2 to, float Gf) {
    return make_float2((float)(from.x - to.x) * Gf, (float)(from.y - to.y) * Gf);
}

}  // namespace vvgpu
