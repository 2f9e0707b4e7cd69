// Local FP32 frames for pairwise kernels.
//
// Every leaf gets an anchor point a = G * (kx, ky) on a power-of-two grid G, stored as FP32
// (exact: |k| < 2^21).  A vortex is stored in FP32 relative to the anchor of its own leaf.
// For a target leaf L and a source leaf q the shift between frames, aq - aL = G (kq - kL),
// is an exact FP32 subtraction, so a source coordinate in the target's frame costs one
// rounded addition and no integer-to-float conversion (those run on the narrow FP64 /
// conversion pipe of sm_103).  Positions of order 100 with spacings of order 1e-3 keep ~1e-7 relative
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

__device__ __forceinline__ float2 anchor_of(double cx, double cy, double G) {
    return make_float2((float)(rint(cx / G) * G), (float)(rint(cy / G) * G));
}

// Exact FP32 shift between two anchors.
__device__ __forceinline__ float2 frame_shift(float2 from, float2 to, float) {
    return make_float2(from.x - to.x, from.y - to.y);
}

}  // namespace vvgpu
