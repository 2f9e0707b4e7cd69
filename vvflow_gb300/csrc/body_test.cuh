// Point-in-body test of libvvhd: TBody::isPointInvalid -> isPointInContour
// (libvvhd/src/TBody.cpp:217-281) with the bounding pre-checks of doFillProperties
// (TBody.cpp:327-342), exact FP64 without contraction.  Shared by move_and_clean and the
// vorticity field (Space::point_is_in_body, libvvhd/headers/TSpace.hpp:140-145).
#pragma once

#include <cfloat>
#include <cmath>

#include "vvgpu_internal.cuh"

namespace vvgpu {

struct BodyTest {
    double blx, bly, trx, try_, cofx, cofy, r2max, axx, axy;
    int64_t first, count;
    int inverted;  // area <= 0: TBody::isInsideValid
};

// Order-preserving integer key of a double: a < b (IEEE) <=> ykey(a) < ykey(b), with -0 and
// +0 one key (as they compare equal); not for NaN.
__device__ __forceinline__ int64_t ykey(double v) {
    uint64_t u = (uint64_t)__double_as_longlong(v);
    if ((u << 1) == 0) u = 0;
    const uint64_t k = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    return (int64_t)(k ^ 0x8000000000000000ull);
}

// TBody::isPointInContour over the corners, exact FP64 (no contraction).  Returns the
// global index of the segment whose centre is nearest, or -1.
__device__ __forceinline__ int64_t point_invalid(const BodyTest& b, const double* __restrict__ cx, const double* __restrict__ cy,
                                 const double* __restrict__ rx, const double* __restrict__ ry, double px, double py) {
    bool in = b.inverted != 0;
    if (!in && (px < b.blx || py < b.bly || px > b.trx || py > b.try_ ||
                dabs2(dsub(px, b.cofx), dsub(py, b.cofy)) > b.r2max))
        return -1;
    // The y-range conditions of an edge are exact comparisons of doubles, made here on
    // order-preserving integer keys (integer pipe); only the few edges whose range holds py
    // take the FP64 products.
    const int64_t f = b.first, n = b.count;
    if (n > 0) {
        const int64_t kpy = ykey(py);
        int64_t kjy = ykey(cy[f + n - 1]);
        for (int64_t i = 0, j = n - 1; i < n; j = i++) {
            const int64_t kiy = ykey(cy[f + i]);
            const bool up = (kiy < kjy) && (kiy < kpy) && (kpy <= kjy);
            const bool down = (kiy > kjy) && (kiy > kpy) && (kpy >= kjy);
            if (up || down) {
                const double vix = cx[f + i], viy = cy[f + i], vjx = cx[f + j], vjy = cy[f + j];
                const double lhs = dmul(dsub(vjy, viy), dsub(px, vix));
                const double rhs = dmul(dsub(vjx, vix), dsub(py, viy));
                if ((up && lhs > rhs) || (down && lhs < rhs)) in = !in;
            }
            kjy = kiy;
        }
    }
    if (!in) return -1;
    int64_t best = -1;
    double bd = DBL_MAX;
    for (int64_t k = 0; k < n; k++) {
        const double d = dabs2(dsub(rx[f + k], px), dsub(ry[f + k], py));
        if (d < bd) { bd = d; best = f + k; }
    }
    return best;
}

// Per-body test geometry, from the host copies of the corners.
inline BodyTest body_test_of(const Ctx& c, const BodyHost& b) {
    BodyTest mb{};
    mb.blx = mb.bly = INFINITY;
    mb.trx = mb.try_ = -INFINITY;
    mb.r2max = 0;
    mb.cofx = b.cofm_x;
    mb.cofy = b.cofm_y;
    for (int64_t k = 0; k < b.count; k++) {
        const double px = c.h_cx[b.first + k], py = c.h_cy[b.first + k];
        const double dx = px - b.cofm_x, dy = py - b.cofm_y;
        const double r2 = dx * dx + dy * dy;
        if (r2 > mb.r2max) mb.r2max = r2;
        if (px > mb.trx) mb.trx = px;
        if (py > mb.try_) mb.try_ = py;
        if (px < mb.blx) mb.blx = px;
        if (py < mb.bly) mb.bly = py;
    }
    mb.axx = b.p.holder_x + b.p.dpos_x;
    mb.axy = b.p.holder_y + b.p.dpos_y;
    mb.first = b.first;
    mb.count = b.count;
    mb.inverted = b.area <= 0;
    return mb;
}

}  // namespace vvgpu
