// Packed FP32 pairs: the sm_100-family f32x2 arithmetic, one instruction for two FP32
// operations, each rounded to nearest as the scalar instruction would round it.
#pragma once

#include <cstdint>

namespace vvgpu {

__device__ __forceinline__ uint64_t f2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void uf2(uint64_t v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t fadd2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fsub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fmul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// Knuth's TwoSum on both halves: (h, l) accumulates v, h + l keeping the rounding errors.
__device__ __forceinline__ void two_sum_acc2(uint64_t& h, uint64_t& l, uint64_t v) {
    const uint64_t s = fadd2(h, v);
    const uint64_t bp = fsub2(s, h);
    l = fadd2(l, fadd2(fsub2(h, fsub2(s, bp)), fsub2(v, bp)));
    h = s;
}

}  // namespace vvgpu
