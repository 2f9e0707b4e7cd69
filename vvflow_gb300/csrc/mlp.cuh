// Shared definitions of the MLP far-field correction (learned.cu: training, inference,
// samples; learned_step.cu: the correction inside the convective pass): network sizes,
// parameter and weight-image layouts, the tcgen05 / mbarrier / TMEM helpers and the model.
#pragma once
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace mlp {

constexpr int TILE = 128;   // samples per tile (MMA M)
constexpr int NF = 20;      // features
constexpr int KIN = 32;     // features padded to a multiple of 16
constexpr int HID = 64;
constexpr int NOUT = 2;
constexpr int NOUTP = 16;   // outputs padded (MMA N >= 16)

// parameter vector (FP32 master copy)
constexpr int P_W1 = 0;                      // [HID][KIN] (columns >= NF stay 0)
constexpr int P_B1 = P_W1 + HID * KIN;
constexpr int P_W2 = P_B1 + HID;             // [HID][HID]
constexpr int P_B2 = P_W2 + HID * HID;
constexpr int P_W3 = P_B2 + HID;             // [NOUT][HID]
constexpr int P_B3 = P_W3 + NOUT * HID;
constexpr int NPARAM = P_B3 + NOUT;
constexpr int PSTRIDE = NPARAM + 2;          // per-tile partials: gradients, then the loss sum
// standardisation: network input k = (feature k - norm[k]) * norm[NF + k]; network output o
// times norm[2 NF + o] is the label
constexpr int NNORM = 2 * NF + NOUT;

// BF16 weight image in shared-memory operand order (core matrices), copied as is
constexpr int I_W1 = 0;                      // B of Z1 = X W1^T : [N = HID][K = KIN]
constexpr int I_W2 = I_W1 + HID * KIN;       // B of Z2 = H1 W2^T : [HID][HID]
constexpr int I_W3 = I_W2 + HID * HID;       // B of Y = H2 W3^T : [NOUTP][HID]
constexpr int I_W3T = I_W3 + NOUTP * HID;    // B of dH2 = dY W3 : [N = HID][K = NOUTP]
constexpr int I_W2T = I_W3T + HID * NOUTP;   // B of dH1 = dZ2 W2 : [N = HID][K = HID]
constexpr int NIMG = I_W2T + HID * HID;
constexpr int NIMG_FWD = I_W3T;              // the forward needs W1, W2, W3 only

// element (r, k) of a K-major operand with kc = K / 8 core matrices per 8-row group
__host__ __device__ __forceinline__ int tile_off(int r, int k, int kc) {
    return ((r >> 3) * kc + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle (descriptor version 1 of the sm_100 family)
__device__ __forceinline__ uint64_t sdesc(const void* p, uint32_t lbo, uint32_t sbo) {
    const uint32_t a = smem_u32(p);
    return (uint64_t)((a >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// kind::f16 instruction descriptor: FP32 accumulate, BF16 A and B, both K-major, M = 128
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TILE >> 4) << 24);
}

// D[128 x n] (+)= A[128 x k] B[n x k]^T; A and B K-major in shared memory; one thread.
__device__ __forceinline__ void mma_issue(uint32_t tmem_d, const __nv_bfloat16* A, const __nv_bfloat16* B, int k, int n,
                                          bool accumulate) {
    const uint32_t kc_bytes = 128, rg_bytes = (uint32_t)(k / 8) * 128;
    const uint32_t id = idesc_bf16(n);
    for (int ks = 0; ks < k / 16; ks++) {
        const uint64_t da = sdesc(A + ks * 128, kc_bytes, rg_bytes);
        const uint64_t db = sdesc(B + ks * 128, kc_bytes, rg_bytes);
        const uint32_t acc = (accumulate || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
            "l"(da), "l"(db), "r"(id), "r"(acc));
    }
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)));
}

// bounded wait for the mbarrier phase `parity` (at most `spins` polls); false on timeout
constexpr uint32_t MBAR_SPINS = 1u << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t spins) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < spins && !done; it++)
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity));
    return done != 0;
}

// 16 consecutive FP32 columns of this warp's 32 lanes (row = 32 * warp + lane)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint32_t tmem_lane_addr(uint32_t base, int warp, int col) {
    return base + ((uint32_t)(32 * warp) << 16) + (uint32_t)col;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }
__device__ __forceinline__ void fence_smem_to_mma() { asm volatile("fence.proxy.async.shared::cta;"); }

// tanh form of GELU and its derivative
constexpr float GC = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float GA = 0.044715f;
__device__ __forceinline__ float gelu(float z) {
    const float t = tanhf(GC * (z + GA * z * z * z));
    return 0.5f * z * (1.f + t);
}
__device__ __forceinline__ float gelu_d(float z) {
    const float t = tanhf(GC * (z + GA * z * z * z));
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * GC * (1.f + 3.f * GA * z * z);
}

// TMEM allocation by warp 0 (ncols a power of two >= 32); the address lands in *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, int ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, int ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Complex moments M2..M4 of every node about its +/- centroids (nd_mom), once per tree and
// circulation state (learned.cu).
void ensure_moments(Ctx& c);

}  // namespace mlp

}  // namespace vvgpu

// The opaque handle of include/vvgpu.h's vvgpu_mlp_* calls.
struct vvgpu_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    vvgpu::DArr<float> params, m1, m2, part, grad, loss, norm;
    vvgpu::DArr<__nv_bfloat16> img;
    vvgpu::DArr<float> feat, lab;        // samples: features [n][NF], labels [n][2]
    int64_t nsamples = 0;
    vvgpu::DArr<int64_t> ids;            // sample order of an epoch, padded with -1 to whole tiles
    vvgpu::DArr<int32_t> err;
    int64_t steps = 0;            // Adam steps taken
    int64_t launches = 0;
    uint32_t wait_spins = vvgpu::mlp::MBAR_SPINS;  // polls of one tensor-core completion wait
};
