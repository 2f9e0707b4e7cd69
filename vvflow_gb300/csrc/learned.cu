// Learned far-field correction: a small MLP that predicts, for one far cell of the tree and
// one target point, the part of the cell's Biot-Savart velocity that the reference's
// monopole far field (the +/- centroids, MConvectiveFast.cpp:139-151) misses.  It lets a
// looser opening criterion keep more of the plain tree's accuracy.
//
// Inputs (20, cell_features): the cell's positive and negative circulations over their
// total G, each centroid's offset from the cell centre over the cell size s = h + w, the
// complex moments M_k = sum g (z - c)^k about each centroid for k = 2, 3, 4 over G s^k, and
// the target's offset from the cell centre over s.  Output (2): the residual velocity
// (exact FP64 direct sum over the cell minus the monopoles) times 2 pi d^3 / (G s^2), with
// d the target's distance from the cell centre.
//
// Network 20 -> 64 -> 64 -> 2 with tanh-GELU, BF16 weights and activations, FP32
// accumulation.  Every product, forward and backward, is one tcgen05.mma shape: M = 128
// rows (a tile of 128 samples, or an output dimension padded to 128), K-major BF16 A and B
// staged in shared memory in the canonical no-swizzle layout (8 x 16-byte core matrices,
// leading byte offset = the next core matrix along K, stride byte offset = the next 8-row
// group), FP32 accumulators in tensor memory, read back with tcgen05.ld.  One elected
// thread issues the MMAs and commits them to an mbarrier; every wait is bounded and sets
// an error flag.  Weight gradients (sum over the tile's samples) are products with the
// samples as K: dW = dZ^T X, with dZ^T and X^T written transposed into shared memory.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "mlp.cuh"

namespace vvgpu {

namespace mlp {

// ---- inference -----------------------------------------------------------------------
// y[i] for i < n from features[i][NF]; persistent over 128-sample tiles.
constexpr int FWD_TMEM = 128;  // Z1 at column 0, Z2 at 64; Y reuses column 0
struct FwdSmem {
    __nv_bfloat16 w[NIMG_FWD];
    __nv_bfloat16 x0[TILE * KIN];
    __nv_bfloat16 h1[TILE * HID];
    __nv_bfloat16 h2[TILE * HID];
    float b1[HID], b2[HID], b3[NOUTP];
    uint64_t mbar;
    uint32_t tmem;
};

__global__ void __launch_bounds__(TILE) k_mlp_forward(int64_t n, const float* __restrict__ feat,
                                                     const __nv_bfloat16* __restrict__ img,
                                                     const float* __restrict__ params,
                                                     const float* __restrict__ norm, float* __restrict__ y,
                                                     int* err, uint32_t spins) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    FwdSmem& S = *reinterpret_cast<FwdSmem*>(smraw);
    const int tid = threadIdx.x, w = tid >> 5;
    for (int i = tid; i < NIMG_FWD; i += TILE) S.w[i] = img[i];
    for (int i = tid; i < HID; i += TILE) { S.b1[i] = params[P_B1 + i]; S.b2[i] = params[P_B2 + i]; }
    if (tid < NOUTP) S.b3[tid] = tid < NOUT ? params[P_B3 + tid] : 0.f;
    if (tid == 0) mbar_init(&S.mbar);
    if (w == 0) tmem_alloc(&S.tmem, FWD_TMEM);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = S.tmem;
    uint32_t phase = 0, lost = 2;  // lost: the phase whose completion a timed-out wait missed
    bool ok = true;
    const int64_t ntiles = (n + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t i = tile * TILE + tid;
        // X0 row tid: features (BF16), zero padding
        for (int k = 0; k < KIN; k++) {
            const float v = (i < n && k < NF) ? (feat[i * NF + k] - norm[k]) * norm[NF + k] : 0.f;
            S.x0[tile_off(tid, k, KIN / 8)] = __float2bfloat16(v);
        }
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) { mma_issue(tm, S.x0, S.w + I_W1, KIN, HID, false); mma_commit(&S.mbar); }
        ok = __syncthreads_and(mbar_wait(&S.mbar, phase, spins));
        if (!ok) lost = phase;
        phase ^= 1;
        fence_after();
        if (!ok) break;
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, c), v);
#pragma unroll
            for (int j = 0; j < 16; j++) S.h1[tile_off(tid, c + j, HID / 8)] = __float2bfloat16(gelu(v[j] + S.b1[c + j]));
        }
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) { mma_issue(tm + 64, S.h1, S.w + I_W2, HID, HID, false); mma_commit(&S.mbar); }
        ok = __syncthreads_and(mbar_wait(&S.mbar, phase, spins));
        if (!ok) lost = phase;
        phase ^= 1;
        fence_after();
        if (!ok) break;
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, 64 + c), v);
#pragma unroll
            for (int j = 0; j < 16; j++) S.h2[tile_off(tid, c + j, HID / 8)] = __float2bfloat16(gelu(v[j] + S.b2[c + j]));
        }
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) { mma_issue(tm, S.h2, S.w + I_W3, HID, NOUTP, false); mma_commit(&S.mbar); }
        ok = __syncthreads_and(mbar_wait(&S.mbar, phase, spins));
        if (!ok) lost = phase;
        phase ^= 1;
        fence_after();
        if (!ok) break;
        {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, 0), v);
            if (i < n) {
                y[i * NOUT + 0] = (v[0] + S.b3[0]) * norm[2 * NF];
                y[i * NOUT + 1] = (v[1] + S.b3[1]) * norm[2 * NF + 1];
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    // a wait that gave up leaves its MMA in flight: let it land (bounded) before the tensor
    // memory it writes is released
    if (lost != 2) mbar_wait(&S.mbar, lost, MBAR_SPINS);
    fence_before();
    __syncthreads();
    if (w == 0) tmem_free(tm, FWD_TMEM);
}

// ---- training: one tile of samples, forward and backward ------------------------------
constexpr int TR_TMEM = 512;
constexpr int C_Z1 = 0, C_Z2 = 64, C_Y = 128, C_DH2 = 160, C_DH1 = 224, C_DW3 = 288, C_DW2 = 352, C_DW1 = 416;
struct TrainSmem {
    __nv_bfloat16 w[NIMG];
    __nv_bfloat16 x0[TILE * KIN], x0t[KIN * TILE];    // X0 [b][k] and X0^T [k][b]
    __nv_bfloat16 h1[TILE * HID], h1t[HID * TILE];
    __nv_bfloat16 h2[TILE * HID], h2t[HID * TILE];
    __nv_bfloat16 dy[TILE * NOUTP];                   // dY [b][o]
    __nv_bfloat16 dz[TILE * HID];                     // dZ2 [b][o]
    __nv_bfloat16 at[TILE * TILE];                    // dY^T / dZ^T [o][b], o padded to 128 (rows beyond stay 0)
    float b1[HID], b2[HID], b3[NOUTP];
    float red[4][HID];                                // per-warp column sums (bias gradients)
    float lred[4];
    uint64_t mbar;
    uint32_t tmem;
};

// column sums over the tile's rows of v[HID] (one value per thread per column): per-warp
// shuffle trees, then the four warps in order
__device__ __forceinline__ void col_sums(TrainSmem& S, const float* v, int ncol, float* out) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = 0; c < ncol; c++) {
        float s = v[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) S.red[w][c] = s;
    }
    __syncthreads();
    if ((int)threadIdx.x < ncol) {
        const int c = threadIdx.x;
        out[c] = ((S.red[0][c] + S.red[1][c]) + S.red[2][c]) + S.red[3][c];
    }
    __syncthreads();
}

// Partial gradients of the loss sum_i |y_i - t_i|^2 * scale over the tile's samples
// sample_ids[tile * TILE ..] (< 0: padding), written to part[tile * PSTRIDE ..] (the loss
// sum at NPARAM).
__global__ void __launch_bounds__(TILE) k_mlp_train_tile(const float* __restrict__ feat, const float* __restrict__ lab,
                                                        const int64_t* __restrict__ sample_ids,
                                                        const __nv_bfloat16* __restrict__ img,
                                                        const float* __restrict__ params,
                                                        const float* __restrict__ norm, float scale,
                                                        float* __restrict__ part, int* err, uint32_t spins) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smraw);
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int64_t sid = sample_ids[(int64_t)blockIdx.x * TILE + tid];
    float* gp = part + (int64_t)blockIdx.x * PSTRIDE;
    for (int i = tid; i < NIMG; i += TILE) S.w[i] = img[i];
    for (int i = tid; i < TILE * TILE; i += TILE) S.at[i] = __float2bfloat16(0.f);
    for (int i = tid; i < HID; i += TILE) { S.b1[i] = params[P_B1 + i]; S.b2[i] = params[P_B2 + i]; }
    if (tid < NOUTP) S.b3[tid] = tid < NOUT ? params[P_B3 + tid] : 0.f;
    if (tid == 0) mbar_init(&S.mbar);
    if (w == 0) tmem_alloc(&S.tmem, TR_TMEM);
    // X0 row and its transpose
    for (int k = 0; k < KIN; k++) {
        const __nv_bfloat16 v =
            __float2bfloat16((sid >= 0 && k < NF) ? (feat[sid * NF + k] - norm[k]) * norm[NF + k] : 0.f);
        S.x0[tile_off(tid, k, KIN / 8)] = v;
        S.x0t[tile_off(k, tid, TILE / 8)] = v;
    }
    fence_smem_to_mma();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = S.tmem;
    uint32_t phase = 0, lost = 2;  // lost: the phase whose completion a timed-out wait missed
    bool ok = true;
    auto sync_mma = [&]() {
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
    };
    // every thread waits, then all agree (tcgen05.ld needs converged warps)
    auto wait = [&]() {
        const bool mine = ok ? mbar_wait(&S.mbar, phase, spins) : false;
        const bool all = __syncthreads_and(mine) != 0;
        if (ok && !all) lost = phase;
        ok = all;
        phase ^= 1;
        fence_after();
    };
    // forward
    if (tid == 0) { mma_issue(tm + C_Z1, S.x0, S.w + I_W1, KIN, HID, false); mma_commit(&S.mbar); }
    wait();
    if (ok) {
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_Z1 + c), v);
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const __nv_bfloat16 h = __float2bfloat16(gelu(v[j] + S.b1[c + j]));
                S.h1[tile_off(tid, c + j, HID / 8)] = h;
                S.h1t[tile_off(c + j, tid, TILE / 8)] = h;
            }
        }
    }
    sync_mma();
    if (tid == 0 && ok) { mma_issue(tm + C_Z2, S.h1, S.w + I_W2, HID, HID, false); mma_commit(&S.mbar); }
    wait();
    if (ok) {
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_Z2 + c), v);
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const __nv_bfloat16 h = __float2bfloat16(gelu(v[j] + S.b2[c + j]));
                S.h2[tile_off(tid, c + j, HID / 8)] = h;
                S.h2t[tile_off(c + j, tid, TILE / 8)] = h;
            }
        }
    }
    sync_mma();
    if (tid == 0 && ok) { mma_issue(tm + C_Y, S.h2, S.w + I_W3, HID, NOUTP, false); mma_commit(&S.mbar); }
    wait();
    // loss and dY = 2 scale (y - t)
    float dyv[NOUT] = {0.f, 0.f};
    float lsum = 0.f;
    if (ok) {
        float v[16];
        tmem_ld16(tmem_lane_addr(tm, w, C_Y), v);
        if (sid >= 0) {
#pragma unroll
            for (int o = 0; o < NOUT; o++) {
                const float r = v[o] + S.b3[o] - lab[sid * NOUT + o] / norm[2 * NF + o];
                lsum += r * r;
                dyv[o] = 2.f * scale * r;
            }
        }
        for (int o = 0; o < NOUTP; o++) S.dy[tile_off(tid, o, NOUTP / 8)] = __float2bfloat16(o < NOUT ? dyv[o] : 0.f);
        for (int o = 0; o < NOUT; o++) S.at[tile_off(o, tid, TILE / 8)] = __float2bfloat16(dyv[o]);
    }
    {
        float s = lsum;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) S.lred[w] = s;
    }
    sync_mma();
    if (tid == 0) gp[NPARAM] = ((S.lred[0] + S.lred[1]) + S.lred[2]) + S.lred[3];
    // dH2 = dY W3, dW3 = dY^T H2
    if (tid == 0 && ok) {
        mma_issue(tm + C_DH2, S.dy, S.w + I_W3T, NOUTP, HID, false);
        mma_issue(tm + C_DW3, S.at, S.h2t, TILE, HID, false);
        mma_commit(&S.mbar);
    }
    wait();
    float dzv[HID];
    if (ok) {
        for (int c = 0; c < HID; c += 16) {
            float d[16], z[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_DH2 + c), d);
            tmem_ld16(tmem_lane_addr(tm, w, C_Z2 + c), z);
#pragma unroll
            for (int j = 0; j < 16; j++) dzv[c + j] = (sid >= 0) ? d[j] * gelu_d(z[j] + S.b2[c + j]) : 0.f;
        }
        for (int c = 0; c < HID; c++) {
            const __nv_bfloat16 h = __float2bfloat16(dzv[c]);
            S.dz[tile_off(tid, c, HID / 8)] = h;
            S.at[tile_off(c, tid, TILE / 8)] = h;
        }
    } else {
        for (int c = 0; c < HID; c++) dzv[c] = 0.f;
    }
    // bias gradients b3 (from dY) and b2 (from dZ2)
    col_sums(S, dyv, NOUT, gp + P_B3);
    col_sums(S, dzv, HID, gp + P_B2);
    sync_mma();
    // dH1 = dZ2 W2, dW2 = dZ2^T H1
    if (tid == 0 && ok) {
        mma_issue(tm + C_DH1, S.dz, S.w + I_W2T, HID, HID, false);
        mma_issue(tm + C_DW2, S.at, S.h1t, TILE, HID, false);
        mma_commit(&S.mbar);
    }
    wait();
    if (ok) {
        for (int c = 0; c < HID; c += 16) {
            float d[16], z[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_DH1 + c), d);
            tmem_ld16(tmem_lane_addr(tm, w, C_Z1 + c), z);
#pragma unroll
            for (int j = 0; j < 16; j++) dzv[c + j] = (sid >= 0) ? d[j] * gelu_d(z[j] + S.b1[c + j]) : 0.f;
        }
        for (int c = 0; c < HID; c++) S.at[tile_off(c, tid, TILE / 8)] = __float2bfloat16(dzv[c]);
    }
    col_sums(S, dzv, HID, gp + P_B1);
    sync_mma();
    // dW1 = dZ1^T X0
    if (tid == 0 && ok) { mma_issue(tm + C_DW1, S.at, S.x0t, TILE, KIN, false); mma_commit(&S.mbar); }
    wait();
    // weight gradients: TMEM rows = output units (lanes 0..63 held by warps 0 and 1)
    if (ok && w < 2) {
        const int o = 32 * w + lane;
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_DW2 + c), v);
#pragma unroll
            for (int j = 0; j < 16; j++) gp[P_W2 + o * HID + c + j] = v[j];
        }
        for (int c = 0; c < KIN; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_DW1 + c), v);
#pragma unroll
            for (int j = 0; j < 16; j++) gp[P_W1 + o * KIN + c + j] = (c + j < NF) ? v[j] : 0.f;
        }
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, C_DW3 + c), v);
            if (o < NOUT)
#pragma unroll
                for (int j = 0; j < 16; j++) gp[P_W3 + o * HID + c + j] = v[j];
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    if (lost != 2) mbar_wait(&S.mbar, lost, MBAR_SPINS);  // the abandoned MMA lands first
    fence_before();
    __syncthreads();
    if (w == 0) tmem_free(tm, TR_TMEM);
}

// Sums the tiles' partial gradients in tile order, applies Adam (bias-corrected) to the
// FP32 master weights and rewrites the BF16 image.  One thread per parameter.
__global__ void k_mlp_adam(int ntiles, const float* __restrict__ part, float* params, float* m1, float* m2, float lr,
                           float beta1, float beta2, float epsilon, float c1, float c2, __nv_bfloat16* img,
                           float* grad_out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    float g = 0.f;
    for (int t = 0; t < ntiles; t++) g += part[(int64_t)t * PSTRIDE + p];
    if (grad_out) grad_out[p] = g;
    if (lr != 0.f) {
        const float a = beta1 * m1[p] + (1.f - beta1) * g;
        const float b = beta2 * m2[p] + (1.f - beta2) * g * g;
        m1[p] = a;
        m2[p] = b;
        float v = params[p] - lr * (a / c1) / (sqrtf(b / c2) + epsilon);
        if (p < P_B1 && (p % KIN) >= NF) v = 0.f;  // padding inputs
        params[p] = v;
    }
    const float v = params[p];
    const __nv_bfloat16 h = __float2bfloat16(v);
    if (p < P_B1) {
        const int o = p / KIN, i = p % KIN;
        img[I_W1 + tile_off(o, i, KIN / 8)] = h;
    } else if (p >= P_W2 && p < P_B2) {
        const int o = (p - P_W2) / HID, i = (p - P_W2) % HID;
        img[I_W2 + tile_off(o, i, HID / 8)] = h;
        img[I_W2T + tile_off(i, o, HID / 8)] = h;
    } else if (p >= P_W3 && p < P_B3) {
        const int o = (p - P_W3) / HID, i = (p - P_W3) % HID;
        img[I_W3 + tile_off(o, i, HID / 8)] = h;
        img[I_W3T + tile_off(i, o, NOUTP / 8)] = h;
    }
}

__global__ void k_loss_sum(int ntiles, const float* __restrict__ part, float* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        float s = 0.f;
        for (int t = 0; t < ntiles; t++) s += part[(int64_t)t * PSTRIDE + NPARAM];
        *out = s;
    }
}

// ---- samples: far (cell, target) pairs ---------------------------------------------------

// Per node, the complex moments about its +/- centroids (nd_cm): M_k = sum g (z - c)^k,
// k = 2, 3, 4, over the node's vortices of that sign; mom[12 k ..] = M2+, M3+, M4+, M2-,
// M3-, M4- (re, im).  Leaves sum their vortices; inner nodes, level by level from the
// bottom, shift their children's moments to their own centroid (binomial expansion of
// (z - c)^k = ((z - c') + d)^k, d = c' - c, with M_0 = the child's circulation and M_1 = 0
// about the child's own centroid).
__device__ __forceinline__ void cmul(double ax, double ay, double bx, double by, double& rx, double& ry) {
    rx = ax * bx - ay * by;
    ry = ax * by + ay * bx;
}

__global__ void k_leaf_moments(int64_t nn, const int32_t* __restrict__ ch1, const int32_t* __restrict__ vf,
                               const int32_t* __restrict__ vl, const double* __restrict__ cm,
                               const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ g, double* mom) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nn || ch1[k] >= 0) return;
    const double* c = cm + 6 * k;
    double a[12];
#pragma unroll
    for (int q = 0; q < 12; q++) a[q] = 0.;
    for (int32_t j = vf[k]; j < vl[k]; j++) {
        const double gj = g[j];
        if (gj == 0.) continue;
        const int o = gj > 0 ? 0 : 6;
        const double wx = x[j] - (gj > 0 ? c[0] : c[3]), wy = y[j] - (gj > 0 ? c[1] : c[4]);
        double px, py;
        cmul(wx, wy, wx, wy, px, py);
#pragma unroll
        for (int e = 0; e < 3; e++) {
            a[o + 2 * e] += gj * px;
            a[o + 2 * e + 1] += gj * py;
            double nx, ny;
            cmul(px, py, wx, wy, nx, ny);
            px = nx;
            py = ny;
        }
    }
#pragma unroll
    for (int q = 0; q < 12; q++) mom[12 * k + q] = a[q];
}

// Moments of inner node k from its two children's (binomial shift to k's centroids).
__device__ void inner_moments(int64_t k, int32_t c1, const double* __restrict__ cm, double* mom) {
    double out[12];
#pragma unroll
    for (int q = 0; q < 12; q++) out[q] = 0.;
    for (int sgn = 0; sgn < 2; sgn++) {
        const double cx = cm[6 * k + 3 * sgn], cy = cm[6 * k + 3 * sgn + 1];
        for (int h = 0; h < 2; h++) {
            const int64_t u = c1 + h;
            const double G = cm[6 * u + 3 * sgn + 2];
            if (G == 0.) continue;
            const double dx = cm[6 * u + 3 * sgn] - cx, dy = cm[6 * u + 3 * sgn + 1] - cy;
            double m[6];  // M2', M3', M4' (written by another thread: read through L2)
#pragma unroll
            for (int q = 0; q < 6; q++) m[q] = __ldcg(mom + 12 * u + 6 * sgn + q);
            double d2x, d2y, d3x, d3y, d4x, d4y;
            cmul(dx, dy, dx, dy, d2x, d2y);
            cmul(d2x, d2y, dx, dy, d3x, d3y);
            cmul(d3x, d3y, dx, dy, d4x, d4y);
            double tx, ty, ux, uy, vx, vy;
            // M2 = M2' + G d^2
            out[6 * sgn + 0] += m[0] + G * d2x;
            out[6 * sgn + 1] += m[1] + G * d2y;
            // M3 = M3' + 3 M2' d + G d^3
            cmul(m[0], m[1], dx, dy, tx, ty);
            out[6 * sgn + 2] += m[2] + 3. * tx + G * d3x;
            out[6 * sgn + 3] += m[3] + 3. * ty + G * d3y;
            // M4 = M4' + 4 M3' d + 6 M2' d^2 + G d^4
            cmul(m[2], m[3], dx, dy, ux, uy);
            cmul(m[0], m[1], d2x, d2y, vx, vy);
            out[6 * sgn + 4] += m[4] + 4. * ux + 6. * vx + G * d4x;
            out[6 * sgn + 5] += m[5] + 4. * uy + 6. * vy + G * d4y;
        }
    }
#pragma unroll
    for (int q = 0; q < 12; q++) mom[12 * k + q] = out[q];
}

// All inner nodes bottom-up in one pass: each leaf's thread climbs, and at each node the
// second child to arrive computes the node (children in the order ch1, ch1 + 1 either way).
__global__ void k_inner_moments(int64_t nn, const int32_t* __restrict__ ch1, const int32_t* __restrict__ parent,
                                const double* __restrict__ cm, double* mom, int32_t* arrive) {
    const int64_t k0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= nn || ch1[k0] >= 0) return;
    int32_t k = (int32_t)k0;
    for (int it = 0; it <= MAX_DEPTH; it++) {
        const int32_t p = parent[k];
        if (p < 0) return;
        __threadfence();  // this subtree's moments before the arrival
        if (atomicAdd(&arrive[p], 1) == 0) return;  // the sibling computes p
        __threadfence();
        inner_moments(p, ch1[p], cm, mom);
        k = p;
    }
}

struct WalkView {
    const double4* geom;
    const int32_t* ch1;
    double fc;
    int64_t nnodes;
};

// far nodes of the leaf holding p, in the reference's depth-first order (FindNearNodes,
// TSortedTree.cpp:199-217, exact FP64 test); fn(node) per far node
template <class F>
__device__ __forceinline__ void far_walk(const WalkView& t, double px, double py, F&& fn) {
    int32_t k = 0;
    for (int it = 0; it <= MAX_DEPTH && t.ch1[k] >= 0; it++) {
        const double4 gm = t.geom[k];
        if (gm.z < gm.w) k = (px < gm.x) ? t.ch1[k] : t.ch1[k] + 1;
        else k = (py < gm.y) ? t.ch1[k] : t.ch1[k] + 1;
    }
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
            fn(u);
            continue;
        }
        const int32_t c1 = t.ch1[u];
        if (c1 >= 0 && sp + 2 <= MAX_DEPTH + 2) {
            stack[sp++] = c1 + 1;
            stack[sp++] = c1;
        }
    }
}

__global__ void k_far_count(int64_t np, const double* __restrict__ px, const double* __restrict__ py, WalkView t,
                            int32_t* cnt) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    int32_t c = 0;
    far_walk(t, px[q], py[q], [&](int32_t) { c++; });
    cnt[q] = c;
}

__global__ void k_far_fill(int64_t np, const double* __restrict__ px, const double* __restrict__ py, WalkView t,
                           const int64_t* __restrict__ off, int32_t* node, int32_t* target, int64_t first_target) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    int64_t o = off[q];
    far_walk(t, px[q], py[q], [&](int32_t u) {
        node[o] = u;
        target[o] = (int32_t)(first_target + q);
        o++;
    });
}

// Features (20), label (2: normalised residual of the exact FP64 sum over the cell) and the
// factor back to velocity for pair i = (target point, far node).
__global__ void k_pair_samples(int64_t npairs, const int32_t* __restrict__ node, const int32_t* __restrict__ target,
                               const double* __restrict__ px, const double* __restrict__ py,
                               const double4* __restrict__ geom, const double* __restrict__ cm,
                               const double* __restrict__ mom, const int32_t* __restrict__ vf,
                               const int32_t* __restrict__ vl, const double* __restrict__ x,
                               const double* __restrict__ y, const double* __restrict__ g, float* feat, float* lab,
                               double* back, int with_label) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npairs) return;
    const int32_t S = node[i];
    const int32_t tq = target[i];
    const double p0 = px[tq], p1 = py[tq];
    const double4 gm = geom[S];
    const double* c = cm + 6 * (size_t)S;
    const double* mo = mom + 12 * (size_t)S;
    const double sz = gm.z + gm.w;
    const double G = c[2] - c[5];
    float* f = feat + i * NF;
    const double dx = p0 - gm.x, dy = p1 - gm.y;
    const double d2 = dx * dx + dy * dy, d = sqrt(d2);
    if (!(G > 0.) || !(sz > 0.)) {
        for (int k = 0; k < NF; k++) f[k] = 0.f;
        if (with_label) { lab[2 * i] = 0.f; lab[2 * i + 1] = 0.f; }
        back[i] = 0.;
        return;
    }
    const double iG = 1. / G, is = 1. / sz;
    f[0] = (float)(c[2] * iG);
    f[1] = (float)(c[5] * iG);
    f[2] = (float)((c[0] - gm.x) * is);
    f[3] = (float)((c[1] - gm.y) * is);
    f[4] = (float)((c[3] - gm.x) * is);
    f[5] = (float)((c[4] - gm.y) * is);
    const double s2 = is * is, sc[3] = {iG * s2, iG * s2 * is, iG * s2 * s2};
#pragma unroll
    for (int sgn = 0; sgn < 2; sgn++)
#pragma unroll
        for (int e = 0; e < 3; e++) {
            f[6 + 6 * sgn + 2 * e] = (float)(mo[6 * sgn + 2 * e] * sc[e]);
            f[6 + 6 * sgn + 2 * e + 1] = (float)(mo[6 * sgn + 2 * e + 1] * sc[e]);
        }
    f[18] = (float)(dx * is);
    f[19] = (float)(dy * is);
    const double norm = 2. * C_PI * d2 * d / (G * sz * sz);
    back[i] = 1. / norm;
    if (!with_label) return;
    // exact sum over the cell's vortices minus the two monopoles (MConvectiveFast.cpp:116-151)
    double ex = 0, ey = 0;
    for (int32_t j = vf[S]; j < vl[S]; j++) {
        const double gj = g[j];
        if (gj == 0.) continue;
        const double rx = p0 - x[j], ry = p1 - y[j];
        const double q = gj / (rx * rx + ry * ry);
        ex -= ry * q;
        ey += rx * q;
    }
    double mx = 0, my = 0;
    for (int sgn = 0; sgn < 2; sgn++) {
        const double gs = c[3 * sgn + 2];
        if (gs == 0.) continue;
        const double rx = p0 - c[3 * sgn], ry = p1 - c[3 * sgn + 1];
        const double q = gs / (rx * rx + ry * ry);
        mx -= ry * q;
        my += rx * q;
    }
    lab[2 * i] = (float)((ex - mx) * C_1_2PI * norm);
    lab[2 * i + 1] = (float)((ey - my) * C_1_2PI * norm);
}

// per target point: sum over its pairs (contiguous, walk order) of y * back
__global__ void k_apply_correction(int64_t np, const int64_t* __restrict__ off, const float* __restrict__ yv,
                                   const double* __restrict__ back, double* vx, double* vy) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    double sx = 0, sy = 0;
    for (int64_t i = off[q]; i < off[q + 1]; i++) {
        sx += (double)yv[2 * i] * back[i];
        sy += (double)yv[2 * i + 1] * back[i];
    }
    vx[q] += sx;
    vy[q] += sy;
}

}  // namespace mlp

}  // namespace vvgpu

// ---- host side ---------------------------------------------------------------------------

using namespace vvgpu;
using namespace vvgpu::mlp;

namespace {

int mfail(vvgpu_mlp* m, int code, const std::string& msg) {
    m->last_error = msg;
    return code;
}

#define MLP_BEGIN(mp)                              \
    if (!(mp)) return VVGPU_ERR_ARG;               \
    vvgpu_mlp& M = *(mp);                          \
    try {                                          \
        VV_CUDA(cudaSetDevice(M.device));
#define MLP_END                                                                                \
    }                                                                                          \
    catch (ApiError & e) { return mfail(&M, e.code, e.msg); }                                  \
    catch (CudaError & e) {                                                                    \
        return mfail(&M, VVGPU_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.err)); \
    }                                                                                          \
    catch (std::bad_alloc&) { return mfail(&M, VVGPU_ERR_NOMEM, "host allocation failed"); }  \
    return 0;

// launches count into the model (the macro VV_LAUNCH_CHECK counts into a context named c)
#define MLP_LAUNCH_CHECK()                 \
    do {                                   \
        VV_CUDA(cudaGetLastError());       \
        ++M.launches;                      \
    } while (0)

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

size_t fwd_smem() { return sizeof(FwdSmem) + 1024; }
size_t train_smem() { return sizeof(TrainSmem) + 1024; }

void check_err(vvgpu_mlp& M) {
    int e = 0;
    VV_CUDA(cudaMemcpyAsync(&e, M.err.p, sizeof e, cudaMemcpyDeviceToHost, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    if (e) throw ApiError{VVGPU_ERR_TIMEOUT, "tensor-core wait timed out"};
}

// rewrites the BF16 image from the master weights (Adam with lr = 0 and no tiles)
void refresh_image(vvgpu_mlp& M) {
    k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, M.stream>>>(0, M.part.p, M.params.p, M.m1.p, M.m2.p, 0.f, 0.9f, 0.999f,
                                                          1e-8f, 1.f, 1.f, M.img.p, nullptr);
    MLP_LAUNCH_CHECK();
}

// one pass over the samples ids[0 .. ntiles * TILE): partial gradients, then Adam (lr > 0)
// or the summed gradient (grad_out)
void train_batch(vvgpu_mlp& M, const int64_t* ids, int ntiles, float scale, float lr, float* grad_out,
                 float* loss_slot) {
    M.part.reserve((size_t)ntiles * PSTRIDE);
    k_mlp_train_tile<<<ntiles, TILE, train_smem(), M.stream>>>(M.feat.p, M.lab.p, ids, M.img.p, M.params.p,
                                                             M.norm.p, scale, M.part.p, M.err.p,
                                                             M.wait_spins);
    MLP_LAUNCH_CHECK();
    float c1 = 1.f, c2 = 1.f;
    if (lr != 0.f) {
        M.steps++;
        c1 = 1.f - std::pow(0.9f, (float)M.steps);
        c2 = 1.f - std::pow(0.999f, (float)M.steps);
    }
    k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, M.stream>>>(ntiles, M.part.p, M.params.p, M.m1.p, M.m2.p, lr, 0.9f,
                                                          0.999f, 1e-8f, c1, c2, M.img.p, grad_out);
    MLP_LAUNCH_CHECK();
    if (loss_slot) {
        k_loss_sum<<<1, 32, 0, M.stream>>>(ntiles, M.part.p, loss_slot);
        MLP_LAUNCH_CHECK();
    }
}

void set_attrs() {
    static bool done = false;  // attributes are per function, identical for every model
    if (done) return;
    VV_CUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem()));
    VV_CUDA(cudaFuncSetAttribute(k_mlp_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
    done = true;
}

// aligned start of the dynamic shared memory is taken care of by the kernels' __align__;
// the extra 1024 bytes are headroom for it

void forward_device(vvgpu_mlp& M, int64_t n, const float* dfeat, float* dy) {
    if (n <= 0) return;
    const int64_t ntiles = (n + TILE - 1) / TILE;
    const int grid = (int)std::min<int64_t>(ntiles, 152 * 4);
    k_mlp_forward<<<grid, TILE, fwd_smem(), M.stream>>>(n, dfeat, M.img.p, M.params.p, M.norm.p, dy, M.err.p,
                                                         M.wait_spins);
    MLP_LAUNCH_CHECK();
}

struct PairSet {
    int64_t npairs = 0;
    DArr<int64_t> off;
    DArr<int32_t> node, target;
    DArr<double> pts, back;
};


// far pairs of np points (device arrays dpx, dpy) in the context's built tree, with features
// (and labels) into feat/lab (device, grown as needed)
void make_pairs(Ctx& c, int64_t np, const double* dpx, const double* dpy, PairSet& ps, DArr<float>& feat,
                DArr<float>& lab, int64_t feat_off, bool with_label) {
    cudaStream_t s = c.st();
    const int64_t nn = c.nnodes;
    ensure_moments(c);
    WalkView wv{c.nd_geom.p, c.nd_ch1.p, c.far_criteria, nn};
    DArr<int32_t> cnt;
    cnt.reserve((size_t)np + 1);
    ps.off.reserve((size_t)np + 1);
    k_far_count<<<grid_for(np, 128), 128, 0, s>>>(np, dpx, dpy, wv, cnt.p);
    VV_LAUNCH_CHECK();
    std::vector<int32_t> hc((size_t)np);
    VV_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, np * 4, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    std::vector<int64_t> ho((size_t)np + 1, 0);
    for (int64_t q = 0; q < np; q++) ho[q + 1] = ho[q] + hc[q];
    ps.npairs = ho[np];
    VV_CUDA(cudaMemcpyAsync(ps.off.p, ho.data(), (np + 1) * 8, cudaMemcpyHostToDevice, s));
    ps.node.reserve((size_t)ps.npairs + 1);
    ps.target.reserve((size_t)ps.npairs + 1);
    ps.back.reserve((size_t)ps.npairs + 1);
    k_far_fill<<<grid_for(np, 128), 128, 0, s>>>(np, dpx, dpy, wv, ps.off.p, ps.node.p, ps.target.p, 0);
    VV_LAUNCH_CHECK();
    const int64_t need = feat_off + ps.npairs;
    feat.reserve((size_t)need * NF + 1, true, (size_t)feat_off * NF, s);
    lab.reserve((size_t)need * 2 + 1, true, (size_t)feat_off * 2, s);
    if (ps.npairs > 0) {
        k_pair_samples<<<grid_for(ps.npairs, 128), 128, 0, s>>>(
            ps.npairs, ps.node.p, ps.target.p, dpx, dpy, c.nd_geom.p, c.nd_cm.p, c.nd_mom.p, c.nd_vf.p, c.nd_vl.p,
            c.x.p, c.y.p, c.g.p, feat.p + feat_off * NF, lab.p + feat_off * 2, ps.back.p, with_label ? 1 : 0);
        VV_LAUNCH_CHECK();
    }
    VV_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

namespace vvgpu {
namespace mlp {

// the moments of every node of the built tree, once per tree
void ensure_moments(Ctx& c) {
    if (c.mom_valid) return;
    cudaStream_t s = c.st();
    const int64_t nn = c.nnodes;
    c.nd_mom.reserve(12 * (size_t)nn + 12);
    k_leaf_moments<<<grid_for(nn, 128), 128, 0, s>>>(nn, c.nd_ch1.p, c.nd_vf.p, c.nd_vl.p, c.nd_cm.p, c.x.p, c.y.p,
                                                     c.g.p, c.nd_mom.p);
    VV_LAUNCH_CHECK();
    c.nd_arrive.reserve(nn + 1);
    VV_CUDA(cudaMemsetAsync(c.nd_arrive.p, 0, nn * sizeof(int32_t), s));
    k_inner_moments<<<grid_for(nn, 128), 128, 0, s>>>(nn, c.nd_ch1.p, c.nd_parent.p, c.nd_cm.p, c.nd_mom.p,
                                                      c.nd_arrive.p);
    VV_LAUNCH_CHECK();
    c.mom_valid = true;
}

}  // namespace mlp
}  // namespace vvgpu

extern "C" {

int vvgpu_mlp_create(int device, uint64_t seed, vvgpu_mlp** out) {
    if (!out) return VVGPU_ERR_ARG;
    *out = nullptr;
    vvgpu_mlp* m = nullptr;
    try {
        m = new vvgpu_mlp();
    } catch (std::bad_alloc&) {
        return VVGPU_ERR_NOMEM;
    }
    vvgpu_mlp& M = *m;
    M.device = device;
    try {
        VV_CUDA(cudaSetDevice(device));
        VV_CUDA(cudaStreamCreateWithFlags(&M.stream, cudaStreamNonBlocking));
        set_attrs();
        M.params.reserve(NPARAM);
        M.m1.reserve(NPARAM);
        M.m2.reserve(NPARAM);
        M.grad.reserve(NPARAM);
        M.img.reserve(NIMG);
        M.err.reserve(1);
        M.part.reserve(PSTRIDE);
        M.norm.reserve(NNORM);
        {
            std::vector<float> hn(NNORM, 1.f);
            for (int k = 0; k < NF; k++) hn[k] = 0.f;
            VV_CUDA(cudaMemcpyAsync(M.norm.p, hn.data(), NNORM * 4, cudaMemcpyHostToDevice, M.stream));
        }
        // Glorot-uniform weights, zero biases
        std::vector<float> h(NPARAM, 0.f);
        uint64_t st = seed;
        auto uni = [&](float a) { return (float)(((splitmix(st) >> 11) * 0x1.0p-53) * 2.0 - 1.0) * a; };
        const float a1 = std::sqrt(6.f / (NF + HID)), a2 = std::sqrt(6.f / (HID + HID)), a3 = std::sqrt(6.f / (HID + NOUT));
        for (int o = 0; o < HID; o++)
            for (int i = 0; i < NF; i++) h[P_W1 + o * KIN + i] = uni(a1);
        for (int q = 0; q < HID * HID; q++) h[P_W2 + q] = uni(a2);
        for (int q = 0; q < NOUT * HID; q++) h[P_W3 + q] = uni(a3);
        VV_CUDA(cudaMemcpyAsync(M.params.p, h.data(), NPARAM * 4, cudaMemcpyHostToDevice, M.stream));
        VV_CUDA(cudaMemsetAsync(M.m1.p, 0, NPARAM * 4, M.stream));
        VV_CUDA(cudaMemsetAsync(M.m2.p, 0, NPARAM * 4, M.stream));
        VV_CUDA(cudaMemsetAsync(M.img.p, 0, NIMG * 2, M.stream));
        VV_CUDA(cudaMemsetAsync(M.err.p, 0, 4, M.stream));
        refresh_image(M);
        VV_CUDA(cudaStreamSynchronize(M.stream));
    } catch (...) {
        if (M.stream) cudaStreamDestroy(M.stream);
        delete m;
        return VVGPU_ERR_CUDA;
    }
    *out = m;
    return 0;
}

int vvgpu_mlp_destroy(vvgpu_mlp* m) {
    if (!m) return 0;
    cudaSetDevice(m->device);
    if (m->stream) {
        cudaStreamSynchronize(m->stream);
        cudaStreamDestroy(m->stream);
    }
    delete m;
    return 0;
}

const char* vvgpu_mlp_last_error(const vvgpu_mlp* m) { return m ? m->last_error.c_str() : "null model"; }

int vvgpu_mlp_set_wait_limit(vvgpu_mlp* m, int64_t spins) {
    MLP_BEGIN(m)
    if (spins < 0) throw ApiError{VVGPU_ERR_ARG, "negative wait limit"};
    M.wait_spins = spins > (int64_t)MBAR_SPINS ? MBAR_SPINS : (uint32_t)spins;
    MLP_END
}

int64_t vvgpu_mlp_num_params(void) { return NPARAM; }

int vvgpu_mlp_get_params(vvgpu_mlp* m, float* out) {
    MLP_BEGIN(m)
    if (!out) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    VV_CUDA(cudaMemcpyAsync(out, M.params.p, NPARAM * 4, cudaMemcpyDeviceToHost, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

int vvgpu_mlp_set_params(vvgpu_mlp* m, const float* in) {
    MLP_BEGIN(m)
    if (!in) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    VV_CUDA(cudaMemcpyAsync(M.params.p, in, NPARAM * 4, cudaMemcpyHostToDevice, M.stream));
    VV_CUDA(cudaMemsetAsync(M.m1.p, 0, NPARAM * 4, M.stream));
    VV_CUDA(cudaMemsetAsync(M.m2.p, 0, NPARAM * 4, M.stream));
    M.steps = 0;
    refresh_image(M);
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

int vvgpu_mlp_set_norm(vvgpu_mlp* m, const float* norm) {
    MLP_BEGIN(m)
    if (!norm) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    VV_CUDA(cudaMemcpyAsync(M.norm.p, norm, NNORM * 4, cudaMemcpyHostToDevice, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

int vvgpu_mlp_get_norm(vvgpu_mlp* m, float* norm) {
    MLP_BEGIN(m)
    if (!norm) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    VV_CUDA(cudaMemcpyAsync(norm, M.norm.p, NNORM * 4, cudaMemcpyDeviceToHost, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

// standardisation from the samples (every k-th sample, at most FIT_MAX of them): per-feature
// mean and 1 / standard deviation (1 where the deviation is 0), per-output root mean square
// of the labels
constexpr int64_t FIT_MAX = 4000000;
int vvgpu_mlp_fit_norm(vvgpu_mlp* m) {
    MLP_BEGIN(m)
    const int64_t total = M.nsamples;
    if (total <= 0) throw ApiError{VVGPU_ERR_ARG, "no samples"};
    const int64_t stride = (total + FIT_MAX - 1) / FIT_MAX;
    const int64_t n = (total + stride - 1) / stride;
    std::vector<float> f((size_t)n * NF), l((size_t)n * 2);
    VV_CUDA(cudaMemcpy2DAsync(f.data(), NF * 4, M.feat.p, stride * NF * 4, NF * 4, n, cudaMemcpyDeviceToHost,
                              M.stream));
    VV_CUDA(cudaMemcpy2DAsync(l.data(), 2 * 4, M.lab.p, stride * 2 * 4, 2 * 4, n, cudaMemcpyDeviceToHost, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    std::vector<double> s1(NF, 0.), s2(NF, 0.), ls(2, 0.);
    for (int64_t i = 0; i < n; i++) {
        for (int k = 0; k < NF; k++) {
            const double v = f[(size_t)i * NF + k];
            s1[k] += v;
            s2[k] += v * v;
        }
        for (int o = 0; o < 2; o++) ls[o] += (double)l[(size_t)i * 2 + o] * l[(size_t)i * 2 + o];
    }
    std::vector<float> hn(NNORM);
    for (int k = 0; k < NF; k++) {
        const double mu = s1[k] / (double)n, var = std::max(0., s2[k] / (double)n - mu * mu);
        hn[k] = (float)mu;
        hn[NF + k] = var > 0. ? (float)(1. / std::sqrt(var)) : 1.f;
    }
    for (int o = 0; o < 2; o++) {
        const double r = std::sqrt(ls[o] / (double)n);
        hn[2 * NF + o] = r > 0. ? (float)r : 1.f;
    }
    VV_CUDA(cudaMemcpyAsync(M.norm.p, hn.data(), NNORM * 4, cudaMemcpyHostToDevice, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

int vvgpu_mlp_set_samples(vvgpu_mlp* m, int64_t n, const float* feat, const float* lab) {
    MLP_BEGIN(m)
    if (n < 0 || (n > 0 && (!feat || !lab))) throw ApiError{VVGPU_ERR_ARG, "bad sample arrays"};
    M.feat.reserve((size_t)n * NF + 1);
    M.lab.reserve((size_t)n * 2 + 1);
    if (n > 0) {
        VV_CUDA(cudaMemcpyAsync(M.feat.p, feat, n * NF * 4, cudaMemcpyHostToDevice, M.stream));
        VV_CUDA(cudaMemcpyAsync(M.lab.p, lab, n * 2 * 4, cudaMemcpyHostToDevice, M.stream));
    }
    M.nsamples = n;
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

int64_t vvgpu_mlp_num_samples(const vvgpu_mlp* m) { return m ? m->nsamples : -1; }

int vvgpu_mlp_get_samples(vvgpu_mlp* m, int64_t first, int64_t n, float* feat, float* lab) {
    MLP_BEGIN(m)
    if (first < 0 || n < 0 || first + n > M.nsamples) throw ApiError{VVGPU_ERR_ARG, "sample range"};
    if (n > 0) {
        if (feat) VV_CUDA(cudaMemcpyAsync(feat, M.feat.p + first * NF, n * NF * 4, cudaMemcpyDeviceToHost, M.stream));
        if (lab) VV_CUDA(cudaMemcpyAsync(lab, M.lab.p + first * 2, n * 2 * 4, cudaMemcpyDeviceToHost, M.stream));
    }
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

int vvgpu_mlp_add_samples(vvgpu_mlp* m, vvgpu_ctx* h, int64_t np, const double* px, const double* py,
                          int64_t* added) {
    MLP_BEGIN(m)
    if (!h || np < 0 || (np > 0 && (!px || !py))) throw ApiError{VVGPU_ERR_ARG, "bad arguments"};
    Ctx& c = h->c;
    VV_CUDA(cudaSetDevice(c.device));
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    PairSet ps;
    ps.pts.reserve(2 * (size_t)np + 2);
    cudaStream_t s = c.st();
    if (np > 0) {
        VV_CUDA(cudaMemcpyAsync(ps.pts.p, px, np * 8, cudaMemcpyHostToDevice, s));
        VV_CUDA(cudaMemcpyAsync(ps.pts.p + np, py, np * 8, cudaMemcpyHostToDevice, s));
    }
    VV_CUDA(cudaStreamSynchronize(M.stream));
    make_pairs(c, np, ps.pts.p, ps.pts.p + np, ps, M.feat, M.lab, M.nsamples, true);
    M.nsamples += ps.npairs;
    if (added) *added = ps.npairs;
    MLP_END
}

// loss = (1/n) sum |y - t|^2 over the first n samples; its gradient (and the loss) without
// changing the weights
int vvgpu_mlp_gradient(vvgpu_mlp* m, int64_t n, float* grad, float* loss) {
    MLP_BEGIN(m)
    if (n <= 0 || n > M.nsamples) throw ApiError{VVGPU_ERR_ARG, "sample count"};
    const int64_t ntiles = (n + TILE - 1) / TILE;
    if (ntiles > 65535) throw ApiError{VVGPU_ERR_LIMIT, "at most 65535 tiles per gradient"};
    std::vector<int64_t> ids((size_t)ntiles * TILE, -1);
    for (int64_t i = 0; i < n; i++) ids[i] = i;
    M.ids.reserve(ids.size());
    M.loss.reserve(1);
    VV_CUDA(cudaMemsetAsync(M.err.p, 0, 4, M.stream));
    VV_CUDA(cudaMemcpyAsync(M.ids.p, ids.data(), ids.size() * 8, cudaMemcpyHostToDevice, M.stream));
    train_batch(M, M.ids.p, (int)ntiles, 1.f / (float)n, 0.f, M.grad.p, M.loss.p);
    check_err(M);
    if (grad) VV_CUDA(cudaMemcpyAsync(grad, M.grad.p, NPARAM * 4, cudaMemcpyDeviceToHost, M.stream));
    float L = 0.f;
    VV_CUDA(cudaMemcpyAsync(&L, M.loss.p, 4, cudaMemcpyDeviceToHost, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    if (loss) *loss = L / (float)n;
    MLP_END
}

// Adam on mini-batches of `batch` samples (a multiple of 128), a fresh shuffle per epoch;
// loss_per_epoch[e] = mean squared error over the epoch's batches (before each update)
int vvgpu_mlp_train(vvgpu_mlp* m, int64_t epochs, int64_t batch, float lr, uint64_t seed, float* loss_per_epoch) {
    MLP_BEGIN(m)
    if (epochs < 0 || batch <= 0 || batch % TILE || !(lr > 0.f) || M.nsamples <= 0)
        throw ApiError{VVGPU_ERR_ARG, "bad training arguments"};
    const int64_t n = M.nsamples;
    const int64_t nb = (n + batch - 1) / batch;
    const int64_t tiles_per_batch = batch / TILE;
    std::vector<int64_t> ids((size_t)nb * batch, -1);
    M.ids.reserve(ids.size());
    M.loss.reserve((size_t)nb);
    uint64_t st = seed;
    std::vector<float> hl((size_t)nb);
    VV_CUDA(cudaMemsetAsync(M.err.p, 0, 4, M.stream));
    for (int64_t e = 0; e < epochs; e++) {
        std::iota(ids.begin(), ids.begin() + n, (int64_t)0);
        for (int64_t i = n - 1; i > 0; i--) std::swap(ids[i], ids[splitmix(st) % (uint64_t)(i + 1)]);
        VV_CUDA(cudaMemcpyAsync(M.ids.p, ids.data(), ids.size() * 8, cudaMemcpyHostToDevice, M.stream));
        // cosine decay from lr to lr / 20 over the epochs
        const double ph = epochs > 1 ? (double)e / (double)(epochs - 1) : 0.;
        const float lre = (float)(lr * (0.05 + 0.95 * 0.5 * (1. + std::cos(C_PI * ph))));
        for (int64_t b = 0; b < nb; b++) {
            const int64_t cnt = std::min<int64_t>(batch, n - b * batch);
            const int nt = (int)((cnt + TILE - 1) / TILE);
            train_batch(M, M.ids.p + b * batch, nt, 1.f / (float)cnt, lre, nullptr, M.loss.p + b);
            (void)tiles_per_batch;
        }
        VV_CUDA(cudaMemcpyAsync(hl.data(), M.loss.p, nb * 4, cudaMemcpyDeviceToHost, M.stream));
        VV_CUDA(cudaStreamSynchronize(M.stream));
        double tot = 0;
        for (int64_t b = 0; b < nb; b++) tot += hl[b];
        if (loss_per_epoch) loss_per_epoch[e] = (float)(tot / (double)n);
    }
    check_err(M);
    MLP_END
}

int vvgpu_mlp_forward(vvgpu_mlp* m, int64_t n, const float* feat, float* y) {
    MLP_BEGIN(m)
    if (n < 0 || (n > 0 && (!feat || !y))) throw ApiError{VVGPU_ERR_ARG, "bad arrays"};
    DArr<float> f, o;
    f.reserve((size_t)n * NF + 1);
    o.reserve((size_t)n * 2 + 1);
    VV_CUDA(cudaMemsetAsync(M.err.p, 0, 4, M.stream));
    if (n > 0) VV_CUDA(cudaMemcpyAsync(f.p, feat, n * NF * 4, cudaMemcpyHostToDevice, M.stream));
    forward_device(M, n, f.p, o.p);
    check_err(M);
    if (n > 0) VV_CUDA(cudaMemcpyAsync(y, o.p, n * 2 * 4, cudaMemcpyDeviceToHost, M.stream));
    VV_CUDA(cudaStreamSynchronize(M.stream));
    MLP_END
}

// MConvectiveFast::velocity(p) of the built tree plus, per far cell of p's leaf, the
// network's residual (the learned correction); npairs_out = the pairs evaluated
int vvgpu_velocity_points_learned(vvgpu_ctx* h, vvgpu_mlp* m, int64_t np, const double* px, const double* py,
                                  double* vx, double* vy, int64_t* npairs_out) {
    MLP_BEGIN(m)
    if (!h || np < 0 || (np > 0 && (!px || !py || !vx || !vy))) throw ApiError{VVGPU_ERR_ARG, "bad arguments"};
    Ctx& c = h->c;
    VV_CUDA(cudaSetDevice(c.device));
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    ensure_full_lists(c);
    cudaStream_t s = c.st();
    PairSet ps;
    ps.pts.reserve(4 * (size_t)np + 4);
    if (np > 0) {
        VV_CUDA(cudaMemcpyAsync(ps.pts.p, px, np * 8, cudaMemcpyHostToDevice, s));
        VV_CUDA(cudaMemcpyAsync(ps.pts.p + np, py, np * 8, cudaMemcpyHostToDevice, s));
    }
    velocity_points_on_device(c, np, ps.pts.p, ps.pts.p + np, ps.pts.p + 2 * np, ps.pts.p + 3 * np);
    DArr<float> feat, lab, yv;
    make_pairs(c, np, ps.pts.p, ps.pts.p + np, ps, feat, lab, 0, false);
    yv.reserve(2 * (size_t)ps.npairs + 2);
    VV_CUDA(cudaMemsetAsync(M.err.p, 0, 4, M.stream));
    forward_device(M, ps.npairs, feat.p, yv.p);
    check_err(M);
    if (np > 0) {
        k_apply_correction<<<grid_for(np, 128), 128, 0, M.stream>>>(np, ps.off.p, yv.p, ps.back.p, ps.pts.p + 2 * np,
                                                                   ps.pts.p + 3 * np);
        MLP_LAUNCH_CHECK();
        VV_CUDA(cudaMemcpyAsync(vx, ps.pts.p + 2 * np, np * 8, cudaMemcpyDeviceToHost, M.stream));
        VV_CUDA(cudaMemcpyAsync(vy, ps.pts.p + 3 * np, np * 8, cudaMemcpyDeviceToHost, M.stream));
    }
    VV_CUDA(cudaStreamSynchronize(M.stream));
    if (npairs_out) *npairs_out = ps.npairs;
    MLP_END
}

}  // extern "C"
