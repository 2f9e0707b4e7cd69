// The learned far-field correction inside the convective pass, and the plain tree as its
// judge and fallback.
//
// The reference's far field (MConvectiveFast.cpp:48-69) expands, about each leaf's centre,
// the two monopoles (+/- centroids) of every far node of the leaf.  Here the MLP of
// learned.cu adds, for every (leaf, far node) pair, its prediction of the part of that
// node's exact velocity the monopoles miss, evaluated at the leaf's centre; the sum over the
// leaf's far nodes corrects the constant terms T1, T2 of the leaf's expansion.  A looser
// opening criterion (theta = 0.8, farCriteria 3.125) then keeps about the accuracy of the
// plain theta = 0.5 tree.
//
// Pairs: the near/far walk keeps every leaf's far nodes (lists.cu, keep_far), compacted in
// leaf order.  One pass over them in tiles of 128 (k_mlp_far_pairs): the per-node inputs
// are precomputed once per tree (k_node_inputs: the 18 cell features, standardised, BF16),
// the two target-offset inputs are formed per pair; layers 1 and 2 run on the tensor cores
// (tcgen05.mma kind::f16, BF16 operands in shared memory, FP32 accumulators in tensor
// memory), the 2-wide output layer on the CUDA cores with the BF16 weights.  Each pair's
// velocity goes to an FP32 buffer, and one warp per leaf sums its pairs in a fixed order
// (deterministic) into a copy of the leaf's coefficients.
//
// Judge: velocity(p) of the plain tree at the judge's far criterion, at sampled vortices
// (convective.cu, k_judge), against the learned pass's convective increments there.  If the
// relative rms gap exceeds the bound, the increments are undone and the pass is redone with
// the plain tree at the judge's criterion (near/far walk again, plain expansion).
#include "frame.cuh"
#include "mlp.cuh"
#include "pair.cuh"

namespace vvgpu {

namespace mlp {

constexpr int NCF = 18;   // cell inputs; inputs 18, 19 are the target's offset

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Per node, one 64-byte record (4 x uint4) with everything a pair reads about the node:
//   q0, q1: standardised cell inputs 0..15 (the features of k_pair_samples, learned.cu), BF16
//   q2: inputs 16, 17 (BF16 pair), 1 / s, G s^2 / 2pi (FP32 bits), 0
//   q3: node centre x, y in its anchor frame and the anchor (FP32, frame.cuh)
// The factor back to velocity is back = G s^2 / (2 pi d^3).  A node with no circulation or
// no extent gets 0 there (no correction), as its samples have.
__global__ void k_node_inputs(int64_t nn, const double4* __restrict__ geom, const double* __restrict__ cm,
                              const double* __restrict__ mom, const float* __restrict__ norm,
                              const float4* __restrict__ nf_geo, const float2* __restrict__ nf_k, uint4* nrec) {
    const int64_t S = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (S >= nn) return;
    const double4 gm = geom[S];
    const double* c = cm + 6 * S;
    const double* mo = mom + 12 * S;
    const double sz = gm.z + gm.w;
    const double G = c[2] - c[5];
    float f[NCF];
#pragma unroll
    for (int k = 0; k < NCF; k++) f[k] = 0.f;
    double is = 0., back0 = 0.;
    if (G > 0. && sz > 0.) {
        const double iG = 1. / G;
        is = 1. / sz;
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
        back0 = G * sz * sz * (0.5 / C_PI);
    }
    uint32_t b[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
        b[k] = pack_bf16((f[2 * k] - norm[2 * k]) * norm[NF + 2 * k], (f[2 * k + 1] - norm[2 * k + 1]) * norm[NF + 2 * k + 1]);
    const float4 gq = nf_geo[S];
    const float2 kq = nf_k[S];
    uint4* r = nrec + 4 * S;
    r[0] = make_uint4(b[0], b[1], b[2], b[3]);
    r[1] = make_uint4(b[4], b[5], b[6], b[7]);
    r[2] = make_uint4(b[8], __float_as_uint((float)is), __float_as_uint((float)back0), 0u);
    r[3] = make_uint4(__float_as_uint(gq.x), __float_as_uint(gq.y), __float_as_uint(kq.x), __float_as_uint(kq.y));
}

__device__ __forceinline__ float tanh_fast(float x) {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The network's tanh-form GELU of (z0 + b0, z1 + b1) with the hardware tanh, rounded to a
// BF16 pair (the rounding is far coarser than the approximation)
__device__ __forceinline__ uint32_t gelu2_bf16(float z0, float z1, float2 b) {
    const uint64_t z = fadd2(f2(z0, z1), f2(b.x, b.y));
    const uint64_t a = fmul2(fmul2(z, z), f2(GA, GA));
    const uint64_t u = fmul2(ffma2(a, z, z), f2(GC, GC));
    float u0, u1;
    uf2(u, u0, u1);
    const uint64_t hz = fmul2(z, f2(0.5f, 0.5f));
    const uint64_t h = ffma2(hz, f2(tanh_fast(u0), tanh_fast(u1)), hz);
    float h0, h1;
    uf2(h, h0, h1);
    return pack_bf16(h0, h1);
}

// 16-byte chunk q (8 consecutive K elements) of row r of a K-major core-matrix operand
__device__ __forceinline__ uint4* chunk_at(__nv_bfloat16* base, int r, int q, int kc) {
    return reinterpret_cast<uint4*>(base + tile_off(r, 8 * q, kc));
}

constexpr int PT_TMEM = 64;   // Z1, then Z2 over it (Z1 is read out before the second MMA)
constexpr int PT_CTAS = 7;    // resident per SM (shared memory ~30 KB, 64 TMEM columns each)
static_assert(PT_CTAS * PT_TMEM <= 512, "tensor-memory columns of the resident CTAs");
struct PairSmem {
    __nv_bfloat16 w[NIMG_FWD];     // W1, W2 and W3 images (learned.cu's layout)
    // the tile's inputs, then its first hidden layer, then its second: each is read by its
    // MMA, which has completed before the next is written
    __nv_bfloat16 h1[TILE * HID];
    float b1[HID], b2[HID];
    float b3[NOUT], onorm[NOUT], inorm[4];
    uint64_t mbar;
    uint32_t tmem;
};

// Velocity correction of every (leaf, far node) pair, pv[p] = network output times the
// output scale times the pair's back factor.  Persistent over tiles of 128 pairs.
__global__ void __launch_bounds__(TILE, PT_CTAS) k_mlp_far_pairs(int64_t np, const int32_t* __restrict__ pnode,
                                                       const int32_t* __restrict__ plnode,
                                                       const uint4* __restrict__ nrec,
                                                       const __nv_bfloat16* __restrict__ img,
                                                       const float* __restrict__ params,
                                                       const float* __restrict__ norm, float2* __restrict__ pv,
                                                       int* err, uint32_t spins) {
    extern __shared__ __align__(128) unsigned char smraw[];
    PairSmem& S = *reinterpret_cast<PairSmem*>(smraw);
    __nv_bfloat16* const x0 = S.h1;  // [TILE][KIN] at the start of h1's space
    const int tid = threadIdx.x, w = tid >> 5;
    for (int i = tid; i < NIMG_FWD; i += TILE) S.w[i] = img[i];
    for (int i = tid; i < HID; i += TILE) {
        S.b1[i] = params[P_B1 + i];
        S.b2[i] = params[P_B2 + i];
    }
    if (tid < NOUT) {
        S.b3[tid] = params[P_B3 + tid];
        S.onorm[tid] = norm[2 * NF + tid];
        S.inorm[tid] = norm[NCF + tid];            // means of inputs 18, 19
        S.inorm[2 + tid] = norm[NF + NCF + tid];   // their inverse deviations
    }
    if (tid == 0) mbar_init(&S.mbar);
    if (w == 0) tmem_alloc(&S.tmem, PT_TMEM);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = S.tmem;
    uint32_t phase = 0, lost = 2;  // lost: the phase whose completion a timed-out wait missed
    bool ok = true;
    const int64_t ntiles = (np + TILE - 1) / TILE;
    // The gather is pipelined over the tiles: the pair indices of the next tile are read at
    // the start of a tile and its node records right after the tile's first MMA is issued,
    // so they arrive while the tile's layers run; the inputs are formed at the next tile.
    auto fetch_idx = [&](int64_t tile, int32_t& node, int32_t& lnode) {
        const int64_t p = tile * TILE + tid;
        node = lnode = -1;
        if (tile < ntiles && p < np) {
            node = pnode[p];
            lnode = plnode[p];
        }
    };
    uint4 r0 = make_uint4(0, 0, 0, 0), r1 = r0, r2 = r0, r3 = r0, rl = r0;  // records of the tile
    auto fetch_rec = [&](int32_t node, int32_t lnode) {
        if (node >= 0) {
            const uint4* rn = nrec + 4 * (size_t)node;
            r0 = rn[0];
            r1 = rn[1];
            r2 = rn[2];
            r3 = rn[3];
            rl = nrec[4 * (size_t)lnode + 3];  // the leaf's centre and anchor
        }
    };
    int32_t nx, nxl;
    fetch_idx(blockIdx.x, nx, nxl);
    fetch_rec(nx, nxl);
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t p = tile * TILE + tid;
        const bool live = nx >= 0;
        fetch_idx(tile + gridDim.x, nx, nxl);
        uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0, c2 = c0;
        float back = 0.f;
        if (live) {
            c0 = r0;
            c1 = r1;
            const uint4 a = r2, gN = r3, gL = rl;
            // the leaf centre's offset from the node centre in FP32 from the node frames (the
            // shift between two anchors is exact); the inputs are rounded to BF16 anyway
            const float dx = (__uint_as_float(gL.z) - __uint_as_float(gN.z)) +
                             (__uint_as_float(gL.x) - __uint_as_float(gN.x));
            const float dy = (__uint_as_float(gL.w) - __uint_as_float(gN.w)) +
                             (__uint_as_float(gL.y) - __uint_as_float(gN.y));
            const float is = __uint_as_float(a.y), back0 = __uint_as_float(a.z);
            const float o0 = (dx * is - S.inorm[0]) * S.inorm[2];
            const float o1 = (dy * is - S.inorm[1]) * S.inorm[3];
            c2 = make_uint4(a.x, pack_bf16(o0, o1), 0u, 0u);  // inputs 16..19, then zeros
            const float d2 = dx * dx + dy * dy;
            const float r = rsqrtf(d2);
            back = (back0 > 0.f && d2 > 0.f) ? back0 * (r * r * r) : 0.f;
        }
        *chunk_at(x0, tid, 0, KIN / 8) = c0;
        *chunk_at(x0, tid, 1, KIN / 8) = c1;
        *chunk_at(x0, tid, 2, KIN / 8) = c2;
        *chunk_at(x0, tid, 3, KIN / 8) = make_uint4(0, 0, 0, 0);
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) { mma_issue(tm, x0, S.w + I_W1, KIN, HID, false); mma_commit(&S.mbar); }
        fetch_rec(nx, nxl);
        ok = __syncthreads_and(mbar_wait(&S.mbar, phase, spins));
        if (!ok) lost = phase;
        phase ^= 1;
        fence_after();
        if (!ok) break;
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, c), v);
            uint32_t q[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                q[j] = gelu2_bf16(v[2 * j], v[2 * j + 1], *reinterpret_cast<const float2*>(&S.b1[c + 2 * j]));
            *chunk_at(S.h1, tid, c / 8, HID / 8) = make_uint4(q[0], q[1], q[2], q[3]);
            *chunk_at(S.h1, tid, c / 8 + 1, HID / 8) = make_uint4(q[4], q[5], q[6], q[7]);
        }
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) { mma_issue(tm, S.h1, S.w + I_W2, HID, HID, false); mma_commit(&S.mbar); }
        ok = __syncthreads_and(mbar_wait(&S.mbar, phase, spins));
        if (!ok) lost = phase;
        phase ^= 1;
        fence_after();
        if (!ok) break;
        for (int c = 0; c < HID; c += 16) {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, c), v);
            uint32_t q[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                q[j] = gelu2_bf16(v[2 * j], v[2 * j + 1], *reinterpret_cast<const float2*>(&S.b2[c + 2 * j]));
            *chunk_at(S.h1, tid, c / 8, HID / 8) = make_uint4(q[0], q[1], q[2], q[3]);
            *chunk_at(S.h1, tid, c / 8 + 1, HID / 8) = make_uint4(q[4], q[5], q[6], q[7]);
        }
        // output layer on the tensor cores too (N padded to 16), as the training forward
        fence_smem_to_mma();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) { mma_issue(tm, S.h1, S.w + I_W3, HID, NOUTP, false); mma_commit(&S.mbar); }
        ok = __syncthreads_and(mbar_wait(&S.mbar, phase, spins));
        if (!ok) lost = phase;
        phase ^= 1;
        fence_after();
        if (!ok) break;
        {
            float v[16];
            tmem_ld16(tmem_lane_addr(tm, w, 0), v);
            if (p < np)
                pv[p] = make_float2((v[0] + S.b3[0]) * S.onorm[0] * back, (v[1] + S.b3[1]) * S.onorm[1] * back);
        }
        fence_before();
        __syncthreads();
        fence_after();
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    if (lost != 2) mbar_wait(&S.mbar, lost, MBAR_SPINS);  // the abandoned MMA lands first
    fence_before();
    __syncthreads();
    if (w == 0) tmem_free(tm, PT_TMEM);
}

// Leaf L's coefficients plus the sum of its pairs' corrections (one warp per leaf: lane
// partials in pair order, then a fixed shuffle tree).
__global__ void k_far_leaf_sum(int64_t nl, const int32_t* __restrict__ off, const float2* __restrict__ pv,
                               const double4* __restrict__ taylor, double4* out) {
    const int64_t L = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (L >= nl) return;
    double sx = 0., sy = 0.;
    for (int32_t k = off[L] + lane; k < off[L + 1]; k += 32) {
        const float2 v = pv[k];
        sx += (double)v.x;
        sy += (double)v.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (lane == 0) {
        double4 t = taylor[L];
        t.x += sx;
        t.y += sy;
        out[L] = t;
    }
}

// (learned - before) at the judged vortices: out[2 k ..]
__global__ void k_judge_gather(int64_t nt, const int32_t* __restrict__ idx, const double* __restrict__ vx,
                               const double* __restrict__ vy, const double* __restrict__ vx0,
                               const double* __restrict__ vy0, double* out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nt) return;
    const int32_t i = idx[q];
    out[2 * q] = vx[i] - vx0[i];
    out[2 * q + 1] = vy[i] - vy0[i];
}

uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

size_t pair_smem() { return sizeof(PairSmem); }

}  // namespace mlp

// The learned convective pass (see the top of this file); returns the judge's verdict.
void convective_learned(Ctx& c, vvgpu_mlp& M, const vvgpu_judge_cfg* jc, vvgpu_judge_out* jo) {
    using namespace mlp;
    cudaStream_t s = c.st();
    if (jc && (jc->targets < 0 || !(jc->far_criteria > 0) || !(jc->bound >= 0)))
        throw ApiError{VVGPU_ERR_ARG, "bad judge parameters"};
    const int64_t n = c.n, nl = c.nleaves, nn = c.nnodes;
    vvgpu_judge_out res{};
    res.gap_rms = res.gap_max = 0.;
    if (n == 0 || nl == 0) {
        if (jo) *jo = res;
        return;
    }
    // the far nodes of every leaf (kept by the walk; one more walk if the lists were built
    // without them)
    c.keep_far = true;
    if (!c.far_kept) {
        c.lists_full = false;
        ensure_full_lists(c);
    }
    ensure_moments(c);
    // the model's weights, as its last call left them
    VV_CUDA(cudaStreamSynchronize(M.stream));
    c.ln_rec.reserve(4 * (size_t)nn + 4);
    if (!c.nf_geo.p || !c.nf_k.p) throw ApiError{VVGPU_ERR_STATE, "node frames missing"};
    k_node_inputs<<<grid_for(nn, 128), 128, 0, s>>>(nn, c.nd_geom.p, c.nd_cm.p, c.nd_mom.p, M.norm.p, c.nf_geo.p,
                                                    c.nf_k.p, c.ln_rec.p);
    VV_LAUNCH_CHECK();
    const int64_t np = c.n_far_pairs;
    c.ln_pv.reserve(np + 1);
    VV_CUDA(cudaMemsetAsync(M.err.p, 0, 4, s));
    {
        KernelTimer kt(c, VVGPU_T_LEARNED);
        if (np > 0) {
            VV_CUDA(cudaFuncSetAttribute(k_mlp_far_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)pair_smem()));
            const int64_t ntiles = (np + TILE - 1) / TILE;
            // persistent: exactly the CTAs that fit at once (PT_CTAS per SM by registers, shared
            // and tensor memory; the runtime's occupancy query answered 1 for this kernel, which
            // left six of every seven slots empty)
            int dev_sms = 0;
            VV_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, c.device));
            const int grid = (int)std::min<int64_t>(ntiles, (int64_t)dev_sms * PT_CTAS);
            k_mlp_far_pairs<<<grid, TILE, pair_smem(), s>>>(np, c.lf_far_node.p, c.lf_far_leaf.p, c.ln_rec.p,
                                                            M.img.p, M.params.p, M.norm.p,
                                                            c.ln_pv.p, M.err.p, M.wait_spins);
            VV_LAUNCH_CHECK();
        }
        c.lf_taylor_l.reserve(nl + 1);
        k_far_leaf_sum<<<grid_for(nl, 8), 256, 0, s>>>(nl, c.lf_far_off.p, c.ln_pv.p, c.lf_taylor.p, c.lf_taylor_l.p);
        VV_LAUNCH_CHECK();
    }
    if (read_i32(c, M.err.p)) throw ApiError{VVGPU_ERR_TIMEOUT, "tensor-core wait timed out"};
    res.pairs = np;
    // the increments are judged: keep the velocities they add to
    const bool judge = jc && jc->targets > 0;
    if (judge) {
        c.ln_v0.reserve(2 * (size_t)n);
        VV_CUDA(cudaMemcpyAsync(c.ln_v0.p, c.vx.p, n * 8, cudaMemcpyDeviceToDevice, s));
        VV_CUDA(cudaMemcpyAsync(c.ln_v0.p + n, c.vy.p, n * 8, cudaMemcpyDeviceToDevice, s));
    }
    std::swap(c.lf_taylor, c.lf_taylor_l);  // the convective pass reads lf_taylor
    try {
        convective(c);
    } catch (...) {
        std::swap(c.lf_taylor, c.lf_taylor_l);
        throw;
    }
    std::swap(c.lf_taylor, c.lf_taylor_l);
    if (!judge) {
        if (jo) *jo = res;
        return;
    }
    // judge: velocity(p) of the plain tree at sampled vortices
    const int64_t nt = jc->targets;
    std::vector<int32_t> idx(nt);
    const uint64_t base = mix64(jc->seed * 0x9E3779B97F4A7C15ull + (uint64_t)(++c.judge_calls));
    for (int64_t k = 0; k < nt; k++) idx[k] = (int32_t)(mix64(base + (uint64_t)k) % (uint64_t)n);
    c.ln_idx.reserve(nt + 1);
    c.ln_judge.reserve(5 * (size_t)nt + 1);
    VV_CUDA(cudaMemcpyAsync(c.ln_idx.p, idx.data(), nt * 4, cudaMemcpyHostToDevice, s));
    {
        KernelTimer kt(c, VVGPU_T_JUDGE);
        judge_velocity(c, nt, c.ln_idx.p, jc->far_criteria, c.ln_judge.p);
        k_judge_gather<<<grid_for(nt, 128), 128, 0, s>>>(nt, c.ln_idx.p, c.vx.p, c.vy.p, c.ln_v0.p, c.ln_v0.p + n,
                                                         c.ln_judge.p + 3 * nt);
        VV_LAUNCH_CHECK();
    }
    std::vector<double> hj(5 * (size_t)nt);
    VV_CUDA(cudaMemcpyAsync(hj.data(), c.ln_judge.p, 5 * nt * 8, cudaMemcpyDeviceToHost, s));
    VV_CUDA(cudaStreamSynchronize(s));
    double se = 0, sm = 0, emax = 0;
    int64_t cnt = 0;
    for (int64_t k = 0; k < nt; k++) {
        if (hj[3 * k + 2] == 0.) continue;
        const double jx = hj[3 * k], jy = hj[3 * k + 1];
        const double lx = hj[3 * nt + 2 * k], ly = hj[3 * nt + 2 * k + 1];
        const double e2 = (lx - jx) * (lx - jx) + (ly - jy) * (ly - jy);
        const double ux = jx - c.inf_vx, uy = jy - c.inf_vy;
        se += e2;
        sm += ux * ux + uy * uy;
        emax = std::max(emax, std::sqrt(e2));
        cnt++;
    }
    res.judged = cnt;
    res.gap_rms = (sm > 0) ? std::sqrt(se / sm) : (se > 0 ? INFINITY : 0.);
    res.gap_max = (sm > 0) ? emax / std::sqrt(sm / (double)std::max<int64_t>(cnt, 1)) : emax;
    if (!(res.gap_rms <= jc->bound)) {
        // revert: undo the increments, then the plain tree at the judge's criterion
        res.reverted = 1;
        VV_CUDA(cudaMemcpyAsync(c.vx.p, c.ln_v0.p, n * 8, cudaMemcpyDeviceToDevice, s));
        VV_CUDA(cudaMemcpyAsync(c.vy.p, c.ln_v0.p + n, n * 8, cudaMemcpyDeviceToDevice, s));
        c.far_criteria = jc->far_criteria;
        c.keep_far = false;
        c.lists_full = false;
        c.far_kept = false;
        ensure_full_lists(c);
        convective(c);
        c.keep_far = true;  // the next tree's walk keeps its far nodes again
    }
    if (jo) *jo = res;
}

}  // namespace vvgpu

using namespace vvgpu;

extern "C" int vvgpu_convective_learned(vvgpu_ctx* h, vvgpu_mlp* m, const vvgpu_judge_cfg* judge,
                                        vvgpu_judge_out* out) {
    if (!h || !m) return VVGPU_ERR_ARG;
    Ctx& c = h->c;
    try {
        VV_CUDA(cudaSetDevice(c.device));
        if (m->device != c.device) throw ApiError{VVGPU_ERR_ARG, "model and context are on different devices"};
        if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
        convective_learned(c, *m, judge, out);
    } catch (ApiError& e) {
        c.last_error = e.msg;
        return e.code;
    } catch (CudaError& e) {
        c.last_error = std::string(e.what) + ": " + cudaGetErrorString(e.err);
        return VVGPU_ERR_CUDA;
    } catch (std::bad_alloc&) {
        c.last_error = "host allocation failed";
        return VVGPU_ERR_NOMEM;
    }
    return VVGPU_OK;
}

extern "C" int vvgpu_keep_far_lists(vvgpu_ctx* h, int on) {
    if (!h) return VVGPU_ERR_ARG;
    h->c.keep_far = on != 0;
    return VVGPU_OK;
}
