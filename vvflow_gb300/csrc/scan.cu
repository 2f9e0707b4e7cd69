// Device-wide exclusive prefix sum over int32 (used by the tree partition and list builds).
// Three passes: per-block totals, a one-block scan of the totals, per-block rescan + offset;
// inputs of at most four tiles take a single one-block pass.
#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

// Inclusive block scan of one value per thread; returns the inclusive prefix and the block total.
__device__ __forceinline__ int32_t block_inclusive(int32_t v, int32_t* warp_tot, int32_t& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_tot[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int32_t w = (lane < SCAN_BLOCK / 32) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < SCAN_BLOCK / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    total = warp_tot[SCAN_BLOCK / 32 - 1];
    int32_t r = v + (wid ? warp_tot[wid - 1] : 0);
    __syncthreads();
    return r;
}

__global__ void k_tile_sums(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums) {
    __shared__ int32_t wt[SCAN_BLOCK / 32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < n) s += in[base + k];
    int32_t total;
    block_inclusive(s, wt, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int32_t* __restrict__ sums, int64_t nb, int32_t* __restrict__ total_out) {
    __shared__ int32_t wt[SCAN_BLOCK / 32];
    int32_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += SCAN_BLOCK) {
        int64_t i = b0 + threadIdx.x;
        int32_t v = (i < nb) ? sums[i] : 0;
        int32_t tot;
        int32_t inc = block_inclusive(v, wt, tot);
        if (i < nb) sums[i] = carry + inc - v;
        carry += tot;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_tile_scan(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ sums,
                            int32_t* __restrict__ out) {
    __shared__ int32_t wt[SCAN_BLOCK / 32];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int32_t v[SCAN_ITEMS];
    int32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int32_t total;
    int32_t inc = block_inclusive(s, wt, total);
    int32_t run = sums[blockIdx.x] + inc - s;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

// Short inputs (at most SMALL_TILES tiles): one block walks the tiles in order, carrying the
// running total, so the scan is one launch instead of three.
constexpr int SMALL_TILES = 4;
__global__ void k_scan_small(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ out) {
    __shared__ int32_t wt[SCAN_BLOCK / 32];
    int32_t carry = 0;
    for (int64_t t0 = 0; t0 < n; t0 += SCAN_TILE) {
        const int64_t base = t0 + (int64_t)threadIdx.x * SCAN_ITEMS;
        int32_t v[SCAN_ITEMS];
        int32_t s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            v[k] = (base + k < n) ? in[base + k] : 0;
            s += v[k];
        }
        int32_t total;
        const int32_t inc = block_inclusive(s, wt, total);
        int32_t run = carry + inc - s;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) {
            if (base + k < n) out[base + k] = run;
            run += v[k];
        }
        carry += total;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

}  // namespace

void exclusive_scan(Ctx& c, const int32_t* in, int32_t* out, int64_t n) {
    if (n <= (int64_t)SMALL_TILES * SCAN_TILE) {
        k_scan_small<<<1, SCAN_BLOCK, 0, c.st()>>>(in, n, out);
        VV_LAUNCH_CHECK();
        return;
    }
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb < 1) nb = 1;
    c.scan_tmp.reserve((size_t)nb);
    k_tile_sums<<<(unsigned)nb, SCAN_BLOCK, 0, c.st()>>>(in, n, c.scan_tmp.p);
    VV_LAUNCH_CHECK();
    k_scan_sums<<<1, SCAN_BLOCK, 0, c.st()>>>(c.scan_tmp.p, nb, out + n);
    VV_LAUNCH_CHECK();
    k_tile_scan<<<(unsigned)nb, SCAN_BLOCK, 0, c.st()>>>(in, n, c.scan_tmp.p, out);
    VV_LAUNCH_CHECK();
}

int32_t read_i32(Ctx& c, const int32_t* p) {
    int32_t v = 0;
    int32_t* dst = c.h_pin ? c.h_pin : &v;
    VV_CUDA(cudaMemcpyAsync(dst, p, sizeof v, cudaMemcpyDeviceToHost, c.st()));
    VV_CUDA(cudaStreamSynchronize(c.st()));
    return *dst;
}

}  // namespace vvgpu
