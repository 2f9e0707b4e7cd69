// Bisection tree of libvvhd (stree/snode, libvvhd/src/TSortedTree.cpp) built on the GPU.
//
// The reference splits a node at the midpoint of its bounding box along the longer side
// and partitions the node's slice of VortexList in place with a two-pointer swap loop
// (DistributeContent, TSortedTree.cpp:81-99).  That loop is a set of disjoint swaps: with
// L = #{key < pivot} in the slice [f, l), the k-th element with key >= pivot inside [f, f+L)
// (counted from the left) trades places with the k-th element with key < pivot inside
// [f+L, l) (counted from the right).  Here every level of the tree is split at once: nodes
// of at most 64 vortices by one warp each (ballots give the ranks, the swap goes through
// shared memory), larger ones by blocks over 1024-vortex chunks (counts per chunk, one
// exclusive scan, then each vortex's rank; the lows of the right part and the highs of the
// left part publish their positions in two tables by rank, and one thread per pair swaps).  Only the
// keys (x, y) and a slot permutation move at each level; the rest of the vortex record
// follows once, after the last level.  The resulting permutation, node boxes and ranges are
// bit-identical to the reference.
// Segment lists (bllist) are split stably (TSortedTree.cpp:139-148).
//
// All decision arithmetic uses explicitly rounded FP64 operations (no FMA contraction),
// matching the reference's x86-64 build.
#include <cfloat>

#include "vvgpu_internal.cuh"

namespace vvgpu {

namespace {

constexpr int TB = 256;

__device__ __forceinline__ void bbox_min_atomic(unsigned long long* slot, double v) { atomicMin(slot, dkey(v)); }
__device__ __forceinline__ void bbox_max_atomic(unsigned long long* slot, double v) { atomicMax(slot, dkey(v)); }

__global__ void k_init_root(int32_t* perm, int64_t n, int32_t* seg_order, int32_t* seg_node_of, int64_t m,
                            unsigned long long* bbox) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) perm[i] = (int32_t)i;
    if (i < m) { seg_order[i] = (int32_t)i; seg_node_of[i] = 0; }
    if (i == 0) {
        bbox[0] = dkey(DBL_MAX); bbox[1] = dkey(DBL_MAX);
        bbox[2] = dkey(-DBL_MAX); bbox[3] = dkey(-DBL_MAX);
    }
}

// Root box over all segment centres and all vortices (snode::Stretch, TSortedTree.cpp:101-137):
// grid-stride, one set of atomics per block.  Boxes are reduced on the order-preserving
// integer keys of the coordinates (dkey), on the integer pipe rather than sm_103's narrow
// FP64 pipe.
__global__ void k_root_bbox(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                            const double* __restrict__ rx, const double* __restrict__ ry, int64_t m,
                            unsigned long long* bbox) {
    __shared__ unsigned long long s_b[TB / 32][4];
    unsigned long long b[4] = {dkey(DBL_MAX), dkey(DBL_MAX), dkey(-DBL_MAX), dkey(-DBL_MAX)};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n + m; i += (int64_t)gridDim.x * blockDim.x) {
        const double px = i < n ? x[i] : rx[i - n], py = i < n ? y[i] : ry[i - n];
        const unsigned long long kx = dkey(px), ky = dkey(py);
        b[0] = kx < b[0] ? kx : b[0];
        b[1] = ky < b[1] ? ky : b[1];
        b[2] = kx > b[2] ? kx : b[2];
        b[3] = ky > b[3] ? ky : b[3];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u[4];
#pragma unroll
        for (int e = 0; e < 4; e++) u[e] = __shfl_xor_sync(0xffffffffu, b[e], o);
        b[0] = u[0] < b[0] ? u[0] : b[0];
        b[1] = u[1] < b[1] ? u[1] : b[1];
        b[2] = u[2] > b[2] ? u[2] : b[2];
        b[3] = u[3] > b[3] ? u[3] : b[3];
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int e = 0; e < 4; e++) s_b[w][e] = b[e];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < TB / 32; q++) {
            b[0] = s_b[q][0] < b[0] ? s_b[q][0] : b[0];
            b[1] = s_b[q][1] < b[1] ? s_b[q][1] : b[1];
            b[2] = s_b[q][2] > b[2] ? s_b[q][2] : b[2];
            b[3] = s_b[q][3] > b[3] ? s_b[q][3] : b[3];
        }
        atomicMin(bbox + 0, b[0]);
        atomicMin(bbox + 1, b[1]);
        atomicMax(bbox + 2, b[2]);
        atomicMax(bbox + 3, b[3]);
    }
}

// Box -> (x, y, h, w) exactly as Stretch: x = (bl+tr).x*0.5, h = (tr-bl).y, w = (tr-bl).x
__device__ __forceinline__ double4 geom_from_bbox(const unsigned long long* b) {
    double blx = dunkey(b[0]), bly = dunkey(b[1]), trx = dunkey(b[2]), try_ = dunkey(b[3]);
    double4 g;
    g.x = dmul(dadd(blx, trx), 0.5);
    g.y = dmul(dadd(bly, try_), 0.5);
    g.z = dsub(try_, bly);
    g.w = dsub(trx, blx);
    return g;
}

__global__ void k_finalize_root(double4* geom, const unsigned long long* bbox, int32_t* vf, int32_t* vl,
                                int32_t* sf, int32_t* sl, int32_t* ch1, int32_t* depth, int64_t* path,
                                int64_t n, int64_t m) {
    geom[0] = geom_from_bbox(bbox);
    vf[0] = 0; vl[0] = (int32_t)n; sf[0] = 0; sl[0] = (int32_t)m;
    ch1[0] = -1; depth[0] = 0; path[0] = 0;
}

// snode::DivideNode's test (TSortedTree.cpp:36-79): split unless small enough; the split is
// at the box midpoint across the longer side.  Returns 1 to split.
__device__ __forceinline__ int decide_vals(double4 gm, int64_t nv, int64_t ns, int32_t depth, double min_node,
                                           double max_node, int32_t* err, int32_t& axis, double& pivot) {
    const double h = gm.z, w = gm.w;
    const double mx = smax(h, w), mn = smin(h, w);
    const int64_t maxlist = nv > ns ? nv : ns;
    const bool leaf = (mx < max_node && mn <= min_node) || (mx < max_node && maxlist < TREE_MAX_LIST_SIZE);
    int s = leaf ? 0 : 1;
    if (s && depth >= MAX_DEPTH) { s = 0; atomicExch(err, 1); }
    const bool byx = h < w;
    axis = byx ? 1 : 0;
    pivot = byx ? gm.x : gm.y;
    return s;
}

// Largest node whose whole subtree one block builds (k_subtree): at most SUB_N vortices,
// or, with segments, at most SUB_N vortices and segments together.
constexpr int SUB_N = 1024;

// split[k]: 0 leaf, 1 split by the level loop, 2 split by k_subtree (no segments and at most
// SUB_N vortices), 3 split by k_subtree with segments (vortices + segments at most SUB_N):
// the node and its descendants are finished after the loop.  Returns 1 for a split by the
// level loop (the flag that allocates its children in this pass).
__device__ __forceinline__ int decide_node(int64_t k, const double4* __restrict__ geom, const int32_t* __restrict__ vf,
                                           const int32_t* __restrict__ vl, const int32_t* __restrict__ sf,
                                           const int32_t* __restrict__ sl, const int32_t* __restrict__ depth,
                                           double min_node, double max_node, int32_t* split, double* pivot,
                                           int32_t* axis, int32_t* err) {
    const int64_t nv = (int64_t)vl[k] - vf[k], ns = (int64_t)sl[k] - sf[k];
    int32_t ax;
    double pv;
    int s = decide_vals(geom[k], nv, ns, depth[k], min_node, max_node, err, ax, pv);
    if (s && ns == 0 && nv <= SUB_N) s = 2;
    else if (s && nv + ns <= SUB_N) s = 3;
    split[k] = s;
    axis[k] = ax;
    pivot[k] = pv;
    return s == 1;
}

__global__ void k_decide(int64_t a, int64_t cnt, const double4* __restrict__ geom, const int32_t* __restrict__ vf,
                         const int32_t* __restrict__ vl, const int32_t* __restrict__ sf, const int32_t* __restrict__ sl,
                         const int32_t* __restrict__ depth, double min_node, double max_node, int32_t* split,
                         int32_t* flags, double* pivot, int32_t* axis, int32_t* err, int32_t* counts) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    if (t == 0) counts[0] = counts[1] = 0;  // the route's counters of this level
    const int64_t k = a + t;
    flags[t] = decide_node(k, geom, vf, vl, sf, sl, depth, min_node, max_node, split, pivot, axis, err);
}

__device__ __forceinline__ void make_children(int64_t k, int64_t c1, int32_t* ch1, int32_t* depth, int64_t* path,
                                              int32_t* parent, unsigned long long* bbox, int32_t* nlow,
                                              int32_t* nlow_s) {
    ch1[k] = (int32_t)c1;
    nlow[k] = 0;
    nlow_s[k] = 0;
    for (int q = 0; q < 2; q++) {
        int64_t c = c1 + q;
        ch1[c] = -1;
        depth[c] = depth[k] + 1;
        path[c] = path[k] * 2 + q;
        parent[c] = (int32_t)k;
        unsigned long long* s = bbox + 4 * c;
        s[0] = dkey(DBL_MAX); s[1] = dkey(DBL_MAX);
        s[2] = dkey(-DBL_MAX); s[3] = dkey(-DBL_MAX);
    }
}

__device__ __forceinline__ bool in_level_split(int32_t k, int64_t a, int64_t b, const int32_t* split) {
    return k >= a && k < b && split[k] == 1;
}

__global__ void k_perm_gather(int64_t n, const int32_t* __restrict__ perm, const double* __restrict__ g,
                              const double* __restrict__ ie, const double* __restrict__ vx,
                              const double* __restrict__ vy, const int64_t* __restrict__ orig, double* tmp,
                              int64_t* otmp) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t p = perm[i];
    tmp[i] = g[p];
    tmp[n + i] = ie[p];
    tmp[2 * n + i] = vx[p];
    tmp[3 * n + i] = vy[p];
    otmp[i] = orig[p];
}

__global__ void k_perm_store(int64_t n, const double* __restrict__ tmp, const int64_t* __restrict__ otmp, double* g,
                             double* ie, double* vx, double* vy, int64_t* orig) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    g[i] = tmp[i];
    ie[i] = tmp[n + i];
    vx[i] = tmp[2 * n + i];
    vy[i] = tmp[3 * n + i];
    orig[i] = otmp[i];
}

// Every split node's vortices are partitioned by one of two routes, chosen by size: one warp
// per node of at most SMALL_N vortices, or blocks over chunks of CH vortices of the larger
// nodes (count, scan, place, swap).  Both give the pairing of the swap loop of
// TSortedTree.cpp:81-99: the kk-th high of the left part (kk = highs to its left) trades
// places with the low of the right part that has kk lows to its right.  Segments are
// partitioned by their own passes whatever the route.
constexpr int SMALL_N = 64;
constexpr int SW = 4;          // warps per block in k_small_split
constexpr int CT = 256;        // threads per chunk block
constexpr int CE = 4;          // vortices per thread in a chunk
constexpr int CH = CT * CE;    // vortices per chunk
constexpr int CNW = CT / 32;

// k_route: counts[0] = warp-route nodes (listed in small_list), counts[1] = chunks; chunk c
// belongs to node chunk_node[c], and node k's chunks are cbase[k] .. cbase[k] + nch - 1 in
// position order.
// Creates the children of the level's split nodes (ids b + 2 * rank among the split
// nodes), then routes each split node.  counts[2] = the level's split count.
__global__ void k_route(int64_t a, int64_t b, int64_t cnt, const int32_t* __restrict__ split,
                        const int32_t* __restrict__ lscan, const int32_t* __restrict__ vf,
                        const int32_t* __restrict__ vl, int32_t* counts, int32_t* small_list, int32_t* cbase,
                        int32_t* chunk_node, int32_t* ch1, int32_t* depth, int64_t* path, int32_t* parent,
                        unsigned long long* bbox, int32_t* nlow, int32_t* nlow_s) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t k = (int32_t)(a + t);
    if (t == 0) counts[2] = lscan[cnt];
    if (t < cnt) {
        if (split[k] == 1) make_children(k, b + 2 * (int64_t)lscan[t], ch1, depth, path, parent, bbox, nlow, nlow_s);
        else ch1[k] = -1;
    }
    bool small = false;
    int nch = 0;
    if (t < cnt && split[k] == 1) {
        const int32_t nv = vl[k] - vf[k];
        if (nv <= SMALL_N) small = true;
        else nch = (nv + CH - 1) / CH;
    }
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1;
    const unsigned ms = __ballot_sync(0xffffffffu, small);
    if (ms) {
        int base = 0;
        if (lane == 0) base = atomicAdd(counts, __popc(ms));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (small) small_list[base + __popc(ms & below)] = k;
    }
    int incl = nch;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    const int tot = __shfl_sync(0xffffffffu, incl, 31);
    if (tot == 0) return;  // warp-uniform
    int wbase = 0;
    if (lane == 0) wbase = atomicAdd(counts + 1, tot);
    wbase = __shfl_sync(0xffffffffu, wbase, 0);
    const int cb = wbase + incl - nch;
    if (nch) cbase[k] = cb;
    unsigned mm = __ballot_sync(0xffffffffu, nch > 0);
    while (mm) {  // the warp writes each node's chunk entries together
        const int src = __ffs(mm) - 1;
        mm &= mm - 1;
        const int b = __shfl_sync(0xffffffffu, cb, src), nc = __shfl_sync(0xffffffffu, nch, src);
        const int32_t kk = __shfl_sync(0xffffffffu, k, src);
        for (int j = lane; j < nc; j += 32) chunk_node[b + j] = kk;
    }
}

__device__ __forceinline__ void bbox_acc(unsigned long long* b, double px, double py) {
    const unsigned long long kx = dkey(px), ky = dkey(py);
    b[0] = kx < b[0] ? kx : b[0];
    b[1] = ky < b[1] ? ky : b[1];
    b[2] = kx > b[2] ? kx : b[2];
    b[3] = ky > b[3] ? ky : b[3];
}
__device__ __forceinline__ void bbox_merge(unsigned long long* b, const unsigned long long* u) {
    b[0] = u[0] < b[0] ? u[0] : b[0];
    b[1] = u[1] < b[1] ? u[1] : b[1];
    b[2] = u[2] > b[2] ? u[2] : b[2];
    b[3] = u[3] > b[3] ? u[3] : b[3];
}
__device__ __forceinline__ void bbox_warp_reduce(unsigned long long* b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u[4];
#pragma unroll
        for (int e = 0; e < 4; e++) u[e] = __shfl_xor_sync(0xffffffffu, b[e], o);
        bbox_merge(b, u);
    }
}
__device__ __forceinline__ void bbox_init(unsigned long long* b) {
    b[0] = b[1] = dkey(DBL_MAX);
    b[2] = b[3] = dkey(-DBL_MAX);
}
// The children's boxes take atomics: other blocks and the segment passes merge into them.
__device__ __forceinline__ void bbox_commit(unsigned long long* dst, const unsigned long long* b) {
    atomicMin(dst + 0, b[0]);
    atomicMin(dst + 1, b[1]);
    atomicMax(dst + 2, b[2]);
    atomicMax(dst + 3, b[3]);
}

// One warp per node of at most SMALL_N vortices.  Every vortex is loaded to registers before
// any is stored, so the in-place scatter to the paired destinations needs no staging.
__global__ void __launch_bounds__(SW * 32) k_small_split(const int32_t* __restrict__ list, int64_t nlist,
                                                         const int32_t* __restrict__ vf, const int32_t* __restrict__ vl,
                                                         const int32_t* __restrict__ axis,
                                                         const double* __restrict__ pivot,
                                                         const int32_t* __restrict__ ch1, double* x, double* y,
                                                         int32_t* perm, int32_t* nlow, unsigned long long* bbox) {
    __shared__ int32_t s_tr[SW][SMALL_N], s_tl[SW][SMALL_N];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t t = (int64_t)blockIdx.x * SW + w;
    if (t >= nlist) return;
    const int32_t k = list[t];
    const int32_t f = vf[k], n = vl[k] - f;
    const bool byx = axis[k] != 0;
    const unsigned long long kp = lt_key_of(pivot[k]);
    double ex[2], ey[2];
    int32_t ep[2];
    bool val[2], low[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int q = lane + 32 * h;
        val[h] = q < n;
        ex[h] = val[h] ? x[f + q] : 0.;
        ey[h] = val[h] ? y[f + q] : 0.;
        ep[h] = val[h] ? perm[f + q] : 0;
        low[h] = val[h] && lt_key(byx ? ex[h] : ey[h], kp);
    }
    const unsigned m0 = __ballot_sync(0xffffffffu, low[0]), m1 = __ballot_sync(0xffffffffu, low[1]);
    const int L = __popc(m0) + __popc(m1);
    const unsigned below = (1u << lane) - 1;
    const int lb[2] = {__popc(m0 & below), __popc(m0) + __popc(m1 & below)};  // lows before q
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int q = lane + 32 * h;
        if (val[h] && q >= L && low[h]) s_tr[w][L - lb[h] - 1] = q;
        if (val[h] && q < L && !low[h]) s_tl[w][q - lb[h]] = q;
    }
    __syncwarp();
    const int32_t c1 = ch1[k];
    unsigned long long b0[4], b1[4];
    bbox_init(b0);
    bbox_init(b1);
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if (!val[h]) continue;
        const int q = lane + 32 * h;
        int dq = q;
        if (q < L && !low[h]) dq = s_tr[w][q - lb[h]];
        if (q >= L && low[h]) dq = s_tl[w][L - lb[h] - 1];
        x[f + dq] = ex[h];
        y[f + dq] = ey[h];
        perm[f + dq] = ep[h];
        if (low[h]) bbox_acc(b0, ex[h], ey[h]);
        else bbox_acc(b1, ex[h], ey[h]);
    }
    bbox_warp_reduce(b0);
    bbox_warp_reduce(b1);
    if (lane == 0) {
        if (L > 0) bbox_commit(bbox + 4 * (size_t)c1, b0);
        if (L < n) bbox_commit(bbox + 4 * (size_t)(c1 + 1), b1);
        nlow[k] = L;
    }
}

struct ChunkPos {
    int32_t k, f, n, j, cb, nch;  // node, its first vortex, its size, chunk index, first chunk, chunks
};
__device__ __forceinline__ ChunkPos chunk_pos(int c, const int32_t* chunk_node, const int32_t* cbase,
                                              const int32_t* vf, const int32_t* vl) {
    ChunkPos p;
    p.k = chunk_node[c];
    p.cb = cbase[p.k];
    p.j = c - p.cb;
    p.f = vf[p.k];
    p.n = vl[p.k] - p.f;
    p.nch = (p.n + CH - 1) / CH;
    return p;
}

// Lows (key < pivot) in each chunk.
__global__ void __launch_bounds__(CT) k_chunk_count(const int32_t* __restrict__ chunk_node,
                                                    const int32_t* __restrict__ cbase, const int32_t* __restrict__ vf,
                                                    const int32_t* __restrict__ vl, const int32_t* __restrict__ axis,
                                                    const double* __restrict__ pivot, const double* __restrict__ x,
                                                    const double* __restrict__ y, int32_t* chunk_cnt) {
    __shared__ int s_c[CNW];
    const ChunkPos p = chunk_pos(blockIdx.x, chunk_node, cbase, vf, vl);
    const double* key = axis[p.k] ? x : y;
    const unsigned long long kp = lt_key_of(pivot[p.k]);
    int cl = 0;
#pragma unroll
    for (int e = 0; e < CE; e++) {
        const int q = p.j * CH + e * CT + threadIdx.x;
        cl += __popc(__ballot_sync(0xffffffffu, q < p.n && lt_key(key[p.f + q], kp)));
    }
    if ((threadIdx.x & 31) == 0) s_c[threadIdx.x >> 5] = cl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < CNW; w++) tot += s_c[w];
        chunk_cnt[blockIdx.x] = tot;
    }
}

// Ranks every vortex of a chunk among the node's lows and highs (pre = exclusive scan of the
// chunk counts), publishes the pairing tables (tab_tr[f + r] = right-part low with r lows to
// its right, tab_tl[f + kk] = left-part high with kk highs to its left), the number of pairs
// npair[k], the split count nlow[k], and the children's boxes.  Reads the keys only.
__global__ void __launch_bounds__(CT) k_chunk_place(const int32_t* __restrict__ chunk_node,
                                                    const int32_t* __restrict__ cbase, const int32_t* __restrict__ vf,
                                                    const int32_t* __restrict__ vl, const int32_t* __restrict__ axis,
                                                    const double* __restrict__ pivot, const int32_t* __restrict__ ch1,
                                                    const double* __restrict__ x, const double* __restrict__ y,
                                                    const int32_t* __restrict__ pre, int32_t* tab_tr, int32_t* tab_tl,
                                                    int32_t* npair, int32_t* nlow, unsigned long long* bbox) {
    __shared__ int s_cnt[CE * CNW], s_pre[CE * CNW];
    __shared__ unsigned long long s_b[CNW][8];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const ChunkPos p = chunk_pos(blockIdx.x, chunk_node, cbase, vf, vl);
    const bool byx = axis[p.k] != 0;
    const unsigned long long kp = lt_key_of(pivot[p.k]);
    const int L = pre[p.cb + p.nch] - pre[p.cb];
    const int before = pre[blockIdx.x] - pre[p.cb];  // lows in the node's earlier chunks
    double ex[CE], ey[CE];
    unsigned lowm[CE];
#pragma unroll
    for (int e = 0; e < CE; e++) {
        const int q = p.j * CH + e * CT + tid;
        const bool v = q < p.n;
        ex[e] = v ? x[p.f + q] : 0.;
        ey[e] = v ? y[p.f + q] : 0.;
        lowm[e] = __ballot_sync(0xffffffffu, v && lt_key(byx ? ex[e] : ey[e], kp));
        if (lane == 0) s_cnt[e * CNW + w] = __popc(lowm[e]);
    }
    __syncthreads();
    if (w == 0) {  // exclusive prefix over (row e, warp w) in position order; CE * CNW = 32
        const int c0 = s_cnt[lane];
        int incl = c0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        s_pre[lane] = incl - c0;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1;
    unsigned long long b0[4], b1[4];
    bbox_init(b0);
    bbox_init(b1);
    const int32_t k = p.k, f = p.f;
    if (p.j == 0 && tid == 0) {
        nlow[k] = L;
        if (L == 0) npair[k] = 0;
    }
#pragma unroll
    for (int e = 0; e < CE; e++) {
        const int q = p.j * CH + e * CT + tid;
        if (q >= p.n) continue;
        const bool low = (lowm[e] >> lane) & 1u;
        const int lb = before + s_pre[e * CNW + w] + __popc(lowm[e] & below);  // lows before q
        if (q >= L && low) tab_tr[f + L - lb - 1] = q;
        if (q < L && !low) tab_tl[f + q - lb] = q;
        if (q == L - 1) npair[k] = L - lb - (low ? 1 : 0);  // highs in the left part
        if (low) bbox_acc(b0, ex[e], ey[e]);
        else bbox_acc(b1, ex[e], ey[e]);
    }
    bbox_warp_reduce(b0);
    bbox_warp_reduce(b1);
    if (lane == 0) {
#pragma unroll
        for (int e = 0; e < 4; e++) { s_b[w][e] = b0[e]; s_b[w][4 + e] = b1[e]; }
    }
    __syncthreads();
    if (tid < 8) {
        // thread 4 child + c merges component c of that child's box over the warps and
        // commits it (min for the lower corner, max for the upper)
        const int comp = tid & 3, chd = tid >> 2;
        unsigned long long v = s_b[0][4 * chd + comp];
        for (int q = 1; q < CNW; q++) {
            const unsigned long long u = s_b[q][4 * chd + comp];
            v = comp < 2 ? (u < v ? u : v) : (u > v ? u : v);
        }
        const int lows = s_pre[CE * CNW - 1] + s_cnt[CE * CNW - 1];
        const int lo = p.j * CH, hi = min(p.n, lo + CH);
        if (chd == 0 ? lows > 0 : lows < hi - lo) {
            unsigned long long* dst = bbox + 4 * (size_t)(ch1[k] + chd) + comp;
            if (comp < 2) atomicMin(dst, v);
            else atomicMax(dst, v);
        }
    }
}

// Swaps the pairs p = j * CH .. of the chunk's node: tab_tl[f + p] <-> tab_tr[f + p].
__global__ void __launch_bounds__(CT) k_chunk_swap(const int32_t* __restrict__ chunk_node,
                                                   const int32_t* __restrict__ cbase, const int32_t* __restrict__ vf,
                                                   const int32_t* __restrict__ vl, const int32_t* __restrict__ npair,
                                                   const int32_t* __restrict__ tab_tr,
                                                   const int32_t* __restrict__ tab_tl, double* x, double* y,
                                                   int32_t* perm) {
    const ChunkPos p = chunk_pos(blockIdx.x, chunk_node, cbase, vf, vl);
    const int H = npair[p.k];
#pragma unroll
    for (int e = 0; e < CE; e++) {
        const int q = p.j * CH + e * CT + threadIdx.x;
        if (q >= H) break;
        const int64_t i = p.f + tab_tl[p.f + q], j = p.f + tab_tr[p.f + q];
        const double tx = x[i], ty = y[i];
        const int32_t tp = perm[i];
        x[i] = x[j]; y[i] = y[j]; perm[i] = perm[j];
        x[j] = tx; y[j] = ty; perm[j] = tp;
    }
}

__global__ void k_sclass(int64_t m, int64_t a, int64_t b, const int32_t* __restrict__ seg_node_of,
                         const int32_t* __restrict__ seg_order, const int32_t* __restrict__ split,
                         const int32_t* __restrict__ axis, const double* __restrict__ pivot,
                         const double* __restrict__ rx, const double* __restrict__ ry, int32_t* flags) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    int32_t k = seg_node_of[q];
    int f = 0;
    if (in_level_split(k, a, b, split)) {
        int32_t s = seg_order[q];
        double key = axis[k] ? rx[s] : ry[s];
        f = key < pivot[k];
    }
    flags[q] = f;
}

__global__ void k_sscatter(int64_t m, int64_t a, int64_t b, const int32_t* __restrict__ seg_node_of,
                           const int32_t* __restrict__ seg_order, const int32_t* __restrict__ split,
                           const int32_t* __restrict__ sf, const int32_t* __restrict__ sl,
                           const int32_t* __restrict__ ch1, const int32_t* __restrict__ flags,
                           const int32_t* __restrict__ S, int32_t* nlow_s, int32_t* seg_order2,
                           int32_t* seg_node_of2, const double* __restrict__ rx, const double* __restrict__ ry,
                           unsigned long long* bbox) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    int32_t k = seg_node_of[q];
    int32_t s = seg_order[q];
    if (!in_level_split(k, a, b, split)) {
        seg_order2[q] = s;
        seg_node_of2[q] = k;
        return;
    }
    int32_t f = sf[k], l = sl[k];
    int32_t nl = S[l] - S[f];
    if (q == f) nlow_s[k] = nl;
    int32_t before = S[q] - S[f];
    bool low = flags[q];
    int32_t nq = low ? f + before : f + nl + ((int32_t)(q - f) - before);
    int32_t child = ch1[k] + (low ? 0 : 1);
    seg_order2[nq] = s;
    seg_node_of2[nq] = child;
    unsigned long long* bb = bbox + 4 * (size_t)child;
    bbox_min_atomic(bb + 0, rx[s]);
    bbox_min_atomic(bb + 1, ry[s]);
    bbox_max_atomic(bb + 2, rx[s]);
    bbox_max_atomic(bb + 3, ry[s]);
}

// The segment split of one level in one block (m <= SEG1_MAX): classify, scan in shared
// memory, then the same stable scatter as k_sscatter.
constexpr int SEG1_MAX = 8192;
constexpr int SEG1_TB = 1024;
__global__ void __launch_bounds__(SEG1_TB) k_seg_level(int64_t m, int64_t a, int64_t b,
                                                      const int32_t* __restrict__ seg_node_of,
                                                      const int32_t* __restrict__ seg_order,
                                                      const int32_t* __restrict__ split, const int32_t* __restrict__ axis,
                                                      const double* __restrict__ pivot, const int32_t* __restrict__ sf,
                                                      const int32_t* __restrict__ sl, const int32_t* __restrict__ ch1,
                                                      int32_t* nlow_s, int32_t* seg_order2, int32_t* seg_node_of2,
                                                      const double* __restrict__ rx, const double* __restrict__ ry,
                                                      unsigned long long* bbox) {
    __shared__ int32_t S[SEG1_MAX + 1];
    __shared__ int32_t wsum[SEG1_TB / 32];
    __shared__ int32_t carry_s;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) carry_s = 0;
    __syncthreads();
    for (int64_t q0 = 0; q0 < m; q0 += SEG1_TB) {
        const int64_t q = q0 + tid;
        int f = 0;
        if (q < m) {
            const int32_t k = seg_node_of[q];
            if (in_level_split(k, a, b, split)) {
                const int32_t sg = seg_order[q];
                const double key = axis[k] ? rx[sg] : ry[sg];
                f = key < pivot[k];
            }
        }
        int v = f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane == 31) wsum[w] = v;
        __syncthreads();
        if (w == 0) {
            int x = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += u;
            }
            wsum[lane] = x;
        }
        __syncthreads();
        const int carry = carry_s;
        if (q < m) S[q] = carry + (w ? wsum[w - 1] : 0) + v - f;  // exclusive
        __syncthreads();
        if (tid == 0) carry_s = carry + wsum[SEG1_TB / 32 - 1];
        __syncthreads();
    }
    if (tid == 0) S[m] = carry_s;
    __syncthreads();
    for (int64_t q = tid; q < m; q += SEG1_TB) {
        const int32_t k = seg_node_of[q];
        const int32_t sg = seg_order[q];
        if (!in_level_split(k, a, b, split)) {
            seg_order2[q] = sg;
            seg_node_of2[q] = k;
            continue;
        }
        const int32_t f = sf[k], l = sl[k];
        const int32_t nl = S[l] - S[f];
        if (q == f) nlow_s[k] = nl;
        const int32_t before = S[q] - S[f];
        const bool low = (S[q + 1] - S[q]) != 0;
        const int32_t nq = low ? f + before : f + nl + ((int32_t)(q - f) - before);
        const int32_t child = ch1[k] + (low ? 0 : 1);
        seg_order2[nq] = sg;
        seg_node_of2[nq] = child;
        unsigned long long* bb = bbox + 4 * (size_t)child;
        bbox_min_atomic(bb + 0, rx[sg]);
        bbox_min_atomic(bb + 1, ry[sg]);
        bbox_max_atomic(bb + 2, rx[sg]);
        bbox_max_atomic(bb + 3, ry[sg]);
    }
}

// Ranges and boxes of the level's children, then their split decisions: the next level's
// nodes are [b, b + 2 nsplit) and their flags go to flags[c - b] for its scan.
__global__ void k_finalize(int64_t a, int64_t b, int64_t cnt, const int32_t* split,
                           const int32_t* __restrict__ ch1, const int32_t* __restrict__ nlow,
                           const int32_t* __restrict__ nlow_s, int32_t* vf, int32_t* vl, int32_t* sf, int32_t* sl,
                           double4* geom, const unsigned long long* bbox, const int32_t* __restrict__ depth,
                           double min_node, double max_node, int32_t* nsplit_flag, double* pivot, int32_t* axis,
                           int32_t* err, int32_t* flags, int32_t* counts) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    if (t == 0) counts[0] = counts[1] = 0;  // the next level's route counters
    int64_t k = a + t;
    if (split[k] != 1) return;
    int32_t c1 = ch1[k], c2 = c1 + 1;
    vf[c1] = vf[k]; vl[c1] = vf[k] + nlow[k];
    vf[c2] = vf[k] + nlow[k]; vl[c2] = vl[k];
    sf[c1] = sf[k]; sl[c1] = sf[k] + nlow_s[k];
    sf[c2] = sf[k] + nlow_s[k]; sl[c2] = sl[k];
    geom[c1] = geom_from_bbox(bbox + 4 * (size_t)c1);
    geom[c2] = geom_from_bbox(bbox + 4 * (size_t)c2);
    for (int q = 0; q < 2; q++) {
        const int64_t c = c1 + q;
        flags[c - b] = decide_node(c, geom, vf, vl, sf, sl, depth, min_node, max_node, nsplit_flag, pivot, axis, err);
    }
}

// ---- subtrees of small nodes, one block each ----
//
// A node without segments and with at most SUB_N vortices (split[k] == 2) is left alone by
// the level loop; afterwards one block loads its vortices into shared memory and builds
// its whole subtree there, level by level, with the same decisions (decide_vals) and the
// same swap pairing as the loop.  The subtree's nodes are numbered breadth-first from 1
// (the root is 0) and recorded in scratch slots 2 vf(root) + id (a subtree of n vortices
// has at most 2 n - 1 nodes, and the roots' vortex ranges are disjoint); k_subtree_place
// then moves them to ids after the loop's nodes.
constexpr int SUB_T = 256;
constexpr int SUB_E = SUB_N / SUB_T;
constexpr int SUB_NW = SUB_T / 32;
static_assert(SUB_N % SUB_T == 0 && SUB_NW <= 32, "subtree block shape");

struct SubNode {  // a node made by k_subtree, before its final id is known
    double4 geom;  // centre x, y, h, w (Stretch)
    int64_t path;
    int32_t vf, vl, sf, sl, ch1, parent, depth, pad;
};
static_assert(sizeof(SubNode) == 80, "SubNode is 80 bytes (2.5 double4)");

constexpr size_t SUB_SMEM = (size_t)SUB_N * (5 * 8 + 2 * 4 + 12 * 2 + 2) + 64 * 4;
// with segments: per segment slot its centre (x, y), global id, and for two levels its
// local index and node slot; per level node (two levels) its segment start and count
constexpr size_t SUB_SMEM_SEG = SUB_SMEM + (size_t)SUB_N * (2 * 8 + 4 + 2 * 2 + 2 * 2 + 2 * 2 + 2 * 2);

// Exclusive prefix of a[0 .. SUB_N) in place (thread-contiguous runs), a[SUB_N] = total.
__device__ __forceinline__ int32_t sub_exscan(int32_t* a, int32_t* wt) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int32_t v[SUB_E], sum = 0;
#pragma unroll
    for (int e = 0; e < SUB_E; e++) { v[e] = a[t * SUB_E + e]; sum += v[e]; }
    int32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) wt[w] = incl;
    __syncthreads();
    if (w == 0) {
        int32_t x = lane < SUB_NW ? wt[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        if (lane < SUB_NW) wt[lane] = x;
    }
    __syncthreads();
    int32_t off = (w ? wt[w - 1] : 0) + incl - sum;
#pragma unroll
    for (int e = 0; e < SUB_E; e++) { a[t * SUB_E + e] = off; off += v[e]; }
    if (t == SUB_T - 1) a[SUB_N] = off;
    __syncthreads();
    return a[SUB_N];
}

__global__ void k_defer_flags(int64_t nn, const int32_t* __restrict__ split, int32_t* flags) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nn) flags[k] = split[k] >= 2;
}
__global__ void k_defer_list(int64_t nn, const int32_t* __restrict__ split, const int32_t* __restrict__ pos,
                             int32_t* roots) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nn && split[k] >= 2) roots[pos[k]] = (int32_t)k;
}

template <bool SEG>
__global__ void __launch_bounds__(SUB_T) k_subtree(const int32_t* __restrict__ roots,
                                                   const int32_t* __restrict__ vf, const int32_t* __restrict__ vl,
                                                   const int32_t* __restrict__ sf, const int32_t* __restrict__ sl,
                                                   const int32_t* __restrict__ depth, const int64_t* __restrict__ path,
                                                   const double* __restrict__ pivot, const int32_t* __restrict__ axis,
                                                   double min_node, double max_node, double* x, double* y,
                                                   int32_t* perm, int32_t* seg_order, const double* __restrict__ rx,
                                                   const double* __restrict__ ry, SubNode* scratch, int32_t* nnew,
                                                   int32_t* err, int32_t* maxdepth) {
    extern __shared__ __align__(16) unsigned char smem[];
    // per vortex: position, permutation, level-node slot (two levels: -1 = in a finished
    // leaf), prefix, pairing tables.  Per level node: pivot, axis, split (the next level's
    // overwrite them once the current level's partition is done), and, for two levels,
    // path, first, size; per current node: rank among the split nodes, lows, pairs; per
    // next node: its parent's slot.
    double* sx = (double*)smem;
    double* sy = sx + SUB_N;
    unsigned long long* lkp = (unsigned long long*)(sy + SUB_N);  // pivot keys (lt_key_of)
    int64_t* lpath = (int64_t*)(lkp + SUB_N);                 // [2][SUB_N]
    int32_t* sp = (int32_t*)(lpath + 2 * SUB_N);
    int32_t* pre = sp + SUB_N;                                // SUB_N + 1
    int32_t* wt = pre + SUB_N + 4;                            // SUB_NW (60 ints reserved)
    int16_t* en = (int16_t*)(wt + 60);                        // [2][SUB_N]
    int16_t* tl = en + 2 * SUB_N;
    int16_t* tr = tl + SUB_N;
    int16_t* lvf = tr + SUB_N;                                // [2][SUB_N]
    int16_t* ln = lvf + 2 * SUB_N;                            // [2][SUB_N]
    int16_t* rank = ln + 2 * SUB_N;
    int16_t* cL = rank + SUB_N;
    int16_t* cH = cL + SUB_N;
    int16_t* par = cH + SUB_N;
    int8_t* lax = (int8_t*)(par + SUB_N);
    int8_t* lsp = lax + SUB_N;
    // segments (SEG): centres by local index, global ids; for two levels the local index at
    // each position, the node slot at each position, and each level node's segment range
    double* gx = (double*)(smem + SUB_SMEM);
    double* gy = gx + SUB_N;
    int32_t* gid = (int32_t*)(gy + SUB_N);
    int16_t* gix = (int16_t*)(gid + SUB_N);  // [2][SUB_N]
    int16_t* gen = gix + 2 * SUB_N;          // [2][SUB_N]
    int16_t* lsf = gen + 2 * SUB_N;          // [2][SUB_N]
    int16_t* lsn = lsf + 2 * SUB_N;          // [2][SUB_N]

    const int t = threadIdx.x;
    const int32_t root = roots[blockIdx.x];
    const int32_t f0 = vf[root], nr = vl[root] - f0;
    const int32_t s0 = sf[root], ns = sl[root] - s0;
    if ((ns > 0) != SEG) return;  // the other kernel's subtree
    if (SEG ? (nr + ns > SUB_N) : (nr > SUB_N || nr < 1)) {  // not a deferred node (cannot happen)
        if (t == 0) { atomicExch(err, 3); nnew[blockIdx.x] = 0; }
        return;
    }
    SubNode* rec = scratch + 2 * ((size_t)f0 + (size_t)s0);  // local id u at rec[u], u < 2 (nr + ns)
    for (int i = t; i < SUB_N; i += SUB_T) {
        if (i < nr) {
            sx[i] = x[f0 + i];
            sy[i] = y[f0 + i];
            sp[i] = perm[f0 + i];
            en[i] = 0;
        } else {
            en[i] = -1;
        }
        if (SEG) {
            if (i < ns) {
                const int32_t sg = seg_order[s0 + i];
                gid[i] = sg;
                gx[i] = rx[sg];
                gy[i] = ry[sg];
                gix[i] = (int16_t)i;
                gen[i] = 0;
            } else {
                gen[i] = -1;
            }
        }
    }
    if (t == 0) {
        lvf[0] = 0; ln[0] = (int16_t)nr; lkp[0] = lt_key_of(pivot[root]); lax[0] = (int8_t)axis[root];
        lsp[0] = 1; lpath[0] = path[root];
        if (SEG) { lsf[0] = 0; lsn[0] = (int16_t)ns; }
    }
    int cur = 0, ncur = 1, base = 0, next_lid = 1;  // base: local id of the level's slot 0
    int32_t dep = depth[root];
    __syncthreads();
    for (int level = 0; level <= MAX_DEPTH; level++) {
        const int co = cur * SUB_N, no = (cur ^ 1) * SUB_N;
        // (a) rank of each split node among the level's split nodes
        for (int j = t; j < SUB_N; j += SUB_T) pre[j] = (j < ncur && lsp[j]) ? 1 : 0;
        __syncthreads();
        const int nsplit = sub_exscan(pre, wt);
        if (nsplit == 0) break;
        if (next_lid + 2 * nsplit > 2 * (nr + ns)) {
            // only a chain of splits that leave one side empty (a box midpoint rounding onto
            // its lower edge) outgrows 2 n - 1 nodes; the level loop reports it as too deep
            if (t == 0) atomicExch(err, 1);
            break;
        }
        for (int j = t; j < ncur; j += SUB_T) rank[j] = (int16_t)pre[j];
        __syncthreads();
        // (b) low flags (key < pivot) of the split nodes' vortices, prefix over positions
#pragma unroll
        for (int e = 0; e < SUB_E; e++) {
            const int i = e * SUB_T + t;
            const int nd = en[co + i];
            bool low = false;
            if (nd >= 0 && lsp[nd]) low = lt_key(lax[nd] ? sx[i] : sy[i], lkp[nd]);
            pre[i] = low ? 1 : 0;
        }
        __syncthreads();
        sub_exscan(pre, wt);
        // (c) lows and pairs of each split node; its children take slots 2 rank, 2 rank + 1
        for (int j = t; j < ncur; j += SUB_T) {
            if (!lsp[j]) continue;
            const int f = lvf[co + j], n = ln[co + j];
            const int L = pre[f + n] - pre[f];
            cL[j] = (int16_t)L;
            cH[j] = (int16_t)(L - (pre[f + L] - pre[f]));  // highs in the left part
            const int r = rank[j];
            if (base + j > 0) rec[base + j].ch1 = next_lid + 2 * r;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int cs = 2 * r + q;
                lvf[no + cs] = (int16_t)(q ? f + L : f);
                ln[no + cs] = (int16_t)(q ? n - L : L);
                lpath[no + cs] = lpath[co + j] * 2 + q;
                par[cs] = (int16_t)j;
            }
        }
        __syncthreads();
        // (d) pairing tables (the pairing of TSortedTree.cpp:81-99, as in the level loop) and
        // each position's slot in the next level
#pragma unroll
        for (int e = 0; e < SUB_E; e++) {
            const int i = e * SUB_T + t;
            const int nd = en[co + i];
            int cs = -1;
            if (nd >= 0 && lsp[nd]) {
                const int f = lvf[co + nd], L = cL[nd], q = i - f, lb = pre[i] - pre[f];
                const bool low = pre[i + 1] != pre[i];
                if (q >= L && low) tr[f + L - lb - 1] = (int16_t)q;
                if (q < L && !low) tl[f + q - lb] = (int16_t)q;
                cs = 2 * rank[nd] + (q >= L ? 1 : 0);
            }
            en[no + i] = (int16_t)cs;
        }
        __syncthreads();
        // (e) swaps
#pragma unroll
        for (int e = 0; e < SUB_E; e++) {
            const int i = e * SUB_T + t;
            const int nd = en[co + i];
            if (nd < 0 || !lsp[nd]) continue;
            const int f = lvf[co + nd], pq = i - f;
            if (pq >= cH[nd]) continue;
            const int ia = f + tl[f + pq], ib = f + tr[f + pq];
            const double tx = sx[ia], ty = sy[ia];
            const int32_t tp = sp[ia];
            sx[ia] = sx[ib]; sy[ia] = sy[ib]; sp[ia] = sp[ib];
            sx[ib] = tx; sy[ib] = ty; sp[ib] = tp;
        }
        __syncthreads();
        if (SEG) {
            // (g) the segment lists of the split nodes, split stably (TSortedTree.cpp:139-148):
            // low flags (centre key < pivot) and their prefix, then each segment's position
            // and child slot in the next level
#pragma unroll
            for (int e = 0; e < SUB_E; e++) {
                const int i = e * SUB_T + t;
                const int nd = gen[co + i];
                bool low = false;
                if (nd >= 0 && lsp[nd]) {
                    const int li = gix[co + i];
                    low = lt_key(lax[nd] ? gx[li] : gy[li], lkp[nd]);
                }
                pre[i] = low ? 1 : 0;
            }
            __syncthreads();
            sub_exscan(pre, wt);
            for (int j = t; j < ncur; j += SUB_T) {
                if (!lsp[j]) continue;
                const int f = lsf[co + j], n = lsn[co + j];
                const int L = pre[f + n] - pre[f];
                cH[j] = (int16_t)L;  // the vortex swaps are done: cH now holds the segment lows
                const int r = rank[j];
                lsf[no + 2 * r] = (int16_t)f;
                lsn[no + 2 * r] = (int16_t)L;
                lsf[no + 2 * r + 1] = (int16_t)(f + L);
                lsn[no + 2 * r + 1] = (int16_t)(n - L);
            }
            __syncthreads();
#pragma unroll
            for (int e = 0; e < SUB_E; e++) {
                const int i = e * SUB_T + t;
                const int nd = gen[co + i];
                if (nd >= 0 && lsp[nd]) {
                    const int f = lsf[co + nd], L = cH[nd], before = pre[i] - pre[f];
                    const bool low = pre[i + 1] != pre[i];
                    const int nq = low ? f + before : f + L + ((i - f) - before);
                    gix[no + nq] = gix[co + i];
                    gen[no + nq] = (int16_t)(2 * rank[nd] + (low ? 0 : 1));
                } else {
                    gix[no + i] = gix[co + i];
                    gen[no + i] = -1;
                }
            }
            __syncthreads();
        }
        // (f) the children: box (a group of G lanes per child), geometry, decision, record
        const int nch = 2 * nsplit;
        const int G = nch <= SUB_NW ? 32 : nch <= 2 * SUB_NW ? 16 : nch <= 4 * SUB_NW ? 8 : 4;
        const int gl = t & (G - 1), ng = SUB_T / G;
        for (int c0 = 0; c0 < nch; c0 += ng) {  // uniform trip count: every lane shuffles
            const int cs = c0 + t / G;
            unsigned long long b4[4];
            bbox_init(b4);
            int f = 0, n = 0, gf = 0, gn = 0;
            if (cs < nch) {
                f = lvf[no + cs];
                n = ln[no + cs];
                for (int i = f + gl; i < f + n; i += G) bbox_acc(b4, sx[i], sy[i]);
                if (SEG) {
                    gf = lsf[no + cs];
                    gn = lsn[no + cs];
                    for (int i = gf + gl; i < gf + gn; i += G) {
                        const int li = gix[no + i];
                        bbox_acc(b4, gx[li], gy[li]);
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                if (o >= G) continue;
                unsigned long long u[4];
#pragma unroll
                for (int e = 0; e < 4; e++) u[e] = __shfl_xor_sync(0xffffffffu, b4[e], o);
                bbox_merge(b4, u);
            }
            if (cs < nch && gl == 0) {
                const double4 gm = geom_from_bbox(b4);
                int32_t ax;
                double pv;
                lsp[cs] = (int8_t)decide_vals(gm, n, gn, dep + 1, min_node, max_node, err, ax, pv);
                lax[cs] = (int8_t)ax;
                lkp[cs] = lt_key_of(pv);
                SubNode o;
                o.geom = gm;
                o.path = lpath[no + cs];
                o.vf = f0 + f;
                o.vl = f0 + f + n;
                o.sf = s0 + gf;
                o.sl = s0 + gf + gn;
                o.ch1 = -1;
                o.parent = base + par[cs];
                o.depth = dep + 1;
                o.pad = 0;
                rec[next_lid + cs] = o;
            }
        }
        base = next_lid;
        next_lid += nch;
        dep++;
        ncur = nch;
        cur ^= 1;
        __syncthreads();
    }
    for (int i = t; i < nr; i += SUB_T) {
        x[f0 + i] = sx[i];
        y[f0 + i] = sy[i];
        perm[f0 + i] = sp[i];
    }
    if (SEG)
        for (int i = t; i < ns; i += SUB_T) seg_order[s0 + i] = gid[gix[cur * SUB_N + i]];
    if (t == 0) {
        nnew[blockIdx.x] = next_lid - 1;
        atomicMax(maxdepth, dep);
    }
}

// Moves subtree r's new nodes (local ids 1 .. nnew) to ids base + pos[r] + id - 1.
__global__ void k_subtree_place(const int32_t* __restrict__ roots, const int32_t* __restrict__ pos,
                                const int32_t* __restrict__ nnew, int64_t base, const SubNode* __restrict__ scratch,
                                double4* geom, int32_t* vf, int32_t* vl, int32_t* sf, int32_t* sl, int32_t* ch1,
                                int32_t* depth, int64_t* path, int32_t* parent) {
    const int32_t root = roots[blockIdx.x];
    const int32_t cnt = nnew[blockIdx.x];
    const int64_t b = base + pos[blockIdx.x] - 1;  // id of local node u >= 1 is b + u
    const SubNode* rec = scratch + 2 * ((size_t)vf[root] + (size_t)sf[root]);
    if (threadIdx.x == 0) ch1[root] = cnt > 0 ? (int32_t)(b + 1) : -1;
    for (int32_t u = 1 + threadIdx.x; u <= cnt; u += blockDim.x) {
        const SubNode o = rec[u];
        const int64_t g = b + u;
        geom[g] = o.geom;
        vf[g] = o.vf;
        vl[g] = o.vl;
        sf[g] = o.sf;
        sl[g] = o.sl;
        ch1[g] = o.ch1 >= 0 ? (int32_t)(b + o.ch1) : -1;
        depth[g] = o.depth;
        path[g] = o.path;
        parent[g] = o.parent > 0 ? (int32_t)(b + o.parent) : root;
    }
}

// ---- centroids (snode::CalculateCMass, TSortedTree.cpp:150-197) and depth-first order ----

__global__ void k_leaf_cm(int64_t nn, const int32_t* __restrict__ ch1, const int32_t* __restrict__ vf,
                          const int32_t* __restrict__ vl, const double4* __restrict__ geom,
                          const double* __restrict__ x, const double* __restrict__ y,
                          const double* __restrict__ g, double* cm, int32_t* lc) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nn || ch1[k] >= 0) return;
    double px = 0, py = 0, pg = 0, mx = 0, my = 0, mg = 0;
    for (int32_t i = vf[k]; i < vl[k]; i++) {
        double gi = g[i];
        if (gi > 0) { px = dadd(px, dmul(x[i], gi)); py = dadd(py, dmul(y[i], gi)); pg = dadd(pg, gi); }
        else        { mx = dadd(mx, dmul(x[i], gi)); my = dadd(my, dmul(y[i], gi)); mg = dadd(mg, gi); }
    }
    double4 gm = geom[k];
    if (pg != 0) { double inv = ddiv(1., pg); px = dmul(px, inv); py = dmul(py, inv); } else { px = gm.x; py = gm.y; }
    if (mg != 0) { double inv = ddiv(1., mg); mx = dmul(mx, inv); my = dmul(my, inv); } else { mx = gm.x; my = gm.y; }
    double* c = cm + 6 * k;
    c[0] = px; c[1] = py; c[2] = pg; c[3] = mx; c[4] = my; c[5] = mg;
    lc[k] = 1;
}

__device__ __forceinline__ void combine_cm(const double* a, const double* b, double* out, double nx, double ny) {
    double sumg = dadd(a[2], b[2]);
    if (sumg != 0) {
        double sx = dadd(dmul(a[0], a[2]), dmul(b[0], b[2]));
        double sy = dadd(dmul(a[1], a[2]), dmul(b[1], b[2]));
        double inv = ddiv(1., sumg);
        out[0] = dmul(sx, inv); out[1] = dmul(sy, inv); out[2] = sumg;
    } else { out[0] = nx; out[1] = ny; out[2] = 0; }
}

// All inner centroids in one pass: each leaf's thread climbs towards the root, and at each
// node the second child to arrive combines both children (always in the order ch1, ch1 + 1,
// so the result does not depend on which arrives last) and climbs on.
// Climbs start at the leaves of nodes [0, nn), and with `split` also at the subtree roots
// (split >= 2), whose subtrees k_subtree_cm has completed.
__global__ void k_tree_cm(int64_t nn, const int32_t* __restrict__ ch1, const int32_t* __restrict__ split,
                          const int32_t* __restrict__ parent, const double4* __restrict__ geom, double* cm,
                          int32_t* lc, int32_t* arrive) {
    const int64_t k0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= nn || (ch1[k0] >= 0 && !(split && split[k0] >= 2))) return;
    int32_t k = (int32_t)k0;
    for (int it = 0; it <= MAX_DEPTH; it++) {
        const int32_t p = parent[k];
        if (p < 0) return;
        __threadfence();  // this subtree's results before the arrival
        if (atomicAdd(&arrive[p], 1) == 0) return;  // the sibling combines
        __threadfence();
        const int32_t c1 = ch1[p];
        const double4 gm = geom[p];
        double A[6], B[6], o[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
            A[q] = __ldcg(cm + 6 * (size_t)c1 + q);
            B[q] = __ldcg(cm + 6 * (size_t)(c1 + 1) + q);
        }
        combine_cm(A, B, o, gm.x, gm.y);
        combine_cm(A + 3, B + 3, o + 3, gm.x, gm.y);
#pragma unroll
        for (int q = 0; q < 6; q++) cm[6 * (size_t)p + q] = o[q];
        lc[p] = __ldcg(lc + c1) + __ldcg(lc + c1 + 1);
        k = p;
    }
}

// Centroids and leaf counts of every subtree built by k_subtree, one block per subtree:
// its vortices are staged in shared memory (one coalesced read), each leaf sums its own in
// the order of k_leaf_cm, then the inner nodes combine their children deepest level first
// as k_tree_cm does (a subtree's ids are breadth-first, so its deepest node is the last).
// The subtree's root is completed here too; the level loop's nodes above it climb later.
__global__ void __launch_bounds__(SUB_T) k_subtree_cm(const int32_t* __restrict__ roots,
                                                      const int32_t* __restrict__ pos,
                                                      const int32_t* __restrict__ nnew, int64_t base0,
                                                      const int32_t* __restrict__ vf, const int32_t* __restrict__ vl,
                                                      const int32_t* __restrict__ ch1,
                                                      const int32_t* __restrict__ depth,
                                                      const double4* __restrict__ geom, const double* __restrict__ x,
                                                      const double* __restrict__ y, const double* __restrict__ g,
                                                      double* cm, int32_t* lc) {
    __shared__ double sx[SUB_N], sy[SUB_N], sg[SUB_N];
    const int t = threadIdx.x;
    const int32_t root = roots[blockIdx.x], cnt = nnew[blockIdx.x];
    const int64_t b = base0 + pos[blockIdx.x] - 1;  // id of local node u >= 1
    const int32_t f0 = vf[root], nr = vl[root] - f0;
    if (cnt <= 0 || nr > SUB_N) return;
    for (int i = t; i < nr; i += SUB_T) {
        sx[i] = x[f0 + i];
        sy[i] = y[f0 + i];
        sg[i] = g[f0 + i];
    }
    __syncthreads();
    for (int32_t u = 1 + t; u <= cnt; u += SUB_T) {
        const int64_t k = b + u;
        if (ch1[k] >= 0) continue;
        double px = 0, py = 0, pg = 0, mx = 0, my = 0, mg = 0;
        for (int32_t i = vf[k] - f0; i < vl[k] - f0; i++) {
            const double gi = sg[i];
            if (gi > 0) { px = dadd(px, dmul(sx[i], gi)); py = dadd(py, dmul(sy[i], gi)); pg = dadd(pg, gi); }
            else        { mx = dadd(mx, dmul(sx[i], gi)); my = dadd(my, dmul(sy[i], gi)); mg = dadd(mg, gi); }
        }
        const double4 gm = geom[k];
        if (pg != 0) { double inv = ddiv(1., pg); px = dmul(px, inv); py = dmul(py, inv); } else { px = gm.x; py = gm.y; }
        if (mg != 0) { double inv = ddiv(1., mg); mx = dmul(mx, inv); my = dmul(my, inv); } else { mx = gm.x; my = gm.y; }
        double* c = cm + 6 * k;
        c[0] = px; c[1] = py; c[2] = pg; c[3] = mx; c[4] = my; c[5] = mg;
        lc[k] = 1;
    }
    const int32_t dmax = depth[b + cnt], droot = depth[root];
    for (int32_t d = dmax - 1; d >= droot; d--) {
        __syncthreads();
        for (int32_t u = t; u <= cnt; u += SUB_T) {
            const int64_t k = u == 0 ? (int64_t)root : b + u;
            const int32_t c1 = ch1[k];
            if (c1 < 0 || depth[k] != d) continue;
            const double4 gm = geom[k];
            double A[6], B[6], o[6];
#pragma unroll
            for (int q = 0; q < 6; q++) {
                A[q] = __ldcg(cm + 6 * (size_t)c1 + q);
                B[q] = __ldcg(cm + 6 * (size_t)(c1 + 1) + q);
            }
            combine_cm(A, B, o, gm.x, gm.y);
            combine_cm(A + 3, B + 3, o + 3, gm.x, gm.y);
#pragma unroll
            for (int q = 0; q < 6; q++) cm[6 * k + q] = o[q];
            lc[k] = __ldcg(lc + c1) + __ldcg(lc + c1 + 1);
        }
    }
}

// Depth-first leaf index of every node (its first leaf): the leaves of the left siblings on
// the way up to the root, summed; leaf_node[dfs] = node for the leaves.
__global__ void k_tree_dfs(int64_t nn, const int32_t* __restrict__ ch1, const int32_t* __restrict__ parent,
                           const int32_t* __restrict__ lc, int32_t* dfs, int32_t* leaf_node) {
    const int64_t k0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 >= nn) return;
    int32_t k = (int32_t)k0, d = 0;
    for (int it = 0; it <= MAX_DEPTH; it++) {
        const int32_t p = parent[k];
        if (p < 0) break;
        const int32_t c1 = ch1[p];
        if (k != c1) d += lc[c1];
        k = p;
    }
    dfs[k0] = d;
    if (ch1[k0] < 0) leaf_node[d] = (int32_t)k0;
}

__global__ void k_leaf_arrays(int64_t nl, const int32_t* __restrict__ leaf_node, const int32_t* __restrict__ vf,
                              const int32_t* __restrict__ vl, const int32_t* __restrict__ sf,
                              const int32_t* __restrict__ sl, const double4* __restrict__ geom, int32_t* lvf,
                              int32_t* lvl, int32_t* lsf, int32_t* lsl, double4* lgeom, int32_t* leaf_of) {
    int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= nl) return;
    int32_t k = leaf_node[L];
    lvf[L] = vf[k]; lvl[L] = vl[k]; lsf[L] = sf[k]; lsl[L] = sl[k];
    lgeom[L] = geom[k];
    for (int32_t i = vf[k]; i < vl[k]; i++) leaf_of[i] = (int32_t)L;
}

}  // namespace

void tree_build(Ctx& c, double far_criteria, double min_node, double max_node) {
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "tree is already built"};
    if (c.n > 0x3fffffff || c.m > 0x3fffffff) throw ApiError{VVGPU_ERR_LIMIT, "too many vortices or segments"};
    check_input(c);
    upload_segments(c);
    c.far_criteria = far_criteria; c.min_node = min_node; c.max_node = max_node;
    const int64_t n = c.n, m = c.m;
    cudaStream_t s = c.st();
    int64_t cap_nodes = 1024;
    auto ensure_nodes = [&](int64_t need) {
        if ((size_t)need <= c.nd_geom.cap) return;
        int64_t keep = c.nnodes;
        c.nd_geom.reserve(need, true, keep, s);
        c.nd_vf.reserve(need, true, keep, s); c.nd_vl.reserve(need, true, keep, s);
        c.nd_sf.reserve(need, true, keep, s); c.nd_sl.reserve(need, true, keep, s);
        c.nd_ch1.reserve(need, true, keep, s); c.nd_depth.reserve(need, true, keep, s);
        c.nd_path.reserve(need, true, keep, s);
        c.nd_bbox.reserve(4 * need, true, 4 * keep, s);
        c.nd_pivot.reserve(need, true, keep, s);
        c.nd_axis.reserve(need, true, keep, s); c.nd_split.reserve(need, true, keep, s);
        c.nd_nlow.reserve(need, true, keep, s); c.nd_nlow_s.reserve(need, true, keep, s);
        c.nd_cbase.reserve(need, true, keep, s); c.nd_npair.reserve(need, true, keep, s);
        c.nd_parent.reserve(need, true, keep, s);
    };
    c.lvl_cnt.reserve(4);
    c.nnodes = 1;
    ensure_nodes(cap_nodes);
    c.flags.reserve(n + m + 2);
    c.scan.reserve(n + m + 2);
    c.tab_rl.reserve(n + 1);
    c.tab_lh.reserve(n + 1);
    c.seg_order.reserve(m + 1); c.seg_order2.reserve(m + 1);
    c.seg_node_of.reserve(m + 1); c.seg_node_of2.reserve(m + 1);
    c.counters.reserve(24);
    VV_CUDA(cudaMemsetAsync(c.counters.p, 0, 16 * sizeof(unsigned long long), s));
    int32_t* err = (int32_t*)c.counters.p;

    int64_t nm = n > m ? n : m;
    c.perm.reserve(n + 1);
    k_init_root<<<grid_for(nm, TB), TB, 0, s>>>(c.perm.p, n, c.seg_order.p, c.seg_node_of.p, m,
                                                c.nd_bbox.p);
    VV_LAUNCH_CHECK();
    if (n + m > 0) {
        k_root_bbox<<<std::min<int64_t>(grid_for(n + m, TB), 152 * 8), TB, 0, s>>>(c.x.p, c.y.p, n, c.s_rx.p, c.s_ry.p, m, c.nd_bbox.p);
        VV_LAUNCH_CHECK();
    }
    VV_CUDA(cudaMemsetAsync(c.nd_parent.p, 0xff, sizeof(int32_t), s));  // the root has none
    k_finalize_root<<<1, 1, 0, s>>>(c.nd_geom.p, c.nd_bbox.p, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p,
                                    c.nd_ch1.p, c.nd_depth.p, c.nd_path.p, n, m);
    VV_LAUNCH_CHECK();

    c.level_begin.assign({0, 1});
    cudaStream_t side = side_stream(c);
    int64_t d = 0;
    for (;; d++) {
        int64_t a = c.level_begin[d], b = c.level_begin[d + 1], cnt = b - a;
        if (cnt <= 0) break;
        ensure_nodes(b + 2 * cnt);
        // this level's flags come from the previous level's k_finalize (kept); the next
        // level's (up to 2 cnt) are written by this level's
        c.flags.reserve(2 * cnt + 2, true, cnt + 1, s);
        c.scan.reserve(cnt + 2);
        c.lvl_list.reserve((size_t)cnt + 1);
        c.chunk_node.reserve((size_t)cnt + (size_t)(n / CH) + 2);
        if (d == 0) {
            k_decide<<<grid_for(cnt, TB), TB, 0, s>>>(a, cnt, c.nd_geom.p, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p,
                                                      c.nd_depth.p, min_node, max_node, c.nd_split.p, c.flags.p,
                                                      c.nd_pivot.p, c.nd_axis.p, err, c.lvl_cnt.p);
            VV_LAUNCH_CHECK();
        }
        exclusive_scan(c, c.flags.p, c.scan.p, cnt);
        // children of the split nodes, then the partition route of each: one warp per small
        // node, chunk blocks over the larger ones
        k_route<<<grid_for(cnt, TB), TB, 0, s>>>(a, b, cnt, c.nd_split.p, c.scan.p, c.nd_vf.p, c.nd_vl.p,
                                                 c.lvl_cnt.p, c.lvl_list.p, c.nd_cbase.p, c.chunk_node.p,
                                                 c.nd_ch1.p, c.nd_depth.p, c.nd_path.p, c.nd_parent.p, c.nd_bbox.p,
                                                 c.nd_nlow.p, c.nd_nlow_s.p);
        VV_LAUNCH_CHECK();
        // The segment split and the warp-per-node splits touch other data than the chunk
        // partition (other nodes' ranges; the children's boxes only through atomic min/max),
        // so they run on the side stream, joined before k_finalize.
        const bool seg1 = m > 0 && m <= SEG1_MAX;
        if (seg1) {
            VV_CUDA(cudaEventRecord(c.ev_fork, s));
            VV_CUDA(cudaStreamWaitEvent(side, c.ev_fork, 0));
            k_seg_level<<<1, SEG1_TB, 0, side>>>(m, a, b, c.seg_node_of.p, c.seg_order.p, c.nd_split.p,
                                                 c.nd_axis.p, c.nd_pivot.p, c.nd_sf.p, c.nd_sl.p, c.nd_ch1.p,
                                                 c.nd_nlow_s.p, c.seg_order2.p, c.seg_node_of2.p, c.s_rx.p, c.s_ry.p,
                                                 c.nd_bbox.p);
            VV_LAUNCH_CHECK();
            std::swap(c.seg_order, c.seg_order2);
            std::swap(c.seg_node_of, c.seg_node_of2);
        }
        int32_t hl[3];
        int32_t* hc = c.h_pin ? c.h_pin + 4 : hl;  // pinned when the context has its words
        VV_CUDA(cudaMemcpyAsync(hc, c.lvl_cnt.p, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        VV_CUDA(cudaStreamSynchronize(s));
        const int32_t nsmall = hc[0], nchunk = hc[1], nsplit = hc[2];
        if (nsplit == 0) {
            if (seg1) {  // nothing split: the side stream's copy of the segment order is unchanged
                VV_CUDA(cudaEventRecord(c.ev_join, side));
                VV_CUDA(cudaStreamWaitEvent(s, c.ev_join, 0));
            }
            break;
        }
        if (nsmall > 0) {
            if (!seg1) {
                VV_CUDA(cudaEventRecord(c.ev_fork, s));
                VV_CUDA(cudaStreamWaitEvent(side, c.ev_fork, 0));
            }
            k_small_split<<<grid_for(nsmall, SW), SW * 32, 0, side>>>(c.lvl_list.p, nsmall, c.nd_vf.p, c.nd_vl.p,
                                                                      c.nd_axis.p, c.nd_pivot.p, c.nd_ch1.p, c.x.p,
                                                                      c.y.p, c.perm.p, c.nd_nlow.p, c.nd_bbox.p);
            VV_LAUNCH_CHECK();
        }
        const bool forked = seg1 || nsmall > 0;
        if (nchunk > 0) {
            c.chunk_cnt.reserve((size_t)nchunk + 1);
            c.chunk_pre.reserve((size_t)nchunk + 1);
            k_chunk_count<<<nchunk, CT, 0, s>>>(c.chunk_node.p, c.nd_cbase.p, c.nd_vf.p, c.nd_vl.p, c.nd_axis.p,
                                                c.nd_pivot.p, c.x.p, c.y.p, c.chunk_cnt.p);
            VV_LAUNCH_CHECK();
            exclusive_scan(c, c.chunk_cnt.p, c.chunk_pre.p, nchunk);
            k_chunk_place<<<nchunk, CT, 0, s>>>(c.chunk_node.p, c.nd_cbase.p, c.nd_vf.p, c.nd_vl.p, c.nd_axis.p,
                                                c.nd_pivot.p, c.nd_ch1.p, c.x.p, c.y.p, c.chunk_pre.p, c.tab_rl.p,
                                                c.tab_lh.p, c.nd_npair.p, c.nd_nlow.p, c.nd_bbox.p);
            VV_LAUNCH_CHECK();
            k_chunk_swap<<<nchunk, CT, 0, s>>>(c.chunk_node.p, c.nd_cbase.p, c.nd_vf.p, c.nd_vl.p, c.nd_npair.p,
                                               c.tab_rl.p, c.tab_lh.p, c.x.p, c.y.p, c.perm.p);
            VV_LAUNCH_CHECK();
        }
        if (m > SEG1_MAX) {
            k_sclass<<<grid_for(m, TB), TB, 0, s>>>(m, a, b, c.seg_node_of.p, c.seg_order.p, c.nd_split.p,
                                                    c.nd_axis.p, c.nd_pivot.p, c.s_rx.p, c.s_ry.p, c.flags.p);
            VV_LAUNCH_CHECK();
            exclusive_scan(c, c.flags.p, c.scan.p, m);
            k_sscatter<<<grid_for(m, TB), TB, 0, s>>>(m, a, b, c.seg_node_of.p, c.seg_order.p, c.nd_split.p,
                                                      c.nd_sf.p, c.nd_sl.p, c.nd_ch1.p, c.flags.p, c.scan.p,
                                                      c.nd_nlow_s.p, c.seg_order2.p, c.seg_node_of2.p, c.s_rx.p,
                                                      c.s_ry.p, c.nd_bbox.p);
            VV_LAUNCH_CHECK();
            std::swap(c.seg_order, c.seg_order2);
            std::swap(c.seg_node_of, c.seg_node_of2);
        }
        if (forked) {
            VV_CUDA(cudaEventRecord(c.ev_join, side));
            VV_CUDA(cudaStreamWaitEvent(s, c.ev_join, 0));
        }
        k_finalize<<<grid_for(cnt, TB), TB, 0, s>>>(a, b, cnt, c.nd_split.p, c.nd_ch1.p, c.nd_nlow.p, c.nd_nlow_s.p,
                                                    c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p, c.nd_geom.p,
                                                    c.nd_bbox.p, c.nd_depth.p, min_node, max_node, c.nd_split.p,
                                                    c.nd_pivot.p, c.nd_axis.p, err, c.flags.p, c.lvl_cnt.p);
        VV_LAUNCH_CHECK();
        c.level_begin.push_back(b + 2 * (int64_t)nsplit);
        c.nnodes = b + 2 * (int64_t)nsplit;
    }
    c.depth = (int64_t)c.level_begin.size() - 1;
    // the subtrees the loop deferred (split == 2), one block each, in node order
    const int64_t nn0 = c.nnodes;
    int32_t ndef = 0;
    {
        c.flags.reserve(nn0 + 2);
        c.scan.reserve(nn0 + 2);
        k_defer_flags<<<grid_for(nn0, TB), TB, 0, s>>>(nn0, c.nd_split.p, c.flags.p);
        VV_LAUNCH_CHECK();
        exclusive_scan(c, c.flags.p, c.scan.p, nn0);
        ndef = read_i32(c, c.scan.p + nn0);
        if (ndef > 0) {
            c.sub_i32.reserve(3 * (size_t)ndef + 4);
            int32_t* roots = c.sub_i32.p;
            int32_t* nnew = roots + ndef;
            int32_t* pos = nnew + ndef + 1;
            k_defer_list<<<grid_for(nn0, TB), TB, 0, s>>>(nn0, c.nd_split.p, c.scan.p, roots);
            VV_LAUNCH_CHECK();
            // two 80-byte records per vortex and per segment (2.5 double4 each)
            c.sub_scratch.reserve(5 * (size_t)(n + m) + 4);
            SubNode* scratch = reinterpret_cast<SubNode*>(c.sub_scratch.p);
            int32_t* maxdep = (int32_t*)(c.counters.p + 5);
            // every root goes to both kernels; each builds the subtrees of its kind (without
            // or with segments) and leaves the others
            VV_CUDA(cudaFuncSetAttribute(k_subtree<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SUB_SMEM));
            k_subtree<false><<<ndef, SUB_T, SUB_SMEM, s>>>(
                roots, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p, c.nd_depth.p, c.nd_path.p, c.nd_pivot.p,
                c.nd_axis.p, min_node, max_node, c.x.p, c.y.p, c.perm.p, c.seg_order.p, c.s_rx.p, c.s_ry.p,
                scratch, nnew, err, maxdep);
            VV_LAUNCH_CHECK();
            if (m > 0) {
                VV_CUDA(cudaFuncSetAttribute(k_subtree<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)SUB_SMEM_SEG));
                k_subtree<true><<<ndef, SUB_T, SUB_SMEM_SEG, s>>>(
                    roots, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p, c.nd_depth.p, c.nd_path.p, c.nd_pivot.p,
                    c.nd_axis.p, min_node, max_node, c.x.p, c.y.p, c.perm.p, c.seg_order.p, c.s_rx.p, c.s_ry.p,
                    scratch, nnew, err, maxdep);
                VV_LAUNCH_CHECK();
            }
            exclusive_scan(c, nnew, pos, ndef);
            const int32_t added = read_i32(c, pos + ndef);
            ensure_nodes(nn0 + added + 1);
            k_subtree_place<<<ndef, 128, 0, s>>>(roots, pos, nnew, nn0, scratch, c.nd_geom.p, c.nd_vf.p, c.nd_vl.p,
                                                 c.nd_sf.p, c.nd_sl.p, c.nd_ch1.p, c.nd_depth.p, c.nd_path.p,
                                                 c.nd_parent.p);
            VV_LAUNCH_CHECK();
            c.nnodes = nn0 + added;
            c.depth = std::max<int64_t>(c.depth, (int64_t)read_i32(c, maxdep) + 1);
        }
    }
    if (n > 0) {
        c.ptmp.reserve(4 * (size_t)n);
        c.otmp.reserve(n);
        k_perm_gather<<<grid_for(n, TB), TB, 0, s>>>(n, c.perm.p, c.g.p, c.ie.p, c.vx.p, c.vy.p, c.orig.p, c.ptmp.p,
                                                     c.otmp.p);
        VV_LAUNCH_CHECK();
        k_perm_store<<<grid_for(n, TB), TB, 0, s>>>(n, c.ptmp.p, c.otmp.p, c.g.p, c.ie.p, c.vx.p, c.vy.p, c.orig.p);
        VV_LAUNCH_CHECK();
    }
    if (read_i32(c, err)) throw ApiError{VVGPU_ERR_LIMIT, "tree deeper than supported"};

    // centroids bottom-up, leaf counts, then depth-first leaf order top-down
    const int64_t nn = c.nnodes;
    c.nd_cm.reserve(6 * nn);
    c.nd_lc.reserve(nn);
    c.nd_dfs.reserve(nn);
    c.nd_arrive.reserve(nn);
    VV_CUDA(cudaMemsetAsync(c.nd_arrive.p, 0, nn * sizeof(int32_t), s));
    // the loop's leaves; the subtrees whole (one block each); then the climbs above them
    k_leaf_cm<<<grid_for(nn0, TB), TB, 0, s>>>(nn0, c.nd_ch1.p, c.nd_vf.p, c.nd_vl.p, c.nd_geom.p, c.x.p, c.y.p,
                                               c.g.p, c.nd_cm.p, c.nd_lc.p);
    VV_LAUNCH_CHECK();
    if (ndef > 0) {
        const int32_t* roots = c.sub_i32.p;
        k_subtree_cm<<<ndef, SUB_T, 0, s>>>(roots, roots + 2 * ndef + 1, roots + ndef, nn0, c.nd_vf.p, c.nd_vl.p,
                                            c.nd_ch1.p, c.nd_depth.p, c.nd_geom.p, c.x.p, c.y.p, c.g.p, c.nd_cm.p,
                                            c.nd_lc.p);
        VV_LAUNCH_CHECK();
    }
    k_tree_cm<<<grid_for(nn0, TB), TB, 0, s>>>(nn0, c.nd_ch1.p, ndef > 0 ? c.nd_split.p : nullptr, c.nd_parent.p,
                                               c.nd_geom.p, c.nd_cm.p, c.nd_lc.p, c.nd_arrive.p);
    VV_LAUNCH_CHECK();
    int32_t nl = read_i32(c, c.nd_lc.p);
    c.nleaves = nl;
    c.leaf_node.reserve(nl + 1);
    k_tree_dfs<<<grid_for(nn, TB), TB, 0, s>>>(nn, c.nd_ch1.p, c.nd_parent.p, c.nd_lc.p, c.nd_dfs.p, c.leaf_node.p);
    VV_LAUNCH_CHECK();
    c.lf_vf.reserve(nl + 1); c.lf_vl.reserve(nl + 1); c.lf_sf.reserve(nl + 1); c.lf_sl.reserve(nl + 1);
    c.lf_geom.reserve(nl + 1);
    c.leaf_of.reserve(n + 1);
    k_leaf_arrays<<<grid_for(nl, TB), TB, 0, s>>>(nl, c.leaf_node.p, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p,
                                                  c.nd_geom.p, c.lf_vf.p, c.lf_vl.p, c.lf_sf.p, c.lf_sl.p,
                                                  c.lf_geom.p, c.leaf_of.p);
    VV_LAUNCH_CHECK();
    tree_lists(c);
    c.built = true;
    c.mom_valid = false;
    c.stats.n_vortices = n;
    c.stats.n_segments = m;
    c.stats.n_nodes = nn;
    c.stats.n_leaves = nl;
    c.stats.tree_depth = c.depth;
}

}  // namespace vvgpu
