// Bisection tree of libvvhd (stree/snode, libvvhd/src/TSortedTree.cpp) built on the GPU.
//
// The reference splits a node at the midpoint of its bounding box along the longer side
// and partitions the node's slice of VortexList in place with a two-pointer swap loop
// (DistributeContent, TSortedTree.cpp:81-99).  That loop is a set of disjoint swaps: with
// L = #{key < pivot} in the slice [f, l), the k-th element with key >= pivot inside [f, f+L)
// (counted from the left) trades places with the k-th element with key < pivot inside
// [f+L, l) (counted from the right).  Here every level of the tree is split at once:
// one exclusive scan of the "low" flags gives every element its rank, the right-side lows
// publish their positions in a table, and each left-side high performs its swap.  Only the
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

// Segmented (by node id, contiguous within the warp) min/max reduction, then one atomic
// per segment head.  node < 0 marks lanes that do not contribute.  The reduction runs on
// the order-preserving integer keys of the coordinates (dkey), so it stays on the integer
// pipe (FP64 min/max would run on sm_103's narrow FP64 pipe).
__device__ __forceinline__ void warp_bbox_update(int node, double px, double py, unsigned long long* bbox) {
    const int lane = threadIdx.x & 31;
    const unsigned long long kx = dkey(px), ky = dkey(py);
    unsigned long long mnx = kx, mny = ky, mxx = kx, mxy = ky;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int on = __shfl_down_sync(0xffffffffu, node, o);
        const unsigned long long a = __shfl_down_sync(0xffffffffu, mnx, o);
        const unsigned long long b = __shfl_down_sync(0xffffffffu, mny, o);
        const unsigned long long cc = __shfl_down_sync(0xffffffffu, mxx, o);
        const unsigned long long d = __shfl_down_sync(0xffffffffu, mxy, o);
        if (lane + o < 32 && on == node) {
            mnx = a < mnx ? a : mnx;
            mny = b < mny ? b : mny;
            mxx = cc > mxx ? cc : mxx;
            mxy = d > mxy ? d : mxy;
        }
    }
    const int prev = __shfl_up_sync(0xffffffffu, node, 1);
    const bool head = (lane == 0) || (prev != node);
    if (head && node >= 0) {
        unsigned long long* s = bbox + 4 * (size_t)node;
        atomicMin(s + 0, mnx);
        atomicMin(s + 1, mny);
        atomicMax(s + 2, mxx);
        atomicMax(s + 3, mxy);
    }
}

__global__ void k_init_root(int32_t* node_of, int32_t* perm, int64_t n, int32_t* seg_order, int32_t* seg_node_of,
                            int64_t m, unsigned long long* bbox) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) { node_of[i] = 0; perm[i] = (int32_t)i; }
    if (i < m) { seg_order[i] = (int32_t)i; seg_node_of[i] = 0; }
    if (i == 0) {
        bbox[0] = dkey(DBL_MAX); bbox[1] = dkey(DBL_MAX);
        bbox[2] = dkey(-DBL_MAX); bbox[3] = dkey(-DBL_MAX);
    }
}

// Root box over all segment centres and all vortices (snode::Stretch, TSortedTree.cpp:101-137).
__global__ void k_root_bbox(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                            const double* __restrict__ rx, const double* __restrict__ ry, int64_t m,
                            unsigned long long* bbox) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int node = -1;
    double px = 0, py = 0;
    if (i < n) { node = 0; px = x[i]; py = y[i]; }
    else if (i - n < m && i >= n) { node = 0; px = rx[i - n]; py = ry[i - n]; }
    warp_bbox_update(node, px, py, bbox);
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

// snode::DivideNode leaf rules (TSortedTree.cpp:36-56).
__global__ void k_decide(int64_t a, int64_t cnt, const double4* __restrict__ geom, const int32_t* __restrict__ vf,
                         const int32_t* __restrict__ vl, const int32_t* __restrict__ sf, const int32_t* __restrict__ sl,
                         const int32_t* __restrict__ depth, double min_node, double max_node, int32_t* split,
                         int32_t* flags, double* pivot, int32_t* axis, int32_t* err) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    int64_t k = a + t;
    double4 gm = geom[k];
    double h = gm.z, w = gm.w;
    double mx = smax(h, w), mn = smin(h, w);
    int64_t nv = (int64_t)vl[k] - vf[k], ns = (int64_t)sl[k] - sf[k];
    int64_t maxlist = nv > ns ? nv : ns;
    bool leaf = (mx < max_node && mn <= min_node) || (mx < max_node && maxlist < TREE_MAX_LIST_SIZE);
    int s = leaf ? 0 : 1;
    if (s && depth[k] >= MAX_DEPTH) { s = 0; atomicExch(err, 1); }
    split[k] = s;
    flags[t] = s;
    bool byx = h < w;
    axis[k] = byx ? 1 : 0;
    pivot[k] = byx ? gm.x : gm.y;
}

__global__ void k_children(int64_t a, int64_t b, int64_t cnt, const int32_t* __restrict__ split,
                           const int32_t* __restrict__ lscan, int32_t* ch1, int32_t* depth, int64_t* path,
                           unsigned long long* bbox, int32_t* nlow, int32_t* nlow_s) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    int64_t k = a + t;
    if (!split[k]) { ch1[k] = -1; return; }
    int64_t c1 = b + 2 * (int64_t)lscan[t];
    ch1[k] = (int32_t)c1;
    nlow[k] = 0;
    nlow_s[k] = 0;
    for (int q = 0; q < 2; q++) {
        int64_t c = c1 + q;
        ch1[c] = -1;
        depth[c] = depth[k] + 1;
        path[c] = path[k] * 2 + q;
        unsigned long long* s = bbox + 4 * c;
        s[0] = dkey(DBL_MAX); s[1] = dkey(DBL_MAX);
        s[2] = dkey(-DBL_MAX); s[3] = dkey(-DBL_MAX);
    }
}

__device__ __forceinline__ bool in_level_split(int32_t k, int64_t a, int64_t b, const int32_t* split) {
    return k >= a && k < b && split[k];
}

__global__ void k_vclass(int64_t n, int64_t a, int64_t b, const int32_t* __restrict__ node_of,
                         const int32_t* __restrict__ split, const int32_t* __restrict__ axis,
                         const double* __restrict__ pivot, const double* __restrict__ x,
                         const double* __restrict__ y, int32_t* flags) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t k = node_of[i];
    int f = 0;
    if (in_level_split(k, a, b, split)) {
        double key = axis[k] ? x[i] : y[i];
        f = key < pivot[k];
    }
    flags[i] = f;
}

__global__ void k_vrank(int64_t n, int64_t a, int64_t b, const int32_t* __restrict__ node_of,
                        const int32_t* __restrict__ split, const int32_t* __restrict__ vf,
                        const int32_t* __restrict__ vl, const int32_t* __restrict__ flags,
                        const int32_t* __restrict__ S, int32_t* nlow, int32_t* tab_rl) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t k = node_of[i];
    if (!in_level_split(k, a, b, split)) return;
    int32_t f = vf[k], l = vl[k];
    int32_t L = S[l] - S[f];
    if (i == f) nlow[k] = L;
    if (i >= f + L && flags[i]) {
        int32_t r = S[l] - S[i + 1];  // lows strictly to the right of i inside the node
        tab_rl[f + r] = (int32_t)i;
    }
}

__global__ void k_vswap(int64_t n, int64_t a, int64_t b, const int32_t* __restrict__ node_of,
                        const int32_t* __restrict__ split, const int32_t* __restrict__ vf,
                        const int32_t* __restrict__ nlow, const int32_t* __restrict__ flags,
                        const int32_t* __restrict__ S, const int32_t* __restrict__ tab_rl, double* x,
                        double* y, int32_t* perm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t k = node_of[i];
    if (!in_level_split(k, a, b, split)) return;
    int32_t f = vf[k], L = nlow[k];
    if (i >= f + L || flags[i]) return;
    int32_t kk = (int32_t)(i - f) - (S[i] - S[f]);  // highs to the left of i inside the node
    int64_t j = tab_rl[f + kk];
    // the keys move at every level; the rest of the record follows once, through perm
    const double tx = x[i], ty = y[i];
    x[i] = x[j]; y[i] = y[j];
    x[j] = tx; y[j] = ty;
    const int32_t tp = perm[i];
    perm[i] = perm[j];
    perm[j] = tp;
}

// Applies the partition's permutation to the rest of the vortex record (two passes through
// staging buffers, so the arrays keep their device addresses).
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

__global__ void k_vassign(int64_t n, int64_t a, int64_t b, int32_t* node_of, const int32_t* __restrict__ split,
                          const int32_t* __restrict__ vf, const int32_t* __restrict__ nlow,
                          const int32_t* __restrict__ ch1, const double* __restrict__ x,
                          const double* __restrict__ y, unsigned long long* bbox) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int node = -1;
    double px = 0, py = 0;
    if (i < n) {
        int32_t k = node_of[i];
        if (in_level_split(k, a, b, split)) {
            node = ch1[k] + ((i >= vf[k] + nlow[k]) ? 1 : 0);
            node_of[i] = node;
            px = x[i]; py = y[i];
        }
    }
    // A block whose elements all go to one child (the rule near the root, where children
    // are large) reduces in shared memory and makes 4 atomics instead of 4 per warp.
    __shared__ int s_node0;
    __shared__ unsigned long long s_red[TB / 32][4];
    if (threadIdx.x == 0) s_node0 = node;
    __syncthreads();
    if (__syncthreads_and(node == s_node0)) {
        if (node < 0) return;
        unsigned long long k0 = dkey(px), k1 = dkey(py), k2 = k0, k3 = k1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long a0 = __shfl_xor_sync(0xffffffffu, k0, o);
            const unsigned long long a1 = __shfl_xor_sync(0xffffffffu, k1, o);
            const unsigned long long a2 = __shfl_xor_sync(0xffffffffu, k2, o);
            const unsigned long long a3 = __shfl_xor_sync(0xffffffffu, k3, o);
            k0 = a0 < k0 ? a0 : k0; k1 = a1 < k1 ? a1 : k1;
            k2 = a2 > k2 ? a2 : k2; k3 = a3 > k3 ? a3 : k3;
        }
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) { s_red[w][0] = k0; s_red[w][1] = k1; s_red[w][2] = k2; s_red[w][3] = k3; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int q = 1; q < (int)(blockDim.x >> 5); q++) {
                k0 = s_red[q][0] < k0 ? s_red[q][0] : k0; k1 = s_red[q][1] < k1 ? s_red[q][1] : k1;
                k2 = s_red[q][2] > k2 ? s_red[q][2] : k2; k3 = s_red[q][3] > k3 ? s_red[q][3] : k3;
            }
            unsigned long long* sb = bbox + 4 * (size_t)node;
            atomicMin(sb + 0, k0);
            atomicMin(sb + 1, k1);
            atomicMax(sb + 2, k2);
            atomicMax(sb + 3, k3);
        }
        return;
    }
    warp_bbox_update(node, px, py, bbox);
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

__global__ void k_finalize(int64_t a, int64_t cnt, const int32_t* __restrict__ split, const int32_t* __restrict__ ch1,
                           const int32_t* __restrict__ nlow, const int32_t* __restrict__ nlow_s, int32_t* vf,
                           int32_t* vl, int32_t* sf, int32_t* sl, double4* geom, const unsigned long long* bbox) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    int64_t k = a + t;
    if (!split[k]) return;
    int32_t c1 = ch1[k], c2 = c1 + 1;
    vf[c1] = vf[k]; vl[c1] = vf[k] + nlow[k];
    vf[c2] = vf[k] + nlow[k]; vl[c2] = vl[k];
    sf[c1] = sf[k]; sl[c1] = sf[k] + nlow_s[k];
    sf[c2] = sf[k] + nlow_s[k]; sl[c2] = sl[k];
    geom[c1] = geom_from_bbox(bbox + 4 * (size_t)c1);
    geom[c2] = geom_from_bbox(bbox + 4 * (size_t)c2);
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

__global__ void k_inner_cm(int64_t a, int64_t cnt, const int32_t* __restrict__ ch1, const double4* __restrict__ geom,
                           double* cm, int32_t* lc) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    int64_t k = a + t;
    int32_t c1 = ch1[k];
    if (c1 < 0) return;
    double4 gm = geom[k];
    const double* A = cm + 6 * (size_t)c1;
    const double* B = cm + 6 * (size_t)(c1 + 1);
    double* o = cm + 6 * k;
    combine_cm(A, B, o, gm.x, gm.y);
    combine_cm(A + 3, B + 3, o + 3, gm.x, gm.y);
    lc[k] = lc[c1] + lc[c1 + 1];
}

__global__ void k_dfs(int64_t a, int64_t cnt, const int32_t* __restrict__ ch1, const int32_t* __restrict__ lc,
                      int32_t* dfs, int32_t* leaf_node) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    int64_t k = a + t;
    if (k == 0) dfs[0] = 0;
    int32_t c1 = ch1[k];
    if (c1 < 0) { leaf_node[dfs[k]] = (int32_t)k; return; }
    dfs[c1] = dfs[k];
    dfs[c1 + 1] = dfs[k] + lc[c1];
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
    };
    c.nnodes = 1;
    ensure_nodes(cap_nodes);
    c.node_of.reserve(n + 1);
    c.flags.reserve(n + m + 2);
    c.scan.reserve(n + m + 2);
    c.tab_rl.reserve(n + 1);
    c.seg_order.reserve(m + 1); c.seg_order2.reserve(m + 1);
    c.seg_node_of.reserve(m + 1); c.seg_node_of2.reserve(m + 1);
    c.counters.reserve(16);
    VV_CUDA(cudaMemsetAsync(c.counters.p, 0, 16 * sizeof(unsigned long long), s));
    int32_t* err = (int32_t*)c.counters.p;

    int64_t nm = n > m ? n : m;
    c.perm.reserve(n + 1);
    k_init_root<<<grid_for(nm, TB), TB, 0, s>>>(c.node_of.p, c.perm.p, n, c.seg_order.p, c.seg_node_of.p, m,
                                                c.nd_bbox.p);
    VV_LAUNCH_CHECK();
    if (n + m > 0) {
        k_root_bbox<<<grid_for(n + m, TB), TB, 0, s>>>(c.x.p, c.y.p, n, c.s_rx.p, c.s_ry.p, m, c.nd_bbox.p);
        VV_LAUNCH_CHECK();
    }
    k_finalize_root<<<1, 1, 0, s>>>(c.nd_geom.p, c.nd_bbox.p, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p,
                                    c.nd_ch1.p, c.nd_depth.p, c.nd_path.p, n, m);
    VV_LAUNCH_CHECK();

    c.level_begin.assign({0, 1});
    int64_t d = 0;
    for (;; d++) {
        int64_t a = c.level_begin[d], b = c.level_begin[d + 1], cnt = b - a;
        if (cnt <= 0) break;
        ensure_nodes(b + 2 * cnt);
        c.flags.reserve(cnt + 1);
        c.scan.reserve(cnt + 2);
        k_decide<<<grid_for(cnt, TB), TB, 0, s>>>(a, cnt, c.nd_geom.p, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p,
                                                  c.nd_depth.p, min_node, max_node, c.nd_split.p, c.flags.p,
                                                  c.nd_pivot.p, c.nd_axis.p, err);
        VV_LAUNCH_CHECK();
        exclusive_scan(c, c.flags.p, c.scan.p, cnt);
        k_children<<<grid_for(cnt, TB), TB, 0, s>>>(a, b, cnt, c.nd_split.p, c.scan.p, c.nd_ch1.p, c.nd_depth.p,
                                                    c.nd_path.p, c.nd_bbox.p, c.nd_nlow.p, c.nd_nlow_s.p);
        VV_LAUNCH_CHECK();
        int32_t nsplit = read_i32(c, c.scan.p + cnt);
        if (nsplit == 0) break;
        if (n > 0) {
            k_vclass<<<grid_for(n, TB), TB, 0, s>>>(n, a, b, c.node_of.p, c.nd_split.p, c.nd_axis.p, c.nd_pivot.p,
                                                    c.x.p, c.y.p, c.flags.p);
            VV_LAUNCH_CHECK();
            exclusive_scan(c, c.flags.p, c.scan.p, n);
            k_vrank<<<grid_for(n, TB), TB, 0, s>>>(n, a, b, c.node_of.p, c.nd_split.p, c.nd_vf.p, c.nd_vl.p,
                                                   c.flags.p, c.scan.p, c.nd_nlow.p, c.tab_rl.p);
            VV_LAUNCH_CHECK();
            k_vswap<<<grid_for(n, TB), TB, 0, s>>>(n, a, b, c.node_of.p, c.nd_split.p, c.nd_vf.p, c.nd_nlow.p,
                                                   c.flags.p, c.scan.p, c.tab_rl.p, c.x.p, c.y.p, c.perm.p);
            VV_LAUNCH_CHECK();
            k_vassign<<<grid_for(n, TB), TB, 0, s>>>(n, a, b, c.node_of.p, c.nd_split.p, c.nd_vf.p, c.nd_nlow.p,
                                                     c.nd_ch1.p, c.x.p, c.y.p, c.nd_bbox.p);
            VV_LAUNCH_CHECK();
        }
        if (m > 0) {
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
        k_finalize<<<grid_for(cnt, TB), TB, 0, s>>>(a, cnt, c.nd_split.p, c.nd_ch1.p, c.nd_nlow.p, c.nd_nlow_s.p,
                                                    c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p, c.nd_geom.p,
                                                    c.nd_bbox.p);
        VV_LAUNCH_CHECK();
        c.level_begin.push_back(b + 2 * (int64_t)nsplit);
        c.nnodes = b + 2 * (int64_t)nsplit;
    }
    c.depth = (int64_t)c.level_begin.size() - 1;
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
    k_leaf_cm<<<grid_for(nn, TB), TB, 0, s>>>(nn, c.nd_ch1.p, c.nd_vf.p, c.nd_vl.p, c.nd_geom.p, c.x.p, c.y.p,
                                              c.g.p, c.nd_cm.p, c.nd_lc.p);
    VV_LAUNCH_CHECK();
    const int64_t nlev = (int64_t)c.level_begin.size() - 1;
    for (int64_t lv = nlev - 1; lv >= 0; lv--) {
        int64_t a = c.level_begin[lv], b = c.level_begin[lv + 1];
        if (b > nn) b = nn;
        if (b <= a) continue;
        k_inner_cm<<<grid_for(b - a, TB), TB, 0, s>>>(a, b - a, c.nd_ch1.p, c.nd_geom.p, c.nd_cm.p, c.nd_lc.p);
        VV_LAUNCH_CHECK();
    }
    int32_t nl = read_i32(c, c.nd_lc.p);
    c.nleaves = nl;
    c.leaf_node.reserve(nl + 1);
    for (int64_t lv = 0; lv < nlev; lv++) {
        int64_t a = c.level_begin[lv], b = c.level_begin[lv + 1];
        if (b > nn) b = nn;
        if (b <= a) continue;
        k_dfs<<<grid_for(b - a, TB), TB, 0, s>>>(a, b - a, c.nd_ch1.p, c.nd_lc.p, c.nd_dfs.p, c.leaf_node.p);
        VV_LAUNCH_CHECK();
    }
    c.lf_vf.reserve(nl + 1); c.lf_vl.reserve(nl + 1); c.lf_sf.reserve(nl + 1); c.lf_sl.reserve(nl + 1);
    c.lf_geom.reserve(nl + 1);
    c.leaf_of.reserve(n + 1);
    k_leaf_arrays<<<grid_for(nl, TB), TB, 0, s>>>(nl, c.leaf_node.p, c.nd_vf.p, c.nd_vl.p, c.nd_sf.p, c.nd_sl.p,
                                                  c.nd_geom.p, c.lf_vf.p, c.lf_vl.p, c.lf_sf.p, c.lf_sl.p,
                                                  c.lf_geom.p, c.leaf_of.p);
    VV_LAUNCH_CHECK();
    tree_lists(c);
    c.built = true;
    c.stats.n_vortices = n;
    c.stats.n_segments = m;
    c.stats.n_nodes = nn;
    c.stats.n_leaves = nl;
    c.stats.tree_depth = c.depth;
}

}  // namespace vvgpu
