// C ABI entry points (include/vvgpu.h): context, Space state, inspection exports.
#include <cmath>
#include <exception>
#include <new>

#include "vvgpu_internal.cuh"

using namespace vvgpu;

namespace {

int fail(Ctx& c, int code, const std::string& msg) {
    c.last_error = msg;
    return code;
}

#define API_BEGIN(ctxp)                                          \
    if (!(ctxp)) return VVGPU_ERR_ARG;                           \
    Ctx& c = (ctxp)->c;                                          \
    try {                                                        \
        VV_CUDA(cudaSetDevice(c.device));

#define API_END                                                                        \
    }                                                                                  \
    catch (ApiError & e) { return fail(c, e.code, e.msg); }                            \
    catch (CudaError & e) {                                                            \
        return fail(c, VVGPU_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.err)); \
    }                                                                                  \
    catch (std::bad_alloc&) { return fail(c, VVGPU_ERR_NOMEM, "host allocation failed"); } \
    catch (std::exception & e) { return fail(c, VVGPU_ERR_ARG, e.what()); }            \
    return VVGPU_OK;

double abs2h(double x, double y) { return x * x + y * y; }

// TBody::doUpdateSegments (TBody.cpp:200-215) and doFillProperties (TBody.cpp:283-343).
void body_update(Ctx& c, BodyHost& b) {
    int64_t f = b.first, n = b.count;
    for (int64_t k = 0; k < n; k++) {
        int64_t i = f + k, j = f + (k + 1) % n;
        c.h_dlx[i] = c.h_cx[j] - c.h_cx[i];
        c.h_dly[i] = c.h_cy[j] - c.h_cy[i];
        c.h_sie[i] = 3.0 / std::sqrt(abs2h(c.h_dlx[i], c.h_dly[i]));
        c.h_rx[i] = (c.h_cx[j] + c.h_cx[i]) * 0.5;
        c.h_ry[i] = (c.h_cy[j] + c.h_cy[i]) * 0.5;
    }
    b.slen = 0;
    b.area = 0;
    for (int64_t k = 0; k < n; k++) {
        int64_t i = f + k;
        b.slen += std::sqrt(abs2h(c.h_dlx[i], c.h_dly[i]));
        b.area += c.h_ry[i] * c.h_dlx[i];
    }
    if (b.area == 0) {
        double lx = 0, ly = 0;
        for (int64_t k = 0; k < n; k++) {
            int64_t i = f + k;
            double l = std::sqrt(abs2h(c.h_dlx[i], c.h_dly[i]));
            lx += c.h_rx[i] * l;
            ly += c.h_ry[i] * l;
        }
        double inv = 1. / b.slen;
        b.cofm_x = lx * inv;
        b.cofm_y = ly * inv;
        b.moi_cofm = 0.;
    } else {
        double sx = 0, sy = 0, m0 = 0;
        for (int64_t k = 0; k < n; k++) {
            int64_t i = f + k, j = f + (k + 1) % n;
            double cr = (-c.h_cy[i]) * c.h_cx[j] + c.h_cx[i] * c.h_cy[j];
            sx -= c.h_rx[i] * cr;
            sy -= c.h_ry[i] * cr;
            m0 -= (abs2h(c.h_cx[i], c.h_cy[i]) + (c.h_cx[i] * c.h_cx[j] + c.h_cy[i] * c.h_cy[j]) +
                   abs2h(c.h_cx[j], c.h_cy[j])) * cr;
        }
        double inv = 1. / (3 * b.area);
        b.cofm_x = sx * inv;
        b.cofm_y = sy * inv;
        b.moi_cofm = m0 / 12. - b.area * abs2h(b.cofm_x, b.cofm_y);
    }
}

template <class T>
void h2d(DArr<T>& d, const T* h, int64_t n, cudaStream_t s) {
    d.reserve((size_t)(n > 0 ? n : 1));
    if (n > 0) VV_CUDA(cudaMemcpyAsync(d.p, h, (size_t)n * sizeof(T), cudaMemcpyHostToDevice, s));
}

template <class T>
void d2h(T* h, const T* d, int64_t n, cudaStream_t s) {
    if (h && n > 0) VV_CUDA(cudaMemcpyAsync(h, d, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, s));
}

__global__ void k_i32_to_i64(const int32_t* in, int64_t* out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}

__global__ void k_iota64(int64_t* out, int64_t n, int64_t base) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = base + i;
}

// orig = 0..n-1, and *bad = 1 if a position or circulation is not finite or an inverse
// epsilon is NaN or negative (+inf is a valid _1_eps: coincident vortices have epsilon 0)
// Device snapshot of the list for the download beside later calls: the five arrays side by
// side (orig as its 64-bit pattern), each only when its host pointer was given (bit k of
// want).  One kernel instead of five device-to-device copies, which the copy engine runs
// at a fraction of the SMs' copy rate.
__global__ void k_snapshot(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ g, const double* __restrict__ ie,
                           const int64_t* __restrict__ orig, unsigned want, double* __restrict__ snap) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (want & 1u) snap[i] = x[i];
    if (want & 2u) snap[n + i] = y[i];
    if (want & 4u) snap[2 * n + i] = g[i];
    if (want & 8u) snap[3 * n + i] = ie[i];
    if (want & 16u) snap[4 * n + i] = __longlong_as_double((long long)orig[i]);
}

__global__ void k_set_orig_check(int64_t n, int64_t* __restrict__ orig, const double* __restrict__ x,
                                 const double* __restrict__ y, const double* __restrict__ g,
                                 const double* __restrict__ ie, int32_t* bad) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool b = false;
    if (i < n) {
        orig[i] = i;
        b = !isfinite(x[i]) || !isfinite(y[i]) || !isfinite(g[i]);
        if (ie) b = b || !(ie[i] >= 0.0);
    }
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) *bad = 1;
}

}  // namespace

namespace vvgpu {

void upload_segments(Ctx& c) {
    if (!c.segs_dirty) return;
    cudaStream_t s = c.st();
    int64_t m = c.m;
    h2d(c.s_cx, c.h_cx.data(), m, s);
    h2d(c.s_cy, c.h_cy.data(), m, s);
    h2d(c.s_rx, c.h_rx.data(), m, s);
    h2d(c.s_ry, c.h_ry.data(), m, s);
    h2d(c.s_dlx, c.h_dlx.data(), m, s);
    h2d(c.s_dly, c.h_dly.data(), m, s);
    h2d(c.s_ie, c.h_sie.data(), m, s);
    h2d(c.s_slip, c.h_slip.data(), m, s);
    VV_CUDA(cudaStreamSynchronize(s));
    c.segs_dirty = false;
}

void collect_kernel_timing(Ctx& c) {
    if (c.ev_rec.empty()) return;
    VV_CUDA(cudaEventSynchronize(c.ev_rec.back().b));
    for (auto& r : c.ev_rec) {
        float ms = 0;
        VV_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        c.t_ms[r.slot] += ms;
        c.t_count[r.slot]++;
        c.ev_free.push_back(r.a);
        c.ev_free.push_back(r.b);
    }
    c.ev_rec.clear();
}

void check_input(Ctx& c) {
    if (!c.in_pending) return;
    c.in_pending = false;
    if (read_i32(c, c.in_bad.p))
        throw ApiError{VVGPU_ERR_ARG, "vortex list holds a non-finite position or circulation, or a NaN or "
                                      "negative inverse epsilon"};
}

void ensure_vortex_capacity(Ctx& c, int64_t n, bool keep) {
    size_t need = (size_t)(n > 0 ? n : 1);
    cudaStream_t s = c.st();
    c.x.reserve(need, keep, c.n, s);
    c.y.reserve(need, keep, c.n, s);
    c.g.reserve(need, keep, c.n, s);
    c.ie.reserve(need, keep, c.n, s);
    c.vx.reserve(need, keep, c.n, s);
    c.vy.reserve(need, keep, c.n, s);
    c.orig.reserve(need, keep, c.n, s);
}

}  // namespace vvgpu

extern "C" {

int vvgpu_ctx_create(const vvgpu_cfg* cfg, vvgpu_ctx** out) {
    if (!out) return VVGPU_ERR_ARG;
    *out = nullptr;
    vvgpu_ctx* h = nullptr;
    try {
        h = new vvgpu_ctx();
    } catch (std::bad_alloc&) {
        return VVGPU_ERR_NOMEM;
    }
    Ctx& c = h->c;
    c.device = cfg ? cfg->device : 0;
    c.precision = cfg ? cfg->precision : VVGPU_FP64;
    if (c.precision != VVGPU_FP64 && c.precision != VVGPU_FP32) {
        delete h;
        return VVGPU_ERR_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || c.device < 0 || c.device >= ndev) {
        cudaGetLastError();
        delete h;
        return VVGPU_ERR_CUDA;
    }
    if (cudaSetDevice(c.device) != cudaSuccess || cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return VVGPU_ERR_CUDA;
    }
    c.stream = c.own_stream;
    // pinned host words for the small device reads of the step (counts, flags)
    if (cudaMallocHost(&c.h_pin, 512) != cudaSuccess) {
        cudaGetLastError();
        c.h_pin = nullptr;  // the reads then go through pageable memory
    }
    try {
        if (cfg && cfg->reserve_vortices > 0) ensure_vortex_capacity(c, cfg->reserve_vortices, false);
    } catch (...) {
        if (c.h_pin) cudaFreeHost(c.h_pin);
        cudaStreamDestroy(c.own_stream);
        delete h;
        return VVGPU_ERR_NOMEM;
    }
    *out = h;
    return VVGPU_OK;
}

int vvgpu_ctx_destroy(vvgpu_ctx* h) {
    if (!h) return VVGPU_ERR_ARG;
    Ctx& c = h->c;
    cudaSetDevice(c.device);
    cudaStreamSynchronize(c.stream);
    if (c.side) cudaStreamSynchronize(c.side);
    if (c.dl_stream) cudaStreamSynchronize(c.dl_stream);
    cudaStream_t own = c.own_stream, side = c.side, dls = c.dl_stream;
    cudaEvent_t e1 = c.ev_fork, e2 = c.ev_join, e3 = c.dl_ready, e4 = c.dl_done;
    for (auto& r : c.ev_rec) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : c.ev_free) cudaEventDestroy(e);
    if (c.h_pin) cudaFreeHost(c.h_pin);
    delete h;  // device arrays are released by their destructors
    if (own) cudaStreamDestroy(own);
    if (side) cudaStreamDestroy(side);
    if (e1) cudaEventDestroy(e1);
    if (e2) cudaEventDestroy(e2);
    if (dls) cudaStreamDestroy(dls);
    if (e3) cudaEventDestroy(e3);
    if (e4) cudaEventDestroy(e4);
    return VVGPU_OK;
}

const char* vvgpu_last_error(const vvgpu_ctx* h) { return h ? h->c.last_error.c_str() : "null context"; }

int vvgpu_set_precision(vvgpu_ctx* h, int precision) {
    API_BEGIN(h)
    if (precision != VVGPU_FP64 && precision != VVGPU_FP32) throw ApiError{VVGPU_ERR_ARG, "unknown precision"};
    c.precision = precision;
    API_END
}

int vvgpu_set_stream(vvgpu_ctx* h, void* stream) {
    API_BEGIN(h)
    VV_CUDA(cudaStreamSynchronize(c.stream));
    c.stream = stream ? (cudaStream_t)stream : c.own_stream;
    API_END
}

int vvgpu_set_eps_round_limit(vvgpu_ctx* h, int64_t max_rounds) {
    API_BEGIN(h)
    if (max_rounds < 1) throw ApiError{VVGPU_ERR_ARG, "the round limit must be at least 1"};
    c.eps_max_rounds = max_rounds;
    API_END
}

int vvgpu_autotune_tiles(vvgpu_ctx* h, int32_t* conv_tile, int32_t* diff_targets, double* ms) {
    API_BEGIN(h)
    autotune_tiles(c, ms);
    if (conv_tile) *conv_tile = c.conv_tile;
    if (diff_targets) *diff_targets = c.diff_targets;
    API_END
}

int vvgpu_set_tiles(vvgpu_ctx* h, int32_t conv_tile, int32_t diff_targets) {
    API_BEGIN(h)
    if (!(conv_tile == 128 || conv_tile == 192 || conv_tile == 256) || !(diff_targets == 1 || diff_targets == 2))
        throw ApiError{VVGPU_ERR_ARG, "tile shapes: conv_tile 128, 192 or 256; diff_targets 1 or 2"};
    c.conv_tile = conv_tile;
    c.diff_targets = diff_targets;
    API_END
}

int vvgpu_get_tiles(vvgpu_ctx* h, int32_t* conv_tile, int32_t* diff_targets) {
    API_BEGIN(h)
    if (conv_tile) *conv_tile = c.conv_tile;
    if (diff_targets) *diff_targets = c.diff_targets;
    API_END
}

int vvgpu_set_autotune(vvgpu_ctx* h, int on) {
    API_BEGIN(h)
    c.tune_pending = on != 0;
    API_END
}

int vvgpu_set_wait_limit(vvgpu_ctx* h, uint32_t spins) {
    API_BEGIN(h)
    c.wait_spins = spins;
    API_END
}

int vvgpu_set_kernel_timing(vvgpu_ctx* h, int on) {
    API_BEGIN(h)
    collect_kernel_timing(c);
    c.timing = on != 0;
    for (int k = 0; k < VVGPU_T_COUNT; k++) { c.t_ms[k] = 0; c.t_count[k] = 0; }
    API_END
}

int vvgpu_get_kernel_timing(vvgpu_ctx* h, double* ms, int64_t* launches) {
    API_BEGIN(h)
    collect_kernel_timing(c);
    for (int k = 0; k < VVGPU_T_COUNT; k++) {
        if (ms) ms[k] = c.t_ms[k];
        if (launches) launches[k] = c.t_count[k];
    }
    API_END
}

int vvgpu_synchronize(vvgpu_ctx* h) {
    API_BEGIN(h)
    VV_CUDA(cudaStreamSynchronize(c.stream));
    API_END
}

int vvgpu_get_stats(const vvgpu_ctx* h, vvgpu_stats* out) {
    if (!h || !out) return VVGPU_ERR_ARG;
    *out = h->c.stats;
    out->reserved[0] = h->c.launches;
    out->reserved[1] = h->c.eps_evaluations;
    out->reserved[2] = h->c.diff_sources;
    out->reserved[3] = h->c.eps_records;
    out->reserved[4] = h->c.walk_loads;
    return VVGPU_OK;
}

int vvgpu_set_params(vvgpu_ctx* h, double re, double dt, double inf_vx, double inf_vy, double inf_g,
                     double time, double gravity_x, double gravity_y) {
    API_BEGIN(h)
    if (!(re > 0)) throw ApiError{VVGPU_ERR_ARG, "re must be > 0"};
    if (!(dt > 0)) throw ApiError{VVGPU_ERR_ARG, "dt must be > 0"};
    c.re = re; c.dt = dt; c.inf_vx = inf_vx; c.inf_vy = inf_vy; c.inf_g = inf_g; c.time = time;
    c.grav_x = gravity_x; c.grav_y = gravity_y;
    API_END
}

int vvgpu_add_body(vvgpu_ctx* h, int64_t nseg, const double* cx, const double* cy, const uint32_t* slip,
                   const vvgpu_body_params* bp) {
    API_BEGIN(h)
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "cannot add a body while the tree is built"};
    if (nseg < 2 || !cx || !cy) throw ApiError{VVGPU_ERR_ARG, "a body needs at least two corners"};
    int64_t m0 = c.m, m = c.m + nseg;
    for (auto* v : {&c.h_cx, &c.h_cy, &c.h_rx, &c.h_ry, &c.h_dlx, &c.h_dly, &c.h_sie}) v->resize(m);
    c.h_slip.resize(m);
    for (int64_t k = 0; k < nseg; k++) {
        c.h_cx[m0 + k] = cx[k];
        c.h_cy[m0 + k] = cy[k];
        c.h_slip[m0 + k] = slip ? slip[k] : 0;
    }
    BodyHost b{};
    b.first = m0;
    b.count = nseg;
    if (bp) {
        b.p = *bp;
    } else {
        b.p = vvgpu_body_params{};
        b.p.density = 1.0;
        b.p.kspring_x = b.p.kspring_y = b.p.kspring_o = INFINITY;
    }
    c.m = m;
    body_update(c, b);
    c.bodies.push_back(b);
    // device-resident per-segment state: g, fric, gsum (grow, keep old values)
    cudaStream_t s = c.st();
    c.s_g.reserve(m, true, m0, s);
    c.s_fric.reserve(m, true, m0, s);
    c.s_gsum.reserve(m, true, m0, s);
    c.s_cp.reserve(m, true, m0, s);
    c.s_fr.reserve(m, true, m0, s);
    c.s_nu.reserve(m, true, m0, s);
    for (auto* a : {&c.s_g, &c.s_fric, &c.s_gsum, &c.s_cp, &c.s_fr, &c.s_nu})
        VV_CUDA(cudaMemsetAsync(a->p + m0, 0, nseg * sizeof(double), s));
    c.segs_dirty = true;
    c.lu_valid = false;
    c.seg_version++;
    API_END
}

int vvgpu_set_segment_g(vvgpu_ctx* h, const double* g) {
    API_BEGIN(h)
    if (!g) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    if (c.m) VV_CUDA(cudaMemcpyAsync(c.s_g.p, g, c.m * sizeof(double), cudaMemcpyHostToDevice, c.st()));
    VV_CUDA(cudaStreamSynchronize(c.st()));
    API_END
}

int vvgpu_set_segment_state(vvgpu_ctx* h, const double* g, const double* fric, const double* gsum) {
    API_BEGIN(h)
    cudaStream_t s = c.st();
    if (c.m) {
        if (g) VV_CUDA(cudaMemcpyAsync(c.s_g.p, g, c.m * sizeof(double), cudaMemcpyHostToDevice, s));
        if (fric) VV_CUDA(cudaMemcpyAsync(c.s_fric.p, fric, c.m * sizeof(double), cudaMemcpyHostToDevice, s));
        if (gsum) VV_CUDA(cudaMemcpyAsync(c.s_gsum.p, gsum, c.m * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    VV_CUDA(cudaStreamSynchronize(s));
    API_END
}

int vvgpu_clear_bodies(vvgpu_ctx* h) {
    API_BEGIN(h)
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "cannot clear bodies while the tree is built"};
    c.bodies.clear();
    c.m = 0;
    for (auto* v : {&c.h_cx, &c.h_cy, &c.h_rx, &c.h_ry, &c.h_dlx, &c.h_dly, &c.h_sie}) v->clear();
    c.h_slip.clear();
    c.segs_dirty = true;
    c.lu_valid = false;
    c.seg_version++;
    API_END
}

int vvgpu_set_body_params(vvgpu_ctx* h, int body, const vvgpu_body_params* params) {
    API_BEGIN(h)
    if (body < 0 || body >= (int)c.bodies.size() || !params) throw ApiError{VVGPU_ERR_ARG, "no such body"};
    c.bodies[body].p = *params;
    API_END
}

int vvgpu_set_velocities(vvgpu_ctx* h, const double* vx, const double* vy) {
    API_BEGIN(h)
    if (c.n && (!vx || !vy)) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    if (c.n) {
        VV_CUDA(cudaMemcpyAsync(c.vx.p, vx, c.n * sizeof(double), cudaMemcpyHostToDevice, c.st()));
        VV_CUDA(cudaMemcpyAsync(c.vy.p, vy, c.n * sizeof(double), cudaMemcpyHostToDevice, c.st()));
    }
    VV_CUDA(cudaStreamSynchronize(c.st()));
    API_END
}

int vvgpu_set_sinks(vvgpu_ctx* h, int64_t n, const double* x, const double* y, const double* g) {
    API_BEGIN(h)
    if (n < 0 || (n && (!x || !y || !g))) throw ApiError{VVGPU_ERR_ARG, "bad sink arrays"};
    h2d(c.k_x, x, n, c.st());
    h2d(c.k_y, y, n, c.st());
    h2d(c.k_g, g, n, c.st());
    VV_CUDA(cudaStreamSynchronize(c.st()));
    c.ns = n;
    API_END
}

static int set_vortices_impl(vvgpu_ctx* h, int64_t n, const double* x, const double* y, const double* g,
                             const double* ie, cudaMemcpyKind kind) {
    API_BEGIN(h)
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "cannot replace vortices while the tree is built"};
    if (n < 0 || (n && (!x || !y || !g))) throw ApiError{VVGPU_ERR_ARG, "bad vortex arrays"};
    if (n > 0x3fffffff) throw ApiError{VVGPU_ERR_LIMIT, "more than 2^30 vortices"};
    ensure_vortex_capacity(c, n, false);
    cudaStream_t s = c.st();
    size_t bytes = (size_t)n * sizeof(double);
    if (n) {
        VV_CUDA(cudaMemcpyAsync(c.x.p, x, bytes, kind, s));
        VV_CUDA(cudaMemcpyAsync(c.y.p, y, bytes, kind, s));
        VV_CUDA(cudaMemcpyAsync(c.g.p, g, bytes, kind, s));
        if (ie) VV_CUDA(cudaMemcpyAsync(c.ie.p, ie, bytes, kind, s));
        else VV_CUDA(cudaMemsetAsync(c.ie.p, 0, bytes, s));
        VV_CUDA(cudaMemsetAsync(c.vx.p, 0, bytes, s));
        VV_CUDA(cudaMemsetAsync(c.vy.p, 0, bytes, s));
        // the check is read by the next call that consumes the list (check_input)
        c.in_bad.reserve(1);
        VV_CUDA(cudaMemsetAsync(c.in_bad.p, 0, 4, s));
        k_set_orig_check<<<grid_for(n, 256), 256, 0, s>>>(n, c.orig.p, c.x.p, c.y.p, c.g.p, ie ? c.ie.p : nullptr,
                                                          c.in_bad.p);
        VV_LAUNCH_CHECK();
        c.in_pending = true;
    } else {
        c.in_pending = false;
    }
    c.n = n;
    c.next_orig = n;
    if (kind == cudaMemcpyHostToDevice) VV_CUDA(cudaStreamSynchronize(s));
    API_END
}

int vvgpu_set_vortices(vvgpu_ctx* h, int64_t n, const double* x, const double* y, const double* g,
                       const double* ie) {
    return set_vortices_impl(h, n, x, y, g, ie, cudaMemcpyHostToDevice);
}

int vvgpu_set_vortices_device(vvgpu_ctx* h, int64_t n, const double* x, const double* y, const double* g,
                              const double* ie) {
    return set_vortices_impl(h, n, x, y, g, ie, cudaMemcpyDeviceToDevice);
}

int64_t vvgpu_num_vortices(const vvgpu_ctx* h) { return h ? h->c.n : -1; }
int64_t vvgpu_num_segments(const vvgpu_ctx* h) { return h ? h->c.m : -1; }

int vvgpu_get_vortices(vvgpu_ctx* h, double* x, double* y, double* g, double* ie, double* vx, double* vy,
                       int64_t* orig) {
    API_BEGIN(h)
    cudaStream_t s = c.st();
    d2h(x, c.x.p, c.n, s);
    d2h(y, c.y.p, c.n, s);
    d2h(g, c.g.p, c.n, s);
    d2h(ie, c.ie.p, c.n, s);
    d2h(vx, c.vx.p, c.n, s);
    d2h(vy, c.vy.p, c.n, s);
    d2h(orig, c.orig.p, c.n, s);
    VV_CUDA(cudaStreamSynchronize(s));
    API_END
}

int vvgpu_get_vortices_async(vvgpu_ctx* h, double* x, double* y, double* g, double* ie, int64_t* orig) {
    API_BEGIN(h)
    if (c.dl_pending) {
        c.dl_pending = false;
        VV_CUDA(cudaEventSynchronize(c.dl_done));
    }
    if (!c.dl_stream) {
        VV_CUDA(cudaStreamCreateWithFlags(&c.dl_stream, cudaStreamNonBlocking));
        VV_CUDA(cudaEventCreateWithFlags(&c.dl_ready, cudaEventDisableTiming));
        VV_CUDA(cudaEventCreateWithFlags(&c.dl_done, cudaEventDisableTiming));
    }
    const int64_t n = c.n;
    if (n > 0) {
        cudaStream_t s = c.st();
        c.dl_snap.reserve((size_t)5 * n);
        double* snap = c.dl_snap.p;
        const size_t bytes = (size_t)n * 8;
        void* dst[5] = {x, y, g, ie, orig};
        unsigned want = 0;
        for (int k = 0; k < 5; k++)
            if (dst[k]) want |= 1u << k;
        k_snapshot<<<grid_for(n, 256), 256, 0, s>>>(n, c.x.p, c.y.p, c.g.p, c.ie.p, c.orig.p, want, snap);
        VV_LAUNCH_CHECK();
        VV_CUDA(cudaEventRecord(c.dl_ready, s));
        VV_CUDA(cudaStreamWaitEvent(c.dl_stream, c.dl_ready, 0));
        for (int k = 0; k < 5; k++)
            if (dst[k]) VV_CUDA(cudaMemcpyAsync(dst[k], snap + k * n, bytes, cudaMemcpyDeviceToHost, c.dl_stream));
        VV_CUDA(cudaEventRecord(c.dl_done, c.dl_stream));
        c.dl_pending = true;
    }
    API_END
}

int vvgpu_wait_vortices(vvgpu_ctx* h) {
    API_BEGIN(h)
    if (c.dl_pending) {
        c.dl_pending = false;
        VV_CUDA(cudaEventSynchronize(c.dl_done));
    }
    API_END
}

int vvgpu_device_arrays(vvgpu_ctx* h, double** x, double** y, double** g, double** ie, double** vx, double** vy) {
    API_BEGIN(h)
    if (x) *x = c.x.p;
    if (y) *y = c.y.p;
    if (g) *g = c.g.p;
    if (ie) *ie = c.ie.p;
    if (vx) *vx = c.vx.p;
    if (vy) *vy = c.vy.p;
    API_END
}

int vvgpu_get_segments(vvgpu_ctx* h, double* rx, double* ry, double* dlx, double* dly, double* ie, double* g,
                       double* fric, double* gsum) {
    API_BEGIN(h)
    int64_t m = c.m;
    auto cp = [&](double* dst, const std::vector<double>& src) {
        if (dst && m) memcpy(dst, src.data(), m * sizeof(double));
    };
    cp(rx, c.h_rx); cp(ry, c.h_ry); cp(dlx, c.h_dlx); cp(dly, c.h_dly); cp(ie, c.h_sie);
    cudaStream_t s = c.st();
    d2h(g, c.s_g.p, m, s);
    d2h(fric, c.s_fric.p, m, s);
    d2h(gsum, c.s_gsum.p, m, s);
    VV_CUDA(cudaStreamSynchronize(s));
    API_END
}

int vvgpu_get_body_geom(vvgpu_ctx* h, int bi, double* area, double* cofm_x, double* cofm_y, double* moi_axis,
                        double* slen) {
    API_BEGIN(h)
    if (bi < 0 || bi >= (int)c.bodies.size()) throw ApiError{VVGPU_ERR_ARG, "no such body"};
    const BodyHost& b = c.bodies[bi];
    double ax = b.p.holder_x + b.p.dpos_x, ay = b.p.holder_y + b.p.dpos_y;
    if (area) *area = b.area;
    if (cofm_x) *cofm_x = b.cofm_x;
    if (cofm_y) *cofm_y = b.cofm_y;
    if (moi_axis) *moi_axis = b.moi_cofm + abs2h(ax - b.cofm_x, ay - b.cofm_y) * b.area;
    if (slen) *slen = b.slen;
    API_END
}

int vvgpu_tree_build(vvgpu_ctx* h, double far_criteria, double min_node, double max_node) {
    API_BEGIN(h)
    if (!(far_criteria > 0) || std::isnan(min_node) || std::isnan(max_node))
        throw ApiError{VVGPU_ERR_ARG, "bad tree parameters"};
    KernelTimer kt(c, VVGPU_T_TREE_BUILD);
    tree_build(c, far_criteria, min_node, max_node);
    API_END
}

int vvgpu_tree_destroy(vvgpu_ctx* h) {
    API_BEGIN(h)
    c.built = false;
    c.lists_full = false;
    c.far_kept = false;
    API_END
}

int vvgpu_eps(vvgpu_ctx* h, int merge, int64_t* merged) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    ensure_full_lists(c);
    {
        KernelTimer kt(c, VVGPU_T_EPS_PASS);
        eps_pass(c, merge, merged);
    }
    c.mom_valid = false;  // merges move circulation
    API_END
}

int vvgpu_convective(vvgpu_ctx* h) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    ensure_full_lists(c);
    convective(c);
    API_END
}

int vvgpu_diffusive(vvgpu_ctx* h) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    ensure_full_lists(c);
    diffusive(c);
    API_END
}

int vvgpu_velocity_points(vvgpu_ctx* h, int64_t n, const double* px, const double* py, double* vx, double* vy) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    if (n < 0 || (n && (!px || !py || !vx || !vy))) throw ApiError{VVGPU_ERR_ARG, "bad point arrays"};
    ensure_full_lists(c);
    velocity_points(c, n, px, py, vx, vy);
    API_END
}

int vvgpu_slae(vvgpu_ctx* h, vvgpu_body_out* out) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    KernelTimer kt(c, VVGPU_T_SLAE);
    slae(c, out);
    API_END
}

int vvgpu_vortex_shed(vvgpu_ctx* h) {
    API_BEGIN(h)
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "shed with the tree built"};
    vortex_shed(c);
    API_END
}

int vvgpu_move_and_clean(vvgpu_ctx* h, int remove, int64_t* cleaned) {
    API_BEGIN(h)
    if (c.built) throw ApiError{VVGPU_ERR_STATE, "move_and_clean with the tree built"};
    move_and_clean(c, remove, cleaned);
    API_END
}

int vvgpu_calc_forces(vvgpu_ctx* h, double* out4) {
    API_BEGIN(h)
    calc_forces(c, out4);
    API_END
}

int vvgpu_zero_forces(vvgpu_ctx* h) {
    API_BEGIN(h)
    zero_forces(c);
    API_END
}

int vvgpu_get_segment_forces(vvgpu_ctx* h, double* cp, double* fr, double* nu) {
    API_BEGIN(h)
    cudaStream_t s = c.st();
    d2h(cp, c.s_cp.p, c.m, s);
    d2h(fr, c.s_fr.p, c.m, s);
    d2h(nu, c.s_nu.p, c.m, s);
    VV_CUDA(cudaStreamSynchronize(s));
    API_END
}

int vvgpu_get_body_params(vvgpu_ctx* h, int body, vvgpu_body_params* out) {
    API_BEGIN(h)
    if (body < 0 || body >= (int)c.bodies.size() || !out) throw ApiError{VVGPU_ERR_ARG, "bad body index"};
    *out = c.bodies[body].p;
    API_END
}

int vvgpu_direct_velocity(vvgpu_ctx* h, int64_t n, const double* px, const double* py, double* vx, double* vy) {
    API_BEGIN(h)
    if (n < 0 || (n && (!px || !py || !vx || !vy))) throw ApiError{VVGPU_ERR_ARG, "bad point arrays"};
    direct_velocity(c, n, px, py, vx, vy);
    API_END
}

int vvgpu_field_velocity(vvgpu_ctx* h, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                         char mode, char ref_frame, float* out) {
    API_BEGIN(h)
    if (!out) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    field_velocity(c, xmin, ymin, dxdy, xres, yres, mode, ref_frame, out);
    API_END
}

int vvgpu_field_streamfunction(vvgpu_ctx* h, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                               double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                               uint16_t* gap_yj, float* gap, int64_t* ngaps) {
    API_BEGIN(h)
    if (!out || gap_cap < 0 || (gap_cap > 0 && (!gap_xi || !gap_yj || !gap)))
        throw ApiError{VVGPU_ERR_ARG, "bad output arrays"};
    field_streamfunction(c, xmin, ymin, dxdy, xres, yres, eps_mult, ref_frame, out, gap_cap, gap_xi, gap_yj, gap,
                         ngaps);
    API_END
}

int vvgpu_field_vorticity(vvgpu_ctx* h, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                          double eps_mult, float* out) {
    API_BEGIN(h)
    if (!out) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    field_vorticity(c, xmin, ymin, dxdy, xres, yres, eps_mult, out);
    API_END
}

int vvgpu_gsum(vvgpu_ctx* h, double* out) {
    API_BEGIN(h)
    if (!out) throw ApiError{VVGPU_ERR_ARG, "null pointer"};
    *out = gsum(c);
    API_END
}

int vvgpu_tree_sizes(vvgpu_ctx* h, int64_t* nnodes, int64_t* nleaves, int64_t* nnear, int64_t* nfar) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    ensure_full_lists(c);
    std::vector<int2> runs(c.n_near_runs);
    d2h(runs.data(), c.near_run.p, c.n_near_runs, c.st());
    VV_CUDA(cudaStreamSynchronize(c.st()));
    int64_t tot = 0;
    for (auto& r : runs) tot += r.y - r.x;
    std::vector<int32_t> foff, fnode;
    if (nfar) tree_lists_exact(c, foff, fnode, false);
    if (nnodes) *nnodes = c.nnodes;
    if (nleaves) *nleaves = c.nleaves;
    if (nnear) *nnear = tot;
    if (nfar) *nfar = foff.empty() ? 0 : (int64_t)foff.back();
    API_END
}

int vvgpu_tree_leaves(vvgpu_ctx* h, double* x, double* y, double* hh, double* w, int64_t* vfirst, int64_t* vlast,
                      int32_t* depth, int64_t* path, int64_t* sfirst, int64_t* slast) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    int64_t nl = c.nleaves;
    cudaStream_t s = c.st();
    std::vector<double4> gm(nl);
    std::vector<int32_t> vf(nl), vl(nl), sf(nl), sl(nl), ln(nl), dep(c.nnodes);
    std::vector<int64_t> pth(c.nnodes);
    d2h(gm.data(), c.lf_geom.p, nl, s);
    d2h(vf.data(), c.lf_vf.p, nl, s);
    d2h(vl.data(), c.lf_vl.p, nl, s);
    d2h(sf.data(), c.lf_sf.p, nl, s);
    d2h(sl.data(), c.lf_sl.p, nl, s);
    d2h(ln.data(), c.leaf_node.p, nl, s);
    d2h(dep.data(), c.nd_depth.p, c.nnodes, s);
    d2h(pth.data(), c.nd_path.p, c.nnodes, s);
    VV_CUDA(cudaStreamSynchronize(s));
    for (int64_t L = 0; L < nl; L++) {
        if (x) x[L] = gm[L].x;
        if (y) y[L] = gm[L].y;
        if (hh) hh[L] = gm[L].z;
        if (w) w[L] = gm[L].w;
        if (vfirst) vfirst[L] = vf[L];
        if (vlast) vlast[L] = vl[L];
        if (sfirst) sfirst[L] = sf[L];
        if (slast) slast[L] = sl[L];
        if (depth) depth[L] = dep[ln[L]];
        if (path) path[L] = pth[ln[L]];
    }
    API_END
}

int vvgpu_tree_nodes(vvgpu_ctx* h, double* x, double* y, double* hh, double* w, int64_t* vfirst, int64_t* vlast,
                     int32_t* depth, int64_t* path, double* cmp_x, double* cmp_y, double* cmp_g, double* cmm_x,
                     double* cmm_y, double* cmm_g) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    int64_t nn = c.nnodes;
    cudaStream_t s = c.st();
    std::vector<double4> gm(nn);
    std::vector<int32_t> vf(nn), vl(nn), dep(nn);
    std::vector<int64_t> pth(nn);
    std::vector<double> cm(6 * nn);
    d2h(gm.data(), c.nd_geom.p, nn, s);
    d2h(vf.data(), c.nd_vf.p, nn, s);
    d2h(vl.data(), c.nd_vl.p, nn, s);
    d2h(dep.data(), c.nd_depth.p, nn, s);
    d2h(pth.data(), c.nd_path.p, nn, s);
    d2h(cm.data(), c.nd_cm.p, 6 * nn, s);
    VV_CUDA(cudaStreamSynchronize(s));
    for (int64_t k = 0; k < nn; k++) {
        if (x) x[k] = gm[k].x;
        if (y) y[k] = gm[k].y;
        if (hh) hh[k] = gm[k].z;
        if (w) w[k] = gm[k].w;
        if (vfirst) vfirst[k] = vf[k];
        if (vlast) vlast[k] = vl[k];
        if (depth) depth[k] = dep[k];
        if (path) path[k] = pth[k];
        if (cmp_x) cmp_x[k] = cm[6 * k + 0];
        if (cmp_y) cmp_y[k] = cm[6 * k + 1];
        if (cmp_g) cmp_g[k] = cm[6 * k + 2];
        if (cmm_x) cmm_x[k] = cm[6 * k + 3];
        if (cmm_y) cmm_y[k] = cm[6 * k + 4];
        if (cmm_g) cmm_g[k] = cm[6 * k + 5];
    }
    API_END
}

int vvgpu_tree_seg_order(vvgpu_ctx* h, int64_t* seg_order) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    std::vector<int32_t> so(c.m);
    d2h(so.data(), c.seg_order.p, c.m, c.st());
    VV_CUDA(cudaStreamSynchronize(c.st()));
    for (int64_t k = 0; k < c.m; k++) seg_order[k] = so[k];
    API_END
}

int vvgpu_tree_lists(vvgpu_ctx* h, int64_t* near_off, int32_t* near_depth, int64_t* near_path, int64_t* far_off,
                     int32_t* far_depth, int64_t* far_path) {
    API_BEGIN(h)
    if (!c.built) throw ApiError{VVGPU_ERR_NOT_BUILT, "tree is not built"};
    ensure_full_lists(c);
    int64_t nl = c.nleaves, nn = c.nnodes;
    cudaStream_t s = c.st();
    std::vector<int32_t> noff(nl + 1), foff, fnode, ln(nl), dep(nn);
    std::vector<int2> runs(c.n_near_runs);
    std::vector<int64_t> pth(nn);
    tree_lists_exact(c, foff, fnode, far_depth || far_path);
    d2h(noff.data(), c.near_off.p, nl + 1, s);
    d2h(runs.data(), c.near_run.p, c.n_near_runs, s);
    d2h(ln.data(), c.leaf_node.p, nl, s);
    d2h(dep.data(), c.nd_depth.p, nn, s);
    d2h(pth.data(), c.nd_path.p, nn, s);
    VV_CUDA(cudaStreamSynchronize(s));
    int64_t k = 0;
    for (int64_t L = 0; L < nl; L++) {
        if (near_off) near_off[L] = k;
        for (int32_t r = noff[L]; r < noff[L + 1]; r++)
            for (int32_t q = runs[r].x; q < runs[r].y; q++) {
                if (near_depth) near_depth[k] = dep[ln[q]];
                if (near_path) near_path[k] = pth[ln[q]];
                k++;
            }
    }
    if (near_off) near_off[nl] = k;
    for (int64_t L = 0; L <= nl; L++)
        if (far_off) far_off[L] = foff[L];
    for (int64_t q = 0; q < (int64_t)fnode.size(); q++) {
        if (far_depth) far_depth[q] = dep[fnode[q]];
        if (far_path) far_path[q] = pth[fnode[q]];
    }
    API_END
}

int64_t vvgpu_slae_size(const vvgpu_ctx* h) {
    if (!h) return -1;
    return h->c.m + 9 * (int64_t)h->c.bodies.size();
}

int vvgpu_slae_export(vvgpu_ctx* h, double* matrix, double* rhs, double* solution) {
    API_BEGIN(h)
    if (!c.neq) throw ApiError{VVGPU_ERR_STATE, "no system filled yet"};
    int64_t n = c.neq;
    cudaStream_t s = c.st();
    d2h(matrix, c.A.p, n * n, s);
    d2h(rhs, c.B.p, n, s);
    d2h(solution, c.X.p, n, s);
    VV_CUDA(cudaStreamSynchronize(s));
    API_END
}

}  // extern "C"
