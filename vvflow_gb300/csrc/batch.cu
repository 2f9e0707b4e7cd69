// Batched sweep: one call advances many independent simulations (contexts of uneven size)
// by one step of simulate() (utils/vvflow/vvflow.cpp:214-255), optionally followed by
// MFlowmove::move_and_clean.  Every context keeps its own stream, buffers, bodies and
// parameters (nu, dt, tree sizes), so each instance computes exactly what it computes alone.
//
// The host side is a pool of threads: each takes the next instance, largest first (longest
// processing time first keeps the tail short with sizes spread over 40x), and issues that
// instance's launches on its stream, so the GPU runs many instances at once while the
// per-level host reads of one instance's tree build overlap the kernels of the others.
// vvgpu_batch_autotune first has every instance time its own kernel shapes in its next step
// (sources per staged tile of the convective near field, targets per pass of the diffusive
// pass; vvgpu_autotune_tiles), then times the pool sizes it is given on real steps and keeps
// the fastest.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "vvgpu_internal.cuh"

namespace {

int run_step(vvgpu_ctx* h, const vvgpu_step_cfg& s) {
    int rc;
    vvgpu_body_out out[64];
    const int nb = (int)h->c.bodies.size();
    std::vector<vvgpu_body_out> big;
    vvgpu_body_out* o = out;
    if (nb > 64) {
        big.resize((size_t)nb);
        o = big.data();
    }
    if ((rc = vvgpu_tree_build(h, s.far_criteria, s.min_node, s.max_node))) return rc;
    if ((rc = vvgpu_slae(h, o))) return rc;
    if ((rc = vvgpu_tree_destroy(h))) return rc;
    if ((rc = vvgpu_vortex_shed(h))) return rc;
    if ((rc = vvgpu_tree_build(h, s.far_criteria, s.min_node, s.max_node))) return rc;
    int64_t merged = 0;
    if ((rc = vvgpu_eps(h, s.merge, &merged))) return rc;
    if ((rc = vvgpu_convective(h))) return rc;
    if ((rc = vvgpu_diffusive(h))) return rc;
    if ((rc = vvgpu_tree_destroy(h))) return rc;
    if (s.move) {
        int64_t cleaned = 0;
        if ((rc = vvgpu_move_and_clean(h, 1, &cleaned))) return rc;
    }
    return vvgpu_synchronize(h);
}

}  // namespace

extern "C" int vvgpu_batch_step(vvgpu_ctx* const* ctxs, int64_t count, const vvgpu_step_cfg* cfgs, int32_t nthreads,
                                double* step_ms, int32_t* status) {
    if (count < 0 || (count > 0 && (!ctxs || !cfgs))) return VVGPU_ERR_ARG;
    for (int64_t i = 0; i < count; i++)
        if (!ctxs[i]) return VVGPU_ERR_ARG;
    if (count == 0) return 0;
    std::vector<int64_t> order((size_t)count);
    for (int64_t i = 0; i < count; i++) order[(size_t)i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return vvgpu_num_vortices(ctxs[a]) > vvgpu_num_vortices(ctxs[b]);
    });
    int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt = (int)std::min<int64_t>(nt, count);
    std::atomic<int64_t> next{0};
    std::vector<int32_t> rcs((size_t)count, 0);
    auto worker = [&] {
        for (;;) {
            const int64_t k = next.fetch_add(1);
            if (k >= count) return;
            const int64_t i = order[(size_t)k];
            const auto t0 = std::chrono::steady_clock::now();
            const int rc = run_step(ctxs[i], cfgs[i]);
            const auto t1 = std::chrono::steady_clock::now();
            rcs[(size_t)i] = rc;
            if (step_ms) step_ms[i] = std::chrono::duration<double, std::milli>(t1 - t0).count();
        }
    };
    std::vector<std::thread> pool;
    pool.reserve((size_t)nt - 1);
    try {
        for (int t = 1; t < nt; t++) pool.emplace_back(worker);
    } catch (...) {
        // fewer threads than asked: the ones that started and this one finish the work
    }
    worker();
    for (auto& th : pool) th.join();
    int first = 0;
    for (int64_t i = 0; i < count; i++) {
        if (status) status[i] = rcs[(size_t)i];
        if (!first && rcs[(size_t)i]) first = rcs[(size_t)i];
    }
    return first;
}

extern "C" int vvgpu_batch_autotune(vvgpu_ctx* const* ctxs, int64_t count, const vvgpu_step_cfg* cfgs,
                                    const int32_t* candidates, int32_t ncand, int32_t* best, double* best_ms) {
    if (!candidates || ncand <= 0 || !best) return VVGPU_ERR_ARG;
    if (count < 0 || (count > 0 && !ctxs)) return VVGPU_ERR_ARG;
    // each instance's kernel shapes, timed on its own tree in the first step below
    for (int64_t i = 0; i < count; i++) {
        if (!ctxs[i]) return VVGPU_ERR_ARG;
        const int rc = vvgpu_set_autotune(ctxs[i], 1);
        if (rc) return rc;
    }
    double bt = 0;
    int32_t bc = -1;
    for (int32_t k = 0; k < ncand; k++) {
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = vvgpu_batch_step(ctxs, count, cfgs, candidates[k], nullptr, nullptr);
        const auto t1 = std::chrono::steady_clock::now();
        if (rc) return rc;
        const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        if (bc < 0 || ms < bt) {
            bt = ms;
            bc = candidates[k];
        }
    }
    *best = bc;
    if (best_ms) *best_ms = bt;
    return 0;
}
