// vvgpu_modules.hpp -- drop-in C++ classes for libvvhd's per-step velocity path.
//
// Header-only templates over the host Space type.  They keep the constructors and methods
// that simulate() and the X* fields use (libvvhd/headers/TSortedTree.hpp:60-92,
// MConvectiveFast.hpp:8-26, MEpsilonFast.hpp:5-18, MDiffusiveFast.hpp:5-11), so a build of
// vvflow switches with four aliases:
//
//     #include "vvgpu_modules.hpp"
//     using TSortedTree     = vvgpu_cxx::stree<Space>;
//     using MConvectiveFast = vvgpu_cxx::MConvectiveFast<Space>;
//     using MEpsilonFast    = vvgpu_cxx::MEpsilonFast<Space>;
//     using MDiffusiveFast  = vvgpu_cxx::MDiffusiveFast<Space>;
//
// The host Space stays the source of truth.  stree::build() uploads the vortex list, the
// bodies and the per-segment state, builds the tree on the GPU and applies the GPU's
// permutation to Space::VortexList in place (the reference permutes it the same way).
// The modules run on the GPU and write their results back into the Space:
//   CalcEpsilonFast -> TObj::r, g, _1_eps;  process_all_lists / process_vort_list -> TObj::v;
//   process_vort_list -> TAtt::fric;  calc_circulation -> TAtt::g and the TBody unknowns.
// Errors raise vvgpu_cxx::error (derived from std::runtime_error) where the reference
// exits; std::invalid_argument where the reference throws it.
//
// Space requirements (duck-typed): VortexList (vector of objects with r.x, r.y, g, v.x, v.y,
// _1_eps), BodyList (vector of shared pointers to bodies with alist of segments having
// corner, g, fric, gsum, slip, and the rigid-body fields of TBody), re, dt and time
// convertible to double, inf_speed(), inf_g, gravity, HeatList.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "vvgpu.h"

namespace vvgpu_cxx {

class error : public std::runtime_error {
   public:
    int code;
    error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(vvgpu_ctx* ctx, int rc, const char* what) {
    if (rc != VVGPU_OK)
        throw error(rc, std::string(what) + " failed (" + std::to_string(rc) + "): " +
                            (ctx ? vvgpu_last_error(ctx) : "no context"));
}

template <class SpaceT>
using obj_t = typename std::decay<decltype(std::declval<SpaceT&>().VortexList[0])>::type;
template <class SpaceT>
using body_t = typename std::decay<decltype(*std::declval<SpaceT&>().BodyList[0])>::type;
template <class SpaceT>
using vec_t = typename std::decay<decltype(std::declval<SpaceT&>().VortexList[0].r)>::type;

template <class SpaceT>
class stree;

// Host view of one tree node with the members snode exposes (TSortedTree.hpp:22-58).
template <class SpaceT>
struct snode {
    using TObj = obj_t<SpaceT>;
    struct range {
        TObj* first = nullptr;
        TObj* last = nullptr;
        size_t size() const { return (size_t)(last - first); }
    };
    double x = 0, y = 0, h = 0, w = 0;
    int i = 0;         // depth
    long long j = 0;   // path bits (ch1 -> 2j, ch2 -> 2j+1)
    TObj CMp{}, CMm{};
    std::vector<TObj*> bllist;
    range vRange, hRange, sRange;
    std::vector<snode*>* NearNodes = nullptr;
    std::vector<snode*>* FarNodes = nullptr;
    snode* ch1 = nullptr;
    snode* ch2 = nullptr;
};

template <class SpaceT>
class stree {
   public:
    using TObj = obj_t<SpaceT>;
    using TVec = vec_t<SpaceT>;
    using node_t = snode<SpaceT>;

    stree(SpaceT* S, int farCriteria, double minNodeSize, double maxNodeSize = std::numeric_limits<double>::max(),
          int precision = VVGPU_FP64, int device = 0)
        : stree(S, (double)farCriteria, minNodeSize, maxNodeSize, precision, device) {}
    stree(SpaceT* S, double farCriteria, double minNodeSize, double maxNodeSize, int precision, int device)
        : S_(S), fc_(farCriteria), min_(minNodeSize), max_(maxNodeSize) {
        vvgpu_cfg cfg{device, precision, 0, 0};
        check(nullptr, vvgpu_ctx_create(&cfg, &ctx_), "vvgpu_ctx_create");
    }
    stree() = delete;
    stree(const stree&) = delete;
    stree& operator=(const stree&) = delete;
    ~stree() {
        if (ctx_) vvgpu_ctx_destroy(ctx_);
    }

    // stree::build (TSortedTree.cpp:232-265); heat and streak lists are not supported.
    void build(bool includeV = true, bool includeB = true, bool includeH = true) {
        (void)includeH;
        if (built_) {
            fprintf(stderr, "Tree is already built\n");
            return;
        }
        if (!S_->HeatList.empty()) throw error(VVGPU_ERR_UNSUPPORTED, "heat particles are not supported");
        sync_params();
        if (includeB) sync_bodies();
        upload_vortices(includeV);
        check(ctx_, vvgpu_tree_build(ctx_, fc_, min_, max_), "vvgpu_tree_build");
        built_ = true;
        apply_permutation();
        mirror_.clear();
    }

    void destroy() {
        check(ctx_, vvgpu_tree_destroy(ctx_), "vvgpu_tree_destroy");
        built_ = false;
        mirror_.clear();
        bottom_.clear();
    }

    const std::vector<node_t*>& getBottomNodes() const {
        if (!built_) {
            fprintf(stderr, "PANIC in stree::getBottomNodes()! Tree isn't built\n");
            return bottom_;
        }
        ensure_mirror();
        return bottom_;
    }

    const node_t* findNode(TVec p) const {
        if (!built_) throw std::invalid_argument("TTree::findNode(): tree is not built");
        ensure_mirror();
        const node_t* n = root_;
        while (n && n->ch1) {
            if (n->h < n->w) n = (p.x < n->x) ? n->ch1 : n->ch2;
            else n = (p.y < n->y) ? n->ch1 : n->ch2;
        }
        return n;
    }

    void printBottomNodes(FILE* f, bool PrintDepth = false) const {
        for (auto* b : getBottomNodes()) {
            fprintf(f, "%g\t%g\t%g\t%g\t", b->x, b->y, b->w, b->h);
            if (PrintDepth) fprintf(f, "\t%d", b->i);
            fprintf(f, "\n");
        }
    }

    // ---- used by the module classes ----
    vvgpu_ctx* gpu() const { return ctx_; }
    SpaceT* space() const { return S_; }
    bool built() const { return built_; }

    // Copies the GPU's vortex list (fields selected by the mask) into Space::VortexList.
    enum { F_R = 1, F_G = 2, F_EPS = 4, F_V = 8 };
    void download_vortices(int fields) const {
        auto& V = S_->VortexList;
        const size_t n = V.size();
        if ((int64_t)n != vvgpu_num_vortices(ctx_)) throw error(VVGPU_ERR_STATE, "vortex list changed size");
        std::vector<double> x(n), y(n), g(n), ie(n), vx(n), vy(n);
        check(ctx_, vvgpu_get_vortices(ctx_, (fields & F_R) ? x.data() : nullptr, (fields & F_R) ? y.data() : nullptr,
                                       (fields & F_G) ? g.data() : nullptr, (fields & F_EPS) ? ie.data() : nullptr,
                                       (fields & F_V) ? vx.data() : nullptr, (fields & F_V) ? vy.data() : nullptr,
                                       nullptr),
              "vvgpu_get_vortices");
        for (size_t k = 0; k < n; k++) {
            if (fields & F_R) { V[k].r.x = x[k]; V[k].r.y = y[k]; }
            if (fields & F_G) V[k].g = g[k];
            if (fields & F_EPS) V[k]._1_eps = ie[k];
            if (fields & F_V) { V[k].v.x = vx[k]; V[k].v.y = vy[k]; }
        }
    }

    void upload_velocities() const {
        auto& V = S_->VortexList;
        std::vector<double> vx(V.size()), vy(V.size());
        for (size_t k = 0; k < V.size(); k++) { vx[k] = V[k].v.x; vy[k] = V[k].v.y; }
        check(ctx_, vvgpu_set_velocities(ctx_, vx.data(), vy.data()), "vvgpu_set_velocities");
    }

    // Segment fields in BodyList order.
    template <class F>
    void for_segments(F f) const {
        for (auto& b : S_->BodyList)
            for (auto& a : b->alist) f(a);
    }

    static vvgpu_body_params body_params(const SpaceT& S, const body_t<SpaceT>& b) {
        vvgpu_body_params p{};
        auto sp = b.speed(double(S.time));
        p.holder_x = b.holder.r.x; p.holder_y = b.holder.r.y; p.holder_o = b.holder.o;
        p.dpos_x = b.dpos.r.x; p.dpos_y = b.dpos.r.y; p.dpos_o = b.dpos.o;
        p.speed_x = sp.r.x; p.speed_y = sp.r.y; p.speed_o = sp.o;
        p.speed_slae_x = b.speed_slae.r.x; p.speed_slae_y = b.speed_slae.r.y; p.speed_slae_o = b.speed_slae.o;
        p.speed_slae_prev_x = b.speed_slae_prev.r.x; p.speed_slae_prev_y = b.speed_slae_prev.r.y;
        p.speed_slae_prev_o = b.speed_slae_prev.o;
        p.friction_prev_x = b.friction_prev.r.x; p.friction_prev_y = b.friction_prev.r.y;
        p.friction_prev_o = b.friction_prev.o;
        p.fdt_dead_x = b.fdt_dead.r.x; p.fdt_dead_y = b.fdt_dead.r.y; p.fdt_dead_o = b.fdt_dead.o;
        p.g_dead = b.g_dead;
        p.density = b.density;
        p.kspring_x = b.kspring.r.x; p.kspring_y = b.kspring.r.y; p.kspring_o = b.kspring.o;
        p.special_segment_no = b.special_segment_no;
        p.bc_kutta = (b.boundary_condition == decltype(b.boundary_condition)::kutta) ? 1 : 0;
        return p;
    }

   private:
    void sync_params() {
        auto inf = S_->inf_speed();
        check(ctx_, vvgpu_set_params(ctx_, S_->re, double(S_->dt), inf.x, inf.y, S_->inf_g, double(S_->time),
                                     S_->gravity.x, S_->gravity.y),
              "vvgpu_set_params");
    }

    void sync_bodies() {
        std::vector<double> corners;
        std::vector<size_t> sizes;
        for (auto& b : S_->BodyList) {
            sizes.push_back(b->alist.size());
            for (auto& a : b->alist) { corners.push_back(a.corner.x); corners.push_back(a.corner.y); }
        }
        if (corners != corners_ || sizes != sizes_) {
            check(ctx_, vvgpu_clear_bodies(ctx_), "vvgpu_clear_bodies");
            for (auto& b : S_->BodyList) {
                const size_t m = b->alist.size();
                std::vector<double> cx(m), cy(m);
                std::vector<uint32_t> slip(m);
                for (size_t k = 0; k < m; k++) {
                    cx[k] = b->alist[k].corner.x;
                    cy[k] = b->alist[k].corner.y;
                    slip[k] = b->alist[k].slip;
                }
                vvgpu_body_params p = body_params(*S_, *b);
                check(ctx_, vvgpu_add_body(ctx_, (int64_t)m, cx.data(), cy.data(), slip.data(), &p), "vvgpu_add_body");
            }
            corners_ = corners;
            sizes_ = sizes;
        } else {
            int bi = 0;
            for (auto& b : S_->BodyList) {
                vvgpu_body_params p = body_params(*S_, *b);
                check(ctx_, vvgpu_set_body_params(ctx_, bi++, &p), "vvgpu_set_body_params");
            }
        }
        std::vector<double> g, fric, gsum;
        for_segments([&](const typename std::decay<decltype(S_->BodyList[0]->alist[0])>::type& a) {
            g.push_back(a.g); fric.push_back(a.fric); gsum.push_back(a.gsum);
        });
        if (!g.empty())
            check(ctx_, vvgpu_set_segment_state(ctx_, g.data(), fric.data(), gsum.data()), "vvgpu_set_segment_state");
    }

    void upload_vortices(bool includeV) {
        auto& V = S_->VortexList;
        const size_t n = includeV ? V.size() : 0;
        std::vector<double> x(n), y(n), g(n), ie(n), vx(n), vy(n);
        for (size_t k = 0; k < n; k++) {
            x[k] = V[k].r.x; y[k] = V[k].r.y; g[k] = V[k].g; ie[k] = V[k]._1_eps;
            vx[k] = V[k].v.x; vy[k] = V[k].v.y;
        }
        check(ctx_, vvgpu_set_vortices(ctx_, (int64_t)n, x.data(), y.data(), g.data(), ie.data()),
              "vvgpu_set_vortices");
        check(ctx_, vvgpu_set_velocities(ctx_, vx.data(), vy.data()), "vvgpu_set_velocities");
    }

    void apply_permutation() {
        auto& V = S_->VortexList;
        const size_t n = vvgpu_num_vortices(ctx_);
        if (n == 0 || n != V.size()) return;
        std::vector<int64_t> orig(n);
        check(ctx_, vvgpu_get_vortices(ctx_, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, orig.data()),
              "vvgpu_get_vortices");
        std::vector<TObj> old(V.begin(), V.end());
        for (size_t k = 0; k < n; k++) V[k] = old[orig[k]];
    }

    // Host mirror of the tree for getBottomNodes()/findNode() (built on first use).
    void ensure_mirror() const {
        if (!mirror_.empty() || !built_) return;
        int64_t nn = 0, nl = 0, nnear = 0, nfar = 0;
        check(ctx_, vvgpu_tree_sizes(ctx_, &nn, &nl, &nnear, &nfar), "vvgpu_tree_sizes");
        std::vector<double> x(nn), y(nn), h(nn), w(nn), px(nn), py(nn), pg(nn), mx(nn), my(nn), mg(nn);
        std::vector<int64_t> vf(nn), vl(nn), path(nn);
        std::vector<int32_t> depth(nn);
        check(ctx_, vvgpu_tree_nodes(ctx_, x.data(), y.data(), h.data(), w.data(), vf.data(), vl.data(), depth.data(),
                                     path.data(), px.data(), py.data(), pg.data(), mx.data(), my.data(), mg.data()),
              "vvgpu_tree_nodes");
        mirror_.resize(nn);
        std::map<std::pair<int, long long>, node_t*> by_id;
        TObj* base = S_->VortexList.empty() ? nullptr : &S_->VortexList[0];
        for (int64_t k = 0; k < nn; k++) {
            node_t& n = mirror_[k];
            n.x = x[k]; n.y = y[k]; n.h = h[k]; n.w = w[k];
            n.i = depth[k]; n.j = path[k];
            n.CMp.r.x = px[k]; n.CMp.r.y = py[k]; n.CMp.g = pg[k];
            n.CMm.r.x = mx[k]; n.CMm.r.y = my[k]; n.CMm.g = mg[k];
            if (base) { n.vRange.first = base + vf[k]; n.vRange.last = base + vl[k]; }
            by_id[{n.i, n.j}] = &n;
        }
        root_ = by_id.count({0, 0}) ? by_id[{0, 0}] : nullptr;
        for (auto& n : mirror_) {
            auto a = by_id.find({n.i + 1, n.j * 2}), b = by_id.find({n.i + 1, n.j * 2 + 1});
            if (a != by_id.end() && b != by_id.end()) { n.ch1 = a->second; n.ch2 = b->second; }
        }
        std::vector<double> lx(nl), ly(nl), lh(nl), lw(nl);
        std::vector<int64_t> lvf(nl), lvl(nl), lpath(nl), lsf(nl), lsl(nl);
        std::vector<int32_t> ldepth(nl);
        check(ctx_, vvgpu_tree_leaves(ctx_, lx.data(), ly.data(), lh.data(), lw.data(), lvf.data(), lvl.data(),
                                      ldepth.data(), lpath.data(), lsf.data(), lsl.data()),
              "vvgpu_tree_leaves");
        std::vector<int64_t> nearo(nl + 1), faro(nl + 1), nearp(nnear), farp(nfar);
        std::vector<int32_t> neard(nnear), fard(nfar);
        check(ctx_, vvgpu_tree_lists(ctx_, nearo.data(), neard.data(), nearp.data(), faro.data(), fard.data(),
                                     farp.data()),
              "vvgpu_tree_lists");
        std::vector<int64_t> seg_order(vvgpu_num_segments(ctx_));
        if (!seg_order.empty()) check(ctx_, vvgpu_tree_seg_order(ctx_, seg_order.data()), "vvgpu_tree_seg_order");
        std::vector<obj_t<SpaceT>*> segs;
        for (auto& b : S_->BodyList)
            for (auto& a : b->alist) segs.push_back(static_cast<obj_t<SpaceT>*>(&a));
        lists_.assign(2 * nl, {});
        bottom_.clear();
        for (int64_t L = 0; L < nl; L++) {
            node_t* n = by_id[{ldepth[L], lpath[L]}];
            bottom_.push_back(n);
            for (int64_t q = lsf[L]; q < lsl[L]; q++) n->bllist.push_back(segs[seg_order[q]]);
            auto& nr = lists_[2 * L];
            auto& fr = lists_[2 * L + 1];
            for (int64_t k = nearo[L]; k < nearo[L + 1]; k++) nr.push_back(by_id[{neard[k], nearp[k]}]);
            for (int64_t k = faro[L]; k < faro[L + 1]; k++) fr.push_back(by_id[{fard[k], farp[k]}]);
            n->NearNodes = &nr;
            n->FarNodes = &fr;
        }
    }

    SpaceT* S_;
    double fc_, min_, max_;
    vvgpu_ctx* ctx_ = nullptr;
    bool built_ = false;
    std::vector<double> corners_;
    std::vector<size_t> sizes_;
    mutable std::vector<node_t> mirror_;
    mutable std::vector<node_t*> bottom_;
    mutable std::vector<std::vector<node_t*>> lists_;
    mutable node_t* root_ = nullptr;
};

// MEpsilonFast (MEpsilonFast.hpp:5-31).
template <class SpaceT>
class MEpsilonFast {
   public:
    MEpsilonFast(SpaceT* S, const stree<SpaceT>* tree) : S_(S), tree_(tree) {}
    void CalcEpsilonFast(bool merge) {
        int64_t m = 0;
        check(tree_->gpu(), vvgpu_eps(tree_->gpu(), merge ? 1 : 0, &m), "vvgpu_eps");
        merged_ = (int)m;
        tree_->download_vortices(stree<SpaceT>::F_R | stree<SpaceT>::F_G | stree<SpaceT>::F_EPS);
    }
    int Merged() { return merged_; }

   private:
    SpaceT* S_;
    const stree<SpaceT>* tree_;
    int merged_ = 0;
};

// MConvectiveFast (MConvectiveFast.hpp:8-75).
template <class SpaceT>
class MConvectiveFast {
   public:
    using TVec = vec_t<SpaceT>;
    MConvectiveFast(SpaceT* S, const stree<SpaceT>* tree) : S_(S), tree_(tree) {}
    MConvectiveFast() = delete;
    MConvectiveFast(const MConvectiveFast&) = delete;
    MConvectiveFast& operator=(const MConvectiveFast&) = delete;

    void process_all_lists() {
        tree_->upload_velocities();
        check(tree_->gpu(), vvgpu_convective(tree_->gpu()), "vvgpu_convective");
        tree_->download_vortices(stree<SpaceT>::F_V);
    }

    TVec velocity(TVec p) const {
        double px = p.x, py = p.y, vx = 0, vy = 0;
        check(tree_->gpu(), vvgpu_velocity_points(tree_->gpu(), 1, &px, &py, &vx, &vy), "vvgpu_velocity_points");
        TVec r = p;
        r.x = vx;
        r.y = vy;
        return r;
    }

    void calc_circulation(const void** collision) {
        if (collision == nullptr)
            throw std::invalid_argument("MConvectiveFast::calc_circulation(): invalid collision pointer");
        if (*collision != nullptr) throw error(VVGPU_ERR_UNSUPPORTED, "collisions are not supported");
        vvgpu_ctx* c = tree_->gpu();
        int bi = 0;
        for (auto& b : S_->BodyList) {
            vvgpu_body_params p = stree<SpaceT>::body_params(*S_, *b);
            check(c, vvgpu_set_body_params(c, bi++, &p), "vvgpu_set_body_params");
        }
        std::vector<vvgpu_body_out> out(S_->BodyList.size());
        check(c, vvgpu_slae(c, out.data()), "vvgpu_slae");
        std::vector<double> g(vvgpu_num_segments(c));
        if (!g.empty())
            check(c, vvgpu_get_segments(c, nullptr, nullptr, nullptr, nullptr, nullptr, g.data(), nullptr, nullptr),
                  "vvgpu_get_segments");
        size_t k = 0;
        bi = 0;
        for (auto& b : S_->BodyList) {
            for (auto& a : b->alist) a.g = g[k++];
            const vvgpu_body_out& o = out[bi++];
            b->speed_slae.r.x = o.speed_slae_x; b->speed_slae.r.y = o.speed_slae_y; b->speed_slae.o = o.speed_slae_o;
            b->force_hydro.r.x = o.force_hydro_x; b->force_hydro.r.y = o.force_hydro_y; b->force_hydro.o = o.force_hydro_o;
            b->force_holder.r.x = o.force_holder_x; b->force_holder.r.y = o.force_holder_y;
            b->force_holder.o = o.force_holder_o;
        }
    }

   private:
    SpaceT* S_;
    const stree<SpaceT>* tree_;
};

// MDiffusiveFast (MDiffusiveFast.hpp:5-18).
template <class SpaceT>
class MDiffusiveFast {
   public:
    MDiffusiveFast(SpaceT* S, const stree<SpaceT>* tree) : S_(S), tree_(tree) {}
    void process_vort_list() {
        vvgpu_ctx* c = tree_->gpu();
        std::vector<double> fric;
        tree_->for_segments([&](const typename std::decay<decltype(S_->BodyList[0]->alist[0])>::type& a) {
            fric.push_back(a.fric);
        });
        if (!fric.empty())
            check(c, vvgpu_set_segment_state(c, nullptr, fric.data(), nullptr), "vvgpu_set_segment_state");
        tree_->upload_velocities();
        check(c, vvgpu_diffusive(c), "vvgpu_diffusive");
        tree_->download_vortices(stree<SpaceT>::F_V);
        if (!fric.empty()) {
            check(c, vvgpu_get_segments(c, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, fric.data(), nullptr),
                  "vvgpu_get_segments");
            size_t k = 0;
            for (auto& b : S_->BodyList)
                for (auto& a : b->alist) a.fric = fric[k++];
        }
    }
    void process_heat_list() {
        if (!S_->HeatList.empty()) throw error(VVGPU_ERR_UNSUPPORTED, "heat particles are not supported");
    }

   private:
    SpaceT* S_;
    const stree<SpaceT>* tree_;
};

}  // namespace vvgpu_cxx
