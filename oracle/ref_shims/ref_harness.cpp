// C entry points over the reference's own hot-path classes (stree, MEpsilonFast,
// MConvectiveFast, MDiffusiveFast, MFlowmove), compiled unmodified from the reference
// sources by oracle/Makefile into oracle/_ref/libvvref.so.  TEST INFRASTRUCTURE ONLY.
//
// The entry points mirror oracle/vvd_oracle.h with the prefix vvr_ instead of vvo_, so
// the same Python wrapper drives the reference and the C restatement. The harness
// reads tree internals for export, so it opens the classes' private sections for this
// translation unit only (the class layout is unchanged).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#define private public
#include "MConvectiveFast.hpp"
#include "MDiffusiveFast.hpp"
#include "MEpsilonFast.hpp"
#include "MFlowmove.hpp"
#include "TSortedTree.hpp"
#include "TSpace.hpp"
#define protected public
#include "XStreamfunction.hpp"
#include "XVelocity.hpp"
#include "XVorticity.hpp"
#undef protected
#undef private

#include "../vvd_oracle.h"

extern std::vector<double> vvr_last_matrix, vvr_last_rhs, vvr_last_solution;

namespace {

struct Handle {
    Space S;
    TSortedTree* tree = nullptr;
    MConvectiveFast* conv = nullptr;
    MEpsilonFast* eps = nullptr;
    MDiffusiveFast* diff = nullptr;
    int fc = -1;
    double minn = 0, maxn = 0;
    bool built = false;
    std::vector<int64_t> orig;  // original index of each VortexList slot

    ~Handle() { drop_modules(); }
    void drop_modules() {
        if (tree) tree->destroy();
        delete conv; delete eps; delete diff; delete tree;
        conv = nullptr; eps = nullptr; diff = nullptr; tree = nullptr;
        built = false;
    }
};

std::string num(double v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

TTime ttime_of(double v, int* ok) {
    TTime t = TTime::makeWithSecondsDecimal(v);
    *ok = (double(t) == v);
    return t;
}

void collect(const snode* nd, std::vector<const snode*>& out) {
    out.push_back(nd);
    if (nd->ch1) { collect(nd->ch1, out); collect(nd->ch2, out); }
}

}  // namespace

extern "C" {

void* vvr_create(void) { return new Handle(); }
void vvr_destroy(void* h) { delete (Handle*)h; }

int vvr_set_params(void* h, double re, double dt, double inf_vx, double inf_vy, double inf_g,
                   double time, double gravity_x, double gravity_y) {
    Handle* H = (Handle*)h;
    int ok1, ok2;
    H->S.re = re;
    H->S.dt = ttime_of(dt, &ok1);
    H->S.time = ttime_of(time, &ok2);
    if (!ok1 || !ok2) return -1;
    H->S.inf_vx = num(inf_vx);
    H->S.inf_vy = num(inf_vy);
    H->S.inf_g = inf_g;
    H->S.gravity = TVec(gravity_x, gravity_y);
    return 0;
}

int vvr_add_body(void* h, int64_t nseg, const double* cx, const double* cy, const uint32_t* slip,
                 const vvo_body_params* bp) {
    Handle* H = (Handle*)h;
    auto b = std::make_shared<TBody>();
    for (int64_t k = 0; k < nseg; k++) b->alist.emplace_back(cx[k], cy[k], slip ? slip[k] != 0 : false);
    if (bp) {
        b->holder = TVec3D(bp->holder_x, bp->holder_y, bp->holder_o);
        b->dpos = TVec3D(bp->dpos_x, bp->dpos_y, bp->dpos_o);
        b->speed_x = num(bp->speed_x);
        b->speed_y = num(bp->speed_y);
        b->speed_o = num(bp->speed_o);
        b->speed_slae = TVec3D(bp->speed_slae_x, bp->speed_slae_y, bp->speed_slae_o);
        b->speed_slae_prev = TVec3D(bp->speed_slae_prev_x, bp->speed_slae_prev_y, bp->speed_slae_prev_o);
        b->friction_prev = TVec3D(bp->friction_prev_x, bp->friction_prev_y, bp->friction_prev_o);
        b->fdt_dead = TVec3D(bp->fdt_dead_x, bp->fdt_dead_y, bp->fdt_dead_o);
        b->g_dead = bp->g_dead;
        b->density = bp->density;
        b->kspring = TVec3D(bp->kspring_x, bp->kspring_y, bp->kspring_o);
        b->special_segment_no = bp->special_segment_no;
        b->boundary_condition = bp->bc_kutta ? bc_t::kutta : bc_t::steady;
    }
    b->doUpdateSegments();
    b->doFillProperties();
    H->S.BodyList.push_back(b);
    return 0;
}

int vvr_set_segment_g(void* h, const double* g) {
    Handle* H = (Handle*)h;
    int64_t k = 0;
    for (auto& b : H->S.BodyList)
        for (auto& a : b->alist) a.g = g[k++];
    return 0;
}

int vvr_set_sinks(void* h, int64_t n, const double* x, const double* y, const double* g) {
    Handle* H = (Handle*)h;
    H->S.SourceList.clear();
    for (int64_t i = 0; i < n; i++) H->S.SourceList.emplace_back(x[i], y[i], g[i]);
    return 0;
}

int vvr_set_vortices(void* h, int64_t n, const double* x, const double* y, const double* g,
                     const double* ie) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    H->S.VortexList.clear();
    H->orig.resize(n);
    for (int64_t i = 0; i < n; i++) {
        TObj o(x[i], y[i], g[i]);
        o._1_eps = ie ? ie[i] : 0.;
        H->S.VortexList.push_back(o);
        H->orig[i] = i;
    }
    return 0;
}

int64_t vvr_num_vortices(void* h) { return (int64_t)((Handle*)h)->S.VortexList.size(); }
int64_t vvr_num_segments(void* h) { return (int64_t)((Handle*)h)->S.total_segment_count(); }

int vvr_get_vortices(void* h, double* x, double* y, double* g, double* ie, double* vx, double* vy,
                     int64_t* orig) {
    Handle* H = (Handle*)h;
    size_t n = H->S.VortexList.size();
    for (size_t i = 0; i < n; i++) {
        const TObj& o = H->S.VortexList[i];
        if (x) x[i] = o.r.x;
        if (y) y[i] = o.r.y;
        if (g) g[i] = o.g;
        if (ie) ie[i] = o._1_eps;
        if (vx) vx[i] = o.v.x;
        if (vy) vy[i] = o.v.y;
        if (orig) orig[i] = H->orig[i];
    }
    return 0;
}

int vvr_get_segments(void* h, double* rx, double* ry, double* dlx, double* dly, double* ie,
                     double* g, double* fric, double* gsum) {
    Handle* H = (Handle*)h;
    int64_t k = 0;
    for (auto& b : H->S.BodyList)
        for (auto& a : b->alist) {
            if (rx) rx[k] = a.r.x;
            if (ry) ry[k] = a.r.y;
            if (dlx) dlx[k] = a.dl.x;
            if (dly) dly[k] = a.dl.y;
            if (ie) ie[k] = a._1_eps;
            if (g) g[k] = a.g;
            if (fric) fric[k] = a.fric;
            if (gsum) gsum[k] = a.gsum;
            k++;
        }
    return 0;
}

int vvr_get_body_geom(void* h, int bi, double* area, double* cofm_x, double* cofm_y,
                      double* moi_axis, double* slen) {
    Handle* H = (Handle*)h;
    if (bi < 0 || bi >= (int)H->S.BodyList.size()) return -1;
    const TBody& b = *H->S.BodyList[bi];
    if (area) *area = b.get_area();
    if (cofm_x) *cofm_x = b.get_cofm().x;
    if (cofm_y) *cofm_y = b.get_cofm().y;
    if (moi_axis) *moi_axis = b.get_moi_axis();
    if (slen) *slen = b.get_slen();
    return 0;
}

int vvr_tree_build(void* h, double far_criteria, double min_node, double max_node) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    int fc = (int)far_criteria;
    if ((double)fc != far_criteria) return -1;  // the reference takes an int
    if (!H->tree || fc != H->fc || min_node != H->minn || max_node != H->maxn) {
        H->drop_modules();
        H->tree = new TSortedTree(&H->S, fc, min_node, max_node);
        H->conv = new MConvectiveFast(&H->S, H->tree);
        H->eps = new MEpsilonFast(&H->S, H->tree);
        H->diff = new MDiffusiveFast(&H->S, H->tree);
        H->fc = fc; H->minn = min_node; H->maxn = max_node;
    }
    // carry the original index through the in-place permutation inside TObj::v
    auto& V = H->S.VortexList;
    std::vector<TVec> saved(V.size());
    for (size_t i = 0; i < V.size(); i++) {
        saved[H->orig[i]] = V[i].v;
        V[i].v = TVec((double)H->orig[i], 0.);
    }
    H->tree->build();
    for (size_t i = 0; i < V.size(); i++) {
        int64_t o = (int64_t)V[i].v.x;
        H->orig[i] = o;
        V[i].v = saved[o];
    }
    H->built = true;
    return 0;
}

int vvr_tree_destroy(void* h) {
    Handle* H = (Handle*)h;
    if (H->tree) H->tree->destroy();
    H->built = false;
    return 0;
}

int vvr_tree_sizes(void* h, int64_t* nnodes, int64_t* nleaves, int64_t* nnear, int64_t* nfar) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    std::vector<const snode*> all;
    collect(H->tree->rootNode, all);
    const auto& bn = H->tree->getBottomNodes();
    int64_t a = 0, b = 0;
    for (auto* L : bn) { a += L->NearNodes->size(); b += L->FarNodes->size(); }
    if (nnodes) *nnodes = (int64_t)all.size();
    if (nleaves) *nleaves = (int64_t)bn.size();
    if (nnear) *nnear = a;
    if (nfar) *nfar = b;
    return 0;
}

static int64_t seg_index(Handle* H, const TObj* p) {
    int64_t base = 0;
    for (auto& b : H->S.BodyList) {
        if (!b->alist.empty() && p >= &b->alist.front() && p <= &b->alist.back())
            return base + (int64_t)((const TAtt*)p - &b->alist.front());
        base += (int64_t)b->alist.size();
    }
    return -1;
}

int vvr_tree_leaves(void* h, double* x, double* y, double* hh, double* w, int64_t* vfirst,
                    int64_t* vlast, int32_t* depth, int64_t* path, int64_t* sfirst, int64_t* slast) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    const TObj* base = H->S.VortexList.empty() ? nullptr : &H->S.VortexList.front();
    const auto& bn = H->tree->getBottomNodes();
    int64_t s = 0;
    for (size_t L = 0; L < bn.size(); L++) {
        const snode* nd = bn[L];
        if (x) x[L] = nd->x;
        if (y) y[L] = nd->y;
        if (hh) hh[L] = nd->h;
        if (w) w[L] = nd->w;
        int64_t f = nd->vRange.first ? (int64_t)(nd->vRange.first - base) : 0;
        int64_t l = nd->vRange.first ? (int64_t)(nd->vRange.last - base) : 0;
        if (vfirst) vfirst[L] = f;
        if (vlast) vlast[L] = l;
        if (depth) depth[L] = nd->i;
        if (path) path[L] = nd->j;
        if (sfirst) sfirst[L] = s;
        s += (int64_t)nd->bllist.size();
        if (slast) slast[L] = s;
    }
    return 0;
}

int vvr_tree_nodes(void* h, double* x, double* y, double* hh, double* w, int64_t* vfirst,
                   int64_t* vlast, int32_t* depth, int64_t* path, double* cmp_x, double* cmp_y,
                   double* cmp_g, double* cmm_x, double* cmm_y, double* cmm_g) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    const TObj* base = H->S.VortexList.empty() ? nullptr : &H->S.VortexList.front();
    std::vector<const snode*> all;
    collect(H->tree->rootNode, all);
    for (size_t k = 0; k < all.size(); k++) {
        const snode* nd = all[k];
        if (x) x[k] = nd->x;
        if (y) y[k] = nd->y;
        if (hh) hh[k] = nd->h;
        if (w) w[k] = nd->w;
        if (vfirst) vfirst[k] = nd->vRange.first ? (int64_t)(nd->vRange.first - base) : 0;
        if (vlast) vlast[k] = nd->vRange.first ? (int64_t)(nd->vRange.last - base) : 0;
        if (depth) depth[k] = nd->i;
        if (path) path[k] = nd->j;
        if (cmp_x) cmp_x[k] = nd->CMp.r.x;
        if (cmp_y) cmp_y[k] = nd->CMp.r.y;
        if (cmp_g) cmp_g[k] = nd->CMp.g;
        if (cmm_x) cmm_x[k] = nd->CMm.r.x;
        if (cmm_y) cmm_y[k] = nd->CMm.r.y;
        if (cmm_g) cmm_g[k] = nd->CMm.g;
    }
    return 0;
}

int vvr_tree_seg_order(void* h, int64_t* seg_order) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    int64_t k = 0;
    for (auto* L : H->tree->getBottomNodes())
        for (TObj* p : L->bllist) seg_order[k++] = seg_index(H, p);
    return 0;
}

int vvr_tree_lists(void* h, int64_t* near_off, int32_t* near_depth, int64_t* near_path,
                   int64_t* far_off, int32_t* far_depth, int64_t* far_path) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    const auto& bn = H->tree->getBottomNodes();
    int64_t a = 0, b = 0;
    for (size_t L = 0; L < bn.size(); L++) {
        if (near_off) near_off[L] = a;
        if (far_off) far_off[L] = b;
        for (auto* n : *bn[L]->NearNodes) {
            if (near_depth) near_depth[a] = n->i;
            if (near_path) near_path[a] = n->j;
            a++;
        }
        for (auto* n : *bn[L]->FarNodes) {
            if (far_depth) far_depth[b] = n->i;
            if (far_path) far_path[b] = n->j;
            b++;
        }
    }
    if (near_off) near_off[bn.size()] = a;
    if (far_off) far_off[bn.size()] = b;
    return 0;
}

int vvr_eps(void* h, int merge, int64_t* merged) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    H->eps->CalcEpsilonFast(merge != 0);
    if (merged) *merged = H->eps->Merged();
    return 0;
}

int vvr_convective(void* h) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    H->conv->process_all_lists();
    return 0;
}

int vvr_diffusive(void* h) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    H->diff->process_vort_list();
    return 0;
}

int vvr_velocity_points(void* h, int64_t n, const double* px, const double* py, double* vx,
                        double* vy) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    for (int64_t i = 0; i < n; i++) {
        TVec v = H->conv->velocity(TVec(px[i], py[i]));
        vx[i] = v.x;
        vy[i] = v.y;
    }
    return 0;
}

int vvr_slae(void* h, vvo_body_out* out) {
    Handle* H = (Handle*)h;
    if (!H->built) return -3;
    const void* collision = nullptr;
    H->conv->calc_circulation(&collision);
    size_t bi = 0;
    for (auto& b : H->S.BodyList) {
        if (out) {
            vvo_body_out& o = out[bi];
            o.speed_slae_x = b->speed_slae.r.x; o.speed_slae_y = b->speed_slae.r.y; o.speed_slae_o = b->speed_slae.o;
            o.force_hydro_x = b->force_hydro.r.x; o.force_hydro_y = b->force_hydro.r.y; o.force_hydro_o = b->force_hydro.o;
            o.force_holder_x = b->force_holder.r.x; o.force_holder_y = b->force_holder.r.y; o.force_holder_o = b->force_holder.o;
        }
        bi++;
    }
    return 0;
}

int64_t vvr_slae_size(void* h) {
    Handle* H = (Handle*)h;
    return (int64_t)(H->S.total_segment_count() + H->S.BodyList.size() * 9);
}

int vvr_slae_export(void* h, double* matrix, double* rhs, double* solution) {
    (void)h;
    if (vvr_last_rhs.empty()) return -3;
    if (matrix) memcpy(matrix, vvr_last_matrix.data(), vvr_last_matrix.size() * sizeof(double));
    if (rhs) memcpy(rhs, vvr_last_rhs.data(), vvr_last_rhs.size() * sizeof(double));
    if (solution) memcpy(solution, vvr_last_solution.data(), vvr_last_solution.size() * sizeof(double));
    return 0;
}

int vvr_vortex_shed(void* h) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    size_t before = H->S.VortexList.size();
    MFlowmove fm(&H->S);
    fm.vortex_shed();
    for (size_t i = before; i < H->S.VortexList.size(); i++) H->orig.push_back((int64_t)i);
    return 0;
}

double vvr_gsum(void* h) { return ((Handle*)h)->S.gsum(); }

int vvr_set_velocities(void* h, const double* vx, const double* vy) {
    Handle* H = (Handle*)h;
    size_t i = 0;
    for (auto& o : H->S.VortexList) { o.v = TVec(vx[i], vy[i]); i++; }
    return 0;
}

// MFlowmove::move_and_clean.  The original index of each surviving vortex is carried
// through the call in TObj::_1_eps (which move_and_clean does not read) and restored after.
int vvr_move_and_clean(void* h, int remove, int64_t* cleaned) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    std::vector<double> ie;
    size_t k = 0;
    for (auto& o : H->S.VortexList) { ie.push_back(o._1_eps); o._1_eps = (double)k++; }
    MFlowmove fm(&H->S);
    const void* collision = nullptr;
    size_t nc = 0;
    fm.move_and_clean(remove != 0, &collision, &nc);
    std::vector<int64_t> orig;
    for (auto& o : H->S.VortexList) {
        const size_t slot = (size_t)o._1_eps;
        orig.push_back(H->orig[slot]);
        o._1_eps = ie[slot];
    }
    H->orig = orig;
    if (cleaned) *cleaned = (int64_t)nc;
    return collision ? -5 : 0;
}

int vvr_set_segment_state(void* h, const double* g, const double* fric, const double* gsum) {
    Handle* H = (Handle*)h;
    int64_t k = 0;
    for (auto& b : H->S.BodyList)
        for (auto& a : b->alist) {
            if (g) a.g = g[k];
            if (fric) a.fric = fric[k];
            if (gsum) a.gsum = gsum[k];
            k++;
        }
    return 0;
}

int vvr_calc_forces(void* h, double* out4) {
    Handle* H = (Handle*)h;
    H->S.calc_forces();
    int bi = 0;
    for (auto& b : H->S.BodyList) {
        if (out4) {
            out4[4 * bi + 0] = b->friction.r.x; out4[4 * bi + 1] = b->friction.r.y;
            out4[4 * bi + 2] = b->friction.o; out4[4 * bi + 3] = b->nusselt;
        }
        bi++;
    }
    return 0;
}

int vvr_zero_forces(void* h) {
    ((Handle*)h)->S.zero_forces();
    return 0;
}

int vvr_get_segment_forces(void* h, double* cp, double* fr, double* nu) {
    Handle* H = (Handle*)h;
    int64_t k = 0;
    for (auto& b : H->S.BodyList)
        for (auto& a : b->alist) {
            if (cp) cp[k] = a.Cp;
            if (fr) fr[k] = a.Fr;
            if (nu) nu[k] = a.Nu;
            k++;
        }
    return 0;
}

int vvr_get_body_params(void* h, int bi, vvo_body_params* out) {
    Handle* H = (Handle*)h;
    if (bi < 0 || bi >= (int)H->S.BodyList.size() || !out) return -1;
    const TBody& b = *H->S.BodyList[bi];
    memset(out, 0, sizeof *out);
    out->holder_x = b.holder.r.x; out->holder_y = b.holder.r.y; out->holder_o = b.holder.o;
    out->dpos_x = b.dpos.r.x; out->dpos_y = b.dpos.r.y; out->dpos_o = b.dpos.o;
    out->speed_slae_x = b.speed_slae.r.x; out->speed_slae_y = b.speed_slae.r.y; out->speed_slae_o = b.speed_slae.o;
    out->speed_slae_prev_x = b.speed_slae_prev.r.x; out->speed_slae_prev_y = b.speed_slae_prev.r.y;
    out->speed_slae_prev_o = b.speed_slae_prev.o;
    out->friction_prev_x = b.friction_prev.r.x; out->friction_prev_y = b.friction_prev.r.y;
    out->friction_prev_o = b.friction_prev.o;
    out->fdt_dead_x = b.fdt_dead.r.x; out->fdt_dead_y = b.fdt_dead.r.y; out->fdt_dead_o = b.fdt_dead.o;
    out->g_dead = b.g_dead;
    out->density = b.density;
    out->kspring_x = b.kspring.r.x; out->kspring_y = b.kspring.r.y; out->kspring_o = b.kspring.o;
    out->special_segment_no = b.special_segment_no;
    out->bc_kutta = b.boundary_condition == bc_t::kutta;
    return 0;
}

// Grid fields: the reference's XVelocity / XStreamfunction / XVorticity constructed on the
// handle's Space (each copies it), evaluated, and XField::map copied out.
static int field_out(XField& f, int32_t xres, int32_t yres, float* out) {
    for (int32_t yj = 0; yj < yres; yj++)
        for (int32_t xi = 0; xi < xres; xi++) out[(int64_t)yj * xres + xi] = f.at(xi, yj);
    return 0;
}

int vvr_field_velocity(void* h, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres, char mode,
                       char ref_frame, float* out) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    try {
        XVelocity f(H->S, xmin, ymin, dxdy, xres, yres);
        f.mode = mode;
        f.ref_frame = ref_frame;
        f.evaluate();
        return field_out(f, xres, yres, out);
    } catch (std::invalid_argument&) {
        return -1;
    }
}

int vvr_field_streamfunction(void* h, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                             double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                             uint16_t* gap_yj, float* gap, int64_t* ngaps) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    try {
        XStreamfunction f(H->S, xmin, ymin, dxdy, xres, yres);
        f.eps_mult = eps_mult;
        f.ref_frame = ref_frame;
        f.evaluate();
        // gaps come in thread order: sort into grid order
        std::vector<TGap> gs(f.gaps.begin(), f.gaps.end());
        std::sort(gs.begin(), gs.end(), [](const TGap& a, const TGap& b) {
            return a.yj != b.yj ? a.yj < b.yj : a.xi < b.xi;
        });
        int64_t k = 0;
        for (const TGap& gp : gs) {
            if (k < gap_cap) { gap_xi[k] = gp.xi; gap_yj[k] = gp.yj; gap[k] = gp.gap; }
            k++;
        }
        if (ngaps) *ngaps = k;
        return field_out(f, xres, yres, out);
    } catch (std::invalid_argument&) {
        return -1;
    }
}

int vvr_field_vorticity(void* h, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                        double eps_mult, float* out) {
    Handle* H = (Handle*)h;
    if (H->built) return -2;
    try {
        XVorticity f(H->S, xmin, ymin, dxdy, xres, yres);
        f.eps_mult = eps_mult;
        f.evaluate();
        return field_out(f, xres, yres, out);
    } catch (std::invalid_argument&) {
        return -1;
    }
}

}  // extern "C"
