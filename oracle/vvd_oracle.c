/*
 * vvd_oracle.c -- sequential FP64 restatement of libvvhd's per-step velocity path.
 *
 * TEST INFRASTRUCTURE ONLY (see vvd_oracle.h).  Every function names the reference
 * file:line it restates.  Compile with -ffp-contract=off: the reference is built for
 * x86-64 without FMA, so a fused multiply-add here would change the last bit of tree
 * decisions on hosts (aarch64) whose compilers contract by default.
 */
#include "vvd_oracle.h"

#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#define C_PI    3.14159265358979323846
#define C_2PI   (2. * C_PI)
#define C_1_2PI (1. / (2. * C_PI))
#define C_1_4PI (1. / (4. * C_PI))
#define C_1_PI  (1. / C_PI)

/* Tree_MaxListSize, libvvhd/src/TSortedTree.cpp:10 */
#define TREE_MAX_LIST_SIZE 16
/* ExpArgRestriction, libvvhd/src/MDiffusiveFast.cpp:6 */
#define EXP_ARG_RESTRICTION (-8.)
/* MFlowmove remove_eps default, libvvhd/headers/MFlowmove.hpp:8 */
#define REMOVE_EPS 1e-10

/* std::max / std::min exactly as libstdc++ defines them (order matters for NaN, -0). */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double sgn(double x) { return (x > 0) ? 1 : ((x < 0) ? -1 : 0); }
static inline double sqr(double x) { return x * x; }
static inline double abs2(double x, double y) { return x * x + y * y; }

typedef struct {
    double x, y, h, w;
    int64_t vf, vl;  /* vortex slots [vf, vl) */
    int64_t sf, sl;  /* seg_order slots [sf, sl) */
    int32_t ch1, ch2;
    int32_t depth;
    int64_t path;
    double cmp_x, cmp_y, cmp_g, cmm_x, cmm_y, cmm_g;
} onode;

typedef struct {
    int64_t first, count;
    vvo_body_params p;
    double slen, area, cofm_x, cofm_y, moi_cofm;
    double friction_x, friction_y, friction_o, nusselt;  /* TBody::friction, nusselt */
} obody;

struct vvo_space {
    double re, dt, inf_vx, inf_vy, inf_g, time, grav_x, grav_y;
    /* Space::VortexList as SoA */
    int64_t n, cap, n_set;
    double *x, *y, *g, *ie, *vx, *vy;
    int64_t* orig;
    /* all TAtt of all bodies, concatenated */
    int64_t m, mcap;
    double *cx, *cy, *rx, *ry, *dlx, *dly, *sie, *sg, *fric, *gsum;
    double *cp, *fr, *nu;  /* TAtt::Cp, Fr, Nu (Space::calc_forces accumulators) */
    uint32_t* slip;
    int nb, nbcap;
    obody* bodies;
    /* Space::SourceList */
    int64_t ns;
    double *snk_x, *snk_y, *snk_g;
    /* tree */
    int built;
    double far_criteria, min_node, max_node;
    onode* nodes;
    int64_t nnodes, nodecap;
    int32_t* leaves;
    int64_t nleaves, leafcap;
    int64_t* seg_order;
    int64_t* near_off; int32_t* near_list; int64_t nnear, nearcap;
    int64_t* far_off;  int32_t* far_list;  int64_t nfar, farcap;
    /* timing sample: phases over leaves process only leaves L with L % stride == 0 */
    int64_t stride;
    double t_partition, t_cmass, t_lists;
    /* SLAE */
    int64_t neq;
    double *mat, *rhs, *sol;
};

static void* xrealloc(void* p, size_t sz) {
    void* q = realloc(p, sz ? sz : 1);
    if (!q) abort();
    return q;
}

vvo_space* vvo_create(void) {
    vvo_space* S = (vvo_space*)calloc(1, sizeof(vvo_space));
    /* Space::Space, libvvhd/src/TSpace.cpp:14-36 */
    S->re = INFINITY;
    S->dt = 1.0;
    S->stride = 1;
    return S;
}

static void free_tree(vvo_space* S) {
    free(S->nodes); S->nodes = NULL; S->nnodes = S->nodecap = 0;
    free(S->leaves); S->leaves = NULL; S->nleaves = S->leafcap = 0;
    free(S->seg_order); S->seg_order = NULL;
    free(S->near_off); S->near_off = NULL; free(S->near_list); S->near_list = NULL;
    S->nnear = S->nearcap = 0;
    free(S->far_off); S->far_off = NULL; free(S->far_list); S->far_list = NULL;
    S->nfar = S->farcap = 0;
    S->built = 0;
}

void vvo_destroy(vvo_space* S) {
    if (!S) return;
    free_tree(S);
    free(S->x); free(S->y); free(S->g); free(S->ie); free(S->vx); free(S->vy); free(S->orig);
    free(S->cx); free(S->cy); free(S->rx); free(S->ry); free(S->dlx); free(S->dly);
    free(S->sie); free(S->sg); free(S->fric); free(S->gsum); free(S->slip);
    free(S->cp); free(S->fr); free(S->nu);
    free(S->bodies);
    free(S->snk_x); free(S->snk_y); free(S->snk_g);
    free(S->mat); free(S->rhs); free(S->sol);
    free(S);
}

int vvo_set_params(vvo_space* S, double re, double dt, double inf_vx, double inf_vy,
                   double inf_g, double time, double gravity_x, double gravity_y) {
    S->re = re; S->dt = dt; S->inf_vx = inf_vx; S->inf_vy = inf_vy; S->inf_g = inf_g;
    S->time = time; S->grav_x = gravity_x; S->grav_y = gravity_y;
    return 0;
}

/* TBody::doUpdateSegments (TBody.cpp:200-215) and doFillProperties (TBody.cpp:283-343). */
static void body_update(vvo_space* S, obody* b) {
    int64_t f = b->first, n = b->count;
    for (int64_t k = 0; k < n; k++) {
        int64_t i = f + k, j = f + (k + 1) % n;
        S->dlx[i] = S->cx[j] - S->cx[i];
        S->dly[i] = S->cy[j] - S->cy[i];
        S->sie[i] = 3.0 / sqrt(abs2(S->dlx[i], S->dly[i]));
        S->rx[i] = (S->cx[j] + S->cx[i]) * 0.5;
        S->ry[i] = (S->cy[j] + S->cy[i]) * 0.5;
    }
    b->slen = 0; b->area = 0;
    for (int64_t k = 0; k < n; k++) {
        int64_t i = f + k;
        b->slen += sqrt(abs2(S->dlx[i], S->dly[i]));
        b->area += S->ry[i] * S->dlx[i];
    }
    if (b->area == 0) {
        double lx = 0, ly = 0;
        for (int64_t k = 0; k < n; k++) {
            int64_t i = f + k;
            double l = sqrt(abs2(S->dlx[i], S->dly[i]));
            lx += S->rx[i] * l; ly += S->ry[i] * l;
        }
        double inv = 1. / b->slen;
        b->cofm_x = lx * inv; b->cofm_y = ly * inv;
        b->moi_cofm = 0.;
    } else {
        double sx = 0, sy = 0, m0 = 0;
        for (int64_t k = 0; k < n; k++) {
            int64_t i = f + k, j = f + (k + 1) % n;
            /* rotl(c_i) * c_{i+1} */
            double cr = (-S->cy[i]) * S->cx[j] + S->cx[i] * S->cy[j];
            sx -= S->rx[i] * cr; sy -= S->ry[i] * cr;
            m0 -= (abs2(S->cx[i], S->cy[i]) + (S->cx[i] * S->cx[j] + S->cy[i] * S->cy[j])
                   + abs2(S->cx[j], S->cy[j])) * cr;
        }
        double inv = 1. / (3 * b->area);
        b->cofm_x = sx * inv; b->cofm_y = sy * inv;
        b->moi_cofm = m0 / 12. - b->area * abs2(b->cofm_x, b->cofm_y);
    }
}

int vvo_add_body(vvo_space* S, int64_t nseg, const double* corner_x, const double* corner_y,
                 const uint32_t* slip, const vvo_body_params* bp) {
    if (nseg < 0) return -1;
    int64_t m = S->m + nseg;
    if (m > S->mcap) {
        S->mcap = m;
        size_t d = sizeof(double) * (size_t)m;
        S->cx = xrealloc(S->cx, d); S->cy = xrealloc(S->cy, d);
        S->rx = xrealloc(S->rx, d); S->ry = xrealloc(S->ry, d);
        S->dlx = xrealloc(S->dlx, d); S->dly = xrealloc(S->dly, d);
        S->sie = xrealloc(S->sie, d); S->sg = xrealloc(S->sg, d);
        S->fric = xrealloc(S->fric, d); S->gsum = xrealloc(S->gsum, d);
        S->cp = xrealloc(S->cp, d); S->fr = xrealloc(S->fr, d); S->nu = xrealloc(S->nu, d);
        S->slip = xrealloc(S->slip, sizeof(uint32_t) * (size_t)m);
    }
    for (int64_t k = 0; k < nseg; k++) {
        int64_t i = S->m + k;
        S->cx[i] = corner_x[k]; S->cy[i] = corner_y[k];
        S->sg[i] = 0; S->fric[i] = 0; S->gsum[i] = 0;
        S->cp[i] = 0; S->fr[i] = 0; S->nu[i] = 0;
        S->slip[i] = slip ? slip[k] : 0;
    }
    if (S->nb == S->nbcap) {
        S->nbcap = S->nbcap ? 2 * S->nbcap : 4;
        S->bodies = xrealloc(S->bodies, sizeof(obody) * (size_t)S->nbcap);
    }
    obody* b = &S->bodies[S->nb++];
    memset(b, 0, sizeof(*b));
    b->first = S->m; b->count = nseg;
    if (bp) b->p = *bp;
    else {
        b->p.density = 1.0;
        b->p.kspring_x = b->p.kspring_y = b->p.kspring_o = INFINITY;
    }
    S->m = m;
    body_update(S, b);
    return 0;
}

int vvo_set_segment_g(vvo_space* S, const double* g) {
    for (int64_t i = 0; i < S->m; i++) S->sg[i] = g[i];
    return 0;
}

int vvo_set_sinks(vvo_space* S, int64_t n, const double* x, const double* y, const double* g) {
    S->ns = n;
    S->snk_x = xrealloc(S->snk_x, sizeof(double) * (size_t)n);
    S->snk_y = xrealloc(S->snk_y, sizeof(double) * (size_t)n);
    S->snk_g = xrealloc(S->snk_g, sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; i++) { S->snk_x[i] = x[i]; S->snk_y[i] = y[i]; S->snk_g[i] = g[i]; }
    return 0;
}

static void vort_reserve(vvo_space* S, int64_t n) {
    if (n <= S->cap) return;
    S->cap = n;
    size_t d = sizeof(double) * (size_t)n;
    S->x = xrealloc(S->x, d); S->y = xrealloc(S->y, d); S->g = xrealloc(S->g, d);
    S->ie = xrealloc(S->ie, d); S->vx = xrealloc(S->vx, d); S->vy = xrealloc(S->vy, d);
    S->orig = xrealloc(S->orig, sizeof(int64_t) * (size_t)n);
}

int vvo_set_vortices(vvo_space* S, int64_t n, const double* x, const double* y,
                     const double* g, const double* inv_eps) {
    if (S->built) return -2;
    vort_reserve(S, n);
    S->n = n; S->n_set = n;
    for (int64_t i = 0; i < n; i++) {
        S->x[i] = x[i]; S->y[i] = y[i]; S->g[i] = g[i];
        S->ie[i] = inv_eps ? inv_eps[i] : 0.;
        S->vx[i] = 0; S->vy[i] = 0; S->orig[i] = i;
    }
    return 0;
}

int64_t vvo_num_vortices(const vvo_space* S) { return S->n; }
int64_t vvo_num_segments(const vvo_space* S) { return S->m; }

int vvo_get_vortices(const vvo_space* S, double* x, double* y, double* g, double* inv_eps,
                     double* vx, double* vy, int64_t* orig) {
    size_t d = sizeof(double) * (size_t)S->n;
    if (x) memcpy(x, S->x, d);
    if (y) memcpy(y, S->y, d);
    if (g) memcpy(g, S->g, d);
    if (inv_eps) memcpy(inv_eps, S->ie, d);
    if (vx) memcpy(vx, S->vx, d);
    if (vy) memcpy(vy, S->vy, d);
    if (orig) memcpy(orig, S->orig, sizeof(int64_t) * (size_t)S->n);
    return 0;
}

int vvo_get_segments(const vvo_space* S, double* rx, double* ry, double* dlx, double* dly,
                     double* inv_eps, double* g, double* fric, double* gsum) {
    size_t d = sizeof(double) * (size_t)S->m;
    if (rx) memcpy(rx, S->rx, d);
    if (ry) memcpy(ry, S->ry, d);
    if (dlx) memcpy(dlx, S->dlx, d);
    if (dly) memcpy(dly, S->dly, d);
    if (inv_eps) memcpy(inv_eps, S->sie, d);
    if (g) memcpy(g, S->sg, d);
    if (fric) memcpy(fric, S->fric, d);
    if (gsum) memcpy(gsum, S->gsum, d);
    return 0;
}

static double body_axis_x(const obody* b) { return b->p.holder_x + b->p.dpos_x; }
static double body_axis_y(const obody* b) { return b->p.holder_y + b->p.dpos_y; }
/* TBody::get_moi_axis, TBody.hpp:129-132 */
static double body_moi_axis(const obody* b) {
    double dx = body_axis_x(b) - b->cofm_x, dy = body_axis_y(b) - b->cofm_y;
    return b->moi_cofm + abs2(dx, dy) * b->area;
}

int vvo_get_body_geom(const vvo_space* S, int bi, double* area, double* cofm_x, double* cofm_y,
                      double* moi_axis, double* slen) {
    if (bi < 0 || bi >= S->nb) return -1;
    const obody* b = &S->bodies[bi];
    if (area) *area = b->area;
    if (cofm_x) *cofm_x = b->cofm_x;
    if (cofm_y) *cofm_y = b->cofm_y;
    if (moi_axis) *moi_axis = body_moi_axis(b);
    if (slen) *slen = b->slen;
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Tree (libvvhd/src/TSortedTree.cpp)                                                   */
/* ------------------------------------------------------------------------------------ */

static int32_t new_node(vvo_space* S) {
    if (S->nnodes == S->nodecap) {
        S->nodecap = S->nodecap ? 2 * S->nodecap : 1024;
        S->nodes = xrealloc(S->nodes, sizeof(onode) * (size_t)S->nodecap);
    }
    onode* nd = &S->nodes[S->nnodes];
    memset(nd, 0, sizeof(*nd));
    nd->ch1 = nd->ch2 = -1;
    /* snode::snode sets CMp._1_eps = CMm._1_eps = inf (TSortedTree.cpp:17); only used as
     * biot_savart's zero smoothing radius, which the far-field code below writes directly. */
    return (int32_t)S->nnodes++;
}

/* snode::Stretch (TSortedTree.cpp:101-137): bbox over bllist then vRange. */
static void stretch(vvo_space* S, onode* nd) {
    double trx = -DBL_MAX, try_ = -DBL_MAX, blx = DBL_MAX, bly = DBL_MAX;
    for (int64_t k = nd->sf; k < nd->sl; k++) {
        int64_t s = S->seg_order[k];
        trx = smax(trx, S->rx[s]); try_ = smax(try_, S->ry[s]);
        blx = smin(blx, S->rx[s]); bly = smin(bly, S->ry[s]);
    }
    for (int64_t i = nd->vf; i < nd->vl; i++) {
        trx = smax(trx, S->x[i]); try_ = smax(try_, S->y[i]);
        blx = smin(blx, S->x[i]); bly = smin(bly, S->y[i]);
    }
    nd->x = (blx + trx) * 0.5;
    nd->y = (bly + try_) * 0.5;
    nd->h = try_ - bly;
    nd->w = trx - blx;
}

static void swap_slots(vvo_space* S, int64_t a, int64_t b) {
    double t;
#define SW(arr) t = S->arr[a]; S->arr[a] = S->arr[b]; S->arr[b] = t;
    SW(x) SW(y) SW(g) SW(ie) SW(vx) SW(vy)
#undef SW
    int64_t o = S->orig[a]; S->orig[a] = S->orig[b]; S->orig[b] = o;
}

static int32_t find_node(const vvo_space* S, double px, double py);

/* snode::DivideNode (TSortedTree.cpp:36-79) with DistributeContent (:81-99, :139-148). */
static void divide(vvo_space* S, int32_t ni) {
    onode nd = S->nodes[ni];
    double mx = smax(nd.h, nd.w), mn = smin(nd.h, nd.w);
    if (mx < S->max_node && mn <= S->min_node) {
        S->leaves[S->nleaves++] = ni;
        return;
    }
    int64_t nv = nd.vl - nd.vf, nsg = nd.sl - nd.sf;
    int64_t maxlist = nv > nsg ? nv : nsg;
    if (mx < S->max_node && maxlist < TREE_MAX_LIST_SIZE) {
        S->leaves[S->nleaves++] = ni;
        return;
    }
    int32_t c1 = new_node(S), c2 = new_node(S);
    int byx = nd.h < nd.w;
    double piv = byx ? nd.x : nd.y;
    /* vortex range: in-place swap partition */
    int64_t f = nd.vf, l = nd.vl, p1 = f, p2 = l;
    const double* key = byx ? S->x : S->y;
    while (p1 < p2) {
        while (p1 < l && key[p1] < piv) p1++;
        do p2--; while (p2 >= f && key[p2] >= piv);
        if (p1 < p2) swap_slots(S, p1, p2);
    }
    /* bllist: stable split */
    const double* skey = byx ? S->rx : S->ry;
    int64_t nlow = 0;
    int64_t* tmp = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(nsg ? nsg : 1));
    for (int64_t k = nd.sf; k < nd.sl; k++)
        if (skey[S->seg_order[k]] < piv) tmp[nlow++] = S->seg_order[k];
    int64_t nh = nlow;
    for (int64_t k = nd.sf; k < nd.sl; k++)
        if (!(skey[S->seg_order[k]] < piv)) tmp[nh++] = S->seg_order[k];
    for (int64_t k = 0; k < nsg; k++) S->seg_order[nd.sf + k] = tmp[k];
    free(tmp);

    onode* a = &S->nodes[c1];
    a->vf = f; a->vl = p1; a->sf = nd.sf; a->sl = nd.sf + nlow;
    a->depth = nd.depth + 1; a->path = nd.path * 2;
    stretch(S, a);
    onode* b = &S->nodes[c2];
    b->vf = p1; b->vl = l; b->sf = nd.sf + nlow; b->sl = nd.sl;
    b->depth = nd.depth + 1; b->path = nd.path * 2 + 1;
    stretch(S, b);
    S->nodes[ni].ch1 = c1; S->nodes[ni].ch2 = c2;
    divide(S, c1);
    divide(S, c2);
}

/* snode::CalculateCMass / CalculateCMassFromScratch (TSortedTree.cpp:150-197). */
static void cmass(vvo_space* S, int32_t ni) {
    onode* nd = &S->nodes[ni];
    if (nd->ch1 < 0) {
        double px = 0, py = 0, pg = 0, mx = 0, my = 0, mg = 0;
        for (int64_t i = nd->vf; i < nd->vl; i++) {
            double g = S->g[i];
            if (g > 0) { px += S->x[i] * g; py += S->y[i] * g; pg += g; }
            else       { mx += S->x[i] * g; my += S->y[i] * g; mg += g; }
        }
        if (pg) { double inv = 1. / pg; px *= inv; py *= inv; } else { px = nd->x; py = nd->y; }
        if (mg) { double inv = 1. / mg; mx *= inv; my *= inv; } else { mx = nd->x; my = nd->y; }
        nd->cmp_x = px; nd->cmp_y = py; nd->cmp_g = pg;
        nd->cmm_x = mx; nd->cmm_y = my; nd->cmm_g = mg;
        return;
    }
    int32_t c1 = nd->ch1, c2 = nd->ch2;
    cmass(S, c1);
    cmass(S, c2);
    nd = &S->nodes[ni];
    const onode* a = &S->nodes[c1];
    const onode* b = &S->nodes[c2];
    double sumg = a->cmp_g + b->cmp_g;
    if (sumg) {
        double sx = a->cmp_x * a->cmp_g + b->cmp_x * b->cmp_g;
        double sy = a->cmp_y * a->cmp_g + b->cmp_y * b->cmp_g;
        double inv = 1. / sumg;
        nd->cmp_x = sx * inv; nd->cmp_y = sy * inv; nd->cmp_g = sumg;
    } else { nd->cmp_x = nd->x; nd->cmp_y = nd->y; nd->cmp_g = 0; }
    sumg = a->cmm_g + b->cmm_g;
    if (sumg) {
        double sx = a->cmm_x * a->cmm_g + b->cmm_x * b->cmm_g;
        double sy = a->cmm_y * a->cmm_g + b->cmm_y * b->cmm_g;
        double inv = 1. / sumg;
        nd->cmm_x = sx * inv; nd->cmm_y = sy * inv; nd->cmm_g = sumg;
    } else { nd->cmm_x = nd->x; nd->cmm_y = nd->y; nd->cmm_g = 0; }
}

static void push_near(vvo_space* S, int32_t v) {
    if (S->nnear == S->nearcap) {
        S->nearcap = S->nearcap ? 2 * S->nearcap : 4096;
        S->near_list = xrealloc(S->near_list, sizeof(int32_t) * (size_t)S->nearcap);
    }
    S->near_list[S->nnear++] = v;
}
static void push_far(vvo_space* S, int32_t v) {
    if (S->nfar == S->farcap) {
        S->farcap = S->farcap ? 2 * S->farcap : 4096;
        S->far_list = xrealloc(S->far_list, sizeof(int32_t) * (size_t)S->farcap);
    }
    S->far_list[S->nfar++] = v;
}

/* snode::FindNearNodes (TSortedTree.cpp:199-217). */
static void find_near(vvo_space* S, const onode* me, int32_t top) {
    const onode* t = &S->nodes[top];
    double dx = t->x - me->x, dy = t->y - me->y;
    double hp = t->h + t->w + me->h + me->w;
    if (abs2(dx, dy) > S->far_criteria * hp * hp) { push_far(S, top); return; }
    if (t->ch1 >= 0) {
        int32_t c1 = t->ch1, c2 = t->ch2;
        find_near(S, me, c1);
        find_near(S, me, c2);
        return;
    }
    push_near(S, top);
}

/* stree::build (TSortedTree.cpp:232-265). */
int vvo_tree_build(vvo_space* S, double far_criteria, double min_node, double max_node) {
    if (S->built) return -2; /* "Tree is already built" */
    free_tree(S);
    S->far_criteria = far_criteria; S->min_node = min_node; S->max_node = max_node;
    S->seg_order = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(S->m ? S->m : 1));
    for (int64_t k = 0; k < S->m; k++) S->seg_order[k] = k;
    S->leafcap = S->n + S->m + 16;
    S->leaves = (int32_t*)xrealloc(NULL, sizeof(int32_t) * (size_t)S->leafcap);
    int32_t root = new_node(S);
    onode* r = &S->nodes[root];
    r->vf = 0; r->vl = S->n; r->sf = 0; r->sl = S->m; r->depth = 0; r->path = 0;
    double t0 = now_s();
    stretch(S, r);
    divide(S, root);
    double t1 = now_s();
    cmass(S, root);
    double t2 = now_s();
    S->near_off = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(S->nleaves + 1));
    S->far_off = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(S->nleaves + 1));
    /* with a timing sample, lists are built for the sampled leaves and for the leaves that
     * hold segment centres (the SLAE right-hand side reads those) */
    char* need = NULL;
    if (S->stride > 1) {
        need = (char*)calloc((size_t)S->nleaves + 1, 1);
        int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * (size_t)S->nnodes);
        for (int64_t L = 0; L < S->nleaves; L++) pos[S->leaves[L]] = (int32_t)L;
        for (int64_t sg = 0; sg < S->m; sg++) need[pos[find_node(S, S->rx[sg], S->ry[sg])]] = 1;
        free(pos);
    }
    for (int64_t L = 0; L < S->nleaves; L++) {
        S->near_off[L] = S->nnear; S->far_off[L] = S->nfar;
        if (need && (L % S->stride) && !need[L]) continue;
        onode me = S->nodes[S->leaves[L]];
        find_near(S, &me, root);
    }
    free(need);
    S->t_partition = t1 - t0;
    S->t_cmass = t2 - t1;
    S->t_lists = now_s() - t2;
    S->near_off[S->nleaves] = S->nnear; S->far_off[S->nleaves] = S->nfar;
    S->built = 1;
    return 0;
}

int vvo_tree_destroy(vvo_space* S) { free_tree(S); return 0; }

int vvo_tree_sizes(const vvo_space* S, int64_t* nnodes, int64_t* nleaves, int64_t* nnear,
                   int64_t* nfar) {
    if (nnodes) *nnodes = S->nnodes;
    if (nleaves) *nleaves = S->nleaves;
    if (nnear) *nnear = S->nnear;
    if (nfar) *nfar = S->nfar;
    return S->built ? 0 : -3;
}

int vvo_tree_leaves(const vvo_space* S, double* x, double* y, double* h, double* w,
                    int64_t* vfirst, int64_t* vlast, int32_t* depth, int64_t* path,
                    int64_t* sfirst, int64_t* slast) {
    if (!S->built) return -3;
    for (int64_t L = 0; L < S->nleaves; L++) {
        const onode* nd = &S->nodes[S->leaves[L]];
        if (x) x[L] = nd->x;
        if (y) y[L] = nd->y;
        if (h) h[L] = nd->h;
        if (w) w[L] = nd->w;
        if (vfirst) vfirst[L] = nd->vf;
        if (vlast) vlast[L] = nd->vl;
        if (depth) depth[L] = nd->depth;
        if (path) path[L] = nd->path;
        if (sfirst) sfirst[L] = nd->sf;
        if (slast) slast[L] = nd->sl;
    }
    return 0;
}

int vvo_tree_nodes(const vvo_space* S, double* x, double* y, double* h, double* w,
                   int64_t* vfirst, int64_t* vlast, int32_t* depth, int64_t* path,
                   double* cmp_x, double* cmp_y, double* cmp_g,
                   double* cmm_x, double* cmm_y, double* cmm_g) {
    if (!S->built) return -3;
    for (int64_t k = 0; k < S->nnodes; k++) {
        const onode* nd = &S->nodes[k];
        if (x) x[k] = nd->x;
        if (y) y[k] = nd->y;
        if (h) h[k] = nd->h;
        if (w) w[k] = nd->w;
        if (vfirst) vfirst[k] = nd->vf;
        if (vlast) vlast[k] = nd->vl;
        if (depth) depth[k] = nd->depth;
        if (path) path[k] = nd->path;
        if (cmp_x) cmp_x[k] = nd->cmp_x;
        if (cmp_y) cmp_y[k] = nd->cmp_y;
        if (cmp_g) cmp_g[k] = nd->cmp_g;
        if (cmm_x) cmm_x[k] = nd->cmm_x;
        if (cmm_y) cmm_y[k] = nd->cmm_y;
        if (cmm_g) cmm_g[k] = nd->cmm_g;
    }
    return 0;
}

int vvo_tree_seg_order(const vvo_space* S, int64_t* seg_order) {
    if (!S->built) return -3;
    memcpy(seg_order, S->seg_order, sizeof(int64_t) * (size_t)S->m);
    return 0;
}

int vvo_tree_lists(const vvo_space* S, int64_t* near_off, int32_t* near_depth, int64_t* near_path,
                   int64_t* far_off, int32_t* far_depth, int64_t* far_path) {
    if (!S->built) return -3;
    for (int64_t L = 0; L <= S->nleaves; L++) {
        if (near_off) near_off[L] = S->near_off[L];
        if (far_off) far_off[L] = S->far_off[L];
    }
    for (int64_t k = 0; k < S->nnear; k++) {
        const onode* nd = &S->nodes[S->near_list[k]];
        if (near_depth) near_depth[k] = nd->depth;
        if (near_path) near_path[k] = nd->path;
    }
    for (int64_t k = 0; k < S->nfar; k++) {
        const onode* nd = &S->nodes[S->far_list[k]];
        if (far_depth) far_depth[k] = nd->depth;
        if (far_path) far_path[k] = nd->path;
    }
    return 0;
}

/* stree::findNode (TSortedTree.cpp:284-303). */
static int32_t find_node(const vvo_space* S, double px, double py) {
    int32_t k = 0;
    while (S->nodes[k].ch1 >= 0) {
        const onode* nd = &S->nodes[k];
        if (nd->h < nd->w) k = (px < nd->x) ? nd->ch1 : nd->ch2;
        else               k = (py < nd->y) ? nd->ch1 : nd->ch2;
    }
    return k;
}

/* ------------------------------------------------------------------------------------ */
/* Epsilon / merge (libvvhd/src/MEpsilonFast.cpp)                                       */
/* ------------------------------------------------------------------------------------ */

/* MEpsilonFast::nearestBodySegment (MEpsilonFast.cpp:214-253) for leaf L. Returns -1 if none. */
static int64_t nearest_body_segment_L(const vvo_space* S, int64_t L, double px, double py) {
    int64_t att = -1;
    double res = DBL_MAX;
    for (int64_t k = S->near_off[L]; k < S->near_off[L + 1]; k++) {
        const onode* nn = &S->nodes[S->near_list[k]];
        for (int64_t q = nn->sf; q < nn->sl; q++) {
            int64_t s = S->seg_order[q];
            double d = abs2(px - S->rx[s], py - S->ry[s]);
            if (d < res) { res = d; att = s; }
        }
    }
    if (att >= 0) return att;
    for (int bi = 0; bi < S->nb; bi++) {
        const obody* b = &S->bodies[bi];
        for (int64_t k = 0; k < b->count; k++) {
            int64_t s = b->first + k;
            double d = abs2(px - S->rx[s], py - S->ry[s]);
            if (d < res) { res = d; att = s; }
            else k += 9; /* "speed up" skip, MEpsilonFast.cpp:248 */
        }
    }
    return att;
}

static int64_t g_merged;

/* MEpsilonFast::MergeVortexes (MEpsilonFast.cpp:111-126). */
static void merge_vortexes(vvo_space* S, int64_t a, int64_t b) {
    g_merged++;
    if (sgn(S->g[a]) == sgn(S->g[b])) {
        double sx = S->x[a] * S->g[a] + S->x[b] * S->g[b];
        double sy = S->y[a] * S->g[a] + S->y[b] * S->g[b];
        double inv = 1. / (S->g[a] + S->g[b]);
        S->x[a] = sx * inv; S->y[a] = sy * inv;
    } else if (fabs(S->g[a]) < fabs(S->g[b])) {
        S->x[a] = S->x[b]; S->y[a] = S->y[b];
    }
    S->g[a] += S->g[b];
    S->g[b] = 0;
}

/* MEpsilonFast::epsv (MEpsilonFast.cpp:128-173). */
static double epsv(vvo_space* S, int64_t L, int64_t lv, double mcs) {
    double res1 = DBL_MAX, res2 = DBL_MAX;
    int64_t lv1 = -1, lv2 = -1;
    for (int64_t k = S->near_off[L]; k < S->near_off[L + 1]; k++) {
        const onode* nn = &S->nodes[S->near_list[k]];
        for (int64_t j = nn->vf; j < nn->vl; j++) {
            if (!S->g[j] || j == lv) continue;
            double d = abs2(S->x[lv] - S->x[j], S->y[lv] - S->y[j]);
            if (res1 > d) { res2 = res1; lv2 = lv1; res1 = d; lv1 = j; }
            else if (res2 > d) { res2 = d; lv2 = j; }
        }
    }
    if (lv1 < 0) return DBL_MIN;
    if (lv2 < 0) return sqrt(res1);
    if (isnan(mcs)) return sqrt(res2);
    if ((res1 < mcs) || ((sgn(S->g[lv1]) == sgn(S->g[lv2])) && (sgn(S->g[lv1]) != sgn(S->g[lv])))) {
        merge_vortexes(S, lv, lv1);
        return epsv(S, L, lv, NAN);
    }
    return sqrt(res2);
}

/* MEpsilonFast::CalcEpsilonFast (MEpsilonFast.cpp:11-63), vortex list only. */
int vvo_eps(vvo_space* S, int merge, int64_t* merged) {
    if (!S->built) return -3;
    g_merged = 0;
    for (int64_t L = 0; L < S->nleaves; L++) {
        if (L % S->stride) continue;
        const onode* nd = &S->nodes[S->leaves[L]];
        double cx = nd->x, cy = nd->y;
        int64_t att = nearest_body_segment_L(S, L, cx, cy);
        double mcs;
        if (merge) {
            mcs = (att >= 0)
                ? 0.16 * abs2(S->dlx[att], S->dly[att]) * (1. + sqrt(abs2(cx - S->rx[att], cy - S->ry[att])))
                : 0;
        } else {
            mcs = NAN;
        }
        double eps_r = (att >= 0) ? sqrt(abs2(S->dlx[att], S->dly[att])) * (1.0 / 3.0) : 0;
        for (int64_t i = nd->vf; i < nd->vl; i++) {
            if (!S->g[i]) continue;
            S->ie[i] = 1.0 / smax(epsv(S, L, i, mcs), eps_r);
        }
    }
    if (merged) *merged = g_merged;
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Convective (libvvhd/src/MConvectiveFast.cpp)                                         */
/* ------------------------------------------------------------------------------------ */

/* near_nodes_influence (MConvectiveFast.cpp:122-137) with biot_savart (:116-120). */
static void near_influence(const vvo_space* S, int64_t L, double px, double py,
                           double* ox, double* oy) {
    double rx = 0, ry = 0;
    for (int64_t k = S->near_off[L]; k < S->near_off[L + 1]; k++) {
        const onode* nn = &S->nodes[S->near_list[k]];
        for (int64_t j = nn->vf; j < nn->vl; j++) {
            if (!S->g[j]) continue;
            double dx = px - S->x[j], dy = py - S->y[j];
            double e = 1. / S->ie[j];
            double s = S->g[j] / (abs2(dx, dy) + e * e);
            rx += (-dy) * s;
            ry += dx * s;
        }
    }
    *ox = rx * C_1_2PI;
    *oy = ry * C_1_2PI;
}

/* The reference writes abs(src.g) without std:: and without a global abs(double) in scope
 * (MConvectiveFast.cpp:166), so C's int abs(int) runs on the circulation truncated to int. */
static double int_abs_of(double g) { return (double)abs((int)g); }

/* sink_list_influence (MConvectiveFast.cpp:153-170). */
static void sink_influence(const vvo_space* S, double px, double py, double* ox, double* oy) {
    double rx = 0, ry = 0;
    const double e2 = S->dt * C_1_PI;
    for (int64_t k = 0; k < S->ns; k++) {
        double dx = px - S->snk_x[k], dy = py - S->snk_y[k];
        double s = S->snk_g[k] / (abs2(dx, dy) + e2 * int_abs_of(S->snk_g[k]));
        rx += dx * s; ry += dy * s;
    }
    *ox = rx * C_1_2PI;
    *oy = ry * C_1_2PI;
}

/* SegmentInfluence_linear_source (MConvectiveFast.cpp:440-457): the velocity of a source
 * sheet of linearly varying strength q1 -> q2 along segment s, in the complex arithmetic of
 * std::complex<double> (libgcc's complex multiply and divide, the C library's clog). */
static void seg_linear_source(const vvo_space* S, int64_t s, double px, double py, double q1, double q2,
                              double* ox, double* oy) {
    const double complex z = CMPLX(px, py);
    const double complex zc = CMPLX(S->rx[s], S->ry[s]);
    const double complex dz = CMPLX(S->dlx[s], S->dly[s]);
    const double complex zs1 = zc - dz * 0.5;
    const double complex zs2 = zc + dz * 0.5;
    const double complex z1 = z - zs1;
    const double complex z2 = z - zs2;
    const double complex zV = ((q2 - q1) - conj(q2 * z1 - q1 * z2) / conj(dz) * clog(conj(z2) / conj(z1))) / conj(dz);
    *ox = creal(zV);
    *oy = cimag(zV);
}

/* body_list_influence (MConvectiveFast.cpp:172-215): slip segments act as smoothed point
 * vortices; a body whose speed_slae is not zero (TVec3D::iszero) carries attached vortex and
 * source sheets of strengths -Vs.dl and -rotl(Vs).dl, Vs the body's velocity at the point of
 * the segment (rotation about get_axis() = holder + dpos, TBody.hpp:124): linear sheets
 * within |dl| of the segment centre, point singularities beyond. */
static void body_influence(const vvo_space* S, double px, double py, double* ox, double* oy) {
    double rx = 0, ry = 0;
    for (int bi = 0; bi < S->nb; bi++) {
        const obody* b = &S->bodies[bi];
        int any = 0;
        for (int64_t k = 0; k < b->count; k++) any = any || S->slip[b->first + k];
        if (any) {
            for (int64_t k = 0; k < b->count; k++) {
                int64_t s = b->first + k;
                if (!S->slip[s]) continue;
                double dx = px - S->rx[s], dy = py - S->ry[s];
                double e = 1. / S->sie[s];
                double sc = S->sg[s] / (abs2(dx, dy) + e * e);
                rx += (-dy) * sc; ry += dx * sc;
            }
        }
        const vvo_body_params* p = &b->p;
        if (fabs(p->speed_slae_x) + fabs(p->speed_slae_y) + fabs(p->speed_slae_o) < 1E-10) continue;
        const double ax = p->holder_x + p->dpos_x, ay = p->holder_y + p->dpos_y;
        const double vx = p->speed_slae_x, vy = p->speed_slae_y, vo = p->speed_slae_o;
        for (int64_t k = 0; k < b->count; k++) {
            const int64_t s = b->first + k;
            const double dlx = S->dlx[s], dly = S->dly[s];
            const double drabs2 = abs2(px - S->rx[s], py - S->ry[s]);
            if (drabs2 < abs2(dlx, dly)) {
                /* Vs1 = V.r + V.o rotl(corner - axis), Vs2 at corner + dl */
                const double c1x = S->cx[s] - ax, c1y = S->cy[s] - ay;
                const double w1x = vx + (-c1y) * vo, w1y = vy + c1x * vo;
                const double g1 = (-w1x) * dlx + (-w1y) * dly;
                const double q1 = w1y * dlx + (-w1x) * dly;
                const double c2x = (S->cx[s] + dlx) - ax, c2y = (S->cy[s] + dly) - ay;
                const double w2x = vx + (-c2y) * vo, w2y = vy + c2x * vo;
                const double g2 = (-w2x) * dlx + (-w2y) * dly;
                const double q2 = w2y * dlx + (-w2x) * dly;
                double ux, uy;
                seg_linear_source(S, s, px, py, g1, g2, &ux, &uy);
                rx += -uy; ry += ux;  /* rotl */
                seg_linear_source(S, s, px, py, q1, q2, &ux, &uy);
                rx += ux; ry += uy;
            } else {
                const double cx = S->rx[s] - ax, cy = S->ry[s] - ay;
                const double wx = vx + (-cy) * vo, wy = vy + cx * vo;
                const double g = (-wx) * dlx + (-wy) * dly;
                const double q = wy * dlx + (-wx) * dly;
                const double dx = px - S->rx[s], dy = py - S->ry[s];
                const double inv = 1. / drabs2;  /* TVec / c is TVec * (1 / c) */
                rx += (dx * q + (-dy) * g) * inv;
                ry += (dy * q + dx * g) * inv;
            }
        }
    }
    *ox = rx * C_1_2PI;
    *oy = ry * C_1_2PI;
}

static int bodies_at_rest(const vvo_space* S) {
    for (int bi = 0; bi < S->nb; bi++) {
        const vvo_body_params* p = &S->bodies[bi].p;
        /* TVec3D::iszero, TVec3D.hpp:17 */
        if (!(fabs(p->speed_slae_x) + fabs(p->speed_slae_y) + fabs(p->speed_slae_o) < 1E-10)) return 0;
    }
    return 1;
}

/* MConvectiveFast::process_all_lists (MConvectiveFast.cpp:36-114), vortex list. */
int vvo_convective(vvo_space* S) {
    if (!S->built) return -3;
    for (int64_t L = 0; L < S->nleaves; L++) {
        if (L % S->stride) continue;
        const onode* nd = &S->nodes[S->leaves[L]];
        double t1 = 0, t2 = 0, t3 = 0, t4 = 0;
        for (int64_t k = S->far_off[L]; k < S->far_off[L + 1]; k++) {
            const onode* fn = &S->nodes[S->far_list[k]];
            double dpx = nd->x - fn->cmp_x, dpy = nd->y - fn->cmp_y;
            double dmx = nd->x - fn->cmm_x, dmy = nd->y - fn->cmm_y;
            double fp1 = fn->cmp_g / abs2(dpx, dpy);
            double fm1 = fn->cmm_g / abs2(dmx, dmy);
            double fp2 = fn->cmp_g / sqr(abs2(dpx, dpy));
            double fm2 = fn->cmm_g / sqr(abs2(dmx, dmy));
            t1 -= (fp1 * dpy + fm1 * dmy);
            t2 += (fp1 * dpx + fm1 * dmx);
            t3 += (fp2 * dpy * dpx + fm2 * dmy * dmx);
            t4 += (fp2 * (sqr(dpy) - sqr(dpx)) + fm2 * (sqr(dmy) - sqr(dmx)));
        }
        t1 *= C_1_2PI; t2 *= C_1_2PI; t3 *= C_1_PI; t4 *= C_1_2PI;
        /* the reference opens one parallel region per leaf (MConvectiveFast.cpp:73-75) */
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = nd->vf; i < nd->vl; i++) {
            if (!S->g[i]) continue;
            double px = S->x[i], py = S->y[i];
            double lx = px - nd->x, ly = py - nd->y;
            double ax, ay;
            S->vx[i] += S->inf_vx; S->vy[i] += S->inf_vy;
            near_influence(S, L, px, py, &ax, &ay); S->vx[i] += ax; S->vy[i] += ay;
            sink_influence(S, px, py, &ax, &ay); S->vx[i] += ax; S->vy[i] += ay;
            body_influence(S, px, py, &ax, &ay); S->vx[i] += ax; S->vy[i] += ay;
            S->vx[i] += t1; S->vy[i] += t2;
            S->vx[i] += t3 * lx + t4 * ly;
            S->vy[i] += t4 * lx + (-t3) * ly;
        }
    }
    return 0;
}

/* MConvectiveFast::velocity (MConvectiveFast.cpp:20-34) with far_nodes_influence (:139-151). */
int vvo_velocity_points(vvo_space* S, int64_t n, const double* px, const double* py,
                        double* vx, double* vy) {
    if (!S->built) return -3;
    int32_t* pos = (int32_t*)xrealloc(NULL, sizeof(int32_t) * (size_t)(S->nnodes ? S->nnodes : 1));
    for (int64_t k = 0; k < S->nnodes; k++) pos[k] = -1;
    for (int64_t t = 0; t < S->nleaves; t++) pos[S->leaves[t]] = (int32_t)t;
    for (int64_t q = 0; q < n; q++) {
        const int64_t L = pos[find_node(S, px[q], py[q])];
        double rx = 0, ry = 0, ax, ay;
        if (L >= 0) {
            near_influence(S, L, px[q], py[q], &ax, &ay); rx += ax; ry += ay;
            double fx = 0, fy = 0;
            for (int64_t t = S->far_off[L]; t < S->far_off[L + 1]; t++) {
                const onode* fn = &S->nodes[S->far_list[t]];
                double dx = px[q] - fn->cmp_x, dy = py[q] - fn->cmp_y;
                double s = fn->cmp_g / (abs2(dx, dy) + 0.);
                fx += (-dy) * s; fy += dx * s;
                dx = px[q] - fn->cmm_x; dy = py[q] - fn->cmm_y;
                s = fn->cmm_g / (abs2(dx, dy) + 0.);
                fx += (-dy) * s; fy += dx * s;
            }
            rx += fx * C_1_2PI; ry += fy * C_1_2PI;
            sink_influence(S, px[q], py[q], &ax, &ay); rx += ax; ry += ay;
            body_influence(S, px[q], py[q], &ax, &ay); rx += ax; ry += ay;
            rx += S->inf_vx; ry += S->inf_vy;
        }
        vx[q] = rx; vy[q] = ry;
    }
    free(pos);
    return 0;
}

int vvo_direct_velocity(const vvo_space* S, int64_t n, const double* px, const double* py,
                        double* vx, double* vy) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t q = 0; q < n; q++) {
        double rx = 0, ry = 0;
        for (int64_t j = 0; j < S->n; j++) {
            if (!S->g[j]) continue;
            double dx = px[q] - S->x[j], dy = py[q] - S->y[j];
            double e = 1. / S->ie[j];
            double s = S->g[j] / (abs2(dx, dy) + e * e);
            rx += (-dy) * s; ry += dx * s;
        }
        double ax, ay, bx, by;
        sink_influence(S, px[q], py[q], &ax, &ay);
        body_influence(S, px[q], py[q], &bx, &by);
        vx[q] = rx * C_1_2PI + ax + bx + S->inf_vx;
        vy[q] = ry * C_1_2PI + ay + by + S->inf_vy;
    }
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Diffusive (libvvhd/src/MDiffusiveFast.cpp)                                           */
/* ------------------------------------------------------------------------------------ */

/* MDiffusiveFast::process_vort_list (MDiffusiveFast.cpp:8-48) with vortex_influence
 * (:94-105) and segment_influence (:108-123). */
int vvo_diffusive(vvo_space* S) {
    if (!S->built) return -3;
    const double re = S->re;
    for (int64_t L = 0; L < S->nleaves; L++) {
        if (L % S->stride) continue;
        const onode* nd = &S->nodes[S->leaves[L]];
        for (int64_t i = nd->vf; i < nd->vl; i++) {
            if (!S->g[i]) continue;
            double s2x = 0, s2y = 0, s3x = 0, s3y = 0, s1 = 0, s0 = 0;
            double xi = S->x[i], yi = S->y[i], gi = S->g[i], ie = S->ie[i];
            for (int64_t k = S->near_off[L]; k < S->near_off[L + 1]; k++) {
                const onode* nn = &S->nodes[S->near_list[k]];
                for (int64_t j = nn->vf; j < nn->vl; j++) {
                    double gj = S->g[j];
                    if (!gj) continue;
                    if (sgn(gi) != sgn(gj)) continue;
                    double dx = xi - S->x[j], dy = yi - S->y[j];
                    if (fabs(dx) + fabs(dy) < 1E-10) continue; /* TVec::iszero */
                    double drabs = sqrt(abs2(dx, dy));
                    double ea = -drabs * ie;
                    if (ea < EXP_ARG_RESTRICTION) continue;
                    double t = gj * exp(ea);
                    double q = t / drabs;
                    s2x += dx * q; s2y += dy * q;
                    s1 += t;
                }
                for (int64_t q = nn->sf; q < nn->sl; q++) {
                    int64_t s = S->seg_order[q];
                    double dx = xi - S->rx[s], dy = yi - S->ry[s];
                    double dr2 = abs2(dx, dy);
                    double dr = sqrt(dr2);
                    double ea = -dr * ie;
                    if (ea < EXP_ARG_RESTRICTION) continue;
                    double ex = exp(ea);
                    double dsx = -S->dly[s], dsy = S->dlx[s];
                    s3x += dsx * ex; s3y += dsy * ex;
                    s0 += (dr * ie + 1) / dr2 * (dx * dsx + dy * dsy) * ex;
                    S->fric[s] += sqr(ie) * gi * ex * sqrt(abs2(dsx, dsy));
                }
            }
            if ((sgn(s1) != sgn(gi)) || (fabs(s1) < fabs(0.1 * gi))) s1 = 0.1 * gi;
            double f = ie / (re * s1);
            S->vx[i] += s2x * f; S->vy[i] += s2y * f;
            if (s0 > C_PI) s0 = C_PI;
            f = sqr(ie) / (re * (C_2PI - s0));
            S->vx[i] += s3x * f; S->vy[i] += s3y * f;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Body SLAE (MConvectiveFast.cpp:235-273, 286-310, 398-418, 459-862, 882-1017)          */
/* ------------------------------------------------------------------------------------ */

static double xi_g_near(double px, double py, double pcx, double pcy, double dlx, double dly,
                        double rd) {
    return ((pcx - px) * dlx + (pcy - py) * dly) / sqr(rd);
}
static double xi_g_dist(double px, double py, double p1x, double p1y, double p2x, double p2y) {
    return 0.5 * log(abs2(px - p2x, py - p2y) / abs2(px - p1x, py - p1y));
}
/* _2PI_Xi_g (MConvectiveFast.cpp:286-310) for segment s at point p with radius rd. */
static double xi_g(const vvo_space* S, double px, double py, int64_t s, double rd) {
    double cx = S->cx[s], cy = S->cy[s], dlx = S->dlx[s], dly = S->dly[s];
    double rd_sqr = sqr(rd);
    double dr1 = abs2(px - cx, py - cy);
    double dr2 = abs2((px - cx) - dlx, (py - cy) - dly);
    if (dr1 >= rd_sqr && dr2 >= rd_sqr) return 0.5 * log(dr2 / dr1);
    if (dr1 <= rd_sqr && dr2 <= rd_sqr) return xi_g_near(px, py, S->rx[s], S->ry[s], dlx, dly, rd);
    double rx = S->rx[s], ry = S->ry[s];
    double a0 = abs2(dlx, dly);
    double b0 = (px - rx) * dlx + (py - ry) * dly;
    double d = sqrt(b0 * b0 - a0 * (abs2(px - rx, py - ry) - rd * rd));
    double k = (b0 + d) / a0;
    if ((k <= -0.5) || (k >= 0.5)) k = (b0 - d) / a0;
    double p3x = rx + dlx * k, p3y = ry + dly * k;
    if (dr1 < rd_sqr)
        return xi_g_near(px, py, (p3x + cx) * 0.5, (p3y + cy) * 0.5, p3x - cx, p3y - cy, rd)
             + xi_g_dist(px, py, p3x, p3y, cx + dlx, cy + dly);
    return xi_g_dist(px, py, cx, cy, p3x, p3y)
         + xi_g_near(px, py, ((cx + dlx) + p3x) * 0.5, ((cy + dly) + p3y) * 0.5,
                     (cx + dlx) - p3x, (cy + dly) - p3y, rd);
}

/* NodeInfluence (MConvectiveFast.cpp:398-418). */
static double node_influence(const vvo_space* S, int64_t L, int64_t s) {
    double res = 0;
    for (int64_t k = S->near_off[L]; k < S->near_off[L + 1]; k++) {
        const onode* nn = &S->nodes[S->near_list[k]];
        for (int64_t j = nn->vf; j < nn->vl; j++) {
            if (!S->g[j]) continue;
            res += xi_g(S, S->x[j], S->y[j], s, 1. / S->ie[j]) * S->g[j];
        }
    }
    double c1x = S->cx[s], c1y = S->cy[s], c2x = S->cx[s] + S->dlx[s], c2y = S->cy[s] + S->dly[s];
    for (int64_t k = S->far_off[L]; k < S->far_off[L + 1]; k++) {
        const onode* fn = &S->nodes[S->far_list[k]];
        res += xi_g_dist(fn->cmp_x, fn->cmp_y, c1x, c1y, c2x, c2y) * fn->cmp_g;
        res += xi_g_dist(fn->cmm_x, fn->cmm_y, c1x, c1y, c2x, c2y) * fn->cmm_g;
    }
    return res * C_1_2PI;
}

double vvo_gsum(const vvo_space* S) {
    double r = 0;
    for (int64_t i = 0; i < S->n; i++) r += S->g[i];
    return r;
}

static int is_rigid(double k) { return !(k >= 0 && isfinite(k)); }

int64_t vvo_slae_size(const vvo_space* S) { return S->m + 9 * (int64_t)S->nb; }

/* LU with partial pivoting (row-major), solves A x = b in place of b.  Any LAPACK-like
 * solver gives the reference's TMatrix.cpp:166-223 result to within rounding. */
static int lu_solve(int64_t n, double* A, double* b) {
    for (int64_t k = 0; k < n; k++) {
        int64_t p = k;
        double best = fabs(A[k * n + k]);
        for (int64_t i = k + 1; i < n; i++) {
            double v = fabs(A[i * n + k]);
            if (v > best) { best = v; p = i; }
        }
        if (best == 0) return -5;
        if (p != k) {
            for (int64_t j = 0; j < n; j++) { double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
            double t = b[k]; b[k] = b[p]; b[p] = t;
        }
        double piv = A[k * n + k];
        for (int64_t i = k + 1; i < n; i++) {
            double l = A[i * n + k] / piv;
            if (l == 0) continue;
            A[i * n + k] = l;
            for (int64_t j = k + 1; j < n; j++) A[i * n + j] -= l * A[k * n + j];
            b[i] -= l * b[k];
        }
    }
    for (int64_t k = n - 1; k >= 0; k--) {
        double s = b[k];
        for (int64_t j = k + 1; j < n; j++) s -= A[k * n + j] * b[j];
        b[k] = s / A[k * n + k];
    }
    return 0;
}

/* MConvectiveFast::calc_circulation + fill_matrix for rigid bodies (no collision, no
 * root bodies, no springs).  Column layout follows the solution pointer map built at
 * MConvectiveFast.cpp:250-267: per body [segments..., speed_slae x,y,o, force_hydro x,y,o,
 * force_holder x,y,o]; rows follow fill_matrix's eq_no order (:896-975). */
int vvo_slae(vvo_space* S, vvo_body_out* out) {
    if (!S->built) return -3;
    for (int bi = 0; bi < S->nb; bi++) {
        const vvo_body_params* p = &S->bodies[bi].p;
        if (!is_rigid(p->kspring_x) || !is_rigid(p->kspring_y) || !is_rigid(p->kspring_o)) return -4;
    }
    int64_t n = vvo_slae_size(S);
    S->neq = n;
    S->mat = xrealloc(S->mat, sizeof(double) * (size_t)(n * n));
    S->rhs = xrealloc(S->rhs, sizeof(double) * (size_t)n);
    S->sol = xrealloc(S->sol, sizeof(double) * (size_t)n);
    memset(S->mat, 0, sizeof(double) * (size_t)(n * n));
    memset(S->rhs, 0, sizeof(double) * (size_t)n);
    double* A = S->mat;
    double* B = S->rhs;
    /* column of body bj's speed/force unknowns */
    int64_t* col0 = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(S->nb + 1));
    {
        int64_t c = 0;
        for (int bi = 0; bi < S->nb; bi++) { col0[bi] = c; c += S->bodies[bi].count + 9; }
        col0[S->nb] = c;
    }
#define SEGCOL(bj, k) (col0[bj] + (k))
#define BCOL(bj, q) (col0[bj] + S->bodies[bj].count + (q))
    const double _1_dt = 1 / S->dt;
    const double _1_2dt = 0.5 / S->dt;
    const double gsum = vvo_gsum(S);
    /* node -> leaf position (the reference's findNode returns the leaf itself) */
    int64_t* leaf_pos = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(S->nnodes ? S->nnodes : 1));
    for (int64_t t = 0; t < S->nleaves; t++) leaf_pos[S->leaves[t]] = t;
    int once = 0;
    for (int bi = 0; bi < S->nb; bi++) {
        const obody* b = &S->bodies[bi];
        const vvo_body_params* p = &b->p;
        for (int64_t k = 0; k < b->count; k++) {
            int64_t eq = col0[bi] + k;
            int64_t s = b->first + k;
            if (k != p->special_segment_no) {
                /* fillSlipEquationForSegment (:459-482) */
                double r = (-S->inf_vy) * S->dlx[s] + S->inf_vx * S->dly[s];
                double sx, sy;
                sink_influence(S, S->rx[s], S->ry[s], &sx, &sy);
                r += (-sy) * S->dlx[s] + sx * S->dly[s];
                int32_t nk = find_node(S, S->rx[s], S->ry[s]);
                r -= node_influence(S, leaf_pos[nk], s);
                B[eq] = r;
                for (int bj = 0; bj < S->nb; bj++) {
                    const obody* jb = &S->bodies[bj];
                    for (int64_t q = 0; q < jb->count; q++) {
                        int64_t sj = jb->first + q;
                        double rd = sqrt(abs2(S->dlx[sj], S->dly[sj])) * 0.25;
                        A[eq * n + SEGCOL(bj, q)] = xi_g(S, S->cx[sj], S->cy[sj], s, rd) * C_1_2PI;
                    }
                    /* _2PI_A123 (:375-396); A3 is 0 for a rigid body with no rotation */
                    double a1 = (bi == bj) ? C_2PI * S->dly[s] : 0;
                    double a2 = (bi == bj) ? -C_2PI * S->dlx[s] : 0;
                    if (!(is_rigid(jb->p.kspring_o) && jb->p.speed_o == 0)) { free(col0); return -4; }
                    A[eq * n + BCOL(bj, 0)] = a1 * C_1_2PI;
                    A[eq * n + BCOL(bj, 1)] = a2 * C_1_2PI;
                    A[eq * n + BCOL(bj, 2)] = 0 * C_1_2PI;
                }
            } else if (p->bc_kutta) {
                /* fillZeroEquationForSegment (:484-492) */
                B[eq] = 0;
                A[eq * n + SEGCOL(bi, k)] = 1;
            } else if (!once++) {
                /* fillInfSteadyEquationForSegment (:508-522) */
                B[eq] = -gsum - S->inf_g;
                for (int bj = 0; bj < S->nb; bj++) {
                    const obody* jb = &S->bodies[bj];
                    for (int64_t q = 0; q < jb->count; q++) A[eq * n + SEGCOL(bj, q)] = 1;
                    A[eq * n + BCOL(bj, 2)] = 2 * jb->area;
                }
            } else {
                /* fillSteadyEquationForSegment (:494-506) */
                B[eq] = p->g_dead + 2 * b->area * p->speed_slae_prev_o;
                for (int64_t q = 0; q < b->count; q++) A[eq * n + SEGCOL(bi, q)] = 1;
                A[eq * n + BCOL(bi, 2)] = 2 * b->area;
            }
        }
        int64_t e0 = col0[bi] + b->count;
        /* fillSpeedX/Y/OEquation (:803-862): rigid bodies (or time <= 0) */
        B[e0 + 0] = p->speed_x; A[(e0 + 0) * n + BCOL(bi, 0)] = 1;
        B[e0 + 1] = p->speed_y; A[(e0 + 1) * n + BCOL(bi, 1)] = 1;
        B[e0 + 2] = p->speed_o; A[(e0 + 2) * n + BCOL(bi, 2)] = 1;

        const double area = b->area, cofx = b->cofm_x, cofy = b->cofm_y;
        const double axx = body_axis_x(b), axy = body_axis_y(b);
        const double rcx = cofx - axx, rcy = cofy - axy;
        const double moi = body_moi_axis(b);
        const double dens = p->density;
        const double pvx = p->speed_slae_prev_x, pvy = p->speed_slae_prev_y, pvo = p->speed_slae_prev_o;
        /* fillHydroXEquation (:533-562) */
        {
            int64_t eq = e0 + 3;
            double tx = cofx * 2 + rcx, ty = cofy * 2 + rcy; /* 2*cofm + r_c_com */
            B[eq] = area * _1_dt * pvx + area * _1_dt * (-ty) * pvo + sqr(pvo) * area * rcx
                  - p->friction_prev_x + p->fdt_dead_x * _1_dt;
            for (int64_t q = 0; q < b->count; q++) A[eq * n + SEGCOL(bi, q)] = _1_dt * (-S->cy[b->first + q]);
            A[eq * n + BCOL(bi, 0)] = area * _1_dt;
            A[eq * n + BCOL(bi, 1)] = 0;
            A[eq * n + BCOL(bi, 2)] = area * _1_dt * (-2 * cofy - rcy);
            A[eq * n + BCOL(bi, 3)] = -1;
            (void)tx;
        }
        /* fillHydroYEquation (:564-593) */
        {
            int64_t eq = e0 + 4;
            double tx = cofx * 2 + rcx;
            B[eq] = area * _1_dt * pvy + area * _1_dt * tx * pvo + sqr(pvo) * area * rcy
                  - p->friction_prev_y + p->fdt_dead_y * _1_dt;
            for (int64_t q = 0; q < b->count; q++) A[eq * n + SEGCOL(bi, q)] = _1_dt * (S->cx[b->first + q]);
            A[eq * n + BCOL(bi, 0)] = 0;
            A[eq * n + BCOL(bi, 1)] = area * _1_dt;
            A[eq * n + BCOL(bi, 2)] = area * _1_dt * (2 * cofx + rcx);
            A[eq * n + BCOL(bi, 4)] = -1;
        }
        /* fillHydroOEquation (:595-623) */
        {
            int64_t eq = e0 + 5;
            double c = area * _1_dt;
            double lx = (-rcy) * c, ly = rcx * c; /* (area*_1_dt) * rotl(r_c_com) */
            B[eq] = (lx * pvx + ly * pvy) + 2 * moi * _1_dt * pvo - p->friction_prev_o + p->fdt_dead_o * _1_2dt;
            for (int64_t q = 0; q < b->count; q++) {
                int64_t s = b->first + q;
                A[eq * n + SEGCOL(bi, q)] = _1_2dt * abs2(S->cx[s] - axx, S->cy[s] - axy);
            }
            A[eq * n + BCOL(bi, 0)] = area * _1_dt * (-rcy);
            A[eq * n + BCOL(bi, 1)] = area * _1_dt * (rcx);
            A[eq * n + BCOL(bi, 2)] = 2 * moi * _1_dt;
            A[eq * n + BCOL(bi, 5)] = -1;
        }
        /* fillNewtonXEquation (:634-667) */
        {
            int64_t eq = e0 + 6;
            B[eq] = -area * _1_dt * dens * pvx + area * _1_dt * dens * rcy * pvo
                  - area * dens * rcx * sqr(pvo) - (dens - 1.0) * S->grav_x * area;
            A[eq * n + BCOL(bi, 0)] = -area * _1_dt * dens;
            A[eq * n + BCOL(bi, 1)] = 0;
            A[eq * n + BCOL(bi, 2)] = area * _1_dt * dens * rcy;
            A[eq * n + BCOL(bi, 3)] = 1;
            A[eq * n + BCOL(bi, 6)] = -1;
        }
        /* fillNewtonYEquation (:669-702) */
        {
            int64_t eq = e0 + 7;
            B[eq] = -area * _1_dt * dens * pvy - area * _1_dt * dens * rcx * pvo
                  - area * dens * rcy * sqr(pvo) - (dens - 1.0) * S->grav_y * area;
            A[eq * n + BCOL(bi, 0)] = 0;
            A[eq * n + BCOL(bi, 1)] = -area * _1_dt * dens;
            A[eq * n + BCOL(bi, 2)] = -area * _1_dt * dens * rcx;
            A[eq * n + BCOL(bi, 4)] = 1;
            A[eq * n + BCOL(bi, 7)] = -1;
        }
        /* fillNewtonOEquation (:704-739) */
        {
            int64_t eq = e0 + 8;
            double rlx = -rcy, rly = rcx; /* rotl(r_c_com) */
            B[eq] = -area * _1_dt * dens * (rlx * pvx + rly * pvy) - moi * _1_dt * dens * pvo
                  - (dens - 1.0) * (rlx * S->grav_x + rly * S->grav_y) * area;
            A[eq * n + BCOL(bi, 0)] = +area * _1_dt * dens * rcy;
            A[eq * n + BCOL(bi, 1)] = -area * _1_dt * dens * rcx;
            A[eq * n + BCOL(bi, 2)] = -moi * _1_dt * dens;
            A[eq * n + BCOL(bi, 5)] = 1;
            A[eq * n + BCOL(bi, 8)] = -1;
        }
    }
    /* solve on a copy so the filled system stays exportable */
    double* LU = (double*)xrealloc(NULL, sizeof(double) * (size_t)(n * n));
    memcpy(LU, A, sizeof(double) * (size_t)(n * n));
    memcpy(S->sol, B, sizeof(double) * (size_t)n);
    int rc = lu_solve(n, LU, S->sol);
    free(LU);
    if (rc) { free(col0); free(leaf_pos); return rc; }
    for (int bi = 0; bi < S->nb; bi++) {
        const obody* b = &S->bodies[bi];
        for (int64_t q = 0; q < b->count; q++) S->sg[b->first + q] = S->sol[SEGCOL(bi, q)];
        const double* u = &S->sol[BCOL(bi, 0)];
        S->bodies[bi].p.speed_slae_x = u[0]; S->bodies[bi].p.speed_slae_y = u[1]; S->bodies[bi].p.speed_slae_o = u[2];
        if (out) {
            vvo_body_out* o = &out[bi];
            o->speed_slae_x = u[0]; o->speed_slae_y = u[1]; o->speed_slae_o = u[2];
            o->force_hydro_x = u[3]; o->force_hydro_y = u[4]; o->force_hydro_o = u[5];
            o->force_holder_x = u[6]; o->force_holder_y = u[7]; o->force_holder_o = u[8];
        }
    }
#undef SEGCOL
#undef BCOL
    free(col0);
    free(leaf_pos);
    return 0;
}

int vvo_set_sample(vvo_space* S, int64_t stride) {
    if (stride < 1) return -1;
    S->stride = stride;
    return 0;
}

/* The reference's steady-state SLAE work per step (time > 0, rigid bodies at rest): the
 * right-hand side of every slip row (fillSlipEquationForSegment with rightColOnly,
 * MConvectiveFast.cpp:459-467; rows sampled with the timing stride) followed by one dense
 * matrix-vector product with the cached inverse (cblas_dgemv, TMatrix.cpp:176-189). */
int vvo_slae_rhs_step(vvo_space* S, double* rhs_out) {
    if (!S->built) return -3;
    int64_t n = vvo_slae_size(S);
    double* inv = (double*)calloc((size_t)(n * n), sizeof(double));
    double* b = (double*)calloc((size_t)n, sizeof(double));
    double* y = (double*)calloc((size_t)n, sizeof(double));
    if (!inv || !b || !y) { free(inv); free(b); free(y); return -7; }
    for (int64_t i = 0; i < n; i++) inv[i * n + i] = 1.0;
    /* node -> leaf position (the reference's findNode returns the leaf itself) */
    int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (size_t)(S->nnodes ? S->nnodes : 1));
    if (!pos) { free(inv); free(b); free(y); return -7; }
    for (int64_t t = 0; t < S->nleaves; t++) pos[S->leaves[t]] = t;
    int64_t row = 0;
    for (int bi = 0; bi < S->nb; bi++) {
        const obody* bd = &S->bodies[bi];
        for (int64_t k = 0; k < bd->count; k++, row++) {
            if (k == bd->p.special_segment_no || (k % S->stride)) continue;
            int64_t s = bd->first + k;
            double r = (-S->inf_vy) * S->dlx[s] + S->inf_vx * S->dly[s];
            int32_t nk = find_node(S, S->rx[s], S->ry[s]);
            r -= node_influence(S, pos[nk], s);
            b[row] = r;
        }
        row += 9;
    }
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) {
        double acc = 0;
        for (int64_t j = 0; j < n; j++) acc += inv[i * n + j] * b[j];
        y[i] = acc;
    }
    if (rhs_out) memcpy(rhs_out, y, sizeof(double) * (size_t)n);
    free(pos); free(inv); free(b); free(y);
    return 0;
}

int vvo_last_timings(const vvo_space* S, double* out3) {
    out3[0] = S->t_partition; out3[1] = S->t_cmass; out3[2] = S->t_lists;
    return 0;
}

int vvo_slae_export(const vvo_space* S, double* matrix, double* rhs, double* solution) {
    if (!S->neq) return -3;
    int64_t n = S->neq;
    if (matrix) memcpy(matrix, S->mat, sizeof(double) * (size_t)(n * n));
    if (rhs) memcpy(rhs, S->rhs, sizeof(double) * (size_t)n);
    if (solution) memcpy(solution, S->sol, sizeof(double) * (size_t)n);
    return 0;
}

/* TBody::isPointInvalid -> isPointInContour over the body's corners (TBody.cpp:217-280):
 * the bounding rectangle / disc of doFillProperties (TBody.cpp:327-342) as a pre-check
 * unless the body is inverted (area <= 0), then crossing-number parity, then the segment
 * whose centre is nearest (first minimum in list order).  Returns the global segment index
 * or -1. */
static int64_t point_invalid(const vvo_space* S, const obody* b, double px, double py) {
    const int64_t f = b->first, n = b->count;
    int in = (b->area <= 0);
    double r2max = 0, blx = INFINITY, bly = INFINITY, trx = -INFINITY, try_ = -INFINITY;
    for (int64_t k = 0; k < n; k++) {
        const double cx = S->cx[f + k], cy = S->cy[f + k];
        const double r2 = abs2(cx - b->cofm_x, cy - b->cofm_y);
        if (r2 > r2max) r2max = r2;
        if (cx > trx) trx = cx;
        if (cy > try_) try_ = cy;
        if (cx < blx) blx = cx;
        if (cy < bly) bly = cy;
    }
    if (!in && (px < blx || py < bly || px > trx || py > try_ || abs2(px - b->cofm_x, py - b->cofm_y) > r2max))
        return -1;
    for (int64_t i = 0, j = n - 1; i < n; j = i++) {
        const double vix = S->cx[f + i], viy = S->cy[f + i], vjx = S->cx[f + j], vjy = S->cy[f + j];
        if (((viy < vjy) && (viy < py) && (py <= vjy) && ((vjy - viy) * (px - vix) > (vjx - vix) * (py - viy))) ||
            ((viy > vjy) && (viy > py) && (py >= vjy) && ((vjy - viy) * (px - vix) < (vjx - vix) * (py - viy))))
            in = !in;
    }
    if (!in) return -1;
    int64_t best = -1;
    double bd = DBL_MAX;
    for (int64_t k = 0; k < n; k++) {
        const double d = abs2(S->rx[f + k] - px, S->ry[f + k] - py);
        if (d < bd) { bd = d; best = f + k; }
    }
    return best;
}

/* MFlowmove::move_and_clean (MFlowmove.cpp:11-215) for rigid bodies at rest: with no
 * spring there is no collision (current_dt = dt) and the bodies do not move (a SLAE speed
 * below 1e-10, the solver's round-off of zero, is not applied), so only the vortex part and
 * the bookkeeping remain.  The order of every FP64 accumulation follows
 * the reference (list order for the removed vortices, body and segment order after). */
int vvo_move_and_clean(vvo_space* S, int remove, int64_t* cleaned) {
    if (S->built) return -2;
    for (int bi = 0; bi < S->nb; bi++) {
        const vvo_body_params* p = &S->bodies[bi].p;
        if (!is_rigid(p->kspring_x) || !is_rigid(p->kspring_y) || !is_rigid(p->kspring_o)) return -4;
        if (p->speed_x != 0 || p->speed_y != 0 || p->speed_o != 0 ||
            !(fabs(p->speed_slae_x) + fabs(p->speed_slae_y) + fabs(p->speed_slae_o) < 1E-10))
            return -4;
    }
    const double dt = S->dt;
    int64_t nc = 0;
    /* r += v * dt (MFlowmove.cpp:104) */
    for (int64_t i = 0; i < S->n; i++) {
        S->x[i] = S->x[i] + S->vx[i] * dt;
        S->y[i] = S->y[i] + S->vy[i] * dt;
    }
    /* erase |g| < remove_eps (:110-114), keeping the order */
    int64_t w = 0;
    for (int64_t i = 0; i < S->n; i++) {
        if (fabs(S->g[i]) < REMOVE_EPS) continue;
        S->x[w] = S->x[i]; S->y[w] = S->y[i]; S->g[w] = S->g[i]; S->ie[w] = S->ie[i];
        S->vx[w] = S->vx[i]; S->vy[w] = S->vy[i]; S->orig[w] = S->orig[i];
        w++;
    }
    S->n = w;
    if (remove) {
        /* erase vortices inside a body, with the dead-vortex bookkeeping (:121-143) */
        w = 0;
        for (int64_t i = 0; i < S->n; i++) {
            int64_t seg = -1;
            int bad = -1;
            for (int bi = 0; bi < S->nb; bi++) {
                seg = point_invalid(S, &S->bodies[bi], S->x[i], S->y[i]);
                if (seg >= 0) { bad = bi; break; }
            }
            if (bad < 0) {
                S->x[w] = S->x[i]; S->y[w] = S->y[i]; S->g[w] = S->g[i]; S->ie[w] = S->ie[i];
                S->vx[w] = S->vx[i]; S->vy[w] = S->vy[i]; S->orig[w] = S->orig[i];
                w++;
                continue;
            }
            vvo_body_params* p = &S->bodies[bad].p;
            const double gi = S->g[i], px = S->x[i], py = S->y[i];
            p->fdt_dead_x += (-py) * gi;
            p->fdt_dead_y += px * gi;
            p->fdt_dead_o += abs2(px - body_axis_x(&S->bodies[bad]), py - body_axis_y(&S->bodies[bad])) * gi;
            S->gsum[seg] -= gi;
            p->g_dead += gi;
            nc++;
        }
        S->n = w;
    }
    /* v = 0 (:192-197) */
    for (int64_t i = 0; i < S->n; i++) { S->vx[i] = 0; S->vy[i] = 0; }
    /* dead segments: |g| < remove_eps or slip (:199-214) */
    for (int bi = 0; bi < S->nb; bi++) {
        obody* b = &S->bodies[bi];
        const double ax = body_axis_x(b), ay = body_axis_y(b);
        for (int64_t k = 0; k < b->count; k++) {
            const int64_t s = b->first + k;
            if (fabs(S->sg[s]) < REMOVE_EPS || S->slip[s]) {
                const double gs = S->sg[s];
                b->p.fdt_dead_x += (-S->cy[s]) * gs;
                b->p.fdt_dead_y += S->cx[s] * gs;
                b->p.fdt_dead_o += abs2(S->cx[s] - ax, S->cy[s] - ay) * gs;
                S->gsum[s] -= gs;
                b->p.g_dead += gs;
            }
        }
    }
    if (cleaned) *cleaned = nc;
    return 0;
}

int vvo_set_segment_state(vvo_space* S, const double* g, const double* fric, const double* gsum) {
    for (int64_t i = 0; i < S->m; i++) {
        if (g) S->sg[i] = g[i];
        if (fric) S->fric[i] = fric[i];
        if (gsum) S->gsum[i] = gsum[i];
    }
    return 0;
}

/* Space::calc_forces (TSpace.cpp:94-117).  No heat here: hsum = 0 and Space::pr = 0, the
 * reference's defaults, are kept in the formulas so that Nu and nusselt match it. */
int vvo_calc_forces(vvo_space* S, double* out4) {
    const double pr = 0., hsum = 0.;
    const double c_nyudt_pi = S->dt / (C_PI * S->re);
    const double c_nyu_pi = 1. / (C_PI * S->re);
    for (int bi = 0; bi < S->nb; bi++) {
        obody* b = &S->bodies[bi];
        double tmp_gsum = 0;
        b->friction_x = b->friction_y = b->friction_o = 0;
        for (int64_t k = 0; k < b->count; k++) {
            const int64_t s = b->first + k;
            const double dlabs = sqrt(abs2(S->dlx[s], S->dly[s]));
            tmp_gsum += S->gsum[s];
            S->cp[s] += tmp_gsum;
            S->fr[s] += S->fric[s] * c_nyudt_pi;
            S->nu[s] += hsum * (S->re * pr / dlabs);
            const double f = S->fric[s] * c_nyu_pi / dlabs;
            b->friction_x -= S->dlx[s] * f;
            b->friction_y -= S->dly[s] * f;
            b->friction_o -= ((-S->ry[s]) * S->dlx[s] + S->rx[s] * S->dly[s]) * f;
            b->nusselt += hsum * (S->re * pr);
        }
        b->nusselt /= S->dt;
        if (out4) {
            out4[4 * bi + 0] = b->friction_x; out4[4 * bi + 1] = b->friction_y;
            out4[4 * bi + 2] = b->friction_o; out4[4 * bi + 3] = b->nusselt;
        }
    }
    return 0;
}

/* Space::zero_forces (TSpace.cpp:122-142); force_hydro/force_holder are not kept here. */
int vvo_zero_forces(vvo_space* S) {
    for (int bi = 0; bi < S->nb; bi++) {
        obody* b = &S->bodies[bi];
        for (int64_t k = 0; k < b->count; k++) {
            const int64_t s = b->first + k;
            S->gsum[s] = 0; S->fric[s] = 0;
        }
        b->p.friction_prev_x = b->friction_x;
        b->p.friction_prev_y = b->friction_y;
        b->p.friction_prev_o = b->friction_o;
        b->friction_x = b->friction_y = b->friction_o = 0;
        b->p.fdt_dead_x = b->p.fdt_dead_y = b->p.fdt_dead_o = 0;
        b->p.g_dead = 0;
        b->nusselt = 0;
    }
    return 0;
}

int vvo_get_segment_forces(const vvo_space* S, double* cp, double* fr, double* nu) {
    for (int64_t i = 0; i < S->m; i++) {
        if (cp) cp[i] = S->cp[i];
        if (fr) fr[i] = S->fr[i];
        if (nu) nu[i] = S->nu[i];
    }
    return 0;
}

int vvo_set_velocities(vvo_space* S, const double* vx, const double* vy) {
    for (int64_t i = 0; i < S->n; i++) { S->vx[i] = vx[i]; S->vy[i] = vy[i]; }
    return 0;
}

int vvo_get_body_params(const vvo_space* S, int b, vvo_body_params* out) {
    if (b < 0 || b >= S->nb || !out) return -1;
    *out = S->bodies[b].p;
    return 0;
}

/* MFlowmove::vortex_shed (MFlowmove.cpp:217-235). */
int vvo_vortex_shed(vvo_space* S) {
    if (S->built) return -2;
    int64_t add = 0;
    for (int64_t s = 0; s < S->m; s++) if (fabs(S->sg[s]) >= REMOVE_EPS && !S->slip[s]) add++;
    vort_reserve(S, S->n + add);
    for (int64_t s = 0; s < S->m; s++) {
        S->gsum[s] += S->sg[s];
        if (fabs(S->sg[s]) >= REMOVE_EPS && !S->slip[s]) {
            int64_t i = S->n++;
            S->x[i] = S->cx[s] + (-S->dly[s]) * 1e-4;
            S->y[i] = S->cy[s] + S->dlx[s] * 1e-4;
            S->g[i] = S->sg[s]; S->ie[i] = 0; S->vx[i] = 0; S->vy[i] = 0;
            S->orig[i] = i;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Grid fields (libvvhd/src/XVelocity.cpp, XStreamfunction.cpp, XVorticity.cpp)          */
/* ------------------------------------------------------------------------------------ */

/* The reference evaluates every field on a private copy of Space (XVelocity.hpp:23 and
 * the others); the copy's vortex list, epsilon and attached-segment sums are saved here
 * and put back afterwards. */
typedef struct {
    int64_t n;
    double *x, *y, *g, *ie, *vx, *vy, *gsum;
    int64_t* orig;
} osnap;

static double* dup_d(const double* a, int64_t n) {
    double* r = (double*)xrealloc(NULL, sizeof(double) * (size_t)(n ? n : 1));
    if (n) memcpy(r, a, sizeof(double) * (size_t)n);
    return r;
}

static void snap_save(const vvo_space* S, osnap* q) {
    q->n = S->n;
    q->x = dup_d(S->x, S->n); q->y = dup_d(S->y, S->n); q->g = dup_d(S->g, S->n);
    q->ie = dup_d(S->ie, S->n); q->vx = dup_d(S->vx, S->n); q->vy = dup_d(S->vy, S->n);
    q->orig = (int64_t*)xrealloc(NULL, sizeof(int64_t) * (size_t)(S->n ? S->n : 1));
    if (S->n) memcpy(q->orig, S->orig, sizeof(int64_t) * (size_t)S->n);
    q->gsum = dup_d(S->gsum, S->m);
}

static void snap_restore(vvo_space* S, osnap* q) {
    free_tree(S);
    S->n = q->n;
    size_t d = sizeof(double) * (size_t)q->n;
    if (q->n) {
        memcpy(S->x, q->x, d); memcpy(S->y, q->y, d); memcpy(S->g, q->g, d);
        memcpy(S->ie, q->ie, d); memcpy(S->vx, q->vx, d); memcpy(S->vy, q->vy, d);
        memcpy(S->orig, q->orig, sizeof(int64_t) * (size_t)q->n);
    }
    if (S->m) memcpy(S->gsum, q->gsum, sizeof(double) * (size_t)S->m);
    free(q->x); free(q->y); free(q->g); free(q->ie); free(q->vx); free(q->vy); free(q->orig); free(q->gsum);
}

/* Space::average_segment_length (TSpace.hpp:119-129): of the first body. */
static double avg_seg_len(const vvo_space* S) {
    if (!S->nb) return 0;
    const obody* b = &S->bodies[0];
    if (b->count <= 1) return 0;
    return b->slen / (double)(b->count - 1);
}

/* XField::XField (XField.cpp:8-24): the grid origin and spacing are stored as float. */
static int field_grid(double xmin, double ymin, double dxdy, int32_t xres, int32_t yres, float* fx, float* fy,
                      float* fd) {
    *fx = (float)xmin; *fy = (float)ymin; *fd = (float)dxdy;
    if (xres <= 1 || yres <= 1) return 0;
    if (!isfinite(*fd) || *fd <= 0) return 0;
    return 1;
}

/* leaf index (DFS) of every node id that is a leaf */
static int32_t* leaf_pos(const vvo_space* S) {
    int32_t* pos = (int32_t*)xrealloc(NULL, sizeof(int32_t) * (size_t)(S->nnodes ? S->nnodes : 1));
    for (int64_t L = 0; L < S->nleaves; L++) pos[S->leaves[L]] = (int32_t)L;
    return pos;
}

/* MEpsilonFast::eps2h (MEpsilonFast.cpp:66-92): squared distance to the second nearest
 * vortex (any circulation, coincident points skipped) over the near leaves of leaf L. */
static double eps2h(const vvo_space* S, int64_t L, double px, double py) {
    double res1 = INFINITY, res2 = INFINITY;
    for (int64_t t = S->near_off[L]; t < S->near_off[L + 1]; t++) {
        const onode* nn = &S->nodes[S->near_list[t]];
        for (int64_t j = nn->vf; j < nn->vl; j++) {
            const double d = abs2(px - S->x[j], py - S->y[j]);
            if (!d) continue;
            else if (d < res1) { res2 = res1; res1 = d; }
            else if (d < res2) res2 = d;
        }
    }
    if (isfinite(res2)) return res2;
    if (isfinite(res1)) return res1;
    return -DBL_MAX;
}

static int ref_speed(const vvo_space* S, char ref_frame, double* rx, double* ry) {
    switch (ref_frame) {
    case 'o': *rx = 0; *ry = 0; return 1;
    case 'f': *rx = S->inf_vx; *ry = S->inf_vy; return 1;
    case 'b':
        if (!S->nb) return 0;
        *rx = S->bodies[0].p.speed_slae_x; *ry = S->bodies[0].p.speed_slae_y;
        return 1;
    default: return 0;
    }
}

/* XVelocity::evaluate (XVelocity.cpp:24-73): tree (8, 20 dl, 0.1), epsilon without merging,
 * then MConvectiveFast::velocity at every node of the grid minus the frame speed. */
int vvo_field_velocity(vvo_space* S, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                       char mode, char ref_frame, float* out) {
    float fx, fy, fd;
    if (!field_grid(xmin, ymin, dxdy, xres, yres, &fx, &fy, &fd)) return -1;
    double rfx, rfy;
    if (!ref_speed(S, ref_frame, &rfx, &rfy)) return -1;
    if (mode != 'x' && mode != 'y') return -1;
    if (S->built) return -2;
    if (!bodies_at_rest(S)) return -4;
    osnap q;
    snap_save(S, &q);
    const double dl = avg_seg_len(S);
    int rc = vvo_tree_build(S, 8, dl * 20, 0.1);
    int64_t merged;
    if (!rc) rc = vvo_eps(S, 0, &merged);
    if (!rc) {
        const int64_t np = (int64_t)xres * yres;
        double* px = (double*)xrealloc(NULL, sizeof(double) * 4 * (size_t)np);
        double *py = px + np, *vx = px + 2 * np, *vy = px + 3 * np;
        for (int32_t yj = 0; yj < yres; yj++)
            for (int32_t xi = 0; xi < xres; xi++) {
                px[(int64_t)yj * xres + xi] = (double)fx + (double)fd * xi;
                py[(int64_t)yj * xres + xi] = (double)fy + (double)fd * yj;
            }
        rc = vvo_velocity_points(S, np, px, py, vx, vy);
        for (int64_t k = 0; !rc && k < np; k++) out[k] = (float)(mode == 'x' ? vx[k] - rfx : vy[k] - rfy);
        free(px);
    }
    snap_restore(S, &q);
    return rc;
}

/* XStreamfunction::evaluate and streamfunction(node, p, gap) (XStreamfunction.cpp:47-212):
 * tree (8, 10 dl, 20 dl); every vortex gets eps^2 = eps_mult^2 max(eps2h / 4, (0.2 dl)^2);
 * psi = [sum over segments, far-node centroids and near vortices of -g log(r^2 + e^2)] / 4pi
 * + [sum over sinks of q atan2] / 2pi + p . rotl(V_inf - V_frame).  Sinks inside the cell
 * (p, p + dxdy] give gap entries, in grid order. */
int vvo_field_streamfunction(vvo_space* S, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                             double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                             uint16_t* gap_yj, float* gap, int64_t* ngaps) {
    float fx, fy, fd;
    if (!field_grid(xmin, ymin, dxdy, xres, yres, &fx, &fy, &fd)) return -1;
    if (eps_mult <= 0) return -1;
    double rfx, rfy;
    if (!ref_speed(S, ref_frame, &rfx, &rfy)) return -1;
    if (S->built) return -2;
    if (!bodies_at_rest(S)) return -4;
    osnap q;
    snap_save(S, &q);
    const double dl = avg_seg_len(S);
    const double rd2 = sqr(0.2 * dl);
    int rc = vvo_tree_build(S, 8, dl > 0 ? dl * 10 : 0, dl > 0 ? dl * 20 : INFINITY);
    int64_t ng = 0;
    if (!rc) {
        double* e2 = (double*)xrealloc(NULL, sizeof(double) * (size_t)(S->n ? S->n : 1));
        for (int64_t L = 0; L < S->nleaves; L++) {
            const onode* nd = &S->nodes[S->leaves[L]];
            for (int64_t i = nd->vf; i < nd->vl; i++)
                e2[i] = sqr(eps_mult) * smax(eps2h(S, L, S->x[i], S->y[i]) * 0.25, sqr(0.2 * dl));
        }
        int32_t* pos = leaf_pos(S);
        const double vfx = S->inf_vx - rfx, vfy = S->inf_vy - rfy;
        for (int32_t yj = 0; yj < yres; yj++)
            for (int32_t xi = 0; xi < xres; xi++) {
                const double px = (double)fx + (double)fd * xi, py = (double)fy + (double)fd * yj;
                const int64_t L = pos[find_node(S, px, py)];
                double t4 = 0, t2 = 0, pgap = 0;
                for (int64_t s = 0; s < S->m; s++) t4 += -S->sg[s] * log(abs2(px - S->rx[s], py - S->ry[s]) + rd2);
                for (int64_t s = 0; s < S->ns; s++) {
                    t2 += S->snk_g[s] * atan2(py - S->snk_y[s], px - S->snk_x[s]);
                    if (px < S->snk_x[s] && S->snk_x[s] <= px + (double)fd && py < S->snk_y[s] &&
                        S->snk_y[s] <= py + (double)fd)
                        pgap += S->snk_g[s];
                }
                for (int64_t t = S->far_off[L]; t < S->far_off[L + 1]; t++) {
                    const onode* fn = &S->nodes[S->far_list[t]];
                    t4 += -fn->cmp_g * log(abs2(px - fn->cmp_x, py - fn->cmp_y) + rd2);
                    t4 += -fn->cmm_g * log(abs2(px - fn->cmm_x, py - fn->cmm_y) + rd2);
                }
                for (int64_t t = S->near_off[L]; t < S->near_off[L + 1]; t++) {
                    const onode* nn = &S->nodes[S->near_list[t]];
                    for (int64_t j = nn->vf; j < nn->vl; j++)
                        t4 += -S->g[j] * log(abs2(px - S->x[j], py - S->y[j]) + e2[j]);
                }
                out[(int64_t)yj * xres + xi] = (float)(t4 * C_1_4PI + t2 * C_1_2PI + (px * (-vfy) + py * vfx));
                if (pgap) {
                    if (ng < gap_cap) {
                        gap_xi[ng] = (uint16_t)xi; gap_yj[ng] = (uint16_t)yj; gap[ng] = (float)pgap;
                    }
                    ng++;
                }
            }
        free(pos);
        free(e2);
    }
    if (ngaps) *ngaps = ng;
    snap_restore(S, &q);
    return rc;
}

/* XVorticity::evaluate and vorticity(node, p) (XVorticity.cpp:26-94): vortex_shed, tree
 * (8, 20 dl, DBL_MAX); every vortex gets a = 1 / (eps_mult^2 max(eps2h, (0.6 dl)^2));
 * omega = 0 inside a body, else [sum over near vortices of g a exp(-a r^2), cut at
 * -a r^2 <= -6] / pi + (erfarg < 3 ? (1 - erf(erfarg)) / 2 : 0) with erfarg = (squared
 * distance to the nearest segment centre of the near leaves) / (dl eps_mult)^2. */
int vvo_field_vorticity(vvo_space* S, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                        double eps_mult, float* out) {
    float fx, fy, fd;
    if (!field_grid(xmin, ymin, dxdy, xres, yres, &fx, &fy, &fd)) return -1;
    if (eps_mult <= 0) return -1;
    if (S->built) return -2;
    if (!bodies_at_rest(S)) return -4;
    osnap q;
    snap_save(S, &q);
    const double dl = avg_seg_len(S);
    int rc = vvo_vortex_shed(S);
    if (!rc) rc = vvo_tree_build(S, 8, dl * 20, DBL_MAX);
    if (!rc) {
        double* a = (double*)xrealloc(NULL, sizeof(double) * 2 * (size_t)(S->n ? S->n : 1));
        double* ag = a + S->n;
        for (int64_t L = 0; L < S->nleaves; L++) {
            const onode* nd = &S->nodes[S->leaves[L]];
            for (int64_t i = nd->vf; i < nd->vl; i++) {
                a[i] = 1. / (sqr(eps_mult) * smax(eps2h(S, L, S->x[i], S->y[i]), sqr(0.6 * dl)));
                ag[i] = a[i] * S->g[i];
            }
        }
        int32_t* pos = leaf_pos(S);
        const double e2 = sqr(dl * eps_mult);
        for (int32_t yj = 0; yj < yres; yj++)
            for (int32_t xi = 0; xi < xres; xi++) {
                const double px = (double)fx + (double)fd * xi, py = (double)fy + (double)fd * yj;
                int inside = 0;
                for (int b = 0; b < S->nb && !inside; b++) inside = point_invalid(S, &S->bodies[b], px, py) >= 0;
                double res = 0;
                if (!inside) {
                    const int64_t L = pos[find_node(S, px, py)];
                    double h2 = INFINITY;
                    for (int64_t t = S->near_off[L]; t < S->near_off[L + 1]; t++) {
                        const onode* nn = &S->nodes[S->near_list[t]];
                        for (int64_t j = nn->vf; j < nn->vl; j++) {
                            const double exparg = -abs2(px - S->x[j], py - S->y[j]) * a[j];
                            res += (exparg > -6) ? ag[j] * exp(exparg) : 0;
                        }
                    }
                    res *= C_1_PI;
                    for (int64_t t = S->near_off[L]; t < S->near_off[L + 1]; t++) {
                        const onode* nn = &S->nodes[S->near_list[t]];
                        for (int64_t k = nn->sf; k < nn->sl; k++) {
                            const int64_t sg = S->seg_order[k];
                            h2 = smin(h2, abs2(px - S->rx[sg], py - S->ry[sg]));
                        }
                    }
                    const double erfarg = h2 / e2;
                    res += (erfarg < 3) ? 0.5 * (1 - erf(erfarg)) : 0;
                }
                out[(int64_t)yj * xres + xi] = (float)res;
            }
        free(pos);
        free(a);
    }
    snap_restore(S, &q);
    return rc;
}
