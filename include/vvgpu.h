/*
 * vvgpu.h -- C ABI of the GB300 implementation of libvvhd's per-step velocity path.
 *
 * One context = one Space (vortices + bodies) resident in device memory, one CUDA
 * stream.  The calls replace the reference's hot-path classes one for one:
 *
 *   vvgpu_tree_build / vvgpu_tree_destroy  <- stree::build / stree::destroy
 *                                             (libvvhd/headers/TSortedTree.hpp:74-75,
 *                                              libvvhd/src/TSortedTree.cpp:232-265, 267-273)
 *   vvgpu_eps                              <- MEpsilonFast::CalcEpsilonFast(bool merge),
 *                                             MEpsilonFast::Merged()
 *                                             (libvvhd/headers/MEpsilonFast.hpp:10-11,
 *                                              libvvhd/src/MEpsilonFast.cpp:11-63)
 *   vvgpu_convective                       <- MConvectiveFast::process_all_lists()
 *                                             (libvvhd/headers/MConvectiveFast.hpp:16,
 *                                              libvvhd/src/MConvectiveFast.cpp:36-114)
 *   vvgpu_velocity_points                  <- MConvectiveFast::velocity(TVec p)
 *                                             (libvvhd/headers/MConvectiveFast.hpp:17,
 *                                              libvvhd/src/MConvectiveFast.cpp:20-34)
 *   vvgpu_slae                             <- MConvectiveFast::calc_circulation(const void**)
 *                                             (libvvhd/headers/MConvectiveFast.hpp:18-26,
 *                                              libvvhd/src/MConvectiveFast.cpp:235-273)
 *   vvgpu_diffusive                        <- MDiffusiveFast::process_vort_list()
 *                                             (libvvhd/headers/MDiffusiveFast.hpp:10,
 *                                              libvvhd/src/MDiffusiveFast.cpp:8-48)
 *   vvgpu_vortex_shed                      <- MFlowmove::vortex_shed()
 *   vvgpu_move_and_clean                   <- MFlowmove::move_and_clean()
 *   vvgpu_calc_forces, vvgpu_zero_forces   <- Space::calc_forces(), Space::zero_forces()
 *                                             (libvvhd/headers/MFlowmove.hpp:12,
 *                                              libvvhd/src/MFlowmove.cpp:217-235)
 *   vvgpu_gsum                             <- Space::gsum() (libvvhd/headers/TSpace.hpp:93-99)
 *   vvgpu_field_velocity, _streamfunction, <- XVelocity, XStreamfunction, XVorticity:
 *   _vorticity                                constructor + mode/ref_frame/eps_mult +
 *                                             evaluate() + XField::map
 *                                             (libvvhd/headers/XVelocity.hpp:10-28,
 *                                              XStreamfunction.hpp:9-29, XVorticity.hpp:7-21)
 *
 * The Space state crosses the boundary as structure-of-arrays of doubles
 * (TObj r.x, r.y, g, _1_eps, v.x, v.y; libvvhd/headers/TObj.hpp:10-35) and body corners
 * (TAtt::corner; libvvhd/headers/TBody.hpp:17-55).  The tree permutes the vortex list in
 * place exactly as the reference does; vvgpu_get_vortices returns the permuted list and,
 * per slot, the index the vortex had when it was set.
 *
 * Errors: every call returns VVGPU_OK (0) or a negative VVGPU_ERR_* code and never exits;
 * vvgpu_last_error gives a message.  The reference reports the same conditions with
 * exit() / std::invalid_argument / stderr (libvvhd/src/TMatrix.cpp:60-61, 201-213,
 * libvvhd/src/MConvectiveFast.cpp:237-239, libvvhd/src/TSortedTree.cpp:234, 279-281).
 *
 * Threading: a context is used from one host thread at a time; all work is queued on the
 * context's stream and the calls that return results to host memory synchronise it.
 */
#ifndef VVGPU_H
#define VVGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    VVGPU_OK = 0,
    VVGPU_ERR_ARG = -1,          /* invalid argument                                     */
    VVGPU_ERR_STATE = -2,        /* wrong call order (e.g. tree already built)            */
    VVGPU_ERR_NOT_BUILT = -3,    /* tree not built                                       */
    VVGPU_ERR_UNSUPPORTED = -4,  /* body kinematics outside this implementation's scope  */
    VVGPU_ERR_SINGULAR = -5,     /* singular SLAE (zero pivot)                           */
    VVGPU_ERR_CUDA = -6,         /* CUDA runtime error                                   */
    VVGPU_ERR_NOMEM = -7,        /* device allocation failed                             */
    VVGPU_ERR_TIMEOUT = -8,      /* an iterative pass did not converge in its bound      */
    VVGPU_ERR_LIMIT = -9         /* size beyond a documented limit                       */
};

/* Arithmetic used for the pairwise sums (convective near/far field, diffusive).
 * Tree decisions, epsilon/merge, the SLAE and circulation totals are FP64 in both. */
enum { VVGPU_FP64 = 0, VVGPU_FP32 = 1 };

typedef struct vvgpu_ctx vvgpu_ctx;

typedef struct vvgpu_cfg {
    int device;                 /* CUDA device ordinal                                  */
    int precision;              /* VVGPU_FP64 or VVGPU_FP32                              */
    int64_t reserve_vortices;   /* optional capacity hint                               */
    int64_t reserve_segments;   /* optional capacity hint                               */
} vvgpu_cfg;

/* Rigid-body parameters (TBody fields, libvvhd/headers/TBody.hpp:57-158); time functions
 * (speed_x/y/o) are passed evaluated at the current time.  Same layout as the oracle's. */
typedef struct vvgpu_body_params {
    double holder_x, holder_y, holder_o;
    double dpos_x, dpos_y, dpos_o;
    double speed_x, speed_y, speed_o;
    double speed_slae_x, speed_slae_y, speed_slae_o;
    double speed_slae_prev_x, speed_slae_prev_y, speed_slae_prev_o;
    double friction_prev_x, friction_prev_y, friction_prev_o;
    double fdt_dead_x, fdt_dead_y, fdt_dead_o;
    double g_dead;
    double density;
    double kspring_x, kspring_y, kspring_o;
    int32_t special_segment_no;
    int32_t bc_kutta;
} vvgpu_body_params;

/* SLAE outputs per body (TBody::speed_slae, force_hydro, force_holder). */
typedef struct vvgpu_body_out {
    double speed_slae_x, speed_slae_y, speed_slae_o;
    double force_hydro_x, force_hydro_y, force_hydro_o;
    double force_holder_x, force_holder_y, force_holder_o;
} vvgpu_body_out;

/* Per-call counters of the last step's work (algorithmic, counted from the built tree). */
typedef struct vvgpu_stats {
    int64_t n_vortices, n_segments, n_nodes, n_leaves, tree_depth;
    int64_t near_pairs;         /* sum over leaves |L| * sum over near leaves |N|        */
    int64_t far_pairs;          /* sum over leaves |Far(L)| (two monopoles each)         */
    int64_t near_runs;          /* near lists stored as runs of consecutive leaves       */
    int64_t merge_rounds;       /* fixed-point rounds of the last epsilon pass           */
    int64_t merged;             /* merges in the last epsilon pass                       */
    int64_t diff_candidates;    /* vortex pairs inside the 8-eps cut-off boxes           */
    int64_t reserved[8];        /* reserved[0]: kernels launched by the context so far;
                                   reserved[1]: target evaluations over all epsilon rounds;
                                   reserved[2]: sources in the candidate leaves of every
                                   8-target chunk of the last FP32 diffusive pass;
                                   reserved[3]: candidate records read by the FP32 filter
                                   of every epsilon evaluation of the last pass;
                                   reserved[4]: node records loaded by the warps of the
                                   last near/far walk (each shared by its 32 leaves) */
} vvgpu_stats;

/* Device time per kernel (vvgpu_get_kernel_timing slots): CUDA events recorded on the
 * context's stream around these launches while timing is on. */
enum {
    VVGPU_T_TREE_BUILD = 0,   /* vvgpu_tree_build, whole call                             */
    VVGPU_T_WALK = 1,         /* near/far walk with the far-field expansion (k_walk_warp)  */
    VVGPU_T_EPS_ROUND = 2,    /* epsilon/merge two-nearest searches, every round           */
    VVGPU_T_EPS_CAND = 3,     /* epsilon/merge candidate leaves, every round               */
    VVGPU_T_EPS_PASS = 4,     /* vvgpu_eps after the walk, whole pass                      */
    VVGPU_T_CONVECTIVE = 5,   /* convective near field and far-field application          */
    VVGPU_T_DIFFUSIVE = 6,    /* diffusive sums                                           */
    VVGPU_T_SLAE = 7,         /* vvgpu_slae, whole call                                   */
    VVGPU_T_LEARNED = 8,      /* learned far-field corrections (network and leaf sums)     */
    VVGPU_T_JUDGE = 9,        /* the judge's plain-tree velocities                         */
    VVGPU_T_COUNT = 10
};

/* ---- context --------------------------------------------------------------------- */
int vvgpu_ctx_create(const vvgpu_cfg* cfg, vvgpu_ctx** out);
int vvgpu_ctx_destroy(vvgpu_ctx* ctx);
const char* vvgpu_last_error(const vvgpu_ctx* ctx);
int vvgpu_set_precision(vvgpu_ctx* ctx, int precision);
/* Use the caller's CUDA stream (cudaStream_t passed as void*); NULL = context's own. */
int vvgpu_set_stream(vvgpu_ctx* ctx, void* stream);
int vvgpu_synchronize(vvgpu_ctx* ctx);
int vvgpu_get_stats(const vvgpu_ctx* ctx, vvgpu_stats* out);
/* Largest number of fixed-point rounds vvgpu_eps may take (default 4096; the passes measured
 * take 5 to 7).  A pass that has not converged within it returns VVGPU_ERR_TIMEOUT and
 * leaves the vortex list as it was; the tree stays built.  The reference's sequential pass
 * has no such bound (MEpsilonFast.cpp:11-63). */
int vvgpu_set_eps_round_limit(vvgpu_ctx* ctx, int64_t max_rounds);
/* Polls of one shared-memory staging wait in the FP32 near field (bulk copies completing
 * on an mbarrier; default 4194304).  A wait that runs out makes the call return
 * VVGPU_ERR_TIMEOUT after its copies in flight have landed; the context stays usable
 * (0 polls: every wait runs out).  No counterpart in the reference (it has no GPU). */
int vvgpu_set_wait_limit(vvgpu_ctx* ctx, uint32_t spins);
/* Kernel shapes of the FP32 pair passes: sources per shared-memory tile of the convective
 * near field (128, 192 or 256; default 256) and the shape of the diffusive pass (1: up to
 * 16 targets of a leaf per pass, 2: up to 8; default 1).  The variants compute the same sums in a different order of their FP32
 * partial sums.  vvgpu_autotune_tiles times every shape on the context's current tree
 * (built; after vvgpu_eps, where the pass would run) and keeps the fastest of each; the
 * velocities and wall friction are left as they were.  ms (may be NULL) receives five
 * device times in ms (convective at 128, 192, 256; diffusive at shapes 1, 2; the best of
 * two runs each; -1 in an FP64 context, which has one shape).  vvgpu_set_autotune(ctx, 1)
 * tunes at the next vvgpu_convective instead (vvgpu_batch_autotune uses it for every
 * instance).  No counterpart in the reference (its OpenMP loops have no tile shapes). */
int vvgpu_autotune_tiles(vvgpu_ctx* ctx, int32_t* conv_tile, int32_t* diff_targets, double* ms);
int vvgpu_set_tiles(vvgpu_ctx* ctx, int32_t conv_tile, int32_t diff_targets);
int vvgpu_get_tiles(vvgpu_ctx* ctx, int32_t* conv_tile, int32_t* diff_targets);
int vvgpu_set_autotune(vvgpu_ctx* ctx, int on);
/* Kernel timing on (1) or off (0); either clears the sums.  No counterpart in the
 * reference (it has no GPU). */
int vvgpu_set_kernel_timing(vvgpu_ctx* ctx, int on);
/* Sums since timing was switched on: ms[k] device milliseconds and launches[k] timed
 * launches of slot k (arrays of VVGPU_T_COUNT; either may be NULL).  Synchronises. */
int vvgpu_get_kernel_timing(vvgpu_ctx* ctx, double* ms, int64_t* launches);

/* ---- Space state (host pointers) -------------------------------------------------- */
/* Space::re, dt, inf_speed(), inf_g, time, gravity (libvvhd/headers/TSpace.hpp:19-36). */
int vvgpu_set_params(vvgpu_ctx* ctx, double re, double dt, double inf_vx, double inf_vy,
                     double inf_g, double time, double gravity_x, double gravity_y);
/* Appends a body (TBody with alist corners in contour order; r, dl and _1_eps are derived
 * as in TBody::doUpdateSegments, libvvhd/src/TBody.cpp:200-215). */
int vvgpu_add_body(vvgpu_ctx* ctx, int64_t nseg, const double* corner_x, const double* corner_y,
                   const uint32_t* slip, const vvgpu_body_params* params);
int vvgpu_set_segment_g(vvgpu_ctx* ctx, const double* g);
/* Per-segment state TAtt::g, fric, gsum (any pointer may be NULL = keep). */
int vvgpu_set_segment_state(vvgpu_ctx* ctx, const double* g, const double* fric, const double* gsum);
/* Removes all bodies (before re-adding bodies whose geometry changed). */
int vvgpu_clear_bodies(vvgpu_ctx* ctx);
/* Updates the parameters of body b (time functions evaluated at the current time). */
int vvgpu_set_body_params(vvgpu_ctx* ctx, int body, const vvgpu_body_params* params);
int vvgpu_set_sinks(vvgpu_ctx* ctx, int64_t n, const double* x, const double* y, const double* g);
/* Replaces the vortex list (v = 0).  inv_eps may be NULL (= 0, a freshly loaded list).
 * The values are checked on the device: the next call that reads the list (tree build,
 * direct sum, move_and_clean) returns VVGPU_ERR_ARG if a position or circulation is not
 * finite or an inverse epsilon is NaN or negative (+inf, epsilon 0, is valid).  The
 * reference does not check and carries NaN through its sums. */
int vvgpu_set_vortices(vvgpu_ctx* ctx, int64_t n, const double* x, const double* y,
                       const double* g, const double* inv_eps);
/* Same with device pointers (data already resident in HBM on the context's device). */
int vvgpu_set_vortices_device(vvgpu_ctx* ctx, int64_t n, const double* x, const double* y,
                              const double* g, const double* inv_eps);
/* Sets TObj::v of the current list (the reference accumulates into v). */
int vvgpu_set_velocities(vvgpu_ctx* ctx, const double* vx, const double* vy);
int64_t vvgpu_num_vortices(const vvgpu_ctx* ctx);
int64_t vvgpu_num_segments(const vvgpu_ctx* ctx);
/* Copies the vortex list back to host memory; any pointer may be NULL. */
int vvgpu_get_vortices(vvgpu_ctx* ctx, double* x, double* y, double* g, double* inv_eps,
                       double* vx, double* vy, int64_t* orig);
/* Starts copying the vortex list's positions, circulations, inverse epsilons and origin
 * indices (as vvgpu_get_vortices; any pointer may be NULL) to host memory and returns
 * without waiting: the list is first copied on the device into a private snapshot, in
 * order on the context's stream, then to the host on a copy stream, so that the copies run
 * beside the context's later calls (after vvgpu_eps, the list does not change again in the
 * step: the convective and diffusive passes write only velocities and wall friction).  The
 * host arrays must stay valid, and must not be read, until vvgpu_wait_vortices returns;
 * with page-locked host memory the copies overlap the kernels.  The context's own small
 * device reads (counts, flags) share the copy engine and queue behind these copies, so a
 * caller starts them after vvgpu_convective (the diffusive pass reads only at its end).  A
 * second call first waits for the first.  The reference keeps the list in host memory (Space::VortexList); this is
 * the drop-in's return path for it after the epsilon pass. */
int vvgpu_get_vortices_async(vvgpu_ctx* ctx, double* x, double* y, double* g, double* inv_eps, int64_t* orig);
/* Waits for the download vvgpu_get_vortices_async started (returns at once without one). */
int vvgpu_wait_vortices(vvgpu_ctx* ctx);
/* Device pointers to the resident SoA arrays (valid until the next call that resizes). */
int vvgpu_device_arrays(vvgpu_ctx* ctx, double** x, double** y, double** g, double** inv_eps,
                        double** vx, double** vy);
int vvgpu_get_segments(vvgpu_ctx* ctx, double* rx, double* ry, double* dlx, double* dly,
                       double* inv_eps, double* g, double* fric, double* gsum);
int vvgpu_get_body_geom(vvgpu_ctx* ctx, int body, double* area, double* cofm_x, double* cofm_y,
                        double* moi_axis, double* slen);

/* ---- hot path --------------------------------------------------------------------- */
/* stree(S, farCriteria, minNodeSize, maxNodeSize).build(); far_criteria is a double here
 * (the reference takes an int; theta = sqrt(2 / far_criteria)).  The build makes the near
 * and far lists of the leaves holding a segment centre (all vvgpu_slae reads); the near
 * lists of the other leaves follow on the first call that needs them. */
int vvgpu_tree_build(vvgpu_ctx* ctx, double far_criteria, double min_node, double max_node);
int vvgpu_tree_destroy(vvgpu_ctx* ctx);
int vvgpu_eps(vvgpu_ctx* ctx, int merge, int64_t* merged);
/* Bodies whose speed_slae is not zero (vvgpu_slae's solution for a body in prescribed
 * translation, or vvgpu_set_body_params) carry the attached vortex and source sheets of
 * body_list_influence (MConvectiveFast.cpp:185-210, SegmentInfluence_linear_source
 * :440-457), rotation about holder + dpos included: in vvgpu_convective,
 * vvgpu_velocity_points and vvgpu_direct_velocity.  Like the reference, every target then
 * visits every segment of the moving bodies (FP64). */
int vvgpu_convective(vvgpu_ctx* ctx);
int vvgpu_diffusive(vvgpu_ctx* ctx);
int vvgpu_velocity_points(vvgpu_ctx* ctx, int64_t n, const double* px, const double* py,
                          double* vx, double* vy);
/* Same as vvgpu_velocity_points, for callers that must not allocate device memory (a fixed
 * device-memory budget, or probes that must not trigger the synchronisation cudaMalloc and
 * cudaFree imply).  It has no counterpart in the reference.  Points and results are staged
 * in one fixed device array of VVGPU_NOALLOC_MAX_POINTS points that every call shares: at
 * most that many points per call (VVGPU_ERR_LIMIT otherwise), and calls whose GPU work
 * overlaps race on the array.  The first call on each device looks the array's device
 * address up (cudaGetSymbolAddress).  It reads the near
 * lists of every leaf, which the tree builds on its first vvgpu_eps, vvgpu_convective,
 * vvgpu_diffusive or vvgpu_velocity_points call; before that it returns VVGPU_ERR_STATE. */
#define VVGPU_NOALLOC_MAX_POINTS 16384
int vvgpu_velocity_points_noalloc(vvgpu_ctx* ctx, int64_t n, const double* px, const double* py,
                                  double* vx, double* vy);
/* calc_circulation with no collision; rigid bodies at rest or in prescribed translation
 * are in scope (VVGPU_ERR_UNSUPPORTED otherwise).  The matrix and its inverse are refilled
 * only when an input of the cells changed (bodies added or cleared, body parameters, dt,
 * precision); otherwise only the right-hand side is filled, as the reference does once
 * its matrix and inverse are in place (MConvectiveFast.cpp:245-246).  The FP32 context
 * evaluates the right-hand side's tree sums in FP32 (cells stay FP64). */
int vvgpu_slae(vvgpu_ctx* ctx, vvgpu_body_out* out);
int vvgpu_vortex_shed(vvgpu_ctx* ctx);
/* MFlowmove::move_and_clean(remove, &collision, &cleaned) (libvvhd/src/MFlowmove.cpp:11-215)
 * for rigid bodies at rest (no collision): r += v dt, erasing |g| < 1e-10 and, with
 * remove != 0, the vortices inside a body with the dead-vortex bookkeeping (TBody::fdt_dead,
 * g_dead, TAtt::gsum), v = 0, and the dead-segment bookkeeping.  The list order is kept.
 * `cleaned` receives the number erased inside bodies.  Call with the tree destroyed. */
int vvgpu_move_and_clean(vvgpu_ctx* ctx, int remove, int64_t* cleaned);
/* Current TBody state of body `body` (g_dead and fdt_dead change in move_and_clean,
 * friction_prev in zero_forces). */
int vvgpu_get_body_params(vvgpu_ctx* ctx, int body, vvgpu_body_params* out);
/* Space::calc_forces (libvvhd/src/TSpace.cpp:94-117): adds to each segment's TAtt::Cp, Fr,
 * Nu and computes each body's friction and nusselt, written to out4[4 b .. 4 b + 3]
 * (friction x, y, o, nusselt; out4 may be NULL).  No heat: hsum = 0, Prandtl number 0. */
int vvgpu_calc_forces(vvgpu_ctx* ctx, double* out4);
/* Space::zero_forces (TSpace.cpp:122-142): TAtt::gsum = fric = 0; per body friction_prev =
 * friction, then friction, fdt_dead, g_dead and nusselt = 0. */
int vvgpu_zero_forces(vvgpu_ctx* ctx);
/* TAtt::Cp, Fr, Nu of every segment (the calc_forces accumulators). */
int vvgpu_get_segment_forces(vvgpu_ctx* ctx, double* cp, double* fr, double* nu);
int vvgpu_gsum(vvgpu_ctx* ctx, double* out);

/* FP64 direct sum (no tree) at n points: every vortex with its own epsilon (biot_savart,
 * MConvectiveFast.cpp:116-120) plus the sink, slip-segment and free-stream terms of
 * velocity(p).  The reference of the tree's own approximation error. */
int vvgpu_direct_velocity(vvgpu_ctx* ctx, int64_t n, const double* px, const double* py, double* vx, double* vy);

/* ---- batched sweep: many independent simulations advanced by one call ------------------ */
/* One simulate() step (utils/vvflow/vvflow.cpp:214-255: tree build, calc_circulation, tree
 * destroy, vortex_shed, tree build, CalcEpsilonFast(merge), process_all_lists,
 * process_vort_list, tree destroy), then, with move != 0, MFlowmove::move_and_clean(true). */
typedef struct vvgpu_step_cfg {
    double far_criteria, min_node, max_node;   /* stree(S, farCriteria, minNode, maxNode) */
    int32_t merge;                             /* CalcEpsilonFast(merge)                 */
    int32_t move;                              /* move_and_clean after the velocities    */
} vvgpu_step_cfg;
/* Advances each of count independent contexts by one step with cfgs[i]: a pool of nthreads
 * host threads (<= 0: one per host core) takes the instances largest first and drives each
 * on its own stream.  Each instance computes exactly what the same calls compute alone.
 * step_ms[i] (may be NULL) = instance i's wall time, its stream synchronised; status[i]
 * (may be NULL) = its return code.  Returns the first non-zero status, else 0. */
int vvgpu_batch_step(vvgpu_ctx* const* ctxs, int64_t count, const vvgpu_step_cfg* cfgs, int32_t nthreads,
                     double* step_ms, int32_t* status);
/* Tunes every instance's kernel shapes in its next step (vvgpu_set_autotune), then runs
 * one batched step per candidate pool size (these steps advance the instances) and returns
 * the fastest in *best (its wall time in *best_ms, may be NULL). */
int vvgpu_batch_autotune(vvgpu_ctx* const* ctxs, int64_t count, const vvgpu_step_cfg* cfgs,
                         const int32_t* candidates, int32_t ncand, int32_t* best, double* best_ms);

/* ---- learned far-field correction (no counterpart in the reference) ------------------- */
/* An MLP 20 -> 64 -> 64 -> 2 (tanh-GELU, BF16 weights and activations, FP32 accumulation on
 * the tensor cores) that predicts, for one far cell of the tree and one target point, the
 * residual of the cell's exact velocity beyond the reference's two-monopole far field
 * (MConvectiveFast.cpp:139-151).  Samples are (target, far cell) pairs of a built tree with
 * FP64 direct-sum labels.  Parameters: W1[64][32] (inputs 20..31 unused), b1[64],
 * W2[64][64], b2[64], W3[2][64], b3[2] as one float vector of vvgpu_mlp_num_params(). */
typedef struct vvgpu_mlp vvgpu_mlp;
int vvgpu_mlp_create(int device, uint64_t seed, vvgpu_mlp** out);
int vvgpu_mlp_destroy(vvgpu_mlp* m);
const char* vvgpu_mlp_last_error(const vvgpu_mlp* m);
/* Polls per tensor-core completion wait (default and largest 2^22).  A wait that runs out
 * makes the call return VVGPU_ERR_TIMEOUT; the kernel lets its MMA land and releases its
 * tensor memory first, so the model and the device stay usable.  0 makes every wait run
 * out at once (the time-out path, exercised without a fault). */
int vvgpu_mlp_set_wait_limit(vvgpu_mlp* m, int64_t spins);
int64_t vvgpu_mlp_num_params(void);
int vvgpu_mlp_get_params(vvgpu_mlp* m, float* out);
int vvgpu_mlp_set_params(vvgpu_mlp* m, const float* in);
/* standardisation, 42 floats: network input k = (feature k - norm[k]) * norm[20 + k], label o
 * = network output o * norm[40 + o] (default: identity); fit_norm sets it from the samples
 * (means, 1 / standard deviations, label root mean squares) */
int vvgpu_mlp_set_norm(vvgpu_mlp* m, const float* norm);
int vvgpu_mlp_get_norm(vvgpu_mlp* m, float* norm);
int vvgpu_mlp_fit_norm(vvgpu_mlp* m);
/* samples: features [n][20] and labels [n][2] (float) */
int vvgpu_mlp_set_samples(vvgpu_mlp* m, int64_t n, const float* feat, const float* lab);
int64_t vvgpu_mlp_num_samples(const vvgpu_mlp* m);
int vvgpu_mlp_get_samples(vvgpu_mlp* m, int64_t first, int64_t n, float* feat, float* lab);
/* appends the (target, far cell) pairs of np points in ctx's built tree, labelled by the
 * FP64 direct sum over each cell; *added = pairs appended */
int vvgpu_mlp_add_samples(vvgpu_mlp* m, vvgpu_ctx* ctx, int64_t np, const double* px, const double* py,
                          int64_t* added);
/* gradient (and loss) of (1/n) sum |y - t|^2 over the first n samples; weights unchanged */
int vvgpu_mlp_gradient(vvgpu_mlp* m, int64_t n, float* grad, float* loss);
/* Adam over all samples, mini-batches of `batch` (a multiple of 128), reshuffled each epoch */
int vvgpu_mlp_train(vvgpu_mlp* m, int64_t epochs, int64_t batch, float lr, uint64_t seed, float* loss_per_epoch);
int vvgpu_mlp_forward(vvgpu_mlp* m, int64_t n, const float* feat, float* y);
/* MConvectiveFast::velocity(p) of ctx's built tree plus the learned correction of each far
 * cell of p's leaf; *npairs = cells evaluated (may be NULL) */
int vvgpu_velocity_points_learned(vvgpu_ctx* ctx, vvgpu_mlp* m, int64_t np, const double* px, const double* py,
                                  double* vx, double* vy, int64_t* npairs);

/* The judge of the learned convective pass: velocity(p) of the plain tree (far criterion
 * far_criteria, e.g. 8 for theta 0.5) at `targets` vortices drawn per call from `seed` and
 * a call counter, against the learned pass's increments there.  gap = rms |learned -
 * plain| / rms |plain - free stream| over the drawn vortices with g != 0. */
typedef struct vvgpu_judge_cfg {
    int64_t targets;            /* vortices judged per call (0: no judge)                */
    double far_criteria;        /* the plain tree's far criterion                        */
    double bound;               /* largest gap accepted                                   */
    uint64_t seed;
} vvgpu_judge_cfg;
typedef struct vvgpu_judge_out {
    double gap_rms, gap_max;    /* gap (above) and the largest single gap, same scale     */
    int64_t pairs;              /* (leaf, far node) pairs the network corrected           */
    int64_t judged;             /* vortices judged (g != 0)                               */
    int32_t reverted;           /* 1: gap above the bound, the plain tree's pass was used */
    int32_t reserved;
} vvgpu_judge_out;
/* MConvectiveFast::process_all_lists (MConvectiveFast.cpp:36-114) with the learned far
 * field: for every (leaf, far node) pair of the built tree, the network's correction of the
 * node's monopole field at the leaf's centre is added to the leaf's constant far-field
 * terms, then the pass runs as vvgpu_convective.  judge (may be NULL: no judge) checks the
 * increments against the plain tree; above the bound they are undone and the pass is redone
 * with the plain tree at the judge's far criterion (the near lists then follow that
 * criterion until the tree is destroyed).  The tree's walk keeps every leaf's far nodes for
 * this; a tree built after vvgpu_keep_far_lists(ctx, 1) keeps them from its first walk,
 * otherwise the first call walks once more.  No counterpart in the reference. */
int vvgpu_convective_learned(vvgpu_ctx* ctx, vvgpu_mlp* m, const vvgpu_judge_cfg* judge, vvgpu_judge_out* out);
/* Makes the near/far walk of later trees keep every leaf's far nodes (on = 1). */
int vvgpu_keep_far_lists(vvgpu_ctx* ctx, int on);

/* ---- grid fields (libvvhd/src/XVelocity.cpp, XStreamfunction.cpp, XVorticity.cpp) ---- */
/* An xres x yres grid p = (xmin, ymin) + dxdy * (xi, yj), with xmin, ymin and dxdy rounded
 * to float as XField stores them (XField.hpp:47); out[yj * xres + xi] as XField::map.
 * The reference evaluates each field on a private copy of Space: the context's vortex
 * list, epsilon and segment gsum are left as they were.  No tree may be built on entry
 * (VVGPU_ERR_STATE) and none is left.  VVGPU_ERR_ARG where XField/X* throw
 * std::invalid_argument (xres or yres <= 1, dxdy not finite or <= 0, eps_mult <= 0, bad
 * mode or ref_frame), VVGPU_ERR_UNSUPPORTED for moving bodies.
 * velocity: tree (8, 20 dl, 0.1), epsilon without merging, then
 *   MConvectiveFast::velocity(p) - frame speed; mode 'x'|'y'; ref_frame 'o' (none),
 *   'f' (free stream), 'b' (first body's speed_slae).  dl = Space::average_segment_length().
 * streamfunction: tree (8, 10 dl, 20 dl); the grid cells (p, p + dxdy] that hold a sink are
 *   reported in grid order: at most gap_cap of them written to gap_xi/gap_yj/gap, their
 *   number in *ngaps (may be NULL).
 * vorticity: vortex_shed, tree (8, 20 dl); 0 inside a body. */
int vvgpu_field_velocity(vvgpu_ctx* ctx, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                         char mode, char ref_frame, float* out);
int vvgpu_field_streamfunction(vvgpu_ctx* ctx, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                               double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                               uint16_t* gap_yj, float* gap, int64_t* ngaps);
int vvgpu_field_vorticity(vvgpu_ctx* ctx, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                          double eps_mult, float* out);

/* ---- inspection (parity tests; same meaning as the oracle's exports) -------------- */
int vvgpu_tree_sizes(vvgpu_ctx* ctx, int64_t* nnodes, int64_t* nleaves, int64_t* nnear,
                     int64_t* nfar);
int vvgpu_tree_leaves(vvgpu_ctx* ctx, double* x, double* y, double* h, double* w,
                      int64_t* vfirst, int64_t* vlast, int32_t* depth, int64_t* path,
                      int64_t* sfirst, int64_t* slast);
int vvgpu_tree_nodes(vvgpu_ctx* ctx, double* x, double* y, double* h, double* w,
                     int64_t* vfirst, int64_t* vlast, int32_t* depth, int64_t* path,
                     double* cmp_x, double* cmp_y, double* cmp_g,
                     double* cmm_x, double* cmm_y, double* cmm_g);
int vvgpu_tree_seg_order(vvgpu_ctx* ctx, int64_t* seg_order);
int vvgpu_tree_lists(vvgpu_ctx* ctx, int64_t* near_off, int32_t* near_depth, int64_t* near_path,
                     int64_t* far_off, int32_t* far_depth, int64_t* far_path);
int64_t vvgpu_slae_size(const vvgpu_ctx* ctx);
int vvgpu_slae_export(vvgpu_ctx* ctx, double* matrix, double* rhs, double* solution);

#ifdef __cplusplus
}
#endif
#endif /* VVGPU_H */
