/*
 * vvd_oracle.h -- CPU oracle for the per-step Viscous Vortex Domains velocity path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a sequential FP64 restatement of the reference
 * libvvhd algorithms (bisection tree, convective Biot-Savart sum, body SLAE fill,
 * diffusive I0..I3 sums, epsilon/merge pass) written in plain C from reading
 * the libvvhd sources.  It is the checker for the CUDA path: only tests/, the smoke
 * entry point and the CPU-baseline leg of bench.py load it.  The product never
 * links it.
 *
 * Pinning: tests/test_oracle_pin.py compares every output of this restatement with
 * the reference's own sources compiled unmodified (oracle/Makefile -> oracle/_ref)
 * on seeded inputs, and with the golden fixtures in tests/golden/ that were produced
 * by that compiled reference.
 *
 * Arithmetic is written operation by operation in the same order as the reference
 * and compiled with -ffp-contract=off, so tree geometry, permutation, neighbour lists,
 * epsilon and merges are bit-identical to the reference on IEEE-754 hosts.
 *
 * The same entry points exist with the prefix vvr_ in oracle/_ref/libvvref.so (the
 * compiled reference behind oracle/ref_shims/ref_harness.cpp), so one Python wrapper
 * drives either.
 */
#ifndef VVD_ORACLE_H
#define VVD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-body parameters of a rigid body (TBody fields, libvvhd/headers/TBody.hpp:57-158).
 * Time functions (speed_x/y/o, force_o) are passed already evaluated at S->time. */
typedef struct vvo_body_params {
    double holder_x, holder_y, holder_o;         /* TBody::holder   */
    double dpos_x, dpos_y, dpos_o;               /* TBody::dpos     */
    double speed_x, speed_y, speed_o;            /* TBody::speed(t) */
    double speed_slae_x, speed_slae_y, speed_slae_o;               /* TBody::speed_slae      */
    double speed_slae_prev_x, speed_slae_prev_y, speed_slae_prev_o; /* TBody::speed_slae_prev */
    double friction_prev_x, friction_prev_y, friction_prev_o;      /* TBody::friction_prev   */
    double fdt_dead_x, fdt_dead_y, fdt_dead_o;                     /* TBody::fdt_dead        */
    double g_dead;                                                 /* TBody::g_dead          */
    double density;                                                /* TBody::density         */
    double kspring_x, kspring_y, kspring_o;      /* TBody::kspring (rigid: inf or <0) */
    int32_t special_segment_no;                  /* TBody::special_segment_no */
    int32_t bc_kutta;                            /* boundary_condition == bc_t::kutta */
} vvo_body_params;

/* SLAE outputs per body: TBody::speed_slae, force_hydro, force_holder. */
typedef struct vvo_body_out {
    double speed_slae_x, speed_slae_y, speed_slae_o;
    double force_hydro_x, force_hydro_y, force_hydro_o;
    double force_holder_x, force_holder_y, force_holder_o;
} vvo_body_out;

typedef struct vvo_space vvo_space;

vvo_space* vvo_create(void);
void vvo_destroy(vvo_space* S);

/* Space scalars: re (1/nu), dt, inf_speed(), inf_g, time, gravity. */
int vvo_set_params(vvo_space* S, double re, double dt, double inf_vx, double inf_vy,
                   double inf_g, double time, double gravity_x, double gravity_y);
/* Appends one body given its corners (TBody::alist[i].corner) in contour order. */
int vvo_add_body(vvo_space* S, int64_t nseg, const double* corner_x, const double* corner_y,
                 const uint32_t* slip, const vvo_body_params* bp);
/* Sets segment circulations (TAtt::g), e.g. from a previous SLAE solve. */
int vvo_set_segment_g(vvo_space* S, const double* g);
int vvo_set_sinks(vvo_space* S, int64_t n, const double* x, const double* y, const double* g);
/* Replaces Space::VortexList (v is zeroed; slot i remembers original index i). */
int vvo_set_vortices(vvo_space* S, int64_t n, const double* x, const double* y,
                     const double* g, const double* inv_eps);
int64_t vvo_num_vortices(const vvo_space* S);
int64_t vvo_num_segments(const vvo_space* S);
/* Current VortexList in its current (tree-permuted) order; orig = index at set time
 * (shed vortices get indices n_set, n_set+1, ...). Any pointer may be NULL. */
int vvo_get_vortices(const vvo_space* S, double* x, double* y, double* g, double* inv_eps,
                     double* vx, double* vy, int64_t* orig);
/* Per segment (all bodies in order): r, dl, _1_eps, g, fric, gsum. Any pointer may be NULL. */
int vvo_get_segments(const vvo_space* S, double* rx, double* ry, double* dlx, double* dly,
                     double* inv_eps, double* g, double* fric, double* gsum);
/* TBody::get_area / get_cofm / get_moi_axis / get_slen of body b. */
int vvo_get_body_geom(const vvo_space* S, int b, double* area, double* cofm_x, double* cofm_y,
                      double* moi_axis, double* slen);

/* stree::build (TSortedTree.cpp:232-265), vortices + bodies only. */
int vvo_tree_build(vvo_space* S, double far_criteria, double min_node, double max_node);
int vvo_tree_destroy(vvo_space* S);
/* Sizes of the built tree: nodes, leaves (bottomNodes), total near and far entries. */
int vvo_tree_sizes(const vvo_space* S, int64_t* nnodes, int64_t* nleaves, int64_t* nnear,
                   int64_t* nfar);
/* Leaves in bottomNodes order: geometry, vortex range, node depth (snode::i) and path
 * bits (snode::j), segment list range in seg_order, and +/- centroids. Any pointer may be NULL. */
int vvo_tree_leaves(const vvo_space* S, double* x, double* y, double* h, double* w,
                    int64_t* vfirst, int64_t* vlast, int32_t* depth, int64_t* path,
                    int64_t* sfirst, int64_t* slast);
/* All nodes (creation order is implementation defined; identify by depth/path). */
int vvo_tree_nodes(const vvo_space* S, double* x, double* y, double* h, double* w,
                   int64_t* vfirst, int64_t* vlast, int32_t* depth, int64_t* path,
                   double* cmp_x, double* cmp_y, double* cmp_g,
                   double* cmm_x, double* cmm_y, double* cmm_g);
/* Segment order (bllist order concatenated over leaves) as global segment indices. */
int vvo_tree_seg_order(const vvo_space* S, int64_t* seg_order);
/* Near/far lists per leaf, CSR: near_off[nleaves+1], near entries as (depth,path);
 * far_off[nleaves+1], far entries as (depth,path). */
int vvo_tree_lists(const vvo_space* S, int64_t* near_off, int32_t* near_depth, int64_t* near_path,
                   int64_t* far_off, int32_t* far_depth, int64_t* far_path);

/* MEpsilonFast::CalcEpsilonFast (MEpsilonFast.cpp:11-63). */
int vvo_eps(vvo_space* S, int merge, int64_t* merged);
/* MConvectiveFast::process_all_lists (MConvectiveFast.cpp:36-114). */
int vvo_convective(vvo_space* S);
/* MDiffusiveFast::process_vort_list (MDiffusiveFast.cpp:8-48). */
int vvo_diffusive(vvo_space* S);
/* MConvectiveFast::velocity(p) (MConvectiveFast.cpp:20-34) for points. */
int vvo_velocity_points(vvo_space* S, int64_t n, const double* px, const double* py,
                        double* vx, double* vy);
/* MConvectiveFast::calc_circulation (MConvectiveFast.cpp:235-273) for rigid bodies:
 * fills and solves the SLAE; writes TAtt::g and the body outputs. The filled system
 * can be read back with vvo_slae_export (row-major, size nseg+9*nbodies). */
int vvo_slae(vvo_space* S, vvo_body_out* out);
int64_t vvo_slae_size(const vvo_space* S);
int vvo_slae_export(const vvo_space* S, double* matrix, double* rhs, double* solution);
/* Timing sample for the CPU baseline: eps/convective/diffusive and the SLAE right-hand
 * side process only leaves (rows) whose index is a multiple of stride (default 1 = all). */
int vvo_set_sample(vvo_space* S, int64_t stride);
/* Seconds spent in the last tree build: partition, centroids, near/far lists. */
int vvo_last_timings(const vvo_space* S, double* out3);
/* Steady-state per-step SLAE work of the reference (right-hand side + dense GEMV). */
int vvo_slae_rhs_step(vvo_space* S, double* rhs_out);
/* MFlowmove::vortex_shed (MFlowmove.cpp:217-235). */
int vvo_vortex_shed(vvo_space* S);
/* MFlowmove::move_and_clean(remove, &collision, &cleaned) (MFlowmove.cpp:11-215) for rigid
 * bodies at rest (no collision): r += v dt, removal of |g| < 1e-10 and (remove != 0) of
 * vortices inside a body with its circulation bookkeeping, v = 0, dead segment terms.
 * Returns -2 with the tree built, -4 for moving or spring-mounted bodies. */
int vvo_move_and_clean(vvo_space* S, int remove, int64_t* cleaned);
int vvo_get_body_params(const vvo_space* S, int b, vvo_body_params* out);
/* TObj::v of every vortex (as left by the convective and diffusive passes). */
int vvo_set_velocities(vvo_space* S, const double* vx, const double* vy);
/* TAtt::g, fric and gsum of every segment. */
int vvo_set_segment_state(vvo_space* S, const double* g, const double* fric, const double* gsum);
/* Space::calc_forces (TSpace.cpp:94-117): per-segment Cp, Fr, Nu accumulation and each
 * body's friction (x, y, o) and nusselt, written to out4[4 b .. 4 b + 3]. */
int vvo_calc_forces(vvo_space* S, double* out4);
/* Space::zero_forces (TSpace.cpp:122-142). */
int vvo_zero_forces(vvo_space* S);
int vvo_get_segment_forces(const vvo_space* S, double* cp, double* fr, double* nu);
/* Space::gsum (TSpace.hpp:93-99). */
double vvo_gsum(const vvo_space* S);

/* Grid fields of libvvhd (XVelocity.cpp, XStreamfunction.cpp, XVorticity.cpp): an
 * xres x yres grid p = (xmin, ymin) + dxdy (xi, yj) with xmin, ymin, dxdy rounded to float
 * (XField.hpp:47), out[yj * xres + xi] as XField::map.  Each evaluates on a private copy of
 * the space (the vortex list, epsilon and segment sums are restored).  Return -1 for
 * arguments the reference rejects with std::invalid_argument, -2 with a tree built, -4 for
 * moving bodies.  The stream function also reports the grid cells that hold a sink (gap
 * entries, grid order, at most gap_cap written; *ngaps = their number). */
int vvo_field_velocity(vvo_space* S, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                       char mode, char ref_frame, float* out);
int vvo_field_streamfunction(vvo_space* S, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                             double eps_mult, char ref_frame, float* out, int64_t gap_cap, uint16_t* gap_xi,
                             uint16_t* gap_yj, float* gap, int64_t* ngaps);
int vvo_field_vorticity(vvo_space* S, double xmin, double ymin, double dxdy, int32_t xres, int32_t yres,
                        double eps_mult, float* out);

/* FP64 direct sums (no tree) used to measure the tree's own error:
 * convective velocity of every non-zero vortex at the given points, with each source's
 * own smoothing radius (biot_savart, MConvectiveFast.cpp:116-120), plus inf_speed. */
int vvo_direct_velocity(const vvo_space* S, int64_t n, const double* px, const double* py,
                        double* vx, double* vy);

#ifdef __cplusplus
}
#endif
#endif
