/*
 * portal_gb300.h -- C ABI of the GB300 (sm_103a) implementation of PORTAL's
 * polarized line-transfer hot path.
 *
 * The reference (PORTAL, Fortran90 + OpenMP) has no library interface: its
 * hot path is the body of two OpenMP loops.  Each entry point below replaces
 * one of those loops *and* its body with one batched call, taking the
 * reference's own arrays in their Fortran layouts (column-major, 1-based
 * node / level ids, 0 = "no node"), so that a Fortran caller passes its
 * arrays unchanged through ISO_C_BINDING.
 *
 * Conventions
 *   - Return value: PORTAL_OK (0) or a negative PORTAL_ERR_* code;
 *     portal_strerror() describes it.  Per-node outcome goes to the optional
 *     `status` array (PORTAL_NODE_* values), the analogue of the reference's
 *     `stop` statements, which abort the whole run instead.
 *   - Input host pointers are borrowed for the duration of the call; the
 *     context owns every device copy.
 *   - A context is not re-entrant: call it from one host thread.  Calls are
 *     synchronous.  The device is the one passed to portal_create.
 *   - Where an output pointer is NULL the result stays resident on the
 *     device, inside the context, for the next call to consume (e.g.
 *     portal_radiation_field with J0 = J2 = NULL followed by
 *     portal_solve_se with J0 = J2 = NULL runs the whole node loop of
 *     main_portal.x without a host round trip).
 */
#ifndef PORTAL_GB300_H
#define PORTAL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct portal_ctx portal_ctx;

enum {
    PORTAL_OK = 0,
    PORTAL_ERR_CUDA = -1,      /* a CUDA call failed (message: portal_last_error) */
    PORTAL_ERR_ARG = -2,       /* invalid argument                                 */
    PORTAL_ERR_STATE = -3,     /* cloud / molecule / preceding result missing      */
    PORTAL_ERR_DEPTH = -4,     /* a walk needed more than n_depth cells            */
    PORTAL_ERR_SINGULAR = -5,  /* an SE matrix was singular                        */
    PORTAL_ERR_NOMEM = -6,     /* device allocation failed                         */
    PORTAL_ERR_NODEVICE = -7   /* no CUDA device / the build has no sm_103a code   */
};

/* per-node status bits */
enum {
    PORTAL_NODE_OK = 0,
    PORTAL_NODE_DEPTH = 1,     /* inverse_rt.f90:206-210 would have stopped        */
    PORTAL_NODE_SINGULAR = 2,  /* em_coefs.f90:170-178 would have stopped          */
    PORTAL_NODE_REFINE = 4,    /* FP32 LU + FP64 refinement did not converge; the
                                  node was solved by the FP64 LU instead           */
    PORTAL_NODE_STAR = 8       /* star mode: star_all's rays exceed nth*nph
                                  (miscellaneous.f90:1203-1206 would have stopped) */
};

const char *portal_strerror(int code);
/* Last CUDA / argument error message of this context (or of the last failed
 * portal_create when ctx is NULL). */
const char *portal_last_error(const portal_ctx *ctx);

/* Create a context on CUDA device `device`.  Replaces nothing in the
 * reference (the Fortran program owns all state in its main program,
 * main_para.f90:1-200); it allocates the stream the context runs on. */
int portal_create(portal_ctx **ctx, int device);
int portal_destroy(portal_ctx *ctx);

/* The molecule after main_para.f90:119-120 and :178-185 (frequencies and
 * level energies in Hz, t_Bij computed), exactly the arrays
 * eat_lime_no_delaunay returns (eat_lime.f90:151-196):
 *   j_lev(nlev), e_levs(nlev) [Hz], r_trans(2,r_num) (lower, upper),
 *   t_Aji(r_num), nu(r_num) [Hz], t_Bij(r_num), kd_v(r_num),
 *   c_trans(2,c_num) (lower, upper), col_temps(c_temp),
 *   t_Cji(c_temp,c_num,c_par) [cm^3/s]. */
int portal_set_molecule(portal_ctx *ctx, int nlev, const int *j_lev, const double *e_levs,
                        int r_num, const int *r_trans, const double *t_Aji, const double *nu,
                        const double *t_Bij, const double *kd_v, int c_num, const int *c_trans,
                        int c_temp, int c_par, const double *col_temps, const double *t_Cji);

/* The LIME cloud after eat_lime_no_delaunay (eat_lime.f90:71-313) and the
 * del_ne compaction of main_para.f90:124-130:
 *   XYZ(3,N) normalised by tx = r_max, vel_all(3,N) [m/s], b_all(N) [m/s],
 *   temp_all(2,N) (kinetic, dust), dust_p(N), h2_dens(N) [m^-3], ab_all(N),
 *   lev_p(nlev,N) [m^-3], bvec_all(3,N) (global_magfield / dipole_magfield
 *   output, main_para.f90:149-155), del_ne(N,maxne) 1-based neighbour ids
 *   sorted ascending per node (unique.f90:43), del_num_ne(N).
 * The call builds the device layout (SoA, neighbour CSR with per-face
 * geometry).  The populations lev_p are the ones the radiation field uses;
 * portal_set_populations replaces them. */
int portal_set_cloud(portal_ctx *ctx, int node_num, int bulk_node_num, int nlev,
                     const double *xyz, const double *vel_all, const double *b_all,
                     const double *temp_all, const double *dust_p, const double *h2_dens,
                     const double *ab_all, const double *lev_p, const double *bvec_all,
                     int maxne, const int *del_ne, const int *del_num_ne, double tx);

/* Replace the level populations lev_p(nlev,N) [m^-3] of the cloud. */
int portal_set_populations(portal_ctx *ctx, const double *lev_p);

/* Radiation field of every bulk node: the inverse_rt half of the node loop
 * main_para.f90:210-257 (trace_node main_sub.f90:82-84 -> inverse_rt
 * inverse_rt.f90:1-137, trace_out :139-214, ray_in :217-344) with the
 * direction set of legendre_all(nth,nph) (miscellaneous.f90:1100-1137), the
 * gauge vector gvec (main_para.f90:172-176) and the trace step dx
 * (main_para.f90:135; PORTAL passes the REAL*4 1E-6).
 * Outputs (any may be NULL):
 *   J0(r_num,N), J2(r_num,N)  profile-averaged J^0_0, J^2_0 per line,
 *                             0 for nodes the reference skips (ab_all <= 0,
 *                             non-bulk nodes);
 *   status(N)                 PORTAL_NODE_* bits;
 *   n_segments                ray segments walked (sum of node_count).
 * In star mode (portal_set_star) nodes inside the star are skipped too and
 * every other node uses its own star_all ray set instead. */
int portal_radiation_field(portal_ctx *ctx, int nth, int nph, int nvel, const double *gvec,
                           double dx, int n_depth, double *J0, double *J2, int *status,
                           long long *n_segments);

/* portal_radiation_field plus the split of J^0_0 that the accelerated Lambda
 * iteration uses (no reference counterpart): J_eff(r_num,N) the profile-
 * averaged J^0_0 without the node's own line emission (the central cell's
 * term S_line (1 - e^-tau) removed, ray_in inverse_rt.f90:320-339) and
 * L_star(r_num,N) = dJ^0_0 / dS_line, the diagonal of the Lambda operator,
 * so that J^0_0 = J_eff + L_star S_line.  A following portal_solve_se with
 * J0 = J2 = NULL solves the preconditioned population equations. */
int portal_radiation_field_split(portal_ctx *ctx, int nth, int nph, int nvel, const double *gvec,
                                 double dx, int n_depth, double *J0, double *J2, double *J_eff,
                                 double *L_star, int *status, long long *n_segments);

/* Polarized statistical equilibrium of every bulk node: make_AC
 * (miscellaneous.f90:288-392) + get_rhovec (em_coefs.f90:115-201, with
 * setup_stateq pop_eqs.f90:361-653) + the packing of trace_node
 * (main_sub.f90:112-137), D0 = 0.  J0/J2 (r_num,N) from the host, or NULL to
 * use the device-resident result of the last portal_radiation_field.
 * Outputs: pol_pops(N, 2*nlev) column-major (rho^0_0, rho^2_0 per level, as
 * main_para.f90:271-275 writes them), rates(N,3,2*nlev) (spontaneous,
 * radiative, collisional; main_para.f90:277-294) or NULL, JJ_20(N,r_num)
 * (= J2/J0, main_sub.f90:139) or NULL, status(N) or NULL. */
int portal_solve_se(portal_ctx *ctx, int kmax, const double *J0, const double *J2,
                    double *pol_pops, double *rates, double *JJ_20, int *status);

/* Depolarising collisions in the statistical equilibrium: the D^(K) rates
 * of setup_stateq's col_dep slot (pop_eqs.f90:642-648), which the reference
 * computes with de_polarization (depol.f90:242-317, the sudden
 * approximation of Morris 1985 from the rates out of the lowest level, first
 * collision partner) and make_depolarization_temp (depol.f90:319-360, times
 * n_H2 1e-6) but never switches on (main_sub.f90:96 passes D0 = 0).
 *   mode 0  off (the default, the reference's run);
 *   mode 1  D^(K) on the K = K' >= 2 diagonal entries of each level, where
 *           setup_stateq assigns col_dep;
 *   mode 2  col_dep as setup_stateq's code reads it: the last assigned value
 *           also enters every later diagonal-block entry (the variable is
 *           never reset), which mode 1 leaves out.
 * Needs j_lev(i) = i - 1 (de_polarization's own assumption); a molecule
 * without it fails the next portal_solve_se with PORTAL_ERR_ARG.  Applies
 * to portal_solve_se, portal_lambda_iterate and batches built afterwards. */
int portal_set_depolarization(portal_ctx *ctx, int mode);

/* Lambda iteration of the node loop: repeat portal_radiation_field +
 * portal_solve_se, setting the level populations of every bulk node from
 * the SE solution between passes, n_J = n_mol sqrt(2J+1) rho^0_0(J)
 * (em_coefs.f90:91-94 with the normalisation em_coefs.f90:158-164), until the
 * largest relative change of rho^0_0 over nodes and levels is below tol, or
 * max_iter passes.  The reference makes exactly one pass
 * (main_para.f90:210-257); iteration 1 from the cloud's populations is that
 * pass.  start_pops(N, 2*nlev) (pol_pops layout) replaces the starting
 * populations of the bulk nodes by those of its rho^0_0 (a warm start), or
 * NULL to start from the cloud's.  ng_period 0 iterates plainly; ng_period
 * >= 3 adds Ng acceleration (no reference counterpart): after every
 * ng_period passes the state moves to the order-2 Ng extrapolation of the
 * last four iterates of rho^0_0 (weights 1/rho^2), clipped to positive
 * values and renormalised per node; convergence is still decided by the
 * change of one plain pass.  local_operator != 0 (no reference counterpart)
 * makes the passes accelerated Lambda iterations: the radiation-field
 * kernel also splits J^0_0 = J_eff + L* S at each node's own cell (L* the
 * diagonal of the Lambda operator) and the SE's population equations take
 * the preconditioned net rates (B_lu n_l - B_ul n_u) J_eff - A (1 - L*) n_u
 * (Rybicki & Hummer 1991); the fixed point is the plain one, and once an
 * accelerated pass changes rho^0_0 by less than tol a plain pass follows and
 * decides convergence.  Outputs (any may be NULL): the last
 * pol_pops(N, 2*nlev), the final lev_p(nlev, N) (they also become the
 * context's populations), the number of passes, residuals(max_iter) per
 * pass, and the total ray segments walked. */
int portal_lambda_iterate(portal_ctx *ctx, int nth, int nph, int nvel, const double *gvec, double dx,
                          int n_depth, int kmax, double tol, int max_iter, int ng_period,
                          int local_operator, const double *start_pops,
                          double *pol_pops, double *lev_p_out, int *iterations, double *residuals,
                          long long *n_segments);

/* Stokes image of one inclination: the pixel mode of finish_portal.x
 * (para_finish.f90:352-448) -- rotate_all_save (miscellaneous.f90:844-907),
 * the population read-back (para_finish.f90:222-240), comp_emcoefs
 * (em_coefs.f90:1-113) per bulk node and line, trace_out_raytrace
 * (raytrace.f90:58-177) per pixel and ray_in_raytrace (:179-323) per pixel,
 * line and channel; star mode as set by portal_set_star.
 *   pol_pops(N, 2*nlev) as main_portal.x wrote it, or NULL for the
 *   device-resident result of portal_solve_se;
 *   lines l1(nlines), l2(nlines) 1-based levels (at most 16 lines; as in
 *   the reference every line takes the frequency of the last pair,
 *   para_finish.f90:173-175); th_inc, ph_az inclination and azimuth
 *   (radians); channels v = i*dvel + v0, i = -nvel..nvel; pixels
 *   (2*im_pix+1)^2 over +-im_size (< 1/sqrt(2), so that every start point
 *   lies inside the unit sphere); alpha the dust polarisation efficiency
 *   (0.15 in para_finish.f90:78); dx the march step (REAL*4 1E-4 there).
 * Outputs (any may be NULL), each (2*im_pix+1, 2*im_pix+1, 2*nvel+1,
 * nlines) column-major, unscaled intensities (para_finish.f90 multiplies
 * I, Q, U by I_to_T = 3.255e39/nu0^2 when it writes them): I, Q, U, tau
 * and the dust I, Q, U, tau; status(pixels) 0 or PORTAL_NODE_DEPTH. */
int portal_image(portal_ctx *ctx, const double *pol_pops, int nlines, const int *l1, const int *l2,
                 double th_inc, double ph_az, int nvel, double dvel, double v0, int im_pix,
                 double im_size, double alpha, double dx, int n_depth_rt, float *I, float *Q,
                 float *U, float *tau, float *dust_I, float *dust_Q, float *dust_U,
                 float *dust_tau, int *status);

/* Star mode (star_mod = 1 of both input files; main_para.f90:75,
 * para_finish.f90:116).  R_star in metres as the input file gives it
 * (divided by the cloud's r_max here, main_para.f90:122); X_star(3) as given
 * -- the reference uses it without scaling, so only a centred star
 * (X_star = 0) is meaningful there and here alike.  star_mod = 0 turns it
 * off.  While on:
 *   - the node loop skips nodes with |X| <= R_star (main_para.f90:232): zero
 *     J and populations;
 *   - every other node integrates over its own ray set from star_all
 *     (miscellaneous.f90:1139-1226; main_sub.f90:56-79): ceil(dOm / (4 pi /
 *     (nth nph))) rays into the star's cone of solid angle
 *     dOm = pi (R_star / |X_star - X|)^2, then nth bands of
 *     ceil(nph sin th) rays over the rest of the sphere; the star rays end
 *     on the star's surface when they meet it (check_neigh_fast
 *     miscellaneous.f90:1056-1069) and start from B(T_star)
 *     (inverse_rt.f90:113-115).  A node whose rays would exceed nth*nph
 *     (the reference stops there) fails with PORTAL_ERR_ARG and status bit
 *     PORTAL_NODE_STAR;
 *   - image rays whose sky position lies on the star's disc start at the
 *     star's front, z = z_star + R_star, from B(T_star) (raytrace.f90:103-115).
 * portal_radiation_field_static has no context and is star_mod = 0 only. */
int portal_set_star(portal_ctx *ctx, int star_mod, double T_star, double R_star, const double *X_star);

/* Per-node maps of one inclination: the pix_mod = 0 mode of finish_portal.x
 * (para_finish.f90:245-350).  As portal_image, but one ray per bulk node,
 * started at the node's rotated sky position (x, y) = XYZ_inc(1:2, node)
 * (:292), and every line's Einstein A taken as t_Aji(l1(j)) -- the radiative
 * transition whose index equals the line's lower level (:303; the pixel mode
 * matches (l1, l2) against r_trans), so l1 must not exceed the number of
 * radiative transitions.  A node whose (x, y) lies outside the unit circle
 * has no start point (the reference leaves its start node undefined): its
 * status is 3 and its outputs NaN.
 * Outputs (any may be NULL): xy(2, n_bulk) = tx * the rotated (x, y), the
 * rows of inc%02d-xy.dat (:266-271); I, Q, U, tau and the dust I, Q, U, tau,
 * each (n_bulk, 2*nvel+1, nlines) column-major and unscaled (the files
 * inc%02d-trans%02d-vel%02d-im.dat hold I_to_T I, I_to_T Q, I_to_T U, tau,
 * :331-349); status(n_bulk). */
int portal_image_nodes(portal_ctx *ctx, const double *pol_pops, int nlines, const int *l1, const int *l2,
                       double th_inc, double ph_az, int nvel, double dvel, double v0, double alpha, double dx,
                       int n_depth_rt, double *xy, float *I, float *Q, float *U, float *tau, float *dust_I,
                       float *dust_Q, float *dust_U, float *dust_tau, int *status);

/* Radiation field for callers that cannot allocate device memory.
 *
 * No counterpart in the reference.  It serves callers that must not call
 * cudaMalloc: a host whose device memory is owned by its own pool (e.g. CUDA
 * Fortran device arrays, a framework that hands out pre-sized buffers), or
 * code that may not allocate between simulation steps.  It computes what
 * portal_radiation_field computes for a run without a star (star_mod = 0:
 * it has no star parameters), needs no context, and allocates nothing:
 *   - every input is a DEVICE pointer to the reference-layout array that
 *     portal_set_cloud takes from the host (xyz(3,N), vel_all(3,N), b_all(N),
 *     temp_all(2,N), dust_p(N), ab_all(N), lev_p(nlev,N), bvec_all(3,N),
 *     del_ne(N,maxne), del_num_ne(N)); the molecule's line data
 *     (j_lev, r_trans(2,r_num), t_Aji, nu, t_Bij, kd_v) and gvec are HOST
 *     pointers;
 *   - J0(r_num,N), J2(r_num,N) and status(N) (or NULL) are DEVICE outputs,
 *     written for every node (0 for the non-bulk nodes and the skipped ones);
 *   - its only scratch is a fixed 64 MiB array inside the library image,
 *     held on every GPU that loads the library until the process exits.
 * The call is asynchronous on cuda_stream (a cudaStream_t, NULL = legacy
 * default stream): synchronise before reading the outputs.  Every call
 * shares the one scratch array (and the line constants), so calls that
 * overlap on the GPU race; serialise them.  The first call on each device
 * looks up the scratch array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  The address is kept for the
 * life of the process, so no cudaDeviceReset may happen while the library
 * is loaded.
 * Limits (PORTAL_ERR_ARG beyond them; portal_radiation_field_static_limits
 * reports them): n_depth <= 857 cells per ray, r_num <= 64 lines,
 * 2*nvel+1 <= 288 channels, nth*nph <= 8192 directions.  Walk overflow is
 * reported per node in status (PORTAL_NODE_DEPTH) with J = 0 there. */
int portal_radiation_field_static(void *cuda_stream, int node_num, int bulk_node_num, int nlev,
                                  const double *xyz, const double *vel_all, const double *b_all,
                                  const double *temp_all, const double *dust_p, const double *ab_all,
                                  const double *lev_p, const double *bvec_all, int maxne,
                                  const int *del_ne, const int *del_num_ne, double tx,
                                  const int *j_lev, int r_num, const int *r_trans,
                                  const double *t_Aji, const double *nu, const double *t_Bij,
                                  const double *kd_v, int nth, int nph, int nvel, const double *gvec,
                                  double dx, int n_depth, double *J0, double *J2, int *status);
/* The size limits of portal_radiation_field_static (any pointer may be NULL). */
void portal_radiation_field_static_limits(int *max_n_depth, int *max_lines, int *max_channels,
                                          int *max_directions, long long *scratch_bytes);

/* Run this context's work on the caller's CUDA stream (a cudaStream_t
 * passed as void*), or on the context's own stream when NULL.  Lets a caller
 * order the library's kernels with its own work and time them with its own
 * events.  No reference counterpart (the reference has no device). */
int portal_set_stream(portal_ctx *ctx, void *cuda_stream);

/* Kernel timing of the last call (CUDA events on the context's stream):
 * times_ms[0] line-table kernel, [1] radiation-field kernel, [2] SE kernel,
 * [3] emission-coefficient kernel, [4] image walk kernel, [5] image
 * integration kernel; launches[i] the number of launches each. */
int portal_last_kernel_times(const portal_ctx *ctx, double *times_ms, int *launches, int n);

/* Copy the device-resident results of the last pass out (any pointer may be
 * NULL): J0, J2 (r_num,N), pol_pops(N, 2*nlev), status(N).  For models run by
 * a batch, whose results stay on the device. */
int portal_get_results(portal_ctx *ctx, double *J0, double *J2, double *pol_pops, int *status);

/* The Delaunay neighbour lists of the cloud, built on the device:
 * adj_list_no_delaunay (miscellaneous.f90:910-1015) with SortUnique's sort
 * and de-duplication of each node's list (unique.f90:43-59), the step of
 * eat_lime_no_delaunay (eat_lime.f90:282) that turns grid.vtk's tetrahedra
 * into del_ne.  del_tri(4, del_num) holds the tetrahedra's vertices as
 * grid.vtk lists them (0-based); outputs: del_ne(node_num, max_ne_temp)
 * column-major (1-based ids, ascending per node, 0 in the unused slots) or
 * NULL, del_num_ne(node_num), max_ne (the longest list, main_para.f90's
 * maxne), and the device time in ms (or NULL).  A node whose unsorted list
 * exceeds max_ne_temp fails with PORTAL_ERR_ARG, as the reference stops
 * there (miscellaneous.f90:995-1000). */
int portal_adj_list(portal_ctx *ctx, int node_num, long long del_num, const int *del_tri, int max_ne_temp,
                    int *del_ne, int *del_num_ne, int *max_ne, double *ms);

/* Ray segments of every node in the last radiation-field pass:
 * segments(N), the sum over the node's rays of trace_out's node_count
 * (inverse_rt.f90:139-214), 0 for skipped and non-bulk nodes.  No
 * reference counterpart (the reference keeps node_count per ray only). */
int portal_node_segments(portal_ctx *ctx, int *segments);

/* ---- many models in one launch (no counterpart in the reference) --------
 *
 * PORTAL post-processes one LIME model per run.  A batch runs the node loop
 * (radiation field + SE, as portal_radiation_field + portal_solve_se) of
 * many models -- each a context with its own cloud and molecule, uneven in
 * point and level counts -- as one persistent radiation-field launch and
 * one SE launch over all models' (model, node) work items, captured once
 * into a CUDA graph and replayed.  portal_batch_prepare picks the launch
 * shapes (line group and blocks per SM of the radiation-field kernel, warps
 * per block of the SE kernel) by timing each candidate on a 1-in-16 sample
 * of the work when autotune != 0.  Results stay in each model's context
 * (portal_get_results).  The contexts must outlive the batch and must not
 * be used on their own while a batch run is in flight. */
typedef struct portal_batch portal_batch;

int portal_batch_create(portal_batch **batch, int device);
int portal_batch_destroy(portal_batch *batch);
const char *portal_batch_last_error(const portal_batch *batch);
/* Add a model (a context with cloud and molecule set, on the batch's
 * device); returns its index (>= 0) or an error code. */
int portal_batch_add(portal_batch *batch, portal_ctx *model);
/* Set up every model for the pass (directions, channels, kmax as in
 * portal_radiation_field / portal_solve_se), tune and capture the graph. */
int portal_batch_prepare(portal_batch *batch, int nth, int nph, int nvel, const double *gvec, double dx,
                         int n_depth, int kmax, int autotune);
/* One pass over every model; use_graph 0 issues the same launches without
 * the graph.  n_segments: ray segments walked; ms: device time of the pass. */
int portal_batch_run(portal_batch *batch, int use_graph, long long *n_segments, double *ms);
/* Launch shapes in use (config[4]: line group, radiation-field blocks per
 * SM, SE warps per block, SE blocks per SM) and the tuner's timings
 * (triples: shape, shape, ms per candidate); returns the number of timing
 * values available. */
int portal_batch_config(const portal_batch *batch, int *config, double *tune, int max_tune);

/* ---- learned warm start (no counterpart in the reference) -------------
 *
 * A small MLP maps per-node features of the cloud and of the first
 * radiation field to the converged level populations, which then start
 * portal_lambda_iterate (start_pops); the plain iteration still decides
 * convergence, so the fixed point it reaches is unchanged.  The network is
 * n_in -> width (SiLU) x depth -> n_out (linear), FP32 master parameters,
 * BF16 operands and FP32 accumulation on the tensor cores in every GEMM of
 * the forward and the backward pass.  Inputs and targets are standardised
 * with statistics held in the model (mean, standard deviation).
 *
 * Parameter layout (flat FP32, portal_mlp_num_params values): per layer
 * l = 0..depth, the weights W_l (fan_out x fan_in, row-major) followed by
 * the bias b_l (fan_out).  Statistics: mean_x(n_in), std_x(n_in),
 * mean_y(n_out), std_y(n_out).  Matrices X(rows, n_in) and Y(rows, n_out)
 * are row-major (a node's features contiguous).  An MLP owns its own CUDA
 * stream on its device; calls are synchronous. */
typedef struct portal_mlp portal_mlp;

int portal_mlp_create(portal_mlp **mlp, int device, int n_in, int width, int depth, int n_out,
                      unsigned long long seed);
int portal_mlp_destroy(portal_mlp *mlp);
const char *portal_mlp_last_error(const portal_mlp *mlp);
long long portal_mlp_num_params(const portal_mlp *mlp);
/* copy parameters / statistics out or in (either pointer may be NULL) */
int portal_mlp_get_params(const portal_mlp *mlp, float *params, float *stats);
int portal_mlp_set_params(portal_mlp *mlp, const float *params, const float *stats);
/* One forward and backward pass on B rows of already standardised inputs X
 * and targets T: the mean squared error over the B*n_out outputs and its
 * gradient with respect to the flat parameters (grads may be NULL). */
int portal_mlp_gradients(portal_mlp *mlp, const float *X, const float *T, int B, float *grads,
                         float *loss);
/* Fit to (X, Y) in raw units, M rows: the standardisation statistics are
 * taken from this set, then `epochs` passes of shuffled minibatches of
 * `batch` rows (the remainder of each pass is dropped) with Adam
 * (beta 0.9 / 0.999, eps 1e-8) at learning rate lr; loss_per_epoch
 * (epochs values, may be NULL) the mean standardised MSE of each pass. */
int portal_mlp_train(portal_mlp *mlp, const float *X, const float *Y, int M, int epochs, int batch,
                     float lr, unsigned long long seed, float *loss_per_epoch);
/* Raw-unit predictions Y(B, n_out) for raw inputs X(B, n_in). */
int portal_mlp_predict(portal_mlp *mlp, const float *X, int B, float *Y);

/* The warm start's node features from the context's cloud and its
 * device-resident radiation field (the last portal_radiation_field call):
 * features(8, N) column-major (a node's 8 values contiguous):
 *   0 log10 n_H2 [cm^-3], 1 log10 T_kin [K],
 *   2 log10 |grad v| [s^-1] (Frobenius norm of the least-squares velocity
 *     gradient over the node's neighbours),
 *   3 cos^2 of the angle between the field and the local J^2_0 axis of
 *     line 1 (the principal axis of the traceless part of the second
 *     moment portal_field_moments returns),
 *   4, 5 log10 J^0_0 / B_nu(T_kin) of lines 1 and 2,
 *   6, 7 100 J^2_0 / J^0_0 of lines 1 and 2
 * (line 1 again for a one-line molecule). */
int portal_warmstart_features(portal_ctx *ctx, float *features);

/* The second moment of line 1's radiation field at every node from the last
 * portal_radiation_field call: moments(6, N) = sum over the node's rays of
 * w Ibar n n (components xx, yy, zz, xy, xz, yz in the cloud's frame; n the
 * ray direction, w its quadrature weight, Ibar its profile-averaged
 * intensity, as J^0_0 = sum w Ibar).  Its traceless part holds J^2_Q in any
 * frame: along a unit vector b, J^2_0 = (3 b.M.b - trace M) / (2 sqrt 2).
 * No reference counterpart (the reference forms J^2_0 in the field frame
 * only, inverse_rt.f90:128-129); 0 for skipped nodes. */
int portal_field_moments(portal_ctx *ctx, double *moments);

/* ---- utilities -------------------------------------------------------- */

/* Wigner 3j and 6j symbols, arguments doubled (2j, 2m) like wigxjpf's
 * fwig3jj / fwig6jj, which the reference calls at pop_eqs.f90:48-61,
 * :127-140, :194, :252-265, :331-344 and em_coefs.f90:42-46.  Exact
 * big-integer Racah sums, rounded once. */
double portal_wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3);
double portal_wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6);
/* SE coupling constants of L&L04 Eqs. 7.20 as pop_eqs.f90 defines them:
 * which = 0 t_abs_const (:1-78), 1 t_stim_const (:80-156), 2 t_spont_const
 * (:158-201; c2 = 0), 3 r_abs_const (:204-281), 4 r_stim_const (:283-359). */
void portal_coupling_constant(int which, int j, int k, int j2, int k2, double *c0, double *c2);

#ifdef __cplusplus
}
#endif
#endif
