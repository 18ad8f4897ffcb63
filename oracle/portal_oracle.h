/*
 * portal_oracle.h -- FP64 CPU restatement of PORTAL's polarized line-transfer
 * hot path.  TEST INFRASTRUCTURE ONLY: this library is the checker for the
 * CUDA path (tests/, __graft_entry__.smoke(), and the cpu_baseline leg of
 * bench.py).  Nothing in the product library links or calls it.
 *
 * Every routine follows the reference routine named in its comment
 * (file:line within the PORTAL source tree).  Array layouts are the
 * reference's Fortran (column-major) layouts, node and level indices are
 * 1-based where the reference stores them (neighbour lists, transition
 * level pairs), and 0 means "no node" exactly as in the reference.
 *
 * Parity pinning (the reference ships no tests or fixtures):
 *   - Wigner 3j/6j against exact sympy values (tests/golden/wigner.json);
 *   - Gauss-Legendre nodes against numpy.polynomial.legendre.leggauss;
 *   - the SE LU against scipy.linalg.lapack dgetrf/dgetri;
 *   - analytic limits (isotropic field => rho^2_0 = 0, collision-dominated
 *     => Boltzmann populations, normalisation sum sqrt(2J+1) rho^0_0 = 1).
 */
#ifndef PORTAL_ORACLE_H
#define PORTAL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Cloud after the reference's ingestion transforms (eat_lime.f90:207-311):
 * xyz normalised by r_max, b_all with thermal broadening added, lev_p as
 * level number densities (fractions * ab * n_H2). */
typedef struct {
    int node_num;          /* all nodes (bulk + surface sink nodes)          */
    int bulk_node_num;     /* nodes that carry a .pop row                      */
    int nlev;              /* e_num                                            */
    int maxne;             /* second extent of del_ne                          */
    const double *xyz;     /* (3,N)                                            */
    const double *vel;     /* (3,N)  m/s                                       */
    const double *b_all;   /* (N)    Doppler b, m/s                            */
    const double *t_kin;   /* (N)    temp_all(1,:)                             */
    const double *t_dust;  /* (N)    temp_all(2,:)                             */
    const double *dust_p;  /* (N)    dust mass density kg/m^3                  */
    const double *h2_dens; /* (N)    m^-3                                      */
    const double *ab_all;  /* (N)                                              */
    const double *lev_p;   /* (nlev,N) m^-3                                    */
    const double *bvec;    /* (3,N)  unit magnetic-field direction            */
    const int *del_ne;     /* (N,maxne) column-major, 1-based, 0 = unused      */
    const int *del_num_ne; /* (N)                                              */
    double tx;             /* r_max in metres                                  */
    /* star mode (star_mod = 1, main_para.f90:75, :122, :216-246): 0 = off.
     * R_star is R_star / tx; X_star is used as read, unscaled, as the
     * reference does (only a centred star is meaningful there). */
    int star_mod;
    double T_star, R_star;
    double X_star[3];
} orc_cloud;

/* Molecule after main_para.f90:119-120 (nu, e_levs in Hz) and
 * main_para.f90:180-185 (t_Bij). */
typedef struct {
    int nlev, r_num, c_num, c_temp, c_par;
    const int *j_lev;       /* (nlev)                                          */
    const double *e_levs;   /* (nlev) Hz                                       */
    const int *r_trans;     /* (2,r_num) (lower, upper), 1-based               */
    const double *A;        /* (r_num) t_Aji                                   */
    const double *nu;       /* (r_num) Hz                                      */
    const double *Bij;      /* (r_num) t_Bij                                   */
    const double *kd_v;     /* (r_num) dust opacity                            */
    const int *c_trans;     /* (2,c_num) (lower, upper), 1-based               */
    const double *col_temps;/* (c_temp)                                        */
    const double *C;        /* (c_temp,c_num,c_par) cm^3/s                     */
    /* depolarising collisions (depol.f90:242-360), D0 of setup_stateq's
     * col_dep slot (pop_eqs.f90:642-648): 0 off (main_sub.f90:96 passes
     * D0 = 0), 1 on the K = K' >= 2 diagonal entries where the reference
     * assigns col_dep, 2 as the reference's code reads col_dep (the last
     * assigned value stays in every later entry of the diagonal blocks). */
    int depol;
} orc_molecule;

enum {
    ORC_OK = 0,
    ORC_ERR_DEPTH = 1,     /* node_count > n_depth (inverse_rt.f90:206-210)    */
    ORC_ERR_LU = 2,        /* singular SE matrix (em_coefs.f90:170-178)        */
    ORC_ERR_ARG = 3
};

/* ---- numerics ---- */
double orc_black_body(double T, double nu0);
void   orc_gauss_legendre(int n, double *x, double *w);
int    orc_legendre_all(int nth, int nph, double *xth /* (3, nth*nph) */);
double orc_wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3);
double orc_wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6);
void   orc_find_dir(const double *bvec, const double *gvec, double th, double ph,
                    double *dir);

/* star_all miscellaneous.f90:1139-1226 with circle_points :1228-1265: the
 * ray set of a node outside the star -- n_star rays into the star's cone
 * around kvec (the node-to-star direction) with solid angle dOm, then nth
 * bands over the rest of the sphere -- as (cos th, ph, weight) relative to
 * bvec (find_angles miscellaneous.f90:86-134).  xth holds nth*nph columns;
 * returns the ray count, or -1 where the reference would run past them. */
int orc_star_all(int nth, int nph, const double *kvec, const double *gvec, const double *bvec,
                 double dOm_star, int *n_star, double *xth);

/* ---- radiation field (main_portal.x hot loop, first half) ---- */
int orc_trace_out(const orc_cloud *c, int node, const double *dir, double dx,
                  int n_depth, int *depth_list /* (2,n_depth+1) */, int *node_count);
int orc_inverse_rt(const orc_cloud *c, const orc_molecule *m, int node,
                   const double *xth, int n_sphere, const double *gvec, int nvel,
                   double dx, int n_depth, double *J0, double *J2,
                   int64_t *n_segments);
/* Nodes node_lo..node_hi (1-based, inclusive) of the bulk; J0/J2 are
 * (r_num, node_num).  Returns the number of nodes whose walk overflowed
 * n_depth (their status entry is ORC_ERR_DEPTH).  Threads: OpenMP, static
 * schedule over nodes like main_para.f90:210. */
int orc_radiation_field(const orc_cloud *c, const orc_molecule *m, int nth, int nph,
                        int nvel, const double *gvec, double dx, int n_depth,
                        int node_lo, int node_hi, int nthreads, double *J0,
                        double *J2, int *status, int64_t *n_segments);
/* The same, with the split of the accelerated Lambda iteration (no
 * reference counterpart): JE(r_num,N) J^0_0 without the node's own line
 * emission, LS(r_num,N) its derivative with respect to the node's line
 * source function (the diagonal of the Lambda operator). */
int orc_radiation_field_split(const orc_cloud *c, const orc_molecule *m, int nth, int nph,
                              int nvel, const double *gvec, double dx, int n_depth, int node_lo,
                              int node_hi, int nthreads, double *J0, double *J2, double *JE,
                              double *LS, int *status, int64_t *n_segments);

/* The node loop over a list of n_nodes 1-based bulk node ids (a sample of a
 * cloud too large to restate whole): J0/J2 (and JE/LS when JE is not NULL)
 * written at the listed nodes' columns, status and seg_per_node (each may
 * be NULL) per list entry.  Returns the number of failed nodes. */
int orc_radiation_field_nodes(const orc_cloud *c, const orc_molecule *m, int nth, int nph, int nvel,
                              const double *gvec, double dx, int n_depth, const int *nodes,
                              int n_nodes, int nthreads, double *J0, double *J2, double *JE,
                              double *LS, int *status, int64_t *seg_per_node);

/* ---- statistical equilibrium ---- */
int orc_setup_count_array(const int *j_lev, int nlev, int kmax, int *count_array);
int orc_all_transitions(const orc_molecule *m, int *all_trans /* (2,r_num+c_num) */);
void orc_make_AC(const orc_molecule *m, double nH2, double Temp, int n_trans,
                 const int *all_trans, const double *J0, const double *J2,
                 double *AC /* (5,n_trans) */);
/* D0 (nlev, kmax/2): the node's depolarisation rates D^(K) [s^-1] of level
 * i for K = 2, 4, .. at D0[(i-1) + nlev (K/2 - 1)], or NULL for D0 = 0;
 * depol as orc_molecule.depol. */
void orc_setup_stateq(int c_dim, const int *count_array, int nlev, const int *j_lev,
                      const int *trans, int ntrans, int kmax, const double *AC,
                      double Temp, const double *D0, int depol, double *Amat, double *A_mat,
                      double *B_mat, double *C_mat);
int orc_get_rhovec(int c_dim, const int *count_array, int nlev, const int *j_lev,
                   int ntrans, const int *trans, const double *AC, int kmax,
                   double Temp, const double *D0, int depol, double *rhovec,
                   double *rates /* (3,c_dim) or NULL */);
/* de_polarization depol.f90:242-317: D0_all (c_temp, nlev, kmax/2), the
 * sudden-approximation depolarisation coefficients [cm^3 s^-1] of every
 * level and K = 2, 4, .. <= min(2J, kmax) from the first partner's rates out
 * of the lowest level.  Returns -1 unless j_lev(i) = i - 1 (the reference's
 * assumption). */
int orc_de_polarization(const orc_molecule *m, int kmax, double *D0_all);
/* make_depolarization_temp depol.f90:319-360: D0 (nlev, kmax/2) [s^-1] at
 * temperature T and n_H2 [m^-3]. */
void orc_make_depolarization_temp(const double *D0_all, int nlev, int nT, int kmax,
                                  const double *col_temps, double T, double nH2, double *D0);
/* trace_node's SE half for nodes node_lo..node_hi: pol_pops (node_num, 2*nlev)
 * column-major, rates (node_num,3,2*nlev) or NULL. */
int orc_solve_se(const orc_cloud *c, const orc_molecule *m, int kmax,
                 const double *J0, const double *J2, int node_lo, int node_hi,
                 int nthreads, double *pol_pops, double *rates, int *status);
/* orc_solve_se over a list of 1-based bulk node ids (status per entry). */
int orc_solve_se_nodes(const orc_cloud *c, const orc_molecule *m, int kmax, const double *J0,
                       const double *J2, const int *nodes, int n_nodes, int nthreads,
                       double *pol_pops, double *rates, int *status);
/* Coupling constants of pop_eqs.f90:1-359 for the tests: which = 0 t_A,
 * 1 t_S, 2 t_E (c0 only), 3 r_A, 4 r_S. */
void orc_coupling_constants(int which, int j, int k, int j2, int k2, double *c0, double *c2);
/* Matrix of one node (before the normalisation row), column-major, for tests. */
int orc_node_matrix(const orc_cloud *c, const orc_molecule *m, int kmax, int node,
                    const double *J0, const double *J2, double *Amat, int *c_dim);

/* ---- Stokes image (finish_portal.x) ---- */
void orc_comp_emcoefs(double r1_0, double r2_0, double r1_2, double r2_2, int j1,
                      int j2, double th, double nu0, double Aji, double *nsI_tot,
                      double *nsQ_tot, double *es_I, double *es_Q);
void orc_rotate_all_save(int node_num, double th_inc, double ph_az, const double *vel,
                         const double *bvec, const double *xyz, double *vel_new,
                         double *bvec_new, double *xyz_new);
int orc_trace_out_raytrace(double x_co, double y_co, int node_num, const double *xyz,
                           const int *del_ne, const int *del_num_ne, int maxne,
                           double dx, int n_depth_rt, int *depth_list, int *node_count);
void orc_polarize_prop(double eta_I, double eta_Q, double eps_I, double eps_Q,
                       double ds, double *I, double *Q, double *U);
void orc_ray_in_raytrace(double vel_obs, int node_count, const int *depth_list,
                         const double *pol_rayt /* (nlines,4,N) */, int nlines, int line,
                         const double *b_all, const double *bvec, const double *dust_p,
                         double alpha, double kd, const double *t_dust,
                         const double *vel_z, double dx, double nu0, double I_in,
                         double *out /* I,Q,U,tau,dI,dQ,dU,dtau */);
/* Pixel-mode image for one inclination (para_finish.f90:352-448).
 * lines: l1/l2 (1-based levels), pol_pops (node_num, 2*nlev) as read back and
 * renormalised by para_finish.f90:222-240.  Output cube layout:
 * out[(((q*n_rt + p)*nlines + j)*nchan + k)] with q = 0..7 the quantities
 * I,Q,U,tau,dust I,Q,U,tau; p the pixel (para_finish.f90:369-376 order). */
int orc_image(const orc_cloud *c, const orc_molecule *m, int nlines, const int *l1,
              const int *l2, const double *pol_pops, double th_inc, double ph_az,
              int nvel, double dvel, double v0, int im_pix, double im_size,
              double alpha, int n_depth_rt, int pix_lo, int pix_hi, int nthreads,
              double *out, int *status);
/* Per-node mode of finish_portal.x (pix_mod = 0, para_finish.f90:245-350) for
 * one inclination: one ray per bulk node started at its rotated (x, y), the
 * line's Einstein A taken as t_Aji(l1(j)) (:303).  xy(2, n_bulk) = tx * the
 * rotated (x, y) (:269-271), or NULL; out as orc_image with p the bulk node,
 * computed for nodes node_lo..node_hi. */
int orc_image_nodes(const orc_cloud *c, const orc_molecule *m, int nlines, const int *l1,
                    const int *l2, const double *pol_pops, double th_inc, double ph_az,
                    int nvel, double dvel, double v0, double alpha, int n_depth_rt, int node_lo,
                    int node_hi, int nthreads, double *xy, double *out, int *status);

#ifdef __cplusplus
}
#endif
#endif
