! ISO_C_BINDING interface to libportal_gb300 (include/portal_gb300.h) for a
! Fortran caller such as PORTAL's main_para.f90 / para_finish.f90: the
! entry points that replace the node loop (main_para.f90:210-257) and the
! image loops (para_finish.f90:286-320, :382-448).  Arrays are passed in the
! reference's own layouts (column-major, 1-based ids where the reference
! uses them); pointers that may be NULL are type(c_ptr) (c_null_ptr or
! c_loc(array)).
module portal_gpu
  use iso_c_binding
  implicit none
  interface
    integer(c_int) function portal_create(ctx, device) bind(C, name="portal_create")
      import :: c_ptr, c_int
      type(c_ptr) :: ctx
      integer(c_int), value :: device
    end function
    integer(c_int) function portal_destroy(ctx) bind(C, name="portal_destroy")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function portal_set_molecule(ctx, nlev, j_lev, e_levs, r_num, r_trans, t_Aji, nu, &
        t_Bij, kd_v, c_num, c_trans, c_temp, c_par, col_temps, t_Cji) bind(C, name="portal_set_molecule")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nlev, r_num, c_num, c_temp, c_par
      integer(c_int) :: j_lev(*), r_trans(2,*), c_trans(2,*)
      real(c_double) :: e_levs(*), t_Aji(*), nu(*), t_Bij(*), kd_v(*), col_temps(*), t_Cji(*)
    end function
    integer(c_int) function portal_set_cloud(ctx, node_num, bulk_node_num, nlev, xyz, vel_all, b_all, &
        temp_all, dust_p, h2_dens, ab_all, lev_p, bvec_all, maxne, del_ne, del_num_ne, tx) &
        bind(C, name="portal_set_cloud")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: node_num, bulk_node_num, nlev, maxne
      real(c_double) :: xyz(3,*), vel_all(3,*), b_all(*), temp_all(2,*), dust_p(*), h2_dens(*), &
                        ab_all(*), lev_p(nlev,*), bvec_all(3,*)
      integer(c_int) :: del_ne(node_num,*), del_num_ne(*)
      real(c_double), value :: tx
    end function
    integer(c_int) function portal_radiation_field(ctx, nth, nph, nvel, gvec, dx, n_depth, J0, J2, &
        status, n_segments) bind(C, name="portal_radiation_field")
      import :: c_ptr, c_int, c_double, c_long_long
      type(c_ptr), value :: ctx
      integer(c_int), value :: nth, nph, nvel, n_depth
      real(c_double) :: gvec(3)
      real(c_double), value :: dx
      type(c_ptr), value :: J0, J2, status      ! c_loc(...) or c_null_ptr (keep on the device)
      integer(c_long_long) :: n_segments
    end function
    integer(c_int) function portal_solve_se(ctx, kmax, J0, J2, pol_pops, rates, JJ_20, status) &
        bind(C, name="portal_solve_se")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int), value :: kmax
      type(c_ptr), value :: J0, J2, pol_pops, rates, JJ_20, status
    end function
    integer(c_int) function portal_image(ctx, pol_pops, nlines, l1, l2, th_inc, ph_az, nvel, dvel, v0, &
        im_pix, im_size, alpha, dx, n_depth_rt, I, Q, U, tau, dI, dQ, dU, dtau, status) &
        bind(C, name="portal_image")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx, pol_pops
      integer(c_int), value :: nlines, nvel, im_pix, n_depth_rt
      integer(c_int) :: l1(*), l2(*)
      real(c_double), value :: th_inc, ph_az, dvel, v0, im_size, alpha, dx
      type(c_ptr), value :: I, Q, U, tau, dI, dQ, dU, dtau, status
    end function
    integer(c_int) function portal_set_star(ctx, star_mod, T_star, R_star, XYZ_star) &
        bind(C, name="portal_set_star")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: star_mod
      real(c_double), value :: T_star, R_star
      real(c_double) :: XYZ_star(3)
    end function
    integer(c_int) function portal_image_nodes(ctx, pol_pops, nlines, l1, l2, th_inc, ph_az, nvel, &
        dvel, v0, alpha, dx, n_depth_rt, xy, I, Q, U, tau, dI, dQ, dU, dtau, status) &
        bind(C, name="portal_image_nodes")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx, pol_pops
      integer(c_int), value :: nlines, nvel, n_depth_rt
      integer(c_int) :: l1(*), l2(*)
      real(c_double), value :: th_inc, ph_az, dvel, v0, alpha, dx
      type(c_ptr), value :: xy, I, Q, U, tau, dI, dQ, dU, dtau, status
    end function
    integer(c_int) function portal_lambda_iterate(ctx, nth, nph, nvel, gvec, dx, n_depth, kmax, tol, &
        max_iter, ng_period, local_operator, start_pops, pol_pops, lev_p_out, iterations, residuals, &
        n_segments) bind(C, name="portal_lambda_iterate")
      import :: c_ptr, c_int, c_double, c_long_long
      type(c_ptr), value :: ctx
      integer(c_int), value :: nth, nph, nvel, n_depth, kmax, max_iter, ng_period, local_operator
      real(c_double) :: gvec(3)
      real(c_double), value :: dx, tol
      type(c_ptr), value :: start_pops, pol_pops, lev_p_out, residuals
      integer(c_int) :: iterations
      integer(c_long_long) :: n_segments
    end function
    integer(c_int) function portal_node_segments(ctx, segments) bind(C, name="portal_node_segments")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int) :: segments(*)
    end function
    integer(c_int) function portal_set_depolarization(ctx, mode) bind(C, name="portal_set_depolarization")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int), value :: mode
    end function
    integer(c_int) function portal_adj_list(ctx, node_num, del_num, del_tri, max_ne_temp, del_ne, &
        del_num_ne, max_ne, ms) bind(C, name="portal_adj_list")
      import :: c_ptr, c_int, c_long_long
      type(c_ptr), value :: ctx
      integer(c_int), value :: node_num, max_ne_temp
      integer(c_long_long), value :: del_num
      integer(c_int) :: del_tri(4,*), del_num_ne(*), max_ne
      type(c_ptr), value :: del_ne, ms
    end function
    integer(c_int) function portal_field_moments(ctx, moments) bind(C, name="portal_field_moments")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double) :: moments(6,*)
    end function
  end interface
end module
