!! mglc_iface.f90 -- iso_c_binding interface to libmglc_gb300.so for the MGLC
!! Fortran drivers.  Source only in this repository: no Fortran compiler is
!! available where it is built and tested; the same C-ABI is exercised from
!! C/C++ and Python.  Every function returns an integer status (0 = OK);
!! mglc_last_error_f returns the context's message.
!!
!! Array arguments are the reference's own arrays, passed without copies:
!!   f(0:18,1:nx,1:ny,1:nz), g(0:6,1:nx,1:ny,1:nz), rho/u/v/w/T(1:nx,1:ny,1:nz).
module mglc_iface
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: MGLC_OK = 0
    integer(c_int), parameter :: MGLC_ERR_INVALID = 1, MGLC_ERR_CUDA = 2, MGLC_ERR_NOMEM = 3, &
                                  MGLC_ERR_STATE = 4, MGLC_ERR_NUMERIC = 5, &
                                  MGLC_ERR_UNSUPPORTED = 6, MGLC_ERR_PARTICLE = 7
    integer(c_int), parameter :: MGLC_FP64 = 0, MGLC_FP32 = 1, MGLC_FP16 = 2, MGLC_BF16 = 3, &
                                  MGLC_FX64 = 4, MGLC_FP16S = 5, MGLC_BF16S = 6
    integer(c_int), parameter :: MGLC_KIND_LID = 1, MGLC_KIND_THERMAL = 2, &
                                  MGLC_KIND_PARTICLE = 3, MGLC_KIND_PARTICLE2D = 4, &
                                  MGLC_KIND_LID2D = 5

    type, bind(C) :: mglc_lid_params
        integer(c_int) :: total_nx, total_ny, total_nz
        real(c_double) :: reynolds, rho0, u0
        integer(c_int) :: top_layer_u0, precision
        integer(c_int) :: in_place = 0   !! 1: AA-pattern streaming on one buffer
    end type

    type, bind(C) :: mglc_thermal_params
        integer(c_int) :: total_nx, total_ny, total_nz
        real(c_double) :: rayleigh, prandtl, mach
        real(c_double) :: t_hot, t_cold, t_ref
        real(c_double) :: ekman
        integer(c_int) :: bc_y_const_t, bc_z_const_t, precision
        integer(c_int) :: in_place = 0   !! 1: AA-pattern streaming of f and g
    end type

    type, bind(C) :: mglc_particle_params
        integer(c_int) :: total_nx, total_ny, total_nz, periodic_x
        real(c_double) :: tauf, rho0, rho_solid, radius
        real(c_double) :: gravity(3), body_force(3)
        real(c_double) :: threshold_wall, threshold_particle
        real(c_double) :: spring_scale_wall, spring_scale_particle
        integer(c_int) :: precision
    end type

    type, bind(C) :: mglc_particle2d_params
        integer(c_int) :: total_nx, total_ny
        real(c_double) :: tauf, rho0, rho_solid, radius, gravity
        real(c_double) :: threshold_wall, stiff_wall, threshold_particle, stiff_particle
        integer(c_int) :: q_bisection
    end type

    type, bind(C) :: mglc_shear2d_params
        integer(c_int) :: total_nx, total_ny
        real(c_double) :: tauf, rho0, rho_solid, radius, u0, uwall
        integer(c_int) :: moving_frame, linear
    end type

    type, bind(C) :: mglc_lid2d_params
        integer(c_int) :: total_nx, total_ny
        real(c_double) :: reynolds, rho0, u0
        integer(c_int) :: precision
    end type

    type, bind(C) :: mglc_nure_status
        integer(c_int) :: time
        real(c_double) :: nu, re, nu_mean, re_mean
        integer(c_int) :: stationary, stationary_time, converged
        real(c_double) :: nu_half_change, re_half_change, nu_mean_change, re_mean_change
    end type

    type, bind(C) :: mglc_info
        integer(c_int) :: kind, precision
        integer(c_int) :: nx, ny, nz
        integer(c_long_long) :: itc
        real(c_double) :: tauf, snu, sq
        real(c_double) :: viscosity, diffusivity, para_a, gbeta, omega_rot
        real(c_double) :: bytes_per_cell_step
        integer(c_long_long) :: device_bytes
    end type

    type, bind(C) :: mglc_server_params
        integer(c_long_long) :: hbm_budget_bytes
        integer(c_int) :: max_active, precision, steps_per_iteration
        real(c_double) :: tol
        integer(c_long_long) :: max_steps
        integer(c_int) :: autotune, keep_results
        integer(c_int) :: in_place = 0   !! 1: one population buffer per solve
    end type

    type, bind(C) :: mglc_request
        integer(c_int) :: kind, n
        real(c_double) :: reynolds, rayleigh, arrival_s
    end type

    type, bind(C) :: mglc_request_result
        integer(c_long_long) :: id
        integer(c_int) :: kind, n
        integer(c_long_long) :: steps
        real(c_double) :: residual
        real(c_double) :: arrival_s, admit_s, finish_s
        integer(c_int) :: converged
    end type

    type, bind(C) :: mglc_server_stats
        integer(c_long_long) :: iterations, steps_total, cell_updates
        real(c_double) :: wall_s, busy_s
        integer(c_int) :: tile_threads, tile_rows, ctas_per_sm
        integer(c_long_long) :: peak_device_bytes
        integer(c_int) :: peak_active
    end type

    interface
        integer(c_int) function mglc_lid_create(p, ctx) bind(C, name="mglc_lid_create")
            import :: c_int, c_ptr, mglc_lid_params
            type(mglc_lid_params), intent(in) :: p
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function mglc_thermal_create(p, ctx) bind(C, name="mglc_thermal_create")
            import :: c_int, c_ptr, mglc_thermal_params
            type(mglc_thermal_params), intent(in) :: p
            type(c_ptr), intent(out) :: ctx
        end function
        subroutine mglc_destroy(ctx) bind(C, name="mglc_destroy")
            import :: c_ptr
            type(c_ptr), value :: ctx
        end subroutine
        type(c_ptr) function mglc_last_error(ctx) bind(C, name="mglc_last_error")
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function mglc_initial(ctx) bind(C, name="mglc_initial")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function mglc_load_state(ctx, f, g, rho, u, v, w, T) &
                bind(C, name="mglc_load_state")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, f, g, rho, u, v, w, T
        end function
        integer(c_int) function mglc_get_f(ctx, f, g) bind(C, name="mglc_get_f")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, f, g
        end function
        integer(c_int) function mglc_step(ctx, nsteps) bind(C, name="mglc_step")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps
        end function
        integer(c_int) function mglc_get_macros(ctx, rho, u, v, w, T) bind(C, name="mglc_get_macros")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, rho, u, v, w, T
        end function
        integer(c_int) function mglc_check(ctx, error_u, error_t) bind(C, name="mglc_check")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: error_u, error_t
        end function
        integer(c_int) function mglc_totals(ctx, mass, energy, heat) bind(C, name="mglc_totals")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: mass, energy, heat
        end function
        integer(c_int) function mglc_nusselt(ctx, nu_vol, re_vol, nu_hot, nu_cold) &
                bind(C, name="mglc_nusselt")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: nu_vol, re_vol, nu_hot, nu_cold
        end function
        !! spheres (D3Q19): centers(3, np)
        integer(c_int) function mglc_particle_create(p, centers, np, ctx) &
                bind(C, name="mglc_particle_create")
            import :: c_int, c_ptr, c_double, mglc_particle_params
            type(mglc_particle_params), intent(in) :: p
            real(c_double), intent(in) :: centers(*)
            integer(c_int), value :: np
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function mglc_get_mask(ctx, owner) bind(C, name="mglc_get_mask")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: owner(*)
        end function
        !! case4 (D2Q9) particles: centers(2, np)
        integer(c_int) function mglc_particle2d_create(p, centers, np, ctx) &
                bind(C, name="mglc_particle2d_create")
            import :: c_int, c_ptr, c_double, mglc_particle2d_params
            type(mglc_particle2d_params), intent(in) :: p
            real(c_double), intent(in) :: centers(*)
            integer(c_int), value :: np
            type(c_ptr), intent(out) :: ctx
        end function
        !! case1 (D2Q9) circles in shear flow, periodic x: centers(2, np)
        integer(c_int) function mglc_shear2d_create(p, centers, np, ctx) &
                bind(C, name="mglc_shear2d_create")
            import :: c_int, c_ptr, c_double, mglc_shear2d_params
            type(mglc_shear2d_params), intent(in) :: p
            real(c_double), intent(in) :: centers(*)
            integer(c_int), value :: np
            type(c_ptr), intent(out) :: ctx
        end function
        !! 2-D lid-driven cavity (2d_revised/mpi_blocked), f(0:8,nx,ny)
        integer(c_int) function mglc_lid2d_create(p, ctx) bind(C, name="mglc_lid2d_create")
            import :: c_int, c_ptr, mglc_lid2d_params
            type(mglc_lid2d_params), intent(in) :: p
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function mglc_particle_state(ctx, xc, uc, omega, force, torque) &
                bind(C, name="mglc_particle_state")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: xc(*), uc(*), omega(*), force(*), torque(*)
        end function
        !! output_Tecplot / getVelocity / output_binary / backupData / reload
        integer(c_int) function mglc_write_tecplot(ctx, path) bind(C, name="mglc_write_tecplot")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        integer(c_int) function mglc_write_profiles(ctx, uz_path, xw_path, u0) &
                bind(C, name="mglc_write_profiles")
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: uz_path(*), xw_path(*)
            real(c_double), value :: u0
        end function
        integer(c_int) function mglc_write_binary(ctx, path) bind(C, name="mglc_write_binary")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        integer(c_int) function mglc_backup_save(ctx, path) bind(C, name="mglc_backup_save")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        integer(c_int) function mglc_backup_load(ctx, path) bind(C, name="mglc_backup_load")
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        !! calNuRe bookkeeping
        integer(c_int) function mglc_nure_create(flow_reversal, flow_reversal_time, m) &
                bind(C, name="mglc_nure_create")
            import :: c_int, c_ptr
            integer(c_int), value :: flow_reversal, flow_reversal_time
            type(c_ptr), intent(out) :: m
        end function
        subroutine mglc_nure_destroy(m) bind(C, name="mglc_nure_destroy")
            import :: c_ptr
            type(c_ptr), value :: m
        end subroutine
        integer(c_int) function mglc_nure_sample(m, ctx, status) bind(C, name="mglc_nure_sample")
            import :: c_int, c_ptr, mglc_nure_status
            type(c_ptr), value :: m, ctx
            type(mglc_nure_status), intent(out) :: status
        end function
        integer(c_int) function mglc_nure_push(m, nu, re, status) bind(C, name="mglc_nure_push")
            import :: c_int, c_ptr, c_double, mglc_nure_status
            type(c_ptr), value :: m
            real(c_double), value :: nu, re
            type(mglc_nure_status), intent(out) :: status
        end function
        !! derived constants and device memory of a context
        integer(c_int) function mglc_get_info(ctx, info) bind(C, name="mglc_get_info")
            import :: c_int, c_ptr, mglc_info
            type(c_ptr), value :: ctx
            type(mglc_info), intent(out) :: info
        end function
        !! the CUDA stream the context launches on (c_null_ptr: its own stream)
        integer(c_int) function mglc_set_stream(ctx, cuda_stream) bind(C, name="mglc_set_stream")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, cuda_stream
        end function
        !! rho, u, v, w (and T) into DEVICE arrays the caller owns
        integer(c_int) function mglc_get_macros_device(ctx, rho, u, v, w, T) &
                bind(C, name="mglc_get_macros_device")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, rho, u, v, w, T
        end function
        !! the writers on host arrays the caller already holds
        integer(c_int) function mglc_tecplot_write_fields(path, nx, ny, nz, u, v, w, s, thermal) &
                bind(C, name="mglc_tecplot_write_fields")
            import :: c_int, c_ptr, c_char
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int), value :: nx, ny, nz
            type(c_ptr), value :: u, v, w, s
            integer(c_int), value :: thermal
        end function
        integer(c_int) function mglc_profiles_write_fields(uz_path, xw_path, nx, ny, nz, u, w, u0) &
                bind(C, name="mglc_profiles_write_fields")
            import :: c_int, c_ptr, c_char, c_double
            character(kind=c_char), intent(in) :: uz_path(*), xw_path(*)
            integer(c_int), value :: nx, ny, nz
            type(c_ptr), value :: u, w
            real(c_double), value :: u0
        end function
        integer(c_int) function mglc_backup_write_fields(path, nx, ny, nz, u, v, w, T, f, g, &
                max_subrecord) bind(C, name="mglc_backup_write_fields")
            import :: c_int, c_ptr, c_char, c_long_long
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int), value :: nx, ny, nz
            type(c_ptr), value :: u, v, w, T, f, g
            integer(c_long_long), value :: max_subrecord
        end function
        integer(c_int) function mglc_backup_read_fields(path, nx, ny, nz, u, v, w, T, f, g) &
                bind(C, name="mglc_backup_read_fields")
            import :: c_int, c_ptr, c_char
            character(kind=c_char), intent(in) :: path(*)
            integer(c_int), value :: nx, ny, nz
            type(c_ptr), value :: u, v, w, T, f, g
        end function
        !! check() on DEVICE arrays the caller owns, without device allocation
        integer(c_int) function mglc_residual_noalloc(n, u, v, w, T, up, vp, wp, Tp, with_w, &
                cuda_stream, error_u, error_t, errbuf, errbuf_len) &
                bind(C, name="mglc_residual_noalloc")
            import :: c_int, c_ptr, c_double, c_long_long, c_char
            integer(c_long_long), value :: n
            type(c_ptr), value :: u, v, w, T, up, vp, wp, Tp
            integer(c_int), value :: with_w
            type(c_ptr), value :: cuda_stream
            real(c_double), intent(out) :: error_u, error_t
            character(kind=c_char), intent(out) :: errbuf(*)
            integer(c_int), value :: errbuf_len
        end function
        !! the sequential FP64 sum of the 2-D particle step's density averages
        integer(c_int) function mglc_sequential_sum(x, keep, n, total, count) &
                bind(C, name="mglc_sequential_sum")
            import :: c_int, c_double, c_long_long
            real(c_double), intent(in) :: x(*)
            integer(c_int), intent(in) :: keep(*)
            integer(c_int), value :: n
            real(c_double), intent(out) :: total
            integer(c_long_long), intent(out) :: count
        end function
        !! batched serving of many cavity solves
        integer(c_int) function mglc_server_create(p, srv) bind(C, name="mglc_server_create")
            import :: c_int, c_ptr, mglc_server_params
            type(mglc_server_params), intent(in) :: p
            type(c_ptr), intent(out) :: srv
        end function
        subroutine mglc_server_destroy(srv) bind(C, name="mglc_server_destroy")
            import :: c_ptr
            type(c_ptr), value :: srv
        end subroutine
        type(c_ptr) function mglc_server_last_error(srv) bind(C, name="mglc_server_last_error")
            import :: c_ptr
            type(c_ptr), value :: srv
        end function
        integer(c_int) function mglc_server_submit(srv, r, id) bind(C, name="mglc_server_submit")
            import :: c_int, c_ptr, c_long_long, mglc_request
            type(c_ptr), value :: srv
            type(mglc_request), intent(in) :: r
            integer(c_long_long), intent(out) :: id
        end function
        integer(c_int) function mglc_server_run(srv, time_limit_s) bind(C, name="mglc_server_run")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: srv
            real(c_double), value :: time_limit_s
        end function
        integer(c_int) function mglc_server_results(srv, results, nmax, count) &
                bind(C, name="mglc_server_results")
            import :: c_int, c_ptr, mglc_request_result
            type(c_ptr), value :: srv
            type(mglc_request_result), intent(out) :: results(*)
            integer(c_int), value :: nmax
            integer(c_int), intent(out) :: count
        end function
        integer(c_int) function mglc_server_get_field(srv, id, fields) &
                bind(C, name="mglc_server_get_field")
            import :: c_int, c_ptr, c_long_long, c_float
            type(c_ptr), value :: srv
            integer(c_long_long), value :: id
            real(c_float), intent(out) :: fields(*)
        end function
        integer(c_int) function mglc_server_get_stats(srv, stats) bind(C, name="mglc_server_get_stats")
            import :: c_int, c_ptr, mglc_server_stats
            type(c_ptr), value :: srv
            type(mglc_server_stats), intent(out) :: stats
        end function
    end interface

contains

    !! Fortran string of the context's last error message.
    function mglc_last_error_f(ctx) result(msg)
        type(c_ptr), intent(in) :: ctx
        character(len=512) :: msg
        character(kind=c_char), pointer :: p(:)
        integer :: i
        msg = ''
        call c_f_pointer(mglc_last_error(ctx), p, [512])
        do i = 1, 512
            if (p(i) == c_null_char) exit
            msg(i:i) = p(i)
        enddo
    end function

end module mglc_iface
