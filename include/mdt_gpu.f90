! mdt_gpu.f90 -- Fortran 2003 iso_c_binding interface to libmdt_gpu.so (mdt_gpu.h).
!
! Lets md_tian2's Fortran host call the GB300 engine directly: arrays are passed in
! the reference's own order (r(3, nbeads, natoms) per trajectory, concatenated), every
! function returns an integer(c_int32_t) status (0 = ok, < 0 = MDT_ERR_*).
module mdt_gpu

    use, intrinsic :: iso_c_binding

    implicit none

    integer(c_int32_t), parameter :: MDT_OK = 0
    integer(c_int32_t), parameter :: MDT_PES_EMT = 2003, MDT_PES_NENE = 2008, MDT_PES_SURROGATE = 2100
    integer(c_int32_t), parameter :: MDT_ENERGY_AND_FORCE = 3001, MDT_ENERGY_ONLY = 3002
    integer(c_int32_t), parameter :: MDT_PREC_FP64 = 0, MDT_PREC_FP32 = 1
    integer(c_int32_t), parameter :: MDT_TRAJ_RUNNING = 0, MDT_TRAJ_EXIT_UPPER = 1, MDT_TRAJ_EXIT_LOWER = 2, &
                                     MDT_TRAJ_STEP_LIMIT = 3, MDT_TRAJ_ERR_DENSITY = -10

    type, bind(C) :: mdt_prop_params
        real(c_double)     :: step, Tsurf, Tproj, pile_tau, andersen_time, gamma_const
        real(c_double)     :: pul, pll
        integer(c_int64_t) :: seed
        integer(c_int32_t) :: use_exit, rng_mode
    end type mdt_prop_params

    type, bind(C) :: mdt_refill_params
        real(c_double)     :: z0, einc_min, einc_max, polar_min, polar_max, azimuth
        integer(c_int64_t) :: seed
    end type mdt_refill_params

    type, bind(C) :: mdt_traj_summary
        integer(c_int32_t) :: status, steps_done
        real(c_double)     :: epot, ekin_p, ekin_l, ebead
    end type mdt_traj_summary

    interface

        integer(c_int32_t) function mdt_create(device, ctx) bind(C, name="mdt_create")
            import :: c_int32_t, c_ptr
            integer(c_int32_t), value :: device
            type(c_ptr), intent(out) :: ctx
        end function

        integer(c_int32_t) function mdt_destroy(ctx) bind(C, name="mdt_destroy")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
        end function

        type(c_ptr) function mdt_last_error(ctx) bind(C, name="mdt_last_error")
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function

        integer(c_int32_t) function mdt_synchronize(ctx) bind(C, name="mdt_synchronize")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
        end function

        integer(c_int32_t) function mdt_emt_set_params(ctx, ntypes, eta2, n0, e0, lambda, v0, kappa, s0, pes) &
                bind(C, name="mdt_emt_set_params")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: ntypes
            real(c_double), intent(in) :: eta2(*), n0(*), e0(*), lambda(*), v0(*), kappa(*), s0(*)
            integer(c_int32_t), intent(in) :: pes(*)
        end function

        integer(c_int32_t) function mdt_batch_define(ctx, ntraj, natoms, nbeads, idx, mass, is_fixed, simbox, &
                ntypes, algo, is_proj) bind(C, name="mdt_batch_define")
            import :: c_int32_t, c_ptr, c_double, c_int8_t
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: ntraj, ntypes
            integer(c_int32_t), intent(in) :: natoms(*), nbeads(*), idx(*), algo(*)
            real(c_double), intent(in) :: mass(*), simbox(*)
            integer(c_int8_t), intent(in) :: is_fixed(*), is_proj(*)
        end function

        integer(c_int32_t) function mdt_state_upload(ctx, r, v) bind(C, name="mdt_state_upload")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: r(*), v(*)
        end function

        integer(c_int32_t) function mdt_state_download(ctx, r, v, f, a, epot, dens) bind(C, name="mdt_state_download")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: r(*), v(*), f(*), a(*), epot(*), dens(*)
        end function

        integer(c_int32_t) function mdt_calc_force(ctx, flag, precision, p) bind(C, name="mdt_calc_force")
            import :: c_int32_t, c_ptr, mdt_prop_params
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: flag, precision
            type(mdt_prop_params), intent(in) :: p
        end function

        integer(c_int32_t) function mdt_propagate_1(ctx, p) bind(C, name="mdt_propagate_1")
            import :: c_int32_t, c_ptr, mdt_prop_params
            type(c_ptr), value :: ctx
            type(mdt_prop_params), intent(in) :: p
        end function

        integer(c_int32_t) function mdt_propagate_2(ctx, p) bind(C, name="mdt_propagate_2")
            import :: c_int32_t, c_ptr, mdt_prop_params
            type(c_ptr), value :: ctx
            type(mdt_prop_params), intent(in) :: p
        end function

        integer(c_int32_t) function mdt_md_steps(ctx, nsteps, precision, p) bind(C, name="mdt_md_steps")
            import :: c_int32_t, c_ptr, mdt_prop_params
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: nsteps, precision
            type(mdt_prop_params), intent(in) :: p
        end function

        integer(c_int32_t) function mdt_set_random_arrays(ctx, randy, zeta, andersen_v, andersen_u) &
                bind(C, name="mdt_set_random_arrays")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, randy, zeta, andersen_v, andersen_u
        end function

        integer(c_int32_t) function mdt_query(ctx, p, out) bind(C, name="mdt_query")
            import :: c_int32_t, c_ptr, mdt_prop_params, mdt_traj_summary
            type(c_ptr), value :: ctx
            type(mdt_prop_params), intent(in) :: p
            type(mdt_traj_summary), intent(out) :: out(*)
        end function

        integer(c_int32_t) function mdt_traj_observables(ctx, turn_pnts, cl_appr, cl_appr_step, r_min_p) &
                bind(C, name="mdt_traj_observables")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int32_t), intent(out) :: turn_pnts(*), cl_appr_step(*)
            real(c_double), intent(out) :: cl_appr(*), r_min_p(*)
        end function

        integer(c_int32_t) function mdt_set_step_limit(ctx, max_steps) bind(C, name="mdt_set_step_limit")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: max_steps
        end function

        integer(c_int32_t) function mdt_refill(ctx, p, generation, nrefilled) bind(C, name="mdt_refill")
            import :: c_int32_t, c_ptr, mdt_refill_params
            type(c_ptr), value :: ctx
            type(mdt_refill_params), intent(in) :: p
            integer(c_int32_t), intent(out) :: generation(*), nrefilled
        end function

        integer(c_int32_t) function mdt_set_pes(ctx, pes_kind, range_margin) bind(C, name="mdt_set_pes")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: pes_kind
            real(c_double), value :: range_margin
        end function

        integer(c_int32_t) function mdt_nn_fast_path(ctx, enable) bind(C, name="mdt_nn_fast_path")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: enable
        end function

        integer(c_int32_t) function mdt_nn_radial_kernel(ctx, enable) bind(C, name="mdt_nn_radial_kernel")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: enable
        end function

        integer(c_int32_t) function mdt_nn_radial_block(ctx, max_block) bind(C, name="mdt_nn_radial_block")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: max_block
        end function

        integer(c_int32_t) function mdt_nn_set_skin(ctx, skin_ang) bind(C, name="mdt_nn_set_skin")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: skin_ang
        end function

    end interface

contains

    ! mdt_last_error as a Fortran string (what the reference would print before stop)
    function mdt_last_error_f(ctx) result(msg)
        type(c_ptr), intent(in) :: ctx
        character(len=:), allocatable :: msg
        character(kind=c_char), pointer :: chars(:)
        type(c_ptr) :: p
        integer :: n
        interface
            integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
                import :: c_ptr, c_size_t
                type(c_ptr), value :: s
            end function
        end interface
        p = mdt_last_error(ctx)
        n = int(c_strlen(p))
        call c_f_pointer(p, chars, [n])
        allocate(character(len=n) :: msg)
        msg = transfer(chars(1:n), msg)
    end function mdt_last_error_f

end module mdt_gpu
