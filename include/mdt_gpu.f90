! mdt_gpu.f90 -- Fortran 2003 iso_c_binding interface to libmdt_gpu.so (mdt_gpu.h).
!
! Lets md_tian2's Fortran host call the GB300 engine directly: arrays are passed in
! the reference's own order (r(3, nbeads, natoms) per trajectory, concatenated), every
! function returns an integer(c_int32_t) status (0 = ok, < 0 = MDT_ERR_*).  Every entry
! point and struct of mdt_gpu.h has its interface here (tests/test_cpu_fortran_abi.py
! checks names, argument counts and C kinds against the header).
!
! C pointers that may be NULL (mdt_state_download's outputs, mdt_set_random_arrays'
! deviates, the optional outputs of the statistics calls) are type(c_ptr), value: pass
! c_loc(array) or c_null_ptr.  Required arrays are assumed-size dummies.
module mdt_gpu

    use, intrinsic :: iso_c_binding

    implicit none

    integer(c_int32_t), parameter :: MDT_OK = 0, MDT_ERR_ARG = -1, MDT_ERR_CUDA = -2, MDT_ERR_STATE = -3, &
                                     MDT_ERR_UNSUPPORTED = -4, MDT_ERR_NOMEM = -5, MDT_ERR_TOO_LARGE = -6
    integer(c_int32_t), parameter :: MDT_PES_EMT = 2003, MDT_PES_NENE = 2008, MDT_PES_SURROGATE = 2100
    integer(c_int32_t), parameter :: MDT_PROP_VERLET = 1001, MDT_PROP_LANGEVIN = 1003, MDT_PROP_ANDERSEN = 1005, &
                                     MDT_PROP_PILE = 1006, MDT_PROP_LANGEVIN_CONST = 1007
    integer(c_int32_t), parameter :: MDT_ENERGY_AND_FORCE = 3001, MDT_ENERGY_ONLY = 3002
    integer(c_int32_t), parameter :: MDT_PREC_FP64 = 0, MDT_PREC_FP32 = 1, MDT_PREC_BF16 = 2, &
                                     MDT_PREC_BF16X3 = 3
    integer(c_int32_t), parameter :: MDT_TRAJ_RUNNING = 0, MDT_TRAJ_EXIT_UPPER = 1, MDT_TRAJ_EXIT_LOWER = 2, &
                                     MDT_TRAJ_STEP_LIMIT = 3, MDT_TRAJ_ERR_DENSITY = -10, &
                                     MDT_TRAJ_ERR_NONFINITE = -11

    type, bind(C) :: mdt_prop_params
        real(c_double)     :: step, Tsurf, Tproj, pile_tau, andersen_time, gamma_const
        real(c_double)     :: pul, pll
        integer(c_int64_t) :: seed
        integer(c_int32_t) :: use_exit, rng_mode
    end type mdt_prop_params

    type, bind(C) :: mdt_traj_summary
        integer(c_int32_t) :: status, steps_done
        real(c_double)     :: epot, ekin_p, ekin_l, ebead
    end type mdt_traj_summary

    ! The HDNNP of read_nene (pes_nene_mod.f90:123): pointers to arrays laid out as in
    ! mdt_gpu.h (per element e and symmetry function s at e*maxsf + s, 0-based), lengths in
    ! bohr and energies in Hartree as inside RuNNer.
    type, bind(C) :: mdt_nn_model
        integer(c_int32_t) :: nelem
        type(c_ptr)        :: z
        integer(c_int32_t) :: maxsf
        type(c_ptr)        :: nsf, sftype
        type(c_ptr)        :: eta, rshift, lambda, zeta, rc
        type(c_ptr)        :: e1, e2
        type(c_ptr)        :: smin, smax, savg
        integer(c_int32_t) :: scalesym, centersym
        real(c_double)     :: scmin, scmax
        integer(c_int32_t) :: cutoff_type
        real(c_double)     :: cutoff_alpha
        integer(c_int32_t) :: nlayers
        integer(c_int32_t) :: maxnodes
        type(c_ptr)        :: nodes, act
        integer(c_int32_t) :: maxweights
        type(c_ptr)        :: weights
        integer(c_int32_t) :: normnodes
        integer(c_int32_t) :: remove_atom_energies
        type(c_ptr)        :: atom_energy
    end type mdt_nn_model

    type, bind(C) :: mdt_train_opts
        real(c_double)     :: w_energy, w_force
        real(c_double)     :: lr, beta1, beta2, eps
        integer(c_int32_t) :: precision
    end type mdt_train_opts

    type, bind(C) :: mdt_refill_params
        real(c_double)     :: z0, einc_min, einc_max, polar_min, polar_max, azimuth
        integer(c_int64_t) :: seed
    end type mdt_refill_params

    interface

        ! ---- context ------------------------------------------------------------
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

        integer(c_int32_t) function mdt_set_stream(ctx, cuda_stream) bind(C, name="mdt_set_stream")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, cuda_stream
        end function

        ! ---- PES parameters -----------------------------------------------------
        integer(c_int32_t) function mdt_emt_set_params(ctx, ntypes, eta2, n0, e0, lambda, v0, kappa, s0, pes) &
                bind(C, name="mdt_emt_set_params")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: ntypes
            real(c_double), intent(in) :: eta2(*), n0(*), e0(*), lambda(*), v0(*), kappa(*), s0(*)
            integer(c_int32_t), intent(in) :: pes(*)
        end function

        integer(c_int32_t) function mdt_nn_set_model(ctx, model, ntypes, z_of_type, max_neighbors) &
                bind(C, name="mdt_nn_set_model")
            import :: c_int32_t, c_ptr, mdt_nn_model
            type(c_ptr), value :: ctx
            type(mdt_nn_model), intent(in) :: model
            integer(c_int32_t), value :: ntypes, max_neighbors
            integer(c_int32_t), intent(in) :: z_of_type(*)
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

        integer(c_int32_t) function mdt_autotune(ctx, precision, nsteps, p, block, skin_ang, ms_per_step) &
                bind(C, name="mdt_autotune")
            import :: c_int32_t, c_ptr, mdt_prop_params
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: precision, nsteps
            type(mdt_prop_params), intent(in) :: p
            type(c_ptr), value :: block, skin_ang, ms_per_step
        end function

        integer(c_int32_t) function mdt_nn_repack(ctx, npacks) bind(C, name="mdt_nn_repack")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, npacks
        end function

        integer(c_int32_t) function mdt_nn_stats(ctx, fallbacks, overflow) bind(C, name="mdt_nn_stats")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, fallbacks, overflow
        end function

        integer(c_int32_t) function mdt_nn_descriptors(ctx, precision, G) bind(C, name="mdt_nn_descriptors")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: precision
            real(c_double), intent(out) :: G(*)
        end function

        integer(c_int32_t) function mdt_nn_neighbors(ctx, counts, words) bind(C, name="mdt_nn_neighbors")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int32_t), intent(out) :: counts(*), words(*)
        end function

        ! ---- training of the network (learned EMT surrogate) --------------------
        integer(c_int32_t) function mdt_train_set_labels(ctx, energy, forces) bind(C, name="mdt_train_set_labels")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: energy(*), forces(*)
        end function

        integer(c_int32_t) function mdt_train_step(ctx, opts, conf_ids, n, stats) bind(C, name="mdt_train_step")
            import :: c_int32_t, c_ptr, mdt_train_opts
            type(c_ptr), value :: ctx
            type(mdt_train_opts), intent(in) :: opts
            integer(c_int32_t), intent(in) :: conf_ids(*)
            integer(c_int32_t), value :: n
            type(c_ptr), value :: stats
        end function

        integer(c_int32_t) function mdt_train_gradient(ctx, opts, conf_ids, n, grad) &
                bind(C, name="mdt_train_gradient")
            import :: c_int32_t, c_ptr, c_double, mdt_train_opts
            type(c_ptr), value :: ctx
            type(mdt_train_opts), intent(in) :: opts
            integer(c_int32_t), intent(in) :: conf_ids(*)
            integer(c_int32_t), value :: n
            real(c_double), intent(out) :: grad(*)
        end function

        integer(c_int32_t) function mdt_train_commit(ctx, weights) bind(C, name="mdt_train_commit")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, weights
        end function

        ! ---- batch geometry and state -------------------------------------------
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
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, r, v, f, a, epot, dens
        end function

        ! ---- hot path -----------------------------------------------------------
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

        integer(c_int32_t) function mdt_set_step_limit(ctx, max_steps) bind(C, name="mdt_set_step_limit")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: max_steps
        end function

        integer(c_int32_t) function mdt_refill(ctx, p, generation, nrefilled) bind(C, name="mdt_refill")
            import :: c_int32_t, c_ptr, mdt_refill_params
            type(c_ptr), value :: ctx
            type(mdt_refill_params), intent(in) :: p
            type(c_ptr), value :: generation
            integer(c_int32_t), intent(out) :: nrefilled
        end function

        integer(c_int32_t) function mdt_refill_draws(ctx, draws) bind(C, name="mdt_refill_draws")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: draws(*)
        end function

        integer(c_int32_t) function mdt_traj_observables(ctx, turn_pnts, cl_appr, cl_appr_step, r_min_p) &
                bind(C, name="mdt_traj_observables")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: ctx, turn_pnts, cl_appr, cl_appr_step, r_min_p
        end function

        integer(c_int32_t) function mdt_traj_bounces(ctx, bounces, interaction_time, is_adsorbed, p) &
                bind(C, name="mdt_traj_bounces")
            import :: c_int32_t, c_ptr, mdt_prop_params
            type(c_ptr), value :: ctx, bounces, interaction_time, is_adsorbed
            type(mdt_prop_params), intent(in) :: p
        end function

        integer(c_int32_t) function mdt_set_adsorption(ctx, ads_start, ads_end) bind(C, name="mdt_set_adsorption")
            import :: c_int32_t, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: ads_start, ads_end
        end function

        integer(c_int32_t) function mdt_query(ctx, p, out) bind(C, name="mdt_query")
            import :: c_int32_t, c_ptr, mdt_prop_params, mdt_traj_summary
            type(c_ptr), value :: ctx
            type(mdt_prop_params), intent(in) :: p
            type(mdt_traj_summary), intent(out) :: out(*)
        end function

        integer(c_int32_t) function mdt_device_state(ctx, ptrs, nslots) bind(C, name="mdt_device_state")
            import :: c_int32_t, c_int64_t, c_ptr
            type(c_ptr), value :: ctx
            type(c_ptr), intent(out) :: ptrs(*)
            integer(c_int64_t), intent(out) :: nslots
        end function

        ! ---- allocation-free EMT (device pointers; see mdt_gpu.h) ---------------
        integer(c_int32_t) function mdt_emt_force_noalloc(natoms, idx, x, y, z, simbox, ntypes, eta2, n0, e0, &
                lambda, v0, kappa, s0, pes, fx, fy, fz, energy, dens, stream) bind(C, name="mdt_emt_force_noalloc")
            import :: c_int32_t, c_ptr, c_double
            integer(c_int32_t), value :: natoms, ntypes
            type(c_ptr), value :: idx, x, y, z
            real(c_double), intent(in) :: simbox(*), eta2(*), n0(*), e0(*), lambda(*), v0(*), kappa(*), s0(*)
            integer(c_int32_t), intent(in) :: pes(*)
            type(c_ptr), value :: fx, fy, fz, energy, dens, stream
        end function

        ! ---- measurement and counters -------------------------------------------
        integer(c_int32_t) function mdt_peak_fma(precision, iters, flops_per_s) bind(C, name="mdt_peak_fma")
            import :: c_int32_t, c_double
            integer(c_int32_t), value :: precision, iters
            real(c_double), intent(out) :: flops_per_s
        end function

        integer(c_int32_t) function mdt_rng_deviates(kind, seed, traj, step, stream, n, out) &
                bind(C, name="mdt_rng_deviates")
            import :: c_int32_t, c_int64_t, c_double
            integer(c_int32_t), value :: kind, traj, step, stream
            integer(c_int64_t), value :: seed, n
            real(c_double), intent(out) :: out(*)
        end function

        integer(c_int32_t) function mdt_wait_check(max_polls, arrive, timed_out, ms) bind(C, name="mdt_wait_check")
            import :: c_int32_t, c_double
            integer(c_int32_t), value :: max_polls, arrive
            integer(c_int32_t), intent(out) :: timed_out
            real(c_double), intent(out) :: ms
        end function

        integer(c_int64_t) function mdt_launch_count(ctx) bind(C, name="mdt_launch_count")
            import :: c_int64_t, c_ptr
            type(c_ptr), value :: ctx
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
