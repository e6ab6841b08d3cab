! hande_gpu_m.f90 -- ISO_C_BINDING interface to the GB300 FCIQMC engine
! (include/hande_gpu.h).  A HANDE build links libhande_gpu.so and replaces the
! body of the Monte Carlo cycle loop of do_fciqmc (src/fciqmc.f90:307-413) and
! the estimator part of end_report_loop with calls to these procedures.
!
! The derived types mirror the C structs field for field (bind(c)); keep the
! two in step.  This module is compiled only where a Fortran compiler exists.
module hande_gpu_m

    use, intrinsic :: iso_c_binding, only: c_int32_t, c_int64_t, c_double, c_ptr, c_char, &
                                           c_null_ptr, c_uint64_t => c_int64_t
    implicit none

    integer(c_int32_t), parameter :: HGPU_OK = 0
    integer(c_int32_t), parameter :: HGPU_SYS_HUB_K = 1, HGPU_SYS_READ_IN = 2
    integer(c_int32_t), parameter :: HGPU_PREC_FP64 = 0, HGPU_PREC_MIXED = 1
    integer, parameter :: HGPU_MAX_WORDS = 2, HGPU_MAX_SPACES = 2

    type, bind(c) :: hgpu_system
        integer(c_int32_t) :: kind, nbasis, nel, nalpha, nbeta, nwords
        type(c_ptr) :: orb_sym, orb_ms, sp_eigv
        integer(c_int32_t) :: nkpoints
        type(c_ptr) :: sym_table, inv_sym
        real(c_double) :: coulomb_k
        integer(c_int32_t) :: norb, nsym_pg
        type(c_ptr) :: h1, v2
        integer(c_int64_t) :: nv2
        real(c_double) :: ecore
        type(c_ptr) :: nbasis_sym_spin
        integer(c_int32_t) :: max_sym_spin
        type(c_ptr) :: sym_spin_basis_fns
    end type hgpu_system

    type, bind(c) :: hgpu_config
        real(c_double) :: tau, shift_damping, initial_shift, vary_shift_from, target_particles
        real(c_double) :: initiator_pop, spawn_cutoff, pattempt_single, pattempt_double, D0_population
        integer(c_int32_t) :: vary_shift_from_proje, excit_gen, real_amplitudes, initiator_approx
        integer(c_int32_t) :: nspaces, ncycles, precision, quadrature_initiator
        integer(c_int64_t) :: seed, walker_length, spawned_walker_length
        integer(c_uint64_t) :: ref_det(HGPU_MAX_WORDS)
        real(c_double) :: pattempt_parallel
        integer(c_int32_t) :: density_matrices, density_matrix_report
        real(c_double) :: power_pitzer_min_weight
        integer(c_int32_t) :: semi_stoch_space, semi_stoch_size
        integer(c_int64_t) :: semi_stoch_start_iter, semi_stoch_shift_iter
        integer(c_int32_t) :: semi_stoch_ci_level, semi_stoch_combined
        real(c_double) :: shift_harmonic_forcing
        integer(c_int32_t) :: target_reference, reserved0
    end type hgpu_config

    type, bind(c) :: hgpu_report
        integer(c_int64_t) :: iteration
        real(c_double) :: shift(HGPU_MAX_SPACES), proj_energy(HGPU_MAX_SPACES)
        real(c_double) :: D0_population(HGPU_MAX_SPACES), nparticles(HGPU_MAX_SPACES)
        integer(c_int32_t) :: vary_shift(HGPU_MAX_SPACES)
        integer(c_int64_t) :: nstates, nspawn_events
        real(c_double) :: rspawn
        integer(c_int64_t) :: nattempts, nspawned
        integer(c_int32_t) :: error_flags, reserved0
        real(c_double) :: device_ms
        real(c_double) :: rdm_energy, rdm_trace
        integer(c_int64_t) :: nblooms
        real(c_double) :: tot_bloom, max_bloom
    end type hgpu_report

    type, bind(c) :: hgpu_launch
        integer(c_int32_t) :: spawn_chunk, spawn_blocks, stream_blocks, sort_blocks
    end type hgpu_launch

    type, bind(c) :: hgpu_state
        integer(c_int64_t) :: iteration
        real(c_double) :: shift(HGPU_MAX_SPACES)
        integer(c_int32_t) :: vary_shift(HGPU_MAX_SPACES)
        real(c_double) :: nparticles_old(HGPU_MAX_SPACES)
        real(c_double) :: tau
        integer(c_int64_t) :: seed
    end type hgpu_state

    interface
        integer(c_int32_t) function hgpu_version() bind(c, name='hgpu_version')
            import :: c_int32_t
        end function hgpu_version

        type(c_ptr) function hgpu_error_string(status) bind(c, name='hgpu_error_string')
            import :: c_ptr, c_int32_t
            integer(c_int32_t), value :: status
        end function hgpu_error_string

        integer(c_int32_t) function hgpu_device_count() bind(c, name='hgpu_device_count')
            import :: c_int32_t
        end function hgpu_device_count

        integer(c_int32_t) function hgpu_create(cfg, sys, h) bind(c, name='hgpu_create')
            import :: hgpu_config, hgpu_system, c_ptr, c_int32_t
            type(hgpu_config), intent(in) :: cfg
            type(hgpu_system), intent(in) :: sys
            type(c_ptr), intent(out) :: h
        end function hgpu_create

        integer(c_int32_t) function hgpu_destroy(h) bind(c, name='hgpu_destroy')
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
        end function hgpu_destroy

        integer(c_int32_t) function hgpu_initial_distribution(h) bind(c, name='hgpu_initial_distribution')
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
        end function hgpu_initial_distribution

        integer(c_int32_t) function hgpu_upload_walkers(h, states, pops, dat, n) bind(c, name='hgpu_upload_walkers')
            import :: c_ptr, c_int32_t, c_int64_t, c_double
            type(c_ptr), value :: h
            integer(c_int64_t), intent(in) :: states(*), pops(*)
            real(c_double), intent(in) :: dat(*)
            integer(c_int64_t), value :: n
        end function hgpu_upload_walkers

        integer(c_int32_t) function hgpu_rdm_download(h, rdm, capacity, n_out) bind(c, name='hgpu_rdm_download')
            import :: c_ptr, c_int32_t, c_int64_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: rdm(*)
            integer(c_int64_t), value :: capacity
            integer(c_int64_t), intent(out) :: n_out
        end function hgpu_rdm_download

        integer(c_int32_t) function hgpu_download_walkers(h, states, pops, dat, capacity, n_out) &
                bind(c, name='hgpu_download_walkers')
            import :: c_ptr, c_int32_t, c_int64_t, c_double
            type(c_ptr), value :: h
            integer(c_int64_t), intent(out) :: states(*), pops(*)
            real(c_double), intent(out) :: dat(*)
            integer(c_int64_t), value :: capacity
            integer(c_int64_t), intent(out) :: n_out
        end function hgpu_download_walkers

        integer(c_int32_t) function hgpu_run_cycles(h, ncycles) bind(c, name='hgpu_run_cycles')
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
            integer(c_int32_t), value :: ncycles
        end function hgpu_run_cycles

        integer(c_int32_t) function hgpu_end_report(h, rep) bind(c, name='hgpu_end_report')
            import :: c_ptr, c_int32_t, hgpu_report
            type(c_ptr), value :: h
            type(hgpu_report), intent(out) :: rep
        end function hgpu_end_report

        integer(c_int32_t) function hgpu_run_report(h, rep) bind(c, name='hgpu_run_report')
            import :: c_ptr, c_int32_t, hgpu_report
            type(c_ptr), value :: h
            type(hgpu_report), intent(out) :: rep
        end function hgpu_run_report

        integer(c_int32_t) function hgpu_checkpoint(h, path) bind(c, name='hgpu_checkpoint')
            import :: c_ptr, c_int32_t, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: path(*)
        end function hgpu_checkpoint

        integer(c_int32_t) function hgpu_restore(h, path) bind(c, name='hgpu_restore')
            import :: c_ptr, c_int32_t, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(in) :: path(*)
        end function hgpu_restore

        ! Scalars of qmc_state_t for a restart-aware do_fciqmc (iteration, shift,
        ! vary_shift, N_w of the last report, tau, seed).
        integer(c_int32_t) function hgpu_get_state(h, st) bind(c, name='hgpu_get_state')
            import :: c_ptr, c_int32_t, hgpu_state
            type(c_ptr), value :: h
            type(hgpu_state), intent(out) :: st
        end function hgpu_get_state

        integer(c_int32_t) function hgpu_set_state(h, st) bind(c, name='hgpu_set_state')
            import :: c_ptr, c_int32_t, hgpu_state
            type(c_ptr), value :: h
            type(hgpu_state), intent(in) :: st
        end function hgpu_set_state

        integer(c_int32_t) function hgpu_snapshot(h, restore) bind(c, name='hgpu_snapshot')
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: h
            integer(c_int32_t), value :: restore
        end function hgpu_snapshot

        integer(c_int32_t) function hgpu_profile_cycle(h, phase_ms, nphase, counts) bind(c, name='hgpu_profile_cycle')
            import :: c_ptr, c_int32_t, c_int64_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: phase_ms(*)
            integer(c_int32_t), value :: nphase
            integer(c_int64_t), intent(out) :: counts(*)
        end function hgpu_profile_cycle

        ! Parity entry points (fixed inputs, results on the host).
        integer(c_int32_t) function hgpu_eval_excitations(h, parents, parent_pops, n, iteration, orbs, pgen, &
                hmatel, allowed, nspawn) bind(c, name='hgpu_eval_excitations')
            import :: c_ptr, c_int32_t, c_int64_t, c_double
            type(c_ptr), value :: h
            integer(c_int64_t), intent(in) :: parents(*), parent_pops(*)
            integer(c_int64_t), value :: n, iteration
            integer(c_int32_t), intent(out) :: orbs(*)
            real(c_double), intent(out) :: pgen(*), hmatel(*)
            integer(c_int32_t), intent(out) :: allowed(*)
            integer(c_int64_t), intent(out) :: nspawn(*)
        end function hgpu_eval_excitations

        integer(c_int32_t) function hgpu_annihilate_fixed(h, sdata, n, iteration) bind(c, name='hgpu_annihilate_fixed')
            import :: c_ptr, c_int32_t, c_int64_t
            type(c_ptr), value :: h
            integer(c_int64_t), intent(in) :: sdata(*)
            integer(c_int64_t), value :: n, iteration
        end function hgpu_annihilate_fixed

        integer(c_int32_t) function hgpu_eval_diagonal(h, dets, n, kii) bind(c, name='hgpu_eval_diagonal')
            import :: c_ptr, c_int32_t, c_int64_t, c_double
            type(c_ptr), value :: h
            integer(c_int64_t), intent(in) :: dets(*)
            integer(c_int64_t), value :: n
            real(c_double), intent(out) :: kii(*)
        end function hgpu_eval_diagonal

        ! Self-annihilation of a device-resident spawned list without device
        ! allocation by the library (d_sdata, d_out and stream are device
        ! pointers / a cudaStream_t passed as c_ptr).
        integer(c_int32_t) function hgpu_self_annihilate_noalloc(d_sdata, n, nwords, nspaces, d_out, n_out, &
                stream) bind(c, name='hgpu_self_annihilate_noalloc')
            import :: c_ptr, c_int32_t, c_int64_t
            type(c_ptr), value :: d_sdata
            integer(c_int64_t), value :: n
            integer(c_int32_t), value :: nwords, nspaces
            type(c_ptr), value :: d_out
            integer(c_int64_t), intent(out) :: n_out
            type(c_ptr), value :: stream
        end function hgpu_self_annihilate_noalloc

        ! Launch shape of a handle's kernels (speed only; results do not depend on it).
        integer(c_int32_t) function hgpu_get_launch(h, l) bind(c, name='hgpu_get_launch')
            import :: c_ptr, c_int32_t, hgpu_launch
            type(c_ptr), value :: h
            type(hgpu_launch), intent(out) :: l
        end function hgpu_get_launch

        integer(c_int32_t) function hgpu_set_launch(h, l) bind(c, name='hgpu_set_launch')
            import :: c_ptr, c_int32_t, hgpu_launch
            type(c_ptr), value :: h
            type(hgpu_launch), intent(in) :: l
        end function hgpu_set_launch

        ! Batches: many handles advanced together, one graph launch per cycle.
        integer(c_int32_t) function hgpu_batch_create(handles, n, batch) bind(c, name='hgpu_batch_create')
            import :: c_ptr, c_int32_t
            type(c_ptr), intent(in) :: handles(*)
            integer(c_int32_t), value :: n
            type(c_ptr), intent(out) :: batch
        end function hgpu_batch_create

        integer(c_int32_t) function hgpu_batch_run_cycles(batch, ncycles) bind(c, name='hgpu_batch_run_cycles')
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: batch
            integer(c_int32_t), value :: ncycles
        end function hgpu_batch_run_cycles

        integer(c_int32_t) function hgpu_batch_destroy(batch) bind(c, name='hgpu_batch_destroy')
            import :: c_ptr, c_int32_t
            type(c_ptr), value :: batch
        end function hgpu_batch_destroy
    end interface

end module hande_gpu_m
