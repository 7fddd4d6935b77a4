! tam.f90 -- Fortran 2008 interface to libtam.so (iso_c_binding).
!
! The module the reference's driver (src/mcpolar.f90) uses to call the GPU
! library in place of its photon loop and heat / damage / property block:
!   tam_read_input_params   replaces src/mcpolar.f90:79-94
!   tam_create              replaces src/mcpolar.f90:55-140 (set-up)
!   tam_mc_pass             replaces src/mcpolar.f90:151-174 (photon loop,
!                           allreduce, normalisation)
!   tam_heat_steps          replaces src/mcpolar.f90:178 (heat_sim_3D)
!   tam_arrhenius           replaces src/mcpolar.f90:180 (Arrhenius)
!   tam_update_props        replaces src/mcpolar.f90:182 (setupThermalCoeff)
!   tam_run                 replaces the whole loop src/mcpolar.f90:148-186
!   tam_finalize            replaces src/mcpolar.f90:196-205
!   tam_write_output        replaces src/writer.f90:6-81
! and, with no reference counterpart: device error word, timing, tuning and
! the autotuner, and the batches of instances (tam_batch_*).
! Arrays are passed as c_loc of the reference's own arrays (FP64,
! column-major, halo lower bound 0 where the reference has one).
!
! Written against include/tam.h; no Fortran compiler was available where
! this library was built, so this file has not been compiled.
module tam_gpu
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: TAM_OK = 0, TAM_E_INVALID = 1, TAM_E_CUDA = 2, TAM_E_NOMEM = 3, &
                                 TAM_E_IO = 4, TAM_E_PARSE = 5, TAM_E_STATE = 6, TAM_E_DEVICE = 7, &
                                 TAM_E_NODEV = 8
    integer(c_int), parameter :: TAM_MODE_REFERENCE = 0, TAM_MODE_CONFIG = 1
    integer(c_int), parameter :: TAM_FP64 = 0, TAM_FP32 = 1
    integer(c_int), parameter :: TAM_PULSE_GAUSSIAN = 0, TAM_PULSE_TOPHAT = 1, TAM_PULSE_TRIANGULAR = 2
    integer(c_int), parameter :: TAM_F_TEMP = 0, TAM_F_RHOKAP = 1, TAM_F_JMEAN = 2, TAM_F_JMEAN_GLOBAL = 3, &
                                 TAM_F_TISSUE = 4, TAM_F_THRESTIME = 5, TAM_F_KAPPA = 6, TAM_F_DENSITY = 7, &
                                 TAM_F_HEATCAP = 8, TAM_F_COEFF = 9, TAM_F_ALPHA = 10, TAM_F_Q = 11, &
                                 TAM_F_WATER = 12, TAM_F_MATERIAL = 13

    ! res/input.params in file order, then the grid and run options
    type, bind(C) :: tam_params
        integer(c_int64_t) :: nphotons
        real(c_double)     :: xmax, ymax, zmax, n1, n2, total_time
        integer(c_int32_t) :: loops
        real(c_double)     :: repetition_rate_1, power, energy_per_pixel, ablate_temp
        integer(c_int32_t) :: pulses_to_do, pulse_type
        integer(c_int32_t) :: nxg, nyg, nzg, numproc, mode, precision, device
    end type

    ! module Heat scalars of the reference (src/3dFD.f90:7-12)
    type, bind(C) :: tam_state
        real(c_double)     :: time, delt, total_time, pulse_count, repetition_count, laser_on
        real(c_double)     :: pulse_length, real_pulse_length, volume_voxel, mass_voxel, qvapor
        real(c_double)     :: dx, dy, dz
        integer(c_int32_t) :: laser_flag, pulse_flag, pulses_done, counter
        integer(c_int64_t) :: n_ablated, mc_passes
    end type

    interface
        integer(c_int) function tam_params_default(p) bind(C)
            import
            type(tam_params), intent(out) :: p
        end function
        ! config-mode extension file; cfg is c_loc of a tam_config buffer (the C struct)
        integer(c_int) function tam_read_config(path, cfg) bind(C)
            import; character(kind=c_char), intent(in) :: path(*); type(c_ptr), value :: cfg
        end function
        integer(c_int) function tam_read_input_params(path, p) bind(C)
            import
            character(kind=c_char), intent(in) :: path(*)
            type(tam_params), intent(inout) :: p
        end function
        integer(c_int) function tam_create(p, cfg, ctx) bind(C)
            import
            type(tam_params), intent(in) :: p
            type(c_ptr), value :: cfg          ! c_null_ptr in reference mode
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function tam_destroy(ctx) bind(C)
            import
            type(c_ptr), value :: ctx
        end function
        type(c_ptr) function tam_last_error(ctx) bind(C)
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function tam_init_opt(ctx) bind(C)
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function tam_gridset(ctx, xmax, ymax, zmax) bind(C)
            import
            type(c_ptr), value :: ctx
            real(c_double), value :: xmax, ymax, zmax
        end function
        integer(c_int) function tam_init_thermal(ctx, delt) bind(C)
            import
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: delt
        end function
        integer(c_int) function tam_mc_pass(ctx, nphotons, seed, stream, jmean_out) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int64_t), value :: nphotons, seed   ! seed: the bits of a uint64
            integer(c_int32_t), value :: stream
            type(c_ptr), value :: jmean_out                ! c_loc(jmeanGLOBAL) or c_null_ptr
        end function
        integer(c_int) function tam_heat_steps(ctx, nsteps, temp_out) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: nsteps
            type(c_ptr), value :: temp_out                 ! c_loc(temp) or c_null_ptr
        end function
        integer(c_int) function tam_arrhenius(ctx) bind(C)
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function tam_update_props(ctx, ablate_temp) bind(C)
            import
            type(c_ptr), value :: ctx
            real(c_double), value :: ablate_temp
        end function
        integer(c_int) function tam_step_coupled(ctx, n, seed) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int32_t), value :: n
            integer(c_int64_t), value :: seed
        end function
        integer(c_int) function tam_run(ctx, seed, max_iters, iters) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int64_t), value :: seed, max_iters
            integer(c_int64_t), intent(out) :: iters
        end function
        integer(c_int) function tam_finalize(ctx) bind(C)
            import
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function tam_get_state(ctx, st) bind(C)
            import
            type(c_ptr), value :: ctx
            type(tam_state), intent(out) :: st
        end function
        integer(c_int) function tam_get_tallies(ctx, absorbed, reflected, transmitted) bind(C)
            import
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: absorbed, reflected, transmitted
        end function
        integer(c_int) function tam_field_bytes(ctx, field, nbytes) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            integer(c_int64_t), intent(out) :: nbytes
        end function
        integer(c_int) function tam_upload(ctx, field, host, nbytes) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            type(c_ptr), value :: host
            integer(c_int64_t), value :: nbytes
        end function
        integer(c_int) function tam_download(ctx, field, host, nbytes) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            type(c_ptr), value :: host
            integer(c_int64_t), value :: nbytes
        end function
        integer(c_int) function tam_write_output(ctx, dir) bind(C)
            import
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: dir(*)
        end function
        integer(c_int) function tam_save_state(ctx, path) bind(C)
            import
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        integer(c_int) function tam_load_state(ctx, path) bind(C)
            import
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function
        integer(c_int) function tam_device_errors(ctx, bits) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int32_t), intent(out) :: bits       ! uint32 bit set
        end function
        integer(c_int) function tam_get_timing(ctx, transport_ms, heat_ms, heat_launches) bind(C)
            import
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: transport_ms, heat_ms
            integer(c_int64_t), intent(out) :: heat_launches
        end function
        integer(c_int) function tam_set_tuning(ctx, key, val) bind(C)
            import
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: key(*)  ! e.g. "heat.zchunk"//c_null_char
            integer(c_int64_t), value :: val
        end function
        integer(c_int) function tam_autotune(ctx, packets, steps, chosen, nchosen) bind(C)
            import
            type(c_ptr), value :: ctx
            integer(c_int64_t), value :: packets
            integer(c_int32_t), value :: steps, nchosen
            integer(c_int64_t), intent(out) :: chosen(*)
        end function
        ! batches: ctxs is an array of the instances' c_ptr handles
        integer(c_int) function tam_batch_step_coupled(ctxs, n, iters, seeds) bind(C)
            import
            type(c_ptr), intent(in) :: ctxs(*)
            integer(c_int32_t), value :: n, iters
            integer(c_int64_t), intent(in) :: seeds(*)    ! the bits of uint64 seeds
        end function
        integer(c_int) function tam_batch_heat_steps(ctxs, n, nsteps) bind(C)
            import
            type(c_ptr), intent(in) :: ctxs(*)
            integer(c_int32_t), value :: n, nsteps
        end function
        integer(c_int) function tam_batch_run(ctxs, n, seeds, max_iters, iters) bind(C)
            import
            type(c_ptr), intent(in) :: ctxs(*)
            integer(c_int32_t), value :: n
            integer(c_int64_t), intent(in) :: seeds(*)
            integer(c_int64_t), value :: max_iters
            integer(c_int64_t), intent(out) :: iters(*)
        end function
        integer(c_int) function tam_batch_autotune(ctxs, n, steps, chosen, nchosen) bind(C)
            import
            type(c_ptr), intent(in) :: ctxs(*)
            integer(c_int32_t), value :: n, steps, nchosen
            integer(c_int64_t), intent(out) :: chosen(*)
        end function
        ! one MC pass of every instance; nphotons and streams may be c_null_ptr
        ! (each context's nphotons x numproc, its count of passes)
        integer(c_int) function tam_batch_mc_pass(ctxs, n, nphotons, seeds, streams) bind(C)
            import
            type(c_ptr), intent(in) :: ctxs(*)
            integer(c_int32_t), value :: n
            type(c_ptr), value :: nphotons
            integer(c_int64_t), intent(in) :: seeds(*)
            type(c_ptr), value :: streams
        end function
        integer(c_int) function tam_measure_tally_atomics(cells, fp32, per_second) bind(C)
            import
            integer(c_int64_t), value :: cells
            integer(c_int32_t), value :: fp32
            real(c_double), intent(out) :: per_second
        end function
    end interface
end module tam_gpu
