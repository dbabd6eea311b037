! gturbo_c.f90 -- ISO_C_BINDING interface to the C-ABI of gturbo.h, for the Fortran driver.
!
! Add this module next to src/modules.f90 and link with -lgturbo_gb300. Every interface below
! matches one declaration of gturbo.h; the routines named in the comments are the reference's
! call points that each one replaces. Field arguments are DEVICE arrays: pass them inside
! `!$acc host_data use_device(...)` (as the reference does for cuFFT in src/fft_dir.f90:11-13).
! Host arrays are marked as such. Every function returns 0 (GT_OK) or an error code, whose
! message gt_last_error returns as a C string.
module gturbo_c
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: GT_OK = 0, GT_ERR_ARG = 1, GT_ERR_CUDA = 2, GT_ERR_NFORC = 3, &
                               GT_ERR_STATE = 4, GT_ERR_NOMEM = 5, GT_ERR_NONFINITE = 6
  integer(c_int), parameter :: GT_NVARIANTS = 6

  ! struct gt_params: params.dat plus the derived switches (src/inieuler.f90:13-36)
  type, bind(C) :: gt_params
    integer(c_int32_t) :: n, rko, truncate, split
    real(c_double) :: xlx, xly, nu, alpnu, mu, alpmu, alpv, dt, rtrunc, famp, k1f, k2f
    integer(c_int32_t) :: ny, ny_pad_
  end type

  interface
    ! inieuler + defk + iniforcing (src/inieuler.f90:22-87, src/defk.f90, src/iniforcing.f90)
    integer(c_int) function gt_create(p, h) bind(C, name="gt_create")
      import :: gt_params, c_int, c_ptr
      type(gt_params), intent(in) :: p
      type(c_ptr), intent(out) :: h
    end function
    integer(c_int) function gt_destroy(h) bind(C, name="gt_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    ! the stream of OpenACC's async queue: acc_get_cuda_stream(acc_async_sync)
    integer(c_int) function gt_set_stream(h, s) bind(C, name="gt_set_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: h, s
    end function
    integer(c_int) function gt_sync(h) bind(C, name="gt_sync")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function
    ! const char* gt_last_error(const gt_handle*): convert with c_f_pointer
    type(c_ptr) function gt_last_error(h) bind(C, name="gt_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function

    ! fft_dir / fft_inv (src/fft_dir.f90:1-24, src/fft_inv.f90:1-16)
    integer(c_int) function gt_fft_dir(h, z) bind(C, name="gt_fft_dir")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*)
    end function
    integer(c_int) function gt_fft_inv(h, z) bind(C, name="gt_fft_inv")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*)
    end function
    ! the real(4) physical field of a dump (src/write.f90:29-51); out: N*N real(4), DEVICE
    integer(c_int) function gt_dump_real4(h, work, out) bind(C, name="gt_dump_real4")
      import :: c_int, c_ptr, c_double, c_float
      type(c_ptr), value :: h
      real(c_double) :: work(*)
      real(c_float) :: out(*)
    end function
    ! restart: readf (src/read.f90:3-27) + fft_dir + trunc (src/main.f90:89-92); in: N*N real(4), DEVICE
    integer(c_int) function gt_load_real4(h, w, z) bind(C, name="gt_load_real4")
      import :: c_int, c_ptr, c_double, c_float
      type(c_ptr), value :: h
      real(c_float) :: w(*)
      real(c_double) :: z(*)
    end function
    ! trunc, produ, nlt (src/trunc.f90, src/produ.f90, src/nlt.f90)
    integer(c_int) function gt_trunc(h, z) bind(C, name="gt_trunc")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*)
    end function
    integer(c_int) function gt_produ(h, z, u, v) bind(C, name="gt_produ")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*), u(*), v(*)
    end function
    integer(c_int) function gt_nlt(h, z, u, v) bind(C, name="gt_nlt")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*), u(*), v(*)
    end function
    ! step / step4 (src/rkstep.f90:2-76, 82-131)
    integer(c_int) function gt_step_rk2(h, z, znl, u, v) bind(C, name="gt_step_rk2")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*), znl(*), u(*), v(*)
    end function
    integer(c_int) function gt_step_rk4(h, z, znl, znew, u, v) bind(C, name="gt_step_rk4")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*), znl(*), znew(*), u(*), v(*)
    end function
    ! forcing (src/forcing.f90:1-36); seed is a HOST integer, updated in place
    integer(c_int) function gt_forcing(h, z, seed) bind(C, name="gt_forcing")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: h
      real(c_double) :: z(*)
      integer(c_int32_t) :: seed
    end function
    ! step / step4 followed by forcing, the kick fused into the final stage (src/main.f90:100-106)
    integer(c_int) function gt_step_rk2_forced(h, z, znl, u, v, seed) bind(C, name="gt_step_rk2_forced")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: h
      real(c_double) :: z(*), znl(*), u(*), v(*)
      integer(c_int32_t) :: seed
    end function
    integer(c_int) function gt_step_rk4_forced(h, z, znl, znew, u, v, seed) &
        bind(C, name="gt_step_rk4_forced")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: h
      real(c_double) :: z(*), znl(*), znew(*), u(*), v(*)
      integer(c_int32_t) :: seed
    end function
    ! rann (src/forcing.f90:40-51), host only
    real(c_float) function gt_rann(seed) bind(C, name="gt_rann")
      import :: c_float, c_int32_t
      integer(c_int32_t) :: seed
    end function
    ! spectrum / fluxes / glob (src/diagnostics.f90); sp, sz, fle, flz, glob are HOST arrays
    integer(c_int) function gt_diag(h, z, znl, sp, sz, fle, flz, glob) bind(C, name="gt_diag")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double) :: z(*), znl(*), sp(*), sz(*), fle(*), flz(*), glob(6)
    end function
    ! the same without a handle and without allocating; outputs are DEVICE arrays
    integer(c_int) function gt_diag_static(p, z, znl, sp, sz, fle, flz, glob, s) &
        bind(C, name="gt_diag_static")
      import :: gt_params, c_int, c_ptr, c_double
      type(gt_params), intent(in) :: p
      real(c_double) :: z(*), znl(*), sp(*), sz(*), fle(*), flz(*), glob(6)
      type(c_ptr), value :: s
    end function

    ! launch variants of the nonlinear-term passes; gt_autotune times them once (after
    ! gt_create, before the time loop) and keeps the fastest. ms_per_step: GT_NVARIANTS values.
    integer(c_int) function gt_set_variant(h, variant) bind(C, name="gt_set_variant")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: h
      integer(c_int32_t), value :: variant
    end function
    integer(c_int) function gt_set_variants(h, col_variant, row_variant) bind(C, name="gt_set_variants")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: h
      integer(c_int32_t), value :: col_variant, row_variant
    end function
    ! field-split column passes (on by default where they apply)
    integer(c_int) function gt_set_col_split(h, on) bind(C, name="gt_set_col_split")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: h
      integer(c_int32_t), value :: on
    end function
    ! programmatic dependent launch of the pass kernels (on by default)
    integer(c_int) function gt_set_pdl(h, on) bind(C, name="gt_set_pdl")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: h
      integer(c_int32_t), value :: on
    end function
    integer(c_int) function gt_autotune(h, steps, ms_per_step, best) bind(C, name="gt_autotune")
      import :: c_int, c_ptr, c_int32_t, c_double
      type(c_ptr), value :: h
      integer(c_int32_t), value :: steps
      real(c_double) :: ms_per_step(*)
      integer(c_int32_t) :: best
    end function
  end interface
end module gturbo_c
