! pqdts_cuda_mod -- iso_c_binding interface of libpqdts_cuda.so for a Fortran
! host such as program pqdts (pqdts.f90).  Declarations mirror
! include/pqdts_cuda.h one to one; arrays are passed as in the reference
! (X(M,N) and P(N,D) column-major, real64), indices 0-based, every function
! returns 0 on success or a negative error code.
!
! Build (needs a Fortran compiler):
!   gfortran -c pqdts_cuda_mod.f90
!   gfortran ... pqdts.f90 pqdts_cuda_mod.o -L<dir> -lpqdts_cuda -Wl,-rpath,<dir>
module pqdts_cuda_mod
  use iso_c_binding, only: c_int32_t, c_int64_t, c_double, c_ptr, c_funptr, c_char
  implicit none

  integer(c_int32_t), parameter :: PQDTS_FP64 = 0, PQDTS_MIXED = 1

  interface
    integer(c_int32_t) function pqdts_cuda_create(device, ctx) bind(C, name="pqdts_cuda_create")
      import :: c_int32_t, c_ptr
      integer(c_int32_t), value :: device
      type(c_ptr) :: ctx
    end function

    integer(c_int32_t) function pqdts_cuda_destroy(ctx) bind(C, name="pqdts_cuda_destroy")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
    end function

    integer(c_int32_t) function pqdts_cuda_last_error(ctx, buf, len) bind(C, name="pqdts_cuda_last_error")
      import :: c_int32_t, c_int64_t, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char) :: buf(*)
      integer(c_int64_t), value :: len
    end function

    ! name: "graphs" or "autotune" (NUL-terminated, e.g. "graphs"//c_null_char)
    integer(c_int32_t) function pqdts_cuda_set_option(ctx, name, value) bind(C, name="pqdts_cuda_set_option")
      import :: c_int32_t, c_int64_t, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char) :: name(*)
      integer(c_int64_t), value :: value
    end function

    integer(c_int32_t) function pqdts_cuda_get_option(ctx, name, value) bind(C, name="pqdts_cuda_get_option")
      import :: c_int32_t, c_int64_t, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char) :: name(*)
      integer(c_int64_t) :: value
    end function

    integer(c_int32_t) function pqdts_cuda_set_verbose(ctx, verbose) bind(C, name="pqdts_cuda_set_verbose")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: verbose
    end function

    ! replaces read_sparse_from_python + band build + P assembly (pqdts.f90:1318-1538)
    integer(c_int32_t) function pqdts_cuda_set_problem_coo(ctx, M, N, D, nnzF, F_row, F_col, F_val, &
                                                           nnzP, P_row, P_col, P_val, gamma, precision) &
      bind(C, name="pqdts_cuda_set_problem_coo")
      import :: c_int32_t, c_int64_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: M, N, D, nnzF, nnzP
      integer(c_int32_t) :: F_row(*), F_col(*), P_row(*), P_col(*)
      real(c_double) :: F_val(*), P_val(*)
      real(c_double), value :: gamma
      integer(c_int32_t), value :: precision
    end function

    ! replaces the Frows bands + dense P (pqdts.f90:77-83, 1528)
    integer(c_int32_t) function pqdts_cuda_set_problem(ctx, M, N, D, band_lo, band_hi, band_vals, P_ND, &
                                                       gamma, precision) bind(C, name="pqdts_cuda_set_problem")
      import :: c_int32_t, c_int64_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: M, N, D
      integer(c_int64_t) :: band_lo(*), band_hi(*)
      real(c_double) :: band_vals(*), P_ND(*)
      real(c_double), value :: gamma
      integer(c_int32_t), value :: precision
    end function

    integer(c_int32_t) function pqdts_cuda_set_x(ctx, X) bind(C, name="pqdts_cuda_set_x")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: X(*)
    end function

    integer(c_int32_t) function pqdts_cuda_get_x(ctx, X) bind(C, name="pqdts_cuda_get_x")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: X(*)
    end function

    integer(c_int32_t) function pqdts_cuda_set_space(ctx, fullspace, maxr) bind(C, name="pqdts_cuda_set_space")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: fullspace
      integer(c_int32_t) :: maxr(*)
    end function

    ! subroutine L(X, val), pqdts.f90:917
    integer(c_int32_t) function pqdts_cuda_L(ctx, val) bind(C, name="pqdts_cuda_L")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: val
    end function

    ! subroutine dL(X, dLdX), pqdts.f90:975
    integer(c_int32_t) function pqdts_cuda_dL(ctx, G) bind(C, name="pqdts_cuda_dL")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: G(*)
    end function

    ! subroutine BF(dd, BX), pqdts.f90:246
    integer(c_int32_t) function pqdts_cuda_BF(ctx, V, HV) bind(C, name="pqdts_cuda_BF")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: V(*), HV(*)
    end function

    ! BF in the mixed-precision solver's FP32 arithmetic (PQDTS_MIXED problems)
    integer(c_int32_t) function pqdts_cuda_BF32(ctx, V, HV) bind(C, name="pqdts_cuda_BF32")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: V(*), HV(*)
    end function

    ! subroutine Bdiag(BD), pqdts.f90:208
    integer(c_int32_t) function pqdts_cuda_Bdiag(ctx, BD) bind(C, name="pqdts_cuda_Bdiag")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: BD(*)
    end function

    ! function pdot(a, b), pqdts.f90:589: sum(a*b) in the reference's order
    integer(c_int32_t) function pqdts_cuda_pdot(ctx, A, B, res) bind(C, name="pqdts_cuda_pdot")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: A(*), B(*)
      real(c_double) :: res
    end function

    ! subroutine doproj(X), pqdts.f90:1120
    integer(c_int32_t) function pqdts_cuda_doproj(ctx) bind(C, name="pqdts_cuda_doproj")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
    end function

    ! subroutine doproj2(X, xmin), pqdts.f90:1142
    integer(c_int32_t) function pqdts_cuda_doproj2(ctx, xmin) bind(C, name="pqdts_cuda_doproj2")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: xmin
    end function

    ! subroutine conv_test(X, dLdX, tprint, conv), pqdts.f90:1034
    integer(c_int32_t) function pqdts_cuda_conv_test(ctx, conv) bind(C, name="pqdts_cuda_conv_test")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: conv
    end function

    ! simplexproj_condat_(y, x, len), condat_simplexproj.c:60
    integer(c_int32_t) function pqdts_cuda_simplexproj(ctx, y, x, len, rows) bind(C, name="pqdts_cuda_simplexproj")
      import :: c_int32_t, c_int64_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: y(*), x(*)
      integer(c_int64_t), value :: len, rows
    end function

    ! one stage of the loop at pqdts.f90:1927-2166
    integer(c_int32_t) function pqdts_cuda_run_stage(ctx, mode, oiter, maxiiter, conv_thres, output, stats) &
      bind(C, name="pqdts_cuda_run_stage")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: mode, oiter, maxiiter, output
      real(c_double), value :: conv_thres
      real(c_double) :: stats(8)
    end function

    ! the minimisation of program pqdts, pqdts.f90:1908-2167
    integer(c_int32_t) function pqdts_cuda_solve(ctx, mode, maxiiter, conv_thres, start_stage, output, &
                                                 stage_cb, user, stats) bind(C, name="pqdts_cuda_solve")
      import :: c_int32_t, c_double, c_ptr, c_funptr
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: mode, maxiiter, start_stage, output
      real(c_double), value :: conv_thres
      type(c_funptr), value :: stage_cb
      type(c_ptr), value :: user
      real(c_double) :: stats(8)
    end function

    integer(c_int32_t) function pqdts_cuda_kernel_launches(ctx, count) bind(C, name="pqdts_cuda_kernel_launches")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t) :: count
    end function

    integer(c_int32_t) function pqdts_cuda_get_bands(ctx, band_lo, band_hi, nnz) bind(C, name="pqdts_cuda_get_bands")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t) :: band_lo(*), band_hi(*), nnz
    end function

    integer(c_int32_t) function pqdts_cuda_init_x(ctx) bind(C, name="pqdts_cuda_init_x")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
    end function

    integer(c_int32_t) function pqdts_cuda_get_stream(ctx, stream) bind(C, name="pqdts_cuda_get_stream")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr) :: stream
    end function

    integer(c_int32_t) function pqdts_cuda_transfer_bytes(ctx, h2d, d2h) bind(C, name="pqdts_cuda_transfer_bytes")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int64_t) :: h2d, d2h
    end function

    integer(c_int32_t) function pqdts_cuda_get_maxr(ctx, maxr) bind(C, name="pqdts_cuda_get_maxr")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int32_t) :: maxr(*)
    end function

    ! redO local part, pqdts.f90:707-736: O(N,D) column-major
    integer(c_int32_t) function pqdts_cuda_redO(ctx, O) bind(C, name="pqdts_cuda_redO")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double) :: O(*)
    end function

    ! device pointers d_y, d_x and a cudaStream_t (no counterpart in the reference)
    integer(c_int32_t) function pqdts_cuda_simplexproj_noalloc(d_y, d_x, len, rows, stream) &
        bind(C, name="pqdts_cuda_simplexproj_noalloc")
      import :: c_int32_t, c_int64_t, c_ptr
      type(c_ptr), value :: d_y, d_x, stream
      integer(c_int64_t), value :: len, rows
    end function

    integer(c_int32_t) function pqdts_cuda_set_objective_target(ctx, target) &
        bind(C, name="pqdts_cuda_set_objective_target")
      import :: c_int32_t, c_double, c_ptr
      type(c_ptr), value :: ctx
      real(c_double), value :: target
    end function

    integer(c_int32_t) function pqdts_cuda_timer(ctx, name, seconds, count) bind(C, name="pqdts_cuda_timer")
      import :: c_int32_t, c_int64_t, c_double, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char) :: name(*)
      real(c_double) :: seconds
      integer(c_int64_t) :: count
    end function

    ! target_L: pass c_null_ptr or c_loc of n_inst targets
    integer(c_int32_t) function pqdts_cuda_solve_batch(device, n_inst, M, N, D, band_lo, band_hi, band_vals, &
                                                       band_row_offset, band_val_offset, P, P_offset, gamma, &
                                                       precision, mode, maxiiter, conv_thres, target_L, X, stats) &
        bind(C, name="pqdts_cuda_solve_batch")
      import :: c_int32_t, c_int64_t, c_double, c_ptr
      integer(c_int32_t), value :: device, n_inst, precision, mode, maxiiter
      integer(c_int64_t) :: M(*), N(*), D(*), band_lo(*), band_hi(*), band_row_offset(*), band_val_offset(*), P_offset(*)
      real(c_double) :: band_vals(*), P(*), gamma(*), X(*), stats(*)
      real(c_double), value :: conv_thres
      type(c_ptr), value :: target_L
    end function

    ! the grouping pqdts_cuda_solve_batch uses (lockstep groups sharing F); host only
    integer(c_int32_t) function pqdts_cuda_batch_groups(n_inst, M, N, D, band_lo, band_hi, band_vals, &
                                                        band_row_offset, band_val_offset, group_of) &
        bind(C, name="pqdts_cuda_batch_groups")
      import :: c_int32_t, c_int64_t, c_double
      integer(c_int32_t), value :: n_inst
      integer(c_int64_t) :: M(*), N(*), D(*), band_lo(*), band_hi(*), band_row_offset(*), band_val_offset(*)
      real(c_double) :: band_vals(*)
      integer(c_int32_t) :: group_of(*)
    end function

    ! smoothing of a restart state, pqdts.f90:1877-1902 (host memory, no context)
    integer(c_int32_t) function pqdts_cuda_smooth(M, N, smo_fact, X) bind(C, name="pqdts_cuda_smooth")
      import :: c_int32_t, c_int64_t, c_double
      integer(c_int64_t), value :: M, N
      real(c_double), value :: smo_fact
      real(c_double) :: X(*)
    end function
  end interface
end module pqdts_cuda_mod
