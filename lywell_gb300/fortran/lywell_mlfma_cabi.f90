! ISO_C_BINDING interface to liblywell_mlfma.so (include/lywell_mlfma.h).
!
! A MLFMAxwell host (gabsantamaria/lywell, Fortran 90) keeps its own geometry
! arrays and calls these in place of its module procedures:
!
!   inicializar_MLFMA (modMLFMA.f90:113)    -> mlf_init
!   MatxVec_MLFMA     (modMLFMA.f90:1901)   -> mlf_matvec      (see matxvec_gpu below)
!   crear_precond/ilu0C (main.f90:851, modIterativo.f90:1805) -> mlf_ilu0
!   lusol0C           (modIterativo.f90:504)-> mlf_ilu0_solve
!   CGSold            (modIterativo.f90:331)-> mlf_cgs
!   generar_onda      (main.f90:1488)       -> mlf_excitation
!   sigmaRCS          (modRCS.f90:91)       -> mlf_rcs
!   destruir_MLFMA    (modMLFMA.f90:85)     -> mlf_free
!
! Arrays keep the host's layout: complex(8) vectors, (3,N) real(8) geometry,
! 1-based integer(4) index arrays.  Every function returns 0 on success.
module lywell_mlfma_cabi
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: MLF_OK = 0, MLF_E_ARG = -1, MLF_E_TOO_SMALL = -2, MLF_E_CUDA = -3
    integer(c_int), parameter :: MLF_FLAG_LEGENDRE_RECURRENCE = 1, MLF_FLAG_DENSE_MOM = 2, MLF_FLAG_FMM = 4
    integer(c_int), parameter :: MLF_PRECOND_NONE = 0, MLF_PRECOND_ILU0 = 1, MLF_PRECOND_NEARINV = 2

    ! context used by matxvec_gpu (the reference's module state is single-instance too)
    type(c_ptr) :: mlf_current = c_null_ptr

    interface
        integer(c_int) function mlf_rwg_build(tris, T, N_out, P_out, p_coord, t_p, e_p, e_t, e_po, &
                                              e_long, e_centro, t_area, t_baric, t_baric_sub) bind(C)
            import :: c_int, c_double, c_ptr
            real(c_double), intent(in) :: tris(*)
            integer(c_int), value :: T
            integer(c_int), intent(out) :: N_out, P_out
            type(c_ptr), value :: p_coord, t_p, e_p, e_t, e_po, e_long, e_centro, t_area, t_baric, t_baric_sub
        end function

        integer(c_int) function mlf_init(ctx, e_centro, N, e_t, e_po, e_long, t_area, t_baric, t_baric_sub, &
                                         p_coord, t_p, e_p, P, T, t_normal, lambda, ladomax, flags) bind(C)
            import :: c_int, c_double, c_ptr
            type(c_ptr), intent(out) :: ctx
            real(c_double), intent(in) :: e_centro(3, *), e_long(*), t_area(*), t_baric(3, *), &
                                          t_baric_sub(3, 9, *), p_coord(3, *), t_normal(3, *)
            integer(c_int), value :: N, P, T, flags
            integer(c_int), intent(in) :: e_t(2, *), e_po(2, *), t_p(3, *), e_p(2, *)
            real(c_double), value :: lambda, ladomax
        end function

        subroutine mlf_free(ctx) bind(C)
            import :: c_ptr
            type(c_ptr), value :: ctx
        end subroutine

        type(c_ptr) function mlf_last_error(ctx) bind(C)
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function

        integer(c_int) function mlf_matvec(ctx, x, y, nrhs, ld) bind(C)
            import :: c_int, c_double_complex, c_ptr
            type(c_ptr), value :: ctx
            complex(c_double_complex), intent(in) :: x(*)
            complex(c_double_complex), intent(out) :: y(*)
            integer(c_int), value :: nrhs, ld
        end function

        integer(c_int) function mlf_near_csr(ctx, nnz, a, ja, ia) bind(C)
            import :: c_int, c_long_long, c_ptr
            type(c_ptr), value :: ctx
            integer(c_long_long), intent(out) :: nnz
            type(c_ptr), value :: a, ja, ia
        end function

        integer(c_int) function mlf_ilu0(ctx, ierr_row) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: ierr_row
        end function

        ! ilu0C(n, a, ja, ia, alu, jlu, ju, iw, ierr) on host arrays (iw kept inside)
        integer(c_int) function mlf_ilu0_csr(n, a, ja, ia, alu, jlu, ju, ierr) bind(C)
            import :: c_int, c_float_complex
            integer(c_int), value :: n
            complex(c_float_complex), intent(in) :: a(*)
            integer(c_int), intent(in) :: ja(*), ia(*)
            complex(c_float_complex), intent(out) :: alu(*)
            integer(c_int), intent(out) :: jlu(*), ju(*), ierr
        end function

        ! overwrite Zesparcida_MLFMA's values on the device
        integer(c_int) function mlf_set_near_values(ctx, a) bind(C)
            import :: c_int, c_float_complex, c_ptr
            type(c_ptr), value :: ctx
            complex(c_float_complex), intent(in) :: a(*)
        end function

        integer(c_int) function mlf_set_stagnation(ctx, window) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: window
        end function

        integer(c_int) function mlf_ilu0_solve(ctx, y, x, nrhs) bind(C)
            import :: c_int, c_double_complex, c_ptr
            type(c_ptr), value :: ctx
            complex(c_double_complex), intent(in) :: y(*)
            complex(c_double_complex), intent(out) :: x(*)
            integer(c_int), value :: nrhs
        end function

        integer(c_int) function mlf_cgs(ctx, b, x0, tol, maxit, nrhs, x, iters, relres, precond_kind, &
                                        status_out) bind(C)
            import :: c_int, c_double, c_double_complex, c_ptr
            type(c_ptr), value :: ctx
            complex(c_double_complex), intent(in) :: b(*)
            type(c_ptr), value :: x0
            real(c_double), value :: tol
            integer(c_int), value :: maxit, nrhs, precond_kind
            complex(c_double_complex), intent(out) :: x(*)
            integer(c_int), intent(out) :: iters(*), status_out(*)
            real(c_double), intent(out) :: relres(*)
        end function

        integer(c_int) function mlf_ilut(ctx, fill_in_prc, droptol, ierr) bind(C)
            import :: c_int, c_double, c_ptr
            type(c_ptr), value :: ctx
            real(c_double), value :: fill_in_prc, droptol
            integer(c_int), intent(out) :: ierr
        end function

        integer(c_int) function mlf_nearinv(ctx, bad_box) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: bad_box
        end function

        integer(c_int) function mlf_solve(ctx, b, x0, tol, maxit, nrhs, precond_kind, mode, inner_tol, &
                                          x, iters, relres, status_out, outer) bind(C)
            import :: c_int, c_double, c_double_complex, c_ptr
            type(c_ptr), value :: ctx
            complex(c_double_complex), intent(in) :: b(*)
            type(c_ptr), value :: x0
            real(c_double), value :: tol, inner_tol
            integer(c_int), value :: maxit, nrhs, precond_kind, mode
            complex(c_double_complex), intent(out) :: x(*)
            integer(c_int), intent(out) :: iters(*), status_out(*), outer
            real(c_double), intent(out) :: relres(*)
        end function

        integer(c_int) function mlf_monostatic(ctx, nang, phis, hh, ctte_re, ctte_im, tol, maxit, &
                                               precond_kind, mode, block, sigma, iters, status_out) bind(C)
            import :: c_int, c_double, c_ptr
            type(c_ptr), value :: ctx, phis
            integer(c_int), value :: nang, hh, maxit, precond_kind, mode, block
            real(c_double), value :: ctte_re, ctte_im, tol
            real(c_double), intent(out) :: sigma(*)
            integer(c_int), intent(out) :: iters(*), status_out(*)
        end function

        integer(c_int) function mlf_excitation(ctx, dirs, pols, ctte_re, ctte_im, nrhs, b) bind(C)
            import :: c_int, c_double, c_double_complex, c_ptr
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: dirs(3, *)
            complex(c_double_complex), intent(in) :: pols(3, *)
            real(c_double), value :: ctte_re, ctte_im
            integer(c_int), value :: nrhs
            complex(c_double_complex), intent(out) :: b(*)
        end function

        integer(c_int) function mlf_rcs(ctx, I, pol, ctte_re, ctte_im, theta, phi, nang, sigma) bind(C)
            import :: c_int, c_double, c_double_complex, c_ptr
            type(c_ptr), value :: ctx
            complex(c_double_complex), intent(in) :: I(*), pol(3)
            real(c_double), value :: ctte_re, ctte_im
            real(c_double), intent(in) :: theta(*), phi(*)
            integer(c_int), value :: nang
            real(c_double), intent(out) :: sigma(*)
        end function

        ! tuning of the mixed-precision and batched paths (optional; no counterpart
        ! in the reference)
        integer(c_int) function mlf_autotune_block(ctx, candidates, ncand, best_block, best_cols, &
                                                   best_engine, per_rhs_ms) bind(C)
            import :: c_int, c_float, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), intent(in) :: candidates(*)
            integer(c_int), value :: ncand
            integer(c_int), intent(out) :: best_block, best_cols, best_engine
            real(c_float), intent(out) :: per_rhs_ms(*)
        end function

        integer(c_int) function mlf_set_block_engine(ctx, engine, cols) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: engine, cols
        end function

        integer(c_int) function mlf_set_gmres_restart(ctx, m) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: m
        end function

        integer(c_int) function mlf_set_gs_passes(ctx, passes) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: passes
        end function

        integer(c_int) function mlf_set_basis_precision(ctx, bits) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: bits
        end function

        integer(c_int) function mlf_set_translation_group(ctx, boxes, cols) bind(C)
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: boxes, cols
        end function
    end interface

contains

    ! Drop-in for the procedure argument of CGSold (modIterativo.f90:357-363):
    ! set mlf_current to the context returned by mlf_init first.
    function matxvec_gpu(vecX) result(res)
        complex(kind=8), intent(in), dimension(:) :: vecX
        complex(kind=8), dimension(size(vecX, 1)) :: res
        integer(c_int) :: st
        st = mlf_matvec(mlf_current, vecX, res, 1_c_int, int(size(vecX, 1), c_int))
        if (st /= MLF_OK) stop 'mlf_matvec failed'
    end function

end module lywell_mlfma_cabi
