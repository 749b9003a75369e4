! s2d_mod.F90 -- ISO_C_BINDING interface to libspectral2d_gb300 (include/s2d.h).
!
! The module a maintainer of the Fortran driver (src/Spectral2D.F90) adds to
! call the GB300 time step.  Scalars pass by VALUE, arrays as assumed-size
! COMPLEX(C_DOUBLE_COMPLEX) in the driver's own (cISize, nyG) layout, the
! handle as TYPE(C_PTR).  Every function returns S2D_OK (0) or a negative
! S2D_ERR_* code.  Not compiled in this repository (no Fortran compiler on the
! build machines); the derived types mirror the C structs field by field.
MODULE s2d_m
   USE ISO_C_BINDING
   IMPLICIT NONE

   INTEGER(C_INT), PARAMETER :: S2D_OK = 0
   INTEGER(C_INT), PARAMETER :: S2D_ERR_INVALID = -1, S2D_ERR_CUDA = -2
   INTEGER(C_INT), PARAMETER :: S2D_ERR_NONFINITE = -3, S2D_ERR_TIMEOUT = -4
   INTEGER(C_INT), PARAMETER :: S2D_ERR_UNSUPPORTED = -5, S2D_ERR_NOMEM = -6
   INTEGER(C_INT32_T), PARAMETER :: S2D_DEALIAS_3_2_RULE = 1
   INTEGER(C_INT32_T), PARAMETER :: S2D_FP64 = 0, S2D_FP32 = 1
   INTEGER(C_INT32_T), PARAMETER :: S2D_NL_BASDEVANT = 0, S2D_NL_CONSERVATIVE = 1
   INTEGER(C_INT32_T), PARAMETER :: S2D_SPECTRUM_SCHUMANN = 0, S2D_SPECTRUM_K4_GAUSS = 1

   TYPE, BIND(C) :: s2d_config_t
      INTEGER(C_INT32_T) :: nx, ny, dealias, precision
      REAL(C_DOUBLE) :: nu, alpha, forcing_amp
      INTEGER(C_INT32_T) :: forcing_k, device, nonlinear_form
   END TYPE s2d_config_t

   TYPE, BIND(C) :: s2d_grid_t
      INTEGER(C_INT32_T) :: nx, ny, dealias, nxG, nyG
      INTEGER(C_INT32_T) :: kxLG, kyLG, kxMG, kyMG, kxLU, kyLU, kxMU, kyMU
      REAL(C_DOUBLE) :: kMax
      INTEGER(C_INT32_T) :: rISize, cISize
   END TYPE s2d_grid_t

   INTERFACE
      INTEGER(C_INT) FUNCTION s2d_get_grid_size(nx, ny, dealias, grid) BIND(C, NAME='s2d_get_grid_size')
         IMPORT :: C_INT, C_INT32_T, s2d_grid_t
         INTEGER(C_INT32_T), VALUE :: nx, ny, dealias
         TYPE(s2d_grid_t), INTENT(OUT) :: grid
      END FUNCTION s2d_get_grid_size

      INTEGER(C_INT) FUNCTION s2d_create(cfg, h) BIND(C, NAME='s2d_create')
         IMPORT :: C_INT, C_PTR, s2d_config_t
         TYPE(s2d_config_t), INTENT(IN) :: cfg
         TYPE(C_PTR), INTENT(OUT) :: h
      END FUNCTION s2d_create

      SUBROUTINE s2d_destroy(h) BIND(C, NAME='s2d_destroy')
         IMPORT :: C_PTR
         TYPE(C_PTR), VALUE :: h
      END SUBROUTINE s2d_destroy

      INTEGER(C_INT) FUNCTION s2d_set_state(h, wC, cISize, nyG) BIND(C, NAME='s2d_set_state')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE_COMPLEX
         TYPE(C_PTR), VALUE :: h
         COMPLEX(C_DOUBLE_COMPLEX), INTENT(IN) :: wC(*)
         INTEGER(C_INT32_T), VALUE :: cISize, nyG
      END FUNCTION s2d_set_state

      INTEGER(C_INT) FUNCTION s2d_get_state(h, wC, psiC, cISize, nyG) BIND(C, NAME='s2d_get_state')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE_COMPLEX
         TYPE(C_PTR), VALUE :: h
         COMPLEX(C_DOUBLE_COMPLEX), INTENT(OUT) :: wC(*), psiC(*)
         INTEGER(C_INT32_T), VALUE :: cISize, nyG
      END FUNCTION s2d_get_state

      INTEGER(C_INT) FUNCTION s2d_integrate_one_step(h, dt) BIND(C, NAME='s2d_integrate_one_step')
         IMPORT :: C_INT, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         REAL(C_DOUBLE), VALUE :: dt
      END FUNCTION s2d_integrate_one_step

      INTEGER(C_INT) FUNCTION s2d_integrate_steps(h, n, dt) BIND(C, NAME='s2d_integrate_steps')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         INTEGER(C_INT32_T), VALUE :: n
         REAL(C_DOUBLE), VALUE :: dt
      END FUNCTION s2d_integrate_steps

      INTEGER(C_INT) FUNCTION s2d_integrate_one_step_host(h, wC, psiC, cISize, nyG, dt) &
            BIND(C, NAME='s2d_integrate_one_step_host')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE, C_DOUBLE_COMPLEX
         TYPE(C_PTR), VALUE :: h
         COMPLEX(C_DOUBLE_COMPLEX), INTENT(INOUT) :: wC(*)
         COMPLEX(C_DOUBLE_COMPLEX), INTENT(OUT) :: psiC(*)
         INTEGER(C_INT32_T), VALUE :: cISize, nyG
         REAL(C_DOUBLE), VALUE :: dt
      END FUNCTION s2d_integrate_one_step_host

      INTEGER(C_INT) FUNCTION s2d_compute_rhs(h, dW, cISize, nyG) BIND(C, NAME='s2d_compute_rhs')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE_COMPLEX
         TYPE(C_PTR), VALUE :: h
         COMPLEX(C_DOUBLE_COMPLEX), INTENT(OUT) :: dW(*)
         INTEGER(C_INT32_T), VALUE :: cISize, nyG
      END FUNCTION s2d_compute_rhs

      INTEGER(C_INT) FUNCTION s2d_spectrum_bins(h) BIND(C, NAME='s2d_spectrum_bins')
         IMPORT :: C_INT, C_PTR
         TYPE(C_PTR), VALUE :: h
      END FUNCTION s2d_spectrum_bins

      INTEGER(C_INT) FUNCTION s2d_spectrum(h, Ek, nbins, tke, eps, enstDiss) BIND(C, NAME='s2d_spectrum')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         REAL(C_DOUBLE), INTENT(OUT) :: Ek(*)
         INTEGER(C_INT32_T), VALUE :: nbins
         REAL(C_DOUBLE), INTENT(OUT) :: tke, eps, enstDiss
      END FUNCTION s2d_spectrum

      INTEGER(C_INT) FUNCTION s2d_minmax_abs(h, out) BIND(C, NAME='s2d_minmax_abs')
         IMPORT :: C_INT, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         REAL(C_DOUBLE), INTENT(OUT) :: out(4)
      END FUNCTION s2d_minmax_abs

      INTEGER(C_INT) FUNCTION s2d_set_taylor_green(h) BIND(C, NAME='s2d_set_taylor_green')
         IMPORT :: C_INT, C_PTR
         TYPE(C_PTR), VALUE :: h
      END FUNCTION s2d_set_taylor_green

      INTEGER(C_INT) FUNCTION s2d_set_turbulent(h, seed, spectrum, k0, urms, tke) BIND(C, NAME='s2d_set_turbulent')
         IMPORT :: C_INT, C_INT32_T, C_INT64_T, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         INTEGER(C_INT64_T), VALUE :: seed
         INTEGER(C_INT32_T), VALUE :: spectrum
         REAL(C_DOUBLE), VALUE :: k0, urms, tke
      END FUNCTION s2d_set_turbulent

      INTEGER(C_INT) FUNCTION s2d_cfl_dt(h, cfl, dt) BIND(C, NAME='s2d_cfl_dt')
         IMPORT :: C_INT, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         REAL(C_DOUBLE), VALUE :: cfl
         REAL(C_DOUBLE), INTENT(OUT) :: dt
      END FUNCTION s2d_cfl_dt

      INTEGER(C_INT) FUNCTION s2d_check_finite(h) BIND(C, NAME='s2d_check_finite')
         IMPORT :: C_INT, C_PTR
         TYPE(C_PTR), VALUE :: h
      END FUNCTION s2d_check_finite

      INTEGER(C_INT) FUNCTION s2d_synchronize(h) BIND(C, NAME='s2d_synchronize')
         IMPORT :: C_INT, C_PTR
         TYPE(C_PTR), VALUE :: h
      END FUNCTION s2d_synchronize

      ! Analysis (src/Analysis.F90:135-225): x and y vorticity-gradient skewness
      INTEGER(C_INT) FUNCTION s2d_skewness(h, xSkew, ySkew) BIND(C, NAME='s2d_skewness')
         IMPORT :: C_INT, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         REAL(C_DOUBLE), INTENT(OUT) :: xSkew, ySkew
      END FUNCTION s2d_skewness

      INTEGER(C_INT) FUNCTION s2d_enstrophy(h, enst) BIND(C, NAME='s2d_enstrophy')
         IMPORT :: C_INT, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         REAL(C_DOUBLE), INTENT(OUT) :: enst
      END FUNCTION s2d_enstrophy

      ! WriteRestart (src/IO.F90:98-143): root_<num>.bin + root_<num>.xmf
      INTEGER(C_INT) FUNCTION s2d_write_restart(h, root, num, nadv, time) BIND(C, NAME='s2d_write_restart')
         IMPORT :: C_INT, C_PTR, C_CHAR, C_INT32_T, C_INT64_T, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         CHARACTER(KIND=C_CHAR), DIMENSION(*), INTENT(IN) :: root   ! NUL-terminated
         INTEGER(C_INT32_T), VALUE :: num
         INTEGER(C_INT64_T), VALUE :: nadv
         REAL(C_DOUBLE), VALUE :: time
      END FUNCTION s2d_write_restart

      INTEGER(C_INT) FUNCTION s2d_read_restart(h, path, nadv, time) BIND(C, NAME='s2d_read_restart')
         IMPORT :: C_INT, C_PTR, C_CHAR, C_INT64_T, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         CHARACTER(KIND=C_CHAR), DIMENSION(*), INTENT(IN) :: path
         INTEGER(C_INT64_T), INTENT(OUT) :: nadv
         REAL(C_DOUBLE), INTENT(OUT) :: time
      END FUNCTION s2d_read_restart

      INTEGER(C_INT) FUNCTION s2d_checkpoint_write(h, path, nadv, time) BIND(C, NAME='s2d_checkpoint_write')
         IMPORT :: C_INT, C_PTR, C_CHAR, C_INT64_T, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         CHARACTER(KIND=C_CHAR), DIMENSION(*), INTENT(IN) :: path
         INTEGER(C_INT64_T), VALUE :: nadv
         REAL(C_DOUBLE), VALUE :: time
      END FUNCTION s2d_checkpoint_write

      INTEGER(C_INT) FUNCTION s2d_checkpoint_read(h, path, nadv, time) BIND(C, NAME='s2d_checkpoint_read')
         IMPORT :: C_INT, C_PTR, C_CHAR, C_INT64_T, C_DOUBLE
         TYPE(C_PTR), VALUE :: h
         CHARACTER(KIND=C_CHAR), DIMENSION(*), INTENT(IN) :: path
         INTEGER(C_INT64_T), INTENT(OUT) :: nadv
         REAL(C_DOUBLE), INTENT(OUT) :: time
      END FUNCTION s2d_checkpoint_read

      ! One run over several MPI ranks (the reference's slab decomposition,
      ! src/Alloc.F90:90-100): per RK3 stage, phases 0, 1, 2 with an
      ! MPI_Alltoallv of the slab's device buffers after phases 0 and 1
      ! (CUDA-aware MPI), byte counts from s2d_slab_exchange.
      INTEGER(C_INT) FUNCTION s2d_slab_partition(nx, nranks, rank, part) BIND(C, NAME='s2d_slab_partition')
         IMPORT :: C_INT, C_INT32_T
         INTEGER(C_INT32_T), VALUE :: nx, nranks, rank
         INTEGER(C_INT32_T), DIMENSION(4), INTENT(OUT) :: part   ! kx0, nkx, y0, ny
      END FUNCTION s2d_slab_partition

      INTEGER(C_INT) FUNCTION s2d_slab_create(cfg, rank, nranks, s) BIND(C, NAME='s2d_slab_create')
         IMPORT :: C_INT, C_INT32_T, C_PTR, s2d_config_t
         TYPE(s2d_config_t), INTENT(IN) :: cfg
         INTEGER(C_INT32_T), VALUE :: rank, nranks
         TYPE(C_PTR), INTENT(OUT) :: s
      END FUNCTION s2d_slab_create

      SUBROUTINE s2d_slab_destroy(s) BIND(C, NAME='s2d_slab_destroy')
         IMPORT :: C_PTR
         TYPE(C_PTR), VALUE :: s
      END SUBROUTINE s2d_slab_destroy

      INTEGER(C_INT) FUNCTION s2d_slab_handle(s, h) BIND(C, NAME='s2d_slab_handle')
         IMPORT :: C_INT, C_PTR
         TYPE(C_PTR), VALUE :: s
         TYPE(C_PTR), INTENT(OUT) :: h
      END FUNCTION s2d_slab_handle

      INTEGER(C_INT) FUNCTION s2d_slab_exchange(s, xchg, sendbuf, recvbuf, sendBytes, recvBytes) &
            BIND(C, NAME='s2d_slab_exchange')
         IMPORT :: C_INT, C_INT32_T, C_INT64_T, C_PTR
         TYPE(C_PTR), VALUE :: s
         INTEGER(C_INT32_T), VALUE :: xchg
         TYPE(C_PTR), INTENT(OUT) :: sendbuf, recvbuf
         INTEGER(C_INT64_T), DIMENSION(*), INTENT(OUT) :: sendBytes, recvBytes
      END FUNCTION s2d_slab_exchange

      INTEGER(C_INT) FUNCTION s2d_slab_phase(s, stage, phase, dt) BIND(C, NAME='s2d_slab_phase')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE
         TYPE(C_PTR), VALUE :: s
         INTEGER(C_INT32_T), VALUE :: stage, phase
         REAL(C_DOUBLE), VALUE :: dt
      END FUNCTION s2d_slab_phase

      INTEGER(C_INT) FUNCTION s2d_slab_get_columns(s, wC, psiC, cISize, nyG) BIND(C, NAME='s2d_slab_get_columns')
         IMPORT :: C_INT, C_INT32_T, C_PTR, C_DOUBLE_COMPLEX
         TYPE(C_PTR), VALUE :: s
         INTEGER(C_INT32_T), VALUE :: cISize, nyG
         COMPLEX(C_DOUBLE_COMPLEX), DIMENSION(cISize, nyG), INTENT(INOUT) :: wC, psiC
      END FUNCTION s2d_slab_get_columns
   END INTERFACE
END MODULE s2d_m
