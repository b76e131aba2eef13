! qs3g_iface.f90 -- iso_c_binding interface of libqs3g.so for the QS3 Fortran
! sources.  A QS3 build links -lqs3g and `use qs3g_iface`; the bodies of the
! routines named in each comment then become these calls.  Every function
! returns 0 on success.  Scalars are passed by reference, arrays as Fortran
! arrays (contiguous, column-major).
module qs3g_iface
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: QS3G_OK = 0, QS3G_HOST = 0, QS3G_DEVICE = 1
  ! added to qs3g_trlan's precision: real Krylov vectors (k = 0 chains, U(1))
  integer(c_int), parameter :: QS3G_REAL = 8

  interface
    ! state set up by read_ip / get_combination / mk_shift_*_SQ
    integer(c_int) function qs3g_create(h, NOS, LX, LY, LZ, NOxxz, p_xxz, sJint) bind(C, name="qs3g_create")
      import :: c_ptr, c_int, c_double
      type(c_ptr) :: h
      integer(c_int) :: NOS, LX, LY, LZ, NOxxz
      integer(c_int) :: p_xxz(2, *)
      real(c_double) :: sJint(*)          ! sJint(1:NOxxz, 2:3) flattened column-major
    end function

    integer(c_int) function qs3g_destroy(h) bind(C, name="qs3g_destroy")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
    end function

    ! allocate_lists_omp_SQ (+ explist)
    integer(c_int) function qs3g_build_sector(h, NOD, KX, KY, KZ, D) bind(C, name="qs3g_build_sector")
      import :: c_ptr, c_int, c_int64_t
      type(c_ptr), value :: h
      integer(c_int) :: NOD, KX, KY, KZ
      integer(c_int64_t) :: D
    end function

    ! allocate_lists_omp_SQ with the reference's default-kind THS (main.f90:28-34);
    ! QS3G_ERANGE when THS or a list_s code does not fit
    integer(c_int) function qs3g_build_sector_i32(h, NOD, KX, KY, KZ, THS) bind(C, name="qs3g_build_sector_i32")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: NOD, KX, KY, KZ
      integer(c_int) :: THS
    end function

    integer(c_int) function qs3g_get_sector_i32(h, list_s, list_r) bind(C, name="qs3g_get_sector_i32")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      integer(c_int) :: list_s(*)
      real(c_double) :: list_r(*)
    end function

    ! a sector the Fortran side enumerated itself (allocate_lists_omp_SQ): checked
    ! against the (NOD, K) sector and adopted; default-kind and 64-bit forms
    integer(c_int) function qs3g_load_sector_i32(h, NOD, KX, KY, KZ, THS, list_s, list_r) &
        bind(C, name="qs3g_load_sector_i32")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      integer(c_int) :: NOD, KX, KY, KZ, THS
      integer(c_int) :: list_s(*)
      real(c_double) :: list_r(*)
    end function

    integer(c_int) function qs3g_load_sector(h, NOD, KX, KY, KZ, D, list_s, list_r) bind(C, name="qs3g_load_sector")
      import :: c_ptr, c_int, c_int64_t, c_double
      type(c_ptr), value :: h
      integer(c_int) :: NOD, KX, KY, KZ
      integer(c_int64_t) :: D
      integer(c_int64_t) :: list_s(*)
      real(c_double) :: list_r(*)
    end function

    ! real FP32 product (H - shift) v1 for k = 0 chain / U(1) sectors
    integer(c_int) function qs3g_hv32_real(h, v0, v1, shift, where) bind(C, name="qs3g_hv32_real")
      import :: c_ptr, c_int, c_float
      type(c_ptr), value :: h
      real(c_float) :: v0(*), v1(*)
      real(c_float) :: shift
      integer(c_int) :: where
    end function

    ! complex(8) H*v from the cached table in double-float arithmetic
    integer(c_int) function qs3g_hv_df(h, v0, v1, where) bind(C, name="qs3g_hv_df")
      import :: c_ptr, c_int, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex) :: v0(*), v1(*)
      integer(c_int) :: where
    end function

    ! cache (on = 1) or drop (on = 0) the sector's connection table
    integer(c_int) function qs3g_hv_cache(h, on, bytes) bind(C, name="qs3g_hv_cache")
      import :: c_ptr, c_int, c_int64_t
      type(c_ptr), value :: h
      integer(c_int) :: on
      integer(c_int64_t) :: bytes
    end function

    ! wall-clock limit of qs3g_trlan, and what the last qs3g_trlan did
    integer(c_int) function qs3g_set_time_limit(h, seconds) bind(C, name="qs3g_set_time_limit")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      real(c_double) :: seconds
    end function

    integer(c_int) function qs3g_trlan_stats(h, hv_fp32, hv_fp64, restarts, seconds, timed_out) &
        bind(C, name="qs3g_trlan_stats")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      integer(c_int) :: hv_fp32, hv_fp64, restarts, timed_out
      real(c_double) :: seconds
    end function

    integer(c_int) function qs3g_get_sector(h, list_s, list_r) bind(C, name="qs3g_get_sector")
      import :: c_ptr, c_int, c_int64_t, c_double
      type(c_ptr), value :: h
      integer(c_int64_t) :: list_s(*)
      real(c_double) :: list_r(*)
    end function

    ! ham_to_vec_wave_vector(v0, v1, lv, NOD, list_s, list_r, explist)
    integer(c_int) function qs3g_hv(h, v0, v1, where) bind(C, name="qs3g_hv")
      import :: c_ptr, c_int, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex) :: v0(*), v1(*)
      integer(c_int) :: where
    end function

    ! the same product on real vectors (sectors with a real symmetric H)
    integer(c_int) function qs3g_hv_real(h, v0, v1, where) bind(C, name="qs3g_hv_real")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      real(c_double) :: v0(*), v1(*)
      integer(c_int) :: where
    end function

    ! lancz_eigen_val_complex (TRLan)
    integer(c_int) function qs3g_trlan(h, NOE, NOK, NOM, maxitr, tol, precision, conv_mode, start_mode, &
        seed, start, ene, psi, iters, resid) bind(C, name="qs3g_trlan")
      import :: c_ptr, c_int, c_double, c_double_complex, c_int64_t
      type(c_ptr), value :: h
      integer(c_int) :: NOE, NOK, NOM, maxitr, precision, conv_mode, start_mode, iters
      real(c_double) :: tol, ene(*), resid(*)
      integer(c_int64_t) :: seed
      complex(c_double_complex) :: start(*), psi(*)
    end function

    ! lancz_eigen_val (plain Lanczos)
    integer(c_int) function qs3g_lanczos(h, maxitr, minitr, itrint, tol, start_mode, seed, start, ene, psi, &
        iters) bind(C, name="qs3g_lanczos")
      import :: c_ptr, c_int, c_double, c_double_complex, c_int64_t
      type(c_ptr), value :: h
      integer(c_int) :: maxitr, minitr, itrint, start_mode, iters
      real(c_double) :: tol, ene
      integer(c_int64_t) :: seed
      complex(c_double_complex) :: start(*), psi(*)
    end function

    ! calcu_Sq_a + calcu_DSF_wavevector, for nq wave vectors at once
    integer(c_int) function qs3g_dsf(h, psi, ene1, spsmsz, nq, qvec, Spos, itr_dsf, rfield, alpha, beta2, &
        norm1, E0, nlev) bind(C, name="qs3g_dsf")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex) :: psi(*)
      real(c_double) :: ene1, qvec(3, *), Spos(3, *), rfield, alpha(*), beta2(*), norm1(*), E0(*)
      integer(c_int) :: spsmsz, nq, itr_dsf, nlev(*)
    end function

    ! DSFLan continued fraction
    integer(c_int) function qs3g_cfrac(nq, ldab, nlev, alpha, beta2, norm1, E0, eta, nomega, omega, compat, S) &
        bind(C, name="qs3g_cfrac")
      import :: c_int, c_double
      integer(c_int) :: nq, ldab, nlev(*), nomega, compat
      real(c_double) :: alpha(*), beta2(*), norm1(*), E0(*), eta, omega(*), S(*)
    end function

    ! U(1)-only basis of source_only_u1 (get_combination + list_fly)
    integer(c_int) function qs3g_build_sector_u1(h, NOD, D) bind(C, name="qs3g_build_sector_u1")
      import :: c_ptr, c_int, c_int64_t
      type(c_ptr), value :: h
      integer(c_int) :: NOD
      integer(c_int64_t) :: D
    end function

    ! get_cf_2_wave_vector + get_lm_2_wave_vector for all NOS**2 pairs
    integer(c_int) function qs3g_correlations(h, psi, szsz, spsm, lm) bind(C, name="qs3g_correlations")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex) :: psi(*), spsm(*)
      real(c_double) :: szsz(*), lm(*)
    end function

    ! write_wf / read_wf record (path is a NUL-terminated character string)
    integer(c_int) function qs3g_write_wf(path, dim, psi) bind(C, name="qs3g_write_wf")
      import :: c_int, c_int64_t, c_char, c_double_complex
      character(kind=c_char) :: path(*)
      integer(c_int64_t) :: dim
      complex(c_double_complex) :: psi(*)
    end function

    integer(c_int) function qs3g_read_wf(path, dim, psi) bind(C, name="qs3g_read_wf")
      import :: c_int, c_int64_t, c_char, c_double_complex
      character(kind=c_char) :: path(*)
      integer(c_int64_t) :: dim
      complex(c_double_complex) :: psi(*)
    end function

    ! alpha_beta_values_*.d lines
    integer(c_int) function qs3g_write_alpha_beta(path, nlines, ex_i, itr, alpha, beta2, norm1, E0, sztot, &
        append) bind(C, name="qs3g_write_alpha_beta")
      import :: c_int, c_char, c_double
      character(kind=c_char) :: path(*)
      integer(c_int) :: nlines, ex_i, itr, append
      real(c_double) :: alpha(*), beta2(*), norm1, E0, sztot
    end function

    integer(c_int) function qs3g_read_alpha_beta(path, cap, alpha, beta2, norm1, E0, sztot, nlines) &
        bind(C, name="qs3g_read_alpha_beta")
      import :: c_int, c_char, c_double
      character(kind=c_char) :: path(*)
      integer(c_int) :: cap, nlines
      real(c_double) :: alpha(*), beta2(*), norm1(*), E0(*), sztot(*)
    end function

    ! energy.dat lines (write / read back for re_wf = 1)
    integer(c_int) function qs3g_write_energy(path, NOE, ene) bind(C, name="qs3g_write_energy")
      import :: c_int, c_char, c_double
      character(kind=c_char) :: path(*)
      integer(c_int) :: NOE
      real(c_double) :: ene(*)
    end function

    integer(c_int) function qs3g_read_energy(path, NOE, ene) bind(C, name="qs3g_read_energy")
      import :: c_int, c_char, c_double
      character(kind=c_char) :: path(*)
      integer(c_int) :: NOE
      real(c_double) :: ene(*)
    end function

    ! calcu_Sq_a alone: the new sector's list_s and S^a(q)|psi>
    integer(c_int) function qs3g_sq_a(h, psi, spsmsz, qvec, Spos, D_new, list_s_new, fn) bind(C, name="qs3g_sq_a")
      import :: c_ptr, c_int, c_int64_t, c_double, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex) :: psi(*), fn(*)
      integer(c_int) :: spsmsz
      real(c_double) :: qvec(3), Spos(3, *)
      integer(c_int64_t) :: D_new, list_s_new(*)
    end function

    ! ALG = 3: Full_diag_routines + make_full_hamiltonian + fulldia_routines_with_momentum
    integer(c_int) function qs3g_full_diag(h, ene, psi) bind(C, name="qs3g_full_diag")
      import :: c_ptr, c_int, c_double, c_double_complex
      type(c_ptr), value :: h
      real(c_double) :: ene(*)
      complex(c_double_complex) :: psi(*)
    end function

    integer(c_int) function qs3g_full_hamiltonian(h, ham) bind(C, name="qs3g_full_hamiltonian")
      import :: c_ptr, c_int, c_double_complex
      type(c_ptr), value :: h
      complex(c_double_complex) :: ham(*)
    end function

    ! DSFLan from a code that cannot allocate device memory
    integer(c_int) function qs3g_cfrac_noalloc(nq, ldab, nlev, alpha, beta2, norm1, E0, eta, nomega, omega, &
        compat, S) bind(C, name="qs3g_cfrac_noalloc")
      import :: c_int, c_double
      integer(c_int) :: nq, ldab, nlev(*), nomega, compat
      real(c_double) :: alpha(*), beta2(*), norm1(*), E0(*), eta, omega(*), S(*)
    end function

    ! message of the handle's last failed call (c_null_ptr: the last global
    ! failure, e.g. of the file routines); a NUL-terminated C string, see
    ! qs3g_error_message below
    type(c_ptr) function qs3g_last_error(h) bind(C, name="qs3g_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function
  end interface

contains

  ! The last error message as a Fortran string (blank-padded to len(msg)).
  subroutine qs3g_error_message(h, msg)
    type(c_ptr), value :: h
    character(len=*), intent(out) :: msg
    character(kind=c_char), pointer :: c(:)
    integer :: i
    msg = ' '
    call c_f_pointer(qs3g_last_error(h), c, [len(msg)])
    do i = 1, len(msg)
      if (c(i) == c_null_char) exit
      msg(i:i) = c(i)
    end do
  end subroutine
end module qs3g_iface
