! rrtmg_sw_gb300_shim.f90 -- Fortran (ISO_C_BINDING) drop-in for the GCM
! interface of RRTMG_SW on top of the GB300 library's C ABI
! (include/rrtmg_sw_gb300.h, librrtmg_sw_gb300.so).
!
! A GCM that calls RRTMG_SW through the modules rrtmg_sw_init
! (rrtmg_sw_ini), mcica_subcol_gen_sw (get_alpha, mcica_subcol_sw) and
! rrtmg_sw_rad (rrtmg_sw) compiles this file in place of those reference
! sources and links librrtmg_sw_gb300.so.  Module names, routine names,
! argument lists, kinds, intents and optional arguments are the
! reference's: rrtmg_sw_init.f90:47, mcica_subcol_gen_sw.f90:66-67 and
! 181-185, rrtmg_sw_rad.f90:99-111 (declarations :220-388).  Kinds: the
! reference's integer(kind=im) is a 4-byte integer and real(kind=rb) an
! 8-byte real (modules/parkind.f90), i.e. c_int32_t and c_double here;
! every kind is explicit, so the file compiles the same under the
! reference's -r8 -i8 build flags.
!
! Arrays keep the reference's shapes and Fortran order.  Each routine hands
! the library c_loc of its arrays; an array that is not one contiguous
! block of the extents the library expects (a section, or a leading
! dimension larger than ncol) is packed into a temporary first and, for
! outputs, unpacked after the call.  A non-zero status prints the
! library's message -- the text of the reference's `stop` for the same
! condition -- and stops with error stop.
!
! Module rrtmg_sw_gb300 adds the library's own controls: the arithmetic
! form (rrtmg_sw_set_form) and release of its device memory
! (rrtmg_sw_finalize).

module rrtmg_sw_gb300_c
  use, intrinsic :: iso_c_binding
  use, intrinsic :: iso_fortran_env, only: error_unit
  implicit none
  private

  public :: rrtmg_sw_args, rrtmg_sw_clouds, buf1_t, buf2_t, buf3_t
  public :: rrtmg_sw_ini_c, rrtmg_sw_c, rrtmg_sw_mcica_c, mcica_subcol_sw_c, get_alpha_c
  public :: rrtmg_sw_set_form_c, rrtmg_sw_finalize_c, rrtmg_sw_errstr_c
  public :: gb300_check, gb300_null_args, gb300_in1, gb300_in2, gb300_in3, gb300_io2
  public :: gb300_out2, gb300_out3, gb300_back2, gb300_back3

  ! Field for field the struct rrtmg_sw_args of include/rrtmg_sw_gb300.h.
  type, bind(c) :: rrtmg_sw_args
     integer(c_int32_t) :: ncol, nlay, icld, iaer
     type(c_ptr) :: play, plev, tlay, tlev, tsfc
     type(c_ptr) :: h2ovmr, o3vmr, co2vmr, ch4vmr, n2ovmr, o2vmr
     type(c_ptr) :: asdir, asdif, aldir, aldif
     type(c_ptr) :: coszen
     real(c_double) :: adjes
     integer(c_int32_t) :: dyofyr
     real(c_double) :: scon
     integer(c_int32_t) :: isolvar
     integer(c_int32_t) :: inflgsw, iceflgsw, liqflgsw
     type(c_ptr) :: cldfmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl
     type(c_ptr) :: ciwpmcl, clwpmcl
     type(c_ptr) :: reicmcl, relqmcl
     type(c_ptr) :: tauaer, ssaaer, asmaer
     type(c_ptr) :: ecaer
     type(c_ptr) :: swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc
     type(c_ptr) :: bndsolvar
     type(c_ptr) :: indsolvar
     type(c_ptr) :: solcycfrac
     type(c_ptr) :: dirdflux, difdflux, uvdflx, nidflx, dirdnuv, difdnuv, dirdnir, difdnir
     integer(c_int32_t) :: idelm
     integer(c_int32_t) :: nthreads
     type(c_ptr) :: bndfu, bndfd, bndfddir, bndcu, bndcd
  end type rrtmg_sw_args

  ! Field for field the struct rrtmg_sw_clouds of include/rrtmg_sw_gb300.h.
  type, bind(c) :: rrtmg_sw_clouds
     integer(c_int32_t) :: permuteseed, irng
     type(c_ptr) :: cldfrac, ciwp, clwp, rei, rel
     type(c_ptr) :: tauc, ssac, asmc, fsfc
     type(c_ptr) :: alpha
  end type rrtmg_sw_clouds

  ! Packing buffers (used only for arrays that are not one contiguous block)
  type :: buf1_t
     real(c_double), allocatable :: v(:)
  end type buf1_t
  type :: buf2_t
     real(c_double), allocatable :: v(:,:)
  end type buf2_t
  type :: buf3_t
     real(c_double), allocatable :: v(:,:,:)
  end type buf3_t

  interface
     function rrtmg_sw_ini_c(cpdair) bind(c, name='rrtmg_sw_ini_c') result(rc)
       import :: c_int, c_double
       real(c_double), value :: cpdair
       integer(c_int) :: rc
     end function rrtmg_sw_ini_c

     function rrtmg_sw_c(a) bind(c, name='rrtmg_sw_c') result(rc)
       import :: c_int, rrtmg_sw_args
       type(rrtmg_sw_args), intent(in) :: a
       integer(c_int) :: rc
     end function rrtmg_sw_c

     function rrtmg_sw_mcica_c(a, c) bind(c, name='rrtmg_sw_mcica_c') result(rc)
       import :: c_int, rrtmg_sw_args, rrtmg_sw_clouds
       type(rrtmg_sw_args), intent(in) :: a
       type(rrtmg_sw_clouds), intent(in) :: c
       integer(c_int) :: rc
     end function rrtmg_sw_mcica_c

     function mcica_subcol_sw_c(ncol, nlay, icld, permuteseed, irng, play, cldfrac, ciwp, clwp, rei, rel, &
                                tauc, ssac, asmc, fsfc, alpha, cldfmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, &
                                taucmcl, ssacmcl, asmcmcl, fsfcmcl) bind(c, name='mcica_subcol_sw_c') result(rc)
       import :: c_int, c_int32_t, c_ptr
       integer(c_int32_t), value :: ncol, nlay, icld, permuteseed, irng
       type(c_ptr), value :: play, cldfrac, ciwp, clwp, rei, rel, tauc, ssac, asmc, fsfc, alpha
       type(c_ptr), value :: cldfmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl
       integer(c_int) :: rc
     end function mcica_subcol_sw_c

     function get_alpha_c(ncol, nlay, icld, idcor, decorr_con, dz, lat, juldat, cldfrac, alpha) &
          bind(c, name='get_alpha_c') result(rc)
       import :: c_int, c_int32_t, c_double, c_ptr
       integer(c_int32_t), value :: ncol, nlay, icld, idcor
       real(c_double), value :: decorr_con
       type(c_ptr), value :: dz, lat
       integer(c_int32_t), value :: juldat
       type(c_ptr), value :: cldfrac, alpha
       integer(c_int) :: rc
     end function get_alpha_c

     function rrtmg_sw_set_form_c(form) bind(c, name='rrtmg_sw_set_form_c') result(rc)
       import :: c_int, c_int32_t
       integer(c_int32_t), value :: form
       integer(c_int) :: rc
     end function rrtmg_sw_set_form_c

     function rrtmg_sw_finalize_c() bind(c, name='rrtmg_sw_finalize_c') result(rc)
       import :: c_int
       integer(c_int) :: rc
     end function rrtmg_sw_finalize_c

     function rrtmg_sw_errstr_c(code) bind(c, name='rrtmg_sw_errstr_c') result(p)
       import :: c_int32_t, c_ptr
       integer(c_int32_t), value :: code
       type(c_ptr) :: p
     end function rrtmg_sw_errstr_c
  end interface

contains

  ! A non-zero library status: print the library's message (the reference's
  ! stop text for the same condition) and stop.
  subroutine gb300_check(rc)
    integer(c_int), intent(in) :: rc
    character(kind=c_char), pointer :: s(:)
    character(len=256) :: msg
    integer :: n
    if (rc == 0) return
    call c_f_pointer(rrtmg_sw_errstr_c(int(rc, c_int32_t)), s, [256])
    msg = ' '
    n = 0
    do while (n < 256)
       if (s(n + 1) == c_null_char) exit
       n = n + 1
       msg(n:n) = s(n)
    end do
    write (error_unit, '(a)') trim(msg)
    error stop 'RRTMG_SW (GB300 library) stopped'
  end subroutine gb300_check

  ! Every pointer of the argument struct to NULL and every scalar to 0.
  subroutine gb300_null_args(a)
    type(rrtmg_sw_args), intent(out) :: a
    a%ncol = 0; a%nlay = 0; a%icld = 0; a%iaer = 0
    a%play = c_null_ptr; a%plev = c_null_ptr; a%tlay = c_null_ptr; a%tlev = c_null_ptr; a%tsfc = c_null_ptr
    a%h2ovmr = c_null_ptr; a%o3vmr = c_null_ptr; a%co2vmr = c_null_ptr; a%ch4vmr = c_null_ptr
    a%n2ovmr = c_null_ptr; a%o2vmr = c_null_ptr
    a%asdir = c_null_ptr; a%asdif = c_null_ptr; a%aldir = c_null_ptr; a%aldif = c_null_ptr
    a%coszen = c_null_ptr
    a%adjes = 0.0_c_double; a%dyofyr = 0; a%scon = 0.0_c_double; a%isolvar = 0
    a%inflgsw = 0; a%iceflgsw = 0; a%liqflgsw = 0
    a%cldfmcl = c_null_ptr; a%taucmcl = c_null_ptr; a%ssacmcl = c_null_ptr; a%asmcmcl = c_null_ptr
    a%fsfcmcl = c_null_ptr; a%ciwpmcl = c_null_ptr; a%clwpmcl = c_null_ptr
    a%reicmcl = c_null_ptr; a%relqmcl = c_null_ptr
    a%tauaer = c_null_ptr; a%ssaaer = c_null_ptr; a%asmaer = c_null_ptr; a%ecaer = c_null_ptr
    a%swuflx = c_null_ptr; a%swdflx = c_null_ptr; a%swhr = c_null_ptr
    a%swuflxc = c_null_ptr; a%swdflxc = c_null_ptr; a%swhrc = c_null_ptr
    a%bndsolvar = c_null_ptr; a%indsolvar = c_null_ptr; a%solcycfrac = c_null_ptr
    a%dirdflux = c_null_ptr; a%difdflux = c_null_ptr; a%uvdflx = c_null_ptr; a%nidflx = c_null_ptr
    a%dirdnuv = c_null_ptr; a%difdnuv = c_null_ptr; a%dirdnir = c_null_ptr; a%difdnir = c_null_ptr
    a%idelm = 1; a%nthreads = 0
    a%bndfu = c_null_ptr; a%bndfd = c_null_ptr; a%bndfddir = c_null_ptr
    a%bndcu = c_null_ptr; a%bndcd = c_null_ptr
  end subroutine gb300_null_args

  ! c_loc of x(1:n) as one contiguous block: x itself when it is that block,
  ! else a copy in b%v.
  function gb300_in1(x, n, b) result(p)
    real(c_double), intent(in), target :: x(:)
    integer(c_int32_t), intent(in) :: n
    type(buf1_t), intent(inout), target :: b
    type(c_ptr) :: p
    if (size(x) == n .and. is_contiguous(x)) then
       p = c_loc(x)
    else
       allocate (b%v(n))
       b%v = x(1:n)
       p = c_loc(b%v)
    end if
  end function gb300_in1

  ! c_loc of x(1:n1,1:n2) as one contiguous (n1,n2) block.
  function gb300_in2(x, n1, n2, b) result(p)
    real(c_double), intent(in), target :: x(:,:)
    integer(c_int32_t), intent(in) :: n1, n2
    type(buf2_t), intent(inout), target :: b
    type(c_ptr) :: p
    if (size(x, 1) == n1 .and. size(x, 2) == n2 .and. is_contiguous(x)) then
       p = c_loc(x)
    else
       allocate (b%v(n1, n2))
       b%v = x(1:n1, 1:n2)
       p = c_loc(b%v)
    end if
  end function gb300_in2

  ! c_loc of x(1:n1,1:n2,1:n3) as one contiguous (n1,n2,n3) block.
  function gb300_in3(x, n1, n2, n3, b) result(p)
    real(c_double), intent(in), target :: x(:,:,:)
    integer(c_int32_t), intent(in) :: n1, n2, n3
    type(buf3_t), intent(inout), target :: b
    type(c_ptr) :: p
    if (size(x, 1) == n1 .and. size(x, 2) == n2 .and. size(x, 3) == n3 .and. is_contiguous(x)) then
       p = c_loc(x)
    else
       allocate (b%v(n1, n2, n3))
       b%v = x(1:n1, 1:n2, 1:n3)
       p = c_loc(b%v)
    end if
  end function gb300_in3

  ! Output or in-out block x(1:n1,1:n2): x itself, or a buffer (copied in
  ! when copyin) that gb300_back2 copies back.
  function gb300_io2(x, n1, n2, b, copyin) result(p)
    real(c_double), intent(inout), target :: x(:,:)
    integer(c_int32_t), intent(in) :: n1, n2
    type(buf2_t), intent(inout), target :: b
    logical, intent(in) :: copyin
    type(c_ptr) :: p
    if (size(x, 1) == n1 .and. size(x, 2) == n2 .and. is_contiguous(x)) then
       p = c_loc(x)
    else
       allocate (b%v(n1, n2))
       if (copyin) b%v = x(1:n1, 1:n2)
       p = c_loc(b%v)
    end if
  end function gb300_io2

  function gb300_out2(x, n1, n2, b) result(p)
    real(c_double), intent(inout), target :: x(:,:)
    integer(c_int32_t), intent(in) :: n1, n2
    type(buf2_t), intent(inout), target :: b
    type(c_ptr) :: p
    p = gb300_io2(x, n1, n2, b, .false.)
  end function gb300_out2

  function gb300_out3(x, n1, n2, n3, b) result(p)
    real(c_double), intent(inout), target :: x(:,:,:)
    integer(c_int32_t), intent(in) :: n1, n2, n3
    type(buf3_t), intent(inout), target :: b
    type(c_ptr) :: p
    if (size(x, 1) == n1 .and. size(x, 2) == n2 .and. size(x, 3) == n3 .and. is_contiguous(x)) then
       p = c_loc(x)
    else
       allocate (b%v(n1, n2, n3))
       p = c_loc(b%v)
    end if
  end function gb300_out3

  subroutine gb300_back2(x, b)
    real(c_double), intent(inout) :: x(:,:)
    type(buf2_t), intent(inout) :: b
    if (allocated(b%v)) then
       x(1:size(b%v, 1), 1:size(b%v, 2)) = b%v
       deallocate (b%v)
    end if
  end subroutine gb300_back2

  subroutine gb300_back3(x, b)
    real(c_double), intent(inout) :: x(:,:,:)
    type(buf3_t), intent(inout) :: b
    if (allocated(b%v)) then
       x(1:size(b%v, 1), 1:size(b%v, 2), 1:size(b%v, 3)) = b%v
       deallocate (b%v)
    end if
  end subroutine gb300_back3

end module rrtmg_sw_gb300_c


! rrtmg_sw_ini (rrtmg_sw_init.f90:47): tables, lookup table and heatfac,
! loaded onto the current GPU.
module rrtmg_sw_init
  use, intrinsic :: iso_c_binding
  use rrtmg_sw_gb300_c
  implicit none
  private
  public :: rrtmg_sw_ini

contains

  subroutine rrtmg_sw_ini(cpdair)
    real(kind=c_double), intent(in) :: cpdair      ! specific heat capacity of dry air
    call gb300_check(rrtmg_sw_ini_c(cpdair))
  end subroutine rrtmg_sw_ini

end module rrtmg_sw_init


! get_alpha and mcica_subcol_sw (mcica_subcol_gen_sw.f90:66-67, 181-185).
module mcica_subcol_gen_sw
  use, intrinsic :: iso_c_binding
  use rrtmg_sw_gb300_c
  implicit none
  private
  public :: get_alpha, mcica_subcol_sw

  integer, parameter :: im = c_int32_t, rb = c_double
  integer(c_int32_t), parameter :: ngptsw = 112, nbndsw = 14

contains

  subroutine get_alpha(iplon, ncol, nlayers, icld, idcor, decorr_con, &
                       dz, lat, juldat, cldfrac, alpha)
    integer(kind=im), intent(in) :: iplon           ! column/longitude dimension
    integer(kind=im), intent(in) :: ncol            ! number of columns
    integer(kind=im), intent(in) :: nlayers         ! number of model layers
    integer(kind=im), intent(in) :: icld            ! clear/cloud, cloud overlap flag
    integer(kind=im), intent(in) :: idcor           ! decorrelation length method
    integer(kind=im), intent(in) :: juldat          ! Julian day of year
    real(kind=rb), intent(in) :: decorr_con         ! decorrelation length, constant (m)
    real(kind=rb), intent(in), target :: dz(:,:)    ! layer thickness (m)
    real(kind=rb), intent(in), target :: lat(:)     ! latitude (degrees)
    real(kind=rb), intent(in), target :: cldfrac(:,:) ! layer cloud fraction
    real(kind=rb), intent(out), target :: alpha(:,:)  ! vertical cloud fraction correlation parameter
    type(buf1_t), target :: b1
    type(buf2_t), target :: b2(3)
    integer(c_int) :: rc
    if (iplon < 0) continue                         ! iplon is unused, as in the reference
    if (ncol == 0) return
    ! alpha keeps its values where get_alpha sets none (icld other than 4, 5)
    rc = get_alpha_c(ncol, nlayers, icld, idcor, decorr_con, gb300_in2(dz, ncol, nlayers, b2(1)), &
                     gb300_in1(lat, ncol, b1), juldat, gb300_in2(cldfrac, ncol, nlayers, b2(2)), &
                     gb300_io2(alpha, ncol, nlayers, b2(3), .true.))
    call gb300_back2(alpha, b2(3))
    call gb300_check(rc)
  end subroutine get_alpha

  subroutine mcica_subcol_sw(iplon, ncol, nlay, icld, permuteseed, irng, play, &
                             cldfrac, ciwp, clwp, rei, rel, tauc, ssac, asmc, fsfc, &
                             alpha, &
                             cldfmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, &
                             taucmcl, ssacmcl, asmcmcl, fsfcmcl)
    integer(kind=im), intent(in) :: iplon           ! column/longitude dimension
    integer(kind=im), intent(in) :: ncol            ! number of columns
    integer(kind=im), intent(in) :: nlay            ! number of model layers
    integer(kind=im), intent(in) :: icld            ! clear/cloud, cloud overlap flag
    integer(kind=im), intent(in) :: permuteseed     ! generator offset between calls
    integer(kind=im), intent(inout) :: irng         ! random number generator: 0 KISS, 1 MT19937
    real(kind=rb), intent(in), target :: play(:,:)       ! layer pressures (mb)
    real(kind=rb), intent(in), target :: cldfrac(:,:)    ! layer cloud fraction
    real(kind=rb), intent(in), target :: tauc(:,:,:)     ! in-cloud optical depth (nbndsw,ncol,nlay)
    real(kind=rb), intent(in), target :: ssac(:,:,:)     ! in-cloud single scattering albedo
    real(kind=rb), intent(in), target :: asmc(:,:,:)     ! in-cloud asymmetry parameter
    real(kind=rb), intent(in), target :: fsfc(:,:,:)     ! in-cloud forward scattering fraction
    real(kind=rb), intent(in), target :: ciwp(:,:)       ! in-cloud ice water path
    real(kind=rb), intent(in), target :: clwp(:,:)       ! in-cloud liquid water path
    real(kind=rb), intent(in), target :: rei(:,:)        ! cloud ice particle size
    real(kind=rb), intent(in), target :: rel(:,:)        ! cloud liquid particle size
    real(kind=rb), intent(in), target :: alpha(:,:)      ! cloud fraction correlation (icld 4, 5)
    real(kind=rb), intent(out), target :: cldfmcl(:,:,:) ! cloud fraction [mcica] (ngptsw,ncol,nlay)
    real(kind=rb), intent(out), target :: ciwpmcl(:,:,:) ! in-cloud ice water path [mcica]
    real(kind=rb), intent(out), target :: clwpmcl(:,:,:) ! in-cloud liquid water path [mcica]
    real(kind=rb), intent(out), target :: relqmcl(:,:)   ! liquid particle size (microns)
    real(kind=rb), intent(out), target :: reicmcl(:,:)   ! ice particle size (microns)
    real(kind=rb), intent(out), target :: taucmcl(:,:,:) ! in-cloud optical depth [mcica]
    real(kind=rb), intent(out), target :: ssacmcl(:,:,:) ! in-cloud single scattering albedo [mcica]
    real(kind=rb), intent(out), target :: asmcmcl(:,:,:) ! in-cloud asymmetry parameter [mcica]
    real(kind=rb), intent(out), target :: fsfcmcl(:,:,:) ! in-cloud forward scattering fraction [mcica]
    type(buf2_t), target :: b2(9)
    type(buf3_t), target :: b3(11)
    type(c_ptr) :: palpha
    integer(c_int) :: rc
    if (iplon < 0) continue                         ! iplon is unused, as in the reference
    if (irng /= 0) irng = 1                          ! mcica_subcol_gen_sw.f90:455
    if (icld == 0) return                            ! clear sky: nothing to generate (:261)
    if (ncol == 0) return
    palpha = c_null_ptr
    if (icld >= 4) palpha = gb300_in2(alpha, ncol, nlay, b2(7))
    rc = mcica_subcol_sw_c(ncol, nlay, icld, permuteseed, irng, &
                           gb300_in2(play, ncol, nlay, b2(1)), gb300_in2(cldfrac, ncol, nlay, b2(2)), &
                           gb300_in2(ciwp, ncol, nlay, b2(3)), gb300_in2(clwp, ncol, nlay, b2(4)), &
                           gb300_in2(rei, ncol, nlay, b2(5)), gb300_in2(rel, ncol, nlay, b2(6)), &
                           gb300_in3(tauc, nbndsw, ncol, nlay, b3(1)), gb300_in3(ssac, nbndsw, ncol, nlay, b3(2)), &
                           gb300_in3(asmc, nbndsw, ncol, nlay, b3(3)), gb300_in3(fsfc, nbndsw, ncol, nlay, b3(4)), &
                           palpha, &
                           gb300_out3(cldfmcl, ngptsw, ncol, nlay, b3(5)), gb300_out3(ciwpmcl, ngptsw, ncol, nlay, b3(6)), &
                           gb300_out3(clwpmcl, ngptsw, ncol, nlay, b3(7)), gb300_out2(reicmcl, ncol, nlay, b2(8)), &
                           gb300_out2(relqmcl, ncol, nlay, b2(9)), gb300_out3(taucmcl, ngptsw, ncol, nlay, b3(8)), &
                           gb300_out3(ssacmcl, ngptsw, ncol, nlay, b3(9)), gb300_out3(asmcmcl, ngptsw, ncol, nlay, b3(10)), &
                           gb300_out3(fsfcmcl, ngptsw, ncol, nlay, b3(11)))
    call gb300_back3(cldfmcl, b3(5)); call gb300_back3(ciwpmcl, b3(6)); call gb300_back3(clwpmcl, b3(7))
    call gb300_back2(reicmcl, b2(8)); call gb300_back2(relqmcl, b2(9))
    call gb300_back3(taucmcl, b3(8)); call gb300_back3(ssacmcl, b3(9))
    call gb300_back3(asmcmcl, b3(10)); call gb300_back3(fsfcmcl, b3(11))
    call gb300_check(rc)
  end subroutine mcica_subcol_sw

end module mcica_subcol_gen_sw


! rrtmg_sw (rrtmg_sw_rad.f90:99-111), McICA version: the subcolumn arrays
! of mcica_subcol_sw in, fluxes and heating rates out.
module rrtmg_sw_rad
  use, intrinsic :: iso_c_binding
  use rrtmg_sw_gb300_c
  implicit none
  private
  public :: rrtmg_sw

  integer, parameter :: im = c_int32_t, rb = c_double
  integer(c_int32_t), parameter :: ngptsw = 112, nbndsw = 14, naerec = 6

contains

  subroutine rrtmg_sw &
       (ncol    ,nlay    ,icld    ,iaer    , &
        play    ,plev    ,tlay    ,tlev    ,tsfc   , &
        h2ovmr , o3vmr   ,co2vmr  ,ch4vmr  ,n2ovmr ,o2vmr , &
        asdir   ,asdif   ,aldir   ,aldif   , &
        coszen  ,adjes   ,dyofyr  ,scon    ,isolvar, &
        inflgsw ,iceflgsw,liqflgsw,cldfmcl , &
        taucmcl ,ssacmcl ,asmcmcl ,fsfcmcl , &
        ciwpmcl ,clwpmcl ,reicmcl ,relqmcl , &
        tauaer  ,ssaaer  ,asmaer  ,ecaer   , &
        swuflx  ,swdflx  ,swhr    ,swuflxc ,swdflxc ,swhrc, &
        bndsolvar,indsolvar,solcycfrac)
    integer(kind=im), intent(in) :: ncol            ! number of horizontal columns
    integer(kind=im), intent(in) :: nlay            ! number of model layers
    integer(kind=im), intent(inout) :: icld         ! cloud overlap method
    integer(kind=im), intent(inout) :: iaer         ! aerosol option flag
    real(kind=rb), intent(in), target :: play(:,:)      ! layer pressures (hPa)
    real(kind=rb), intent(in), target :: plev(:,:)      ! interface pressures (hPa)
    real(kind=rb), intent(in), target :: tlay(:,:)      ! layer temperatures (K)
    real(kind=rb), intent(in), target :: tlev(:,:)      ! interface temperatures (K)
    real(kind=rb), intent(in), target :: tsfc(:)        ! surface temperature (K)
    real(kind=rb), intent(in), target :: h2ovmr(:,:)    ! H2O volume mixing ratio
    real(kind=rb), intent(in), target :: o3vmr(:,:)     ! O3 volume mixing ratio
    real(kind=rb), intent(in), target :: co2vmr(:,:)    ! CO2 volume mixing ratio
    real(kind=rb), intent(in), target :: ch4vmr(:,:)    ! methane volume mixing ratio
    real(kind=rb), intent(in), target :: n2ovmr(:,:)    ! nitrous oxide volume mixing ratio
    real(kind=rb), intent(in), target :: o2vmr(:,:)     ! oxygen volume mixing ratio
    real(kind=rb), intent(in), target :: asdir(:)       ! UV/vis surface albedo, direct
    real(kind=rb), intent(in), target :: aldir(:)       ! near-IR surface albedo, direct
    real(kind=rb), intent(in), target :: asdif(:)       ! UV/vis surface albedo, diffuse
    real(kind=rb), intent(in), target :: aldif(:)       ! near-IR surface albedo, diffuse
    integer(kind=im), intent(in) :: dyofyr          ! day of the year (Earth-Sun distance)
    real(kind=rb), intent(in) :: adjes              ! flux adjustment for Earth-Sun distance
    real(kind=rb), intent(in), target :: coszen(:)      ! cosine of solar zenith angle
    real(kind=rb), intent(in) :: scon               ! solar constant (W/m2)
    integer(kind=im), intent(in) :: isolvar         ! solar variability method
    real(kind=rb), intent(in), optional, target :: indsolvar(:) ! facular and sunspot amplitudes
    real(kind=rb), intent(in), optional, target :: bndsolvar(:) ! solar variability scale factors
    real(kind=rb), intent(in), optional, target :: solcycfrac   ! fraction of the 11-year solar cycle
    integer(kind=im), intent(in) :: inflgsw         ! cloud optical properties flag
    integer(kind=im), intent(in) :: iceflgsw        ! ice particle specification flag
    integer(kind=im), intent(in) :: liqflgsw        ! liquid droplet specification flag
    real(kind=rb), intent(in), target :: cldfmcl(:,:,:)  ! cloud fraction [mcica] (ngptsw,ncol,nlay)
    real(kind=rb), intent(in), target :: taucmcl(:,:,:)  ! in-cloud optical depth
    real(kind=rb), intent(in), target :: ssacmcl(:,:,:)  ! in-cloud single scattering albedo
    real(kind=rb), intent(in), target :: asmcmcl(:,:,:)  ! in-cloud asymmetry parameter
    real(kind=rb), intent(in), target :: fsfcmcl(:,:,:)  ! in-cloud forward scattering fraction
    real(kind=rb), intent(in), target :: ciwpmcl(:,:,:)  ! in-cloud ice water path (g/m2)
    real(kind=rb), intent(in), target :: clwpmcl(:,:,:)  ! in-cloud liquid water path (g/m2)
    real(kind=rb), intent(in), target :: reicmcl(:,:)    ! cloud ice effective radius (microns)
    real(kind=rb), intent(in), target :: relqmcl(:,:)    ! cloud drop effective radius (microns)
    real(kind=rb), intent(in), target :: tauaer(:,:,:)   ! aerosol optical depth (iaer=10) (ncol,nlay,nbndsw)
    real(kind=rb), intent(in), target :: ssaaer(:,:,:)   ! aerosol single scattering albedo (iaer=10)
    real(kind=rb), intent(in), target :: asmaer(:,:,:)   ! aerosol asymmetry parameter (iaer=10)
    real(kind=rb), intent(in), target :: ecaer(:,:,:)    ! aerosol optical depth at 0.55 um (iaer=6) (ncol,nlay,naerec)
    real(kind=rb), intent(out), target :: swuflx(:,:)    ! total sky upward flux (W/m2) (ncol,nlay+1)
    real(kind=rb), intent(out), target :: swdflx(:,:)    ! total sky downward flux (W/m2)
    real(kind=rb), intent(out), target :: swhr(:,:)      ! total sky heating rate (K/d) (ncol,nlay)
    real(kind=rb), intent(out), target :: swuflxc(:,:)   ! clear sky upward flux (W/m2)
    real(kind=rb), intent(out), target :: swdflxc(:,:)   ! clear sky downward flux (W/m2)
    real(kind=rb), intent(out), target :: swhrc(:,:)     ! clear sky heating rate (K/d)
    type(rrtmg_sw_args) :: a
    type(buf1_t), target :: b1(8)
    type(buf2_t), target :: b2(18)
    type(buf3_t), target :: b3(11)
    integer(c_int) :: rc
    integer(c_int32_t) :: icld_eff, iaer_eff

    ! the driver's clamps (rrtmg_sw_rad.f90:589,597), visible to the caller
    ! through intent(inout); icld 4 and 5 are accepted by the library
    icld_eff = icld
    if (icld_eff < 0 .or. icld_eff > 5) icld_eff = 2
    iaer_eff = iaer
    if (iaer_eff /= 0 .and. iaer_eff /= 6 .and. iaer_eff /= 10) iaer_eff = 0
    icld = icld_eff
    iaer = iaer_eff
    if (ncol == 0) return

    call gb300_null_args(a)
    a%ncol = ncol; a%nlay = nlay; a%icld = icld_eff; a%iaer = iaer_eff
    a%play = gb300_in2(play, ncol, nlay, b2(1))
    a%plev = gb300_in2(plev, ncol, nlay + 1_c_int32_t, b2(2))
    a%tlay = gb300_in2(tlay, ncol, nlay, b2(3))
    ! tlev, tsfc and n2ovmr enter nothing the shortwave solve returns
    a%h2ovmr = gb300_in2(h2ovmr, ncol, nlay, b2(4))
    a%o3vmr = gb300_in2(o3vmr, ncol, nlay, b2(5))
    a%co2vmr = gb300_in2(co2vmr, ncol, nlay, b2(6))
    a%ch4vmr = gb300_in2(ch4vmr, ncol, nlay, b2(7))
    a%o2vmr = gb300_in2(o2vmr, ncol, nlay, b2(8))
    a%asdir = gb300_in1(asdir, ncol, b1(1))
    a%asdif = gb300_in1(asdif, ncol, b1(2))
    a%aldir = gb300_in1(aldir, ncol, b1(3))
    a%aldif = gb300_in1(aldif, ncol, b1(4))
    a%coszen = gb300_in1(coszen, ncol, b1(5))
    a%adjes = adjes; a%dyofyr = dyofyr; a%scon = scon; a%isolvar = isolvar
    a%inflgsw = inflgsw; a%iceflgsw = iceflgsw; a%liqflgsw = liqflgsw
    if (icld_eff >= 1) then
       a%cldfmcl = gb300_in3(cldfmcl, ngptsw, ncol, nlay, b3(1))
       a%taucmcl = gb300_in3(taucmcl, ngptsw, ncol, nlay, b3(2))
       a%ssacmcl = gb300_in3(ssacmcl, ngptsw, ncol, nlay, b3(3))
       a%asmcmcl = gb300_in3(asmcmcl, ngptsw, ncol, nlay, b3(4))
       a%fsfcmcl = gb300_in3(fsfcmcl, ngptsw, ncol, nlay, b3(5))
       a%ciwpmcl = gb300_in3(ciwpmcl, ngptsw, ncol, nlay, b3(6))
       a%clwpmcl = gb300_in3(clwpmcl, ngptsw, ncol, nlay, b3(7))
       a%reicmcl = gb300_in2(reicmcl, ncol, nlay, b2(9))
       a%relqmcl = gb300_in2(relqmcl, ncol, nlay, b2(10))
    end if
    if (iaer_eff == 10) then
       a%tauaer = gb300_in3(tauaer, ncol, nlay, nbndsw, b3(8))
       a%ssaaer = gb300_in3(ssaaer, ncol, nlay, nbndsw, b3(9))
       a%asmaer = gb300_in3(asmaer, ncol, nlay, nbndsw, b3(10))
    else if (iaer_eff == 6) then
       a%ecaer = gb300_in3(ecaer, ncol, nlay, naerec, b3(11))
    end if
    a%swuflx = gb300_out2(swuflx, ncol, nlay + 1_c_int32_t, b2(11))
    a%swdflx = gb300_out2(swdflx, ncol, nlay + 1_c_int32_t, b2(12))
    a%swhr = gb300_out2(swhr, ncol, nlay, b2(13))
    a%swuflxc = gb300_out2(swuflxc, ncol, nlay + 1_c_int32_t, b2(14))
    a%swdflxc = gb300_out2(swdflxc, ncol, nlay + 1_c_int32_t, b2(15))
    a%swhrc = gb300_out2(swhrc, ncol, nlay, b2(16))
    if (present(bndsolvar)) a%bndsolvar = gb300_in1(bndsolvar, nbndsw, b1(6))
    if (present(indsolvar)) a%indsolvar = gb300_in1(indsolvar, 2_c_int32_t, b1(7))
    if (present(solcycfrac)) a%solcycfrac = c_loc(solcycfrac)
    a%idelm = 1                                      ! rrtmg_sw_rad.f90:605

    rc = rrtmg_sw_c(a)

    call gb300_back2(swuflx, b2(11)); call gb300_back2(swdflx, b2(12)); call gb300_back2(swhr, b2(13))
    call gb300_back2(swuflxc, b2(14)); call gb300_back2(swdflxc, b2(15)); call gb300_back2(swhrc, b2(16))
    call gb300_check(rc)
  end subroutine rrtmg_sw

end module rrtmg_sw_rad


! Controls of the GB300 library that the reference does not have.
module rrtmg_sw_gb300
  use, intrinsic :: iso_c_binding
  use rrtmg_sw_gb300_c
  implicit none
  private
  public :: rrtmg_sw_set_form, rrtmg_sw_finalize
  public :: RRTMG_SW_FORM_FP64, RRTMG_SW_FORM_FP32

  integer(c_int32_t), parameter :: RRTMG_SW_FORM_FP64 = 0, RRTMG_SW_FORM_FP32 = 1

contains

  ! Arithmetic form of later solves (include/rrtmg_sw_gb300.h, default FP64).
  subroutine rrtmg_sw_set_form(form)
    integer(c_int32_t), intent(in) :: form
    call gb300_check(rrtmg_sw_set_form_c(form))
  end subroutine rrtmg_sw_set_form

  ! Release the library's device tables and workspace.
  subroutine rrtmg_sw_finalize()
    call gb300_check(rrtmg_sw_finalize_c())
  end subroutine rrtmg_sw_finalize

end module rrtmg_sw_gb300
