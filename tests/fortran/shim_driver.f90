! shim_driver.f90 -- test program for rrtmg_sw_gb300_shim.f90: a GCM-style
! caller of RRTMG_SW's modules with arrays whose leading dimension (pcols)
! is larger than ncol, as GCM physics buffers are.
!
! Usage: shim_driver <input file> <output file>
! Input (stream, native byte order): ncol, nlay, pcols as int32, then the
! arrays below in the order read.  Output: c_sizeof of the two bind(c)
! types (int64), then the six outputs (columns 1..ncol) of a clear-sky
! call, then those of a McICA call (mcica_subcol_sw, irng = 0, icld = 2).
program shim_driver
  use, intrinsic :: iso_c_binding
  use rrtmg_sw_init, only: rrtmg_sw_ini
  use mcica_subcol_gen_sw, only: mcica_subcol_sw
  use rrtmg_sw_rad, only: rrtmg_sw
  use rrtmg_sw_gb300_c, only: rrtmg_sw_args, rrtmg_sw_clouds
  implicit none
  integer(c_int32_t) :: ncol, nlay, pcols, icld, iaer, irng
  integer(c_int32_t), parameter :: ng = 112, nb = 14
  real(c_double), allocatable :: play(:,:), plev(:,:), tlay(:,:), tlev(:,:), tsfc(:)
  real(c_double), allocatable :: h2o(:,:), o3(:,:), co2(:,:), ch4(:,:), n2o(:,:), o2(:,:)
  real(c_double), allocatable :: asdir(:), asdif(:), aldir(:), aldif(:), coszen(:)
  real(c_double), allocatable :: cldfrac(:,:), ciwp(:,:), clwp(:,:), rei(:,:), rel(:,:), alpha(:,:)
  real(c_double), allocatable :: tauc(:,:,:), ssac(:,:,:), asmc(:,:,:), fsfc(:,:,:)
  real(c_double), allocatable :: cldfmcl(:,:,:), ciwpmcl(:,:,:), clwpmcl(:,:,:), taucmcl(:,:,:)
  real(c_double), allocatable :: ssacmcl(:,:,:), asmcmcl(:,:,:), fsfcmcl(:,:,:), reicmcl(:,:), relqmcl(:,:)
  real(c_double), allocatable :: tauaer(:,:,:), ssaaer(:,:,:), asmaer(:,:,:), ecaer(:,:,:)
  real(c_double), allocatable :: swuflx(:,:), swdflx(:,:), swhr(:,:), swuflxc(:,:), swdflxc(:,:), swhrc(:,:)
  type(rrtmg_sw_args) :: a
  type(rrtmg_sw_clouds) :: c
  character(len=1024) :: fin, fout
  integer :: u, pass

  call get_command_argument(1, fin)
  call get_command_argument(2, fout)
  open (newunit=u, file=trim(fin), access='stream', form='unformatted', status='old')
  read (u) ncol, nlay, pcols
  allocate (play(pcols, nlay), plev(pcols, nlay + 1), tlay(pcols, nlay), tlev(pcols, nlay + 1), tsfc(pcols))
  allocate (h2o(pcols, nlay), o3(pcols, nlay), co2(pcols, nlay), ch4(pcols, nlay), n2o(pcols, nlay), o2(pcols, nlay))
  allocate (asdir(pcols), asdif(pcols), aldir(pcols), aldif(pcols), coszen(pcols))
  allocate (cldfrac(pcols, nlay), ciwp(pcols, nlay), clwp(pcols, nlay), rei(pcols, nlay), rel(pcols, nlay))
  allocate (alpha(pcols, nlay))
  allocate (tauc(nb, pcols, nlay), ssac(nb, pcols, nlay), asmc(nb, pcols, nlay), fsfc(nb, pcols, nlay))
  read (u) play, plev, tlay, tlev, tsfc, h2o, o3, co2, ch4, n2o, o2, asdir, asdif, aldir, aldif, coszen
  read (u) cldfrac, ciwp, clwp, rei, rel
  close (u)
  tauc = 0.0_c_double; ssac = 1.0_c_double; asmc = 0.0_c_double; fsfc = 0.0_c_double; alpha = 0.0_c_double
  allocate (cldfmcl(ng, pcols, nlay), ciwpmcl(ng, pcols, nlay), clwpmcl(ng, pcols, nlay), taucmcl(ng, pcols, nlay))
  allocate (ssacmcl(ng, pcols, nlay), asmcmcl(ng, pcols, nlay), fsfcmcl(ng, pcols, nlay))
  allocate (reicmcl(pcols, nlay), relqmcl(pcols, nlay))
  allocate (tauaer(pcols, nlay, nb), ssaaer(pcols, nlay, nb), asmaer(pcols, nlay, nb), ecaer(pcols, nlay, 6))
  tauaer = 0.0_c_double; ssaaer = 1.0_c_double; asmaer = 0.0_c_double; ecaer = 0.0_c_double
  allocate (swuflx(pcols, nlay + 1), swdflx(pcols, nlay + 1), swhr(pcols, nlay))
  allocate (swuflxc(pcols, nlay + 1), swdflxc(pcols, nlay + 1), swhrc(pcols, nlay))

  call rrtmg_sw_ini(1.004e3_c_double)
  open (newunit=u, file=trim(fout), access='stream', form='unformatted', status='replace')
  write (u) int(c_sizeof(a), c_int64_t), int(c_sizeof(c), c_int64_t)
  do pass = 1, 2
     icld = 0
     if (pass == 2) then
        icld = 2
        irng = 0
        call mcica_subcol_sw(1_c_int32_t, ncol, nlay, icld, 112_c_int32_t, irng, play, cldfrac, ciwp, clwp, rei, rel, &
                             tauc, ssac, asmc, fsfc, alpha, cldfmcl, ciwpmcl, clwpmcl, reicmcl, relqmcl, &
                             taucmcl, ssacmcl, asmcmcl, fsfcmcl)
     else
        cldfmcl = 0.0_c_double; ciwpmcl = 0.0_c_double; clwpmcl = 0.0_c_double; taucmcl = 0.0_c_double
        ssacmcl = 1.0_c_double; asmcmcl = 0.0_c_double; fsfcmcl = 0.0_c_double
        reicmcl = 0.0_c_double; relqmcl = 0.0_c_double
     end if
     iaer = 0
     call rrtmg_sw(ncol, nlay, icld, iaer, play, plev, tlay, tlev, tsfc, &
                   h2o, o3, co2, ch4, n2o, o2, asdir, asdif, aldir, aldif, &
                   coszen, 1.0_c_double, 0_c_int32_t, 1360.85_c_double, 0_c_int32_t, &
                   2_c_int32_t, 3_c_int32_t, 1_c_int32_t, cldfmcl, taucmcl, ssacmcl, asmcmcl, fsfcmcl, &
                   ciwpmcl, clwpmcl, reicmcl, relqmcl, tauaer, ssaaer, asmaer, ecaer, &
                   swuflx, swdflx, swhr, swuflxc, swdflxc, swhrc)
     write (u) swuflx(1:ncol, :), swdflx(1:ncol, :), swhr(1:ncol, :)
     write (u) swuflxc(1:ncol, :), swdflxc(1:ncol, :), swhrc(1:ncol, :)
  end do
  close (u)
end program shim_driver
