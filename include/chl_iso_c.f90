!-----------------------------------------------------------------------!
! ISO_C_BINDING interface to libchl (include/chl.h) and a drop-in      !
! replacement of the reference's time-step layer.                      !
!                                                                       !
! Module chl_iso_c declares the C entry points.  Module                 !
! time_integration_gpu provides compute_time_step_RK3 and compute_dt    !
! with the names and (no-argument) calling convention of the reference  !
! (time_integration.f90:24 and :102); they read and write the same      !
! module variables of `global` (U, V, W, nu_t, dt, t, dPdx, alpha_x).   !
!                                                                       !
! Only the single-process form is offered: one rank holds the whole     !
! domain on one GPU (the global arrays of a P=1 run, whose loop ranges  !
! are the union of the reference's per-rank ranges).                    !
!-----------------------------------------------------------------------!
Module chl_iso_c
  Use, Intrinsic :: iso_c_binding
  Implicit None

  Type, bind(C) :: chl_grid_desc
     Integer(c_int) :: nx, ny, nz
     Type(c_ptr)    :: x, y, z
     Real(c_double) :: nu, CFL, dPdx
     Integer(c_int) :: x_mass_cte, LES_model, Dirichlet_nu_t, wall_model
     Real(c_double) :: Cs, Re_tau
  End Type chl_grid_desc

  Interface
     Integer(c_int) Function chl_create(desc, h) bind(C, name='chl_create')
       Import :: c_int, c_ptr, chl_grid_desc
       Type(chl_grid_desc), Intent(In) :: desc
       Type(c_ptr), Intent(Out) :: h
     End Function chl_create

     Integer(c_int) Function chl_destroy(h) bind(C, name='chl_destroy')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
     End Function chl_destroy

     Integer(c_int) Function chl_upload(h, inst, U, V, W) bind(C, name='chl_upload')
       Import :: c_int, c_ptr, c_double
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: inst
       Real(c_double), Intent(In) :: U(*), V(*), W(*)
     End Function chl_upload

     Integer(c_int) Function chl_set_fields(h, inst, U, V, W) bind(C, name='chl_set_fields')
       Import :: c_int, c_ptr, c_double
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: inst
       Real(c_double), Intent(In) :: U(*), V(*), W(*)
     End Function chl_set_fields

     ! pointers so that unwanted fields can be passed as c_null_ptr
     Integer(c_int) Function chl_download(h, inst, U, V, W, P, nu_t) bind(C, name='chl_download')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: inst
       Type(c_ptr), Value :: U, V, W, P, nu_t
     End Function chl_download

     Integer(c_int) Function chl_set_wall_stress(h, inst, alpha_x) bind(C, name='chl_set_wall_stress')
       Import :: c_int, c_ptr, c_double
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: inst
       Real(c_double), Intent(In) :: alpha_x(*)
     End Function chl_set_wall_stress

     Integer(c_int) Function chl_get_scalars(h, inst, s) bind(C, name='chl_get_scalars')
       Import :: c_int, c_ptr, c_double
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: inst
       Real(c_double), Intent(Out) :: s(4)
     End Function chl_get_scalars

     Integer(c_int) Function chl_set_scalars(h, inst, s) bind(C, name='chl_set_scalars')
       Import :: c_int, c_ptr, c_double
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: inst
       Real(c_double), Intent(In) :: s(4)
     End Function chl_set_scalars

     Integer(c_int) Function chl_compute_dt(h) bind(C, name='chl_compute_dt')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
     End Function chl_compute_dt

     Integer(c_int) Function chl_compute_time_step_RK3(h) bind(C, name='chl_compute_time_step_RK3')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
     End Function chl_compute_time_step_RK3

     Integer(c_int) Function chl_rk3_step(h, nsteps) bind(C, name='chl_rk3_step')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
       Integer(c_int), Value :: nsteps
     End Function chl_rk3_step

     Integer(c_int) Function chl_compute_pressure(h) bind(C, name='chl_compute_pressure')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
     End Function chl_compute_pressure

     Integer(c_int) Function chl_synchronize(h) bind(C, name='chl_synchronize')
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: h
     End Function chl_synchronize

     Type(c_ptr) Function chl_last_error(h) bind(C, name='chl_last_error')
       Import :: c_ptr
       Type(c_ptr), Value :: h
     End Function chl_last_error
  End Interface
End Module chl_iso_c

Module time_integration_gpu
  Use iso_fortran_env, Only : error_unit, Int32, Int64
  Use, Intrinsic :: iso_c_binding
  Use global
  Use chl_iso_c
  Implicit None

  Type(c_ptr), Save :: chl_h = c_null_ptr
  Logical, Save :: chl_ready = .False.

Contains

  Subroutine chl_check(rc, where)
    Integer(c_int), Intent(In) :: rc
    Character(*), Intent(In) :: where
    If (rc /= 0) Then
       Write(error_unit,*) 'libchl error in ', where, ' code ', rc
       Stop 'libchl failure'
    End If
  End Subroutine chl_check

  ! Called once after initialize (initialization.f90:23): creates the
  ! device instance from the global grid and parameters and uploads U,V,W.
  Subroutine chl_initialize(wall_model)
    Integer(c_int), Intent(In) :: wall_model
    Type(chl_grid_desc) :: d
    Real(c_double), Target, Save, Allocatable :: xs(:), ys(:), zs(:)
    xs = x_global; ys = y_global; zs = z_global
    d%nx = nx_global; d%ny = ny_global; d%nz = nz_global
    d%x = c_loc(xs); d%y = c_loc(ys); d%z = c_loc(zs)
    d%nu = nu; d%CFL = CFL; d%dPdx = dPdx
    d%x_mass_cte = x_mass_cte; d%LES_model = LES_model; d%Dirichlet_nu_t = Dirichlet_nu_t
    d%wall_model = wall_model; d%Cs = 0.1d0; d%Re_tau = 0d0
    Call chl_check(chl_create(d, chl_h), 'chl_create')
    Call chl_check(chl_upload(chl_h, 0_c_int, U, V, W), 'chl_upload')
    Call chl_check(chl_set_wall_stress(chl_h, 0_c_int, alpha_x), 'chl_set_wall_stress')
    chl_ready = .True.
  End Subroutine chl_initialize

  ! Drop-in for time_integration.f90:102 (dt left on the device and copied back)
  Subroutine compute_dt
    Real(c_double) :: s(4)
    Call chl_check(chl_compute_dt(chl_h), 'chl_compute_dt')
    Call chl_check(chl_get_scalars(chl_h, 0_c_int, s), 'chl_get_scalars')
    dt = s(1)
  End Subroutine compute_dt

  ! Drop-in for time_integration.f90:24: U, V, W, nu_t, t and dPdx of
  ! `global` are updated from the device after the step.
  Subroutine compute_time_step_RK3
    Real(c_double) :: s(4)
    Call chl_check(chl_set_wall_stress(chl_h, 0_c_int, alpha_x), 'chl_set_wall_stress')
    Call chl_check(chl_get_scalars(chl_h, 0_c_int, s), 'chl_get_scalars')
    s(1) = dt; s(2) = t
    Call chl_check(chl_set_scalars(chl_h, 0_c_int, s), 'chl_set_scalars')
    Call chl_check(chl_compute_time_step_RK3(chl_h), 'chl_compute_time_step_RK3')
    Call chl_check(chl_download(chl_h, 0_c_int, c_loc(U), c_loc(V), c_loc(W), c_null_ptr, &
                                c_loc(nu_t)), 'chl_download')
    Call chl_check(chl_get_scalars(chl_h, 0_c_int, s), 'chl_get_scalars')
    t = s(2); dPdx = s(3)
  End Subroutine compute_time_step_RK3

  Subroutine chl_finalize
    If (chl_ready) Call chl_check(chl_destroy(chl_h), 'chl_destroy')
    chl_ready = .False.
  End Subroutine chl_finalize

End Module time_integration_gpu
