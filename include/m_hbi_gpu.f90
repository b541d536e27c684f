! m_hbi_gpu.f90 -- Fortran binding of libhbigpu (include/hbi_gpu.h) under
! HACApK's own names, so that HBI's driver (main_LH.f90) switches to the GPU
! library by replacing
!
!     use m_HACApK_solve
!     use m_HACApK_base
!     use m_HACApK_use
!     use m_HACApK_calc_entry_ij
!
! with `use m_hbi_gpu`.  The module defines the derived types main_LH.f90
! touches, with the components it reads or writes (st_HACApK_lcontrol%param,
! %lpmd, %time; st_HACApK_calc_entry%xcol ... %problem, %v, %md, %w;
! st_HACApK_leafmtxp%ndlfs; st_HACApK_latticevec%ndc, %lodc, %vs), and the
! HACApK routines of the hot path with the reference's argument lists:
!
!   HACApK_init(nd, st_ctl, st_bemv, icomma)                m_HACApK_base.f90:246
!   HACApK_generate(st_leafmtxp, st_bemv, st_ctl, coord, ztol)   m_HACApK_use.f90:133
!   HACApK_construct_LH(st_LHp, st_leafmtxp, st_bemv, st_ctl, coord, ztol)
!                                                           m_HACApK_use.f90:263
!   HACApK_gen_lattice_vector(st_vec, st_leafmtxp, st_ctl)  m_HACApK_base.f90:3449
!   HACApK_adot_lattice_hyp(st_au, st_LHp, st_ctl, wws, st_u)  m_HACApK_solve.f90:220
!   HACApK_free_leafmtxp(st_leafmtxp)                       m_HACApK_base.f90:3084
!   HACApK_finalize(st_ctl)                                 m_HACApK_base.f90:385
!
! Each wraps one extern "C" entry point of hbi_gpu.h through ISO_C_BINDING.
! The GPU library owns the H-matrix: the Fortran types carry an opaque handle
! (component h) next to the components the driver uses.  Like the reference,
! the routines return 0 and stop the program on a fatal error (the C entry
! points themselves never abort; they return a status and a message).
!
! One MPI rank: the communicators of lpmd(1), (31) and (35) are the icomma
! the driver passes, ranks lpmd(3), (33), (37) are 0 and sizes lpmd(2), (32),
! (36) are 1, as HACApK sets them for a single process.
!
! The factor storage of HACApK_construct_LH is the module variable
! hbi_factor_storage (HBI_STORE_F64 unless the driver sets it).
module m_hbi_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: HBI_STORE_F64 = 0, HBI_STORE_F32 = 1, HBI_STORE_BF16 = 2
  integer(c_int), parameter :: HBI_2DVS = 1, HBI_3DPH = 2, HBI_3DNR = 3, HBI_3DNT = 4, &
                               HBI_2DPH = 5, HBI_2DN = 6, HBI_3DHT = 7
  integer(c_int) :: hbi_factor_storage = HBI_STORE_F64

  ! st_HACApK_calc_entry (m_HACApK_calc_entry_ij.f90:7-19)
  type :: st_HACApK_calc_entry
    real(8), pointer :: ao(:) => null()
    character(128) :: problem = ''
    integer :: nd = 0, lp61 = 0
    real(8), pointer :: xcol(:) => null(), ycol(:) => null(), zcol(:) => null()
    real(8), pointer :: xel(:) => null(), xer(:) => null(), yel(:) => null(), yer(:) => null()
    real(8), pointer :: ang(:) => null(), angd(:) => null(), rake(:) => null()
    real(8), pointer :: xs1(:) => null(), xs2(:) => null(), xs3(:) => null(), xs4(:) => null()
    real(8), pointer :: zs1(:) => null(), zs2(:) => null(), zs3(:) => null(), zs4(:) => null()
    real(8), pointer :: ys1(:) => null(), ys2(:) => null(), ys3(:) => null(), ys4(:) => null()
    real(8), pointer :: ev11(:) => null(), ev12(:) => null(), ev13(:) => null()
    real(8), pointer :: ev21(:) => null(), ev22(:) => null(), ev23(:) => null()
    real(8), pointer :: ev31(:) => null(), ev32(:) => null(), ev33(:) => null()
    real(8), pointer :: ds(:) => null(), dsl(:) => null(), dsd(:) => null()
    real(8) :: w = 0d0
    character(128) :: v = 's', md = 's'
  end type st_HACApK_calc_entry

  ! st_HACApK_lcontrol (m_HACApK_base.f90:146-161)
  type :: st_HACApK_lcontrol
    integer(4) :: lf_umpi = 1
    real(8), pointer :: param(:) => null()
    real(8), pointer :: time(:) => null()
    integer(4), pointer :: lpmd(:) => null()
    integer(4), pointer :: lod(:) => null()
    type(c_ptr) :: h = c_null_ptr            ! hbi_ctl*
  end type st_HACApK_lcontrol

  ! st_HACApK_leafmtxp (m_HACApK_base.f90:108-136)
  type :: st_HACApK_leafmtxp
    integer(4) :: nd = 0, nlf = 0, ktmax = 0
    integer(4) :: ndlfs = 0, ndtfs = 0
    type(c_ptr) :: h = c_null_ptr            ! hbi_leafmtxp*
  end type st_HACApK_leafmtxp

  ! st_HACApK_LHp (m_HACApK_base.f90:164-182)
  type :: st_HACApK_LHp
    integer(4) :: nd = 0, nlf = 0
    integer(4) :: ndlfs = 0, ndtfs = 0
    type(c_ptr) :: h = c_null_ptr            ! hbi_lhp*
  end type st_HACApK_LHp

  ! st_HACApK_latticevec (m_HACApK_base.f90:185-211)
  type :: st_HACApK_latticevec
    integer(4) :: ndc = 0, nlfc = 1
    integer(4), pointer :: lodc(:) => null()
    real(8), pointer :: vs(:) => null()
  end type st_HACApK_latticevec

  ! hbi_bemv (include/hbi_gpu.h)
  type, bind(c) :: hbi_bemv_c
    integer(c_int) :: problem, nd
    character(kind=c_char) :: v, md
    type(c_ptr) :: xcol, ycol, zcol, xel, xer, ang, angd, dsl, dsd, rake
    real(c_double) :: w
    type(c_ptr) :: xs1, xs2, xs3, ys1, ys2, ys3, zs1, zs2, zs3
    type(c_ptr) :: ev11, ev12, ev13, ev21, ev22, ev23, ev31, ev32, ev33
    type(c_ptr) :: yel, yer
  end type hbi_bemv_c

  ! ---- the C ABI (include/hbi_gpu.h) ------------------------------------
  interface
    function hbi_last_error() bind(c, name='hbi_last_error') result(msg)
      import :: c_ptr
      type(c_ptr) :: msg
    end function hbi_last_error
    function hbi_init(nd, ctl) bind(c, name='hbi_init') result(rc)
      import :: c_int, c_ptr
      integer(c_int), value :: nd
      type(c_ptr) :: ctl
      integer(c_int) :: rc
    end function hbi_init
    function hbi_param_set(ctl, param100) bind(c, name='hbi_param_set') result(rc)
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctl
      real(c_double) :: param100(100)
      integer(c_int) :: rc
    end function hbi_param_set
    function hbi_param_get(ctl, param100) bind(c, name='hbi_param_get') result(rc)
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctl
      real(c_double) :: param100(100)
      integer(c_int) :: rc
    end function hbi_param_get
    function hbi_finalize(ctl) bind(c, name='hbi_finalize') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctl
      integer(c_int) :: rc
    end function hbi_finalize
    function hbi_generate(lf, bemv, ctl, coord, ztol) bind(c, name='hbi_generate') result(rc)
      import :: c_int, c_ptr, c_double, hbi_bemv_c
      type(c_ptr) :: lf
      type(hbi_bemv_c) :: bemv
      type(c_ptr), value :: ctl
      real(c_double) :: coord(*)
      real(c_double), value :: ztol
      integer(c_int) :: rc
    end function hbi_generate
    function hbi_free_leafmtxp(lf) bind(c, name='hbi_free_leafmtxp') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: lf
      integer(c_int) :: rc
    end function hbi_free_leafmtxp
    function hbi_construct_lh(lh, lf, ctl, storage) bind(c, name='hbi_construct_lh') result(rc)
      import :: c_int, c_ptr
      type(c_ptr) :: lh
      type(c_ptr), value :: lf, ctl
      integer(c_int), value :: storage
      integer(c_int) :: rc
    end function hbi_construct_lh
    function hbi_free_lh(lh) bind(c, name='hbi_free_lh') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: lh
      integer(c_int) :: rc
    end function hbi_free_lh
    function hbi_gen_lattice_vector(ctl, ndc, lodc) bind(c, name='hbi_gen_lattice_vector') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctl
      integer(c_int) :: ndc
      type(c_ptr), value :: lodc
      integer(c_int) :: rc
    end function hbi_gen_lattice_vector
    function hbi_adot_lattice_hyp(au, lh, ctl, wws, u) bind(c, name='hbi_adot_lattice_hyp') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: au, lh, ctl, wws, u
      integer(c_int) :: rc
    end function hbi_adot_lattice_hyp
    function hbi_get_lod(ctl, lod) bind(c, name='hbi_get_lod') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: ctl, lod
      integer(c_int) :: rc
    end function hbi_get_lod
    function hbi_leaf_count(lf, nleaf, ktmax) bind(c, name='hbi_leaf_count') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: lf
      integer(c_int) :: nleaf, ktmax
      integer(c_int) :: rc
    end function hbi_leaf_count
    function hbi_lh_check_error(lh) bind(c, name='hbi_lh_check_error') result(rc)
      import :: c_int, c_ptr
      type(c_ptr), value :: lh
      integer(c_int) :: rc
    end function hbi_lh_check_error
    function c_strlen(s) bind(c, name='strlen') result(n)
      import :: c_ptr, c_size_t
      type(c_ptr), value :: s
      integer(c_size_t) :: n
    end function c_strlen
  end interface

  private :: hbi_bemv_c, check, problem_id, bemv_of, vptr, c_strlen

contains

  ! message of the last failed call, then stop (the reference stops too)
  subroutine check(rc, where)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: m(:)
    type(c_ptr) :: p
    integer :: n, i
    character(512) :: msg
    if (rc == 0) return
    p = hbi_last_error()
    msg = ''
    if (c_associated(p)) then
      n = int(min(c_strlen(p), 512_c_size_t))
      call c_f_pointer(p, m, [n])
      do i = 1, n
        msg(i:i) = m(i)
      end do
    end if
    print *, trim(where), ': error ', rc, ': ', trim(msg)
    error stop 1
  end subroutine check

  ! st_bemv%problem (the names HACApK_entry_ij selects on,
  ! m_HACApK_calc_entry_ij.f90:31-88) to the HBI_* kinds of the C ABI
  integer(c_int) function problem_id(name)
    character(*), intent(in) :: name
    select case (trim(name))
    case ('2dvs'); problem_id = HBI_2DVS
    case ('3dph', '3dhr'); problem_id = HBI_3DPH
    case ('3dnr'); problem_id = HBI_3DNR
    case ('3dnt', '3dn'); problem_id = HBI_3DNT
    case ('2dph', '2dnh'); problem_id = HBI_2DPH
    case ('2dn'); problem_id = HBI_2DN
    case ('3dht', '3dh'); problem_id = HBI_3DHT
    case default; problem_id = -1
    end select
  end function problem_id

  type(c_ptr) function vptr(a)
    real(8), pointer, intent(in) :: a(:)
    if (associated(a)) then
      vptr = c_loc(a(1))
    else
      vptr = c_null_ptr
    end if
  end function vptr

  type(hbi_bemv_c) function bemv_of(st_bemv)
    type(st_HACApK_calc_entry), intent(in) :: st_bemv
    bemv_of%problem = problem_id(st_bemv%problem)
    bemv_of%nd = st_bemv%nd
    bemv_of%v = st_bemv%v(1:1)
    bemv_of%md = st_bemv%md(1:1)
    bemv_of%w = st_bemv%w
    bemv_of%xcol = vptr(st_bemv%xcol); bemv_of%ycol = vptr(st_bemv%ycol); bemv_of%zcol = vptr(st_bemv%zcol)
    bemv_of%xel = vptr(st_bemv%xel); bemv_of%xer = vptr(st_bemv%xer)
    bemv_of%yel = vptr(st_bemv%yel); bemv_of%yer = vptr(st_bemv%yer)
    bemv_of%ang = vptr(st_bemv%ang); bemv_of%angd = vptr(st_bemv%angd)
    bemv_of%dsl = vptr(st_bemv%dsl); bemv_of%dsd = vptr(st_bemv%dsd); bemv_of%rake = vptr(st_bemv%rake)
    bemv_of%xs1 = vptr(st_bemv%xs1); bemv_of%xs2 = vptr(st_bemv%xs2); bemv_of%xs3 = vptr(st_bemv%xs3)
    bemv_of%ys1 = vptr(st_bemv%ys1); bemv_of%ys2 = vptr(st_bemv%ys2); bemv_of%ys3 = vptr(st_bemv%ys3)
    bemv_of%zs1 = vptr(st_bemv%zs1); bemv_of%zs2 = vptr(st_bemv%zs2); bemv_of%zs3 = vptr(st_bemv%zs3)
    bemv_of%ev11 = vptr(st_bemv%ev11); bemv_of%ev12 = vptr(st_bemv%ev12); bemv_of%ev13 = vptr(st_bemv%ev13)
    bemv_of%ev21 = vptr(st_bemv%ev21); bemv_of%ev22 = vptr(st_bemv%ev22); bemv_of%ev23 = vptr(st_bemv%ev23)
    bemv_of%ev31 = vptr(st_bemv%ev31); bemv_of%ev32 = vptr(st_bemv%ev32); bemv_of%ev33 = vptr(st_bemv%ev33)
  end function bemv_of

  ! HACApK_init (m_HACApK_base.f90:246-345)
  integer function HACApK_init(nd, st_ctl, st_bemv, icomma)
    integer, intent(in) :: nd
    type(st_HACApK_lcontrol) :: st_ctl
    type(st_HACApK_calc_entry) :: st_bemv
    integer, optional :: icomma
    integer :: icomm
    icomm = 0
    if (present(icomma)) icomm = icomma
    allocate (st_ctl%param(100), st_ctl%time(10), st_ctl%lpmd(50), st_ctl%lod(nd))
    st_ctl%time = 0d0
    st_ctl%lpmd = 0
    st_ctl%lpmd(1) = icomm; st_ctl%lpmd(2) = 1; st_ctl%lpmd(3) = 0; st_ctl%lpmd(20) = 1
    st_ctl%lpmd(31) = icomm; st_ctl%lpmd(32) = 1; st_ctl%lpmd(33) = 0
    st_ctl%lpmd(35) = icomm; st_ctl%lpmd(36) = 1; st_ctl%lpmd(37) = 0
    st_ctl%lod = 0
    st_bemv%nd = nd
    call check(hbi_init(int(nd, c_int), st_ctl%h), 'HACApK_init')
    call check(hbi_param_get(st_ctl%h, st_ctl%param), 'HACApK_init')
    HACApK_init = 0
  end function HACApK_init

  ! HACApK_generate (m_HACApK_use.f90:133-260): tree, leaves and ACA+ on the GPU
  integer function HACApK_generate(st_leafmtxp, st_bemv, st_ctl, coord, ztol)
    type(st_HACApK_leafmtxp) :: st_leafmtxp
    type(st_HACApK_calc_entry) :: st_bemv
    type(st_HACApK_lcontrol) :: st_ctl
    real(8) :: coord(st_bemv%nd, *)
    real(8) :: ztol
    type(hbi_bemv_c) :: b
    integer(c_int) :: nlf, ktmax
    b = bemv_of(st_bemv)
    call check(hbi_param_set(st_ctl%h, st_ctl%param), 'HACApK_generate')
    call check(hbi_generate(st_leafmtxp%h, b, st_ctl%h, coord, real(ztol, c_double)), 'HACApK_generate')
    call check(hbi_param_get(st_ctl%h, st_ctl%param), 'HACApK_generate')
    call check(hbi_get_lod(st_ctl%h, c_loc(st_ctl%lod(1))), 'HACApK_generate')
    call check(hbi_leaf_count(st_leafmtxp%h, nlf, ktmax), 'HACApK_generate')
    st_leafmtxp%nd = st_bemv%nd
    st_leafmtxp%nlf = nlf
    st_leafmtxp%ktmax = ktmax
    st_leafmtxp%ndlfs = st_bemv%nd
    st_leafmtxp%ndtfs = st_bemv%nd
    HACApK_generate = 0
  end function HACApK_generate

  ! HACApK_construct_LH (m_HACApK_use.f90:263-366): the matvec operator with
  ! factors stored as hbi_factor_storage
  integer function HACApK_construct_LH(st_LHp, st_leafmtxp, st_bemv, st_ctl, coord, ztol)
    type(st_HACApK_LHp) :: st_LHp
    type(st_HACApK_leafmtxp) :: st_leafmtxp
    type(st_HACApK_calc_entry) :: st_bemv
    type(st_HACApK_lcontrol) :: st_ctl
    real(8) :: coord(st_bemv%nd, *)
    real(8) :: ztol
    call check(hbi_construct_lh(st_LHp%h, st_leafmtxp%h, st_ctl%h, hbi_factor_storage), 'HACApK_construct_LH')
    st_LHp%nd = st_leafmtxp%nd
    st_LHp%nlf = 1
    st_LHp%ndlfs = st_leafmtxp%nd
    st_LHp%ndtfs = st_leafmtxp%nd
    HACApK_construct_LH = 0
  end function HACApK_construct_LH

  ! HACApK_gen_lattice_vector (m_HACApK_base.f90:3449-3500): ndc, lodc, vs
  integer function HACApK_gen_lattice_vector(st_vec, st_leafmtxp, st_ctl)
    type(st_HACApK_latticevec) :: st_vec
    type(st_HACApK_leafmtxp) :: st_leafmtxp
    type(st_HACApK_lcontrol) :: st_ctl
    integer(c_int) :: ndc
    call check(hbi_gen_lattice_vector(st_ctl%h, ndc, c_null_ptr), 'HACApK_gen_lattice_vector')
    st_vec%ndc = ndc
    st_vec%nlfc = 1
    allocate (st_vec%lodc(ndc), st_vec%vs(ndc))
    st_vec%vs = 0d0
    call check(hbi_gen_lattice_vector(st_ctl%h, ndc, c_loc(st_vec%lodc(1))), 'HACApK_gen_lattice_vector')
    HACApK_gen_lattice_vector = 0
  end function HACApK_gen_lattice_vector

  ! HACApK_adot_lattice_hyp (m_HACApK_solve.f90:220-337): st_au%vs = H st_u%vs
  subroutine HACApK_adot_lattice_hyp(st_au, st_LHp, st_ctl, wws, st_u)
    type(st_HACApK_latticevec) :: st_au, st_u
    type(st_HACApK_LHp) :: st_LHp
    type(st_HACApK_lcontrol) :: st_ctl
    real(8) :: wws(:)
    call check(hbi_adot_lattice_hyp(c_loc(st_au%vs(1)), st_LHp%h, st_ctl%h, c_null_ptr, c_loc(st_u%vs(1))), &
               'HACApK_adot_lattice_hyp')
  end subroutine HACApK_adot_lattice_hyp

  ! HACApK_free_leafmtxp (m_HACApK_base.f90:3084)
  integer function HACApK_free_leafmtxp(st_leafmtxp)
    type(st_HACApK_leafmtxp) :: st_leafmtxp
    call check(hbi_free_leafmtxp(st_leafmtxp%h), 'HACApK_free_leafmtxp')
    st_leafmtxp%h = c_null_ptr
    HACApK_free_leafmtxp = 0
  end function HACApK_free_leafmtxp

  ! HACApK_finalize (m_HACApK_base.f90:385-393)
  integer function HACApK_finalize(st_ctl)
    type(st_HACApK_lcontrol) :: st_ctl
    call check(hbi_finalize(st_ctl%h), 'HACApK_finalize')
    st_ctl%h = c_null_ptr
    HACApK_finalize = 0
  end function HACApK_finalize

end module m_hbi_gpu
