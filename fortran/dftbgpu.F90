!> iso_c_binding interface of libdftbgpu.so (include/dftbgpu.h) for the DFTB+ host, to be added as
!> src/dftbp/extlibs/dftbgpu.F90 beside the MAGMA binding (extlibs/magma.F90:30-60), which binds
!> extlibs/magmac.c the same way. Every routine returns 0 on success or a DFTBGPU_ERR_* code.
!>
!> Not compiled in this repository: neither the build machine nor the GPU host has a Fortran
!> compiler. tests/test_abi_layout.py parses the bind(C) derived types below and checks, with a
!> C program compiled against include/dftbgpu.h, that their field order, kinds and offsets are the
!> C structs' (dftbgpu_scc_opts, dftbgpu_energies), and that every interface below names an entry
!> point the header declares with the same number of arguments.
module dftbp_extlibs_dftbgpu
  use, intrinsic :: iso_c_binding, only : c_ptr, c_int, c_double, c_char, c_null_ptr, c_associated, &
      & c_f_pointer
  implicit none
  private

  public :: TDftbGpuOpts, TDftbGpuEnergies
  public :: dftbgpu_default_opts, dftbgpu_create, dftbgpu_destroy, dftbgpu_last_error
  public :: dftbgpu_set_model, dftbgpu_set_geometry, dftbgpu_set_geometry_neighbours, dftbgpu_scc
  public :: dftbgpu_scc_history
  public :: dftbgpu_gradients, dftbgpu_n_orbitals, dftbgpu_get_orbital_populations
  public :: dftbgpu_set_tensor_cores, dftbgpu_set_fp64_emulation, dftbgpu_set_two_stage
  public :: dftbgpu_set_panel_mode, dftbgpu_set_digit_gemm_kernel, dftbgpu_set_fp32_emulation
  public :: dftbgpu_set_dc_staging
  public :: dftbgpuErrorMessage
  public :: DFTBGPU_OK, DFTBGPU_ERR_ARGS, DFTBGPU_ERR_CUDA, DFTBGPU_ERR_NOT_POSDEF, &
      & DFTBGPU_ERR_SCC_NOT_CONVERGED, DFTBGPU_ERR_FERMI, DFTBGPU_ERR_ITER_CAP, DFTBGPU_ERR_STATE, &
      & DFTBGPU_ERR_NO_DEVICE, DFTBGPU_PREC_FP64, DFTBGPU_PREC_MIXED

  !> Status codes (enum in include/dftbgpu.h)
  integer(c_int), parameter :: DFTBGPU_OK = 0
  integer(c_int), parameter :: DFTBGPU_ERR_ARGS = 1
  integer(c_int), parameter :: DFTBGPU_ERR_CUDA = 2
  integer(c_int), parameter :: DFTBGPU_ERR_NOT_POSDEF = 3
  integer(c_int), parameter :: DFTBGPU_ERR_SCC_NOT_CONVERGED = 4
  integer(c_int), parameter :: DFTBGPU_ERR_FERMI = 5
  integer(c_int), parameter :: DFTBGPU_ERR_ITER_CAP = 6
  integer(c_int), parameter :: DFTBGPU_ERR_STATE = 7
  integer(c_int), parameter :: DFTBGPU_ERR_NO_DEVICE = 8

  !> Precision forms (Solver = GpuScc { Precision = FP64 | Mixed })
  integer(c_int), parameter :: DFTBGPU_PREC_FP64 = 0
  integer(c_int), parameter :: DFTBGPU_PREC_MIXED = 1

  !> SCC options (dftbgpu_scc_opts); the fields carry the HSD settings of the Hamiltonian block
  type, bind(C) :: TDftbGpuOpts
    real(c_double) :: kT              ! Filling = Fermi { Temperature }
    real(c_double) :: sccTol          ! SCCTolerance
    integer(c_int) :: maxIter         ! MaxSCCIterations
    integer(c_int) :: minIter         ! MinSCCIterations
    real(c_double) :: mixAlpha        ! Mixer = Broyden { MixingParameter }
    real(c_double) :: mixOmega0       ! InverseJacobiWeight
    real(c_double) :: mixMinWeight    ! MinimalWeight
    real(c_double) :: mixMaxWeight    ! MaximalWeight
    real(c_double) :: mixWeightFac    ! WeightFactor
    real(c_double) :: netCharge       ! Charge
    integer(c_int) :: precision       ! DFTBGPU_PREC_*
    integer(c_int) :: convergentOnly  ! ConvergentSCCOnly
    real(c_double) :: mixedSwitchTol  ! Precision = Mixed: leave the FP32 eigensolves below this error
  end type TDftbGpuOpts

  !> Energy terms (dftbgpu_energies), copied into dftbEnergy(1) by the caller
  type, bind(C) :: TDftbGpuEnergies
    real(c_double) :: EnonSCC
    real(c_double) :: Escc
    real(c_double) :: Erep
    real(c_double) :: Eband
    real(c_double) :: TS
    real(c_double) :: E0
    real(c_double) :: Etotal
    real(c_double) :: EMermin
  end type TDftbGpuEnergies

  interface

    subroutine dftbgpu_default_opts(opts) bind(C, name="dftbgpu_default_opts")
      import :: TDftbGpuOpts
      type(TDftbGpuOpts), intent(out) :: opts
    end subroutine dftbgpu_default_opts

    function dftbgpu_create(ctx, device) result(stat) bind(C, name="dftbgpu_create")
      import :: c_ptr, c_int
      type(c_ptr), intent(out) :: ctx
      integer(c_int), value :: device
      integer(c_int) :: stat
    end function dftbgpu_create

    function dftbgpu_destroy(ctx) result(stat) bind(C, name="dftbgpu_destroy")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int) :: stat
    end function dftbgpu_destroy

    function dftbgpu_last_error(ctx) result(msg) bind(C, name="dftbgpu_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
      type(c_ptr) :: msg
    end function dftbgpu_last_error

    !> Species and SK tables of the SK containers (parser.F90:3668-3886, getFullTable :4061-4130)
    function dftbgpu_set_model(ctx, nSpecies, nShell, angShell, onsite, hubbU, refOcc, skDist, skRows,&
        & skNInt, skHam, skOver, repNSpline, repData) result(stat) bind(C, name="dftbgpu_set_model")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nSpecies
      integer(c_int), intent(in) :: nShell(*), angShell(*), skRows(*), skNInt(*), repNSpline(*)
      real(c_double), intent(in) :: onsite(*), hubbU(*), refOcc(*), skDist(*), skHam(*), skOver(*)
      real(c_double), intent(in) :: repData(*)
      integer(c_int) :: stat
    end function dftbgpu_set_model

    !> Geometry in place of buildH0/buildS (main.F90:1219-1222): coords(3, nAtom) in Bohr,
    !> species 0-based (species0 - 1)
    function dftbgpu_set_geometry(ctx, nAtom, coords, species) result(stat)&
        & bind(C, name="dftbgpu_set_geometry")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nAtom
      real(c_double), intent(in) :: coords(3, *)
      integer(c_int), intent(in) :: species(*)
      integer(c_int) :: stat
    end function dftbgpu_set_geometry

    !> Geometry with the host's neighbour list (cluster case): nNeighbourSK(nAtom) and
    !> iNeighbour(0:maxNeighbour, nAtom) of TNeighbourList (dftb/periodic.F90), passed 0-based
    !> (iNeighbour - 1, species0 - 1); the GPU then keeps the host's pairs instead of its own
    function dftbgpu_set_geometry_neighbours(ctx, nAtom, coords, species, nNeighbourSK, iNeighbour,&
        & maxNeighbour) result(stat) bind(C, name="dftbgpu_set_geometry_neighbours")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: nAtom
      integer(c_int), value :: maxNeighbour
      real(c_double), intent(in) :: coords(3, *)
      integer(c_int), intent(in) :: species(*), nNeighbourSK(*), iNeighbour(0:maxNeighbour, *)
      integer(c_int) :: stat
    end function dftbgpu_set_geometry_neighbours

    !> SCC cycle in place of the lpSCC body (main.F90:1429-1563). qInit(nAtom) atomic populations
    !> (pass the reference q0 to start from neutral atoms); outputs as in include/dftbgpu.h
    function dftbgpu_scc(ctx, opts, qInit, energies, ef, eigen, filling, qOut, nIter, converged)&
        & result(stat) bind(C, name="dftbgpu_scc")
      import :: c_ptr, c_int, c_double, TDftbGpuOpts, TDftbGpuEnergies
      type(c_ptr), value :: ctx
      type(TDftbGpuOpts), intent(in) :: opts
      real(c_double), intent(in) :: qInit(*)
      type(TDftbGpuEnergies), intent(out) :: energies
      real(c_double), intent(out) :: ef, eigen(*), filling(*), qOut(*)
      integer(c_int), intent(out) :: nIter, converged
      integer(c_int) :: stat
    end function dftbgpu_scc

    !> Per-iteration SCC table (printSccHeader/printSccInfo, mainio.F90:4781-4845)
    function dftbgpu_scc_history(ctx, cap, energy, error, precision, ms) result(nIter)&
        & bind(C, name="dftbgpu_scc_history")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: cap
      real(c_double), intent(out) :: energy(*), error(*), ms(*)
      integer(c_int), intent(out) :: precision(*)
      integer(c_int) :: nIter
    end function dftbgpu_scc_history

    !> Energy gradient (this%derivs) in place of main.F90:1777-1800
    function dftbgpu_gradients(ctx, grad) result(stat) bind(C, name="dftbgpu_gradients")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: grad(3, *)
      integer(c_int) :: stat
    end function dftbgpu_gradients

    function dftbgpu_n_orbitals(ctx, nOrb) result(stat) bind(C, name="dftbgpu_n_orbitals")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int), intent(out) :: nOrb
      integer(c_int) :: stat
    end function dftbgpu_n_orbitals

    !> Orbital-resolved Mulliken populations (qOutput collapsed to the nOrb orbitals in atom order)
    function dftbgpu_get_orbital_populations(ctx, qOrb) result(stat)&
        & bind(C, name="dftbgpu_get_orbital_populations")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: qOrb(*)
      integer(c_int) :: stat
    end function dftbgpu_get_orbital_populations

    !> Solver = GpuScc { TensorCores, Fp64Emulation, TwoStage }: process-wide switches of the mixed
    !> form; each returns the previous setting
    function dftbgpu_set_tensor_cores(enable) result(prev) bind(C, name="dftbgpu_set_tensor_cores")
      import :: c_int
      integer(c_int), value :: enable
      integer(c_int) :: prev
    end function dftbgpu_set_tensor_cores

    function dftbgpu_set_fp64_emulation(enable) result(prev) bind(C, name="dftbgpu_set_fp64_emulation")
      import :: c_int
      integer(c_int), value :: enable
      integer(c_int) :: prev
    end function dftbgpu_set_fp64_emulation

    !> Fp32Emulation: the FP32 eigensolves' large products as exact digit-slice tensor-core products
    function dftbgpu_set_fp32_emulation(enable) result(prev) bind(C, name="dftbgpu_set_fp32_emulation")
      import :: c_int
      integer(c_int), value :: enable
      integer(c_int) :: prev
    end function dftbgpu_set_fp32_emulation

    !> TwoStage = 0 (one-stage), 1 (two-stage) or 2 (by size, the default); -1 for an invalid mode
    function dftbgpu_set_two_stage(mode) result(prev) bind(C, name="dftbgpu_set_two_stage")
      import :: c_int
      integer(c_int), value :: mode
      integer(c_int) :: prev
    end function dftbgpu_set_two_stage

    !> PanelKernel = 1 (trailing tiles on chip per panel, the default), 0 (re-read per column) or 2
    !> (on-chip kernel with small limits, tests); -1 for an invalid mode
    function dftbgpu_set_panel_mode(mode) result(prev) bind(C, name="dftbgpu_set_panel_mode")
      import :: c_int
      integer(c_int), value :: mode
      integer(c_int) :: prev
    end function dftbgpu_set_panel_mode

    !> DcStaging = 1 (merges of the tridiagonal divide and conquer deflated in shared memory where
    !> they fit, the default) or 0 (all in global memory); returns the previous setting
    function dftbgpu_set_dc_staging(enable) result(prev) bind(C, name="dftbgpu_set_dc_staging")
      import :: c_int
      integer(c_int), value :: enable
      integer(c_int) :: prev
    end function dftbgpu_set_dc_staging

    !> Fp64EmulationKernel = 0 (single-stage, the default) or 1 (TMA-pipelined); -1 for an invalid mode
    function dftbgpu_set_digit_gemm_kernel(mode) result(prev) bind(C, name="dftbgpu_set_digit_gemm_kernel")
      import :: c_int
      integer(c_int), value :: mode
      integer(c_int) :: prev
    end function dftbgpu_set_digit_gemm_kernel

  end interface

contains

  !> Message of the last failed call of a context, for @:RAISE_ERROR(errStatus, stat, msg)
  function dftbgpuErrorMessage(ctx) result(msg)
    type(c_ptr), intent(in) :: ctx
    character(len=:), allocatable :: msg
    character(kind=c_char), pointer :: chars(:)
    type(c_ptr) :: cmsg
    integer :: ii

    cmsg = dftbgpu_last_error(ctx)
    if (.not. c_associated(cmsg)) then
      msg = "dftbgpu: no message"
      return
    end if
    call c_f_pointer(cmsg, chars, [1024])
    ii = 0
    do while (ii < 1024)
      if (chars(ii + 1) == achar(0)) exit
      ii = ii + 1
    end do
    allocate(character(len=ii) :: msg)
    do ii = 1, len(msg)
      msg(ii:ii) = chars(ii)
    end do
  end function dftbgpuErrorMessage

end module dftbp_extlibs_dftbgpu
