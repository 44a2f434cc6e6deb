!> Solver glue of the GpuScc electronic solver for processGeometry (dftbplus/main.F90), to be added
!> as src/dftbp/elecsolvers/gpuscc.F90. It owns one dftbgpu context and turns the plain arrays the
!> host already holds into the library's calls; statuses come back as (stat, message) pairs that
!> the caller raises with @:RAISE_ERROR(errStatus, stat, msg), so ConvergentSCCOnly keeps its
!> meaning (main.F90:1679-1690). Where each call goes in processGeometry, and how the SK containers
!> map onto setModel's packed arrays, is in INTEGRATION.md.
!>
!> Not compiled in this repository (no Fortran compiler on the build machine or the GPU host).
module dftbp_elecsolvers_gpuscc
  use, intrinsic :: iso_c_binding, only : c_ptr, c_int, c_double, c_null_ptr, c_associated
  use dftbp_extlibs_dftbgpu
  implicit none
  private

  public :: TGpuSccSolver, TGpuSccSolver_init

  !> One GPU context and the SCC settings parsed from Solver = GpuScc { ... }
  type :: TGpuSccSolver
    type(c_ptr) :: ctx = c_null_ptr
    type(TDftbGpuOpts) :: opts
    integer :: nAtom = 0
    integer :: nOrb = 0
  contains
    procedure :: setModel
    procedure :: setGeometry
    procedure :: runScc
    procedure :: getGradients
    procedure :: sccTable
    final :: TGpuSccSolver_final
  end type TGpuSccSolver

contains

  !> Create the context on a device and take the HSD settings (defaults of parser.F90:5786-5790
  !> for anything not given)
  subroutine TGpuSccSolver_init(this, device, kT, sccTol, maxIter, mixAlpha, netCharge, precision,&
      & convergentOnly, stat, msg)
    type(TGpuSccSolver), intent(out) :: this
    integer, intent(in) :: device, maxIter, precision
    real(c_double), intent(in) :: kT, sccTol, mixAlpha, netCharge
    logical, intent(in) :: convergentOnly
    integer, intent(out) :: stat
    character(len=:), allocatable, intent(out) :: msg

    call dftbgpu_default_opts(this%opts)
    this%opts%kT = kT
    this%opts%sccTol = sccTol
    this%opts%maxIter = int(maxIter, c_int)
    this%opts%mixAlpha = mixAlpha
    this%opts%netCharge = netCharge
    this%opts%precision = int(precision, c_int)
    this%opts%convergentOnly = merge(1_c_int, 0_c_int, convergentOnly)
    stat = dftbgpu_create(this%ctx, int(device, c_int))
    if (stat /= DFTBGPU_OK) then
      msg = "dftbgpu: no usable CUDA device"
    else
      msg = ""
    end if
  end subroutine TGpuSccSolver_init

  !> Upload species data and SK tables once (packed as dftbgpu_set_model documents)
  subroutine setModel(this, nShell, angShell, onsite, hubbU, refOcc, skDist, skRows, skNInt, skHam,&
      & skOver, repNSpline, repData, stat, msg)
    class(TGpuSccSolver), intent(inout) :: this
    integer(c_int), intent(in) :: nShell(:), angShell(:), skRows(:), skNInt(:), repNSpline(:)
    real(c_double), intent(in) :: onsite(:), hubbU(:), refOcc(:), skDist(:), skHam(:), skOver(:)
    real(c_double), intent(in) :: repData(:)
    integer, intent(out) :: stat
    character(len=:), allocatable, intent(out) :: msg

    stat = dftbgpu_set_model(this%ctx, int(size(nShell), c_int), nShell, angShell, onsite, hubbU,&
        & refOcc, skDist, skRows, skNInt, skHam, skOver, repNSpline, repData)
    call fillMessage(this, stat, msg)
  end subroutine setModel

  !> New coordinates (Bohr): H0, S and the Cholesky factor of S are built on the GPU
  subroutine setGeometry(this, coord, species0, stat, msg)
    class(TGpuSccSolver), intent(inout) :: this
    real(c_double), intent(in) :: coord(:,:)
    integer, intent(in) :: species0(:)
    integer, intent(out) :: stat
    character(len=:), allocatable, intent(out) :: msg
    integer(c_int), allocatable :: sp(:)
    integer(c_int) :: nOrb

    this%nAtom = size(species0)
    sp = int(species0 - 1, c_int)
    stat = dftbgpu_set_geometry(this%ctx, int(this%nAtom, c_int), coord, sp)
    if (stat == DFTBGPU_OK) then
      stat = dftbgpu_n_orbitals(this%ctx, nOrb)
      this%nOrb = nOrb
    end if
    call fillMessage(this, stat, msg)
  end subroutine setGeometry

  !> The SCC cycle: results into the host fields processGeometry fills itself (dftbEnergy(1),
  !> Ef(1), eigen(:,1,1), filling(:,1,1), atomic populations of qOutput)
  subroutine runScc(this, qInit, energies, ef, eigen, filling, qOut, nIter, tConverged, stat, msg)
    class(TGpuSccSolver), intent(inout) :: this
    real(c_double), intent(in) :: qInit(:)
    type(TDftbGpuEnergies), intent(out) :: energies
    real(c_double), intent(out) :: ef, eigen(:), filling(:), qOut(:)
    integer, intent(out) :: nIter
    logical, intent(out) :: tConverged
    integer, intent(out) :: stat
    character(len=:), allocatable, intent(out) :: msg
    integer(c_int) :: it, conv

    stat = dftbgpu_scc(this%ctx, this%opts, qInit, energies, ef, eigen, filling, qOut, it, conv)
    nIter = it
    tConverged = (conv /= 0)
    call fillMessage(this, stat, msg)
  end subroutine runScc

  !> Energy gradient of the converged state into derivs(3, nAtom)
  subroutine getGradients(this, derivs, stat, msg)
    class(TGpuSccSolver), intent(inout) :: this
    real(c_double), intent(out) :: derivs(:,:)
    integer, intent(out) :: stat
    character(len=:), allocatable, intent(out) :: msg

    stat = dftbgpu_gradients(this%ctx, derivs)
    call fillMessage(this, stat, msg)
  end subroutine getGradients

  !> Per-iteration lines of the last SCC call for the SCC table the host prints
  subroutine sccTable(this, energy, error, precision, nIter)
    class(TGpuSccSolver), intent(in) :: this
    real(c_double), allocatable, intent(out) :: energy(:), error(:)
    integer(c_int), allocatable, intent(out) :: precision(:)
    integer, intent(out) :: nIter
    real(c_double), allocatable :: ms(:)

    ! first call with cap 0 only counts the iterations (nothing is written)
    allocate(energy(1), error(1), precision(1), ms(1))
    nIter = dftbgpu_scc_history(this%ctx, 0_c_int, energy, error, precision, ms)
    deallocate(energy, error, precision, ms)
    allocate(energy(max(nIter, 1)), error(max(nIter, 1)), precision(max(nIter, 1)), ms(max(nIter, 1)))
    nIter = dftbgpu_scc_history(this%ctx, int(nIter, c_int), energy, error, precision, ms)
  end subroutine sccTable

  subroutine fillMessage(this, stat, msg)
    class(TGpuSccSolver), intent(in) :: this
    integer, intent(in) :: stat
    character(len=:), allocatable, intent(out) :: msg

    if (stat == DFTBGPU_OK) then
      msg = ""
    else
      msg = dftbgpuErrorMessage(this%ctx)
    end if
  end subroutine fillMessage

  subroutine TGpuSccSolver_final(this)
    type(TGpuSccSolver), intent(inout) :: this
    integer(c_int) :: stat

    if (c_associated(this%ctx)) then
      stat = dftbgpu_destroy(this%ctx)
      this%ctx = c_null_ptr
    end if
  end subroutine TGpuSccSolver_final

end module dftbp_elecsolvers_gpuscc
