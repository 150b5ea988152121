!!
!! transportOperatorGPU -- a SCONE transportOperator whose transport (and collision processing) runs
!! on one GB300 through libsconegpu's C ABI (scone_gpu_mod).
!!
!! Registered in new_transportOperator (TransportOperator/transportOperatorFactory_func.f90:36-60) as
!! 'transportOperatorGPU' (transportOperatorFactory.patch).  Unlike the scalar operators it is never
!! called per particle: a GPU needs whole banks, so the physics packages' `gen:` loops
!! (fixedSourcePhysicsPackage_class.f90:198-261, eigenPhysicsPackage_class.f90:211-275) call it once
!! per cycle (physicsPackages.patch):
!!   transportBank   -> the gen loop over thisCycle: fission sites into nextCycle in brood order,
!!                      scores into the operator's device tally admin (sg_transport_bank);
!!   eigenCycle      -> the whole eigenvalue cycle body, normSize_Repr included, on the device, with
!!                      the dungeons staying in host memory (sg_eigen_cycle_bank).
!! The collision operator of the deck is then not used for these particles: neutronMGstd /
!! neutronCEstd (or the *imp processors set with sg_set_collision) run in the same kernel.
!!
!! Sample input dictionary:
!!   transportOperator { type transportOperatorGPU; tracking DT; cache 1; cutoff 0.9;
!!                       precision mixed; form history; maxBank 2500000; device 0; }
!!   tracking  ST | DT | HT (transportOperatorST/DT/HT), cache and cutoff as those operators read them
!!   precision fp64 (all-FP64 verification form) | mixed (FP32 XS and distances, FP64 positions/tallies)
!!
!! Problem data reach the device as the C ABI's descriptors (upload): the geometry tables that
!! geometryStd%init builds, the MG or CE data and the tally clerks.  Building those descriptors from a
!! SCONE input deck is the deck converter's job and is not part of this file.
!!
!! Not compiled in this repository (no Fortran compiler is available to its builds).
!!
module transportOperatorGPU_class

  use iso_c_binding
  use numPrecision
  use universalVariables
  use errors_mod,              only : fatalError
  use particle_class,          only : particle, particleState
  use particleDungeon_class,   only : particleDungeon
  use dictionary_class,        only : dictionary
  use RNG_class,               only : RNG
  use tallyAdmin_class,        only : tallyAdmin
  use transportOperator_inter, only : transportOperator, init_super => init
  use scone_gpu_mod

  implicit none
  private

  !!
  !! Host staging of one dungeon as the SoA arrays of particleStateData (particle_class.f90:50-65)
  !!
  type :: soaBank
    real(c_double), dimension(:), pointer, contiguous     :: wgt => null(), time => null(), E => null()
    real(c_double), dimension(:,:), pointer, contiguous   :: r => null(), dir => null()
    integer(c_int32_t), dimension(:), pointer, contiguous :: G => null(), brood => null()
  contains
    procedure :: reserve
    procedure :: view
    procedure :: free
  end type soaBank

  type, public, extends(transportOperator) :: transportOperatorGPU
    type(c_ptr)        :: h = c_null_ptr
    type(sg_config)    :: cfg
    integer(c_int32_t) :: admin = -1       ! device tally admin of the active cycles
    integer(c_int32_t) :: atch = -1        ! its attachment holding the k clerk (eigenvalue runs)
    logical(defBool)   :: isCE = .false.
    type(soaBank)      :: inBank, outBank
  contains
    procedure :: init
    procedure :: kill
    procedure :: transit => gpuTransit
    procedure :: upload
    procedure :: transportBank
    procedure :: eigenCycle
    procedure :: closeCycle
    procedure :: getBins
    procedure :: check
  end type transportOperatorGPU

contains

  !!
  !! Reads the operator options and creates the device handle
  !!
  subroutine init(self, dict)
    class(transportOperatorGPU), intent(inout) :: self
    class(dictionary), intent(in)              :: dict
    character(nameLen)                         :: tracking, precision, form
    integer(shortInt)                          :: cache, device, maxBank
    real(defReal)                              :: cutoff
    character(100), parameter :: Here = 'init (transportOperatorGPU_class.f90)'

    call init_super(self, dict)
    call dict % getOrDefault(tracking, 'tracking', 'DT')
    call dict % getOrDefault(precision, 'precision', 'mixed')
    call dict % getOrDefault(form, 'form', 'history')
    call dict % getOrDefault(cache, 'cache', 1)
    call dict % getOrDefault(cutoff, 'cutoff', 0.9_defReal)
    call dict % getOrDefault(device, 'device', 0)
    call dict % getOrDefault(maxBank, 'maxBank', 2500000)

    select case (trim(tracking))
      case ('ST')
        self % cfg % transport = merge(SG_TRANSPORT_ST, SG_TRANSPORT_ST_NOCACHE, cache /= 0)
      case ('DT')
        self % cfg % transport = SG_TRANSPORT_DT
      case ('HT')
        self % cfg % transport = merge(SG_TRANSPORT_HT, SG_TRANSPORT_HT_NOCACHE, cache /= 0)
      case default
        call fatalError(Here, 'Unknown tracking: ' // trim(tracking) // ' (ST, DT or HT)')
    end select
    select case (trim(precision))
      case ('fp64')
        self % cfg % precision = SG_PREC_FP64
      case ('mixed')
        self % cfg % precision = SG_PREC_MIXED
      case default
        call fatalError(Here, 'Unknown precision: ' // trim(precision) // ' (fp64 or mixed)')
    end select
    self % cfg % form = merge(SG_FORM_EVENT, SG_FORM_HISTORY, trim(form) == 'event')
    self % cfg % device = int(device, c_int32_t)
    self % cfg % max_bank = int(maxBank, c_int32_t)
    self % cfg % record_histories = 0
    self % cfg % ht_cutoff = real(cutoff, c_double)

    call self % check(sg_create(self % cfg, self % h), Here)

  end subroutine init

  !!
  !! Uploads the problem: geometry, MG or CE data, the active-cycle tally admin and (eigenvalue runs)
  !! its k attachment.  The descriptors' arrays are copied to the device during the calls.
  !!
  subroutine upload(self, geom, tallies, mg, ce, kTally)
    class(transportOperatorGPU), intent(inout)   :: self
    type(sg_geometry_desc), intent(in)           :: geom
    type(sg_tally_desc), intent(in)              :: tallies
    type(sg_mg_desc), intent(in), optional       :: mg
    type(sg_ce_desc), intent(in), optional       :: ce
    type(sg_tally_desc), intent(in), optional    :: kTally
    character(100), parameter :: Here = 'upload (transportOperatorGPU_class.f90)'

    call self % check(sg_upload_geometry(self % h, geom), Here)
    if (present(mg)) then
      call self % check(sg_upload_mg(self % h, mg), Here)
    else if (present(ce)) then
      call self % check(sg_upload_ce(self % h, ce), Here)
      self % isCE = .true.
    else
      call fatalError(Here, 'MG or CE data are required')
    end if
    call self % check(sg_upload_tally(self % h, tallies, self % admin), Here)
    if (present(kTally)) then
      call self % check(sg_upload_tally(self % h, kTally, self % atch), Here)
      call self % check(sg_attach_tally(self % h, self % admin, self % atch), Here)
    end if

  end subroutine upload

  !!
  !! The transportOperator interface moves one particle; this operator moves whole banks
  !!
  subroutine gpuTransit(self, p, tally, thisCycle, nextCycle)
    class(transportOperatorGPU), intent(inout) :: self
    class(particle), intent(inout)             :: p
    type(tallyAdmin), intent(inout)            :: tally
    class(particleDungeon), intent(inout)      :: thisCycle
    class(particleDungeon), intent(inout)      :: nextCycle
    character(100), parameter :: Here = 'gpuTransit (transportOperatorGPU_class.f90)'

    call fatalError(Here, 'transportOperatorGPU transports whole dungeons: call transportBank or eigenCycle')

  end subroutine gpuTransit

  !!
  !! The gen loop over thisCycle (its particle n uses pRNG strided by n, as the physics packages do):
  !! transport and collisions of every history on the device, scores into the device admin, fission
  !! sites detained into nextCycle in brood order.  pRNG is not advanced (the caller strides it as
  !! after its own gen loop).
  !!
  subroutine transportBank(self, thisCycle, nextCycle, pRNG, k_eff, stats)
    class(transportOperatorGPU), intent(inout) :: self
    class(particleDungeon), intent(inout)      :: thisCycle
    class(particleDungeon), intent(inout)      :: nextCycle
    class(RNG), intent(in)                     :: pRNG
    real(defReal), intent(in)                  :: k_eff
    type(sg_cycle_stats), intent(out)          :: stats
    integer(shortInt)                          :: n, cap
    type(sg_bank)                              :: bIn, bOut
    character(100), parameter :: Here = 'transportBank (transportOperatorGPU_class.f90)'

    n = thisCycle % popSize()
    cap = int(self % cfg % max_bank, shortInt)
    call packDungeon(thisCycle, self % inBank, n)
    call self % outBank % reserve(cap)
    bIn = self % inBank % view(self % isCE)
    bOut = self % outBank % view(self % isCE)
    call self % check(sg_transport_bank(self % h, self % admin, bIn, int(n, c_int32_t), &
                                        int(pRNG % currentState(), c_int64_t), real(k_eff, c_double), &
                                        bOut, int(cap, c_int32_t), stats), Here)
    call unpackDungeon(self % outBank, int(stats % n_next, shortInt), nextCycle)

  end subroutine transportBank

  !!
  !! The whole eigenvalue cycle (eigenPhysicsPackage_class.f90:203-338) on the device: gen loop,
  !! cleanPop, stride(totalPop + 1), reportCycleEnd, normSize_Repr(totalPop), stride(1) and the k
  !! estimate.  thisCycle is consumed (cleanPop); nextCycle receives the normalised bank; pRNG and
  !! k_eff advance as the cycle body advances them (k_eff in: the k of this cycle's fission weights;
  !! out: the new estimate).  nextCycle%k_eff is read as end%k_eff of reportCycleEnd.  The caller
  !! flips the dungeons and loads the new k into the next dungeon, as the physics package does.
  !!
  subroutine eigenCycle(self, thisCycle, nextCycle, pRNG, k_eff, stats)
    class(transportOperatorGPU), intent(inout) :: self
    class(particleDungeon), intent(inout)      :: thisCycle
    class(particleDungeon), intent(inout)      :: nextCycle
    class(RNG), intent(inout)                  :: pRNG
    real(defReal), intent(inout)               :: k_eff
    type(sg_cycle_stats), intent(out)          :: stats
    integer(shortInt)                          :: n
    integer(c_int64_t)                         :: master
    real(c_double)                             :: k
    type(sg_bank)                              :: bIn, bOut
    character(100), parameter :: Here = 'eigenCycle (transportOperatorGPU_class.f90)'

    if (self % atch < 0) call fatalError(Here, 'eigenvalue cycles need a k tally (upload kTally)')
    n = thisCycle % popSize()
    call packDungeon(thisCycle, self % inBank, n)
    call self % outBank % reserve(n)
    bIn = self % inBank % view(self % isCE)
    bOut = self % outBank % view(self % isCE)
    master = int(pRNG % currentState(), c_int64_t)
    k = real(k_eff, c_double)
    call self % check(sg_eigen_cycle_bank(self % h, self % admin, self % atch, bIn, int(n, c_int32_t), master, &
                                          k, real(nextCycle % k_eff, c_double), bOut, stats), Here)
    call thisCycle % cleanPop()
    call unpackDungeon(self % outBank, n, nextCycle)
    call pRNG % setSeed(int(master, longInt))
    k_eff = real(k, defReal)

  end subroutine eigenCycle

  !!
  !! tallyAdmin%reportCycleEnd for the device admin (transportBank cycles)
  !!
  subroutine closeCycle(self, endPopWeight, k_end)
    class(transportOperatorGPU), intent(inout) :: self
    real(defReal), intent(in)                  :: endPopWeight, k_end
    character(100), parameter :: Here = 'closeCycle (transportOperatorGPU_class.f90)'

    call self % check(sg_tally_cycle_end(self % h, self % admin, real(endPopWeight, c_double), &
                                         real(k_end, c_double)), Here)

  end subroutine closeCycle

  !!
  !! scoreMemory bins(N, {BIN, CSUM, CSUM2}) of the device admin (scoreMemory_class.f90:16-18)
  !!
  subroutine getBins(self, bins)
    class(transportOperatorGPU), intent(inout)             :: self
    real(defReal), dimension(:,:), allocatable, intent(out) :: bins
    integer(c_int64_t)                                     :: N
    real(c_double), dimension(:,:), allocatable, target    :: b
    character(100), parameter :: Here = 'getBins (transportOperatorGPU_class.f90)'

    call self % check(sg_tally_size(self % h, self % admin, N), Here)
    allocate(b(N, 3))
    call self % check(sg_get_bins(self % h, self % admin, b, N), Here)
    bins = real(b, defReal)

  end subroutine getBins

  !!
  !! Maps a nonzero status to fatalError with the library's message (errors_mod.f90:32-69)
  !!
  subroutine check(self, rc, where)
    class(transportOperatorGPU), intent(inout) :: self
    integer(c_int32_t), intent(in)             :: rc
    character(*), intent(in)                   :: where
    character(kind=c_char), dimension(512)     :: buf
    character(512)                             :: msg
    integer                                    :: i, ierr

    if (rc == SG_OK) return
    buf = c_null_char
    ierr = sg_last_error(self % h, buf, int(size(buf), c_size_t))
    msg = ''
    do i = 1, size(buf)
      if (buf(i) == c_null_char) exit
      msg(i:i) = buf(i)
    end do
    call fatalError(where, 'libsconegpu status ' // trim(adjustl(itoa(int(rc)))) // ': ' // trim(msg))

  end subroutine check

  !!
  !! Frees the device handle and the staging banks
  !!
  subroutine kill(self)
    class(transportOperatorGPU), intent(inout) :: self
    integer(c_int32_t)                         :: ierr

    if (c_associated(self % h)) ierr = sg_destroy(self % h)
    self % h = c_null_ptr
    call self % inBank % free()
    call self % outBank % free()

  end subroutine kill

  ! ---------------------------------------------------------------- staging of the dungeons

  subroutine packDungeon(d, b, n)
    class(particleDungeon), intent(in) :: d
    type(soaBank), intent(inout)       :: b
    integer(shortInt), intent(in)      :: n
    integer(shortInt)                  :: i

    call b % reserve(max(n, 1))
    do i = 1, n
      associate (s => d % prisoners(i))
        b % wgt(i) = s % wgt
        b % r(:, i) = s % r
        b % dir(:, i) = s % dir
        b % E(i) = s % E
        b % G(i) = s % G
        b % time(i) = s % time
        b % brood(i) = s % broodID
      end associate
    end do

  end subroutine packDungeon

  subroutine unpackDungeon(b, n, d)
    type(soaBank), intent(in)             :: b
    integer(shortInt), intent(in)         :: n
    class(particleDungeon), intent(inout) :: d
    type(particleState)                   :: s
    integer(shortInt)                     :: i

    do i = 1, n
      s % wgt = b % wgt(i)
      s % r = b % r(:, i)
      s % dir = b % dir(:, i)
      s % E = b % E(i)
      s % G = b % G(i)
      s % isMG = (b % G(i) > 0)
      s % type = P_NEUTRON
      s % time = b % time(i)
      s % broodID = b % brood(i)
      call d % detain(s)
    end do

  end subroutine unpackDungeon

  subroutine reserve(self, n)
    class(soaBank), intent(inout) :: self
    integer(shortInt), intent(in) :: n

    if (associated(self % wgt)) then
      if (size(self % wgt) >= n) return
      call self % free()
    end if
    allocate(self % wgt(n), self % time(n), self % E(n), self % r(3, n), self % dir(3, n), &
             self % G(n), self % brood(n))
    self % E = 0.0_c_double
    self % G = 0

  end subroutine reserve

  function view(self, isCE) result(b)
    class(soaBank), intent(in) :: self
    logical(defBool), intent(in) :: isCE
    type(sg_bank)              :: b

    b % wgt = c_loc(self % wgt)
    b % r = c_loc(self % r)
    b % dir = c_loc(self % dir)
    b % G = c_loc(self % G)
    b % time = c_loc(self % time)
    b % brood_id = c_loc(self % brood)
    b % E = merge(c_loc(self % E), c_null_ptr, isCE)

  end function view

  subroutine free(self)
    class(soaBank), intent(inout) :: self

    if (associated(self % wgt)) deallocate(self % wgt, self % time, self % E, self % r, self % dir, &
                                           self % G, self % brood)

  end subroutine free

  function itoa(i) result(s)
    integer, intent(in) :: i
    character(16)       :: s

    write(s, '(I0)') i

  end function itoa

end module transportOperatorGPU_class
