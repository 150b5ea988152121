!!
!! scone_gpu_mod -- ISO_C_BINDING view of libsconegpu's C ABI (include/scone_gpu.h) for SCONE.
!!
!! The derived types mirror the C structs field for field (bind(C): same order, kinds and
!! alignment; C pointers are type(c_ptr), filled with c_loc of TARGET arrays the caller owns), and
!! every entry point of the header has an interface block here, all returning the int32 status
!! (SG_OK = 0, negative SG_ERR_* codes; sg_last_error gives the message).  uint64_t RNG states are
!! integer(c_int64_t): SCONE's 63-bit LCG state (RNG_class.f90:20-35) is always non-negative.
!!
!! This module has no SCONE dependencies; transportOperatorGPU_class uses it.  It is not compiled
!! in this repository (no Fortran compiler is available to its builds); tests/test_fortran_binding.py
!! checks every type's field offsets and size against the C structs and every interface against the
!! header's prototypes.
!!
module scone_gpu_mod
  use iso_c_binding
  implicit none
  public

  ! status codes
  integer(c_int32_t), parameter :: SG_OK = 0, SG_ERR_BAD_ARG = -1, SG_ERR_OOM = -2, &
                                   SG_ERR_BANK_OVERFLOW = -3, SG_ERR_UNDEF_MAT = -4, SG_ERR_OVERLAP = -5, &
                                   SG_ERR_NAN = -6, SG_ERR_TIMEOUT = -7, SG_ERR_CUDA = -8, &
                                   SG_ERR_STATE = -9, SG_ERR_LOST = -10
  ! precision forms, execution forms, transport operators
  integer(c_int32_t), parameter :: SG_PREC_FP64 = 0, SG_PREC_MIXED = 1
  integer(c_int32_t), parameter :: SG_FORM_EVENT = 0, SG_FORM_HISTORY = 1
  integer(c_int32_t), parameter :: SG_TRANSPORT_ST = 1, SG_TRANSPORT_DT = 2, SG_TRANSPORT_ST_NOCACHE = 3, &
                                   SG_TRANSPORT_HT = 4, SG_TRANSPORT_HT_NOCACHE = 5
  ! clerks, map axes, grids, responses, boundary conditions
  integer(c_int32_t), parameter :: SG_CLERK_COLLISION = 1, SG_CLERK_TRACK = 2, SG_CLERK_KEFF_ANALOG = 3, &
                                   SG_CLERK_KEFF_IMPLICIT = 4, SG_CLERK_SURFACE_CURRENT = 5
  integer(c_int32_t), parameter :: SG_AXIS_X = 1, SG_AXIS_Y = 2, SG_AXIS_Z = 3, SG_AXIS_GROUP = 4, &
                                   SG_AXIS_MATERIAL = 5, SG_AXIS_ENERGY = 6, SG_AXIS_CELL = 7
  integer(c_int32_t), parameter :: SG_GRID_DEFAULT = 0, SG_GRID_LIN = 1, SG_GRID_LOG = 2, SG_GRID_UNSTRUCT = 3
  integer(c_int32_t), parameter :: SG_RESP_FLUX = 0
  integer(c_int32_t), parameter :: SG_BC_VACUUM = 0, SG_BC_REFLECTIVE = 1, SG_BC_PERIODIC = 2
  integer(c_int32_t), parameter :: SG_COLL_STD = 0, SG_COLL_IMP = 1
  integer(c_int32_t), parameter :: SG_SURF_NPAR = 6, SG_MAX_NEST = 12
  integer(c_int32_t), parameter :: SG_NOALLOC_MAX_HISTORIES = 16384, SG_NOALLOC_MAX_SITES = 32768

  type, bind(C) :: sg_geometry_desc
    integer(c_int32_t) :: n_surf
    type(c_ptr)        :: surf_type, surf_par
    integer(c_int32_t) :: border_surf
    integer(c_int32_t) :: bc(6)
    integer(c_int32_t) :: n_cell
    type(c_ptr)        :: cell_ptr, cell_surf
    integer(c_int32_t) :: n_uni
    type(c_ptr)        :: uni_type, uni_origin, uni_iptr, uni_ipar, uni_dptr, uni_dpar, uni_fptr, uni_fill
    integer(c_int32_t) :: root_uni
    type(c_ptr)        :: uni_rot
  end type sg_geometry_desc

  type, bind(C) :: sg_mg_desc
    integer(c_int32_t) :: n_mat, n_g
    type(c_ptr)        :: capture, fission, nu, chi, p0, prod, fissile
    real(c_double)     :: avg_dist
    type(c_ptr)        :: p1
  end type sg_mg_desc

  type, bind(C) :: sg_ce_desc
    integer(c_int32_t) :: n_nuc
    type(c_ptr)        :: nuc_ptr, e, xs, A, kT
    integer(c_int32_t) :: n_mat
    type(c_ptr)        :: mat_ptr, mat_nuc, mat_dens
    integer(c_int32_t) :: majorant
    real(c_double)     :: min_e, max_e, thresh_e, thresh_a, avg_dist
  end type sg_ce_desc

  type, bind(C) :: sg_axis_desc
    integer(c_int32_t) :: kind, n
    real(c_double)     :: min, max
    integer(c_int32_t) :: grid, cell_rest
    type(c_ptr)        :: bounds, cells
  end type sg_axis_desc

  type, bind(C) :: sg_clerk_desc
    integer(c_int32_t) :: type, handle_virtual, n_resp
    integer(c_int32_t) :: resp(4)
    integer(c_int32_t) :: n_axes
    type(sg_axis_desc) :: axes(3)
    integer(c_int32_t) :: filter_g_top, filter_g_low, current_axis, n_planes
    real(c_double)     :: planes(8)
  end type sg_clerk_desc

  type, bind(C) :: sg_tally_desc
    integer(c_int32_t) :: n_clerks
    type(c_ptr)        :: clerks
    integer(c_int32_t) :: batch_size, norm_clerk
    real(c_double)     :: norm_val
  end type sg_tally_desc

  type, bind(C) :: sg_point_source_desc
    real(c_double)     :: r(3), dir(3)
    integer(c_int32_t) :: isotropic, G, n_prob_g
    type(c_ptr)        :: prob_g
    real(c_double)     :: E
  end type sg_point_source_desc

  type, bind(C) :: sg_config
    integer(c_int32_t) :: precision, transport, device, max_bank, record_histories, form
    real(c_double)     :: ht_cutoff
  end type sg_config

  type, bind(C) :: sg_bank
    type(c_ptr) :: wgt, r, dir, G, time, brood_id, E
  end type sg_bank

  type, bind(C) :: sg_cycle_stats
    integer(c_int64_t) :: n_histories, n_events, n_collisions, n_next
    real(c_double)     :: start_weight, end_weight, k_eff, k_new, transport_ms, cycle_ms
    integer(c_int64_t) :: n_kernels
  end type sg_cycle_stats

  type, bind(C) :: sg_collision_desc
    integer(c_int32_t) :: kind, imp_abs, roulette, split, weight_windows, max_split
    real(c_double)     :: min_wgt, max_wgt, av_wgt
    integer(c_int32_t) :: ww_n_axes
    type(sg_axis_desc) :: ww_axes(3)
    type(c_ptr)        :: ww_lower, ww_upper
    real(c_double)     :: ww_const_survival
    integer(c_int32_t) :: buffer_depth
  end type sg_collision_desc

  type, bind(C) :: sg_event_tuning
    integer(c_int32_t) :: rounds_per_check, tail_min, tail_divisor
  end type sg_event_tuning

  type, bind(C) :: sg_batch_config
    integer(c_int32_t) :: precision, transport, device, max_problems
    integer(c_int64_t) :: arena_bytes
    integer(c_int32_t) :: max_work_items, reserved
    real(c_double)     :: ht_cutoff
  end type sg_batch_config

  type, bind(C) :: sg_problem_desc
    type(c_ptr)        :: geometry, mg, source, tally
    integer(c_int32_t) :: pop, cycles
    integer(c_int64_t) :: master_state
  end type sg_problem_desc

  type, bind(C) :: sg_batch_tuning
    integer(c_int32_t) :: item_histories, blocks_per_sm, block_threads, order
  end type sg_batch_tuning

  type, bind(C) :: sg_batch_stats
    integer(c_int64_t) :: n_histories, n_events, n_collisions
    integer(c_int32_t) :: n_problems, n_items
    real(c_double)     :: kernel_ms, run_ms
    integer(c_int64_t) :: n_kernels
  end type sg_batch_stats

  interface

    function sg_create(cfg, out) bind(C, name="sg_create")
      import
      type(sg_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: out
      integer(c_int32_t) :: sg_create
    end function sg_create

    function sg_destroy(h) bind(C, name="sg_destroy")
      import
      type(c_ptr), value :: h
      integer(c_int32_t) :: sg_destroy
    end function sg_destroy

    function sg_last_error(h, buf, len) bind(C, name="sg_last_error")
      import
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: buf
      integer(c_size_t), value :: len
      integer(c_int32_t) :: sg_last_error
    end function sg_last_error

    function sg_upload_geometry(h, g) bind(C, name="sg_upload_geometry")
      import
      type(c_ptr), value :: h
      type(sg_geometry_desc), intent(in) :: g
      integer(c_int32_t) :: sg_upload_geometry
    end function sg_upload_geometry

    function sg_upload_mg(h, mg) bind(C, name="sg_upload_mg")
      import
      type(c_ptr), value :: h
      type(sg_mg_desc), intent(in) :: mg
      integer(c_int32_t) :: sg_upload_mg
    end function sg_upload_mg

    function sg_upload_ce(h, ce) bind(C, name="sg_upload_ce")
      import
      type(c_ptr), value :: h
      type(sg_ce_desc), intent(in) :: ce
      integer(c_int32_t) :: sg_upload_ce
    end function sg_upload_ce

    function sg_upload_tally(h, t, admin_out) bind(C, name="sg_upload_tally")
      import
      type(c_ptr), value :: h
      type(sg_tally_desc), intent(in) :: t
      integer(c_int32_t), intent(inout) :: admin_out
      integer(c_int32_t) :: sg_upload_tally
    end function sg_upload_tally

    function sg_attach_tally(h, admin, attachment) bind(C, name="sg_attach_tally")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      integer(c_int32_t), value :: attachment
      integer(c_int32_t) :: sg_attach_tally
    end function sg_attach_tally

    function sg_set_point_source(h, src) bind(C, name="sg_set_point_source")
      import
      type(c_ptr), value :: h
      type(sg_point_source_desc), intent(in) :: src
      integer(c_int32_t) :: sg_set_point_source
    end function sg_set_point_source

    function sg_generate_source(h, master_state, n, out) bind(C, name="sg_generate_source")
      import
      type(c_ptr), value :: h
      integer(c_int64_t), value :: master_state
      integer(c_int32_t), value :: n
      type(sg_bank), intent(inout) :: out
      integer(c_int32_t) :: sg_generate_source
    end function sg_generate_source

    function sg_transport_bank(h, admin, in, n, master_state, k_eff, next, next_cap, stats) bind(C, name="sg_transport_bank")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      type(sg_bank), intent(in) :: in
      integer(c_int32_t), value :: n
      integer(c_int64_t), value :: master_state
      real(c_double), value :: k_eff
      type(sg_bank), intent(inout) :: next
      integer(c_int32_t), value :: next_cap
      type(sg_cycle_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_transport_bank
    end function sg_transport_bank

    function sg_tally_cycle_start(h, admin, start_pop_weight) bind(C, name="sg_tally_cycle_start")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      real(c_double), value :: start_pop_weight
      integer(c_int32_t) :: sg_tally_cycle_start
    end function sg_tally_cycle_start

    function sg_tally_cycle_end(h, admin, end_pop_weight, k_end) bind(C, name="sg_tally_cycle_end")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      real(c_double), value :: end_pop_weight
      real(c_double), value :: k_end
      integer(c_int32_t) :: sg_tally_cycle_end
    end function sg_tally_cycle_end

    function sg_tally_size(h, admin, n_bins) bind(C, name="sg_tally_size")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      integer(c_int64_t), intent(inout) :: n_bins
      integer(c_int32_t) :: sg_tally_size
    end function sg_tally_size

    function sg_get_bins(h, admin, bins, n_bins) bind(C, name="sg_get_bins")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      real(c_double), dimension(*), intent(inout) :: bins
      integer(c_int64_t), value :: n_bins
      integer(c_int32_t) :: sg_get_bins
    end function sg_get_bins

    function sg_get_keff(h, admin, k, std) bind(C, name="sg_get_keff")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      real(c_double), intent(inout) :: k
      real(c_double), intent(inout) :: std
      integer(c_int32_t) :: sg_get_keff
    end function sg_get_keff

    function sg_bank_write_file(path, bank, n, binary) bind(C, name="sg_bank_write_file")
      import
      character(kind=c_char), dimension(*) :: path
      type(sg_bank), intent(in) :: bank
      integer(c_int32_t), value :: n
      integer(c_int32_t), value :: binary
      integer(c_int32_t) :: sg_bank_write_file
    end function sg_bank_write_file

    function sg_bank_count_file(path, binary, n) bind(C, name="sg_bank_count_file")
      import
      character(kind=c_char), dimension(*) :: path
      integer(c_int32_t), value :: binary
      integer(c_int64_t), intent(inout) :: n
      integer(c_int32_t) :: sg_bank_count_file
    end function sg_bank_count_file

    function sg_bank_read_file(path, binary, bank, cap, n) bind(C, name="sg_bank_read_file")
      import
      character(kind=c_char), dimension(*) :: path
      integer(c_int32_t), value :: binary
      type(sg_bank), intent(inout) :: bank
      integer(c_int32_t), value :: cap
      integer(c_int32_t), intent(inout) :: n
      integer(c_int32_t) :: sg_bank_read_file
    end function sg_bank_read_file

    function sg_set_file_source(h, particles, n) bind(C, name="sg_set_file_source")
      import
      type(c_ptr), value :: h
      type(sg_bank), intent(in) :: particles
      integer(c_int32_t), value :: n
      integer(c_int32_t) :: sg_set_file_source
    end function sg_set_file_source

    function sg_eigen_init(h, pop, master_state, k0) bind(C, name="sg_eigen_init")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: pop
      integer(c_int64_t), value :: master_state
      real(c_double), value :: k0
      integer(c_int32_t) :: sg_eigen_init
    end function sg_eigen_init

    function sg_eigen_cycle(h, admin, atch, stats) bind(C, name="sg_eigen_cycle")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      integer(c_int32_t), value :: atch
      type(sg_cycle_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_eigen_cycle
    end function sg_eigen_cycle

    function sg_eigen_cycle_bank(h, admin, atch, in, pop, master_state, k_eff, k_end, out, stats) &
        bind(C, name="sg_eigen_cycle_bank")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      integer(c_int32_t), value :: atch
      type(sg_bank), intent(in) :: in
      integer(c_int32_t), value :: pop
      integer(c_int64_t), intent(inout) :: master_state
      real(c_double), intent(inout) :: k_eff
      real(c_double), value :: k_end
      type(sg_bank), intent(inout) :: out
      type(sg_cycle_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_eigen_cycle_bank
    end function sg_eigen_cycle_bank

    function sg_eigen_state(h, master_state, k) bind(C, name="sg_eigen_state")
      import
      type(c_ptr), value :: h
      integer(c_int64_t), intent(inout) :: master_state
      real(c_double), intent(inout) :: k
      integer(c_int32_t) :: sg_eigen_state
    end function sg_eigen_state

    function sg_eigen_get_bank(h, out, cap, pop) bind(C, name="sg_eigen_get_bank")
      import
      type(c_ptr), value :: h
      type(sg_bank), intent(inout) :: out
      integer(c_int32_t), value :: cap
      integer(c_int32_t), intent(inout) :: pop
      integer(c_int32_t) :: sg_eigen_get_bank
    end function sg_eigen_get_bank

    function sg_fixed_source_cycle(h, admin, n, master_state, stats) bind(C, name="sg_fixed_source_cycle")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      integer(c_int32_t), value :: n
      integer(c_int64_t), intent(inout) :: master_state
      type(sg_cycle_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_fixed_source_cycle
    end function sg_fixed_source_cycle

    function sg_fixed_source_cycle_shard(h, admin, share, total, master_state, stats) bind(C, name="sg_fixed_source_cycle_shard")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      integer(c_int32_t), value :: share
      integer(c_int32_t), value :: total
      integer(c_int64_t), intent(inout) :: master_state
      type(sg_cycle_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_fixed_source_cycle_shard
    end function sg_fixed_source_cycle_shard

    function sg_normalise_shard(h, sites, n, sites_before, tot_sites, tot_pop, master_state, out, out_cap, n_out) &
        bind(C, name="sg_normalise_shard")
      import
      type(c_ptr), value :: h
      type(sg_bank), intent(in) :: sites
      integer(c_int32_t), value :: n
      integer(c_int64_t), value :: sites_before
      integer(c_int64_t), value :: tot_sites
      integer(c_int32_t), value :: tot_pop
      integer(c_int64_t), value :: master_state
      type(sg_bank), intent(inout) :: out
      integer(c_int32_t), value :: out_cap
      integer(c_int32_t), intent(inout) :: n_out
      integer(c_int32_t) :: sg_normalise_shard
    end function sg_normalise_shard

    function sg_tally_get_scores(h, admin, scores, n_bins) bind(C, name="sg_tally_get_scores")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      real(c_double), dimension(*), intent(inout) :: scores
      integer(c_int64_t), value :: n_bins
      integer(c_int32_t) :: sg_tally_get_scores
    end function sg_tally_get_scores

    function sg_tally_set_scores(h, admin, scores, n_bins) bind(C, name="sg_tally_set_scores")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      real(c_double), dimension(*), intent(in) :: scores
      integer(c_int64_t), value :: n_bins
      integer(c_int32_t) :: sg_tally_set_scores
    end function sg_tally_set_scores

    function sg_transport_bank_noalloc(h, admin, dev_in, n, master_state, k_eff, dev_next, next_cap, n_next) &
        bind(C, name="sg_transport_bank_noalloc")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), value :: admin
      type(sg_bank), intent(in) :: dev_in
      integer(c_int32_t), value :: n
      integer(c_int64_t), value :: master_state
      real(c_double), value :: k_eff
      type(sg_bank), intent(inout) :: dev_next
      integer(c_int32_t), value :: next_cap
      integer(c_int32_t), intent(inout) :: n_next
      integer(c_int32_t) :: sg_transport_bank_noalloc
    end function sg_transport_bank_noalloc

    function sg_set_collision(h, d) bind(C, name="sg_set_collision")
      import
      type(c_ptr), value :: h
      type(sg_collision_desc), intent(in) :: d
      integer(c_int32_t) :: sg_set_collision
    end function sg_set_collision

    function sg_set_event_tuning(h, t) bind(C, name="sg_set_event_tuning")
      import
      type(c_ptr), value :: h
      type(sg_event_tuning), intent(in) :: t
      integer(c_int32_t) :: sg_set_event_tuning
    end function sg_set_event_tuning

    function sg_get_event_tuning(h, t) bind(C, name="sg_get_event_tuning")
      import
      type(c_ptr), value :: h
      type(sg_event_tuning), intent(inout) :: t
      integer(c_int32_t) :: sg_get_event_tuning
    end function sg_get_event_tuning

    function sg_batch_create(cfg, out) bind(C, name="sg_batch_create")
      import
      type(sg_batch_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: out
      integer(c_int32_t) :: sg_batch_create
    end function sg_batch_create

    function sg_batch_destroy(b) bind(C, name="sg_batch_destroy")
      import
      type(c_ptr), value :: b
      integer(c_int32_t) :: sg_batch_destroy
    end function sg_batch_destroy

    function sg_batch_last_error(b, buf, len) bind(C, name="sg_batch_last_error")
      import
      type(c_ptr), value :: b
      character(kind=c_char), dimension(*) :: buf
      integer(c_size_t), value :: len
      integer(c_int32_t) :: sg_batch_last_error
    end function sg_batch_last_error

    function sg_batch_add(b, p, slot) bind(C, name="sg_batch_add")
      import
      type(c_ptr), value :: b
      type(sg_problem_desc), intent(in) :: p
      integer(c_int32_t), intent(inout) :: slot
      integer(c_int32_t) :: sg_batch_add
    end function sg_batch_add

    function sg_batch_instance(b, parent, pop, cycles, master_state, slot) bind(C, name="sg_batch_instance")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: parent
      integer(c_int32_t), value :: pop
      integer(c_int32_t), value :: cycles
      integer(c_int64_t), value :: master_state
      integer(c_int32_t), intent(inout) :: slot
      integer(c_int32_t) :: sg_batch_instance
    end function sg_batch_instance

    function sg_batch_remove(b, slot) bind(C, name="sg_batch_remove")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: slot
      integer(c_int32_t) :: sg_batch_remove
    end function sg_batch_remove

    function sg_batch_memory(b, used, capacity) bind(C, name="sg_batch_memory")
      import
      type(c_ptr), value :: b
      integer(c_int64_t), intent(inout) :: used
      integer(c_int64_t), intent(inout) :: capacity
      integer(c_int32_t) :: sg_batch_memory
    end function sg_batch_memory

    function sg_batch_set_tuning(b, t) bind(C, name="sg_batch_set_tuning")
      import
      type(c_ptr), value :: b
      type(sg_batch_tuning), intent(in) :: t
      integer(c_int32_t) :: sg_batch_set_tuning
    end function sg_batch_set_tuning

    function sg_batch_get_tuning(b, t) bind(C, name="sg_batch_get_tuning")
      import
      type(c_ptr), value :: b
      type(sg_batch_tuning), intent(inout) :: t
      integer(c_int32_t) :: sg_batch_get_tuning
    end function sg_batch_get_tuning

    function sg_batch_run(b, slots, n, stats) bind(C, name="sg_batch_run")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), dimension(*), intent(in) :: slots
      integer(c_int32_t), value :: n
      type(sg_batch_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_batch_run
    end function sg_batch_run

    function sg_batch_run_plain(b, slots, n, form, stats) bind(C, name="sg_batch_run_plain")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), dimension(*), intent(in) :: slots
      integer(c_int32_t), value :: n
      integer(c_int32_t), value :: form
      type(sg_batch_stats), intent(inout) :: stats
      integer(c_int32_t) :: sg_batch_run_plain
    end function sg_batch_run_plain

    function sg_batch_autotune(b, slots, n, best) bind(C, name="sg_batch_autotune")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), dimension(*), intent(in) :: slots
      integer(c_int32_t), value :: n
      type(sg_batch_tuning), intent(inout) :: best
      integer(c_int32_t) :: sg_batch_autotune
    end function sg_batch_autotune

    function sg_batch_autotune_plain(b, slots, n, best) bind(C, name="sg_batch_autotune_plain")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), dimension(*), intent(in) :: slots
      integer(c_int32_t), value :: n
      type(sg_event_tuning), intent(inout) :: best
      integer(c_int32_t) :: sg_batch_autotune_plain
    end function sg_batch_autotune_plain

    function sg_batch_tally_size(b, slot, n_bins) bind(C, name="sg_batch_tally_size")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: slot
      integer(c_int64_t), intent(inout) :: n_bins
      integer(c_int32_t) :: sg_batch_tally_size
    end function sg_batch_tally_size

    function sg_batch_get_bins(b, slot, bins, n_bins) bind(C, name="sg_batch_get_bins")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: slot
      real(c_double), dimension(*), intent(inout) :: bins
      integer(c_int64_t), value :: n_bins
      integer(c_int32_t) :: sg_batch_get_bins
    end function sg_batch_get_bins

    function sg_batch_clear_tally(b, slot) bind(C, name="sg_batch_clear_tally")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: slot
      integer(c_int32_t) :: sg_batch_clear_tally
    end function sg_batch_clear_tally

    function sg_serve_start(b, wave_histories, item_histories) bind(C, name="sg_serve_start")
      import
      type(c_ptr), value :: b
      integer(c_int64_t), value :: wave_histories
      integer(c_int32_t), value :: item_histories
      integer(c_int32_t) :: sg_serve_start
    end function sg_serve_start

    function sg_serve_submit(b, slot) bind(C, name="sg_serve_submit")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: slot
      integer(c_int32_t) :: sg_serve_submit
    end function sg_serve_submit

    function sg_serve_pump(b, wait, done_slots, latency_s, cap, n_done) bind(C, name="sg_serve_pump")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: wait
      integer(c_int32_t), dimension(*), intent(inout) :: done_slots
      real(c_double), dimension(*), intent(inout) :: latency_s
      integer(c_int32_t), value :: cap
      integer(c_int32_t), intent(inout) :: n_done
      integer(c_int32_t) :: sg_serve_pump
    end function sg_serve_pump

    function sg_serve_stop(b) bind(C, name="sg_serve_stop")
      import
      type(c_ptr), value :: b
      integer(c_int32_t) :: sg_serve_stop
    end function sg_serve_stop

    function sg_serve_status(b, queued, active, waves) bind(C, name="sg_serve_status")
      import
      type(c_ptr), value :: b
      integer(c_int64_t), intent(inout) :: queued
      integer(c_int32_t), intent(inout) :: active
      integer(c_int64_t), intent(inout) :: waves
      integer(c_int32_t) :: sg_serve_status
    end function sg_serve_status

    function sg_serve_share(b, blocks_per_sm, on) bind(C, name="sg_serve_share")
      import
      type(c_ptr), value :: b
      integer(c_int32_t), value :: blocks_per_sm
      integer(c_int32_t), value :: on
      integer(c_int32_t) :: sg_serve_share
    end function sg_serve_share

    function sg_serve_counts(b, histories, events) bind(C, name="sg_serve_counts")
      import
      type(c_ptr), value :: b
      integer(c_int64_t), intent(inout) :: histories
      integer(c_int64_t), intent(inout) :: events
      integer(c_int32_t) :: sg_serve_counts
    end function sg_serve_counts

    function sg_serve_clock() bind(C, name="sg_serve_clock")
      import
      real(c_double) :: sg_serve_clock
    end function sg_serve_clock

    function sg_get_history_records(h, collisions, rng_end, n) bind(C, name="sg_get_history_records")
      import
      type(c_ptr), value :: h
      integer(c_int32_t), dimension(*), intent(inout) :: collisions
      integer(c_int64_t), dimension(*), intent(inout) :: rng_end
      integer(c_int32_t), value :: n
      integer(c_int32_t) :: sg_get_history_records
    end function sg_get_history_records

    function sg_rng_draws(state, out, n) bind(C, name="sg_rng_draws")
      import
      integer(c_int64_t), intent(inout) :: state
      real(c_double), dimension(*), intent(inout) :: out
      integer(c_int32_t), value :: n
      integer(c_int32_t) :: sg_rng_draws
    end function sg_rng_draws

    function sg_rng_skip(state, k) bind(C, name="sg_rng_skip")
      import
      integer(c_int64_t), value :: state
      integer(c_int64_t), value :: k
      integer(c_int64_t) :: sg_rng_skip
    end function sg_rng_skip

  end interface

end module scone_gpu_mod
