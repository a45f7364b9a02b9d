!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!
!!!!!   examd_gpu_mod.f90
!!!!!
!!!!!   ISO_C_BINDING interface of the GB300 midpoint Lennard-Jones library
!!!!!   (include/examd_gb300.h, libexamd_gb300.so) for the exaMD Fortran
!!!!!   driver.  Interfaces only, in the style of the driver's existing C
!!!!!   bindings (SRC/exaMD_metis_interface.f90:31-41): every entry point of the
!!!!!   header, with bind(C, name=...) and the header's argument order and
!!!!!   types.  Scalars passed by value in C carry the Value attribute; C
!!!!!   pointers to arrays are assumed-size dummies; nullable pointers are
!!!!!   Type(c_ptr), Value (pass c_null_ptr or c_loc(x)).
!!!!!
!!!!!   Every function returns Integer(c_int) status 0 (EXAMD_OK) on success.
!!!!!   109 keeps the reference's MPI_Abort code for a position outside the
!!!!!   block grid (SRC/exaMD_module.f90:118-123).
!!!!!
!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!

Module examd_gpu_mod

  Use, Intrinsic :: iso_c_binding

  Implicit None

  ! Status codes (include/examd_gb300.h)
  Integer(c_int), Parameter :: EXAMD_OK = 0
  Integer(c_int), Parameter :: EXAMD_ERR_OUTSIDE = 109
  Integer(c_int), Parameter :: EXAMD_ERR_ARG = 201
  Integer(c_int), Parameter :: EXAMD_ERR_NB_TOO_SMALL = 202
  Integer(c_int), Parameter :: EXAMD_ERR_CELL_OVERFLOW = 203
  Integer(c_int), Parameter :: EXAMD_ERR_NONFINITE = 204
  Integer(c_int), Parameter :: EXAMD_ERR_TIMEOUT = 205
  Integer(c_int), Parameter :: EXAMD_ERR_CUDA = 206
  Integer(c_int), Parameter :: EXAMD_ERR_NOMEM = 207
  Integer(c_int), Parameter :: EXAMD_ERR_STATE = 208
  Integer(c_int), Parameter :: EXAMD_ERR_NO_DEVICE = 209
  Integer(c_int), Parameter :: EXAMD_ERR_IO = 210
  Integer(c_int), Parameter :: EXAMD_ERR_PAIRFN = 211
  Integer(c_int), Parameter :: EXAMD_ERR_CHECK = 212

  Integer(c_int), Parameter :: EXAMD_MAX_TYPES = 4
  Integer(c_int), Parameter :: EXAMD_POT_LJ = 0, EXAMD_POT_LJ_SHIFTED = 1, EXAMD_POT_WCA = 2
  Integer(c_int), Parameter :: EXAMD_FP64 = 0, EXAMD_MIXED = 1
  Integer(c_int64_t), Parameter :: EXAMD_STATIC_MAX_ATOMS = 1048576_c_int64_t
  Integer(c_int), Parameter :: EXAMD_STATIC_MAX_BOXES = 4096

  ! struct examd_params: same field order and C types.  The type tables are
  ! row-major [a*ntypes+b] in C; for the single-type case eps(1), sigma(1)
  ! and rc(1) take prmvdw(1,1), prmvdw(1,2) and prmvdw(1,5).
  Type, bind(C) :: examd_params
     Integer(c_int) :: precision
     Integer(c_int) :: ntypes
     Real(c_double) :: eps(EXAMD_MAX_TYPES * EXAMD_MAX_TYPES)
     Real(c_double) :: sigma(EXAMD_MAX_TYPES * EXAMD_MAX_TYPES)
     Real(c_double) :: rc(EXAMD_MAX_TYPES * EXAMD_MAX_TYPES)
     Real(c_double) :: mass(EXAMD_MAX_TYPES)
     Real(c_double) :: cell_edge
     Integer(c_int) :: tile(3)
     Integer(c_int) :: warps
     Integer(c_int) :: strict_box
     Integer(c_int) :: device
     Integer(c_int) :: potential
     Integer(c_int) :: pair_tables
     Integer(c_int) :: tile_balance
     Real(c_double) :: pair_skin
     Integer(c_int) :: pair_list_capacity
  End Type examd_params

  ! struct examd_box
  Type, bind(C) :: examd_box
     Real(c_double) :: L(3)
     Integer(c_int64_t) :: natoms
  End Type examd_box

  ! struct examd_stats
  Type, bind(C) :: examd_stats
     Real(c_double) :: epot
     Real(c_double) :: virial
     Real(c_double) :: ekin
     Integer(c_int64_t) :: steps
     Real(c_double) :: ms
  End Type examd_stats

  Interface

     Subroutine examd_default_params(p) bind(C, name="examd_default_params")
       Import :: examd_params
       Type(examd_params), Intent(out) :: p
     End Subroutine examd_default_params

     Integer(c_int) Function examd_gpu_create(params, nboxes, boxes, ctx) bind(C, name="examd_gpu_create")
       Import :: c_int, c_ptr, examd_params, examd_box
       Type(examd_params), Intent(in) :: params
       Integer(c_int), Value :: nboxes
       Type(examd_box), Intent(in) :: boxes(*)
       Type(c_ptr), Intent(out) :: ctx
     End Function examd_gpu_create

     Subroutine examd_gpu_destroy(ctx) bind(C, name="examd_gpu_destroy")
       Import :: c_ptr
       Type(c_ptr), Value :: ctx
     End Subroutine examd_gpu_destroy

     Integer(c_int) Function examd_gpu_set_atoms(ctx, n, pos, type, vel) bind(C, name="examd_gpu_set_atoms")
       Import :: c_int, c_int64_t, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int64_t), Value :: n
       Real(c_double), Intent(in) :: pos(3, *)
       Type(c_ptr), Value :: type   ! c_null_ptr: every atom type 0
       Type(c_ptr), Value :: vel    ! c_null_ptr: zero velocities
     End Function examd_gpu_set_atoms

     Integer(c_int) Function examd_gpu_forces(ctx, forces, epot, virial, accumulate) bind(C, name="examd_gpu_forces")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double), Intent(inout) :: forces(3, *)
       Type(c_ptr), Value :: epot, virial   ! per-box arrays, or c_null_ptr
       Integer(c_int), Value :: accumulate
     End Function examd_gpu_forces

     Integer(c_int) Function examd_gpu_forces_at(ctx, pos, forces, epot, virial, accumulate) &
          bind(C, name="examd_gpu_forces_at")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double), Intent(in) :: pos(3, *)
       Real(c_double), Intent(inout) :: forces(3, *)
       Type(c_ptr), Value :: epot, virial   ! per-box arrays, or c_null_ptr
       Integer(c_int), Value :: accumulate
     End Function examd_gpu_forces_at

     Integer(c_int) Function examd_gpu_run(ctx, nsteps, dt, graph_chunk, energies, stats) bind(C, name="examd_gpu_run")
       Import :: c_int, c_double, c_ptr, examd_stats
       Type(c_ptr), Value :: ctx
       Integer(c_int), Value :: nsteps
       Real(c_double), Value :: dt
       Integer(c_int), Value :: graph_chunk
       Type(c_ptr), Value :: energies       ! nsteps*nboxes*2 doubles, or c_null_ptr
       Type(examd_stats), Intent(out) :: stats
     End Function examd_gpu_run

     Integer(c_int) Function examd_gpu_prepare_run(ctx, dt, graph_chunk, energies) bind(C, name="examd_gpu_prepare_run")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double), Value :: dt
       Integer(c_int), Value :: graph_chunk
       Integer(c_int), Value :: energies
     End Function examd_gpu_prepare_run

     Integer(c_int) Function examd_gpu_time_phases(ctx, nsteps, dt, ms) bind(C, name="examd_gpu_time_phases")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int), Value :: nsteps
       Real(c_double), Value :: dt
       Real(c_double), Intent(out) :: ms(3)
     End Function examd_gpu_time_phases

     Integer(c_int) Function examd_gpu_time_rebuild(ctx, reps, ms) bind(C, name="examd_gpu_time_rebuild")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int), Value :: reps
       Real(c_double), Intent(out) :: ms
     End Function examd_gpu_time_rebuild

     Integer(c_int) Function examd_gpu_list_info(ctx, builds, capacity, longest, fallback_tiles) &
          bind(C, name="examd_gpu_list_info")
       Import :: c_int, c_int64_t, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int64_t), Intent(out) :: builds
       Integer(c_int), Intent(out) :: capacity, longest, fallback_tiles
     End Function examd_gpu_list_info

     Integer(c_int) Function examd_gpu_get_state(ctx, pos, vel) bind(C, name="examd_gpu_get_state")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ctx
       Type(c_ptr), Value :: pos, vel       ! 3*n doubles each, or c_null_ptr
     End Function examd_gpu_get_state

     Integer(c_int) Function examd_gpu_kinetic(ctx, ekin) bind(C, name="examd_gpu_kinetic")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double), Intent(out) :: ekin(*)
     End Function examd_gpu_kinetic

     Integer(c_int) Function examd_kinetic_static(device, natoms, nboxes, atom0, vx, vy, vz, type, ntypes, mass, &
          ekin, stream, errbuf, errbuf_len) bind(C, name="examd_kinetic_static")
       Import :: c_int, c_int64_t, c_double, c_ptr, c_char
       Integer(c_int), Value :: device
       Integer(c_int64_t), Value :: natoms
       Integer(c_int), Value :: nboxes
       Integer(c_int64_t), Intent(in) :: atom0(*)
       Type(c_ptr), Value :: vx, vy, vz, type   ! device arrays (type may be c_null_ptr)
       Integer(c_int), Value :: ntypes
       Real(c_double), Intent(in) :: mass(*)
       Real(c_double), Intent(out) :: ekin(*)
       Type(c_ptr), Value :: stream
       Character(kind=c_char), Intent(out) :: errbuf(*)
       Integer(c_int), Value :: errbuf_len
     End Function examd_kinetic_static

     Integer(c_int) Function examd_gpu_scale_velocities(ctx, factor) bind(C, name="examd_gpu_scale_velocities")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Real(c_double), Intent(in) :: factor(*)
     End Function examd_gpu_scale_velocities

     Integer(c_int) Function examd_autotune(params, nboxes, boxes, n, pos, type, cache_path, best, best_ms) &
          bind(C, name="examd_autotune")
       Import :: c_int, c_int64_t, c_double, c_ptr, examd_params, examd_box
       Type(examd_params), Intent(in) :: params
       Integer(c_int), Value :: nboxes
       Type(examd_box), Intent(in) :: boxes(*)
       Integer(c_int64_t), Value :: n
       Real(c_double), Intent(in) :: pos(3, *)
       Type(c_ptr), Value :: type
       Type(c_ptr), Value :: cache_path     ! c_loc of a NUL-terminated name, or c_null_ptr
       Type(examd_params), Intent(out) :: best
       Real(c_double), Intent(out) :: best_ms
     End Function examd_autotune

     Integer(c_int) Function examd_gpu_time_forces(ctx, reps, ms, kernel_ms) bind(C, name="examd_gpu_time_forces")
       Import :: c_int, c_double, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int), Value :: reps
       Real(c_double), Intent(out) :: ms, kernel_ms
     End Function examd_gpu_time_forces

     Integer(c_int) Function examd_gpu_counters(ctx, candidates, accepted, evaluated, tiles, max_tile_atoms) &
          bind(C, name="examd_gpu_counters")
       Import :: c_int, c_int64_t, c_ptr
       Type(c_ptr), Value :: ctx
       Integer(c_int64_t), Intent(out) :: candidates, accepted, evaluated, tiles, max_tile_atoms
     End Function examd_gpu_counters

     Integer(c_int) Function examd_own_table(rows, lut) bind(C, name="examd_own_table")
       Import :: c_int, c_signed_char
       Integer(c_signed_char), Intent(out) :: rows(26)
       Integer(c_signed_char), Intent(out) :: lut(1625)   ! unsigned char in C: masks 0..31
     End Function examd_own_table

     Integer(c_int) Function examd_tile_split(nb, last_width, tile_len, tile_balance, starts, nt) &
          bind(C, name="examd_tile_split")
       Import :: c_int, c_double
       Integer(c_int), Value :: nb
       Real(c_double), Value :: last_width
       Integer(c_int), Value :: tile_len, tile_balance
       Integer(c_int), Intent(out) :: starts(*)
       Integer(c_int), Intent(out) :: nt
     End Function examd_tile_split

     Type(c_ptr) Function examd_gpu_strerror(code) bind(C, name="examd_gpu_strerror")
       Import :: c_int, c_ptr
       Integer(c_int), Value :: code
     End Function examd_gpu_strerror

     Type(c_ptr) Function examd_gpu_last_error(ctx) bind(C, name="examd_gpu_last_error")
       Import :: c_ptr
       Type(c_ptr), Value :: ctx
     End Function examd_gpu_last_error

     Integer(c_int) Function examd_host_alloc(ptr, bytes) bind(C, name="examd_host_alloc")
       Import :: c_int, c_int64_t, c_ptr
       Type(c_ptr), Intent(out) :: ptr
       Integer(c_int64_t), Value :: bytes
     End Function examd_host_alloc

     Integer(c_int) Function examd_host_free(ptr) bind(C, name="examd_host_free")
       Import :: c_int, c_ptr
       Type(c_ptr), Value :: ptr
     End Function examd_host_free

     Integer(c_int) Function examd_read_particles(path, natoms, L, pos, capacity) bind(C, name="examd_read_particles")
       Import :: c_int, c_int64_t, c_double, c_char, c_ptr
       Character(kind=c_char), Intent(in) :: path(*)   ! NUL-terminated
       Integer(c_int64_t), Intent(out) :: natoms
       Real(c_double), Intent(out) :: L(3)
       Type(c_ptr), Value :: pos                       ! c_null_ptr: sizes only
       Integer(c_int64_t), Value :: capacity
     End Function examd_read_particles

     Integer(c_int) Function examd_write_particles(path, natoms, L, pos) bind(C, name="examd_write_particles")
       Import :: c_int, c_int64_t, c_double, c_char
       Character(kind=c_char), Intent(in) :: path(*)
       Integer(c_int64_t), Value :: natoms
       Real(c_double), Intent(in) :: L(3)
       Real(c_double), Intent(in) :: pos(3, *)
     End Function examd_write_particles

     Integer(c_int) Function examd_gen_fcc(nc, rho, pos, L) bind(C, name="examd_gen_fcc")
       Import :: c_int, c_double
       Integer(c_int), Value :: nc
       Real(c_double), Value :: rho
       Real(c_double), Intent(out) :: pos(3, *)
       Real(c_double), Intent(out) :: L
     End Function examd_gen_fcc

     Integer(c_int) Function examd_gen_velocities(n, type, mass, T, seed, vel) bind(C, name="examd_gen_velocities")
       Import :: c_int, c_int64_t, c_double, c_ptr
       Integer(c_int64_t), Value :: n
       Type(c_ptr), Value :: type, mass
       Real(c_double), Value :: T
       Integer(c_int64_t), Value :: seed      ! uint64_t in C
       Real(c_double), Intent(out) :: vel(3, *)
     End Function examd_gen_velocities

     Integer(c_int) Function examd_gen_random(n, n_fixed, L, lo, hi, dmin, seed, max_tries, pos) &
          bind(C, name="examd_gen_random")
       Import :: c_int, c_int64_t, c_double
       Integer(c_int64_t), Value :: n, n_fixed
       Real(c_double), Intent(in) :: L(3), lo(3), hi(3)
       Real(c_double), Value :: dmin
       Integer(c_int64_t), Value :: seed      ! uint64_t in C
       Integer(c_int64_t), Value :: max_tries
       Real(c_double), Intent(inout) :: pos(3, *)
     End Function examd_gen_random

     Integer(c_int) Function examd_gen_jittered_sc(m, rho, jitter, frac_b, seed, pos, type, L) &
          bind(C, name="examd_gen_jittered_sc")
       Import :: c_int, c_int64_t, c_double
       Integer(c_int), Value :: m
       Real(c_double), Value :: rho, jitter, frac_b
       Integer(c_int64_t), Value :: seed      ! uint64_t in C
       Real(c_double), Intent(out) :: pos(3, *)
       Integer(c_int), Intent(out) :: type(*)
       Real(c_double), Intent(out) :: L
     End Function examd_gen_jittered_sc

  End Interface

End Module examd_gpu_mod
