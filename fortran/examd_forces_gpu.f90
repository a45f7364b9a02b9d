!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!
!!!!!   examd_forces_gpu.f90
!!!!!
!!!!!   Drop-in for the force call of the exaMD driver on one GB300.  The
!!!!!   driver keeps its blocks, block lists and output; this module gathers
!!!!!   the positions of its own blocks into one contiguous posn(3,n) array in
!!!!!   locblocks order, makes one call to the GPU library, and adds the
!!!!!   returned forces back into the blocks, as the reference accumulates into
!!!!!   grid(:,:,:)%forces (SRC/exaMD_forces.f90:538-542).
!!!!!
!!!!!   In exaMD.f90, after exaMD_setup_midpoint_interactions (:230):
!!!!!
!!!!!     Call exaMD_forces_gpu_setup(cutoff, EXAMD_FP64)      ! or EXAMD_MIXED
!!!!!     (or, with pair lists: Call exaMD_forces_gpu_setup(cutoff, EXAMD_MIXED, 0.4_PRC))
!!!!!
!!!!!   and in place of the force call at exaMD.f90:247-251:
!!!!!
!!!!!     Call exaMD_forces_midpoint_gpu()
!!!!!
!!!!!   (both branches of the reference, _all and _overlap, compute the same
!!!!!   forces; one GPU has no halo to overlap).  The t1/t2 timers around the
!!!!!   call stay as they are.  At the end: Call exaMD_forces_gpu_finalize().
!!!!!
!!!!!   Module state used from the reference (SRC/exaMD_module.f90:17-82,
!!!!!   user_func.f90:16-18): grid, locblocks, nblocks_loc, globalbox,
!!!!!   COMM_EXAMD, prmvdw.  One rank per GPU: with noprocs == 1 every block is
!!!!!   local (SRC/exaMD_partitioning.f90:448-451).
!!!!!
!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!!

Module examd_forces_gpu_mod

  Use, Intrinsic :: iso_c_binding
  Use exaMD_mod
  Use user_func_mod, Only: prmvdw
  Use examd_gpu_mod

  Implicit None

  Private
  Public :: exaMD_forces_gpu_setup, exaMD_forces_midpoint_gpu, exaMD_forces_gpu_finalize

  Type(c_ptr), Save :: ctx = c_null_ptr
  Integer(c_int64_t), Save :: natms_gpu = 0
  ! page-locked (examd_host_alloc): from the second call with the same
  ! arrays the library replays the call as a captured CUDA graph
  Type(c_ptr), Save :: pos_mem = c_null_ptr, frc_mem = c_null_ptr, ep_mem = c_null_ptr, vir_mem = c_null_ptr
  Real(c_double), Pointer, Save :: posbuf(:,:) => Null(), fbuf(:,:) => Null()
  Real(c_double), Pointer, Save :: epot(:) => Null(), virial(:) => Null()

Contains

  !!  The atom count of this rank's blocks (all blocks when noprocs == 1).
  Integer(c_int64_t) Function local_atoms()
    Integer :: b
    local_atoms = 0
    Do b = 1, nblocks_loc
       local_atoms = local_atoms + grid(locblocks(1,b), locblocks(2,b), locblocks(3,b))%natms
    End Do
  End Function local_atoms

  !!  posbuf(:, 1:n) <- grid(:,:,:)%posn in locblocks order.
  Subroutine gather_positions()
    Integer :: b, i, j, k, na, m
    m = 0
    Do b = 1, nblocks_loc
       i = locblocks(1,b); j = locblocks(2,b); k = locblocks(3,b)
       na = grid(i,j,k)%natms
       If (na > 0) posbuf(:, m+1:m+na) = Real(grid(i,j,k)%posn(:, 1:na), c_double)
       m = m + na
    End Do
  End Subroutine gather_positions

  !!  grid(:,:,:)%forces += fbuf(:, 1:n) in locblocks order.
  Subroutine scatter_forces()
    Integer :: b, i, j, k, na, m
    m = 0
    Do b = 1, nblocks_loc
       i = locblocks(1,b); j = locblocks(2,b); k = locblocks(3,b)
       na = grid(i,j,k)%natms
       If (na > 0) grid(i,j,k)%forces(:, 1:na) = grid(i,j,k)%forces(:, 1:na) &
            + Real(fbuf(:, m+1:m+na), Kind(grid(i,j,k)%forces))
       m = m + na
    End Do
  End Subroutine scatter_forces

  !!  A status other than EXAMD_OK stops the run as the reference stops on
  !!  its own fatal errors: MPI_Abort with the status as the error code.
  Subroutine check(rc, where)
    Integer(c_int), Intent(in) :: rc
    Character(len=*), Intent(in) :: where
    Character(kind=c_char), Pointer :: msg(:)
    Integer :: n, ierr2
    If (rc == EXAMD_OK) Return
    Call c_f_pointer(examd_gpu_strerror(rc), msg, [256])
    n = 0
    Do While (n < 256)
       If (msg(n+1) == c_null_char) Exit
       n = n + 1
    End Do
    Write(*, '(3A,I0,2A)') 'exaMD GPU: ', where, ' returned ', rc, ': ', Transfer(msg(1:n), Repeat(' ', n))
    Call MPI_Abort(COMM_EXAMD, Int(rc), ierr2)
  End Subroutine check

  !!  Create the GPU context for this rank's atoms: the box (globalbox), the
  !!  LJ parameters of the driver's set-up (prmvdw(1,1:5) = eps, sigma, -, -,
  !!  rc: exaMD.f90:199-202), the reference's cell edge rc/2 (exaMD.f90:56),
  !!  and the current positions.  precision: EXAMD_FP64 (the reference's
  !!  arithmetic) or EXAMD_MIXED.  skin (optional, EXAMD_MIXED only): the
  !!  per-tile pair lists' skin in sigma; the library rebuilds its cells and
  !!  lists at the calls whose atoms moved more than half of it since the last
  !!  build, and the cell edge becomes (rc + skin)/2.
  Subroutine exaMD_forces_gpu_setup(cutoff, precision, skin)
    Real(kind=PRC), Intent(in) :: cutoff
    Integer(c_int), Intent(in) :: precision
    Real(kind=PRC), Intent(in), Optional :: skin
    Type(examd_params) :: p, best
    Type(examd_box) :: box(1)
    Real(c_double) :: ms
    Integer(c_int) :: rc

    Call examd_default_params(p)
    p%precision = precision
    p%eps(1) = Real(prmvdw(1,1), c_double)
    p%sigma(1) = Real(prmvdw(1,2), c_double)
    p%rc(1) = Real(cutoff, c_double)
    p%cell_edge = 0.0_c_double
    If (Present(skin)) p%pair_skin = Real(skin, c_double)
    box(1)%L = Real(globalbox, c_double)
    natms_gpu = local_atoms()
    box(1)%natoms = natms_gpu

    rc = examd_host_alloc(pos_mem, 24_c_int64_t * Max(natms_gpu, 1_c_int64_t))
    Call check(rc, 'examd_host_alloc')
    rc = examd_host_alloc(frc_mem, 24_c_int64_t * Max(natms_gpu, 1_c_int64_t))
    Call check(rc, 'examd_host_alloc')
    rc = examd_host_alloc(ep_mem, 8_c_int64_t)
    Call check(rc, 'examd_host_alloc')
    rc = examd_host_alloc(vir_mem, 8_c_int64_t)
    Call check(rc, 'examd_host_alloc')
    Call c_f_pointer(pos_mem, posbuf, [3_c_int64_t, Max(natms_gpu, 1_c_int64_t)])
    Call c_f_pointer(frc_mem, fbuf, [3_c_int64_t, Max(natms_gpu, 1_c_int64_t)])
    Call c_f_pointer(ep_mem, epot, [1])
    Call c_f_pointer(vir_mem, virial, [1])

    Call gather_positions()
    ! tile shape, CTA width and tile split timed on these atoms (a few seconds, once)
    rc = examd_autotune(p, 1_c_int, box, natms_gpu, posbuf, c_null_ptr, c_null_ptr, best, ms)
    If (rc == EXAMD_OK) p = best
    rc = examd_gpu_create(p, 1_c_int, box, ctx)
    Call check(rc, 'examd_gpu_create')
    rc = examd_gpu_set_atoms(ctx, natms_gpu, posbuf, c_null_ptr, c_null_ptr)
    Call check(rc, 'examd_gpu_set_atoms')
  End Subroutine exaMD_forces_gpu_setup

  !!  The counterpart of Call exaMD_forces_midpoint_all(lennardjones_12,
  !!  cutoff, noprocs) (SRC/exaMD_forces.f90:308-390): forces at the blocks'
  !!  current positions, added to grid(:,:,:)%forces.  The potential energy
  !!  and virial come back in epot(1) and virial(1) (the reference's e12 slot
  !!  is zero, user_func.f90:71).
  Subroutine exaMD_forces_midpoint_gpu()
    Integer(c_int) :: rc
    Call gather_positions()
    rc = examd_gpu_forces_at(ctx, posbuf, fbuf, ep_mem, vir_mem, 0_c_int)
    Call check(rc, 'examd_gpu_forces_at')
    Call scatter_forces()
  End Subroutine exaMD_forces_midpoint_gpu

  Subroutine exaMD_forces_gpu_finalize()
    Integer(c_int) :: rc
    If (c_associated(ctx)) Call examd_gpu_destroy(ctx)
    ctx = c_null_ptr
    If (c_associated(pos_mem)) rc = examd_host_free(pos_mem)
    If (c_associated(frc_mem)) rc = examd_host_free(frc_mem)
    If (c_associated(ep_mem)) rc = examd_host_free(ep_mem)
    If (c_associated(vir_mem)) rc = examd_host_free(vir_mem)
    pos_mem = c_null_ptr; frc_mem = c_null_ptr; ep_mem = c_null_ptr; vir_mem = c_null_ptr
    Nullify(posbuf, fbuf, epot, virial)
  End Subroutine exaMD_forces_gpu_finalize

End Module examd_forces_gpu_mod
