/*
 * examd_gb300.h -- C ABI of the GB300 (sm_103a) midpoint Lennard-Jones force
 * path.  Plain C types only: pointers, sizes, a POD parameter struct.  Every
 * entry point returns an int status (0 = EXAMD_OK); nothing throws across the
 * boundary.  One host thread per context; calls are synchronous on the
 * context's own CUDA stream.
 *
 * Reference interface this replaces:
 *   Subroutine exaMD_forces_midpoint_all(user_func, cutoff, noprocs)
 *     SRC/exaMD_forces.f90:308-318, called from exaMD.f90:247-251.
 *   Its inputs are module state: grid(:,:,:)%posn/%natms (SRC/exaMD_module.f90:
 *   34-54), globalbox/globalboxi (:54), the 63-entry interactions table
 *   (:276-346) and the pair plug-in lennardjones_12 with its parameters
 *   prmvdw(1,1:5) (user_func.f90:16-18,40-75).  Its output is
 *   grid(:,:,:)%forces, accumulated (+=).
 * The GPU replacement takes the same information as explicit arguments: the
 * atoms gathered into one contiguous posn(3,n) array, the box, and the LJ
 * parameters; it returns forces in the same (3,n) order plus the potential
 * energy and virial that the reference's e12 slot was meant to carry
 * (user_func.f90:71 leaves it zero).
 */
#ifndef EXAMD_GB300_H
#define EXAMD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------
 * 109 keeps the reference's MPI_Abort code for an atom whose block number is
 * out of range (SRC/exaMD_module.f90:118-123).  The others are new: the
 * reference prints and aborts (codes 101-109) or has no check at all. */
#define EXAMD_OK 0
#define EXAMD_ERR_OUTSIDE 109       /* position outside the box (strict mode) */
#define EXAMD_ERR_ARG 201           /* bad argument or parameter              */
#define EXAMD_ERR_NB_TOO_SMALL 202  /* fewer than 5 cells on an axis          */
#define EXAMD_ERR_CELL_OVERFLOW 203 /* a tile's staged atoms exceed capacity  */
#define EXAMD_ERR_NONFINITE 204     /* NaN/Inf position or force              */
#define EXAMD_ERR_TIMEOUT 205       /* a bounded device wait gave up (reserved:
                                       no current kernel waits on another CTA) */
#define EXAMD_ERR_CUDA 206          /* CUDA runtime error                     */
#define EXAMD_ERR_NOMEM 207         /* device or pinned allocation failed     */
#define EXAMD_ERR_STATE 208         /* call order (e.g. no atoms set)         */
#define EXAMD_ERR_NO_DEVICE 209     /* no CUDA device / wrong architecture    */
#define EXAMD_ERR_IO 210            /* file missing, unreadable or malformed  */
#define EXAMD_ERR_PAIRFN 211        /* the pair function returned an error    */
#define EXAMD_ERR_CHECK 212         /* checked build (-DEXAMD_CHECKED): an index
                                       of a kernel fell outside its array      */

#define EXAMD_MAX_TYPES 4

/* Pair functions (examd_params.potential), the counterpart of the reference's
 * External :: user_func (SRC/exaMD_forces.f90:532) and its return codes: 0
 * apply the pair, > 0 skip it, < 0 error (EXAMD_ERR_PAIRFN; coincident atoms,
 * r^2 < 1e-12, are an error for every potential). */
#define EXAMD_POT_LJ 0         /* lennardjones_12 (user_func.f90:40-75): cut at
                                  rc, unshifted; energy 4 eps (s^12 - s^6)   */
#define EXAMD_POT_LJ_SHIFTED 1 /* same forces, energy shifted to 0 at rc     */
#define EXAMD_POT_WCA 2        /* LJ cut at 2^(1/6) sigma and shifted up by
                                  eps (purely repulsive); rc only bounds the
                                  candidate pairs and must be >= that range  */

/* Precision forms. */
#define EXAMD_FP64 0  /* FP64 end to end                                       */
#define EXAMD_MIXED 1 /* FP32 pair forces on tile-frame offsets, Kahan-merged  */
                      /* FP32 per-atom sums, FP64 integration/wrap/reductions  */

typedef struct examd_params {
  int precision;      /* EXAMD_FP64 or EXAMD_MIXED                            */
  int ntypes;         /* 1..EXAMD_MAX_TYPES                                   */
  /* ntypes x ntypes tables, row-major [a*ntypes+b], symmetric.  eps = prmvdw
   * (1,1), sigma = prmvdw(1,2), rc = prmvdw(1,5) for the single-type case. */
  double eps[EXAMD_MAX_TYPES * EXAMD_MAX_TYPES];
  double sigma[EXAMD_MAX_TYPES * EXAMD_MAX_TYPES];
  double rc[EXAMD_MAX_TYPES * EXAMD_MAX_TYPES];
  double mass[EXAMD_MAX_TYPES]; /* 0 = 1.0                                     */
  /* block_length: the cell edge, >= max(rc)/2; 0 = max(rc)/2 as the reference
   * (exaMD.f90:56).  Rounded up to the nearest value with at most 14
   * significant bits so that every cell origin c*block_length is exact in
   * FP32.  nb = Int(L/block_length) cells per axis with the last cell
   * absorbing the remainder (SRC/exaMD_utils.f90:179,
   * SRC/exaMD_module.f90:109-113). */
  double cell_edge;
  int tile[3];        /* home cells per CTA tile per axis; 0 = default        */
  int warps;          /* warps per CTA in the pair kernel; 0 = default        */
  int strict_box;     /* 1: positions outside [0,L) are an error (109);       */
                      /* 0: they are wrapped periodically                     */
  int device;         /* CUDA device ordinal                                  */
  int potential;      /* EXAMD_POT_*                                          */
  int pair_tables;    /* mixed form's per-warp tables in the pair kernel:     */
                      /* 0 = chosen by occupancy, 1 = wide, 2 = compact       */
  int tile_balance;   /* split of an axis into tiles: 0 = by cell count;      */
                      /* 1 = by width, where the last cell (which absorbs the */
                      /* box's remainder) is >= 1.5 edges wide it counts as   */
                      /* two, so its tile has one cell fewer and the largest  */
                      /* tile, which sizes shared memory, is smaller          */
  /* pair_skin: 0 = the reference's schedule, cells and candidate pairs
   * rebuilt at every force evaluation.  > 0 (EXAMD_MIXED only): pair-list
   * mode.  Each tile keeps the list of its pairs within rc + pair_skin, built
   * by the same midpoint ownership; later evaluations compute the forces from
   * the lists, and the cells and lists are rebuilt, on the device, at the
   * first evaluation at which some atom has moved more than pair_skin / 2
   * (less 1e-4) since the last build.  Every pair within rc is still
   * computed exactly once, with the same FP32 expression.  The cell edge
   * becomes at least (max(rc) + pair_skin) / 2. */
  double pair_skin;
  /* pair_list_capacity: pair-list mode's list entries per atom (the pairs it
   * owns in its tile), a multiple of 8 up to 1024; 0 = sized by the library
   * (the most at the first build + 20 %, grown when an atom outgrows it).  A
   * tile with an atom whose pairs do not fit is computed by enumeration at
   * every evaluation until the next build. */
  int pair_list_capacity;
} examd_params;

/* One independent periodic box of a batched ensemble. */
typedef struct examd_box {
  double L[3];
  int64_t natoms;
} examd_box;

typedef struct examd_stats {
  double epot;     /* potential energy, FP64 reduction                        */
  double virial;   /* W = sum over pairs of r_ij . f_ij                       */
  double ekin;     /* kinetic energy after the last step                      */
  int64_t steps;   /* steps taken                                             */
  double ms;       /* device time of the call, CUDA events                    */
} examd_stats;

typedef struct examd_ctx examd_ctx;

/* Fill *p with the reference defaults: FP64, one type, eps = sigma = 1,
 * rc = 2.5, reference cell rule, default tiles. */
void examd_default_params(examd_params *p);

/* Create a context for nboxes independent boxes (1 for the reference's single
 * domain).  Fails with EXAMD_ERR_NB_TOO_SMALL if any box has fewer than 5
 * cells on an axis: with 4 or fewer, separations +2 and -2 name the same cell
 * pair and the 63-entry table would count it twice. */
int examd_gpu_create(const examd_params *params, int nboxes,
                     const examd_box *boxes, examd_ctx **out);
void examd_gpu_destroy(examd_ctx *ctx);

/* Upload atoms.  pos: 3*n doubles, posn(3,n) order, boxes concatenated in
 * order; n must equal the sum of the boxes' natoms.  type: n ints or NULL
 * (all type 0).  vel: 3*n doubles or NULL (zero). */
int examd_gpu_set_atoms(examd_ctx *ctx, int64_t n, const double *pos,
                        const int *type, const double *vel);

/* One force evaluation at the current positions: the drop-in for
 * exaMD_forces_midpoint_all.  forces: 3*n doubles in the caller's atom order,
 * overwritten (accumulate = 0) or added to (accumulate = 1, the reference's
 * += semantics).  epot, virial: per-box arrays of nboxes doubles, or NULL. */
int examd_gpu_forces(examd_ctx *ctx, double *forces, double *epot,
                     double *virial, int accumulate);

/* Same as examd_gpu_forces but with new positions given in the same call
 * (one host->device copy, the pair path, one device->host copy). */
int examd_gpu_forces_at(examd_ctx *ctx, const double *pos, double *forces,
                        double *epot, double *virial, int accumulate);

/* nsteps velocity-Verlet steps of size dt (rebinning every step; in
 * pair-list mode at the steps that rebuild the lists).  When
 * graph_chunk > 0 the step loop is captured once as a CUDA graph of
 * graph_chunk steps and replayed.  energies: when non-NULL, per-box
 * (ekin, epot) pairs after every step: nsteps * nboxes * 2 doubles. */
int examd_gpu_run(examd_ctx *ctx, int nsteps, double dt, int graph_chunk,
                  double *energies, examd_stats *stats);

/* Capture, without running any step, the CUDA graph that the next
 * examd_gpu_run(ctx, nsteps, dt, graph_chunk, energies ? buf : NULL, ...)
 * replays, so that the capture and instantiation stay out of a timed run (the
 * reference times its force call alone, exaMD.f90:241-253).  Also sizes the
 * per-step energy buffers and computes the forces at the current positions
 * if none are held.  A no-op for graph_chunk = 0. */
int examd_gpu_prepare_run(examd_ctx *ctx, double dt, int graph_chunk,
                          int energies);

/* Device time of the step's phases, averaged over nsteps eager steps of size
 * dt: ms[0] the kick with drift, wrap and binning count (pair-list mode: the
 * offsets and displacement since the build instead of the count); ms[1] the
 * rest of the binning, scan and scatter (pair-list mode: the rebuild
 * decision, and the binning and list build of the steps that rebuild);
 * ms[2] the pair kernel and the mixed form's redo pass.  CUDA events on the context's stream around each phase (the
 * reference stamps its force call with MPI_WTIME, exaMD.f90:234-263).  The
 * steps use the merged kick of the captured loop (v += dt F/m), so they
 * advance the state but are not a velocity-Verlet trajectory from a state
 * that examd_gpu_run left at full step: for timing only. */
int examd_gpu_time_phases(examd_ctx *ctx, int nsteps, double dt, double *ms);

/* Pair-list mode: device time of reps rebuilds of the cells and the pair
 * lists at the current positions (the work of a step whose atoms moved more
 * than half the skin), in ms per rebuild; the forces are computed again at
 * the next call that needs them.  EXAMD_ERR_ARG without pair lists. */
int examd_gpu_time_rebuild(examd_ctx *ctx, int reps, double *ms);

/* Pair-list mode's state (zeros without it): the builds since the context
 * was created, the list entries per atom, the most entries of one atom at
 * the builds since the last call, and the tiles computed by enumeration
 * because an atom's list did not fit or they outgrew the staged-atom
 * capacity (until the next build). */
int examd_gpu_list_info(examd_ctx *ctx, int64_t *builds, int *capacity,
                        int *longest, int *fallback_tiles);

/* Current positions and velocities in the caller's order (3*n each, NULL to
 * skip). */
int examd_gpu_get_state(examd_ctx *ctx, double *pos, double *vel);

/* Per-box kinetic energy (sum m v^2 / 2) at the current velocities. */
int examd_gpu_kinetic(examd_ctx *ctx, double *ekin);

/* Per-box kinetic energy of atoms in the CALLER's device arrays, with no
 * device allocation (no counterpart in the reference, which has no device
 * memory).  For callers that own their device memory and cannot let a library
 * allocate between steps: a host MD code whose CUDA Fortran / OpenACC arrays or
 * pool allocator hold the free HBM, where cudaMalloc can fail or fragment the
 * pool and cudaFree would synchronise the device under the caller's streams.
 * Scratch is one fixed static device array per device, so:
 *   - natoms <= EXAMD_STATIC_MAX_ATOMS and 1 <= nboxes <= EXAMD_STATIC_MAX_BOXES,
 *     else EXAMD_ERR_ARG before any device work;
 *   - every call shares that array: calls whose device work overlaps (other
 *     threads, or unordered streams) race; sequential calls are safe;
 *   - the first call on a device sets up the array's address
 *     (cudaGetSymbolAddress); make it before any stream capture begins.  The
 *     address is kept for the life of the process: do not call this entry
 *     point on a device after a cudaDeviceReset of it;
 *   - a call that fails after queueing device work waits for that work before
 *     it returns, so sequential calls stay safe on error paths too.
 * atom0: host, nboxes+1 offsets (0 .. natoms) of each box's contiguous atoms.
 * vx, vy, vz: device, natoms doubles each.  type: device, natoms ints in
 * [0, ntypes), or NULL for all type 0.  mass: host, ntypes doubles.  ekin:
 * host, nboxes doubles.  stream: a cudaStream_t, or NULL for the default
 * stream; the call synchronises it before returning.  errbuf (may be NULL):
 * receives a one-line reason when the status is not EXAMD_OK. */
#define EXAMD_STATIC_MAX_ATOMS 1048576
#define EXAMD_STATIC_MAX_BOXES 4096
int examd_kinetic_static(int device, int64_t natoms, int nboxes,
                         const int64_t *atom0, const double *vx,
                         const double *vy, const double *vz, const int *type,
                         int ntypes, const double *mass, double *ekin,
                         void *stream, char *errbuf, int errbuf_len);

/* Scale all velocities of box b by factor[b] (thermostat / melt protocol). */
int examd_gpu_scale_velocities(examd_ctx *ctx, const double *factor);

/* Autotuner (no counterpart in the reference, whose decomposition is the
 * METIS partition and whose block edge is a parameter, SRC/exaMD_utils.f90:
 * 167-190, set to rc/2 by the driver, exaMD.f90:56): time the pair kernel on
 * these atoms for tile shapes of 3-6 home cells per axis, 4 or 8 warps per
 * CTA and, where a box has a last cell of about 1.5 edges or more, both tile
 * splits (tile_balance); then the cell edge at 1.1 and 1.2 times the
 * caller's (rc/2 by default) with the four fastest of those.  Returns the
 * fastest in *best (a copy of *params with tile, warps, tile_balance and
 * cell_edge set) and its time per launch in *best_ms.
 * cache_path (may be NULL): a text file of earlier choices keyed by device,
 * precision, types, cutoff, box count, atom count and density; a hit returns
 * without timing, a miss is appended.  pos/type as in examd_gpu_set_atoms. */
int examd_autotune(const examd_params *params, int nboxes,
                   const examd_box *boxes, int64_t n, const double *pos,
                   const int *type, const char *cache_path,
                   examd_params *best, double *best_ms);

/* Device time in ms of `reps` force evaluations (positions already resident),
 * measured with CUDA events on the context's stream.  kernel_ms, when
 * non-NULL, receives the average duration of the pair kernel alone. */
int examd_gpu_time_forces(examd_ctx *ctx, int reps, double *ms,
                          double *kernel_ms);

/* Counters of one force evaluation at the current positions: candidate pairs
 * (the reference's particle-interaction calls: every atom pair of every owned
 * cell pair, SRC/exaMD_forces.f90:349-377), accepted pairs (r <= rc),
 * evaluated pairs (distance tests the kernel actually ran after skipping cells
 * beyond rc), tiles, and the largest staged atom count of a tile.  Any
 * pointer may be NULL. */
int examd_gpu_counters(examd_ctx *ctx, int64_t *candidates, int64_t *accepted,
                       int64_t *evaluated, int64_t *tiles,
                       int64_t *max_tile_atoms);

/* Introspection (no counterpart in the reference): the row structure and the
 * per-position-class ownership masks the pair kernel derives from the 63-entry
 * table (SRC/exaMD_module.f90:276-346).  rows: 13*2 (dy, dz); lut: 125*13
 * masks over dx = -2..2, lut[class*13 + row].  Host-only; returns EXAMD_ERR_ARG if the table does
 * not have the expected shape. */
int examd_own_table(signed char *rows, unsigned char *lut);

/* Introspection: the split of one box axis of nb cells (nb < 1024) into tiles
 * of at most tile_len cells that examd_gpu_create uses (tile_balance as in
 * examd_params; last_width: the last cell's width in cell edges, in [1, 2)).
 * starts: room for nb/2 + 2 ints; receives *nt + 1 tile starts, the last one
 * nb.  Host-only. */
int examd_tile_split(int nb, double last_width, int tile_len, int tile_balance,
                     int *starts, int *nt);

/* Text of a status code; never NULL. */
const char *examd_gpu_strerror(int code);

/* Last CUDA error text seen by the context (empty if none). */
const char *examd_gpu_last_error(examd_ctx *ctx);

/* Page-locked host buffers for fast copies (cudaHostAlloc). */
int examd_host_alloc(void **ptr, int64_t bytes);
int examd_host_free(void *ptr);

/* ---- the reference's particle file (host code, no device use) ----------- */

/* Read exaMD_particles.dat: natms_tot, globalbox(3), then x y z per atom, as
 * Fortran list-directed records (SRC/exaMD_input_formats.f90:128-192).  With
 * pos = NULL only *natoms and L[3] are filled; then call again with pos of
 * capacity >= 3 * natoms doubles.  EXAMD_ERR_IO: missing, short or malformed
 * file. */
int examd_read_particles(const char *path, int64_t *natoms, double *L,
                         double *pos, int64_t capacity);

/* Write the same format (exaMD_write_particles, :211-235) with 17
 * significant digits, so that the reference reads back the same doubles. */
int examd_write_particles(const char *path, int64_t natoms, const double *L,
                          const double *pos);

/* ---- input generators (host code, no device use) ------------------------ */

/* FCC lattice of 4*nc^3 atoms at density rho, box edge L = nc*(4/rho)^(1/3).
 * pos: 3*4*nc^3 doubles.  Returns the box edge in *L. */
int examd_gen_fcc(int nc, double rho, double *pos, double *L);

/* Maxwell-Boltzmann velocities at temperature T (k_B = 1) with zero net
 * momentum and the kinetic temperature rescaled to exactly T
 * (3(n-1) degrees of freedom).  mass: per-type masses or NULL (1). */
int examd_gen_velocities(int64_t n, const int *type, const double *mass,
                         double T, uint64_t seed, double *vel);

/* Uniform random positions in [lo, hi) of a box L with a minimum pair
 * separation dmin enforced by rejection against a cell grid (periodic).  The
 * first n_fixed atoms of pos are already placed and are kept.  Returns
 * EXAMD_ERR_ARG if an atom could not be placed in max_tries attempts. */
int examd_gen_random(int64_t n, int64_t n_fixed, const double L[3],
                     const double lo[3], const double hi[3], double dmin,
                     uint64_t seed, int64_t max_tries, double *pos);

/* Simple-cubic lattice of m^3 atoms at density rho with uniform jitter of
 * amplitude jitter*a per coordinate; types drawn with P(type 1) = frac_b. */
int examd_gen_jittered_sc(int m, double rho, double jitter, double frac_b,
                          uint64_t seed, double *pos, int *type, double *L);

#ifdef __cplusplus
}
#endif
#endif
