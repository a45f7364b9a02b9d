/*
 * examd_oracle.h -- CPU oracle for the midpoint Lennard-Jones force path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (examd_gb300/, include/,
 * bench.py's GPU arm) links or calls this code.  It is used by tests/, by
 * __graft_entry__.smoke() as the checker, and by bench.py's cpu_baseline leg
 * and reference arm.
 *
 * Parity status: UNPINNED against the reference binary.  The reference
 * (exaMD, Fortran 90 + MPI) ships no tests, fixtures or golden vectors, and it
 * cannot be compiled on this machine (no Fortran compiler, MPI or METIS).  The
 * restatement in examd_oracle.c follows the reference sources line by line and
 * is pinned instead by analytic known-answer tests and by an independent
 * O(N^2) brute-force pair sum (examd_oracle_ext.c).
 */
#ifndef EXAMD_ORACLE_H
#define EXAMD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes.  109 keeps the reference's MPI_Abort code for "block number out
 * of range" (SRC/exaMD_module.f90:118-123). */
#define EXO_OK 0
#define EXO_ERR_OUTSIDE 109
#define EXO_ERR_NB_TOO_SMALL 201
#define EXO_ERR_ARG 202
#define EXO_ERR_NOMEM 203

typedef struct exo_counts {
  int64_t candidates; /* calls of the particle-interaction routine            */
  int64_t accepted;   /* calls whose pair function returned retval == 0       */
  int64_t zero_d2;    /* calls with |d2| < 0.001 (the reference prints these) */
} exo_counts;

/* ---- restated reference path (examd_oracle.c) --------------------------- */

/* nblocks_xyz = Int(globalbox / block_length)  (SRC/exaMD_utils.f90:179). */
void exo_domain_create(const double box[3], double block_length, int nb[3]);

/* Block of one position, 1-based, last block absorbing the remainder
 * (SRC/exaMD_module.f90:101-125).  Returns the linear block number or -109. */
int exo_identify_block(const double pos[3], double block_length,
                       const int nb[3], int bxyz[3]);

/* Slot table of the midpoint method: 63 (slot_a, slot_b) pairs, slots 1..27
 * (SRC/exaMD_module.f90:276-346).  out[2*k], out[2*k+1] for k = 0..62. */
void exo_midpoint_table(int *out);

/* One force evaluation of exaMD_forces_midpoint_all with noprocs == 1
 * (SRC/exaMD_forces.f90:308-390, 492-551; user_func.f90:40-75).
 * pos: 3*n doubles, atom-major (Fortran posn(3,n) order).
 * forces: 3*n doubles, ACCUMULATED (+=) as the reference does.
 * eps, sigma, cutoff: prmvdw(1,1), prmvdw(1,2), prmvdw(1,5). */
int exo_forces_midpoint_all(int64_t n, const double *pos, const double box[3],
                            double block_length, double eps, double sigma,
                            double cutoff, double *forces, exo_counts *counts);

/* ---- extensions (examd_oracle_ext.c): not in the reference ------------- */

/* Typed LJ with potential energy and virial, same block loops.
 * type: n ints in [0, ntypes) (NULL = all 0).  eps/sigma/rc: ntypes^2 tables.
 * epot, virial (scalar W = sum r_ij . f_ij), virial9 (tensor, may be NULL). */
int exo_forces_typed(int64_t n, const double *pos, const int *type,
                     const double box[3], double block_length, int ntypes,
                     const double *eps, const double *sigma, const double *rc,
                     double *forces, double *epot, double *virial,
                     double *virial9, exo_counts *counts);

/* Same sums as exo_forces_typed over all unordered pairs, O(N^2), minimum
 * image.  Independent of the block decomposition. */
int exo_forces_bruteforce(int64_t n, const double *pos, const int *type,
                          const double box[3], int ntypes, const double *eps,
                          const double *sigma, const double *rc,
                          double *forces, double *epot, double *virial);

/* exo_forces_typed parallelised over home blocks with OpenMP (nthreads <= 0:
 * all).  Per-thread force buffers; the stand-in for the reference's MPI ranks. */
int exo_forces_typed_omp(int64_t n, const double *pos, const int *type,
                         const double box[3], double block_length, int ntypes,
                         const double *eps, const double *sigma,
                         const double *rc, double *forces, double *epot,
                         double *virial, int nthreads, exo_counts *counts);

/* Velocity-Verlet: nsteps of v += dt/2 F/m; x += dt v; wrap; F(x); v += dt/2
 * F/m.  forces must hold F(x) on entry and holds F on exit.  ekin/epot per
 * step are written to energies[2*s], energies[2*s+1] when non-NULL. */
int exo_vv_run(int64_t n, double *pos, double *vel, const int *type,
               const double *mass, const double box[3], double block_length,
               int ntypes, const double *eps, const double *sigma,
               const double *rc, double dt, int nsteps, int nthreads,
               double *forces, double *energies);

/* Periodic wrap into [0, L): x - floor(x / L) * L, then one fix-up. */
double exo_wrap(double x, double L, double Linv);

#ifdef __cplusplus
}
#endif
#endif
