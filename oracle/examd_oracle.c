/*
 * examd_oracle.c -- CPU restatement of exaMD's serial midpoint force path.
 *
 * TEST INFRASTRUCTURE ONLY (see examd_oracle.h).  Parity status: UNPINNED
 * against the reference binary (no reference tests or golden vectors exist and
 * the Fortran cannot be compiled here); pinned by known-answer tests and a
 * brute-force pair sum instead.
 *
 * Every routine below restates one reference routine, keeping its loop nesting
 * and floating-point operation order.  Build with -ffp-contract=off so that no
 * multiply-add is fused where the Fortran has two roundings.  The one choice
 * the Fortran leaves to its compiler is the expansion of (sig2*d2i)**3; this
 * file uses (t*t)*t.
 */
#include "examd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* The 63 block-pair classes of the midpoint method, as (slot_a, slot_b) with
 * slot = (ii+1) + 3(jj+1) + 9(kk+1) + 1 over neighbour offsets ii,jj,kk in
 * {-1,0,1} (ii fastest).  Slot 14 is the home block.  The pairs are data that
 * define which block owns each block pair, so they are reproduced exactly
 * (SRC/exaMD_module.f90:282-344). */
static const int kTable[63][2] = {
    {14, 14}, {14, 15}, {14, 16}, {14, 17}, {14, 18}, {14, 19}, {14, 20},
    {14, 21}, {14, 22}, {14, 23}, {14, 24}, {14, 25}, {14, 26}, {14, 27},
    {10, 18}, {10, 27}, {11, 17}, {11, 18}, {11, 25}, {11, 26}, {11, 27},
    {12, 16}, {12, 17}, {12, 25}, {13, 15}, {13, 18}, {13, 24}, {13, 27},
    {15, 16}, {15, 19}, {15, 22}, {15, 25}, {16, 21}, {16, 24}, {17, 19},
    {17, 20}, {17, 21}, {18, 19}, {19, 5},  {19, 9},  {20, 5},  {20, 7},
    {20, 8},  {20, 9},  {21, 5},  {21, 7},  {22, 5},  {22, 6},  {22, 9},
    {23, 5},  {24, 5},  {24, 4},  {24, 7},  {25, 5},  {25, 3},  {25, 6},
    {26, 5},  {26, 2},  {26, 3},  {27, 1},  {27, 2},  {27, 4},  {27, 5}};

void exo_midpoint_table(int *out) {
  for (int k = 0; k < 63; ++k) {
    out[2 * k] = kTable[k][0];
    out[2 * k + 1] = kTable[k][1];
  }
}

/* SRC/exaMD_utils.f90:179 -- nblocks_xyz = Int(globalbox/block_length). */
void exo_domain_create(const double box[3], double block_length, int nb[3]) {
  for (int a = 0; a < 3; ++a) nb[a] = (int)(box[a] / block_length);
}

/* SRC/exaMD_module.f90:109-123.  Int() truncates toward zero.  The reference
 * only range-checks the linear number; this restatement also rejects a
 * per-axis index below 1 (a position below 0), which the reference would
 * misfile into another block. */
int exo_identify_block(const double pos[3], double block_length,
                       const int nb[3], int b[3]) {
  for (int a = 0; a < 3; ++a) {
    double q = pos[a] / block_length + 1.0;
    if (!(q >= 1.0)) return -EXO_ERR_OUTSIDE; /* also catches NaN */
    b[a] = (int)q;
    if (b[a] > nb[a]) b[a] = nb[a];
  }
  long blocknum = b[0] + (long)(b[1] - 1) * nb[0] + (long)(b[2] - 1) * nb[0] * nb[1];
  if (blocknum < 1 || blocknum > (long)nb[0] * nb[1] * nb[2]) return -EXO_ERR_OUTSIDE;
  return (int)blocknum;
}

/* Blocks as CSR in the reference's linked-list order: the atoms of a block in
 * ascending atom index (SRC/exaMD_input_formats.f90:66-92 inserts in order
 * i = 1..natms_tot and exaMD_partition_work copies the list in that order,
 * SRC/exaMD_partitioning.f90:958-962). */
typedef struct {
  int nb[3];
  int64_t nblocks;
  int64_t *start; /* nblocks + 1 */
  int64_t *atom;  /* n atom indices, grouped by block */
} exo_grid;

static void grid_free(exo_grid *g) {
  free(g->start);
  free(g->atom);
  g->start = g->atom = NULL;
}

static int grid_build(exo_grid *g, int64_t n, const double *pos,
                      const double box[3], double block_length) {
  memset(g, 0, sizeof(*g));
  exo_domain_create(box, block_length, g->nb);
  /* With fewer than 5 blocks on an axis the separations +2 and -2 name the
   * same block pair and the table counts it twice; the reference has no
   * guard (SRC/exaMD_partitioning.f90:789-791). */
  for (int a = 0; a < 3; ++a)
    if (g->nb[a] < 5) return EXO_ERR_NB_TOO_SMALL;
  g->nblocks = (int64_t)g->nb[0] * g->nb[1] * g->nb[2];
  g->start = (int64_t *)calloc((size_t)g->nblocks + 1, sizeof(int64_t));
  g->atom = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int *blk = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
  if (!g->start || !g->atom || !blk) {
    free(blk);
    grid_free(g);
    return EXO_ERR_NOMEM;
  }
  for (int64_t i = 0; i < n; ++i) {
    int b[3];
    int num = exo_identify_block(pos + 3 * i, block_length, g->nb, b);
    if (num < 0) {
      free(blk);
      grid_free(g);
      return EXO_ERR_OUTSIDE;
    }
    blk[i] = num - 1;
    g->start[num] += 1;
  }
  for (int64_t c = 0; c < g->nblocks; ++c) g->start[c + 1] += g->start[c];
  int64_t *fill = (int64_t *)malloc((size_t)g->nblocks * sizeof(int64_t));
  if (!fill) {
    free(blk);
    grid_free(g);
    return EXO_ERR_NOMEM;
  }
  memcpy(fill, g->start, (size_t)g->nblocks * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) g->atom[fill[blk[i]]++] = i;
  free(fill);
  free(blk);
  return EXO_OK;
}

/* neighrefs of block (i,j,k), 1-based, for kk, jj, ii in -1..1 with ii
 * fastest and a periodic Mod wrap (SRC/exaMD_partitioning.f90:783-798).
 * Returned as 0-based linear block numbers, slot s at refs[s-1]. */
static void neighrefs(const int nb[3], int i, int j, int k, int64_t refs[27]) {
  int cnt = 0;
  for (int kk = -1; kk <= 1; ++kk)
    for (int jj = -1; jj <= 1; ++jj)
      for (int ii = -1; ii <= 1; ++ii) {
        int iii = (i + ii + nb[0] - 1) % nb[0] + 1;
        int jjj = (j + jj + nb[1] - 1) % nb[1] + 1;
        int kkk = (k + kk + nb[2] - 1) % nb[2] + 1;
        refs[cnt++] = (int64_t)(iii - 1) + (int64_t)(jjj - 1) * nb[0] +
                      (int64_t)(kkk - 1) * nb[0] * nb[1];
      }
}

/* user_func.f90:40-75, lennardjones_12.  e12 is left at zero as in the
 * reference; the energy-returning variant lives in examd_oracle_ext.c. */
static int lennardjones_12(double dx, double dy, double dz, double d2,
                           double eps, double sigma, double cutoff,
                           double f12[3]) {
  if (d2 > cutoff * cutoff) return 1;
  double eps24 = 24.0 * eps;
  double sig2 = sigma * sigma;
  double d2i = 1.0 / d2;
  double t = sig2 * d2i;
  double d6 = (t * t) * t;
  double d12 = d6 * d6;
  double dg = -((eps24 * (2.0 * d12 - d6)) * d2i);
  f12[0] = dg * dx;
  f12[1] = dg * dy;
  f12[2] = dg * dz;
  return 0;
}

/* Fortran NINT: nearest integer, halves away from zero. */
static double fnint(double x) { return (double)llround(x); }

/* SRC/exaMD_forces.f90:492-551, exaMD_particle_interaction. */
static void particle_interaction(const double *pos, double *forces,
                                 int64_t a1, int64_t a2, const double box[3],
                                 const double boxi[3], double eps,
                                 double sigma, double cutoff,
                                 exo_counts *cnt) {
  const double *p1 = pos + 3 * a1, *p2 = pos + 3 * a2;
  double dx = p2[0] - p1[0];
  double dy = p2[1] - p1[1];
  double dz = p2[2] - p1[2];
  double bt0 = fnint(dx * boxi[0]);
  double bt1 = fnint(dy * boxi[1]);
  double bt2 = fnint(dz * boxi[2]);
  dx = dx - bt0 * box[0];
  dy = dy - bt1 * box[1];
  dz = dz - bt2 * box[2];
  double d2 = dx * dx + dy * dy + dz * dz;
  cnt->candidates++;
  if (fabs(d2) < 0.001) cnt->zero_d2++;
  double f12[3];
  if (lennardjones_12(dx, dy, dz, d2, eps, sigma, cutoff, f12) == 0) {
    cnt->accepted++;
    double *f1 = forces + 3 * a1, *f2 = forces + 3 * a2;
    f1[0] = f1[0] + f12[0];
    f1[1] = f1[1] + f12[1];
    f1[2] = f1[2] + f12[2];
    f2[0] = f2[0] - f12[0];
    f2[1] = f2[1] - f12[1];
    f2[2] = f2[2] - f12[2];
  }
}

/* SRC/exaMD_forces.f90:308-390, exaMD_forces_midpoint_all with noprocs == 1:
 * every block is interior (SRC/exaMD_partitioning.f90:448-451,735-746) and the
 * boundary routine and the comms tests do nothing.  Home blocks run in the
 * interior_blks order, k outer, i inner (SRC/exaMD_partitioning.f90:764-780). */
int exo_forces_midpoint_all(int64_t n, const double *pos, const double box[3],
                            double block_length, double eps, double sigma,
                            double cutoff, double *forces, exo_counts *counts) {
  if (n < 0 || (n > 0 && (!pos || !forces)) || block_length <= 0.0)
    return EXO_ERR_ARG;
  exo_counts cnt = {0, 0, 0};
  exo_grid g;
  int rc = grid_build(&g, n, pos, box, block_length);
  if (rc != EXO_OK) return rc;
  double boxi[3];
  for (int a = 0; a < 3; ++a) boxi[a] = 1.0 / box[a]; /* SRC/exaMD_utils.f90:188 */
  int64_t refs[27];
  for (int k = 1; k <= g.nb[2]; ++k)
    for (int j = 1; j <= g.nb[1]; ++j)
      for (int i = 1; i <= g.nb[0]; ++i) {
        neighrefs(g.nb, i, j, k, refs);
        int64_t home = refs[13];
        int64_t h0 = g.start[home], natm1 = g.start[home + 1] - h0;
        /* local interactions on the home block first (:349-356) */
        if (natm1 > 1)
          for (int64_t a1 = 0; a1 < natm1 - 1; ++a1)
            for (int64_t a2 = a1 + 1; a2 < natm1; ++a2)
              particle_interaction(pos, forces, g.atom[h0 + a1],
                                   g.atom[h0 + a2], box, boxi, eps, sigma,
                                   cutoff, &cnt);
        /* the other 62 block-pair classes (:359-378) */
        for (int pair = 1; pair < 63; ++pair) {
          int64_t b1 = refs[kTable[pair][0] - 1], b2 = refs[kTable[pair][1] - 1];
          int64_t s1 = g.start[b1], m1 = g.start[b1 + 1] - s1;
          int64_t s2 = g.start[b2], m2 = g.start[b2 + 1] - s2;
          if (m1 >= 1 && m2 >= 1)
            for (int64_t a1 = 0; a1 < m1; ++a1)
              for (int64_t a2 = 0; a2 < m2; ++a2)
                particle_interaction(pos, forces, g.atom[s1 + a1],
                                     g.atom[s2 + a2], box, boxi, eps, sigma,
                                     cutoff, &cnt);
        }
      }
  grid_free(&g);
  if (counts) *counts = cnt;
  return EXO_OK;
}
