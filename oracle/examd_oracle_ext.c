/*
 * examd_oracle_ext.c -- oracle extensions that the reference does not have.
 *
 * TEST INFRASTRUCTURE ONLY (see examd_oracle.h).  The reference returns no
 * energy (user_func.f90:71 sets e12 = 0), no virial, has a single species
 * (only prmvdw(1,:) is read, user_func.f90:52-59) and no integrator.  These
 * routines add those on top of the same block loops as examd_oracle.c, kept
 * in this separate file so that the restated code stays as the reference has
 * it.  Energy and virial parity are therefore unpinned by construction.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "examd_oracle.h"

double exo_wrap(double x, double L, double Linv) {
  double y = x - floor(x * Linv) * L;
  if (y >= L) y = y - L;
  if (y < 0.0) y = y + L;
  return y;
}

typedef struct {
  int nt;
  const double *eps, *sigma, *rc;
} lj_table;

/* LJ 12-6 for one pair with the reference's operation order
 * (user_func.f90:52-69) plus e12 = 4 eps (d12 - d6) and the pair virial
 * w = r_12 . f_12 = -dg d2. */
static inline int lj_pair(const lj_table *t, int ta, int tb, double dx,
                          double dy, double dz, double d2, double f12[3],
                          double *e12, double *dgo) {
  int k = ta * t->nt + tb;
  double cutoff = t->rc[k];
  if (d2 > cutoff * cutoff) return 1;
  double eps = t->eps[k], sigma = t->sigma[k];
  double eps24 = 24.0 * eps;
  double sig2 = sigma * sigma;
  double d2i = 1.0 / d2;
  double q = sig2 * d2i;
  double d6 = (q * q) * q;
  double d12 = d6 * d6;
  double dg = -((eps24 * (2.0 * d12 - d6)) * d2i);
  f12[0] = dg * dx;
  f12[1] = dg * dy;
  f12[2] = dg * dz;
  *e12 = (4.0 * eps) * (d12 - d6);
  *dgo = dg;
  return 0;
}

typedef struct {
  int nb[3];
  int64_t nblocks;
  int64_t *start, *atom;
} grid_t;

static int build_grid(grid_t *g, int64_t n, const double *pos,
                      const double box[3], double bl) {
  memset(g, 0, sizeof(*g));
  exo_domain_create(box, bl, g->nb);
  for (int a = 0; a < 3; ++a)
    if (g->nb[a] < 5) return EXO_ERR_NB_TOO_SMALL;
  g->nblocks = (int64_t)g->nb[0] * g->nb[1] * g->nb[2];
  g->start = (int64_t *)calloc((size_t)g->nblocks + 1, sizeof(int64_t));
  g->atom = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t *blk = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  if (!g->start || !g->atom || !blk) {
    free(g->start); free(g->atom); free(blk);
    return EXO_ERR_NOMEM;
  }
  for (int64_t i = 0; i < n; ++i) {
    int b[3];
    int num = exo_identify_block(pos + 3 * i, bl, g->nb, b);
    if (num < 0) {
      free(g->start); free(g->atom); free(blk);
      return EXO_ERR_OUTSIDE;
    }
    blk[i] = num - 1;
    g->start[num]++;
  }
  for (int64_t c = 0; c < g->nblocks; ++c) g->start[c + 1] += g->start[c];
  int64_t *fill = (int64_t *)malloc((size_t)g->nblocks * sizeof(int64_t));
  memcpy(fill, g->start, (size_t)g->nblocks * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) g->atom[fill[blk[i]]++] = i;
  free(fill);
  free(blk);
  return EXO_OK;
}

static void refs_of(const int nb[3], int64_t lin, int64_t refs[27]) {
  int i = (int)(lin % nb[0]) + 1;
  int j = (int)((lin / nb[0]) % nb[1]) + 1;
  int k = (int)(lin / ((int64_t)nb[0] * nb[1])) + 1;
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

typedef struct {
  double epot, vir, vir9[9];
  exo_counts cnt;
} acc_t;

static inline void pair_typed(const double *pos, const int *type, double *f,
                              int64_t a1, int64_t a2, const double box[3],
                              const double boxi[3], const lj_table *t,
                              acc_t *acc, int want9) {
  const double *p1 = pos + 3 * a1, *p2 = pos + 3 * a2;
  double dx = p2[0] - p1[0], dy = p2[1] - p1[1], dz = p2[2] - p1[2];
  double bt0 = (double)llround(dx * boxi[0]);
  double bt1 = (double)llround(dy * boxi[1]);
  double bt2 = (double)llround(dz * boxi[2]);
  dx = dx - bt0 * box[0];
  dy = dy - bt1 * box[1];
  dz = dz - bt2 * box[2];
  double d2 = dx * dx + dy * dy + dz * dz;
  acc->cnt.candidates++;
  if (fabs(d2) < 0.001) acc->cnt.zero_d2++;
  double f12[3], e12, dg;
  int ta = type ? type[a1] : 0, tb = type ? type[a2] : 0;
  if (lj_pair(t, ta, tb, dx, dy, dz, d2, f12, &e12, &dg) == 0) {
    acc->cnt.accepted++;
    double *f1 = f + 3 * a1, *f2 = f + 3 * a2;
    f1[0] += f12[0]; f1[1] += f12[1]; f1[2] += f12[2];
    f2[0] -= f12[0]; f2[1] -= f12[1]; f2[2] -= f12[2];
    acc->epot += e12;
    acc->vir += -dg * d2;
    if (want9) {
      double d[3] = {dx, dy, dz};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) acc->vir9[3 * a + b] += -(d[a] * f12[b]);
    }
  }
}

/* The block loops of exo_forces_midpoint_all for one home block. */
static void home_block(const grid_t *g, int64_t lin, const int kt[63][2],
                       const double *pos, const int *type, double *f,
                       const double box[3], const double boxi[3],
                       const lj_table *t, acc_t *acc, int want9) {
  int64_t refs[27];
  refs_of(g->nb, lin, refs);
  int64_t home = refs[13];
  int64_t h0 = g->start[home], n1 = g->start[home + 1] - h0;
  for (int64_t a1 = 0; a1 + 1 < n1; ++a1)
    for (int64_t a2 = a1 + 1; a2 < n1; ++a2)
      pair_typed(pos, type, f, g->atom[h0 + a1], g->atom[h0 + a2], box, boxi,
                 t, acc, want9);
  for (int p = 1; p < 63; ++p) {
    int64_t b1 = refs[kt[p][0] - 1], b2 = refs[kt[p][1] - 1];
    int64_t s1 = g->start[b1], m1 = g->start[b1 + 1] - s1;
    int64_t s2 = g->start[b2], m2 = g->start[b2 + 1] - s2;
    for (int64_t a1 = 0; a1 < m1; ++a1)
      for (int64_t a2 = 0; a2 < m2; ++a2)
        pair_typed(pos, type, f, g->atom[s1 + a1], g->atom[s2 + a2], box,
                   boxi, t, acc, want9);
  }
}

static int check_types(int64_t n, const int *type, int ntypes) {
  if (ntypes < 1) return EXO_ERR_ARG;
  if (type)
    for (int64_t i = 0; i < n; ++i)
      if (type[i] < 0 || type[i] >= ntypes) return EXO_ERR_ARG;
  return EXO_OK;
}

int exo_forces_typed(int64_t n, const double *pos, const int *type,
                     const double box[3], double bl, int ntypes,
                     const double *eps, const double *sigma, const double *rc,
                     double *forces, double *epot, double *virial,
                     double *virial9, exo_counts *counts) {
  if (check_types(n, type, ntypes) != EXO_OK || bl <= 0.0) return EXO_ERR_ARG;
  int kt[63][2];
  exo_midpoint_table((int *)kt);
  grid_t g;
  int e = build_grid(&g, n, pos, box, bl);
  if (e != EXO_OK) return e;
  double boxi[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  lj_table t = {ntypes, eps, sigma, rc};
  acc_t acc;
  memset(&acc, 0, sizeof(acc));
  for (int64_t lin = 0; lin < g.nblocks; ++lin)
    home_block(&g, lin, (const int(*)[2])kt, pos, type, forces, box, boxi, &t,
               &acc, virial9 != NULL);
  free(g.start);
  free(g.atom);
  if (epot) *epot = acc.epot;
  if (virial) *virial = acc.vir;
  if (virial9) memcpy(virial9, acc.vir9, sizeof(acc.vir9));
  if (counts) *counts = acc.cnt;
  return EXO_OK;
}

int exo_forces_typed_omp(int64_t n, const double *pos, const int *type,
                         const double box[3], double bl, int ntypes,
                         const double *eps, const double *sigma,
                         const double *rc, double *forces, double *epot,
                         double *virial, int nthreads, exo_counts *counts) {
  if (check_types(n, type, ntypes) != EXO_OK || bl <= 0.0) return EXO_ERR_ARG;
  int kt[63][2];
  exo_midpoint_table((int *)kt);
  grid_t g;
  int e = build_grid(&g, n, pos, box, bl);
  if (e != EXO_OK) return e;
  double boxi[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  lj_table t = {ntypes, eps, sigma, rc};
  int nt = 1;
#ifdef _OPENMP
  nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
  double *buf = (double *)calloc((size_t)nt * 3 * (size_t)(n > 0 ? n : 1), sizeof(double));
  acc_t *accs = (acc_t *)calloc((size_t)nt, sizeof(acc_t));
  if (!buf || !accs) {
    free(buf); free(accs); free(g.start); free(g.atom);
    return EXO_ERR_NOMEM;
  }
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *fl = buf + (size_t)tid * 3 * (size_t)n;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int64_t lin = 0; lin < g.nblocks; ++lin)
      home_block(&g, lin, (const int(*)[2])kt, pos, type, fl, box, boxi, &t,
                 &accs[tid], 0);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int64_t i = 0; i < 3 * n; ++i) {
      double s = 0.0;
      for (int r = 0; r < nt; ++r) s += buf[(size_t)r * 3 * (size_t)n + i];
      forces[i] += s;
    }
  }
  acc_t tot;
  memset(&tot, 0, sizeof(tot));
  for (int r = 0; r < nt; ++r) {
    tot.epot += accs[r].epot;
    tot.vir += accs[r].vir;
    tot.cnt.candidates += accs[r].cnt.candidates;
    tot.cnt.accepted += accs[r].cnt.accepted;
    tot.cnt.zero_d2 += accs[r].cnt.zero_d2;
  }
  free(buf);
  free(accs);
  free(g.start);
  free(g.atom);
  if (epot) *epot = tot.epot;
  if (virial) *virial = tot.vir;
  if (counts) *counts = tot.cnt;
  return EXO_OK;
}

int exo_forces_bruteforce(int64_t n, const double *pos, const int *type,
                          const double box[3], int ntypes, const double *eps,
                          const double *sigma, const double *rc,
                          double *forces, double *epot, double *virial) {
  if (check_types(n, type, ntypes) != EXO_OK) return EXO_ERR_ARG;
  double boxi[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  lj_table t = {ntypes, eps, sigma, rc};
  acc_t acc;
  memset(&acc, 0, sizeof(acc));
  for (int64_t a = 0; a < n; ++a)
    for (int64_t b = a + 1; b < n; ++b)
      pair_typed(pos, type, forces, a, b, box, boxi, &t, &acc, 0);
  if (epot) *epot = acc.epot;
  if (virial) *virial = acc.vir;
  return EXO_OK;
}

int exo_vv_run(int64_t n, double *pos, double *vel, const int *type,
               const double *mass, const double box[3], double bl, int ntypes,
               const double *eps, const double *sigma, const double *rc,
               double dt, int nsteps, int nthreads, double *forces,
               double *energies) {
  double Li[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  double hdt = 0.5 * dt;
  for (int s = 0; s < nsteps; ++s) {
    for (int64_t i = 0; i < n; ++i) {
      double im = 1.0 / (mass ? mass[type ? type[i] : 0] : 1.0);
      for (int a = 0; a < 3; ++a) {
        double v = vel[3 * i + a] + (hdt * im) * forces[3 * i + a];
        vel[3 * i + a] = v;
        pos[3 * i + a] = exo_wrap(pos[3 * i + a] + dt * v, box[a], Li[a]);
      }
    }
    memset(forces, 0, sizeof(double) * 3 * (size_t)n);
    double ep = 0.0, w = 0.0;
    int e = (nthreads == 1)
                ? exo_forces_typed(n, pos, type, box, bl, ntypes, eps, sigma,
                                   rc, forces, &ep, &w, NULL, NULL)
                : exo_forces_typed_omp(n, pos, type, box, bl, ntypes, eps,
                                       sigma, rc, forces, &ep, &w, nthreads,
                                       NULL);
    if (e != EXO_OK) return e;
    double ek = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      double m = mass ? mass[type ? type[i] : 0] : 1.0;
      double im = 1.0 / m;
      double v2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        double v = vel[3 * i + a] + (hdt * im) * forces[3 * i + a];
        vel[3 * i + a] = v;
        v2 += v * v;
      }
      ek += 0.5 * m * v2;
    }
    if (energies) {
      energies[2 * s] = ek;
      energies[2 * s + 1] = ep;
    }
  }
  return EXO_OK;
}
