// gen.cpp -- seeded synthetic inputs (host code).
//
// The reference generates a uniform random gas with rejection of any atom
// closer than PROXIMITY = 1.0 to one already placed, testing the 27 nearby
// blocks through per-block linked lists (SRC/exaMD_input_formats.f90:41-96,
// SRC/exaMD_module.f90:28,173-256); its Random_number stream is never seeded
// (:69).  examd_gen_random keeps that rejection rule with a seeded, portable
// generator (splitmix64) and a caller-chosen minimum distance and region; the
// lattice and velocity generators serve the LJ-liquid workloads.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/examd_gb300.h"

namespace {

struct Rng {  // splitmix64 (Steele, Lea, Flood 2014)
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
  double normal() {  // Box-Muller
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

}  // namespace

extern "C" {

int examd_gen_fcc(int nc, double rho, double* pos, double* L) {
  if (nc < 1 || !(rho > 0) || !pos || !L) return EXAMD_ERR_ARG;
  const double a = std::cbrt(4.0 / rho);
  const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
  int64_t n = 0;
  for (int k = 0; k < nc; ++k)
    for (int j = 0; j < nc; ++j)
      for (int i = 0; i < nc; ++i)
        for (int b = 0; b < 4; ++b) {
          pos[3 * n] = (i + basis[b][0]) * a;
          pos[3 * n + 1] = (j + basis[b][1]) * a;
          pos[3 * n + 2] = (k + basis[b][2]) * a;
          ++n;
        }
  *L = nc * a;
  return EXAMD_OK;
}

int examd_gen_velocities(int64_t n, const int* type, const double* mass, double T, uint64_t seed, double* vel) {
  if (n < 0 || !(T >= 0) || (n > 0 && !vel)) return EXAMD_ERR_ARG;
  if (n == 0) return EXAMD_OK;
  Rng r(seed);
  double P[3] = {0, 0, 0}, M = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double m = mass ? mass[type ? type[i] : 0] : 1.0;
    const double sd = std::sqrt(T / m);
    for (int a = 0; a < 3; ++a) {
      vel[3 * i + a] = sd * r.normal();
      P[a] += m * vel[3 * i + a];
    }
    M += m;
  }
  double ke2 = 0;  // sum m v^2 after removing the centre-of-mass velocity
  for (int64_t i = 0; i < n; ++i) {
    const double m = mass ? mass[type ? type[i] : 0] : 1.0;
    for (int a = 0; a < 3; ++a) {
      vel[3 * i + a] -= P[a] / M;
      ke2 += m * vel[3 * i + a] * vel[3 * i + a];
    }
  }
  const double dof = 3.0 * (double)(n > 1 ? n - 1 : 1);
  if (ke2 > 0) {
    const double f = std::sqrt(T * dof / ke2);
    for (int64_t i = 0; i < 3 * n; ++i) vel[i] *= f;
  }
  return EXAMD_OK;
}

int examd_gen_random(int64_t n, int64_t n_fixed, const double L[3], const double lo[3], const double hi[3],
                     double dmin, uint64_t seed, int64_t max_tries, double* pos) {
  if (n < 0 || n_fixed < 0 || n_fixed > n || !L || !lo || !hi || !pos || dmin < 0 || max_tries < 1)
    return EXAMD_ERR_ARG;
  for (int a = 0; a < 3; ++a)
    if (!(L[a] > 0) || !(lo[a] >= 0) || !(hi[a] <= L[a]) || !(hi[a] > lo[a])) return EXAMD_ERR_ARG;
  // cell grid with edge >= dmin for the proximity test (27 cells, periodic)
  int nb[3];
  for (int a = 0; a < 3; ++a) {
    nb[a] = dmin > 0 ? (int)(L[a] / dmin) : 1;
    if (nb[a] < 1) nb[a] = 1;
    if (nb[a] > 2048) nb[a] = 2048;
  }
  const int64_t ncell = (int64_t)nb[0] * nb[1] * nb[2];
  std::vector<int64_t> head((size_t)ncell, -1), next((size_t)n, -1);
  auto cell = [&](const double* p, int c[3]) {
    for (int a = 0; a < 3; ++a) {
      c[a] = (int)(p[a] / L[a] * nb[a]);
      if (c[a] >= nb[a]) c[a] = nb[a] - 1;
      if (c[a] < 0) c[a] = 0;
    }
    return (int64_t)c[0] + (int64_t)nb[0] * (c[1] + (int64_t)nb[1] * c[2]);
  };
  auto insert = [&](int64_t i) {
    int c[3];
    int64_t k = cell(pos + 3 * i, c);
    next[(size_t)i] = head[(size_t)k];
    head[(size_t)k] = i;
  };
  const double d2min = dmin * dmin;
  auto too_close = [&](const double* p) {
    int c[3];
    cell(p, c);
    const int span[3] = {nb[0] >= 3 ? 1 : 0, nb[1] >= 3 ? 1 : 0, nb[2] >= 3 ? 1 : 0};
    for (int dz = -span[2]; dz <= span[2]; ++dz)
      for (int dy = -span[1]; dy <= span[1]; ++dy)
        for (int dx = -span[0]; dx <= span[0]; ++dx) {
          int q[3] = {(c[0] + dx + nb[0]) % nb[0], (c[1] + dy + nb[1]) % nb[1], (c[2] + dz + nb[2]) % nb[2]};
          for (int64_t j = head[(size_t)(q[0] + (int64_t)nb[0] * (q[1] + (int64_t)nb[1] * q[2]))]; j >= 0;
               j = next[(size_t)j]) {
            double r2 = 0;
            for (int a = 0; a < 3; ++a) {
              double d = pos[3 * j + a] - p[a];
              d -= std::nearbyint(d / L[a]) * L[a];
              r2 += d * d;
            }
            if (r2 < d2min) return true;
          }
        }
    return false;
  };
  for (int64_t i = 0; i < n_fixed; ++i) insert(i);
  Rng r(seed);
  for (int64_t i = n_fixed; i < n; ++i) {
    int64_t t = 0;
    for (; t < max_tries; ++t) {
      double p[3];
      for (int a = 0; a < 3; ++a) {
        p[a] = lo[a] + r.uniform() * (hi[a] - lo[a]);
        if (p[a] >= L[a]) p[a] = 0.0;
      }
      if (dmin > 0 && too_close(p)) continue;
      for (int a = 0; a < 3; ++a) pos[3 * i + a] = p[a];
      insert(i);
      break;
    }
    if (t == max_tries) return EXAMD_ERR_ARG;
  }
  return EXAMD_OK;
}

int examd_gen_jittered_sc(int m, double rho, double jitter, double frac_b, uint64_t seed, double* pos, int* type,
                          double* L) {
  if (m < 1 || !(rho > 0) || jitter < 0 || jitter >= 0.5 || frac_b < 0 || frac_b > 1 || !pos || !L)
    return EXAMD_ERR_ARG;
  const double a = std::cbrt(1.0 / rho);
  Rng r(seed);
  int64_t n = 0;
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        const int g[3] = {i, j, k};
        for (int c = 0; c < 3; ++c) pos[3 * n + c] = (g[c] + 0.5 + jitter * (2.0 * r.uniform() - 1.0)) * a;
        if (type) type[n] = r.uniform() < frac_b ? 1 : 0;
        ++n;
      }
  *L = m * a;
  return EXAMD_OK;
}

}  // extern "C"
