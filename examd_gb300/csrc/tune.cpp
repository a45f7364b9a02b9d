// tune.cpp -- the cell edge, tile shape and CTA width of the pair kernel,
// picked per system by timing.
//
// The reference has no counterpart: its work decomposition is the METIS
// partition of the block graph (SRC/exaMD_partitioning.f90), fixed by the
// process count, and its block edge is a parameter (exaMD_domain_create,
// SRC/exaMD_utils.f90:167-190) that the driver sets to rc/2 (exaMD.f90:56).
// Here the unit of work is a CTA tile of home cells; its
// shape (cubes of 3-6 cells, cubes stretched by one cell on one or two axes,
// and a few stretched by two along x) trades halo overhead against shared memory per CTA and CTAs per SM,
// and the warps per CTA trade latency hiding against tail imbalance.  Where
// a box's last cell on some axis is at least about 1.5 edges wide (it
// absorbs the box's remainder), each shape is also tried with the tiles split
// by width (examd_params.tile_balance = 1): the tile that holds that cell has
// one cell fewer, which shrinks the largest tile and so the shared memory of
// every CTA, at the price of a few more tiles.  The cell edge is then tried
// at 1.1 and 1.2 times the reference's rc/2 with the four fastest
// configurations: a larger edge puts more atoms in a cell (more candidate
// pairs per atom, fewer cells and tile halos); anything at or above rc/2
// keeps the 63-entry table exact, and a smaller one would break it.
//
// Each candidate gets its own context on the caller's atoms; the pair kernel
// is timed with CUDA events (one warm-up launch, then kReps launches; in
// pair-list mode the kernel that computes the forces from the lists, which
// runs at every step, while the build runs only at the steps that rebuild).
// With pair lists the reference's edge is (rc + skin) / 2, and a candidate's
// score adds a fifth of the time of a rebuild of its cells and lists.  A
// candidate that does not fit (capacity, memory, fewer than 5 cells on an
// axis) is skipped.  Choices can be kept in a text cache keyed by device,
// precision, types, cutoff, box count, atom count and density.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/examd_gb300.h"

namespace {

constexpr int kReps = 3;
// pair-list mode: steps per rebuild assumed in the score (a thermal liquid at
// a skin of 0.3 sigma and the usual time steps rebuilds every 4 to 9 steps)
constexpr double kStepsPerBuild = 5.0;

std::string cache_key(const examd_params& p, int nboxes, const examd_box* boxes, int64_t n) {
  cudaDeviceProp pr;
  std::string dev = "unknown";
  if (cudaGetDeviceProperties(&pr, p.device) == cudaSuccess)
    dev = std::string(pr.name) + "/" + std::to_string(pr.multiProcessorCount);
  for (char& c : dev)
    if (c == ' ') c = '_';
  double vol = 0.0, rcmax = 0.0;
  for (int b = 0; b < nboxes; ++b) vol += boxes[b].L[0] * boxes[b].L[1] * boxes[b].L[2];
  for (int k = 0; k < p.ntypes * p.ntypes; ++k) rcmax = std::fmax(rcmax, p.rc[k]);
  char buf[256];
  // atom count in quarter-octaves, density to 0.05; "ce": choices that include the cell edge; the pair
  // lists' skin
  std::snprintf(buf, sizeof buf, "%s|%s|nt%d|rc%.4g|boxes%d|n%.2f|rho%.2f|ce|sk%.4g", dev.c_str(),
                p.precision == EXAMD_FP64 ? "fp64" : "mixed", p.ntypes, rcmax, nboxes,
                std::round(std::log2((double)(n > 0 ? n : 1)) * 4.0) / 4.0, std::round(n / vol * 20.0) / 20.0,
                p.pair_skin);
  return buf;
}

bool cache_lookup(const char* path, const std::string& key, int tile[3], int* warps, int* balance, double* edge,
                  double* ms) {
  if (!path) return false;
  std::FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[512];
  bool hit = false;
  while (std::fgets(line, sizeof line, f)) {
    char* sep = std::strrchr(line, '|');
    if (!sep || (size_t)(sep - line) != key.size() || std::strncmp(line, key.c_str(), key.size()) != 0) continue;
    int t0, t1, t2, w, tb;
    double m, ce;
    if (std::sscanf(sep + 1, "%d %d %d %d %lf %d %lf", &t0, &t1, &t2, &w, &m, &tb, &ce) == 7 &&
        (tb == 0 || tb == 1) && ce >= 0.0) {
      tile[0] = t0;
      tile[1] = t1;
      tile[2] = t2;
      *warps = w;
      *balance = tb;
      *edge = ce;
      *ms = m;
      hit = true;  // the last entry wins
    }
  }
  std::fclose(f);
  return hit;
}

// The key's fields are joined by '|'; the choice follows the last '|'.
void cache_store(const char* path, const std::string& key, const int tile[3], int warps, int balance, double edge,
                 double ms) {
  if (!path) return;
  std::FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s|%d %d %d %d %.17g %d %.17g\n", key.c_str(), tile[0], tile[1], tile[2], warps, ms, balance,
               edge);
  std::fclose(f);
}

// Whether some box has a last cell of about 1.5 edges or more on some axis
// (the cell edge before its rounding to 14 significant bits, which moves it
// by less than 1e-4 of itself; the margin covers that).
bool has_wide_cell(const examd_params& p, int nboxes, const examd_box* boxes) {
  double rcmax = 0.0;
  for (int k = 0; k < p.ntypes * p.ntypes; ++k) rcmax = std::fmax(rcmax, p.rc[k]);
  const double bl = p.cell_edge > 0 ? p.cell_edge : 0.5 * (rcmax + p.pair_skin);
  if (!(bl > 0)) return false;
  for (int b = 0; b < nboxes; ++b)
    for (int a = 0; a < 3; ++a) {
      const double q = boxes[b].L[a] / bl;
      if (q - std::floor(q) >= 0.45) return true;
    }
  return false;
}

}  // namespace

extern "C" int examd_autotune(const examd_params* params, int nboxes, const examd_box* boxes, int64_t n,
                              const double* pos, const int* type, const char* cache_path, examd_params* best,
                              double* best_ms) {
  if (!params || !boxes || nboxes < 1 || n < 0 || (n > 0 && !pos) || !best) return EXAMD_ERR_ARG;
  const std::string key = cache_key(*params, nboxes, boxes, n);
  examd_params out = *params;
  double ms = 0.0;
  if (cache_lookup(cache_path, key, out.tile, &out.warps, &out.tile_balance, &out.cell_edge, &ms)) {
    *best = out;
    if (best_ms) *best_ms = ms;
    return EXAMD_OK;
  }
  const int shapes[][3] = {{3, 3, 3}, {4, 3, 3}, {4, 4, 3}, {4, 4, 4}, {5, 4, 4}, {6, 4, 4}, {5, 5, 4},
                           {6, 5, 4}, {5, 5, 5}, {6, 5, 5}, {6, 6, 5}, {6, 6, 6}};
  const int widths[] = {8, 4};
  const int nbal = has_wide_cell(*params, nboxes, boxes) ? 2 : 1;
  int last_rc = EXAMD_ERR_CELL_OVERFLOW;
  struct Cand {
    examd_params p;
    double t;
  };
  std::vector<Cand> done;
  // one candidate: its own context on the caller's atoms, kReps timed launches
  auto time_one = [&](const examd_params& p, double* t) {
    examd_ctx* ctx = nullptr;
    int rc = examd_gpu_create(&p, nboxes, boxes, &ctx);
    if (rc == EXAMD_OK) rc = examd_gpu_set_atoms(ctx, n, pos, type, nullptr);
    if (rc == EXAMD_OK) rc = examd_gpu_time_forces(ctx, kReps, nullptr, t);
    if (rc == EXAMD_OK && p.pair_skin > 0.0) {  // the score: a step's share of a rebuild too
      double tb = 0.0;
      rc = examd_gpu_time_rebuild(ctx, 2, &tb);
      *t += tb / kStepsPerBuild;
    }
    if (ctx) examd_gpu_destroy(ctx);
    return rc;
  };
  for (int tb = 0; tb < nbal; ++tb)
    for (const auto& sh : shapes)
      for (int w : widths) {
        examd_params p = *params;
        for (int a = 0; a < 3; ++a) p.tile[a] = sh[a];
        p.warps = w;
        p.tile_balance = tb;
        double t = 0.0;
        const int rc = time_one(p, &t);
        if (rc == EXAMD_ERR_NO_DEVICE || rc == EXAMD_ERR_ARG || rc == EXAMD_ERR_OUTSIDE) return rc;
        if (rc != EXAMD_OK) {
          last_rc = rc;
          continue;
        }
        done.push_back({p, t});
      }
  if (done.empty()) return last_rc;
  // the cell edge: 1.1 and 1.2 x the caller's edge (rc/2 by default) with the
  // four fastest configurations so far
  std::stable_sort(done.begin(), done.end(), [](const Cand& x, const Cand& y) { return x.t < y.t; });
  double rcmax = 0.0;
  for (int k = 0; k < params->ntypes * params->ntypes; ++k) rcmax = std::fmax(rcmax, params->rc[k]);
  const double edge0 = params->cell_edge > 0 ? params->cell_edge : 0.5 * (rcmax + params->pair_skin);
  const size_t ntop = std::min<size_t>(4, done.size());
  for (double scale : {1.1, 1.2})
    for (size_t k = 0; k < ntop; ++k) {
      examd_params p = done[k].p;
      p.cell_edge = edge0 * scale;
      double t = 0.0;
      const int rc = time_one(p, &t);
      if (rc == EXAMD_ERR_NO_DEVICE) return rc;
      if (rc == EXAMD_OK) done.push_back({p, t});
    }
  const Cand* pick = &done[0];
  for (const Cand& c : done)
    if (c.t < pick->t) pick = &c;
  out = pick->p;
  cache_store(cache_path, key, out.tile, out.warps, out.tile_balance, out.cell_edge, pick->t);
  *best = out;
  if (best_ms) *best_ms = pick->t;
  return EXAMD_OK;
}
