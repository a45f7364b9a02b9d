// api.cu -- the C ABI (include/examd_gb300.h): context, buffers, step
// sequencing, CUDA-graph capture of the step loop.
//
// Host-side counterpart of the reference's setup and driver sequence:
// exaMD_domain_create (SRC/exaMD_utils.f90:167-190), the neighbour-slot and
// midpoint tables (SRC/exaMD_partitioning.f90:783-798,
// SRC/exaMD_module.f90:276-346) and the timed force call (exaMD.f90:241-253).
// The METIS partition of blocks over ranks (SRC/exaMD_partitioning.f90:65-455)
// becomes a fixed partition of cells into CTA tiles.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

using namespace examd;

namespace {

// The 63 (slot_a, slot_b) block-pair classes of the midpoint method, slot =
// (ii+1) + 3(jj+1) + 9(kk+1) + 1 with ii fastest, 14 = home.  This table is
// the ownership rule itself, so it is carried as the same data
// (SRC/exaMD_module.f90:282-344).
const int kMidpointTable[63][2] = {
    {14, 14}, {14, 15}, {14, 16}, {14, 17}, {14, 18}, {14, 19}, {14, 20}, {14, 21}, {14, 22},
    {14, 23}, {14, 24}, {14, 25}, {14, 26}, {14, 27}, {10, 18}, {10, 27}, {11, 17}, {11, 18},
    {11, 25}, {11, 26}, {11, 27}, {12, 16}, {12, 17}, {12, 25}, {13, 15}, {13, 18}, {13, 24},
    {13, 27}, {15, 16}, {15, 19}, {15, 22}, {15, 25}, {16, 21}, {16, 24}, {17, 19}, {17, 20},
    {17, 21}, {18, 19}, {19, 5},  {19, 9},  {20, 5},  {20, 7},  {20, 8},  {20, 9},  {21, 5},
    {21, 7},  {22, 5},  {22, 6},  {22, 9},  {23, 5},  {24, 5},  {24, 4},  {24, 7},  {25, 5},
    {25, 3},  {25, 6},  {26, 5},  {26, 2},  {26, 3},  {27, 1},  {27, 2},  {27, 4},  {27, 5}};

void slot_offset(int s, int o[3]) {  // SRC/exaMD_partitioning.f90:786-795
  s -= 1;
  o[0] = s % 3 - 1;
  o[1] = (s / 3) % 3 - 1;
  o[2] = s / 9 - 1;
}

bool class_ok(int cls, int h) {  // home offset h keeps the home cell inside the tile
  switch (cls) {
    case 0: return h == 1;   // halo cell before the tile
    case 1: return h >= 0;   // first cell
    case 2: return true;     // interior
    case 3: return h <= 0;   // last cell
    default: return h == -1; // halo cell after the tile
  }
}

// Derive the row structure and the per-class ownership masks from the table.
// Returns false if the table does not have the expected shape.
bool build_own_lut(OwnLut& L) {
  std::memset(&L, 0, sizeof(L));
  std::vector<std::pair<int, int>> rows;
  std::map<std::pair<int, int>, std::map<int, std::array<int, 3>>> byrow;
  for (int p = 1; p < 63; ++p) {
    int a[3], b[3];
    slot_offset(kMidpointTable[p][0], a);
    slot_offset(kMidpointTable[p][1], b);
    int d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    auto key = std::make_pair(d[1], d[2]);
    if (!byrow.count(key) && key != std::make_pair(0, 0)) rows.push_back(key);
    if (byrow[key].count(d[0])) return false;  // duplicate separation
    byrow[key][d[0]] = {-a[0], -a[1], -a[2]};  // home = A - slot_a
  }
  if (rows.size() != 12 || byrow.size() != 13) return false;
  rows.push_back({0, 0});
  for (int r = 0; r < kRows; ++r) {
    L.rows[r][0] = (signed char)rows[r].first;
    L.rows[r][1] = (signed char)rows[r].second;
    const auto& m = byrow[rows[r]];
    if (r < 12) {
      if (m.size() != 5) return false;
    } else if (m.size() != 2 || !m.count(1) || !m.count(2)) {
      return false;
    }
  }
  for (int cx = 0; cx < 5; ++cx)
    for (int cy = 0; cy < 5; ++cy)
      for (int cz = 0; cz < 5; ++cz) {
        const int cls = cx * 25 + cy * 5 + cz;
        for (int r = 0; r < kRows; ++r) {
          unsigned mask = 0;
          for (const auto& kv : byrow[rows[r]]) {
            const auto& h = kv.second;
            if (class_ok(cx, h[0]) && class_ok(cy, h[1]) && class_ok(cz, h[2])) mask |= 1u << (kv.first + 2);
          }
          if (r == kRows - 1 && class_ok(cx, 0) && class_ok(cy, 0) && class_ok(cz, 0)) mask |= 1u << 2;
          if (mask) {
            L.lut[cls][L.nrow[cls]] = (unsigned char)mask;  // by position in the class's row list
            L.rlist[cls][L.nrow[cls]++] = (unsigned char)r;
          }
        }
      }
  return true;
}

int round_block_length(double want, double* out, int* q_out, int* k_out) {
  if (!(want > 0.0) || !std::isfinite(want)) return EXAMD_ERR_ARG;
  // largest k with ceil(want * 2^k) < 2^14: c * bl then needs <= 24 bits
  int k = 13 - (int)std::floor(std::log2(want));
  double bl = 0.0;
  for (; k > -60; --k) {
    double q = std::ceil(want * std::ldexp(1.0, k));
    if (q < 16384.0) {
      bl = std::ldexp(q, -k);
      *q_out = (int)q;
      *k_out = k;
      break;
    }
  }
  if (!(bl >= want)) return EXAMD_ERR_ARG;
  *out = bl;  // = q * 2^-k
  return EXAMD_OK;
}

// Split of one box axis of nb cells into tiles of at most tile_len cells (an
// even split: tile_len or tile_len - 1 cells), so that the largest staged
// tile, which sizes shared memory, stays (tile_len + 2)^3 cells; every tile
// keeps >= 2 cells.  balance = 1: a last cell at least 1.5 edges wide (it
// absorbs the remainder of L / edge) counts as two cells in the split, so the
// tile that holds it has one cell fewer.  Writes nt + 1 starts, returns nt.
int split_axis(int nb, double last_width, int tile_len, int balance, int* starts) {
  const int nv = nb + (balance == 1 && last_width >= 1.5 ? 1 : 0);
  const int nt = std::max(1, std::min(nb / 2, (nv + tile_len - 1) / tile_len));
  for (int k = 0; k < nt; ++k) starts[k] = (int)((int64_t)k * nv / nt);
  starts[nt] = nb;
  if (nt > 1 && starts[nt] - starts[nt - 1] < 2)  // keep >= 2 cells: the even split
    for (int k = 0; k <= nt; ++k) starts[k] = (int)((int64_t)k * nb / nt);
  return nt;
}

}  // namespace

int examd_tile_split(int nb, double last_width, int tile_len, int tile_balance, int* starts, int* nt) {
  if (!starts || !nt || nb < 1 || nb >= 1024 || tile_len < 1 || tile_balance < 0 || tile_balance > 1 ||
      !(last_width >= 1.0) || !(last_width < 2.0))
    return EXAMD_ERR_ARG;
  *nt = split_axis(nb, last_width, tile_len, tile_balance, starts);
  return EXAMD_OK;
}

constexpr int kIoChunks = 4;            // host <-> device transfers of the force call, in chunks
constexpr int64_t kIoMinChunk = 1 << 16;  // atoms; smaller calls use fewer chunks

struct examd_ctx {
  examd_params p{};
  int nboxes = 0;
  std::vector<examd_box> boxes;
  std::vector<BoxDev> bh;
  std::vector<int> tile0;  // nboxes + 1
  std::vector<int64_t> atom0;
  int64_t N = 0;
  int NC = 0, ntiles = 0, ne_max = 0, ext_max = 0;
  double bl = 0.0;
  LJTable lj{};
  PairConfig pc;
  int cap = 0, smem = 0, smem_limit = 0;
  int cap_redo = 0;     // mixed form: staged-atom capacity of the redo pass
  int pair_tables = 0;  // examd_params.pair_tables
  int dev = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
  std::string lasterr;

  // device buffers
  BoxDev* d_boxes = nullptr;
  int4* d_tiles = nullptr;
  int* d_order = nullptr;  // pair-kernel launch order of the tiles
  int* d_tile0 = nullptr;
  unsigned char* d_bmask = nullptr;
  double* X[2][3] = {};
  double* V[2][3] = {};
  int* meta[2] = {};
  int* id[2] = {};
  int cur = 0;
  float4* U = nullptr;
  int* cellS = nullptr;
  int* cellOld = nullptr;
  int* slot = nullptr;
  int* count = nullptr;
  int* cstart = nullptr;
  int* bsum = nullptr;
  void* Fown = nullptr;
  void* P = nullptr;
  double* tileE = nullptr;
  double* tileW = nullptr;
  long long* tileC = nullptr;
  int* redo = nullptr;  // mixed form: tiles for the redo pass (large pair-force terms)
  int* redo_n = nullptr;  // [0] count, [1] done counter of the redo pass
  double* boxE = nullptr;  // per box (graph chunk: [chunk][nboxes])
  double* boxW = nullptr;
  double* boxKE = nullptr;
  int* status = nullptr;
  int* d_occ = nullptr;
  double* stage = nullptr;   // 3N doubles (AoS I/O)
  double* stage2 = nullptr;  // 3N doubles
  int* d_meta_in = nullptr;
  double* d_factor = nullptr;
  int64_t* d_atom0 = nullptr;
  double* keAtom = nullptr;
  double* partial = nullptr;  // chunk partial sums of the per-box reductions
  int* h_status = nullptr;    // pinned host copy of the status word
  // caller-order I/O in chunks, copies on a second stream
  int* inv = nullptr;         // caller index -> sorted slot
  bool inv_valid = false;     // inv matches the current sorted order
  cudaStream_t st2 = nullptr;
  cudaStream_t stc = nullptr;  // pair-list mode: captures the rebuild into a conditional node's body
  cudaEvent_t ev_io[3 * kIoChunks + 1] = {};
  int maxc_atoms = 1, maxc_tiles = 1;
  int ebuf_steps = 0;

  bool atoms_set = false;
  bool forces_valid = false;  // Fown/P hold F(X[cur])
  bool energy_valid = false;

  // pair-list mode (examd_params.pair_skin > 0): the offsets Ub of the last
  // build, the per-tile lists (lslots staged atoms of lk entries each) and
  // their counts, the staged atoms per tile, the fallback tiles and the list
  // words (ListWord); list_gen counts the reallocations of the lists (a
  // captured graph names one generation)
  bool list = false;
  float disp_thr2 = 0.f;  // rebuild when an atom moved more than this squared
  float4* Ub = nullptr;
  unsigned short* plist = nullptr;
  unsigned short* plraw = nullptr;   // the build's scratch (each atom's entries in staged order)
  unsigned short* plperm = nullptr;  // the staged atoms in the order of their entry counts
  unsigned short* plcnt = nullptr;
  int lk = 0, lslots = 0, list_gen = 0;
  int* lcount = nullptr;
  int* fb = nullptr;
  int* lw = nullptr;
  int* h_lw = nullptr;  // pinned host copy of the list words
  int64_t host_builds = 0;  // builds the host asked for (the device counts the others)

  // graph cache
  cudaGraphExec_t gexec = nullptr;
  int g_parity = -1, g_chunk = 0, g_energy = -1, g_cap = 0, g_list_gen = 0;
  double g_dt = 0.0;
  // the force call at new positions (examd_gpu_forces_at) as a CUDA graph,
  // one per parity of the sort's double buffer, for a caller that passes the
  // same pinned buffers every time (an MD driver's arrays)
  struct IoGraph {
    cudaGraphExec_t exec = nullptr;
    const void *pos = nullptr, *forces = nullptr, *epot = nullptr, *virial = nullptr;
    int accumulate = -1, cap = 0, cap_redo = 0, list_gen = 0;
    bool pack = false;
  } io_graph[2];

  int cuda_fail(cudaError_t e, const char* what) {
    lasterr = std::string(what) + ": " + cudaGetErrorString(e);
    return EXAMD_ERR_CUDA;
  }
};

#define CK(call)                                                    \
  do {                                                              \
    cudaError_t _e = (call);                                        \
    if (_e != cudaSuccess) return ctx->cuda_fail(_e, #call);        \
  } while (0)

namespace {

template <class T>
int dalloc(examd_ctx* ctx, T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    ctx->lasterr = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    *p = nullptr;
    return EXAMD_ERR_NOMEM;
  }
  return EXAMD_OK;
}

void free_all(examd_ctx* ctx) {
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  ctx->gexec = nullptr;
  for (auto& g : ctx->io_graph)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  void* ptrs[] = {ctx->d_boxes, ctx->d_tiles, ctx->d_order, ctx->d_tile0, ctx->d_bmask, ctx->U, ctx->cellS,
                  ctx->cellOld, ctx->slot, ctx->count, ctx->cstart, ctx->bsum,
                  ctx->Fown, ctx->P, ctx->tileE, ctx->tileW, ctx->tileC, ctx->boxE, ctx->boxW, ctx->boxKE,
                  ctx->status, ctx->d_occ, ctx->stage, ctx->stage2, ctx->d_meta_in, ctx->d_factor,
                  ctx->d_atom0, ctx->keAtom, ctx->partial, ctx->redo, ctx->redo_n,
                  ctx->Ub, ctx->plist, ctx->plraw, ctx->plperm, ctx->plcnt, ctx->lcount, ctx->fb, ctx->lw};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  for (int b = 0; b < 2; ++b) {
    for (int a = 0; a < 3; ++a) {
      if (ctx->X[b][a]) cudaFree(ctx->X[b][a]);
      if (ctx->V[b][a]) cudaFree(ctx->V[b][a]);
    }
    if (ctx->meta[b]) cudaFree(ctx->meta[b]);
    if (ctx->id[b]) cudaFree(ctx->id[b]);
  }
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->h_lw) cudaFreeHost(ctx->h_lw);
  if (ctx->inv) cudaFree(ctx->inv);
  for (cudaEvent_t e : ctx->ev_io)
    if (e) cudaEventDestroy(e);
  if (ctx->st2) cudaStreamDestroy(ctx->st2);
  if (ctx->stc) cudaStreamDestroy(ctx->stc);
  if (ctx->e0) cudaEventDestroy(ctx->e0);
  if (ctx->e1) cudaEventDestroy(ctx->e1);
  if (ctx->e2) cudaEventDestroy(ctx->e2);
  if (ctx->e3) cudaEventDestroy(ctx->e3);
  if (ctx->st) cudaStreamDestroy(ctx->st);
}

int status_to_code(int st) {
  if (st & ST_PAIRFN) return EXAMD_ERR_PAIRFN;
  if (st & ST_NONFINITE) return EXAMD_ERR_NONFINITE;
  if (st & ST_OUTSIDE) return EXAMD_ERR_OUTSIDE;
  if (st & ST_OVERFLOW) return EXAMD_ERR_CELL_OVERFLOW;
  if (st & ST_TIMEOUT) return EXAMD_ERR_TIMEOUT;
  if (st & ST_BOUNDS) return EXAMD_ERR_CHECK;
  return EXAMD_OK;
}

// Largest staged-atom count of any tile (ext cells), for the smem capacity.
__global__ void k_tile_occupancy(const int4* __restrict__ tiles, const BoxDev* __restrict__ boxes,
                                 const int* __restrict__ cstart, int* __restrict__ occ) {
  __shared__ int part[32];
  const int tile = blockIdx.x;
  const int4 t0 = tiles[2 * tile], t1 = tiles[2 * tile + 1];
  const BoxDev& B = boxes[t0.x];
  const int EX = t1.x + 2, EY = t1.y + 2, EZ = t1.z + 2, NE = EX * EY * EZ;
  int s = 0;
  for (int e = threadIdx.x; e < NE; e += blockDim.x) {
    int lx = e % EX, rr = e / EX, ly = rr % EY, lz = rr / EY;
    int g[3] = {t0.y + lx - 1, t0.z + ly - 1, t0.w + lz - 1};
    for (int a = 0; a < 3; ++a) {
      if (g[a] < 0) g[a] += B.nb[a];
      if (g[a] >= B.nb[a]) g[a] -= B.nb[a];
    }
    int gc = B.cell0 + g[0] + B.nb[0] * (g[1] + B.nb[1] * g[2]);
    s += cstart[gc + 1] - cstart[gc];
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    atomicMax(&occ[0], t);
  }
}

}  // namespace

// --------------------------------------------------------------------------
extern "C" {

void examd_default_params(examd_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->precision = EXAMD_FP64;
  p->ntypes = 1;
  p->eps[0] = 1.0;
  p->sigma[0] = 1.0;
  p->rc[0] = 2.5;
  p->mass[0] = 1.0;
}

const char* examd_gpu_strerror(int code) {
  switch (code) {
    case EXAMD_OK: return "ok";
    case EXAMD_ERR_OUTSIDE: return "position outside the box (block number out of range)";
    case EXAMD_ERR_ARG: return "invalid argument or parameter";
    case EXAMD_ERR_NB_TOO_SMALL: return "fewer than 5 cells on an axis: the 63-entry table would count pairs twice";
    case EXAMD_ERR_CELL_OVERFLOW: return "a tile holds more atoms than its shared-memory capacity";
    case EXAMD_ERR_NONFINITE: return "non-finite position";
    case EXAMD_ERR_TIMEOUT: return "a bounded device wait gave up";
    case EXAMD_ERR_CUDA: return "CUDA runtime error";
    case EXAMD_ERR_NOMEM: return "out of device or pinned memory";
    case EXAMD_ERR_STATE: return "invalid call order";
    case EXAMD_ERR_NO_DEVICE: return "no usable sm_103 CUDA device";
    case EXAMD_ERR_IO: return "file missing, unreadable or malformed";
    case EXAMD_ERR_PAIRFN: return "the pair function returned an error (e.g. coincident atoms)";
    case EXAMD_ERR_CHECK: return "an index check of the checked build failed";
    default: return "unknown status";
  }
}

const char* examd_gpu_last_error(examd_ctx* ctx) { return ctx ? ctx->lasterr.c_str() : ""; }

int examd_own_table(signed char* rows, unsigned char* lut) {
  if (!rows || !lut) return EXAMD_ERR_ARG;
  OwnLut L;
  if (!build_own_lut(L)) return EXAMD_ERR_ARG;
  std::memcpy(rows, L.rows, sizeof(L.rows));
  std::memset(lut, 0, sizeof(L.lut));  // by row, as the header documents it
  for (int c = 0; c < kClasses; ++c)
    for (int n = 0; n < L.nrow[c]; ++n) lut[c * kRows + L.rlist[c][n]] = L.lut[c][n];
  return EXAMD_OK;
}

int examd_host_alloc(void** ptr, int64_t bytes) {
  if (!ptr || bytes < 0) return EXAMD_ERR_ARG;
  return cudaHostAlloc(ptr, (size_t)std::max<int64_t>(bytes, 1), cudaHostAllocDefault) == cudaSuccess
             ? EXAMD_OK
             : EXAMD_ERR_NOMEM;
}
int examd_host_free(void* ptr) { return cudaFreeHost(ptr) == cudaSuccess ? EXAMD_OK : EXAMD_ERR_CUDA; }

int examd_gpu_create(const examd_params* params, int nboxes, const examd_box* boxes, examd_ctx** out) {
  if (!params || !boxes || !out || nboxes < 1) return EXAMD_ERR_ARG;
  *out = nullptr;
  const examd_params& p = *params;
  if (p.ntypes < 1 || p.ntypes > EXAMD_MAX_TYPES) return EXAMD_ERR_ARG;
  if (p.precision != EXAMD_FP64 && p.precision != EXAMD_MIXED) return EXAMD_ERR_ARG;
  if (p.potential < EXAMD_POT_LJ || p.potential > EXAMD_POT_WCA) return EXAMD_ERR_ARG;
  const int nt = p.ntypes;
  double rcmax = 0.0;
  for (int a = 0; a < nt; ++a)
    for (int b = 0; b < nt; ++b) {
      const int k = a * nt + b, kt = b * nt + a;
      if (!(p.eps[k] > 0) || !(p.sigma[k] > 0) || !(p.rc[k] > 0)) return EXAMD_ERR_ARG;
      if (p.eps[k] != p.eps[kt] || p.sigma[k] != p.sigma[kt] || p.rc[k] != p.rc[kt]) return EXAMD_ERR_ARG;
      rcmax = std::max(rcmax, p.rc[k]);
    }
  // pair-list mode: the cells must hold every pair within rc + skin in the
  // 63-entry table's reach, so their edge is at least (rc + skin) / 2
  const double skin = p.pair_skin;
  if (!(skin >= 0.0) || !std::isfinite(skin) || (skin > 0.0 && p.precision != EXAMD_MIXED)) return EXAMD_ERR_ARG;
  if (skin > 0.0 && skin < 1e-3) return EXAMD_ERR_ARG;  // below the displacement test's margin
  if (p.pair_list_capacity < 0 || p.pair_list_capacity > 1024 || p.pair_list_capacity % 8 != 0) return EXAMD_ERR_ARG;
  const double reach = rcmax + skin;
  double want = p.cell_edge > 0 ? p.cell_edge : 0.5 * reach;
  if (want < 0.5 * reach) return EXAMD_ERR_ARG;
  double bl;
  int blq = 0, blk = 0;
  if (round_block_length(want, &bl, &blq, &blk) != EXAMD_OK) return EXAMD_ERR_ARG;

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1 || p.device < 0 || p.device >= ndev)
    return EXAMD_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, p.device) != cudaSuccess) return EXAMD_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return EXAMD_ERR_NO_DEVICE;  // built for sm_103a only

  examd_ctx* ctx = new examd_ctx();
  ctx->p = p;
  ctx->nboxes = nboxes;
  ctx->boxes.assign(boxes, boxes + nboxes);
  ctx->bl = bl;
  ctx->dev = p.device;
  ctx->smem_limit = (int)prop.sharedMemPerBlockOptin;
  cudaSetDevice(ctx->dev);

  // pair-kernel configuration
  ctx->pc.fp64 = p.precision == EXAMD_FP64;
  ctx->pc.multi = nt > 1;
  ctx->pc.cut = p.potential == EXAMD_POT_WCA;
  ctx->pc.pack = p.pair_tables == 2;
  ctx->pair_tables = p.pair_tables;
  if (p.pair_tables < 0 || p.pair_tables > 2 || p.tile_balance < 0 || p.tile_balance > 1) {
    delete ctx;
    return EXAMD_ERR_ARG;
  }
  ctx->list = skin > 0.0;
  ctx->pc.list = ctx->list;
  // an atom that moved d since the build is tested in FP32 against skin/2
  // less a margin of 1e-4 that covers the offsets' rounding many times over
  ctx->disp_thr2 = ctx->list ? (float)((0.5 * skin - 1e-4) * (0.5 * skin - 1e-4)) : 0.f;
  ctx->pc.warps = p.warps > 0 ? p.warps : 8;
  if (ctx->pc.warps < 4 || ctx->pc.warps > 8) {
    delete ctx;
    return EXAMD_ERR_ARG;
  }
  const int deftile = 4;
  int T[3];
  for (int a = 0; a < 3; ++a) {
    T[a] = p.tile[a] > 0 ? p.tile[a] : deftile;
    if (T[a] < 2 || T[a] > 14) {
      delete ctx;
      return EXAMD_ERR_ARG;
    }
  }

  // LJ tables
  LJTable& lj = ctx->lj;
  lj.nt = nt;
  float rc2max = 0.f;
  lj.pot = p.potential;
  for (int k = 0; k < nt * nt; ++k) {
    const double e = p.eps[k], s = p.sigma[k], r = p.rc[k];
    lj.p64[k].sig2 = s * s;      // sig2 = prmvdw(1,2)**2   (user_func.f90:59)
    lj.p64[k].eps24 = 24.0 * e;  // eps24 = twentyfour*eps  (user_func.f90:58)
    lj.p64[k].eps4 = 4.0 * e;
    lj.p64[k].rc2 = r * r;       // prmvdw(1,5)**2           (user_func.f90:52)
    // the potential's own range and energy shift
    double rcut2 = r * r, eshift = 0.0;
    if (p.potential == EXAMD_POT_LJ_SHIFTED) {
      const double s6 = std::pow(s * s / (r * r), 3);
      eshift = 4.0 * e * s6 * (s6 - 1.0);
    } else if (p.potential == EXAMD_POT_WCA) {
      rcut2 = std::cbrt(2.0) * s * s;  // (2^(1/6) sigma)^2
      eshift = -e;                     // U(2^(1/6) sigma) = -eps
      if (rcut2 > r * r) {  // rc must cover the potential's range
        delete ctx;
        return EXAMD_ERR_ARG;
      }
    }
    lj.p64[k].rcut2 = rcut2;
    lj.p64[k].eshift = eshift;
    lj.p32[k].sig2 = (float)(s * s);
    lj.p32[k].m24eps = (float)(-24.0 * e);
    lj.p32[k].c4eps = (float)(4.0 * e);
    lj.p32[k].rc2 = (float)(r * r);
    // the mixed form's own range test only where the potential ends inside
    // rc (WCA); for the LJ forms the range is rc itself, which the candidate
    // test decides, in FP64 at the border (an FP32 re-test there would drop
    // a pair that the FP64 form applies)
    lj.p32[k].rcut2 = p.potential == EXAMD_POT_WCA ? (float)rcut2 : INFINITY;
    lj.p32[k].eshift = (float)eshift;
    lj.p32[k].rl2 = (float)((r + skin) * (r + skin));
    {
      // |F(r)| = 24 eps (2 s^12 - s^6) / r, s = sigma / r, falls monotonically
      // from r -> 0 to its zero at 2^(1/6) sigma: bisect for |F| = kFixMaxForce,
      // then widen by 1e-4 (the FP32 d2 of a pair and the FP32 force differ
      // from the exact ones by far less)
      auto fmag = [&](double rr) {
        const double s6 = std::pow(s / rr, 6.0);
        return 24.0 * e * (2.0 * s6 * s6 - s6) / rr;
      };
      double lo = 1e-3 * s, hi = std::pow(2.0, 1.0 / 6.0) * s;
      if (!(fmag(lo) > kFixMaxForce)) {
        hi = lo;
      } else {
        for (int it = 0; it < 200; ++it) {
          const double mid = 0.5 * (lo + hi);
          (fmag(mid) > kFixMaxForce ? lo : hi) = mid;
        }
      }
      lj.p32[k].r2big = (float)(hi * hi * (1.0 + 1e-4));
    }
    rc2max = std::max(rc2max, lj.p32[k].rc2);
  }
  lj.rc2max = rc2max;
  // pair-list mode: atoms may be up to skin/2 outside the cells they were
  // sorted into, so an enumeration between builds prunes at rc + skin/2
  const double reach_now = rcmax + 0.5 * skin + 1e-4;
  lj.prune2 = (float)(reach_now * reach_now);
  lj.prune2_list = (float)((reach + 1e-4) * (reach + 1e-4));
  for (int a = 0; a < EXAMD_MAX_TYPES; ++a) {
    double m = (a < nt && p.mass[a] > 0) ? p.mass[a] : 1.0;
    lj.mass[a] = m;
    lj.minv[a] = 1.0 / m;
  }

  // Tiles of a batch: the tile edge T is the densest box's.  A box with fewer
  // atoms per cell gets tiles up to 2 cells longer per axis, as long as its
  // expected staged atoms, (T + 2 + g)^3 per cell times its atoms per cell,
  // stay within the densest box's (the largest tile sizes shared memory for
  // the whole launch): fewer halo cells per home cell, the same footprint.
  double dens_max = 0.0;
  std::vector<double> dens(nboxes, 0.0);
  for (int b = 0; b < nboxes; ++b) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) cells *= std::max(1.0, std::floor(boxes[b].L[a] / bl));
    dens[b] = (double)boxes[b].natoms / cells;
    dens_max = std::max(dens_max, dens[b]);
  }

  // boxes, cells, tiles
  std::vector<int4> tiles;
  std::vector<unsigned char> bmask;
  int cell0 = 0;
  int64_t a0 = 0;
  for (int b = 0; b < nboxes; ++b) {
    const examd_box& X = boxes[b];
    BoxDev B{};
    if (X.natoms < 0) {
      delete ctx;
      return EXAMD_ERR_ARG;
    }
    for (int a = 0; a < 3; ++a) {
      if (!(X.L[a] > 0) || !std::isfinite(X.L[a])) {
        delete ctx;
        return EXAMD_ERR_ARG;
      }
      B.L[a] = X.L[a];
      B.Li[a] = 1.0 / X.L[a];  // globalboxi = one/globalbox (SRC/exaMD_utils.f90:188)
      B.Lf[a] = (float)X.L[a];
      double q = X.L[a] / bl;  // nblocks_xyz = Int(globalbox/block_length) (:179)
      if (q < 5.0) {
        delete ctx;
        return EXAMD_ERR_NB_TOO_SMALL;
      }
      if (q >= 1024.0) {
        delete ctx;
        return EXAMD_ERR_ARG;
      }
      B.nb[a] = (int)q;
    }
    B.bl = bl;
    B.bli = 1.0 / bl;
    B.blq = blq;
    B.blk = blk;
    for (int a = 0; a < 3; ++a) B.remf[a] = (float)(B.L[a] - B.nb[a] * bl);  // nb*bl is exact
    B.blf = (float)bl;
    B.blif = (float)(1.0 / bl);
    B.cell0 = cell0;
    B.tile0 = (int)tiles.size() / 2;
    int Tb[3] = {T[0], T[1], T[2]};
    for (int g = 2; g > 0 && dens[b] > 0.0; --g) {
      const double grown = (double)(T[0] + 2 + g) * (T[1] + 2 + g) * (T[2] + 2 + g) * dens[b];
      if (grown <= (double)(T[0] + 2) * (T[1] + 2) * (T[2] + 2) * dens_max) {
        for (int a = 0; a < 3; ++a) Tb[a] = T[a] + g;
        break;
      }
    }
    int starts[3][1025];
    for (int a = 0; a < 3; ++a) {
      const double wide = (B.L[a] - (B.nb[a] - 1) * bl) / bl;  // the last cell's width in edges
      B.nt[a] = split_axis(B.nb[a], wide, Tb[a], p.tile_balance, starts[a]);
      for (int k = 0; k < B.nt[a]; ++k)
        if (starts[a][k + 1] - starts[a][k] + 2 > kMaxExt) {
          delete ctx;
          return EXAMD_ERR_ARG;
        }
    }
    ctx->tile0.push_back(B.tile0);
    for (int kz = 0; kz < B.nt[2]; ++kz)
      for (int ky = 0; ky < B.nt[1]; ++ky)
        for (int kx = 0; kx < B.nt[0]; ++kx) {
          int4 d0 = make_int4(b, starts[0][kx], starts[1][ky], starts[2][kz]);
          int4 d1 = make_int4(starts[0][kx + 1] - starts[0][kx], starts[1][ky + 1] - starts[1][ky],
                              starts[2][kz + 1] - starts[2][kz], 0);
          tiles.push_back(d0);
          tiles.push_back(d1);
          ctx->ne_max = std::max(ctx->ne_max, (d1.x + 2) * (d1.y + 2) * (d1.z + 2));
          ctx->ext_max = std::max(ctx->ext_max, std::max(d1.x, std::max(d1.y, d1.z)) + 2);
        }
    // boundary mask per cell: first or last cell of its tile on each axis
    std::vector<unsigned char> edge[3];
    for (int a = 0; a < 3; ++a) {
      edge[a].assign(B.nb[a], 0);
      for (int k = 0; k < B.nt[a]; ++k) {
        edge[a][starts[a][k]] = 1;
        edge[a][starts[a][k + 1] - 1] = 1;
      }
    }
    for (int cz = 0; cz < B.nb[2]; ++cz)
      for (int cy = 0; cy < B.nb[1]; ++cy)
        for (int cx = 0; cx < B.nb[0]; ++cx)
          bmask.push_back((unsigned char)(edge[0][cx] | (edge[1][cy] << 1) | (edge[2][cz] << 2)));
    cell0 += B.nb[0] * B.nb[1] * B.nb[2];
    ctx->atom0.push_back(a0);
    a0 += X.natoms;
    ctx->bh.push_back(B);
  }
  ctx->tile0.push_back((int)tiles.size() / 2);
  ctx->atom0.push_back(a0);
  ctx->N = a0;
  ctx->NC = cell0;
  ctx->ntiles = (int)tiles.size() / 2;
  if (ctx->N >= (int64_t)1 << 31 || (int64_t)cell0 >= ((int64_t)1 << 31) - 1 ||
      (cell0 + kScanTileHost - 1) / kScanTileHost > 8192 || nboxes >= (1 << 23)) {
    delete ctx;
    return EXAMD_ERR_ARG;
  }
  // Launch order of the pair kernel: the tiles by estimated cost, costliest
  // first, so that the grid ends on its cheapest CTAs (longest processing
  // time first; the per-tile outputs keep the tile's index).  The estimate is
  // the tile's staged atoms plus twice its home atoms times the atoms per cell
  // (its pair work), from cell volumes: the last cell of an axis is wider.
  std::vector<int> order(ctx->ntiles);
  {
    std::vector<double> cost(ctx->ntiles);
    for (int t = 0; t < ctx->ntiles; ++t) {
      const int4 d0 = tiles[2 * t], d1 = tiles[2 * t + 1];
      const BoxDev& B = ctx->bh[d0.x];
      const int org[3] = {d0.y, d0.z, d0.w}, len[3] = {d1.x, d1.y, d1.z};
      double vh = 1.0, ve = 1.0;
      for (int a = 0; a < 3; ++a) {
        const double wide = (B.L[a] - (B.nb[a] - 1) * B.bl) / B.bl;  // the last cell's width in cell edges
        double h = 0.0, e = 0.0;
        for (int c = org[a] - 1; c <= org[a] + len[a]; ++c) {
          const int g = (c + B.nb[a]) % B.nb[a];
          const double w = g == B.nb[a] - 1 ? wide : 1.0;
          e += w;
          if (c >= org[a] && c < org[a] + len[a]) h += w;
        }
        vh *= h;
        ve *= e;
      }
      const double n = (double)boxes[d0.x].natoms * B.bl * B.bl * B.bl / (B.L[0] * B.L[1] * B.L[2]);
      cost[t] = n * (ve + 2.0 * vh * n);
    }
    for (int t = 0; t < ctx->ntiles; ++t) order[t] = t;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  }

  OwnLut lut;
  if (!build_own_lut(lut)) {
    delete ctx;
    return EXAMD_ERR_ARG;
  }
  int rc = EXAMD_OK;
#define ALLOC(ptr, cnt)                                   \
  do {                                                    \
    if ((rc = dalloc(ctx, &(ptr), (cnt))) != EXAMD_OK) {  \
      free_all(ctx);                                      \
      delete ctx;                                         \
      return rc;                                          \
    }                                                     \
  } while (0)
  if (upload_own_lut(lut) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&ctx->e0) != cudaSuccess || cudaEventCreate(&ctx->e1) != cudaSuccess ||
      cudaEventCreate(&ctx->e2) != cudaSuccess || cudaEventCreate(&ctx->e3) != cudaSuccess) {
    free_all(ctx);
    delete ctx;
    return EXAMD_ERR_CUDA;
  }
  if (cudaHostAlloc((void**)&ctx->h_status, sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
    ctx->h_status = nullptr;
    free_all(ctx);
    delete ctx;
    return EXAMD_ERR_NOMEM;
  }
  *ctx->h_status = 0;
  bool io_ok = cudaStreamCreateWithFlags(&ctx->st2, cudaStreamNonBlocking) == cudaSuccess &&
               cudaStreamCreateWithFlags(&ctx->stc, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaEvent_t& e : ctx->ev_io) io_ok = io_ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!io_ok) {
    free_all(ctx);
    delete ctx;
    return EXAMD_ERR_CUDA;
  }
  const size_t N = (size_t)ctx->N, NC = (size_t)ctx->NC;
  ALLOC(ctx->d_boxes, nboxes);
  ALLOC(ctx->d_tiles, tiles.size());
  ALLOC(ctx->d_order, ctx->ntiles);
  ALLOC(ctx->d_tile0, nboxes + 1);
  ALLOC(ctx->d_bmask, NC);
  for (int b = 0; b < 2; ++b) {
    for (int a = 0; a < 3; ++a) {
      ALLOC(ctx->X[b][a], N);
      ALLOC(ctx->V[b][a], N);
    }
    ALLOC(ctx->meta[b], N);
    ALLOC(ctx->id[b], N);
  }
  ALLOC(ctx->U, N);
  ALLOC(ctx->cellS, N);
  ALLOC(ctx->cellOld, N);
  ALLOC(ctx->slot, N);
  ALLOC(ctx->count, NC);
  ALLOC(ctx->cstart, NC + 1);
  ALLOC(ctx->bsum, 8192);
  if (ctx->pc.fp64) {
    double* f;
    ALLOC(f, 3 * N);
    ctx->Fown = f;
    ALLOC(f, 7 * 3 * N);
    ctx->P = f;
  } else {
    float4* f;
    ALLOC(f, N);
    ctx->Fown = f;
    ALLOC(f, 7 * N);
    ctx->P = f;
    ALLOC(ctx->redo, std::max(1, ctx->ntiles));
    ALLOC(ctx->redo_n, 2);
  }
  ALLOC(ctx->tileE, ctx->ntiles);
  ALLOC(ctx->tileW, ctx->ntiles);
  ALLOC(ctx->tileC, 3 * (size_t)ctx->ntiles);
  ALLOC(ctx->boxE, nboxes);
  ALLOC(ctx->boxW, nboxes);
  ALLOC(ctx->boxKE, nboxes);
  ALLOC(ctx->status, 1);
  ALLOC(ctx->d_occ, 2);
  ALLOC(ctx->stage, 3 * N);
  ALLOC(ctx->stage2, 3 * N);
  ALLOC(ctx->d_meta_in, N);
  ALLOC(ctx->d_factor, nboxes);
  ALLOC(ctx->d_atom0, nboxes + 1);
  ALLOC(ctx->keAtom, N);
  ALLOC(ctx->inv, N);
  if (ctx->list) {
    ALLOC(ctx->Ub, N);
    ALLOC(ctx->lcount, ctx->ntiles);
    ALLOC(ctx->fb, ctx->ntiles);
    ALLOC(ctx->lw, LW_WORDS);
    if (cudaHostAlloc((void**)&ctx->h_lw, LW_WORDS * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
      ctx->h_lw = nullptr;
      free_all(ctx);
      delete ctx;
      return EXAMD_ERR_NOMEM;
    }
  }
  {
    int64_t maxa = 1, maxt = 1;
    for (int b = 0; b < nboxes; ++b) {
      maxa = std::max<int64_t>(maxa, ctx->atom0[b + 1] - ctx->atom0[b]);
      maxt = std::max<int64_t>(maxt, ctx->tile0[b + 1] - ctx->tile0[b]);
    }
    ctx->maxc_atoms = red_chunks(maxa);
    ctx->maxc_tiles = red_chunks(maxt);
    ALLOC(ctx->partial, std::max((size_t)nboxes * ctx->maxc_atoms, (size_t)2 * nboxes * ctx->maxc_tiles));
  }
#undef ALLOC
  cudaStream_t st = ctx->st;
  bool ok = cudaMemcpyAsync(ctx->d_boxes, ctx->bh.data(), nboxes * sizeof(BoxDev), cudaMemcpyHostToDevice, st) ==
                cudaSuccess &&
            cudaMemcpyAsync(ctx->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, st) ==
                cudaSuccess &&
            cudaMemcpyAsync(ctx->d_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, st) ==
                cudaSuccess &&
            cudaMemcpyAsync(ctx->d_tile0, ctx->tile0.data(), (nboxes + 1) * sizeof(int), cudaMemcpyHostToDevice,
                            st) == cudaSuccess &&
            cudaMemcpyAsync(ctx->d_bmask, bmask.data(), NC, cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(ctx->d_atom0, ctx->atom0.data(), (nboxes + 1) * sizeof(int64_t),
                            cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemsetAsync(ctx->count, 0, NC * sizeof(int), st) == cudaSuccess &&
            cudaMemsetAsync(ctx->status, 0, sizeof(int), st) == cudaSuccess &&
            (!ctx->redo_n || cudaMemsetAsync(ctx->redo_n, 0, 2 * sizeof(int), st) == cudaSuccess) &&
            (!ctx->lw || cudaMemsetAsync(ctx->lw, 0, LW_WORDS * sizeof(int), st) == cudaSuccess) &&
            cudaStreamSynchronize(st) == cudaSuccess;
  if (!ok) {
    free_all(ctx);
    delete ctx;
    return EXAMD_ERR_CUDA;
  }
  *out = ctx;
  return EXAMD_OK;
}

void examd_gpu_destroy(examd_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->dev);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  free_all(ctx);
  delete ctx;
}

}  // extern "C"

// --------------------------------------------------------------------------
namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

// Scan and final ordering after a counting pass; swaps the buffers.
// want_inv: also record the caller -> sorted map (for the caller-order I/O).
// Pair-list mode: the sorted arrays are copied back into the current buffer
// (a step loop captured as a graph names fixed buffers, and whether a step
// rebuilds is decided on the device), the offsets are kept as the build's
// Ub, the caller map is always recorded, and gate (a device word, or
// nullptr) makes the whole sequence conditional.
int finish_binning(examd_ctx* ctx, bool want_inv, const int* gate = nullptr) {
  cudaStream_t st = ctx->st;
  const int nc = ctx->NC;
  const int nsb = (nc + kScanTileHost - 1) / kScanTileHost;
  const int s = ctx->cur, d = 1 - ctx->cur;
  const bool list = ctx->list;
  if (list) want_inv = true;
  k_scan_reduce<<<nsb, 256, 0, st>>>(nc, ctx->count, ctx->bsum, gate);
  k_scan_final<<<nsb, 256, 0, st>>>(nc, ctx->count, ctx->bsum, ctx->cstart, gate);
  if (ctx->N > 0) {
    k_finalize<<<nblk(ctx->N), 256, 0, st>>>(ctx->N, ctx->cellOld, ctx->slot, ctx->cstart, ctx->d_boxes,
                                              ctx->X[s][0], ctx->X[s][1], ctx->X[s][2], ctx->V[s][0],
                                              ctx->V[s][1], ctx->V[s][2], ctx->meta[s], ctx->id[s],
                                              ctx->X[d][0], ctx->X[d][1], ctx->X[d][2], ctx->V[d][0],
                                              ctx->V[d][1], ctx->V[d][2], ctx->meta[d], ctx->id[d], ctx->U,
                                              list ? ctx->Ub : nullptr, ctx->cellS, want_inv ? ctx->inv : nullptr,
                                              ctx->NC, ctx->status, gate);
    if (list)
      k_copy_back<<<nblk(ctx->N), 256, 0, st>>>(ctx->N, ctx->X[d][0], ctx->X[d][1], ctx->X[d][2], ctx->V[d][0],
                                                 ctx->V[d][1], ctx->V[d][2], ctx->meta[d], ctx->id[d], ctx->X[s][0],
                                                 ctx->X[s][1], ctx->X[s][2], ctx->V[s][0], ctx->V[s][1],
                                                 ctx->V[s][2], ctx->meta[s], ctx->id[s], gate);
  }
  CK(cudaGetLastError());
  if (!list) ctx->cur = d;
  ctx->inv_valid = want_inv;
  return EXAMD_OK;
}

// Chunk c of n atoms for the caller-order I/O: [i0, i1).
int io_chunks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(kIoChunks, n / kIoMinChunk)); }
void io_range(int64_t n, int nch, int c, int64_t& i0, int64_t& i1) {
  i0 = n * c / nch;
  i1 = n * (c + 1) / nch;
}

// The caller -> sorted map of the current order, if the last binning did not
// record it.
cudaError_t ensure_inv(examd_ctx* ctx) {
  if (ctx->inv_valid || ctx->N == 0) return cudaSuccess;
  k_inverse<<<nblk(ctx->N), 256, 0, ctx->st>>>(ctx->N, ctx->id[ctx->cur], ctx->inv);
  ctx->inv_valid = true;
  return cudaGetLastError();
}

// The status word after work already synchronised: its copy to the pinned
// host word was queued before that synchronisation (queue_status).
int take_status(examd_ctx* ctx) {
  const int h = *ctx->h_status;
  if (h) {
    CK(cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  return status_to_code(h);
}

cudaError_t queue_status(examd_ctx* ctx) {
  return cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
}

int check_status(examd_ctx* ctx) {
  CK(queue_status(ctx));
  CK(cudaStreamSynchronize(ctx->st));
  return take_status(ctx);
}

// Staged-atom capacities of a tile from the current binning: +25% + 64
// headroom for the FP64 form and for the mixed form's redo pass; +6% + 32 for
// the mixed form's first pass (a tile that outgrows it before the next update
// is computed in full by the redo pass, at the redo capacity).
int update_capacity(examd_ctx* ctx, bool* grew = nullptr) {
  if (grew) *grew = false;
  CK(cudaMemsetAsync(ctx->d_occ, 0, 2 * sizeof(int), ctx->st));
  k_tile_occupancy<<<ctx->ntiles, 128, 0, ctx->st>>>(ctx->d_tiles, ctx->d_boxes, ctx->cstart, ctx->d_occ);
  CK(cudaGetLastError());
  int occ = 0;
  CK(cudaMemcpyAsync(&occ, ctx->d_occ, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  int want_r = std::max(((occ + occ / 4 + 64) + 7) & ~7, ctx->cap_redo);
  int want = ctx->pc.fp64 ? want_r : ((occ + occ / 16 + 32) + 7) & ~7;
  if (want <= ctx->cap) return EXAMD_OK;
  // mixed form with pair_tables = 0: the compact per-warp tables where they
  // fit more CTAs on an SM at this capacity (or where only they fit at all)
  auto choose = [&](int cap) {
    PairConfig c = ctx->pc;
    if (c.fp64 || ctx->pair_tables != 0) return c;
    PairConfig w = c, k = c;
    w.pack = false;
    k.pack = true;
    for (int e = 0; e < 2; ++e) {  // the occupancy query needs the opt-in limit set
      PairConfig q = e ? k : w;
      if (pair_prepare(q, ctx->smem_limit) != cudaSuccess) return c;
    }
    c.pack = pair_smem_bytes(w, cap, want_r, ctx->ne_max, ctx->ext_max) > ctx->smem_limit ||
             pair_blocks_per_sm(k, cap, ctx->ne_max, ctx->ext_max) > pair_blocks_per_sm(w, cap, ctx->ne_max, ctx->ext_max);
    return c;
  };
  PairConfig pc = choose(want);
  int bytes = pair_smem_bytes(pc, want, want_r, ctx->ne_max, ctx->ext_max);
  if (bytes > ctx->smem_limit) {
    // fall back to the exact need if the headroom does not fit
    want = want_r = (occ + 7) & ~7;
    pc = choose(want);
    bytes = pair_smem_bytes(pc, want, want_r, ctx->ne_max, ctx->ext_max);
    if (bytes > ctx->smem_limit) return EXAMD_ERR_CELL_OVERFLOW;
  }
  ctx->pc.pack = pc.pack;
  ctx->cap = want;
  ctx->cap_redo = want_r;
  ctx->smem = bytes;
  if (grew) *grew = true;
  // all variants used by this context
  PairConfig c = ctx->pc;
  for (int e = 0; e < 2; ++e)
    for (int n = 0; n < 2; ++n) {
      c.energy = e;
      c.count = n;
      CK(pair_prepare(c, bytes));
    }
  return EXAMD_OK;
}

PairArgs pair_args(examd_ctx* ctx) {
  PairArgs a{};
  a.tiles = ctx->d_tiles;
  a.order = ctx->d_order;
  a.boxes = ctx->d_boxes;
  a.cstart = ctx->cstart;
  a.U = ctx->U;
  a.X0 = ctx->X[ctx->cur][0];
  a.X1 = ctx->X[ctx->cur][1];
  a.X2 = ctx->X[ctx->cur][2];
  a.Fown = ctx->Fown;
  a.P = ctx->P;
  a.N = ctx->N;
  a.tileE = ctx->tileE;
  a.tileW = ctx->tileW;
  a.tileC = ctx->tileC;
  a.status = ctx->status;
  a.cap = ctx->cap;
  a.cap_redo = ctx->cap_redo;
  a.ne_max = ctx->ne_max;
  a.ext_max = ctx->ext_max;
  a.lj = ctx->lj;
  a.redo = ctx->redo;
  a.redo_n = ctx->redo_n;
  a.redo_done = (unsigned*)(ctx->redo_n + 1);
  a.list = ctx->plist;
  a.lraw = ctx->plraw;
  a.lperm = ctx->plperm;
  a.lcnt = ctx->plcnt;
  a.lcount = ctx->lcount;
  a.lk = ctx->lk;
  a.lslots = ctx->lslots;
  a.ntiles = ctx->ntiles;
  a.fb = ctx->fb;
  a.lw = ctx->lw;
  a.gate = nullptr;
  return a;
}

// Pair-list mode: the lists of every tile at the current cells.  gate: a
// device word that makes the build conditional (eager steps), or nullptr:
// build now, with the fallback list emptied first (host: a build the host
// asked for, counted here; otherwise the body of a captured rebuild, which
// the device counts).
int build_lists(examd_ctx* ctx, const int* gate, bool host = true) {
  if (!gate) CK(cudaMemsetAsync(ctx->lw + LW_FBN, 0, sizeof(int), ctx->st));
  if (!gate && host) ++ctx->host_builds;
  PairArgs a = pair_args(ctx);
  a.gate = gate;
  CK(launch_pair_build(ctx->pc, a, ctx->ntiles, ctx->smem, ctx->st));
  return EXAMD_OK;
}

// Pair-list mode: cells and lists rebuilt at the current positions (gate and
// host as for build_lists).
int rebuild(examd_ctx* ctx, const int* gate, bool host = true) {
  const int s = ctx->cur;
  if (ctx->N > 0) {
    k_bin_count<<<nblk(ctx->N), 256, 0, ctx->st>>>(ctx->N, ctx->X[s][0], ctx->X[s][1], ctx->X[s][2],
                                                    ctx->meta[s], ctx->d_boxes, ctx->cellOld, ctx->slot,
                                                    ctx->count, ctx->status, gate);
    CK(cudaGetLastError());
  }
  const int rc = finish_binning(ctx, true, gate);
  return rc ? rc : build_lists(ctx, gate, host);
}

// Pair-list mode, after new positions: the device decides whether some atom
// moved more than half the skin since the build (or a rebuild was asked
// for).  Eager, the rebuild's kernels run or return at once on that
// decision.  Under stream capture (the step loop's graphs, the captured
// force call) the rebuild is captured, ungated, as the body of a conditional
// graph node whose value the decision sets, so a step without a rebuild
// launches none of its kernels.
int maybe_rebuild(examd_ctx* ctx) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(ctx->st, &cs));
  if (cs != cudaStreamCaptureStatusActive) {
    k_list_decide<<<1, 1, 0, ctx->st>>>(ctx->lw, ctx->disp_thr2, cudaGraphConditionalHandle{}, 0);
    CK(cudaGetLastError());
    return rebuild(ctx, ctx->lw + LW_GATE);
  }
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(ctx->st, &cs, nullptr, &g, &deps, &edges, &nd));
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  k_list_decide<<<1, 1, 0, ctx->st>>>(ctx->lw, ctx->disp_thr2, h, 1);
  CK(cudaGetLastError());
  CK(cudaStreamGetCaptureInfo(ctx->st, &cs, nullptr, &g, &deps, &edges, &nd));
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeIf;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, edges, nd, &np));
  CK(cudaStreamUpdateCaptureDependencies(ctx->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  // the body: the rebuild's kernels, captured from a stream of their own
  cudaGraph_t body = np.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(ctx->stc, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  cudaStream_t main = ctx->st;
  ctx->st = ctx->stc;
  const int rc = rebuild(ctx, nullptr, false);
  ctx->st = main;
  cudaGraph_t captured = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(ctx->stc, &captured);
  if (rc) return rc;
  if (ce != cudaSuccess) return ctx->cuda_fail(ce, "cudaStreamEndCapture (rebuild body)");
  return EXAMD_OK;
}

// Pair-list mode: lists of `want` entries per staged atom, for the current
// staged-atom capacity.  The captured graphs name the old lists, so they are
// dropped.
int set_list_capacity(examd_ctx* ctx, int want) {
  const int slots = (ctx->cap + 31) & ~31;
  if (want == ctx->lk && slots == ctx->lslots && ctx->plist) return EXAMD_OK;
  CK(cudaStreamSynchronize(ctx->st));
  for (unsigned short** q : {&ctx->plist, &ctx->plraw, &ctx->plperm, &ctx->plcnt}) {
    if (*q) cudaFree(*q);
    *q = nullptr;
  }
  ctx->lk = ctx->lslots = 0;
  const size_t atoms = (size_t)ctx->ntiles * (size_t)slots;
  int rc;
  if ((rc = dalloc(ctx, &ctx->plist, atoms * (size_t)want)) || (rc = dalloc(ctx, &ctx->plraw, atoms * (size_t)want)) ||
      (rc = dalloc(ctx, &ctx->plperm, atoms)) || (rc = dalloc(ctx, &ctx->plcnt, atoms)))
    return rc;
  ctx->lk = want;
  ctx->lslots = slots;
  ++ctx->list_gen;
  if (ctx->gexec) {
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  for (auto& g : ctx->io_graph) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = examd_ctx::IoGraph{};
  }
  return EXAMD_OK;
}

// Pair-list mode: the list words, read after the stream's work; the longest
// list since the last read is reset.
int read_list_words(examd_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_lw, ctx->lw, LW_WORDS * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemsetAsync(ctx->lw + LW_LMAX, 0, sizeof(int), ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return EXAMD_OK;
}

// entries per atom: a multiple of 8 (a list pass reads eight at a time), at
// most 1024 (the list pass's count histogram)
int list_capacity_for(int longest) { return std::min(((longest + longest / 5 + 8) + 7) & ~7, 1024); }

// Pair-list mode, after a binning with the atoms in their cells: the lists
// built now at a capacity that fits the atom with the most entries, with 20 %
// headroom (the first build at an estimate from the densest box: 1.6 times
// the pairs in half a sphere of radius rc + skin).
int init_lists(examd_ctx* ctx) {
  if (ctx->p.pair_list_capacity > 0) {  // the caller's capacity, never resized
    const int rc = set_list_capacity(ctx, ctx->p.pair_list_capacity);
    return rc ? rc : build_lists(ctx, nullptr);
  }
  if (!ctx->plist) {
    double rho = 0.0, reach = 0.0;
    for (int b = 0; b < ctx->nboxes; ++b)
      rho = std::max(rho, (double)ctx->boxes[b].natoms / (ctx->boxes[b].L[0] * ctx->boxes[b].L[1] * ctx->boxes[b].L[2]));
    for (int k = 0; k < ctx->lj.nt * ctx->lj.nt; ++k) reach = std::max(reach, std::sqrt((double)ctx->lj.p32[k].rl2));
    const double est = 1.6 * (2.0943951 * reach * reach * reach * rho) + 16.0;
    const int rc = set_list_capacity(ctx, list_capacity_for((int)std::min(est, 4096.0)));
    if (rc) return rc;
  } else {
    const int rc = set_list_capacity(ctx, ctx->lk);  // new slots if the staged-atom capacity grew
    if (rc) return rc;
  }
  for (int it = 0; it < 4; ++it) {
    int rc = build_lists(ctx, nullptr);
    if (rc) return rc;
    rc = read_list_words(ctx);
    if (rc) return rc;
    const int longest = ctx->h_lw[LW_LMAX];
    const int want = list_capacity_for(longest);
    if (longest <= ctx->lk && ctx->lk <= 2 * want) return EXAMD_OK;
    rc = set_list_capacity(ctx, want);  // grow to fit, or shrink an estimate far too large
    if (rc) return rc;
  }
  return EXAMD_OK;  // any tile still over its list is computed by enumeration
}

int run_pair(examd_ctx* ctx, bool energy, bool count, double* boxE = nullptr, double* boxW = nullptr);

// Pair-list mode, between runs of steps: a tile with an atom whose list
// outgrew its capacity since the last check, or with more staged atoms than
// the lists have slots, is computed by enumeration meanwhile.  The lists get
// room for it: new lists, which a build at the current positions fills, after
// a fresh sort (a build needs every atom inside its cell), and the forces
// again in the new order.  A staged-atom capacity that grew within the slots
// makes the next step rebuild, so that the tiles over the old one get lists.
int update_lists(examd_ctx* ctx, bool cap_grew) {
  int rc = read_list_words(ctx);
  if (rc) return rc;
  const int longest = ctx->h_lw[LW_LMAX];
  const bool fixed = ctx->p.pair_list_capacity > 0;
  const int want = fixed ? ctx->lk : std::max(ctx->lk, list_capacity_for(longest));
  if (want != ctx->lk || ctx->cap > ctx->lslots) {
    if ((rc = set_list_capacity(ctx, want)) || (rc = rebuild(ctx, nullptr)) || (rc = run_pair(ctx, false, false)))
      return rc;
    return read_list_words(ctx);
  }
  if (cap_grew) {
    const int one = 1;
    CK(cudaMemcpyAsync(ctx->lw + LW_FORCE, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  return EXAMD_OK;
}

int run_pair(examd_ctx* ctx, bool energy, bool count, double* boxE, double* boxW) {
  PairConfig c = ctx->pc;
  c.energy = energy;
  c.count = count;
  CK(launch_pair(c, pair_args(ctx), ctx->ntiles, ctx->smem, ctx->st));
  if (energy)
    CK(launch_reduce_tiles(ctx->nboxes, ctx->d_tile0, ctx->maxc_tiles, ctx->tileE, ctx->tileW, ctx->partial,
                           boxE ? boxE : ctx->boxE,
                           boxW ? boxW : ctx->boxW, ctx->st));
  return EXAMD_OK;
}

StepArgs step_args(examd_ctx* ctx) {
  StepArgs s{};
  s.boxes = ctx->d_boxes;
  s.bmask = ctx->d_bmask;
  s.cellS = ctx->cellS;
  s.Fown = ctx->Fown;
  s.P = ctx->P;
  s.N = ctx->N;
  s.fp64 = ctx->pc.fp64;
  s.nc = ctx->NC;
  s.status = ctx->status;
  return s;
}

// The pair path at the resident positions, then the forces to the caller in
// chunks of its own order: the device->host copy of chunk c (second stream)
// overlaps the gather of chunk c + 1.  With accumulate, the caller's forces
// come in on the second stream while the pair kernel runs.
// The work of the force call, queued on the context's streams; the second
// stream rejoins the first at the end (so the sequence can be captured).
int enqueue_forces(examd_ctx* ctx, double* forces, double* epot, double* virial, int accumulate) {
  cudaStream_t st = ctx->st, st2 = ctx->st2;
  const bool energy = epot || virial;
  const int64_t N = ctx->N;
  const int nch = io_chunks(N);
  cudaEvent_t* ev_acc = ctx->ev_io + 2 * kIoChunks;
  if (forces && accumulate && N > 0) {
    CK(cudaEventRecord(ctx->ev_io[3 * kIoChunks], st));  // stage is free once earlier work is done
    CK(cudaStreamWaitEvent(st2, ctx->ev_io[3 * kIoChunks], 0));
    for (int c = 0; c < nch; ++c) {
      int64_t i0, i1;
      io_range(N, nch, c, i0, i1);
      CK(cudaMemcpyAsync(ctx->stage + 3 * i0, forces + 3 * i0, 3 * (i1 - i0) * sizeof(double),
                         cudaMemcpyHostToDevice, st2));
      CK(cudaEventRecord(ev_acc[c], st2));
    }
  }
  int rc = run_pair(ctx, energy, false);
  if (rc) return rc;
  if (forces && N > 0) {
    CK(ensure_inv(ctx));
    for (int c = 0; c < nch; ++c) {
      int64_t i0, i1;
      io_range(N, nch, c, i0, i1);
      if (accumulate) CK(cudaStreamWaitEvent(st, ev_acc[c], 0));
      CK(launch_forces_out(step_args(ctx), i0, i1, ctx->inv, ctx->stage, accumulate, st));
      CK(cudaEventRecord(ctx->ev_io[kIoChunks + c], st));
      CK(cudaStreamWaitEvent(st2, ctx->ev_io[kIoChunks + c], 0));
      CK(cudaMemcpyAsync(forces + 3 * i0, ctx->stage + 3 * i0, 3 * (i1 - i0) * sizeof(double),
                         cudaMemcpyDeviceToHost, st2));
    }
  }
  if (epot) CK(cudaMemcpyAsync(epot, ctx->boxE, ctx->nboxes * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (virial) CK(cudaMemcpyAsync(virial, ctx->boxW, ctx->nboxes * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(ctx->ev_io[3 * kIoChunks], st2));
  CK(cudaStreamWaitEvent(st, ctx->ev_io[3 * kIoChunks], 0));
  return EXAMD_OK;
}

// Waits for the force call and reads its status word.
int finish_forces(examd_ctx* ctx) {
  CK(queue_status(ctx));
  CK(cudaStreamSynchronize(ctx->st));
  const int rc = take_status(ctx);
  if (rc) return rc;
  ctx->forces_valid = true;
  return EXAMD_OK;
}

int forces_common(examd_ctx* ctx, double* forces, double* epot, double* virial, int accumulate) {
  const int rc = enqueue_forces(ctx, forces, epot, virial, accumulate);
  return rc ? rc : finish_forces(ctx);
}

bool pinned(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

}  // namespace

extern "C" {

int examd_gpu_set_atoms(examd_ctx* ctx, int64_t n, const double* pos, const int* type, const double* vel) {
  if (!ctx || (n > 0 && !pos) || n != ctx->N) return EXAMD_ERR_ARG;
  cudaSetDevice(ctx->dev);
  cudaStream_t st = ctx->st;
  std::vector<int> meta((size_t)n);
  for (int b = 0; b < ctx->nboxes; ++b)
    for (int64_t i = ctx->atom0[b]; i < ctx->atom0[b + 1]; ++i) {
      int t = type ? type[i] : 0;
      if (t < 0 || t >= ctx->p.ntypes) return EXAMD_ERR_ARG;
      meta[(size_t)i] = (b << 8) | t;
    }
  if (n > 0) {
    CK(cudaMemcpyAsync(ctx->stage, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    if (vel) CK(cudaMemcpyAsync(ctx->stage2, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->d_meta_in, meta.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  CK(cudaMemsetAsync(ctx->status, 0, sizeof(int), st));
  const int s = ctx->cur;
  if (n > 0) {
    k_load_bin<<<nblk(n), 256, 0, st>>>(n, ctx->stage, vel ? ctx->stage2 : nullptr, ctx->d_meta_in, ctx->d_boxes,
                                        ctx->p.strict_box, ctx->X[s][0], ctx->X[s][1], ctx->X[s][2], ctx->V[s][0],
                                        ctx->V[s][1], ctx->V[s][2], ctx->meta[s], ctx->id[s], ctx->cellOld,
                                        ctx->slot, ctx->count, ctx->status);
    CK(cudaGetLastError());
  }
  int rc = finish_binning(ctx, true);
  if (rc) return rc;
  CK(cudaStreamSynchronize(st));
  rc = check_status(ctx);
  if (rc) return rc;
  rc = update_capacity(ctx);
  if (rc) return rc;
  if (ctx->list) {
    CK(cudaMemsetAsync(ctx->lw, 0, LW_WORDS * sizeof(int), st));
    rc = init_lists(ctx);
    if (rc) return rc;
    rc = check_status(ctx);
    if (rc) return rc;
  }
  ctx->atoms_set = true;
  ctx->forces_valid = false;
  return EXAMD_OK;
}

int examd_gpu_forces(examd_ctx* ctx, double* forces, double* epot, double* virial, int accumulate) {
  if (!ctx) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  return forces_common(ctx, forces, epot, virial, accumulate);
}

}  // extern "C"

namespace {

// The force call at new positions, queued (see examd_gpu_forces_at).
int enqueue_forces_at(examd_ctx* ctx, const double* pos, double* forces, double* epot, double* virial,
                      int accumulate) {
  cudaStream_t st = ctx->st, st2 = ctx->st2;
  const int s = ctx->cur;
  const int64_t N = ctx->N;
  if (N > 0) {
    // positions in chunks of the caller's order: the host->device copy of
    // chunk c + 1 (second stream) overlaps the gather and binning count of chunk c
    CK(ensure_inv(ctx));
    CK(cudaEventRecord(ctx->ev_io[3 * kIoChunks], st));
    CK(cudaStreamWaitEvent(st2, ctx->ev_io[3 * kIoChunks], 0));
    const int nch = io_chunks(N);
    for (int c = 0; c < nch; ++c) {
      int64_t i0, i1;
      io_range(N, nch, c, i0, i1);
      CK(cudaMemcpyAsync(ctx->stage2 + 3 * i0, pos + 3 * i0, 3 * (i1 - i0) * sizeof(double),
                         cudaMemcpyHostToDevice, st2));
      CK(cudaEventRecord(ctx->ev_io[c], st2));
      CK(cudaStreamWaitEvent(st, ctx->ev_io[c], 0));
      if (ctx->list) {
        CK(launch_gather_pos_list(i0, i1, ctx->stage2, ctx->d_boxes, ctx->p.strict_box, ctx->X[s][0],
                                  ctx->X[s][1], ctx->X[s][2], ctx->meta[s], ctx->inv, ctx->cellS, ctx->U, ctx->Ub,
                                  ctx->lw, ctx->status, st));
      } else {
        k_gather_pos_bin_range<<<nblk(i1 - i0), 256, 0, st>>>(i0, i1, ctx->stage2, ctx->d_boxes,
                                                              ctx->p.strict_box, ctx->X[s][0], ctx->X[s][1],
                                                              ctx->X[s][2], ctx->meta[s], ctx->inv, ctx->cellOld,
                                                              ctx->slot, ctx->count, ctx->status);
        CK(cudaGetLastError());
      }
    }
  }
  int rc = ctx->list ? maybe_rebuild(ctx) : finish_binning(ctx, true);
  if (rc) return rc;
  return enqueue_forces(ctx, forces, epot, virial, accumulate);
}

int finish_forces_at_eager(examd_ctx* ctx, const double* pos, double* forces, double* epot, double* virial,
                           int accumulate) {
  const int rc = enqueue_forces_at(ctx, pos, forces, epot, virial, accumulate);
  return rc ? rc : finish_forces(ctx);
}

}  // namespace

extern "C" {

int examd_gpu_forces_at(examd_ctx* ctx, const double* pos, double* forces, double* epot, double* virial,
                        int accumulate) {
  if (!ctx || (ctx->N > 0 && !pos)) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  CK(ensure_inv(ctx));  // outside any captured sequence
  if (ctx->N < kIoMinChunk || !pinned(pos) || !pinned(forces) || !pinned(epot) || !pinned(virial))
    return finish_forces_at_eager(ctx, pos, forces, epot, virial, accumulate);
  // same pinned buffers as last time at this parity: replay the captured call
  auto& g = ctx->io_graph[ctx->cur];
  const bool hit = g.exec && g.pos == pos && g.forces == forces && g.epot == epot && g.virial == virial &&
                   g.accumulate == accumulate && g.cap == ctx->cap && g.cap_redo == ctx->cap_redo &&
                   g.pack == ctx->pc.pack && g.list_gen == ctx->list_gen;
  if (!hit) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = examd_ctx::IoGraph{};
    const int parity = ctx->cur;
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_forces_at(ctx, pos, forces, epot, virial, accumulate);
    cudaError_t ce = cudaStreamEndCapture(ctx->st, &graph);
    ctx->cur = parity;  // capture only recorded the work
    if (rc) return rc;
    if (ce != cudaSuccess) return ctx->cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      g.exec = nullptr;
      return ctx->cuda_fail(ce, "cudaGraphInstantiate");
    }
    g.pos = pos;
    g.forces = forces;
    g.epot = epot;
    g.virial = virial;
    g.accumulate = accumulate;
    g.cap = ctx->cap;
    g.cap_redo = ctx->cap_redo;
    g.pack = ctx->pc.pack;
    g.list_gen = ctx->list_gen;
  }
  CK(cudaGraphLaunch(g.exec, ctx->st));
  if (!ctx->list) ctx->cur = 1 - ctx->cur;  // the host-side effects of the captured call
  ctx->inv_valid = true;
  return finish_forces(ctx);
}

}  // extern "C"

namespace {

KickArgs kick_args(examd_ctx* ctx, double ckick, double dt, bool drift, double hk, double* boxKE) {
  KickArgs k{};
  k.s = step_args(ctx);
  const int c = ctx->cur;
  for (int a = 0; a < 3; ++a) {
    k.X[a] = ctx->X[c][a];
    k.V[a] = ctx->V[c][a];
  }
  k.meta = ctx->meta[c];
  k.ckick = ckick;
  k.dt = dt;
  k.drift = drift;
  k.hk = hk;
  for (int t = 0; t < EXAMD_MAX_TYPES; ++t) {
    k.ckm[t] = ckick * ctx->lj.minv[t];
    k.hkm[t] = hk * ctx->lj.minv[t];
  }
  k.boxKE = boxKE;
  k.keAtom = ctx->keAtom;
  k.partial = ctx->partial;
  k.maxc = ctx->maxc_atoms;
  k.atom0 = ctx->d_atom0;
  k.nboxes = ctx->nboxes;
  k.lj = ctx->lj;
  k.cellOld = ctx->cellOld;
  k.slot = ctx->slot;
  k.count = ctx->count;
  k.status = ctx->status;
  k.list = ctx->list;
  k.U = ctx->U;
  k.Ub = ctx->Ub;
  k.lw = ctx->lw;
  return k;
}

// One step after the first: kick(ck) + drift + bin, pair.  keSlot receives the
// kinetic energy at the start of this step, eSlot the potential energy after.
// Pair-list mode: the binning and the lists only on the steps that the
// device decides to rebuild.
int step_once(examd_ctx* ctx, double ck, double dt, double* keSlot, double* eSlot, double* wSlot) {
  const double h = 0.5 * dt;
  CK(launch_kick(kick_args(ctx, ck, dt, true, keSlot ? h : 0.0, keSlot), ctx->st));
  int rc = ctx->list ? maybe_rebuild(ctx) : finish_binning(ctx, false);
  if (rc) return rc;
  return run_pair(ctx, eSlot != nullptr, false, eSlot, wSlot);
}

int ensure_ebuf(examd_ctx* ctx, int steps) {
  if (steps <= ctx->ebuf_steps) return EXAMD_OK;
  if (ctx->boxE) cudaFree(ctx->boxE);
  if (ctx->boxW) cudaFree(ctx->boxW);
  if (ctx->boxKE) cudaFree(ctx->boxKE);
  ctx->boxE = ctx->boxW = ctx->boxKE = nullptr;
  size_t n = (size_t)(steps + 1) * ctx->nboxes;
  int rc;
  if ((rc = dalloc(ctx, &ctx->boxE, n)) || (rc = dalloc(ctx, &ctx->boxW, n)) || (rc = dalloc(ctx, &ctx->boxKE, n)))
    return rc;
  ctx->ebuf_steps = steps;
  // every captured graph that names the old energy buffers is stale: the step
  // loop's and the force call's (whose energy variant writes and reads boxE,
  // boxW)
  if (ctx->gexec) {
    cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
  }
  for (auto& g : ctx->io_graph) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = examd_ctx::IoGraph{};
  }
  return EXAMD_OK;
}

// The steady-state step loop of `chunk` steps (merged kicks) as one CUDA
// graph for buffer parity `parity`, captured and instantiated unless the
// cached one already matches.  Captures only: no step runs.
int ensure_chunk_graph(examd_ctx* ctx, int chunk, double dt, bool wantE, int parity) {
  const bool stale = !ctx->gexec || ctx->g_parity != parity || ctx->g_chunk != chunk ||
                     ctx->g_energy != (int)wantE || ctx->g_dt != dt || ctx->g_cap != ctx->cap ||
                     ctx->g_list_gen != ctx->list_gen;
  if (!stale) return EXAMD_OK;
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  ctx->gexec = nullptr;
  const int nb = ctx->nboxes;
  const int saved = ctx->cur;
  ctx->cur = parity;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
  int src = EXAMD_OK;
  for (int j = 0; j < chunk && src == EXAMD_OK; ++j)
    src = step_once(ctx, dt, dt, wantE ? ctx->boxKE + (size_t)j * nb : nullptr,
                    wantE ? ctx->boxE + (size_t)j * nb : nullptr, wantE ? ctx->boxW + (size_t)j * nb : nullptr);
  cudaError_t ce = cudaStreamEndCapture(ctx->st, &g);
  // capture advanced the host-side parity; the graph leaves it unchanged (chunk
  // even; pair-list mode: no step swaps the buffers)
  ctx->cur = saved;
  if (src != EXAMD_OK) return src;
  if (ce != cudaSuccess) return ctx->cuda_fail(ce, "cudaStreamEndCapture");
  ce = cudaGraphInstantiate(&ctx->gexec, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) {
    ctx->gexec = nullptr;
    return ctx->cuda_fail(ce, "cudaGraphInstantiate");
  }
  ctx->g_parity = parity;
  ctx->g_chunk = chunk;
  ctx->g_energy = wantE;
  ctx->g_dt = dt;
  ctx->g_cap = ctx->cap;
  ctx->g_list_gen = ctx->list_gen;
  return EXAMD_OK;
}

}  // namespace

extern "C" {

int examd_gpu_run(examd_ctx* ctx, int nsteps, double dt, int graph_chunk, double* energies, examd_stats* stats) {
  if (!ctx || nsteps < 0 || !(dt > 0) || graph_chunk < 0) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  cudaStream_t st = ctx->st;
  const int nb = ctx->nboxes;
  const bool wantE = energies != nullptr;
  int chunk = graph_chunk > 0 ? (graph_chunk + 1) / 2 * 2 : 0;
  int rc = ensure_ebuf(ctx, std::max(chunk, 1) + 1);
  if (rc) return rc;
  if (!ctx->forces_valid) {
    rc = run_pair(ctx, false, false);
    if (rc) return rc;
    ctx->forces_valid = true;
  }
  if (nsteps == 0) return EXAMD_OK;
  const double h = 0.5 * dt;
  CK(cudaEventRecord(ctx->e0, st));
  // step 1: half kick + drift, then forces
  rc = step_once(ctx, h, dt, nullptr, wantE ? ctx->boxE : nullptr, wantE ? ctx->boxW : nullptr);
  if (rc) return rc;
  if (wantE) {
    // energies[0] epot now; ekin later
    for (int b = 0; b < nb; ++b)
      CK(cudaMemcpyAsync(&energies[2 * b + 1], ctx->boxE + b, sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  int done = 1;
  // steady state: merged kicks v += dt F/m
  while (done < nsteps) {
    const int left = nsteps - done;
    if (chunk > 0 && left >= chunk) {
      rc = ensure_chunk_graph(ctx, chunk, dt, wantE, ctx->cur);
      if (rc) return rc;
      CK(cudaGraphLaunch(ctx->gexec, st));
      if (wantE) {
        // slot j: ekin at the start of local step j (= after global step done + j), epot after it
        for (int j = 0; j < chunk; ++j)
          for (int b = 0; b < nb; ++b) {
            const size_t gs = (size_t)(done + j);  // global 0-based step index of epot
            CK(cudaMemcpyAsync(&energies[2 * ((gs - 1) * nb + b)], ctx->boxKE + (size_t)j * nb + b,
                               sizeof(double), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(&energies[2 * (gs * nb + b) + 1], ctx->boxE + (size_t)j * nb + b, sizeof(double),
                               cudaMemcpyDeviceToHost, st));
          }
        CK(cudaStreamSynchronize(st));  // buffers are reused by the next replay
      }
      done += chunk;
      // the capacities may need to grow as the density fluctuates
      CK(cudaStreamSynchronize(st));
      rc = check_status(ctx);
      if (rc) return rc;
      bool grew = false;
      rc = update_capacity(ctx, &grew);
      if (rc) return rc;
      if (ctx->list && (rc = update_lists(ctx, grew))) return rc;
    } else {
      double* ke = nullptr;
      if (wantE) ke = ctx->boxKE;
      rc = step_once(ctx, dt, dt, ke, wantE ? ctx->boxE : nullptr, wantE ? ctx->boxW : nullptr);
      if (rc) return rc;
      if (wantE)
        for (int b = 0; b < nb; ++b) {
          CK(cudaMemcpyAsync(&energies[2 * ((size_t)(done - 1) * nb + b)], ctx->boxKE + b, sizeof(double),
                             cudaMemcpyDeviceToHost, st));
          CK(cudaMemcpyAsync(&energies[2 * ((size_t)done * nb + b) + 1], ctx->boxE + b, sizeof(double),
                             cudaMemcpyDeviceToHost, st));
        }
      if (wantE) CK(cudaStreamSynchronize(st));
      done += 1;
    }
  }
  // closing half kick: v(t_n) = v(t_n - h) + h F/m
  CK(launch_kick(kick_args(ctx, h, dt, false, wantE ? h : 0.0, ctx->boxKE), st));
  if (wantE)
    for (int b = 0; b < nb; ++b)
      CK(cudaMemcpyAsync(&energies[2 * ((size_t)(nsteps - 1) * nb + b)], ctx->boxKE + b, sizeof(double),
                         cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(ctx->e1, st));
  CK(cudaStreamSynchronize(st));
  rc = check_status(ctx);
  if (rc) return rc;
  ctx->forces_valid = true;
  if (stats) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->e0, ctx->e1));
    std::memset(stats, 0, sizeof(*stats));
    stats->ms = ms;
    stats->steps = nsteps;
    if (wantE) {
      for (int b = 0; b < nb; ++b) {
        stats->ekin += energies[2 * ((size_t)(nsteps - 1) * nb + b)];
        stats->epot += energies[2 * ((size_t)(nsteps - 1) * nb + b) + 1];
      }
    }
  }
  return EXAMD_OK;
}

int examd_gpu_prepare_run(examd_ctx* ctx, double dt, int graph_chunk, int energies) {
  if (!ctx || !(dt > 0) || graph_chunk < 0) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  const int chunk = graph_chunk > 0 ? (graph_chunk + 1) / 2 * 2 : 0;
  int rc = ensure_ebuf(ctx, std::max(chunk, 1) + 1);
  if (rc) return rc;
  if (!ctx->forces_valid) {
    rc = run_pair(ctx, false, false);
    if (rc) return rc;
    rc = check_status(ctx);
    if (rc) return rc;
    ctx->forces_valid = true;
  }
  if (chunk == 0) return EXAMD_OK;
  // the run's first step flips the sort's double buffer: its graph chunks
  // run at the other parity (pair-list mode: at this one)
  rc = ensure_chunk_graph(ctx, chunk, dt, energies != 0, ctx->list ? ctx->cur : 1 - ctx->cur);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->st));
  return EXAMD_OK;
}

int examd_gpu_time_phases(examd_ctx* ctx, int nsteps, double dt, double* ms) {
  if (!ctx || nsteps < 1 || !(dt > 0) || !ms) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  cudaStream_t st = ctx->st;
  int rc;
  if (!ctx->forces_valid) {
    rc = run_pair(ctx, false, false);
    if (rc) return rc;
    ctx->forces_valid = true;
  }
  double acc[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < nsteps; ++k) {
    // one steady-state step (merged kick), as the captured loop runs it
    CK(cudaEventRecord(ctx->e0, st));
    CK(launch_kick(kick_args(ctx, dt, dt, true, 0.0, nullptr), st));
    CK(cudaEventRecord(ctx->e1, st));
    rc = ctx->list ? maybe_rebuild(ctx) : finish_binning(ctx, false);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->e2, st));
    rc = run_pair(ctx, false, false);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->e3, st));
    CK(cudaStreamSynchronize(st));
    float t01 = 0.f, t12 = 0.f, t23 = 0.f;
    CK(cudaEventElapsedTime(&t01, ctx->e0, ctx->e1));
    CK(cudaEventElapsedTime(&t12, ctx->e1, ctx->e2));
    CK(cudaEventElapsedTime(&t23, ctx->e2, ctx->e3));
    acc[0] += t01;
    acc[1] += t12;
    acc[2] += t23;
  }
  rc = check_status(ctx);
  if (rc) return rc;
  for (int a = 0; a < 3; ++a) ms[a] = acc[a] / nsteps;
  return EXAMD_OK;
}

int examd_gpu_time_rebuild(examd_ctx* ctx, int reps, double* ms) {
  if (!ctx || reps < 1 || !ms) return EXAMD_ERR_ARG;
  if (!ctx->list) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  CK(cudaEventRecord(ctx->e0, ctx->st));
  for (int r = 0; r < reps; ++r) {
    const int rc = rebuild(ctx, nullptr);
    if (rc) return rc;
  }
  CK(cudaEventRecord(ctx->e1, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->e0, ctx->e1));
  *ms = t / reps;
  ctx->forces_valid = false;  // the sorted order changed
  return check_status(ctx);
}

int examd_gpu_list_info(examd_ctx* ctx, int64_t* builds, int* capacity, int* longest, int* fallback_tiles) {
  if (!ctx) return EXAMD_ERR_ARG;
  int64_t b = 0;
  int c = 0, l = 0, f = 0;
  if (ctx->list) {
    cudaSetDevice(ctx->dev);
    const int rc = read_list_words(ctx);
    if (rc) return rc;
    b = ctx->h_lw[LW_BUILDS] + ctx->host_builds;
    c = ctx->lk;
    l = ctx->h_lw[LW_LMAX];
    f = ctx->h_lw[LW_FBN];
  }
  if (builds) *builds = b;
  if (capacity) *capacity = c;
  if (longest) *longest = l;
  if (fallback_tiles) *fallback_tiles = f;
  return EXAMD_OK;
}

int examd_gpu_get_state(examd_ctx* ctx, double* pos, double* vel) {
  if (!ctx) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  const int c = ctx->cur;
  if (pos) {
    CK(launch_state_out(ctx->N, ctx->X[c], ctx->id[c], ctx->stage, ctx->st));
    CK(cudaMemcpyAsync(pos, ctx->stage, 3 * ctx->N * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  }
  if (vel) {
    CK(launch_state_out(ctx->N, ctx->V[c], ctx->id[c], ctx->stage2, ctx->st));
    CK(cudaMemcpyAsync(vel, ctx->stage2, 3 * ctx->N * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  }
  CK(cudaStreamSynchronize(ctx->st));
  return EXAMD_OK;
}

int examd_gpu_kinetic(examd_ctx* ctx, double* ekin) {
  if (!ctx || !ekin) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  const int c = ctx->cur;
  CK(launch_kinetic(ctx->N, ctx->nboxes, ctx->d_atom0, ctx->maxc_atoms, ctx->V[c], ctx->meta[c], ctx->lj,
                    ctx->keAtom, ctx->partial, ctx->boxKE,
                    ctx->st));
  CK(cudaMemcpyAsync(ekin, ctx->boxKE, ctx->nboxes * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return EXAMD_OK;
}

int examd_gpu_scale_velocities(examd_ctx* ctx, const double* factor) {
  if (!ctx || !factor) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  const int c = ctx->cur;
  CK(cudaMemcpyAsync(ctx->d_factor, factor, ctx->nboxes * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  CK(launch_scale_v(ctx->N, ctx->V[c], ctx->meta[c], ctx->d_factor, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return EXAMD_OK;
}

int examd_gpu_time_forces(examd_ctx* ctx, int reps, double* ms, double* kernel_ms) {
  if (!ctx || reps < 1) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  cudaStream_t st = ctx->st;
  int rc = run_pair(ctx, false, false);  // warm-up
  if (rc) return rc;
  CK(cudaEventRecord(ctx->e0, st));
  for (int r = 0; r < reps; ++r) {
    rc = run_pair(ctx, false, false);
    if (rc) return rc;
  }
  CK(cudaEventRecord(ctx->e1, st));
  CK(cudaStreamSynchronize(st));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->e0, ctx->e1));
  if (ms) *ms = t;
  if (kernel_ms) *kernel_ms = t / reps;
  rc = check_status(ctx);
  if (rc) return rc;
  ctx->forces_valid = true;
  return EXAMD_OK;
}

int examd_gpu_counters(examd_ctx* ctx, int64_t* candidates, int64_t* accepted, int64_t* evaluated,
                       int64_t* tiles, int64_t* max_tile_atoms) {
  if (!ctx) return EXAMD_ERR_ARG;
  if (!ctx->atoms_set) return EXAMD_ERR_STATE;
  cudaSetDevice(ctx->dev);
  int rc;
  // pair-list mode: the counts are the enumeration's, which needs every atom
  // inside its cell: a fresh sort and lists first
  if (ctx->list && (rc = rebuild(ctx, nullptr))) return rc;
  rc = run_pair(ctx, false, true);
  if (rc) return rc;
  std::vector<long long> c(3 * (size_t)ctx->ntiles);
  CK(cudaMemcpyAsync(c.data(), ctx->tileC, c.size() * sizeof(long long), cudaMemcpyDeviceToHost, ctx->st));
  int occ = 0;
  CK(cudaMemsetAsync(ctx->d_occ, 0, 2 * sizeof(int), ctx->st));
  k_tile_occupancy<<<ctx->ntiles, 128, 0, ctx->st>>>(ctx->d_tiles, ctx->d_boxes, ctx->cstart, ctx->d_occ);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&occ, ctx->d_occ, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  rc = check_status(ctx);
  if (rc) return rc;
  long long s1 = 0, s2 = 0, s3 = 0;
  for (int t = 0; t < ctx->ntiles; ++t) {
    s1 += c[3 * t];
    s2 += c[3 * t + 1];
    s3 += c[3 * t + 2];
  }
  if (candidates) *candidates = s1;
  if (accepted) *accepted = s2;
  if (evaluated) *evaluated = s3;
  if (tiles) *tiles = ctx->ntiles;
  if (max_tile_atoms) *max_tile_atoms = occ;
  ctx->forces_valid = true;
  return EXAMD_OK;
}

}  // extern "C"
