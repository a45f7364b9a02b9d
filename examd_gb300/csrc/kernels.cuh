// kernels.cuh -- host-side launchers of the device kernels (one per .cu file).
#pragma once

#include "common.cuh"

namespace examd {

// ---- bin.cu -----------------------------------------------------------------
__global__ void k_load_bin(int64_t n, const double* aos, const double* vaos, const int* meta_in,
                           const BoxDev* boxes, int strict, double* X0, double* X1, double* X2, double* V0,
                           double* V1, double* V2, int* meta, int* id, int* cellOld, int* slot,
                           int* count, int* status);
__global__ void k_gather_pos_bin_range(int64_t i0, int64_t i1, const double* aos, const BoxDev* boxes, int strict,
                                       double* X0, double* X1, double* X2, const int* meta, const int* inv,
                                       int* cellOld, int* slot, int* count, int* status);
__global__ void k_inverse(int64_t n, const int* id, int* inv);
// gate: nullptr, or a device word; zero makes the launch return at once (the
// pair-list mode's conditional rebuild inside a captured step loop).
__global__ void k_scan_reduce(int nc, const int* count, int* bsum, const int* gate);
__global__ void k_scan_final(int nc, int* count, const int* bsum, int* cstart, const int* gate);
__global__ void k_finalize(int64_t n, const int* cellOld, const int* slot, const int* cstart, const BoxDev* boxes,
                           const double* X0, const double* X1, const double* X2, const double* V0,
                           const double* V1, const double* V2, const int* meta, const int* id, double* Y0,
                           double* Y1, double* Y2, double* W0, double* W1, double* W2, int* meta2, int* id2,
                           float4* U, float4* Ub, int* cellS, int* inv, int nc, int* status, const int* gate);
// Pair-list mode's rebuild: the binning count at the current positions, and
// the sorted arrays copied back into the primary buffer (the step loop's
// buffers stay fixed whether a step rebuilds or not).
__global__ void k_bin_count(int64_t n, const double* X0, const double* X1, const double* X2, const int* meta,
                            const BoxDev* boxes, int* cellOld, int* slot, int* count, int* status, const int* gate);
__global__ void k_copy_back(int64_t n, const double* Y0, const double* Y1, const double* Y2, const double* W0,
                            const double* W1, const double* W2, const int* meta2, const int* id2, double* X0,
                            double* X1, double* X2, double* V0, double* V1, double* V2, int* meta, int* id,
                            const int* gate);
// Pair-list mode: decide whether this step rebuilds (largest displacement
// since the build against thr2 = (skin/2 - margin)^2, or a forced rebuild);
// in a captured step loop (cond) also the value of the conditional graph
// node that holds the rebuild.
__global__ void k_list_decide(int* lw, float thr2, cudaGraphConditionalHandle h, int cond);
constexpr int kScanTileHost = 2048;  // cells per scan block (kScanThreads * kScanItems)

// ---- pair.cu ----------------------------------------------------------------
struct PairArgs {
  const int4* tiles;  // 2 int4 per tile
  const int* order;   // launch order: CTA b computes tile order[b] (the costliest tiles first)
  const BoxDev* boxes;
  const int* cstart;
  const float4* U;
  const double* X0;
  const double* X1;
  const double* X2;
  void* Fown;  // mixed: float4[N]; fp64: double[3][N]
  void* P;     // mixed: float4[7][N]; fp64: double[7][3][N]
  int64_t N;
  double* tileE;     // per tile potential energy
  double* tileW;     // per tile virial
  long long* tileC;  // per tile (candidates, accepted)
  int* status;
  int cap;     // staged-atom capacity of a tile (mixed form: of the first pass)
  int cap_redo;  // mixed form: capacity of the redo pass
  int ne_max;  // largest ext-cell count of a tile
  int ext_max;  // largest ext extent of a tile on one axis
  LJTable lj;
  // mixed form: tiles whose pair-force terms exceeded the fixed-point range,
  // for the redo pass (ntiles entries; count and done counter zero between launches)
  int* redo;
  int* redo_n;
  unsigned* redo_done;
  // pair-list mode, per tile (lslots staged-atom slots, a multiple of 32, of
  // up to lk entries each, lk a multiple of 8 and at most 1024): the staged
  // atoms in the order of their entry counts, most first (lperm), and their
  // counts in that order (lcnt); the entries, the staged indices m of the
  // pairs (i, m) that the tile owns within the list cutoff, in that order by
  // groups of 32 atoms, entries k..k+3 of the group's 32 atoms side by side
  // (list[tile][p / 32][k / 4][p % 32][k % 4] for the atom at position p),
  // every atom's entries padded up to its group's longest count with the
  // tile's staged-atom count (an index the list passes stage beyond every
  // cutoff);
  // the build's scratch, each atom's entries in staged order
  // (lraw[tile][i][k]); per tile the staged atoms, or -1 when the tile is in
  // the fallback list fb (computed by enumeration every step); the list
  // words (ListWord); the build's gate (nullptr: build unconditionally)
  unsigned short* list;
  unsigned short* lraw;
  unsigned short* lperm;
  unsigned short* lcnt;
  int* lcount;
  int lk;
  int lslots;
  int ntiles;
  int* fb;
  int* lw;
  const int* gate;
};

struct PairConfig {
  bool fp64 = false;
  bool multi = false;   // more than one atom type
  bool pack = false;    // mixed form: compact per-warp tables (more CTAs per SM)
  bool energy = false;  // potential energy and virial
  bool count = false;   // candidate / accepted counters
  bool list = false;    // mixed form: pair-list mode (forces from the per-tile lists)
  bool cut = true;      // list pass: the potential's own range is finite (WCA) and tested
  int warps = 8;
};

// Dynamic shared memory for the tile capacities: the larger of the first
// pass's need at cap and, mixed form, the redo pass's at cap_redo.
int pair_smem_bytes(const PairConfig& cfg, int cap, int cap_redo, int ne_max, int ext_max);
cudaError_t pair_prepare(const PairConfig& cfg, int smem_bytes);  // opt-in smem attribute
// Resident CTAs per SM of the pair kernel at this capacity (occupancy calculator).
int pair_blocks_per_sm(const PairConfig& cfg, int cap, int ne_max, int ext_max);
cudaError_t launch_pair(const PairConfig& cfg, const PairArgs& a, int ntiles, int smem_bytes, cudaStream_t st);
// Pair-list mode: build the per-tile lists (gated by a.gate).
cudaError_t launch_pair_build(const PairConfig& cfg, const PairArgs& a, int ntiles, int smem_bytes, cudaStream_t st);
cudaError_t upload_own_lut(const OwnLut& lut);

// ---- step.cu ----------------------------------------------------------------
struct StepArgs {
  const BoxDev* boxes;
  const unsigned char* bmask;  // per global cell: bit a set when the cell is first/last of its tile on axis a
  const int* cellS;
  const void* Fown;
  const void* P;
  int64_t N;
  bool fp64;
  int nc;       // cells (the bmask length; index checks of the checked build)
  int* status;  // the status word (index checks of the checked build)
};

// F = Fown + halo partials, in caller order, AoS doubles (out[3*id + a]); += if accumulate.
cudaError_t launch_forces_out(const StepArgs& s, int64_t i0, int64_t i1, const int* inv, double* out, int accumulate,
                              cudaStream_t st);
// Per-box sums of the per-tile energy/virial partials (FP64, fixed order).
// Per-box sums in two fixed-order levels (chunks of 4096 entries, then the
// box's chunks in order); partial holds nboxes * maxc doubles (tiles: twice).
int red_chunks(int64_t max_per_box);
cudaError_t launch_reduce_tiles(int nboxes, const int* tile0, int maxc, const double* tileE, const double* tileW,
                                double* partial, double* boxE, double* boxW, cudaStream_t st);
cudaError_t launch_box_sums(int nboxes, const int64_t* atom0, int maxc, const double* v, double* partial,
                            double* out, cudaStream_t st);
// Velocity-Verlet pieces.  kick: v += c_kick F / m.  With drift: x += dt v, wrap, bin.
struct KickArgs {
  StepArgs s;
  double* X[3];
  double* V[3];
  const int* meta;
  double ckick;  // dt or dt/2
  double dt;
  bool drift;
  double hk;        // > 0: also the kinetic energy at v + hk F / m, per box
  double ckm[4];    // ckick / m per type
  double hkm[4];    // hk / m per type
  double* keAtom;   // per-atom kinetic energy scratch (N)
  double* boxKE;    // per-box kinetic energy (fixed-order reduction of keAtom)
  double* partial;  // chunk partial sums of that reduction
  int maxc;         // chunks per box
  const int64_t* atom0;  // nboxes + 1 atom offsets (sorted order is grouped by box)
  int nboxes;
  LJTable lj;
  // binning outputs (drift only)
  int* cellOld;
  int* slot;
  int* count;
  int* status;
  // pair-list mode (drift only, instead of the binning count): the FP32
  // offsets U from each atom's cell at the last build, and the largest
  // squared displacement from the offsets Ub of that build (lw[LW_DISP])
  bool list;
  float4* U;
  const float4* Ub;
  int* lw;
};
cudaError_t launch_kick(const KickArgs& k, cudaStream_t st);
// Pair-list mode: new positions for the caller's atoms [i0, i1) at their
// sorted slots, with the offsets from their cells at the last build and the
// displacement since then (the force call at new positions).
cudaError_t launch_gather_pos_list(int64_t i0, int64_t i1, const double* aos, const BoxDev* boxes, int strict,
                                   double* X0, double* X1, double* X2, const int* meta, const int* inv,
                                   const int* cellS, float4* U, const float4* Ub, int* lw, int* status,
                                   cudaStream_t st);
cudaError_t launch_kinetic(int64_t n, int nboxes, const int64_t* atom0, int maxc, const double* const V[3],
                           const int* meta, LJTable lj, double* keAtom, double* partial, double* boxKE,
                           cudaStream_t st);
cudaError_t launch_reduce_atoms(int nboxes, const int64_t* atom0, const double* v, double* out, cudaStream_t st);
cudaError_t launch_scale_v(int64_t n, double* V[3], const int* meta, const double* factor, cudaStream_t st);
cudaError_t launch_state_out(int64_t n, const double* const A[3], const int* id, double* out, cudaStream_t st);

}  // namespace examd
