// pair.cu -- the midpoint pair kernel: one CTA per tile of home cells.
//
// Replaces exaMD_forces_midpoint_all / _bdry / _overlap, exaMD_particle_
// interaction and lennardjones_12 (SRC/exaMD_forces.f90:41-551,
// user_func.f90:40-75).  A tile owns every cell pair whose home block -- given
// by the reference's 63-entry table (SRC/exaMD_module.f90:276-346) -- lies in
// the tile; the tile plus a one-cell halo is staged in shared memory with the
// periodic images folded into the staged coordinates (the SMEM counterpart of
// the MPI halo exchange, SRC/exaMD_comms.f90:44-244).
//
// Work order.  The 62 non-self table entries are, per cell A, 12 full x-rows
// of 5 cells (dy, dz fixed, dx = -2..2) plus the half row dx = +1, +2; with
// the pairs inside A that makes 13 "rows" r.  A warp turns (staged atom,
// row) pairs into items: the contiguous j-ranges of the cells of row r that
// the table assigns to this tile (ownership masks per position class),
// trimmed to the cells whose box comes within rc of the atom (the accepted
// pairs are unchanged).  Only rows with a nonzero mask for the atom's class
// are visited, 32 (atom, row) pairs per step whatever the atom; the items
// of one step (at most 32) have their candidate pairs laid end to end and
// tested 32 at a time, one per lane.  Accepted pairs are queued and their
// forces computed in batches of 32, both atoms' sums updated (Newton's third
// law).  The FP64 form builds items per (ext cell, row) instead: the block
// of the cell's atoms against the row's owned j-cells, untrimmed, tested with
// an FP32 prefilter on a widened cutoff; the queued pairs are computed in
// FP64.  Its batches then hold pairs of many different i atoms, so their FP64
// shared-memory atomics (the FP64 form's bound) rarely hit one address.
//
// Accumulation.  Mixed form: each per-atom force component is an exact 32-bit
// fixed-point sum in shared memory (scale 2^17, native integer atomics), so
// the result does not depend on the order of the terms and is reproducible
// bit for bit.  A term of magnitude >= 2048 (r < 0.74 sigma at eps = 1) is
// left out and flags the tile, so every fixed-point term is below 2^28 and a
// component's sum could leave the int32 range only through more than 8
// near-maximal terms of one sign on one atom, i.e. 8 neighbours within about
// 0.75 sigma on one side, which no physical configuration has (the repulsive
// cores of 8 such neighbours do not fit in one hemisphere).  A second
// launch (k_pair_redo) recomputes the flagged tiles, sums their large terms
// in FP32 and adds them to the outputs; thermal configurations flag no tile
// and the launch returns at once (only the rare FP32 sums' order can vary
// between runs).  FP64 form: FP64 shared-memory atomics.
//
// Output: forces of the tile's home atoms go to Fown, those of halo copies to
// the partial slot P[s] (s = bitmask of the axes on which the copy is a halo
// copy); the integrator sums an atom's 1..8 partials in a fixed order.
#include <algorithm>
#include <type_traits>

#include <cuda_fp16.h>

// The list build returns before the write-back that the other passes of the
// same tile body run (its instantiation has that code unreachable, by design).
#pragma nv_diag_suppress 128

#include "common.cuh"
#include "kernels.cuh"
#include "pairfn.cuh"

namespace examd {

__constant__ OwnLut c_own;

cudaError_t upload_own_lut(const OwnLut& lut) { return cudaMemcpyToSymbol(c_own, &lut, sizeof(OwnLut)); }

constexpr int kDT = 6;        // origin differences for d = -2..3
constexpr int kQueue = 64;    // per-warp queue of accepted pairs
constexpr int kParts = 2;     // work units per 32 staged atoms (1, 3 and 4 measured slower)
// Warps per CTA of the list build, whatever the other passes use: the build
// needs one count word per atom where they keep three force sums, and in the
// room 12 warps fit 3 CTAs on an SM at the tiles of a dense liquid (36 warps
// against 24 with 8), to hide its shared-memory latency.
constexpr int kBuildWarps = 12;
// Fixed-point scale 2^17: each term is rounded to 2^-18 in absolute value.
// With the pairs at the cutoff decided in FP64, the mixed form's error on an
// equilibrated 1M-atom liquid was 2.38e-6 RMS of F_rms at 2^16, about 1.6e-6
// of it the sums' rounding (55 terms an atom at F_rms ~ 35) and the rest the
// FP32 separations; 2^17 halves the rounding share.  Every kept term is below
// kFixMaxForce, so below 2^28 in fixed point: a component's int32 sum (exact
// modulo 2^32 whatever the order) leaves the range only through more than 8
// near-maximal terms of one sign on one atom, which no physical
// configuration has.
constexpr float kFix = 131072.f;
constexpr float kFixInv = 1.f / 131072.f;
constexpr int kRedoBlocks = 152;       // grid of the redo pass (1 per SM)
// Passes of the mixed form's tile body: the first pass; the redo pass's two
// kinds of tile, one whose large terms were left out (only those are summed
// and added) and one that overflowed the first pass's capacity (computed in
// full at the redo capacity, large terms in an FP32 side array).  Pair-list
// mode: the list build (the first pass's enumeration at the list cutoff,
// writing the tile's pairs instead of their forces), the forces from the
// list, and the redo of a listed tile's large terms.
constexpr int kMain = 0, kRedoBig = 1, kRedoFull = 2, kListBuild = 3, kList = 4, kListBig = 5;
constexpr int kFullBit = 1 << 30;      // redo-list entry: tile | kFullBit for an overflowed tile
constexpr int kSeg = 4;                // lanes per segment of the i-side force sums
constexpr int kMaxListK = 1024;        // pair-list mode: most list entries of one atom
// Mixed form: a pair whose FP32 r^2 lies within this fraction of rc^2 (a few
// times the FP32 separation's rounding) is accepted or not on its FP64 r^2,
// as the FP64 form decides it, so that no pair straddling the cutoff enters
// one form's sums and not the other's (about 1e-4 of an atom's pairs)
constexpr float kBorder = 4e-6f;

// Shared-memory carve-up, identical on host and device.
struct Layout {
  int lstart, gfirst, ox, oy, oz, dyt, dzt, img, cw, r2l, lut, ljt, queue;
  int pf, fa, px, code, fr;
  int perm, hist;  // pair-list passes: the staged atoms by entry count, and the counts' histogram
  int bytes;
};

// Per-warp tables after the accepted-pair queues.  Mixed form: one step's
// items by rank (ptA float4 + ptB) and the work unit's atoms by rank (btA
// float4 + btB); wide: ptB int4, btB float4 of full values; compact: ptB
// int2 with two 16-bit offsets, the atom's squared x-gaps as FP16 rounded
// toward zero (so the pruning stays conservative) and btB int2.  The host
// takes the compact tables where they fit more CTAs on an SM.  FP64 form: one
// step's items by lane (float4).
constexpr int kWarpTabWide = 32 * 16 + 32 * 16 + 32 * 16 + 32 * 16;
constexpr int kWarpTabCompact = 32 * 16 + 32 * 8 + 32 * 16 + 32 * 8;
constexpr int kWarpTabFp64 = 32 * 16;

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// mode: kMain, kRedoBig (fr: the large terms' FP32 sums, over the
// accepted-pair queues, which that pass does not use, when they fit there)
// or kRedoFull (fr after everything else); kListBuild (the per-warp tables
// without queues, the count order and its histogram); kList, kListBig (no
// queues, no ownership table: the queue region holds only the scan and
// reduction scratch; kListBig's fr after everything).
// ne_max, ext_max: the largest tile's ext cells and ext extent on one axis.
__host__ __device__ inline Layout make_layout(bool fp64, int cap, int ne_max, int ext_max, int nw, int mode,
                                              bool pack) {
  const bool from_list = mode == kList || mode == kListBig;
  Layout L;
  int o = 0;
  L.lstart = o; o = align16(o + 2 * (ne_max + 1));  // < 2^16: at most the capacity
  L.gfirst = o; o = align16(o + 4 * ne_max);
  L.ox = o;     o = align16(o + 4 * (ext_max + 1));
  L.oy = o;     o = align16(o + 4 * (ext_max + 1));
  L.oz = o;     o = align16(o + 4 * (ext_max + 1));
  L.dyt = o;    o = align16(o + 8 * ext_max * kDT);  // float2 (row origin offset, near face) per (l, d)
  L.dzt = o;    o = align16(o + 8 * ext_max * kDT);
  L.img = o;    o = align16(o + (fp64 ? 3 * 32 : 0));  // periodic image per ext coordinate (FP64 form)
  L.cw = o;     o = align16(o + 16);  // unit counter, large-term flag, staged-atom total
  L.r2l = o;    o = align16(o + (fp64 ? 64 * nw : 0));  // rank -> lane tables (FP64 form)
  L.lut = o;    o = align16(o + (from_list ? 0 : (int)sizeof(OwnLut)));
  // the LJ table per ordered type pair (several types): per-lane type indices
  // would serialise on the kernel-parameter bank, shared memory serves them at once
  L.ljt = o;    o = align16(o + (int)sizeof(LJ64) * EXAMD_MAX_TYPES * EXAMD_MAX_TYPES);
  const int tab = pack ? kWarpTabCompact : kWarpTabWide;
  const int qbytes = (fp64 ? 4 * kQueue + kWarpTabFp64
                           : (from_list ? 64 : (mode == kListBuild ? 0 : 16) * kQueue + tab)) * nw;
  L.queue = o;  o = align16(o + qbytes);
  L.pf = o;     o = align16(o + 16 * (from_list ? cap + 1 : cap));  // list passes: + the padding atom
  if (fp64) {
    L.fa = o;   o = align16(o + 3 * 8 * cap);  // FP64 force sums
    L.px = o;   o = align16(o + 3 * 8 * cap);  // FP64 positions
  } else {
    L.fa = o;   o = align16(o + (mode == kListBuild ? 1 : 3) * 4 * cap);  // fixed-point force sums (build: counts)
    L.px = o;
  }
  L.code = o;   o = align16(o + 2 * cap);
  L.perm = L.hist = o;
  if (mode == kListBuild) {  // the build orders the atoms by entry count, at its end:
    // in the per-warp tables' region, which the enumeration no longer uses then, if it fits
    if (align16(2 * cap) + 4 * (kMaxListK + 1) <= qbytes) {
      L.perm = L.queue;
      L.hist = L.queue + align16(2 * cap);
    } else {
      L.perm = o; o = align16(o + 2 * cap);
      L.hist = o; o = align16(o + 4 * (kMaxListK + 1));
    }
  }
  L.fr = L.queue;
  if (!fp64 && (mode == kRedoFull || mode == kListBig || (mode == kRedoBig && 3 * 4 * cap > 16 * kQueue * nw))) {
    L.fr = o;   o = align16(o + 3 * 4 * cap);
  }
  L.bytes = o;
  return L;
}

static int redo_smem_bytes(const PairConfig& cfg, int cap_redo, int ne_max, int ext_max) {
  const int b = std::max(make_layout(false, cap_redo, ne_max, ext_max, cfg.warps, kRedoBig, cfg.pack).bytes,
                         make_layout(false, cap_redo, ne_max, ext_max, cfg.warps, kRedoFull, cfg.pack).bytes);
  return cfg.list ? std::max(b, make_layout(false, cap_redo, ne_max, ext_max, cfg.warps, kListBig, cfg.pack).bytes)
                  : b;
}

// The first pass's layout: the enumeration's, or in pair-list mode (without
// counters, which the enumeration gives) the list pass's.
static int main_smem_bytes(const PairConfig& cfg, int cap, int ne_max, int ext_max) {
  const int mode = (cfg.list && !cfg.count && !cfg.fp64) ? kList : kMain;
  return make_layout(cfg.fp64, cap, ne_max, ext_max, cfg.warps, mode, cfg.pack).bytes;
}

static int build_smem_bytes(const PairConfig& cfg, int cap, int ne_max, int ext_max) {
  return make_layout(false, cap, ne_max, ext_max, kBuildWarps, kListBuild, cfg.pack).bytes;
}

int pair_smem_bytes(const PairConfig& cfg, int cap, int cap_redo, int ne_max, int ext_max) {
  int b = make_layout(cfg.fp64, cap, ne_max, ext_max, cfg.warps, kMain, cfg.pack).bytes;
  if (cfg.fp64) return b;
  b = std::max(b, redo_smem_bytes(cfg, cap_redo, ne_max, ext_max));
  if (cfg.list) b = std::max(b, std::max(main_smem_bytes(cfg, cap, ne_max, ext_max),
                                         build_smem_bytes(cfg, cap, ne_max, ext_max)));
  return b;
}

// Exact sum of FP32 terms in 64-bit fixed point (2^-32 resolution): the total
// does not depend on the order of the terms.  A term of magnitude >= 30000
// (a pair closer than ~0.46 sigma) goes to an FP32 side sum.
struct FixSum {
  long long v = 0;
  float side = 0.f;
  __device__ __forceinline__ void add(float x) {
    if (fabsf(x) < 30000.f) {
      const float hs = x * 65536.f;  // exact power-of-two scaling
      const int h = __float2int_rz(hs);
      const int l = __float2int_rn((hs - (float)h) * 65536.f);  // hs - h is exact
      v += ((long long)h << 16) + l;
    } else {
      side += x;
    }
  }
};

// The force of one accepted pair per lane (act), from registers: d = x_j -
// x_i with d.w = r^2, P the type pair's parameters; i = -1 on a lane outside
// the batch, which also ends any run of equal i.  Lanes that hold a pair
// that was not accepted keep their i, add nothing, and do not break the run.
template <bool ENERGY, bool COUNT, bool SIDE, class FA, class FR>
__device__ __forceinline__ void pair_force32(bool act, int i, int m, float4 d, const LJ32& P, FA& fa, FR& fr,
                                             int cap, const PairArgs& A, FixSum& ek, FixSum& wk, int& nacc,
                                             int* big_flag) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  bool big = false;
  if (act) {
    big = d.w < P.r2big;  // left to the redo pass
    float dg = 0.f, e = 0.f;
    const int rv = pair_fn32<ENERGY>(A.lj.pot, d.w, P, dg, e);
    if (rv == 0) {
      const float dgs = kFix * dg;
      fx = dgs * d.x;
      fy = dgs * d.y;
      fz = dgs * d.z;
      if (ENERGY) {
        ek.add(e);
        wk.add(-dg * d.w);
      }
      if (COUNT) ++nacc;
    } else if (rv < 0) {
      atomicOr(A.status, ST_PAIRFN);
    }
  }
  int ix = 0, iy = 0, iz = 0;
  if (act && !big) {
    ix = __float2int_rn(fx);
    iy = __float2int_rn(fy);
    iz = __float2int_rn(fz);
    atomicAdd(&fa[m], -ix);
    atomicAdd(&fa[cap + m], -iy);
    atomicAdd(&fa[2 * cap + m], -iz);
  }
  if (big) {
    if (SIDE) {
      atomicAdd(&fr[i], fx * kFixInv);
      atomicAdd(&fr[cap + i], fy * kFixInv);
      atomicAdd(&fr[2 * cap + i], fz * kFixInv);
      atomicAdd(&fr[m], -fx * kFixInv);
      atomicAdd(&fr[cap + m], -fy * kFixInv);
      atomicAdd(&fr[2 * cap + m], -fz * kFixInv);
    } else {
      *big_flag = 1;
    }
  }
  // i side: sum over runs of equal i (lanes outside the batch form one run
  // with i = -1), in segments of kSeg lanes from the run's first one: each
  // segment's last lane adds the segment's total (4: measured against 2, 8
  // and 16)
  const int ip = __shfl_up_sync(FULL, i, 1);
  const unsigned hb = __ballot_sync(FULL, lane == 0 || ip != i);
  const int dist = (lane - (31 - __clz(hb & (FULL >> (31 - lane))))) & (kSeg - 1);
#pragma unroll
  for (int o = 1; o < kSeg; o <<= 1) {
    const int yx = __shfl_up_sync(FULL, ix, o), yy = __shfl_up_sync(FULL, iy, o), yz = __shfl_up_sync(FULL, iz, o);
    if (o <= dist) {
      ix += yx;
      iy += yy;
      iz += yz;
    }
  }
  const bool tail = lane == 31 || dist == kSeg - 1 || ((hb >> (lane + 1)) & 1u);
  if (i >= 0 && tail && (ix | iy | iz) != 0) {
    atomicAdd(&fa[i], ix);
    atomicAdd(&fa[cap + i], iy);
    atomicAdd(&fa[2 * cap + i], iz);
  }
}

// Forces of cnt queued accepted pairs, one per lane: entry = (d = x_j - x_i,
// key) with key = i | j << 14 | type_i << 28 | type_j << 30; r^2 is recomputed
// with the distance test's expression, so it has the same bits.  user_func.f90:58-69
// in FP32: dg = -24 eps (2 s^12 - s^6) / r^2, f_i += dg d, f_j -= dg d.
// The queue keeps an atom's accepted pairs next to each other, so the i-side
// fixed-point terms are first summed over segments of each run of lanes with
// the same i (a segmented shuffle scan; integer sums, so the result is exact)
// and each segment's last lane adds its total: one shared atomic per segment
// instead of one per pair on the same address.
// A pair-force term too large for the fixed-point sums (|F| >= kFixMaxForce,
// decided on r^2 < r2big of the type pair: r < ~0.74 sigma at eps = 1, which
// thermal configurations do not reach) is left out here and raises the
// tile's flag (*big_flag); the redo pass adds it.  SIDE (the full redo pass):
// such terms go to the FP32 side sums fr instead.
template <bool MULTI, bool ENERGY, bool COUNT, bool SIDE, class QD, class FA, class FR>
__device__ __forceinline__ void force_batch(int cnt, int qh, const QD& qd, FA& fa, FR& fr, int cap, const PairArgs& A,
                                            const LJ32* ljs, FixSum& ek, FixSum& wk, int& nacc, int* big_flag) {
  const int lane = threadIdx.x & 31;
  const bool act = lane < cnt;
  int i = -1, m = 0;
  float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
  LJ32 P = A.lj.p32[0];
  if (act) {
    const int slot = (qh + lane) & (kQueue - 1);
    d = qd[slot];
    const unsigned key = __float_as_uint(d.w);
    d.w = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));  // r^2 exactly as the distance test computed it
    i = key & 0x3fff;
    m = (key >> 14) & 0x3fff;
    if (MULTI) P = ljs[((key >> 28) & 3) * A.lj.nt + (key >> 30)];
  }
  pair_force32<ENERGY, COUNT, SIDE>(act, i, m, d, P, fa, fr, cap, A, ek, wk, nacc, big_flag);
}

// FP64 form: the reference's arithmetic for cnt queued pairs that passed the
// FP32 prefilter, one per lane (key as in force_batch).  The separation is
// x_j - x_i plus the difference of the two staged copies' periodic images,
// (n_j - n_i) L, which is exact (Sterbenz) and equals the reference's
// dx - Nint(dx/L) L (SRC/exaMD_forces.f90:509-523); then user_func.f90:52-69.
template <bool MULTI, bool ENERGY, bool COUNT, class QK, class PD, class CODE, class IMG, class FD>
__device__ __forceinline__ void force_batch64(int cnt, const QK& qk, const PD& pd, const CODE& code, const IMG& img,
                                              const double* Lbox, FD& fd, int cap, const LJTable& lj,
                                              const LJ64* ljs, double& esum, double& wsum, int* status, int& nacc,
                                              int qh) {
  const int lane = threadIdx.x & 31;
  if (lane >= cnt) return;
  const unsigned key = (unsigned)qk[(qh + lane) & (kQueue - 1)];
  const int i = key & 0x3fff, m = (key >> 14) & 0x3fff;
  const int ci = code[i], cm = code[m];
  // difference of the copies' periodic images per axis: -1, 0 or +1 box
  const int nx = img[cm & 31] - img[ci & 31];
  const int ny = img[32 + ((cm >> 5) & 31)] - img[32 + ((ci >> 5) & 31)];
  const int nz = img[64 + (cm >> 10)] - img[64 + (ci >> 10)];
  double dx = __dsub_rn(pd[m], pd[i]);
  double dy = __dsub_rn(pd[cap + m], pd[cap + i]);
  double dz = __dsub_rn(pd[2 * cap + m], pd[2 * cap + i]);
  if (nx) dx = __dadd_rn(dx, nx > 0 ? Lbox[0] : -Lbox[0]);
  if (ny) dy = __dadd_rn(dy, ny > 0 ? Lbox[1] : -Lbox[1]);
  if (nz) dz = __dadd_rn(dz, nz > 0 ? Lbox[2] : -Lbox[2]);
  const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  LJ64 P = lj.p64[0];
  if (MULTI) P = ljs[((key >> 28) & 3) * lj.nt + (key >> 30)];
  double dg = 0.0, e = 0.0;
  const int rv = pair_fn64<ENERGY>(lj.pot, d2, P, dg, e);
  if (rv == 0) {
    const double fx = __dmul_rn(dg, dx), fy = __dmul_rn(dg, dy), fz = __dmul_rn(dg, dz);
    atomicAdd(&fd[i], fx);
    atomicAdd(&fd[cap + i], fy);
    atomicAdd(&fd[2 * cap + i], fz);
    atomicAdd(&fd[m], -fx);
    atomicAdd(&fd[cap + m], -fy);
    atomicAdd(&fd[2 * cap + m], -fz);
    if (ENERGY) {
      esum += e;
      wsum += -__dmul_rn(dg, d2);
    }
    if (COUNT) ++nacc;
  } else if (rv < 0) {
    atomicOr(status, ST_PAIRFN);
  }
}

// One tile.  MODE (mixed form; the FP64 form has only kMain):
// - kMain: the first pass, at capacity A.cap; a tile with more staged atoms
//   is listed for a full redo, one with a large term for a large-term redo;
// - kRedoBig (without energy or counters): recomputes the tile's pairs, sums
//   only the large terms (FP32 shared atomics) and adds them to the outputs
//   that the first pass wrote;
// - kRedoFull: the whole tile at capacity A.cap_redo, large terms in FP32
//   side sums, outputs, energy and counters written as the first pass would.
// Pair-list mode:
// - kListBuild: the first pass's enumeration at the list cutoff (rl2, with
//   prune2_list), which writes the tile's accepted pairs as staged-index
//   entries to its list instead of computing them; a tile over capacity or
//   with more pairs than its list holds goes to the fallback list;
// - kList: the tile's forces from its list, with the same per-pair FP32
//   expressions as the first pass (the same bits when the atoms are where
//   the list was built), outputs, energy and the large-term flag as there;
// - kListBig: kRedoBig from the list.
// CUT (list pass): the potential's own range rcut2 is tested (WCA; infinite otherwise).
template <bool FP64, bool MULTI, bool ENERGY, bool COUNT, int MODE, bool PACK, bool CUT = true>
__device__ __forceinline__ void pair_tile(const PairArgs& A, const int tile) {
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int4 t0 = A.tiles[2 * tile], t1 = A.tiles[2 * tile + 1];
  const BoxDev& B = A.boxes[t0.x];
  const int X0 = t0.y, Y0 = t0.z, Z0 = t0.w;
  const int tx = t1.x, ty = t1.y, tz = t1.z;
  const int EX = tx + 2, EY = ty + 2, EZ = tz + 2;
  const int NE = EX * EY * EZ;
  constexpr bool kFromList = MODE == kList || MODE == kListBig;
  if (kFromList && MODE == kList && A.lcount[tile] < 0) return;  // a fallback tile: the redo pass computes it
  const int cap = (MODE == kMain || MODE == kListBuild || MODE == kList) ? A.cap : A.cap_redo;
  const Layout L = make_layout(FP64, cap, A.ne_max, A.ext_max, nw, MODE, PACK);
  // shared-memory arrays (index-checked in the checked build)
  int* const st = A.status;  // the index checks' status word (checked build)
  (void)st;
  auto lstart = EXAMD_ARR(unsigned short, smem + L.lstart, A.ne_max + 1, st);
  auto gfirst = EXAMD_ARR(int, smem + L.gfirst, A.ne_max, st);
  auto ox = EXAMD_ARR(float, smem + L.ox, A.ext_max + 1, st);
  auto oy = EXAMD_ARR(float, smem + L.oy, A.ext_max + 1, st);
  auto oz = EXAMD_ARR(float, smem + L.oz, A.ext_max + 1, st);
  auto dyt = EXAMD_ARR(float2, smem + L.dyt, A.ext_max * kDT, st);
  auto dzt = EXAMD_ARR(float2, smem + L.dzt, A.ext_max * kDT, st);
  auto img = EXAMD_ARR(signed char, smem + L.img, FP64 ? 96 : 1, st);
  double* red = (double*)(smem + L.queue);  // scan and reduction scratch, before and after the queues' use
  int* cw = (int*)(smem + L.cw);
  OwnLut* sown = (OwnLut*)(smem + L.lut);
  const signed char* srows = &sown->rows[0][0];
  LJ32* ljs32 = (LJ32*)(smem + L.ljt);
  LJ64* ljs64 = (LJ64*)(smem + L.ljt);
  auto pf = EXAMD_ARR(float4, smem + L.pf, kFromList ? cap + 1 : cap, st);
  auto code = EXAMD_ARR(unsigned short, smem + L.code, cap, st);
  auto U = EXAMD_ARR(const float4, A.U, A.N, st);

  // (1) ext cells: global cell, count, first atom; ownership tables to smem
  for (int e = tid; e < NE; e += blockDim.x) {
    int lx = e % EX, rr = e / EX, ly = rr % EY, lz = rr / EY;
    int gx = X0 + lx - 1, gy = Y0 + ly - 1, gz = Z0 + lz - 1;
    gx += (gx < 0) ? B.nb[0] : 0;
    gx -= (gx >= B.nb[0]) ? B.nb[0] : 0;
    gy += (gy < 0) ? B.nb[1] : 0;
    gy -= (gy >= B.nb[1]) ? B.nb[1] : 0;
    gz += (gz < 0) ? B.nb[2] : 0;
    gz -= (gz >= B.nb[2]) ? B.nb[2] : 0;
    int gc = B.cell0 + gx + B.nb[0] * (gy + B.nb[1] * gz);
    int s0 = A.cstart[gc];
    gfirst[e] = s0;
    lstart[e] = (unsigned short)min(A.cstart[gc + 1] - s0, 0xffff);  // a larger count overflows any capacity
  }
  {
    const uint4* src = reinterpret_cast<const uint4*>(&c_own);
    uint4* dst = reinterpret_cast<uint4*>(sown);
    if (!kFromList)
      for (int k = tid; k < (int)(sizeof(OwnLut) / 16); k += blockDim.x) dst[k] = src[k];
    if (MULTI)
      for (int k = tid; k < A.lj.nt * A.lj.nt; k += blockDim.x) {
        if (FP64)
          ljs64[k] = A.lj.p64[k];
        else
          ljs32[k] = A.lj.p32[k];
      }
  }
  // Per-axis tables.  Ext coordinate l (cell X0 + l - 1, l = 0..E; l = E is
  // the far edge of the last ext cell) has origin (g0 + l - 1)*bl + n*r, with
  // n = -1, 0, +1 its periodic image and r = L - nb*bl the extra width of the
  // box's last cell.  o*[l]: origin relative to the tile centre, FP32 (the
  // multiple of bl is exact, so the value is rounded once).  d*t[l*6 + d + 2]
  // (y, z): the origin difference between ext rows l and l + d (d = -2..3),
  // rounded once, and o*[l + d + (d < 0)], the near face of row l + d seen
  // from row l (the same value as the o* entry).  img[32a + l] (FP64 form): n.
  {
    const int a = tid >> 5, l = tid & 31;
    if (a < 3) {
      const int E = a == 0 ? EX : (a == 1 ? EY : EZ);
      const int g0 = a == 0 ? X0 : (a == 1 ? Y0 : Z0);
      const int t = a == 0 ? tx : (a == 1 ? ty : tz);
      const int nb = B.nb[a];
      const float blf = B.blf, rf = B.remf[a];
      auto nimg = [&](int ll) {
        const int g = g0 + ll - 1;
        return g < 0 ? -1 : (g >= nb ? 1 : 0);
      };
      if (l <= E) {
        const int n = nimg(l);
        (a == 0 ? ox : (a == 1 ? oy : oz))[l] = fmaf((float)(2 * (l - 1) - t), 0.5f * blf, (float)n * rf);
        if (l < E) {
          if (FP64) img[32 * a + l] = (signed char)n;
          if (a > 0) {
            auto dt = a == 1 ? dyt : dzt;
#pragma unroll
            for (int d = -2; d <= 3; ++d) {
              const int l2 = l + d, ln = l + d + (d < 0);
              const float off = (l2 >= 0 && l2 <= E) ? fmaf((float)(nimg(l2) - n), rf, (float)d * blf) : 0.f;
              const float near =
                  (ln >= 0 && ln <= E) ? fmaf((float)(2 * (ln - 1) - t), 0.5f * blf, (float)nimg(ln) * rf) : 0.f;
              dt[l * kDT + d + 2] = make_float2(off, near);
            }
          }
        }
      }
    }
  }
  __syncthreads();

  // (2) exclusive scan of the ext-cell counts
  {
    const int per = (NE + blockDim.x - 1) / blockDim.x;
    const int b = tid * per, e = min(b + per, NE);
    int s = 0;
    for (int k = b; k < e; ++k) s += lstart[k];
    int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    int* wsum = (int*)red;
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; ++w) base += wsum[w];
    int run = base + x - s;
    for (int k = b; k < e; ++k) {
      int c = lstart[k];
      lstart[k] = run;
      run += c;
    }
    if (tid == blockDim.x - 1) {
      lstart[NE] = (unsigned short)run;
      cw[2] = run;
    }
    __syncthreads();
  }
  const int total = cw[2];
  if (kFromList && A.lcount[tile] != total) {  // the lists of another binning: not computed from
    if (tid == 0) atomicOr(A.status, ST_BOUNDS);
    return;
  }
  if (kFromList && !(A.lj.pot == EXAMD_POT_LJ || A.lj.pot == EXAMD_POT_LJ_SHIFTED || A.lj.pot == EXAMD_POT_WCA)) {
    if (tid == 0) atomicOr(A.status, ST_PAIRFN);  // a potential the list passes do not evaluate
    return;
  }
  if (MODE == kListBuild && (total > cap || total > A.lslots)) {  // no list: the redo pass enumerates it every step
    if (tid == 0) {
      A.lcount[tile] = -1;
      A.fb[atomicAdd(&A.lw[LW_FBN], 1)] = tile;
    }
    return;
  }
  if (!FP64 && MODE == kMain && total > cap) {  // the redo pass computes it at its capacity
    if (tid == 0) A.redo[atomicAdd(A.redo_n, 1)] = tile | kFullBit;
    return;
  }
  if (total > cap) {
    if (tid == 0) {
      atomicOr(A.status, ST_OVERFLOW);
      if (ENERGY) {
        A.tileE[tile] = 0.0;
        A.tileW[tile] = 0.0;
      }
      if (COUNT) {
        A.tileC[3 * tile] = 0;
        A.tileC[3 * tile + 1] = 0;
        A.tileC[3 * tile + 2] = 0;
      }
    }
    return;
  }
  // (3) stage atoms, one thread per ext cell
  auto fa = EXAMD_ARR(int, smem + L.fa, (MODE == kListBuild ? 1 : 3) * cap, st);
  auto fr = EXAMD_ARR(float, smem + L.fr, 3 * cap, st);  // redo pass: FP32 sums of the large terms
  auto fd = EXAMD_ARR(double, smem + L.fa, 3 * cap, st);
  auto pd = EXAMD_ARR(double, smem + L.px, 3 * cap, st);
  for (int e = tid; e < NE; e += blockDim.x) {
    const int lx = e % EX, rr = e / EX, ly = rr % EY, lz = rr / EY;
    const int a0 = lstart[e], a1 = lstart[e + 1], g0 = gfirst[e];
    const unsigned short cc = (unsigned short)(lx | (ly << 5) | (lz << 10));
    for (int t = a0; t < a1; ++t) {
      const int g = g0 + (t - a0);
      const float4 u = U[g];
      if (FP64) {
        pf[t] = make_float4(ox[lx] + u.x, oy[ly] + u.y, oz[lz] + u.z, u.w);
        pd[t] = A.X0[EXAMD_IDX(g, A.N, st)];
        pd[cap + t] = A.X1[EXAMD_IDX(g, A.N, st)];
        pd[2 * cap + t] = A.X2[EXAMD_IDX(g, A.N, st)];
#pragma unroll
        for (int c = 0; c < 3; ++c) fd[c * cap + t] = 0.0;
      } else {
        // from a list: the type and the ext-cell code in w (the list pass
        // reads both atoms' rows from them)
        pf[t] = make_float4(ox[lx] + u.x, u.y, u.z,
                            kFromList ? __int_as_float((__float_as_int(u.w) & 3) | ((int)cc << 2)) : u.w);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (MODE == kRedoBig || MODE == kRedoFull || MODE == kListBig) fr[c * cap + t] = 0.f;
          // (list build: fa holds the atoms' entry counts, one word each)
          if (MODE == kMain || MODE == kRedoFull || MODE == kList || (MODE == kListBuild && c == 0))
            fa[c * cap + t] = 0;
        }
      }
      code[t] = cc;
    }
  }
  int* big_flag = cw + 1;  // mixed form: a term was too large for the fixed-point sums
  // list passes: the padding entries' atom, beyond every cutoff
  if (kFromList && tid == 0) pf[total] = make_float4(1e30f, 0.f, 0.f, 0.f);
  if (tid == 0) {
    cw[0] = 0;  // work-unit counter
    cw[3] = 0;  // list build: the tile's entries so far
    *big_flag = 0;
  }
  __syncthreads();

  const LJ32 q32 = A.lj.p32[0];
  const float rcpre = A.lj.rc2max * 1.0001f + 1e-4f;  // FP32 prefilter of the FP64 form
  double esum = 0.0, wsum = 0.0;  // FP64 form
  FixSum ek, wk;                  // mixed form: exact fixed-point sums of FP32 terms
  int ncand = 0, neval = 0, nacc = 0;
  // per-warp queue of accepted pairs (mixed form: the separation and the key
  // in one 16-byte entry, r^2 recomputed from it; FP64 form: the key only)
  // bytes per queue entry (the list build writes its pairs to the lists directly)
  constexpr int kQe = FP64 ? 4 : (MODE == kListBuild ? 0 : 16);
  auto qd = EXAMD_ARR(float4, (float4*)(smem + L.queue) + warp * kQueue, kQueue, st);
  auto qk = EXAMD_ARR(int, (int*)(smem + L.queue) + warp * kQueue, kQueue, st);
  // per-warp tables (kWarpTab*): one step's items (ptA, ptB) and, mixed
  // form, the work unit's atoms (bt)
  unsigned char* wtab =
      smem + L.queue + kQe * kQueue * nw + warp * (FP64 ? kWarpTabFp64 : (PACK ? kWarpTabCompact : kWarpTabWide));
  auto ptA = EXAMD_ARR(float4, wtab, 32, st);
  auto ptB2 = EXAMD_ARR(int2, wtab + 32 * 16, 32, st);  // the compact layout's view
  auto ptB4 = EXAMD_ARR(int4, wtab + 32 * 16, 32, st);  // the wide layout's view
  auto btA = EXAMD_ARR(float4, wtab + (PACK ? 32 * 24 : 32 * 32), 32, st);
  auto btB2 = EXAMD_ARR(int2, wtab + (PACK ? 32 * 40 : 32 * 48), 32, st);
  auto btB4 = EXAMD_ARR(float4, wtab + (PACK ? 32 * 40 : 32 * 48), 32, st);
  int qn = 0, qh = 0;  // queued pairs and the ring's head
  const unsigned lt = (1u << lane) - 1u;
  const unsigned le = FULL >> (31 - lane);
  auto r2l = EXAMD_ARR(unsigned char, smem + L.r2l + 64 * warp, FP64 ? 64 : 1, st);  // FP64 form: two rank -> lane tables of 32
  // ---- accepted pairs go to the warp's queue (a ring of kQueue entries);
  // their forces are computed in full batches of 32 ----
  // list build: an accepted pair (i, m) is entry k of atom i in the scratch
  // (i's entries side by side, lk per atom), k from the atom's counter (fa);
  // entries beyond lk are counted, not written (the tile then goes to the
  // fallback list)
  const size_t ltile = (size_t)tile * A.lslots;
  auto list_add = [&](bool acc, int key) {
    if (!acc) return;
    const int i = key & 0x3fff, m = (key >> 14) & 0x3fff;
    const int k = atomicAdd(&fa[i], 1);
    if (k < A.lk)
      A.lraw[EXAMD_IDX((ltile + i) * A.lk + k, (size_t)A.ntiles * A.lslots * A.lk, st)] = (unsigned short)m;
  };
  auto enqueue = [&](bool acc, const float4& dq, int key) {
    const unsigned bal = __ballot_sync(FULL, acc);
    if (acc) {
      const int p = (qh + qn + __popc(bal & lt)) & (kQueue - 1);
      if (FP64)
        qk[p] = key;
      else
        qd[p] = make_float4(dq.x, dq.y, dq.z, __int_as_float(key));
    }
    qn += __popc(bal);
    if (qn >= 32) {  // a batch only moves the ring's head
      __syncwarp();
      if (FP64)
        force_batch64<MULTI, ENERGY, COUNT>(32, qk, pd, code, img, B.L, fd, cap, A.lj, ljs64, esum, wsum, A.status,
                                            nacc, qh);
      else
        force_batch<MULTI, ENERGY, COUNT, MODE == kRedoFull>(32, qh, qd, fa, fr, cap, A, ljs32, ek, wk, nacc,
                                                             big_flag);
      __syncwarp();
      qh = (qh + 32) & (kQueue - 1);
      qn -= 32;
    }
  };

  // ---- mixed form: the FP64 cutoff test of a pair of staged atoms (a, b)
  // at the border, r^2 from the FP64 positions as the FP64 form and the
  // reference form it: the difference, then the periodic image (the pair is
  // far nearer than half a box), SRC/exaMD_forces.f90:509-523 ----
  auto inside64 = [&](int a, int b, int ta, int tb) -> bool {
    auto gidx = [&](int t) {
      const int c = code[t];
      const int e = (c & 31) + EX * (((c >> 5) & 31) + EY * (c >> 10));
      return (int64_t)gfirst[e] + (t - (int)lstart[e]);
    };
    const int64_t ga = EXAMD_IDX(gidx(a), A.N, st), gb = EXAMD_IDX(gidx(b), A.N, st);
    const double* Xs[3] = {A.X0, A.X1, A.X2};
    double d2 = 0.0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      double d = __dsub_rn(Xs[ax][gb], Xs[ax][ga]);
      d = __dsub_rn(d, __dmul_rn(rint(__dmul_rn(d, B.Li[ax])), B.L[ax]));
      d2 = ax == 0 ? __dmul_rn(d, d) : __dadd_rn(d2, __dmul_rn(d, d));
    }
    return d2 <= A.lj.p64[ta * A.lj.nt + tb].rc2;
  };

  // ---- redo pass: the force of each accepted pair at once; only the large
  // terms, decided exactly as force_batch decides them, are summed (both atoms)
  auto redo_pair = [&](bool acc, const float4& dq, int key) {
    if (!acc) return;
    const int i = key & 0x3fff, m = (key >> 14) & 0x3fff;
    LJ32 P = A.lj.p32[0];
    if (MULTI) P = ljs32[((key >> 28) & 3) * A.lj.nt + ((unsigned)key >> 30)];
    float dg = 0.f, e = 0.f;
    if (pair_fn32<false>(A.lj.pot, dq.w, P, dg, e) != 0) return;
    const float dgs = kFix * dg;
    const float fx = dgs * dq.x, fy = dgs * dq.y, fz = dgs * dq.z;
    if (!(dq.w < P.r2big)) return;
    atomicAdd(&fr[i], fx * kFixInv);
    atomicAdd(&fr[cap + i], fy * kFixInv);
    atomicAdd(&fr[2 * cap + i], fz * kFixInv);
    atomicAdd(&fr[m], -fx * kFixInv);
    atomicAdd(&fr[cap + m], -fy * kFixInv);
    atomicAdd(&fr[2 * cap + m], -fz * kFixInv);
  };

  // ---- mixed form: consume one step's (atom, row) items, at most one per
  // lane (nt = 0: none).  The items' candidate pairs are laid end to end and
  // the warp walks them 32 at a time, one pair per lane, so no lane idles
  // while another finishes a long j-range.  A lane finds its item from the
  // bitmask of the items that start in the current 32 candidates, and reads
  // the item's data from the per-warp tables by its rank.
  auto consume = [&](int i, float cy, float cz, int lo1, int n1, int lo2, int n2) {
    const int nt = n1 + n2;
    const unsigned hb = __ballot_sync(FULL, nt > 0);
    if (hb == 0u) return;
    // exclusive scan of the items' candidate counts
    int incl = nt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const int s0 = incl - nt;
    const int T = __shfl_sync(FULL, incl, 31);
    if (nt > 0) {
      // the atom's position moved into the j-cells' frame: d = x_j + C
      // (y, z relative to the cell origin; cy, cz: the j-row's origin offset)
      const float4 pi = pf[i];
      // by rank: the item's key base and frame shift, and the offsets that map
      // candidate k to its staged atom: m = k + (k < e1 ? o1 : o2)
      const int rk = __popc(hb & lt);
      ptA[rk] = make_float4(-pi.x, cy - pi.y, cz - pi.z, __int_as_float(MULTI ? i | (__float_as_int(pi.w) << 28) : i));
      if (PACK)
        ptB2[rk] = make_int2(((lo1 - s0) & 0xffff) | ((lo2 - n1 - s0) << 16), s0 + n1);
      else
        ptB4[rk] = make_int4(lo1 - s0, s0 + n1, lo2 - n1 - s0, 0);
    }
    __syncwarp();
    // distance tests; accepted pairs go to the queue
    int qb = 0;  // items that start before K
    const int sw = nt > 0 ? s0 >> 5 : -1;  // the 32-candidate window in which the item starts
    const unsigned sbit = 1u << (s0 & 31);
    for (int K = 0, kw = 0; K < T; K += 32, ++kw) {
      const unsigned M = __reduce_or_sync(FULL, sw == kw ? sbit : 0u);
      const int qr = qb + __popc(M & le) - 1;  // >= 0: the first item starts at 0
      qb += __popc(M);
      const float4 a = ptA[qr];
      int o1, e1, o2;
      if (PACK) {
        const int2 b = ptB2[qr];
        o1 = (int)(short)(b.x & 0xffff);
        o2 = b.x >> 16;
        e1 = b.y;
      } else {
        const int4 b = ptB4[qr];
        o1 = b.x;
        e1 = b.y;
        o2 = b.z;
      }
      const int k = K + lane;
      const bool valid = k < T;
      const int m = (k < e1 ? o1 : o2) + k;
      const float4 pj = pf[valid ? m : 0];
      float4 dq;
      dq.x = pj.x + a.x;
      dq.y = pj.y + a.y;
      dq.z = pj.z + a.z;
      dq.w = fmaf(dq.x, dq.x, fmaf(dq.y, dq.y, dq.z * dq.z));
      const int tj = __float_as_int(pj.w);
      const int kb = __float_as_int(a.w);
      if (COUNT && valid) ++neval;
      const float thr = MODE == kListBuild ? (MULTI ? ljs32[((kb >> 28) & 3) * A.lj.nt + tj].rl2 : q32.rl2)
                                           : (MULTI ? ljs32[((kb >> 28) & 3) * A.lj.nt + tj].rc2 : q32.rc2);
      // disjoint bit fields: the sum is the OR, in one instruction
      const int key = (int)((unsigned)kb + ((unsigned)m << 14) + (MULTI ? (unsigned)tj << 30 : 0u));
      bool acc = valid && dq.w <= thr;
      if ((MODE == kMain || MODE == kRedoFull) && valid && fabsf(dq.w - thr) <= kBorder * thr)
        acc = inside64(kb & 0x3fff, m, MULTI ? (kb >> 28) & 3 : 0, MULTI ? tj : 0);  // at the border: FP64
      if (MODE == kRedoBig)
        redo_pair(acc, dq, key);
      else if (MODE == kListBuild)
        list_add(acc, key);
      else
        enqueue(acc, dq, key);
    }
    __syncwarp();
  };

  // ---- FP64 form: consume one step's (ext cell, row) blocks ----
  // Item (at most one per lane): atoms [i0, i0 + ni) of one cell against the
  // j-range(s) [lo1, lo1 + n1) and [lo2, lo2 + n2) of one owned row; in the
  // row through the cell itself (self) only j > i.  The items' ni * nj
  // candidate pairs are laid end to end and tested 32 at a time, one per lane,
  // against the FP32 prefilter.  A lane finds its item from the bitmask of
  // item starts and splits its index into (i, j) by a float division
  // corrected to the exact quotient.  Consecutive queued pairs then share an
  // i only within one block (a few pairs), which keeps the FP64 batches'
  // shared-memory atomics on i from serialising; the atom-item order of the
  // mixed form would put one atom's whole row list (~30 pairs) in a batch.
  auto consume_cells = [&](int i0, int ni, int lo1, int n1, int lo2, int n2, bool self) {
    const int nj = n1 + n2;
    const int nt = ni * nj;
    const unsigned hb = __ballot_sync(FULL, nt > 0);
    if (hb == 0u) return;
    int incl = nt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const int s0 = incl - nt;
    const int T = __shfl_sync(FULL, incl, 31);
    const int pa = i0 | (ni << 16), p1 = lo1 | (n1 << 16), l2 = lo2 - n1, pn = nj | (self ? 1 << 16 : 0);
    if (nt > 0) {
      ptA[lane] = make_float4(0.f, 0.f, 1.0f / (float)nj, __int_as_float(s0));
      r2l[32 + __popc(hb & lt)] = (unsigned char)lane;
    }
    __syncwarp();
    int qb = 0;  // items that start before K
    const int sw = nt > 0 ? s0 >> 5 : -1;  // the 32-candidate window in which the item starts
    const unsigned sbit = 1u << (s0 & 31);
    for (int K = 0, kw = 0; K < T; K += 32, ++kw) {
      const unsigned M = __reduce_or_sync(FULL, sw == kw ? sbit : 0u);
      const int qr = qb + __popc(M & le) - 1;  // >= 0: the first item starts at 0
      qb += __popc(M);
      const int ql = r2l[32 + qr];
      const int bpa = __shfl_sync(FULL, pa, ql), bp1 = __shfl_sync(FULL, p1, ql);
      const int bl2 = __shfl_sync(FULL, l2, ql), bpn = __shfl_sync(FULL, pn, ql);
      const float4 a = ptA[ql];
      const int k = K + lane;
      const int kl = k - __float_as_int(a.w);
      const int bnj = bpn & 0xffff;
      int ia = __float2int_rz(((float)kl + 0.5f) * a.z);
      int jb = kl - ia * bnj;
      if (jb < 0) {
        --ia;
        jb += bnj;
      } else if (jb >= bnj) {
        ++ia;
        jb -= bnj;
      }
      const bool valid = k < T && (!(bpn >> 16) || jb > ia);
      const int i = (bpa & 0xffff) + ia;
      const int m = jb < (bp1 >> 16) ? (bp1 & 0xffff) + jb : bl2 + jb;
      const float4 pi = pf[valid ? i : 0], pj = pf[valid ? m : 0];
      float4 dq;  // positions are in the tile frame: no row offset
      dq.x = pj.x - pi.x;
      dq.y = pj.y - pi.y;
      dq.z = pj.z - pi.z;
      dq.w = fmaf(dq.x, dq.x, fmaf(dq.y, dq.y, dq.z * dq.z));
      const int ti = __float_as_int(pi.w), tj = __float_as_int(pj.w);
      if (COUNT && valid) {
        ++ncand;
        ++neval;
      }
      enqueue(valid && dq.w <= rcpre, dq, i | (m << 14) | (ti << 28) | (tj << 30));
    }
    __syncwarp();
  };

  int* ucnt = cw;  // work-unit counter
  if constexpr (kFromList) {
    // ---- forces from the tile's lists ----
    // The build ordered the staged atoms by entry count, most first; a warp
    // takes 32 consecutive atoms of that order, one per lane, so its lanes
    // have about as many entries each and few idle while the longest runs
    // out.  A lane reads four entries at a time, the warp's 32 lanes' four
    // side by side (one 256-byte load per warp), the next four loaded
    // ahead.  Entry m of atom i is the pair (i, m).  The separation is
    // formed as the first pass forms it: x in the tile frame, y and z from
    // the atoms' cell offsets and the origin offset between their rows (read
    // from the rows in the staged codes); the same bits when the atoms are
    // where the lists were built.  Atom i's terms add up in registers (exact
    // integer sums) and go to shared memory once; m's go at once.
    const int lk = A.lk;
    const unsigned short* lst = A.list + ltile * lk;
    const unsigned short* perm = A.lperm + ltile;
    const unsigned short* cnts = A.lcnt + ltile;
    const int ng = (total + 31) >> 5;
    bool bigl = false, perr = false;  // a large term left out; a pair-function error
    // The origin offset between rows l and l + d (d = -2..2 for a listed
    // pair) is fmaf(image difference, r, d bl) in the tables: d bl itself
    // (exact) unless the tile reaches the box's periodic face on that axis
    // and the box's last cell is wider by r != 0.  Such tiles read the
    // tables; the others form d bl in registers, the same bits.
    const bool taby = B.remf[1] != 0.f && (Y0 == 0 || Y0 + ty >= B.nb[1]);
    const bool tabz = B.remf[2] != 0.f && (Z0 == 0 || Z0 + tz >= B.nb[2]);
    const float blf = B.blf;
    // d as a float, exactly, without a conversion instruction (|d| < 2^22)
    auto dfloat = [](int d) { return __fsub_rn(__int_as_float(0x4B400000 + d), 12582912.f); };
    while (true) {
      int g = 0;
      if (lane == 0) g = atomicAdd(ucnt, 1);
      g = __shfl_sync(FULL, g, 0);
      if (g >= ng) break;
      const int r = g * 32 + lane;
      const bool vi = r < total;
      const int i = vi ? perm[r] : 0;
      const int cnt = vi ? cnts[r] : 0;
      const int gm = __shfl_sync(FULL, cnt, 0);  // the order puts the group's longest first
      const float4 pi = pf[i];
      const int wi = __float_as_int(pi.w);
      const int ti = wi & 3;
      const int lyi = (wi >> 7) & 31, lzi = (wi >> 12) & 31;
      // entries k..k+3 of this lane: 8 bytes at brick k / 4 of the group
      const uint2* col = reinterpret_cast<const uint2*>(lst + (size_t)g * 32 * lk) + lane;
      // (every lane's bricks hold entries up to the group's longest, the
      // padding entries naming the far atom `total`: no per-lane count test)
      auto four = [&](int k) { return k < gm ? __ldcs(col + (size_t)(k >> 2) * 32) : make_uint2(0u, 0u); };
      uint2 nxt = four(0);
      int sx = 0, sy = 0, sz = 0;  // atom i's fixed-point sums
      // the entries, in one of two versions: row offsets from the tables or
      // formed in registers (no table load)
      auto walk = [&](auto tables) {
      constexpr bool TAB = decltype(tables)::value;
      for (int k0 = 0; k0 < gm; k0 += 4) {
        const uint2 cur = nxt;
        nxt = four(k0 + 4);
        const unsigned wv[2] = {cur.x, cur.y};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int m = (int)((wv[q >> 1] >> (16 * (q & 1))) & 0xffffu);
          const float4 pj = pf[m];
          const int wj = __float_as_int(pj.w);
          const int lyj = (wj >> 7) & 31, lzj = (wj >> 12) & 31;
          // (the table entry of rows l, l + d: l kDT + d + 2)
          float cy, cz;
          if constexpr (TAB) {
            cy = dyt[lyi * (kDT - 1) + 2 + lyj].x;
            cz = dzt[lzi * (kDT - 1) + 2 + lzj].x;
          } else {
            cy = __fmul_rn(dfloat(lyj - lyi), blf);
            cz = __fmul_rn(dfloat(lzj - lzi), blf);
          }
          float4 dq;
          dq.x = pj.x + (-pi.x);
          dq.y = pj.y + (cy - pi.y);
          dq.z = pj.z + (cz - pi.z);
          dq.w = fmaf(dq.x, dq.x, fmaf(dq.y, dq.y, dq.z * dq.z));
          const int tj = wj & 3;
          const LJ32 P = MULTI ? ljs32[ti * A.lj.nt + tj] : q32;
          bool acc = dq.w <= P.rc2;
          if (MODE == kList && fabsf(dq.w - P.rc2) <= kBorder * P.rc2)
            acc = inside64(i, m, ti, tj);  // at the border: the FP64 test
          if (MODE == kListBig) {
            redo_pair(acc, dq, i | (m << 14) | (ti << 28) | (tj << 30));
          } else {
            // The LJ family's expression of pair_fn32 (the potential was
            // checked per tile) for every entry, its result kept where the
            // entry applies: some lane of the warp takes nearly every entry,
            // so a branch would only add reconvergence, and without it the
            // four entries' arithmetic interleaves.  The same expressions:
            // the same bits as pair_fn32 where it applies.
            const float ri = rcp_approx(dq.w);
            const float s2 = P.sig2 * ri;
            const float s6 = s2 * s2 * s2;
            const float dg = P.m24eps * s6 * fmaf(2.f, s6, -1.f) * ri;
            perr |= acc && !(dq.w >= kR2Min32);  // pair_fn32's error return
            const bool app = acc && dq.w >= kR2Min32 && !(CUT && dq.w > P.rcut2);
            if (ENERGY && app) {
              ek.add(P.c4eps * s6 * (s6 - 1.f) - P.eshift);
              wk.add(-dg * dq.w);
            }
            const bool big = app && dq.w < P.r2big;  // left to the redo pass
            bigl |= big;
            const bool fix = app && !big;
            const float dgs = fix ? kFix * dg : 0.f;
            const int ix = __float2int_rn(dgs * dq.x), iy = __float2int_rn(dgs * dq.y),
                      iz = __float2int_rn(dgs * dq.z);
            if (fix) {
              atomicAdd(&fa[m], -ix);
              atomicAdd(&fa[cap + m], -iy);
              atomicAdd(&fa[2 * cap + m], -iz);
            }
            sx += ix;
            sy += iy;
            sz += iz;
          }
        }
      }
      };
      if (taby || tabz)
        walk(std::true_type{});
      else
        walk(std::false_type{});
      if (MODE == kList && (sx | sy | sz) != 0) {
        atomicAdd(&fa[i], sx);
        atomicAdd(&fa[cap + i], sy);
        atomicAdd(&fa[2 * cap + i], sz);
      }
    }
    if (bigl) *big_flag = 1;
    if (perr) atomicOr(A.status, ST_PAIRFN);
  } else if constexpr (!FP64) {
    // ---- item building: (staged atom, owned row) pairs, laid end to end ----
    // A unit is 32 consecutive staged atoms and one of kParts shares of each
    // atom's list of owned rows (the rows whose ownership mask for the atom's
    // position class is nonzero; ordinals n = kParts m + part).  The warp lays
    // the unit's (atom, row) pairs end to end and builds one item per lane per
    // step, so lanes do not idle on atoms that own few rows (the halo).  Units are handed out by a
    // shared counter: their cost varies, and the force sums do not depend on the
    // order.  An item is the atom's j-range(s) in the row: the owned cells,
    // trimmed to those whose box comes within rc of the atom (the 1e-4 margin in
    // prune2 covers the FP32 rounding; the accepted pairs are unchanged).
    const int nunits = kParts * ((total + 31) >> 5);
    const float prune2 = MODE == kListBuild ? A.lj.prune2_list : A.lj.prune2;
    while (true) {
      int u = 0;
      if (lane == 0) u = atomicAdd(ucnt, 1);
      u = __shfl_sync(FULL, u, 0);
      if (u >= nunits) break;
      const int c = u / kParts, part = u - c * kParts;
      // per-atom quantities of lane l's atom c*32 + l
      const int ia = c * 32 + lane;
      const bool va = ia < total;
      const int cia = code[va ? ia : 0];
      const int ax = cia & 31, ay = (cia >> 5) & 31, az = cia >> 10;
      const int acls = pos_class(ax - 1, tx) * 25 + pos_class(ay - 1, ty) * 5 + pos_class(az - 1, tz);
      const int aw = va ? (sown->nrow[acls] + kParts - 1 - part) / kParts : 0;
      const float4 pa = pf[va ? ia : 0];
      const float apy = FP64 ? pa.y : oy[ay] + pa.y;  // tile-frame y, z
      const float apz = FP64 ? pa.z : oz[az] + pa.z;
      // squared x-gaps to the cells dx = -2, -1, +1, +2 (ox has EX + 1 entries)
      const float gm2 = fmaxf(pa.x - ox[max(ax - 1, 0)], 0.f), gm1 = fmaxf(pa.x - ox[ax], 0.f);
      const float gp1 = fmaxf(ox[min(ax + 1, EX)] - pa.x, 0.f), gp2 = fmaxf(ox[min(ax + 2, EX)] - pa.x, 0.f);
      const float am2 = gm2 * gm2, am1 = gm1 * gm1, ap1 = gp1 * gp1, ap2 = gp2 * gp2;
      int incl = aw;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int as0 = incl - aw, W = __shfl_sync(FULL, incl, 31);
      const unsigned wb = __ballot_sync(FULL, aw > 0);
      if (aw > 0) {  // the working atoms' data by rank (as0 < 512, ia < 2^14, acls < 128)
        const int rk = __popc(wb & lt);
        const int wa = as0 | (ia << 9), wc = cia | (acls << 15);
        if (PACK) {
          const __half2 hm = __halves2half2(__float2half_rz(am2), __float2half_rz(am1));
          const __half2 hp = __halves2half2(__float2half_rz(ap1), __float2half_rz(ap2));
          btA[rk] = make_float4(apy, apz, *reinterpret_cast<const float*>(&hm), *reinterpret_cast<const float*>(&hp));
          btB2[rk] = make_int2(wa, wc);
        } else {
          btA[rk] = make_float4(apy, apz, am2, am1);
          btB4[rk] = make_float4(ap1, ap2, __int_as_float(wa), __int_as_float(wc));
        }
      }
      __syncwarp();
      int qb = 0;  // working atoms that start before K
      const int aww = aw > 0 ? as0 >> 5 : -1;  // the 32-item window in which the atom's items start
      const unsigned abit = 1u << (as0 & 31);
      for (int K = 0, kw = 0; K < W; K += 32, ++kw) {
        const unsigned M = __reduce_or_sync(FULL, aww == kw ? abit : 0u);
        const int qr = qb + __popc(M & (FULL >> (31 - lane))) - 1;  // >= 0: the first worker starts at 0
        qb += __popc(M);
        const int k = K + lane;
        const bool valid = k < W;
        const float4 b0v = btA[qr];
        const float py = b0v.x, pz = b0v.y;
        float xm2, xm1, xp1, xp2;
        int sq, cc;
        if (PACK) {
          const float2 gm = __half22float2(*reinterpret_cast<const __half2*>(&b0v.z));
          const float2 gp = __half22float2(*reinterpret_cast<const __half2*>(&b0v.w));
          const int2 b1v = btB2[qr];
          xm2 = gm.x;
          xm1 = gm.y;
          xp1 = gp.x;
          xp2 = gp.y;
          sq = b1v.x;
          cc = b1v.y;
        } else {
          const float4 b1v = btB4[qr];
          xm2 = b0v.z;
          xm1 = b0v.w;
          xp1 = b1v.x;
          xp2 = b1v.y;
          sq = __float_as_int(b1v.z);
          cc = __float_as_int(b1v.w);
        }
        const int s_q = sq & 511, i = sq >> 9;
        const int ci = cc & 0x7fff, cls = cc >> 15;
        const int lx = ci & 31, ly = (ci >> 5) & 31, lz = ci >> 10;
        int r = 0, mask = 0;
        if (valid) {
          r = sown->rlist[cls][kParts * (k - s_q) + part];
          mask = sown->lut[cls][kParts * (k - s_q) + part];
        }
        int lo1 = 0, n1 = 0, lo2 = 0, n2 = 0;
        float cy = 0.f, cz = 0.f;
        if (mask) {
          const int dy = srows[2 * r], dz = srows[2 * r + 1];
          const int rowbase = ((ly + dy) + EY * (lz + dz)) * EX + lx - 2;  // + bit b -> ext cell of dx = b - 2
          const float2 ry = dyt[ly * kDT + dy + 2], rz = dzt[lz * kDT + dz + 2];
          cy = ry.x;
          cz = rz.x;
          if (COUNT) {  // every atom of the owned cells, as the reference visits them
            for (int b = 0; b < 5; ++b)
              if ((mask >> b) & 1) {
                const int e = rowbase + b;
                ncand += (r == kRows - 1 && b == 2) ? lstart[e + 1] - i - 1 : lstart[e + 1] - lstart[e];
              }
          }
          // distance from the atom to the row's cell boxes
          // (the row's near face comes with its origin offset)
          const float ty = ry.y - py, tz = rz.y - pz;
          const float gy = dy == 0 ? 0.f : fmaxf(dy > 0 ? ty : -ty, 0.f);
          const float gz = dz == 0 ? 0.f : fmaxf(dz > 0 ? tz : -tz, 0.f);
          const float g2 = gy * gy + gz * gz;
          const float tr = prune2 - g2;
          if (tr < 0.f) mask = 0;
          mask &= ~((xm2 > tr ? 1 : 0) | (xm1 > tr ? 2 : 0) | (xp1 > tr ? 8 : 0) | (xp2 > tr ? 16 : 0));
          if (mask) {
            const int b0 = __ffs(mask) - 1, b1 = 31 - __clz(mask);
            const int mm = mask >> b0;
            lo1 = lstart[rowbase + b0];
            int hi1 = lstart[rowbase + b1 + 1];
            if (mm & (mm + 1)) {  // two runs: [b0, e1) and [b2, b1]
              const int e1 = b0 + __ffs(~mm) - 1;
              const int b2 = __ffs(mask & ~((1 << e1) - 1)) - 1;
              lo2 = lstart[rowbase + b2];
              n2 = hi1 - lo2;
              hi1 = lstart[rowbase + e1];
            }
            n1 = hi1 - lo1;
            if (r == kRows - 1 && b0 == 2) {  // pairs inside the cell: a2 > a1
              n1 -= i + 1 - lo1;
              lo1 = i + 1;
            }
            if (n1 <= 0) {
              lo1 = lo2;
              n1 = n2;
              lo2 = 0;
              n2 = 0;
            }
          }
        }
        consume(i, cy, cz, lo1, n1, lo2, n2);
      }
      __syncwarp();
    }
  } else {
    // ---- item building: (ext cell, owned row) pairs, laid end to end ----
    // A unit is 32 consecutive ext cells and one of kCellParts shares of each
    // cell's owned rows; empty cells have no work.  An item is the row's owned
    // j-cells as at most two contiguous runs (no per-atom trimming: the block
    // is tested in full).
    constexpr int kCellParts = 4;
    const int nunits = kCellParts * ((NE + 31) >> 5);
    while (true) {
      int u = 0;
      if (lane == 0) u = atomicAdd(ucnt, 1);
      u = __shfl_sync(FULL, u, 0);
      if (u >= nunits) break;
      const int c = u / kCellParts, part = u - c * kCellParts;
      const int e = c * 32 + lane;
      const bool ve = e < NE;
      const int ee = ve ? e : 0;
      const int ex = ee % EX, er = ee / EX, ey = er % EY, ez = er / EY;
      const int ai0 = lstart[ee], ana = ve ? lstart[ee + 1] - ai0 : 0;
      const int acls = pos_class(ex - 1, tx) * 25 + pos_class(ey - 1, ty) * 5 + pos_class(ez - 1, tz);
      const int aw = ana > 0 ? (sown->nrow[acls] + kCellParts - 1 - part) / kCellParts : 0;
      int incl = aw;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int as0 = incl - aw, W = __shfl_sync(FULL, incl, 31);
      const unsigned wb = __ballot_sync(FULL, aw > 0);
      if (aw > 0) r2l[__popc(wb & lt)] = (unsigned char)lane;
      __syncwarp();
      const int ageo = ex | (ey << 5) | (ez << 10) | (acls << 15);
      const int apa = ai0 | (ana << 16);
      int qb = 0;
      const int aww = aw > 0 ? as0 >> 5 : -1;  // the 32-item window in which the cell's items start
      const unsigned abit = 1u << (as0 & 31);
      for (int K = 0, kw = 0; K < W; K += 32, ++kw) {
        const unsigned M = __reduce_or_sync(FULL, aww == kw ? abit : 0u);
        const int qr = qb + __popc(M & le) - 1;
        qb += __popc(M);
        const int k = K + lane;
        const bool valid = k < W;
        const int ql = r2l[qr];
        const int s_q = __shfl_sync(FULL, as0, ql);
        const int geo = __shfl_sync(FULL, ageo, ql);
        const int qpa = __shfl_sync(FULL, apa, ql);
        const int lx = geo & 31, ly = (geo >> 5) & 31, lz = (geo >> 10) & 31, cls = geo >> 15;
        int r = 0, mask = 0;
        if (valid) {
          r = sown->rlist[cls][kCellParts * (k - s_q) + part];
          mask = sown->lut[cls][kCellParts * (k - s_q) + part];
        }
        int lo1 = 0, n1 = 0, lo2 = 0, n2 = 0;
        bool self = false;
        if (mask) {
          const int dy = srows[2 * r], dz = srows[2 * r + 1];
          const int rowbase = ((ly + dy) + EY * (lz + dz)) * EX + lx - 2;  // + bit b -> ext cell of dx = b - 2
          const int b0 = __ffs(mask) - 1, b1 = 31 - __clz(mask);
          const int mm = mask >> b0;
          lo1 = lstart[rowbase + b0];
          int hi1 = lstart[rowbase + b1 + 1];
          if (mm & (mm + 1)) {  // two runs: [b0, e1) and [b2, b1]
            const int e1 = b0 + __ffs(~mm) - 1;
            const int b2 = __ffs(mask & ~((1 << e1) - 1)) - 1;
            lo2 = lstart[rowbase + b2];
            n2 = hi1 - lo2;
            hi1 = lstart[rowbase + e1];
          }
          n1 = hi1 - lo1;
          self = r == kRows - 1 && b0 == 2;  // the first run starts at the cell itself
          if (n1 <= 0 && !self) {
            lo1 = lo2;
            n1 = n2;
            lo2 = 0;
            n2 = 0;
          }
        }
        consume_cells(qpa & 0xffff, qpa >> 16, lo1, n1, lo2, n2, self);
      }
      __syncwarp();
    }
  }
  if (qn > 0) {  // the last, partial batch
    __syncwarp();
    if (FP64)
      force_batch64<MULTI, ENERGY, COUNT>(qn, qk, pd, code, img, B.L, fd, cap, A.lj, ljs64, esum, wsum, A.status,
                                          nacc, qh);
    else
      force_batch<MULTI, ENERGY, COUNT, MODE == kRedoFull>(qn, qh, qd, fa, fr, cap, A, ljs32, ek, wk, nacc,
                                                           big_flag);
  }
  __syncthreads();
  // a large term was left out: list the tile for the redo pass
  if (!FP64 && (MODE == kMain || MODE == kList) && tid == 0 && *big_flag) A.redo[atomicAdd(A.redo_n, 1)] = tile;
  if (MODE == kListBuild) {
    // The atoms in the order of their entry counts, most first (a counting
    // sort), and the entries moved from the scratch into that order; a tile
    // with an atom over lk goes to the fallback list.
    const int lk = A.lk;
    auto perm = EXAMD_ARR(unsigned short, smem + L.perm, cap, st);
    auto hist = EXAMD_ARR(int, smem + L.hist, kMaxListK + 1, st);
    int mx = 0;
    for (int c = tid; c <= lk; c += blockDim.x) hist[c] = 0;
    __syncthreads();
    for (int t = tid; t < total; t += blockDim.x) {
      const int c = fa[t];
      mx = max(mx, c);
      atomicAdd(&hist[min(c, lk)], 1);
    }
    mx = warp_max(mx);
    if (lane == 0) atomicMax(&cw[3], mx);
    __syncthreads();
    if (warp == 0) {  // exclusive scan from the largest count down
      int run = 0;
      for (int c0 = lk; c0 >= 0; c0 -= 32) {
        const int c = c0 - lane;
        const int h = c >= 0 ? hist[c] : 0;
        int x = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL, x, o);
          if (lane >= o) x += y;
        }
        if (c >= 0) hist[c] = run + x - h;
        run += __shfl_sync(FULL, x, 31);
      }
    }
    __syncthreads();
    for (int t = tid; t < total; t += blockDim.x) perm[atomicAdd(&hist[min((int)fa[t], lk)], 1)] = (unsigned short)t;
    __syncthreads();
    // a lane moves its atom's entries eight at a time (16 bytes from the
    // atom's scratch row, two 8-byte bricks that the warp's lanes store side
    // by side); every lane fills the group's bricks up to the group's longest
    // count, the entries past its own count naming the padding atom `total`
    // (staged by the list passes beyond every cutoff), so that the list pass
    // tests no per-lane count
    const size_t nbrick = (size_t)A.ntiles * A.lslots * lk / 4;
    const unsigned short* raw = A.lraw + ltile * lk;
    (void)nbrick;
    for (int g = warp; g * 32 < total; g += nw) {
      const int p = g * 32 + lane;
      const int t = p < total ? perm[p] : 0;
      const int c = p < total ? min((int)fa[t], lk) : 0;
      A.lperm[EXAMD_IDX(ltile + p, (size_t)A.lslots * A.ntiles, st)] = (unsigned short)t;
      A.lcnt[EXAMD_IDX(ltile + p, (size_t)A.lslots * A.ntiles, st)] = (unsigned short)c;
      const int gm = __shfl_sync(FULL, c, 0);
      const uint4* src = reinterpret_cast<const uint4*>(raw + (size_t)t * lk);
      const size_t b0 = (ltile + (size_t)g * 32) * lk / 4 + lane;  // brick k / 4 of this lane: b0 + (k / 4) * 32
      uint2* dst = reinterpret_cast<uint2*>(A.list);
      // 32 entries a round: the four 16-byte reads issued before the stores
      const unsigned dd = (unsigned)total * 0x10001u;  // two padding entries
      // word w of a 16-byte piece holds entries 2w, 2w + 1; n of the piece are the atom's
      auto pad = [&](unsigned w, int n) { return n >= 2 ? w : (n == 1 ? (w & 0xffffu) | (dd & 0xffff0000u) : dd); };
      for (int k0 = 0; k0 < gm; k0 += 32) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = k0 + 8 * u < c ? src[(k0 >> 3) + u] : make_uint4(dd, dd, dd, dd);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = k0 + 8 * u;
          if (k < gm) {
            const int n = c - k;
            if (n < 8) v[u] = make_uint4(pad(v[u].x, n), pad(v[u].y, n - 2), pad(v[u].z, n - 4), pad(v[u].w, n - 6));
            dst[EXAMD_IDX(b0 + (size_t)(k >> 2) * 32, nbrick, st)] = make_uint2(v[u].x, v[u].y);
            if (k + 4 < gm)
              dst[EXAMD_IDX(b0 + (size_t)((k >> 2) + 1) * 32, nbrick, st)] = make_uint2(v[u].z, v[u].w);
          }
        }
      }
    }
    if (tid == 0) {
      const int n = cw[3];
      atomicMax(&A.lw[LW_LMAX], n);
      if (n > lk) {
        A.lcount[tile] = -1;
        A.fb[atomicAdd(&A.lw[LW_FBN], 1)] = tile;
      } else {
        A.lcount[tile] = total;
      }
    }
    return;
  }

  // (4) write-back: home atoms -> Fown, halo copies -> P[slot]
  for (int t = tid; t < total; t += blockDim.x) {
    const int ci = code[t];
    const int lx = ci & 31, ly = (ci >> 5) & 31, lz = ci >> 10;
    const int slot = ((lx == 0 || lx == EX - 1) ? 1 : 0) | ((ly == 0 || ly == EY - 1) ? 2 : 0) |
                     ((lz == 0 || lz == EZ - 1) ? 4 : 0);
    const int e = lx + EX * (ly + EY * lz);
    const int64_t g = gfirst[e] + (t - lstart[e]);
    if (FP64) {
      double* F = slot == 0 ? (double*)A.Fown : (double*)A.P + (size_t)(slot - 1) * 3 * A.N;
#pragma unroll
      for (int c = 0; c < 3; ++c) F[EXAMD_IDX(c * A.N + g, 3 * A.N, st)] = fd[c * cap + t];
    } else {
      float4* F = slot == 0 ? (float4*)A.Fown : (float4*)A.P + (size_t)(slot - 1) * A.N;
      if (MODE == kRedoBig || MODE == kListBig) {
        // this copy's output was written by the first pass and by this tile
        // only (a copy's slot pattern is unique to one tile)
        const float x = fr[t], y = fr[cap + t], z = fr[2 * cap + t];
        if (x != 0.f || y != 0.f || z != 0.f) {
          const int64_t gg = EXAMD_IDX(g, A.N, st);
          float4 v = F[gg];
          v.x += x;
          v.y += y;
          v.z += z;
          F[gg] = v;
        }
      } else {
        float f[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
          f[c] = MODE == kRedoFull ? fmaf((float)fa[c * cap + t], kFixInv, fr[c * cap + t])
                                   : (float)fa[c * cap + t] * kFixInv;
        F[EXAMD_IDX(g, A.N, st)] = make_float4(f[0], f[1], f[2], 0.f);
      }
    }
  }

  // (5) per-tile energy / virial / counters
  if (ENERGY || COUNT) {
    // mixed form: exact integer sums (the same bits whatever the order);
    // FP64 form: FP64 sums
    double e = 0.0, w = 0.0;
    long long ev = 0, wv = 0;
    if (ENERGY) {
      if (FP64) {
        e = esum;
        w = wsum;
      } else {
        ev = ek.v;
        wv = wk.v;
        e = (double)ek.side;
        w = (double)wk.side;
      }
    }
    e = warp_sum(e);
    w = warp_sum(w);
    ev = warp_sum(ev);
    wv = warp_sum(wv);
    const long long c1 = warp_sum((long long)ncand), c2 = warp_sum((long long)nacc),
                    c3 = warp_sum((long long)neval);
    long long* redl = (long long*)red;
    __syncthreads();
    if (lane == 0) {
      red[8 * warp] = e;
      red[8 * warp + 1] = w;
      redl[8 * warp + 2] = ev;
      redl[8 * warp + 3] = wv;
      redl[8 * warp + 4] = c1;
      redl[8 * warp + 5] = c2;
      redl[8 * warp + 6] = c3;
    }
    __syncthreads();
    if (tid == 0) {
      double se = 0, sw = 0;
      long long sev = 0, swv = 0, s1 = 0, s2 = 0, s3 = 0;
      for (int k = 0; k < nw; ++k) {
        se += red[8 * k];
        sw += red[8 * k + 1];
        sev += redl[8 * k + 2];
        swv += redl[8 * k + 3];
        s1 += redl[8 * k + 4];
        s2 += redl[8 * k + 5];
        s3 += redl[8 * k + 6];
      }
      if (ENERGY) {
        A.tileE[tile] = (double)sev * 0x1.0p-32 + se;
        A.tileW[tile] = (double)swv * 0x1.0p-32 + sw;
      }
      if (COUNT) {
        A.tileC[3 * tile] = s1;
        A.tileC[3 * tile + 1] = s2;
        A.tileC[3 * tile + 2] = s3;
      }
    }
  }
}

template <bool FP64, bool MULTI, bool ENERGY, bool COUNT, bool PACK>
__global__ void __launch_bounds__(256, FP64 ? 3 : 4) k_pair(const PairArgs A) {
  pair_tile<FP64, MULTI, ENERGY, COUNT, kMain, PACK>(A, A.order[blockIdx.x]);
}

// Pair-list mode: the forces of every tile from its list (fallback tiles
// return at once: the redo pass enumerates them).
template <bool MULTI, bool ENERGY, bool CUT>
__global__ void __launch_bounds__(256, 4) k_pair_list(const PairArgs A) {
  pair_tile<false, MULTI, ENERGY, false, kList, false, CUT>(A, A.order[blockIdx.x]);
}

// Pair-list mode: the lists of every tile, on the steps whose gate is set.
template <bool MULTI, bool PACK>
__global__ void __launch_bounds__(32 * kBuildWarps, 3) k_pair_build(const PairArgs A) {
  if (A.gate && !*A.gate) return;
  pair_tile<false, MULTI, false, false, kListBuild, PACK>(A, A.order[blockIdx.x]);
}

// Mixed form: the redo pass over the tiles that k_pair listed (normally none,
// and the blocks return at once).  The block that finishes last empties the
// list: every block has read its length (a read that its loop and barrier
// depend on) before its thread 0 counts the block done.  LIST (pair-list
// mode): the listed tiles' large terms are redone from their lists, and the
// fallback tiles (over capacity or with lists that did not fit when they were
// built) are computed in full by enumeration, every step until the next build.
template <bool MULTI, bool PACK, bool ENERGY, bool COUNT, bool LIST>
__global__ void __launch_bounds__(256, 3) k_pair_redo(const PairArgs A) {
  const int n = *(volatile const int*)A.redo_n;
  const int nfb = LIST ? *(volatile const int*)&A.lw[LW_FBN] : 0;
  for (int j = blockIdx.x; j < n + nfb; j += gridDim.x) {
    const int w = j < n ? A.redo[j] : (A.fb[j - n] | kFullBit);
    if (w & kFullBit)
      pair_tile<false, MULTI, ENERGY, COUNT, kRedoFull, PACK>(A, w & ~kFullBit);
    else if (LIST)
      pair_tile<false, MULTI, false, false, kListBig, PACK>(A, w);
    else
      pair_tile<false, MULTI, false, false, kRedoBig, PACK>(A, w);
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (atomicAdd(A.redo_done, 1u) == gridDim.x - 1) {
      *A.redo_n = 0;
      *A.redo_done = 0;
    }
  }
}

template <bool FP64, bool MULTI, bool ENERGY, bool COUNT, bool PACK>
static void* kfn() {
  return (void*)&k_pair<FP64, MULTI, ENERGY, COUNT, PACK>;
}

// The enumeration's first pass.  The FP64 form has one table layout (PACK = false).
static void* pick_enum(const PairConfig& c) {
#define EXAMD_PICK(F, M, P)                                            \
  if (c.energy && c.count) return kfn<F, M, true, true, P>();         \
  if (c.energy) return kfn<F, M, true, false, P>();                   \
  if (c.count) return kfn<F, M, false, true, P>();                    \
  return kfn<F, M, false, false, P>();
  if (c.fp64) {
    if (c.multi) { EXAMD_PICK(true, true, false) }
    EXAMD_PICK(true, false, false)
  }
  if (c.pack) {
    if (c.multi) { EXAMD_PICK(false, true, true) }
    EXAMD_PICK(false, false, true)
  }
  if (c.multi) { EXAMD_PICK(false, true, false) }
  EXAMD_PICK(false, false, false)
#undef EXAMD_PICK
}

// The first pass: in pair-list mode (the counters excepted, which the
// enumeration counts) the list pass.
static bool uses_list(const PairConfig& c) { return c.list && !c.fp64 && !c.count; }

static void* pick(const PairConfig& c) {
  if (uses_list(c)) {
    if (c.cut) {
      if (c.multi) return c.energy ? (void*)&k_pair_list<true, true, true> : (void*)&k_pair_list<true, false, true>;
      return c.energy ? (void*)&k_pair_list<false, true, true> : (void*)&k_pair_list<false, false, true>;
    }
    if (c.multi) return c.energy ? (void*)&k_pair_list<true, true, false> : (void*)&k_pair_list<true, false, false>;
    return c.energy ? (void*)&k_pair_list<false, true, false> : (void*)&k_pair_list<false, false, false>;
  }
  return pick_enum(c);
}

static void* pick_build(const PairConfig& c) {
  if (c.pack) return c.multi ? (void*)&k_pair_build<true, true> : (void*)&k_pair_build<false, true>;
  return c.multi ? (void*)&k_pair_build<true, false> : (void*)&k_pair_build<false, false>;
}

template <bool MULTI, bool PACK, bool LIST>
static void* pick_redo_ec(const PairConfig& c) {
  if (c.energy && c.count) return (void*)&k_pair_redo<MULTI, PACK, true, true, LIST>;
  if (c.energy) return (void*)&k_pair_redo<MULTI, PACK, true, false, LIST>;
  if (c.count) return (void*)&k_pair_redo<MULTI, PACK, false, true, LIST>;
  return (void*)&k_pair_redo<MULTI, PACK, false, false, LIST>;
}

template <bool LIST>
static void* pick_redo_l(const PairConfig& c) {
  if (c.pack) return c.multi ? pick_redo_ec<true, true, LIST>(c) : pick_redo_ec<false, true, LIST>(c);
  return c.multi ? pick_redo_ec<true, false, LIST>(c) : pick_redo_ec<false, false, LIST>(c);
}

static void* pick_redo(const PairConfig& c) { return uses_list(c) ? pick_redo_l<true>(c) : pick_redo_l<false>(c); }

cudaError_t pair_prepare(const PairConfig& cfg, int smem_bytes) {
  cudaError_t e = cudaFuncSetAttribute(pick(cfg), cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
  if (e != cudaSuccess || cfg.fp64) return e;
  e = cudaFuncSetAttribute(pick_redo(cfg), cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
  if (e != cudaSuccess || !uses_list(cfg)) return e;
  return cudaFuncSetAttribute(pick_build(cfg), cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
}

// Occupancy of the enumeration's first pass (the pair-list mode's build uses
// the same tables).
int pair_blocks_per_sm(const PairConfig& cfg, int cap, int ne_max, int ext_max) {
  PairConfig c = cfg;
  c.list = false;
  const int smem = make_layout(c.fp64, cap, ne_max, ext_max, c.warps, kMain, c.pack).bytes;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pick_enum(c), 32 * c.warps, (size_t)smem) != cudaSuccess)
    return 0;
  return n;
}

cudaError_t launch_pair(const PairConfig& cfg, const PairArgs& a, int ntiles, int smem_bytes, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  void* fn = pick(cfg);
  void* args[] = {(void*)&a};
  // smem_bytes (the larger of the passes' needs) bounds every launch
  const int main_smem = main_smem_bytes(cfg, a.cap, a.ne_max, a.ext_max);
  if (main_smem > smem_bytes) return cudaErrorInvalidValue;
  cudaError_t e = cudaLaunchKernel(fn, dim3(ntiles), dim3(32 * cfg.warps), args, (size_t)main_smem, st);
  if (e != cudaSuccess || cfg.fp64) return e;
  // the redo pass: a few blocks per SM at most; nothing to do in a thermal system
  const int redo_smem = redo_smem_bytes(cfg, a.cap_redo, a.ne_max, a.ext_max);
  if (redo_smem > smem_bytes) return cudaErrorInvalidValue;
  return cudaLaunchKernel(pick_redo(cfg), dim3(std::min(ntiles, kRedoBlocks)), dim3(32 * cfg.warps), args,
                          (size_t)redo_smem, st);
}

cudaError_t launch_pair_build(const PairConfig& cfg, const PairArgs& a, int ntiles, int smem_bytes, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  void* args[] = {(void*)&a};
  const int smem = build_smem_bytes(cfg, a.cap, a.ne_max, a.ext_max);
  if (smem > smem_bytes) return cudaErrorInvalidValue;
  return cudaLaunchKernel(pick_build(cfg), dim3(ntiles), dim3(32 * kBuildWarps), args, (size_t)smem, st);
}

}  // namespace examd
