// bin.cu -- cell binning: a counting sort of the atoms into the reference's
// block grid, rebuilt on every step.
//
// Replaces exaMD_identify_block (SRC/exaMD_module.f90:101-125) and the
// per-block linked lists built once by exaMD_particles_generate /
// exaMD_read_particles (SRC/exaMD_input_formats.f90:66-92, 169-192).  Cells
// come in the reference's (z, y, x) block order; inside a cell the atoms keep
// the order in which the counting pass drew their slots.  Neither form's
// results depend on that order: the mixed form's force and energy sums are
// exact fixed point and each pair's FP32 term is antisymmetric in its two
// atoms, and the FP64 form's shared-memory atomics fix no order anyway.
// HBM-bound work.
#include "common.cuh"
#include "kernels.cuh"

namespace examd {

__device__ __forceinline__ void bin_one(int s, double x, double y, double z, int meta,
                                        const BoxDev* __restrict__ boxes, int* __restrict__ cellOld,
                                        int* __restrict__ slot, int* __restrict__ count, int* __restrict__ status) {
  const BoxDev& B = boxes[meta >> 8];
  if (!(finite_bits(x) && finite_bits(y) && finite_bits(z))) {
    atomicOr(status, ST_NONFINITE);
    x = y = z = 0.0;
  }
  const int gc = cell_of(x, y, z, B);
  cellOld[s] = gc;
  slot[s] = atomicAdd(&count[EXAMD_IDX(gc, B.cell0 + B.nb[0] * B.nb[1] * B.nb[2], status)], 1);
}

// Load caller-order AoS positions (and velocities) into the SoA master arrays,
// wrapping (or, in strict mode, rejecting) positions outside [0, L), and bin.
__global__ void k_load_bin(int64_t n, const double* __restrict__ aos, const double* __restrict__ vaos,
                           const int* __restrict__ meta_in, const BoxDev* __restrict__ boxes, int strict,
                           double* __restrict__ X0, double* __restrict__ X1, double* __restrict__ X2,
                           double* __restrict__ V0, double* __restrict__ V1, double* __restrict__ V2,
                           int* __restrict__ meta, int* __restrict__ id, int* __restrict__ cellOld,
                           int* __restrict__ slot, int* __restrict__ count, int* __restrict__ status) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  int mt = meta_in[s];
  const BoxDev& B = boxes[mt >> 8];
  double p[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double x = aos[3 * s + a];
    if (strict && !in_range_bits(x, B.L[a])) atomicOr(status, ST_OUTSIDE);
    p[a] = finite_bits(x) ? wrap_coord(x, B.L[a], B.Li[a]) : x;
  }
  X0[s] = p[0];
  X1[s] = p[1];
  X2[s] = p[2];
  if (vaos) {
    V0[s] = vaos[3 * s];
    V1[s] = vaos[3 * s + 1];
    V2[s] = vaos[3 * s + 2];
  } else {
    V0[s] = V1[s] = V2[s] = 0.0;
  }
  meta[s] = mt;
  id[s] = (int)s;
  bin_one((int)s, p[0], p[1], p[2], mt, boxes, cellOld, slot, count, status);
}

// New positions for the caller's atoms [i0, i1) (AoS, caller order, as they
// arrive in chunks): wrap, store at the atom's sorted slot inv[i], bin.
__global__ void k_gather_pos_bin_range(int64_t i0, int64_t i1, const double* __restrict__ aos,
                                       const BoxDev* __restrict__ boxes, int strict, double* __restrict__ X0,
                                       double* __restrict__ X1, double* __restrict__ X2,
                                       const int* __restrict__ meta, const int* __restrict__ inv,
                                       int* __restrict__ cellOld, int* __restrict__ slot, int* __restrict__ count,
                                       int* __restrict__ status) {
  const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= i1) return;
  const int s = inv[i];
  const int mt = meta[s];
  const BoxDev& B = boxes[mt >> 8];
  double p[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double x = aos[3 * i + a];
    if (strict && !in_range_bits(x, B.L[a])) atomicOr(status, ST_OUTSIDE);
    p[a] = finite_bits(x) ? wrap_coord(x, B.L[a], B.Li[a]) : x;
  }
  X0[s] = p[0];
  X1[s] = p[1];
  X2[s] = p[2];
  bin_one(s, p[0], p[1], p[2], mt, boxes, cellOld, slot, count, status);
}

// ---- exclusive scan of the cell counts (two passes) ------------------------
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh, int& total) {
  // sh: kScanThreads/32 ints
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    int t = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) sh[lane] = t;
  }
  __syncthreads();
  int base = w > 0 ? sh[w - 1] : 0;
  total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return base + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(int nc, const int* __restrict__ count,
                                                              int* __restrict__ bsum, const int* gate) {
  __shared__ int sh[kScanThreads / 32];
  if (gate && !*gate) return;
  int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) s += (base + k < nc) ? count[base + k] : 0;
  int total;
  block_exclusive_scan(s, sh, total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Final pass: cstart = exclusive scan, cstart[nc] = the atom count; counts
// are zeroed for the next binning.  Each block first sums the earlier blocks'
// sums itself (a few hundred to a few thousand values), which saves a launch
// over a separate scan of them.
__global__ void __launch_bounds__(kScanThreads) k_scan_final(int nc, int* __restrict__ count,
                                                             const int* __restrict__ bsum,
                                                             int* __restrict__ cstart, const int* gate) {
  __shared__ int sh[kScanThreads / 32];
  if (gate && !*gate) return;
  int pre = 0;
  for (int k = threadIdx.x; k < (int)blockIdx.x; k += blockDim.x) pre += bsum[k];
  int offset;
  block_exclusive_scan(pre, sh, offset);  // offset: the block-wide sum
  int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < nc) ? count[base + k] : 0;
    s += v[k];
  }
  int total;
  int ex = block_exclusive_scan(s, sh, total) + offset;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) cstart[nc] = offset + total;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < nc) {
      cstart[base + k] = ex;
      count[base + k] = 0;
    }
    ex += v[k];
  }
}

// Final order: every atom goes to its cell's range at the slot it drew in the
// counting pass, and each per-atom array is scattered into the other buffer.
// The pair kernel's FP32 cell offsets U are computed here from the FP64
// position (the same exact rule as the cell), not carried from the counting
// pass: 32 B less memory traffic per atom.  Pair-list mode: the offsets are
// also kept as Ub, the reference for the displacement test of later steps.
__global__ void k_finalize(int64_t n, const int* __restrict__ cellOld, const int* __restrict__ slot,
                           const int* __restrict__ cstart, const BoxDev* __restrict__ boxes,
                           const double* __restrict__ X0, const double* __restrict__ X1,
                           const double* __restrict__ X2, const double* __restrict__ V0,
                           const double* __restrict__ V1, const double* __restrict__ V2,
                           const int* __restrict__ meta, const int* __restrict__ id, double* __restrict__ Y0,
                           double* __restrict__ Y1, double* __restrict__ Y2, double* __restrict__ W0,
                           double* __restrict__ W1, double* __restrict__ W2, int* __restrict__ meta2,
                           int* __restrict__ id2, float4* __restrict__ U, float4* __restrict__ Ub,
                           int* __restrict__ cellS, int* __restrict__ inv, int nc, int* __restrict__ status,
                           const int* gate) {
  if (gate && !*gate) return;
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int c = (int)EXAMD_IDX(cellOld[s], nc, status);
  const int d = (int)EXAMD_IDX(cstart[c] + slot[s], n, status);
  const int myid = id[s], mt = meta[s];
  double x = X0[s], y = X1[s], z = X2[s];
  Y0[d] = x;
  Y1[d] = y;
  Y2[d] = z;
  W0[d] = V0[s];
  W1[d] = V1[s];
  W2[d] = V2[s];
  meta2[d] = mt;
  id2[d] = myid;
  if (!(finite_bits(x) && finite_bits(y) && finite_bits(z))) x = y = z = 0.0;  // as binned
  const BoxDev& B = boxes[mt >> 8];
  float4 u;
  cell_offset(x, B, 0, u.x);
  cell_offset(y, B, 1, u.y);
  cell_offset(z, B, 2, u.z);
  u.w = __int_as_float(mt & 0xff);
  U[d] = u;
  if (Ub) Ub[d] = u;
  cellS[d] = c;
  if (inv) inv[EXAMD_IDX(myid, n, status)] = d;  // caller index -> sorted slot, when the caller's order is needed next
}

// Pair-list mode's binning count: the cell and slot of every atom at its
// current position (the counting pass that the plain step fuses into the
// kick, here only on the steps that rebuild).
__global__ void k_bin_count(int64_t n, const double* __restrict__ X0, const double* __restrict__ X1,
                            const double* __restrict__ X2, const int* __restrict__ meta,
                            const BoxDev* __restrict__ boxes, int* __restrict__ cellOld, int* __restrict__ slot,
                            int* __restrict__ count, int* __restrict__ status, const int* gate) {
  if (gate && !*gate) return;
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  bin_one((int)s, X0[s], X1[s], X2[s], meta[s], boxes, cellOld, slot, count, status);
}

// Pair-list mode: the sorted arrays back into the primary buffer.
__global__ void k_copy_back(int64_t n, const double* __restrict__ Y0, const double* __restrict__ Y1,
                            const double* __restrict__ Y2, const double* __restrict__ W0,
                            const double* __restrict__ W1, const double* __restrict__ W2,
                            const int* __restrict__ meta2, const int* __restrict__ id2, double* __restrict__ X0,
                            double* __restrict__ X1, double* __restrict__ X2, double* __restrict__ V0,
                            double* __restrict__ V1, double* __restrict__ V2, int* __restrict__ meta,
                            int* __restrict__ id, const int* gate) {
  if (gate && !*gate) return;
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  X0[s] = Y0[s];
  X1[s] = Y1[s];
  X2[s] = Y2[s];
  V0[s] = W0[s];
  V1[s] = W1[s];
  V2[s] = W2[s];
  meta[s] = meta2[s];
  id[s] = id2[s];
}

// Pair-list mode: one thread decides whether this step rebuilds and resets
// the displacement maximum and the forced-rebuild request for the next step.
// A rebuild empties the fallback list (the build fills it again).  Inside a
// captured step loop the rebuild is the body of a conditional graph node,
// whose value is set here: a step that does not rebuild launches none of it.
__global__ void k_list_decide(int* lw, float thr2, cudaGraphConditionalHandle h, int cond) {
  const int rb = (__int_as_float(lw[LW_DISP]) > thr2 || lw[LW_FORCE] != 0) ? 1 : 0;
  if (cond) cudaGraphSetConditional(h, (unsigned)rb);
  lw[LW_GATE] = rb;
  lw[LW_DISP] = 0;
  lw[LW_FORCE] = 0;
  if (rb) {
    lw[LW_FBN] = 0;
    lw[LW_BUILDS] += 1;
  }
}

// inv[id[s]] = s: the caller-order map of the current sorted order.
__global__ void k_inverse(int64_t n, const int* __restrict__ id, int* __restrict__ inv) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s < n) inv[id[s]] = (int)s;
}

}  // namespace examd
