// step.cu -- per-atom kernels around the pair kernel: halo-partial gather,
// velocity-Verlet kick/drift fused with the next binning, kinetic energy,
// per-box reductions and the caller-order output.
//
// The reference has no integrator (one force evaluation, exaMD.f90:247-251);
// the gather replaces its reverse force exchange, which adds received halo
// forces into the owner's blocks (SRC/exaMD_comms.f90:330-376).  All of these
// are HBM-bound; FP64 is used only where positions, velocities and the
// reductions need it.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace examd {

__device__ __forceinline__ void bin_store(int s, double x, double y, double z, const BoxDev& B,
                                          int* __restrict__ cellOld, int* __restrict__ slot,
                                          int* __restrict__ count, int nc, int* status) {
  // same rule as bin.cu: exact cell of the FP64 position on the grid c * bl
  const int gc = (int)EXAMD_IDX(cell_of(x, y, z, B), nc, status);
  cellOld[s] = gc;
  slot[s] = atomicAdd(&count[gc], 1);
}

// Pair-list mode.  Between two builds an atom keeps the cell it was sorted
// into; its FP32 offset is taken from that cell's origin, so it may leave the
// cell's range by up to half the skin.

// x rounded to the nearest float, either sign, on the integer pipe.
__device__ __forceinline__ float d2f_rn_signed(double x) {
  const long long b = __double_as_longlong(x);
  const float m = d2f_rn_nonneg(__longlong_as_double(b & 0x7fffffffffffffffll));
  return b < 0 ? -m : m;
}

// The periodic image of an atom that crossed the box boundary since the
// build, seen from its build cell (rare: out of line, so that its FP64
// instructions are not run speculatively by every thread).
static __device__ __noinline__ double offset_wrapped(double u, double L) { return u > 0.0 ? u - L : u + L; }

// Offset of coordinate x (in [0, L)) from the origin of cell c on axis a,
// rounded once to FP32: x - c*bl is exact (both are within a factor of two,
// or c = 0), and an atom that crossed the periodic boundary is taken at its
// image nearest the cell (it moved less than half the skin).
__device__ __forceinline__ float list_offset(double x, int c, const BoxDev& B, int a) {
  double u = x - mul_pow2((unsigned)(c * B.blq), B.blk);
  const long long b = __double_as_longlong(u) & 0x7fffffffffffffffll;
  if (d2f_trunc(__longlong_as_double(b)) > 0.5f * B.Lf[a]) u = offset_wrapped(u, B.L[a]);
  return d2f_rn_signed(u);
}

// The list-mode offsets of one atom from its build cell (global cell gc),
// and its squared displacement since the build (from the offsets Ub then).
__device__ __forceinline__ float list_update(int64_t s, const double x[3], int gc, int type, const BoxDev& B,
                                             float4* __restrict__ U, const float4* __restrict__ Ub) {
  const int cl = gc - B.cell0;
  const int q = cl / B.nb[0];
  const int cx = cl - q * B.nb[0];
  const int cz = q / B.nb[1];
  const int cy = q - cz * B.nb[1];
  float4 u;
  u.x = list_offset(x[0], cx, B, 0);
  u.y = list_offset(x[1], cy, B, 1);
  u.z = list_offset(x[2], cz, B, 2);
  u.w = __int_as_float(type);
  U[s] = u;
  const float4 b = Ub[s];
  const float dx = u.x - b.x, dy = u.y - b.y, dz = u.z - b.z;
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// The block's largest squared displacement into lw[LW_DISP] (non-negative
// floats order as their bit patterns).  Every thread of the block calls it.
// One atomic per block at most, and none when the block's maximum is not
// above the value already there: atomics on one word serialise in L2, and
// one per warp cost a third of the kick at 16.8M atoms.
__device__ __forceinline__ void disp_max(float d2, int* lw) {
  __shared__ unsigned wmax[32];
  const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wmax[w] = m;
  __syncthreads();
  if (w == 0) {
    const unsigned b = __reduce_max_sync(0xffffffffu, lane < (int)(blockDim.x >> 5) ? wmax[lane] : 0u);
    if (lane == 0 && b != 0u && (int)b > *(volatile int*)&lw[LW_DISP]) atomicMax(&lw[LW_DISP], (int)b);
  }
}

// Sum of an atom's force partials: the owning tile's, then the halo slots in
// increasing order (fixed order: deterministic).  Mixed form: Kahan in FP32.
__device__ __forceinline__ void gather_force(const StepArgs& a, int64_t s, double f[3]) {
  s = EXAMD_IDX(s, a.N, a.status);
  const int m = a.bmask[EXAMD_IDX(a.cellS[s], a.nc, a.status)];
  if (a.fp64) {
    const double* Fo = (const double*)a.Fown;
    const double* P = (const double*)a.P;
    double fx = Fo[s], fy = Fo[a.N + s], fz = Fo[2 * a.N + s];
    for (int sl = 1; sl < 8; ++sl) {
      if ((sl & m) != sl) continue;
      const double* q = P + (size_t)(sl - 1) * 3 * a.N;
      fx += q[s];
      fy += q[a.N + s];
      fz += q[2 * a.N + s];
    }
    f[0] = fx;
    f[1] = fy;
    f[2] = fz;
  } else {
    const float4* Fo = (const float4*)a.Fown;
    const float4* P = (const float4*)a.P;
    float4 v = Fo[s];
    if (m == 0) {
      f[0] = f2d_exact(v.x);
      f[1] = f2d_exact(v.y);
      f[2] = f2d_exact(v.z);
      return;
    }
    KSum kx, ky, kz;
    kx.s = v.x;
    ky.s = v.y;
    kz.s = v.z;
    for (int sl = 1; sl < 8; ++sl) {
      if ((sl & m) != sl) continue;
      float4 q = P[(size_t)(sl - 1) * a.N + s];
      kx.add(q.x);
      ky.add(q.y);
      kz.add(q.z);
    }
    f[0] = f2d_exact(kx.s - kx.c);
    f[1] = f2d_exact(ky.s - ky.c);
    f[2] = f2d_exact(kz.s - kz.c);
  }
}

// Forces of the caller's atoms [i0, i1) in caller order (AoS): the atom's
// partials gathered at its sorted slot inv[i]; written or added (acc).
__global__ void k_forces_out(const StepArgs a, int64_t i0, int64_t i1, const int* __restrict__ inv,
                             double* __restrict__ out, int acc) {
  const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= i1) return;
  double f[3];
  gather_force(a, inv[i], f);
  if (acc) {
    out[3 * i] += f[0];
    out[3 * i + 1] += f[1];
    out[3 * i + 2] += f[2];
  } else {
    out[3 * i] = f[0];
    out[3 * i + 1] = f[1];
    out[3 * i + 2] = f[2];
  }
}

cudaError_t launch_forces_out(const StepArgs& s, int64_t i0, int64_t i1, const int* inv, double* out, int accumulate,
                              cudaStream_t st) {
  if (i1 <= i0) return cudaSuccess;
  k_forces_out<<<(unsigned)((i1 - i0 + 255) / 256), 256, 0, st>>>(s, i0, i1, inv, out, accumulate);
  return cudaGetLastError();
}

// Per-box FP64 sums of per-tile partials: one block per box, fixed-order tree.
// Per-box sums of per-atom or per-tile values over the boxes' contiguous
// ranges, in two fixed-order levels so that a box of millions of atoms does
// not fall on one block: block (c, b) sums chunk c (kRedChunk entries from the
// box's first one) with a fixed tree, then one block per box sums its chunks
// in order.  Reproducible bit for bit.  NV = 1 or 2 arrays.
constexpr int kRedChunk = 4096;

template <typename Off, int NV>
__global__ void k_chunk_sums(const Off* __restrict__ off, const double* __restrict__ v0,
                             const double* __restrict__ v1, int maxc, double* __restrict__ partial) {
  __shared__ double sh[NV][256];
  const int c = blockIdx.x, b = blockIdx.y;
  const int64_t a0 = (int64_t)off[b] + (int64_t)c * kRedChunk;
  const int64_t a1 = min((int64_t)off[b + 1], a0 + kRedChunk);
  double s0 = 0.0, s1 = 0.0;
  for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    s0 += v0[i];
    if (NV > 1) s1 += v1[i];
  }
  sh[0][threadIdx.x] = s0;
  if (NV > 1) sh[NV - 1][threadIdx.x] = s1;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      if (NV > 1) sh[NV - 1][threadIdx.x] += sh[NV - 1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[(size_t)b * maxc + c] = sh[0][0];
    if (NV > 1) partial[((size_t)gridDim.y + b) * maxc + c] = sh[NV - 1][0];
  }
}

template <int NV>
__global__ void k_box_sums(const double* __restrict__ partial, int maxc, int nboxes, double* __restrict__ out0,
                           double* __restrict__ out1) {
  __shared__ double sh[NV][256];
  const int b = blockIdx.x;
  double s0 = 0.0, s1 = 0.0;
  for (int c = threadIdx.x; c < maxc; c += blockDim.x) {
    s0 += partial[(size_t)b * maxc + c];
    if (NV > 1) s1 += partial[((size_t)nboxes + b) * maxc + c];
  }
  sh[0][threadIdx.x] = s0;
  if (NV > 1) sh[NV - 1][threadIdx.x] = s1;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      if (NV > 1) sh[NV - 1][threadIdx.x] += sh[NV - 1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out0[b] = sh[0][0];
    if (NV > 1) out1[b] = sh[NV - 1][0];
  }
}

int red_chunks(int64_t max_per_box) { return (int)std::max<int64_t>(1, (max_per_box + kRedChunk - 1) / kRedChunk); }

cudaError_t launch_box_sums(int nboxes, const int64_t* atom0, int maxc, const double* v, double* partial,
                            double* out, cudaStream_t st) {
  k_chunk_sums<int64_t, 1><<<dim3(maxc, nboxes), 256, 0, st>>>(atom0, v, nullptr, maxc, partial);
  k_box_sums<1><<<nboxes, 256, 0, st>>>(partial, maxc, nboxes, out, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_reduce_tiles(int nboxes, const int* tile0, int maxc, const double* tileE, const double* tileW,
                                double* partial, double* boxE, double* boxW, cudaStream_t st) {
  k_chunk_sums<int, 2><<<dim3(maxc, nboxes), 256, 0, st>>>(tile0, tileE, tileW, maxc, partial);
  k_box_sums<2><<<nboxes, 256, 0, st>>>(partial, maxc, nboxes, boxE, boxW);
  return cudaGetLastError();
}

// Per-box sums of a per-atom quantity over the boxes' contiguous atom ranges
// (atoms are sorted by box): one block per box, fixed assignment and tree
// order, so the result is reproducible bit for bit.
__global__ void k_reduce_atoms(const int64_t* __restrict__ atom0, const double* __restrict__ v,
                               double* __restrict__ out) {
  __shared__ double sh[256];
  const int b = blockIdx.x;
  const int64_t a0 = atom0[b], a1 = atom0[b + 1];
  double s = 0.0;
  for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) s += v[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[b] = sh[0];
}

cudaError_t launch_reduce_atoms(int nboxes, const int64_t* atom0, const double* v, double* out, cudaStream_t st) {
  k_reduce_atoms<<<nboxes, 256, 0, st>>>(atom0, v, out);
  return cudaGetLastError();
}

// v += ckick F/m; optional kinetic energy at v + hk F/m; optional drift
// x += dt v with periodic wrap followed by the binning count of the next step
// (pair-list mode: by the offsets from the build cells and the displacement
// since the build instead).
__global__ void k_kick(const KickArgs k) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool in = s < k.s.N;
  const int64_t ss = in ? s : 0;
  double f[3];
  gather_force(k.s, ss, f);
  const int mt = k.meta[ss];
  const int type = mt & 0xff, box = mt >> 8;
  const double ck = k.ckm[type];
  double v[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) v[a] = k.V[a][ss];
  if (k.hk > 0.0) {
    const double hm = k.hkm[type];
    double ke = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double vt = v[a] + hm * f[a];
      ke += vt * vt;
    }
    ke *= 0.5 * k.lj.mass[type];
    if (in) k.keAtom[s] = ke;
  }
  float d2 = 0.f;  // pair-list mode: squared displacement since the build
  if (in) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      v[a] = v[a] + ck * f[a];
      k.V[a][s] = v[a];
    }
    if (k.drift) {
      const BoxDev& B = k.s.boxes[box];
      double x[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        x[a] = wrap_coord(fma(k.dt, v[a], k.X[a][s]), B.L[a], B.Li[a]);
        k.X[a][s] = x[a];
      }
      if (!(finite_bits(x[0]) && finite_bits(x[1]) && finite_bits(x[2]))) {
        atomicOr(k.status, ST_NONFINITE);
        x[0] = x[1] = x[2] = 0.0;
      }
      if (k.list)
        d2 = list_update(s, x, k.s.cellS[s], type, B, k.U, k.Ub);
      else
        bin_store((int)s, x[0], x[1], x[2], B, k.cellOld, k.slot, k.count, k.s.nc, k.status);
    }
  }
  if (k.list && k.drift) disp_max(d2, k.lw);
}

// Pair-list mode: new positions for the caller's atoms [i0, i1) (AoS, caller
// order): wrap, store at the sorted slot inv[i], offsets from the build cell
// and the displacement since the build.
__global__ void k_gather_pos_list(int64_t i0, int64_t i1, const double* __restrict__ aos,
                                  const BoxDev* __restrict__ boxes, int strict, double* __restrict__ X0,
                                  double* __restrict__ X1, double* __restrict__ X2, const int* __restrict__ meta,
                                  const int* __restrict__ inv, const int* __restrict__ cellS, float4* __restrict__ U,
                                  const float4* __restrict__ Ub, int* __restrict__ lw, int* __restrict__ status) {
  const int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float d2 = 0.f;
  if (i < i1) {
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
    if (!(finite_bits(p[0]) && finite_bits(p[1]) && finite_bits(p[2]))) {
      atomicOr(status, ST_NONFINITE);
      p[0] = p[1] = p[2] = 0.0;
    }
    d2 = list_update(s, p, cellS[s], mt & 0xff, B, U, Ub);
  }
  disp_max(d2, lw);
}

cudaError_t launch_gather_pos_list(int64_t i0, int64_t i1, const double* aos, const BoxDev* boxes, int strict,
                                   double* X0, double* X1, double* X2, const int* meta, const int* inv,
                                   const int* cellS, float4* U, const float4* Ub, int* lw, int* status,
                                   cudaStream_t st) {
  if (i1 <= i0) return cudaSuccess;
  k_gather_pos_list<<<(unsigned)((i1 - i0 + 255) / 256), 256, 0, st>>>(i0, i1, aos, boxes, strict, X0, X1, X2, meta,
                                                                       inv, cellS, U, Ub, lw, status);
  return cudaGetLastError();
}

cudaError_t launch_kick(const KickArgs& k, cudaStream_t st) {
  if (k.s.N > 0) k_kick<<<(unsigned)((k.s.N + 255) / 256), 256, 0, st>>>(k);
  if (k.hk > 0.0) return launch_box_sums(k.nboxes, k.atom0, k.maxc, k.keAtom, k.partial, k.boxKE, st);
  return cudaGetLastError();
}

__global__ void k_kinetic(int64_t n, const double* __restrict__ V0, const double* __restrict__ V1,
                          const double* __restrict__ V2, const int* __restrict__ meta, const LJTable lj,
                          double* __restrict__ keAtom) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  keAtom[s] = 0.5 * lj.mass[meta[s] & 0xff] * (V0[s] * V0[s] + V1[s] * V1[s] + V2[s] * V2[s]);
}

cudaError_t launch_kinetic(int64_t n, int nboxes, const int64_t* atom0, int maxc, const double* const V[3],
                           const int* meta, LJTable lj, double* keAtom, double* partial, double* boxKE,
                           cudaStream_t st) {
  if (n > 0) k_kinetic<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, V[0], V[1], V[2], meta, lj, keAtom);
  return launch_box_sums(nboxes, atom0, maxc, keAtom, partial, boxKE, st);
}

__global__ void k_scale_v(int64_t n, double* __restrict__ V0, double* __restrict__ V1, double* __restrict__ V2,
                          const int* __restrict__ meta, const double* __restrict__ factor) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double f = factor[meta[s] >> 8];
  V0[s] *= f;
  V1[s] *= f;
  V2[s] *= f;
}

cudaError_t launch_scale_v(int64_t n, double* V[3], const int* meta, const double* factor, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_scale_v<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, V[0], V[1], V[2], meta, factor);
  return cudaGetLastError();
}

__global__ void k_state_out(int64_t n, const double* __restrict__ A0, const double* __restrict__ A1,
                            const double* __restrict__ A2, const int* __restrict__ id, double* __restrict__ out) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  int64_t i = id[s];
  out[3 * i] = A0[s];
  out[3 * i + 1] = A1[s];
  out[3 * i + 2] = A2[s];
}

cudaError_t launch_state_out(int64_t n, const double* const A[3], const int* id, double* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_state_out<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, A[0], A[1], A[2], id, out);
  return cudaGetLastError();
}

}  // namespace examd
