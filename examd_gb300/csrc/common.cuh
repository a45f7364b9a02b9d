// common.cuh -- shared device-side definitions of the GB300 midpoint LJ path.
//
// Layout in HBM (all per-atom arrays in "sorted order": atoms grouped by cell,
// cells in (box, z, y, x) order, atoms of a cell in ascending caller index,
// i.e. the reference's block order and linked-list order,
// SRC/exaMD_input_formats.f90:66-92):
//   X[3][N], V[3][N]  FP64 positions / velocities (SoA), double-buffered
//   meta[N]           box << 8 | type
//   id[N]             caller index
//   U[N]              float4 (u_x, u_y, u_z, type bits): position relative to
//                     the atom's cell origin c * block_length, FP32
//   cellS[N]          global cell id
//   cstart[NC+1]      CSR offsets of cells
//   Fown[N], P[7][N]  force partials: the owning tile's sum, and the sums of
//                     up to 7 neighbouring tiles whose halo holds the atom
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/examd_gb300.h"

namespace examd {

constexpr int kRows = 13;     // 12 full x-rows of 5 cells + the half self row
constexpr int kClasses = 125; // 5 position classes per axis inside a tile
constexpr int kMaxExt = 31;   // ext-cell coordinate packing: 5 bits per axis

// Status word bits (device -> host).
enum StatusBits : int {
  ST_OVERFLOW = 1,   // a tile has more staged atoms than the smem capacity
  ST_NONFINITE = 2,  // NaN / Inf position
  ST_OUTSIDE = 4,    // position outside [0,L) in strict mode
  ST_TIMEOUT = 8,    // a bounded wait gave up
  ST_PAIRFN = 16,    // the pair function returned an error
  ST_BOUNDS = 32,    // checked build: an index check failed (the access went to index 0)
};

// Pair-list mode: the device words that carry the list's state between the
// kernels of a step (no host round trip, so that a step loop stays one CUDA
// graph).
enum ListWord : int {
  LW_DISP = 0,    // largest squared displacement since the last build (float bits, atomicMax)
  LW_GATE = 1,    // nonzero: this step rebuilds the cells and the lists (k_list_decide)
  LW_FORCE = 2,   // nonzero: rebuild at the next step whatever the displacement
  LW_FBN = 3,     // tiles in the fallback list (computed by enumeration every step)
  LW_LMAX = 4,    // largest list length of a tile since the host last read it
  LW_BUILDS = 5,  // builds since the context was created
  LW_WORDS = 8
};

// Index-checked arrays of the checked build (-DEXAMD_CHECKED, the
// counterpart of a memory checker on a pool where none may run): every
// subscript is tested against the array's length; an index outside it sets
// ST_BOUNDS in the status word and reads or writes element 0 instead, so the
// kernel records the fault and finishes without touching memory outside its
// buffers.  Without EXAMD_CHECKED an array is its plain pointer and the
// checks cost nothing.
#ifdef EXAMD_CHECKED
template <class T>
struct ChkArr {
  T* p;
  long long n;
  int* st;
  __device__ __forceinline__ T& operator[](long long i) const {
    if (i < 0 || i >= n) {
      atomicOr(st, ST_BOUNDS);
      i = 0;
    }
    return p[i];
  }
};
#define EXAMD_ARR(T, ptr, len, status) (examd::ChkArr<T>{(T*)(ptr), (long long)(len), (status)})
#define EXAMD_IDX(i, len, status) examd::chk_index((i), (long long)(len), (status))
__device__ __forceinline__ long long chk_index(long long i, long long n, int* st) {
  if (i < 0 || i >= n) {
    atomicOr(st, ST_BOUNDS);
    return 0;
  }
  return i;
}
#else
#define EXAMD_ARR(T, ptr, len, status) ((T*)(ptr))
#define EXAMD_IDX(i, len, status) (i)
#endif

struct BoxDev {
  double L[3], Li[3];
  double bl, bli;  // block_length (cell edge) and its inverse
  int blq, blk;    // bl = blq * 2^-blk exactly (blq < 2^14)
  float blf, blif, Lf[3];
  float remf[3];   // L - nb*bl: the extra width of the last cell, FP32
  int nb[3];
  int cell0;       // first global cell id of the box
  int tile0;       // first tile of the box
  int nt[3];       // tiles per axis
};

// LJ parameters per ordered type pair, FP32 (mixed) and FP64.
// rc2: the candidate cutoff (distance test, queue); rcut2: the potential's
// own range (<= rc2; FP32 table: infinite where it is rc2, which the
// candidate test decides); eshift: subtracted from the pair energy.
struct LJ32 {
  // the fields every list entry reads first, in one 16-byte word
  float sig2, m24eps, rc2;  // m24eps = -24 eps (dg prefactor)
  float r2big;  // r^2 below which |F| >= kFixMaxForce (mixed form: left to the redo pass)
  float c4eps, eshift, rcut2;
  float rl2;    // pair-list mode: (rc + skin)^2, the list's cutoff for this type pair
};

// Mixed form: pair-force magnitude at which a term leaves the fixed-point sums
// (2^17 scale, int32) for the redo pass (r < ~0.74 sigma at eps = 1); every
// component of a kept term is below 2^28 in fixed point, so a component's
// int32 sum needs more than 8 near-maximal terms of one sign to overflow.
constexpr float kFixMaxForce = 2048.f;
struct LJ64 {
  double sig2, eps24, eps4, rc2;   // as user_func.f90:58-59 computes them
  double rcut2, eshift;
};

struct LJTable {
  int nt;
  int pot;       // EXAMD_POT_*
  float rc2max;
  float prune2;  // (max rc + 1e-4)^2: cell boxes farther than this hold no pair
                 // (pair-list mode: (max rc + skin/2 + 1e-4)^2, atoms may have
                 // left their cells by up to skin/2 since the list was built)
  float prune2_list;  // pair-list mode: (max rc + skin + 1e-4)^2, for the list build
  LJ32 p32[EXAMD_MAX_TYPES * EXAMD_MAX_TYPES];
  LJ64 p64[EXAMD_MAX_TYPES * EXAMD_MAX_TYPES];
  double minv[EXAMD_MAX_TYPES];
  double mass[EXAMD_MAX_TYPES];
};

// Ownership masks of the midpoint table, filled once per process.
//   c_rows[r] = (dy, dz) of row r (r = 12: the self row (0,0))
//   lut[cls][n] = 5-bit mask over dx = -2..2 of the cell pairs (A, A+d) of
//   row rlist[cls][n] owned by the tile when A's position class is cls (by
//   position in the class's row list, so that a kernel reads the row and its
//   mask side by side).  Row 12 uses bit 2 for the pairs inside A (a1 < a2)
//   and bits 3, 4 for dx = +1, +2.
// 16-byte aligned so that a CTA copies it to shared memory as uint4 words.
struct __align__(16) OwnLut {
  unsigned char lut[kClasses][kRows];     // dx mask per position class and row-list position
  signed char rows[kRows][2];             // (dy, dz) of row r
  unsigned char nrow[kClasses];           // rows with a nonzero mask
  unsigned char rlist[kClasses][kRows];   // those rows, ascending
};

__host__ __device__ inline int pos_class(int l, int t) {
  return l < 0 ? 0 : (l == 0 ? 1 : (l < t - 1 ? 2 : (l == t - 1 ? 3 : 4)));
}

// Tile descriptor: int4 {box, x0, y0, z0}, int4 {tx, ty, tz, 0}.

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Kahan-compensated FP32 accumulator.
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// FP64 arithmetic and the FP32 <-> FP64 conversions both run on this part's
// FP64 pipe, 1/64 of the FP32 rate.  The per-atom kernels therefore decide
// range, finiteness and cell membership of an FP64 coordinate on its bits
// with integer operations, and spend FP64 instructions only on the arithmetic
// that needs them.

// 0 <= x < L (either zero), for L > 0: non-negative doubles are ordered as
// their bit patterns, and every negative one has the sign bit set.
__device__ __forceinline__ bool in_range_bits(double x, double L) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return b < (unsigned long long)__double_as_longlong(L) || b == 0x8000000000000000ull;
}

__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// A float within one FP32 ulp of x (mantissa truncated), for estimates only;
// 0 for |x| < 2^-126.  x must be below 2^128 in magnitude.
__device__ __forceinline__ float d2f_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 1023 - 126) return 0.f;
  return __uint_as_float((unsigned)(b >> 32 & 0x80000000u) | ((unsigned)(e - 1023 + 127) << 23) |
                         (unsigned)((b >> 29) & 0x7fffff));
}

// x rounded to the nearest float, ties to even, for 0 <= x < 2^128; values
// below 2^-126 become 0 (no subnormals).  Same result as (float)x in the
// normal range.
__device__ __forceinline__ float d2f_rn_nonneg(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  const int e = (int)(b >> 52);
  if (e < 1023 - 126) return 0.f;
  const unsigned mf = (unsigned)((b >> 29) & 0x7fffff);
  const unsigned long long rest = b & 0x1fffffffull;  // the 29 dropped mantissa bits
  unsigned bits = ((unsigned)(e - 1023 + 127) << 23) | mf;
  if (rest > 0x10000000ull || (rest == 0x10000000ull && (mf & 1u))) ++bits;  // a carry rounds up the exponent
  return __uint_as_float(bits);
}

// float -> double, exact, by rebuilding the bit pattern on the integer pipe
// (GB300 converts FP32 to FP64 on the FP64 pipe, at about 2 per clock per
// SM).  Infinities and NaNs carry over; FP32 subnormals become signed zeros.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu, sign = b & 0x80000000u;
  if (e == 0u) return __hiloint2double((int)sign, 0);
  const unsigned ee = e == 0xffu ? 0x7ffu : e + (1023u - 127u);
  return __hiloint2double((int)(sign | (ee << 20) | ((b & 0x7fffffu) >> 3)), (int)((b & 7u) << 29));
}

// n * 2^-k exactly, for 0 < n < 2^31 (0 for n = 0).
__device__ __forceinline__ double mul_pow2(unsigned n, int k) {
  if (n == 0u) return 0.0;
  const int p = 31 - __clz(n);
  const unsigned long long mant = ((unsigned long long)n << (52 - p)) & 0xfffffffffffffull;
  return __longlong_as_double((long long)(((unsigned long long)(p - k + 1023) << 52) | mant));
}

// Cell c = Int(x / bl) of the exact quotient, clamped to the last cell (which
// absorbs the remainder, SRC/exaMD_module.f90:109-113), and the offset
// u = x - c*bl rounded once to FP32, for 0 <= x < L.  One FP64 subtraction:
// the FP32 estimate of c is within one of the exact cell, c*bl and (c+1)*bl
// are built exactly from their integer multiples of 2^-k and compared with x
// as bit patterns, and x - c*bl is then exact.
__device__ __forceinline__ int cell_offset(double x, const BoxDev& B, int a, float& u) {
  const int nb = B.nb[a];
  int c = (int)(d2f_trunc(x) * B.blif);
  c = min(max(c, 0), nb - 1);
  long long bx = __double_as_longlong(x);
  if (bx == (long long)0x8000000000000000ull) bx = 0;  // -0
  if (bx < __double_as_longlong(mul_pow2((unsigned)(c * B.blq), B.blk))) {
    c = max(c - 1, 0);  // the estimate was one too high
  } else if (c < nb - 1 && bx >= __double_as_longlong(mul_pow2((unsigned)((c + 1) * B.blq), B.blk))) {
    ++c;  // one too low
  }
  u = d2f_rn_nonneg(x - mul_pow2((unsigned)(c * B.blq), B.blk));
  return c;
}

// Global cell of a position inside its box (the offsets are not needed).
__device__ __forceinline__ int cell_of(double x, double y, double z, const BoxDev& B) {
  float u;
  const int cx = cell_offset(x, B, 0, u);
  const int cy = cell_offset(y, B, 1, u);
  const int cz = cell_offset(z, B, 2, u);
  return B.cell0 + cx + B.nb[0] * (cy + B.nb[1] * cz);
}

// Periodic wrap of an FP64 coordinate into [0, L).  The in-range case is
// decided on the bits; the rare out-of-range case is a separate function so
// that its FP64 instructions are not executed speculatively by every thread.
static __device__ __noinline__ double wrap_slow(double x, double L, double Li) {
  double y = x - floor(x * Li) * L;
  if (y >= L) y -= L;
  if (y < 0.0) y += L;
  return y;
}

__device__ __forceinline__ double wrap_coord(double x, double L, double Li) {
  return in_range_bits(x, L) ? x : wrap_slow(x, L, Li);
}

}  // namespace examd
