// pair.cu -- the midpoint pair kernel: one CTA per tile of home cells.
//
// Replaces exaMD_forces_midpoint_all / _bdry / _overlap, exaMD_particle_
// interaction and lennardjones_12 (SRC/exaMD_forces.f90:41-551,
// user_func.f90:40-75).  A tile owns every cell pair whose home block -- given
// by the reference's 63-entry table (SRC/exaMD_module.f90:276-346) -- lies in
// the tile; the tile plus a one-cell halo is staged in shared memory (periodic
// images folded into the staged coordinates: the HBM/SMEM counterpart of the
// MPI halo exchange in SRC/exaMD_comms.f90:44-244).
//
// Work order.  The 62 non-self table entries are, per home-relative cell A,
// 12 full x-rows of 5 cells (dy, dz fixed, dx = -2..2) plus the half row
// dx = +1, +2; with the self pairs that is 13 "rows" r.  Phase r: each warp
// takes chunks of 32 consecutive staged i-atoms from its own block of x-rows;
// lane l owns atom i = c0 + l and the contiguous j-ranges of the cells in row
// r that the table assigns to this tile (ownership masks per position class).
// The warp walks the ranges along diagonals: at step k lane l handles
// j = l + k, so no two lanes touch the same j at once and the Newton's-third-
// law update of f_j is a plain shared-memory read-modify-write: deterministic
// and free of atomics.  Warps own disjoint x-rows, and a phase shifts every
// row by the same (dy, dz), so warps never share j atoms inside a phase;
// phases are separated by __syncthreads().
//
// Output: the forces of the tile's home atoms go to Fown, those of halo atoms
// to the partial slot P[s] (s = bitmask of the axes on which the copy is a
// halo copy); the integrator sums an atom's 1..8 partials in a fixed order.
#include <climits>

#include "common.cuh"
#include "kernels.cuh"

namespace examd {

__constant__ OwnLut c_own;

cudaError_t upload_own_lut(const OwnLut& lut) { return cudaMemcpyToSymbol(c_own, &lut, sizeof(OwnLut)); }

// Shared-memory carve-up, identical on host and device.
struct Layout {
  int lstart, gfirst, rowb, ox, oy, oz, dyt, dzt, imx, imy, imz, red;
  int pf, fi, fj, fic, fjc, px, gidx, code;
  int bytes;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

__host__ __device__ inline Layout make_layout(bool fp64, bool kahan, int cap, int ne_max, int nw) {
  Layout L;
  int o = 0;
  L.lstart = o; o = align16(o + 4 * (ne_max + 1));
  L.gfirst = o; o = align16(o + 4 * ne_max);
  L.rowb = o;   o = align16(o + 4 * (nw + 1));
  L.ox = o;     o = align16(o + 4 * kMaxExt);
  L.oy = o;     o = align16(o + 4 * kMaxExt);
  L.oz = o;     o = align16(o + 4 * kMaxExt);
  L.dyt = o;    o = align16(o + 4 * kMaxExt * 5);
  L.dzt = o;    o = align16(o + 4 * kMaxExt * 5);
  L.imx = o;    o = align16(o + 8 * kMaxExt);
  L.imy = o;    o = align16(o + 8 * kMaxExt);
  L.imz = o;    o = align16(o + 8 * kMaxExt);
  L.red = o;    o = align16(o + 8 * 4 * nw);
  const int fs = fp64 ? 8 : 4;
  L.pf = o;     o = align16(o + 16 * cap);
  L.fi = o;     o = align16(o + 3 * fs * cap);
  L.fj = o;     o = align16(o + 3 * fs * cap);
  const bool comp = kahan && !fp64;
  L.fic = o;    o = align16(o + (comp ? 3 * 4 * cap : 0));
  L.fjc = o;    o = align16(o + (comp ? 3 * 4 * cap : 0));
  L.px = o;     o = align16(o + (fp64 ? 3 * 8 * cap : 0));
  L.gidx = o;   o = align16(o + 4 * cap);
  L.code = o;   o = align16(o + 2 * cap);
  L.bytes = o;
  return L;
}

int pair_smem_bytes(const PairConfig& cfg, int cap, int ne_max) {
  return make_layout(cfg.fp64, cfg.kahan, cap, ne_max, cfg.warps).bytes;
}
int pair_bytes_per_atom(const PairConfig& cfg) {
  return make_layout(cfg.fp64, cfg.kahan, 1024, 0, 1).bytes / 1024;
}

template <bool FP64>
struct Acc;
template <>
struct Acc<false> {
  using T = float;
};
template <>
struct Acc<true> {
  using T = double;
};

template <bool FP64, bool MULTI, bool KAHAN, bool ENERGY, bool COUNT>
__global__ void __launch_bounds__(256) k_pair(const PairArgs A) {
  using T = typename Acc<FP64>::T;
  constexpr bool COMP = KAHAN && !FP64;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int tile = blockIdx.x;
  const int4 t0 = A.tiles[2 * tile], t1 = A.tiles[2 * tile + 1];
  const BoxDev& B = A.boxes[t0.x];
  const int X0 = t0.y, Y0 = t0.z, Z0 = t0.w;
  const int tx = t1.x, ty = t1.y, tz = t1.z;
  const int EX = tx + 2, EY = ty + 2, EZ = tz + 2;
  const int NE = EX * EY * EZ, NR = EY * EZ;
  const Layout L = make_layout(FP64, KAHAN, A.cap, A.ne_max, nw);
  int* lstart = (int*)(smem + L.lstart);
  int* gfirst = (int*)(smem + L.gfirst);
  int* rowb = (int*)(smem + L.rowb);
  float* ox = (float*)(smem + L.ox);
  float* oy = (float*)(smem + L.oy);
  float* oz = (float*)(smem + L.oz);
  float* dyt = (float*)(smem + L.dyt);
  float* dzt = (float*)(smem + L.dzt);
  double* imx = (double*)(smem + L.imx);
  double* imy = (double*)(smem + L.imy);
  double* imz = (double*)(smem + L.imz);
  double* red = (double*)(smem + L.red);
  float4* pf = (float4*)(smem + L.pf);
  T* fi = (T*)(smem + L.fi);
  T* fj = (T*)(smem + L.fj);
  float* fic = (float*)(smem + L.fic);
  float* fjc = (float*)(smem + L.fjc);
  double* pd = (double*)(smem + L.px);
  int* gidx = (int*)(smem + L.gidx);
  unsigned short* code = (unsigned short*)(smem + L.code);
  const int cap = A.cap;

  // (1) ext cells: global cell, count, first atom
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
    lstart[e] = A.cstart[gc + 1] - s0;
  }
  // Per-axis tables.  Ext coordinate l (0-based; cell X0 + l - 1) has origin
  // g*bl + n*L, g the wrapped cell, n its periodic image.  Tile-frame origins
  // are taken relative to the tile centre; dyt/dzt hold the exact origin
  // difference between ext rows l and l + d (d = -2..2), rounded once.
  {
    const int a = tid >> 5, l = tid & 31;
    if (a < 3) {
      const int E = a == 0 ? EX : (a == 1 ? EY : EZ);
      const int g0 = a == 0 ? X0 : (a == 1 ? Y0 : Z0);
      const int t = a == 0 ? tx : (a == 1 ? ty : tz);
      const int nb = B.nb[a];
      if (l < E) {
        int g = g0 + l - 1, n = 0;
        if (g < 0) { g += nb; n = -1; }
        if (g >= nb) { g -= nb; n = 1; }
        double org = (double)((float)g * B.blf) + n * B.L[a];
        double centre = (double)((float)g0 * B.blf) + 0.5 * t * B.bl;
        float o = (float)(org - centre);
        (a == 0 ? ox : (a == 1 ? oy : oz))[l] = o;
        (a == 0 ? imx : (a == 1 ? imy : imz))[l] = n * B.L[a];
        if (a > 0) {
          float* dt = a == 1 ? dyt : dzt;
#pragma unroll
          for (int d = -2; d <= 2; ++d) {
            int l2 = l + d;
            float v = 0.f;
            if (l2 >= 0 && l2 < E) {
              int g2 = g0 + l2 - 1, n2 = 0;
              if (g2 < 0) { g2 += nb; n2 = -1; }
              if (g2 >= nb) { g2 -= nb; n2 = 1; }
              double org2 = (double)((float)g2 * B.blf) + n2 * B.L[a];
              v = (float)(org2 - org);
            }
            dt[l * 5 + d + 2] = v;
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
      int y = __shfl_up_sync(0xffffffffu, x, o);
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
    if (tid == blockDim.x - 1) lstart[NE] = run;
    __syncthreads();
  }
  const int total = lstart[NE];
  if (total > cap) {
    if (tid == 0) {
      atomicOr(A.status, ST_OVERFLOW);
      if (ENERGY) {
        A.tileE[tile] = 0.0;
        A.tileW[tile] = 0.0;
      }
      if (COUNT) {
        A.tileC[2 * tile] = 0;
        A.tileC[2 * tile + 1] = 0;
      }
    }
    return;
  }
  // (3) warp row blocks balanced by atoms; rows never split across warps
  if (tid <= nw) {
    long target = (long)tid * total / nw;
    int lo = 0, hi = NR;  // first row R with start(R) >= target
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (lstart[mid * EX] >= target) hi = mid;
      else lo = mid + 1;
    }
    rowb[tid] = (tid == nw) ? NR : lo;
  }
  // (4) stage atoms row by row
  for (int R = warp; R < NR; R += nw) {
    const int e0 = R * EX, a0 = lstart[e0], a1 = lstart[e0 + EX];
    const int ly = R % EY, lz = R / EY;
    for (int t = a0 + lane; t < a1; t += 32) {
      int lx = 0;
      for (int k = 1; k < EX; ++k) lx += (lstart[e0 + k] <= t);
      const int e = e0 + lx;
      const int g = gfirst[e] + (t - lstart[e]);
      const float4 u = A.U[g];
      float4 p;
      if (FP64) {
        p = make_float4(ox[lx] + u.x, oy[ly] + u.y, oz[lz] + u.z, u.w);
        pd[t] = A.X0[g];
        pd[cap + t] = A.X1[g];
        pd[2 * cap + t] = A.X2[g];
      } else {
        p = make_float4(ox[lx] + u.x, u.y, u.z, u.w);
      }
      pf[t] = p;
      gidx[t] = g;
      code[t] = (unsigned short)(lx | (ly << 5) | (lz << 10));
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        fi[c * cap + t] = T(0);
        fj[c * cap + t] = T(0);
        if (COMP) {
          fic[c * cap + t] = 0.f;
          fjc[c * cap + t] = 0.f;
        }
      }
    }
  }
  __syncthreads();

  const int ib = lstart[rowb[warp] * EX], ie = lstart[rowb[warp + 1] * EX];
  const LJ32 q32 = A.lj.p32[0];
  const LJ64 q64 = A.lj.p64[0];
  const float rcpre = A.lj.rc2max * 1.0001f + 1e-4f;  // FP32 prefilter of the FP64 form
  T esum = T(0), wsum = T(0);
  KSum ek, wk;
  int ncand = 0, nacc = 0;

  for (int r = 0; r < kRows; ++r) {
    const int dy = c_own.rows[r][0], dz = c_own.rows[r][1];
    for (int c0 = ib; c0 < ie; c0 += 32) {
      const int i = c0 + lane;
      const bool vi = i < ie;
      const int ci = vi ? code[i] : 0;
      const int lx = ci & 31, ly = (ci >> 5) & 31, lz = ci >> 10;  // 0-based ext coords
      int mask = 0;
      if (vi)
        mask = c_own.lut[pos_class(lx - 1, tx) * 25 + pos_class(ly - 1, ty) * 5 + pos_class(lz - 1, tz)][r];
      if (__ballot_sync(0xffffffffu, mask != 0) == 0u) continue;
      int lo1 = 0, n1 = 0, lo2 = 0, n2 = 0;
      if (mask) {
        const int rowbase = ((ly + dy) + EY * (lz + dz)) * EX + lx - 2;  // + bit b -> ext cell of dx = b - 2
        const int b0 = __ffs(mask) - 1;
        int b1 = b0;
        while (b1 < 4 && ((mask >> (b1 + 1)) & 1)) ++b1;
        lo1 = lstart[rowbase + b0];
        const int hi1 = lstart[rowbase + b1 + 1];
        if (r == kRows - 1 && b0 == 2) lo1 = i + 1;  // pairs inside A: a2 > a1
        n1 = hi1 - lo1;
        const int m2 = mask & ~((2 << b1) - 1);
        if (m2) {
          const int c0b = __ffs(m2) - 1, c1b = 31 - __clz(m2);
          lo2 = lstart[rowbase + c0b];
          n2 = lstart[rowbase + c1b + 1] - lo2;
        }
      }
      int kmn = INT_MAX, kmx = INT_MIN;
      if (n1 > 0) { kmn = lo1 - lane; kmx = lo1 + n1 - 1 - lane; }
      if (n2 > 0) { kmn = min(kmn, lo2 - lane); kmx = max(kmx, lo2 + n2 - 1 - lane); }
      kmn = warp_min(kmn);
      kmx = warp_max(kmx);
      if (kmn > kmx) continue;

      const float4 pi = pf[vi ? i : 0];
      const int ti = __float_as_int(pi.w);
      // per-lane constants of this row: d = p_j + C
      float Cx = -pi.x, Cy, Cz;
      double xi = 0, yi = 0, zi = 0, sy = 0, sz = 0, sxi = 0;
      if (FP64) {
        Cy = -pi.y;
        Cz = -pi.z;
        xi = pd[vi ? i : 0];
        yi = pd[cap + (vi ? i : 0)];
        zi = pd[2 * cap + (vi ? i : 0)];
        const int lyj = min(max(ly + dy, 0), EY - 1), lzj = min(max(lz + dz, 0), EZ - 1);
        sy = imy[lyj] - imy[ly];
        sz = imz[lzj] - imz[lz];
        sxi = imx[lx];
      } else {
        Cy = dyt[ly * 5 + dy + 2] - pi.y;
        Cz = dzt[lz * 5 + dz + 2] - pi.z;
      }
      T ax = T(0), ay = T(0), az = T(0);
      KSum kx, ky, kz;

      for (int k = kmn; k <= kmx; ++k) {
        const int m = lane + k;
        const bool v = ((unsigned)(m - lo1) < (unsigned)n1) | ((unsigned)(m - lo2) < (unsigned)n2);
        if (v) {
          const float4 q = pf[m];
          if (COUNT) ++ncand;
          if (!FP64) {
            const float dx = q.x + Cx, dyv = q.y + Cy, dzv = q.z + Cz;
            const float r2 = fmaf(dx, dx, fmaf(dyv, dyv, dzv * dzv));
            LJ32 P = q32;
            if (MULTI) P = A.lj.p32[ti * A.lj.nt + __float_as_int(q.w)];
            if (r2 <= P.rc2) {
              const float ri = rcp_approx(r2);
              const float s2 = P.sig2 * ri;
              const float s6 = s2 * s2 * s2;
              const float dg = P.m24eps * s6 * fmaf(2.f, s6, -1.f) * ri;
              const float fx = dg * dx, fy = dg * dyv, fz = dg * dzv;
              if (COMP) {
                kx.add(fx);
                ky.add(fy);
                kz.add(fz);
                float* sj = (float*)fj;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                  const float f = c == 0 ? -fx : (c == 1 ? -fy : -fz);
                  float s = sj[c * cap + m], cc = fjc[c * cap + m];
                  float y = f - cc, t = s + y;
                  fjc[c * cap + m] = (t - s) - y;
                  sj[c * cap + m] = t;
                }
              } else {
                ax += fx;
                ay += fy;
                az += fz;
                fj[m] -= fx;
                fj[cap + m] -= fy;
                fj[2 * cap + m] -= fz;
              }
              if (ENERGY) {
                ek.add(P.c4eps * s6 * (s6 - 1.f));
                wk.add(-dg * r2);
              }
              if (COUNT) ++nacc;
            }
          } else {
            // FP32 prefilter on tile-frame coordinates, then the reference's
            // FP64 arithmetic (SRC/exaMD_forces.f90:509-523, user_func.f90:52-69)
            const float fxp = q.x - pi.x, fyp = q.y - pi.y, fzp = q.z - pi.z;
            const float r2f = fmaf(fxp, fxp, fmaf(fyp, fyp, fzp * fzp));
            if (r2f <= rcpre) {
              const int lxj = code[m] & 31;
              const double sx = imx[lxj] - sxi;
              double dx = __dsub_rn(pd[m], xi);
              double dyv = __dsub_rn(pd[cap + m], yi);
              double dzv = __dsub_rn(pd[2 * cap + m], zi);
              // periodic image: physical separation = (x_j - x_i) + (n_j - n_i) L,
              // exact (Sterbenz), equal to the reference's dx - Nint(dx/L) L
              if (sx != 0.0) dx = __dadd_rn(dx, sx);
              if (sy != 0.0) dyv = __dadd_rn(dyv, sy);
              if (sz != 0.0) dzv = __dadd_rn(dzv, sz);
              const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dyv, dyv)), __dmul_rn(dzv, dzv));
              LJ64 P = q64;
              if (MULTI) P = A.lj.p64[ti * A.lj.nt + __float_as_int(q.w)];
              if (d2 <= P.rc2) {
                const double d2i = __drcp_rn(d2);
                const double t = __dmul_rn(P.sig2, d2i);
                const double d6 = __dmul_rn(__dmul_rn(t, t), t);
                const double d12 = __dmul_rn(d6, d6);
                const double dg = -__dmul_rn(__dmul_rn(P.eps24, __dsub_rn(__dmul_rn(2.0, d12), d6)), d2i);
                const double fx = __dmul_rn(dg, dx), fy = __dmul_rn(dg, dyv), fz = __dmul_rn(dg, dzv);
                ax += fx;
                ay += fy;
                az += fz;
                fj[m] -= fx;
                fj[cap + m] -= fy;
                fj[2 * cap + m] -= fz;
                if (ENERGY) {
                  esum += __dmul_rn(P.eps4, __dsub_rn(d12, d6));
                  wsum += -__dmul_rn(dg, d2);
                }
                if (COUNT) ++nacc;
              }
            }
          }
        }
        __syncwarp();
      }
      if (vi) {
        if (COMP) {
          float* si = (float*)fi;
          const float part[3] = {kx.s - kx.c, ky.s - ky.c, kz.s - kz.c};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float s = si[c * cap + i], cc = fic[c * cap + i];
            float y = part[c] - cc, t = s + y;
            fic[c * cap + i] = (t - s) - y;
            si[c * cap + i] = t;
          }
        } else {
          fi[i] += ax;
          fi[cap + i] += ay;
          fi[2 * cap + i] += az;
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }

  // (5) write-back: home atoms -> Fown, halo copies -> P[slot]
  for (int t = tid; t < total; t += blockDim.x) {
    const int ci = code[t];
    const int lx = ci & 31, ly = (ci >> 5) & 31, lz = ci >> 10;
    const int slot = ((lx == 0 || lx == EX - 1) ? 1 : 0) | ((ly == 0 || ly == EY - 1) ? 2 : 0) |
                     ((lz == 0 || lz == EZ - 1) ? 4 : 0);
    const int64_t g = gidx[t];
    if (FP64) {
      double* F = slot == 0 ? (double*)A.Fown : (double*)A.P + (size_t)(slot - 1) * 3 * A.N;
#pragma unroll
      for (int c = 0; c < 3; ++c) F[c * A.N + g] = (double)fi[c * cap + t] + (double)fj[c * cap + t];
    } else {
      float f[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (COMP) {
          KSum k;
          k.s = ((float*)fi)[c * cap + t];
          k.c = fic[c * cap + t];
          k.add(((float*)fj)[c * cap + t]);
          k.add(-fjc[c * cap + t]);
          f[c] = k.s - k.c;
        } else {
          f[c] = (float)fi[c * cap + t] + (float)fj[c * cap + t];
        }
      }
      float4* F = slot == 0 ? (float4*)A.Fown : (float4*)A.P + (size_t)(slot - 1) * A.N;
      F[g] = make_float4(f[0], f[1], f[2], 0.f);
    }
  }

  // (6) per-tile energy / virial / counters
  if (ENERGY || COUNT) {
    double e = 0.0, w = 0.0;
    if (ENERGY) {
      if (FP64) {
        e = (double)esum;
        w = (double)wsum;
      } else {
        e = (double)ek.s - (double)ek.c;
        w = (double)wk.s - (double)wk.c;
      }
    }
    e = warp_sum(e);
    w = warp_sum(w);
    long long c1 = warp_sum((long long)ncand), c2 = warp_sum((long long)nacc);
    __syncthreads();
    if (lane == 0) {
      red[4 * warp] = e;
      red[4 * warp + 1] = w;
      red[4 * warp + 2] = (double)c1;
      red[4 * warp + 3] = (double)c2;
    }
    __syncthreads();
    if (tid == 0) {
      double se = 0, sw = 0, s1 = 0, s2 = 0;
      for (int k = 0; k < nw; ++k) {
        se += red[4 * k];
        sw += red[4 * k + 1];
        s1 += red[4 * k + 2];
        s2 += red[4 * k + 3];
      }
      if (ENERGY) {
        A.tileE[tile] = se;
        A.tileW[tile] = sw;
      }
      if (COUNT) {
        A.tileC[2 * tile] = (long long)s1;
        A.tileC[2 * tile + 1] = (long long)s2;
      }
    }
  }
}

template <bool FP64, bool MULTI, bool KAHAN, bool ENERGY, bool COUNT>
static void* kfn() {
  return (void*)&k_pair<FP64, MULTI, KAHAN, ENERGY, COUNT>;
}

static void* pick(const PairConfig& c) {
  // FP64 ignores KAHAN; instantiate the combinations that are used.
#define EXAMD_PICK(F, M, K)                                              \
  if (c.energy && c.count) return kfn<F, M, K, true, true>();            \
  if (c.energy) return kfn<F, M, K, true, false>();                      \
  if (c.count) return kfn<F, M, K, false, true>();                       \
  return kfn<F, M, K, false, false>();
  if (c.fp64) {
    if (c.multi) { EXAMD_PICK(true, true, false) }
    EXAMD_PICK(true, false, false)
  }
  if (c.multi) {
    if (c.kahan) { EXAMD_PICK(false, true, true) }
    EXAMD_PICK(false, true, false)
  }
  if (c.kahan) { EXAMD_PICK(false, false, true) }
  EXAMD_PICK(false, false, false)
#undef EXAMD_PICK
}

cudaError_t pair_prepare(const PairConfig& cfg, int smem_bytes) {
  return cudaFuncSetAttribute(pick(cfg), cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
}

cudaError_t launch_pair(const PairConfig& cfg, const PairArgs& a, int ntiles, int smem_bytes, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  void* fn = pick(cfg);
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(fn, dim3(ntiles), dim3(32 * cfg.warps), args, (size_t)smem_bytes, st);
}

}  // namespace examd
