// ewald.cu -- reciprocal-space Ewald (FURIR forces.f:1217-1339, INIFUR
// forces.f:1356-1449) and the excluded-pair correction (ETERMS
// forces.f:1482-1676).
//
// The reference loops k-vectors x atoms with one sin and one cos per term.
// Here the k-set INIFUR builds is regrouped into columns of fixed (nx, ny)
// and a contiguous nz range.  With per-atom phase tables
//   X_j(n) = Q_j e^{i n theta_x}, Y_j(n) = e^{i n theta_y}, Z_j(n) = e^{i n theta_z}
// (theta_a = 2 PI a / L_a, PI = 3.1415926536 as the reference truncates it,
// common_inc.f:31), e^{i k.r_j} = X_j(nx) Y_j(ny) Z_j(nz):
//   S(k)   = sum_j T_j(c) Z_j(nz),            T_j(c) = X_j(nx) Y_j(ny)
//   F_j    = sum_c [RXV_c, RYV_c] Im(T_j(c) U_j(c)),  Fz = Im(T_j(c) V_j(c))
//   U_j(c) = sum_{nz} W_k Z_j(nz), V_j(c) = sum_{nz} RZV_k W_k Z_j(nz),
//   W_k    = 2 AKC_k conj(S_k)
// with no transcendental per (k, atom) term.  INIFUR's k-set is symmetric
// in nz within each column (apart from the k = (0, 0, nz > 0) column), and
// Z_j(-n) = conj(Z_j(n)), so both passes take nz = +p and -p together:
//   S(c, +p) = (A1 - A2, A3 + A4),  S(c, -p) = (A1 + A2, A4 - A3)
//   with A1 = sum T.re a, A2 = sum T.im b, A3 = sum T.re b, A4 = sum T.im a,
//   Z_j(p) = a + i b  (4 fused multiply-adds per atom for two k),
//   U += P a + i M b,  P = W(+p) + W(-p),  M = W(+p) - W(-p)  (and V with
//   RZV W), 4 fused multiply-adds per atom for two k.
// Mathematically this is the reference's sum; in FP64 the difference is
// rounding (the recurrence adds about |n| ulp).
//
// Tables are stored n-major (tab[n * N + atom]) so that a warp of atoms
// reads one coalesced row per n.
//
// Mixed path: tables rounded to FP32 after an FP64 recurrence, products and
// the per-slice sums in FP32, S(k) accumulated across slices in FP64, W in
// FP32 for the force pass, forces accumulated per column in 64-bit fixed
// point.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "mdx_internal.cuh"

namespace {

constexpr double PI_REF = 3.1415926536;  // common_inc.f:31
constexpr int CH = 8;                    // nz per chunk of the S(k) kernel
constexpr int SLICE = 512;               // atoms per slice of the S(k) kernel
constexpr int TILE = 32;                 // atoms staged in shared memory
constexpr size_t SFAC_SMEM_MAX = 227 * 1024;

struct Chunk {
  int col, nz0, len, k0;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
template <typename C2>
__device__ __forceinline__ C2 conj_if(C2 v, bool neg) {
  if (neg) v.y = -v.y;
  return v;
}

// Asynchronous global -> shared copies (8 bytes), grouped per staged tile.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait1() {
  asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait0() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Phase tables: thread per (axis, atom), FP64 recurrence from one sincos.
// hexy (hexagonal cell, FP64 path): the x phase is 2 pi (x / BOXL + y / (2
// BOYL)), which makes k . r = IKX theta_x + IKY theta_y + IKZ theta_z with
// RYV = 2 pi IKY + pi IKX (forces.f:1399-1403); 0 otherwise.
__global__ void k_tables(int n, int ldn, const dbl4 *__restrict__ pos, double ibx,
                         double iby, double ibz, int kx, int ky, int kz,
                         double2 *__restrict__ tx, double2 *__restrict__ ty,
                         double2 *__restrict__ tz, float2 *__restrict__ txf,
                         float2 *__restrict__ tyf, float2 *__restrict__ tzf,
                         const int4 *__restrict__ posi, double hexy) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * n) return;
  const int a = t / n, i = t - a * n;
  if (txf) {
    // mixed path, FP32 table (row stride ldn): every entry from its own
    // phase.  k times the 32-bit fixed-point coordinate is k x / L modulo
    // one turn, exactly (integer wrap-around), a signed fraction of half a
    // turn in units of 2^-31.  Its top 24 bits are exact in FP32 and go to
    // sincospif; the low 8 bits (under 3.7e-7 rad) rotate the result to
    // first order.  No recurrence, no FP64 work.
    // hexagonal cell (hexy != 0): the y word is y / (2 BOYL), and the X
    // table's phase is x / BOXL + y / (2 BOYL) (RYV = 2 pi IKY + pi IKX,
    // forces.f:1402): the sum of the words; the Y table's, twice the y word
    const int4 pq = posi[i];
    const bool hex = hexy != 0.0;
    const unsigned u = a == 0   ? (hex ? (unsigned)pq.x + (unsigned)pq.y : (unsigned)pq.x)
                       : a == 1 ? (hex ? 2u * (unsigned)pq.y : (unsigned)pq.y)
                                : (unsigned)pq.z;
    const float qf = a == 0 ? (float)pos[i].w : 1.0f;
    const int len = a == 0 ? kx : a == 1 ? ky : kz;
    float2 *dst = (a == 0 ? txf : a == 1 ? tyf : tzf) + i;
    for (int k = 0; k < len; ++k) {
      const int ph = (int)((unsigned)k * u);
      const int hi = ph & ~0xff, lo = ph - hi;
      float s, c;
      sincospif((float)hi * 4.656612873077393e-10f, &s, &c);  // 2^-31
      const float d = (float)lo * 1.4629180792671596e-09f;    // pi 2^-31
      dst[(size_t)k * ldn] = make_float2(qf * fmaf(-s, d, c), qf * fmaf(c, d, s));
    }
    return;
  }
  const dbl4 p = pos[i];
  double x = a == 0 ? p.x * ibx : a == 1 ? p.y * iby : p.z * ibz;
  if (a == 0 && hexy != 0.0) x = fma(p.y, hexy, x);
  double s, c;
  sincos(2.0 * PI_REF * x, &s, &c);
  const double2 e = make_double2(c, s);
  // rows n = 0..K (negative n are the conjugates, never stored)
  const int len = a == 0 ? kx : a == 1 ? ky : kz;
  const double q = a == 0 ? p.w : 1.0;
  double2 v = make_double2(1.0, 0.0);
  double2 *dst = (a == 0 ? tx : a == 1 ? ty : tz) + i;
  for (int k = 0; k < len; ++k) {
    dst[(size_t)k * n] = make_double2(q * v.x, q * v.y);
    v = cmul(v, e);
  }
}

// Write one paired accumulator as S(c, +p) and S(c, -p) (each only if the
// k-vector exists): slice partial (summed in a fixed order by k_sfac_sum) or
// atomic.
__device__ __forceinline__ void sfac_out(const KCol &col, int p, double A1, double A2,
                                         double A3, double A4, double2 *part, double2 *sk) {
  const int z = kcol_z(col, p);
  const int kp = kcol_k(col, z), km = z > 0 ? kcol_k(col, -z) : -1;
  const double2 vp = make_double2(A1 - A2, A3 + A4), vm = make_double2(A1 + A2, A4 - A3);
  if (part) {
    if (kp >= 0) part[kp] = vp;
    if (km >= 0) part[km] = vm;
  } else {
    if (kp >= 0) {
      atomicAdd(&sk[kp].x, vp.x);
      atomicAdd(&sk[kp].y, vp.y);
    }
    if (km >= 0) {
      atomicAdd(&sk[km].x, vm.x);
      atomicAdd(&sk[km].y, vm.y);
    }
  }
}

// FP64 S(k): thread per chunk (column, CH consecutive p from p0), block.y =
// slice of SLICE atoms staged TILE at a time in shared memory.
__global__ void __launch_bounds__(128) k_sfac(
    int n, int nchunk, const Chunk *__restrict__ chunks,
    const KCol *__restrict__ cols, const double2 *__restrict__ tx,
    const double2 *__restrict__ ty, const double2 *__restrict__ tz, int kx, int ky,
    int kz, double2 *__restrict__ sk, double2 *__restrict__ part, int nkv) {
  extern __shared__ unsigned char smem_raw[];
  double2 *sx = reinterpret_cast<double2 *>(smem_raw);  // [atom][n]
  double2 *sy = sx + TILE * kx;
  double2 *sz = sy + TILE * ky;
  const int ch = blockIdx.x * blockDim.x + threadIdx.x;
  const int a0 = blockIdx.y * SLICE, a1 = min(n, a0 + SLICE);
  Chunk cc{0, 0, 0, 0};
  KCol col{0, 0, 0, 0, 0, 0, 0, 0, 0, 1};
  if (ch < nchunk) {
    cc = chunks[ch];
    col = cols[cc.col];
  }
  const int ny = col.ny < 0 ? -col.ny : col.ny;
  const bool nyneg = col.ny < 0;
  double A[CH][4];
#pragma unroll
  for (int t = 0; t < CH; ++t) A[t][0] = A[t][1] = A[t][2] = A[t][3] = 0.0;
  for (int base = a0; base < a1; base += TILE) {
    const int m = min(TILE, a1 - base);
    __syncthreads();
    for (int k = threadIdx.x; k < m * kx; k += blockDim.x) {
      const int nn = k / m, j = k - nn * m;
      sx[j * kx + nn] = tx[(size_t)nn * n + base + j];
    }
    for (int k = threadIdx.x; k < m * ky; k += blockDim.x) {
      const int nn = k / m, j = k - nn * m;
      sy[j * ky + nn] = ty[(size_t)nn * n + base + j];
    }
    for (int k = threadIdx.x; k < m * kz; k += blockDim.x) {
      const int nn = k / m, j = k - nn * m;
      sz[j * kz + nn] = tz[(size_t)nn * n + base + j];
    }
    __syncthreads();
    if (ch < nchunk) {
      for (int j = 0; j < m; ++j) {
        const double2 X = sx[j * kx + col.nx];
        const double2 Y = conj_if(sy[j * ky + ny], nyneg);
        const double tr = fma(X.x, Y.x, -X.y * Y.y), ti = fma(X.x, Y.y, X.y * Y.x);
        const double2 *zr = sz + j * kz + kcol_z(col, cc.nz0);
        const int zs = col.zstep;
        // chunks are sorted by length, so a warp's lanes mostly leave
        // together and a short chunk issues only its own FMAs
#pragma unroll
        for (int t = 0; t < CH; ++t) {
          if (t >= cc.len) break;
          const double2 Z = zr[zs * t];
          A[t][0] = fma(tr, Z.x, A[t][0]);
          A[t][1] = fma(ti, Z.y, A[t][1]);
          A[t][2] = fma(tr, Z.y, A[t][2]);
          A[t][3] = fma(ti, Z.x, A[t][3]);
        }
      }
    }
  }
  if (ch < nchunk) {
    double2 *pp = part ? part + (size_t)blockIdx.y * nkv : nullptr;
#pragma unroll
    for (int t = 0; t < CH; ++t)
      if (t < cc.len) sfac_out(col, cc.nz0 + t, A[t][0], A[t][1], A[t][2], A[t][3], pp, sk);
  }
}

// Mixed S(k) pass.  A work item is (column group, window of SCH values of p
// from p0); a thread accumulates 4 columns x SCH paired sums (A1..A4) in
// FP32 registers over one slice of atoms, staged TILE at a time in shared
// memory as one row per atom: X(0..KMAX), Y(0..KMAY), Z(0..KMAZ) and SCH
// zeros (windows past KMAZ and padding columns read zeros).  Tiles are
// double buffered: the next tile's cp.async copies run under this tile's
// FMAs.  Items are sorted by p0 so the lanes of a warp mostly read the same
// z entries (shared-memory broadcast).  The slice length is chosen on the
// host so the grid is one full wave of resident blocks.
constexpr int SCH = 4;
struct SItem {
  int g, t0;
};

// 4 blocks a SM (128 registers, a few spilled): measured 4 % faster than 3
template <int ZS>
__global__ void __launch_bounds__(128, 4) k_sfac32(
    int n, int nitem, const SItem *__restrict__ items, const KGroup *__restrict__ groups,
    const KCol *__restrict__ cols, const float2 *__restrict__ tab, int ldn, int kx, int ky,
    int kz, int slice, double2 *__restrict__ sk, double2 *__restrict__ part, int nkv) {
  // tab: the X, Y and Z tables back to back, row r at tab + r * ldn;
  // ZS: the z step of the records, 2 for the octahedron's k-set (a window
  // reads every other z); a template parameter, so that the rectangular
  // and hexagonal windows keep constant offsets
  constexpr int zstep = ZS;
  extern __shared__ float2 srow[];  // [2][TILE][kx + ky + kz + SCH zstep], double buffer
  const int zpad = kx + ky + kz;    // first zero entry of a row
  const int nzp = SCH * zstep;      // zeros after the z rows
  const int rowlen = zpad + nzp;
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  const int a0 = blockIdx.y * slice, a1 = min(n, a0 + slice);
  const bool active = it < nitem;
  int xo[KGRP], yo[KGRP];
  unsigned ysg[KGRP];  // sign bit flips Im Y for ny < 0
  int zo = 0;
  {
    const SItem si = active ? items[it] : SItem{0, 0};
    const KGroup &G = groups[si.g];
#pragma unroll
    for (int c = 0; c < KGRP; ++c) {
      const int ci = active ? G.col[c] : -1;
      const KCol col = ci >= 0 ? cols[ci] : KCol{0, 0, 0, 0, 0, 0, 0, 0, 0, 1};
      xo[c] = ci >= 0 ? col.nx : zpad;  // padding column: X = 0
      yo[c] = kx + (col.ny < 0 ? -col.ny : col.ny);
      ysg[c] = col.ny < 0 ? 0x80000000u : 0u;
    }
    zo = kx + ky + G.zoff + zstep * si.t0;
  }
  // the four sums of (column c, p) as two pairs, P = (A1, A3) and
  // Q = (A4, A2) of the paired-record scheme, each advanced by one paired
  // FP32 FMA (FFMA2) per atom: P += (tr, tr) (Z.re, Z.im), Q += (ti, ti)
  // (Z.re, Z.im).  Each half is the same rounded FMA in the same order as a
  // scalar fmaf, so the sums are those of four scalar accumulators.
  float2 P[KGRP][SCH], Q[KGRP][SCH];
#pragma unroll
  for (int c = 0; c < KGRP; ++c)
#pragma unroll
    for (int s = 0; s < SCH; ++s) P[c][s] = Q[c][s] = make_float2(0.f, 0.f);
  const int bufsz = TILE * rowlen;
  for (int k = threadIdx.x; k < 2 * TILE * nzp; k += blockDim.x)
    srow[(k / nzp) * rowlen + zpad + k % nzp] = make_float2(0.f, 0.f);
  // stage a tile of atoms asynchronously (cp.async, one group per tile)
  auto stage = [&](int buf, int base) {
    const int m = min(TILE, a1 - base);
    float2 *dst = srow + buf * bufsz;
    for (int k = threadIdx.x; k < m * zpad; k += blockDim.x) {
      const int r = k / m, j = k - r * m;
      cp_async8(dst + j * rowlen + r, tab + (size_t)r * ldn + base + j);
    }
  };
  if (a0 < a1) stage(0, a0);
  cp_async_commit();
  int t = 0;
  for (int base = a0; base < a1; base += TILE, ++t) {
    if (base + TILE < a1) stage((t + 1) & 1, base + TILE);
    cp_async_commit();
    cp_async_wait1();
    __syncthreads();
    const int m = min(TILE, a1 - base);
    if (active) {
#pragma unroll 2  // two atoms' loads in flight (measured 7 % faster than 1 and 4)
      for (int j = 0; j < m; ++j) {
        const float2 *row = srow + (t & 1) * bufsz + j * rowlen;
        float tr[KGRP], ti[KGRP];
#pragma unroll
        for (int c = 0; c < KGRP; ++c) {
          const float2 X = row[xo[c]];
          const float2 Y = row[yo[c]];
          const float yy = __uint_as_float(__float_as_uint(Y.y) ^ ysg[c]);
          tr[c] = fmaf(X.x, Y.x, -X.y * yy);
          ti[c] = fmaf(X.x, yy, X.y * Y.x);
        }
        const float2 *zr = row + zo;
#pragma unroll
        for (int s = 0; s < SCH; ++s) {
          const float2 Z = zr[zstep * s];
#pragma unroll
          for (int c = 0; c < KGRP; ++c) {
            P[c][s] = __ffma2_rn(make_float2(tr[c], tr[c]), Z, P[c][s]);
            Q[c][s] = __ffma2_rn(make_float2(ti[c], ti[c]), Z, Q[c][s]);
          }
        }
      }
    }
    __syncthreads();  // buffer (t & 1) is restaged two tiles later
  }
  cp_async_wait0();
  if (!active) return;
  const SItem si = items[it];
  const KGroup &G = groups[si.g];
  double2 *pp = part ? part + (size_t)blockIdx.y * nkv : nullptr;
#pragma unroll
  for (int c = 0; c < KGRP; ++c) {
    const int ci = G.col[c];
    if (ci < 0) continue;
    const KCol col = cols[ci];
#pragma unroll
    for (int s = 0; s < SCH; ++s)
      if (si.t0 + s <= G.m)
        sfac_out(col, si.t0 + s, (double)P[c][s].x, (double)Q[c][s].y, (double)P[c][s].y,
                 (double)Q[c][s].x, pp, sk);
  }
}

// S(k) = sum of the slice partials in slice order (deterministic).
constexpr int SUM_K = 32, SUM_G = 8;  // k-vectors and slice groups of a block

// S(k) = the sum of the slice partials: thread (k, g) adds slices g, g +
// SUM_G, ... in order, then the groups are added in group order (a fixed
// order: deterministic); reads are coalesced over k.
__global__ void __launch_bounds__(SUM_K * SUM_G) k_sfac_sum(int nkv, int nslice,
                                                         const double2 *__restrict__ part,
                                                         double2 *__restrict__ sk) {
  __shared__ double2 sh[SUM_G][SUM_K];
  const int kl = threadIdx.x % SUM_K, g = threadIdx.x / SUM_K;
  const int k = blockIdx.x * SUM_K + kl;
  double x = 0.0, y = 0.0;
  if (k < nkv)
    for (int s = g; s < nslice; s += SUM_G) {
      const double2 v = part[(size_t)s * nkv + k];
      x += v.x;
      y += v.y;
    }
  sh[g][kl] = make_double2(x, y);
  __syncthreads();
  if (g == 0 && k < nkv) {
#pragma unroll
    for (int q = 1; q < SUM_G; ++q) {
      x += sh[q][kl].x;
      y += sh[q][kl].y;
    }
    sk[k] = make_double2(x, y);
  }
}

// Per k: energy and virial terms (forces.f:1316-1331), W_k and RZV W_k.
// Per-k constants of FURIR that depend on the box and alpha only (forces.f:
// 1316-1331): AKC, (RXV^2, RYV^2, RZV^2) AKV and RZV, five doubles per k,
// and the column's (RXV, RYV); rebuilt when the box or alpha changes.
// hexk: pi for the hexagonal cell (RYV = 2 pi IKY + pi IKX, forces.f:1402),
// 0 otherwise.
__global__ void k_kconst(int ncol, const KCol *__restrict__ cols, double bx, double by,
                         double bz, double alp2, double cfur, double *__restrict__ kc,
                         double2 *__restrict__ colrv, float2 *__restrict__ colrvf,
                         double hexk) {
  const double twopi = 2.0 * PI_REF;
  for (int c = blockIdx.x; c < ncol; c += gridDim.x) {
    const KCol col = cols[c];
    const int len = (col.nzhi - col.nzlo) / col.zstep + 1;
    const double ryv = hexk != 0.0 ? twopi * col.ny + hexk * col.nx : twopi * col.ny;
    if (threadIdx.x == 0) {
      const double rx = (twopi * col.nx) / bx, ry = ryv / by;
      colrv[c] = make_double2(rx, ry);
      colrvf[c] = make_float2((float)rx, (float)ry);
    }
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int k = col.koff + t;
      const int nz = col.nzlo + col.zstep * t;
      const double RXV = (twopi * col.nx) / bx;
      const double RYV = ryv / by;
      const double RZV = (twopi * nz) / bz;
      const double RK2 = RXV * RXV + RYV * RYV + RZV * RZV;
      const double AKC = cfur * exp(-0.25 * RK2 / alp2) / RK2;
      const double AKV = 0.5 * AKC * (4. * alp2 + RK2) / (alp2 * RK2);
      double *q = kc + 5 * (size_t)k;
      q[0] = AKC;
      q[1] = (RXV * RXV) * AKV;
      q[2] = (RYV * RYV) * AKV;
      q[3] = (RZV * RZV) * AKV;
      q[4] = RZV;
    }
  }
}

// Per k: energy and virial terms (forces.f:1316-1331), W_k and RZV W_k, from
// S(k) and the per-k constants (the same products as the reference's
// expressions, in its order).
__global__ void k_kterms(int nkv, const double2 *__restrict__ sk,
                         const double *__restrict__ kc, dbl4 *__restrict__ wk, Dst6 dst) {
  double acc[4] = {0, 0, 0, 0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nkv; k += gridDim.x * blockDim.x) {
    const double2 S = sk[k];
    const double SCS = S.x, SSN = S.y;
    const double *q = kc + 5 * (size_t)k;
    const double AKC = q[0];
    const double S2 = SSN * SSN + SCS * SCS;
    acc[0] += AKC * S2;
    acc[1] -= q[1] * S2;
    acc[2] -= q[2] * S2;
    acc[3] -= q[3] * S2;
    const double AK2 = 2.0 * AKC;
    dbl4 W;
    W.x = AK2 * SCS;
    W.y = -AK2 * SSN;
    W.z = q[4] * W.x;
    W.w = q[4] * W.y;
    wk[k] = W;
  }
  block_add<4>(acc, dst);
}

// Paired W per (column, p): P = W(+p) + W(-p), M = W(+p) - W(-p) for U, the
// same of RZV W for V (a missing k counts as W = 0; p = 0 gives P = W(0),
// M = 0).  FP64: wp64[2 (poff + p) + {0, 1}] = {P_U, M_U}, {P_V, M_V};
// mixed: the group-interleaved FP32 records of KGroup.
__global__ void k_wpairs(int ncol, const KCol *__restrict__ cols, const dbl4 *__restrict__ wk,
                         dbl4 *__restrict__ wp64, float4 *__restrict__ wp32) {
  for (int c = blockIdx.x; c < ncol; c += gridDim.x) {
    const KCol col = cols[c];
    for (int p = threadIdx.x; p <= col.m; p += blockDim.x) {
      const int z = kcol_z(col, p);
      const int kp = kcol_k(col, z), km = z > 0 ? kcol_k(col, -z) : -1;
      dbl4 a, b;
      a.x = a.y = a.z = a.w = 0.0;
      b = a;
      if (kp >= 0) a = wk[kp];
      if (km >= 0) b = wk[km];
      dbl4 u, v;  // {P, M} of W, of RZV W
      u.x = a.x + b.x;
      u.y = a.y + b.y;
      u.z = a.x - b.x;
      u.w = a.y - b.y;
      v.x = a.z + b.z;
      v.y = a.w + b.w;
      v.z = a.z - b.z;
      v.w = a.w - b.w;
      if (wp32) {
        float4 *r = wp32 + col.wpos + 8 * (size_t)p;  // wpos = 8 woff + 2 slot
        r[0] = make_float4((float)u.x, (float)u.y, (float)u.z, (float)u.w);
        r[1] = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
      } else {
        wp64[2 * (size_t)(col.poff + p)] = u;
        wp64[2 * (size_t)(col.poff + p) + 1] = v;
      }
    }
  }
}

// QPE into PELS1 and the three virial projections (forces.f:1333-1336).
__global__ void k_qpe_fold(mdx_scalars *sc, double *qpe) {
  const double Q = *qpe;
  sc->virx = sc->virx + Q;
  sc->viry = sc->viry + Q;
  sc->virz = sc->virz + Q;
  sc->pels1 = sc->pels1 + Q;
  sc->qpe = Q;
  *qpe = 0.0;
}

// Force passes: a block is RF_ATOMS atoms x RF_PARTS column parts (one warp
// per part); part p takes columns p, p + RF_PARTS, ... and the parts are
// added in part order through shared memory, so the sum is deterministic.
constexpr int RF_ATOMS = 32;
constexpr int RF_PARTS = 4;

// FP64 force pass: U = sum_p P_U a + i M_U b over p = 0..m of each column
// (Z(p) = a + i b), V the same with P_V, M_V; then F += rv Im(T U), Im(T V).
__global__ void __launch_bounds__(RF_ATOMS *RF_PARTS) k_rforce64(
    int n, int ncol, const KCol *__restrict__ cols, const dbl4 *__restrict__ wp,
    const double2 *__restrict__ tx, const double2 *__restrict__ ty,
    const double2 *__restrict__ tz, const double2 *__restrict__ colrv,
    double *__restrict__ gx, double *__restrict__ gy, double *__restrict__ gz) {
  __shared__ double red[3][RF_PARTS][RF_ATOMS];
  const int lane = threadIdx.x % RF_ATOMS, part = threadIdx.x / RF_ATOMS;
  const int i = blockIdx.x * RF_ATOMS + lane;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (i < n) {
    const double2 *Z = tz + i;
    for (int c = part; c < ncol; c += RF_PARTS) {
      const KCol col = cols[c];
      double ux = 0., uy = 0., vx = 0., vy = 0.;
      const dbl4 *w = wp + 2 * (size_t)col.poff;
#pragma unroll 4
      for (int p = 0; p <= col.m; ++p) {
        const double2 z = Z[(size_t)kcol_z(col, p) * n];
        const dbl4 u = w[2 * p], v = w[2 * p + 1];
        ux = fma(u.x, z.x, ux);
        ux = fma(-u.w, z.y, ux);
        uy = fma(u.y, z.x, uy);
        uy = fma(u.z, z.y, uy);
        vx = fma(v.x, z.x, vx);
        vx = fma(-v.w, z.y, vx);
        vy = fma(v.y, z.x, vy);
        vy = fma(v.z, z.y, vy);
      }
      const int ny = col.ny < 0 ? -col.ny : col.ny;
      const double2 T = cmul(tx[(size_t)col.nx * n + i],
                             conj_if(ty[(size_t)ny * n + i], col.ny < 0));
      const double imTU = fma(T.x, uy, T.y * ux);
      const double imTV = fma(T.x, vy, T.y * vx);
      const double2 rv = colrv[c];
      fx = fma(rv.x, imTU, fx);
      fy = fma(rv.y, imTU, fy);
      fz += imTV;
    }
  }
  red[0][part][lane] = fx;
  red[1][part][lane] = fy;
  red[2][part][lane] = fz;
  __syncthreads();
  if (part == 0 && i < n) {
#pragma unroll
    for (int p = 1; p < RF_PARTS; ++p) {
      fx += red[0][p][lane];
      fy += red[1][p][lane];
      fz += red[2][p][lane];
    }
    gx[i] += fx;
    gy[i] += fy;
    gz[i] += fz;
  }
}

// Mixed force pass over column groups.  A block holds RF_APT x 32 atoms (a
// thread takes atoms lane and lane + 32) and RF_PARTS warps; the groups are
// cut into nsplit x RF_PARTS contiguous ranges (parts[], balanced by W
// records) and warp w of block (tile, s) takes range s RF_PARTS + w, whose
// paired-W records are contiguous too.  nsplit > 1 spreads one atom tile
// over several blocks so the grid fills the last wave of resident blocks;
// their fixed-point partials meet in integer atomics (order independent).  The block's Z rows (p = 0..KMAZ) are staged in shared
// memory ([row][atom], conflict-free); X and Y (read once per column) come
// through L1/L2.  Each warp streams its records through a two-batch
// shared-memory ring with cp.async (RF_WB records of 8 float4 a batch, one
// 16-byte copy per lane), so W latency hides under the FMAs of the previous
// batch.  Per p and atom one z load; per p eight broadcast loads feed 32 FMAs
// per atom covering 8 k-vectors.
constexpr int RF_APT = 2;
constexpr int RF_BATOMS = 32 * RF_APT;
constexpr int RF_REC = 2 * KGRP;  // float4 per record (4 columns x {U, V})
constexpr int RF_WB = 32 / RF_REC;  // records per batch (one float4 per lane)

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

template <int ZS>
__global__ void __launch_bounds__(32 * RF_PARTS, 6) k_rforce32(
    int n, const int *__restrict__ parts, const KGroup *__restrict__ groups,
    const KCol *__restrict__ cols,
    const float4 *__restrict__ wg, const float2 *__restrict__ tab, int ldn, int kx, int ky,
    int kz, const float2 *__restrict__ colrv, FixScale fsc,
    unsigned long long *__restrict__ gfix) {
  constexpr int zstep = ZS;  // z step of the records (2: truncated octahedron)
  // tab: the X, Y and Z tables back to back, row r at tab + r * ldn
  extern __shared__ float2 srf[];  // [kz][RF_BATOMS]
  __shared__ long long red[3][RF_PARTS][RF_BATOMS];
  __shared__ float4 ring[RF_PARTS][2][RF_WB * RF_REC];
  const int lane = threadIdx.x % 32, part = threadIdx.x / 32;
  const int i0 = blockIdx.x * RF_BATOMS;
  const float2 *tz = tab + (size_t)(kx + ky) * ldn;
  for (int k = threadIdx.x; k < kz * RF_BATOMS; k += blockDim.x) {
    const int r = k / RF_BATOMS, j = k - r * RF_BATOMS;
    srf[k] = i0 + j < n ? tz[(size_t)r * ldn + i0 + j] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // per atom and axis: the group sums (4 columns, FP32) accumulated with
  // Kahan compensation (fs, fc), fixed order -> deterministic
  float fs[RF_APT][3], fc[RF_APT][3];
#pragma unroll
  for (int q = 0; q < RF_APT; ++q)
#pragma unroll
    for (int a = 0; a < 3; ++a) fs[q][a] = fc[q][a] = 0.f;
  int iq[RF_APT];  // this thread's atoms, clamped for the table reads
#pragma unroll
  for (int q = 0; q < RF_APT; ++q) iq[q] = min(i0 + lane + 32 * q, n - 1);
  const float2 *Z = srf + lane;  // row p = 0
  const int gs = parts[blockIdx.y * RF_PARTS + part];
  const int ge = parts[blockIdx.y * RF_PARTS + part + 1];
  if (gs < ge) {
    const int rs = groups[gs].woff;
    const int re = groups[ge - 1].woff + groups[ge - 1].len;
    float4 *wr = &ring[part][0][0];
    // lane copies float4 lane % RF_REC of record (batch start + lane / RF_REC)
    auto issue = [&](int buf, int rec0) {
      const int rec = rec0 + lane / RF_REC;
      if (rec < re)
        cp_async16(wr + buf * RF_WB * RF_REC + lane, wg + (size_t)RF_REC * rec + lane % RF_REC);
    };
    issue(0, rs);
    cp_async_commit();
    int r = rs, next = rs + RF_WB;
    for (int g = gs; g < ge; ++g) {
      const KGroup G = groups[g];
      float u[RF_APT][KGRP][2], v[RF_APT][KGRP][2];
#pragma unroll
      for (int q = 0; q < RF_APT; ++q)
#pragma unroll
        for (int c = 0; c < KGRP; ++c) u[q][c][0] = u[q][c][1] = v[q][c][0] = v[q][c][1] = 0.f;
      for (int p = 0; p < G.len; ++p, ++r) {
        const int qb = r - rs;
        if (qb % RF_WB == 0) {  // batch boundary: this batch landed, prefetch the next
          cp_async_wait0();
          __syncwarp();
          if (next < re) issue((qb / RF_WB + 1) & 1, next);
          cp_async_commit();
          next += RF_WB;
        }
        const float4 *w = wr + (((qb / RF_WB) & 1) * RF_WB + qb % RF_WB) * RF_REC;
        float2 zz[RF_APT];
#pragma unroll
        for (int q = 0; q < RF_APT; ++q) zz[q] = Z[(G.zoff + zstep * p) * RF_BATOMS + 32 * q];
#pragma unroll
        for (int c = 0; c < KGRP; ++c) {
          const float4 pu = w[2 * c], pv = w[2 * c + 1];  // {P.re, P.im, M.re, M.im}
#pragma unroll
          for (int q = 0; q < RF_APT; ++q) {
            u[q][c][0] = fmaf(pu.x, zz[q].x, u[q][c][0]);
            u[q][c][0] = fmaf(-pu.w, zz[q].y, u[q][c][0]);
            u[q][c][1] = fmaf(pu.y, zz[q].x, u[q][c][1]);
            u[q][c][1] = fmaf(pu.z, zz[q].y, u[q][c][1]);
            v[q][c][0] = fmaf(pv.x, zz[q].x, v[q][c][0]);
            v[q][c][0] = fmaf(-pv.w, zz[q].y, v[q][c][0]);
            v[q][c][1] = fmaf(pv.y, zz[q].x, v[q][c][1]);
            v[q][c][1] = fmaf(pv.z, zz[q].y, v[q][c][1]);
          }
        }
      }
      float gs[RF_APT][3];
#pragma unroll
      for (int q = 0; q < RF_APT; ++q) gs[q][0] = gs[q][1] = gs[q][2] = 0.f;
#pragma unroll
      for (int c = 0; c < KGRP; ++c) {
        if (G.col[c] < 0) continue;
        const KCol col = cols[G.col[c]];
        const int ny = col.ny < 0 ? -col.ny : col.ny;
        const float2 rv = colrv[G.col[c]];
#pragma unroll
        for (int q = 0; q < RF_APT; ++q) {
          const float2 T = cmulf(__ldg(&tab[(size_t)col.nx * ldn + iq[q]]),
                                 conj_if(__ldg(&tab[(size_t)(kx + ny) * ldn + iq[q]]), col.ny < 0));
          const float imTU = fmaf(T.x, u[q][c][1], T.y * u[q][c][0]);
          const float imTV = fmaf(T.x, v[q][c][1], T.y * v[q][c][0]);
          gs[q][0] = fmaf(rv.x, imTU, gs[q][0]);
          gs[q][1] = fmaf(rv.y, imTU, gs[q][1]);
          gs[q][2] += imTV;
        }
      }
#pragma unroll
      for (int q = 0; q < RF_APT; ++q)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float y = gs[q][a] - fc[q][a];
          const float t = fs[q][a] + y;
          fc[q][a] = (t - fs[q][a]) - y;
          fs[q][a] = t;
        }
    }
    cp_async_wait0();
  }
  // to 64-bit fixed point (scale a power of two: exact products)
  const float sc = fsc.scalef;
#pragma unroll
  for (int q = 0; q < RF_APT; ++q)
#pragma unroll
    for (int a = 0; a < 3; ++a)
      red[a][part][lane + 32 * q] = f2ll_rn(fs[q][a] * sc) - f2ll_rn(fc[q][a] * sc);
  __syncthreads();
  for (int j = threadIdx.x; j < RF_BATOMS; j += blockDim.x) {
    const int i = i0 + j;
    if (i >= n) continue;
    long long sx = 0, sy = 0, sz = 0;
#pragma unroll
    for (int p = 0; p < RF_PARTS; ++p) {
      sx += red[0][p][j];
      sy += red[1][p][j];
      sz += red[2][p][j];
    }
    if (gridDim.y == 1) {
      gfix[i] += (unsigned long long)sx;
      gfix[n + i] += (unsigned long long)sy;
      gfix[2 * n + i] += (unsigned long long)sz;
    } else {
      atomicAdd(&gfix[i], (unsigned long long)sx);
      atomicAdd(&gfix[n + i], (unsigned long long)sy);
      atomicAdd(&gfix[2 * n + i], (unsigned long long)sz);
    }
  }
}

// ETERMS (forces.f:1482-1676): thread per atom ISP over its bound partners
// JSP < ISP (normal types), or over all intramolecular pairs of EE types.
// R = double: the FP64 path; R = float (mixed path, gfix set): the pair's
// FP64 minimum-image vector rounded to FP32, the rest in FP32, forces to
// 64-bit fixed point with FP32 operations only.  Energy and virial sums are
// FP64 either way.
template <typename R>
__device__ __forceinline__ void eterms_pair(
    int isp, int jsp, int ityp, const dbl4 &pi, const dbl4 &pj, double coulf,
    double alphad, double bx, double by, double bz, const CellPbc &cell, const TypeConst &tc,
    R *acc, double *gx, double *gy, double *gz,
    unsigned long long *gfix, int n, float fscalef) {
  double DXd = pi.x - pj.x, DYd = pi.y - pj.y, DZd = pi.z - pj.z;
  if (cell.icell == 0) pbc_rect(DXd, DYd, DZd, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
  else pbc_cell(DXd, DYd, DZd, cell);  // forces.f:1516-1551
  const R QIJ = (R)(coulf * pi.w * pj.w);
  const R DX = (R)DXd, DY = (R)DYd, DZ = (R)DZd;
  const R R2 = DX * DX + DY * DY + DZ * DZ;
  const R R2I = R(1) / R2;
  const R R1 = sqrt(R2);
  const R R1I = R1 * R2I;
  const R ALPHAR = (R)alphad * R1;
  const R TTT = R(1) / (R(1) + (R)MDX_B1 * ALPHAR);
  const R EXP2A = exp(-(ALPHAR * ALPHAR));
  const R ERFC = (((((R)MDX_A5 * TTT + (R)MDX_A4) * TTT + (R)MDX_A3) * TTT + (R)MDX_A2) * TTT +
                  (R)MDX_A1) * TTT * EXP2A;
  const R EES = QIJ * (ERFC - R(1)) * R1I;
  acc[0] += EES;
  if (tc.lmove[ityp]) {
    const R FES = QIJ * (((R)MDX_TOTPI * ALPHAR * EXP2A + ERFC) - R(1)) * R1I * R2I;
    const R FX = FES * DX, FY = FES * DY, FZ = FES * DZ;
    if (gfix) {
      const long long qx = f2ll_rn((float)FX * fscalef), qy = f2ll_rn((float)FY * fscalef),
                      qz = f2ll_rn((float)FZ * fscalef);
      atomicAdd(&gfix[isp], (unsigned long long)qx);
      atomicAdd(&gfix[n + isp], (unsigned long long)qy);
      atomicAdd(&gfix[2 * n + isp], (unsigned long long)qz);
      atomicAdd(&gfix[jsp], (unsigned long long)-qx);
      atomicAdd(&gfix[n + jsp], (unsigned long long)-qy);
      atomicAdd(&gfix[2 * n + jsp], (unsigned long long)-qz);
    } else {
      atomicAdd(&gx[isp], (double)FX);
      atomicAdd(&gy[isp], (double)FY);
      atomicAdd(&gz[isp], (double)FZ);
      atomicAdd(&gx[jsp], -(double)FX);
      atomicAdd(&gy[jsp], -(double)FY);
      atomicAdd(&gz[jsp], -(double)FZ);
    }
    acc[1] += FES * (DX * DX);
    acc[2] += FES * (DY * DY);
    acc[3] += FES * (DZ * DZ);
  }
}

template <typename R>
__global__ void k_eterms(int n, const dbl4 *__restrict__ pos,
                         const int4 *__restrict__ ainfo,
                         const int *__restrict__ nnbb,
                         const int *__restrict__ inbb, int nbdmax,
                         const int *__restrict__ mol_first, TypeConst tc,
                         double coulf, double alphad, double bx, double by,
                         double bz, CellPbc cell, double *gx, double *gy, double *gz,
                         unsigned long long *gfix, float fscalef, Dst6 dst,
                         double *spee) {
  __shared__ double spee_sh[MDX_NT];
  if (threadIdx.x < MDX_NT) spee_sh[threadIdx.x] = 0.0;
  __syncthreads();
  R acc[4] = {0, 0, 0, 0};  // a thread's few terms: FP32 sums on the mixed path
  const int isp = blockIdx.x * blockDim.x + threadIdx.x;
  int typ = -1;
  if (isp < n) {
    const int4 ai = ainfo[isp];
    const int ityp = ai.x;
    typ = ityp;
    const dbl4 pi = pos[isp];
    if (tc.iee[ityp] != 0) {
      const int nb = nnbb[isp];
      for (int k = 0; k < nb; ++k) {
        int jf = inbb[isp * nbdmax + k];
        int jsp = (jf < 0 ? -jf : jf) - 1;
        if (isp > jsp)
          eterms_pair<R>(isp, jsp, ityp, pi, pos[jsp], coulf, alphad, bx, by, bz, cell, tc,
                         acc, gx, gy, gz, gfix, n, fscalef);
      }
    } else {
      // EE molecule: every intramolecular pair JSM < ISM (forces.f:1585-1594)
      const int f = mol_first[ai.y];
      for (int jsp = f; jsp < isp; ++jsp)
        eterms_pair<R>(isp, jsp, ityp, pi, pos[jsp], coulf, alphad, bx, by, bz, cell, tc,
                       acc, gx, gy, gz, gfix, n, fscalef);
    }
    // SPEE of the atom's type: the thread's own sum (one shared atomic per
    // thread, not per pair)
    if (sizeof(R) == sizeof(double) && acc[0] != R(0)) atomicAdd(&spee_sh[ityp], (double)acc[0]);
  }
  if (sizeof(R) == sizeof(double)) {
    double a[4] = {(double)acc[0], (double)acc[1], (double)acc[2], (double)acc[3]};
    block_add<4>(a, dst);
  } else {
    // warp sums in FP32 (a few terms a lane), then the FP64 block sums; SPEE
    // by warp when the warp's atoms share a type
    const int lane = threadIdx.x & 31;
    const int t0 = __shfl_sync(0xffffffffu, typ, 0);
    const bool uni = __all_sync(0xffffffffu, typ == t0 || typ < 0);
    if (!uni && typ >= 0 && acc[0] != R(0)) atomicAdd(&spee_sh[typ], (double)acc[0]);
    double a[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = (double)warp_sumf((float)acc[k]);
    if (uni && lane == 0 && t0 >= 0 && a[0] != 0.0) atomicAdd(&spee_sh[t0], a[0]);
    block_add_core<4, true>(a, dst.p, dst.part, dst.ctr);
  }
  if (threadIdx.x < MDX_NT && spee_sh[threadIdx.x] != 0.0)
    atomicAdd(&spee[threadIdx.x], spee_sh[threadIdx.x]);
}

struct SelfEnergy {
  double spei, speei[MDX_NT];
};

__global__ void k_eterms_init(mdx_scalars *sc, SelfEnergy se, int ntypes) {
  sc->spe = se.spei;
  for (int t = 0; t < MDX_NT; ++t) sc->spee[t] = t < ntypes ? se.speei[t] : 0.0;
}


}  // namespace

std::mutex g_smem_mu;
cudaError_t raise_smem_limit_fn(const void *kernel, size_t bytes) {
  std::lock_guard<std::mutex> lock(g_smem_mu);
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kernel);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// INIFUR: the reference's k-set (forces.f:1366-1424) regrouped in columns,
// and the self-energy SPEEI/SPEI (forces.f:1426-1447).
int host_inifur(mdx_ctx *ctx) {
  const int icell = ctx->p.icell;
  DevData &d = ctx->dv;
  ctx->drop_graphs();  // k-set buffers are reallocated below
  const double alphad = ctx->p.alphad;
  const double ALP2 = alphad * alphad;
  const double CUTK2 = 4.0 * ALP2 * ctx->p.fexp;
  const double CUTK = std::sqrt(CUTK2);
  const double TWOPI = 2.0 * PI_REF;
  const int KMAX = (int)(CUTK * ctx->boxl / TWOPI + 1);
  const int KMAY = (int)(CUTK * ctx->boyl / TWOPI + 1);
  const int KMAZ = (int)(CUTK * ctx->bozl / TWOPI + 1);
  // the z index of a k-vector: IKZ, or -IKX + IKY + 2 IKZ in the truncated
  // octahedron (forces.f:1392-1406)
  const int MZ = icell == 1 ? KMAX + KMAY + 2 * KMAZ : KMAZ;
  const int NY = 2 * KMAY + 1, NZ = 2 * MZ + 1;
  std::vector<unsigned char> in((size_t)(KMAX + 1) * NY * NZ, 0);
  int nkv = 0;
  for (int IKZ = -KMAZ; IKZ <= KMAZ; ++IKZ)
    for (int IKX = 0; IKX <= KMAX; ++IKX) {
      int KY1 = IKX == 0 ? (IKZ > 0 ? 0 : 1) : -KMAY;
      for (int IKY = KY1; IKY <= KMAY; ++IKY) {
        const int iz = icell == 1 ? -IKX + IKY + 2 * IKZ : IKZ;
        double RXV = TWOPI * IKX, RYV = TWOPI * IKY, RZV = TWOPI * iz;
        if (icell == 2) RYV = TWOPI * IKY + PI_REF * IKX;
        double rx = RXV / ctx->boxl, ry = RYV / ctx->boyl, rz = RZV / ctx->bozl;
        double RK2 = rx * rx + ry * ry + rz * rz;
        if (RK2 <= CUTK2) {
          ++nkv;
          in[((size_t)IKX * NY + (IKY + KMAY)) * NZ + (iz + MZ)] = 1;
        }
      }
    }
  if (nkv > ctx->d.nkv_max) {
    ctx->err = "max number of reciprocal vectors exceeded (NKVM)";
    return MDX_ERR_KVEC;
  }
  std::vector<KCol> cols;
  std::vector<Chunk> chunks;
  int koff = 0, poff = 0, mzmax = 0;
  const int zstep = icell == 1 ? 2 : 1;
  for (int ix = 0; ix <= KMAX; ++ix)
    for (int iy = -KMAY; iy <= KMAY; ++iy) {
      int lo = 1 << 30, hi = -(1 << 30), cnt = 0;
      for (int iz = -MZ; iz <= MZ; ++iz)
        if (in[((size_t)ix * NY + (iy + KMAY)) * NZ + (iz + MZ)]) {
          lo = std::min(lo, iz);
          hi = std::max(hi, iz);
          ++cnt;
        }
      if (!cnt) continue;
      bool steps = cnt == (hi - lo) / zstep + 1 && (hi - lo) % zstep == 0;
      for (int iz = lo; steps && iz <= hi; iz += zstep)
        steps = in[((size_t)ix * NY + (iy + KMAY)) * NZ + (iz + MZ)] != 0;
      if (!steps) {
        ctx->err = "k-set column is not contiguous";
        return MDX_ERR_UNSUPPORTED;
      }
      const int c = (int)cols.size();
      const int zmax = std::max(std::abs(lo), std::abs(hi));
      const int zoff = zmax % zstep;
      const int m = (zmax - zoff) / zstep;
      mzmax = std::max(mzmax, zmax);
      cols.push_back(KCol{ix, iy, lo, hi, koff, 0, m, poff, zoff, zstep});
      for (int p0 = 0; p0 <= m; p0 += CH)
        chunks.push_back(Chunk{c, p0, std::min(CH, m - p0 + 1), 0});
      koff += cnt;
      poff += m + 1;
    }
  // longest chunks first (stable): the lanes of a warp share a length
  std::stable_sort(chunks.begin(), chunks.end(),
                   [](const Chunk &a, const Chunk &b) { return a.len > b.len; });
  // column groups of the mixed passes: columns sorted by m and z offset
  // (then by column index), four at a time, the last group of an (m, zoff)
  // padded; a group's columns share their z records (the octahedron's
  // columns hold the nz of one parity: zoff 0 or 1, zstep 2)
  std::vector<int> order(cols.size());
  for (size_t c = 0; c < cols.size(); ++c) order[c] = (int)c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return cols[a].m != cols[b].m ? cols[a].m < cols[b].m : cols[a].zoff < cols[b].zoff;
  });
  std::vector<KGroup> groups;
  int woff = 0;
  for (size_t p = 0; p < order.size();) {
    const int m = cols[order[p]].m, zo = cols[order[p]].zoff;
    KGroup g{m, m + 1, woff, zo, {-1, -1, -1, -1}};
    for (int s = 0; s < KGRP && p < order.size() && cols[order[p]].m == m &&
                    cols[order[p]].zoff == zo;
         ++s, ++p) {
      g.col[s] = order[p];
      cols[order[p]].wpos = RF_REC * woff + 2 * s;
    }
    woff += g.len;
    groups.push_back(g);
  }
  const size_t nwg = (size_t)RF_REC * std::max(1, woff);
  std::vector<SItem> items;
  for (size_t g = 0; g < groups.size(); ++g)
    for (int t0 = 0; t0 < groups[g].len; t0 += SCH) items.push_back(SItem{(int)g, t0});
  std::stable_sort(items.begin(), items.end(),
                   [](const SItem &a, const SItem &b) { return a.t0 < b.t0; });
  const int kx = KMAX + 1, ky = KMAY + 1, kz = (icell == 1 ? mzmax : KMAZ) + 1;
  d.ldn = ((d.n + 127) / 128) * 128;  // row stride of the FP32 tables
  const bool realloc_tables = kx != d.kx || ky != d.ky || kz != d.kz;
  d.kx = kx;
  d.ky = ky;
  d.kz = kz;
  d.zstep = zstep;
  d.nkv = nkv;
  d.ncol = (int)cols.size();
  ctx->nkv = nkv;
  ctx_free(ctx, d.cols);
  ctx_free(ctx, d.kchunks);
  ctx_free(ctx, d.kgroups);
  ctx_free(ctx, d.sitems);
  d.cols = nullptr;
  d.kchunks = nullptr;
  d.kgroups = nullptr;
  d.sitems = nullptr;
  MDX_CUDA(ctx_alloc(ctx, &d.sitems, sizeof(SItem) * std::max<size_t>(1, items.size())));
  MDX_CUDA(ctx_copy(ctx->stream, d.sitems, items.data(), sizeof(SItem) * items.size(),
                      cudaMemcpyHostToDevice));
  d.nsitem = (int)items.size();
  MDX_CUDA(ctx_alloc(ctx, &d.kgroups, sizeof(KGroup) * std::max<size_t>(1, groups.size())));
  MDX_CUDA(ctx_copy(ctx->stream, d.kgroups, groups.data(), sizeof(KGroup) * groups.size(),
                      cudaMemcpyHostToDevice));
  d.ngroup = (int)groups.size();
  MDX_CUDA(ctx_alloc(ctx, &d.cols, sizeof(KCol) * std::max<size_t>(1, cols.size())));
  MDX_CUDA(ctx_alloc(ctx, &d.kchunks, sizeof(Chunk) * std::max<size_t>(1, chunks.size())));
  MDX_CUDA(ctx_copy(ctx->stream, d.cols, cols.data(), sizeof(KCol) * cols.size(), cudaMemcpyHostToDevice));
  MDX_CUDA(ctx_copy(ctx->stream, d.kchunks, chunks.data(), sizeof(Chunk) * chunks.size(),
                      cudaMemcpyHostToDevice));
  d.nchunk = (int)chunks.size();
  // shared-memory tile of the S(k) kernels: TILE atoms x all table rows
  const size_t sh = ctx->mixed() ? 2 * sizeof(float2) * TILE * (kx + ky + kz + SCH * zstep)
                                 : sizeof(double2) * TILE * (kx + ky + kz);
  if (sh > SFAC_SMEM_MAX) {
    ctx->err = "reciprocal k-set too large for the structure-factor tile";
    return MDX_ERR_UNSUPPORTED;
  }
  // the dynamic shared memory of the mixed force pass plus its static
  // reduction buffer must also fit
  const size_t shr = sizeof(float2) * RF_BATOMS * kz;
  if (ctx->mixed() && shr + sizeof(long long) * 3 * RF_PARTS * RF_BATOMS +
                             sizeof(float4) * RF_PARTS * 2 * RF_WB * RF_REC >
                         SFAC_SMEM_MAX) {
    ctx->err = "reciprocal k-set too large for the force-pass tile";
    return MDX_ERR_UNSUPPORTED;
  }
  // the dynamic shared-memory limit of a kernel is process-wide, shared by
  // every context: only ever raise it
  if (ctx->mixed()) {
    MDX_CUDA(raise_smem_limit(k_rforce32<1>, shr));
    MDX_CUDA(raise_smem_limit(k_rforce32<2>, shr));
    MDX_CUDA(raise_smem_limit(k_sfac32<1>, sh));
    MDX_CUDA(raise_smem_limit(k_sfac32<2>, sh));
  } else {
    MDX_CUDA(raise_smem_limit(k_sfac, sh));
  }
  // mixed force pass: blocks per atom tile (nsplit) so that the grid ends
  // close to a whole number of waves, then contiguous group ranges per warp,
  // balanced by W records (woff is cumulative in group order)
  if (ctx->mixed()) {
    int nsm = 0, dev = 0, per_sm = 0;
    MDX_CUDA(cudaGetDevice(&dev));
    MDX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    MDX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, zstep == 2 ? k_rforce32<2> : k_rforce32<1>, 32 * RF_PARTS, shr));
    const double slots = (double)std::max(1, per_sm) * nsm;
    const double tiles = (double)((d.n + RF_BATOMS - 1) / RF_BATOMS);
    int best = 1;
    double best_eff = 0.0;
    for (int s = 1; s <= 8; ++s) {
      const double w = tiles * s / slots;
      const double eff = w / std::ceil(w);
      if (eff > best_eff + 0.02) {  // a larger split must gain clearly
        best_eff = eff;
        best = s;
      }
    }
    d.rf_nsplit = best;
    const int np = best * RF_PARTS;
    std::vector<int> parts(np + 1);
    int g = 0;
    parts[0] = 0;
    for (int p = 1; p < np; ++p) {
      const long long target = (long long)woff * p / np;
      while (g < (int)groups.size() && groups[g].woff < target) ++g;
      parts[p] = g;
    }
    parts[np] = (int)groups.size();
    ctx_free(ctx, d.rf_part);
    d.rf_part = nullptr;
    MDX_CUDA(ctx_alloc(ctx, &d.rf_part, sizeof(int) * parts.size()));
    MDX_CUDA(ctx_copy(ctx->stream, d.rf_part, parts.data(), sizeof(int) * parts.size(),
                        cudaMemcpyHostToDevice));
  }
  // mixed tensor-core passes (when their shared-memory tiles fit; the
  // CUDA-core passes above stay set up).  MDX_EWALD_TC: 0 = none, 1 (the
  // default) = force pass, 2 = force pass and S(k).  The S(k) GEMM
  // accumulates each 1024-atom partial in the tensor memory's FP32, which
  // biases |S(k)|^2: the reciprocal energy is off by about 3e-5 relative
  // against 1e-8 for the FP32 FMA pass, so it is not the default.
  if (ctx->mixed()) {
    const char *env = std::getenv("MDX_EWALD_TC");
    // the octahedron's stepped z records: the CUDA-core passes only
    const int mode = icell == 1 ? 0 : env && env[0] >= '0' && env[0] <= '2' ? env[0] - '0' : 1;
    d.tc_on = d.tcs_on = false;
    if (mode >= 1 && tc_force_setup(ctx, cols, KMAZ) < 0) return MDX_ERR_CUDA;
    if (mode >= 2 && tc_sfac_setup(ctx, cols) < 0) return MDX_ERR_CUDA;
  }
  // mixed S(k): slices sized so the grid is one wave of resident blocks
  size_t nslice_max = ((size_t)d.n + SLICE - 1) / SLICE;
  if (ctx->mixed()) {
    int nsm = 0, dev = 0, per_sm = 0;
    MDX_CUDA(cudaGetDevice(&dev));
    MDX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    MDX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, zstep == 2 ? k_sfac32<2> : k_sfac32<1>, 128, sh));
    const int nib = std::max(1, ((int)items.size() + 127) / 128);
    int ns = std::max(1, std::max(1, per_sm) * nsm / nib);
    ns = std::min(ns, std::max(1, d.n / 128));  // at least 128 atoms a slice
    d.sfac_slice = (d.n + ns - 1) / ns;
    d.sfac_nslice = (d.n + d.sfac_slice - 1) / d.sfac_slice;
    nslice_max = std::max(nslice_max, (size_t)d.sfac_nslice);
  }
  if (realloc_tables) {
    ctx_free(ctx, d.tabx);
    ctx_free(ctx, d.tabxf);
    d.tabx = d.taby = d.tabz = nullptr;
    d.tabxf = d.tabyf = d.tabzf = nullptr;
    const size_t per = (size_t)kx + ky + kz;
    if (ctx->mixed()) {
      // rows padded to ldn atoms (zero past n): row starts stay 1 KB aligned
      // for the bulk copies of the tensor-core passes
      MDX_CUDA(ctx_alloc(ctx, &d.tabxf, sizeof(float2) * per * d.ldn));
      MDX_CUDA(cudaMemsetAsync(d.tabxf, 0, sizeof(float2) * per * d.ldn, ctx->stream));
      d.tabyf = d.tabxf + (size_t)kx * d.ldn;
      d.tabzf = d.tabyf + (size_t)ky * d.ldn;
    } else {
      MDX_CUDA(ctx_alloc(ctx, &d.tabx, sizeof(double2) * per * d.n));
      d.taby = d.tabx + (size_t)kx * d.n;
      d.tabz = d.taby + (size_t)ky * d.n;
    }
  }
  ctx_free(ctx, d.sk);
  ctx_free(ctx, d.kconst);
  d.kconst = nullptr;
  ctx->kc_box[0] = -1.0;  // per-k constants rebuilt at the next FURIR
  const size_t nk = (size_t)std::max(1, nkv);
  MDX_CUDA(ctx_alloc(ctx, &d.kconst, sizeof(double) * 5 * nk));
  const size_t nkp = (nk + 1) & ~(size_t)1;  // keeps wk 32-byte aligned
  const size_t nc = std::max<size_t>(1, cols.size());
  const size_t np64 = ctx->mixed() ? 0 : 2 * (size_t)poff;  // dbl4 records
  const size_t np32 = ctx->mixed() ? nwg : 0;                // float4 records
  MDX_CUDA(ctx_alloc(ctx, &d.sk,
                     sizeof(double2) * (nkp + 2 * nk + 2 * np64 + np32 + 2 * nc)));
  d.wk = reinterpret_cast<dbl4 *>(d.sk + nkp);
  d.wp64 = d.wk + nk;
  d.wkf = reinterpret_cast<float4 *>(d.wp64 + np64);
  // padding slots of the grouped W stay zero; k_wpairs writes the others
  if (np32) MDX_CUDA(cudaMemsetAsync(d.wkf, 0, sizeof(float4) * np32, ctx->stream));
  d.colrv = reinterpret_cast<double2 *>(d.wkf + np32);
  d.colrvf = reinterpret_cast<float2 *>(d.colrv + nc);
  // per-slice partials of S(k), summed in slice order
  ctx_free(ctx, d.sk_part);
  d.sk_part = nullptr;
  if (ctx_alloc(ctx, &d.sk_part, sizeof(double2) * nslice_max * nk) != cudaSuccess) {
    // the ordered slice sum is what makes S(k) reproducible: no fallback
    d.sk_part = nullptr;
    cudaGetLastError();
    ctx->err = "S(k) slice partials: device allocation failed";
    return MDX_ERR_NOMEM;
  }
  // self-energy (forces.f:1426-1447)
  const double ABC = alphad / std::sqrt(PI_REF);
  ctx->spei = 0.0;
  for (int t = 0; t < ctx->d.ntypes; ++t) {
    double SPET = 0.0;
    const double ESCI = ctx->tc.iee[t] == 0 ? ctx->p.ec_me : 1.0;
    for (int I = 1; I <= ctx->nsits[t]; ++I) {
      const int IS = ctx->isadr[t] + I;
      const double eq = ESCI * ctx->h_charge[IS - 1];
      const double QII = ctx->p.coulf * (eq * eq);
      SPET = SPET - ctx->nspec[t] * ABC * QII;
    }
    ctx->speei[t] = SPET;
    ctx->spei = ctx->spei + SPET;
  }
  return MDX_OK;
}

int sfac_slices(const mdx_ctx *ctx) {
  const DevData &d = ctx->dv;
  return ctx->mixed() ? d.sfac_nslice : (d.n + SLICE - 1) / SLICE;
}

// FURIR's first half (forces.f:1217-1290): the k-set check against the box
// (INIFUR again past the 5 % window), the phase tables and S(k) of the
// current positions and charges into d.sk.  *skip: nothing to do (no Ewald,
// empty k-set or a single molecule).
int furir_sfac(mdx_ctx *ctx, bool *skip) {
  DevData &d = ctx->dv;
  *skip = ctx->p.alphad <= 0.0;
  if (*skip) return MDX_OK;
  const double FKTX = 1.05, FKTS = 0.95;
  int rc;
  if (!ctx->furir_init) {
    ctx->furir_init = true;
    ctx->boxlo = ctx->boxl;
    ctx->boylo = ctx->boyl;
    ctx->bozlo = ctx->bozl;
    if ((rc = host_inifur(ctx))) return rc;
  }
  const double DBX = ctx->boxl / ctx->boxlo, DBY = ctx->boyl / ctx->boylo,
               DBZ = ctx->bozl / ctx->bozlo;
  if (DBX > FKTX || DBX < FKTS || DBY > FKTX || DBY < FKTS || DBZ > FKTX ||
      DBZ < FKTS) {
    ctx->boxlo = ctx->boxl;
    ctx->boylo = ctx->boyl;
    ctx->bozlo = ctx->bozl;
    if ((rc = host_inifur(ctx))) return rc;
  }
  *skip = d.nkv == 0 || (ctx->d.ntypes == 1 && ctx->nspec[0] == 1);
  if (*skip) return MDX_OK;
  const double ibx = 1.0 / ctx->boxl, iby = 1.0 / ctx->boyl, ibz = 1.0 / ctx->bozl;
  const Chunk *chunks = reinterpret_cast<const Chunk *>(d.kchunks);
  const int nchunk = d.nchunk;
  const bool mx = ctx->mixed();
  {
    MDX_TIMER(ctx, MDX_T_EW_TABLES);
    k_tables<<<(3 * d.n + 255) / 256, 256, 0, ctx->stream>>>(
        d.n, d.ldn, d.pos, ibx, iby, ibz, d.kx, d.ky, d.kz, d.tabx, d.taby, d.tabz,
        d.tabxf, d.tabyf, d.tabzf, mx ? d.posi : nullptr,
        ctx->p.icell == 2 ? 0.5 * iby : 0.0);
    MDX_LAUNCHED(ctx);
    if (mx && (rc = tc_zimages_launch(ctx))) return rc;
  }
  MDX_CUDA(cudaMemsetAsync(d.sk, 0, sizeof(double2) * d.nkv, ctx->stream));
  {
    MDX_TIMER(ctx, MDX_T_EW_SFAC);
    const size_t sh = mx ? 2 * sizeof(float2) * TILE * (d.kx + d.ky + d.kz + SCH * d.zstep)
                         : sizeof(double2) * TILE * (d.kx + d.ky + d.kz);
    dim3 grid;
    if (mx && d.tcs_on) {
      if ((rc = tc_sfac_launch(ctx))) return rc;
    } else {
      if (mx) {
        grid = dim3((d.nsitem + 127) / 128, d.sfac_nslice);
        auto kern = d.zstep == 2 ? k_sfac32<2> : k_sfac32<1>;
        kern<<<grid, 128, sh, ctx->stream>>>(
            d.n, d.nsitem, reinterpret_cast<const SItem *>(d.sitems), d.kgroups, d.cols,
            d.tabxf, d.ldn, d.kx, d.ky, d.kz, d.sfac_slice, d.sk, d.sk_part, d.nkv);
      } else {
        grid = dim3((nchunk + 127) / 128, (d.n + SLICE - 1) / SLICE);
        k_sfac<<<grid, 128, sh, ctx->stream>>>(
            d.n, nchunk, chunks, d.cols, d.tabx, d.taby, d.tabz, d.kx, d.ky, d.kz, d.sk,
            d.sk_part, d.nkv);
      }
      MDX_LAUNCHED(ctx);
    }
    if (d.sk_part && !(mx && d.tcs_on)) {
      k_sfac_sum<<<(d.nkv + SUM_K - 1) / SUM_K, SUM_K * SUM_G, 0, ctx->stream>>>(d.nkv, (int)grid.y,
                                                                d.sk_part, d.sk);
      MDX_LAUNCHED(ctx);
    }
  }
  return MDX_OK;
}

// Per-k constants AKC, RXV^2 AKV, RYV^2 AKV, RZV^2 AKV, RZV (forces.f:1296-1305)
// for the current box, rebuilt only when the box or alpha changed.
int ensure_kconst(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  double vol = ctx->boxl * ctx->boyl * ctx->bozl;
  if (ctx->p.icell == 1) vol = 0.5 * vol;  // the octahedron is half its cube (service.f:602)
  const double alp2 = ctx->p.alphad * ctx->p.alphad;
  const double cfur = 4.0 * PI_REF * ctx->p.coulf / vol;
  if (ctx->kc_box[0] != ctx->boxl || ctx->kc_box[1] != ctx->boyl ||
      ctx->kc_box[2] != ctx->bozl || ctx->kc_box[3] != alp2 || ctx->kc_box[4] != cfur) {
    k_kconst<<<std::min(d.ncol, 1024), 64, 0, ctx->stream>>>(
        d.ncol, d.cols, ctx->boxl, ctx->boyl, ctx->bozl, alp2, cfur, d.kconst, d.colrv,
        d.colrvf, ctx->p.icell == 2 ? PI_REF : 0.0);
    MDX_LAUNCHED(ctx);
    ctx->kc_box[0] = ctx->boxl;
    ctx->kc_box[1] = ctx->boyl;
    ctx->kc_box[2] = ctx->bozl;
    ctx->kc_box[3] = alp2;
    ctx->kc_box[4] = cfur;
  }
  return MDX_OK;
}

int launch_furir(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  bool skip = false;
  int rc;
  if ((rc = furir_sfac(ctx, &skip)) || skip) return rc;
  const bool mx = ctx->mixed();
  double *qpe = d.red + 40;
  mdx_scalars *sc = d.sc;
  {
    MDX_TIMER(ctx, MDX_T_EW_KTERMS);
    if ((rc = ensure_kconst(ctx))) return rc;
    const int kb = std::max(1, std::min((d.nkv + 127) / 128, 2 * ctx->nsm));
    Dst6 dst = dst6(ctx, kb, 4, qpe, &sc->virx, &sc->viry, &sc->virz);
    k_kterms<<<kb, 128, 0, ctx->stream>>>(d.nkv, d.sk, d.kconst, d.wk, dst);
    MDX_LAUNCHED(ctx);
    if (!(mx && d.tc_on)) {
      k_wpairs<<<std::min(d.ncol, 1024), 64, 0, ctx->stream>>>(
          d.ncol, d.cols, d.wk, mx ? nullptr : d.wp64, mx ? d.wkf : nullptr);
      MDX_LAUNCHED(ctx);
    }
    k_qpe_fold<<<1, 1, 0, ctx->stream>>>(sc, qpe);
    MDX_LAUNCHED(ctx);
  }
  MDX_TIMER(ctx, MDX_T_EW_FORCE);
  const int rblocks = (d.n + RF_ATOMS - 1) / RF_ATOMS;
  if (mx && d.tc_on) {
    return tc_force_launch(ctx);
  } else if (mx) {
    const size_t shr = sizeof(float2) * RF_BATOMS * d.kz;
    const dim3 grid((d.n + RF_BATOMS - 1) / RF_BATOMS, d.rf_nsplit);
    auto kern = d.zstep == 2 ? k_rforce32<2> : k_rforce32<1>;
    kern<<<grid, 32 * RF_PARTS, shr, ctx->stream>>>(
        d.n, d.rf_part, d.kgroups, d.cols, d.wkf, d.tabxf, d.ldn, d.kx, d.ky, d.kz, d.colrvf,
        ctx->fix, d.gfix);
  } else {
    k_rforce64<<<rblocks, RF_ATOMS * RF_PARTS, 0, ctx->stream>>>(
        d.n, d.ncol, d.cols, d.wp64, d.tabx, d.taby, d.tabz, d.colrv, d.gx, d.gy, d.gz);
  }
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_eterms(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_ETERMS);
  DevData &d = ctx->dv;
  if (ctx->p.lmnbl) return MDX_OK;
  SelfEnergy se;
  se.spei = ctx->spei;
  for (int t = 0; t < MDX_NT; ++t) se.speei[t] = ctx->speei[t];
  k_eterms_init<<<1, 1, 0, ctx->stream>>>(d.sc, se, ctx->d.ntypes);
  MDX_LAUNCHED(ctx);
  mdx_scalars *sc = d.sc;
  Dst6 dst = dst6(ctx, (d.n + 127) / 128, 4, &sc->spe, &sc->virx, &sc->viry, &sc->virz);
  if (ctx->mixed())
    k_eterms<float><<<(d.n + 127) / 128, 128, 0, ctx->stream>>>(
        d.n, d.pos, d.ainfo, d.nnbb, d.inbb, d.nbdmax, d.mol_first, ctx->tc, ctx->p.coulf,
        ctx->p.alphad, ctx->boxl, ctx->boyl, ctx->bozl, cell_pbc(ctx), d.gx, d.gy, d.gz,
        d.gfix, ctx->fix.scalef, dst, sc->spee);
  else
    k_eterms<double><<<(d.n + 127) / 128, 128, 0, ctx->stream>>>(
        d.n, d.pos, d.ainfo, d.nnbb, d.inbb, d.nbdmax, d.mol_first, ctx->tc, ctx->p.coulf,
        ctx->p.alphad, ctx->boxl, ctx->boyl, ctx->bozl, cell_pbc(ctx), d.gx, d.gy, d.gz,
        nullptr, 0.f, dst, sc->spee);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}
