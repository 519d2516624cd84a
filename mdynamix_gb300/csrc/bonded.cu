// bonded.cu -- intramolecular forces into H:
//   GETBND forces.f:113-204  (harmonic / Morse bonds)
//   GETANG forces.f:216-309  (harmonic angle in theta)
//   GETTRS forces.f:323-513  (AMBER, MM3 Tors1, Tors5, improper)
//   STRBND forces.f:530-800  (flexible SPC water, IPOT 1/2)
// One thread per term.  Bond vectors are formed in FP64 with the reference's
// minimum image (vec_r can take them from the fixed-point positions instead;
// launch_bonded leaves that off); the rest of the arithmetic runs in R
// (double on the FP64 path, float on the mixed path, whose forces go to
// 64-bit fixed point with FP32 operations only).
// PINT, VIRB and VIRFX.. are block-reduced in FP64; the per-record averages
// BR/BE, AR/AE, TR/TE are only formed when the caller asks for them.
#include <cmath>

#include <algorithm>

#include "mdx_internal.cuh"

namespace {

struct BondOut {
  double *hx, *hy, *hz;
  unsigned long long *hfix;
  int n;
  double fscale;
  float fscalef;      // the same power of two as FP32
  const int4 *posi;   // mixed: fixed-point positions (bond vectors by integer wrap)
  float sx, sy, sz;   // box / 2^32
  float limx, limy, limz;  // 0.99 x half box: below it no minimum-image shift
  CellPbc cell;            // cell shape (FP64 path: hexagonal / octahedral PBC)
};

// Fixed-point force term: R = float rounds v * 2^k with FP32 operations only
// (the product is exact, so this equals the FP64 rounding of the same value;
// 64-bit conversion instructions issue on the narrow FP64 pipe).
template <typename R>
__device__ __forceinline__ long long fix_term(const BondOut &o, R v) {
  if (sizeof(R) == sizeof(float)) return f2ll_rn((float)v * o.fscalef);
  return __double2ll_rn((double)v * o.fscale);
}

template <typename R>
__device__ __forceinline__ void add_force(const BondOut &o, int i, R fx, R fy, R fz) {
  if (o.hfix) {
    atomicAdd(&o.hfix[i], (unsigned long long)fix_term<R>(o, fx));
    atomicAdd(&o.hfix[o.n + i], (unsigned long long)fix_term<R>(o, fy));
    atomicAdd(&o.hfix[2 * o.n + i], (unsigned long long)fix_term<R>(o, fz));
  } else {
    atomicAdd(&o.hx[i], (double)fx);
    atomicAdd(&o.hy[i], (double)fy);
    atomicAdd(&o.hz[i], (double)fz);
  }
}

__device__ __forceinline__ void vec(const dbl4 *pos, int a, int b, double bx,
                                    double by, double bz, double &x, double &y,
                                    double &z, const CellPbc &c) {
  const dbl4 pa = pos[a], pb = pos[b];
  x = pa.x - pb.x;
  y = pa.y - pb.y;
  z = pa.z - pb.z;
  if (c.icell == 0) pbc_rect(x, y, z, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
  else pbc_cell(x, y, z, c);  // PBC (forces.f:149, 248, 359)
}

// Bond vector a - b in R: FP64 minimum image of the FP64 positions, or on
// the mixed path (float, posi set) the wrapped difference of the 32-bit
// fixed-point positions (exact minimum image by integer wrap-around).
template <typename R>
__device__ __forceinline__ void vec_r(const dbl4 *pos, const BondOut &o, int a, int b, double bx,
                                      double by, double bz, R &x, R &y, R &z) {
  if (sizeof(R) == sizeof(float) && o.posi) {
    const int4 pa = o.posi[a], pb = o.posi[b];
    x = (R)fixdiff(pa.x, pb.x, o.sx);
    y = (R)fixdiff(pa.y, pb.y, o.sy);
    z = (R)fixdiff(pa.z, pb.z, o.sz);
  } else if (sizeof(R) == sizeof(float)) {
    // FP64 difference rounded to FP32; the minimum-image test runs on the
    // FP32 value against 0.99 x half box (bond vectors lie far inside it)
    // and only a vector near or past it takes the FP64 test and shift:
    // the same result as vec()
    const dbl4 pa = pos[a], pb = pos[b];
    double xd = pa.x - pb.x, yd = pa.y - pb.y, zd = pa.z - pb.z;
    x = (R)xd;
    y = (R)yd;
    z = (R)zd;
    if (fabsf((float)x) > o.limx || fabsf((float)y) > o.limy || fabsf((float)z) > o.limz) {
      pbc_rect(xd, yd, zd, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
      x = (R)xd;
      y = (R)yd;
      z = (R)zd;
    }
  } else {
    double xd, yd, zd;
    vec(pos, a, b, bx, by, bz, xd, yd, zd, o.cell);
    x = (R)xd;
    y = (R)yd;
    z = (R)zd;
  }
}

template <typename R>
__device__ __forceinline__ R rsqrt_t(R x);
template <>
__device__ __forceinline__ double rsqrt_t<double>(double x) { return 1.0 / sqrt(x); }
template <>
__device__ __forceinline__ float rsqrt_t<float>(float x) { return 1.0f / sqrtf(x); }

// Per-record average accumulation into shared arrays (only when averaging).
__device__ __forceinline__ void avg_add(double *sh, double *gl, int m, int nrec,
                                        double v) {
  if (m < nrec && nrec <= 256)
    atomicAdd(&sh[m], v);
  else
    atomicAdd(&gl[m], v);
}

// Non-atomic add for a thread that owns every atom it touches (the
// molecule-local kernel); the same per-term rounding as add_force.
template <typename R>
__device__ __forceinline__ void add_force_own(const BondOut &o, int i, R fx, R fy, R fz) {
  if (o.hfix) {
    o.hfix[i] += (unsigned long long)fix_term<R>(o, fx);
    o.hfix[o.n + i] += (unsigned long long)fix_term<R>(o, fy);
    o.hfix[2 * o.n + i] += (unsigned long long)fix_term<R>(o, fz);
  } else {
    o.hx[i] += (double)fx;
    o.hy[i] += (double)fy;
    o.hz[i] += (double)fz;
  }
}

// One bond (GETBND forces.f:140-196): harmonic, or Morse for ID = 1 within
// 2 REQ.  acc: PINT VIRB VIRFX VIRFY VIRFZ; *bd, *eb: length and energy.
template <typename R, bool OWN, typename A = double>
__device__ __forceinline__ void bond_term(const dbl4 *__restrict__ pos, int I, int J, int M,
                                          const int *__restrict__ bid,
                                          const double *__restrict__ rb,
                                          const double *__restrict__ fb,
                                          const double *__restrict__ db,
                                          const double *__restrict__ ro, int lmove,
                                          double bx, double by, double bz,
                                          const BondOut &o, A *acc, R *bd, R *eb) {
  R BX, BY, BZ;
  vec_r<R>(pos, o, J, I, bx, by, bz, BX, BY, BZ);
  const R REQ = (R)rb[M];
  const R BSQ = BX * BX + BY * BY + BZ * BZ;
  const R BD = sqrt(BSQ);
  const R R1I = R(1) / BD;
  const R BBB = BD - REQ;
  R EBDD, FORB;
  if (bid[M] != 1 || BBB > REQ) {
    const R DBND = BBB * (R)fb[M];
    EBDD = DBND * BBB;
    FORB = R(-2) * DBND * R1I;
  } else {
    const R DDIS = (R)db[M], ROH = (R)ro[M];
    const R EXM = exp(-ROH * BBB);
    const R EXMP = R(1) - EXM;
    EBDD = DDIS * (EXMP * EXMP);
    FORB = R(-2) * DDIS * ROH * EXM * EXMP * R1I;
  }
  acc[0] += (A)EBDD;
  *bd = BD;
  *eb = EBDD;
  if (lmove) {
    if (OWN) {
      add_force_own<R>(o, I, -BX * FORB, -BY * FORB, -BZ * FORB);
      add_force_own<R>(o, J, BX * FORB, BY * FORB, BZ * FORB);
    } else {
      add_force<R>(o, I, -BX * FORB, -BY * FORB, -BZ * FORB);
      add_force<R>(o, J, BX * FORB, BY * FORB, BZ * FORB);
    }
    acc[1] += (A)(FORB * BSQ);
    acc[2] += (A)(FORB * (BX * BX));
    acc[3] += (A)(FORB * (BY * BY));
    acc[4] += (A)(FORB * (BZ * BZ));
  }
}

// One angle (GETANG forces.f:230-303), harmonic in theta.
// acc: PINT VIRB(unused) VIRFX VIRFY VIRFZ; *alf, *ea: angle and energy.
template <typename R, bool OWN, typename A = double>
__device__ __forceinline__ void angle_term(const dbl4 *__restrict__ pos, int I, int J, int K,
                                           int M, const double *__restrict__ ra,
                                           const double *__restrict__ fa, int lmove,
                                           double bx, double by, double bz,
                                           const BondOut &o, A *acc, R *alf, R *ea) {
  const R FCN = (R)fa[M], AEQ = (R)ra[M];
  R AX, AY, AZ, BX, BY, BZ;
  vec_r<R>(pos, o, I, J, bx, by, bz, AX, AY, AZ);
  vec_r<R>(pos, o, K, J, bx, by, bz, BX, BY, BZ);
  const R ASQ = AX * AX + AY * AY + AZ * AZ;
  const R ASQI = R(1) / ASQ;
  const R BSQ = BX * BX + BY * BY + BZ * BZ;
  const R BSQI = R(1) / BSQ;
  const R AB = sqrt(ASQ * BSQ);
  const R ABI = R(1) / AB;
  R COSA = AX * BX + AY * BY + AZ * BZ;
  COSA = COSA * ABI;
  COSA = fmin(COSA, R(1));
  COSA = fmax(COSA, R(-1));
  const R ALF = acos(COSA);
  const R SINA = sin(ALF);
  const R SINAI = R(1) / SINA;
  const R DALF = ALF - AEQ;
  const R ABC = DALF * FCN;
  const R EANG = ABC * DALF;
  acc[0] += (A)EANG;
  *alf = ALF;
  *ea = EANG;
  if (lmove) {
    const R SAB = R(-2) * ABC * SINAI;
    const R CAB = SAB * COSA;
    const R FAB = SAB * ABI;
    const R FAA = CAB * ASQI;
    const R FBB = CAB * BSQI;
    const R FAX = FAB * BX - FAA * AX, FAY = FAB * BY - FAA * AY, FAZ = FAB * BZ - FAA * AZ;
    const R FBX = FAB * AX - FBB * BX, FBY = FAB * AY - FBB * BY, FBZ = FAB * AZ - FBB * BZ;
    if (OWN) {
      add_force_own<R>(o, I, -FAX, -FAY, -FAZ);
      add_force_own<R>(o, J, FAX + FBX, FAY + FBY, FAZ + FBZ);
      add_force_own<R>(o, K, -FBX, -FBY, -FBZ);
    } else {
      add_force<R>(o, I, -FAX, -FAY, -FAZ);
      add_force<R>(o, J, FAX + FBX, FAY + FBY, FAZ + FBZ);
      add_force<R>(o, K, -FBX, -FBY, -FBZ);
    }
    acc[2] += (A)(-AX * FAX - BX * FBX);
    acc[3] += (A)(-AY * FAY - BY * FBY);
    acc[4] += (A)(-AZ * FAZ - BZ * FBZ);
  }
}

template <typename R, bool ENER>
__global__ void k_getbnd(int nrbt, const int *__restrict__ ibi,
                         const int *__restrict__ jbj, const int *__restrict__ ibuk,
                         const int *__restrict__ bid, const double *__restrict__ rb,
                         const double *__restrict__ fb, const double *__restrict__ db,
                         const double *__restrict__ ro, const dbl4 *__restrict__ pos,
                         const int4 *__restrict__ ainfo, TypeConst tc,
                         const int *__restrict__ nspec, double bx, double by, double bz,
                         BondOut o, Dst6 dst, int nrbb, int laver,
                         double *br, double *be) {
  __shared__ double sbr[256], sbe[256];
  if (laver) {
    for (int k = threadIdx.x; k < 256; k += blockDim.x) sbr[k] = sbe[k] = 0.0;
    __syncthreads();
  }
  double acc[5] = {0, 0, 0, 0, 0};  // PINT VIRB VIRFX VIRFY VIRFZ
  const int N = blockIdx.x * blockDim.x + threadIdx.x;
  if (N < nrbt) {
    const int I = ibi[N], J = jbj[N], M = ibuk[N];
    const int ityp = ainfo[I].x;
    R BD, EB;
    bond_term<R, false>(pos, I, J, M, bid, rb, fb, db, ro, tc.lmove[ityp], bx, by, bz, o,
                        acc, &BD, &EB);
    if (laver) {
      const double fnspi = 1.0 / (double)nspec[ityp];
      avg_add(sbr, br, M, nrbb, (double)BD * fnspi);
      avg_add(sbe, be, M, nrbb, (double)EB * fnspi);
    }
  }
  if (ENER) block_add<5>(acc, dst);
  if (laver && nrbb <= 256) {
    __syncthreads();
    for (int k = threadIdx.x; k < nrbb; k += blockDim.x) {
      if (sbr[k] != 0.0) atomicAdd(&br[k], sbr[k]);
      if (sbe[k] != 0.0) atomicAdd(&be[k], sbe[k]);
    }
  }
}

template <typename R, bool ENER>
__global__ void k_getang(int nrat, const int *__restrict__ iai,
                         const int *__restrict__ jaj, const int *__restrict__ kak,
                         const int *__restrict__ iauk, const double *__restrict__ ra,
                         const double *__restrict__ fa, const dbl4 *__restrict__ pos,
                         const int4 *__restrict__ ainfo, TypeConst tc,
                         const int *__restrict__ nspec, double bx, double by, double bz,
                         BondOut o, Dst6 dst, int nraa, int laver, double *ar,
                         double *ae) {
  __shared__ double sar[256], sae[256];
  if (laver) {
    for (int k = threadIdx.x; k < 256; k += blockDim.x) sar[k] = sae[k] = 0.0;
    __syncthreads();
  }
  double acc[5] = {0, 0, 0, 0, 0};  // PINT (VIRB) VIRFX VIRFY VIRFZ
  const int N = blockIdx.x * blockDim.x + threadIdx.x;
  if (N < nrat) {
    const int I = iai[N], J = jaj[N], K = kak[N], M = iauk[N];
    const int ityp = ainfo[I].x;
    R ALF, EA;
    angle_term<R, false>(pos, I, J, K, M, ra, fa, tc.lmove[ityp], bx, by, bz, o, acc, &ALF,
                         &EA);
    if (laver) {
      const double fnspi = 1.0 / (double)nspec[ityp];
      avg_add(sar, ar, M, nraa, (double)ALF * fnspi);
      avg_add(sae, ae, M, nraa, (double)EA * fnspi);
    }
  }
  if (ENER) {
    double a4[4] = {acc[0], acc[2], acc[3], acc[4]};
    block_add<4>(a4, dst);
  }
  if (laver && nraa <= 256) {
    __syncthreads();
    for (int k = threadIdx.x; k < nraa; k += blockDim.x) {
      if (sar[k] != 0.0) atomicAdd(&ar[k], sar[k]);
      if (sae[k] != 0.0) atomicAdd(&ae[k], sae[k]);
    }
  }
}

// Bonds and angles of small molecule types, one thread per molecule: every
// atom a thread touches belongs to its molecule, so forces are added
// without atomics (same per-term rounding, so the sums are identical).
template <typename R, bool ENER>
__global__ void __launch_bounds__(128) k_molbonded(
    int ntpl, const MolTpl *__restrict__ tpl, const int *__restrict__ bid,
    const double *__restrict__ rb, const double *__restrict__ fb,
    const double *__restrict__ db, const double *__restrict__ ro,
    const double *__restrict__ ra, const double *__restrict__ fa,
    const dbl4 *__restrict__ pos, TypeConst tc, const int *__restrict__ nspec, double bx,
    double by, double bz, BondOut o, Dst6 dst, int nrbb, int nraa, int laver, double *br,
    double *be, double *ar, double *ae) {
  __shared__ double sav[4][256];  // BR BE AR AE per record (laver)
  if (laver) {
    for (int k = threadIdx.x; k < 4 * 256; k += blockDim.x) sav[k / 256][k % 256] = 0.0;
    __syncthreads();
  }
  R acc[5] = {0, 0, 0, 0, 0};  // PINT VIRB VIRFX VIRFY VIRFZ (a molecule's few terms)
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  int t = 0;
  while (t < ntpl && g >= tpl[t].nmol) {
    g -= tpl[t].nmol;
    ++t;
  }
  // a warp whose molecules all share one template adds to the same records
  // in the same order: its statistics go out as one warp sum per record
  // (shared-memory FP64 atomics from every lane serialise on those records)
  // (every lane takes part in both warp operations: no short-circuit
  // around them)
  const int t0 = __shfl_sync(0xffffffffu, t, 0);
  const bool same_tpl = t < ntpl && t == t0;
  const bool wsum = __all_sync(0xffffffffu, same_tpl) && laver;
  auto add = [&](double *sh, double *gl, int M, int nr, double v) {
    if (wsum) {
      v = warp_sum(v);
      if ((threadIdx.x & 31) == 0) avg_add(sh, gl, M, nr, v);
    } else {
      avg_add(sh, gl, M, nr, v);
    }
  };
  if (t < ntpl) {
    const MolTpl &T = tpl[t];
    const int base = T.first + g * T.nsit;
    const int lmove = tc.lmove[T.type];
    const double fnspi = laver ? 1.0 / (double)nspec[T.type] : 0.0;
    for (int b = 0; b < T.nb; ++b) {
      const int M = T.bm[b];
      R BD, EB;
      bond_term<R, true, R>(pos, base + T.bi[b], base + T.bj[b], M, bid, rb, fb, db, ro, lmove,
                         bx, by, bz, o, acc, &BD, &EB);
      if (laver) {
        add(sav[0], br, M, nrbb, (double)BD * fnspi);
        add(sav[1], be, M, nrbb, (double)EB * fnspi);
      }
    }
    for (int a = 0; a < T.na; ++a) {
      const int M = T.am[a];
      R ALF, EA;
      angle_term<R, true, R>(pos, base + T.ai[a], base + T.aj[a], base + T.ak[a], M, ra, fa,
                          lmove, bx, by, bz, o, acc, &ALF, &EA);
      if (laver) {
        add(sav[2], ar, M, nraa, (double)ALF * fnspi);
        add(sav[3], ae, M, nraa, (double)EA * fnspi);
      }
    }
  }
  if (ENER) {
    double a[5];
    if (sizeof(R) == sizeof(double)) {
#pragma unroll
      for (int k = 0; k < 5; ++k) a[k] = (double)acc[k];
      block_add<5>(a, dst);
    } else {  // warp sums in FP32, then the FP64 block sums
#pragma unroll
      for (int k = 0; k < 5; ++k) a[k] = (double)warp_sumf((float)acc[k]);
      block_add_core<5, true>(a, dst.p, dst.part, dst.ctr);
    }
  }
  if (laver) {
    __syncthreads();
    if (nrbb <= 256)
      for (int k = threadIdx.x; k < nrbb; k += blockDim.x) {
        if (sav[0][k] != 0.0) atomicAdd(&br[k], sav[0][k]);
        if (sav[1][k] != 0.0) atomicAdd(&be[k], sav[1][k]);
      }
    if (nraa <= 256)
      for (int k = threadIdx.x; k < nraa; k += blockDim.x) {
        if (sav[2][k] != 0.0) atomicAdd(&ar[k], sav[2][k]);
        if (sav[3][k] != 0.0) atomicAdd(&ae[k], sav[3][k]);
      }
  }
}

struct TorsTab {
  const int *itors, *nmul;
  const double *ft, *rt, *ft1, *ft2, *ft3, *ft4, *ft5;
};

template <typename R>
__global__ void k_gettrs(int nrrt, const int *__restrict__ iti,
                         const int *__restrict__ jtj, const int *__restrict__ ktk,
                         const int *__restrict__ ltl, const int *__restrict__ ituk,
                         TorsTab tt, const dbl4 *__restrict__ pos,
                         const int4 *__restrict__ ainfo, TypeConst tc,
                         const int *__restrict__ nspec, double bxl, double byl,
                         double bzl, BondOut o, Dst6 dst, int nrtt, int laver,
                         double *trv, double *tev) {
  double acc[4] = {0, 0, 0, 0};  // PINT VIRFX VIRFY VIRFZ
  const int N = blockIdx.x * blockDim.x + threadIdx.x;
  if (N < nrrt) {
    const int I = iti[N], J = jtj[N], K = ktk[N], L = ltl[N], M = ituk[N];
    const int ityp = ainfo[I].x;
    double a0, a1, a2, b0, b1, b2, c0, c1, c2;
    vec(pos, J, I, bxl, byl, bzl, a0, a1, a2, o.cell);
    vec(pos, K, J, bxl, byl, bzl, b0, b1, b2, o.cell);
    vec(pos, L, K, bxl, byl, bzl, c0, c1, c2, o.cell);
    const R ax = (R)a0, ay = (R)a1, az = (R)a2;
    const R bx = (R)b0, by = (R)b1, bz = (R)b2;
    const R cx = (R)c0, cy = (R)c1, cz = (R)c2;
    const R ab = ax * bx + ay * by + az * bz;
    const R bc = bx * cx + by * cy + bz * cz;
    const R ac = ax * cx + ay * cy + az * cz;
    const R at = ax * ax + ay * ay + az * az;
    const R bt = bx * bx + by * by + bz * bz;
    const R ct = cx * cx + cy * cy + cz * cz;
    R axb = (at * bt) - (ab * ab);
    R bxc = (bt * ct) - (bc * bc);
    const R fnum = (ab * bc) - (ac * bt);
    R den = axb * bxc;
    if (den > R(1.0e-10)) {
      den = sqrt(den);
      R co = fnum / den;
      co = fmin(co, R(1));
      co = fmax(co, R(-1));
      const R signum = ax * (by * cz - cy * bz) + ay * (bz * cx - cz * bx) + az * (bx * cy - cx * by);
      const R arg = copysign(acos(co), signum);
      const R SIN1F = sin(arg);
      R si = SIN1F;
      if (fabs(si) < R(1.0e-10)) si = copysign(R(1.0e-10), si);
      R POTT = 0, DERI = 0;
      const int it = tt.itors[M];
      bool ok = true;
      if (it == 0) {
        const R FCN = (R)tt.ft[M], TEQ = (R)tt.rt[M];
        const int MUL = tt.nmul[M];
        const R EARG = MUL * arg - TEQ;
        POTT = FCN * (R(1) + cos(EARG));
        DERI = -FCN * MUL * sin(EARG);
      } else if (it == 1) {
        const R FN1 = (R)tt.ft1[M], FN2 = (R)tt.ft2[M], FN3 = (R)tt.ft3[M];
        const R COS1F = cos(arg);
        const R COS2F = R(2) * (COS1F * COS1F) - R(1);
        const R COS3F = COS1F * (R(2) * COS2F - R(1));
        const R SIN2F = R(2) * SIN1F * COS1F;
        const R SIN3F = SIN1F * COS2F + SIN2F * COS1F;
        POTT = FN1 * (R(1) + COS1F) + FN2 * (R(1) - COS2F) + FN3 * (R(1) + COS3F);
        DERI = -FN1 * SIN1F + R(2) * FN2 * SIN2F - R(3) * FN3 * SIN3F;
      } else if (it == 5) {
        const R FN0 = (R)tt.ft[M], FN1 = (R)tt.ft1[M], FN2 = (R)tt.ft2[M], FN3 = (R)tt.ft3[M],
                FN4 = (R)tt.ft4[M], FN5 = (R)tt.ft5[M], TEQ = (R)tt.rt[M];
        const R EARG = arg - TEQ;
        const R COSI = cos(EARG);
        const R COSI2 = COSI * COSI, COSI3 = COSI * COSI2, COSI4 = COSI * COSI3,
                COSI5 = COSI * COSI4;
        const R SINI = sin(EARG);
        POTT = FN0 + FN1 * COSI + FN2 * COSI2 + FN3 * COSI3 + FN4 * COSI4 + FN5 * COSI5;
        DERI = -SINI * (FN1 + R(2) * FN2 * COSI + R(3) * FN3 * COSI2 + R(4) * FN4 * COSI3 +
                        R(5) * FN5 * COSI4);
      } else if (it == -1) {
        const R FCN = (R)tt.ft[M], TEQ = (R)tt.rt[M];
        const R EARG = arg - TEQ;
        POTT = FCN * (EARG * EARG);
        DERI = R(2) * FCN * EARG;
      } else {
        ok = false;
      }
      if (ok) {
        acc[0] = (double)POTT;
        if (laver) {
          const double fnspi = 1.0 / (double)nspec[ityp];
          atomicAdd(&trv[M], fabs((double)arg * fnspi));
          atomicAdd(&tev[M], (double)POTT * fnspi);
        }
        if (tc.lmove[ityp]) {
          const R de1 = DERI / den / si;
          axb = axb / den * co;
          bxc = bxc / den * co;
          R dnum, dden;
          dnum = cx * bt - bx * bc;
          dden = (ab * bx - ax * bt) * bxc;
          const R FFI1 = (dnum - dden) * de1;
          dnum = ((bx - ax) * bc - ab * cx) + (R(2) * ac * bx - cx * bt);
          dden = axb * (bc * cx - bx * ct) + (ax * bt - at * bx - ab * (bx - ax)) * bxc;
          const R FFJ1 = (dnum - dden) * de1;
          dnum = ab * bx - ax * bt;
          dden = axb * (bt * cx - bc * bx);
          const R FFL1 = (dnum - dden) * de1;
          const R FFK1 = -(FFI1 + FFJ1 + FFL1);
          dnum = cy * bt - by * bc;
          dden = (ab * by - ay * bt) * bxc;
          const R FFI2 = (dnum - dden) * de1;
          dnum = ((by - ay) * bc - ab * cy) + (R(2) * ac * by - cy * bt);
          dden = axb * (bc * cy - by * ct) + (ay * bt - at * by - ab * (by - ay)) * bxc;
          const R FFJ2 = (dnum - dden) * de1;
          dnum = ab * by - ay * bt;
          dden = axb * (bt * cy - bc * by);
          const R FFL2 = (dnum - dden) * de1;
          const R FFK2 = -(FFI2 + FFJ2 + FFL2);
          dnum = cz * bt - bz * bc;
          dden = (ab * bz - az * bt) * bxc;
          const R FFI3 = (dnum - dden) * de1;
          dnum = ((bz - az) * bc - ab * cz) + (R(2) * ac * bz - cz * bt);
          dden = axb * (bc * cz - bz * ct) + (az * bt - at * bz - ab * (bz - az)) * bxc;
          const R FFJ3 = (dnum - dden) * de1;
          dnum = ab * bz - az * bt;
          dden = axb * (bt * cz - bc * bz);
          const R FFL3 = (dnum - dden) * de1;
          const R FFK3 = -(FFI3 + FFJ3 + FFL3);
          add_force<R>(o, I, FFI1, FFI2, FFI3);
          add_force<R>(o, J, FFJ1, FFJ2, FFJ3);
          add_force<R>(o, K, FFK1, FFK2, FFK3);
          add_force<R>(o, L, FFL1, FFL2, FFL3);
          acc[1] = (double)(-(ax + bx) * FFI1 - bx * FFJ1 + cx * FFL1);
          acc[2] = (double)(-(ay + by) * FFI2 - by * FFJ2 + cy * FFL2);
          acc[3] = (double)(-(az + bz) * FFI3 - bz * FFJ3 + cz * FFL3);
        }
      }
    }
  }
  block_add<4>(acc, dst);
}

struct WaterPar {
  int ipt, first, nmol, lmove, i1;
  double roh1, roh2, rh1h2, aaa, bbb, ccc, eee, fff, ggg, ro1, ro2, aadd, bbdd;
};

template <typename R>
__global__ void k_strbnd(WaterPar w, const dbl4 *__restrict__ pos, double bxl,
                         double byl, double bzl, BondOut o, Dst6 dst, int laver,
                         double *br, double *be) {
  const R BBM = (R)(double)1.3f;  // BBMA, a REAL*4 literal (forces.f:566)
  double acc[5] = {0, 0, 0, 0, 0};  // PINT VIRB VIRFX VIRFY VIRFZ
  const int N = blockIdx.x * blockDim.x + threadIdx.x;
  double brs[3] = {0, 0, 0}, bes[3] = {0, 0, 0};
  if (N < w.nmol) {
    const int I = w.first + 3 * N, J = I + 1, K = I + 2;
    const dbl4 pi = pos[I], pj = pos[J], pk = pos[K];
    double a0 = pj.x - pi.x, a1 = pj.y - pi.y, a2 = pj.z - pi.z;
    double b0 = pk.x - pi.x, b1 = pk.y - pi.y, b2 = pk.z - pi.z;
    double c0 = pk.x - pj.x, c1 = pk.y - pj.y, c2 = pk.z - pj.z;
    if (w.ipt == 2) {  // only the Morse variant applies PBC (forces.f:626-640)
      if (o.cell.icell == 0) {
        pbc_rect(a0, a1, a2, bxl, byl, bzl, 0.5 * bxl, 0.5 * byl, 0.5 * bzl);
        pbc_rect(b0, b1, b2, bxl, byl, bzl, 0.5 * bxl, 0.5 * byl, 0.5 * bzl);
        pbc_rect(c0, c1, c2, bxl, byl, bzl, 0.5 * bxl, 0.5 * byl, 0.5 * bzl);
      } else {
        pbc_cell(a0, a1, a2, o.cell);
        pbc_cell(b0, b1, b2, o.cell);
        pbc_cell(c0, c1, c2, o.cell);
      }
    }
    const R AX = (R)a0, AY = (R)a1, AZ = (R)a2, BX = (R)b0, BY = (R)b1, BZ = (R)b2,
            CX = (R)c0, CY = (R)c1, CZ = (R)c2;
    const R ASS = sqrt(AX * AX + AY * AY + AZ * AZ);
    const R BSS = sqrt(BX * BX + BY * BY + BZ * BZ);
    const R CSS = sqrt(CX * CX + CY * CY + CZ * CZ);
    const R SA = ASS - (R)w.roh1, SB = BSS - (R)w.roh2, SH = CSS - (R)w.rh1h2;
    const R AAA = (R)w.aaa, BBB = (R)w.bbb, CCC = (R)w.ccc, EEE = (R)w.eee,
            FFF = (R)w.fff, GGG = (R)w.ggg;
    R WB1, WB2, WB3, FB3A, FB3B, FB3C;
    R EXPA = 0, EXPAM = 0, EXPB = 0, EXPBM = 0;
    if (w.ipt == 2) {
      EXPA = exp(-(R)w.ro1 * SA);
      EXPAM = R(1) - EXPA;
      EXPB = exp(-(R)w.ro2 * SB);
      EXPBM = R(1) - EXPB;
      WB1 = AAA * (EXPAM * EXPAM) + EEE * SA * SH;
      WB2 = BBB * (EXPBM * EXPBM) + FFF * SB * SH;
      WB3 = CCC * SH * SH + GGG * SA * SB;
    } else {
      WB1 = AAA * SA * SA + EEE * SA * SH;
      WB2 = BBB * SB * SB + FFF * SB * SH;
      WB3 = CCC * SH * SH + GGG * SA * SB;
    }
    acc[0] = (double)WB1 + (double)WB2 + (double)WB3;
    if (laver) {
      const double f = 1.0 / (double)w.nmol;
      brs[0] = (double)ASS * f; brs[1] = (double)BSS * f; brs[2] = (double)CSS * f;
      bes[0] = (double)WB1 * f; bes[1] = (double)WB2 * f; bes[2] = (double)WB3 * f;
    }
    if (w.lmove) {
      if (w.ipt == 2) {
        FB3A = ASS > BBM ? R(-2) * SA * (R)w.aadd * (R)w.ro1 : R(-2) * (R)w.aadd * EXPA * EXPAM;
        FB3A = FB3A - EEE * SH - GGG * SB;
        // the reference uses RO(I1) here (forces.f:676)
        FB3B = BSS > BBM ? R(-2) * SB * (R)w.bbdd * (R)w.ro1 : R(-2) * (R)w.bbdd * EXPB * EXPBM;
        FB3B = FB3B - FFF * SH - GGG * SA;
        FB3C = R(-2) * CCC * SH - EEE * SA - FFF * SB;
      } else {
        FB3A = R(-2) * AAA * SA - EEE * SH - GGG * SB;
        FB3B = R(-2) * BBB * SB - FFF * SH - GGG * SA;
        FB3C = R(-2) * CCC * SH - EEE * SA - FFF * SB;
      }
      FB3A = FB3A / ASS;
      FB3B = FB3B / BSS;
      FB3C = FB3C / CSS;
      const R AXX = FB3A * AX, AYY = FB3A * AY, AZZ = FB3A * AZ;
      const R BXX = FB3B * BX, BYY = FB3B * BY, BZZ = FB3B * BZ;
      const R CXX = FB3C * CX, CYY = FB3C * CY, CZZ = FB3C * CZ;
      add_force<R>(o, I, -AXX - BXX, -AYY - BYY, -AZZ - BZZ);
      add_force<R>(o, J, AXX - CXX, AYY - CYY, AZZ - CZZ);
      add_force<R>(o, K, BXX + CXX, BYY + CYY, BZZ + CZZ);
      const R VIX = AX * AXX + BX * BXX + CX * CXX;
      const R VIY = AY * AYY + BY * BYY + CY * CYY;
      const R VIZ = AZ * AZZ + BZ * BZZ + CZ * CZZ;
      acc[1] = (double)VIX + (double)VIY + (double)VIZ;
      acc[2] = (double)VIX;
      acc[3] = (double)VIY;
      acc[4] = (double)VIZ;
    }
  }
  block_add<5>(acc, dst);
  if (laver) {
    // second reduction: its own partials region and counter
    Dst6 d6{{&br[w.i1], &br[w.i1 + 1], &br[w.i1 + 2], &be[w.i1], &be[w.i1 + 1], &be[w.i1 + 2]},
            dst.part ? dst.part + (size_t)gridDim.x * 8 : nullptr, dst.ctr ? dst.ctr + 1 : nullptr};
    double v6[6] = {brs[0], brs[1], brs[2], bes[0], bes[1], bes[2]};
    block_add<6>(v6, d6);
  }
}

}  // namespace

int launch_bonded(mdx_ctx *ctx, int laver, bool ener) {
  MDX_TIMER(ctx, MDX_T_BONDED);
  DevData &d = ctx->dv;
  mdx_scalars *sc = d.sc;
  const bool mx = ctx->mixed();
  // bond vectors stay FP64 differences on both paths: the fixed-point ones
  // cost the mixed path 40 % more force error (stiff bonds turn small
  // length errors into large force errors) for 0.06 ms a long step
  BondOut o{d.hx, d.hy, d.hz, mx ? d.hfix : nullptr, d.n, ctx->fix.scale, ctx->fix.scalef,
            nullptr, (float)(ctx->boxl / 4294967296.0),
            (float)(fix_period_y(ctx) / 4294967296.0), (float)(ctx->bozl / 4294967296.0),
            (float)(0.495 * ctx->boxl), (float)(0.495 * ctx->boyl), (float)(0.495 * ctx->bozl),
            cell_pbc(ctx)};
  const int T = 128;
  const double bx = ctx->boxl, by = ctx->boyl, bz = ctx->bozl;
  const int *nspec = d.nspec_d;
  if (laver) {
    if (d.nrbb) MDX_CUDA(cudaMemsetAsync(d.br, 0, sizeof(double) * 2 * d.nrbb, ctx->stream));
    if (d.nraa) MDX_CUDA(cudaMemsetAsync(d.ar, 0, sizeof(double) * 2 * d.nraa, ctx->stream));
    if (d.nrtt) MDX_CUDA(cudaMemsetAsync(d.tr, 0, sizeof(double) * 2 * d.nrtt, ctx->stream));
  }
  // STRBND first, as GETBND calls it (forces.f:125-127)
  for (int t = 0; t < ctx->d.ntypes; ++t) {
    const int ipt = ctx->tc.ipot[t];
    if (ipt != 1 && ipt != 2) continue;
    const int i1 = ctx->iadb[t] - 1;  // 0-based bond record
    WaterPar w;
    w.ipt = ipt;
    w.first = ctx->isaddr[t];
    w.nmol = ctx->nspec[t];
    w.lmove = ctx->tc.lmove[t];
    w.i1 = i1;
    w.roh1 = ctx->h_rb[i1];
    w.roh2 = ctx->h_rb[i1 + 1];
    w.rh1h2 = ctx->h_rb[i1 + 2];
    w.aaa = ipt == 2 ? ctx->h_db[i1] : ctx->h_fb[i1];
    w.bbb = ipt == 2 ? ctx->h_db[i1 + 1] : ctx->h_fb[i1 + 1];
    w.ccc = ctx->h_fb[i1 + 2];
    w.eee = -884.63 * ctx->p.efact;
    w.fff = -884.63 * ctx->p.efact;
    w.ggg = 467.31 * ctx->p.efact;
    w.ro1 = ctx->h_ro[i1];
    w.ro2 = ctx->h_ro[i1 + 1];
    w.aadd = w.aaa * w.ro1;
    w.bbdd = w.bbb * w.ro2;
    Dst6 dst = dst6(ctx, (w.nmol + T - 1) / T, 14, &sc->pint, &sc->virb, &sc->virfx, &sc->virfy, &sc->virfz);
    if (mx)
      k_strbnd<float><<<(w.nmol + T - 1) / T, T, 0, ctx->stream>>>(w, d.pos, bx, by, bz, o, dst, laver, d.br, d.be);
    else
      k_strbnd<double><<<(w.nmol + T - 1) / T, T, 0, ctx->stream>>>(w, d.pos, bx, by, bz, o, dst, laver, d.br, d.be);
    MDX_LAUNCHED(ctx);
  }
  if (d.ntpl > 0) {
    const int nb = (d.ntpl_mol + T - 1) / T;
    Dst6 dst = dst6(ctx, nb, 5, &sc->pint, &sc->virb, &sc->virfx, &sc->virfy, &sc->virfz);
#define GM(R, E)                                                                       \
  k_molbonded<R, E><<<nb, T, 0, ctx->stream>>>(                                         \
      d.ntpl, d.moltpl, d.bid, d.brb, d.bfb, d.bdb, d.bro, d.ara, d.afa, d.pos, ctx->tc, \
      nspec, bx, by, bz, o, dst, d.nrbb, d.nraa, laver, d.br, d.be, d.ar, d.ae)
    if (mx) {
      if (ener) GM(float, true); else GM(float, false);
    } else {
      if (ener) GM(double, true); else GM(double, false);
    }
#undef GM
    MDX_LAUNCHED(ctx);
  }
  if (d.nrbt > 0) {
    Dst6 dst = dst6(ctx, (d.nrbt + T - 1) / T, 5, &sc->pint, &sc->virb, &sc->virfx, &sc->virfy, &sc->virfz);
#define GB(R, E)                                                                       \
  k_getbnd<R, E><<<(d.nrbt + T - 1) / T, T, 0, ctx->stream>>>(                         \
      d.nrbt, d.ibi, d.jbj, d.ibuk, d.bid, d.brb, d.bfb, d.bdb, d.bro, d.pos, d.ainfo, \
      ctx->tc, nspec, bx, by, bz, o, dst, d.nrbb, laver, d.br, d.be)
    if (mx) {
      if (ener) GB(float, true); else GB(float, false);
    } else {
      if (ener) GB(double, true); else GB(double, false);
    }
#undef GB
    MDX_LAUNCHED(ctx);
  }
  if (d.nrat > 0) {
    Dst6 dst = dst6(ctx, (d.nrat + T - 1) / T, 4, &sc->pint, &sc->virfx, &sc->virfy, &sc->virfz);
#define GA(R, E)                                                                       \
  k_getang<R, E><<<(d.nrat + T - 1) / T, T, 0, ctx->stream>>>(                         \
      d.nrat, d.iai, d.jaj, d.kak, d.iauk, d.ara, d.afa, d.pos, d.ainfo, ctx->tc,      \
      nspec, bx, by, bz, o, dst, d.nraa, laver, d.ar, d.ae)
    if (mx) {
      if (ener) GA(float, true); else GA(float, false);
    } else {
      if (ener) GA(double, true); else GA(double, false);
    }
#undef GA
    MDX_LAUNCHED(ctx);
  }
  if (d.nrrt > 0) {
    Dst6 dst = dst6(ctx, (d.nrrt + T - 1) / T, 4, &sc->pint, &sc->virfx, &sc->virfy, &sc->virfz);
    TorsTab tt{d.titors, d.tnmul, d.tft, d.trt, d.tft1, d.tft2, d.tft3, d.tft4, d.tft5};
#define GT(R)                                                                          \
  k_gettrs<R><<<(d.nrrt + T - 1) / T, T, 0, ctx->stream>>>(                            \
      d.nrrt, d.iti, d.jtj, d.ktk, d.ltl, d.ituk, tt, d.pos, d.ainfo, ctx->tc, nspec,  \
      bx, by, bz, o, dst, d.nrtt, laver, d.tr, d.te)
    if (mx) GT(float); else GT(double);
#undef GT
    MDX_LAUNCHED(ctx);
  }
  return MDX_OK;
}

// GETAVR's per-term statistics (aver.f:45-100) accumulated on the device: the
// per-record averages BR/BE (bonds), AR/AE (angles), TR/TE (torsions) that
// the bonded kernels have just formed under LAVER are added, with their
// squares, to running sums, one sample per long step.  Layout of sums:
// [0] samples; then the values of BR, BE, AR, AE, TR, TE back to back
// (nrbb, nrbb, nraa, nraa, nrtt, nrtt entries: L in all), then their squares.
__global__ void k_acc_bonded(int nrbb, int nraa, int nrtt, const double *__restrict__ br,
                             const double *__restrict__ be, const double *__restrict__ ar,
                             const double *__restrict__ ae, const double *__restrict__ tr,
                             const double *__restrict__ te, double *__restrict__ sums) {
  const int L = 2 * (nrbb + nraa + nrtt);
  if (blockIdx.x == 0 && threadIdx.x == 0) sums[0] += 1.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
    int r = k;
    const double *src;
    if (r < nrbb) src = br;
    else if ((r -= nrbb) < nrbb) src = be;
    else if ((r -= nrbb) < nraa) src = ar;
    else if ((r -= nraa) < nraa) src = ae;
    else if ((r -= nraa) < nrtt) src = tr;
    else { r -= nrtt; src = te; }
    const double v = src[r];
    sums[1 + k] += v;
    sums[1 + L + k] += v * v;
  }
}

int bonded_sums_len(const mdx_ctx *ctx) {
  return 1 + 4 * (ctx->dv.nrbb + ctx->dv.nraa + ctx->dv.nrtt);
}

int launch_acc_bonded(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  if (!d.avsum) return MDX_OK;
  const int L = 2 * (d.nrbb + d.nraa + d.nrtt);
  k_acc_bonded<<<std::max(1, (L + 255) / 256), 256, 0, ctx->stream>>>(
      d.nrbb, d.nraa, d.nrtt, d.br, d.be, d.ar, d.ae, d.tr, d.te, d.avsum);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}
