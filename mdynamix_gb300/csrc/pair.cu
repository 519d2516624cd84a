// pair.cu -- real-space LJ + erfc-Coulomb over the neighbour rows:
//   LOCALF (forces.f:813-998) on the short rows into H,
//   FORCES (forces.f:1014-1202) on the long rows into G.
//
// FP64 path: one warp per owner atom walks its half row (every pair once,
// as in the reference list); the owner's force is reduced in registers and
// the partner's goes out with FP64 atomics.  The arithmetic is the
// reference's, statement by statement.
//
// Mixed path: rows are full (both atoms of a pair hold it), so a warp writes
// only its own atom and there is no scattered atomic at all.  Pair geometry
// comes from 32-bit fixed-point coordinates (x / L * 2^32): the difference of
// two such integers is exact and wraps to the minimum image by itself, and is
// converted to FP32 only as a short vector.  Pair and LJ math is FP32; per
// lane partial forces are rounded to 64-bit fixed point and summed as
// integers, so the result does not depend on the order of the sums.  Energy
// and virial lane partials go the same way into 64-bit integer slots.
#include <algorithm>
#include <cmath>

#include "mdx_internal.cuh"
#include "pair_math.cuh"
#include "tune_table.cuh"

namespace {

// Per-pair parameters (forces.f:838-862 / 1040-1066).
struct PairTables {
  const double *a6lj, *b12lj, *a6lj0, *b12lj0, *a6_14, *b12_14;
  const float *a6f, *b12f, *a60f, *b120f, *a614f, *b1214f;
  const float2 *abf;  // (A6, B12) FP32 pairs: [kind][i*nnbt + j], kind 0 inter, 1 intra, 2 1-4
  int nn;             // nnbt^2
};

// Output slots of one pair sweep.
enum {
  P_EES = 0,   // PELS1/PELS2
  P_ESR,       // PE1/PE2
  P_VIR,       // VIR1/VIR2
  P_VX, P_VY, P_VZ,  // VIRX.. (FORCES) or VIRFX.. (LOCALF)
  P_EE_SAME, P_EE_DIFF, P_ESR_SAME, P_ESR_DIFF,
  P_WIR,       // WIRSS (mixed LOCALF only)
  P_NSLOT
};

__device__ __forceinline__ double ewald_erfc_poly(double ttt, double exp2a) {
  return ((((MDX_A5 * ttt + MDX_A4) * ttt + MDX_A3) * ttt + MDX_A2) * ttt +
          MDX_A1) * ttt * exp2a;
}
__device__ __forceinline__ float ewald_erfc_polyf(float ttt, float exp2a) {
  return (((((float)MDX_A5 * ttt + (float)MDX_A4) * ttt + (float)MDX_A3) * ttt +
           (float)MDX_A2) * ttt + (float)MDX_A1) * ttt * exp2a;
}

// ---------------------------------------------------------------- FP64 ---
template <bool SHORT, bool SPLIT, bool ENER>
__global__ void __launch_bounds__(256) k_pair64(
    int n, const dbl4 *__restrict__ pos, const int4 *__restrict__ ainfo,
    const double *__restrict__ qsite, const int *__restrict__ cnt,
    const int *__restrict__ idx, int cap, PairTables tb, TypeConst tc,
    PairConst pc, double bx, double by, double bz, CellPbc cp, double *__restrict__ fx,
    double *__restrict__ fy, double *__restrict__ fz,
    Dst6 dst, double *__restrict__ split) {
  __shared__ double s_split[2 * MDX_NTPP + 2 * MDX_NT];
  if (SPLIT) {
    for (int k = threadIdx.x; k < 2 * MDX_NTPP + 2 * MDX_NT; k += blockDim.x) s_split[k] = 0.0;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  // ABS(D) > HBOX tests as integer compares of the magnitudes' bit patterns
  // (the same order as the FP64 compare for finite values; no FP64 issue)
  const long long hbxb = __double_as_longlong(0.5 * bx), hbyb = __double_as_longlong(0.5 * by);
  // LOCALF tests DZ against HBOXL (forces.f:871); FORCES against HBOZL
  const long long hbzb = __double_as_longlong(SHORT ? 0.5 * bx : 0.5 * bz);
  const long long rc2b = __double_as_longlong(pc.rc2);
  const bool rae_on = pc.lmdee && pc.raex != 0.0;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  if (i < n) {
    const dbl4 pi = pos[i];
    const int4 ai = ainfo[i];
    const int ti = ai.x, mi = ai.y, ni = ai.z;
    const double qsi = qsite[i];
    const int c = cnt[i];
    double fix = 0.0, fiy = 0.0, fiz = 0.0;
    const int *row = idx + (size_t)i * cap;
    for (int k = lane; k < c; k += 32) {
      const int v = row[k];
      const bool is14 = SHORT && v < 0;
      const int j = v & 0x7fffffff;
      const dbl4 pj = pos[j];
      const int4 aj = ainfo[j];
      const int tj = aj.x, nj = aj.z;
      const bool same = aj.y == mi;
      const int mtr = tc.mdx[ti][tj];
      double QIJ, A6, B12;
      bool rae = false;  // RAEX shifts this pair's distance (MDEE)
      const int tix = ni * pc.nnbt + nj;
      if (same) {
        if (is14) {
          QIJ = qsi * qsite[j] * pc.coulf * tc.c14el[ti];
          A6 = __ldg(&tb.a6_14[tix]) * tc.c14lj[ti];
          B12 = __ldg(&tb.b12_14[tix]) * tc.c14lj[ti];
        } else {
          QIJ = qsi * qsite[j] * pc.coulf;
          A6 = __ldg(&tb.a6lj0[tix]);
          B12 = __ldg(&tb.b12lj0[tix]);
        }
      } else {
        QIJ = pi.w * pj.w * pc.coulf;
        A6 = __ldg(&tb.a6lj[tix]);
        B12 = __ldg(&tb.b12lj[tix]);
        rae = rae_on && tc.iee[ti] * tc.iee[tj] == 0;
      }
      double DX = pi.x - pj.x, DY = pi.y - pj.y, DZ = pi.z - pj.z;
      constexpr long long MAG = 0x7fffffffffffffffLL;
      if (cp.icell == 0) {
        if ((__double_as_longlong(DX) & MAG) > hbxb) DX = DX - fsign(bx, DX);
        if ((__double_as_longlong(DZ) & MAG) > hbzb) DZ = DZ - fsign(bz, DZ);
        if ((__double_as_longlong(DY) & MAG) > hbyb) DY = DY - fsign(by, DY);
      } else {  // hexagonal / truncated octahedron (forces.f:872-906, 1077-1111)
        pbc_cell(DX, DY, DZ, cp, SHORT ? cp.hbx : cp.hbz);
      }
      const double RR = DX * DX + DY * DY + DZ * DZ;
      if (!SHORT && __double_as_longlong(RR) > rc2b) continue;  // skin mode: listed beyond RCUT
      // one reciprocal square root instead of a square root and a division
      // (within an ulp of DSQRT and 1/R1)
      const double R1I = rsqrt(RR);
      const double R1 = RR * R1I;
      double R1E = R1, R1EI = R1I;
      if (rae) {
        R1E = R1 + pc.raex;
        R1EI = 1. / R1E;
      }
      double EE1, EES, FORCE;
      if (is14 || (same && tc.iee[ti] == 0)) {
        if (SHORT) {
          EE1 = QIJ * R1I;
          FORCE = tc.lmove[ti] ? EE1 * (R1I * R1I) : 0.0;
        } else {
          EE1 = QIJ / R1;
          FORCE = tc.lmove[ti] ? EE1 / (R1 * R1) : 0.0;
        }
        EES = EE1;
      } else if (pc.lmnbl) {
        EE1 = QIJ * (1.0 / R1E - 0.5 * pc.rff2 * (R1E * R1E) + pc.rff);
        EES = EE1;
        if (SHORT) {
          FORCE = QIJ * (1. / (R1E * R1E * R1E) + pc.rff2);
          if (ENER) acc[P_VIR] += QIJ * (1.5 * pc.rff2 / (R1E * R1E) - pc.rff);
        } else {
          FORCE = QIJ * (1.0 / ((R1E * R1E) * R1) + pc.rff2);
          if (ENER) acc[P_VIR] += QIJ * (1.5 * pc.rff2 * RR - pc.rff);
        }
      } else {
        const double ALPHAR = pc.alphad * R1;
        const double TTT = rcp_nr(1.0 + MDX_B1 * ALPHAR);
        const double EXP2A = exp_neg(ALPHAR * ALPHAR);
        const double ERFCT = ewald_erfc_poly(TTT, EXP2A);
        EE1 = QIJ * R1EI;
        EES = EE1 * ERFCT;
        FORCE = EE1 * (MDX_TOTPI * pc.alphad * EXP2A + ERFCT * R1EI) * R1I;
      }
      if (SPLIT) {
        if (same) atomicAdd(&s_split[2 * MDX_NTPP + ti], EE1);
        else atomicAdd(&s_split[mtr], EE1);
      }
      if (ENER) acc[P_EES] += EES;
      if ((__double_as_longlong(B12) << 1) != 0) {  // B12 != 0
        const double R2I = R1EI * R1EI;
        const double R6I = R2I * R2I * R2I;
        double ESR = (A6 + B12 * R6I) * R6I;
        const double FSR = (6.0 * A6 + 12.0 * B12 * R6I) * R6I * R1EI;
        FORCE = FORCE + FSR * R1I;
        if (same) {
          if (SHORT) {
            if (tc.lmove[ti]) {
              if (SPLIT) atomicAdd(&s_split[2 * MDX_NTPP + MDX_NT + ti], ESR);
              if (ENER) acc[P_VIR] += FSR * R1;
            } else {
              ESR = 0.0;
              FORCE = 0.0;
            }
          } else {
            if (ENER && tc.lmove[ti]) acc[P_VIR] += FSR * R1;
            if (SPLIT) atomicAdd(&s_split[2 * MDX_NTPP + MDX_NT + ti], ESR);
          }
        } else {
          if (SPLIT) atomicAdd(&s_split[MDX_NTPP + mtr], ESR);
          if (ENER) acc[P_VIR] += FSR * R1;
        }
        if (ENER) acc[P_ESR] += ESR;
      }
      const double gxv = FORCE * DX, gyv = FORCE * DY, gzv = FORCE * DZ;
      if (SHORT || !same || tc.lmove[ti]) {  // FORCE DX^2 as (FORCE DX) DX
        if (ENER) acc[3] += gxv * DX;
        if (ENER) acc[4] += gyv * DY;
        if (ENER) acc[5] += gzv * DZ;
      }
      fix += gxv;
      fiy += gyv;
      fiz += gzv;
      atomicAdd(&fx[j], -gxv);
      atomicAdd(&fy[j], -gyv);
      atomicAdd(&fz[j], -gzv);
    }
    fix = warp_sum(fix);
    fiy = warp_sum(fiy);
    fiz = warp_sum(fiz);
    if (lane == 0 && c > 0) {
      atomicAdd(&fx[i], fix);
      atomicAdd(&fy[i], fiy);
      atomicAdd(&fz[i], fiz);
    }
  }
  if (ENER) block_add<6>(acc, dst);
  if (SPLIT) {
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * MDX_NTPP + 2 * MDX_NT; k += blockDim.x)
      if (s_split[k] != 0.0) atomicAdd(&split[k], s_split[k]);
  }
}

// WIRSS / WIRS: -sum F . (S - COM(molecule)) (forces.f:991-995,
// scalar.f:77-82), FP64 path.
__global__ void k_wir(int n, const dbl4 *__restrict__ pos,
                      const int4 *__restrict__ ainfo, const double *__restrict__ X,
                      const double *__restrict__ Y, const double *__restrict__ Z,
                      const double *__restrict__ fx, const double *__restrict__ fy,
                      const double *__restrict__ fz, Dst6 dst) {
  double w[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const dbl4 p = pos[i];
    const int m = ainfo[i].y;
    w[0] = w[0] - fx[i] * (p.x - X[m]) - fy[i] * (p.y - Y[m]) - fz[i] * (p.z - Z[m]);
  }
  block_add<1>(w, dst);
}

// WIRSS on the mixed path: the short-row sweep has just stored the pair
// forces as fixed point; the bonded terms have not been added yet.
__global__ void k_wir_fix(int n, const dbl4 *__restrict__ pos,
                          const int4 *__restrict__ ainfo, const double *__restrict__ X,
                          const double *__restrict__ Y, const double *__restrict__ Z,
                          const unsigned long long *__restrict__ f, double inv,
                          Dst6 dst) {
  double w[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const dbl4 p = pos[i];
    const int m = ainfo[i].y;
    const double fx = (double)(long long)f[i] * inv;
    const double fy = (double)(long long)f[n + i] * inv;
    const double fz = (double)(long long)f[2 * n + i] * inv;
    w[0] = w[0] - fx * (p.x - X[m]) - fy * (p.y - Y[m]) - fz * (p.z - Z[m]);
  }
  block_add<1>(w, dst);
}

// ---------------------------------------------------------------- mixed ---
constexpr int PAIR32_BLOCKS = 6;  // resident blocks per SM the register cap aims at
// Resident blocks per SM of the paired sweeps: 4 (64 registers), and 6 (40
// registers, a few spilled) for the forces-only short sweep of the
// intermediate short steps, which waits on its loads and gains more from
// resident warps than it loses to the spills (0.289 against 0.310 ms per long
// step at 98,304 atoms).
constexpr int PAIR32X2_BLOCKS = 4;
constexpr int PAIR32X2_BLOCKS_SHORT = 6;

__device__ __forceinline__ float idiff(int a, int b, float s) { return fixdiff(a, b, s); }

// Register cap for occupancy: the sweeps wait on gathered neighbour records,
// and more resident warps hide more of that (6 blocks of 256: 40 registers;
// measured 12 % faster than the uncapped 44-64 registers).
template <bool SHORT, bool SPLIT, bool ENER, int TPO>
__global__ void __launch_bounds__(256, PAIR32_BLOCKS) k_pair32(
    int n, const int4 *__restrict__ posi, const int4 *__restrict__ posn,
    const float4 *__restrict__ stab,
    const int *__restrict__ cnt, const int *__restrict__ idx, int cap,
    PairTables tb, TypeConst tc, PairConst pc, float sx, float sy, float sz,
    FixScale fsc, unsigned long long *__restrict__ ffix,
    const double *__restrict__ X, const double *__restrict__ Y,
    const double *__restrict__ Z, double escale,
    unsigned long long *__restrict__ slots, double *__restrict__ split,
    const int *__restrict__ owner_of, CellF cf) {
  __shared__ double s_split[2 * MDX_NTPP + 2 * MDX_NT];
  if (SPLIT) {
    for (int k = threadIdx.x; k < 2 * MDX_NTPP + 2 * MDX_NT; k += blockDim.x) s_split[k] = 0.0;
    __syncthreads();
  }
  // TPO adjacent lanes per owner atom stride its row: short rows (about 50
  // entries, tiled: list_slot puts entry k of 32 atoms in one 128-byte line)
  // take a few lanes, long rows (several hundred entries) up to a warp.  The
  // split is a tuning choice (tune_table.cuh); the forces' integer sums do
  // not depend on it, the FP32 lane partials before them do.
  // owner_of (long rows, stored whole per atom): owners are taken in the
  // cell order of the last build (slot -> atom), so that the owners of a
  // block are neighbours in space and share their neighbours' records in
  // L1; null (short rows, tiled by 32 atoms): atom order.
  const int lane = threadIdx.x & 31;
  const int sl = (blockIdx.x * blockDim.x + threadIdx.x) / TPO;
  const int i = owner_of && sl < n ? owner_of[sl] : sl;
  const int k0 = lane % TPO, kstep = TPO;
  long long tot[P_NSLOT];
#pragma unroll
  for (int k = 0; k < P_NSLOT; ++k) tot[k] = 0;
  float a[P_NSLOT];
#pragma unroll
  for (int k = 0; k < P_NSLOT; ++k) a[k] = 0.f;
  long long qx = 0, qy = 0, qz = 0;
  if (i < n) {
    // one 16-byte record per atom: fixed-point x, y, z and (molecule, site);
    // charges and types come from the per-site table (L1-resident)
    constexpr unsigned SITE_MASK = (1u << MDX_SITE_BITS) - 1u;
    const int4 pi = owner_of ? posn[sl] : posi[i];
    const float4 sti = __ldg(&stab[(unsigned)pi.w & SITE_MASK]);
    const unsigned mi = (unsigned)pi.w >> MDX_SITE_BITS;
    const int ti = __float_as_int(sti.w), ni = __float_as_int(sti.z);
    const float qi = sti.x;
    const float qsi = sti.y;
    const float coulf = (float)pc.coulf, alphad = (float)pc.alphad;
    const float raex = (float)pc.raex;
    // per-owner constants of the type tables, hoisted out of the row
    const int eei = tc.iee[ti], lmovei = tc.lmove[ti];
    const float c14e = tc.c14elf[ti], c14l = tc.c14ljf[ti];
    const float qsc = qsi * coulf, qic = qi * coulf;
    const float2 *abrow = tb.abf + ni * pc.nnbt;
    const int c = cnt[i];
    float fxa = 0.f, fya = 0.f, fza = 0.f;
    const int *row = idx + list_slot(i, 0, cap, SHORT);
    const int rs = SHORT ? 32 : 1;  // stride of consecutive entries
    // the next entry's index and record are loaded while this one computes
    // entries are cell-order slots of posn (the neighbours' records in the
    // order of the cell grid: neighbours of one owner lie in a few runs)
    int v = k0 < c ? row[(size_t)k0 * rs] : 0;
    int4 pj = posn[v & 0x7fffffff];
    for (int k = k0; k < c; k += kstep) {
      int vn = 0;
      int4 pjn = pj;
      if (k + kstep < c) {
        vn = row[(size_t)(k + kstep) * rs];
        pjn = posn[vn & 0x7fffffff];
      }
      const bool is14 = SHORT && v < 0;
      const float4 stj = __ldg(&stab[(unsigned)pj.w & SITE_MASK]);
      const int tj = __float_as_int(stj.w), nj = __float_as_int(stj.z);
      const bool same = ((unsigned)pj.w >> MDX_SITE_BITS) == mi;
      // one (A6, B12) load: inter-molecular, intra-molecular or 1-4 table
      const int kind = same ? (is14 ? 2 : 1) : 0;
      const float2 ab = __ldg(&abrow[kind * tb.nn + nj]);
      float QIJ, A6, B12, RAE = 0.f;
      if (same) {
        QIJ = is14 ? qsc * stj.y * c14e : qsc * stj.y;
        A6 = is14 ? ab.x * c14l : ab.x;
        B12 = is14 ? ab.y * c14l : ab.y;
      } else {
        QIJ = qic * stj.x;
        A6 = ab.x;
        B12 = ab.y;
        if (pc.lmdee) RAE = (eei * tc.iee[tj] == 0) ? raex : 0.f;
      }
      float DX = idiff(pi.x, pj.x, sx);
      float DY = idiff(pi.y, pj.y, sy);
      float DZ = idiff(pi.z, pj.z, sz);
      if (cf.kind) pbc_cellf(DX, DY, DZ, cf);
      const float RR = DX * DX + DY * DY + DZ * DZ;
      if (SHORT || RR <= pc.rc2f) {  // skin mode: long-row pairs beyond RCUT skipped
        const float R1I = rsqrtf(RR);
        const float R1 = RR * R1I;
        const float R1EI = RAE == 0.f ? R1I : __fdividef(1.f, R1 + RAE);
        const float R1E = R1 + RAE;
        float EE1, EES, FORCE;
        if (is14 || (same && eei == 0)) {
          EE1 = QIJ * R1I;
          FORCE = lmovei ? EE1 * (R1I * R1I) : 0.f;
          EES = EE1;
        } else if (pc.lmnbl) {
          const float rff = (float)pc.rff, rff2 = (float)pc.rff2;
          EE1 = QIJ * (1.f / R1E - 0.5f * rff2 * (R1E * R1E) + rff);
          EES = EE1;
          if (SHORT) {
            FORCE = QIJ * (R1EI * R1EI * R1EI + rff2);
            if (ENER) a[P_VIR] += QIJ * (1.5f * rff2 * R1EI * R1EI - rff);
          } else {
            FORCE = QIJ * (R1EI * R1EI * R1I + rff2);
            if (ENER) a[P_VIR] += QIJ * (1.5f * rff2 * RR - rff);
          }
        } else {
          const float ALPHAR = alphad * R1;
          const float TTT = __fdividef(1.f, 1.f + (float)MDX_B1 * ALPHAR);
          const float EXP2A = __expf(-(ALPHAR * ALPHAR));
          const float ERFCT = ewald_erfc_polyf(TTT, EXP2A);
          EE1 = QIJ * R1EI;
          EES = EE1 * ERFCT;
          FORCE = EE1 * ((float)MDX_TOTPI * alphad * EXP2A + ERFCT * R1EI) * R1I;
        }
        if (SPLIT) {
          const int mtr = tc.mdx[ti][tj];
          if (same) atomicAdd(&s_split[2 * MDX_NTPP + ti], (double)EE1);
          else atomicAdd(&s_split[mtr], (double)EE1);
        }
        if (ENER) {
          if (same) a[P_EE_SAME] += EE1;
          else a[P_EE_DIFF] += EE1;
        }
        if (ENER) a[P_EES] += EES;
        if (B12 != 0.f) {
          const float R2I = R1EI * R1EI;
          const float R6I = R2I * R2I * R2I;
          float ESR = (A6 + B12 * R6I) * R6I;
          const float FSR = (6.f * A6 + 12.f * B12 * R6I) * R6I * R1EI;
          FORCE = FORCE + FSR * R1I;
          bool count_esr_split = true;
          if (same) {
            if (SHORT) {
              if (lmovei) {
                if (ENER) a[P_VIR] += FSR * R1;
              } else {
                ESR = 0.f;
                FORCE = 0.f;
                count_esr_split = false;
              }
            } else {
              if (ENER && lmovei) a[P_VIR] += FSR * R1;
            }
            if (count_esr_split) {
              if (ENER) a[P_ESR_SAME] += ESR;
              if (SPLIT) atomicAdd(&s_split[2 * MDX_NTPP + MDX_NT + ti], (double)ESR);
            }
          } else {
            if (ENER) a[P_ESR_DIFF] += ESR;
            if (SPLIT) atomicAdd(&s_split[MDX_NTPP + tc.mdx[ti][tj]], (double)ESR);
            if (ENER) a[P_VIR] += FSR * R1;
          }
          if (ENER) a[P_ESR] += ESR;
        }
        if (SHORT || !same || lmovei) {
          if (ENER) a[P_VX] += FORCE * (DX * DX);
          if (ENER) a[P_VY] += FORCE * (DY * DY);
          if (ENER) a[P_VZ] += FORCE * (DZ * DZ);
        }
        fxa += FORCE * DX;
        fya += FORCE * DY;
        fza += FORCE * DZ;
      }
      v = vn;
      pj = pjn;
    }
    // forces: lane partials -> fixed point (-> integer warp sum) -> one store
    // (no 64-bit conversion instruction: those issue on the FP64 pipe)
    qx = f2ll_rn(fxa * fsc.scalef);
    qy = f2ll_rn(fya * fsc.scalef);
    qz = f2ll_rn(fza * fsc.scalef);
  }
  // the owner's lanes are adjacent; every lane of the warp takes part
#pragma unroll
  for (int o = 1; o < TPO; o <<= 1) {
    qx += __shfl_xor_sync(0xffffffffu, qx, o);
    qy += __shfl_xor_sync(0xffffffffu, qy, o);
    qz += __shfl_xor_sync(0xffffffffu, qz, o);
  }
  if (i < n && lane % TPO == 0) {
    ffix[i] = (unsigned long long)qx;
    ffix[n + i] = (unsigned long long)qy;
    ffix[2 * n + i] = (unsigned long long)qz;
  }
  if (ENER) {
#pragma unroll
    for (int k = 0; k < P_WIR; ++k) {
      float t = warp_sumf(a[k]);
      if (lane == 0) tot[k] = f2ll_rn(t * fsc.escalef);
    }
  }
  if (!ENER) return;  // forces only: no energy or virial slots
  // block sum of the integer slots, one atomic per slot per block
  __shared__ long long sh[8][P_NSLOT];
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < P_NSLOT; ++k) sh[wid][k] = tot[k];
  }
  __syncthreads();
  if (threadIdx.x < P_NSLOT) {
    long long s = 0;
    for (int w = 0; w < nw; ++w) s += sh[w][threadIdx.x];
    if (s != 0) atomicAdd(&slots[threadIdx.x], (unsigned long long)s);
  }
  if (SPLIT) {
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * MDX_NTPP + 2 * MDX_NT; k += blockDim.x)
      if (s_split[k] != 0.0) atomicAdd(&split[k], 0.5 * s_split[k]);
  }
}

// ------------------------------------------------------- mixed, paired ---
// The common case of the mixed sweeps (Ewald, no energy split by type pair,
// no MDEE shift): each lane evaluates two row entries per iteration with the
// paired FP32 instructions of this GPU (__ffma2_rn / __fmul2_rn /
// __fadd2_rn: two FP32 operations per issued instruction).  The sweeps are
// issue-bound, and pairing halves their FP32 instructions.  Entries of the
// owner's own molecule (intramolecular non-bonded and 1-4 pairs; water has
// none) are evaluated one at a time by pair_same.

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 splat(float a) { return make_float2(a, a); }

// Per-thread asynchronous copies into shared memory (the thread reads back
// only its own slots, so no barrier is involved).
__device__ __forceinline__ void cpa4(int *smem, const int *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpa16(int4 *smem, const int4 *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Sums of one lane: element .x and .y of each are independent partials.
struct Acc2 {
  float2 fx, fy, fz;              // force on the owner
  float2 ees, ee, esr, vir;       // PELS, unscreened Coulomb, PE, VIR (all pairs)
  float2 vx, vy, vz;              // diagonal virial
  float ee_same, esr_same;        // the owner's own molecule's share of ee, esr
};

// One entry of the owner's own molecule (forces.f:868-998 / 1071-1198 with
// SAME set): scaled 1-4 or plain Coulomb for an ion-free site (IEE = 0), the
// Ewald real-space term otherwise; LJ only where B12 is nonzero.
template <bool SHORT, bool ENER>
__device__ __forceinline__ void pair_same(float DX, float DY, float DZ, bool is14, float QIJ,
                                          float A6, float B12, int eei, int lmovei,
                                          float alphad, float rc2f, Acc2 &s) {
  const float RR = DX * DX + DY * DY + DZ * DZ;
  if (!(SHORT || RR <= rc2f)) return;
  const float R1I = rsqrtf(RR);
  const float R1 = RR * R1I;
  float EE1, EES, FORCE;
  if (is14 || eei == 0) {
    EE1 = QIJ * R1I;
    FORCE = lmovei ? EE1 * (R1I * R1I) : 0.f;
    EES = EE1;
  } else {
    const float ALPHAR = alphad * R1;
    const float TTT = __fdividef(1.f, 1.f + (float)MDX_B1 * ALPHAR);
    const float EXP2A = __expf(-(ALPHAR * ALPHAR));
    const float ERFCT = ewald_erfc_polyf(TTT, EXP2A);
    EE1 = QIJ * R1I;
    EES = EE1 * ERFCT;
    FORCE = EE1 * ((float)MDX_TOTPI * alphad * EXP2A + ERFCT * R1I) * R1I;
  }
  if (ENER) {
    s.ee.x += EE1;
    s.ee_same += EE1;
    s.ees.x += EES;
  }
  if (B12 != 0.f) {
    const float R2I = R1I * R1I;
    const float R6I = R2I * R2I * R2I;
    float ESR = (A6 + B12 * R6I) * R6I;
    const float FSR = (6.f * A6 + 12.f * B12 * R6I) * R6I * R1I;
    FORCE = FORCE + FSR * R1I;
    if (SHORT && !lmovei) {
      ESR = 0.f;
      FORCE = 0.f;
    }
    if (ENER) {
      if (lmovei) s.vir.x += FSR * R1;
      s.esr.x += ESR;
      s.esr_same += ESR;
    }
  }
  if (ENER && (SHORT || lmovei)) {
    s.vx.x += FORCE * (DX * DX);
    s.vy.x += FORCE * (DY * DY);
    s.vz.x += FORCE * (DZ * DZ);
  }
  s.fx.x += FORCE * DX;
  s.fy.x += FORCE * DY;
  s.fz.x += FORCE * DZ;
}

// Block sum of a sweep's integer energy/virial slots: warp sums of the lane
// partials, fixed point, one atomic per slot per block.
__device__ __forceinline__ void slots_out(const float (&a)[P_NSLOT], float escalef,
                                          unsigned long long *__restrict__ slots) {
  const int lane = threadIdx.x & 31;
  long long tot[P_WIR];
#pragma unroll
  for (int k = 0; k < P_WIR; ++k) {
    const float t = warp_sumf(a[k]);
    tot[k] = lane == 0 ? f2ll_rn(t * escalef) : 0;
  }
  __shared__ long long sh[8][P_WIR];
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < P_WIR; ++k) sh[wid][k] = tot[k];
  }
  __syncthreads();
  if (threadIdx.x < P_WIR) {
    long long s = 0;
    for (int w = 0; w < nw; ++w) s += sh[w][threadIdx.x];
    if (s != 0) atomicAdd(&slots[threadIdx.x], (unsigned long long)s);
  }
}

template <bool SHORT, bool ENER, int TPO, bool CELL>
__global__ void __launch_bounds__(256, (SHORT && !ENER) ? PAIR32X2_BLOCKS_SHORT : PAIR32X2_BLOCKS)
k_pair32x2(
    int n, const int4 *__restrict__ posi, const int4 *__restrict__ posn,
    const float4 *__restrict__ stab, const int *__restrict__ cnt, const int *__restrict__ idx,
    int cap, PairTables tb, TypeConst tc, PairConst pc, float sx, float sy, float sz,
    FixScale fsc, unsigned long long *__restrict__ ffix,
    unsigned long long *__restrict__ slots, const int *__restrict__ owner_of, CellF cf) {
  // TPO adjacent lanes per owner atom; lane k0 of an owner takes entries
  // k0 + 2 TPO m and k0 + TPO + 2 TPO m as one pair.  Owner order as in
  // k_pair32.
  const int lane = threadIdx.x & 31;
  const int sl = (blockIdx.x * blockDim.x + threadIdx.x) / TPO;
  const int i = owner_of && sl < n ? owner_of[sl] : sl;
  const int k0 = lane % TPO;
  Acc2 s;
  s.fx = s.fy = s.fz = splat(0.f);
  s.ees = s.ee = s.esr = s.vir = splat(0.f);
  s.vx = s.vy = s.vz = splat(0.f);
  s.ee_same = s.esr_same = 0.f;
  long long qx = 0, qy = 0, qz = 0;
  if (i < n) {
    constexpr unsigned SITE_MASK = (1u << MDX_SITE_BITS) - 1u;
    const int4 pi = owner_of ? posn[sl] : posi[i];
    const float4 sti = __ldg(&stab[(unsigned)pi.w & SITE_MASK]);
    const unsigned mi = (unsigned)pi.w >> MDX_SITE_BITS;
    const int ti = __float_as_int(sti.w), ni = __float_as_int(sti.z);
    const float coulf = (float)pc.coulf, alphad = (float)pc.alphad;
    const int eei = tc.iee[ti], lmovei = tc.lmove[ti];
    const float c14e = tc.c14elf[ti], c14l = tc.c14ljf[ti];
    const float qsc = sti.y * coulf, qic = sti.x * coulf;
    const float2 *abrow = tb.abf + ni * pc.nnbt;
    const int c = cnt[i];
    const int *row = idx + list_slot(i, 0, cap, SHORT);
    const size_t rs = SHORT ? 32 : 1;
    const float2 sx2 = splat(sx), sy2 = splat(sy), sz2 = splat(sz);
    const float2 al2 = splat(alphad), qic2 = splat(qic);
    const float2 tpa2 = splat((float)MDX_TOTPI * alphad);
    // one iteration: row entries va, vb (vb a copy of va when hb is false)
    // with their neighbour records pa, pb
    auto pair2 = [&](const int va, const int vb, const int4 pa, const int4 pb, const bool hb) {
      const float4 sa = __ldg(&stab[(unsigned)pa.w & SITE_MASK]);
      const float4 sb = __ldg(&stab[(unsigned)pb.w & SITE_MASK]);
      const bool same_a = ((unsigned)pa.w >> MDX_SITE_BITS) == mi;
      const bool same_b = hb && ((unsigned)pb.w >> MDX_SITE_BITS) == mi;
      if (same_a || same_b) {
        float dxa = fixdiff(pi.x, pa.x, sx), dya = fixdiff(pi.y, pa.y, sy);
        float dza = fixdiff(pi.z, pa.z, sz);
        float dxb = fixdiff(pi.x, pb.x, sx), dyb = fixdiff(pi.y, pb.y, sy);
        float dzb = fixdiff(pi.z, pb.z, sz);
        if (CELL) {
          pbc_cellf(dxa, dya, dza, cf);
          pbc_cellf(dxb, dyb, dzb, cf);
        }
        // the owner's own molecule: one entry at a time, other entry too
        const int nja = __float_as_int(sa.z), njb = __float_as_int(sb.z);
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          if (e == 1 && !hb) break;
          const int v = e ? vb : va;
          const bool same = e ? same_b : same_a;
          const float4 st = e ? sb : sa;
          const bool is14 = SHORT && v < 0;
          const float2 ab = __ldg(&abrow[(same ? (is14 ? 2 : 1) : 0) * tb.nn + (e ? njb : nja)]);
          const float QIJ = same ? (is14 ? qsc * st.y * c14e : qsc * st.y) : qic * st.x;
          const float A6 = is14 ? ab.x * c14l : ab.x, B12 = is14 ? ab.y * c14l : ab.y;
          const float DX = e ? dxb : dxa, DY = e ? dyb : dya, DZ = e ? dzb : dza;
          if (same) {
            pair_same<SHORT, ENER>(DX, DY, DZ, is14, QIJ, A6, B12, eei, lmovei, alphad,
                                   pc.rc2f, s);
          } else {
            // an inter-molecular entry beside one of the own molecule: the
            // paired arithmetic below with the other half empty
            const float RR = DX * DX + DY * DY + DZ * DZ;
            if (SHORT || RR <= pc.rc2f) {
              const float R1I = rsqrtf(RR);
              const float R1 = RR * R1I;
              const float ALPHAR = alphad * R1;
              const float TTT = __fdividef(1.f, 1.f + (float)MDX_B1 * ALPHAR);
              const float EXP2A = __expf(-(ALPHAR * ALPHAR));
              const float ERFCT = ewald_erfc_polyf(TTT, EXP2A);
              const float EE1 = QIJ * R1I;
              float FORCE = EE1 * ((float)MDX_TOTPI * alphad * EXP2A + ERFCT * R1I) * R1I;
              const float R2I = R1I * R1I;
              const float R6I = R2I * R2I * R2I;
              const float ESR = (A6 + B12 * R6I) * R6I;
              const float FSR = (6.f * A6 + 12.f * B12 * R6I) * R6I * R1I;
              FORCE = FORCE + FSR * R1I;
              if (ENER) {
                s.ees.x += EE1 * ERFCT;
                s.ee.x += EE1;
                s.esr.x += ESR;
                s.vir.x += FSR * R1;
                s.vx.x += FORCE * (DX * DX);
                s.vy.x += FORCE * (DY * DY);
                s.vz.x += FORCE * (DZ * DZ);
              }
              s.fx.x += FORCE * DX;
              s.fy.x += FORCE * DY;
              s.fz.x += FORCE * DZ;
            }
          }
        }
        return;
      }
      // two inter-molecular entries (or one and an empty half)
      const float2 aba = __ldg(&abrow[__float_as_int(sa.z)]);
      const float2 abb = __ldg(&abrow[__float_as_int(sb.z)]);
      float2 DX = mul2(make_float2((float)(int)((unsigned)pi.x - (unsigned)pa.x),
                                   (float)(int)((unsigned)pi.x - (unsigned)pb.x)), sx2);
      float2 DY = mul2(make_float2((float)(int)((unsigned)pi.y - (unsigned)pa.y),
                                   (float)(int)((unsigned)pi.y - (unsigned)pb.y)), sy2);
      float2 DZ = mul2(make_float2((float)(int)((unsigned)pi.z - (unsigned)pa.z),
                                   (float)(int)((unsigned)pi.z - (unsigned)pb.z)), sz2);
      if (CELL) {  // a non-rectangular cell (a template parameter: no cost otherwise)
        pbc_cellf(DX.x, DY.x, DZ.x, cf);
        pbc_cellf(DX.y, DY.y, DZ.y, cf);
      }
      float2 RR = fma2(DZ, DZ, fma2(DY, DY, mul2(DX, DX)));
      // an empty half or a pair beyond RCUT (skin mode) contributes nothing
      const bool oka = SHORT || RR.x <= pc.rc2f;
      const bool okb = hb && (SHORT || RR.y <= pc.rc2f);
      float2 QIJ = mul2(make_float2(sa.x, sb.x), qic2);
      float2 A6 = make_float2(aba.x, abb.x), B12 = make_float2(aba.y, abb.y);
      if (!oka) { QIJ.x = 0.f; A6.x = 0.f; B12.x = 0.f; RR.x = 1.f; }
      if (!okb) { QIJ.y = 0.f; A6.y = 0.f; B12.y = 0.f; RR.y = 1.f; }
      const float2 R1I = make_float2(rsqrtf(RR.x), rsqrtf(RR.y));
      const float2 R1 = mul2(RR, R1I);
      const float2 ALPHAR = mul2(al2, R1);
      const float2 den = fma2(splat((float)MDX_B1), ALPHAR, splat(1.f));
      const float2 TTT = make_float2(__fdividef(1.f, den.x), __fdividef(1.f, den.y));
      const float2 A2 = mul2(ALPHAR, ALPHAR);
      const float2 EXP2A = make_float2(__expf(-A2.x), __expf(-A2.y));
      float2 P = fma2(splat((float)MDX_A5), TTT, splat((float)MDX_A4));
      P = fma2(P, TTT, splat((float)MDX_A3));
      P = fma2(P, TTT, splat((float)MDX_A2));
      P = fma2(P, TTT, splat((float)MDX_A1));
      const float2 ERFCT = mul2(mul2(P, TTT), EXP2A);
      const float2 EE1 = mul2(QIJ, R1I);
      float2 FORCE = mul2(mul2(EE1, fma2(tpa2, EXP2A, mul2(ERFCT, R1I))), R1I);
      // LJ (A6 is zero in the tables wherever B12 is, so no test is needed)
      const float2 R2I = mul2(R1I, R1I);
      const float2 R6I = mul2(mul2(R2I, R2I), R2I);
      const float2 FSR = mul2(mul2(fma2(mul2(splat(12.f), B12), R6I, mul2(splat(6.f), A6)), R6I), R1I);
      FORCE = fma2(FSR, R1I, FORCE);
      if (ENER) {
        const float2 ESR = mul2(fma2(B12, R6I, A6), R6I);
        s.ees = fma2(EE1, ERFCT, s.ees);
        s.ee = add2(s.ee, EE1);
        s.esr = add2(s.esr, ESR);
        s.vir = fma2(FSR, R1, s.vir);
        s.vx = fma2(mul2(FORCE, DX), DX, s.vx);
        s.vy = fma2(mul2(FORCE, DY), DY, s.vy);
        s.vz = fma2(mul2(FORCE, DZ), DZ, s.vz);
      }
      s.fx = fma2(FORCE, DX, s.fx);
      s.fy = fma2(FORCE, DY, s.fy);
      s.fz = fma2(FORCE, DZ, s.fz);
    };
    if constexpr (SHORT) {
      // short rows (a few dozen entries) are too short for a pipeline
      for (int k = k0; k < c; k += 2 * TPO) {
        const bool hb = k + TPO < c;
        const int va = row[(size_t)k * rs];
        const int vb = hb ? row[(size_t)(k + TPO) * rs] : va;
        pair2(va, vb, posn[va & 0x7fffffff], posn[vb & 0x7fffffff], hb);
      }
    } else {
      // Software pipeline through shared memory: the row entries of
      // iteration m + 3 and the neighbour records of iteration m + 1 are in
      // flight (cp.async groups, in commit order) while iteration m
      // computes, so the index -> record load chain does not stall every
      // iteration and holds no registers.  Each thread reads back only its
      // own slots.  Entry slots: ring of 4 iterations; records: ring of 2.
      __shared__ int s_v[4][2][256];
      __shared__ int4 s_p[2][2][256];
      const int t = threadIdx.x;
      auto issue_idx = [&](int m) {
        const int e = k0 + 2 * TPO * m;
        if (e < c) cpa4(&s_v[m & 3][0][t], row + (size_t)e * rs);
        if (e + TPO < c) cpa4(&s_v[m & 3][1][t], row + (size_t)(e + TPO) * rs);
        cpa_commit();
      };
      auto issue_rec = [&](int m) {
        const int e = k0 + 2 * TPO * m;
        if (e < c) cpa16(&s_p[m & 1][0][t], posn + (s_v[m & 3][0][t] & 0x7fffffff));
        if (e + TPO < c) cpa16(&s_p[m & 1][1][t], posn + (s_v[m & 3][1][t] & 0x7fffffff));
        cpa_commit();
      };
      const int nit = c > k0 ? (c - k0 + 2 * TPO - 1) / (2 * TPO) : 0;
      issue_idx(0);
      issue_idx(1);
      issue_idx(2);
      cpa_wait<2>();  // entries of iteration 0
      issue_rec(0);
      cpa_wait<1>();  // entries of iterations 1 and 2
      for (int m = 0; m < nit; ++m) {
        const bool hb = k0 + 2 * TPO * m + TPO < c;
        issue_rec(m + 1);
        issue_idx(m + 3);
        cpa_wait<2>();  // records of iteration m, entries of iteration m + 2
        const int va = s_v[m & 3][0][t];
        const int vb = hb ? s_v[m & 3][1][t] : va;
        const int4 pa = s_p[m & 1][0][t];
        const int4 pb = hb ? s_p[m & 1][1][t] : pa;
        pair2(va, vb, pa, pb, hb);
      }
      cpa_wait<0>();  // nothing of this thread left in flight
    }
    qx = f2ll_rn((s.fx.x + s.fx.y) * fsc.scalef);
    qy = f2ll_rn((s.fy.x + s.fy.y) * fsc.scalef);
    qz = f2ll_rn((s.fz.x + s.fz.y) * fsc.scalef);
  }
#pragma unroll
  for (int o = 1; o < TPO; o <<= 1) {
    qx += __shfl_xor_sync(0xffffffffu, qx, o);
    qy += __shfl_xor_sync(0xffffffffu, qy, o);
    qz += __shfl_xor_sync(0xffffffffu, qz, o);
  }
  if (i < n && lane % TPO == 0) {
    ffix[i] = (unsigned long long)qx;
    ffix[n + i] = (unsigned long long)qy;
    ffix[2 * n + i] = (unsigned long long)qz;
  }
  if (!ENER) return;
  float a[P_NSLOT];
  const float ee = s.ee.x + s.ee.y, esr = s.esr.x + s.esr.y;
  a[P_EES] = s.ees.x + s.ees.y;
  a[P_ESR] = esr;
  a[P_VIR] = s.vir.x + s.vir.y;
  a[P_VX] = s.vx.x + s.vx.y;
  a[P_VY] = s.vy.x + s.vy.y;
  a[P_VZ] = s.vz.x + s.vz.y;
  a[P_EE_SAME] = s.ee_same;
  a[P_EE_DIFF] = ee - s.ee_same;
  a[P_ESR_SAME] = s.esr_same;
  a[P_ESR_DIFF] = esr - s.esr_same;
  a[P_WIR] = 0.f;
  slots_out(a, fsc.escalef, slots);
}

// Fold the integer slots of a mixed sweep into mdx_scalars (full rows count
// each pair twice, hence the 1/2 on pair sums).
__global__ void k_fold_slots(unsigned long long *__restrict__ slots, double einv,
                             mdx_scalars *__restrict__ sc, int which, int ntypes,
                             int split) {
  // thread k folds slot k into its own scalar (the slots' sums are
  // independent): one conversion deep instead of P_NSLOT in a row
  const int k = threadIdx.x;
  if (k >= P_NSLOT) return;
  double v = (double)(long long)slots[k] * einv;
  slots[k] = 0ull;
  if (k < P_WIR) v *= 0.5;
  double *dst = nullptr;
  switch (k) {
    case P_EES: dst = which == 1 ? &sc->pels2 : &sc->pels1; break;
    case P_ESR: dst = which == 1 ? &sc->pe2 : &sc->pe1; break;
    case P_VIR: dst = which == 1 ? &sc->vir2 : &sc->vir1; break;
    case P_VX: dst = which == 1 ? &sc->virfx : &sc->virx; break;
    case P_VY: dst = which == 1 ? &sc->virfy : &sc->viry; break;
    case P_VZ: dst = which == 1 ? &sc->virfz : &sc->virz; break;
    case P_WIR: dst = which == 1 ? &sc->wirss : nullptr; break;
    case P_EE_DIFF: dst = ntypes == 1 && !split ? &sc->pote1[0] : nullptr; break;
    case P_ESR_DIFF: dst = ntypes == 1 && !split ? &sc->potl1[0] : nullptr; break;
    case P_EE_SAME: dst = ntypes == 1 && !split ? &sc->pes141[0] : nullptr; break;
    case P_ESR_SAME: dst = ntypes == 1 && !split ? &sc->psr141[0] : nullptr; break;
  }
  if (dst) *dst += v;
}

// Copy the split accumulators (POTE1, POTL1, PES141, PSR141) out.
__global__ void k_fold_split(double *split, mdx_scalars *sc) {
  int k = threadIdx.x;
  if (k < MDX_NTPP) {
    sc->pote1[k] += split[k];
    sc->potl1[k] += split[MDX_NTPP + k];
    split[k] = 0.0;
    split[MDX_NTPP + k] = 0.0;
  }
  if (k < MDX_NT) {
    sc->pes141[k] += split[2 * MDX_NTPP + k];
    sc->psr141[k] += split[2 * MDX_NTPP + MDX_NT + k];
    split[2 * MDX_NTPP + k] = 0.0;
    split[2 * MDX_NTPP + MDX_NT + k] = 0.0;
  }
}

// FP64 path with one molecule type: POTE1 etc. from same/different sums is
// not available (the FP64 sweep sums totals only), so the split sweep is used
// whenever the caller asks for the per-type energies.

PairTables tables(const DevData &d) {
  return PairTables{d.a6lj, d.b12lj, d.a6lj0, d.b12lj0, d.a6_14, d.b12_14,
                    d.a6f,  d.b12f,  d.a60f,  d.b120f,  d.a614f, d.b1214f,
                    d.abf,  d.nnbt * d.nnbt};
}

__global__ void k_pack_lj(int nn, const float *__restrict__ f, float2 *__restrict__ abf) {
  // f: a6f, b12f, a60f, b120f, a614f, b1214f back to back (nn each)
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nn) return;
  // A6 is kept only where B12 is nonzero: the sweeps add the LJ term only
  // for B12 != 0 (forces.f:955, 1166), and the paired sweeps then need no test
  auto ab = [](float a6, float b12) { return make_float2(b12 != 0.f ? a6 : 0.f, b12); };
  abf[k] = ab(f[k], f[nn + k]);
  abf[nn + k] = ab(f[2 * nn + k], f[3 * nn + k]);
  abf[2 * nn + k] = ab(f[4 * nn + k], f[5 * nn + k]);
}

// ener = false: forces only (an intermediate short step of DOUBLE, whose fast
// energies and virials are zeroed again by the next FFORCES before anything
// reads them, forces.f:36-49).
int launch_pair(mdx_ctx *ctx, bool shrt, bool split, bool ener) {
  DevData &d = ctx->dv;
  if (ctx->mixed() && !ctx->tune.tpo_short) resolve_tuning(ctx);
  const int T = 256, WPB = T / 32;
  const int grid = (d.n + WPB - 1) / WPB;
  const int *cnt = shrt ? d.ns_cnt : d.nl_cnt;
  const int *idx = shrt ? d.ns_idx : d.nl_idx;
  const int cap = shrt ? d.cap_s : d.cap_l;
  double *split_buf = d.red + 64;
  if (!ctx->mixed()) {
    double *fx = shrt ? d.hx : d.gx, *fy = shrt ? d.hy : d.gy, *fz = shrt ? d.hz : d.gz;
    mdx_scalars *sc = d.sc;
    Dst6 ddst = shrt ? dst6(ctx, grid, 6, &sc->pels2, &sc->pe2, &sc->vir2, &sc->virfx, &sc->virfy, &sc->virfz)
                     : dst6(ctx, grid, 6, &sc->pels1, &sc->pe1, &sc->vir1, &sc->virx, &sc->viry, &sc->virz);
#define LP64(S, P)                                                                \
  if (ener) k_pair64<S, P, true><<<grid, T, 0, ctx->stream>>>(                    \
      d.n, d.pos, d.ainfo, d.qsite, cnt, idx, cap, tables(d), ctx->tc, ctx->pc,   \
      ctx->boxl, ctx->boyl, ctx->bozl, cell_pbc(ctx), fx, fy, fz, ddst, split_buf); \
  else k_pair64<S, P, false><<<grid, T, 0, ctx->stream>>>(                        \
      d.n, d.pos, d.ainfo, d.qsite, cnt, idx, cap, tables(d), ctx->tc, ctx->pc,   \
      ctx->boxl, ctx->boyl, ctx->bozl, cell_pbc(ctx), fx, fy, fz, ddst, split_buf)
    if (shrt) {
      if (split) { LP64(true, true); } else { LP64(true, false); }
    } else {
      if (split) { LP64(false, true); } else { LP64(false, false); }
    }
#undef LP64
    MDX_LAUNCHED(ctx);
  } else {
    unsigned long long *ffix = shrt ? d.hfix : d.gfix;
    unsigned long long *slots = reinterpret_cast<unsigned long long *>(d.red);
    const double sxs = ctx->boxl / 4294967296.0, sys = fix_period_y(ctx) / 4294967296.0,
                 szs = ctx->bozl / 4294967296.0;
    const double escale = ctx->fix.escale;
    // the cell's fold after the fixed-point differences (the hexagonal
    // cell's y period is 2 BOYL); BOXY3 and 0.5 / cos30 as cell_pbc forms them
    CellF cf{};
    if (ctx->p.icell != 0) {
      const CellPbc c = cell_pbc(ctx);
      cf = CellF{ctx->p.icell, (float)c.hbx, (float)c.bx, (float)c.by, (float)c.boxy3,
                 (float)(0.5 / (double)0.8660254037844386f)};
    }
    // threads per owner atom: the context's tuning (the energy-split sweeps
    // of RECINT keep the defaults)
    const int tpo = split ? (shrt ? TPO_SHORT_DEFAULT : TPO_LONG_DEFAULT)
                          : (shrt ? ctx->tune.tpo_short : ctx->tune.tpo_long);
    const int grid32 = (int)(((long long)tpo * d.n + T - 1) / T);
#define LP32(S, P, E, K)                                                          \
  k_pair32<S, P, E, K><<<grid32, T, 0, ctx->stream>>>(                            \
      d.n, d.posi, d.cell_pos, d.stab, cnt, idx, cap, tables(d),                 \
      ctx->tc, ctx->pc, (float)sxs, (float)sys, (float)szs, ctx->fix, ffix, d.X,  \
      d.Y, d.Z, escale, slots, split_buf, S ? nullptr : d.cell_list, cf)
#define LP32X2C(S, E, K, C)                                                       \
  k_pair32x2<S, E, K, C><<<grid32, T, 0, ctx->stream>>>(                          \
      d.n, d.posi, d.cell_pos, d.stab, cnt, idx, cap, tables(d), ctx->tc, ctx->pc, \
      (float)sxs, (float)sys, (float)szs, ctx->fix, ffix, slots, S ? nullptr : d.cell_list, cf)
#define LP32X2(S, E, K)                        \
  do {                                         \
    if (cf.kind) LP32X2C(S, E, K, true);       \
    else LP32X2C(S, E, K, false);              \
  } while (0)
    // the paired sweeps cover Ewald without MDEE's shifted Coulomb
    const bool paired = !ctx->pc.lmnbl && !ctx->pc.lmdee;
#define LP32E(S, K)                            \
  do {                                         \
    if (paired) {                              \
      if (ener) LP32X2(S, true, K);            \
      else LP32X2(S, false, K);                \
    } else if (ener) LP32(S, false, true, K);  \
    else LP32(S, false, false, K);             \
  } while (0)
    if (split) {
      if (shrt) {
        if (ener) LP32(true, true, true, TPO_SHORT_DEFAULT);
        else LP32(true, true, false, TPO_SHORT_DEFAULT);
      } else {
        if (ener) LP32(false, true, true, TPO_LONG_DEFAULT);
        else LP32(false, true, false, TPO_LONG_DEFAULT);
      }
    } else if (shrt) {
      if (tpo == 2) LP32E(true, 2);
      else if (tpo == 8) LP32E(true, 8);
      else LP32E(true, 4);
    } else {
      if (tpo == 4) LP32E(false, 4);
      else if (tpo == 8) LP32E(false, 8);
      else if (tpo == 16) LP32E(false, 16);
      else LP32E(false, 32);
    }
#undef LP32E
#undef LP32X2
#undef LP32X2C
#undef LP32
    MDX_LAUNCHED(ctx);
    if (ener) {
      k_fold_slots<<<1, 32, 0, ctx->stream>>>(slots, 1.0 / escale, d.sc, shrt ? 1 : 2,
                                              ctx->d.ntypes, split ? 1 : 0);
      MDX_LAUNCHED(ctx);
    }
  }
  if (split) {
    k_fold_split<<<1, 64, 0, ctx->stream>>>(split_buf, d.sc);
    MDX_LAUNCHED(ctx);
  }
  return MDX_OK;
}

template <int N>
int tune_pick(const TuneCell (&cells)[N], int n, double row, int dflt) {
  for (const TuneCell &c : cells)
    if (n <= c.max_atoms && row <= c.max_row) return c.tpo;
  return dflt;
}

}  // namespace

CellPbc cell_pbc(const mdx_ctx *ctx) {
  CellPbc c{};
  c.icell = ctx->p.icell;
  c.bx = ctx->boxl;
  c.by = ctx->boyl;
  c.bz = ctx->bozl;
  c.hbx = 0.5 * ctx->boxl;
  c.hby = 0.5 * ctx->boyl;
  c.hbz = 0.5 * ctx->bozl;
  c.boxy3 = 0.66666666666666666667 * ctx->boyl;  // RECLEN (service.f:579)
  return c;
}

int red_blocks(const mdx_ctx *ctx) {
  return std::max(1, std::min(ctx->nsm, (ctx->dv.n + 255) / 256));
}

// The tuning table's split for this system, from its sizes alone: atoms and
// the mean full-row lengths rho (4/3) pi r^3 of the short and long lists.
void resolve_tuning(mdx_ctx *ctx) {
  if (ctx->tune.tpo_short) return;
  const double vol = ctx->boxl * ctx->boyl * ctx->bozl;
  const double rho = vol > 0 ? ctx->dv.n / vol : 0.0, c = 4.0 / 3.0 * 3.141592653589793;
  const double rs = ctx->p.rshort, rl = ctx->p.rcut + ctx->p.rskin;
  const double row_s = rho * c * rs * rs * rs, row_l = rho * c * (rl * rl * rl - rs * rs * rs);
  ctx->tune.tpo_short = tune_pick(TUNE_SHORT, ctx->dv.n, row_s, TPO_SHORT_DEFAULT);
  ctx->tune.tpo_long = tune_pick(TUNE_LONG, ctx->dv.n, row_l, TPO_LONG_DEFAULT);
  ctx->tune.source = 1;
}

// The interleaved FP32 (A6, B12) tables of the mixed sweeps, from the FP32
// tables (after the topology upload and every RECINT).
int pack_lj_tables(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  const int nn = d.nnbt * d.nnbt;
  if (!d.abf || nn <= 0) return MDX_OK;
  k_pack_lj<<<(nn + 127) / 128, 128, 0, ctx->stream>>>(nn, d.a6f, d.abf);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}


int launch_localf(mdx_ctx *ctx, bool split, bool ener) {
  MDX_TIMER(ctx, MDX_T_PAIR_SHORT); return launch_pair(ctx, true, split, ener); }
int launch_forces_long(mdx_ctx *ctx, bool split) {
  MDX_TIMER(ctx, MDX_T_PAIR_LONG); return launch_pair(ctx, false, split, true); }

int launch_wir(mdx_ctx *ctx, int which) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  double *dst = which == 1 ? &d.sc->wirss : &d.sc->wirs;
  if (which == 1 && ctx->mixed()) {
    const int nb = red_blocks(ctx);
    k_wir_fix<<<nb, 256, 0, ctx->stream>>>(d.n, d.pos, d.ainfo, d.X, d.Y, d.Z, d.hfix,
                                           ctx->fix.inv, dst6(ctx, nb, 1, dst));
    MDX_LAUNCHED(ctx);
    return MDX_OK;
  }
  const double *fx = which == 1 ? d.hx : d.gx, *fy = which == 1 ? d.hy : d.gy,
               *fz = which == 1 ? d.hz : d.gz;
  const int nbw = red_blocks(ctx);
  k_wir<<<nbw, 256, 0, ctx->stream>>>(d.n, d.pos, d.ainfo, d.X, d.Y, d.Z, fx, fy, fz,
                                      dst6(ctx, nbw, 1, dst));
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}
