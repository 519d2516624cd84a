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
    unsigned long long *__restrict__ slots, double *__restrict__ split) {
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
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) / TPO;
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
    const int4 pi = posi[i];
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
      const float DX = idiff(pi.x, pj.x, sx);
      const float DY = idiff(pi.y, pj.y, sy);
      const float DZ = idiff(pi.z, pj.z, sz);
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
  abf[k] = make_float2(f[k], f[nn + k]);
  abf[nn + k] = make_float2(f[2 * nn + k], f[3 * nn + k]);
  abf[2 * nn + k] = make_float2(f[4 * nn + k], f[5 * nn + k]);
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
    const double sxs = ctx->boxl / 4294967296.0, sys = ctx->boyl / 4294967296.0,
                 szs = ctx->bozl / 4294967296.0;
    const double escale = ctx->fix.escale;
    // threads per owner atom: the context's tuning (the energy-split sweeps
    // of RECINT keep the defaults)
    const int tpo = split ? (shrt ? TPO_SHORT_DEFAULT : TPO_LONG_DEFAULT)
                          : (shrt ? ctx->tune.tpo_short : ctx->tune.tpo_long);
    const int grid32 = (int)(((long long)tpo * d.n + T - 1) / T);
#define LP32(S, P, E, K)                                                          \
  k_pair32<S, P, E, K><<<grid32, T, 0, ctx->stream>>>(                            \
      d.n, d.posi, d.cell_pos, d.stab, cnt, idx, cap, tables(d),                 \
      ctx->tc, ctx->pc, (float)sxs, (float)sys, (float)szs, ctx->fix, ffix, d.X,  \
      d.Y, d.Z, escale, slots, split_buf)
#define LP32E(S, K)                      \
  do {                                   \
    if (ener) LP32(S, false, true, K);   \
    else LP32(S, false, false, K);       \
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
      if (tpo == 8) LP32E(false, 8);
      else if (tpo == 16) LP32E(false, 16);
      else LP32E(false, 32);
    }
#undef LP32E
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
