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
// so each (k, atom) term costs one complex multiply-add per pass (4 fused
// multiply-adds) and no transcendental.  Mathematically this is the
// reference's sum; in FP64 the difference is rounding (the recurrence adds
// about |n| ulp).
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

// Phase tables: thread per (axis, atom), FP64 recurrence from one sincos.
__global__ void k_tables(int n, const dbl4 *__restrict__ pos, double ibx,
                         double iby, double ibz, int kx, int ky, int kz,
                         double2 *__restrict__ tx, double2 *__restrict__ ty,
                         double2 *__restrict__ tz, float2 *__restrict__ txf,
                         float2 *__restrict__ tyf, float2 *__restrict__ tzf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * n) return;
  const int a = t / n, i = t - a * n;
  const dbl4 p = pos[i];
  const double x = a == 0 ? p.x * ibx : a == 1 ? p.y * iby : p.z * ibz;
  double s, c;
  sincos(2.0 * PI_REF * x, &s, &c);
  const double2 e = make_double2(c, s);
  // x and y tables hold n = 0..K; the z table holds n = -K..K (conjugates
  // stored) at index n + K, so the inner loops need no sign test
  const int kzo = (kz - 1) / 2;
  const int len = a == 0 ? kx : a == 1 ? ky : kzo + 1;
  const int off = a == 2 ? kzo : 0;
  const double q = a == 0 ? p.w : 1.0;
  double2 v = make_double2(1.0, 0.0);
  if (txf) {  // mixed path: FP64 recurrence, FP32 table
    float2 *dst = (a == 0 ? txf : a == 1 ? tyf : tzf) + i;
    for (int k = 0; k < len; ++k) {
      dst[(size_t)(off + k) * n] = make_float2((float)(q * v.x), (float)(q * v.y));
      if (a == 2) dst[(size_t)(off - k) * n] = make_float2((float)v.x, (float)-v.y);
      v = cmul(v, e);
    }
  } else {
    double2 *dst = (a == 0 ? tx : a == 1 ? ty : tz) + i;
    for (int k = 0; k < len; ++k) {
      dst[(size_t)(off + k) * n] = make_double2(q * v.x, q * v.y);
      if (a == 2) dst[(size_t)(off - k) * n] = make_double2(v.x, -v.y);
      v = cmul(v, e);
    }
  }
}

// S(k): thread per chunk (column, up to CH consecutive nz), block.y = slice
// of atoms staged TILE at a time in shared memory.
template <typename R, typename C2>
__global__ void __launch_bounds__(128) k_sfac(
    int n, int nchunk, const Chunk *__restrict__ chunks,
    const KCol *__restrict__ cols, const C2 *__restrict__ tx,
    const C2 *__restrict__ ty, const C2 *__restrict__ tz, int kx, int ky, int kz,
    double2 *__restrict__ sk, double2 *__restrict__ part, int nkv) {
  extern __shared__ unsigned char smem_raw[];
  C2 *sx = reinterpret_cast<C2 *>(smem_raw);  // [atom][n]
  C2 *sy = sx + TILE * kx;
  C2 *sz = sy + TILE * ky;
  const int ch = blockIdx.x * blockDim.x + threadIdx.x;
  const int a0 = blockIdx.y * SLICE, a1 = min(n, a0 + SLICE);
  Chunk cc{0, 0, 0, 0};
  KCol col{0, 0, 0, 0, 0};
  if (ch < nchunk) {
    cc = chunks[ch];
    col = cols[cc.col];
  }
  const int ny = col.ny < 0 ? -col.ny : col.ny;
  const bool nyneg = col.ny < 0;
  const int kzo = (kz - 1) / 2;
  R sr[CH], si[CH];
#pragma unroll
  for (int t = 0; t < CH; ++t) sr[t] = si[t] = R(0);
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
        const C2 X = sx[j * kx + col.nx];
        const C2 Y = conj_if(sy[j * ky + ny], nyneg);
        const R tr = fma(X.x, Y.x, -X.y * Y.y), ti = fma(X.x, Y.y, X.y * Y.x);
        const C2 *zr = sz + j * kz;
#pragma unroll
        for (int t = 0; t < CH; ++t) {
          if (t < cc.len) {
            const C2 Z = zr[cc.nz0 + t + kzo];
            sr[t] = fma(tr, Z.x, sr[t]);
            sr[t] = fma(-ti, Z.y, sr[t]);
            si[t] = fma(tr, Z.y, si[t]);
            si[t] = fma(ti, Z.x, si[t]);
          }
        }
      }
    }
  }
  if (ch < nchunk) {
#pragma unroll
    for (int t = 0; t < CH; ++t)
      if (t < cc.len) {
        if (part) {  // slice partial, summed in slice order by k_sfac_sum
          part[(size_t)blockIdx.y * nkv + cc.k0 + t] = make_double2((double)sr[t], (double)si[t]);
        } else {
          atomicAdd(&sk[cc.k0 + t].x, (double)sr[t]);
          atomicAdd(&sk[cc.k0 + t].y, (double)si[t]);
        }
      }
  }
}

// S(k) = sum of the slice partials in slice order (deterministic).
__global__ void k_sfac_sum(int nkv, int nslice, const double2 *__restrict__ part,
                           double2 *__restrict__ sk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nkv) return;
  double x = 0.0, y = 0.0;
  for (int s = 0; s < nslice; ++s) {
    const double2 v = part[(size_t)s * nkv + k];
    x += v.x;
    y += v.y;
  }
  sk[k] = make_double2(x, y);
}

// Per k: energy and virial terms (forces.f:1316-1331), W_k and RZV W_k.
__global__ void k_kterms(int ncol, const KCol *__restrict__ cols,
                         const double2 *__restrict__ sk, double bx, double by,
                         double bz, double alp2, double cfur,
                         dbl4 *__restrict__ wk, float4 *__restrict__ wkf,
                         double2 *__restrict__ colrv, float2 *__restrict__ colrvf,
                         Dst6 dst) {
  double acc[4] = {0, 0, 0, 0};
  const double twopi = 2.0 * PI_REF;
  for (int c = blockIdx.x; c < ncol; c += gridDim.x) {
    const KCol col = cols[c];
    const int len = col.nzhi - col.nzlo + 1;
    if (threadIdx.x == 0) {
      const double rx = (twopi * col.nx) / bx, ry = (twopi * col.ny) / by;
      colrv[c] = make_double2(rx, ry);
      colrvf[c] = make_float2((float)rx, (float)ry);
    }
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int k = col.koff + t;
      const int nz = col.nzlo + t;
      const double RXV = (twopi * col.nx) / bx;
      const double RYV = (twopi * col.ny) / by;
      const double RZV = (twopi * nz) / bz;
      const double RK2 = RXV * RXV + RYV * RYV + RZV * RZV;
      const double2 S = sk[k];
      const double SCS = S.x, SSN = S.y;
      const double AKC = cfur * exp(-0.25 * RK2 / alp2) / RK2;
      const double S2 = SSN * SSN + SCS * SCS;
      acc[0] += AKC * S2;
      const double AKV = 0.5 * AKC * (4. * alp2 + RK2) / (alp2 * RK2);
      acc[1] -= (RXV * RXV) * AKV * S2;
      acc[2] -= (RYV * RYV) * AKV * S2;
      acc[3] -= (RZV * RZV) * AKV * S2;
      const double AK2 = 2.0 * AKC;
      dbl4 W;
      W.x = AK2 * SCS;
      W.y = -AK2 * SSN;
      W.z = RZV * W.x;
      W.w = RZV * W.y;
      if (wkf)
        wkf[k] = make_float4((float)W.x, (float)W.y, (float)W.z, (float)W.w);
      else
        wk[k] = W;
    }
  }
  block_add<4>(acc, dst);
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

// Column sums U = sum_nz W_k Z(nz), V = sum_nz RZV_k W_k Z(nz) over the
// signed z table (Z points at row nz = 0 of this atom).  wk holds
// (Re W, Im W, Re RZV W, Im RZV W) per k.
template <typename R, typename W4, typename C2>
__device__ __forceinline__ void column_sums(const C2 *__restrict__ Z, int n,
                                            const W4 *__restrict__ wk,
                                            const KCol &col, R &ux, R &uy,
                                            R &vx, R &vy) {
  const C2 *z = Z + (long long)col.nzlo * n;
  const W4 *w = wk + col.koff;
  const int len = col.nzhi - col.nzlo + 1;
#pragma unroll 4
  for (int t = 0; t < len; ++t) {
    const C2 zz = z[(long long)t * n];
    const W4 a = w[t];
    ux = fma(a.x, zz.x, ux);
    ux = fma(-a.y, zz.y, ux);
    uy = fma(a.x, zz.y, uy);
    uy = fma(a.y, zz.x, uy);
    vx = fma(a.z, zz.x, vx);
    vx = fma(-a.w, zz.y, vx);
    vy = fma(a.z, zz.y, vy);
    vy = fma(a.w, zz.x, vy);
  }
}

// Force passes: a block is RF_ATOMS atoms x RF_PARTS column parts (one warp
// per part); part p takes columns p, p + RF_PARTS, ... and the parts are
// added in part order through shared memory, so the sum is deterministic.
constexpr int RF_ATOMS = 32;
constexpr int RF_PARTS = 4;

__global__ void __launch_bounds__(RF_ATOMS *RF_PARTS) k_rforce64(
    int n, int ncol, const KCol *__restrict__ cols, const dbl4 *__restrict__ wk,
    const double2 *__restrict__ tx, const double2 *__restrict__ ty,
    const double2 *__restrict__ tz, int kzo, const double2 *__restrict__ colrv,
    double *__restrict__ gx, double *__restrict__ gy, double *__restrict__ gz) {
  __shared__ double red[3][RF_PARTS][RF_ATOMS];
  const int lane = threadIdx.x % RF_ATOMS, part = threadIdx.x / RF_ATOMS;
  const int i = blockIdx.x * RF_ATOMS + lane;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (i < n) {
    const double2 *Z = tz + (size_t)kzo * n + i;
    for (int c = part; c < ncol; c += RF_PARTS) {
      const KCol col = cols[c];
      double ux = 0., uy = 0., vx = 0., vy = 0.;
      column_sums<double, dbl4, double2>(Z, n, wk, col, ux, uy, vx, vy);
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

__global__ void __launch_bounds__(RF_ATOMS *RF_PARTS) k_rforce32(
    int n, int ncol, const KCol *__restrict__ cols, const float4 *__restrict__ wk,
    const float2 *__restrict__ tx, const float2 *__restrict__ ty,
    const float2 *__restrict__ tz, int kzo, const float2 *__restrict__ colrv,
    FixScale fsc, unsigned long long *__restrict__ gfix) {
  __shared__ long long red[3][RF_PARTS][RF_ATOMS];
  const int lane = threadIdx.x % RF_ATOMS, part = threadIdx.x / RF_ATOMS;
  const int i = blockIdx.x * RF_ATOMS + lane;
  const float sc = fsc.scalef;
  long long ax = 0, ay = 0, az = 0;
  if (i < n) {
    const float2 *Z = tz + (size_t)kzo * n + i;
    for (int c = part; c < ncol; c += RF_PARTS) {
      const KCol col = cols[c];
      float ux = 0.f, uy = 0.f, vx = 0.f, vy = 0.f;
      column_sums<float, float4, float2>(Z, n, wk, col, ux, uy, vx, vy);
      const int ny = col.ny < 0 ? -col.ny : col.ny;
      const float2 T = cmulf(tx[(size_t)col.nx * n + i],
                             conj_if(ty[(size_t)ny * n + i], col.ny < 0));
      const float imTU = fmaf(T.x, uy, T.y * ux);
      const float imTV = fmaf(T.x, vy, T.y * vx);
      // per-column partials go to 64-bit fixed point (order independent)
      const float2 rv = colrv[c];
      ax += f2ll_rn(rv.x * imTU * sc);
      ay += f2ll_rn(rv.y * imTU * sc);
      az += f2ll_rn(imTV * sc);
    }
  }
  red[0][part][lane] = ax;
  red[1][part][lane] = ay;
  red[2][part][lane] = az;
  __syncthreads();
  if (part == 0 && i < n) {
#pragma unroll
    for (int p = 1; p < RF_PARTS; ++p) {
      ax += red[0][p][lane];
      ay += red[1][p][lane];
      az += red[2][p][lane];
    }
    gfix[i] += (unsigned long long)ax;
    gfix[n + i] += (unsigned long long)ay;
    gfix[2 * n + i] += (unsigned long long)az;
  }
}

// ETERMS (forces.f:1482-1676): thread per atom ISP over its bound partners
// JSP < ISP (normal types), or over all intramolecular pairs of EE types.
__device__ __forceinline__ void eterms_pair(
    int isp, int jsp, int ityp, const dbl4 &pi, const dbl4 &pj, double coulf,
    double alphad, double bx, double by, double bz, const TypeConst &tc,
    double *acc, double *spee_sh, double *gx, double *gy, double *gz,
    unsigned long long *gfix, int n, double fscale) {
  const double QIJ = coulf * pi.w * pj.w;
  double DX = pi.x - pj.x, DY = pi.y - pj.y, DZ = pi.z - pj.z;
  pbc_rect(DX, DY, DZ, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
  const double R2 = DX * DX + DY * DY + DZ * DZ;
  const double R2I = 1.0 / R2;
  const double R1 = sqrt(R2);
  const double R1I = R1 * R2I;
  const double ALPHAR = alphad * R1;
  const double TTT = 1.0 / (1.0 + MDX_B1 * ALPHAR);
  const double EXP2A = exp(-(ALPHAR * ALPHAR));
  const double ERFC =
      ((((MDX_A5 * TTT + MDX_A4) * TTT + MDX_A3) * TTT + MDX_A2) * TTT + MDX_A1) * TTT * EXP2A;
  const double EES = QIJ * (ERFC - 1.0) * R1I;
  acc[0] += EES;
  atomicAdd(&spee_sh[ityp], EES);
  if (tc.lmove[ityp]) {
    const double FES = QIJ * ((MDX_TOTPI * ALPHAR * EXP2A + ERFC) - 1.0) * R1I * R2I;
    if (gfix) {
      fix_add(&gfix[isp], FES * DX, fscale);
      fix_add(&gfix[n + isp], FES * DY, fscale);
      fix_add(&gfix[2 * n + isp], FES * DZ, fscale);
      fix_add(&gfix[jsp], -FES * DX, fscale);
      fix_add(&gfix[n + jsp], -FES * DY, fscale);
      fix_add(&gfix[2 * n + jsp], -FES * DZ, fscale);
    } else {
      atomicAdd(&gx[isp], FES * DX);
      atomicAdd(&gy[isp], FES * DY);
      atomicAdd(&gz[isp], FES * DZ);
      atomicAdd(&gx[jsp], -FES * DX);
      atomicAdd(&gy[jsp], -FES * DY);
      atomicAdd(&gz[jsp], -FES * DZ);
    }
    acc[1] += FES * (DX * DX);
    acc[2] += FES * (DY * DY);
    acc[3] += FES * (DZ * DZ);
  }
}

__global__ void k_eterms(int n, const dbl4 *__restrict__ pos,
                         const int4 *__restrict__ ainfo,
                         const int *__restrict__ nnbb,
                         const int *__restrict__ inbb, int nbdmax,
                         const int *__restrict__ mol_first, TypeConst tc,
                         double coulf, double alphad, double bx, double by,
                         double bz, double *gx, double *gy, double *gz,
                         unsigned long long *gfix, double fscale, Dst6 dst,
                         double *spee) {
  __shared__ double spee_sh[MDX_NT];
  if (threadIdx.x < MDX_NT) spee_sh[threadIdx.x] = 0.0;
  __syncthreads();
  double acc[4] = {0, 0, 0, 0};
  const int isp = blockIdx.x * blockDim.x + threadIdx.x;
  if (isp < n) {
    const int4 ai = ainfo[isp];
    const int ityp = ai.x;
    const dbl4 pi = pos[isp];
    if (tc.iee[ityp] != 0) {
      const int nb = nnbb[isp];
      for (int k = 0; k < nb; ++k) {
        int jf = inbb[isp * nbdmax + k];
        int jsp = (jf < 0 ? -jf : jf) - 1;
        if (isp > jsp)
          eterms_pair(isp, jsp, ityp, pi, pos[jsp], coulf, alphad, bx, by, bz,
                      tc, acc, spee_sh, gx, gy, gz, gfix, n, fscale);
      }
    } else {
      // EE molecule: every intramolecular pair JSM < ISM (forces.f:1585-1594)
      const int f = mol_first[ai.y];
      for (int jsp = f; jsp < isp; ++jsp)
        eterms_pair(isp, jsp, ityp, pi, pos[jsp], coulf, alphad, bx, by, bz, tc,
                    acc, spee_sh, gx, gy, gz, gfix, n, fscale);
    }
  }
  block_add<4>(acc, dst);
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

// INIFUR: the reference's k-set (forces.f:1366-1424) regrouped in columns,
// and the self-energy SPEEI/SPEI (forces.f:1426-1447).
int host_inifur(mdx_ctx *ctx) {
  if (ctx->p.icell != 0) {
    ctx->err = "Ewald sum for non-rectangular cells is not built";
    return MDX_ERR_UNSUPPORTED;
  }
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
  const int NY = 2 * KMAY + 1, NZ = 2 * KMAZ + 1;
  std::vector<unsigned char> in((size_t)(KMAX + 1) * NY * NZ, 0);
  int nkv = 0;
  for (int IKZ = -KMAZ; IKZ <= KMAZ; ++IKZ)
    for (int IKX = 0; IKX <= KMAX; ++IKX) {
      int KY1 = IKX == 0 ? (IKZ > 0 ? 0 : 1) : -KMAY;
      for (int IKY = KY1; IKY <= KMAY; ++IKY) {
        double RXV = TWOPI * IKX, RYV = TWOPI * IKY, RZV = TWOPI * IKZ;
        double rx = RXV / ctx->boxl, ry = RYV / ctx->boyl, rz = RZV / ctx->bozl;
        double RK2 = rx * rx + ry * ry + rz * rz;
        if (RK2 <= CUTK2) {
          ++nkv;
          in[((size_t)IKX * NY + (IKY + KMAY)) * NZ + (IKZ + KMAZ)] = 1;
        }
      }
    }
  if (nkv > ctx->d.nkv_max) {
    ctx->err = "max number of reciprocal vectors exceeded (NKVM)";
    return MDX_ERR_KVEC;
  }
  std::vector<KCol> cols;
  std::vector<Chunk> chunks;
  int koff = 0;
  for (int ix = 0; ix <= KMAX; ++ix)
    for (int iy = -KMAY; iy <= KMAY; ++iy) {
      int lo = 1 << 30, hi = -(1 << 30), cnt = 0;
      for (int iz = -KMAZ; iz <= KMAZ; ++iz)
        if (in[((size_t)ix * NY + (iy + KMAY)) * NZ + (iz + KMAZ)]) {
          lo = std::min(lo, iz);
          hi = std::max(hi, iz);
          ++cnt;
        }
      if (!cnt) continue;
      if (cnt != hi - lo + 1) {
        ctx->err = "k-set column is not contiguous";
        return MDX_ERR_UNSUPPORTED;
      }
      const int c = (int)cols.size();
      cols.push_back(KCol{ix, iy, lo, hi, koff});
      for (int z0 = lo; z0 <= hi; z0 += CH)
        chunks.push_back(Chunk{c, z0, std::min(CH, hi - z0 + 1), koff + (z0 - lo)});
      koff += cnt;
    }
  const int kx = KMAX + 1, ky = KMAY + 1, kz = 2 * KMAZ + 1;
  const bool realloc_tables = kx != d.kx || ky != d.ky || kz != d.kz;
  d.kx = kx;
  d.ky = ky;
  d.kz = kz;
  d.nkv = nkv;
  d.ncol = (int)cols.size();
  ctx->nkv = nkv;
  if (d.cols) cudaFree(d.cols);
  if (d.kchunks) cudaFree(d.kchunks);
  d.cols = nullptr;
  d.kchunks = nullptr;
  MDX_CUDA(cudaMalloc(&d.cols, sizeof(KCol) * std::max<size_t>(1, cols.size())));
  MDX_CUDA(cudaMalloc(&d.kchunks, sizeof(Chunk) * std::max<size_t>(1, chunks.size())));
  MDX_CUDA(cudaMemcpy(d.cols, cols.data(), sizeof(KCol) * cols.size(), cudaMemcpyHostToDevice));
  MDX_CUDA(cudaMemcpy(d.kchunks, chunks.data(), sizeof(Chunk) * chunks.size(),
                      cudaMemcpyHostToDevice));
  d.nchunk = (int)chunks.size();
  // shared-memory tile of the S(k) kernel: TILE atoms x all table rows
  const size_t sh = (ctx->mixed() ? sizeof(float2) : sizeof(double2)) * TILE * (kx + ky + kz);
  if (sh > SFAC_SMEM_MAX) {
    ctx->err = "reciprocal k-set too large for the structure-factor tile";
    return MDX_ERR_UNSUPPORTED;
  }
  if (sh > 48 * 1024) {
    if (ctx->mixed())
      MDX_CUDA(cudaFuncSetAttribute(k_sfac<float, float2>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
    else
      MDX_CUDA(cudaFuncSetAttribute(k_sfac<double, double2>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  }
  if (realloc_tables) {
    cudaFree(d.tabx);
    cudaFree(d.tabxf);
    d.tabx = d.taby = d.tabz = nullptr;
    d.tabxf = d.tabyf = d.tabzf = nullptr;
    const size_t per = (size_t)kx + ky + kz;
    if (ctx->mixed()) {
      MDX_CUDA(cudaMalloc(&d.tabxf, sizeof(float2) * per * d.n));
      d.tabyf = d.tabxf + (size_t)kx * d.n;
      d.tabzf = d.tabyf + (size_t)ky * d.n;
    } else {
      MDX_CUDA(cudaMalloc(&d.tabx, sizeof(double2) * per * d.n));
      d.taby = d.tabx + (size_t)kx * d.n;
      d.tabz = d.taby + (size_t)ky * d.n;
    }
  }
  if (d.sk) cudaFree(d.sk);
  const size_t nk = (size_t)std::max(1, nkv);
  const size_t nkp = (nk + 1) & ~(size_t)1;  // keeps wk 32-byte aligned
  const size_t nc = std::max<size_t>(1, cols.size());
  MDX_CUDA(cudaMalloc(&d.sk, sizeof(double2) * (nkp + 3 * nk + 2 * nc)));
  d.wk = reinterpret_cast<dbl4 *>(d.sk + nkp);
  d.wkf = reinterpret_cast<float4 *>(d.wk + nk);
  d.colrv = reinterpret_cast<double2 *>(d.wkf + nk);
  d.colrvf = reinterpret_cast<float2 *>(d.colrv + nc);
  // per-slice partials of S(k), summed in slice order
  if (d.sk_part) cudaFree(d.sk_part);
  d.sk_part = nullptr;
  const size_t nslice = ((size_t)d.n + SLICE - 1) / SLICE;
  if (cudaMalloc(reinterpret_cast<void **>(&d.sk_part), sizeof(double2) * nslice * nk) !=
      cudaSuccess) {
    d.sk_part = nullptr;  // falls back to atomic slice sums
    cudaGetLastError();
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

int launch_furir(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  if (ctx->p.alphad <= 0.0) return MDX_OK;
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
  if (d.nkv == 0 || (ctx->d.ntypes == 1 && ctx->nspec[0] == 1)) return MDX_OK;
  const double ibx = 1.0 / ctx->boxl, iby = 1.0 / ctx->boyl, ibz = 1.0 / ctx->bozl;
  const double vol = ctx->boxl * ctx->boyl * ctx->bozl;
  const double alp2 = ctx->p.alphad * ctx->p.alphad;
  const double cfur = 4.0 * PI_REF * ctx->p.coulf / vol;
  const Chunk *chunks = reinterpret_cast<const Chunk *>(d.kchunks);
  const int nchunk = d.nchunk;
  const bool mx = ctx->mixed();
  {
    MDX_TIMER(ctx, MDX_T_EW_TABLES);
    k_tables<<<(3 * d.n + 255) / 256, 256, 0, ctx->stream>>>(
        d.n, d.pos, ibx, iby, ibz, d.kx, d.ky, d.kz, d.tabx, d.taby, d.tabz,
        d.tabxf, d.tabyf, d.tabzf);
    MDX_LAUNCHED(ctx);
  }
  MDX_CUDA(cudaMemsetAsync(d.sk, 0, sizeof(double2) * d.nkv, ctx->stream));
  {
    MDX_TIMER(ctx, MDX_T_EW_SFAC);
    dim3 grid((nchunk + 127) / 128, (d.n + SLICE - 1) / SLICE);
    const size_t sh = (mx ? sizeof(float2) : sizeof(double2)) * TILE * (d.kx + d.ky + d.kz);
    if (mx) {
      k_sfac<float, float2><<<grid, 128, sh, ctx->stream>>>(
          d.n, nchunk, chunks, d.cols, d.tabxf, d.tabyf, d.tabzf, d.kx, d.ky, d.kz, d.sk,
          d.sk_part, d.nkv);
    } else {
      k_sfac<double, double2><<<grid, 128, sh, ctx->stream>>>(
          d.n, nchunk, chunks, d.cols, d.tabx, d.taby, d.tabz, d.kx, d.ky, d.kz, d.sk,
          d.sk_part, d.nkv);
    }
    MDX_LAUNCHED(ctx);
    if (d.sk_part) {
      k_sfac_sum<<<(d.nkv + 255) / 256, 256, 0, ctx->stream>>>(d.nkv, (int)grid.y,
                                                                d.sk_part, d.sk);
      MDX_LAUNCHED(ctx);
    }
  }
  double *qpe = d.red + 40;
  mdx_scalars *sc = d.sc;
  {
    MDX_TIMER(ctx, MDX_T_EW_KTERMS);
    Dst6 dst = dst6(ctx, std::min(d.ncol, 1024), 4, qpe, &sc->virx, &sc->viry, &sc->virz);
    k_kterms<<<std::min(d.ncol, 1024), 64, 0, ctx->stream>>>(
        d.ncol, d.cols, d.sk, ctx->boxl, ctx->boyl, ctx->bozl, alp2, cfur, d.wk,
        mx ? d.wkf : nullptr, d.colrv, d.colrvf, dst);
    MDX_LAUNCHED(ctx);
    k_qpe_fold<<<1, 1, 0, ctx->stream>>>(sc, qpe);
    MDX_LAUNCHED(ctx);
  }
  MDX_TIMER(ctx, MDX_T_EW_FORCE);
  const int kzo = (d.kz - 1) / 2;
  const int rblocks = (d.n + RF_ATOMS - 1) / RF_ATOMS;
  if (mx) {
    k_rforce32<<<rblocks, RF_ATOMS * RF_PARTS, 0, ctx->stream>>>(
        d.n, d.ncol, d.cols, d.wkf, d.tabxf, d.tabyf, d.tabzf, kzo, d.colrvf, ctx->fix,
        d.gfix);
  } else {
    k_rforce64<<<rblocks, RF_ATOMS * RF_PARTS, 0, ctx->stream>>>(
        d.n, d.ncol, d.cols, d.wk, d.tabx, d.taby, d.tabz, kzo, d.colrv, d.gx, d.gy, d.gz);
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
  k_eterms<<<(d.n + 127) / 128, 128, 0, ctx->stream>>>(
      d.n, d.pos, d.ainfo, d.nnbb, d.inbb, d.nbdmax, d.mol_first, ctx->tc,
      ctx->p.coulf, ctx->p.alphad, ctx->boxl, ctx->boyl, ctx->bozl, d.gx, d.gy,
      d.gz, ctx->mixed() ? d.gfix : nullptr, ctx->fix.scale, dst, sc->spee);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}
