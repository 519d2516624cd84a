// mdee.cu -- energy differences between expanded-ensemble subensembles for
// the Metropolis move of CHENS (mdee.f:142-262): DIFFUR (reciprocal Ewald,
// self and intramolecular Ewald terms, mdee.f:265-376) and DIFEN (LJ and
// real-space Ewald over the neighbour lists, mdee.f:379-536), on the device.
//
// The subensemble changes only the expanded-ensemble (EE) molecules: their
// charges scale as EC^PW1, their LJ coefficients with other molecules as
// EC^PW1, and their pair distances shift by BEE (1 - EC^PW2).  So:
//  - reciprocal sum: S_old(k) is FURIR's structure factor of the current
//    charges (its first half, run here at the current positions), and
//    S_new(k) = S_old(k) + sum over EE atoms of (QN - QO) e^{i k.r}, one
//    sincos per (k, EE atom); the reference sums both over all atoms;
//  - pair terms: only list pairs with an EE atom on one side and another
//    molecule on the other contribute; both the short and the long rows are
//    swept once (FP64 half rows: all rows; mixed full rows: the EE atoms'
//    rows, pairs of two EE atoms halved);
//  - self terms: host arithmetic on the site charges.
// Returned: EFN, EFO (DIFFUR), EEN, EEO (DIFEN), internal energy units, the
// reference's quantities before CHENS adds the LJ tail change and BETA.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mdx_internal.cuh"

#define RC(x)            \
  do {                   \
    int rc_ = (x);       \
    if (rc_) return rc_; \
  } while (0)

namespace {

constexpr double PI_REF = 3.1415926536;  // common_inc.f:31

// DIFFUR 4.1: per k (block per column, thread per nz), |S_old|^2 and
// |S_new|^2 weighted by AKC.
__global__ void k_ee_recip(int ncol, const KCol *__restrict__ cols,
                           const double *__restrict__ kconst, const double2 *__restrict__ sk,
                           int nee, const int *__restrict__ ee_atom,
                           const double *__restrict__ dq, const dbl4 *__restrict__ pos,
                           double bx, double by, double bz, double hexk, Dst6 dst) {
  // hexk: pi for the hexagonal cell's RYV = 2 pi IKY + pi IKX, else 0; the
  // octahedral columns step nz by 2 (KCol.zstep)
  const double twopi = 2.0 * PI_REF;
  double acc[2] = {0.0, 0.0};  // EFN, EFO
  for (int c = blockIdx.x; c < ncol; c += gridDim.x) {
    const KCol col = cols[c];
    const int len = (col.nzhi - col.nzlo) / col.zstep + 1;
    const double ryv = hexk != 0.0 ? twopi * col.ny + hexk * col.nx : twopi * col.ny;
    const double RXV = (twopi * col.nx) / bx, RYV = ryv / by;
    for (int t = threadIdx.x; t < len; t += blockDim.x) {
      const int k = col.koff + t;
      const double RZV = (twopi * (col.nzlo + col.zstep * t)) / bz;
      double dr = 0.0, di = 0.0;
      for (int e = 0; e < nee; ++e) {
        const dbl4 p = pos[ee_atom[e]];
        double s, cs;
        sincos(RXV * p.x + RYV * p.y + RZV * p.z, &s, &cs);
        dr = fma(dq[e], cs, dr);
        di = fma(dq[e], s, di);
      }
      const double2 S = sk[k];
      const double AKC = kconst[5 * (size_t)k];
      acc[1] += (S.y * S.y + S.x * S.x) * AKC;
      const double nr = S.x + dr, ni = S.y + di;
      acc[0] += (ni * ni + nr * nr) * AKC;
    }
  }
  block_add<2>(acc, dst);
}

__device__ __forceinline__ double erfc_ref(double alphar, double *exp2a) {
  const double TTT = 1.0 / (1.0 + MDX_B1 * alphar);
  const double E = exp(-(alphar * alphar));
  if (exp2a) *exp2a = E;
  return ((((MDX_A5 * TTT + MDX_A4) * TTT + MDX_A3) * TTT + MDX_A2) * TTT + MDX_A1) * TTT * E;
}

// DIFFUR 4.2.2: the reciprocal sum's intramolecular part removed for every
// site pair of an EE molecule (thread per EE atom, partners later in its
// molecule).
__global__ void k_ee_intra(int nee, const int *__restrict__ ee_atom, const dbl4 *__restrict__ pos,
                           const int *__restrict__ mol_first, const int *__restrict__ mol_nat,
                           const int4 *__restrict__ ainfo, const double *__restrict__ qsite,
                           double coulf, double aleen2, double alphad, double bx, double by,
                           double bz, CellPbc cell, Dst6 dst) {
  double acc[2] = {0.0, 0.0};  // EFN, EFO
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nee; e += gridDim.x * blockDim.x) {
    const int i = ee_atom[e];
    const int m = ainfo[i].y, last = mol_first[m] + mol_nat[m];
    const dbl4 pi = pos[i];
    for (int j = i + 1; j < last; ++j) {
      const dbl4 pj = pos[j];
      const double QIJO = coulf * pi.w * pj.w;
      const double QIJN = coulf * aleen2 * qsite[i] * qsite[j];
      double DX = pi.x - pj.x, DY = pi.y - pj.y, DZ = pi.z - pj.z;
      if (cell.icell == 0) pbc_rect(DX, DY, DZ, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
      else pbc_cell(DX, DY, DZ, cell);  // mdee.f:351
      const double R2 = DX * DX + DY * DY + DZ * DZ;
      const double R2I = 1.0 / R2;
      const double R1 = sqrt(R2);
      const double R1I = R1 * R2I;
      const double ERFR = (erfc_ref(alphad * R1, nullptr) - 1.0) * R1I;
      acc[1] += QIJO * ERFR;
      acc[0] += QIJN * ERFR;
    }
  }
  block_add<2>(acc, dst);
}

struct EEPair {
  double coulf, alphad, ealn1, rsho, rshn;
  int nnbt;
  CellPbc cell;  // PBC of the pair (mdee.f:432, 502)
};

// DIFEN's pair term for one listed pair (mdee.f:404-455 / 466-519); adds to
// e[0..1] = EEN, EEO.
__device__ __forceinline__ void ee_pair(int i, int j, const dbl4 *__restrict__ pos,
                                        const int4 *__restrict__ ainfo,
                                        const double *__restrict__ qsite, const TypeConst &tc,
                                        const double *__restrict__ a6lj,
                                        const double *__restrict__ b12lj,
                                        const double *__restrict__ a6lj0,
                                        const double *__restrict__ b12lj0, const EEPair &c,
                                        double bx, double by, double bz, double w, double *e) {
  const int4 ai = ainfo[i], aj = ainfo[j];
  if (tc.iee[ai.x] * tc.iee[aj.x] == 1 || ai.y == aj.y) return;
  const int ix = ai.z * c.nnbt + aj.z;
  const double A6O = a6lj[ix], B12O = b12lj[ix];
  const dbl4 pi = pos[i], pj = pos[j];
  const double QIJO = pi.w * pj.w * c.coulf;
  double ESCI = tc.iee[ai.x] == 0 ? c.ealn1 : 1.0;
  double ESCL = ESCI;
  if (tc.iee[aj.x] == 0) {
    ESCL = ESCI * c.ealn1;
    ESCI = c.ealn1;
  }
  const double A6N = ESCI * a6lj0[ix], B12N = ESCI * b12lj0[ix];
  const double QIJN = ESCL * qsite[i] * qsite[j] * c.coulf;
  double DX = pi.x - pj.x, DY = pi.y - pj.y, DZ = pi.z - pj.z;
  if (c.cell.icell == 0) pbc_rect(DX, DY, DZ, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
  else pbc_cell(DX, DY, DZ, c.cell);
  const double RR = DX * DX + DY * DY + DZ * DZ;
  const double R1 = sqrt(RR);
  const double R1OI = 1. / (R1 + c.rsho), R1NI = 1. / (R1 + c.rshn);
  const double ERFCR = erfc_ref(c.alphad * R1, nullptr);
  const double EESO = QIJO * ERFCR * R1OI, EESN = QIJN * ERFCR * R1NI;
  const double R2O = R1OI * R1OI, R2N = R1NI * R1NI;
  const double R6IO = R2O * R2O * R2O, R6IN = R2N * R2N * R2N;
  const double ESRO = (A6O + B12O * R6IO) * R6IO, ESRN = (A6N + B12N * R6IN) * R6IN;
  e[0] += w * (EESN + ESRN);
  e[1] += w * (EESO + ESRO);
}

// DIFEN over rows: warp per owner.  full == 0: FP64 half rows of atom
// numbers, every row; full == 1: mixed full rows of cell-order slots, the
// EE atoms' rows only (a pair of two EE atoms is in both: weight 1/2).
__global__ void k_ee_pairs(int nown, const int *__restrict__ owners, int full,
                           const int *__restrict__ cnt, const int *__restrict__ idx, int cap,
                           bool tiled, const int *__restrict__ slot_atom,
                           const dbl4 *__restrict__ pos, const int4 *__restrict__ ainfo,
                           const double *__restrict__ qsite, TypeConst tc,
                           const double *__restrict__ a6lj, const double *__restrict__ b12lj,
                           const double *__restrict__ a6lj0, const double *__restrict__ b12lj0,
                           EEPair c, double bx, double by, double bz, Dst6 dst) {
  double e[2] = {0.0, 0.0};
  const int lane = threadIdx.x & 31;
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w < nown) {
    const int i = owners ? owners[w] : w;
    const int n = cnt[i];
    for (int k = lane; k < n; k += 32) {
      const int v = idx[list_slot(i, k, cap, tiled)] & 0x7fffffff;
      const int j = full ? slot_atom[v] : v;
      double wt = 1.0;
      if (full && tc.iee[ainfo[j].x] == 0) wt = 0.5;
      ee_pair(i, j, pos, ainfo, qsite, tc, a6lj, b12lj, a6lj0, b12lj0, c, bx, by, bz, wt, e);
    }
  }
  block_add<2>(e, dst);
}

}  // namespace

extern "C" int mdx_ee_delta(mdx_ctx *ctx, double ec_old, double ec_new, double pw1, double pw2,
                            double bee, double *out) {
  if (!ctx || !out) return MDX_ERR_ARG;
  RC(api_require(ctx, true, true, true));
  if (!ctx->have_lists) {
    ctx->err = "mdx_ee_delta: neighbour lists not built";
    return MDX_ERR_STATE;
  }
  if (ctx->p.lmnbl) {
    ctx->err = "mdx_ee_delta: reaction field not built";
    return MDX_ERR_UNSUPPORTED;
  }
  DevData &d = ctx->dv;
  const int nt = ctx->d.ntypes;
  // EE atoms and their charge change QN - QO (DIFFUR 4.1: QN = CHARGE EC^PW1)
  const double aleeo = std::pow(ec_old, pw1), aleen = std::pow(ec_new, pw1);
  std::vector<int> ee;
  std::vector<double> dq;
  for (int i = 0; i < d.n; ++i) {
    const int t = ctx->h_itype[i] - 1;
    if (ctx->tc.iee[t] != 0) continue;
    ee.push_back(i);
    dq.push_back(ctx->h_charge[ctx->h_nsite[i] - 1] * aleen - ctx->h_q[i]);
  }
  double *acc = d.red + 500;  // EFN, EFO, EEN, EEO
  MDX_CUDA(cudaMemsetAsync(acc, 0, 4 * sizeof(double), ctx->stream));
  const int nee = (int)ee.size();
  int *dee = nullptr;
  double *ddq = nullptr;
  if (nee > 0) {
    MDX_CUDA(ctx_alloc(ctx, &dee, sizeof(int) * nee));
    MDX_CUDA(ctx_alloc(ctx, &ddq, sizeof(double) * nee));
    MDX_CUDA(ctx_copy(ctx->stream, dee, ee.data(), sizeof(int) * nee, cudaMemcpyHostToDevice));
    MDX_CUDA(ctx_copy(ctx->stream, ddq, dq.data(), sizeof(double) * nee, cudaMemcpyHostToDevice));
  }
  const double bx = ctx->boxl, by = ctx->boyl, bz = ctx->bozl;
  int rc = MDX_OK;
  // DIFFUR 4.1
  if (ctx->p.alphad > 0.0) {
    bool skip = false;
    rc = furir_sfac(ctx, &skip);
    if (!rc && !skip) rc = ensure_kconst(ctx);
    if (!rc && !skip) {
      const int nb = std::min(d.ncol, 2 * ctx->nsm);
      k_ee_recip<<<nb, 64, 0, ctx->stream>>>(d.ncol, d.cols, d.kconst, d.sk, nee, dee, ddq,
                                             d.pos, bx, by, bz,
                                             ctx->p.icell == 2 ? PI_REF : 0.0,
                                             dst6(ctx, nb, 2, acc, acc + 1));
      ctx->launches++;
      if (cudaGetLastError() != cudaSuccess) rc = MDX_ERR_CUDA;
    }
    // DIFFUR 4.2.2 (EE types of more than one site)
    if (!rc && nee > 0) {
      const int nb = (nee + 127) / 128;
      k_ee_intra<<<nb, 128, 0, ctx->stream>>>(nee, dee, d.pos, d.mol_first, d.mol_nat, d.ainfo,
                                              d.qsite, ctx->p.coulf, aleen * aleen,
                                              ctx->p.alphad, bx, by, bz, cell_pbc(ctx),
                                              dst6(ctx, nb, 2, acc, acc + 1));
      ctx->launches++;
      if (cudaGetLastError() != cudaSuccess) rc = MDX_ERR_CUDA;
    }
  }
  // DIFEN over the long and the short rows
  if (!rc) {
    const EEPair c{ctx->p.coulf, ctx->p.alphad, aleen, bee * (1. - std::pow(ec_old, pw2)),
                   bee * (1. - std::pow(ec_new, pw2)), ctx->d.nnbt, cell_pbc(ctx)};
    const bool full = ctx->mixed();
    const int nown = full ? nee : d.n;
    if (nown > 0) {
      const int nb = (nown + 7) / 8;
      for (int pass = 0; pass < 2 && !rc; ++pass) {
        const bool shrt = pass == 1;
        k_ee_pairs<<<nb, 256, 0, ctx->stream>>>(
            nown, full ? dee : nullptr, full ? 1 : 0, shrt ? d.ns_cnt : d.nl_cnt,
            shrt ? d.ns_idx : d.nl_idx, shrt ? d.cap_s : d.cap_l, full && shrt, d.cell_list,
            d.pos, d.ainfo, d.qsite, ctx->tc, d.a6lj, d.b12lj, d.a6lj0, d.b12lj0, c, bx, by, bz,
            dst6(ctx, nb, 2, acc + 2, acc + 3));
        ctx->launches++;
        if (cudaGetLastError() != cudaSuccess) rc = MDX_ERR_CUDA;
      }
    }
  }
  double h[4] = {0, 0, 0, 0};
  if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = MDX_ERR_CUDA;
  if (!rc && ctx_copy(ctx->stream, h, acc, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = MDX_ERR_CUDA;
  ctx_free(ctx, dee);
  ctx_free(ctx, ddq);
  if (rc) {
    if (rc == MDX_ERR_CUDA && ctx->err.empty()) ctx->err = "mdx_ee_delta: CUDA error";
    return rc;
  }
  RC(api_check_err(ctx));
  // DIFFUR 4.2.1: the self terms of the EE types' charges
  if (ctx->p.alphad > 0.0) {
    const double ABC = ctx->p.alphad / std::sqrt(PI_REF);
    for (int t = 0; t < nt; ++t) {
      if (ctx->tc.iee[t] != 0) continue;
      for (int II = 1; II <= ctx->nsits[t]; ++II) {
        const double ch = ctx->h_charge[ctx->isadr[t] + II - 1];
        h[1] -= ctx->p.coulf * (aleeo * ch) * (aleeo * ch) * ABC * ctx->nspec[t];
        h[0] -= ctx->p.coulf * (aleen * ch) * (aleen * ch) * ABC * ctx->nspec[t];
      }
    }
  }
  for (int k = 0; k < 4; ++k) out[k] = h[k];
  return MDX_OK;
}
