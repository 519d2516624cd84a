// integrate.cu -- collectors and integrator pieces of the step:
//   ZEROFS service.f:397-453, SCLFRC service.f:182-287, CM_ADDLA
//   scalar.f:88-116, GETCOM service.f:463-563, GETEMP service.f:35-117,
//   SCALING mdstep.f:534-1093 (as device stages), SHEJK mdstep.f:1105-1283,
//   and the kick/drift loops of DOUBLE (mdstep.f:346-431) and SULTAN
//   (mdstep.f:89-113).
// All state stays on the device; scalar logic (thermostat, barostat) runs in
// single-thread stage kernels that read and write the mdx_thermo block, so a
// whole step is a fixed sequence of launches with no host round trip.
#include <cmath>

#include <algorithm>

#include <cstring>

#include "mdx_internal.cuh"

namespace {

// ------------------------------------------------------------- zeroing ---
__global__ void k_zero_scalars(mdx_scalars *sc, int which, int molint, int ntypes) {
  int k = threadIdx.x;
  if (k < molint) {
    sc->pote1[k] = 0.0;
    sc->potl1[k] = 0.0;
  }
  if (k < ntypes) {
    sc->pes141[k] = 0.0;
    sc->psr141[k] = 0.0;
  }
  if (k == 0) {
    if (which == 1) {
      sc->pels2 = 0.; sc->pint = 0.; sc->pe2 = 0.; sc->virb = 0.; sc->vir2 = 0.;
      sc->wirss = 0.; sc->virfx = 0.; sc->virfy = 0.; sc->virfz = 0.;
    } else {
      sc->wirs = 0.; sc->vir1 = 0.; sc->pe1 = 0.; sc->pels1 = 0.;
      sc->virx = 0.; sc->viry = 0.; sc->virz = 0.; sc->qpe = 0.;
      sc->lscfl = 0;
    }
  }
}

__global__ void k_fix_fold(int n, const unsigned long long *__restrict__ f,
                           double inv, double *__restrict__ x,
                           double *__restrict__ y, double *__restrict__ z) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = (double)(long long)f[i] * inv;
  y[i] = (double)(long long)f[n + i] * inv;
  z[i] = (double)(long long)f[2 * n + i] * inv;
}

// SCLFRC (service.f:182-287)
__global__ void k_sclfrc(int n, double fct, const double *__restrict__ massdi,
                         double *x, double *y, double *z, mdx_scalars *sc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double f = x[i] * x[i] + y[i] * y[i] + z[i] * z[i];
  f = sqrt(f) * fct * massdi[i];
  if (f > 1.0) {
    if (f > 1.0e20) {
      x[i] = 0.; y[i] = 0.; z[i] = 0.;
    } else {
      x[i] = x[i] / f; y[i] = y[i] / f; z[i] = z[i] / f;
    }
    sc->lscfl = 1;
  }
}

// CM_ADDLA: F = G + H (scalar.f:106-113)
__global__ void k_sum_forces(int n, const double *gx, const double *gy,
                             const double *gz, const double *hx,
                             const double *hy, const double *hz, double *fx,
                             double *fy, double *fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fx[i] = gx[i] + hx[i];
  fy[i] = gy[i] + hy[i];
  fz[i] = gz[i] + hz[i];
}

// ----------------------------------------------------------------- GETCOM
struct MolConst {
  double summas[MDX_NT];
  double rsummas[MDX_NT];  // 1 / summas (mixed path's centre of mass)
  CellPbc cell;            // cell shape of the centres' PBC (service.f:530-537)
};

// PBC of a centre of mass: the rectangular fold, or the cell's
__device__ __forceinline__ void pbc_com(double &x, double &y, double &z, double bx, double by,
                                        double bz, const MolConst &mc) {
  if (mc.cell.icell == 0) pbc_rect(x, y, z, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
  else pbc_cell(x, y, z, mc.cell);
}

// GETCOM (service.f:463-563); with posi set it also refreshes the
// fixed-point mirror of the wrapped positions (what k_mirror writes for the
// sweeps), so a short step needs no separate mirror pass.  The FP32 mirror
// posf only feeds the list build, which refreshes it itself.
__global__ void k_getcom(int nop, const int *__restrict__ mol_first,
                         const int *__restrict__ mol_nat,
                         const int *__restrict__ mol_type,
                         const double *__restrict__ amass, dbl4 *pos, double *X,
                         double *Y, double *Z, MolConst mc, double bx, double by,
                         double bz, float4 *__restrict__ posf, int4 *__restrict__ posi,
                         const int *__restrict__ pinfo) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nop) return;
  const int f = mol_first[m], na = mol_nat[m];
  const double summ = mc.summas[mol_type[m]];
  double x = 0., y = 0., z = 0.;
  for (int k = 0; k < na; ++k) {
    const dbl4 p = pos[f + k];
    const double ms = amass[f + k];
    x = x + ms * p.x;
    y = y + ms * p.y;
    z = z + ms * p.z;
  }
  x = x / summ;
  y = y / summ;
  z = z / summ;
  double xw = x, yw = y, zw = z;
  pbc_com(xw, yw, zw, bx, by, bz, mc);
  X[m] = xw;
  Y[m] = yw;
  Z[m] = zw;
  // the reference rebuilds every coordinate as (S - X) + Xw (service.f:549-552)
  // the fixed-point y word has period 2 BOYL in the hexagonal cell
  const double two32 = 4294967296.0, ibx = 1.0 / bx, ibz = 1.0 / bz;
  const double iby = mc.cell.icell == 2 ? 0.5 / by : 1.0 / by;
  for (int k = 0; k < na; ++k) {
    dbl4 p = pos[f + k];
    p.x = (p.x - x) + xw;
    p.y = (p.y - y) + yw;
    p.z = (p.z - z) + zw;
    pos[f + k] = p;
    if (posi) {
      const long long xi = __double2ll_rn(p.x * ibx * two32);
      const long long yi = __double2ll_rn(p.y * iby * two32);
      const long long zi = __double2ll_rn(p.z * ibz * two32);
      posi[f + k] = make_int4((int)(unsigned)(unsigned long long)xi,
                              (int)(unsigned)(unsigned long long)yi,
                              (int)(unsigned)(unsigned long long)zi, pinfo[f + k]);
    }
  }
}

// ------------------------------------------------------------ kick/drift
struct MoveConst {
  int lmove[MDX_NT];
};

// bx set: a second kick with h2 right after (the same values as two passes)
__global__ void k_kick(int n, const int4 *__restrict__ ainfo, MoveConst mv,
                       double h, const double *__restrict__ ax,
                       const double *__restrict__ ay, const double *__restrict__ az,
                       double *vx, double *vy, double *vz,
                       const double *__restrict__ vscale, double h2 = 0.0,
                       const double *__restrict__ bx = nullptr,
                       const double *__restrict__ by = nullptr,
                       const double *__restrict__ bz = nullptr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int t = ainfo[i].x;
  if (!mv.lmove[t]) return;
  double x = vx[i], y = vy[i], z = vz[i];
  if (vscale) {  // thermostat factor of SCALING applied first (mdstep.f:818-828)
    const double s = vscale[t];
    x = x * s;
    y = y * s;
    z = z * s;
  }
  x = x + h * ax[i];
  y = y + h * ay[i];
  z = z + h * az[i];
  if (bx) {
    x = x + h2 * bx[i];
    y = y + h2 * by[i];
    z = z + h2 * bz[i];
  }
  vx[i] = x;
  vy[i] = y;
  vz[i] = z;
}

// DOUBLE 2.3.5.3-2.3.5.4 (mdstep.f:366-373), optionally preceded by the
// closing fast half-kick of the previous short step (mdstep.f:407-409).
__global__ void k_kick_drift(int n, const int4 *__restrict__ ainfo, MoveConst mv,
                             double htsteb, double tsteb, int prev,
                             const double *__restrict__ hx,
                             const double *__restrict__ hy,
                             const double *__restrict__ hz,
                             const double *__restrict__ massdi, double *vx,
                             double *vy, double *vz, dbl4 *pos) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!mv.lmove[ainfo[i].x]) return;
  double x = vx[i], y = vy[i], z = vz[i];
  const double fx = hx[i], fy = hy[i], fz = hz[i];
  if (prev) {
    x = x + htsteb * fx;
    y = y + htsteb * fy;
    z = z + htsteb * fz;
  }
  x = x + htsteb * fx;
  y = y + htsteb * fy;
  z = z + htsteb * fz;
  vx[i] = x;
  vy[i] = y;
  vz[i] = z;
  dbl4 p = pos[i];
  const double mi = massdi[i];
  p.x = x * tsteb * mi + p.x;
  p.y = y * tsteb * mi + p.y;
  p.z = z * tsteb * mi + p.z;
  pos[i] = p;
}

constexpr int KD_MAXA = 4;  // atoms per molecule of the register path below

// One short step of DOUBLE's inner loop up to the fast forces, thread per
// molecule: the kick and drift of k_kick_drift for each of its atoms
// (mdstep.f:383-397), then GETCOM's centre of mass and wrap (service.f:
// 463-563) and the fixed-point mirror, all in the order the separate
// kernels use.  hfix (mixed path): the previous short step's fast forces are read
// as fixed point, so that step needs no fold to FP64.
__device__ __forceinline__ void kick_drift_com_body(int m, int nop, const int *__restrict__ mol_first,
                                 const int *__restrict__ mol_nat,
                                 const int *__restrict__ mol_type,
                                 const int4 *__restrict__ ainfo, MoveConst mv,
                                 MolConst mc, double htsteb, double tsteb, int prev,
                                 const double *__restrict__ hx, const double *__restrict__ hy,
                                 const double *__restrict__ hz,
                                 const unsigned long long *__restrict__ hfix, int n,
                                 double inv, const double *__restrict__ massdi,
                                 const double *__restrict__ amass, double *__restrict__ vx,
                                 double *__restrict__ vy, double *__restrict__ vz,
                                 dbl4 *__restrict__ pos, double *__restrict__ X,
                                 double *__restrict__ Y, double *__restrict__ Z,
                                 double bx, double by, double bz, double3 ibs,
                                 int4 *__restrict__ posi, const int *__restrict__ pinfo,
                                 int4 *__restrict__ posc, const int *__restrict__ slot_of) {
  // ibs: 2^32 / box per axis (host-computed: no FP64 division per thread);
  // posi set (mixed path): centre of mass by the reciprocal mass, the
  // fixed-point mirror refreshed, and (posc set) its cell-order copy
  if (m >= nop) return;
  const int f = mol_first[m], na = mol_nat[m];
  if (posi && na <= KD_MAXA) {
    // Mixed path, small molecules: the atoms stay in registers between the
    // centre of mass and the wrap, each position is stored once, and the
    // update takes fewer FP64 operations (the two half kicks of one force
    // as one, 1/2^k folded into the kick factor, the drift factor TSTEB /
    // m formed once per atom, coordinates rebuilt around the wrapped centre
    // only when it moved).  The same update up to FP64 rounding.
    const double hk = prev ? 2.0 * htsteb : htsteb, hkf = hk * inv;
    dbl4 pr[KD_MAXA];
    double x = 0., y = 0., z = 0.;
#pragma unroll
    for (int k = 0; k < KD_MAXA; ++k) {
      if (k < na) {
        const int i = f + k;
        dbl4 p = pos[i];
        if (mv.lmove[ainfo[i].x]) {
          double u = vx[i], v = vy[i], w = vz[i];
          if (hfix) {
            u = fma((double)(long long)hfix[i], hkf, u);
            v = fma((double)(long long)hfix[n + i], hkf, v);
            w = fma((double)(long long)hfix[2 * n + i], hkf, w);
          } else {
            u = fma(hx[i], hk, u);
            v = fma(hy[i], hk, v);
            w = fma(hz[i], hk, w);
          }
          vx[i] = u;
          vy[i] = v;
          vz[i] = w;
          const double tm = tsteb * massdi[i];
          p.x = fma(u, tm, p.x);
          p.y = fma(v, tm, p.y);
          p.z = fma(w, tm, p.z);
        }
        pr[k] = p;
        const double ms = amass[i];
        x = fma(ms, p.x, x);
        y = fma(ms, p.y, y);
        z = fma(ms, p.z, z);
      }
    }
    const double rs = mc.rsummas[mol_type[m]];
    x = x * rs;
    y = y * rs;
    z = z * rs;
    double xw = x, yw = y, zw = z;
    pbc_com(xw, yw, zw, bx, by, bz, mc);
    X[m] = xw;
    Y[m] = yw;
    Z[m] = zw;
    const bool moved = xw != x || yw != y || zw != z;
#pragma unroll
    for (int k = 0; k < KD_MAXA; ++k) {
      if (k < na) {
        dbl4 p = pr[k];
        if (moved) {
          p.x = (p.x - x) + xw;
          p.y = (p.y - y) + yw;
          p.z = (p.z - z) + zw;
        }
        pos[f + k] = p;
        const int4 q =
            make_int4(fix32_rn(__dmul_rn(p.x, ibs.x)), fix32_rn(__dmul_rn(p.y, ibs.y)),
                      fix32_rn(__dmul_rn(p.z, ibs.z)), pinfo[f + k]);
        posi[f + k] = q;
        if (posc) posc[slot_of[f + k]] = q;
      }
    }
    return;
  }
  double x = 0., y = 0., z = 0.;
  for (int k = 0; k < na; ++k) {
    const int i = f + k;
    dbl4 p = pos[i];
    if (mv.lmove[ainfo[i].x]) {
      double u = vx[i], v = vy[i], w = vz[i];
      double fx, fy, fz;
      if (hfix) {
        fx = (double)(long long)hfix[i] * inv;
        fy = (double)(long long)hfix[n + i] * inv;
        fz = (double)(long long)hfix[2 * n + i] * inv;
      } else {
        fx = hx[i];
        fy = hy[i];
        fz = hz[i];
      }
      if (prev) {
        u = u + htsteb * fx;
        v = v + htsteb * fy;
        w = w + htsteb * fz;
      }
      u = u + htsteb * fx;
      v = v + htsteb * fy;
      w = w + htsteb * fz;
      vx[i] = u;
      vy[i] = v;
      vz[i] = w;
      const double mi = massdi[i];
      p.x = u * tsteb * mi + p.x;
      p.y = v * tsteb * mi + p.y;
      p.z = w * tsteb * mi + p.z;
    }
    pos[i] = p;
    const double ms = amass[i];
    x = x + ms * p.x;
    y = y + ms * p.y;
    z = z + ms * p.z;
  }
  if (posi) {
    const double rs = mc.rsummas[mol_type[m]];
    x = x * rs;
    y = y * rs;
    z = z * rs;
  } else {
    const double summ = mc.summas[mol_type[m]];
    x = x / summ;
    y = y / summ;
    z = z / summ;
  }
  double xw = x, yw = y, zw = z;
  pbc_com(xw, yw, zw, bx, by, bz, mc);
  X[m] = xw;
  Y[m] = yw;
  Z[m] = zw;
  for (int k = 0; k < na; ++k) {
    dbl4 p = pos[f + k];
    p.x = (p.x - x) + xw;
    p.y = (p.y - y) + yw;
    p.z = (p.z - z) + zw;
    pos[f + k] = p;
    if (posi) {
      const int4 q = make_int4(fix32_rn(__dmul_rn(p.x, ibs.x)), fix32_rn(__dmul_rn(p.y, ibs.y)),
                               fix32_rn(__dmul_rn(p.z, ibs.z)), pinfo[f + k]);
      posi[f + k] = q;
      if (posc) posc[slot_of[f + k]] = q;
    }
  }
}

__global__ void k_kick_drift_com(int nop, const int *__restrict__ mol_first,
                                 const int *__restrict__ mol_nat,
                                 const int *__restrict__ mol_type,
                                 const int4 *__restrict__ ainfo, MoveConst mv,
                                 MolConst mc, double htsteb, double tsteb, int prev,
                                 const double *__restrict__ hx, const double *__restrict__ hy,
                                 const double *__restrict__ hz,
                                 const unsigned long long *__restrict__ hfix, int n,
                                 double inv, const double *__restrict__ massdi,
                                 const double *__restrict__ amass, double *__restrict__ vx,
                                 double *__restrict__ vy, double *__restrict__ vz,
                                 dbl4 *__restrict__ pos, double *__restrict__ X,
                                 double *__restrict__ Y, double *__restrict__ Z,
                                 double bx, double by, double bz, double3 ibs,
                                 int4 *__restrict__ posi, const int *__restrict__ pinfo,
                                 int4 *__restrict__ posc, const int *__restrict__ slot_of) {
  kick_drift_com_body(blockIdx.x * blockDim.x + threadIdx.x, nop, mol_first, mol_nat, mol_type,
                      ainfo, mv, mc, htsteb, tsteb, prev, hx, hy, hz, hfix, n, inv, massdi,
                      amass, vx, vy, vz, pos, X, Y, Z, bx, by, bz, ibs, posi, pinfo, posc,
                      slot_of);
}

// SULTAN 1.3.1-1.3.2.2 (mdstep.f:89-113): OX = SX, V += TSTEP F,
// SX += TSTEP V MASSDI.
// save != 0: the new positions also go to fx/fy/fz (SHEJK's copy of the
// unconstrained positions, mdstep.f:1128-1132; the forces are not needed
// again before the next ALLFORCE).
__global__ void k_leapfrog(int n, const int4 *__restrict__ ainfo, MoveConst mv,
                           double tstep, double *fx, double *fy, double *fz,
                           const double *__restrict__ massdi, double *vx,
                           double *vy, double *vz, dbl4 *pos, double *ox,
                           double *oy, double *oz, int save) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!mv.lmove[ainfo[i].x]) return;
  dbl4 p = pos[i];
  ox[i] = p.x;
  oy[i] = p.y;
  oz[i] = p.z;
  const double x = vx[i] + tstep * fx[i];
  const double y = vy[i] + tstep * fy[i];
  const double z = vz[i] + tstep * fz[i];
  vx[i] = x;
  vy[i] = y;
  vz[i] = z;
  const double mi = massdi[i];
  p.x = p.x + tstep * x * mi;
  p.y = p.y + tstep * y * mi;
  p.z = p.z + tstep * z * mi;
  pos[i] = p;
  if (save) {
    fx[i] = p.x;
    fy[i] = p.y;
    fz[i] = p.z;
  }
}

// ------------------------------------------------------------------ GETEMP
// ekin layout as the reference's EKIN: [0..ntypes-1] per type, then total,
// VIRKX, VIRKY, VIRKZ.
// NT >= ntypes: per-type sums carried (NT + 4 values reduced; the unused
// types of ekacc are left alone).  R = float (mixed path): the per-atom
// terms and the warp sums in FP32 (a few atoms a thread, 32 threads a warp),
// the block and grid sums in FP64.
// KICK: a half kick folded into the pass, before the kinetic energy is taken
// (pre) and/or after it (post): V += h1 A (+ h2 B) for the movable atoms,
// the operations of k_kick in the same order, so the pass gives the values
// of kick, GETEMP, kick launched one after the other.
// vs (pre only): SCALING's per-type velocity factor applied first, as
// k_scale_atoms (mode 0) and k_kick do.
struct KickArgs {
  double h1, h2;
  const double *ax, *ay, *az;  // null: no kick
  const double *bx, *by, *bz;  // null: one force only
  const double *vs;            // null: no velocity factor
};

__device__ __forceinline__ void kick_atom(const KickArgs &k, int i, double &x, double &y,
                                          double &z) {
  if (!k.ax) return;
  x = x + k.h1 * k.ax[i];
  y = y + k.h1 * k.ay[i];
  z = z + k.h1 * k.az[i];
  if (k.bx) {
    x = x + k.h2 * k.bx[i];
    y = y + k.h2 * k.by[i];
    z = z + k.h2 * k.bz[i];
  }
}

template <int NT, typename R, bool KICK, bool ROW>
__device__ __forceinline__ void getemp_body(int n, const int4 *__restrict__ ainfo,
                                            const MoveConst &mv, int ntypes,
                                            const double *__restrict__ massdi, double *vx,
                                            double *vy, double *vz, double *ekacc, double *part,
                                            unsigned *ctr, const KickArgs &pre,
                                            const KickArgs &post) {
  R e[NT + 4];
#pragma unroll
  for (int k = 0; k < NT + 4; ++k) e[k] = R(0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const int t = ainfo[i].x;
    if (!mv.lmove[t]) continue;
    double px = vx[i], py = vy[i], pz = vz[i];
    if (KICK && pre.vs) {
      const double f = pre.vs[t];
      px = px * f;
      py = py * f;
      pz = pz * f;
    }
    if (KICK) kick_atom(pre, i, px, py, pz);
    const R m = (R)massdi[i], ux = (R)px, uy = (R)py, uz = (R)pz;
    const R VVX = m * (ux * ux);
    const R VVY = m * (uy * uy);
    const R VVZ = m * (uz * uz);
    const R VSC = VVX + VVY + VVZ;
    e[NT + 1] += VVX;
    e[NT + 2] += VVY;
    e[NT + 3] += VVZ;
    e[NT] += VSC;
#pragma unroll
    for (int k = 0; k < NT; ++k)
      if (k == t) e[k] += R(0.5) * VSC;
    if (KICK) {
      kick_atom(post, i, px, py, pz);
      vx[i] = px;
      vy[i] = py;
      vz[i] = pz;
    }
  }
  // value k < NT -> ekacc[k] (type k), NT + j -> ekacc[MDX_NT + j]
  double *dst[NT + 4];
#pragma unroll
  for (int k = 0; k < NT + 4; ++k)
    dst[k] = k < NT ? (k < ntypes ? ekacc + k : nullptr) : ekacc + MDX_NT + (k - NT);
  double ed[NT + 4];
  if (sizeof(R) == sizeof(double)) {
#pragma unroll
    for (int k = 0; k < NT + 4; ++k) ed[k] = (double)e[k];
    block_add_core<NT + 4, false, ROW>(ed, dst, part, ctr);
  } else {
#pragma unroll
    for (int k = 0; k < NT + 4; ++k) ed[k] = (double)warp_sumf((float)e[k]);
    block_add_core<NT + 4, true, ROW>(ed, dst, part, ctr);
  }
}

template <int NT, typename R, bool KICK>
__global__ void k_getemp(int n, const int4 *__restrict__ ainfo, MoveConst mv,
                         int ntypes, const double *__restrict__ massdi,
                         double *vx, double *vy, double *vz, double *ekacc,
                         double *part, unsigned *ctr, KickArgs pre, KickArgs post) {
  getemp_body<NT, R, KICK, false>(n, ainfo, mv, ntypes, massdi, vx, vy, vz, ekacc, part, ctr,
                                  pre, post);
}

// Device scratch of SCALING between stages.
struct ScalScratch {
  double dpe[5];
  double dke;
  double dte[MDX_NT];
  double vscale[MDX_NT];  // per-type velocity factor of the next kick
  double scvx, scvy, scvz, drcx, drcy, drcz, drcv, dxc;
  double ekacc[MDX_NT + 4];
  int iskk;
};

// The stages run on one thread, and an FP64 division there is a long
// dependent sequence on this GPU's FP64 pipe: the quotients of constants are
// formed on the host (rtrtemp = 1 / TRTEMP, tlow = TRTEMP / CHKTF, dqt_f =
// c.dqt_f, c3_fnst = 3 / FNST, c3_fnop = 3 / FNOP) and the pressure stage
// takes one reciprocal of VOL; the values equal the reference's divisions to
// rounding.
struct ScalConst {
  int ntypes, lnvt, lnpt, lsep, lsctd, lp_xy, lshejk, lsclt, icell;
  double tstep, htstep, trtemp, tdelt, trpres, trpresx, trpresy, trpresz, dqt,
      dqp, rtp, fnst, fnop, unitp, vird, tridm_coef, tridee_coef, convet, chktf;
  double rtrtemp, tlow, dqt_f, c3_fnst, c3_fnop, rfnst;
  double tfact[MDX_NT];
  int lmove[MDX_NT];
};

// GETEMP finalisation (service.f:63-80) from the block sums.
__device__ void getemp_fold(const ScalConst &c, ScalScratch *ss, mdx_thermo *th,
                            int *err) {
  const int nt = c.ntypes;
  for (int t = 0; t < nt; ++t) th->ekin[t] = ss->ekacc[t];
  // TEMPR(NTYP1) = 0.5*VSQ
  const double tke = 0.5 * ss->ekacc[MDX_NT];
  th->ekin[nt] = tke;
  th->ekin[nt + 1] = ss->ekacc[MDX_NT + 1];
  th->ekin[nt + 2] = ss->ekacc[MDX_NT + 2];
  th->ekin[nt + 3] = ss->ekacc[MDX_NT + 3];
  th->tke = tke;
  th->virkx = th->ekin[nt + 1];
  th->virky = th->ekin[nt + 2];
  th->virkz = th->ekin[nt + 3];
  for (int t = 0; t < nt + 4; ++t) th->tempr[t] = th->ekin[t];
  for (int t = 0; t < nt; ++t) th->tempr[t] = th->ekin[t] * c.tfact[t];
  th->temp = th->tke * c.convet;
  for (int k = 0; k < MDX_NT + 4; ++k) ss->ekacc[k] = 0.0;
  if (c.chktf > 0.0 && (th->temp > c.chktf * c.trtemp || th->temp <= c.tlow))
    atomicOr(err, DERR_TEMP);
  if (!(th->temp == th->temp)) atomicOr(err, DERR_NAN);
}

__device__ void npt_guard(ScalScratch *ss, mdx_thermo *th, double f, int *err) {
  if (fabs(f) >= 0.1) {
    th->npt_fail += 1;
    if (th->npt_fail > 100) atomicOr(err, DERR_NPT);
  }
}

// Stage codes of the SCALING sequence.
enum {
  ST_GETEMP = 1,   // fold GETEMP
  ST_PRESS,        // 3.3.2-3.3.3 pressures and deviations
  ST_1A,           // IAL=1: 3.4.1 + 3.4.2.1-3.4.2.3
  ST_1NVT,         // IAL=1 NVT velocity factor (3.4.3)
  ST_1RECLEN,      // IAL=1 NPT box
  ST_EABS,         // 3.4.4 / 3.5.7 / 3.6.4
  ST_2V,           // IAL=2 3.5.1 factor
  ST_2NPTV,        // IAL=2 3.5.2 factor
  ST_2SCL,         // IAL=2 3.5.4-3.5.5
  ST_2SC,          // IAL=2 3.5.6
  ST_3V,           // IAL=3 3.2 factor
  ST_3A,           // IAL=3 3.6.1-3.6.2.3
  ST_3B,           // IAL=3 3.6.2.5-3.6.2.6 (box, SC)
  ST_SCLT,         // 3.7 factor
  ST_MSTEP1,       // SULTAN first step correction factor (mdstep.f:131-139)
};

// RECLEN (service.f:572-605): the hexagonal cell keeps BOYL = BOXL cos30,
// the truncated octahedron a cube of the mean factor and half its volume.
__device__ void reclen_dev(mdx_thermo *th, double sx, double sy, double sz, int icell) {
  th->boxl = sx * th->boxl;
  if (icell == 2) {
    th->boyl = th->boxl * (double)0.8660254037844386f;
    th->bozl = sz * th->bozl;
  } else if (icell == 1) {
    th->boxl = (sx + sy + sz) * th->boxl / (3. * sx);
    th->boyl = th->boxl;
    th->bozl = th->boxl;
  } else {
    th->boyl = sy * th->boyl;
    th->bozl = sz * th->bozl;
  }
  th->vol = th->boxl * th->boyl * th->bozl;
  if (icell == 1) th->vol = 0.5 * th->vol;
}

__device__ void scal_stage(int stage, const ScalConst &c, ScalScratch *ss, mdx_thermo *th,
                           const mdx_scalars *s, int *err) {
  const double TSTEP = c.tstep, HTSTEP = c.htstep, FNST = c.fnst;
  const double DQT = c.dqt, DQP = c.dqp, RTP = c.rtp;
  const double VOL = th->vol;
  switch (stage) {
    case ST_GETEMP:
      getemp_fold(c, ss, th, err);
      break;
    case ST_PRESS: {
      const double VIRSUM = s->vir1 + s->vir2 + s->virb + s->pels1 + s->pels2 + s->spe +
                            c.vird + th->vira[0] + th->vira[1] + th->vira[2];
      const double WIRSUM =
          s->vir1 + s->vir2 + s->pels1 + s->pels2 + s->spe + c.vird + s->wirs + s->wirss;
      const double RV = 1.0 / VOL, UPV = c.unitp * RV, UPV3 = UPV * (1.0 / 3.0);
      const double TRIDEE = c.tridee_coef * RV;
      const double TRIDEE3 = TRIDEE * (1.0 / 3.0), VIRD3 = c.vird * (1.0 / 3.0);
      const double TRID = 2. * th->tke * UPV3 - TRIDEE;
      const double TRIDM = c.tridm_coef * th->temp * RV - TRIDEE;
      const double TRIDX = th->virkx * UPV - TRIDEE3;
      const double TRIDY = th->virky * UPV - TRIDEE3;
      const double TRIDZ = th->virkz * UPV - TRIDEE3;
      th->tryck = VIRSUM * UPV3 + TRID;
      th->tryckm = WIRSUM * UPV3 + TRIDM;
      th->tryckx = (s->virx + s->virfx + VIRD3 + th->vira[0]) * UPV + TRIDX;
      th->trycky = (s->viry + s->virfy + VIRD3 + th->vira[1]) * UPV + TRIDY;
      th->tryckz = (s->virz + s->virfz + VIRD3 + th->vira[2]) * UPV + TRIDZ;
      ss->dke = th->temp * c.rtrtemp - 1.0;
      for (int t = 0; t < c.ntypes; ++t) ss->dte[t] = th->tempr[t] * c.rtrtemp - 1.0;
      if (s->lscfl) {
        for (int k = 1; k <= 4; ++k) ss->dpe[k] = 0.;
      } else {
        ss->dpe[1] = c.lshejk ? th->tryckm - c.trpres : th->tryck - c.trpres;
        ss->dpe[2] = th->tryckx - c.trpresx;
        ss->dpe[3] = th->trycky - c.trpresy;
        if (c.lp_xy) {
          ss->dpe[2] = 0.5 * (ss->dpe[2] + ss->dpe[3]);
          ss->dpe[3] = ss->dpe[2];
        }
        ss->dpe[4] = th->tryckz - c.trpresz;
      }
      break;
    }
    case ST_1A: {
      if (c.lsctd) {
        double SCA = 0.;
        for (int t = 0; t < c.ntypes; ++t) {
          th->scm[t] = th->scm[t] + ss->dte[t] * DQT * HTSTEP;
          SCA = SCA + th->scm[t] * th->ekin[t];
        }
        th->sc = SCA / th->tke;
      } else {
        th->sc = th->sc + ss->dke * DQT * HTSTEP;
      }
      if (c.lnpt) {
        if (c.lsctd) {
          double SCA = 0.;
          for (int t = 0; t < c.ntypes; ++t) {
            th->scm[t] = th->scm[t] + (th->scl * th->scl * RTP - c.dqt_f) * HTSTEP;
            SCA = SCA + th->scm[t] * th->ekin[t];
          }
          th->sc = SCA / th->tke;
        } else {
          th->sc = th->sc + (th->scl * th->scl * RTP - c.dqt_f) * HTSTEP;
        }
        const double *DPE = ss->dpe;
        if (c.lsep) {
          th->sclx = th->sclx + DQP * (VOL * DPE[2] + 2. * th->tke * c.rfnst - th->sclx * th->sc) * HTSTEP;
          th->scly = th->scly + DQP * (VOL * DPE[3] + 2. * th->tke * c.rfnst - th->scly * th->sc) * HTSTEP;
          if (c.lp_xy) {
            th->sclx = 0.5 * (th->sclx + th->scly);
            th->scly = th->sclx;
          }
          th->sclz = th->sclz + DQP * (VOL * DPE[4] + 2. * th->tke * c.rfnst - th->sclz * th->sc) * HTSTEP;
          th->scl = th->sclx + th->scly + th->sclz;
        } else {
          th->scl = th->scl + DQP * (3. * VOL * DPE[1] + 6. * th->tke * c.rfnst - th->scl * th->sc) * HTSTEP;
          th->sclx = th->scl;
          th->scly = th->scl;
          th->sclz = th->scl;
          npt_guard(ss, th, th->scl * HTSTEP, err);
        }
        double SCVX = 1. - ((1. - c.c3_fnst) * th->sclx + th->sc) * HTSTEP;
        double SCVY = 1. - ((1. - c.c3_fnst) * th->scly + th->sc) * HTSTEP;
        double SCVZ = 1. - ((1. - c.c3_fnst) * th->sclz + th->sc) * HTSTEP;
        if (c.lp_xy) {
          SCVX = 0.5 * (SCVX + SCVY);
          SCVY = SCVX;
        }
        double DRCX = TSTEP * th->sclx, DRCY = TSTEP * th->scly, DRCZ = TSTEP * th->sclz;
        const double DRC = (DRCX + DRCY + DRCZ) * (1.0 / 3.0);
        ss->drcv = DRC * HTSTEP;
        ss->drcx = 1. + DRCX + 0.5 * (DRCX * DRCX);
        ss->drcy = 1. + DRCY + 0.5 * (DRCY * DRCY);
        ss->drcz = 1. + DRCZ + 0.5 * (DRCZ * DRCZ);
        ss->scvx = SCVX;
        ss->scvy = SCVY;
        ss->scvz = SCVZ;
      }
      break;
    }
    case ST_1RECLEN:
      reclen_dev(th, ss->drcx, ss->drcy, ss->drcz, c.icell);
      break;
    case ST_1NVT:
    case ST_2V:
      for (int t = 0; t < MDX_NT; ++t)
        ss->vscale[t] = c.lsctd ? 1. - th->scm[t] * HTSTEP : 1. - th->sc * HTSTEP;
      break;
    case ST_3V:
      for (int t = 0; t < MDX_NT; ++t)
        ss->vscale[t] = c.lsctd ? 1. - th->scm[t] * TSTEP : 1. - th->sc * TSTEP;
      break;
    case ST_EABS:
      th->eabs = th->eabs - (th->sc + th->scl * (1. - c.c3_fnst)) * th->tke * TSTEP;
      break;
    case ST_2NPTV: {
      double SCVX = 1. - (1. - c.c3_fnop) * th->sclx * HTSTEP;
      double SCVY = 1. - (1. - c.c3_fnop) * th->scly * HTSTEP;
      double SCVZ = 1. - (1. - c.c3_fnop) * th->sclz * HTSTEP;
      if (c.lp_xy) {
        SCVX = 0.5 * (SCVX + SCVY);
        SCVY = SCVX;
      }
      ss->scvx = SCVX;
      ss->scvy = SCVY;
      ss->scvz = SCVZ;
      break;
    }
    case ST_2SCL: {
      const double *DPE = ss->dpe;
      if (c.lsep) {
        th->sclx = th->sclx + DQP * (VOL * DPE[2] + 2. * th->tke * c.rfnst - th->sclx * th->sc) * HTSTEP;
        th->scly = th->scly + DQP * (VOL * DPE[3] + 2. * th->tke * c.rfnst - th->scly * th->sc) * HTSTEP;
        if (c.lp_xy) {
          th->sclx = 0.5 * (th->sclx + th->scly);
          th->scly = th->sclx;
        }
        th->sclz = th->sclz + DQP * (VOL * DPE[4] + 2. * th->tke * c.rfnst - th->sclz * th->sc) * HTSTEP;
        th->scl = th->sclx + th->scly + th->sclz;
      } else {
        th->scl = th->scl + DQP * (3. * VOL * DPE[1] + 6. * th->tke * c.rfnst - th->scl * th->sc) * HTSTEP;
        th->sclx = th->scl;
        th->scly = th->scl;
        th->sclz = th->scl;
        npt_guard(ss, th, th->scl * HTSTEP, err);
      }
      th->sc = th->sc + (th->scl * th->scl * RTP - c.dqt_f) * HTSTEP;
      if (c.lsctd)
        for (int t = 0; t < c.ntypes; ++t)
          th->scm[t] = th->scm[t] + (th->scl * th->scl * RTP - c.dqt_f) * HTSTEP;
      break;
    }
    case ST_2SC: {
      if (c.lsctd) {
        double SCA = 0.;
        for (int t = 0; t < c.ntypes; ++t) {
          const double DTE = th->tempr[t] * c.rtrtemp - 1.0;
          th->scm[t] = th->scm[t] + DTE * DQT * HTSTEP;
          SCA = SCA + th->scm[t] * th->ekin[t];
        }
        th->sc = SCA / th->tke;
      } else {
        const double DKE = th->temp * c.rtrtemp - 1.0;
        th->sc = th->sc + DKE * DQT * HTSTEP;
      }
      th->eabs = th->eabs - (th->sc + th->scl * (1. - c.c3_fnst)) * th->tke * TSTEP;
      break;
    }
    case ST_3A: {
      th->sc = th->sc + ss->dke * DQT * TSTEP;
      if (c.lsctd) {
        double SCA = 0.;
        for (int t = 0; t < c.ntypes; ++t) {
          th->scm[t] = th->scm[t] + ss->dte[t] * DQT * TSTEP;
          SCA = SCA + th->scm[t] * th->ekin[t];
        }
        th->sc = SCA / th->tke;
      }
      if (c.lnpt) {
        const double *DPE = ss->dpe;
        if (c.lsep) {
          th->sclx = th->sclx + DQP * (VOL * DPE[2] + 2. * th->tke * c.rfnst - th->sclx * th->sc) * TSTEP;
          th->scly = th->scly + DQP * (VOL * DPE[3] + 2. * th->tke * c.rfnst - th->scly * th->sc) * TSTEP;
          if (c.lp_xy) {
            th->sclx = 0.5 * (th->sclx + th->scly);
            th->scly = th->sclx;
          }
          th->sclz = th->sclz + DQP * (VOL * DPE[4] + 2. * th->tke * c.rfnst - th->sclz * th->sc) * TSTEP;
          th->scl = th->sclx + th->scly + th->sclz;
        } else {
          th->scl = th->scl + DQP * (3. * VOL * DPE[1] + 6. * th->tke * c.rfnst - th->scl * th->sc) * TSTEP;
          th->sclx = th->scl;
          th->scly = th->scl;
          th->sclz = th->scl;
          npt_guard(ss, th, th->scl * TSTEP, err);
        }
        ss->dxc = ((1. - c.c3_fnst) * th->scl) * TSTEP;  // SCV of 3.6.2.2
        ss->drcx = TSTEP * th->sclx;
        ss->drcy = TSTEP * th->scly;
        ss->drcz = TSTEP * th->sclz;
      }
      break;
    }
    case ST_3B: {
      reclen_dev(th, ss->drcx + 1., ss->drcy + 1., ss->drcz + 1., c.icell);
      th->sc = th->sc + (th->scl * th->scl * RTP - c.dqt_f) * TSTEP;
      if (c.lsctd) {
        double SCA = 0.;
        for (int t = 0; t < c.ntypes; ++t) {
          th->scm[t] = th->scm[t] + (th->scl * th->scl * RTP - c.dqt_f) * TSTEP;
          SCA = SCA + th->scm[t] * th->ekin[t];
        }
        th->sc = SCA / th->tke;
      }
      break;
    }
    case ST_SCLT: {
      for (int t = 0; t < MDX_NT; ++t) ss->vscale[t] = 1.0;
      if (c.lsctd) {
        for (int t = 0; t < c.ntypes; ++t)
          if (fabs(c.trtemp - th->tempr[t]) > c.tdelt && c.lmove[t]) {
            ss->vscale[t] = sqrt(c.trtemp / th->tempr[t]);
            th->nscale += 1;
          }
      } else if (fabs(c.trtemp - th->temp) > c.tdelt) {
        const double SCV = sqrt(c.trtemp / th->temp);
        for (int t = 0; t < MDX_NT; ++t) ss->vscale[t] = SCV;
        th->nscale += 1;
      }
      break;
    }
    case ST_MSTEP1: {
      const double FTMP = sqrt(c.trtemp / th->temp);
      for (int t = 0; t < MDX_NT; ++t) ss->vscale[t] = FTMP;
      break;
    }
  }
}

// Several consecutive SCALING stages in one launch (one thread, in order:
// the same as one launch each).
struct StageList {
  int n;
  int st[8];
};
__device__ __forceinline__ void copy_words(void *dst, const void *src, int bytes) {
  int *d = static_cast<int *>(dst);
  const int *s = static_cast<const int *>(src);
  for (int k = threadIdx.x; k < bytes / 4; k += blockDim.x) d[k] = s[k];
}

// The stages are one serial chain of scalar arithmetic; from global memory
// each of its loads would be a round trip.  The block brings the scratch,
// the thermostat state and the scalars into shared memory at once, thread 0
// runs the stages there, and the block writes the first two back.
__device__ __forceinline__ void scal_list_body(const StageList &L, const ScalConst &c,
                                               ScalScratch *ss, mdx_thermo *th,
                                               const mdx_scalars *s, int *err) {
  __shared__ ScalScratch ss_s;
  __shared__ mdx_thermo th_s;
  __shared__ mdx_scalars s_s;
  static_assert(sizeof(ScalScratch) % 4 == 0 && sizeof(mdx_thermo) % 4 == 0 &&
                    sizeof(mdx_scalars) % 4 == 0,
                "word copies");
  copy_words(&ss_s, ss, sizeof(ScalScratch));
  copy_words(&th_s, th, sizeof(mdx_thermo));
  copy_words(&s_s, s, sizeof(mdx_scalars));
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < L.n; ++k) scal_stage(L.st[k], c, &ss_s, &th_s, &s_s, err);
  __syncthreads();
  copy_words(ss, &ss_s, sizeof(ScalScratch));
  copy_words(th, &th_s, sizeof(mdx_thermo));
}

__global__ void k_scal_list(StageList L, ScalConst c, ScalScratch *ss, mdx_thermo *th,
                            const mdx_scalars *s, int *err) {
  scal_list_body(L, c, ss, th, s, err);
}

// ------------------------------------------------ bead ensembles (PIMD) ---
// The integrator passes of every bead of a PIMD ensemble in one launch each:
// grid row blockIdx.y (the stage blocks: blockIdx.x) is the bead, its arrays
// come from a device table.  A bead's blocks, per-atom operations and sums
// are those of the single-context launches, so the values are the same.
struct BeadMove {
  dbl4 *pos;
  double *vx, *vy, *vz;
  const double *f[3][3];  // forces H, G, F; x, y, z
  double *X, *Y, *Z;
  int4 *posi, *posc;
  const int *slot_of;
  double *part;
  unsigned *ctr;
  ScalScratch *ss;
  mdx_thermo *th;
  const mdx_scalars *sc;
  int *err;
};

struct KickW {  // KickSpec by force index, resolved per bead on the device
  int w1, w2, vs;
  double h1, h2;
};

__device__ __forceinline__ KickArgs bead_kick(const BeadMove &b, const KickW &k) {
  KickArgs a{};
  a.h1 = k.h1;
  a.h2 = k.h2;
  if (k.w1) {
    a.ax = b.f[k.w1 - 1][0];
    a.ay = b.f[k.w1 - 1][1];
    a.az = b.f[k.w1 - 1][2];
  }
  if (k.w2) {
    a.bx = b.f[k.w2 - 1][0];
    a.by = b.f[k.w2 - 1][1];
    a.bz = b.f[k.w2 - 1][2];
  }
  a.vs = k.vs ? b.ss->vscale : nullptr;
  return a;
}

template <int NT, typename R, bool KICK>
__global__ void k_getemp_beads(int n, const int4 *__restrict__ ainfo, MoveConst mv, int ntypes,
                               const double *__restrict__ massdi,
                               const BeadMove *__restrict__ beads, KickW pre, KickW post) {
  const BeadMove &b = beads[blockIdx.y];
  const KickArgs a = bead_kick(b, pre), c = bead_kick(b, post);
  getemp_body<NT, R, KICK, true>(n, ainfo, mv, ntypes, massdi, b.vx, b.vy, b.vz, b.ss->ekacc,
                                 b.part, b.ctr, a, c);
}

__global__ void k_scal_list_beads(StageList L, ScalConst c, const BeadMove *__restrict__ beads) {
  const BeadMove &b = beads[blockIdx.x];
  scal_list_body(L, c, b.ss, b.th, b.sc, b.err);
}

// Velocity (and position) scaling of the SCALING stages.
// mode 0: V *= vscale[type] (LMOVE atoms); mode 1: all atoms (SULTAN first
// step); mode 2: IAL=1 NPT (V *= SCV?, S = S*DRC? + V*DRCV*MASSDI);
// mode 3: IAL=2 NPT V *= SCV?.
__global__ void k_scale_atoms(int n, int mode, const int4 *__restrict__ ainfo,
                              MoveConst mv, const ScalScratch *ss,
                              const double *__restrict__ massdi, double *vx,
                              double *vy, double *vz, dbl4 *pos) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int t = ainfo[i].x;
  if (mode != 1 && !mv.lmove[t]) return;
  if (mode <= 1) {
    const double s = ss->vscale[t];
    vx[i] = vx[i] * s;
    vy[i] = vy[i] * s;
    vz[i] = vz[i] * s;
  } else {
    const double x = vx[i] * ss->scvx, y = vy[i] * ss->scvy, z = vz[i] * ss->scvz;
    vx[i] = x;
    vy[i] = y;
    vz[i] = z;
    if (mode == 2) {
      dbl4 p = pos[i];
      const double mi = massdi[i];
      p.x = p.x * ss->drcx + x * ss->drcv * mi;
      p.y = p.y * ss->drcy + y * ss->drcv * mi;
      p.z = p.z * ss->drcz + z * ss->drcv * mi;
      pos[i] = p;
    }
  }
}

// SCALING(3) NPT molecular correction (mdstep.f:953-1003): per molecule.
__global__ void k_com_scale(int nop, const int *__restrict__ mol_first,
                            const int *__restrict__ mol_nat,
                            const int *__restrict__ mol_type,
                            const double *__restrict__ amass, MolConst mc,
                            MoveConst mv, const ScalScratch *ss, double *vx,
                            double *vy, double *vz, dbl4 *pos) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nop) return;
  const int t = mol_type[m];
  if (!mv.lmove[t]) return;
  const int f = mol_first[m], na = mol_nat[m];
  const double SUMM = mc.summas[t];
  double XC = 0., YC = 0., ZC = 0., PXC = 0., PYC = 0., PZC = 0.;
  for (int k = 0; k < na; ++k) {
    const dbl4 p = pos[f + k];
    const double ms = amass[f + k];
    XC = XC + ms * p.x;
    YC = YC + ms * p.y;
    ZC = ZC + ms * p.z;
    PXC = PXC + vx[f + k];
    PYC = PYC + vy[f + k];
    PZC = PZC + vz[f + k];
  }
  XC = XC / SUMM;
  YC = YC / SUMM;
  ZC = ZC / SUMM;
  const double SCV = ss->dxc;
  const double DVX = PXC * SCV, DVY = PYC * SCV, DVZ = PZC * SCV;
  const double DXC = XC * ss->drcx, DYC = YC * ss->drcy, DZC = ZC * ss->drcz;
  for (int k = 0; k < na; ++k) {
    const double FAC = amass[f + k] / SUMM;
    vx[f + k] = vx[f + k] - DVX * FAC;
    vy[f + k] = vy[f + k] - DVY * FAC;
    vz[f + k] = vz[f + k] - DVZ * FAC;
    dbl4 p = pos[f + k];
    p.x = p.x + DXC;
    p.y = p.y + DYC;
    p.z = p.z + DZC;
    pos[f + k] = p;
  }
}

// ------------------------------------------------------------------ SHEJK
struct ShakeConst {
  int iadb[MDX_NT], nrb[MDX_NT], ishejk[MDX_NT];
  int maxit;
  double tol2, tstep;
  CellPbc cell;
};

// SHEJK (mdstep.f:1105-1283) over independent constraint clusters.  The
// reference sweeps all constraints of a molecule in record order until no
// bond needs adjusting; constraints that share no atom (e.g. the CH2 and CH3
// groups of a lipid under SHAKE on bonds to hydrogen) never see each
// other's updates, so each cluster runs the same sweeps on its own and ends
// in the same positions bit for bit; the molecule's iteration count is the
// largest of its clusters'.  Thread per (molecule, cluster); the positions
// before SHAKE are in fx/fy/fz (written by the leap-frog pass).
__global__ void k_shake_cluster(int nitem, const int2 *__restrict__ items,
                                const int2 *__restrict__ clusters,
                                const int *__restrict__ recs,
                                const int *__restrict__ mol_first,
                                const int *__restrict__ mol_type, MoveConst mv,
                                ShakeConst sk, const int *__restrict__ bib,
                                const int *__restrict__ bjb,
                                const double *__restrict__ brb,
                                const double *__restrict__ massdi, dbl4 *pos,
                                const double *__restrict__ ox,
                                const double *__restrict__ oy,
                                const double *__restrict__ oz, double bx, double by,
                                double bz, mdx_thermo *th, int *__restrict__ mfail) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nitem) return;
  const int2 item = items[it];
  const int m = item.x, t = mol_type[m];
  if (!(mv.lmove[t] && sk.ishejk[t] > 0)) return;
  const int2 cl = clusters[item.y];  // (first record slot, records)
  const int *rr = recs + cl.x;
  const int f = mol_first[m];
  // MOVING / MOVED flags as bit masks over the molecule's atoms (<= 128)
  unsigned long long moving[2] = {0, 0}, moved[2] = {0, 0};
  for (int q = 0; q < cl.y; ++q) {
    const int b = rr[q];
    const int li = bib[b] - 1, lj = bjb[b] - 1;
    moved[li >> 6] |= 1ull << (li & 63);
    moved[lj >> 6] |= 1ull << (lj & 63);
  }
  int ITER = 0;
  bool DONE = false;
  for (;;) {
    if (ITER > sk.maxit || DONE) break;
    DONE = true;
    for (int q = 0; q < cl.y; ++q) {
      const int b = rr[q];
      const int li = bib[b] - 1, lj = bjb[b] - 1;
      const bool mvi = (moved[li >> 6] >> (li & 63)) & 1ull;
      const bool mvj = (moved[lj >> 6] >> (lj & 63)) & 1ull;
      if (!(mvi || mvj)) continue;
      const int I = f + li, J = f + lj;
      const double rbb = brb[b];
      const double BNDSQ = rbb * rbb;
      dbl4 pi = pos[I], pj = pos[J];
      double BXN = pi.x - pj.x, BYN = pi.y - pj.y, BZN = pi.z - pj.z;
      if (sk.cell.icell == 0) pbc_rect(BXN, BYN, BZN, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
      else pbc_cell(BXN, BYN, BZN, sk.cell);  // mdstep.f:1175
      const double BSQ = BXN * BXN + BYN * BYN + BZN * BZN;
      const double DIFFSQ = BNDSQ - BSQ;
      if (fabs(DIFFSQ) > (BNDSQ * sk.tol2)) {
        double DXN = ox[I] - ox[J], DYN = oy[I] - oy[J], DZN = oz[I] - oz[J];
        if (sk.cell.icell == 0) pbc_rect(DXN, DYN, DZN, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
        else pbc_cell(DXN, DYN, DZN, sk.cell);  // mdstep.f:1186
        const double VDOT = BXN * DXN + BYN * DYN + BZN * DZN;
        const double RMA = massdi[I], RMB = massdi[J];
        const double GAB = DIFFSQ / (2.0 * (RMA + RMB) * VDOT);
        DXN = DXN * GAB;
        DYN = DYN * GAB;
        DZN = DZN * GAB;
        pi.x = pi.x + RMA * DXN;
        pi.y = pi.y + RMA * DYN;
        pi.z = pi.z + RMA * DZN;
        pj.x = pj.x - RMB * DXN;
        pj.y = pj.y - RMB * DYN;
        pj.z = pj.z - RMB * DZN;
        pos[I] = pi;
        pos[J] = pj;
        moving[li >> 6] |= 1ull << (li & 63);
        moving[lj >> 6] |= 1ull << (lj & 63);
        DONE = false;
      }
    }
    // MOVED := MOVING restricted to constrained atoms; MOVING := 0
    moved[0] = moving[0];
    moved[1] = moving[1];
    moving[0] = moving[1] = 0;
    ITER = ITER + 1;
  }
  atomicMax(&th->shake_iter_max, ITER);
  if (ITER >= sk.maxit) mfail[m] = 1;
}

// SHEJK's end per molecule (mdstep.f:1240-1275): velocity correction and
// constraint virial from the displacement SHAKE made, the count of
// molecules past MAXIT.  Thread per molecule (the virial sums in molecule
// order).
__global__ void k_shake_finish(int nop, const int *__restrict__ mol_first,
                               const int *__restrict__ mol_nat,
                               const int *__restrict__ mol_type, MoveConst mv,
                               ShakeConst sk, const double *__restrict__ massdi,
                               const dbl4 *__restrict__ pos, double *vx, double *vy,
                               double *vz, const double *__restrict__ ox,
                               const double *__restrict__ oy,
                               const double *__restrict__ oz, const double *__restrict__ fx,
                               const double *__restrict__ fy,
                               const double *__restrict__ fz, mdx_thermo *th, int *err,
                               int *__restrict__ mfail, Dst6 vdst) {
  double vir[3] = {0, 0, 0};
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < nop) {
    const int t = mol_type[m];
    if (mv.lmove[t] && sk.ishejk[t] > 0 && sk.nrb[t] > 0) {
      if (mfail[m]) {
        mfail[m] = 0;
        atomicAdd(&th->shake_fail, 1);
        atomicOr(err, DERR_SHAKE);
      }
      const int f = mol_first[m], na = mol_nat[m];
      const double TS = sk.tstep;
      for (int k = 0; k < na; ++k) {
        const int I = f + k;
        const dbl4 p = pos[I];
        const double DIX = (p.x - fx[I]) / (massdi[I] * TS);
        const double DIY = (p.y - fy[I]) / (massdi[I] * TS);
        const double DIZ = (p.z - fz[I]) / (massdi[I] * TS);
        vir[0] += DIX * ox[I] / TS;
        vir[1] += DIY * oy[I] / TS;
        vir[2] += DIZ * oz[I] / TS;
        vx[I] = vx[I] + DIX;
        vy[I] = vy[I] + DIY;
        vz[I] = vz[I] + DIZ;
      }
    }
  }
  block_add<3>(vir, vdst);
}

__global__ void k_shake_prep(mdx_thermo *th) {
  th->viran[0] = th->viran[1] = th->viran[2] = 0.0;
  th->shake_iter_max = 0;
}
__global__ void k_vira_from_viran(mdx_thermo *th) {
  th->vira[0] = th->viran[0];
  th->vira[1] = th->viran[1];
  th->vira[2] = th->viran[2];
}
__global__ void k_vira_zero(mdx_thermo *th) {
  th->vira[0] = th->vira[1] = th->vira[2] = 0.0;
}

// ------------------------------------------------------------------ record
__global__ void k_record(mdx_step_record *rec, int slot, int mstep,
                         const mdx_scalars *s, const mdx_thermo *th, int *ctr,
                         int cap) {
  if (ctr) {  // graph replay: slot and step number come from device counters
    slot = ctr[0];
    mstep = ctr[1];
    ctr[0] = slot + 1;
    ctr[1] = mstep + 1;
    if (slot >= cap) return;
  }
  mdx_step_record &r = rec[slot];
  r.mstep = mstep;
  r.mbsh = s->mbsh;
  r.mbln = s->mbln;
  r.shake_iter = th->shake_iter_max;
  r.pe1 = s->pe1; r.pels1 = s->pels1; r.pe2 = s->pe2; r.pels2 = s->pels2;
  r.spe = s->spe; r.pint = s->pint;
  r.vir1 = s->vir1; r.vir2 = s->vir2; r.virb = s->virb;
  r.virx = s->virx; r.viry = s->viry; r.virz = s->virz;
  r.virfx = s->virfx; r.virfy = s->virfy; r.virfz = s->virfz;
  r.wirs = s->wirs; r.wirss = s->wirss;
  r.tke = th->tke; r.temp = th->temp; r.sc = th->sc; r.scl = th->scl;
  r.tryck = th->tryck; r.tryckm = th->tryckm;
  r.boxl = th->boxl; r.boyl = th->boyl; r.bozl = th->bozl; r.vol = th->vol;
  r.eabs = th->eabs;
}

// ------------------------------------------------------------- host side
MoveConst move_const(mdx_ctx *ctx) {
  MoveConst m{};
  for (int t = 0; t < MDX_NT; ++t) m.lmove[t] = ctx->tc.lmove[t];
  return m;
}
// ------------------------------------------------------------- observables
// INV3B3 (util.f:89-125): inverse of a 3 x 3 matrix by cofactors; ier 1 when
// |DET| < 1e-6 |trace|^3, 2 when DET = 0 (inverse set to zero).
__device__ __forceinline__ void inv3b3(const double *A, double *AI, int &ier) {
  AI[0] = A[4] * A[8] - A[5] * A[7];
  AI[1] = A[2] * A[7] - A[1] * A[8];
  AI[2] = A[1] * A[5] - A[2] * A[4];
  AI[3] = A[5] * A[6] - A[3] * A[8];
  AI[4] = A[0] * A[8] - A[2] * A[6];
  AI[5] = A[2] * A[3] - A[0] * A[5];
  AI[6] = A[3] * A[7] - A[4] * A[6];
  AI[7] = A[1] * A[6] - A[0] * A[7];
  AI[8] = A[0] * A[4] - A[1] * A[3];
  const double det = A[0] * AI[0] + A[3] * AI[1] + A[6] * AI[2];
  const double spur = A[0] + A[4] + A[8];
  ier = fabs(det) < 1.e-6 * fabs(spur * spur * spur) ? 1 : 0;
  double r = 0.0;
  if (fabs(det) > 0.0) {
    r = 1.0 / det;
  } else {
    ier = 2;
  }
  for (int k = 0; k < 9; ++k) AI[k] = r * AI[k];
}

struct KinConst {
  double summd[MDX_NT];  // SUMMAS / (AVSNO 1000 UNITM NBEADS)
  double summas[MDX_NT];
};

// GETKIN (service.f:611-735), thread per molecule: linear momentum and
// translational kinetic energy, the inertia tensor of the site vectors W
// (site position minus the molecule's centre, as GETCOM leaves them) with
// MASSD = 1 / MASSDI, the angular momentum of the site momenta relative to
// the molecule's, and the rotational kinetic energy (the reference's
// fallback when the tensor is singular); EKTR, EKROT, TKE block-summed.
__global__ void k_getkin(int nop, const int *__restrict__ mol_first,
                         const int *__restrict__ mol_nat, const int *__restrict__ mol_type,
                         KinConst kc, const double *__restrict__ amass,
                         const double *__restrict__ massdi, const double *__restrict__ vx,
                         const double *__restrict__ vy, const double *__restrict__ vz,
                         const dbl4 *__restrict__ pos, const double *__restrict__ X,
                         const double *__restrict__ Y, const double *__restrict__ Z, Dst6 dst) {
  double acc[3] = {0.0, 0.0, 0.0};  // EKTR EKROT TKE
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < nop) {
    const int f = mol_first[m], na = mol_nat[m], t = mol_type[m];
    double PX = 0.0, PY = 0.0, PZ = 0.0, tke = 0.0;
    double TOR[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, TORI[9];
    for (int k = 0; k < na; ++k) {
      const int i = f + k;
      const double u = vx[i], v = vy[i], w = vz[i];
      PX = PX + u;
      PY = PY + v;
      PZ = PZ + w;
      tke = tke + 0.5 * (u * u + v * v + w * w) * massdi[i];
      const dbl4 p = pos[i];
      const double wx = p.x - X[m], wy = p.y - Y[m], wz = p.z - Z[m];
      const double md = 1.0 / massdi[i];
      TOR[0] = TOR[0] + md * (wy * wy + wz * wz);
      TOR[4] = TOR[4] + md * (wx * wx + wz * wz);
      TOR[8] = TOR[8] + md * (wx * wx + wy * wy);
      TOR[1] = TOR[1] - md * wx * wy;
      TOR[2] = TOR[2] - md * wx * wz;
      TOR[5] = TOR[5] - md * wy * wz;
    }
    TOR[3] = TOR[1];
    TOR[6] = TOR[2];
    TOR[7] = TOR[5];
    int ier;
    inv3b3(TOR, TORI, ier);
    acc[0] = 0.5 * (PX * PX + PY * PY + PZ * PZ) / kc.summd[t];
    acc[2] = tke;
    double RX = 0.0, RY = 0.0, RZ = 0.0;
    for (int k = 0; k < na; ++k) {
      const int i = f + k;
      const double fac = amass[i] / kc.summas[t];
      const double vtx = vx[i] - PX * fac, vty = vy[i] - PY * fac, vtz = vz[i] - PZ * fac;
      const dbl4 p = pos[i];
      const double wx = p.x - X[m], wy = p.y - Y[m], wz = p.z - Z[m];
      RX = RX + (vty * wz - wy * vtz);
      RY = RY + (vtz * wx - wz * vtx);
      RZ = RZ + (vtx * wy - wx * vty);
    }
    if (ier == 0) {
      acc[1] = 0.5 * (TORI[0] * RX * RX + (TORI[1] + TORI[3]) * RX * RY + TORI[4] * RY * RY +
                      (TORI[2] + TORI[6]) * RX * RZ + TORI[8] * RZ * RZ +
                      (TORI[5] + TORI[7]) * RY * RZ);
    } else {
      const double PP = RX * RX + RY * RY + RZ * RZ;
      if (PP >= 1.e-50) {
        double ROTM = 0.0;
        for (int k = 0; k < na; ++k) {
          const int i = f + k;
          const dbl4 p = pos[i];
          const double wx = p.x - X[m], wy = p.y - Y[m], wz = p.z - Z[m];
          const double SS = wx * wx + wy * wy + wz * wz;
          const double SP = wx * RX + wy * RY + wz * RZ;
          ROTM = ROTM + (1.0 / massdi[i]) * (SS * PP - SP * SP);
        }
        acc[1] = ROTM >= 1.e-50 ? 0.5 * PP * PP / ROTM : 0.0;
      }
    }
  }
  block_add<3>(acc, dst);
}

// CHKMOM (service.f:1081-1125): total momentum of all atoms, then
// V -= (P / SUMASD) / MASSDI.
__global__ void k_mom_sum(int n, const double *__restrict__ vx, const double *__restrict__ vy,
                          const double *__restrict__ vz, Dst6 dst) {
  double acc[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    acc[0] += vx[i];
    acc[1] += vy[i];
    acc[2] += vz[i];
  }
  block_add<3>(acc, dst);
}

__global__ void k_mom_remove(int n, double sumasd, const double *__restrict__ pt,
                             const double *__restrict__ massdi, double *vx, double *vy,
                             double *vz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dvx = pt[0] / sumasd, dvy = pt[1] / sumasd, dvz = pt[2] / sumasd;
  vx[i] = vx[i] - dvx / massdi[i];
  vy[i] = vy[i] - dvy / massdi[i];
  vz[i] = vz[i] - dvz / massdi[i];
}

MolConst mol_const(mdx_ctx *ctx) {
  MolConst m{};
  for (int t = 0; t < MDX_NT; ++t) {
    m.summas[t] = ctx->summas[t];
    m.rsummas[t] = ctx->summas[t] != 0.0 ? 1.0 / ctx->summas[t] : 0.0;
  }
  m.cell = cell_pbc(ctx);
  return m;
}

}  // namespace

int launch_getemp(mdx_ctx *ctx);

// Scratch of the SCALING stages lives at a fixed place of the context.
static ScalScratch *scratch(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  return reinterpret_cast<ScalScratch *>(ctx->dv.scal_scratch);
}

size_t scal_scratch_bytes() { return sizeof(ScalScratch); }

static ScalConst scal_const(mdx_ctx *ctx) {
  const mdx_params &p = ctx->p;
  ScalConst c{};
  c.ntypes = ctx->d.ntypes;
  c.lnvt = p.lnvt; c.lnpt = p.lnpt; c.lsep = p.lsep; c.lsctd = p.lsctd;
  c.lp_xy = p.lp_xy; c.lshejk = p.lshejk; c.lsclt = p.lsclt; c.icell = p.icell;
  c.tstep = p.tstep; c.htstep = 0.5 * p.tstep; c.trtemp = p.trtemp; c.tdelt = p.tdelt;
  c.trpres = p.trpres; c.trpresx = p.trpresx; c.trpresy = p.trpresy; c.trpresz = p.trpresz;
  c.dqt = p.dqt; c.dqp = p.dqp; c.rtp = p.rtp; c.fnst = p.fnst; c.fnop = p.fnop;
  c.unitp = p.unitp; c.vird = p.vird; c.tridm_coef = p.tridm_coef;
  c.tridee_coef = p.tridee_coef; c.convet = p.convet; c.chktf = p.chktf;
  c.rtrtemp = 1.0 / p.trtemp;
  c.tlow = p.chktf > 0.0 ? p.trtemp / p.chktf : 0.0;
  c.dqt_f = p.dqt / p.fnst;
  c.c3_fnst = 3. / p.fnst;
  c.c3_fnop = 3. / p.fnop;
  c.rfnst = 1.0 / p.fnst;
  for (int t = 0; t < MDX_NT; ++t) {
    c.tfact[t] = p.tfact[t];
    c.lmove[t] = ctx->tc.lmove[t];
  }
  return c;
}

static int stage(mdx_ctx *ctx, int st) {
  StageList L{};
  L.n = 1;
  L.st[0] = st;
  k_scal_list<<<1, 128, 0, ctx->stream>>>(L, scal_const(ctx), scratch(ctx), ctx->dv.th,
                                            ctx->dv.sc, ctx->dv.err);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// Queue of SCALING stages launched together; flushed before any kernel that
// reads what they write (the per-atom scalings) or writes what they read.
struct StageQ {
  mdx_ctx *ctx;
  StageList L{};
  void push(int st) { L.st[L.n++] = st; }
  int flush() {
    if (!L.n) return MDX_OK;
    k_scal_list<<<1, 128, 0, ctx->stream>>>(L, scal_const(ctx), scratch(ctx), ctx->dv.th,
                                            ctx->dv.sc, ctx->dv.err);
    MDX_LAUNCHED(ctx);
    L.n = 0;
    return MDX_OK;
  }
};

// DOUBLE-style drift of every bead (no kick before it: htsteb applies to H)
__global__ void k_kick_drift_com_beads(int nop, const int *__restrict__ mol_first,
                                       const int *__restrict__ mol_nat,
                                       const int *__restrict__ mol_type,
                                       const int4 *__restrict__ ainfo, MoveConst mv, MolConst mc,
                                       double htsteb, double tsteb, int n,
                                       const double *__restrict__ massdi,
                                       const double *__restrict__ amass, double bx, double by,
                                       double bz, double3 ibs, const int *__restrict__ pinfo,
                                       const BeadMove *__restrict__ beads) {
  const BeadMove &b = beads[blockIdx.y];
  kick_drift_com_body(blockIdx.x * blockDim.x + threadIdx.x, nop, mol_first, mol_nat, mol_type,
                      ainfo, mv, mc, htsteb, tsteb, 0, b.f[0][0], b.f[0][1], b.f[0][2], nullptr,
                      n, 0.0, massdi, amass, b.vx, b.vy, b.vz, b.pos, b.X, b.Y, b.Z, bx, by, bz,
                      ibs, b.posi, pinfo, b.posc, b.slot_of);
}

static KickArgs kick_args(mdx_ctx *ctx, const KickSpec &k) {
  DevData &d = ctx->dv;
  KickArgs a{};
  auto set = [&](int w, const double *&x, const double *&y, const double *&z) {
    x = w == 1 ? d.hx : w == 2 ? d.gx : w == 3 ? d.fx : nullptr;
    y = w == 1 ? d.hy : w == 2 ? d.gy : w == 3 ? d.fy : nullptr;
    z = w == 1 ? d.hz : w == 2 ? d.gz : w == 3 ? d.fz : nullptr;
  };
  set(k.w1, a.ax, a.ay, a.az);
  set(k.w2, a.bx, a.by, a.bz);
  a.h1 = k.h1;
  a.h2 = k.h2;
  a.vs = k.vscale ? scratch(ctx)->vscale : nullptr;
  return a;
}

// The kinetic-energy reduction of GETEMP, with kicks folded in (pre, post;
// w1 = 0: none); its fold is the ST_GETEMP stage.
static int getemp_kernel(mdx_ctx *ctx, const KickSpec &pre = {}, const KickSpec &post = {}) {
  DevData &d = ctx->dv;
  const int nt = ctx->d.ntypes;
  const KickArgs a = kick_args(ctx, pre), b = kick_args(ctx, post);
  const bool kick = a.ax || b.ax || a.vs;
#define GETEMP_K(NT, R, K)                                                             \
  k_getemp<NT, R, K><<<red_blocks(ctx), 256, 0, ctx->stream>>>(                               \
      d.n, d.ainfo, move_const(ctx), nt, d.massdi, d.vx, d.vy, d.vz,                   \
      scratch(ctx)->ekacc, d.red_part, d.red_ctr, a, b)
#define GETEMP(NT)                                                                    \
  do {                                                                                \
    if (ctx->mixed()) {                                                               \
      if (kick) GETEMP_K(NT, float, true);                                            \
      else GETEMP_K(NT, float, false);                                                \
    } else {                                                                          \
      if (kick) GETEMP_K(NT, double, true);                                           \
      else GETEMP_K(NT, double, false);                                               \
    }                                                                                 \
  } while (0)
  if (nt <= 1) GETEMP(1);
  else if (nt <= 2) GETEMP(2);
  else if (nt <= 4) GETEMP(4);
  else GETEMP(MDX_NT);
#undef GETEMP
#undef GETEMP_K
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// kick(s), GETEMP, kick(s) in one pass over the atoms, then the ST_GETEMP fold
int launch_getemp_kick(mdx_ctx *ctx, const KickSpec &pre, const KickSpec &post) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  const int rc = getemp_kernel(ctx, pre, post);
  return rc ? rc : stage(ctx, ST_GETEMP);
}

int launch_getemp(mdx_ctx *ctx) {
  const int rc = getemp_kernel(ctx);
  return rc ? rc : stage(ctx, ST_GETEMP);
}

static int scale_atoms(mdx_ctx *ctx, int mode) {
  DevData &d = ctx->dv;
  k_scale_atoms<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(
      d.n, mode, d.ainfo, move_const(ctx), scratch(ctx), d.massdi, d.vx, d.vy, d.vz, d.pos);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

#define RC(x)                  \
  do {                         \
    int rc_ = (x);             \
    if (rc_) return rc_;       \
  } while (0)

// SCALING(IAL).  For IAL=1 in NVT (no NPT) the final velocity factor is left
// in the scratch for the following slow half-kick, which applies it first
// (same operation order as the reference: V*SCV, then V + HTSTEP*G);
// *pending_vscale tells the caller.
int launch_scaling(mdx_ctx *ctx, int ial, bool *pending_vscale, const KickSpec *kick_first) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  const mdx_params &p = ctx->p;
  StageQ q{ctx};
  KickSpec scv;  // V *= SCV (per type) folded into the GETEMP pass that follows it
  scv.vscale = true;
  if (pending_vscale) *pending_vscale = false;
  if (ial == 3 && p.lnvt) {
    q.push(ST_3V);
    RC(q.flush());
    RC(scale_atoms(ctx, 0));
  }
  RC(getemp_kernel(ctx, kick_first ? *kick_first : KickSpec{}));
  q.push(ST_GETEMP);
  q.push(ST_PRESS);
  if (ial == 1) {
    if (p.lnvt) {
      q.push(ST_1A);
      if (p.lnpt) {
        RC(q.flush());
        RC(scale_atoms(ctx, 2));
        q.push(ST_1RECLEN);
      } else {
        // 3.4.3 calls GETEMP again on unchanged velocities: same values
        q.push(ST_1NVT);
        if (pending_vscale) {
          *pending_vscale = true;
        } else {
          RC(q.flush());
          RC(scale_atoms(ctx, 0));
        }
      }
      q.push(ST_EABS);
    }
  } else if (ial == 2) {
    if (p.lnvt) {
      q.push(ST_2V);
      RC(q.flush());
      if (p.lnpt) {
        RC(scale_atoms(ctx, 0));
        q.push(ST_2NPTV);
        RC(q.flush());
        RC(scale_atoms(ctx, 3));
        RC(getemp_kernel(ctx));
        q.push(ST_GETEMP);
        q.push(ST_2SCL);
      } else {
        RC(getemp_kernel(ctx, scv));
        q.push(ST_GETEMP);
      }
      q.push(ST_2SC);
    }
  } else if (ial == 3) {
    if (p.lnvt) {
      q.push(ST_3A);
      if (p.lnpt) {
        RC(q.flush());
        DevData &d = ctx->dv;
        k_com_scale<<<(d.nop + 127) / 128, 128, 0, ctx->stream>>>(
            d.nop, d.mol_first, d.mol_nat, d.mol_type, d.amass, mol_const(ctx),
            move_const(ctx), scratch(ctx), d.vx, d.vy, d.vz, d.pos);
        MDX_LAUNCHED(ctx);
        q.push(ST_3B);
      }
      q.push(ST_EABS);
    }
  }
  if (p.lsclt && (ial == 2 || ial == 3)) {
    q.push(ST_SCLT);
    RC(q.flush());
    RC(getemp_kernel(ctx, scv));
    q.push(ST_GETEMP);
  }
  return q.flush();
}

int launch_mstep1_rescale(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  RC(launch_getemp(ctx));
  RC(stage(ctx, ST_MSTEP1));
  return scale_atoms(ctx, 1);
}

int launch_zero_fast(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  k_zero_scalars<<<1, 64, 0, ctx->stream>>>(d.sc, 1, ctx->p.molint, ctx->d.ntypes);
  MDX_LAUNCHED(ctx);
  if (ctx->mixed()) {
    MDX_CUDA(cudaMemsetAsync(d.hfix, 0, sizeof(unsigned long long) * 3 * d.n, ctx->stream));
  } else {
    MDX_CUDA(cudaMemsetAsync(d.hx, 0, sizeof(double) * 3 * d.n, ctx->stream));
  }
  return MDX_OK;
}

int launch_zero_slow(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  k_zero_scalars<<<1, 64, 0, ctx->stream>>>(d.sc, 2, ctx->p.molint, ctx->d.ntypes);
  MDX_LAUNCHED(ctx);
  if (ctx->mixed()) {
    MDX_CUDA(cudaMemsetAsync(d.gfix, 0, sizeof(unsigned long long) * 3 * d.n, ctx->stream));
  } else {
    MDX_CUDA(cudaMemsetAsync(d.gx, 0, sizeof(double) * 3 * d.n, ctx->stream));
  }
  return MDX_OK;
}

int launch_fix_to_double(mdx_ctx *ctx, int which) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  const unsigned long long *f = which == 1 ? d.hfix : d.gfix;
  double *x = which == 1 ? d.hx : d.gx, *y = which == 1 ? d.hy : d.gy,
         *z = which == 1 ? d.hz : d.gz;
  k_fix_fold<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, f, ctx->fix.inv, x, y, z);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_sclfrc(mdx_ctx *ctx, int nnn) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  if (!ctx->p.lscft) return MDX_OK;
  DevData &d = ctx->dv;
  const double fct = nnn == 1 ? ctx->p.ftscl * ctx->p.ftimes : ctx->p.ftscl;
  double *x = nnn == 1 ? d.hx : nnn == 2 ? d.gx : d.fx;
  double *y = nnn == 1 ? d.hy : nnn == 2 ? d.gy : d.fy;
  double *z = nnn == 1 ? d.hz : nnn == 2 ? d.gz : d.fz;
  k_sclfrc<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, fct, d.massdi, x, y, z, d.sc);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// PULLBACK (forces.f:1756-1799) on G: drag on chosen types, harmonic wells
// on chosen atoms, external field along z at FULTIM = TIM + NSTEP DT.
struct PullConst {
  int ldrag, npull, iext;
  int ldragt[MDX_NT];
  double fdrag[MDX_NT];
  double rlr, exampl, exfreq, tim, dt;
};

// Thread per atom, the reference's order on each atom: drag, well, field.
// well[i]: the atom's well (-1: none; the last one if listed twice).
__global__ void k_pullback(int n, const int4 *__restrict__ ainfo,
                           const double *__restrict__ massdi, const dbl4 *__restrict__ pos,
                           PullConst pc, const int *__restrict__ well,
                           const double *__restrict__ ref, const int *__restrict__ nstep,
                           double *gx, double *gy, double *gz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int t = ainfo[i].x;
  const dbl4 p = pos[i];
  if (pc.ldrag && pc.ldragt[t]) gz[i] = gz[i] + (1.0 / massdi[i]) * pc.fdrag[t];
  if (pc.npull > 0) {
    const int w = well[i];
    if (w >= 0) {
      gx[i] = gx[i] - pc.rlr * (p.x - ref[w]);
      gy[i] = gy[i] - pc.rlr * (p.y - ref[pc.npull + w]);
      gz[i] = gz[i] - pc.rlr * (p.z - ref[2 * pc.npull + w]);
    }
  }
  if (pc.iext == 1) {
    const double FULTIM = pc.tim + (*nstep) * pc.dt;
    const double EFIELD = pc.exampl * cos(pc.exfreq * FULTIM * 0.5 / MDX_PI);
    gz[i] = gz[i] + p.w * EFIELD;
  }
}

__global__ void k_step_tick(int *nstep) { *nstep = *nstep + 1; }

int launch_pullback(mdx_ctx *ctx) {
  if (!ctx->pullback) return MDX_OK;
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  PullConst pc{};
  pc.ldrag = ctx->pb.ldrag;
  pc.npull = ctx->pb.npull;
  pc.iext = ctx->pb.iext;
  for (int t = 0; t < MDX_NT; ++t) {
    pc.ldragt[t] = ctx->pb.ldragt[t];
    pc.fdrag[t] = ctx->pb.fdrag[t];
  }
  pc.rlr = ctx->pb.rlr;
  pc.exampl = ctx->pb.exampl;
  pc.exfreq = ctx->pb.exfreq;
  pc.tim = ctx->pb.tim;
  pc.dt = ctx->pb.dt;
  k_pullback<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, d.ainfo, d.massdi, d.pos, pc,
                                                        d.pull_atom, d.pull_ref, d.pull_step,
                                                        d.gx, d.gy, d.gz);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_step_tick(mdx_ctx *ctx) {
  if (!ctx->pullback) return MDX_OK;
  k_step_tick<<<1, 1, 0, ctx->stream>>>(ctx->dv.pull_step);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_sum_forces(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  k_sum_forces<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, d.gx, d.gy, d.gz, d.hx,
                                                           d.hy, d.hz, d.fx, d.fy, d.fz);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_getcom(mdx_ctx *ctx, bool mirror) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  k_getcom<<<(d.nop + 127) / 128, 128, 0, ctx->stream>>>(
      d.nop, d.mol_first, d.mol_nat, d.mol_type, d.amass, d.pos, d.X, d.Y, d.Z,
      mol_const(ctx), ctx->boxl, ctx->boyl, ctx->bozl, nullptr,
      mirror && ctx->mixed() ? d.posi : nullptr, d.pinfo);
  MDX_LAUNCHED(ctx);
  return mirror ? launch_cell_refresh(ctx) : MDX_OK;
}

int launch_kick(mdx_ctx *ctx, int which, double h, bool apply_vscale) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  const double *x = which == 1 ? d.hx : which == 2 ? d.gx : d.fx;
  const double *y = which == 1 ? d.hy : which == 2 ? d.gy : d.fy;
  const double *z = which == 1 ? d.hz : which == 2 ? d.gz : d.fz;
  k_kick<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(
      d.n, d.ainfo, move_const(ctx), h, x, y, z, d.vx, d.vy, d.vz,
      apply_vscale ? scratch(ctx)->vscale : nullptr);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// Two kicks in one pass: forces `which1` with h1, then `which2` with h2.
int launch_kick2(mdx_ctx *ctx, int which1, double h1, int which2, double h2) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  auto set = [&](int w, const double *&x, const double *&y, const double *&z) {
    x = w == 1 ? d.hx : w == 2 ? d.gx : d.fx;
    y = w == 1 ? d.hy : w == 2 ? d.gy : d.fy;
    z = w == 1 ? d.hz : w == 2 ? d.gz : d.fz;
  };
  const double *ax, *ay, *az, *bx, *by, *bz;
  set(which1, ax, ay, az);
  set(which2, bx, by, bz);
  k_kick<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, d.ainfo, move_const(ctx), h1, ax, ay,
                                                     az, d.vx, d.vy, d.vz, nullptr, h2, bx, by,
                                                     bz);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_kick_drift(mdx_ctx *ctx, double htsteb, double tsteb, int prev) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  k_kick_drift<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(
      d.n, d.ainfo, move_const(ctx), htsteb, tsteb, prev, d.hx, d.hy, d.hz, d.massdi,
      d.vx, d.vy, d.vz, d.pos);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_kick_drift_com(mdx_ctx *ctx, double htsteb, double tsteb, int prev, bool from_fix) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  // a warp per block: the molecules spread over the SMs evenly (this pass
  // waits on its FP64 chains; 0.4 % of the mixed step against 128 threads)
  k_kick_drift_com<<<(d.nop + 31) / 32, 32, 0, ctx->stream>>>(
      d.nop, d.mol_first, d.mol_nat, d.mol_type, d.ainfo, move_const(ctx), mol_const(ctx),
      htsteb, tsteb, prev, d.hx, d.hy, d.hz, from_fix ? d.hfix : nullptr, d.n, ctx->fix.inv,
      d.massdi, d.amass, d.vx, d.vy, d.vz, d.pos, d.X, d.Y, d.Z, ctx->boxl, ctx->boyl,
      ctx->bozl,
      make_double3(4294967296.0 * (1.0 / ctx->boxl), 4294967296.0 * (1.0 / fix_period_y(ctx)),
                   4294967296.0 * (1.0 / ctx->bozl)),
      ctx->mixed() ? d.posi : nullptr, d.pinfo,
      ctx->mixed() && ctx->have_lists ? d.cell_pos : nullptr, d.slot_of);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// ------------------------------------------ bead ensembles: host side ---
size_t bead_move_bytes() { return sizeof(BeadMove); }

// One bead's entry of the device table (pointers only; written once the
// bead's lists exist, they stay valid for the context's life).
void bead_move_fill(mdx_ctx *ctx, void *out) {
  DevData &d = ctx->dv;
  BeadMove b{};
  b.pos = d.pos;
  b.vx = d.vx;
  b.vy = d.vy;
  b.vz = d.vz;
  const double *f[3][3] = {{d.hx, d.hy, d.hz}, {d.gx, d.gy, d.gz}, {d.fx, d.fy, d.fz}};
  for (int w = 0; w < 3; ++w)
    for (int a = 0; a < 3; ++a) b.f[w][a] = f[w][a];
  b.X = d.X;
  b.Y = d.Y;
  b.Z = d.Z;
  b.posi = ctx->mixed() ? d.posi : nullptr;
  b.posc = ctx->mixed() && ctx->have_lists ? d.cell_pos : nullptr;
  b.slot_of = d.slot_of;
  b.part = d.red_part;
  b.ctr = d.red_ctr;
  b.ss = reinterpret_cast<ScalScratch *>(d.scal_scratch);
  b.th = d.th;
  b.sc = d.sc;
  b.err = d.err;
  std::memcpy(out, &b, sizeof b);
}

static KickW kick_w(const KickSpec &k) {
  KickW w{};
  w.w1 = k.w1;
  w.w2 = k.w2;
  w.vs = k.vscale ? 1 : 0;
  w.h1 = k.h1;
  w.h2 = k.h2;
  return w;
}

// kick(s), GETEMP, kick(s) and the ST_GETEMP fold of all P beads (c0: any
// bead; the beads share sizes, topology and parameters), on stream st.
int launch_getemp_beads(mdx_ctx *c0, int P, const void *table, cudaStream_t st,
                        const KickSpec &pre, const KickSpec &post) {
  MDX_TIMER(c0, MDX_T_MOVE);
  DevData &d = c0->dv;
  const int nt = c0->d.ntypes;
  const KickW a = kick_w(pre), b = kick_w(post);
  const bool kick = a.w1 || b.w1 || a.vs;
  const BeadMove *tab = static_cast<const BeadMove *>(table);
  const dim3 grid(red_blocks(c0), P);
#define GB_K(NT, R, K)                                                                   \
  k_getemp_beads<NT, R, K><<<grid, 256, 0, st>>>(d.n, d.ainfo, move_const(c0), nt, d.massdi, \
                                                 tab, a, b)
#define GB(NT)                                   \
  do {                                           \
    if (c0->mixed()) {                           \
      if (kick) GB_K(NT, float, true);           \
      else GB_K(NT, float, false);               \
    } else {                                     \
      if (kick) GB_K(NT, double, true);          \
      else GB_K(NT, double, false);              \
    }                                            \
  } while (0)
  if (nt <= 1) GB(1);
  else if (nt <= 2) GB(2);
  else if (nt <= 4) GB(4);
  else GB(MDX_NT);
#undef GB
#undef GB_K
  MDX_LAUNCHED(c0);
  StageList L{};
  L.n = 1;
  L.st[0] = ST_GETEMP;
  k_scal_list_beads<<<P, 128, 0, st>>>(L, scal_const(c0), tab);
  MDX_LAUNCHED(c0);
  return MDX_OK;
}

// drift (after a kick of htsteb on H), GETCOM and the coordinate mirrors of
// all P beads, on stream st
int launch_kick_drift_com_beads(mdx_ctx *c0, int P, const void *table, cudaStream_t st,
                                double htsteb, double tsteb) {
  MDX_TIMER(c0, MDX_T_MOVE);
  DevData &d = c0->dv;
  const dim3 grid((d.nop + 127) / 128, P);
  k_kick_drift_com_beads<<<grid, 128, 0, st>>>(
      d.nop, d.mol_first, d.mol_nat, d.mol_type, d.ainfo, move_const(c0), mol_const(c0), htsteb,
      tsteb, d.n, d.massdi, d.amass, c0->boxl, c0->boyl, c0->bozl,
      make_double3(4294967296.0 * (1.0 / c0->boxl), 4294967296.0 * (1.0 / fix_period_y(c0)),
                   4294967296.0 * (1.0 / c0->bozl)),
      d.pinfo, static_cast<const BeadMove *>(table));
  MDX_LAUNCHED(c0);
  return MDX_OK;
}

int launch_leapfrog_shake(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  k_leapfrog<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(
      d.n, d.ainfo, move_const(ctx), ctx->p.tstep, d.fx, d.fy, d.fz, d.massdi, d.vx,
      d.vy, d.vz, d.pos, d.ox, d.oy, d.oz, ctx->p.lshejk ? 1 : 0);
  MDX_LAUNCHED(ctx);
  k_shake_prep<<<1, 1, 0, ctx->stream>>>(d.th);
  MDX_LAUNCHED(ctx);
  if (ctx->p.lshejk) {
    ShakeConst sk{};
    for (int t = 0; t < MDX_NT; ++t) {
      sk.iadb[t] = ctx->iadb[t];
      sk.nrb[t] = ctx->nrb[t];
      sk.ishejk[t] = ctx->ishejk[t];
    }
    sk.maxit = ctx->p.maxit > 0 ? ctx->p.maxit : 2000;
    sk.tol2 = ctx->p.toler * ctx->p.toler;
    sk.tstep = ctx->p.tstep;
    sk.cell = cell_pbc(ctx);
    if (d.shk_nitem > 0) {
      k_shake_cluster<<<(d.shk_nitem + 63) / 64, 64, 0, ctx->stream>>>(
          d.shk_nitem, d.shk_item, d.shk_cl, d.shk_rec, d.mol_first, d.mol_type,
          move_const(ctx), sk, d.bib, d.bjb, d.brb, d.massdi, d.pos, d.ox, d.oy, d.oz,
          ctx->boxl, ctx->boyl, ctx->bozl, d.th, d.shk_mfail);
      MDX_LAUNCHED(ctx);
    }
    k_shake_finish<<<(d.nop + 63) / 64, 64, 0, ctx->stream>>>(
        d.nop, d.mol_first, d.mol_nat, d.mol_type, move_const(ctx), sk, d.massdi, d.pos,
        d.vx, d.vy, d.vz, d.ox, d.oy, d.oz, d.fx, d.fy, d.fz, d.th, d.err, d.shk_mfail,
        dst6(ctx, (d.nop + 63) / 64, 3, &d.th->viran[0], &d.th->viran[1], &d.th->viran[2]));
    MDX_LAUNCHED(ctx);
  }
  return MDX_OK;
}

int launch_vira(mdx_ctx *ctx, int from_viran) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  if (from_viran)
    k_vira_from_viran<<<1, 1, 0, ctx->stream>>>(ctx->dv.th);
  else
    k_vira_zero<<<1, 1, 0, ctx->stream>>>(ctx->dv.th);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int launch_record(mdx_ctx *ctx, int slot, int mstep) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  // slot < 0: take slot and step number from the device counters
  int *ctr = slot < 0 ? ctx->dv.shake_iter + 16 : nullptr;
  k_record<<<1, 1, 0, ctx->stream>>>(ctx->dv.rec, slot, mstep, ctx->dv.sc, ctx->dv.th, ctr,
                                     ctx->dv.rec_cap);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// GETKIN on the device; out = EKTR, EKROT, TKE (summed in block order).
int launch_getkin(mdx_ctx *ctx, const double *summd, double *out) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  KinConst kc{};
  for (int t = 0; t < MDX_NT; ++t) {
    kc.summd[t] = t < ctx->d.ntypes ? summd[t] : 1.0;
    kc.summas[t] = ctx->summas[t] != 0.0 ? ctx->summas[t] : 1.0;
  }
  double *acc = d.red + 480;  // scratch of the observables
  MDX_CUDA(cudaMemsetAsync(acc, 0, 3 * sizeof(double), ctx->stream));
  const int nb = (d.nop + 127) / 128;
  k_getkin<<<nb, 128, 0, ctx->stream>>>(d.nop, d.mol_first, d.mol_nat, d.mol_type, kc, d.amass,
                                        d.massdi, d.vx, d.vy, d.vz, d.pos, d.X, d.Y, d.Z,
                                        dst6(ctx, nb, 3, acc, acc + 1, acc + 2));
  MDX_LAUNCHED(ctx);
  MDX_CUDA(ctx_copy(ctx->stream, out, acc, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  return MDX_OK;
}

// CHKMOM on the device; pt = the total momentum removed.
int launch_chkmom(mdx_ctx *ctx, double sumasd, double *pt) {
  MDX_TIMER(ctx, MDX_T_MOVE);
  DevData &d = ctx->dv;
  double *acc = d.red + 484;
  MDX_CUDA(cudaMemsetAsync(acc, 0, 3 * sizeof(double), ctx->stream));
  const int nb = red_blocks(ctx);
  k_mom_sum<<<nb, 256, 0, ctx->stream>>>(d.n, d.vx, d.vy, d.vz,
                                         dst6(ctx, nb, 3, acc, acc + 1, acc + 2));
  MDX_LAUNCHED(ctx);
  k_mom_remove<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, sumasd, acc, d.massdi, d.vx,
                                                           d.vy, d.vz);
  MDX_LAUNCHED(ctx);
  RC(launch_getemp(ctx));  // GETEMP of the corrected momenta (service.f:1116)
  MDX_CUDA(ctx_copy(ctx->stream, pt, acc, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  return MDX_OK;
}
