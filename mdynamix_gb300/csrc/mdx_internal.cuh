// mdx_internal.cuh -- device data layout and shared helpers of libmdxgpu.
//
// One context holds one system resident in HBM.  Layout (structure of
// arrays, one entry per atom unless noted):
//   pos     dbl4 {x, y, z, Q}       master coordinates + (EE-scaled) charge
//   posf    float4  {x, y, z, Q}       FP32 mirror for the mixed path
//   vx..vz  double                     momenta (the reference's VX/VY/VZ)
//   ainfo   int4 {type, molecule, LJ type, site}   all 0-based
//   gx..hz  double                     slow (G) and fast (H) forces
//   gfix..  long long                  64-bit fixed-point force sums (mixed)
//   lists   int [atom][cap]            per-owner neighbour rows (see nblist)
// Scalars (energies, virials) live in one mdx_scalars block, thermostat state
// in one mdx_thermo block, both in device memory so that a whole long step
// runs without a host round trip.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mdx_gpu.h"

#define MDX_NT MDX_NTPS

// 32-byte aligned double4: one 256-bit load per atom record.
typedef double4_32a dbl4;

// Constants of the reference (common_inc.f:22-33).
#define MDX_A1 0.254829592
#define MDX_A2 (-0.284496736)
#define MDX_A3 1.421413741
#define MDX_A4 (-1.453152027)
#define MDX_A5 1.061405429
#define MDX_B1 0.3275911
#define MDX_PI 3.1415926536
#define MDX_TOTPI 1.128379169

// Device error word bits.
enum : int {
  DERR_LIST_SHORT = 1,
  DERR_LIST_LONG = 2,
  DERR_NAN = 4,
  DERR_SHAKE = 8,
  DERR_NPT = 16,
  DERR_TEMP = 32,
  DERR_CELL = 64,
  DERR_TIMEOUT = 128,  // a bounded device wait (tensor-core pipeline) ran out
};

// Per-type constants passed by value to kernels.
struct TypeConst {
  int ntypes;
  int lmove[MDX_NT];
  int iee[MDX_NT];
  int ipot[MDX_NT];
  double c14el[MDX_NT];
  double c14lj[MDX_NT];
  float c14elf[MDX_NT];
  float c14ljf[MDX_NT];
  int mdx[MDX_NT][MDX_NT];  // 0-based type pair index
};

// Box and electrostatics parameters for the force kernels.
struct PairConst {
  double coulf, alphad, raex, rff, rff2;
  int lmnbl, lmdee, nnbt;
  // squared cutoff the long-row sweeps test each pair against: RCUT^2 in
  // skin mode (rows reach RCUT + skin), above every distance otherwise (the
  // reference evaluates every listed pair)
  double rc2;
  float rc2f;
};

// Threads per owner atom of the mixed pair sweeps when nothing else is chosen.
constexpr int TPO_SHORT_DEFAULT = 4;
constexpr int TPO_LONG_DEFAULT = 32;
void resolve_tuning(mdx_ctx *ctx);  // pair.cu: the tuning table's choice, once
// Blocks of the grid-stride per-atom reductions (GETEMP, WIRS, momenta):
// one per SM, or one per 256 atoms when that is fewer (a small system's
// reduction then is not spread over mostly idle blocks).  A function of the
// atom count alone, so the sums' order is fixed for a system.
struct mdx_ctx;
int red_blocks(const mdx_ctx *ctx);
struct CellPbc;
CellPbc cell_pbc(const mdx_ctx *ctx);  // the context's cell and box (pair.cu)

// Cell grid used by the list build.
struct CellGrid {
  int nx, ny, nz, ncell;
  double cx, cy, cz;  // cell edge lengths
};

// Ewald k-space layout: k-vectors grouped in columns of fixed (nx, ny) with
// an nz range in steps of zstep; tables of per-atom phase factors
// e^{i n theta}.  Record p of a column pairs nz = +z(p) and -z(p), z(p) =
// zoff + zstep p: rectangular and hexagonal cells zoff 0, zstep 1; the
// truncated octahedron's k-set (forces.f:1392-1397: RZV = 2 pi (-IKX + IKY +
// 2 IKZ)) has in each column the nz of one parity, zoff = that parity,
// zstep 2.
struct KCol {
  int nx, ny, nzlo, nzhi;  // integer k components
  int koff;                // first k of the column in the column-ordered list
  int wpos;                // mixed: slot of (group, p = 0) in the paired W array
  int m;                   // last record: the column pairs nz = +z(p) and -z(p), p = 0..m
  int poff;                // FP64: first paired-W record of the column
  int zoff, zstep;         // z(p) = zoff + zstep p
};

// k index of (column, nz), -1 outside the column's set.
__host__ __device__ __forceinline__ int kcol_k(const KCol &c, int nz) {
  if (nz < c.nzlo || nz > c.nzhi) return -1;
  const int d = nz - c.nzlo;
  if (c.zstep == 1) return c.koff + d;
  return d % c.zstep ? -1 : c.koff + d / c.zstep;
}
__host__ __device__ __forceinline__ int kcol_z(const KCol &c, int p) {
  return c.zoff + c.zstep * p;
}

// Bonds and angles of one small molecule type, atoms as offsets within the
// molecule, for the molecule-local bonded kernel.
constexpr int ML_MAXS = 8, ML_MAXB = 16, ML_MAXA = 24;
struct MolTpl {
  int first, nmol, nsit, nb, na, type;
  unsigned char bi[ML_MAXB], bj[ML_MAXB];
  short bm[ML_MAXB];
  unsigned char ai[ML_MAXA], aj[ML_MAXA], ak[ML_MAXA];
  short am[ML_MAXA];
};

constexpr int MDX_SITE_BITS = 13;

// Slot of entry k of atom i's neighbour row.  Rows back to back (a warp walks
// one row) except the mixed path's short list ("tiled"): 32 atoms' rows
// interleaved, entry k of the 32 atoms of a tile adjacent, so a thread per
// atom reads its row with coalesced loads.  Tiled storage holds
// ceil(n / 32) * 32 rows.
__host__ __device__ __forceinline__ size_t list_slot(int i, int k, int cap, bool tiled) {
  return tiled ? ((size_t)(i >> 5) * cap + k) * 32 + (i & 31) : (size_t)i * cap + k;
}  // sites < 8192, molecules < 2^19 (mixed path)

// Four columns with the same m = max |nz|, for the mixed Ewald passes.  The
// force pass reads, per p = 0..m, one record of 8 float4: for each column
// slot s, {P_U, M_U} then {P_V, M_V} (paired W, see k_wpairs) at
// wg[8 (woff + p) + 2 s + half]; one z-table load feeds four columns and
// both signs of nz.  col[s] < 0 marks a padding slot (W = 0).
constexpr int KGRP = 4;
struct KGroup {
  int m, len, woff;  // len = m + 1 records
  int zoff;          // the columns' common z offset: record p is z = zoff + zstep p
  int col[KGRP];
};

// Scratch for fixed-point accumulation of the mixed path: forces are stored
// as round(F * 2^fx_shift) in 64-bit integers.
struct FixScale {
  double scale, inv;    // forces
  double escale, einv;  // energies and virials
  float scalef, escalef;  // the same scales as FP32 (powers of two: exact)
};

// Destination pointers of a block reduction, passed by value to kernels,
// with the partials buffer and counter of the deterministic reduction.
struct Dst6 {
  double *p[6];
  double *part;
  unsigned *ctr;
};

struct DevData {
  int n, nop, ntypes, nnbt, nbdmax;
  dbl4 *pos;
  float4 *posf;      // FP32 mirror (list prefilter)
  int4 *posi;        // 32-bit fixed-point coordinates + FP32 charge bits
  float *qsitef;     // CHARGE(NSITE(i)) in FP32
  double *vx, *vy, *vz;
  double *massdi, *amass, *qsite;
  int4 *ainfo;
  int *nnbb, *inbb;  // inbb[i*nbdmax + k] = signed 1-based partner (Fortran value)
  // molecules
  int *mol_first, *mol_nat, *mol_type;
  double *X, *Y, *Z;
  // forces
  double *gx, *gy, *gz, *hx, *hy, *hz, *fx, *fy, *fz;
  double *ox, *oy, *oz;
  unsigned long long *gfix, *hfix;  // 3n each, x then y then z
  // lists
  int cap_s, cap_l;
  int *ns_cnt, *nl_cnt, *ns_idx, *nl_idx;
  int *cell_cnt, *cell_start, *cell_list, *atom_cell;
  // per cell-sorted slot: the candidate record k_build reads; on the mixed
  // path also the neighbour records of the pair sweeps, whose lists hold
  // slots (kept equal to posi[cell_list[slot]] by every posi writer)
  int4 *cell_pos;
  int *slot_of;  // mixed path: slot of atom i in the cell order of the last build
  dbl4 *pos_ref; // skin mode: positions at the last build (displacement check)
  // LJ tables [i*nnbt + j]
  double *a6lj, *b12lj, *a6lj0, *b12lj0, *a6_14, *b12_14;
  float *a6f, *b12f, *a60f, *b120f, *a614f, *b1214f;
  float2 *abf;  // (A6, B12) FP32 pairs for the mixed sweeps: inter, intra, 1-4
  // bonded
  int nrbb, nraa, nrtt, nrbt, nrat, nrrt;
  int *bid, *bib, *bjb;
  double *brb, *bfb, *bdb, *bro;
  int *ibi, *jbj, *ibuk;
  double *ara, *afa;
  int *iai, *jaj, *kak, *iauk;
  int *titors, *tnmul;
  double *tft, *trt, *tft1, *tft2, *tft3, *tft4, *tft5;
  int *iti, *jtj, *ktk, *ltl, *ituk;
  double *br, *be, *ar, *ae, *tr, *te;
  // SHAKE (per type: first bond record, bond count)
  // Ewald
  int nkv, ncol, kx, ky, kz;  // table rows: n = 0..KMAX, 0..KMAY, 0..KMAZ
  int zstep;                    // z step of a column's records (2: truncated octahedron)
  int ldn;                      // row stride (atoms) of the FP32 tables, n rounded up to 128
  KCol *cols;
  void *kchunks;                // column chunks of the S(k) kernel
  int nchunk;
  double2 *tabx, *taby, *tabz;  // [n][atom], n >= 0 (negative n: conjugates)
  float2 *tabxf, *tabyf, *tabzf;
  double2 *sk;                  // structure factors, column order
  dbl4 *wk;                     // (W, RZV W) per k, W = AK2*conj(S)
  double *kconst;               // per k: AKC, RXV^2 AKV, RYV^2 AKV, RZV^2 AKV, RZV
  dbl4 *wp64;                   // FP64 paired W: 2 per (column, p), at poff + p
  float4 *wkf;                  // mixed paired W, grouped (KGroup)
  // mixed pair path: posi.w = (molecule << MDX_SITE_BITS) | site, and per
  // site {Q (EE-scaled), CHARGE, LJ type, molecule type} as float4 bits
  float4 *stab;
  int *pinfo;
  // small molecule types handled per molecule (bonds, angles); the instance
  // lists ibi.. / iai.. then hold only the other types' terms
  MolTpl *moltpl;
  int ntpl, ntpl_mol;
  KGroup *kgroups;              // column groups of the mixed force pass
  int ngroup;
  void *sitems;                 // work items of the mixed S(k) pass
  int nsitem;
  int sfac_slice, sfac_nslice;  // atoms per slice and slices of that pass
  // mixed tensor-core force pass: column slots (sorted by m, -1 = padding)
  // and K-steps per tile of 32 columns; B tiles (hi, lo) rebuilt per step
  bool tc_on;
  int *tc_slot, *tc_ks;
  float *tc_w;
  float4 *tc_meta;  // per slot {nx, ny, rv} for the epilogue
  unsigned char *tc_zimg;  // Z image (A operand), per 128-atom tile
  int tc_ntile, tc_kp;
  // mixed tensor-core S(k) pass: slice partials (FP32) and (column, p) items
  bool tcs_on;
  float *tcs_part;
  int *tcs_cp0;
  unsigned char *tcs_zimg;  // Z image (B operand), per 32-atom chunk
  double *tcs_red;          // partials reduced per M-tile (FP64)
  int tcs_np, tcs_ntm, tcs_nslice, tcs_slice, tcs_items, tcs_gps, tcs_ncg;
  int *rf_part;                 // group ranges of the mixed force pass's warps
  int rf_nsplit;                // blocks per atom tile of that pass
  double2 *colrv;               // per column (RXV, RYV) at the current box
  float2 *colrvf;
  double *kscal;                // per-k scratch of the energy/virial kernel
  // scalars and state blocks
  mdx_scalars *sc;
  mdx_thermo *th;
  mdx_step_record *rec;
  int rec_cap;
  int *err;
  int *shake_iter;   // [4..5]: list capacity needed after an overflow
  double *red;       // reduction scratch
  void *scal_scratch;  // SCALING stage scratch (integrate.cu)
  int *nspec_d;        // NSPEC per type
  double *red_part;    // per-block partials of the deterministic reductions
  unsigned *red_ctr;
  size_t red_cap;      // doubles in red_part
  double2 *sk_part;    // per-slice S(k) partials (deterministic slice sum)
  double *snap;        // mdx_snapshot: positions unpacked for the copy out (3n)
  double *avsum;       // mdx_set_averaging: running sums of the bonded statistics
  // SHEJK work: (molecule, cluster) items; per cluster (first slot, count)
  // into shk_rec, the cluster's constraint records in record order; a
  // failure flag per molecule
  int2 *shk_item, *shk_cl;
  int *shk_rec, *shk_mfail;
  int shk_nitem;
  // PULLBACK: restrained atoms and their wells; the device's NSTEP
  int *pull_atom;
  double *pull_ref;   // 3 x npull: x, y, z
  int *pull_step;
  size_t sk_part_cap;
};

struct mdx_ctx {
  mdx_dims d{};
  mdx_params p{};
  TypeConst tc{};
  PairConst pc{};
  DevData dv{};
  cudaStream_t stream = nullptr;
  int device = 0;
  int nsm = 1;  // SMs of the device: grid of the grid-stride reductions (one block each)
  double kc_box[5] = {-1.0, 0.0, 0.0, 0.0, 0.0};  // box, alpha^2, CFUR of dv.kconst
  int64_t launches = 0;
  bool have_topo = false, have_params = false, have_state = false,
       have_lists = false, have_com = false;
  std::string err;
  // host copies of what the host logic needs
  std::vector<int> h_itype, h_nnum, h_nsite;
  std::vector<double> h_charge, h_mass;
  int nspec[MDX_NT], nsits[MDX_NT], isadr[MDX_NT + 1], isaddr[MDX_NT + 1],
      iaddr[MDX_NT + 1], nrb[MDX_NT], iadb[MDX_NT], ishejk[MDX_NT];
  double summas[MDX_NT];
  std::vector<double> h_a6lj0, h_b12lj0, h_q, h_rb, h_fb, h_db, h_ro;
  std::vector<int> h_inbt;
  // box mirror (host), Ewald bookkeeping
  double boxl = 0, boyl = 0, bozl = 0;
  double boxlo = 0, boylo = 0, bozlo = 0;
  bool furir_init = false;
  int nkv = 0;
  double spei = 0, speei[MDX_NT]{};
  CellGrid grid{};
  double list_rl2 = 0;  // squared list radius used by the last build
  // reaction field: largest distance of an atom of a small molecule from the
  // molecule's centre of mass (+ 1 A for flexing), set at the state upload
  double mol_reach = 0;
  bool q_dirty = true;  // the device charges (pos.w) lag the host's (topology upload)
  FixScale fix{};
  // CUDA graphs of one long step: [rebuild?] + 2 * [records?] + 4 * [SULTAN?]
  cudaGraphExec_t gexec[8] = {};
  int64_t glaunches[8] = {};
  bool use_graphs = true;
  bool averaging = false;  // mdx_set_averaging: LAVER forces + statistics every long step
  // threads per owner atom of the mixed pair sweeps (0: not chosen yet;
  // source 1: the tuning table, 2: mdx_set_tuning)
  mdx_tuning tune{};
  bool pullback = false;   // mdx_set_pullback: drag, wells or field on
  mdx_pullback pb{};       // its constants (array pointers not kept)
  void drop_graphs() {
    for (auto &g : gexec)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }
  int mbsh = 0, mbln = 0;
  cudaEvent_t snap_ev[MDX_SNAPSHOT_SLOTS] = {};  // completion of mdx_snapshot per slot
  // device timers (mdx_set_timers)
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  struct Span {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<Span> spans;
  double t_ms[MDX_NTIMERS]{};
  int64_t t_cnt[MDX_NTIMERS]{};
  bool mixed() const { return d.precision == MDX_MIXED; }
  cudaEvent_t take_event() {
    if (ev_pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = ev_pool.back();
    ev_pool.pop_back();
    return e;
  }
};

// Period of the mixed path's fixed-point y coordinate (y / period * 2^32,
// kept modulo 2^32): BOYL, or 2 BOYL in the hexagonal cell, whose lattice
// holds (BOXL / 2, BOYL) and (0, 2 BOYL) but not (0, BOYL), so that the
// integer difference of two positions is always a lattice image of their
// separation.
inline double fix_period_y(const mdx_ctx *ctx) {
  return ctx->p.icell == 2 ? 2.0 * ctx->boyl : ctx->boyl;
}

// Reduction destinations for a launch of nblocks blocks reducing nv values:
// deterministic (partials + ordered sum) whenever the partials buffer is
// large enough.
inline Dst6 dst6(const mdx_ctx *ctx, size_t nblocks, int nv, double *a,
                 double *b = nullptr, double *c = nullptr, double *d = nullptr,
                 double *e = nullptr, double *f = nullptr) {
  Dst6 r{{a, b, c, d, e, f}, nullptr, nullptr};
  if (ctx->dv.red_part && nblocks * (size_t)nv <= ctx->dv.red_cap) {
    r.part = ctx->dv.red_part;
    r.ctr = ctx->dv.red_ctr;
  }
  return r;
}

// Brackets the launches of one scope with CUDA events when timers are on.
struct TimerScope {
  mdx_ctx *ctx;
  int id;
  cudaEvent_t a = nullptr;
  TimerScope(mdx_ctx *c, int i) : ctx(c), id(i) {
    if (ctx->timing) {
      a = ctx->take_event();
      cudaEventRecord(a, ctx->stream);
    }
  }
  ~TimerScope() {
    if (ctx->timing && a) {
      cudaEvent_t b = ctx->take_event();
      cudaEventRecord(b, ctx->stream);
      ctx->spans.push_back({id, a, b});
    }
  }
};
#define MDX_TIMER(ctx, id) TimerScope mdx_timer_scope_(ctx, id)

// --------------------------------------------------------------- helpers --
#define MDX_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return MDX_ERR_CUDA;                                                  \
    }                                                                       \
  } while (0)

#define MDX_LAUNCHED(ctx)                                                   \
  do {                                                                      \
    (ctx)->launches++;                                                      \
    cudaError_t e_ = cudaGetLastError();                                    \
    if (e_ != cudaSuccess) {                                                \
      (ctx)->err = std::string("launch: ") + cudaGetErrorString(e_);        \
      return MDX_ERR_CUDA;                                                  \
    }                                                                       \
  } while (0)

// Fortran SIGN(a, b) for b != -0 handling as gfortran on IEEE (sign bit).
__device__ __forceinline__ double fsign(double a, double b) {
  return copysign(fabs(a), b);
}
__device__ __forceinline__ float fsignf(float a, float b) {
  return copysignf(fabsf(a), b);
}

// Minimum image of the reference's inlined PBC for a rectangular cell
// (service.f:953-990 with LHEX = LOCT = false); hbz is the half box used for
// the z test (HBOXL in LOCALF, forces.f:871; HBOZL elsewhere).
__device__ __forceinline__ void pbc_rect(double &dx, double &dy, double &dz,
                                         double bx, double by, double bz,
                                         double hbx, double hby, double hbz) {
  if (fabs(dx) > hbx) dx = dx - fsign(bx, dx);
  if (fabs(dz) > hbz) dz = dz - fsign(bz, dz);
  if (fabs(dy) > hby) dy = dy - fsign(by, dy);
}
// Minimum image of the three cell shapes of PBC (service.f:953-990, and
// its inlined copies in LOCALF, FORCES, ETERMS and CHCNB): ICELL 0
// rectangular; 2 hexagonal (the x-y lattice (BOXL, 0), (HBOXL, BOYL), BOYL =
// BOXL cos30, minimum image up to 1.5 BOXL from the centre); 1 truncated
// octahedron (the cube's image, then the fold |x| + |y| + |z| < 0.75 BOXL).
// cos30 and 4/3 are the reference's REAL*4 literals (common_inc.f:33,
// service.f:985).  hbz: HBOZL, or HBOXL in LOCALF (forces.f:873).
struct CellPbc {
  int icell;
  double bx, by, bz, hbx, hby, hbz, boxy3;
};

__device__ __forceinline__ void pbc_cell(double &xx, double &yy, double &zz, const CellPbc &c,
                                         double hbz) {
  if (fabs(xx) > c.hbx) xx = xx - fsign(c.bx, xx);
  if (fabs(zz) > hbz) zz = zz - fsign(c.bz, zz);
  if (c.icell == 2) {
    const double cos30 = (double)0.8660254037844386f;
    const double boxyc = 0.5 / cos30;
    double xy = boxyc * xx;
    if (yy > c.boxy3 - xy && (xx > 0. || yy > 2. * c.boxy3 - xy)) {
      yy = yy - c.by;
      xx = xx - c.hbx;
      xy = boxyc * xx;
    }
    if (yy < -c.boxy3 - xy && (xx < 0. || yy < -2. * c.boxy3 - xy)) {
      yy = yy + c.by;
      xx = xx + c.hbx;
      xy = boxyc * xx;
    }
    if (yy > c.boxy3 + xy) {
      yy = yy - c.by;
      xx = xx + c.hbx;
      xy = boxyc * xx;
    }
    if (yy < -c.boxy3 + xy) {
      yy = yy + c.by;
      xx = xx - c.hbx;
    }
  } else {
    if (fabs(yy) > c.hby) yy = yy - fsign(c.by, yy);
  }
  if (c.icell == 1) {
    const double corss =
        c.hbx * (double)(int)((double)(4.0f / 3.0f) * (fabs(xx) + fabs(yy) + fabs(zz)) / c.bx);
    xx = xx - fsign(corss, xx);
    yy = yy - fsign(corss, yy);
    zz = zz - fsign(corss, zz);
  }
}
__device__ __forceinline__ void pbc_cell(double &xx, double &yy, double &zz, const CellPbc &c) {
  pbc_cell(xx, yy, zz, c, c.hbz);
}

__device__ __forceinline__ void pbc_rectf(float &dx, float &dy, float &dz,
                                          float bx, float by, float bz,
                                          float hbx, float hby, float hbz) {
  if (fabsf(dx) > hbx) dx = dx - fsignf(bx, dx);
  if (fabsf(dz) > hbz) dz = dz - fsignf(bz, dz);
  if (fabsf(dy) > hby) dy = dy - fsignf(by, dy);
}

// The non-rectangular cells' part of PBC (service.f:956-988) in FP32, for
// the mixed path's pair vectors, which arrive as fixed-point differences
// (x within +-BOXL/2, z within +-BOZL/2, y within +-BOYL in the hexagonal
// cell and +-BOYL/2 otherwise): the hexagonal cell's four tests in the
// reference's order, or the truncated octahedron's corner fold.  kind 0:
// rectangular, nothing to do.
struct CellF {
  int kind;  // ICELL
  float hbx, bx, by, boxy3, boxyc;
};
__device__ __forceinline__ void pbc_hexf(float &xx, float &yy, const CellF &h) {
  float xy = h.boxyc * xx;
  if (yy > h.boxy3 - xy && (xx > 0.f || yy > 2.f * h.boxy3 - xy)) {
    yy = yy - h.by;
    xx = xx - h.hbx;
    xy = h.boxyc * xx;
  }
  if (yy < -h.boxy3 - xy && (xx < 0.f || yy < -2.f * h.boxy3 - xy)) {
    yy = yy + h.by;
    xx = xx + h.hbx;
    xy = h.boxyc * xx;
  }
  if (yy > h.boxy3 + xy) {
    yy = yy - h.by;
    xx = xx + h.hbx;
    xy = h.boxyc * xx;
  }
  if (yy < -h.boxy3 + xy) {
    yy = yy + h.by;
    xx = xx - h.hbx;
  }
}
__device__ __forceinline__ void pbc_cellf(float &xx, float &yy, float &zz, const CellF &c) {
  if (c.kind == 2) {
    pbc_hexf(xx, yy, c);
  } else if (c.kind == 1) {  // CORSS: 4/3 is the reference's REAL*4 constant
    const float corss =
        c.hbx * (float)(int)((4.0f / 3.0f) * (fabsf(xx) + fabsf(yy) + fabsf(zz)) / c.bx);
    xx = xx - copysignf(corss, xx);
    yy = yy - copysignf(corss, yy);
    zz = zz - copysignf(corss, zz);
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NV doubles added to *dst[k] (null pointers skipped).  All
// threads of the block must call it.
//
// With a partials buffer the result is deterministic: every block stores its
// totals at part[block * NV + k], and the last block to finish (counted on
// *ctr) sums the partials in block order and adds once to dst, then resets
// the counter for the next launch on the stream.  Without one, each block
// adds with atomicAdd (order-dependent in the last bit).
// WARP_DONE: the caller has already summed each value over its warp (lane 0
// holds the warp totals), e.g. in FP32 for a few terms a thread.
// ROW: blocks of one grid row (blockIdx.y) reduce together, each row with its
// own part / ctr (batched launches over several systems).
template <int NV, bool WARP_DONE = false, bool ROW = false>
__device__ __forceinline__ void block_add_core(double (&v)[NV], double *const *dst,
                                               double *part, unsigned *ctr) {
  __shared__ double sh[32][NV];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  if (!WARP_DONE) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[wid][k] = v[k];
  }
  __syncthreads();
  const unsigned nblk = ROW ? gridDim.x : gridDim.x * gridDim.y;
  const unsigned blin = ROW ? blockIdx.x : blockIdx.y * gridDim.x + blockIdx.x;
  // the block's total of value k is formed by warp k % nw (the same sums in
  // the same order as one warp doing all of them, NV times shorter)
  for (int k = wid; k < NV; k += nw) {
    double t = lane < nw ? sh[lane][k] : 0.0;
    t = warp_sum(t);
    if (lane == 0) {
      if (part) {
        part[(size_t)blin * NV + k] = t;
        __threadfence();
      } else if (dst[k]) {
        atomicAdd(dst[k], t);
      }
    }
  }
  if (part) {
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ctr, 1u) == nblk - 1;
    __syncthreads();
    if (last) {
      __threadfence();
      for (int k = wid; k < NV; k += nw) {
        double t = 0.0;
        for (unsigned b = lane; b < nblk; b += 32) t += __ldcg(&part[(size_t)b * NV + k]);
        t = warp_sum(t);
        if (lane == 0 && dst[k]) *dst[k] += t;
      }
      if (threadIdx.x == 0) *ctr = 0u;
    }
  }
  __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_add(double (&v)[NV], const Dst6 &d) {
  block_add_core<NV>(v, d.p, d.part, d.ctr);
}

// Round-to-nearest-even float -> 64-bit integer from the bits of y with
// integer operations only: no conversion instruction (on this GPU those
// issue on the narrow FP64 pipe).  |y| = M 2^e with the 24-bit significand
// M; e >= 0 shifts left, -24 <= e < 0 shifts right and rounds half to even
// on the dropped bits, smaller e gives 0.  Equal to __float2ll_rn(y) for
// |y| < 2^63.
__device__ __forceinline__ long long f2ll_rn(float y) {
  const unsigned b = __float_as_uint(y);
  const int e = min((int)((b >> 23) & 0xffu) - 150, 39);
  const unsigned m = (b & 0x7fffffu) | 0x800000u;
  unsigned long long r = 0;
  if (e >= 0) {
    r = (unsigned long long)m << e;
  } else if (e >= -24) {
    const int s = -e;
    const unsigned q = m >> s, rem = m & ((1u << s) - 1u), half = 1u << (s - 1);
    r = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
  }
  return (b >> 31) ? -(long long)r : (long long)r;
}

// Wrapped difference a - b of two 32-bit fixed-point coordinates as FP32,
// times the scale s (box length / 2^32): the minimum-image vector component.
// (An exact integer + FMA replacement of the int-to-float conversion was
// measured slower in the pair sweeps, which are issue-bound: 0.39 against
// 0.37 ms per long-row sweep at 98,304 atoms.)
__device__ __forceinline__ float fixdiff(int a, int b, float s) {
  return (float)(int)((unsigned)a - (unsigned)b) * s;
}

// Low 32 bits of round-to-nearest-even(t) for |t| < 2^51: adding 1.5 x 2^52
// leaves the rounded integer in the low mantissa bits (the bias itself has
// none there).  One FP64 add instead of a 64-bit conversion; equal to
// (int)(unsigned long long)__double2ll_rn(t) in that range.  __dadd_rn keeps
// the compiler from fusing the add with the product that forms t.
__device__ __forceinline__ int fix32_rn(double t) {
  return __double2loint(__dadd_rn(t, 6755399441055744.0));
}

// Fixed-point force accumulation of the mixed path: two's complement in an
// unsigned 64-bit word, so that integer addition is associative and the sum
// is independent of the order of contributions.
__device__ __forceinline__ void fix_add(unsigned long long *a, double v,
                                        double scale) {
  long long q = __double2ll_rn(v * scale);
  atomicAdd(a, (unsigned long long)q);
}
__device__ __forceinline__ void fix_addf(unsigned long long *a, float v,
                                         float scale) {
  long long q = __float2ll_rn(v * scale);
  atomicAdd(a, (unsigned long long)q);
}

// Device memory of a context is stream-ordered (cudaMallocAsync /
// cudaFreeAsync on the context's stream): freeing never synchronises the
// whole device, so contexts can open and close while others run.  An
// allocation is followed by a sync of the context's own stream, so host-side
// copies into it may follow at once.
inline cudaError_t ctx_alloc(mdx_ctx *ctx, void **p, size_t bytes) {
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return e;
}
// Copy on a context's stream and wait: ordered after the stream's kernels
// (device-to-host reads see their results) and complete on return (host
// buffers may go away).  The contexts' streams are non-blocking, so a plain
// cudaMemcpy / cudaMemset on the legacy default stream would race with them.
inline cudaError_t ctx_copy(cudaStream_t s, void *dst, const void *src, size_t bytes,
                            cudaMemcpyKind kind) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}
template <typename T>
inline cudaError_t ctx_alloc(mdx_ctx *ctx, T **p, size_t bytes) {
  return ctx_alloc(ctx, reinterpret_cast<void **>(p), bytes);
}
inline void ctx_free(mdx_ctx *ctx, void *p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

// ---------------------------------------------------------- host launchers
// nblist.cu
int launch_build_lists(mdx_ctx *ctx);
int launch_list_update(mdx_ctx *ctx, int mstep);  // CHCNB when due (ICHNB or skin)
bool list_update_every_step(const mdx_ctx *ctx);  // skin mode: the update is in every step
int export_lists(mdx_ctx *ctx, int32_t *nbs1, int32_t *nbs2, int32_t cap_s,
                 int32_t *nbl1, int32_t *nbl2, int32_t cap_l);
// pair.cu
int launch_localf(mdx_ctx *ctx, bool split, bool ener = true);
int pack_lj_tables(mdx_ctx *ctx);  // abf from the FP32 tables
int launch_forces_long(mdx_ctx *ctx, bool split);
int launch_wir(mdx_ctx *ctx, int which);  // WIRSS (1) / WIRS (2)
// ewald.cu
int host_inifur(mdx_ctx *ctx);
int launch_furir(mdx_ctx *ctx);
int furir_sfac(mdx_ctx *ctx, bool *skip);  // k-set check, phase tables, S(k) into d.sk
int ensure_kconst(mdx_ctx *ctx);           // per-k constants of the current box
int launch_eterms(mdx_ctx *ctx);
int sfac_slices(const mdx_ctx *ctx);  // slices of the S(k) partial sums
// 1: set up; 0: the k-set's tiles do not fit (the CUDA-core pass runs);
// -1: a CUDA error (ctx->err says which step)
int tc_force_setup(mdx_ctx *ctx, const std::vector<KCol> &cols, int kmaz);
int tc_sfac_setup(mdx_ctx *ctx, const std::vector<KCol> &cols);
int tc_sfac_launch(mdx_ctx *ctx);
int tc_zimages_launch(mdx_ctx *ctx);
int tc_force_launch(mdx_ctx *ctx);
// Dynamic shared-memory limit of a kernel: process-wide, shared by every
// context, so it is only ever raised (under a lock).
cudaError_t raise_smem_limit_fn(const void *kernel, size_t bytes);
template <typename K>
cudaError_t raise_smem_limit(K kernel, size_t bytes) {
  return raise_smem_limit_fn(reinterpret_cast<const void *>(kernel), bytes);
}
// mdx_api.cu, for the allocation-free entry point in noalloc.cu
int api_require(mdx_ctx *ctx, bool topo, bool par, bool state);
int api_check_err(mdx_ctx *ctx);
int api_copy_scalars(mdx_ctx *ctx, mdx_scalars *out);
int api_do_slforces(mdx_ctx *ctx, bool split, bool mirrored = false);
int api_do_fforces(mdx_ctx *ctx, int laver, bool split, bool mirrored = false);
// bonded.cu: running sums of the per-record bonded statistics
int launch_acc_bonded(mdx_ctx *ctx);
int bonded_sums_len(const mdx_ctx *ctx);
// integrate.cu
int launch_zero_fast(mdx_ctx *ctx);
int launch_zero_slow(mdx_ctx *ctx);
int launch_fix_to_double(mdx_ctx *ctx, int which);  // mixed: int64 -> G/H
int launch_sclfrc(mdx_ctx *ctx, int nnn);
int launch_sum_forces(mdx_ctx *ctx);                // F = G + H
int launch_pullback(mdx_ctx *ctx);                  // PULLBACK into G
int launch_step_tick(mdx_ctx *ctx);                 // NSTEP += 1 on the device
int launch_getcom(mdx_ctx *ctx, bool mirror = false);  // mirror: refresh posf/posi too
int launch_getkin(mdx_ctx *ctx, const double *summd, double *out);  // EKTR, EKROT, TKE
int launch_chkmom(mdx_ctx *ctx, double sumasd, double *pt);        // removed momentum
// DOUBLE's kick + drift + GETCOM + mirrors in one pass (from_fix: fast
// forces read as fixed point, mixed path)
int launch_kick_drift_com(mdx_ctx *ctx, double htsteb, double tsteb, int prev, bool from_fix);
int launch_kick_drift(mdx_ctx *ctx, double htsteb, double tsteb, int prev);
int launch_record(mdx_ctx *ctx, int slot, int mstep);
int launch_getemp(mdx_ctx *ctx);
int launch_kick(mdx_ctx *ctx, int which, double h, bool apply_vscale);
int launch_kick2(mdx_ctx *ctx, int which1, double h1, int which2, double h2);
// a kick on forces w1 (1 H, 2 G, 3 F; 0 none) with h1, then w2 with h2
struct KickSpec {
  int w1 = 0;
  double h1 = 0.0;
  int w2 = 0;
  double h2 = 0.0;
  bool vscale = false;  // SCALING's per-type velocity factor first (GETEMP passes only)
};
int launch_getemp_kick(mdx_ctx *ctx, const KickSpec &pre, const KickSpec &post);
// PIMD bead ensembles: one device table entry per bead, then the integrator
// passes of all beads in one launch each (integrate.cu)
size_t bead_move_bytes();
void bead_move_fill(mdx_ctx *ctx, void *out);
int launch_getemp_beads(mdx_ctx *c0, int P, const void *table, cudaStream_t st,
                        const KickSpec &pre = {}, const KickSpec &post = {});
int launch_kick_drift_com_beads(mdx_ctx *c0, int P, const void *table, cudaStream_t st,
                                double htsteb, double tsteb);
int launch_vira(mdx_ctx *ctx, int from_viran);
// nblist.cu
int launch_mirror_f32(mdx_ctx *ctx);
int launch_cell_refresh(mdx_ctx *ctx);  // mixed: cell_pos from posi (after posi writers)
int upload_site_table(mdx_ctx *ctx);  // mdx_api.cu: stab from the current charges
