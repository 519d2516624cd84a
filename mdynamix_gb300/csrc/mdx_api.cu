// mdx_api.cu -- the C ABI of include/mdx_gpu.h: context lifetime, uploads,
// the force collectors FFORCES/SLFORCES/ALLFORCE (forces.f:36-100) and the
// DOUBLE / SULTAN step loops (mdstep.f:29-530), all device resident.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mdx_internal.cuh"

// integrate.cu
int launch_getemp(mdx_ctx *ctx);
int launch_scaling(mdx_ctx *ctx, int ial, bool *pending_vscale,
                   const KickSpec *kick_first = nullptr);
int launch_mstep1_rescale(mdx_ctx *ctx);
int launch_kick(mdx_ctx *ctx, int which, double h, bool apply_vscale);
int launch_leapfrog_shake(mdx_ctx *ctx);
int launch_vira(mdx_ctx *ctx, int from_viran);
size_t scal_scratch_bytes();
// bonded.cu
int launch_bonded(mdx_ctx *ctx, int laver, bool ener = true);

namespace {

#define RC(x)                \
  do {                       \
    int rc_ = (x);           \
    if (rc_) return rc_;     \
  } while (0)

template <typename T>
int dmalloc(mdx_ctx *ctx, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(p), sizeof(T) * n, ctx->stream);
  if (e != cudaSuccess) {
    ctx->err = std::string("cudaMallocAsync: ") + cudaGetErrorString(e);
    return MDX_ERR_NOMEM;
  }
  cudaMemsetAsync(*p, 0, sizeof(T) * n, ctx->stream);
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    ctx->err = std::string("allocation: ") + cudaGetErrorString(e);
    return MDX_ERR_CUDA;
  }
  return MDX_OK;
}

template <typename T>
int upload(mdx_ctx *ctx, T *dst, const T *src, size_t n) {
  if (!n) return MDX_OK;
  if (!src) {
    ctx->err = "null input array";
    return MDX_ERR_ARG;
  }
  MDX_CUDA(ctx_copy(ctx->stream, dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  return MDX_OK;
}

__global__ void k_com_only(int nop, const int *mol_first, const int *mol_nat,
                           const int *mol_type, const double *amass,
                           const dbl4 *pos, double *X, double *Y, double *Z,
                           const double *summas, double bx, double by,
                           double bz, CellPbc cell) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nop) return;
  const int f = mol_first[m], na = mol_nat[m];
  double x = 0., y = 0., z = 0.;
  for (int k = 0; k < na; ++k) {
    const dbl4 p = pos[f + k];
    x = x + amass[f + k] * p.x;
    y = y + amass[f + k] * p.y;
    z = z + amass[f + k] * p.z;
  }
  const double s = summas[mol_type[m]];
  x = x / s;
  y = y / s;
  z = z / s;
  if (cell.icell == 0) pbc_rect(x, y, z, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
  else pbc_cell(x, y, z, cell);
  X[m] = x;
  Y[m] = y;
  Z[m] = z;
}

__global__ void k_set_pos(int n, const double *sx, const double *sy,
                          const double *sz, const double *q, dbl4 *pos) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dbl4 p;
  p.x = sx[i];
  p.y = sy[i];
  p.z = sz[i];
  p.w = q ? q[i] : pos[i].w;  // q null: the charges already on the device stay
  pos[i] = p;
}

__global__ void k_get_pos(int n, const dbl4 *pos, double *sx, double *sy,
                          double *sz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const dbl4 p = pos[i];
  sx[i] = p.x;
  sy[i] = p.y;
  sz[i] = p.z;
}

__global__ void k_set_q(int n, const double *q, dbl4 *pos) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  pos[i].w = q[i];
}

int check_err(mdx_ctx *ctx) {
  int herr = 0;
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  MDX_CUDA(ctx_copy(ctx->stream, &herr, ctx->dv.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (!herr) return MDX_OK;
  MDX_CUDA(cudaMemsetAsync(ctx->dv.err, 0, sizeof(int), ctx->stream));
  if (herr & (DERR_LIST_SHORT | DERR_LIST_LONG)) {
    int need[2] = {0, 0};
    ctx_copy(ctx->stream, need, ctx->dv.shake_iter + 4, sizeof(int) * 2, cudaMemcpyDeviceToHost);
    char b[256];
    snprintf(b, sizeof b,
             "neighbour list overfilled: short row needs %d (cap %d), long row "
             "needs %d (cap %d); reopen with larger cap_short/cap_long",
             need[0], ctx->dv.cap_s, need[1], ctx->dv.cap_l);
    ctx->err = b;
    return MDX_ERR_LIST_OVERFLOW;
  }
  if (herr & DERR_TEMP) {
    ctx->err = "Temperature control stopped the program";
    return MDX_ERR_NAN;
  }
  if (herr & DERR_NAN) {
    ctx->err = "non-finite value";
    return MDX_ERR_NAN;
  }
  if (herr & DERR_NPT) {
    ctx->err = "repeated failure of NPT-algorithm";
    return MDX_ERR_NAN;
  }
  if (herr & DERR_TIMEOUT) {
    ctx->err = "a bounded wait of the tensor-core Ewald pass ran out";
    return MDX_ERR_TIMEOUT;
  }
  if (herr & DERR_SHAKE) {
    // the reference prints and continues (mdstep.f:1264-1269); the count is
    // in mdx_thermo.shake_fail
    return MDX_OK;
  }
  ctx->err = "device error";
  return MDX_ERR_CUDA;
}

int copy_scalars(mdx_ctx *ctx, mdx_scalars *out) {
  if (!out) return MDX_OK;
  MDX_CUDA(ctx_copy(ctx->stream, out, ctx->dv.sc, sizeof(mdx_scalars), cudaMemcpyDeviceToHost));
  out->nkv = ctx->nkv;
  return MDX_OK;
}

// fixed-point scales of the mixed path: a force count is 1e-10 kJ/mol/A and
// an energy count 1e-9 kJ/mol, rounded to powers of two
void set_fix_scales(mdx_ctx *ctx) {
  const double efact = ctx->p.efact > 0 ? ctx->p.efact : 1.0;
  const double fs = std::exp2(std::round(std::log2(1.0e10 / efact)));
  const double es = std::exp2(std::round(std::log2(1.0e9 / efact)));
  ctx->fix.scale = fs;
  ctx->fix.inv = 1.0 / fs;
  ctx->fix.escale = es;
  ctx->fix.einv = 1.0 / es;
  ctx->fix.scalef = (float)fs;
  ctx->fix.escalef = (float)es;
}

int require(mdx_ctx *ctx, bool topo, bool par, bool state) {
  if ((topo && !ctx->have_topo) || (par && !ctx->have_params) ||
      (state && !ctx->have_state)) {
    ctx->err = "call order: topology, parameters and state must be uploaded first";
    return MDX_ERR_STATE;
  }
  return MDX_OK;
}

// ---------------------------------------------------------------- forces
// ener = false: an intermediate short step of DOUBLE, whose fast energies
// and virials the next FFORCES zeroes before anything reads them; the pair
// sweep then computes forces only, and on the mixed path nothing needs
// zeroing (the short sweep stores every atom's fixed-point force before the
// bonded terms add to it).  mirrored: GETCOM has just refreshed the FP32 and
// fixed-point mirrors of the positions.
int do_fforces(mdx_ctx *ctx, int laver, bool split, bool ener = true, bool mirrored = false,
               bool fold = true) {
  if (ener || !ctx->mixed()) RC(launch_zero_fast(ctx));
  if (ctx->mixed() && !mirrored) RC(launch_mirror_f32(ctx));
  RC(launch_localf(ctx, split, ener));
  if (ener) RC(launch_wir(ctx, 1));  // WIRSS from the pair forces, before the bonded terms
  RC(launch_bonded(ctx, laver, ener));
  // fold = false: the next step's kick reads the fixed-point forces itself
  if (ctx->mixed() && fold) RC(launch_fix_to_double(ctx, 1));
  RC(launch_sclfrc(ctx, 1));
  return MDX_OK;
}

int do_slow_parts(mdx_ctx *ctx, bool split, bool mirrored = false) {
  if (ctx->mixed()) {
    if (!mirrored) RC(launch_mirror_f32(ctx));
    RC(launch_forces_long(ctx, split));  // stores G first
    RC(launch_furir(ctx));
    RC(launch_eterms(ctx));
    RC(launch_fix_to_double(ctx, 2));
  } else {
    RC(launch_furir(ctx));
    RC(launch_eterms(ctx));
    RC(launch_forces_long(ctx, split));
  }
  return MDX_OK;
}

int do_slforces(mdx_ctx *ctx, bool split, bool mirrored = false) {
  RC(launch_zero_slow(ctx));
  RC(do_slow_parts(ctx, split, mirrored));
  RC(launch_wir(ctx, 2));
  RC(launch_pullback(ctx));
  RC(launch_sclfrc(ctx, 2));
  return MDX_OK;
}

int do_allforce(mdx_ctx *ctx, bool split, bool laver = false) {
  RC(launch_zero_fast(ctx));
  RC(launch_zero_slow(ctx));
  if (ctx->mixed()) RC(launch_mirror_f32(ctx));
  RC(launch_localf(ctx, split));
  RC(launch_wir(ctx, 1));  // WIRSS from the pair forces, before the bonded terms
  RC(launch_bonded(ctx, split || laver ? 1 : 0));
  if (ctx->mixed()) RC(launch_fix_to_double(ctx, 1));
  RC(do_slow_parts(ctx, split));
  RC(launch_wir(ctx, 2));
  RC(launch_sum_forces(ctx));
  // PULLBACK adds to G after CM_ADDLA has formed F (forces.f:88-95): SULTAN,
  // which moves with F, does not see it -- the reference's order, kept
  RC(launch_pullback(ctx));
  RC(launch_sclfrc(ctx, 3));
  return MDX_OK;
}

int sync_box_from_device(mdx_ctx *ctx) {
  double b[3];
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  MDX_CUDA(ctx_copy(ctx->stream, b, &ctx->dv.th->boxl, sizeof b, cudaMemcpyDeviceToHost));
  ctx->boxl = b[0];
  ctx->boyl = b[1];
  ctx->bozl = b[2];
  return MDX_OK;
}

// one long step of DOUBLE (mdstep.f:324-436)
int double_step(mdx_ctx *ctx, int mstep, int slot) {
  const mdx_params &p = ctx->p;
  const int NFREQ = p.nfreq, NFREQ2 = NFREQ / 2 + 1;
  const double HTSTEP = 0.5 * p.tstep, TSTEB = p.tsteb, HTSTEB = 0.5 * p.tsteb;
  bool pend = false;
  RC(launch_step_tick(ctx));  // NSTEP = NSTEP + 1 (mdstep.f:325)
  RC(launch_scaling(ctx, 1, &pend));
  if (p.lnpt) RC(sync_box_from_device(ctx));
  RC(launch_kick(ctx, 2, HTSTEP, pend));
  // mixed path, intermediate short steps: the fast forces stay in fixed
  // point (no fold) unless SCLFRC needs them in FP64
  const bool keep_fix = ctx->mixed() && !p.lscft;
  for (int s = 1; s <= NFREQ; ++s) {
    // kick, drift, GETCOM and the mirrors; positions then stay put until the
    // next short step
    RC(launch_kick_drift_com(ctx, HTSTEB, TSTEB, s > 1 ? 1 : 0, keep_fix && s > 1));
    if (s == NFREQ2) RC(launch_list_update(ctx, mstep));
    if (s == NFREQ) {
      RC(do_slforces(ctx, false, true));
      // the bonded statistics of the step (GETBND..GETTRS form them at every
      // FFORCES, forces.f:113-513) when averages are kept on the device
      RC(do_fforces(ctx, ctx->averaging ? 1 : 0, false, true, true));
      if (ctx->averaging) RC(launch_acc_bonded(ctx));
    } else {
      RC(do_fforces(ctx, 0, false, false, true, !keep_fix));
    }
  }
  // the two closing half kicks (mdstep.f:405-430) in SCALING(2)'s first GETEMP pass
  const KickSpec closing{1, HTSTEB, 2, HTSTEP};
  RC(launch_scaling(ctx, 2, nullptr, &closing));
  if (p.lnpt) RC(sync_box_from_device(ctx));
  if (slot != -2) RC(launch_record(ctx, slot, mstep));  // -1: device counters
  return MDX_OK;
}

// one step of SULTAN (mdstep.f:83-162)
int sultan_step(mdx_ctx *ctx, int mstep, int slot) {
  const mdx_params &p = ctx->p;
  RC(launch_step_tick(ctx));  // NSTEP = NSTEP + 1 (mdstep.f:75)
  RC(launch_leapfrog_shake(ctx));
  if (mstep == 1) RC(launch_mstep1_rescale(ctx));
  RC(launch_vira(ctx, 1));
  RC(launch_scaling(ctx, 3, nullptr));
  if (p.lnpt) RC(sync_box_from_device(ctx));
  RC(launch_getcom(ctx));
  RC(launch_list_update(ctx, mstep));
  RC(do_allforce(ctx, false, ctx->averaging));
  if (ctx->averaging) RC(launch_acc_bonded(ctx));
  if (slot != -2) RC(launch_record(ctx, slot, mstep));  // -1: device counters
  return MDX_OK;
}

int ensure_records(mdx_ctx *ctx, int n) {
  if (n <= ctx->dv.rec_cap) return MDX_OK;
  ctx_free(ctx, ctx->dv.rec);
  RC(dmalloc(ctx, &ctx->dv.rec, (size_t)n));
  ctx->dv.rec_cap = n;
  return MDX_OK;
}

// One DOUBLE or SULTAN long step replayed from its captured graph
// (captured on first use; four variants each: list rebuild or not x
// records or not).
int graph_step(mdx_ctx *ctx, int mstep, bool rec, bool dbl) {
  const bool list = list_update_every_step(ctx) || mstep % ctx->p.ichnb == 0;
  const int g = (list ? 1 : 0) + (rec ? 2 : 0) + (dbl ? 0 : 4);
  if (!ctx->gexec[g]) {
    const int64_t l0 = ctx->launches;
    MDX_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = dbl ? double_step(ctx, mstep, rec ? -1 : -2) : sultan_step(ctx, mstep, rec ? -1 : -2);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) {
      ctx->err = std::string("graph capture: ") + cudaGetErrorString(e);
      return MDX_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&ctx->gexec[g], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      ctx->gexec[g] = nullptr;
      ctx->err = std::string("graph instantiate: ") + cudaGetErrorString(e);
      return MDX_ERR_CUDA;
    }
    ctx->glaunches[g] = ctx->launches - l0;
    ctx->launches = l0;
  }
  MDX_CUDA(cudaGraphLaunch(ctx->gexec[g], ctx->stream));
  ctx->launches += ctx->glaunches[g];
  return MDX_OK;
}

int run_steps(mdx_ctx *ctx, bool dbl, int32_t nsteps, int32_t mstep0,
              mdx_step_record *rec) {
  RC(require(ctx, true, true, true));
  if (!ctx->have_lists) {
    ctx->err = "neighbour lists not built (call the prologue first)";
    return MDX_ERR_STATE;
  }
  if (rec) RC(ensure_records(ctx, nsteps));
  // CUDA-graph replay of whole long steps: DOUBLE and SULTAN at constant
  // volume have a fixed launch sequence, with or without the list rebuild
  // (SULTAN's first step, with its temperature rescale, runs eagerly).
  const bool graphs = !ctx->p.lnpt && !ctx->timing && ctx->use_graphs;
  if (graphs && rec) {
    int c0[2] = {0, mstep0 + 1};
    MDX_CUDA(cudaMemcpyAsync(ctx->dv.shake_iter + 16, c0, sizeof c0, cudaMemcpyHostToDevice,
                             ctx->stream));
    MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  for (int s = 1; s <= nsteps; ++s) {
    const int mstep = mstep0 + s;
    if (graphs && (dbl || mstep != 1)) {
      RC(graph_step(ctx, mstep, rec != nullptr, dbl));
    } else if (dbl) {
      RC(double_step(ctx, mstep, rec ? s - 1 : -2));
    } else {
      // with graphs on, the records' slot counter on the device is in use
      RC(sultan_step(ctx, mstep, rec ? (graphs ? -1 : s - 1) : -2));
    }
  }
  RC(check_err(ctx));
  if (rec) {
    MDX_CUDA(ctx_copy(ctx->stream, rec, ctx->dv.rec, sizeof(mdx_step_record) * nsteps,
                        cudaMemcpyDeviceToHost));
  }
  return MDX_OK;
}

}  // namespace

// ================================================================== C ABI
extern "C" {

int mdx_version(void) { return 1; }

const char *mdx_strerror(int code) {
  switch (code) {
    case MDX_OK: return "ok";
    case MDX_ERR_ARG: return "bad argument";
    case MDX_ERR_CUDA: return "CUDA error";
    case MDX_ERR_LIST_OVERFLOW: return "neighbour list overflow";
    case MDX_ERR_SHAKE: return "SHAKE did not converge";
    case MDX_ERR_NAN: return "non-finite value or watchdog";
    case MDX_ERR_TIMEOUT: return "device wait timed out";
    case MDX_ERR_STATE: return "call order";
    case MDX_ERR_NOMEM: return "device allocation failed";
    case MDX_ERR_KVEC: return "too many k-vectors";
    case MDX_ERR_UNSUPPORTED: return "unsupported option";
  }
  return "unknown";
}

const char *mdx_last_error(const mdx_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

int mdx_open(const mdx_dims *dims, mdx_ctx **out) {
  if (!dims || !out) return MDX_ERR_ARG;
  *out = nullptr;
  if (dims->nstot <= 0 || dims->nop <= 0 || dims->ntypes <= 0 ||
      dims->ntypes > MDX_NT || dims->nnbt <= 0 || dims->nsites <= 0 ||
      (dims->precision != MDX_FP64 && dims->precision != MDX_MIXED))
    return MDX_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MDX_ERR_CUDA;
  mdx_ctx *ctx = new (std::nothrow) mdx_ctx();
  if (!ctx) return MDX_ERR_NOMEM;
  ctx->d = *dims;
  if (ctx->d.cap_short <= 0) ctx->d.cap_short = 64;
  if (ctx->d.cap_long <= 0) ctx->d.cap_long = 1000;
  if (ctx->d.nkv_max <= 0) ctx->d.nkv_max = 100000;
  if (ctx->d.precision == MDX_MIXED) {  // full rows hold both copies of a pair
    ctx->d.cap_short *= 2;
    ctx->d.cap_long *= 2;
  }
  cudaGetDevice(&ctx->device);
  if (cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device) !=
          cudaSuccess ||
      ctx->nsm < 1)
    ctx->nsm = 1;
  {
    const char *g = getenv("MDX_GRAPHS");
    if (g && g[0] == '0') ctx->use_graphs = false;
  }
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return MDX_ERR_CUDA;
  }
  DevData &d = ctx->dv;
  const size_t n = dims->nstot;
  d.n = dims->nstot;
  d.nop = dims->nop;
  d.ntypes = dims->ntypes;
  d.nnbt = dims->nnbt;
  d.nbdmax = std::max(1, dims->nbdmax);
  d.cap_s = ctx->d.cap_short;
  d.cap_l = ctx->d.cap_long;
  int rc = MDX_OK;
#define AL(p, cnt) \
  if (!rc) rc = dmalloc(ctx, &p, cnt)
  AL(d.pos, n);
  AL(d.posf, n);
  AL(d.posi, n);
  AL(d.qsitef, n);
  AL(d.vx, 3 * n);
  AL(d.massdi, n);
  AL(d.amass, n);
  AL(d.qsite, n);
  AL(d.ainfo, n);
  AL(d.nnbb, n);
  AL(d.inbb, n * d.nbdmax);
  AL(d.mol_first, (size_t)dims->nop);
  AL(d.mol_nat, (size_t)dims->nop);
  AL(d.mol_type, (size_t)dims->nop);
  AL(d.X, 3 * (size_t)dims->nop);
  AL(d.gx, 9 * n);
  AL(d.ox, 3 * n);
  AL(d.ns_cnt, n);
  AL(d.nl_cnt, n);
  // mixed short rows are tiled by 32 atoms (list_slot): whole tiles stored
  const size_t nrow = dims->precision == MDX_MIXED ? (n + 31) / 32 * 32 : n;
  AL(d.ns_idx, nrow * d.cap_s);
  AL(d.nl_idx, n * d.cap_l);
  AL(d.atom_cell, n);
  AL(d.cell_list, n);
  AL(d.cell_pos, n);
  AL(d.slot_of, n);
  AL(d.sc, 1);
  AL(d.th, 1);
  AL(d.err, 4);
  AL(d.shake_iter, 32);
  AL(d.red, 512);
  AL(d.red_part, (size_t)1 << 21);
  AL(d.red_ctr, 8);
  d.red_cap = (size_t)1 << 21;
  if (!rc) {
    unsigned char *ss = nullptr;
    rc = dmalloc(ctx, &ss, scal_scratch_bytes());
    d.scal_scratch = ss;
  }
  if (!rc && dims->precision == MDX_MIXED) {
    AL(d.gfix, 3 * n);
    AL(d.hfix, 3 * n);
  }
#undef AL
  if (rc) {
    std::string e = ctx->err;
    mdx_close(ctx);
    return rc;
  }
  d.vy = d.vx + n;
  d.vz = d.vy + n;
  d.Y = d.X + dims->nop;
  d.Z = d.Y + dims->nop;
  d.gy = d.gx + n;
  d.gz = d.gy + n;
  d.hx = d.gz + n;
  d.hy = d.hx + n;
  d.hz = d.hy + n;
  d.fx = d.hz + n;
  d.fy = d.fx + n;
  d.fz = d.fy + n;
  d.oy = d.ox + n;
  d.oz = d.oy + n;
  *out = ctx;
  return MDX_OK;
}

int mdx_close(mdx_ctx *ctx) {
  if (!ctx) return MDX_OK;
  DevData &d = ctx->dv;
  void *ptrs[] = {d.pos, d.posf, d.posi, d.qsitef, d.stab, d.pinfo, d.moltpl, d.vx, d.massdi, d.amass, d.qsite,
                  d.ainfo, d.nnbb, d.inbb, d.mol_first, d.mol_nat, d.mol_type, d.X,
                  d.gx, d.ox, d.gfix, d.hfix, d.ns_cnt, d.nl_cnt, d.ns_idx, d.nl_idx,
                  d.cell_cnt, d.cell_start, d.cell_list, d.cell_pos, d.slot_of, d.pos_ref, d.atom_cell, d.a6lj, d.a6f, d.abf,
                  d.bid, d.brb, d.ibi, d.ara, d.iai, d.titors, d.tft, d.iti, d.br,
                  d.ar, d.tr, d.cols, d.kchunks, d.kgroups, d.kconst, d.rf_part, d.tc_slot, d.tc_w, d.tc_meta, d.tcs_part, d.tcs_cp0, d.tc_zimg, d.tcs_zimg, d.tcs_red, d.sitems, d.tabx, d.tabxf, d.sk, d.sc, d.th,
                  d.rec, d.err, d.shake_iter, d.red, d.scal_scratch, d.nspec_d,
                  d.red_part, d.red_ctr, d.sk_part, d.snap, d.avsum, d.shk_item,
                  d.shk_cl, d.shk_rec, d.shk_mfail, d.pull_atom, d.pull_ref, d.pull_step};
  if (ctx->stream) {
    for (void *p : ptrs) ctx_free(ctx, p);
    cudaStreamSynchronize(ctx->stream);
  }
  ctx->drop_graphs();
  for (auto e : ctx->snap_ev)
    if (e) cudaEventDestroy(e);
  for (auto &sp : ctx->spans) {
    cudaEventDestroy(sp.a);
    cudaEventDestroy(sp.b);
  }
  for (auto e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MDX_OK;
}

// Bonds and angles of small molecule types (at most ML_MAXS sites, no
// STRBND water potential, no torsions, the same terms in every molecule, in
// BNDLST's per-molecule order) become one template per type for the
// molecule-local kernel; every other instance stays in the lists.
static int split_bonded(mdx_ctx *ctx, const mdx_topo *t) {
  DevData &d = ctx->dv;
  const int nt = ctx->d.ntypes, nb_all = ctx->d.nrbt, na_all = ctx->d.nrat;
  std::vector<char> ok(nt, 0);
  std::vector<MolTpl> tpl(nt);
  std::vector<int> first(nt), nsit(nt);
  for (int k = 0; k < nt; ++k) {
    first[k] = t->isaddr[k];
    nsit[k] = t->nsits[k];
    ok[k] = t->nsits[k] <= ML_MAXS && t->ipot[k] != 1 && t->ipot[k] != 2 && t->nspec[k] > 0;
    MolTpl &m = tpl[k];
    std::memset(&m, 0, sizeof m);
    m.first = first[k];
    m.nmol = t->nspec[k];
    m.nsit = nsit[k];
    m.type = k;
  }
  auto typ = [&](int atom0) { return t->itype[atom0] - 1; };
  for (int N = 0; N < ctx->d.nrrt; ++N) ok[typ(t->iti[N] - 1)] = 0;
  // templates from each type's first molecule
  for (int N = 0; N < nb_all; ++N) {
    const int I = t->ibi[N] - 1, J = t->jbj[N] - 1, k = typ(I);
    if (!ok[k] || I - first[k] >= nsit[k]) continue;
    MolTpl &m = tpl[k];
    if (m.nb == ML_MAXB || J - first[k] >= nsit[k] || J < first[k]) { ok[k] = 0; continue; }
    m.bi[m.nb] = (unsigned char)(I - first[k]);
    m.bj[m.nb] = (unsigned char)(J - first[k]);
    m.bm[m.nb] = (short)(t->ibuk[N] - 1);
    ++m.nb;
  }
  for (int N = 0; N < na_all; ++N) {
    const int I = t->iai[N] - 1, J = t->jaj[N] - 1, K = t->kak[N] - 1, k = typ(I);
    if (!ok[k] || I - first[k] >= nsit[k]) continue;
    MolTpl &m = tpl[k];
    if (m.na == ML_MAXA || J < first[k] || K < first[k] || J - first[k] >= nsit[k] ||
        K - first[k] >= nsit[k]) { ok[k] = 0; continue; }
    m.ai[m.na] = (unsigned char)(I - first[k]);
    m.aj[m.na] = (unsigned char)(J - first[k]);
    m.ak[m.na] = (unsigned char)(K - first[k]);
    m.am[m.na] = (short)(t->iauk[N] - 1);
    ++m.na;
  }
  // every molecule must repeat its type's template in order
  std::vector<int> seen(nt, 0);
  for (int N = 0; N < nb_all; ++N) {
    const int I = t->ibi[N] - 1, k = typ(I);
    if (!ok[k]) continue;
    const MolTpl &m = tpl[k];
    const int q = seen[k]++, b = m.nb ? q % m.nb : 0, base = first[k] + (m.nb ? q / m.nb : 0) * nsit[k];
    if (!m.nb || I != base + m.bi[b] || t->jbj[N] - 1 != base + m.bj[b] || t->ibuk[N] - 1 != m.bm[b])
      ok[k] = 0;
  }
  for (int k = 0; k < nt; ++k)
    if (ok[k] && seen[k] != tpl[k].nb * tpl[k].nmol) ok[k] = 0;
  std::fill(seen.begin(), seen.end(), 0);
  for (int N = 0; N < na_all; ++N) {
    const int I = t->iai[N] - 1, k = typ(I);
    if (!ok[k]) continue;
    const MolTpl &m = tpl[k];
    const int q = seen[k]++, a = m.na ? q % m.na : 0, base = first[k] + (m.na ? q / m.na : 0) * nsit[k];
    if (!m.na || I != base + m.ai[a] || t->jaj[N] - 1 != base + m.aj[a] ||
        t->kak[N] - 1 != base + m.ak[a] || t->iauk[N] - 1 != m.am[a])
      ok[k] = 0;
  }
  for (int k = 0; k < nt; ++k)
    if (ok[k] && seen[k] != tpl[k].na * tpl[k].nmol) ok[k] = 0;
  // templates in use and the remaining instance lists
  std::vector<MolTpl> use;
  for (int k = 0; k < nt; ++k)
    if (ok[k] && (tpl[k].nb || tpl[k].na)) use.push_back(tpl[k]);
    else ok[k] = 0;
  std::vector<int> bi, bj, bm, ai, aj, ak, am;
  for (int N = 0; N < nb_all; ++N)
    if (!ok[typ(t->ibi[N] - 1)]) {
      bi.push_back(t->ibi[N] - 1);
      bj.push_back(t->jbj[N] - 1);
      bm.push_back(t->ibuk[N] - 1);
    }
  for (int N = 0; N < na_all; ++N)
    if (!ok[typ(t->iai[N] - 1)]) {
      ai.push_back(t->iai[N] - 1);
      aj.push_back(t->jaj[N] - 1);
      ak.push_back(t->kak[N] - 1);
      am.push_back(t->iauk[N] - 1);
    }
  d.nrbt = (int)bi.size();
  d.nrat = (int)ai.size();
  if (d.nrbt) {
    RC(upload(ctx, d.ibi, bi.data(), d.nrbt));
    RC(upload(ctx, d.jbj, bj.data(), d.nrbt));
    RC(upload(ctx, d.ibuk, bm.data(), d.nrbt));
  }
  if (d.nrat) {
    RC(upload(ctx, d.iai, ai.data(), d.nrat));
    RC(upload(ctx, d.jaj, aj.data(), d.nrat));
    RC(upload(ctx, d.kak, ak.data(), d.nrat));
    RC(upload(ctx, d.iauk, am.data(), d.nrat));
  }
  ctx_free(ctx, d.moltpl);
  d.moltpl = nullptr;
  d.ntpl = (int)use.size();
  d.ntpl_mol = 0;
  for (const MolTpl &m : use) d.ntpl_mol += m.nmol;
  if (d.ntpl) {
    RC(dmalloc(ctx, &d.moltpl, use.size()));
    RC(upload(ctx, d.moltpl, use.data(), use.size()));
  }
  return MDX_OK;
}

// SHEJK work items.  A molecule type's constraints (records flagged in
// lcon, or with ID != 2) fall into clusters connected through shared atoms;
// updates in one cluster never touch another's atoms, so each cluster can
// run the reference's sweeps on its own (see k_shake_cluster).  One item
// per (molecule, cluster); clusters list their records in record order.
static int shake_clusters(mdx_ctx *ctx, const mdx_topo *t) {
  DevData &d = ctx->dv;
  std::vector<int> rec;
  std::vector<int2> cl, items;
  for (int k = 0; k < ctx->d.ntypes; ++k) {
    const int nb = t->nrb[k], ns = t->nsits[k], nb0 = t->iadb[k] - 1;
    if (nb <= 0 || ns > 128) continue;
    std::vector<int> root(ns);
    for (int a = 0; a < ns; ++a) root[a] = a;
    auto find = [&](int a) {
      while (root[a] != a) a = root[a] = root[root[a]];
      return a;
    };
    auto con = [&](int b) { return t->lcon ? t->lcon[nb0 + b] != 0 : t->id[nb0 + b] != 2; };
    for (int b = 0; b < nb; ++b)
      if (con(b)) {
        const int x = find(t->ib[nb0 + b] - 1), y = find(t->jb[nb0 + b] - 1);
        if (x != y) root[std::max(x, y)] = std::min(x, y);
      }
    std::vector<int> cid(ns, -1);
    const int c0 = (int)cl.size();
    for (int b = 0; b < nb; ++b) {
      if (!con(b)) continue;
      const int r = find(t->ib[nb0 + b] - 1);
      if (cid[r] < 0) {
        cid[r] = (int)cl.size();
        cl.push_back(make_int2(0, 0));
      }
    }
    // records of each cluster, in record order
    for (int c = c0; c < (int)cl.size(); ++c) {
      cl[c].x = (int)rec.size();
      for (int b = 0; b < nb; ++b)
        if (con(b) && cid[find(t->ib[nb0 + b] - 1)] == c) rec.push_back(nb0 + b);
      cl[c].y = (int)rec.size() - cl[c].x;
    }
    for (int mm = 0; mm < t->nspec[k]; ++mm)
      for (int c = c0; c < (int)cl.size(); ++c) items.push_back(make_int2(t->iaddr[k] + mm, c));
  }
  ctx_free(ctx, d.shk_item);
  ctx_free(ctx, d.shk_cl);
  ctx_free(ctx, d.shk_rec);
  d.shk_item = d.shk_cl = nullptr;
  d.shk_rec = nullptr;
  d.shk_nitem = (int)items.size();
  if (!d.shk_mfail) RC(dmalloc(ctx, &d.shk_mfail, (size_t)d.nop));
  if (d.shk_nitem) {
    RC(dmalloc(ctx, &d.shk_item, items.size()));
    RC(dmalloc(ctx, &d.shk_cl, cl.size()));
    RC(dmalloc(ctx, &d.shk_rec, rec.size()));
    RC(upload(ctx, d.shk_item, items.data(), items.size()));
    RC(upload(ctx, d.shk_cl, cl.data(), cl.size()));
    RC(upload(ctx, d.shk_rec, rec.data(), rec.size()));
  }
  return MDX_OK;
}

int mdx_upload_topology(mdx_ctx *ctx, const mdx_topo *t) {
  if (!ctx || !t) return MDX_ERR_ARG;
  DevData &d = ctx->dv;
  const int n = d.n, nt = ctx->d.ntypes, ns = ctx->d.nsites, nb = ctx->d.nnbt;
  ctx->h_itype.assign(t->itype, t->itype + n);
  ctx->h_nnum.assign(t->nnum, t->nnum + n);
  ctx->h_nsite.assign(t->nsite, t->nsite + n);
  ctx->h_charge.assign(t->charge, t->charge + ns);
  ctx->h_mass.assign(t->mass, t->mass + ns);
  for (int i = 0; i < n; ++i)
    if (t->itype[i] < 1 || t->itype[i] > nt || t->nnum[i] < 1 ||
        t->nnum[i] > ctx->d.nop || t->nsite[i] < 1 || t->nsite[i] > ns) {
      ctx->err = "ITYPE/NNUM/NSITE out of range";
      return MDX_ERR_ARG;
    }
  // per type
  TypeConst &tc = ctx->tc;
  tc = TypeConst{};
  tc.ntypes = nt;
  for (int k = 0; k < nt; ++k) {
    tc.lmove[k] = t->lmove[k];
    tc.iee[k] = t->iee[k];
    tc.ipot[k] = t->ipot[k];
    tc.c14el[k] = t->c14el[k];
    tc.c14lj[k] = t->c14lj[k];
    tc.c14elf[k] = (float)t->c14el[k];
    tc.c14ljf[k] = (float)t->c14lj[k];
    for (int j = 0; j < nt; ++j) tc.mdx[k][j] = t->mdx[(size_t)k + (size_t)j * t->ld_mdx] - 1;
    ctx->nspec[k] = t->nspec[k];
    ctx->nsits[k] = t->nsits[k];
    ctx->isadr[k] = t->isadr[k];
    ctx->isaddr[k] = t->isaddr[k];
    ctx->iaddr[k] = t->iaddr[k];
    ctx->nrb[k] = t->nrb[k];
    ctx->iadb[k] = t->iadb[k];
    ctx->ishejk[k] = t->ishejk[k];
    ctx->summas[k] = t->summas[k];
  }
  // per atom
  std::vector<int4> ai(n);
  std::vector<double> amass(n), qsite(n);
  std::vector<float> qsitef(n);
  for (int i = 0; i < n; ++i) {
    const int site = t->nsite[i] - 1;
    ai[i] = make_int4(t->itype[i] - 1, t->nnum[i] - 1, t->inbt[site] - 1, site);
    amass[i] = t->mass[site];
    qsite[i] = t->charge[site];
    qsitef[i] = (float)t->charge[site];
  }
  RC(upload(ctx, d.ainfo, ai.data(), n));
  RC(upload(ctx, d.massdi, t->massdi, n));
  RC(upload(ctx, d.amass, amass.data(), n));
  RC(upload(ctx, d.qsite, qsite.data(), n));
  RC(upload(ctx, d.qsitef, qsitef.data(), n));
  ctx->h_q.assign(t->q, t->q + n);
  ctx->q_dirty = true;
  if (ctx->mixed()) {
    if (ns >= (1 << MDX_SITE_BITS) || d.nop >= (1 << (32 - MDX_SITE_BITS))) {
      ctx->err = "mixed path: at most 8191 sites and 524287 molecules";
      return MDX_ERR_UNSUPPORTED;
    }
    std::vector<int> pinfo(n);
    for (int i = 0; i < n; ++i)
      pinfo[i] = (int)(((unsigned)(t->nnum[i] - 1) << MDX_SITE_BITS) | (unsigned)(t->nsite[i] - 1));
    RC(dmalloc(ctx, &d.pinfo, n));
    RC(dmalloc(ctx, &d.stab, (size_t)ns));
    RC(upload(ctx, d.pinfo, pinfo.data(), n));
  }
  // molecules: atoms are contiguous per molecule, molecules per type
  std::vector<int> mf(d.nop, -1), mn(d.nop, 0), mt(d.nop, 0);
  for (int i = 0; i < n; ++i) {
    const int m = t->nnum[i] - 1;
    if (mf[m] < 0) mf[m] = i;
    mn[m] += 1;
    mt[m] = t->itype[i] - 1;
  }
  for (int m = 0; m < d.nop; ++m)
    if (mn[m] > 128) {
      ctx->err = "molecules above 128 atoms are not supported by SHEJK";
      return MDX_ERR_UNSUPPORTED;
    }
  RC(upload(ctx, d.mol_first, mf.data(), d.nop));
  RC(upload(ctx, d.mol_nat, mn.data(), d.nop));
  RC(upload(ctx, d.mol_type, mt.data(), d.nop));
  // exclusions INBB(ld, nbdmax) -> row-major [atom][k]
  std::vector<int> inbb((size_t)n * d.nbdmax, 0);
  for (int k = 0; k < ctx->d.nbdmax; ++k)
    for (int i = 0; i < n; ++i) inbb[(size_t)i * d.nbdmax + k] = t->inbb[(size_t)i + (size_t)k * t->ld_inbb];
  RC(upload(ctx, d.nnbb, t->nnbb, n));
  RC(upload(ctx, d.inbb, inbb.data(), inbb.size()));
  // LJ tables (column-major ld_lj) -> [i*nnbt + j], double and float
  const size_t nn = (size_t)nb * nb;
  if (!d.a6lj) {
    RC(dmalloc(ctx, &d.a6lj, 6 * nn));
    RC(dmalloc(ctx, &d.a6f, 6 * nn));
    RC(dmalloc(ctx, &d.abf, 3 * nn));
  }
  d.b12lj = d.a6lj + nn; d.a6lj0 = d.b12lj + nn; d.b12lj0 = d.a6lj0 + nn;
  d.a6_14 = d.b12lj0 + nn; d.b12_14 = d.a6_14 + nn;
  d.b12f = d.a6f + nn; d.a60f = d.b12f + nn; d.b120f = d.a60f + nn;
  d.a614f = d.b120f + nn; d.b1214f = d.a614f + nn;
  std::vector<double> lj(6 * nn);
  std::vector<float> ljf(6 * nn);
  const double *src[6] = {t->a6lj, t->b12lj, t->a6lj0, t->b12lj0, t->a6_14, t->b12_14};
  for (int k = 0; k < 6; ++k)
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        double v = src[k][(size_t)i + (size_t)j * t->ld_lj];
        lj[k * nn + (size_t)i * nb + j] = v;
        ljf[k * nn + (size_t)i * nb + j] = (float)v;
      }
  RC(upload(ctx, d.a6lj, lj.data(), lj.size()));
  RC(upload(ctx, d.a6f, ljf.data(), ljf.size()));
  RC(pack_lj_tables(ctx));
  ctx->h_a6lj0.assign(lj.begin() + 2 * nn, lj.begin() + 3 * nn);
  ctx->h_b12lj0.assign(lj.begin() + 3 * nn, lj.begin() + 4 * nn);
  ctx->h_inbt.assign(t->inbt, t->inbt + ns);
  // bonded: records and instances (indices to 0-based)
  d.nrbb = ctx->d.nrbb; d.nraa = ctx->d.nraa; d.nrtt = ctx->d.nrtt;
  d.nrbt = ctx->d.nrbt; d.nrat = ctx->d.nrat; d.nrrt = ctx->d.nrrt;
  ctx->h_rb.assign(t->rb, t->rb + d.nrbb);
  ctx->h_fb.assign(t->fb, t->fb + d.nrbb);
  ctx->h_db.assign(t->db, t->db + d.nrbb);
  ctx->h_ro.assign(t->ro, t->ro + d.nrbb);
  auto m1 = [](const int32_t *a, int cnt) {
    std::vector<int> v(cnt);
    for (int i = 0; i < cnt; ++i) v[i] = a[i] - 1;
    return v;
  };
  if (!d.bid) {
    RC(dmalloc(ctx, &d.bid, 3 * (size_t)std::max(1, d.nrbb)));
    RC(dmalloc(ctx, &d.brb, 4 * (size_t)std::max(1, d.nrbb)));
    RC(dmalloc(ctx, &d.ibi, 3 * (size_t)std::max(1, d.nrbt)));
    RC(dmalloc(ctx, &d.ara, 2 * (size_t)std::max(1, d.nraa)));
    RC(dmalloc(ctx, &d.iai, 4 * (size_t)std::max(1, d.nrat)));
    RC(dmalloc(ctx, &d.titors, 2 * (size_t)std::max(1, d.nrtt)));
    RC(dmalloc(ctx, &d.tft, 7 * (size_t)std::max(1, d.nrtt)));
    RC(dmalloc(ctx, &d.iti, 5 * (size_t)std::max(1, d.nrrt)));
    RC(dmalloc(ctx, &d.br, 2 * (size_t)std::max(1, d.nrbb)));
    RC(dmalloc(ctx, &d.ar, 2 * (size_t)std::max(1, d.nraa)));
    RC(dmalloc(ctx, &d.tr, 2 * (size_t)std::max(1, d.nrtt)));
    RC(dmalloc(ctx, &d.nspec_d, MDX_NT));
  }
  const int rbb = std::max(1, d.nrbb);
  d.bib = d.bid + rbb; d.bjb = d.bib + rbb;
  d.bfb = d.brb + rbb; d.bdb = d.bfb + rbb; d.bro = d.bdb + rbb;
  d.jbj = d.ibi + std::max(1, d.nrbt); d.ibuk = d.jbj + std::max(1, d.nrbt);
  d.afa = d.ara + std::max(1, d.nraa);
  d.jaj = d.iai + std::max(1, d.nrat); d.kak = d.jaj + std::max(1, d.nrat);
  d.iauk = d.kak + std::max(1, d.nrat);
  d.tnmul = d.titors + std::max(1, d.nrtt);
  {
    const int r = std::max(1, d.nrtt);
    d.trt = d.tft + r; d.tft1 = d.trt + r; d.tft2 = d.tft1 + r; d.tft3 = d.tft2 + r;
    d.tft4 = d.tft3 + r; d.tft5 = d.tft4 + r;
  }
  {
    const int r = std::max(1, d.nrrt);
    d.jtj = d.iti + r; d.ktk = d.jtj + r; d.ltl = d.ktk + r; d.ituk = d.ltl + r;
  }
  d.be = d.br + std::max(1, d.nrbb);
  d.ae = d.ar + std::max(1, d.nraa);
  d.te = d.tr + std::max(1, d.nrtt);
  RC(upload(ctx, d.bid, t->id, d.nrbb));
  RC(upload(ctx, d.bib, t->ib, d.nrbb));
  RC(upload(ctx, d.bjb, t->jb, d.nrbb));
  RC(upload(ctx, d.brb, t->rb, d.nrbb));
  RC(upload(ctx, d.bfb, t->fb, d.nrbb));
  RC(upload(ctx, d.bdb, t->db, d.nrbb));
  RC(upload(ctx, d.bro, t->ro, d.nrbb));
  RC(upload(ctx, d.ara, t->ra, d.nraa));
  RC(upload(ctx, d.afa, t->fa, d.nraa));
  RC(split_bonded(ctx, t));
  RC(upload(ctx, d.titors, t->itors, d.nrtt));
  RC(upload(ctx, d.tnmul, t->nmul, d.nrtt));
  RC(upload(ctx, d.tft, t->ft, d.nrtt));
  RC(upload(ctx, d.trt, t->rt, d.nrtt));
  RC(upload(ctx, d.tft1, t->ft1, d.nrtt));
  RC(upload(ctx, d.tft2, t->ft2, d.nrtt));
  RC(upload(ctx, d.tft3, t->ft3, d.nrtt));
  RC(upload(ctx, d.tft4, t->ft4, d.nrtt));
  RC(upload(ctx, d.tft5, t->ft5, d.nrtt));
  if (d.nrrt) {
    auto a = m1(t->iti, d.nrrt), b = m1(t->jtj, d.nrrt), c = m1(t->ktk, d.nrrt),
         e = m1(t->ltl, d.nrrt), f = m1(t->ituk, d.nrrt);
    RC(upload(ctx, d.iti, a.data(), d.nrrt));
    RC(upload(ctx, d.jtj, b.data(), d.nrrt));
    RC(upload(ctx, d.ktk, c.data(), d.nrrt));
    RC(upload(ctx, d.ltl, e.data(), d.nrrt));
    RC(upload(ctx, d.ituk, f.data(), d.nrrt));
  }
  RC(upload(ctx, d.nspec_d, t->nspec, nt));
  RC(shake_clusters(ctx, t));
  if (ctx->mixed()) RC(upload_site_table(ctx));
  ctx->have_topo = true;
  return MDX_OK;
}

int mdx_set_params(mdx_ctx *ctx, const mdx_params *p) {
  if (!ctx || !p) return MDX_ERR_ARG;
  if (p->icell < 0 || p->icell > 2) {
    ctx->err = "ICELL must be 0 (rectangular), 1 (truncated octahedron) or 2 (hexagonal)";
    return MDX_ERR_ARG;
  }
  if (p->icell != 0 && p->rskin > 0.0) {
    ctx->err = "non-rectangular cells: the reference's list mode only (no Verlet skin)";
    return MDX_ERR_UNSUPPORTED;
  }
  if (p->boxl <= 0 || p->boyl <= 0 || p->bozl <= 0 || p->rcut <= 0 || p->nfreq < 1 ||
      p->ichnb < 1) {
    ctx->err = "bad box, cutoff, NFREQ or ICHNB";
    return MDX_ERR_ARG;
  }
  if (p->rskin < 0.0 || (p->rskin > 0.0 && p->lnpt)) {
    ctx->err = "Verlet skin: rskin >= 0, and constant volume only";
    return p->rskin < 0.0 ? MDX_ERR_ARG : MDX_ERR_UNSUPPORTED;
  }
  if (p->rskin > 0.0 && p->lmnbl) {
    ctx->err = "Verlet skin: not with the reaction-field molecular cutoff";
    return MDX_ERR_UNSUPPORTED;
  }
  if (p->lmnbl && 2.0 * p->rcut > std::min(p->boxl, std::min(p->boyl, p->bozl)) + 1e-9) {
    ctx->err = "reaction field: RCUT must be within half the box (main.f:745-749)";
    return MDX_ERR_ARG;
  }
  if (p->rskin > 0.0 &&
      p->rcut + p->rskin > 0.5 * std::min(p->boxl, std::min(p->boyl, p->bozl))) {
    ctx->err = "Verlet skin: RCUT + skin must stay within half the box";
    return MDX_ERR_ARG;
  }
  ctx->drop_graphs();  // kernel arguments baked into the step graphs change
  if (ctx->have_params && p->rskin != ctx->p.rskin) {
    // a new list mode: the next step needs a fresh CHCNB
    ctx->have_lists = false;
    ctx_free(ctx, ctx->dv.pos_ref);
    ctx->dv.pos_ref = nullptr;
  }
  ctx->p = *p;
  ctx->pc.coulf = p->coulf;
  ctx->pc.alphad = p->alphad;
  ctx->pc.raex = p->raex;
  ctx->pc.rff = p->rff;
  ctx->pc.rff2 = p->rff2;
  ctx->pc.lmnbl = p->lmnbl;
  ctx->pc.lmdee = p->lmdee;
  ctx->pc.nnbt = ctx->d.nnbt;
  ctx->pc.rc2 = p->rskin > 0.0 ? p->rcut * p->rcut : 1e300;
  ctx->pc.rc2f = p->rskin > 0.0 ? (float)(p->rcut * p->rcut) : 3.0e38f;
  ctx->boxl = p->boxl;
  ctx->boyl = p->boyl;
  ctx->bozl = p->bozl;
  ctx->furir_init = false;
  set_fix_scales(ctx);
  ctx->have_params = true;
  return MDX_OK;
}

int mdx_upload_state(mdx_ctx *ctx, const double *sx, const double *sy,
                     const double *sz, const double *vx, const double *vy,
                     const double *vz, const mdx_thermo *th) {
  if (!ctx || !sx || !sy || !sz || !vx || !vy || !vz) return MDX_ERR_ARG;
  RC(require(ctx, true, true, false));
  DevData &d = ctx->dv;
  const size_t n = d.n;
  double *tmp = nullptr;
  RC(dmalloc(ctx, &tmp, 4 * n));
  int rc = MDX_OK;
  rc = rc ? rc : upload(ctx, tmp, sx, n);
  rc = rc ? rc : upload(ctx, tmp + n, sy, n);
  rc = rc ? rc : upload(ctx, tmp + 2 * n, sz, n);
  // the charges (kept in step with RECINT on the device) go up only once
  const bool charges = !ctx->have_state || ctx->q_dirty;
  if (charges) rc = rc ? rc : upload(ctx, tmp + 3 * n, ctx->h_q.data(), n);
  if (!rc) {
    k_set_pos<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, tmp, tmp + n, tmp + 2 * n,
                                                         charges ? tmp + 3 * n : nullptr,
                                                         d.pos);
    ctx->launches++;
  }
  ctx_free(ctx, tmp);
  cudaStreamSynchronize(ctx->stream);
  if (rc) return rc;
  ctx->q_dirty = false;
  RC(upload(ctx, d.vx, vx, n));
  RC(upload(ctx, d.vy, vy, n));
  RC(upload(ctx, d.vz, vz, n));
  if (ctx->p.lmnbl) {
    // reach of small molecules (at most 5 sites) from their centres of mass,
    // for the search radius of the reaction field's molecular cutoff list
    // (unknown, -1, when the state came without that list: the build then
    // searches the whole box)
    double reach = 0.0;
    const double hb[3] = {0.5 * ctx->boxl, 0.5 * ctx->boyl, 0.5 * ctx->bozl};
    const double bl[3] = {ctx->boxl, ctx->boyl, ctx->bozl};
    for (size_t i = 0; i < n;) {
      const int m = ctx->h_nnum[i];
      size_t e = i;
      while (e < n && ctx->h_nnum[e] == m) ++e;
      if (e - i <= 5) {
        double c[3] = {0, 0, 0}, mt = 0.0;
        const double *xs[3] = {sx, sy, sz};
        for (size_t a = i; a < e; ++a) {
          const double w = ctx->h_mass[ctx->h_nsite[a] - 1];
          mt += w;
          for (int k = 0; k < 3; ++k) {
            double dxk = xs[k][a] - xs[k][i];
            if (std::fabs(dxk) > hb[k]) dxk -= std::copysign(bl[k], dxk);
            c[k] += w * dxk;
          }
        }
        for (size_t a = i; a < e; ++a) {
          double r2 = 0.0;
          for (int k = 0; k < 3; ++k) {
            double dxk = xs[k][a] - xs[k][i];
            if (std::fabs(dxk) > hb[k]) dxk -= std::copysign(bl[k], dxk);
            dxk -= c[k] / mt;
            r2 += dxk * dxk;
          }
          reach = std::max(reach, std::sqrt(r2));
        }
      }
      i = e;
    }
    ctx->mol_reach = reach + 1.0;
  } else {
    ctx->mol_reach = -1.0;
  }
  mdx_thermo h{};
  if (th) h = *th;
  if (h.boxl > 0) {
    ctx->boxl = h.boxl;
    ctx->boyl = h.boyl;
    ctx->bozl = h.bozl;
  } else {
    h.boxl = ctx->boxl;
    h.boyl = ctx->boyl;
    h.bozl = ctx->bozl;
  }
  h.vol = h.boxl * h.boyl * h.bozl;
  if (ctx->p.icell == 1) h.vol = 0.5 * h.vol;  // RECLEN (service.f:602)
  RC(upload(ctx, d.th, &h, 1));
  // molecular centres (the driver's last GETCOM left them consistent)
  std::vector<double> sm(MDX_NT, 1.0);
  for (int t = 0; t < ctx->d.ntypes; ++t) sm[t] = ctx->summas[t];
  double *dsm = d.red + 256;
  RC(upload(ctx, dsm, sm.data(), MDX_NT));
  k_com_only<<<(d.nop + 127) / 128, 128, 0, ctx->stream>>>(
      d.nop, d.mol_first, d.mol_nat, d.mol_type, d.amass, d.pos, d.X, d.Y, d.Z, dsm,
      ctx->boxl, ctx->boyl, ctx->bozl, cell_pbc(ctx));
  ctx->launches++;
  RC(launch_mirror_f32(ctx));
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  // lists and forces persist, as the reference's COMMON blocks do, until the
  // caller asks for CHCNB / the force routines again
  ctx->have_state = true;
  return MDX_OK;
}

int mdx_download_state(mdx_ctx *ctx, double *sx, double *sy, double *sz,
                       double *vx, double *vy, double *vz, mdx_thermo *th) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  DevData &d = ctx->dv;
  const size_t n = d.n;
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (sx || sy || sz) {
    double *tmp = nullptr;
    RC(dmalloc(ctx, &tmp, 3 * n));
    k_get_pos<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, d.pos, tmp, tmp + n, tmp + 2 * n);
    ctx->launches++;
    cudaStreamSynchronize(ctx->stream);
    if (sx) ctx_copy(ctx->stream, sx, tmp, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (sy) ctx_copy(ctx->stream, sy, tmp + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (sz) ctx_copy(ctx->stream, sz, tmp + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    ctx_free(ctx, tmp);
  }
  if (vx) MDX_CUDA(ctx_copy(ctx->stream, vx, d.vx, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (vy) MDX_CUDA(ctx_copy(ctx->stream, vy, d.vy, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (vz) MDX_CUDA(ctx_copy(ctx->stream, vz, d.vz, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (th) MDX_CUDA(ctx_copy(ctx->stream, th, d.th, sizeof(mdx_thermo), cudaMemcpyDeviceToHost));
  return MDX_OK;
}

int mdx_snapshot(mdx_ctx *ctx, int32_t slot, double *sx, double *sy, double *sz,
                 double *vx, double *vy, double *vz, mdx_thermo *th) {
  if (!ctx || slot < 0 || slot >= MDX_SNAPSHOT_SLOTS || !sx || !sy || !sz || !vx || !vy ||
      !vz)
    return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  DevData &d = ctx->dv;
  const size_t n = d.n;
  if (!d.snap) RC(dmalloc(ctx, &d.snap, 3 * n));  // first call: waits for the stream once
  if (!ctx->snap_ev[slot])
    MDX_CUDA(cudaEventCreateWithFlags(&ctx->snap_ev[slot], cudaEventDisableTiming));
  k_get_pos<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, d.pos, d.snap, d.snap + n,
                                                       d.snap + 2 * n);
  MDX_LAUNCHED(ctx);
  double *dst[6] = {sx, sy, sz, vx, vy, vz};
  const double *src[6] = {d.snap, d.snap + n, d.snap + 2 * n, d.vx, d.vy, d.vz};
  for (int k = 0; k < 6; ++k)
    MDX_CUDA(cudaMemcpyAsync(dst[k], src[k], sizeof(double) * n, cudaMemcpyDeviceToHost,
                             ctx->stream));
  if (th)
    MDX_CUDA(cudaMemcpyAsync(th, d.th, sizeof(mdx_thermo), cudaMemcpyDeviceToHost, ctx->stream));
  MDX_CUDA(cudaEventRecord(ctx->snap_ev[slot], ctx->stream));
  return MDX_OK;
}

int mdx_snapshot_wait(mdx_ctx *ctx, int32_t slot) {
  if (!ctx || slot < 0 || slot >= MDX_SNAPSHOT_SLOTS || !ctx->snap_ev[slot]) return MDX_ERR_ARG;
  const cudaError_t e = cudaEventSynchronize(ctx->snap_ev[slot]);
  return e == cudaSuccess ? MDX_OK : MDX_ERR_CUDA;
}

int mdx_get_bonded_averages(mdx_ctx *ctx, double *br, double *be, double *ar, double *ae,
                            double *tr, double *te) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, false, false));
  DevData &d = ctx->dv;
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  double *dst[6] = {br, be, ar, ae, tr, te};
  const double *src[6] = {d.br, d.be, d.ar, d.ae, d.tr, d.te};
  const int len[6] = {d.nrbb, d.nrbb, d.nraa, d.nraa, d.nrtt, d.nrtt};
  for (int k = 0; k < 6; ++k)
    if (dst[k] && len[k] > 0)
      MDX_CUDA(ctx_copy(ctx->stream, dst[k], src[k], sizeof(double) * len[k],
                        cudaMemcpyDeviceToHost));
  return MDX_OK;
}

int mdx_set_pullback(mdx_ctx *ctx, const mdx_pullback *pb) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, false, false));
  DevData &d = ctx->dv;
  ctx->drop_graphs();  // the step's launches change
  if (!pb) {
    ctx->pullback = false;
    return MDX_OK;
  }
  if (pb->npull < 0 || (pb->npull > 0 && (!pb->inpl || !pb->xpl || !pb->ypl || !pb->zpl))) {
    ctx->err = "mdx_set_pullback: NPULL wells need INPL, XPL, YPL, ZPL";
    return MDX_ERR_ARG;
  }
  std::vector<int> well(d.n, -1);
  for (int k = 0; k < pb->npull; ++k) {
    if (pb->inpl[k] < 1 || pb->inpl[k] > d.n) {
      ctx->err = "mdx_set_pullback: INPL out of range";
      return MDX_ERR_ARG;
    }
    well[pb->inpl[k] - 1] = k;
  }
  ctx_free(ctx, d.pull_atom);
  ctx_free(ctx, d.pull_ref);
  d.pull_atom = nullptr;
  d.pull_ref = nullptr;
  RC(dmalloc(ctx, &d.pull_atom, (size_t)d.n));
  RC(upload(ctx, d.pull_atom, well.data(), (size_t)d.n));
  if (pb->npull > 0) {
    std::vector<double> ref(3 * (size_t)pb->npull);
    for (int k = 0; k < pb->npull; ++k) {
      ref[k] = pb->xpl[k];
      ref[pb->npull + k] = pb->ypl[k];
      ref[2 * (size_t)pb->npull + k] = pb->zpl[k];
    }
    RC(dmalloc(ctx, &d.pull_ref, ref.size()));
    RC(upload(ctx, d.pull_ref, ref.data(), ref.size()));
  }
  if (!d.pull_step) RC(dmalloc(ctx, &d.pull_step, 1));
  RC(upload(ctx, d.pull_step, &pb->nstep, 1));
  ctx->pb = *pb;
  ctx->pb.inpl = nullptr;
  ctx->pb.xpl = ctx->pb.ypl = ctx->pb.zpl = nullptr;
  ctx->pullback = pb->ldrag || pb->npull > 0 || pb->iext == 1;
  return MDX_OK;
}

int mdx_set_averaging(mdx_ctx *ctx, int on) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, false, false));
  DevData &d = ctx->dv;
  if (on && !d.avsum) RC(dmalloc(ctx, &d.avsum, (size_t)bonded_sums_len(ctx)));
  if ((on != 0) != ctx->averaging) ctx->drop_graphs();  // the step's launches change
  ctx->averaging = on != 0;
  return MDX_OK;
}

int mdx_get_bonded_sums(mdx_ctx *ctx, double *sums, int32_t clear) {
  if (!ctx || !sums) return MDX_ERR_ARG;
  DevData &d = ctx->dv;
  const int len = bonded_sums_len(ctx);
  if (!d.avsum) {
    std::fill(sums, sums + len, 0.0);
    return MDX_OK;
  }
  MDX_CUDA(ctx_copy(ctx->stream, sums, d.avsum, sizeof(double) * len, cudaMemcpyDeviceToHost));
  if (clear) MDX_CUDA(cudaMemsetAsync(d.avsum, 0, sizeof(double) * len, ctx->stream));
  return MDX_OK;
}

int mdx_download_forces(mdx_ctx *ctx, int which, double *fx, double *fy, double *fz) {
  if (!ctx || !fx || !fy || !fz || which < 1 || which > 3) return MDX_ERR_ARG;
  DevData &d = ctx->dv;
  const double *x = which == 1 ? d.hx : which == 2 ? d.gx : d.fx;
  const double *y = which == 1 ? d.hy : which == 2 ? d.gy : d.fy;
  const double *z = which == 1 ? d.hz : which == 2 ? d.gz : d.fz;
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  MDX_CUDA(ctx_copy(ctx->stream, fx, x, sizeof(double) * d.n, cudaMemcpyDeviceToHost));
  MDX_CUDA(ctx_copy(ctx->stream, fy, y, sizeof(double) * d.n, cudaMemcpyDeviceToHost));
  MDX_CUDA(ctx_copy(ctx->stream, fz, z, sizeof(double) * d.n, cudaMemcpyDeviceToHost));
  return MDX_OK;
}

int mdx_inifur(mdx_ctx *ctx, int32_t *nkv) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, false));
  RC(host_inifur(ctx));
  ctx->furir_init = true;
  ctx->boxlo = ctx->boxl;
  ctx->boylo = ctx->boyl;
  ctx->bozlo = ctx->bozl;
  if (nkv) *nkv = ctx->nkv;
  return MDX_OK;
}

int mdx_chcnb(mdx_ctx *ctx, int32_t *mbsh, int32_t *mbln) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  RC(launch_build_lists(ctx));
  RC(check_err(ctx));
  int c[2];
  MDX_CUDA(ctx_copy(ctx->stream, c, &ctx->dv.sc->mbsh, sizeof c, cudaMemcpyDeviceToHost));
  ctx->mbsh = c[0];
  ctx->mbln = c[1];
  if (mbsh) *mbsh = c[0];
  if (mbln) *mbln = c[1];
  return MDX_OK;
}

int mdx_get_lists(mdx_ctx *ctx, int32_t *nbs1, int32_t *nbs2, int32_t cap_s,
                  int32_t *nbl1, int32_t *nbl2, int32_t cap_l) {
  if (!ctx || !nbs1 || !nbs2 || !nbl1 || !nbl2) return MDX_ERR_ARG;
  if (!ctx->have_lists) {
    ctx->err = "no lists built";
    return MDX_ERR_STATE;
  }
  return export_lists(ctx, nbs1, nbs2, cap_s, nbl1, nbl2, cap_l);
}

int mdx_getcom(mdx_ctx *ctx) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  RC(launch_getcom(ctx));
  return check_err(ctx);
}

int mdx_getkin(mdx_ctx *ctx, const double *summd, double enerf_tempf, double fnop,
               double fnstr, double fnsti, mdx_kin *out) {
  if (!ctx || !summd || !out) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));  // the centres: state upload, GETCOM, every step
  double s[3];
  RC(launch_getkin(ctx, summd, s));
  RC(check_err(ctx));
  // the tail of GETKIN (service.f:706-722), on the host
  mdx_kin k{};
  k.ektr = s[0];
  k.ekrot = s[1];
  k.tke = s[2];
  k.ekint = k.tke - k.ektr - k.ekrot;
  k.ttr = fnop > 1.1 ? k.ektr * enerf_tempf / (fnop - 1.0) : k.ektr * enerf_tempf / fnop;
  if (fnstr > 0.01) {
    k.trot = 3. * k.ekrot * enerf_tempf / fnstr;
  } else {
    double temp = 0.0;
    MDX_CUDA(ctx_copy(ctx->stream, &temp, &ctx->dv.th->temp, sizeof(double),
                      cudaMemcpyDeviceToHost));
    k.trot = temp;
  }
  k.tint = fnsti > 0.01 ? 3.0 * k.ekint * enerf_tempf / fnsti : 0.0;
  *out = k;
  return MDX_OK;
}

int mdx_chkmom(mdx_ctx *ctx, double sumasd, double *dv) {
  if (!ctx || !(sumasd > 0.0)) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  double pt[3];
  RC(launch_chkmom(ctx, sumasd, pt));
  RC(check_err(ctx));
  if (dv) {
    dv[0] = pt[0] / sumasd;
    dv[1] = pt[1] / sumasd;
    dv[2] = pt[2] / sumasd;
  }
  return MDX_OK;
}

int mdx_fforces(mdx_ctx *ctx, int laver, mdx_scalars *out) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  if (!ctx->have_lists) {
    ctx->err = "lists not built";
    return MDX_ERR_STATE;
  }
  RC(do_fforces(ctx, laver, true));
  RC(check_err(ctx));
  return copy_scalars(ctx, out);
}

int mdx_slforces(mdx_ctx *ctx, mdx_scalars *out) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  if (!ctx->have_lists) {
    ctx->err = "lists not built";
    return MDX_ERR_STATE;
  }
  RC(do_slforces(ctx, true));
  RC(check_err(ctx));
  return copy_scalars(ctx, out);
}

int mdx_allforce(mdx_ctx *ctx, mdx_scalars *out) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  if (!ctx->have_lists) {
    ctx->err = "lists not built";
    return MDX_ERR_STATE;
  }
  RC(do_allforce(ctx, true));
  RC(check_err(ctx));
  return copy_scalars(ctx, out);
}

int mdx_double_steps(mdx_ctx *ctx, int32_t nsteps, int32_t mstep0, mdx_step_record *rec) {
  if (!ctx || nsteps < 0) return MDX_ERR_ARG;
  return run_steps(ctx, true, nsteps, mstep0, rec);
}

int mdx_double(mdx_ctx *ctx, int32_t nsteps, int32_t nsttot, mdx_step_record *rec) {
  if (!ctx || nsteps < 0) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  RC(launch_vira(ctx, 0));
  RC(launch_build_lists(ctx));
  RC(launch_getcom(ctx));
  RC(do_slforces(ctx, false));
  RC(do_fforces(ctx, 1, false));
  RC(check_err(ctx));
  return run_steps(ctx, true, nsteps, nsttot, rec);
}

int mdx_double_enqueue(mdx_ctx *ctx, int32_t nsteps, int32_t mstep0, int32_t prologue) {
  if (!ctx || nsteps < 0) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  if (ctx->p.lnpt || ctx->timing || !ctx->use_graphs) {
    ctx->err = "enqueued steps need graph replay: constant volume, timers off";
    return MDX_ERR_STATE;
  }
  if (prologue) {  // DOUBLE's prologue, mdstep.f:296-310
    RC(launch_vira(ctx, 0));
    RC(launch_build_lists(ctx));
    RC(launch_getcom(ctx));
    RC(do_slforces(ctx, false));
    RC(do_fforces(ctx, 1, false));
  } else if (!ctx->have_lists) {
    ctx->err = "neighbour lists not built (enqueue with the prologue first)";
    return MDX_ERR_STATE;
  }
  for (int s = 1; s <= nsteps; ++s) RC(graph_step(ctx, mstep0 + s, false, true));
  return MDX_OK;
}

int mdx_poll(mdx_ctx *ctx, int32_t *done) {
  if (!ctx || !done) return MDX_ERR_ARG;
  const cudaError_t e = cudaStreamQuery(ctx->stream);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return MDX_OK;
  }
  if (e != cudaSuccess) {
    ctx->err = std::string("stream: ") + cudaGetErrorString(e);
    return MDX_ERR_CUDA;
  }
  *done = 1;
  return check_err(ctx);
}

int mdx_pending_cuda_error(void) { return (int)cudaPeekAtLastError(); }

int mdx_device_memory(size_t *free_bytes, size_t *total_bytes) {
  size_t f = 0, t = 0;
  if (cudaMemGetInfo(&f, &t) != cudaSuccess) return MDX_ERR_CUDA;
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return MDX_OK;
}

int mdx_get_path_info(const mdx_ctx *ctx, mdx_path_info *out) {
  if (!ctx || !out) return MDX_ERR_ARG;
  const DevData &d = ctx->dv;
  const bool mx = ctx->mixed();
  out->precision = ctx->d.precision;
  out->ewald_force_pass = !mx ? 0 : d.tc_on ? 2 : 1;
  out->ewald_sfac_pass = !mx ? 0 : d.tcs_on ? 2 : 1;
  out->sfac_slices = ctx->furir_init ? sfac_slices(ctx) : 0;
  out->sfac_ordered = (mx && d.tcs_on) || d.sk_part != nullptr ? 1 : 0;
  out->list_mode = ctx->p.rskin > 0.0 ? 1 : 0;
  out->graphs = ctx->use_graphs ? 1 : 0;
  out->nkv = ctx->nkv;
  return MDX_OK;
}

int mdx_set_tuning(mdx_ctx *ctx, const mdx_tuning *t) {
  if (!ctx) return MDX_ERR_ARG;
  if (t) {
    const bool ok_s = t->tpo_short == 2 || t->tpo_short == 4 || t->tpo_short == 8;
    const bool ok_l =
        t->tpo_long == 4 || t->tpo_long == 8 || t->tpo_long == 16 || t->tpo_long == 32;
    if (!ok_s || !ok_l) {
      ctx->err = "tuning: tpo_short must be 2, 4 or 8 and tpo_long 4, 8, 16 or 32";
      return MDX_ERR_ARG;
    }
    ctx->tune = mdx_tuning{t->tpo_short, t->tpo_long, 2, 0};
  } else {
    ctx->tune = mdx_tuning{};
  }
  ctx->drop_graphs();  // the step graphs hold the sweeps' launch shapes
  return MDX_OK;
}

int mdx_get_tuning(mdx_ctx *ctx, mdx_tuning *out) {
  if (!ctx || !out) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  resolve_tuning(ctx);
  *out = ctx->tune;
  return MDX_OK;
}

int mdx_pool_usage(size_t *used_bytes, size_t *reserved_bytes) {
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess)
    return MDX_ERR_CUDA;
  uint64_t u = 0, r = 0;
  if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u) != cudaSuccess ||
      cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r) != cudaSuccess)
    return MDX_ERR_CUDA;
  if (used_bytes) *used_bytes = (size_t)u;
  if (reserved_bytes) *reserved_bytes = (size_t)r;
  return MDX_OK;
}

int mdx_sultan_steps(mdx_ctx *ctx, int32_t nsteps, int32_t mstep0, mdx_step_record *rec) {
  if (!ctx || nsteps < 0) return MDX_ERR_ARG;
  return run_steps(ctx, false, nsteps, mstep0, rec);
}

int mdx_sultan(mdx_ctx *ctx, int32_t nsteps, int32_t nsttot, mdx_step_record *rec) {
  if (!ctx || nsteps < 0) return MDX_ERR_ARG;
  RC(require(ctx, true, true, true));
  RC(launch_build_lists(ctx));
  RC(launch_getemp(ctx));
  RC(do_allforce(ctx, false));
  RC(check_err(ctx));
  return run_steps(ctx, false, nsteps, nsttot, rec);
}

// RECINT (mdee.f:86-140)
int mdx_set_lambda(mdx_ctx *ctx, double ec, double pw1, double pw2, double bee) {
  if (!ctx) return MDX_ERR_ARG;
  RC(require(ctx, true, true, false));
  DevData &d = ctx->dv;
  const int nt = ctx->d.ntypes, nb = ctx->d.nnbt;
  const size_t nn = (size_t)nb * nb;
  std::vector<double> a6(nn), b12(nn);
  std::vector<float> a6f(nn), b12f(nn);
  MDX_CUDA(ctx_copy(ctx->stream, a6.data(), d.a6lj, sizeof(double) * nn, cudaMemcpyDeviceToHost));
  MDX_CUDA(ctx_copy(ctx->stream, b12.data(), d.b12lj, sizeof(double) * nn, cudaMemcpyDeviceToHost));
  ctx->spei = 0.0;
  for (int t = 0; t < nt; ++t) {
    const double ESCI = ctx->tc.iee[t] == 0 ? std::pow(ec, pw1) : 1.0;
    for (int I = ctx->isadr[t] + 1; I <= ctx->isadr[t] + ctx->nsits[t]; ++I) {
      const int IS = ctx->h_inbt[I - 1] - 1;
      for (int u = 0; u < nt; ++u) {
        double ESCL = ESCI;
        if (ctx->tc.iee[u] == 0) ESCL = std::pow(ec, pw1);
        for (int J = ctx->isadr[u] + 1; J <= ctx->isadr[u] + ctx->nsits[u]; ++J) {
          const int JS = ctx->h_inbt[J - 1] - 1;
          a6[(size_t)IS * nb + JS] = ESCL * ctx->h_a6lj0[(size_t)IS * nb + JS];
          b12[(size_t)IS * nb + JS] = ESCL * ctx->h_b12lj0[(size_t)IS * nb + JS];
        }
      }
    }
    for (int ISP = ctx->isaddr[t] + 1; ISP <= ctx->isaddr[t] + ctx->nsits[t] * ctx->nspec[t]; ++ISP)
      ctx->h_q[ISP - 1] = ESCI * ctx->h_charge[ctx->h_nsite[ISP - 1] - 1];
    double SPET = 0.0;
    for (int I = 1; I <= ctx->nsits[t]; ++I) {
      const int IS = ctx->isadr[t] + I;
      const double eq = ESCI * ctx->h_charge[IS - 1];
      const double QII = ctx->p.coulf * (eq * eq);
      SPET = SPET - ctx->nspec[t] * ctx->p.alphad * QII / std::sqrt(3.1415926536);
    }
    ctx->speei[t] = SPET;
    ctx->spei = ctx->spei + SPET;
  }
  for (size_t k = 0; k < nn; ++k) {
    a6f[k] = (float)a6[k];
    b12f[k] = (float)b12[k];
  }
  RC(upload(ctx, d.a6lj, a6.data(), nn));
  RC(upload(ctx, d.b12lj, b12.data(), nn));
  RC(upload(ctx, d.a6f, a6f.data(), nn));
  RC(upload(ctx, d.b12f, b12f.data(), nn));
  RC(pack_lj_tables(ctx));
  ctx->p.raex = bee * (1. - std::pow(ec, pw2));
  ctx->p.ec_me = ec;
  ctx->pc.raex = ctx->p.raex;
  ctx->drop_graphs();
  if (ctx->have_state) {
    double *dq = nullptr;
    RC(dmalloc(ctx, &dq, d.n));
    RC(upload(ctx, dq, ctx->h_q.data(), d.n));
    k_set_q<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(d.n, dq, d.pos);
    ctx->launches++;
    ctx_free(ctx, dq);
    cudaStreamSynchronize(ctx->stream);
  }
  if (ctx->mixed()) RC(upload_site_table(ctx));
  return MDX_OK;
}

int mdx_set_timers(mdx_ctx *ctx, int on) {
  if (!ctx) return MDX_ERR_ARG;
  ctx->timing = on != 0;
  return MDX_OK;
}

int mdx_get_timers(mdx_ctx *ctx, double *ms, int64_t *count) {
  if (!ctx) return MDX_ERR_ARG;
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto &sp : ctx->spans) {
    float t = 0.f;
    cudaEventElapsedTime(&t, sp.a, sp.b);
    ctx->t_ms[sp.id] += t;
    ctx->t_cnt[sp.id] += 1;
    ctx->ev_pool.push_back(sp.a);
    ctx->ev_pool.push_back(sp.b);
  }
  ctx->spans.clear();
  for (int k = 0; k < MDX_NTIMERS; ++k) {
    if (ms) ms[k] = ctx->t_ms[k];
    if (count) count[k] = ctx->t_cnt[k];
    ctx->t_ms[k] = 0.0;
    ctx->t_cnt[k] = 0;
  }
  return MDX_OK;
}

void *mdx_stream(mdx_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }
int64_t mdx_launch_count(const mdx_ctx *ctx) { return ctx ? ctx->launches : 0; }
int mdx_sync(mdx_ctx *ctx) {
  if (!ctx) return MDX_ERR_ARG;
  return check_err(ctx);
}

}  // extern "C"

// Site table of the mixed pair kernels: per site the EE-scaled charge Q (the
// same for every atom of a site: RECINT scales by molecule type,
// mdee.f:119-127), the raw CHARGE, the LJ type and the molecule type.
static float int_bits(int v) {
  float f;
  std::memcpy(&f, &v, sizeof f);
  return f;
}

int upload_site_table(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  const int n = d.n, ns = ctx->d.nsites;
  std::vector<float4> st(ns);
  std::vector<char> seen(ns, 0);
  for (int i = 0; i < n; ++i) {
    const int site = ctx->h_nsite[i] - 1;
    const float q = (float)ctx->h_q[i];
    if (seen[site] && st[site].x != q) {
      ctx->err = "mixed path: atoms of one site carry different charges";
      return MDX_ERR_UNSUPPORTED;
    }
    seen[site] = 1;
    st[site] = make_float4(q, (float)ctx->h_charge[site],
                           int_bits(ctx->h_inbt[site] - 1),
                           int_bits(ctx->h_itype[i] - 1));
  }
  for (int s = 0; s < ns; ++s)
    if (!seen[s]) st[s] = make_float4(0.f, (float)ctx->h_charge[s], int_bits(ctx->h_inbt[s] - 1),
                                      int_bits(0));
  return upload(ctx, d.stab, st.data(), (size_t)ns);
}

// Linkage for noalloc.cu and pimd.cu (the helpers above have internal
// linkage).
int api_require(mdx_ctx *ctx, bool topo, bool par, bool state) {
  return require(ctx, topo, par, state);
}
int api_check_err(mdx_ctx *ctx) { return check_err(ctx); }
int api_copy_scalars(mdx_ctx *ctx, mdx_scalars *out) { return copy_scalars(ctx, out); }
int api_do_slforces(mdx_ctx *ctx, bool split, bool mirrored) {
  return do_slforces(ctx, split, mirrored);
}
int api_do_fforces(mdx_ctx *ctx, int laver, bool split, bool mirrored) {
  return do_fforces(ctx, laver, split, true, mirrored);
}
