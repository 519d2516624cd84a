// pimd.cu -- path-integral MD over bead replicas (PIMD, pimd.f:18-316;
// PIFORCES pimd.f:321-395; BEADNOSE pimd.f:402-444).
//
// The reference runs one bead per MPI rank; every short step the ranks
// exchange coordinates (ring springs) and kinetic energies (bead
// thermostats).  Here the NBEADS contexts stay on one GPU.  The integrator
// passes of all beads run as one launch each on the ensemble's stream
// (grid row = bead, the bead's arrays from a device table:
// launch_getemp_beads, launch_kick_drift_com_beads); each bead's lists and
// forces run on the bead's own stream, concurrently with the other beads
// (fork/join); the two cross-bead operations run on the ensemble's stream:
//   k_pi_nose     BEADNOSE: per atom, kinetic energy summed over beads
//                 drives a Nose-Hoover chain shared by the atom's beads;
//   k_pi_springs  forces / NBEADS, then PIFORCES: springs to bead b-1 and
//                 b+1 with their coordinates rounded to single precision
//                 (the reference sends them as REAL*4, pimd.f:450-486).
// Per long step (NFREQ short steps, no NVT/NPT scaling: PI_SCALING only
// evaluates GETEMP then):
//   [GETEMP, V += HTSTEP G, V += HTSTEB H], nose
//   for each short step:
//     [drift, GETCOM], fork [CHCNB?, SLFORCES+FFORCES | FFORCES] join, springs
//     [V += HTSTEB H, GETEMP, (next: V += HTSTEB H) | (last: V += HTSTEP G)],
//     (nose | GETEMP, record)
// Long steps are captured once (with and without the list rebuild) and
// replayed.  Spring energies and virials are summed per bead in block order
// (deterministic).
#include <vector>

#include "mdx_internal.cuh"

#define RC(x)            \
  do {                   \
    int rc_ = (x);       \
    if (rc_) return rc_; \
  } while (0)

namespace {

struct PiBead {
  dbl4 *pos;
  double *vx, *vy, *vz;
  double *gx, *gy, *gz, *hx, *hy, *hz;
  mdx_scalars *sc;
  mdx_thermo *th;
};

constexpr int PI_THREADS = 256;
constexpr int PI_NV = 5;  // QEK, VIRPI, VIRFX, VIRFY, VIRFZ

// BEADNOSE (pimd.f:406-440), thread per atom.  THERMO(I, J) at th[J*n + I].
__global__ void k_pi_nose(int n, int P, const PiBead *__restrict__ b,
                          const double *__restrict__ massdi, double *th, int jnh,
                          double conveq, double trtemp, double dqqt, double fnh,
                          double tsteb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double fek = 0.0;
  for (int k = 0; k < P; ++k) {
    const double x = b[k].vx[i], y = b[k].vy[i], z = b[k].vz[i];
    fek = fek + 0.5 * (x * x + y * y + z * z) * massdi[i];
  }
  const double atemp = fek * conveq;
  const double dke = atemp / trtemp - 1.0;
  th[i] = th[i] + dke * dqqt * tsteb;
  for (int j = 1; j < jnh; ++j) {
    const double prev = th[(size_t)(j - 1) * n + i];
    th[(size_t)j * n + i] = th[(size_t)j * n + i] + (prev * prev - fnh) * tsteb;
    th[(size_t)(j - 1) * n + i] = prev * (1. - th[(size_t)j * n + i] * tsteb);
  }
  const double scv = 1. - th[i] * tsteb;
  for (int k = 0; k < P; ++k) {
    b[k].vx[i] = b[k].vx[i] * scv;
    b[k].vy[i] = b[k].vy[i] * scv;
    b[k].vz[i] = b[k].vz[i] * scv;
  }
}

// Forces / NBEADS (G too on a slow step), then PIFORCES (pimd.f:333-376);
// block (blockIdx.x, bead blockIdx.y), per-block partial sums in part.
__global__ void __launch_bounds__(PI_THREADS) k_pi_springs(
    int n, int P, const PiBead *__restrict__ b, const double *__restrict__ smass,
    double beadfac, double bx, double by, double bz, int slow, double *part) {
  const int k = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[PI_NV] = {0, 0, 0, 0, 0};
  if (i < n) {
    const PiBead me = b[k];
    const double dP = (double)P;
    if (slow) {
      me.gx[i] = me.gx[i] / dP;
      me.gy[i] = me.gy[i] / dP;
      me.gz[i] = me.gz[i] / dP;
    }
    double fx = me.hx[i] / dP, fy = me.hy[i] / dP, fz = me.hz[i] / dP;
    const dbl4 p = me.pos[i];
    for (int dir = 0; dir < 2; ++dir) {
      const dbl4 o = b[dir == 0 ? (k + P - 1) % P : (k + 1) % P].pos[i];
      double BX = p.x - (double)(float)o.x;
      double BY = p.y - (double)(float)o.y;
      double BZ = p.z - (double)(float)o.z;
      pbc_rect(BX, BY, BZ, bx, by, bz, 0.5 * bx, 0.5 * by, 0.5 * bz);
      const double BSQ = BX * BX + BY * BY + BZ * BZ;
      const double BBB = sqrt(BSQ);
      const double R1I = 1.0 / BBB;
      const double DBND = BBB * beadfac * smass[i];
      const double EBDD = DBND * BBB;
      const double FORB = -2.0 * DBND * R1I;
      fx = fx + BX * FORB;
      fy = fy + BY * FORB;
      fz = fz + BZ * FORB;
      acc[0] += EBDD;
      if (dir == 0) {
        acc[1] += FORB * BSQ;
        acc[2] += FORB * (BX * BX) * dP;
        acc[3] += FORB * (BY * BY) * dP;
        acc[4] += FORB * (BZ * BZ) * dP;
      }
    }
    me.hx[i] = fx;
    me.hy[i] = fy;
    me.hz[i] = fz;
  }
  __shared__ double red[PI_NV][PI_THREADS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < PI_NV; ++v) {
    const double s = warp_sum(acc[v]);
    if (lane == 0) red[v][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < PI_NV) {
    double s = 0.0;
    for (int q = 0; q < PI_THREADS / 32; ++q) s += red[threadIdx.x][q];
    part[((size_t)k * gridDim.x + blockIdx.x) * PI_NV + threadIdx.x] = s;
  }
}

// Per bead: block partials in block order; VIRF into the bead's scalars;
// QEK = 0.5 * sum over beads added to the short-step accumulator.
__global__ void k_pi_springs_sum(int P, int nblk, const double *__restrict__ part,
                                 const PiBead *__restrict__ b, double *bead, double *qeks) {
  extern __shared__ double q[];
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    double s[PI_NV] = {0, 0, 0, 0, 0};
    for (int blk = 0; blk < nblk; ++blk)
      for (int v = 0; v < PI_NV; ++v) s[v] += part[((size_t)k * nblk + blk) * PI_NV + v];
    b[k].sc->virfx = b[k].sc->virfx + s[2];
    b[k].sc->virfy = b[k].sc->virfy + s[3];
    b[k].sc->virfz = b[k].sc->virfz + s[4];
    bead[2 * k] = s[0];
    bead[2 * k + 1] = s[1];
    q[k] = s[0];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < P; ++k) t += q[k];
    *qeks = *qeks + 0.5 * t;
  }
}

// ctr[0]: records written since the start of the call, ctr[1]: MSTEP of the
// step before the first (graph replays need the step number from memory).
__global__ void k_pi_record(int P, const PiBead *__restrict__ b, const double *__restrict__ bead,
                            double *qeks, int nfreq, mdx_pimd_record *rec, int *ctr) {
  mdx_pimd_record r;
  r.mstep = ctr[1] + ctr[0] + 1;
  r.qek = *qeks / nfreq;
  r.virpi = r.pe = r.tke = r.temp = 0.0;
  for (int k = 0; k < P; ++k) {
    const mdx_scalars *s = b[k].sc;
    r.virpi += bead[2 * k + 1];
    r.pe += s->pe1 + s->pe2 + s->pels1 + s->pels2 + s->spe + s->pint;
    r.tke += b[k].th->tke;
    r.temp += b[k].th->temp;
  }
  r.temp /= P;
  *qeks = 0.0;
  if (rec) rec[ctr[0]] = r;
  ctr[0] = ctr[0] + 1;
}

__global__ void k_pi_start(int *ctr, int mstep0) {
  ctr[0] = 0;
  ctr[1] = mstep0;
}

}  // namespace

struct mdx_pimd {
  int P = 0, n = 0;
  mdx_pimd_params pp{};
  std::vector<mdx_ctx *> beads;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  PiBead *db = nullptr;      // [P]
  double *thermo = nullptr;  // [jnh][n]
  double *smass = nullptr;   // MASS(NSITE(i)) per atom
  double *part = nullptr;    // [P][nblk][PI_NV]
  double *bead = nullptr;    // [P][2]: QEK, VIRPI of the last spring pass
  double *qeks = nullptr;    // QEKS accumulator of the long step
  mdx_pimd_record *rec = nullptr;
  int *rec_ctr = nullptr;
  int rec_cap = 0;
  cudaGraphExec_t g[2] = {nullptr, nullptr};
  void *mv_tab = nullptr;            // [P] bead table of the batched integrator passes
  std::vector<unsigned char> mv_host;  // its host image
  std::string err;
  int nblk() const { return (n + PI_THREADS - 1) / PI_THREADS; }
};

namespace {

int pi_cuda(mdx_pimd *pi, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return MDX_OK;
  pi->err = std::string(what) + ": " + cudaGetErrorString(e);
  return MDX_ERR_CUDA;
}
#define PI_CUDA(x) RC(pi_cuda(pi, (x), #x))

int pi_alloc(mdx_pimd *pi, void **p, size_t bytes) {
  PI_CUDA(cudaMallocAsync(p, bytes, pi->stream));
  PI_CUDA(cudaMemsetAsync(*p, 0, bytes, pi->stream));
  return MDX_OK;
}

int fork(mdx_pimd *pi) {
  PI_CUDA(cudaEventRecord(pi->fork, pi->stream));
  for (mdx_ctx *c : pi->beads) PI_CUDA(cudaStreamWaitEvent(c->stream, pi->fork, 0));
  return MDX_OK;
}

int join(mdx_pimd *pi) {
  for (int k = 0; k < pi->P; ++k) {
    PI_CUDA(cudaEventRecord(pi->join[k], pi->beads[k]->stream));
    PI_CUDA(cudaStreamWaitEvent(pi->stream, pi->join[k], 0));
  }
  return MDX_OK;
}

int bead_err(mdx_pimd *pi, int k, int rc) {
  if (rc) pi->err = "bead " + std::to_string(k) + ": " + pi->beads[k]->err;
  return rc;
}

#define EACH_BEAD(body)                                        \
  for (int k = 0; k < pi->P; ++k) {                            \
    mdx_ctx *ctx = pi->beads[k];                               \
    (void)ctx;                                                 \
    int rc_b = [&]() -> int { body; return MDX_OK; }();        \
    if (rc_b) return bead_err(pi, k, rc_b);                    \
  }

int nose(mdx_pimd *pi) {
  mdx_ctx *c0 = pi->beads[0];
  k_pi_nose<<<(pi->n + 255) / 256, 256, 0, pi->stream>>>(
      pi->n, pi->P, pi->db, c0->dv.massdi, pi->thermo, pi->pp.jnh, pi->pp.conveq,
      c0->p.trtemp, pi->pp.dqqt, pi->pp.fnh, c0->p.tsteb);
  PI_CUDA(cudaGetLastError());
  return MDX_OK;
}

int springs(mdx_pimd *pi, bool slow) {
  mdx_ctx *c0 = pi->beads[0];
  dim3 grid(pi->nblk(), pi->P);
  k_pi_springs<<<grid, PI_THREADS, 0, pi->stream>>>(pi->n, pi->P, pi->db, pi->smass,
                                                    pi->pp.beadfac, c0->boxl, c0->boyl,
                                                    c0->bozl, slow ? 1 : 0, pi->part);
  PI_CUDA(cudaGetLastError());
  k_pi_springs_sum<<<1, 64, sizeof(double) * pi->P, pi->stream>>>(pi->P, pi->nblk(), pi->part,
                                                                  pi->db, pi->bead, pi->qeks);
  PI_CUDA(cudaGetLastError());
  return MDX_OK;
}

// 1.2 of pimd.f (lines 48-72), eager.
int prologue(mdx_pimd *pi) {
  RC(fork(pi));
  EACH_BEAD(RC(launch_vira(ctx, 0)); RC(launch_build_lists(ctx)); RC(launch_getcom(ctx));
            RC(api_do_slforces(ctx, false)); RC(api_do_fforces(ctx, 0, false)));
  RC(join(pi));
  RC(springs(pi, true));
  PI_CUDA(cudaMemsetAsync(pi->qeks, 0, sizeof(double), pi->stream));
  return MDX_OK;
}

// The bead table of the batched integrator passes (pointers only: written
// before a run, once every bead has its lists).
int fill_bead_table(mdx_pimd *pi) {
  const size_t b = bead_move_bytes();
  pi->mv_host.resize(b * pi->P);
  for (int k = 0; k < pi->P; ++k) bead_move_fill(pi->beads[k], pi->mv_host.data() + b * k);
  PI_CUDA(ctx_copy(pi->stream, pi->mv_tab, pi->mv_host.data(), b * pi->P, cudaMemcpyHostToDevice));
  return MDX_OK;
}

// One long step (pimd.f:84-194).  The integrator passes of all beads run as
// one launch each on the ensemble's stream (kicks and GETEMP share a pass
// over the atoms; the drift carries GETCOM and the coordinate mirrors): the
// same operations in the same order as per-bead kernels.  The forces run
// per bead, forked across the bead streams.
int long_step(mdx_pimd *pi, int mstep) {
  mdx_ctx *c0 = pi->beads[0];
  const mdx_params &p = c0->p;
  const int NFREQ = p.nfreq, NFREQ2 = NFREQ / 2 + 1, P = pi->P;
  const double HTSTEP = 0.5 * p.tstep, TSTEB = p.tsteb, HTSTEB = 0.5 * p.tsteb;
  cudaStream_t st = pi->stream;
  RC(launch_getemp_beads(c0, P, pi->mv_tab, st, {}, {2, HTSTEP, 1, HTSTEB}));
  RC(nose(pi));
  for (int s = 1; s <= NFREQ; ++s) {
    RC(launch_kick_drift_com_beads(c0, P, pi->mv_tab, st, 0.0, TSTEB));
    RC(fork(pi));
    EACH_BEAD(if (s == NFREQ2) RC(launch_list_update(ctx, mstep));
              if (s == NFREQ) {
                RC(api_do_slforces(ctx, false, true));
                RC(api_do_fforces(ctx, 1, false, true));
              } else {
                RC(api_do_fforces(ctx, 0, false, true));
              });
    RC(join(pi));
    RC(springs(pi, s == NFREQ));
    if (s < NFREQ) {
      RC(launch_getemp_beads(c0, P, pi->mv_tab, st, {1, HTSTEB}, {1, HTSTEB}));
      RC(nose(pi));
    } else {
      RC(launch_getemp_beads(c0, P, pi->mv_tab, st, {1, HTSTEB}, {2, HTSTEP}));
      RC(launch_getemp_beads(c0, P, pi->mv_tab, st));
    }
  }
  k_pi_record<<<1, 1, 0, pi->stream>>>(pi->P, pi->db, pi->bead, pi->qeks, NFREQ, pi->rec,
                                        pi->rec_ctr);
  PI_CUDA(cudaGetLastError());
  return MDX_OK;
}

int graph_long_step(mdx_pimd *pi, int mstep) {
  mdx_ctx *c0 = pi->beads[0];
  const int g = list_update_every_step(c0) || mstep % c0->p.ichnb == 0 ? 1 : 0;
  if (!pi->g[g]) {
    PI_CUDA(cudaStreamBeginCapture(pi->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = long_step(pi, mstep);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(pi->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    PI_CUDA(e);
    const cudaError_t ei = cudaGraphInstantiate(&pi->g[g], graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) pi->g[g] = nullptr;
    PI_CUDA(ei);
  }
  PI_CUDA(cudaGraphLaunch(pi->g[g], pi->stream));
  return MDX_OK;
}

int finish(mdx_pimd *pi, int32_t nsteps, mdx_pimd_record *rec) {
  PI_CUDA(cudaStreamSynchronize(pi->stream));
  for (int k = 0; k < pi->P; ++k) RC(bead_err(pi, k, api_check_err(pi->beads[k])));
  if (rec && nsteps > 0)
    PI_CUDA(ctx_copy(pi->stream, rec, pi->rec, sizeof(mdx_pimd_record) * nsteps, cudaMemcpyDeviceToHost));
  return MDX_OK;
}

int run(mdx_pimd *pi, int32_t nsteps, int32_t mstep0, bool with_prologue,
        mdx_pimd_record *rec) {
  if (nsteps > pi->rec_cap) {
    if (pi->rec) PI_CUDA(cudaFreeAsync(pi->rec, pi->stream));
    pi->rec = nullptr;
    RC(pi_alloc(pi, reinterpret_cast<void **>(&pi->rec), sizeof(mdx_pimd_record) * nsteps));
    pi->rec_cap = nsteps;
    for (auto &g : pi->g)  // graphs hold the old record buffer
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }
  if (with_prologue) RC(prologue(pi));
  RC(fill_bead_table(pi));
  k_pi_start<<<1, 1, 0, pi->stream>>>(pi->rec_ctr, mstep0);
  PI_CUDA(cudaGetLastError());
  const bool graphs = pi->beads[0]->use_graphs;
  for (int s = 1; s <= nsteps; ++s) {
    if (graphs) RC(graph_long_step(pi, mstep0 + s));
    else RC(long_step(pi, mstep0 + s));
  }
  return finish(pi, nsteps, rec);
}

}  // namespace

extern "C" {

int mdx_pimd_open(mdx_ctx *const *beads, const mdx_pimd_params *par, mdx_pimd **out) {
  if (!beads || !par || !out || par->nbeads < 2 || par->jnh < 1) return MDX_ERR_ARG;
  *out = nullptr;
  mdx_ctx *c0 = beads[0];
  for (int k = 0; k < par->nbeads; ++k) {
    mdx_ctx *c = beads[k];
    if (!c || !c->have_topo || !c->have_params || !c->have_state) return MDX_ERR_STATE;
    if (c->dv.n != c0->dv.n || c->dv.nop != c0->dv.nop || c->d.ntypes != c0->d.ntypes ||
        c->d.precision != c0->d.precision || c->device != c0->device)
      return MDX_ERR_ARG;
    if (c->p.lnvt || c->p.lnpt || c->p.icell != 0) {
      c0->err = "PIMD: bead thermostats only (no NVT/NPT scaling), rectangular cell";
      return MDX_ERR_UNSUPPORTED;
    }
    if (c->timing) return MDX_ERR_STATE;
  }
  mdx_pimd *pi = new mdx_pimd();
  pi->P = par->nbeads;
  pi->n = c0->dv.n;
  pi->pp = *par;
  pi->beads.assign(beads, beads + par->nbeads);
  int rc = MDX_OK;
  auto fail = [&](int r) {
    mdx_pimd_close(pi);
    return r;
  };
  if (cudaStreamCreateWithFlags(&pi->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&pi->fork, cudaEventDisableTiming) != cudaSuccess)
    return fail(MDX_ERR_CUDA);
  pi->join.resize(pi->P, nullptr);
  for (auto &e : pi->join)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(MDX_ERR_CUDA);
  std::vector<PiBead> hb(pi->P);
  for (int k = 0; k < pi->P; ++k) {
    DevData &d = beads[k]->dv;
    hb[k] = PiBead{d.pos, d.vx, d.vy, d.vz, d.gx, d.gy, d.gz, d.hx, d.hy, d.hz, d.sc, d.th};
  }
  std::vector<double> sm(pi->n);
  for (int i = 0; i < pi->n; ++i) sm[i] = c0->h_mass[c0->h_nsite[i] - 1];
  if ((rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->db), sizeof(PiBead) * pi->P)) ||
      (rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->thermo),
                     sizeof(double) * (size_t)par->jnh * pi->n)) ||
      (rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->smass), sizeof(double) * pi->n)) ||
      (rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->part),
                     sizeof(double) * (size_t)pi->P * pi->nblk() * PI_NV)) ||
      (rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->bead), sizeof(double) * 2 * pi->P)) ||
      (rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->qeks), sizeof(double))) ||
      (rc = pi_alloc(pi, reinterpret_cast<void **>(&pi->rec_ctr), 2 * sizeof(int))) ||
      (rc = pi_alloc(pi, &pi->mv_tab, bead_move_bytes() * pi->P)))
    return fail(rc);
  if (cudaStreamSynchronize(pi->stream) != cudaSuccess ||
      ctx_copy(pi->stream, pi->db, hb.data(), sizeof(PiBead) * pi->P, cudaMemcpyHostToDevice) != cudaSuccess ||
      ctx_copy(pi->stream, pi->smass, sm.data(), sizeof(double) * pi->n, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(MDX_ERR_CUDA);
  *out = pi;
  return MDX_OK;
}

int mdx_pimd_close(mdx_pimd *pi) {
  if (!pi) return MDX_OK;
  for (auto &g : pi->g)
    if (g) cudaGraphExecDestroy(g);
  if (pi->stream) {
    void *ptrs[] = {pi->db, pi->thermo, pi->smass, pi->part, pi->bead, pi->qeks, pi->rec,
                    pi->rec_ctr, pi->mv_tab};
    for (void *p : ptrs)
      if (p) cudaFreeAsync(p, pi->stream);
    cudaStreamSynchronize(pi->stream);
    cudaStreamDestroy(pi->stream);
  }
  if (pi->fork) cudaEventDestroy(pi->fork);
  for (auto e : pi->join)
    if (e) cudaEventDestroy(e);
  delete pi;
  return MDX_OK;
}

int mdx_pimd_run(mdx_pimd *pi, int32_t nsteps, int32_t nsttot, mdx_pimd_record *rec) {
  if (!pi || nsteps < 0) return MDX_ERR_ARG;
  return run(pi, nsteps, nsttot, true, rec);
}

int mdx_pimd_steps(mdx_pimd *pi, int32_t nsteps, int32_t mstep0, mdx_pimd_record *rec) {
  if (!pi || nsteps < 0) return MDX_ERR_ARG;
  for (mdx_ctx *c : pi->beads)
    if (!c->have_lists) return MDX_ERR_STATE;
  return run(pi, nsteps, mstep0, false, rec);
}

void *mdx_pimd_stream(mdx_pimd *pi) { return pi ? (void *)pi->stream : nullptr; }

int mdx_pimd_get_thermo(mdx_pimd *pi, double *thermo) {
  if (!pi || !thermo) return MDX_ERR_ARG;
  if (cudaStreamSynchronize(pi->stream) != cudaSuccess ||
      ctx_copy(pi->stream, thermo, pi->thermo, sizeof(double) * (size_t)pi->pp.jnh * pi->n,
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    return MDX_ERR_CUDA;
  return MDX_OK;
}

int mdx_pimd_set_thermo(mdx_pimd *pi, const double *thermo) {
  if (!pi || !thermo) return MDX_ERR_ARG;
  if (cudaStreamSynchronize(pi->stream) != cudaSuccess ||
      ctx_copy(pi->stream, pi->thermo, thermo, sizeof(double) * (size_t)pi->pp.jnh * pi->n,
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return MDX_ERR_CUDA;
  return MDX_OK;
}

}  // extern "C"
