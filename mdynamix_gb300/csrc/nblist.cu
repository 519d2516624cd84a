// nblist.cu -- CHCNB (forces.f:1813-2205) as an O(N) cell-grid build.
//
// The reference scans all pairs in "parity strips": outer atom I takes
// J = I-2, I-4, ... (same parity, J < I) and J = I+1, I+3, ... (opposite
// parity, J > I).  That rule fixes which atom owns each pair; it is kept here
// so that every owner row holds about half of the atom's neighbours (load
// balance for free) and so that the export reproduces the reference's lists
// entry for entry (the mixed path keeps full rows: both owners).  Cells are
// at least half the list radius wide; candidates come from the 5 x 5 x 5 (or
// fewer, for small boxes) neighbouring cells, a stencil row of consecutive
// cells read as one run of the cell-ordered candidate records; each
// candidate is classified with the reference's exact
// FP64 arithmetic (minimum image, RR2 <= RSSQ, RR2 <= SHORT2, the 8 A bound
// on the intramolecular bonded check, 1-4 pairs to the short list), after an
// FP32 prefilter that only decides pairs far from every boundary.
//
// Rows: nl_idx[i*cap_l + k] (long), ns_idx[i*cap_s + k] (short; bit 31 marks
// a 1-4 pair; the mixed path tiles short rows by 32 owners), counts in
// nl_cnt / ns_cnt.  Entries are atom numbers (FP64 path) or cell-order slots
// of the neighbour records (mixed path; mdx_get_lists maps them back).  Row
// order is deterministic.
#include <algorithm>
#include <cmath>

#include "mdx_internal.cuh"

namespace {

struct BoxD {
  double bx, by, bz, hbx, hby, hbz;
  int icell;     // ICELL: 0 rectangular, 1 truncated octahedron, 2 hexagonal
  double boxy3;  // BOXY3 of the hexagonal cell
};

// CHCNB's minimum image for the box's cell shape (forces.f:1840-1875)
__device__ __forceinline__ void pbc_box(double &dx, double &dy, double &dz, const BoxD &b) {
  if (b.icell == 0) {
    pbc_rect(dx, dy, dz, b.bx, b.by, b.bz, b.hbx, b.hby, b.hbz);
  } else {
    const CellPbc c{b.icell, b.bx, b.by, b.bz, b.hbx, b.hby, b.hbz, b.boxy3};
    pbc_cell(dx, dy, dz, c);
  }
}

// Skin mode: the list kernels of a step run only when the displacement check
// of that step asked for a rebuild (gate == nullptr: always).
__device__ __forceinline__ bool closed(const int *gate) { return gate && *gate == 0; }

__device__ __forceinline__ int wrap_cell(double x, double L, double cw, int n) {
  double u = (x + 0.5 * L) / cw;
  int c = (int)floor(u);
  c %= n;
  if (c < 0) c += n;
  return c;
}

__global__ void k_cell_count(int n, const dbl4 *__restrict__ pos, BoxD b,
                             CellGrid g, int *__restrict__ cell_cnt,
                             int *__restrict__ atom_cell, const int *__restrict__ gate) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || closed(gate)) return;
  dbl4 p = pos[i];
  int cx = wrap_cell(p.x, b.bx, g.cx, g.nx);
  int cy = wrap_cell(p.y, b.by, g.cy, g.ny);
  int cz = wrap_cell(p.z, b.bz, g.cz, g.nz);
  int c = (cz * g.ny + cy) * g.nx + cx;
  atom_cell[i] = c;
  atomicAdd(&cell_cnt[c], 1);
}

// Single-block exclusive scan of the cell counts (ncell is small).
__global__ void k_cell_scan(int ncell, const int *__restrict__ cnt,
                            int *__restrict__ start, int *__restrict__ fill,
                            const int *__restrict__ gate) {
  __shared__ int sh[1024];
  if (closed(gate)) return;
  int carry = 0;
  for (int base = 0; base < ncell; base += 1024) {
    int i = base + threadIdx.x;
    int v = i < ncell ? cnt[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < ncell) {
      start[i] = carry + sh[threadIdx.x] - v;
      fill[i] = 0;
    }
    int tot = sh[1023];
    __syncthreads();
    carry += tot;
  }
  if (threadIdx.x == 0) start[ncell] = carry;
}

__global__ void k_cell_scatter(int n, const int *__restrict__ atom_cell,
                               const int *__restrict__ start,
                               int *__restrict__ fill,
                               int *__restrict__ list, const int *__restrict__ gate) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || closed(gate)) return;
  int c = atom_cell[i];
  int k = atomicAdd(&fill[c], 1);
  list[start[c] + k] = i;
}

// Sort each cell's atoms by index (one warp per cell, odd-even transposition
// over the small cell population) so that rows come out in a fixed order.
__global__ void k_cell_sort(int ncell, const int *__restrict__ start,
                            int *__restrict__ list, const int *__restrict__ gate) {
  int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (c >= ncell || closed(gate)) return;
  int b = start[c], e = start[c + 1], m = e - b;
  for (int pass = 0; pass < m; ++pass) {
    int par = pass & 1;
    for (int k = par + 2 * lane; k + 1 < m; k += 64) {
      int a0 = list[b + k], a1 = list[b + k + 1];
      if (a0 > a1) {
        list[b + k] = a1;
        list[b + k + 1] = a0;
      }
    }
    __syncwarp();
  }
}

// Candidate records in cell order, beside cell_list: the fixed-point
// position and packed (molecule, site) word (mixed path), or the FP32
// mirror's x, y, z bits and the molecule (FP64 path).  k_build then reads a
// run of neighbour cells as one coalesced stream, with no gather through
// the atom index.
__global__ void k_cell_gather(int n, const int *__restrict__ list, const int4 *__restrict__ posi,
                              const float4 *__restrict__ posf, const int4 *__restrict__ ainfo,
                              int4 *__restrict__ cell_pos, int *__restrict__ slot_of,
                              const int *__restrict__ gate = nullptr) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || closed(gate)) return;
  const int j = list[k];
  if (slot_of) slot_of[j] = k;
  if (posi) {
    cell_pos[k] = posi[j];
  } else {
    const float4 f = posf[j];
    cell_pos[k] = make_int4(__float_as_int(f.x), __float_as_int(f.y), __float_as_int(f.z),
                            ainfo[j].y);
  }
}

constexpr int CELL_REACH = 2;  // list cells per list radius (a row of 5 thin cells is one run)

// Ownership of pair (i, j) in the strip loop: i owns it when (i-j) is even
// and j < i, or (i-j) is odd and j > i (forces.f:1834, 2014).
__device__ __forceinline__ bool owns(int i, int j) {
  return (((i - j) & 1) == 0) ? (j < i) : (j > i);
}

// Reaction field (LMNBL): small molecules (at most MMOL = 5 sites) enter
// the lists whole, by the distance of their centres of mass
// (forces.f:1882-1936).
struct MolCut {
  int lmnbl;
  int nsits[MDX_NT];
  const double *X, *Y, *Z;  // centres of mass of the last GETCOM
  const int4 *ainfo;
};

// Exact classification (forces.f:1938-1981): 0 none, 1 short, 2 long,
// 3 short 1-4, -1 excluded bonded pair.  LMNBL: the molecular cutoff (a
// template parameter, so the atomic-cutoff build carries none of its code
// or its runtime-indexed per-type table).
template <bool LMNBL>
__device__ __forceinline__ int classify_exact(
    int i, int j, bool same_mol, const dbl4 &pi, const dbl4 &pj,
    const BoxD &b, double short2, double rl2, const int *__restrict__ nnbb,
    const int *__restrict__ inbb, int nbdmax, const MolCut &mc) {
  double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
  pbc_box(dx, dy, dz, b);
  double rr2 = dx * dx + dy * dy + dz * dz;
  double rrm = rr2;
  if (LMNBL) {
    constexpr int MMOL = 5;
    const int4 ai = mc.ainfo[i], aj = mc.ainfo[j];
    const int nmi = mc.nsits[ai.x], nmj = mc.nsits[aj.x];
    if (!(nmi > MMOL && nmj > MMOL)) {
      double ex, ey, ez;
      if (nmi > MMOL) {
        ex = pi.x - mc.X[aj.y]; ey = pi.y - mc.Y[aj.y]; ez = pi.z - mc.Z[aj.y];
      } else if (nmj > MMOL) {
        ex = mc.X[ai.y] - pj.x; ey = mc.Y[ai.y] - pj.y; ez = mc.Z[ai.y] - pj.z;
      } else {
        ex = mc.X[ai.y] - mc.X[aj.y]; ey = mc.Y[ai.y] - mc.Y[aj.y]; ez = mc.Z[ai.y] - mc.Z[aj.y];
      }
      pbc_box(ex, ey, ez, b);
      rrm = ex * ex + ey * ey + ez * ez;
    }
  }
  if (same_mol && rr2 <= 64.0) {
    int nb = nnbb[i];
    const int jf = j + 1;
    for (int k = 0; k < nb; ++k) {
      int v = inbb[i * nbdmax + k];
      if (v == jf) return -1;
      if (v == -jf) return 3;
    }
  }
  if (rrm <= short2) return 1;
  if (rrm <= rl2) return 2;
  return 0;
}

template <int BLK, bool LMNBL>
__global__ void __launch_bounds__(BLK) k_build(
    int n, const dbl4 *__restrict__ pos, const float4 *__restrict__ posf,
    const int4 *__restrict__ ainfo, const int *__restrict__ nnbb,
    const int *__restrict__ inbb, int nbdmax, BoxD b, CellGrid g,
    const int *__restrict__ atom_cell, const int *__restrict__ cell_start,
    const int *__restrict__ cell_list, const int4 *__restrict__ cell_pos, double short2,
    double rl2, int cap_s,
    int cap_l, int *__restrict__ ns_cnt, int *__restrict__ nl_cnt,
    int *__restrict__ ns_idx, int *__restrict__ nl_idx, int *__restrict__ err,
    int *__restrict__ need, int full, const int4 *__restrict__ posi, float sxf, float syf,
    float szf, dbl4 *__restrict__ pos_ref, const int *__restrict__ gate, MolCut mc) {
  // posi (mixed path): the prefilter takes the wrapped differences of the
  // fixed-point positions and the molecule from their packed word, one
  // 16-byte gather per candidate
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (BLK / 32) + (threadIdx.x >> 5);
  if (i >= n || closed(gate)) return;
  const dbl4 pi = pos[i];
  if (pos_ref && lane == 0) pos_ref[i] = pi;  // skin mode: positions of this build
  const float4 pf = posf[i];
  const int imol = ainfo[i].y;
  const int4 qi = posi ? posi[i] : make_int4(0, 0, 0, 0);
  const int c0 = atom_cell[i];
  const int cx0 = c0 % g.nx, cy0 = (c0 / g.nx) % g.ny, cz0 = c0 / (g.nx * g.ny);
  const float fbx = (float)b.bx, fby = (float)b.by, fbz = (float)b.bz;
  const float fhx = (float)b.hbx, fhy = (float)b.hby, fhz = (float)b.hbz;
  const float rl2f_hi = (float)(rl2 * (1.0 + 1e-4)), rl2f_lo = (float)(rl2 * (1.0 - 1e-4));
  const float s2f_hi = (float)(short2 * (1.0 + 1e-4)), s2f_lo = (float)(short2 * (1.0 - 1e-4));
  int ns = 0, nl = 0;
  constexpr int R = CELL_REACH, W = 2 * CELL_REACH + 1;
  const int ox0 = g.nx >= W ? -R : 0, ox1 = g.nx >= W ? R : g.nx - 1;
  const int oy0 = g.ny >= W ? -R : 0, oy1 = g.ny >= W ? R : g.ny - 1;
  const int oz0 = g.nz >= W ? -R : 0, oz1 = g.nz >= W ? R : g.nz - 1;
  // offsets stay within one period (|o| <= R < W <= n): a conditional wrap,
  // no integer division
  auto wrap = [](int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); };
  auto wrapx = [&](int ox) { return g.nx >= W ? wrap(cx0 + ox, g.nx) : ox; };
  for (int oz = oz0; oz <= oz1; ++oz)
    for (int oy = oy0; oy <= oy1; ++oy) {
      const int cy = g.ny >= W ? wrap(cy0 + oy, g.ny) : oy;
      const int cz = g.nz >= W ? wrap(cz0 + oz, g.nz) : oz;
      const int crow = (cz * g.ny + cy) * g.nx;
      // the row's stencil cells in stencil order, consecutive cells merged
      // into one run of the cell-sorted arrays (the order of candidates is
      // unchanged)
      for (int ox = ox0; ox <= ox1;) {
        const int cxa = wrapx(ox);
        int cxb = cxa;
        while (ox < ox1 && wrapx(ox + 1) == cxb + 1) {
          ++ox;
          ++cxb;
        }
        ++ox;
        const int s = cell_start[crow + cxa], e = cell_start[crow + cxb + 1];
        for (int base = s; base < e; base += 32) {
          int kind = 0;
          int j = -1;
          if (base + lane < e) {
            j = cell_list[base + lane];
            const int4 qj = cell_pos[base + lane];  // independent of the load of j
            if (j != i && (full || owns(i, j))) {
              const bool same =
                  posi ? ((unsigned)qj.w >> MDX_SITE_BITS) == ((unsigned)qi.w >> MDX_SITE_BITS)
                       : qj.w == imol;
              // the molecular cutoff and the non-rectangular cells: exact test only
              if (same || LMNBL || b.icell) {
                kind = classify_exact<LMNBL>(i, j, same, pi, pos[j], b, short2, rl2,
                                      nnbb, inbb, nbdmax, mc);
              } else {
                float dx, dy, dz;
                if (posi) {
                  dx = fixdiff(qi.x, qj.x, sxf);
                  dy = fixdiff(qi.y, qj.y, syf);
                  dz = fixdiff(qi.z, qj.z, szf);
                } else {
                  dx = pf.x - __int_as_float(qj.x);
                  dy = pf.y - __int_as_float(qj.y);
                  dz = pf.z - __int_as_float(qj.z);
                  pbc_rectf(dx, dy, dz, fbx, fby, fbz, fhx, fhy, fhz);
                }
                float d2 = dx * dx + dy * dy + dz * dz;
                if (d2 > rl2f_hi) {
                  kind = 0;
                } else if (d2 < rl2f_lo && (d2 < s2f_lo || d2 > s2f_hi)) {
                  kind = d2 < s2f_lo ? 1 : 2;
                } else {
                  kind = classify_exact<LMNBL>(i, j, false, pi, pos[j], b, short2, rl2,
                                        nnbb, inbb, nbdmax, mc);
                }
              }
            }
          }
          unsigned ms = __ballot_sync(0xffffffffu, kind == 1 || kind == 3);
          unsigned ml = __ballot_sync(0xffffffffu, kind == 2);
          unsigned lower = (1u << lane) - 1u;
          // full rows (mixed path) hold the neighbour's cell-order slot
          const int v = full ? base + lane : j;
          if (kind == 1 || kind == 3) {
            int k = ns + __popc(ms & lower);
            if (k < cap_s)
              ns_idx[list_slot(i, k, cap_s, full)] = v | (kind == 3 ? (int)0x80000000 : 0);
          } else if (kind == 2) {
            int k = nl + __popc(ml & lower);
            if (k < cap_l) nl_idx[list_slot(i, k, cap_l, false)] = v;
          }
          ns += __popc(ms);
          nl += __popc(ml);
        }
      }
    }
  if (lane == 0) {
    ns_cnt[i] = min(ns, cap_s);
    nl_cnt[i] = min(nl, cap_l);
    if (ns > cap_s) {
      atomicOr(err, DERR_LIST_SHORT);
      atomicMax(&need[0], ns);
    }
    if (nl > cap_l) {
      atomicOr(err, DERR_LIST_LONG);
      atomicMax(&need[1], nl);
    }
  }
}

// FP32 mirror for the list prefilter and, for the mixed path, 32-bit
// fixed-point coordinates: round(x / L * 2^32) kept modulo 2^32.
__global__ void k_mirror(int n, const dbl4 *__restrict__ pos,
                         float4 *__restrict__ posf, int4 *__restrict__ posi,
                         const int *__restrict__ pinfo, double ibx, double iby,
                         double ibz, const int *__restrict__ gate = nullptr) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || closed(gate)) return;
  dbl4 p = pos[i];
  posf[i] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
  if (posi) {
    const double two32 = 4294967296.0;
    long long xi = __double2ll_rn(p.x * ibx * two32);
    long long yi = __double2ll_rn(p.y * iby * two32);
    long long zi = __double2ll_rn(p.z * ibz * two32);
    posi[i] = make_int4((int)(unsigned)(unsigned long long)xi,
                        (int)(unsigned)(unsigned long long)yi,
                        (int)(unsigned)(unsigned long long)zi, pinfo[i]);
  }
}

__global__ void k_count_totals(int n, const int *__restrict__ ns_cnt,
                               const int *__restrict__ nl_cnt,
                               mdx_scalars *sc, int *__restrict__ builds,
                               const int *__restrict__ gate) {
  if (closed(gate)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(builds, 1);  // once per build
  int s = 0, l = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    s += ns_cnt[i];
    l += nl_cnt[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    l += __shfl_xor_sync(0xffffffffu, l, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&sc->mbsh, s);
    atomicAdd(&sc->mbln, l);
  }
}

__global__ void k_halve_counts(mdx_scalars *sc, const int *__restrict__ gate) {
  if (closed(gate)) return;
  sc->mbsh /= 2;
  sc->mbln /= 2;
}

// Zero n ints when the gate is open (a memset that a skin-mode step skips).
__global__ void k_zero_gated(int *__restrict__ p, int n, const int *__restrict__ gate) {
  if (closed(gate)) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    p[k] = 0;
}

// Skin mode: opens the gate when some atom has moved more than half the skin
// (minimum image) since the last build.  The gate word was zeroed just before.
__global__ void k_skin_check(int n, const dbl4 *__restrict__ pos,
                             const dbl4 *__restrict__ pos_ref, BoxD b, double h2,
                             int *__restrict__ gate) {
  bool far = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const dbl4 p = pos[i], r = pos_ref[i];
    double dx = p.x - r.x, dy = p.y - r.y, dz = p.z - r.z;
    pbc_rect(dx, dy, dz, b.bx, b.by, b.bz, b.hbx, b.hby, b.hbz);
    far |= dx * dx + dy * dy + dz * dz > h2;
  }
  if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) *gate = 1;
}

__global__ void k_gate_zero(int *__restrict__ gate) { *gate = 0; }

}  // namespace

int launch_mirror_f32(mdx_ctx *ctx) {
  MDX_TIMER(ctx, MDX_T_OTHER);
  DevData &d = ctx->dv;
  k_mirror<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(
      d.n, d.pos, d.posf, ctx->mixed() ? d.posi : nullptr, d.pinfo, 1.0 / ctx->boxl,
      1.0 / fix_period_y(ctx), 1.0 / ctx->bozl);
  MDX_LAUNCHED(ctx);
  return launch_cell_refresh(ctx);
}

int launch_cell_refresh(mdx_ctx *ctx) {
  if (!ctx->mixed() || !ctx->have_lists) return MDX_OK;
  DevData &d = ctx->dv;
  k_cell_gather<<<(d.n + 255) / 256, 256, 0, ctx->stream>>>(
      d.n, d.cell_list, d.posi, d.posf, d.ainfo, d.cell_pos, nullptr);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

static MolCut mol_cut(const mdx_ctx *ctx) {
  MolCut m{};
  m.lmnbl = ctx->p.lmnbl;
  for (int t = 0; t < MDX_NT; ++t) m.nsits[t] = ctx->nsits[t];
  m.X = ctx->dv.X;
  m.Y = ctx->dv.Y;
  m.Z = ctx->dv.Z;
  m.ainfo = ctx->dv.ainfo;
  return m;
}

// CHCNB.  gate != nullptr (skin mode, inside a step): every kernel of the
// build runs only if the displacement check of this step opened the gate, so
// a captured step graph holds the build whether or not it happens.
static int build_lists(mdx_ctx *ctx, const int *gate) {
  MDX_TIMER(ctx, MDX_T_LIST);
  DevData &d = ctx->dv;
  // CHCNB puts every pair within SHORT in the short list even when SHORT
  // exceeds the cutoff (forces.f:1964-1976), so the search radius covers both
  const double rl = std::max(ctx->p.rcut + ctx->p.rskin, ctx->p.rshort);
  // the molecular cutoff lists atoms up to twice a small molecule's reach
  // from its centre of mass beyond the cutoff
  const double rsearch =
      !ctx->p.lmnbl ? rl
      : ctx->mol_reach >= 0.0
          ? rl + 2.0 * ctx->mol_reach
          : rl + std::min(ctx->boxl, std::min(ctx->boyl, ctx->bozl));  // reach unknown
  BoxD b{ctx->boxl, ctx->boyl, ctx->bozl, 0.5 * ctx->boxl, 0.5 * ctx->boyl,
         0.5 * ctx->bozl, ctx->p.icell, 0.66666666666666666667 * ctx->boyl};
  CellGrid g;
  // cells at least rl / CELL_REACH wide, stencil +-CELL_REACH cells (a
  // (2 R + 1)^3 stencil of thinner cells tests fewer far candidates than
  // 27 cells of width rl); below 2 R + 1 cells a dimension is scanned whole.
  // A non-rectangular cell's nearest image need not lie in the rectangular
  // stencil: one cell, every pair tested (as the reference's CHCNB does).
  const bool whole = ctx->p.icell != 0;
  g.nx = whole ? 1 : std::max(1, (int)std::floor(CELL_REACH * ctx->boxl / rsearch));
  g.ny = whole ? 1 : std::max(1, (int)std::floor(CELL_REACH * ctx->boyl / rsearch));
  g.nz = whole ? 1 : std::max(1, (int)std::floor(CELL_REACH * ctx->bozl / rsearch));
  g.cx = ctx->boxl / g.nx;
  g.cy = ctx->boyl / g.ny;
  g.cz = ctx->bozl / g.nz;
  g.ncell = g.nx * g.ny * g.nz;
  if (g.ncell != ctx->grid.ncell) {
    if (gate) {  // a gated build never allocates (the box is fixed in skin mode)
      ctx->err = "skin mode: the cell grid changed inside a step";
      return MDX_ERR_STATE;
    }
    ctx->drop_graphs();
    ctx_free(ctx, d.cell_cnt);
    ctx_free(ctx, d.cell_start);
    MDX_CUDA(ctx_alloc(ctx, &d.cell_cnt, sizeof(int) * (g.ncell + 1) * 2));
    MDX_CUDA(ctx_alloc(ctx, &d.cell_start, sizeof(int) * (g.ncell + 1)));
  }
  if (ctx->p.rskin > 0.0 && !d.pos_ref) {
    if (gate) {
      ctx->err = "skin mode: no list built before the step";
      return MDX_ERR_STATE;
    }
    MDX_CUDA(ctx_alloc(ctx, &d.pos_ref, sizeof(dbl4) * (size_t)d.n));
  }
  dbl4 *pos_ref = ctx->p.rskin > 0.0 ? d.pos_ref : nullptr;
  ctx->grid = g;
  ctx->list_rl2 = rl * rl;
  int *fill = d.cell_cnt + (g.ncell + 1);
  const int T = 256;
  k_zero_gated<<<(g.ncell + 1 + T - 1) / T, T, 0, ctx->stream>>>(d.cell_cnt, g.ncell + 1, gate);
  MDX_LAUNCHED(ctx);
  k_mirror<<<(d.n + T - 1) / T, T, 0, ctx->stream>>>(
      d.n, d.pos, d.posf, ctx->mixed() ? d.posi : nullptr, d.pinfo, 1.0 / ctx->boxl,
      1.0 / fix_period_y(ctx), 1.0 / ctx->bozl, gate);
  MDX_LAUNCHED(ctx);
  k_cell_count<<<(d.n + T - 1) / T, T, 0, ctx->stream>>>(d.n, d.pos, b, g,
                                                          d.cell_cnt,
                                                          d.atom_cell, gate);
  MDX_LAUNCHED(ctx);
  k_cell_scan<<<1, 1024, 0, ctx->stream>>>(g.ncell, d.cell_cnt, d.cell_start,
                                           fill, gate);
  MDX_LAUNCHED(ctx);
  k_cell_scatter<<<(d.n + T - 1) / T, T, 0, ctx->stream>>>(
      d.n, d.atom_cell, d.cell_start, fill, d.cell_list, gate);
  MDX_LAUNCHED(ctx);
  k_cell_sort<<<(g.ncell + 7) / 8, 256, 0, ctx->stream>>>(g.ncell, d.cell_start,
                                                          d.cell_list, gate);
  MDX_LAUNCHED(ctx);
  k_cell_gather<<<(d.n + T - 1) / T, T, 0, ctx->stream>>>(
      d.n, d.cell_list, ctx->mixed() ? d.posi : nullptr, d.posf, d.ainfo, d.cell_pos,
      ctx->mixed() ? d.slot_of : nullptr, gate);
  MDX_LAUNCHED(ctx);
  int *need = d.shake_iter + 4;  // two ints of scratch after the SHAKE counter
  k_zero_gated<<<1, 32, 0, ctx->stream>>>(need, 2, gate);
  MDX_LAUNCHED(ctx);
  const int BLK = 256;
#define KB(L)                                                                              \
  k_build<BLK, L><<<(d.n + BLK / 32 - 1) / (BLK / 32), BLK, 0, ctx->stream>>>(              \
      d.n, d.pos, d.posf, d.ainfo, d.nnbb, d.inbb, d.nbdmax, b, g, d.atom_cell,            \
      d.cell_start, d.cell_list, d.cell_pos, ctx->p.rshort * ctx->p.rshort, rl * rl,       \
      d.cap_s, d.cap_l, d.ns_cnt, d.nl_cnt, d.ns_idx, d.nl_idx, d.err, need,               \
      ctx->mixed() ? 1 : 0, ctx->mixed() ? d.posi : nullptr,                               \
      (float)(ctx->boxl / 4294967296.0), (float)(fix_period_y(ctx) / 4294967296.0),               \
      (float)(ctx->bozl / 4294967296.0), pos_ref, gate, mol_cut(ctx))
  if (ctx->p.lmnbl) KB(true);
  else KB(false);
#undef KB
  MDX_LAUNCHED(ctx);
  k_zero_gated<<<1, 32, 0, ctx->stream>>>(&d.sc->mbsh, 2, gate);
  MDX_LAUNCHED(ctx);
  k_count_totals<<<64, 256, 0, ctx->stream>>>(d.n, d.ns_cnt, d.nl_cnt, d.sc,
                                              &d.th->list_builds, gate);
  MDX_LAUNCHED(ctx);
  if (ctx->mixed()) {  // full rows count every pair twice
    k_halve_counts<<<1, 1, 0, ctx->stream>>>(d.sc, gate);
    MDX_LAUNCHED(ctx);
  }
  ctx->have_lists = true;
  return MDX_OK;
}

int launch_build_lists(mdx_ctx *ctx) { return build_lists(ctx, nullptr); }

bool list_update_every_step(const mdx_ctx *ctx) { return ctx->p.rskin > 0.0; }

// The list update of long step mstep: CHCNB every ICHNB-th step (the
// reference's rule), or in skin mode a rebuild whenever an atom has moved
// more than half the skin since the last build, decided on the device.
int launch_list_update(mdx_ctx *ctx, int mstep) {
  if (ctx->p.rskin <= 0.0) return mstep % ctx->p.ichnb == 0 ? build_lists(ctx, nullptr) : MDX_OK;
  DevData &d = ctx->dv;
  if (!d.pos_ref) {
    ctx->err = "skin mode: no list built before the step";
    return MDX_ERR_STATE;
  }
  int *gate = d.shake_iter + 6;
  BoxD b{ctx->boxl, ctx->boyl, ctx->bozl, 0.5 * ctx->boxl, 0.5 * ctx->boyl,
         0.5 * ctx->bozl, 0, 0.0};  // skin mode: rectangular cells only
  {
    MDX_TIMER(ctx, MDX_T_LIST);
    k_gate_zero<<<1, 1, 0, ctx->stream>>>(gate);
    MDX_LAUNCHED(ctx);
    k_skin_check<<<ctx->nsm, 256, 0, ctx->stream>>>(d.n, d.pos, d.pos_ref, b,
                                                    0.25 * ctx->p.rskin * ctx->p.rskin, gate);
    MDX_LAUNCHED(ctx);
  }
  return build_lists(ctx, gate);
}

// Reference layout and order of the lists (forces.f:1956-1957, 2127-2140):
// outer atom I ascending; inside, the even strip (J = I-2, I-4, ...) and then
// the odd strip (J = I+1, I+3, ...); a normal pair is stored (larger, smaller)
// and a 1-4 pair (-I, J).
int export_lists(mdx_ctx *ctx, int32_t *nbs1, int32_t *nbs2, int32_t cap_s,
                 int32_t *nbl1, int32_t *nbl2, int32_t cap_l) {
  DevData &d = ctx->dv;
  const int n = d.n;
  const bool tiled = ctx->mixed();
  const size_t nrow = tiled ? ((size_t)n + 31) / 32 * 32 : (size_t)n;
  std::vector<int> cs(n), cl(n), rs(nrow * d.cap_s), rl((size_t)n * d.cap_l);
  MDX_CUDA(cudaStreamSynchronize(ctx->stream));
  MDX_CUDA(ctx_copy(ctx->stream, cs.data(), d.ns_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost));
  MDX_CUDA(ctx_copy(ctx->stream, cl.data(), d.nl_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost));
  MDX_CUDA(ctx_copy(ctx->stream, rs.data(), d.ns_idx, sizeof(int) * rs.size(), cudaMemcpyDeviceToHost));
  MDX_CUDA(ctx_copy(ctx->stream, rl.data(), d.nl_idx, sizeof(int) * rl.size(), cudaMemcpyDeviceToHost));
  std::vector<int> slot_atom;  // mixed path: rows hold cell-order slots
  if (tiled) {
    slot_atom.resize(n);
    MDX_CUDA(ctx_copy(ctx->stream, slot_atom.data(), d.cell_list, sizeof(int) * n,
                      cudaMemcpyDeviceToHost));
  }
  long ks = 0, kl = 0;
  std::vector<int> row;
  for (int i = 0; i < n; ++i) {
    const int I = i + 1;
    for (int pass = 0; pass < 2; ++pass) {
      const int cnt = pass == 0 ? cs[i] : cl[i];
      row.clear();
      for (int k = 0; k < cnt; ++k) {
        int src_k = pass == 0 ? rs[list_slot(i, k, d.cap_s, tiled)]
                              : rl[list_slot(i, k, d.cap_l, false)];
        if (tiled) src_k = (src_k & (int)0x80000000) | slot_atom[src_k & 0x7fffffff];
        // the mixed path keeps full rows (each pair in both atoms' rows);
        // the reference list holds the owner's copy only
        const int j = src_k & 0x7fffffff;
        const bool own = ((i - j) & 1) == 0 ? (j < i) : (j > i);
        if (own) row.push_back(src_k);
      }
      std::sort(row.begin(), row.end(), [I](int a, int b) {
        int ja = (a & 0x7fffffff) + 1, jb = (b & 0x7fffffff) + 1;
        long ka = ja < I ? (long)(I - ja) : (1L << 40) + (ja - I);
        long kb = jb < I ? (long)(I - jb) : (1L << 40) + (jb - I);
        return ka < kb;
      });
      for (int v : row) {
        const bool is14 = (v & 0x80000000) != 0;
        const int J = (v & 0x7fffffff) + 1;
        int a, b2;
        if (is14) {
          a = -I;
          b2 = J;
        } else {
          a = std::max(I, J);
          b2 = std::min(I, J);
        }
        if (pass == 0) {
          if (ks < cap_s) {
            nbs1[ks] = a;
            nbs2[ks] = b2;
          }
          ++ks;
        } else {
          if (kl < cap_l) {
            nbl1[kl] = a;
            nbl2[kl] = b2;
          }
          ++kl;
        }
      }
    }
  }
  if (ks > cap_s || kl > cap_l) {
    ctx->err = "export buffers too small";
    return MDX_ERR_ARG;
  }
  return MDX_OK;
}
