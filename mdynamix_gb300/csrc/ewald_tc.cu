// ewald_tc.cu -- mixed-precision reciprocal Ewald force pass on the tensor
// cores (FURIR's force loop, forces.f:1286-1314).
//
// With Z_j(p) = a + i b (p = 0..KMAZ) and the paired W of each column
// (P = W(+p) + W(-p), M = W(+p) - W(-p)), the per-atom column sums
//   U.re = sum_p P.re a - M.im b,   U.im = sum_p P.im a + M.re b
// (and V the same with RZV W) are one real matrix product
//   D[atom][4 c + t] = sum_k A[atom][k] B[4 c + t][k],
//   A[atom][2p] = a, A[atom][2p+1] = b,  K = 2 (KMAZ + 1) rounded up to 8,
// so the whole force pass is an (atoms x K) x (K x 4 ncol) GEMM followed by
// F_j += sum_c rv_c Im(T_j(c) U_j(c)), Fz += Im(T_j(c) V_j(c)).
//
// The GEMM runs as TF32 tcgen05 MMAs (M = 128 atoms, N = 128 = 32 columns,
// K = 8 per instruction) with FP32 accumulators in tensor memory.  Each
// operand is split into two TF32 parts, x = hi + lo, and three products
// hi*hi + hi*lo + lo*hi keep close to FP32 accuracy (the dropped lo*lo term
// is 2^-22 relative).  Columns are sorted by m = max |nz| (descending) so a
// tile of 32 columns only runs the K-steps its largest m needs.
//
// A CTA owns 128 atoms: it stages their Z rows (hi and lo) once, then walks
// the column tiles with two shared-memory B buffers and two tensor-memory
// accumulators: MMA(t + 1) runs while the CTA's four warps read tile t's
// accumulator (tcgen05.ld) and fold it into the forces.  The B tiles (hi and
// lo, already in the MMA's core-matrix order) are built once per step by
// k_wtiles from the per-k W values.
#include <algorithm>
#include <vector>

#include "mdx_internal.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int TC_M = 128;         // atoms per CTA (MMA M)
constexpr int TC_N = 128;         // accumulator columns per tile (32 k-columns)
constexpr int TC_COLS = TC_N / 4;  // k-columns per tile
constexpr uint32_t TC_POLLS = 1u << 20;  // bounded mbarrier waits

// Byte offset of element (row r, k) in a K-major, unswizzled tile of kp
// columns: core matrix (r / 8, k / 4) of 128 bytes, SBO = 32 kp, LBO = 128.
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k, int kp) {
  return (uint32_t)((((r >> 3) * (kp >> 2) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}

// B tiles of one step: thread per (tile, row r, 4 consecutive k).  Row r of
// tile t is column slot[32 t + r / 4], component r % 4 (U.re, U.im, V.re,
// V.im); k = 2p takes the a-coefficient, k = 2p + 1 the b-coefficient.  The
// threads with r % 4 = 0 and k = 0 also write the slot's epilogue record
// {nx, ny (int bits; nx = -1 for padding), rv.x, rv.y}.
__global__ void k_wtiles(int ntile, int kp, const int *__restrict__ slot,
                         const KCol *__restrict__ cols, const dbl4 *__restrict__ wk,
                         const float2 *__restrict__ colrv, float *__restrict__ tw,
                         float4 *__restrict__ meta) {
  const int q = kp >> 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntile * TC_N * q) return;
  const int kc = t % q, r = (t / q) % TC_N, tile = t / (q * TC_N);
  const int c = slot[tile * TC_COLS + (r >> 2)];
  const int comp = r & 3;
  if (comp == 0 && kc == 0) {
    float4 mt = make_float4(__int_as_float(-1), 0.f, 0.f, 0.f);
    if (c >= 0) {
      const float2 rv = colrv[c];
      mt = make_float4(__int_as_float(cols[c].nx), __int_as_float(cols[c].ny), rv.x, rv.y);
    }
    meta[tile * TC_COLS + (r >> 2)] = mt;
  }
  float v[4] = {0.f, 0.f, 0.f, 0.f};
  if (c >= 0) {
    const KCol col = cols[c];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int p = 2 * kc + e;
      if (p > col.m) break;
      const int kpl = kcol_k(col, p), kmi = p > 0 ? kcol_k(col, -p) : -1;
      dbl4 a, b;
      a.x = a.y = a.z = a.w = 0.0;
      b = a;
      if (kpl >= 0) a = wk[kpl];
      if (kmi >= 0) b = wk[kmi];
      // {W.re, W.im} for U, {RZV W.re, RZV W.im} for V
      const double wpr = comp < 2 ? a.x : a.z, wpi = comp < 2 ? a.y : a.w;
      const double wmr = comp < 2 ? b.x : b.z, wmi = comp < 2 ? b.y : b.w;
      const double Pr = wpr + wmr, Pi = wpi + wmi, Mr = wpr - wmr, Mi = wpi - wmi;
      v[2 * e] = (float)((comp & 1) ? Pi : Pr);
      v[2 * e + 1] = (float)((comp & 1) ? Mr : -Mi);
    }
  }
  float4 hi, lo;
  tc::tf32_split(v[0], hi.x, lo.x);
  tc::tf32_split(v[1], hi.y, lo.y);
  tc::tf32_split(v[2], hi.z, lo.z);
  tc::tf32_split(v[3], hi.w, lo.w);
  const size_t tsz = (size_t)TC_N * kp;  // floats per part
  float *base = tw + (size_t)tile * 2 * tsz + core_off(r, 4 * kc, kp) / 4;
  *reinterpret_cast<float4 *>(base) = hi;
  *reinterpret_cast<float4 *>(base + tsz) = lo;
}

// Force pass: one CTA of 4 warps per 128 atoms.  Shared memory (1024-byte
// aligned): A hi | A lo | B0 hi | B0 lo | B1 hi | B1 lo | X, Y rows of the
// CTA's atoms ([row][atom], float2).  Thread 0 issues the bulk copies of the
// B tiles (one tile ahead of the MMAs) and the MMAs; all four warps read the
// accumulators.  Barriers: bfull[b] (B tile landed in buffer b), mdone[b]
// (MMAs into accumulator b done, so B buffer b is free again).
__global__ void __launch_bounds__(128, 1) k_rforce_tc(
    int n, int ntile, int kp, const int *__restrict__ tile_ks, const float4 *__restrict__ meta,
    const float4 *__restrict__ tw, const float2 *__restrict__ tab, int kx, int ky, int kz,
    FixScale fsc, unsigned long long *__restrict__ gfix, int *__restrict__ err) {
  // tab: the X, Y and Z tables back to back, row r at tab + r * n
  extern __shared__ unsigned char dsm_raw[];
  __shared__ __align__(8) unsigned long long bfull[2], mdone[2];
  __shared__ uint32_t tmem_base_sh;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = blockIdx.x * TC_M;
  const uint32_t raw = tc::smem_addr(dsm_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  unsigned char *dsm = dsm_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t part = (uint32_t)TC_M * kp * 4;  // bytes of one hi or lo tile
  const uint32_t sA = sbase, sB = sbase + 2 * part;
  float2 *sxy = reinterpret_cast<float2 *>(dsm + 6 * (size_t)part);  // [kx + ky][TC_M]

  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base_sh), 2 * TC_N);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(tc::smem_addr(&bfull[b]), 1);
      tc::mbar_init(tc::smem_addr(&mdone[b]), 1);
    }
    tc::mbar_init_fence();
  }
  __syncthreads();  // barriers initialised before the first copy arrives on them
  // B tile t -> buffer b: one bulk copy of both parts (2 part bytes)
  auto copy_b = [&](int t, int b) {
    const uint32_t bar = tc::smem_addr(&bfull[b]);
    tc::mbar_arrive_expect_tx(bar, 2 * part);
    tc::bulk_g2s(sB + (uint32_t)b * 2 * part, tw + (size_t)t * (2 * part / 16), 2 * part, bar);
  };
  if (tid == 0) {
    if (ntile > 0) copy_b(0, 0);
    if (ntile > 1) copy_b(1, 1);
  }
  // A: this CTA's Z rows, hi and lo parts (rows past n are zero)
  {
    const int i = i0 + tid;
    const float2 *tz = tab + (size_t)(kx + ky) * n;
    for (int kc = 0; kc < (kp >> 2); ++kc) {
      float z[4];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int p = 2 * kc + e;
        float2 v = make_float2(0.f, 0.f);
        if (i < n && p < kz) v = tz[(size_t)p * n + i];
        z[2 * e] = v.x;
        z[2 * e + 1] = v.y;
      }
      float4 hi, lo;
      tc::tf32_split(z[0], hi.x, lo.x);
      tc::tf32_split(z[1], hi.y, lo.y);
      tc::tf32_split(z[2], hi.z, lo.z);
      tc::tf32_split(z[3], hi.w, lo.w);
      const uint32_t o = core_off(tid, 4 * kc, kp);
      *reinterpret_cast<float4 *>(dsm + o) = hi;
      *reinterpret_cast<float4 *>(dsm + part + o) = lo;
    }
  }
  // X and Y rows of the CTA's atoms (clamped past n; those rows are unused)
  for (int k = tid; k < (kx + ky) * TC_M; k += blockDim.x) {
    const int r = k / TC_M, a = k - r * TC_M;
    sxy[k] = tab[(size_t)r * n + min(i0 + a, n - 1)];
  }
  const uint32_t idesc = tc::idesc_tf32(TC_M, TC_N);
  const uint32_t lbo = 128, sbo = 32u * kp;
  bool ok = true;
  auto issue = [&](int t, int b, uint32_t tbase) {
    if (!tc::mbar_wait(tc::smem_addr(&bfull[b]), (uint32_t)(t >> 1) & 1u, TC_POLLS)) ok = false;
    tc::fence_after_sync();
    const int ks = tile_ks[t];
    const uint32_t d = tbase + (uint32_t)(b * TC_N);
    const uint32_t bh = sB + (uint32_t)b * 2 * part, bl = bh + part;
    for (int s = 0; s < ks; ++s) {
      const uint32_t ko = (uint32_t)s * 256;  // 8 TF32 = two core matrices along K
      const uint64_t ah = tc::sdesc(sA + ko, lbo, sbo), al = tc::sdesc(sA + part + ko, lbo, sbo);
      const uint64_t bhd = tc::sdesc(bh + ko, lbo, sbo), bld = tc::sdesc(bl + ko, lbo, sbo);
      tc::mma_tf32(d, ah, bhd, idesc, s > 0 ? 1u : 0u);
      tc::mma_tf32(d, ah, bld, idesc, 1u);
      tc::mma_tf32(d, al, bhd, idesc, 1u);
    }
    tc::mma_commit(tc::smem_addr(&mdone[b]));
  };

  tc::fence_proxy_async();  // A visible to the tensor cores
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base_sh;
  if (tid == 0 && ntile > 0) issue(0, 0, tbase);

  const int i = i0 + 32 * warp + lane;
  const float2 *xa = sxy + 32 * warp + lane;  // this thread's atom, row 0
  float fs[3] = {0.f, 0.f, 0.f}, fc[3] = {0.f, 0.f, 0.f};
  for (int t = 0; t < ntile; ++t) {
    const int b = t & 1;
    // MMA(t) done: accumulator b ready, B buffer b free for tile t + 2
    if (!tc::mbar_wait(tc::smem_addr(&mdone[b]), (uint32_t)(t >> 1) & 1u, TC_POLLS)) ok = false;
    tc::fence_after_sync();
    if (tid == 0 && t + 2 < ntile) copy_b(t + 2, b);
    tc::fence_before_sync();
    __syncthreads();  // epilogue(t - 1) done: accumulator b ^ 1 free
    if (tid == 0 && t + 1 < ntile) {
      tc::fence_after_sync();
      issue(t + 1, b ^ 1, tbase);
    }
    __syncwarp();  // warp 0 converged again before the warp-wide tcgen05.ld
    // epilogue of tile t: 4 chunks of 8 columns (32 accumulator columns)
    float gs[3] = {0.f, 0.f, 0.f};
    for (int h = 0; h < TC_N / 32; ++h) {
      float v[32];
      tc::tmem_ld32(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)(b * TC_N + 32 * h), v);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 mt = __ldg(&meta[t * TC_COLS + 8 * h + j]);  // nx, ny, rv
        const int nx = __float_as_int(mt.x), nys = __float_as_int(mt.y);
        if (nx < 0) continue;  // padding slot
        const float2 X = xa[nx * TC_M];
        float2 Y = xa[(kx + (nys < 0 ? -nys : nys)) * TC_M];
        if (nys < 0) Y.y = -Y.y;
        const float Tr = fmaf(X.x, Y.x, -X.y * Y.y), Ti = fmaf(X.x, Y.y, X.y * Y.x);
        const float imTU = fmaf(Tr, v[4 * j + 1], Ti * v[4 * j]);
        const float imTV = fmaf(Tr, v[4 * j + 3], Ti * v[4 * j + 2]);
        gs[0] = fmaf(mt.z, imTU, gs[0]);
        gs[1] = fmaf(mt.w, imTU, gs[1]);
        gs[2] += imTV;
      }
    }
    tc::fence_before_sync();
#pragma unroll
    for (int a = 0; a < 3; ++a) {  // Kahan-compensated sum over tiles
      const float y = gs[a] - fc[a];
      const float s = fs[a] + y;
      fc[a] = (s - fs[a]) - y;
      fs[a] = s;
    }
  }
  __syncthreads();  // every tensor-memory read is done
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, 2 * TC_N);
  }
  if (!ok) {
    atomicOr(err, DERR_TIMEOUT);
    return;
  }
  if (i < n) {
    const float sc = fsc.scalef;
    gfix[i] += (unsigned long long)(f2ll_rn(fs[0] * sc) - f2ll_rn(fc[0] * sc));
    gfix[n + i] += (unsigned long long)(f2ll_rn(fs[1] * sc) - f2ll_rn(fc[1] * sc));
    gfix[2 * n + i] += (unsigned long long)(f2ll_rn(fs[2] * sc) - f2ll_rn(fc[2] * sc));
  }
}

// Shared memory of the force pass: operands plus the X, Y rows, at least
// 80 KB so that no more than two CTAs (2 x 256 tensor-memory columns) share
// an SM.
size_t tc_smem_bytes(int kp, int kxy) {
  return std::max<size_t>(80 * 1024, 1024 + 6 * (size_t)TC_M * kp * 4 +
                                         (size_t)kxy * TC_M * sizeof(float2));
}

}  // namespace

// Column order and tile table of the tensor-core force pass (host, from the
// k-set columns).  Returns false when the pass does not apply (K too large
// for the shared-memory tiles).
bool tc_force_setup(mdx_ctx *ctx, const std::vector<KCol> &cols, int kmaz) {
  DevData &d = ctx->dv;
  const int kp = ((2 * (kmaz + 1) + 7) / 8) * 8;
  d.tc_on = false;
  const int kxy = d.kx + d.ky;
  if (tc_smem_bytes(kp, kxy) > 227 * 1024) return false;
  std::vector<int> order(cols.size());
  for (size_t c = 0; c < cols.size(); ++c) order[c] = (int)c;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cols[a].m > cols[b].m; });
  const int ntile = ((int)cols.size() + TC_COLS - 1) / TC_COLS;
  std::vector<int> slot((size_t)ntile * TC_COLS, -1), ks(ntile, 0);
  for (size_t s = 0; s < order.size(); ++s) slot[s] = order[s];
  for (int t = 0; t < ntile; ++t) {
    const int m = cols[order[(size_t)t * TC_COLS]].m;  // largest m of the tile
    ks[t] = (2 * (m + 1) + 7) / 8;
  }
  ctx_free(ctx, d.tc_slot);
  ctx_free(ctx, d.tc_w);
  ctx_free(ctx, d.tc_meta);
  d.tc_slot = nullptr;
  d.tc_w = nullptr;
  d.tc_meta = nullptr;
  if (ctx_alloc(ctx, &d.tc_slot, sizeof(int) * (slot.size() + ks.size())) != cudaSuccess ||
      ctx_alloc(ctx, &d.tc_w, sizeof(float) * (size_t)ntile * 2 * TC_N * kp) != cudaSuccess ||
      ctx_alloc(ctx, &d.tc_meta, sizeof(float4) * slot.size()) != cudaSuccess)
    return false;
  d.tc_ks = d.tc_slot + slot.size();
  if (cudaMemcpy(d.tc_slot, slot.data(), sizeof(int) * slot.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(d.tc_ks, ks.data(), sizeof(int) * ks.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess)
    return false;
  if (raise_smem_limit(k_rforce_tc, tc_smem_bytes(kp, kxy)) != cudaSuccess) return false;
  d.tc_ntile = ntile;
  d.tc_kp = kp;
  d.tc_on = true;
  return true;
}

// One step's tensor-core force pass: B tiles from W, then the GEMM + fold.
int tc_force_launch(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  const int q = d.tc_kp / 4;
  const int nth = d.tc_ntile * TC_N * q;
  k_wtiles<<<(nth + 255) / 256, 256, 0, ctx->stream>>>(d.tc_ntile, d.tc_kp, d.tc_slot, d.cols,
                                                       d.wk, d.colrvf, d.tc_w, d.tc_meta);
  MDX_LAUNCHED(ctx);
  k_rforce_tc<<<(d.n + TC_M - 1) / TC_M, 128, tc_smem_bytes(d.tc_kp, d.kx + d.ky),
                ctx->stream>>>(d.n, d.tc_ntile, d.tc_kp, d.tc_ks, d.tc_meta,
                               reinterpret_cast<const float4 *>(d.tc_w), d.tabxf, d.kx, d.ky,
                               d.kz, ctx->fix, d.gfix, d.err);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}
