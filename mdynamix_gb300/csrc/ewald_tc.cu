// ewald_tc.cu -- mixed-precision reciprocal Ewald on the tensor cores: the
// structure factors and the force pass of FURIR (forces.f:1286-1314).
//
// With per-atom phase tables X_j(nx) (charge included), Y_j(ny), Z_j(p) =
// a + i b (p = 0..KMAZ) and the k-set in columns (nx, ny) whose nz = +p and
// -p are taken together (Z_j(-p) = conj Z_j(p)):
//
// * S(k): with T_j(c) = X_j(nx) Y_j(ny), the four sums of a (column, p) pair
//     A1 = sum T.re a, A2 = sum T.im b, A3 = sum T.re b, A4 = sum T.im a
//   are the entries of D = A B^T, A[2c + e][j] = (T.re, T.im)_j(c),
//   B[2p + e][j] = (a, b)_j(p), K running over atoms; then
//   S(c, +p) = (A1 - A2, A3 + A4), S(c, -p) = (A1 + A2, A4 - A3).
// * forces: with the paired W of each column (P = W(+p) + W(-p),
//   M = W(+p) - W(-p)), U.re = sum_p P.re a - M.im b, U.im = sum_p P.im a +
//   M.re b (V the same with RZV W) are D[j][4c + t] = sum_k A[j][k] B[4c+t][k]
//   with A[j][2p] = a, A[j][2p + 1] = b (K = 2 (KMAZ + 1) rounded up to 8);
//   then F_j += sum_c rv_c Im(T_j(c) U_j(c)), Fz += Im(T_j(c) V_j(c)).
//
// Both GEMMs run as TF32 tcgen05 MMAs (M = 128, K = 8 per instruction) into
// FP32 accumulators in tensor memory.  Each operand is split into two TF32
// parts, x = hi + lo, and three products hi*hi + hi*lo + lo*hi keep close to
// FP32 accuracy (the dropped lo*lo term is 2^-22 relative).  The Z operands
// of both passes are written once per step (k_zimages) as images in the
// MMA's core-matrix order, so the passes bring them in with bulk copies; the
// X and Y rows of their atoms come in as one tiled TMA box of the tables
// (the FP32 tables have a row stride of ldn atoms, a multiple of 128, zero
// past n).
#include <cuda.h>

#include <algorithm>
#include <vector>

#include "mdx_internal.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int TC_M = 128;          // atoms per CTA of the force pass (MMA M)
constexpr int TC_N = 128;          // accumulator columns per tile (32 k-columns)
constexpr int TC_COLS = TC_N / 4;  // k-columns per tile
constexpr uint32_t TC_POLLS = 1u << 20;  // bounded mbarrier waits

// Force-pass operand layout (128 rows, K-major, unswizzled), K-step major:
// the 8 K of MMA step s = k / 8 fill 8 KB, [hi | lo] of 4 KB each, and
// within a part core matrix (r / 8, k / 4) of 128 bytes sits at
// ((k / 4) % 2) 2048 + (r / 8) 128: LBO (along K) = 2048, SBO (along M/N)
// = 128.  A tile whose columns need ks steps is then its first ks x 8 KB.
constexpr uint32_t TC_STEP = 8192;  // bytes of one K step (hi and lo)
constexpr uint32_t TC_LO = 4096;    // lo part within a step
constexpr uint32_t TC_LBO = 2048, TC_SBO = 128;
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k) {  // hi part
  return (uint32_t)((k >> 3) * TC_STEP + ((k >> 2) & 1) * TC_LBO + (r >> 3) * TC_SBO +
                    ((r & 7) << 4) + ((k & 3) << 2));
}

// S-pass operand layout: 32 atoms (K) per chunk, core matrices along K
// 144 bytes apart (128 + 16 spreads the shared-memory banks), SBO = 8 x 144.
constexpr int SK_ROWS = 128;  // rows of an M-tile (64 columns x re/im)
constexpr int SK_CH = 32;     // atoms per chunk (K of one stage)
constexpr int SK_LBO = 144;
constexpr int SK_SBO = 8 * SK_LBO;
constexpr uint32_t SK_APART = (SK_ROWS / 8) * SK_SBO;  // bytes of one A part
constexpr int SK_GCH = 32;  // chunks per partial sum written out (1024 atoms)

__host__ __device__ __forceinline__ uint32_t sk_off(int row, int q) {  // (row, atom quad)
  return (uint32_t)((row >> 3) * SK_SBO + q * SK_LBO + ((row & 7) << 4));
}
__host__ __device__ __forceinline__ uint32_t sk_bpart(int np) {  // bytes of one B part
  return (uint32_t)(np / 8) * SK_SBO;
}

// Z images of one step: thread per (p, atom), atoms up to ldn (rows past n
// are zero in the table).  zf: force-pass A operand, per 128-atom tile
// kp / 8 K steps of [hi | lo]; zs: S-pass B operand, per 32-atom chunk [hi | lo]
// of np x 32.  Entries with p >= kz stay zero (set once at allocation).
__global__ void k_zimages(int ldn, int kz, int kp, int np, const float2 *__restrict__ tz,
                          unsigned char *__restrict__ zf, unsigned char *__restrict__ zs) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)kz * ldn) return;
  const int p = (int)(t / ldn), i = (int)(t - (size_t)p * ldn);
  const float2 z = tz[t];
  float ah, al, bh, bl;
  tc::tf32_split(z.x, ah, al);
  tc::tf32_split(z.y, bh, bl);
  if (zf) {
    unsigned char *base = zf + (size_t)(i >> 7) * 1024 * kp;
    const uint32_t o = core_off(i & 127, 2 * p);  // k = 2p and 2p + 1: adjacent
    *reinterpret_cast<float2 *>(base + o) = make_float2(ah, bh);
    *reinterpret_cast<float2 *>(base + TC_LO + o) = make_float2(al, bl);
  }
  if (zs) {
    const uint32_t bp = sk_bpart(np);
    unsigned char *base = zs + (size_t)(i >> 5) * 2 * bp;
    const int j = i & 31;
    const uint32_t o0 = sk_off(2 * p, j >> 2) + 4 * (j & 3);
    const uint32_t o1 = sk_off(2 * p + 1, j >> 2) + 4 * (j & 3);
    *reinterpret_cast<float *>(base + o0) = ah;
    *reinterpret_cast<float *>(base + o1) = bh;
    *reinterpret_cast<float *>(base + bp + o0) = al;
    *reinterpret_cast<float *>(base + bp + o1) = bl;
  }
}

// B tiles of the force pass, one step: thread per (tile, row r, 4
// consecutive k).  Row r of tile t is column slot[32 t + r / 4], component
// r % 4 (U.re, U.im, V.re, V.im); k = 2p takes the a-coefficient, k = 2p + 1
// the b-coefficient.  The threads with r % 4 = 0 and k = 0 also write the
// slot's epilogue record {nx, ny (int bits; nx = -1 for padding), rv.x, rv.y}.
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
  float *base = tw + (size_t)tile * 2 * TC_N * kp + core_off(r, 4 * kc) / 4;
  *reinterpret_cast<float4 *>(base) = hi;
  *reinterpret_cast<float4 *>(base + TC_LO / 4) = lo;
}

// Force pass: one CTA per 128 atoms, warp-specialised.  Warp 16 (lane 0) is
// the producer: bulk copies (once: the tile's Z image, its X and Y rows as
// one TMA box, the epilogue records of all column tiles; then the first
// ks K steps of each B tile) and the MMAs.  Warps 0-15 are the epilogue: warp w reads the accumulator
// lanes 32 (w % 4) .. + 31, columns 32 (w / 4) .. + 31 of each tile (8 of
// its k-columns).  Shared memory (1024-byte aligned): A | B0 | B1 (K steps
// of [hi | lo]) | X, Y rows ([row][atom], float2) | records.
// Barriers: abar (A, X, Y, records landed), bfull[b] (B tile in buffer b
// landed), mdone[b] (MMAs into accumulator b done: B buffer b free,
// accumulator b readable), afree[b] (the 16 epilogue warps are done with
// accumulator b).
constexpr int TC_EPI_WARPS = 16;
constexpr int TC_THREADS = 32 * (TC_EPI_WARPS + 1);
constexpr int TC_REC_BYTES = TC_COLS * 16;  // 32 epilogue records of a tile

__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_rforce_tc(
    int n, int ntile, int kp, const int *__restrict__ tile_ks, const float4 *__restrict__ meta,
    const unsigned char *__restrict__ tw, const unsigned char *__restrict__ zimg,
    const __grid_constant__ CUtensorMap tmxy, int kx, int ky, FixScale fsc,
    unsigned long long *__restrict__ gfix, int *__restrict__ err) {
  // tw: per tile [B hi | B lo]; meta: per column slot {nx, ny, rv.x, rv.y};
  // tmxy: the FP32 tables as a [row][2 ldn] float tensor, box 2 TC_M x
  // (kx + ky)
  extern __shared__ unsigned char dsm_raw[];
  __shared__ __align__(8) unsigned long long abar, bfull[2], mdone[2], afree[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ float red[3][6][TC_M];  // partials of column quarters 1-3 (sum, compensation)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = blockIdx.x * TC_M;
  const uint32_t raw = tc::smem_addr(dsm_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  unsigned char *dsm = dsm_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t btile = (uint32_t)TC_M * kp * 8;  // bytes of one operand tile (hi, lo)
  const int kxy = kx + ky;
  const uint32_t sA = sbase, sB = sbase + btile, oXY = 3 * btile;
  const uint32_t oRec = oXY + (uint32_t)kxy * TC_M * 8;

  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base_sh), 2 * TC_N);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_addr(&abar), 1);
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(tc::smem_addr(&bfull[b]), 1);
      tc::mbar_init(tc::smem_addr(&mdone[b]), 1);
      tc::mbar_init(tc::smem_addr(&afree[b]), TC_EPI_WARPS);
    }
    tc::mbar_init_fence();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base_sh;
  bool ok = true;

  if (warp == TC_EPI_WARPS) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      auto copy_b = [&](int t, int b) {  // the K steps tile t uses
        const uint32_t bar = tc::smem_addr(&bfull[b]);
        const uint32_t bytes = (uint32_t)tile_ks[t] * TC_STEP;
        tc::mbar_arrive_expect_tx(bar, bytes);
        tc::bulk_g2s(sB + (uint32_t)b * btile, tw + (size_t)t * btile, bytes, bar);
      };
      {
        const uint32_t bar = tc::smem_addr(&abar);
        const uint32_t recb = (uint32_t)ntile * TC_REC_BYTES;
        tc::mbar_arrive_expect_tx(bar, btile + (uint32_t)kxy * TC_M * 8 + recb);
        tc::bulk_g2s(sA, zimg + (size_t)blockIdx.x * btile, btile, bar);
        tc::tma_load_2d(sbase + oXY, &tmxy, 2 * i0, 0, bar);
        if (recb) tc::bulk_g2s(sbase + oRec, meta, recb, bar);
      }
      if (ntile > 0) copy_b(0, 0);
      if (ntile > 1) copy_b(1, 1);
      if (!tc::mbar_wait(tc::smem_addr(&abar), 0u, TC_POLLS)) ok = false;
      const uint32_t idesc = tc::idesc_tf32(TC_M, TC_N);
      for (int t = 0; t < ntile; ++t) {
        const int b = t & 1;
        if (!tc::mbar_wait(tc::smem_addr(&bfull[b]), (uint32_t)(t >> 1) & 1u, TC_POLLS))
          ok = false;
        if (t >= 2 && !tc::mbar_wait(tc::smem_addr(&afree[b]), (uint32_t)((t - 2) >> 1) & 1u,
                                      TC_POLLS))
          ok = false;
        tc::fence_after_sync();
        const int ks = tile_ks[t];
        const uint32_t d = tbase + (uint32_t)(b * TC_N);
        const uint32_t bh = sB + (uint32_t)b * btile;
        for (int s = 0; s < ks; ++s) {
          const uint32_t ko = (uint32_t)s * TC_STEP;  // 8 TF32 = two core matrices along K
          const uint64_t ah = tc::sdesc(sA + ko, TC_LBO, TC_SBO);
          const uint64_t al = tc::sdesc(sA + ko + TC_LO, TC_LBO, TC_SBO);
          const uint64_t bhd = tc::sdesc(bh + ko, TC_LBO, TC_SBO);
          const uint64_t bld = tc::sdesc(bh + ko + TC_LO, TC_LBO, TC_SBO);
          tc::mma_tf32(d, ah, bhd, idesc, s > 0 ? 1u : 0u);
          tc::mma_tf32(d, ah, bld, idesc, 1u);
          tc::mma_tf32(d, al, bhd, idesc, 1u);
        }
        tc::mma_commit(tc::smem_addr(&mdone[b]));
        // B buffer b ^ 1 (tile t - 1) refilled with tile t + 1 once MMA(t - 1)
        // is done; MMA(t) runs meanwhile
        if (t >= 1 && t + 1 < ntile) {
          if (!tc::mbar_wait(tc::smem_addr(&mdone[b ^ 1]), (uint32_t)((t - 1) >> 1) & 1u,
                             TC_POLLS))
            ok = false;
          copy_b(t + 1, b ^ 1);
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int quarter = warp & 3, h = warp >> 2;  // lane quarter, column chunk
    const int row = 32 * quarter + lane;          // this thread's atom within the tile
    const float2 *xa = reinterpret_cast<const float2 *>(dsm + oXY) + row;  // X, Y rows
    if (!tc::mbar_wait(tc::smem_addr(&abar), 0u, TC_POLLS)) ok = false;
    float fs[3] = {0.f, 0.f, 0.f}, fc[3] = {0.f, 0.f, 0.f};
    for (int t = 0; t < ntile; ++t) {
      const int b = t & 1;
      if (!tc::mbar_wait(tc::smem_addr(&mdone[b]), (uint32_t)(t >> 1) & 1u, TC_POLLS))
        ok = false;
      tc::fence_after_sync();
      __syncwarp();
      const float4 *rec = reinterpret_cast<const float4 *>(dsm + oRec) + t * TC_COLS;
      float gs[3] = {0.f, 0.f, 0.f};
      {
        float v[32];
        tc::tmem_ld32(tbase + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(b * TC_N + 32 * h),
                      v);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 mt = rec[8 * h + j];  // nx, ny (int bits), rv
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
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tc::smem_addr(&afree[b]));
#pragma unroll
      for (int a = 0; a < 3; ++a) {  // Kahan-compensated sum over tiles
        const float y = gs[a] - fc[a];
        const float s = fs[a] + y;
        fc[a] = (s - fs[a]) - y;
        fs[a] = s;
      }
    }
    if (h > 0) {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        red[h - 1][a][row] = fs[a];
        red[h - 1][3 + a][row] = fc[a];
      }
    }
    __syncwarp();
    named_sync(1, 32 * TC_EPI_WARPS);  // epilogue warps only: column quarters meet
    const int i = i0 + row;
    if (h == 0 && i < n) {
      const float sc = fsc.scalef;
      long long q[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {  // fixed point, integer sums: order independent
        q[a] = f2ll_rn(fs[a] * sc) - f2ll_rn(fc[a] * sc);
#pragma unroll
        for (int k = 0; k < 3; ++k)
          q[a] += f2ll_rn(red[k][a][row] * sc) - f2ll_rn(red[k][3 + a][row] * sc);
      }
      gfix[i] += (unsigned long long)q[0];
      gfix[n + i] += (unsigned long long)q[1];
      gfix[2 * n + i] += (unsigned long long)q[2];
    }
  }
  tc::fence_before_sync();
  __syncthreads();  // every MMA waited for, every tensor-memory read done
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, 2 * TC_N);
  }
  if (!ok) atomicOr(err, DERR_TIMEOUT);
}

// Shared memory of the force pass: A, two B tiles, X and Y rows, records.
size_t tc_smem_bytes(int kp, int kxy, int ntile) {
  return 1024 + 6 * (size_t)TC_M * kp * 4 + (size_t)kxy * TC_M * sizeof(float2) +
         (size_t)ntile * TC_REC_BYTES;
}

__device__ __forceinline__ void st_split(unsigned char *hi, unsigned char *lo, float a, float b,
                                         float c, float d) {
  float4 h, l;
  tc::tf32_split_fast(a, h.x, l.x);
  tc::tf32_split_fast(b, h.y, l.y);
  tc::tf32_split_fast(c, h.z, l.z);
  tc::tf32_split_fast(d, h.w, l.w);
  *reinterpret_cast<float4 *>(hi) = h;
  *reinterpret_cast<float4 *>(lo) = l;
}

// S-pass, warp-specialised: a CTA (one per SM) takes MT <= 4 M-tiles of 64
// columns (128 rows each) and a slice of atoms (a multiple of 32), np <= 64.
// Warp 16 (lane 0) is the producer: per chunk of 32 atoms it brings in the
// chunk's X and Y rows (one TMA box) and its Z image (the B operand, shared
// by the MT tiles) SK_NB - 1 chunks ahead, and issues the MMAs.  Warps 0-15
// form T = X Y for one tile's columns at a time (a job = (chunk, tile)) into
// the A operand (two buffers) and write out the accumulators.  Tensor
// memory: two regions of 256 columns, tile m at column 64 m of a region;
// group g of SK_GCH chunks accumulates in region g % 2 and is written out as
// partial gps * slice + g while group g + 1 runs.  Barriers: full[s] (X, Y
// rows and Z image of the chunk in stage s landed), afull[b] (A of the job
// in buffer b written: 16 warp arrivals), adone[b] (MMAs of that job done),
// sdone[s] (MMAs of the chunk in stage s done), gdone[r] (the group in
// region r done), rfree[r] (region r written out: 16 arrivals).
constexpr int SK_NB = 4;  // copy stages (chunks in flight)
constexpr int SK_MT = 4;  // M-tiles per CTA at most
constexpr int SK_GEN_WARPS = 16;
constexpr int SK_THREADS = 32 * (SK_GEN_WARPS + 1);
constexpr int SK_GEN = 32 * SK_GEN_WARPS;  // 512 A items per job: 1 per thread
static_assert(SK_GEN == (SK_ROWS / 2) * (SK_CH / 4), "one A item per generator thread");

__global__ void __launch_bounds__(SK_THREADS, 1) k_sfac_tc(
    int n, int ncol, int ntm, int np, int slice, int gps, const KCol *__restrict__ cols,
    const __grid_constant__ CUtensorMap tmxy, const unsigned char *__restrict__ zimg, int kx,
    int ky, float *__restrict__ part, int *__restrict__ err) {
  // tmxy: the FP32 tables as a [row][2 ldn] float tensor, box 2 SK_CH x (kx + ky)
  extern __shared__ unsigned char dsm_raw[];
  __shared__ __align__(8) unsigned long long full[SK_NB], sdone[SK_NB], afull[2], adone[2],
      gdone[2], rfree[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int2 cxy[SK_MT][SK_ROWS / 2];  // (nx, ny) of the tiles' columns (nx < 0: none)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // this CTA's tiles [mt0, mt0 + MT): the ntm tiles spread evenly over gridDim.x
  const int mt0 = (int)((long long)blockIdx.x * ntm / gridDim.x);
  const int MT = (int)((long long)(blockIdx.x + 1) * ntm / gridDim.x) - mt0;
  const int a0 = blockIdx.y * slice, a1 = min(n, a0 + slice);
  const uint32_t raw = tc::smem_addr(dsm_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  unsigned char *dsm = dsm_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t bpart = sk_bpart(np);
  const int kxy = kx + ky;
  const uint32_t xysz = (uint32_t)kxy * SK_CH * 8;  // X, Y rows of one chunk
  // A0 (hi, lo) | A1 (hi, lo) | SK_NB x B (hi, lo) | SK_NB x X, Y rows [kxy][32]
  const uint32_t oB = 4 * SK_APART, oX = oB + SK_NB * 2 * bpart;
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base_sh), 512);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < SK_NB; ++s) {
      tc::mbar_init(tc::smem_addr(&full[s]), 1);
      tc::mbar_init(tc::smem_addr(&sdone[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(tc::smem_addr(&afull[b]), SK_GEN_WARPS);
      tc::mbar_init(tc::smem_addr(&adone[b]), 1);
      tc::mbar_init(tc::smem_addr(&gdone[b]), 1);
      tc::mbar_init(tc::smem_addr(&rfree[b]), SK_GEN_WARPS);
    }
    tc::mbar_init_fence();
  }
  for (int k = tid; k < SK_MT * (SK_ROWS / 2); k += blockDim.x) {
    const int m = k / (SK_ROWS / 2), c = (mt0 + m) * (SK_ROWS / 2) + k % (SK_ROWS / 2);
    int2 v = make_int2(-1, 0);
    if (m < MT && c < ncol) v = make_int2(cols[c].nx, cols[c].ny);
    cxy[m][k % (SK_ROWS / 2)] = v;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = tmem_base_sh;
  const int nchunk = (a1 - a0 + SK_CH - 1) / SK_CH;
  const int ngroup = (nchunk + SK_GCH - 1) / SK_GCH;
  bool ok = true;
  auto wait = [&](unsigned long long &bar, int phase) {
    if (!tc::mbar_wait(tc::smem_addr(&bar), (uint32_t)phase & 1u, TC_POLLS)) ok = false;
  };

  if (warp == SK_GEN_WARPS) {
    // ------------------------------------------------------------ producer
    // (the warp's other lanes wait at the closing barrier)
    if (lane == 0) {
      auto copy_in = [&](int c) {  // X, Y rows and Z image of chunk c -> stage c % SK_NB
        const int s = c % SK_NB;
        const uint32_t bar = tc::smem_addr(&full[s]);
        tc::mbar_arrive_expect_tx(bar, xysz + 2 * bpart);
        tc::tma_load_2d(sbase + oX + (uint32_t)s * xysz, &tmxy, 2 * (a0 + c * SK_CH), 0, bar);
        tc::bulk_g2s(sbase + oB + (uint32_t)s * 2 * bpart,
                     zimg + (size_t)(a0 / SK_CH + c) * 2 * bpart, 2 * bpart, bar);
      };
      for (int c = 0; c < min(nchunk, SK_NB - 1); ++c) copy_in(c);
      const uint32_t idesc = tc::idesc_tf32(SK_ROWS, np);
      for (int c = 0; c < nchunk; ++c) {
        const int s = c % SK_NB;
        const int g = c / SK_GCH, cg = c - g * SK_GCH;
        wait(full[s], c / SK_NB);
        if (cg == 0 && g >= 2) wait(rfree[g & 1], (g - 2) >> 1);  // region written out
        for (int m = 0; m < MT; ++m) {
          const int j = c * MT + m, b = j & 1;
          wait(afull[b], j >> 1);  // A of job j written (X, Y of chunk c read)
          tc::fence_after_sync();
          const uint32_t d = tbase + (uint32_t)(256 * (g & 1) + 64 * m);
          const uint32_t ah = sbase + (uint32_t)b * 2 * SK_APART, al = ah + SK_APART;
          const uint32_t bh = sbase + oB + (uint32_t)s * 2 * bpart, bl = bh + bpart;
          for (int k = 0; k < SK_CH / 8; ++k) {
            const uint32_t ko = (uint32_t)k * 2 * SK_LBO;  // 8 atoms = two core matrices
            const uint64_t dah = tc::sdesc(ah + ko, SK_LBO, SK_SBO);
            const uint64_t dal = tc::sdesc(al + ko, SK_LBO, SK_SBO);
            const uint64_t dbh = tc::sdesc(bh + ko, SK_LBO, SK_SBO);
            const uint64_t dbl = tc::sdesc(bl + ko, SK_LBO, SK_SBO);
            tc::mma_tf32(d, dah, dbh, idesc, (cg > 0 || k > 0) ? 1u : 0u);
            tc::mma_tf32(d, dah, dbl, idesc, 1u);
            tc::mma_tf32(d, dal, dbh, idesc, 1u);
          }
          tc::mma_commit(tc::smem_addr(&adone[b]));
        }
        tc::mma_commit(tc::smem_addr(&sdone[s]));
        if (cg == SK_GCH - 1 || c == nchunk - 1) tc::mma_commit(tc::smem_addr(&gdone[g & 1]));
        // stage of chunk c - 1 refilled with chunk c + SK_NB - 1: its X, Y
        // rows were read (afull), its Z image once the MMAs of chunk c - 1
        // are done
        if (c + SK_NB - 1 < nchunk) {
          if (c >= 1) wait(sdone[(c - 1) % SK_NB], (c - 1) / SK_NB);
          copy_in(c + SK_NB - 1);
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ generators
    // write out the accumulators of group g (region g % 2) as partial
    // gps * blockIdx.y + g: warp w reads lanes 32 (w % 4) .. of tile w / 4,
    // np <= 64 columns
    auto flush = [&](int g) {
      wait(gdone[g & 1], g >> 1);
      tc::fence_after_sync();
      __syncwarp();
      const int q4 = warp & 3, m = warp >> 2;
      const int row = 32 * q4 + lane;
      if (m < MT) {
        float *dst = part + (((size_t)(gps * blockIdx.y + g) * ntm + mt0 + m) * SK_ROWS + row) * np;
        for (int h = 0; h < np; h += 32) {
          float v[32];
          tc::tmem_ld32(tbase + ((uint32_t)(32 * q4) << 16) + (uint32_t)(256 * (g & 1) + 64 * m + h),
                        v);
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (h + j < np) dst[h + j] = v[j];
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tc::smem_addr(&rfree[g & 1]));
    };
    // this thread's A item: column cl of the job's tile, atom quad q ->
    // rows 2 cl (T.re), 2 cl + 1 (T.im)
    const int cl = tid >> 3, q = tid & 7;
    const uint32_t o0 = sk_off(2 * cl, q), o1 = sk_off(2 * cl + 1, q);
    int gf = 0;  // next group to write out
    for (int c = 0; c < nchunk; ++c) {
      const int s = c % SK_NB;
      const unsigned char *sxy = dsm + oX + (size_t)s * xysz;
      wait(full[s], c / SK_NB);
      for (int m = 0; m < MT; ++m) {
        const int j = c * MT + m, b = j & 1;
        unsigned char *sa = dsm + (size_t)b * 2 * SK_APART;
        if (j >= 2) wait(adone[b], (j - 2) >> 1);  // A buffer b free
        const int2 xy = cxy[m][cl];
        float re[4] = {0.f, 0.f, 0.f, 0.f}, im[4] = {0.f, 0.f, 0.f, 0.f};
        if (xy.x >= 0) {
          const bool neg = xy.y < 0;
          const float4 *X = reinterpret_cast<const float4 *>(sxy + (xy.x * SK_CH + 4 * q) * 8);
          const float4 *Y = reinterpret_cast<const float4 *>(
              sxy + ((kx + (neg ? -xy.y : xy.y)) * SK_CH + 4 * q) * 8);
          const float4 x01 = X[0], x23 = X[1], y01 = Y[0], y23 = Y[1];
          const float xr[4] = {x01.x, x01.z, x23.x, x23.z};
          const float xi[4] = {x01.y, x01.w, x23.y, x23.w};
          const float yr[4] = {y01.x, y01.z, y23.x, y23.z};
          float yi[4] = {y01.y, y01.w, y23.y, y23.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (neg) yi[u] = -yi[u];
            re[u] = fmaf(xr[u], yr[u], -xi[u] * yi[u]);
            im[u] = fmaf(xr[u], yi[u], xi[u] * yr[u]);
          }
        }
        st_split(sa + o0, sa + SK_APART + o0, re[0], re[1], re[2], re[3]);
        st_split(sa + o1, sa + SK_APART + o1, im[0], im[1], im[2], im[3]);
        tc::fence_proxy_async();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(tc::smem_addr(&afull[b]));
      }
      // the previous group is written out one chunk into the next one
      if (c - (c / SK_GCH) * SK_GCH == 1 && gf < c / SK_GCH) flush(gf++);
    }
    while (gf < ngroup) flush(gf++);
  }
  tc::fence_before_sync();
  __syncthreads();  // every MMA waited for, every tensor-memory read done
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tbase, 512);
  }
  if (!ok) atomicOr(err, DERR_TIMEOUT);
}

// Partials -> one FP64 block per M-tile: thread per element of the
// [ntm][128][np] block, partials added in FP64 in a fixed order
// (deterministic; coalesced over the elements).
__global__ void k_sfac_tc_reduce(int nel, int npart, const float *__restrict__ part,
                                 double *__restrict__ red) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  double a = 0.0;
  for (int s = 0; s < npart; ++s) a += (double)part[(size_t)s * nel + e];
  red[e] = a;
}

// S(k) from the reduced blocks: thread per (column, p <= m).
__global__ void k_sfac_tc_form(int ncol, int np, const KCol *__restrict__ cols,
                               const int *__restrict__ cp0, const double *__restrict__ red,
                               double2 *__restrict__ sk) {
  // cp0[c] = first (column, p) item of column c; cp0[ncol] = items
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cp0[ncol]) return;
  int lo = 0, hi = ncol;  // column of item t: cp0[c] <= t < cp0[c + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (cp0[mid] <= t) lo = mid;
    else hi = mid;
  }
  const int c = lo, p = t - cp0[c];
  const int mt = c / (SK_ROWS / 2), r = 2 * (c % (SK_ROWS / 2));
  const double *d = red + (size_t)mt * SK_ROWS * np;
  const double A1 = d[(size_t)r * np + 2 * p], A3 = d[(size_t)r * np + 2 * p + 1];
  const double A4 = d[(size_t)(r + 1) * np + 2 * p], A2 = d[(size_t)(r + 1) * np + 2 * p + 1];
  const KCol col = cols[c];
  const int kp = kcol_k(col, p), km = p > 0 ? kcol_k(col, -p) : -1;
  if (kp >= 0) sk[kp] = make_double2(A1 - A2, A3 + A4);
  if (km >= 0) sk[km] = make_double2(A1 + A2, A4 - A3);
}

size_t sk_smem_bytes(int np, int kxy) {
  return 1024 + 4 * (size_t)SK_APART + SK_NB * (2 * (size_t)sk_bpart(np) + (size_t)kxy * SK_CH * 8);
}

}  // namespace

// Column order and tile table of the tensor-core force pass (host, from the
// k-set columns) and its Z image.  Returns false when the pass does not
// apply (its shared-memory tiles do not fit).
// A failed set-up step of a tensor-core pass is an error of the call (no
// silent switch to another pass): the message names the step and the CUDA
// error, which is consumed.
static int tc_fail(mdx_ctx *ctx, const char *what) {
  const cudaError_t e = cudaGetLastError();
  ctx->err = std::string(what) + (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : "");
  return -1;
}

int tc_force_setup(mdx_ctx *ctx, const std::vector<KCol> &cols, int kmaz) {
  DevData &d = ctx->dv;
  const int kp = ((2 * (kmaz + 1) + 7) / 8) * 8;
  d.tc_on = false;
  const int kxy = d.kx + d.ky;
  const int ntile = ((int)cols.size() + TC_COLS - 1) / TC_COLS;
  if (tc_smem_bytes(kp, kxy, ntile) > 227 * 1024) return 0;  // tiles do not fit: CUDA cores
  std::vector<int> order(cols.size());
  for (size_t c = 0; c < cols.size(); ++c) order[c] = (int)c;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cols[a].m > cols[b].m; });
  std::vector<int> slot((size_t)ntile * TC_COLS, -1), ks(ntile, 0);
  for (size_t s = 0; s < order.size(); ++s) slot[s] = order[s];
  for (int t = 0; t < ntile; ++t) {
    const int m = cols[order[(size_t)t * TC_COLS]].m;  // largest m of the tile
    ks[t] = (2 * (m + 1) + 7) / 8;
  }
  ctx_free(ctx, d.tc_slot);
  ctx_free(ctx, d.tc_w);
  ctx_free(ctx, d.tc_meta);
  ctx_free(ctx, d.tc_zimg);
  d.tc_slot = nullptr;
  d.tc_w = nullptr;
  d.tc_meta = nullptr;
  d.tc_zimg = nullptr;
  const size_t zbytes = (size_t)(d.ldn / TC_M) * 1024 * kp;
  if (ctx_alloc(ctx, &d.tc_slot, sizeof(int) * (slot.size() + ks.size())) != cudaSuccess ||
      ctx_alloc(ctx, &d.tc_w, sizeof(float) * (size_t)ntile * 2 * TC_N * kp) != cudaSuccess ||
      ctx_alloc(ctx, &d.tc_meta, sizeof(float4) * slot.size()) != cudaSuccess ||
      ctx_alloc(ctx, &d.tc_zimg, zbytes) != cudaSuccess)
    return tc_fail(ctx, "tensor-core force pass: device allocation");
  d.tc_ks = d.tc_slot + slot.size();
  if (ctx_copy(ctx->stream, d.tc_slot, slot.data(), sizeof(int) * slot.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      ctx_copy(ctx->stream, d.tc_ks, ks.data(), sizeof(int) * ks.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemsetAsync(d.tc_zimg, 0, zbytes, ctx->stream) != cudaSuccess)  // K columns past 2 kz stay zero
    return tc_fail(ctx, "tensor-core force pass: table upload");
  if (raise_smem_limit(k_rforce_tc, tc_smem_bytes(kp, kxy, ntile)) != cudaSuccess)
    return tc_fail(ctx, "tensor-core force pass: shared-memory limit");
  d.tc_ntile = ntile;
  d.tc_kp = kp;
  d.tc_on = true;
  return 1;
}

// Tables of the tensor-core S(k) pass: M-tiles (up to SK_MT per CTA), slices
// (about one wave of one CTA per SM), partial buffer, item offsets, Z image.  Returns false when it
// does not apply.
int tc_sfac_setup(mdx_ctx *ctx, const std::vector<KCol> &cols) {
  DevData &d = ctx->dv;
  d.tcs_on = false;
  const int np = ((2 * d.kz + 15) / 16) * 16;
  const int kxy = d.kx + d.ky;
  if (np > 64 || sk_smem_bytes(np, kxy) > 227 * 1024) return 0;  // does not fit
  const int ncol = (int)cols.size();
  const int ntm = (ncol + SK_ROWS / 2 - 1) / (SK_ROWS / 2);
  int nsm = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return tc_fail(ctx, "tensor-core S(k): device query");
  const int ncg = (ntm + SK_MT - 1) / SK_MT;  // CTAs per slice (up to SK_MT tiles each)
  int ns = std::max(1, nsm / ncg);
  int slice = (d.n + ns - 1) / ns;
  slice = std::max(SK_CH, ((slice + SK_CH - 1) / SK_CH) * SK_CH);
  ns = (d.n + slice - 1) / slice;
  const int gps = (slice / SK_CH + SK_GCH - 1) / SK_GCH;  // partials per slice
  std::vector<int> cp0(ncol + 1, 0);
  for (int c = 0; c < ncol; ++c) cp0[c + 1] = cp0[c] + cols[c].m + 1;
  ctx_free(ctx, d.tcs_part);
  ctx_free(ctx, d.tcs_cp0);
  ctx_free(ctx, d.tcs_zimg);
  ctx_free(ctx, d.tcs_red);
  d.tcs_part = nullptr;
  d.tcs_cp0 = nullptr;
  d.tcs_zimg = nullptr;
  d.tcs_red = nullptr;
  const size_t pbytes = sizeof(float) * (size_t)ns * gps * ntm * SK_ROWS * np;
  const size_t zbytes = (size_t)(d.ldn / SK_CH) * 2 * sk_bpart(np);
  if (ctx_alloc(ctx, &d.tcs_part, pbytes) != cudaSuccess ||
      ctx_alloc(ctx, &d.tcs_cp0, sizeof(int) * cp0.size()) != cudaSuccess ||
      ctx_alloc(ctx, &d.tcs_zimg, zbytes) != cudaSuccess ||
      ctx_alloc(ctx, &d.tcs_red, sizeof(double) * (size_t)ntm * SK_ROWS * np) != cudaSuccess)
    return tc_fail(ctx, "tensor-core S(k): device allocation");
  if (ctx_copy(ctx->stream, d.tcs_cp0, cp0.data(), sizeof(int) * cp0.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      // partials past the last slice's atoms are never written: they stay zero;
      // image rows 2p, 2p + 1 with p >= kz too
      cudaMemsetAsync(d.tcs_part, 0, pbytes, ctx->stream) != cudaSuccess ||
      cudaMemsetAsync(d.tcs_zimg, 0, zbytes, ctx->stream) != cudaSuccess)
    return tc_fail(ctx, "tensor-core S(k): table upload");
  if (raise_smem_limit(k_sfac_tc, sk_smem_bytes(np, kxy)) != cudaSuccess)
    return tc_fail(ctx, "tensor-core S(k): shared-memory limit");
  d.tcs_np = np;
  d.tcs_ntm = ntm;
  d.tcs_nslice = ns;
  d.tcs_slice = slice;
  d.tcs_items = cp0[ncol];
  d.tcs_gps = gps;
  d.tcs_ncg = ncg;
  d.tcs_on = true;
  return 1;
}

// Tensor map of the FP32 tables: a [kx + ky + kz][2 ldn] float tensor, box
// of box_atoms atoms (2 box_atoms floats, 8 to 1024 bytes) x (kx + ky) rows.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static int encode_xy_map(mdx_ctx *ctx, CUtensorMap *m, int box_atoms) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
      ctx->err = "cuTensorMapEncodeTiled is not available";
      return MDX_ERR_CUDA;
    }
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  const DevData &d = ctx->dv;
  const cuuint64_t dim[2] = {(cuuint64_t)2 * d.ldn, (cuuint64_t)(d.kx + d.ky + d.kz)};
  const cuuint64_t stride[1] = {(cuuint64_t)2 * d.ldn * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)(2 * box_atoms), (cuuint32_t)(d.kx + d.ky)};
  const cuuint32_t estr[2] = {1, 1};
  if (fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, d.tabxf, dim, stride, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    ctx->err = "cuTensorMapEncodeTiled rejected the phase-table map";
    return MDX_ERR_CUDA;
  }
  return MDX_OK;
}

// Z images of this step (after the phase tables), for whichever tensor-core
// pass is on.
int tc_zimages_launch(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  if (!d.tc_on && !d.tcs_on) return MDX_OK;
  const size_t nth = (size_t)d.kz * d.ldn;
  k_zimages<<<(unsigned)((nth + 255) / 256), 256, 0, ctx->stream>>>(
      d.ldn, d.kz, d.tc_kp, d.tcs_np, d.tabzf, d.tc_on ? d.tc_zimg : nullptr,
      d.tcs_on ? d.tcs_zimg : nullptr);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

int tc_sfac_launch(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  CUtensorMap tm;
  int rc = encode_xy_map(ctx, &tm, SK_CH);
  if (rc) return rc;
  k_sfac_tc<<<dim3(d.tcs_ncg, d.tcs_nslice), SK_THREADS, sk_smem_bytes(d.tcs_np, d.kx + d.ky),
              ctx->stream>>>(d.n, d.ncol, d.tcs_ntm, d.tcs_np, d.tcs_slice, d.tcs_gps, d.cols, tm,
                             d.tcs_zimg, d.kx, d.ky, d.tcs_part, d.err);
  MDX_LAUNCHED(ctx);
  const int nel = d.tcs_ntm * SK_ROWS * d.tcs_np;
  k_sfac_tc_reduce<<<(nel + 255) / 256, 256, 0, ctx->stream>>>(nel, d.tcs_nslice * d.tcs_gps,
                                                                d.tcs_part, d.tcs_red);
  MDX_LAUNCHED(ctx);
  k_sfac_tc_form<<<(d.tcs_items + 127) / 128, 128, 0, ctx->stream>>>(
      d.ncol, d.tcs_np, d.cols, d.tcs_cp0, d.tcs_red, d.sk);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}

// One step's tensor-core force pass: B tiles from W, then the GEMM + fold.
int tc_force_launch(mdx_ctx *ctx) {
  DevData &d = ctx->dv;
  const int q = d.tc_kp / 4;
  const int nth = d.tc_ntile * TC_N * q;
  k_wtiles<<<(nth + 255) / 256, 256, 0, ctx->stream>>>(d.tc_ntile, d.tc_kp, d.tc_slot, d.cols,
                                                       d.wk, d.colrvf, d.tc_w, d.tc_meta);
  MDX_LAUNCHED(ctx);
  CUtensorMap tm;
  int rc = encode_xy_map(ctx, &tm, TC_M);
  if (rc) return rc;
  k_rforce_tc<<<(d.n + TC_M - 1) / TC_M, TC_THREADS,
                tc_smem_bytes(d.tc_kp, d.kx + d.ky, d.tc_ntile), ctx->stream>>>(
      d.n, d.tc_ntile, d.tc_kp, d.tc_ks, d.tc_meta,
      reinterpret_cast<const unsigned char *>(d.tc_w), d.tc_zimg, tm, d.kx, d.ky, ctx->fix,
      d.gfix, d.err);
  MDX_LAUNCHED(ctx);
  return MDX_OK;
}
