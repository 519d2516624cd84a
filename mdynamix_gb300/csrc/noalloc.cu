// noalloc.cu -- mdx_slforces_static: SLFORCES (forces.f:55-73) without any
// device allocation.
//
// mdx_slforces evaluates the slow forces with buffers the context owns; the
// one scratch buffer of that path, the per-slice partial sums of the Ewald
// structure factors S(k) (written by k_sfac / k_sfac32, summed in slice order
// by k_sfac_sum), lives in a device block allocated with the k-set.  This entry
// point runs the same kernels with that scratch taken from a file-scope
// static device array instead, and refuses (never allocates) whenever the
// path would need device memory it does not already have:
//  - the reciprocal k-set must exist (mdx_inifur, or one mdx_slforces /
//    mdx_allforce / mdx_double before), and the box must be inside the 5 %
//    window in which FURIR keeps that k-set (forces.f:1251-1265), else
//    MDX_ERR_STATE;
//  - the partial sums (slices x k-vectors x 16 bytes) must fit in
//    MDX_SK_STATIC_BYTES, else MDX_ERR_UNSUPPORTED (not checked, and the
//    scratch not used, when the mixed path's tensor-core S(k) pass is on:
//    that pass keeps its partials in buffers of the k-set);
//  - device timers must be off (they create events), else MDX_ERR_STATE.
// Nothing in the static scratch has to start at zero: every (slice, k)
// partial is written by the S(k) kernel before k_sfac_sum reads it.
// The scratch is one per device and per process: two calls whose kernels
// overlap on the device (two contexts on two streams, two host threads) race
// on it and corrupt each other's S(k).  Serialise such calls.
// Set-up: the first call on a device looks up the scratch's device address
// with cudaGetSymbolAddress, with that device current; make that first call
// before any stream capture that is to contain later calls.  Under CUDA's
// lazy module loading that first lookup is also what loads this file's
// module and with it the 4 MiB array: the first call per device can still
// fail for want of device memory (MDX_ERR_CUDA), later calls cannot.  The
// cached address belongs to the device context of the process; after a
// cudaDeviceReset it is stale, so do not reset a device between calls.
#include <mutex>

#include "mdx_internal.cuh"

#define RC(x)            \
  do {                   \
    int rc_ = (x);       \
    if (rc_) return rc_; \
  } while (0)

namespace {

__device__ __align__(256) unsigned char g_sk_scratch[MDX_SK_STATIC_BYTES];

constexpr int kMaxDevices = 64;
void *g_sk_scratch_addr[kMaxDevices] = {};
std::mutex g_sk_scratch_mu;

int scratch_address(mdx_ctx *ctx, void **addr) {
  int dev = -1;
  MDX_CUDA(cudaGetDevice(&dev));
  if (dev != ctx->device) {
    ctx->err = "mdx_slforces_static: the context's device must be current";
    return MDX_ERR_STATE;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    ctx->err = "mdx_slforces_static: device ordinal out of range";
    return MDX_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_sk_scratch_mu);
  if (!g_sk_scratch_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sk_scratch);
    if (e != cudaSuccess || !p) {
      ctx->err = std::string("mdx_slforces_static: cudaGetSymbolAddress: ") +
                 cudaGetErrorString(e);
      return MDX_ERR_CUDA;
    }
    g_sk_scratch_addr[dev] = p;
  }
  *addr = g_sk_scratch_addr[dev];
  return MDX_OK;
}

}  // namespace

extern "C" int mdx_slforces_static(mdx_ctx *ctx, mdx_scalars *out) {
  if (!ctx) return MDX_ERR_ARG;
  RC(api_require(ctx, true, true, true));
  if (!ctx->have_lists) {
    ctx->err = "lists not built";
    return MDX_ERR_STATE;
  }
  if (ctx->timing) {
    ctx->err = "mdx_slforces_static: device timers must be off";
    return MDX_ERR_STATE;
  }
  DevData &d = ctx->dv;
  if (ctx->p.alphad > 0.0) {
    if (!ctx->furir_init) {
      ctx->err = "mdx_slforces_static: no k-set yet; call mdx_inifur first";
      return MDX_ERR_STATE;
    }
    const double r[3] = {ctx->boxl / ctx->boxlo, ctx->boyl / ctx->boylo, ctx->bozl / ctx->bozlo};
    for (double v : r)
      if (v > 1.05 || v < 0.95) {
        ctx->err = "mdx_slforces_static: the box moved more than 5 % since the k-set was "
                   "built; a new k-set needs device memory (call mdx_inifur)";
        return MDX_ERR_STATE;
      }
  }
  // the tensor-core S(k) pass (mixed path) keeps its partials in buffers of
  // the k-set and never touches the slice scratch
  const bool uses_scratch = !(ctx->mixed() && d.tcs_on);
  const size_t need = (size_t)sfac_slices(ctx) * (size_t)std::max(1, d.nkv) * sizeof(double2);
  if (uses_scratch && need > MDX_SK_STATIC_BYTES) {
    char b[200];
    snprintf(b, sizeof b,
             "mdx_slforces_static: S(k) partial sums need %zu bytes; the static scratch "
             "holds %zu (MDX_SK_STATIC_BYTES)",
             need, (size_t)MDX_SK_STATIC_BYTES);
    ctx->err = b;
    return MDX_ERR_UNSUPPORTED;
  }
  if (!uses_scratch) {
    RC(api_do_slforces(ctx, true));
    RC(api_check_err(ctx));
    return api_copy_scalars(ctx, out);
  }
  void *scratch = nullptr;
  RC(scratch_address(ctx, &scratch));
  double2 *own = d.sk_part;
  d.sk_part = reinterpret_cast<double2 *>(scratch);
  const int rc = api_do_slforces(ctx, true);
  d.sk_part = own;
  RC(rc);
  RC(api_check_err(ctx));
  return api_copy_scalars(ctx, out);
}
