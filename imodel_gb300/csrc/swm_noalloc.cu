// Compensated weighted sums with no device allocation.
//
// Same two-pass Neumaier reduction as the diagnostics kernels (block partial
// sums, then one block per quantity), but the block partials live in a
// file-scope __device__ array instead of a buffer the caller's handle
// allocated.  Compiled with --fmad=false: the compensation terms rely on each
// product being rounded on its own.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "imodel_swm.h"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 32;                  // elements per thread
constexpr int kMaxBlocks = 4096;
constexpr int kQ = 4;                       // sum w, sum w f, sum w f^2, max |f|
constexpr int64_t kMaxN = static_cast<int64_t>(kMaxBlocks) * kThreads * kItems;
constexpr int kMaxDevices = 64;

// Block partials: kQ quantities x kMaxBlocks blocks x (sum, compensation),
// 256 KiB.  Every GPU that loads this library holds it until the process
// exits.  Each launch overwrites every partial it later reads, so nothing in
// it has to start at zero; it keeps the last call's partials.
__device__ __align__(256) double g_partials[kQ * kMaxBlocks * 2];

// max that keeps a NaN: fmax alone returns the other operand when one is NaN,
// so a field holding NaN would report a finite maximum
__device__ __forceinline__ double nanmax(double a, double b) {
  return (a != a || b != b) ? a + b : fmax(a, b);
}

struct KSum {
  double s, c;
  __device__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x))
      c = c + ((s - t) + x);
    else
      c = c + ((x - t) + s);
    s = t;
  }
  __device__ void merge(double os, double oc) {
    add(os);
    c = c + oc;
  }
};

__global__ void __launch_bounds__(kThreads) k_wsum_partials(const double *__restrict__ w,
                                                            const double *__restrict__ f,
                                                            int64_t n,
                                                            double *__restrict__ partials) {
  KSum a[3] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
  double mx = 0.0;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kThreads * kItems;
  for (int k = 0; k < kItems; ++k) {
    const int64_t i = base + static_cast<int64_t>(k) * kThreads + threadIdx.x;
    if (i < n) {
      const double wi = w[i], fi = f[i];
      a[0].add(wi);
      a[1].add(wi * fi);
      a[2].add(wi * (fi * fi));
      mx = nanmax(mx, fabs(fi));
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    for (int q = 0; q < 3; ++q) {
      const double os = __shfl_down_sync(0xffffffffu, a[q].s, off);
      const double oc = __shfl_down_sync(0xffffffffu, a[q].c, off);
      a[q].merge(os, oc);
    }
    mx = nanmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
  }
  __shared__ double sh[kThreads / 32][kQ][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    for (int q = 0; q < 3; ++q) {
      sh[warp][q][0] = a[q].s;
      sh[warp][q][1] = a[q].c;
    }
    sh[warp][3][0] = mx;
    sh[warp][3][1] = 0.0;
  }
  __syncthreads();
  if (threadIdx.x < kQ) {
    const int q = threadIdx.x;
    KSum t{0.0, 0.0};
    double m = 0.0;
    for (int wv = 0; wv < kThreads / 32; ++wv) {
      if (q < 3)
        t.merge(sh[wv][q][0], sh[wv][q][1]);
      else
        m = nanmax(m, sh[wv][q][0]);
    }
    const size_t slot = (static_cast<size_t>(q) * kMaxBlocks + blockIdx.x) * 2;
    partials[slot] = q < 3 ? t.s : m;
    partials[slot + 1] = q < 3 ? t.c : 0.0;
  }
}

// one block per quantity over the nblk partials written by the launch above
__global__ void __launch_bounds__(kThreads) k_wsum_final(const double *__restrict__ partials,
                                                         int nblk, double *__restrict__ out) {
  const int q = blockIdx.x;
  __shared__ double ss[kThreads], sc[kThreads];
  KSum a{0.0, 0.0};
  double m = 0.0;
  for (int b = threadIdx.x; b < nblk; b += kThreads) {
    const size_t slot = (static_cast<size_t>(q) * kMaxBlocks + b) * 2;
    if (q < 3)
      a.merge(partials[slot], partials[slot + 1]);
    else
      m = nanmax(m, partials[slot]);
  }
  ss[threadIdx.x] = q < 3 ? a.s : m;
  sc[threadIdx.x] = q < 3 ? a.c : 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (q < 3) {
      KSum r{0.0, 0.0};
      for (int t = 0; t < kThreads; ++t) r.merge(ss[t], sc[t]);
      out[q] = r.s + r.c;
    } else {
      double r = 0.0;
      for (int t = 0; t < kThreads; ++t) r = nanmax(r, ss[t]);
      out[q] = r;
    }
  }
}

// device address of g_partials per device, with the context it was looked up
// in: a caller that makes another context current on the device (or resets
// the device) gets the address looked up again
struct PartialsAddr {
  CUcontext ctx;
  double *addr;
};
PartialsAddr g_partials_addr[kMaxDevices] = {};
std::mutex g_partials_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &qr) !=
            cudaSuccess ||
        qr != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

}  // namespace

extern "C" int imodel_swm_weighted_sums_noalloc(const double *w, const double *f, int64_t n,
                                                double *out, void *stream) {
  if (!w || !f || !out || n <= 0) return IMODEL_SWM_EINVAL;
  if (n > kMaxN) return IMODEL_SWM_ETOOBIG;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return IMODEL_SWM_ENODEV;
  if (dev < 0 || dev >= kMaxDevices) return IMODEL_SWM_EINVAL;
  // the current context (null before the runtime first touches the device;
  // cudaGetSymbolAddress below then makes the primary context current)
  CtxGetCurrentFn get_ctx = ctx_get_current();
  CUcontext ctx = nullptr;
  if (get_ctx && get_ctx(&ctx) != CUDA_SUCCESS) return IMODEL_SWM_ECUDA;
  double *partials = nullptr;
  {
    // first call on this device (or in this context): host code may not use
    // g_partials itself (it names a host-side stand-in), so ask the runtime
    // for its device address
    std::lock_guard<std::mutex> lock(g_partials_mu);
    PartialsAddr &slot = g_partials_addr[dev];
    if (!slot.addr || (ctx && slot.ctx != ctx)) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_partials) != cudaSuccess || !p) return IMODEL_SWM_ECUDA;
      if (get_ctx && !ctx && get_ctx(&ctx) != CUDA_SUCCESS) return IMODEL_SWM_ECUDA;
      slot.addr = static_cast<double *>(p);
      slot.ctx = ctx;
    }
    partials = slot.addr;
  }
  const int nblk = static_cast<int>((n + static_cast<int64_t>(kThreads) * kItems - 1) /
                                    (static_cast<int64_t>(kThreads) * kItems));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // launched through cudaLaunchKernel so that each launch's own status is
  // returned: cudaGetLastError would also report (and clear) an error the
  // caller left pending before this call
  void *a1[] = {&w, &f, &n, &partials};
  if (cudaLaunchKernel(reinterpret_cast<const void *>(k_wsum_partials), dim3(nblk),
                       dim3(kThreads), a1, 0, s) != cudaSuccess)
    return IMODEL_SWM_ECUDA;
  int nb = nblk;
  void *a2[] = {&partials, &nb, &out};
  if (cudaLaunchKernel(reinterpret_cast<const void *>(k_wsum_final), dim3(kQ), dim3(kThreads), a2,
                       0, s) != cudaSuccess)
    return IMODEL_SWM_ECUDA;
  return IMODEL_SWM_OK;
}
