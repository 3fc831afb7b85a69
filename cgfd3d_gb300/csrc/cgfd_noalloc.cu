/*
 * cgfd_noalloc.cu -- wavefield finiteness check that allocates nothing.
 *
 * Some callers cannot call cudaMalloc: code that runs while another
 * framework owns the device memory pool (a caching allocator that must see
 * every allocation), processes under a hard device-memory cap, or health
 * checks issued between the launches of a tightly scheduled time loop where
 * an allocation would synchronise the device.  For them this file provides
 * cgfd_check_finite_noalloc(): the same NaN/Inf test as
 * cgfd_solver_check_finite(), on a device array the caller owns, with its
 * scratch (one partial flag per block plus the result word) in a file-scope
 * __device__ array instead of memory from cudaMalloc.
 *
 * The scratch array is g_nf_scratch below, CGFD_NOALLOC_MAX_BLOCKS + 1 ints
 * (256 KiB + 4 bytes); every GPU that loads this library holds it until the
 * process exits.  That caps the input at CGFD_NOALLOC_MAX_FLOATS values.
 *
 * Host code cannot pass g_nf_scratch to a kernel: in host code the name is a
 * host-side stand-in, not a device address.  The device address is looked
 * up with cudaGetSymbolAddress once per device, with that device current, on
 * the first call made on that device; that first call therefore should come
 * before any stream capture.  Every call shares the one array and keeps the
 * last call's contents, so each call writes every slot it later reads, and
 * calls that overlap on the GPU (different threads or streams on the same
 * device) race on it.
 */
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/cgfd3d_gpu.h"

#define NF_THREADS 256
#define NF_PER_THREAD 64

static __device__ __align__(256) int g_nf_scratch[CGFD_NOALLOC_MAX_BLOCKS + 1];

/* error reporting shared with the rest of the library (cgfd_solver.cu);
 * the message is returned by cgfd_last_error() */
__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

static int na_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

/* one partial flag per block: 1 if its chunk holds a NaN or an Inf */
__global__ void k_nf_partial(const float *__restrict__ d, unsigned long long n,
                             unsigned long long chunk, int *part)
{
  unsigned long long b0 = blockIdx.x * chunk;
  unsigned long long b1 = b0 + chunk < n ? b0 + chunk : n;
  int bad = 0;
  for (unsigned long long t = b0 + threadIdx.x; t < b1; t += blockDim.x)
    bad |= !isfinite(d[t]);
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) part[blockIdx.x] = bad;
}

/* result word = OR of the partials the previous launch wrote */
__global__ void k_nf_final(const int *part, int nb, int *out)
{
  int bad = 0;
  for (int t = threadIdx.x; t < nb; t += blockDim.x) bad |= part[t];
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) *out = bad;
}

static std::mutex g_na_mutex;
#define NA_MAX_DEVICES 64
/* device address of g_nf_scratch per device, with the context it was looked
 * up in: the module (and so the array) is loaded per context, and a
 * cudaDeviceReset or another current context on the same device loads it
 * at a new address, so a cached address is used only while the context it
 * belongs to is the current one */
static int *g_na_ptr[NA_MAX_DEVICES];
static void *g_na_ctx[NA_MAX_DEVICES];

/* the calling thread's current context (a CUcontext), or null */
static void *na_current_context(void)
{
  typedef int (*get_ctx_t)(void **);
  static get_ctx_t fn = nullptr;
  static bool looked = false;
  if (!looked) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (get_ctx_t)p;
    looked = true;
  }
  void *ctx = nullptr;
  if (fn && fn(&ctx) != 0) ctx = nullptr;
  return ctx;
}

extern "C" int cgfd_check_finite_noalloc(const float *d_data, size_t n,
                                         int *nonfinite)
{
  if (!nonfinite) return na_err(CGFD_EINVAL, "nonfinite output pointer is null");
  *nonfinite = 0;
  if (n == 0) return CGFD_OK;
  if (!d_data) return na_err(CGFD_EINVAL, "device data pointer is null");
  if (n > (size_t)CGFD_NOALLOC_MAX_FLOATS)
    return na_err(CGFD_EINVAL,
                  "cgfd_check_finite_noalloc: %zu values exceed the maximum of %llu "
                  "(scratch holds %d block flags)",
                  n, (unsigned long long)CGFD_NOALLOC_MAX_FLOATS, CGFD_NOALLOC_MAX_BLOCKS);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return na_err(CGFD_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= NA_MAX_DEVICES)
    return na_err(CGFD_EINVAL,
                  "cgfd_check_finite_noalloc: device index %d is beyond the %d devices "
                  "this entry point keeps scratch addresses for",
                  dev, NA_MAX_DEVICES);
  int *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    /* the first call in a context (after cudaSetDevice makes it current,
     * or after a reset) looks the address up; later calls reuse it */
    void *ctx = na_current_context();
    if (!g_na_ptr[dev] || !ctx || ctx != g_na_ctx[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_nf_scratch);
      if (e != cudaSuccess || !p)
        return na_err(CGFD_ECUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      g_na_ptr[dev] = (int *)p;
      g_na_ctx[dev] = na_current_context();
    }
    scratch = g_na_ptr[dev];
  }
  const unsigned long long chunk = (unsigned long long)NF_THREADS * NF_PER_THREAD;
  int nb = (int)((n + chunk - 1) / chunk);
  k_nf_partial<<<nb, NF_THREADS>>>(d_data, (unsigned long long)n, chunk, scratch);
  k_nf_final<<<1, 1024>>>(scratch, nb, scratch + CGFD_NOALLOC_MAX_BLOCKS);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_err(CGFD_ECUDA, "launch: %s", cudaGetErrorString(e));
  int h = 0;
  e = cudaMemcpy(&h, scratch + CGFD_NOALLOC_MAX_BLOCKS, sizeof(int),
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return na_err(CGFD_ECUDA, "cudaMemcpy: %s", cudaGetErrorString(e));
  *nonfinite = h;
  return CGFD_OK;
}
