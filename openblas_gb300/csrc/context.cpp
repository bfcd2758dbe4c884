// Per-thread execution context, error state, scratch memory, host<->device
// staging and the xerbla error hook of libgbblas.
//
// The reference keeps a process-wide thread server and a scratch pool
// (driver/others/blas_server.c, driver/others/memory.c:1161).  On the GPU
// the equivalent state is one CUDA stream per calling host thread plus a
// stream-ordered memory pool: concurrent callers never share a stream, and
// scratch comes from cudaMallocAsync on that stream, cached by the pool.
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "gb_internal.h"

namespace gb {

namespace {
struct ErrorState {
  int status = GB_SUCCESS;
  char msg[512] = {0};
  char xerbla_name[16] = {0};
  int xerbla_info = 0;
};
thread_local ErrorState t_err;
thread_local Context t_ctx;
std::once_flag g_cfg_once;
Config g_cfg;
std::mutex g_pool_mu;
bool g_pool_ready[64] = {false};

// Fork safety (the reference re-initialises its memory pool in a forked
// child, driver/others/memory.c:432-443 pthread_atfork).  A CUDA context does
// not survive fork(): a child of a process that already called into CUDA
// through this library cannot use the GPU, so the child is marked and every
// entry point reports GB_ERR_NO_DEVICE with that reason instead of failing
// in CUDA in an undefined way.
std::atomic<int> g_cuda_touched{0};
std::atomic<int> g_forked_child{0};
std::once_flag g_atfork_once;
void atfork_child() {
  if (g_cuda_touched.load()) g_forked_child.store(1);
}
}  // namespace

int set_error(int status, const char *fmt, ...) {
  t_err.status = status;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err.msg, sizeof(t_err.msg), fmt, ap);
  va_end(ap);
  if (config().verbose || status != GB_ERR_INVALID_VALUE)
    fprintf(stderr, "libgbblas: %s\n", t_err.msg);
  return status;
}

int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return GB_SUCCESS;
  int st = (e == cudaErrorMemoryAllocation) ? GB_ERR_ALLOC
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? GB_ERR_NO_DEVICE
                                                                          : GB_ERR_CUDA;
  return set_error(st, "%s failed: %s", what, cudaGetErrorString(e));
}

const Config &config() {
  std::call_once(g_cfg_once, [] {
    const char *m = getenv("GB_DGEMM_MODE");
    if (m) {
      if (!strcmp(m, "emulated") || !strcmp(m, "ozaki")) g_cfg.dgemm_mode = GB_DGEMM_EMULATED;
      else if (!strcmp(m, "auto")) g_cfg.dgemm_mode = GB_DGEMM_AUTO;
      else g_cfg.dgemm_mode = GB_DGEMM_NATIVE;
    }
    const char *s = getenv("GB_OZAKI_SLICES");
    if (s) g_cfg.ozaki_slices = atoi(s);
    const char *v = getenv("GB_VERBOSE");
    if (v) g_cfg.verbose = atoi(v);
    const char *sm = getenv("GB_SGEMM_MODE");
    if (sm) g_cfg.sgemm_mode = !strcmp(sm, "simt") ? 1 : !strcmp(sm, "tensor") ? 2 : 0;
    const char *tol = getenv("GB_OZAKI_TOL");
    if (tol && atof(tol) > 0.0) g_cfg.ozaki_tol = atof(tol);
    const char *om = getenv("GB_OZAKI_MODULAR");
    if (om) g_cfg.ozaki_modular = atoi(om) != 0;
    const char *la = getenv("GB_LU_LOOKAHEAD");
    if (la) g_cfg.lu_lookahead = atoi(la) != 0;
    const char *g = getenv("GB_OZAKI_GROUP_M");
    if (g && atoi(g) > 0) g_cfg.ozaki_group_m = atoi(g);
  });
  return g_cfg;
}

Context &ctx() { return t_ctx; }

int ensure_init() {
  std::call_once(g_atfork_once, [] { pthread_atfork(nullptr, nullptr, atfork_child); });
  if (g_forked_child.load())
    return set_error(GB_ERR_NO_DEVICE,
                     "this process was forked after its parent used CUDA through libgbblas; a "
                     "CUDA context does not survive fork(), so the child cannot use the GPU "
                     "(fork before the first call, or use spawn)");
  g_cuda_touched.store(1);
  Context &c = t_ctx;
  if (c.stream && c.d_status) return GB_SUCCESS;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return check_cuda(e, "cudaGetDevice");
  int ndev = 0;
  e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return check_cuda(e == cudaSuccess ? cudaErrorNoDevice : e,
                                                       "cudaGetDeviceCount");
  c.device = dev;
  if (!c.stream) {
    GB_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  }
  if (!c.d_status) {
    GB_CUDA(cudaMalloc(&c.d_status, sizeof(int) * STATUS_WORDS));
    GB_CUDA(cudaMemsetAsync(c.d_status, 0, sizeof(int) * STATUS_WORDS, c.stream));
  }
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (dev < 64 && !g_pool_ready[dev]) {
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;  // keep freed scratch cached in the pool
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
      }
      g_pool_ready[dev] = true;
    }
  }
  return GB_SUCCESS;
}

cudaStream_t stream() { return t_ctx.stream; }

int lookahead_streams(cudaStream_t *panel, cudaEvent_t *to_panel, cudaEvent_t *to_main) {
  Context &c = t_ctx;
  if (!c.panel) {
    int least = 0, greatest = 0;
    GB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    GB_CUDA(cudaStreamCreateWithPriority(&c.panel, cudaStreamNonBlocking, greatest));
  }
  for (int i = 0; i < 2; ++i)
    if (!c.la_ev[i]) GB_CUDA(cudaEventCreateWithFlags(&c.la_ev[i], cudaEventDisableTiming));
  *panel = c.panel;
  *to_panel = c.la_ev[0];
  *to_main = c.la_ev[1];
  return GB_SUCCESS;
}

static thread_local int t_sm_reserve = 0;
int persistent_ctas() {
  const int n = sm_count() - t_sm_reserve;
  return n > 0 ? n : 1;
}
SmReserve::SmReserve(int sms) : prev(t_sm_reserve) { t_sm_reserve = sms; }
SmReserve::~SmReserve() { t_sm_reserve = prev; }

int copy_streams(cudaStream_t *in, cudaStream_t *out) {
  Context &c = t_ctx;
  if (!c.copy_in) GB_CUDA(cudaStreamCreateWithFlags(&c.copy_in, cudaStreamNonBlocking));
  if (!c.copy_out) GB_CUDA(cudaStreamCreateWithFlags(&c.copy_out, cudaStreamNonBlocking));
  *in = c.copy_in;
  *out = c.copy_out;
  return GB_SUCCESS;
}

void *scratch_alloc(size_t bytes, cudaStream_t s) {
  if (bytes == 0) bytes = 256;
  void *p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, bytes, s);
  if (e != cudaSuccess) {
    check_cuda(e, "cudaMallocAsync(scratch)");
    return nullptr;
  }
  return p;
}

void scratch_free(void *p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

bool is_device_pointer(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int stage_in(void *dst_dev, const void *src_host, size_t ld, size_t m, size_t n, size_t esize,
             cudaStream_t s) {
  if (m == 0 || n == 0) return GB_SUCCESS;
  GB_CUDA(cudaMemcpy2DAsync(dst_dev, m * esize, src_host, ld * esize, m * esize, n,
                            cudaMemcpyHostToDevice, s));
  return GB_SUCCESS;
}

int stage_out(void *dst_host, const void *src_dev, size_t ld, size_t m, size_t n, size_t esize,
              cudaStream_t s) {
  if (m == 0 || n == 0) return GB_SUCCESS;
  GB_CUDA(cudaMemcpy2DAsync(dst_host, ld * esize, src_dev, m * esize, m * esize, n,
                            cudaMemcpyDeviceToHost, s));
  return GB_SUCCESS;
}

// Called from the xerbla_ entry point (also when the application overrides
// xerbla_, the library records the argument error before calling it).
void record_xerbla(const char *name, int info) {
  size_t n = strnlen(name, sizeof(t_err.xerbla_name) - 1);
  memcpy(t_err.xerbla_name, name, n);
  t_err.xerbla_name[n] = 0;
  t_err.xerbla_info = info;
  t_err.status = GB_ERR_INVALID_VALUE;
  snprintf(t_err.msg, sizeof(t_err.msg), "%s: parameter %d had an illegal value",
           t_err.xerbla_name, info);
}

// ---------------------------------------------------------------------------
// instrumentation
// ---------------------------------------------------------------------------
namespace {
std::atomic<int64_t> g_launches{0};
struct ProfileRec {
  std::string name;
  cudaEvent_t e0, e1;
};
thread_local bool t_prof_on = false;
thread_local std::vector<ProfileRec> t_prof;
}  // namespace

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

ProfileScope::ProfileScope(const char *nm, cudaStream_t st) : name(nm), s(st) {
  if (!t_prof_on) return;
  if (cudaEventCreate(&e0) != cudaSuccess) {
    e0 = nullptr;
    return;
  }
  cudaEventRecord(e0, s);
}

ProfileScope::~ProfileScope() {
  if (!e0) return;
  cudaEvent_t e1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return;
  }
  cudaEventRecord(e1, s);
  t_prof.push_back({name, e0, e1});
}

}  // namespace gb

// ---------------------------------------------------------------------------
// public control API
// ---------------------------------------------------------------------------
extern "C" {

__attribute__((weak)) int xerbla_(const char *name, const blasint *info, blasint len) {
  // The whole routine name, padded to at least six columns (driver/others/
  // xerbla.c:58); a Fortran caller passes it without a terminator, so the
  // hidden length bounds it.
  char buf[16];
  const size_t cap = (len > 0 && len < 15) ? (size_t)len : 15;
  size_t n = strnlen(name, cap);
  memcpy(buf, name, n);
  buf[n] = 0;
  printf(" ** On entry to %6s parameter number %2d had an illegal value\n", buf, *info);
  fflush(stdout);
  return 0;
}

int gb_set_stream(void *s) {
  int st = gb::ensure_init();
  if (st) return st;
  gb::Context &c = gb::ctx();
  if (s) {
    c.stream = (cudaStream_t)s;
    c.user_stream = true;
  } else if (c.user_stream) {
    c.user_stream = false;
    c.stream = nullptr;
    return gb::ensure_init();
  }
  return GB_SUCCESS;
}

void *gb_get_stream(void) {
  if (gb::ensure_init()) return nullptr;
  return (void *)gb::stream();
}

int gb_synchronize(void) {
  int st = gb::ensure_init();
  if (st) return st;
  GB_CUDA(cudaStreamSynchronize(gb::stream()));
  int h[4] = {0, 0, 0, 0};
  GB_CUDA(cudaMemcpy(h, gb::ctx().d_status, sizeof(h), cudaMemcpyDeviceToHost));
  if (h[0]) {
    cudaMemset(gb::ctx().d_status, 0, sizeof(h));
    return gb::set_error(GB_ERR_KERNEL, "kernel reported error code %d (site %d)", h[0], h[1]);
  }
  return GB_SUCCESS;
}

int gb_last_error(char *msg, int len) {
  if (msg && len > 0) {
    strncpy(msg, gb::t_err.msg, (size_t)len - 1);
    msg[len - 1] = 0;
  }
  return gb::t_err.status;
}

void gb_clear_error(void) {
  gb::t_err.status = GB_SUCCESS;
  gb::t_err.msg[0] = 0;
  gb::t_err.xerbla_info = 0;
  gb::t_err.xerbla_name[0] = 0;
}

int gb_last_xerbla(char *name, int len) {
  if (name && len > 0) {
    strncpy(name, gb::t_err.xerbla_name, (size_t)len - 1);
    name[len - 1] = 0;
  }
  return gb::t_err.xerbla_info;
}

static thread_local int t_dgemm_mode = -1;
static thread_local int t_ozaki_slices = -1;
static thread_local int t_ozaki_modular = -1;
static thread_local int t_sgemm_mode = -1;

int gb_set_sgemm_mode(int mode) {
  if (mode < GB_SGEMM_AUTO || mode > GB_SGEMM_TENSOR)
    return gb::set_error(GB_ERR_INVALID_VALUE, "gb_set_sgemm_mode: bad mode %d", mode);
  t_sgemm_mode = mode;
  return GB_SUCCESS;
}

int gb_get_sgemm_mode(void) {
  return t_sgemm_mode >= 0 ? t_sgemm_mode : gb::config().sgemm_mode;
}

int gb_set_dgemm_mode(int mode) {
  if (mode < GB_DGEMM_NATIVE || mode > GB_DGEMM_AUTO)
    return gb::set_error(GB_ERR_INVALID_VALUE, "gb_set_dgemm_mode: bad mode %d", mode);
  t_dgemm_mode = mode;
  return GB_SUCCESS;
}

int gb_get_dgemm_mode(void) {
  return t_dgemm_mode >= 0 ? t_dgemm_mode : gb::config().dgemm_mode;
}

int gb_set_ozaki_slices(int slices) {
  if (slices < 0 || slices > 12)
    return gb::set_error(GB_ERR_INVALID_VALUE, "gb_set_ozaki_slices: %d not in [0,12]", slices);
  t_ozaki_slices = slices;
  return GB_SUCCESS;
}

int gb_get_ozaki_slices_internal(void) {
  return t_ozaki_slices >= 0 ? t_ozaki_slices : gb::config().ozaki_slices;
}

int gb_last_ozaki_slices(void) {
  if (!gb::ctx().d_status || !gb::ctx().stream) return 0;
  cudaError_t e = cudaStreamSynchronize(gb::stream());
  if (e != cudaSuccess) return -gb::check_cuda(e, "gb_last_ozaki_slices");
  int v = 0;
  e = cudaMemcpy(&v, gb::ctx().d_status + gb::STATUS_LAST_SLICES, sizeof(int),
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return -gb::check_cuda(e, "gb_last_ozaki_slices");
  return v;
}

int gb_last_ozaki_moduli(void) {
  if (!gb::ctx().d_status || !gb::ctx().stream) return 0;
  cudaError_t e = cudaStreamSynchronize(gb::stream());
  if (e != cudaSuccess) return -gb::check_cuda(e, "gb_last_ozaki_moduli");
  int v = 0;
  e = cudaMemcpy(&v, gb::ctx().d_status + gb::STATUS_LAST_MODULI, sizeof(int),
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return -gb::check_cuda(e, "gb_last_ozaki_moduli");
  return v;
}

int gb_set_ozaki_modular(int on) {
  t_ozaki_modular = on != 0;
  return GB_SUCCESS;
}

const char *gb_version(void) { return "libgbblas 0.1 (sm_103a)"; }

int64_t gb_kernel_launches(void) { return gb::g_launches.load(); }

int gb_profile_enable(int on) {
  gb::t_prof_on = on != 0;
  return GB_SUCCESS;
}

double gb_profile_kernel_ms(const char *name, int *launches, int reset) {
  double total = 0.0;
  int cnt = 0;
  for (auto &r : gb::t_prof) {
    if (name && r.name != name) continue;
    cudaEventSynchronize(r.e1);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.e0, r.e1) == cudaSuccess) total += ms;
    ++cnt;
  }
  if (launches) *launches = cnt;
  if (reset) {
    for (auto &r : gb::t_prof) {
      cudaEventDestroy(r.e0);
      cudaEventDestroy(r.e1);
    }
    gb::t_prof.clear();
  }
  return total;
}

}  // extern "C"

namespace gb {
int ozaki_caller_slices() {
  const int s = gb_get_ozaki_slices_internal();
  return s > 0 ? s : OZAKI_SLICES_AUTO;
}
bool ozaki_modular_enabled() {
  return t_ozaki_modular >= 0 ? t_ozaki_modular != 0 : config().ozaki_modular != 0;
}
}  // namespace gb
