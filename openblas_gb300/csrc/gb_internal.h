// Internal declarations shared by the host dispatcher and the CUDA kernels
// of libgbblas.  Nothing here is part of the public ABI (include/gbblas.h).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbblas.h"
#include "gemm_blocks.h"
#include "per_device.h"

namespace gb {

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
// Records a library error (status code + message) for the calling thread and
// prints it once to stderr.  Never aborts the process.
int set_error(int status, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
#define GB_CUDA(call)                                                         \
  do {                                                                        \
    cudaError_t _e = (call);                                                  \
    if (_e != cudaSuccess) return gb::check_cuda(_e, #call);                  \
  } while (0)

// ---------------------------------------------------------------------------
// per-thread execution context
// ---------------------------------------------------------------------------
struct Context {
  int device = -1;
  cudaStream_t stream = nullptr;     // library stream (or user stream)
  bool user_stream = false;
  int *d_status = nullptr;           // device status words (STATUS_WORDS ints, see below)
  cudaStream_t copy_in = nullptr;    // host->device uploads of pipelined calls
  cudaStream_t copy_out = nullptr;   // device->host downloads of pipelined calls
  cudaStream_t panel = nullptr;      // the LU's look-ahead panel stream (highest priority)
  cudaEvent_t la_ev[2] = {nullptr, nullptr};  // ordering events between it and `stream`
};
// d_status[0..3]: kernel error code and site (read and cleared by
// gb_synchronize / the blocking entries); d_status[STATUS_LAST_SLICES]: the
// largest slice count the last automatic-mode emulated DGEMM chose;
// d_status[STATUS_LAST_MODULI]: its moduli count (0: no modular tile).
constexpr int STATUS_WORDS = 8;
constexpr int STATUS_LAST_SLICES = 4;
constexpr int STATUS_LAST_MODULI = 5;
Context &ctx();
// Lazily initialise CUDA for this thread; returns GB_SUCCESS or an error.
int ensure_init();
cudaStream_t stream();
// The two copy streams of this thread (created on first use).
int copy_streams(cudaStream_t *in, cudaStream_t *out);
// The look-ahead panel stream of this thread (highest priority) and its two
// ordering events (created on first use).
int lookahead_streams(cudaStream_t *panel, cudaEvent_t *to_panel, cudaEvent_t *to_main);

// CTAs of a persistent (one CTA per SM) kernel launched by this thread: the
// SM count less the SMs the thread keeps free for concurrent work (the LU's
// look-ahead panel), set for a scope by SmReserve.
int persistent_ctas();
struct SmReserve {
  int prev;
  explicit SmReserve(int sms);
  ~SmReserve();
};

// Stream-ordered device scratch (cudaMallocAsync from a pool that keeps its
// memory cached between calls, so repeated calls do not hit the driver).
void *scratch_alloc(size_t bytes, cudaStream_t s);
void scratch_free(void *p, cudaStream_t s);

// RAII holder of a scratch allocation.
struct Scratch {
  void *p = nullptr;
  cudaStream_t s = nullptr;
  Scratch() = default;
  Scratch(size_t bytes, cudaStream_t st) : p(scratch_alloc(bytes, st)), s(st) {}
  ~Scratch() {
    if (p) scratch_free(p, s);
  }
  Scratch(const Scratch &) = delete;
  Scratch &operator=(const Scratch &) = delete;
  template <class T>
  T *as() const { return reinterpret_cast<T *>(p); }
};

// True when `p` is device-accessible memory owned by CUDA (device or managed).
bool is_device_pointer(const void *p);

// Host<->device staging of a column-major m x n block whose host copy has
// leading dimension ld (elements of `esize` bytes).  The device copy is
// packed (leading dimension m), so only the m x n elements cross the link;
// rows between m and ld on the host are neither read nor written.
int stage_in(void *dst_dev, const void *src_host, size_t ld, size_t m, size_t n,
             size_t esize, cudaStream_t s);
int stage_out(void *dst_host, const void *src_dev, size_t ld, size_t m, size_t n,
              size_t esize, cudaStream_t s);

// Kernel-launch accounting (every launch site calls count_launch) and the
// optional event bracketing of a named kernel on its stream.
void count_launch(int n = 1);
struct ProfileScope {
  const char *name;
  cudaStream_t s;
  cudaEvent_t e0 = nullptr;
  ProfileScope(const char *nm, cudaStream_t st);
  ~ProfileScope();
};

// Library configuration read from the environment once.
struct Config {
  int dgemm_mode = GB_DGEMM_NATIVE;   // GB_DGEMM_MODE=native|emulated|auto
  int ozaki_slices = 0;               // GB_OZAKI_SLICES (0 = auto)
  int verbose = 0;                    // GB_VERBOSE
  int sgemm_mode = 0;                 // GB_SGEMM_MODE: 0 auto, 1 simt, 2 tensor
  int ozaki_group_m = 8;              // GB_OZAKI_GROUP_M: m-tiles per slice-GEMM tile group
  double ozaki_tol = 8.0;             // GB_OZAKI_TOL: automatic slice count's bound, units of 2^-52
  int ozaki_modular = 1;              // GB_OZAKI_MODULAR: automatic mode may take the modular scheme
  int lu_lookahead = 1;               // GB_LU_LOOKAHEAD: factor the next LU panel ahead (0: off)
};
const Config &config();

// ---------------------------------------------------------------------------
// kernels (device pointers, stream-ordered)
// ---------------------------------------------------------------------------
// C <- beta*C (beta==0 stores zeros).  kernel/generic/gemm_beta.c:41-94
void launch_dgemm_beta(int64_t m, int64_t n, double beta, double *C, int64_t ldc,
                       cudaStream_t s);
void launch_sgemm_beta(int64_t m, int64_t n, float beta, float *C, int64_t ldc,
                       cudaStream_t s);
// Native FP64 GEMM (DFMA).  Assumes m,n,k > 0 and alpha != 0.
void launch_dgemm_fp64(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                       const double *A, int64_t lda, const double *B, int64_t ldb,
                       double beta, double *C, int64_t ldc, cudaStream_t s);
// Same, writing only one triangle of C: tri 0 full, 1 lower (i>=j), 2 upper.
void launch_dgemm_fp64_tri(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double *A, int64_t lda, const double *B, int64_t ldb,
                           double beta, double *C, int64_t ldc, int tri, cudaStream_t s,
                           const int *skip = nullptr);
// Triangular beta scaling of an n x n C (tri as above).
void launch_dbeta_tri(int64_t n, double beta, double *C, int64_t ldc, int tri, cudaStream_t s);
// Number of SMs of the current device.
int sm_count();
// Ordinal of the calling thread's current device (0 if it cannot be read).
inline int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  return dev;
}
// Native FP32 GEMM (FFMA).
void launch_sgemm_fp32(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha,
                       const float *A, int64_t lda, const float *B, int64_t ldb,
                       float beta, float *C, int64_t ldc, cudaStream_t s);
// Same, restricted to a triangle of C (tri as launch_dgemm_fp64_tri) and
// cancelled on the device when *skip != 0.
void launch_sgemm_fp32_tri(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha,
                           const float *A, int64_t lda, const float *B, int64_t ldb, float beta,
                           float *C, int64_t ldc, int tri, cudaStream_t s, const int *skip);
// Slice count argument meaning "choose per 256-column tile of C from the
// operands and the accuracy target" (see ozaki.cu).
constexpr int OZAKI_SLICES_AUTO = -1;
// Slice count argument meaning "the modular scheme on every tile, with no
// choice" (the internal default of the factorisations' updates).
constexpr int OZAKI_MODULAR_FIXED = -2;
// The count for a caller-facing emulated GEMM: the thread's fixed setting
// (gb_set_ozaki_slices / GB_OZAKI_SLICES), or OZAKI_SLICES_AUTO when unset/0.
int ozaki_caller_slices();
// Whether the calling thread's automatic mode may take the modular scheme
// (gb_set_ozaki_modular / GB_OZAKI_MODULAR).
bool ozaki_modular_enabled();
// Whether the thread's DGEMM mode selects the emulated GEMM for an m x n x k
// product (auto mode: from 384^3 on, with k >= 64).
bool dgemm_mode_emulated(int64_t m, int64_t n, int64_t k);
// Emulated-FP64 GEMM (Ozaki schemes on the bf16 tensor cores).  slices = 0:
// the default form (the modular scheme on every tile, or 7 digit slices
// when the thread turned it off); 1-8: that many digit slices;
// OZAKI_SLICES_AUTO: chosen per tile on the device.  tri = 1 (2): only C(i,j) with i >= j (i <= j) is written,
// tiles wholly in the other triangle are skipped (SYRK-shaped updates).
// skip: device flag; when nonzero at run time C is left unchanged.
int dgemm_emulated(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                   const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                   double *C, int64_t ldc, int slices, cudaStream_t s, int tri = 0,
                   const int *skip = nullptr);
// Column-blocked emulated DGEMM (k <= 16384): op(A) is prepared once per K
// segment; for each block of nb columns of op(B) and C, hooks->before
// supplies device pointers to the block (after making it available, e.g.
// waiting for its upload) and hooks->after runs once C's block is final
// (e.g. to start its download), so transfers overlap the other blocks' work.
// K segment of the digit-slice engine: every int32 level sum of one segment
// is exact (8 products x 4096 x 255^2 < 2^31); longer K runs segment by
// segment (the automatic mode's modular scheme takes segments of twice
// this).
constexpr int64_t EMU_K_SEGMENT = 4096;
// hooks->segment(j0, jn, k0, kk) runs before the K range [k0, k0 + kk) of
// the block is used (e.g. to wait for that range of op(A) and op(B)), and
// hooks->a_range(k0, kk) before op(A)'s columns [k0, k0 + kk) are first read.
// hooks->block_cols(j0, nb) gives the width of the block starting at column
// j0 (a multiple of 256, at most nb; the default: nb).  When
// hooks->a_row_block() is positive (a multiple of 128), op(A) arrives in
// blocks of that many rows, and with a single K segment each block's row
// maxima, exponents and residues are prepared as it arrives;
// hooks->a_rows(i0, rb) runs before rows [i0, i0 + rb) of op(A) are read.
struct EmuBlockHooks {
  virtual int before(int64_t j0, int64_t jn, const double **Bj, int64_t *ldb, double **Cj,
                     int64_t *ldc) = 0;
  virtual int segment(int64_t, int64_t, int64_t, int64_t) { return GB_SUCCESS; }
  virtual int a_range(int64_t, int64_t) { return GB_SUCCESS; }
  virtual int64_t block_cols(int64_t, int64_t nb) { return nb; }
  virtual int64_t a_row_block() { return 0; }
  virtual int a_rows(int64_t, int64_t) { return GB_SUCCESS; }
  virtual int after(int64_t j0, int64_t jn) = 0;
  virtual ~EmuBlockHooks() = default;
};
// The K segment the emulated engine runs for a slice-count argument.
int64_t emulated_k_segment(int slices);
int dgemm_emulated_blocked(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double *A, int64_t lda, double beta, int slices, int64_t nb,
                           EmuBlockHooks *hooks, cudaStream_t s);
// FP32 GEMM on the bf16 tensor cores (three-term split, FP32 accuracy).
// Assumes m, n, k > 0.
int sgemm_tc(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha, const float *A,
             int64_t lda, const float *B, int64_t ldb, float beta, float *C, int64_t ldc,
             cudaStream_t s, int tri = 0, const int *skip = nullptr);
// FP64 GEMM on a triangle of C (tri 0 full, 1 lower, 2 upper) with the
// engine the DGEMM mode selects (native DFMA or emulated); k > 0, alpha != 0.
int dgemm_select(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha, const double *A,
                 int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
                 int tri, cudaStream_t s);
// FP32 GEMM behind sgemm_/cblas_sgemm and the FP32 LU: the tensor-core form
// for shapes large enough to fill the GPU (GB_SGEMM_MODE=auto, default), or
// always SIMT / always tensor (GB_SGEMM_MODE=simt|tensor).
int sgemm_dispatch(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha, const float *A,
                   int64_t lda, const float *B, int64_t ldb, float beta, float *C, int64_t ldc,
                   cudaStream_t s);

}  // namespace gb
