// Level-3 BLAS entry points of libgbblas: dgemm_/cblas_dgemm, sgemm_/
// cblas_sgemm, dtrsm_/cblas_dtrsm, dsyrk_/cblas_dsyrk, cblas_dgemm_batch,
// and their device-pointer variants.
//
// Argument decoding, the order of the checks (so the same parameter
// position reaches xerbla), the row-major -> column-major operand swap and
// the quick returns restate interface/gemm.c:181-476, interface/trsm.c:114-
// 351 and interface/syrk.c:96-340.  Instead of the reference's thread-count
// decision and scratch buffer, the call is dispatched to the GPU stream.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "gb_internal.h"
#include "operand.h"

extern "C" int gb_get_ozaki_slices_internal(void);

namespace gb {

void call_xerbla(const char *name, int info) {
  record_xerbla(name, info);
  blasint i = info;
  xerbla_(name, &i, (blasint)strlen(name));
}

int finish_blocking(cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return check_cuda(e, "cudaStreamSynchronize");
  int h = 0;
  e = cudaMemcpy(&h, ctx().d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return check_cuda(e, "cudaMemcpy(status)");
  if (h) {
    int site[4] = {0, 0, 0, 0};
    cudaMemcpy(site, ctx().d_status, sizeof(site), cudaMemcpyDeviceToHost);
    cudaMemset(ctx().d_status, 0, sizeof(site));
    return set_error(GB_ERR_KERNEL, "kernel reported error code %d (site %d)", site[0], site[1]);
  }
  return GB_SUCCESS;
}

// transa/transb code: 0 = N, 1 = T, -1 = invalid (interface/gemm.c:243-262;
// for real types 'R' means N and 'C' means T)
static inline int trans_code(char t) {
  t = upch(t);
  if (t == 'N' || t == 'R') return 0;
  if (t == 'T' || t == 'C') return 1;
  return -1;
}
static inline int cblas_trans_code(int t) {
  if (t == CblasNoTrans || t == CblasConjNoTrans) return 0;
  if (t == CblasTrans || t == CblasConjTrans) return 1;
  return -1;
}

// C <- alpha*op(A)op(B) + beta*C on device pointers, native FP64.
static int dgemm_native(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                        const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                        double *C, int64_t ldc, cudaStream_t s) {
  if (m == 0 || n == 0) return GB_SUCCESS;
  if (k == 0 || alpha == 0.0) {
    launch_dgemm_beta(m, n, beta, C, ldc, s);
  } else {
    launch_dgemm_fp64(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
  }
  return check_cuda(cudaGetLastError(), "dgemm launch");
}


static bool dgemm_wants_emulated(int64_t m, int64_t n, int64_t k) {
  return dgemm_mode_emulated(m, n, k);
}

// Selected by the DGEMM mode: emulated when requested, or in auto mode when
// the product is large enough for the split/recombine passes to pay off.
static int dgemm_dispatch(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                          const double *A, int64_t lda, const double *B, int64_t ldb,
                          double beta, double *C, int64_t ldc, cudaStream_t s) {
  if (dgemm_wants_emulated(m, n, k) && k > 0 && alpha != 0.0)
    return dgemm_emulated(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          ozaki_caller_slices(), s);
  return dgemm_native(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

// Host-pointer emulated DGEMM pipelined over column blocks of op(B) and C.
// With one engine K segment and op(A) = A^T, op(A) goes up in row blocks,
// each prepared (row maxima, exponents, residues) while the next uploads;
// otherwise op(A) and every block of op(B) go up in 4096-deep K pieces, so
// the first slice GEMM starts once the first segment is on the device.  Block j+1 uploads on
// the copy-in stream while block j computes, and C's block j comes down on
// the copy-out stream while later blocks compute.  The result is the one of the
// single-call emulated GEMM bit for bit (each C(i,j) sees only row i of
// op(A) and column j of op(B)).  The upload of block j+1 and the download of
// block j-1 are issued after block j's kernels, so that pageable host
// buffers (whose copies the CUDA runtime performs synchronously) still
// overlap with the GPU.
namespace {
constexpr int64_t PIPE_K_SEGMENT = EMU_K_SEGMENT;  // upload piece of op(A) and op(B) along K

// Column blocks of the pipelined DGEMM, in 256-column tiles of C (block
// starts, the last entry n; *nb the widest block).  The first block's
// upload and the last block's download lie outside any overlap, so both
// are at most one wave of the persistent GEMM's tiles (one 128 x 256 tile
// per CTA); the two or three blocks between them are picked with a
// timeline model: uploads run back to back from the start, block b's
// compute starts when its upload and block b - 1 are done and takes whole
// waves of tiles, its download follows it and the previous download.  The
// model's constants are this part's measured rates: ~200 GB/s up and
// ~190 GB/s down the host link, ~0.84 ms per wave of modular-scheme tiles
// per 8192 of K, ~0.8 ms per 8192^2 of op(A) preparation and ~0.12 ms of
// fixed work per block.  The plan changes only the overlap, never the
// result.
std::vector<int64_t> pipeline_blocks(int64_t m, int64_t n, int64_t k, int64_t *nb) {
  const int64_t T = (n + 255) / 256, mt = (m + 127) / 128, P = persistent_ctas();
  const double a_up = (double)m * k * 8 / 200e9 * 1e3;
  const double a_prep = 0.8 * ((double)m * k / (8192.0 * 8192.0));
  const double up_t = 256.0 * k * 8 / 200e9 * 1e3, dn_t = 256.0 * m * 8 / 190e9 * 1e3;
  const double wave = 0.843 * k / 8192.0;
  auto cost = [&](const std::vector<int64_t> &t) {
    double up = a_up, comp = a_up + a_prep, dn = 0.0;
    for (int64_t b : t) {
      up += b * up_t;
      comp = (comp > up ? comp : up) + (double)((mt * b + P - 1) / P) * wave + 0.12;
      dn = (comp > dn ? comp : dn) + b * dn_t;
    }
    return dn;
  };
  // the even split into blocks of ~4096 columns, and the edge-block plans
  int64_t nu = n / 4096;
  nu = nu < 2 ? 2 : nu > 8 ? 8 : nu;
  std::vector<int64_t> best;
  for (int64_t i = 0; i < nu; ++i) best.push_back(T * (i + 1) / nu - T * i / nu);
  double best_cost = cost(best);
  int64_t e = P / mt;
  e = e < 1 ? 1 : e;
  const int64_t R = T - 2 * e;
  auto consider = [&](const std::vector<int64_t> &t) {
    const double c = cost(t);
    if (c < best_cost - 1e-9) {
      best_cost = c;
      best = t;
    }
  };
  for (int64_t x = 1; R >= 2 && x < R; ++x) {
    consider({e, x, R - x, e});
    for (int64_t y = 1; x + y < R; ++y) consider({e, x, y, R - x - y, e});
  }
  std::vector<int64_t> starts{0};
  *nb = 0;
  for (int64_t b : best) {
    const int64_t j1 = starts.back() + b * 256 < n ? starts.back() + b * 256 : n;
    *nb = j1 - starts.back() > *nb ? j1 - starts.back() : *nb;
    starts.push_back(j1);
  }
  return starts;
}

struct PipelinedDgemm : EmuBlockHooks {
  cudaStream_t s = nullptr, cin = nullptr, cout = nullptr;
  int ta = 0, tb = 0;
  int64_t m = 0, n = 0, k = 0, nseg = 1, lda = 0, ldb = 0, ldc = 0;
  std::vector<int64_t> bs;  // column blocks: block j is [bs[j], bs[j + 1])
  int64_t block_of(int64_t j0) const {
    return (int64_t)(std::upper_bound(bs.begin(), bs.end(), j0) - bs.begin()) - 1;
  }
  const double *A = nullptr, *B = nullptr;
  double *C = nullptr;
  bool load_c = false;
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int64_t dlda = 0, dldb = 0;
  std::vector<cudaEvent_t> a_up, up, done;  // a_up[seg], up[block * nseg + seg], done[block]
  // op(A) in row blocks of arb rows (0: in K pieces), ar_up[row block]
  int64_t arb = 0;
  std::vector<cudaEvent_t> ar_up;
  // GB_VERBOSE >= 3: a timeline of the copies and blocks (timing events)
  struct Mark {
    cudaEvent_t e;
    const char *what;
    int64_t idx;
  };
  std::vector<Mark> marks;
  bool trace = false;
  void mark(cudaStream_t st, const char *what, int64_t idx) {
    if (!trace) return;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, st);
    marks.push_back({e, what, idx});
  }
  std::chrono::steady_clock::time_point h0, h1, h2;  // host: entry, enqueued, finished
  void report() {
    if (marks.empty()) return;
    auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    fprintf(stderr, "[gbblas] pipelined dgemm host: %.3f ms enqueueing, %.3f ms to completion\n",
            ms(h0, h1), ms(h0, h2));
    cudaEventSynchronize(marks.back().e);
    for (const Mark &mk : marks) {
      float ms = 0.f;
      cudaEventSynchronize(mk.e);
      cudaEventElapsedTime(&ms, marks.front().e, mk.e);
      fprintf(stderr, "[gbblas] pipelined dgemm %8.3f ms  %s %lld\n", ms, mk.what,
              (long long)mk.idx);
    }
    for (const Mark &mk : marks) cudaEventDestroy(mk.e);
    marks.clear();
  }

  int64_t seg_len(int64_t sg) const {
    const int64_t k0 = sg * PIPE_K_SEGMENT;
    return (k - k0) < PIPE_K_SEGMENT ? (k - k0) : PIPE_K_SEGMENT;
  }
  // segment sg of op(A): columns of A (ta = 0) or rows of A (ta = 1)
  int upload_a(int64_t sg) {
    const int64_t k0 = sg * PIPE_K_SEGMENT, kk = seg_len(sg);
    if (ta)
      GB_CUDA(cudaMemcpy2DAsync(dA + k0, dlda * 8, A + k0, lda * 8, kk * 8, m,
                                cudaMemcpyHostToDevice, cin));
    else
      GB_CUDA(cudaMemcpy2DAsync(dA + k0 * dlda, dlda * 8, A + k0 * lda, lda * 8, m * 8, kk,
                                cudaMemcpyHostToDevice, cin));
    GB_CUDA(cudaEventRecord(a_up[sg], cin));
    mark(cin, "op(A) segment uploaded", sg);
    return GB_SUCCESS;
  }
  // rows [b arb, b arb + arb) of op(A): rows of A (ta = 0) or columns of A
  int upload_a_rows(int64_t b) {
    const int64_t i0 = b * arb, rb = (m - i0) < arb ? (m - i0) : arb;
    if (ta)
      GB_CUDA(cudaMemcpy2DAsync(dA + i0 * dlda, dlda * 8, A + i0 * lda, lda * 8, k * 8, rb,
                                cudaMemcpyHostToDevice, cin));
    else
      GB_CUDA(cudaMemcpy2DAsync(dA + i0, dlda * 8, A + i0, lda * 8, rb * 8, k,
                                cudaMemcpyHostToDevice, cin));
    GB_CUDA(cudaEventRecord(ar_up[b], cin));
    mark(cin, "op(A) row block uploaded", b);
    return GB_SUCCESS;
  }
  int64_t a_row_block() override { return arb; }
  int a_rows(int64_t i0, int64_t) override {
    GB_CUDA(cudaStreamWaitEvent(s, ar_up[i0 / arb], 0));
    return GB_SUCCESS;
  }
  // segment sg of block j of op(B) (and C's block with the first segment)
  int upload(int64_t j, int64_t sg) {
    const int64_t j0 = bs[j], jn = bs[j + 1] - bs[j];
    const int64_t k0 = sg * PIPE_K_SEGMENT, kk = seg_len(sg);
    if (tb)  // op(B) = B^T: rows j0.. and columns k0.. of the n x k matrix B
      GB_CUDA(cudaMemcpy2DAsync(dB + j0 + k0 * dldb, dldb * 8, B + j0 + k0 * ldb, ldb * 8, jn * 8,
                                kk, cudaMemcpyHostToDevice, cin));
    else
      GB_CUDA(cudaMemcpy2DAsync(dB + j0 * dldb + k0, dldb * 8, B + j0 * ldb + k0, ldb * 8, kk * 8,
                                jn, cudaMemcpyHostToDevice, cin));
    if (load_c && sg == 0) {
      int st = stage_in(dC + j0 * m, C + j0 * ldc, ldc, m, jn, 8, cin);
      if (st) return st;
    }
    GB_CUDA(cudaEventRecord(up[j * nseg + sg], cin));
    mark(cin, "op(B) block segment uploaded", j * nseg + sg);
    return GB_SUCCESS;
  }
  int upload_block(int64_t j) {
    for (int64_t sg = 0; sg < nseg; ++sg) {
      int st = upload(j, sg);
      if (st) return st;
    }
    return GB_SUCCESS;
  }
  int download(int64_t j) {
    const int64_t j0 = bs[j], jn = bs[j + 1] - bs[j];
    GB_CUDA(cudaStreamWaitEvent(cout, done[j], 0));
    const int st = stage_out(C + j0 * ldc, dC + j0 * m, ldc, m, jn, 8, cout);
    mark(cout, "C block downloaded", j);
    return st;
  }
  int before(int64_t j0, int64_t, const double **Bj, int64_t *ldbj, double **Cj,
             int64_t *ldcj) override {
    *Bj = tb ? dB + j0 : dB + j0 * dldb;
    *ldbj = dldb;
    *Cj = dC + j0 * m;
    *ldcj = m;
    return GB_SUCCESS;
  }
  // every upload piece overlapping [k0, k0 + kk)
  // op(A) is complete on the device: its last row block, or its K pieces
  int wait_a(int64_t k0, int64_t kk) {
    if (arb > 0) {
      GB_CUDA(cudaStreamWaitEvent(s, ar_up.back(), 0));
      return GB_SUCCESS;
    }
    for (int64_t sg = k0 / PIPE_K_SEGMENT; sg * PIPE_K_SEGMENT < k0 + kk; ++sg)
      GB_CUDA(cudaStreamWaitEvent(s, a_up[sg], 0));
    return GB_SUCCESS;
  }
  int segment(int64_t j0, int64_t, int64_t k0, int64_t kk) override {
    int st = wait_a(k0, kk);
    if (st) return st;
    for (int64_t sg = k0 / PIPE_K_SEGMENT; sg * PIPE_K_SEGMENT < k0 + kk; ++sg)
      GB_CUDA(cudaStreamWaitEvent(s, up[block_of(j0) * nseg + sg], 0));
    return GB_SUCCESS;
  }
  int a_range(int64_t k0, int64_t kk) override { return wait_a(k0, kk); }
  int64_t block_cols(int64_t j0, int64_t) override {
    const int64_t j = block_of(j0);
    return bs[j + 1] - bs[j];
  }
  int after(int64_t j0, int64_t) override {
    const int64_t j = block_of(j0), nblk = (int64_t)done.size();
    GB_CUDA(cudaEventRecord(done[j], s));
    mark(s, "C block computed", j);
    int st = GB_SUCCESS;
    if (j + 1 < nblk && (st = upload_block(j + 1))) return st;
    if (j > 0 && (st = download(j - 1))) return st;
    if (j + 1 == nblk) return download(j);
    return GB_SUCCESS;
  }
};
}  // namespace

// Returns 1 when the call was handled (successfully or with a recorded
// error), 0 when the pipelined form does not apply.
static int dgemm_host_pipelined(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                                const double *A, int64_t lda, const double *B, int64_t ldb,
                                double beta, double *C, int64_t ldc) {
  if (k <= 0 || alpha == 0.0 || k > 16384 || n < 6144 || m < 2048) return 0;
  if (m > GEMM_BLOCK_EXTENT || n > GEMM_BLOCK_EXTENT) return 0;  // the blocked device path
  if (!dgemm_wants_emulated(m, n, k)) return 0;
  if (is_device_pointer(A) || is_device_pointer(B) || is_device_pointer(C)) return 0;
  PipelinedDgemm p;
  p.h0 = std::chrono::steady_clock::now();
  p.s = stream();
  if (copy_streams(&p.cin, &p.cout)) return 1;
  int64_t nb = 0;
  p.bs = pipeline_blocks(m, n, k, &nb);
  const int64_t nblk = (int64_t)p.bs.size() - 1;
  p.ta = ta;
  p.tb = tb;
  p.m = m;
  p.n = n;
  p.k = k;
  p.nseg = (k + PIPE_K_SEGMENT - 1) / PIPE_K_SEGMENT;
  p.A = A;
  p.lda = lda;
  p.B = B;
  p.ldb = ldb;
  p.C = C;
  p.ldc = ldc;
  p.load_c = beta != 0.0;
  const int64_t ra = ta ? k : m, ca = ta ? m : k;
  p.dlda = ra;
  p.dldb = tb ? n : k;
  Scratch ws(((size_t)ra * ca + (size_t)n * k + (size_t)m * n) * 8, p.s);
  if (!ws.p) {
    set_error(GB_ERR_ALLOC, "dgemm: device staging of %lld x %lld x %lld", (long long)m,
              (long long)n, (long long)k);
    return 1;
  }
  double *dA = p.dA = ws.as<double>();
  p.dB = dA + ra * ca;
  p.dC = p.dB + n * k;
  p.a_up.assign(p.nseg, nullptr);
  p.up.assign(nblk * p.nseg, nullptr);
  p.done.assign(nblk, nullptr);
  // one K segment in the engine and op(A) = A^T (its rows are A's contiguous
  // columns): op(A) goes up in eight row blocks (at least 512 rows each),
  // each prepared while the next uploads.  With op(A) = A the rows are
  // strided on the host: a block's 2D copy moves runs of 8 x rows bytes, at
  // 96, 107, 180 and 210 GB/s for 4, 8, 16 and 32 KB runs, so such blocks
  // are at least 4096 rows (up to eight of them), and smaller operands go
  // up in K pieces.
  if (emulated_k_segment(ozaki_caller_slices()) >= k) {
    if (ta) {
      const int64_t rb = ((m + 7) / 8 + 127) / 128 * 128;
      p.arb = rb < 512 ? 512 : rb;
    } else if (m >= 2 * 4096) {
      const int64_t nbk = m / 4096 < 8 ? m / 4096 : 8;
      p.arb = ((m + nbk - 1) / nbk + 127) / 128 * 128;
    }
    if (p.arb >= m) p.arb = 0;
  }
  p.ar_up.assign(p.arb > 0 ? (m + p.arb - 1) / p.arb : 0, nullptr);
  cudaEvent_t ready = nullptr, out_done = nullptr;
  auto run = [&]() -> int {
    for (auto *v : {&p.a_up, &p.up, &p.done, &p.ar_up})
      for (cudaEvent_t &e : *v) GB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    GB_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    GB_CUDA(cudaEventCreateWithFlags(&out_done, cudaEventDisableTiming));
    // the staging buffer was allocated on the compute stream
    GB_CUDA(cudaEventRecord(ready, p.s));
    GB_CUDA(cudaStreamWaitEvent(p.cin, ready, 0));
    p.mark(p.cin, "start", 0);
    // op(A) and block 0 of op(B) engine segment by engine segment: all of
    // op(A)'s pieces of a segment first (its preparation needs the whole
    // segment and overlaps block 0's upload), then block 0's
    int st;
    if (p.arb > 0) {  // op(A) by row blocks, then block 0 of op(B)
      for (int64_t b = 0; b < (int64_t)p.ar_up.size(); ++b)
        if ((st = p.upload_a_rows(b))) return st;
      for (int64_t sg = 0; sg < p.nseg; ++sg)
        if ((st = p.upload(0, sg))) return st;
    }
    const int64_t eseg = emulated_k_segment(ozaki_caller_slices()) / PIPE_K_SEGMENT;
    for (int64_t g0 = 0; p.arb == 0 && g0 < p.nseg; g0 += eseg) {
      const int64_t g1 = g0 + eseg < p.nseg ? g0 + eseg : p.nseg;
      for (int64_t sg = g0; sg < g1; ++sg)
        if ((st = p.upload_a(sg))) return st;
      for (int64_t sg = g0; sg < g1; ++sg)
        if ((st = p.upload(0, sg))) return st;
    }
    st = dgemm_emulated_blocked(ta, tb, m, n, k, alpha, dA, ra, beta,
                                ozaki_caller_slices(), nb, &p, p.s);
    // the staging buffer is released on the compute stream after the last download
    GB_CUDA(cudaEventRecord(out_done, p.cout));
    GB_CUDA(cudaStreamWaitEvent(p.s, out_done, 0));
    return st;
  };
  p.trace = config().verbose >= 3;
  int st = run();
  p.h1 = std::chrono::steady_clock::now();
  cudaStreamSynchronize(p.cin);
  cudaStreamSynchronize(p.cout);
  p.h2 = std::chrono::steady_clock::now();
  p.report();
  if (!st) finish_blocking(p.s);
  else cudaStreamSynchronize(p.s);
  for (auto *v : {&p.a_up, &p.up, &p.done, &p.ar_up})
    for (cudaEvent_t e : *v)
      if (e) cudaEventDestroy(e);
  if (ready) cudaEventDestroy(ready);
  if (out_done) cudaEventDestroy(out_done);
  return 1;
}

// Blocking host-pointer DGEMM after argument checks (column-major form).
static void dgemm_blocking(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double *A, int64_t lda, const double *B, int64_t ldb,
                           double beta, double *C, int64_t ldc) {
  if (m == 0 || n == 0) return;  // interface/gemm.c:494
  if (ensure_init()) return;
  if (dgemm_host_pipelined(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc)) return;
  cudaStream_t s = stream();
  bool need_ab = k > 0 && alpha != 0.0;
  Operand a(A, ta ? k : m, ta ? m : k, lda, 8), b(B, tb ? n : k, tb ? k : n, ldb, 8);
  Operand c(C, m, n, ldc, 8);
  if (need_ab && (a.bind(true, s) || b.bind(true, s))) return;
  if (c.bind(beta != 0.0, s)) return;
  if (dgemm_dispatch(ta, tb, m, n, k, alpha, a.d<double>(), a.dld, b.d<double>(), b.dld, beta,
                     c.d<double>(), c.dld, s))
    return;
  c.unbind(s);
  finish_blocking(s);
}

static void sgemm_blocking(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha,
                           const float *A, int64_t lda, const float *B, int64_t ldb, float beta,
                           float *C, int64_t ldc) {
  if (m == 0 || n == 0) return;
  if (ensure_init()) return;
  cudaStream_t s = stream();
  bool need_ab = k > 0 && alpha != 0.0f;
  Operand a(A, ta ? k : m, ta ? m : k, lda, 4), b(B, tb ? n : k, tb ? k : n, ldb, 4);
  Operand c(C, m, n, ldc, 4);
  if (need_ab && (a.bind(true, s) || b.bind(true, s))) return;
  if (c.bind(beta != 0.0f, s)) return;
  if (!need_ab) {
    launch_sgemm_beta(m, n, beta, c.d<float>(), c.dld, s);
    if (check_cuda(cudaGetLastError(), "sgemm launch")) return;
  } else if (sgemm_dispatch(ta, tb, m, n, k, alpha, a.d<float>(), a.dld, b.d<float>(), b.dld,
                            beta, c.d<float>(), c.dld, s)) {
    return;
  }
  c.unbind(s);
  finish_blocking(s);
}

// Device-side drivers defined in the other translation units.
int dtrsm_device(int side, int uplo, int trans, int unit, int64_t m, int64_t n, double alpha,
                 const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s);
int dsyrk_device(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                 int64_t lda, double beta, double *C, int64_t ldc, cudaStream_t s);
int dtrsm_select(int side, int uplo, int trans, int unit, int64_t m, int64_t n, double alpha,
                 const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s);
int gb_dgemm_batch_grouped(int order, const int *ta, const int *tb, const blasint *m,
                           const blasint *n, const blasint *k, const double *alpha,
                           const double **A, const blasint *lda, const double **B,
                           const blasint *ldb, const double *beta, double **C,
                           const blasint *ldc, blasint group_count, const blasint *group_size);

static void dtrsm_blocking(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                           double alpha, const double *A, int64_t lda, double *B, int64_t ldb) {
  if (m == 0 || n == 0) return;  // interface/trsm.c:355
  if (ensure_init()) return;
  cudaStream_t s = stream();
  int64_t na = side ? n : m;
  Operand a(A, na, na, lda, 8), b(B, m, n, ldb, 8);
  if (alpha != 0.0 && a.bind(true, s)) return;
  if (b.bind(alpha != 0.0, s)) return;
  if (dtrsm_select(side, uplo, trans, unit, m, n, alpha, a.d<double>(), a.dld, b.d<double>(),
                   b.dld, s))
    return;
  b.unbind(s);
  finish_blocking(s);
}

int dgemmt_device(int uplo, int ta, int tb, int64_t m, int64_t k, double alpha, const double *A,
                  int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                  int64_t ldc, cudaStream_t s);
int dsyr2k_device(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                  int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
                  cudaStream_t s);
int dtrmm_device(int side, int uplo, int trans, int unit_code, int64_t m, int64_t n,
                 double alpha, const double *A, int64_t lda, double *B, int64_t ldb,
                 cudaStream_t s);

static void dgemmt_blocking(int uplo, int ta, int tb, int64_t m, int64_t k, double alpha,
                            const double *A, int64_t lda, const double *B, int64_t ldb,
                            double beta, double *C, int64_t ldc) {
  if (m == 0) return;  // interface/gemmt.c: quick return
  if (ensure_init()) return;
  cudaStream_t s = stream();
  const bool need_ab = k > 0 && alpha != 0.0;
  Operand a(A, ta ? k : m, ta ? m : k, lda, 8), b(B, tb ? m : k, tb ? k : m, ldb, 8);
  Operand c(C, m, m, ldc, 8);
  if (need_ab && (a.bind(true, s) || b.bind(true, s))) return;
  if (c.bind(true, s)) return;  // the other triangle must survive the round trip
  if (dgemmt_device(uplo, ta, tb, m, k, alpha, a.d<double>(), a.dld, b.d<double>(), b.dld, beta,
                    c.d<double>(), c.dld, s))
    return;
  c.unbind(s);
  finish_blocking(s);
}

static void dsyr2k_blocking(int uplo, int trans, int64_t n, int64_t k, double alpha,
                            const double *A, int64_t lda, const double *B, int64_t ldb,
                            double beta, double *C, int64_t ldc) {
  if (n == 0) return;
  if (ensure_init()) return;
  cudaStream_t s = stream();
  const bool need_ab = k > 0 && alpha != 0.0;
  Operand a(A, trans ? k : n, trans ? n : k, lda, 8), b(B, trans ? k : n, trans ? n : k, ldb, 8);
  Operand c(C, n, n, ldc, 8);
  if (need_ab && (a.bind(true, s) || b.bind(true, s))) return;
  if (c.bind(true, s)) return;
  if (dsyr2k_device(uplo, trans, n, k, alpha, a.d<double>(), a.dld, b.d<double>(), b.dld, beta,
                    c.d<double>(), c.dld, s))
    return;
  c.unbind(s);
  finish_blocking(s);
}

static void dtrmm_blocking(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                           double alpha, const double *A, int64_t lda, double *B, int64_t ldb) {
  if (m == 0 || n == 0) return;
  if (ensure_init()) return;
  cudaStream_t s = stream();
  const int64_t na = side ? n : m;
  Operand a(A, na, na, lda, 8), b(B, m, n, ldb, 8);
  if (alpha != 0.0 && a.bind(true, s)) return;
  if (b.bind(alpha != 0.0, s)) return;
  if (dtrmm_device(side, uplo, trans, unit, m, n, alpha, a.d<double>(), a.dld, b.d<double>(),
                   b.dld, s))
    return;
  b.unbind(s);
  finish_blocking(s);
}

static void dsyrk_blocking(int uplo, int trans, int64_t n, int64_t k, double alpha,
                           const double *A, int64_t lda, double beta, double *C, int64_t ldc) {
  if (n == 0) return;  // interface/syrk.c:344
  if (ensure_init()) return;
  cudaStream_t s = stream();
  Operand a(A, trans ? k : n, trans ? n : k, lda, 8), c(C, n, n, ldc, 8);
  if (k > 0 && alpha != 0.0 && a.bind(true, s)) return;
  // the untouched triangle must survive the round trip, so C is always staged in
  if (c.bind(true, s)) return;
  if (dsyrk_device(uplo, trans, n, k, alpha, a.d<double>(), a.dld, beta, c.d<double>(), c.dld,
                   s))
    return;
  c.unbind(s);
  finish_blocking(s);
}

}  // namespace gb

using namespace gb;

// interface/gemm.c:374-471: row-major is the column-major product of the
// transposes, so A<->B, m<->n and transa<->transb swap.
template <typename T, void (*Blocking)(int, int, int64_t, int64_t, int64_t, T, const T *, int64_t,
                                       const T *, int64_t, T, T *, int64_t)>
static void cblas_gemm_t(int order, int TransA, int TransB, blasint m, blasint n, blasint k,
                         T alpha, const T *a, blasint lda, const T *b, blasint ldb, T beta, T *c,
                         blasint ldc, const char *name) {
  int info = -1, ta = -1, tb = -1;
  int64_t M = m, N = n;
  const T *pa = a, *pb = b;
  int64_t la = lda, lb = ldb;
  if (order == CblasColMajor) {
    ta = cblas_trans_code(TransA);
    tb = cblas_trans_code(TransB);
  } else if (order == CblasRowMajor) {
    M = n;
    N = m;
    pa = b;
    pb = a;
    la = ldb;
    lb = lda;
    ta = cblas_trans_code(TransB);
    tb = cblas_trans_code(TransA);
  }
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = gemm_check(ta, tb, M, N, k, la, lb, ldc);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla(name, info);
    return;
  }
  Blocking(ta, tb, M, N, k, alpha, pa, la, pb, lb, beta, c, ldc);
}

extern "C" {

// ---------------------------------------------------------------------------
// GEMM
// ---------------------------------------------------------------------------
void dgemm_(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
            const blasint *K, const double *alpha, const double *A, const blasint *ldA,
            const double *B, const blasint *ldB, const double *beta, double *C,
            const blasint *ldC) {
  int ta = trans_code(*TRANSA), tb = trans_code(*TRANSB);
  int info = gemm_check(ta, tb, *M, *N, *K, *ldA, *ldB, *ldC);
  if (info) {
    call_xerbla("DGEMM ", info);
    return;
  }
  dgemm_blocking(ta, tb, *M, *N, *K, *alpha, A, *ldA, B, *ldB, *beta, C, *ldC);
}

void sgemm_(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
            const blasint *K, const float *alpha, const float *A, const blasint *ldA,
            const float *B, const blasint *ldB, const float *beta, float *C,
            const blasint *ldC) {
  int ta = trans_code(*TRANSA), tb = trans_code(*TRANSB);
  int info = gemm_check(ta, tb, *M, *N, *K, *ldA, *ldB, *ldC);
  if (info) {
    call_xerbla("SGEMM ", info);
    return;
  }
  sgemm_blocking(ta, tb, *M, *N, *K, *alpha, A, *ldA, B, *ldB, *beta, C, *ldC);
}

void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_TRANSPOSE TransB, blasint m, blasint n, blasint k, double alpha,
                 const double *a, blasint lda, const double *b, blasint ldb, double beta,
                 double *c, blasint ldc) {
  cblas_gemm_t<double, dgemm_blocking>(order, TransA, TransB, m, n, k, alpha, a, lda, b, ldb,
                                       beta, c, ldc, "DGEMM ");
}

void cblas_sgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_TRANSPOSE TransB, blasint m, blasint n, blasint k, float alpha,
                 const float *a, blasint lda, const float *b, blasint ldb, float beta, float *c,
                 blasint ldc) {
  cblas_gemm_t<float, sgemm_blocking>(order, TransA, TransB, m, n, k, alpha, a, lda, b, ldb,
                                      beta, c, ldc, "SGEMM ");
}

// ---------------------------------------------------------------------------
// TRSM (interface/trsm.c)
// ---------------------------------------------------------------------------
static int trsm_check(int side, int uplo, int trans, int unit, int64_t m, int64_t n, int64_t lda,
                      int64_t ldb) {
  int64_t nrowa = (side & 1) ? n : m;
  int info = 0;
  if (ldb < (m > 1 ? m : 1)) info = 11;
  if (lda < (nrowa > 1 ? nrowa : 1)) info = 9;
  if (n < 0) info = 6;
  if (m < 0) info = 5;
  if (unit < 0) info = 4;
  if (trans < 0) info = 3;
  if (uplo < 0) info = 2;
  if (side < 0) info = 1;
  return info;
}

void dtrsm_(const char *SIDE, const char *UPLO, const char *TRANSA, const char *DIAG,
            const blasint *M, const blasint *N, const double *alpha, const double *A,
            const blasint *ldA, double *B, const blasint *ldB) {
  char sd = upch(SIDE), up = upch(UPLO), tr = upch(TRANSA), dg = upch(DIAG);
  int side = sd == 'L' ? 0 : sd == 'R' ? 1 : -1;
  int uplo = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int trans = (tr == 'N' || tr == 'R') ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  int unit = dg == 'U' ? 0 : dg == 'N' ? 1 : -1;
  int info = trsm_check(side, uplo, trans, unit, *M, *N, *ldA, *ldB);
  if (info) {
    call_xerbla("DTRSM ", info);
    return;
  }
  dtrsm_blocking(side, uplo, trans, unit, *M, *N, *alpha, A, *ldA, B, *ldB);
}

void cblas_dtrsm(enum CBLAS_ORDER order, enum CBLAS_SIDE Side, enum CBLAS_UPLO Uplo,
                 enum CBLAS_TRANSPOSE Trans, enum CBLAS_DIAG Diag, blasint m, blasint n,
                 double alpha, const double *a, blasint lda, double *b, blasint ldb) {
  // interface/trsm.c:276-351: row-major swaps m<->n, Left<->Right, Upper<->Lower
  int side = -1, uplo = -1, trans = -1, unit = -1, info = -1;
  int64_t M = m, N = n;
  if (order == CblasColMajor) {
    side = Side == CblasLeft ? 0 : Side == CblasRight ? 1 : -1;
    uplo = Uplo == CblasUpper ? 0 : Uplo == CblasLower ? 1 : -1;
  } else if (order == CblasRowMajor) {
    M = n;
    N = m;
    side = Side == CblasLeft ? 1 : Side == CblasRight ? 0 : -1;
    uplo = Uplo == CblasUpper ? 1 : Uplo == CblasLower ? 0 : -1;
  }
  trans = cblas_trans_code(Trans);
  unit = Diag == CblasUnit ? 0 : Diag == CblasNonUnit ? 1 : -1;
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = trsm_check(side, uplo, trans, unit, M, N, lda, ldb);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla("DTRSM ", info);
    return;
  }
  dtrsm_blocking(side, uplo, trans, unit, M, N, alpha, a, lda, b, ldb);
}

// ---------------------------------------------------------------------------
// SYRK (interface/syrk.c)
// ---------------------------------------------------------------------------
static int syrk_check(int uplo, int trans, int64_t n, int64_t k, int64_t lda, int64_t ldc) {
  int64_t nrowa = (trans & 1) ? k : n;
  int info = 0;
  if (ldc < (n > 1 ? n : 1)) info = 10;
  if (lda < (nrowa > 1 ? nrowa : 1)) info = 7;
  if (k < 0) info = 4;
  if (n < 0) info = 3;
  if (trans < 0) info = 2;
  if (uplo < 0) info = 1;
  return info;
}

void dsyrk_(const char *UPLO, const char *TRANS, const blasint *N, const blasint *K,
            const double *alpha, const double *A, const blasint *ldA, const double *beta,
            double *C, const blasint *ldC) {
  char up = upch(UPLO), tr = upch(TRANS);
  int uplo = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int trans = tr == 'N' ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  int info = syrk_check(uplo, trans, *N, *K, *ldA, *ldC);
  if (info) {
    call_xerbla("DSYRK ", info);
    return;
  }
  dsyrk_blocking(uplo, trans, *N, *K, *alpha, A, *ldA, *beta, C, *ldC);
}

void cblas_dsyrk(enum CBLAS_ORDER order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE Trans,
                 blasint n, blasint k, double alpha, const double *a, blasint lda, double beta,
                 double *c, blasint ldc) {
  // interface/syrk.c:291-335: row-major flips uplo and trans
  int uplo = -1, trans = -1, info = -1;
  if (order == CblasColMajor) {
    uplo = Uplo == CblasUpper ? 0 : Uplo == CblasLower ? 1 : -1;
    trans = cblas_trans_code(Trans);
  } else if (order == CblasRowMajor) {
    uplo = Uplo == CblasUpper ? 1 : Uplo == CblasLower ? 0 : -1;
    int t = cblas_trans_code(Trans);
    trans = t < 0 ? -1 : 1 - t;
  }
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = syrk_check(uplo, trans, n, k, lda, ldc);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla("DSYRK ", info);
    return;
  }
  dsyrk_blocking(uplo, trans, n, k, alpha, a, lda, beta, c, ldc);
}

// ---------------------------------------------------------------------------
// TRMM (interface/trsm.c built with TRMM: same checks and row-major mapping)
// ---------------------------------------------------------------------------
void dtrmm_(const char *SIDE, const char *UPLO, const char *TRANSA, const char *DIAG,
            const blasint *M, const blasint *N, const double *alpha, const double *A,
            const blasint *ldA, double *B, const blasint *ldB) {
  char sd = upch(SIDE), up = upch(UPLO), tr = upch(TRANSA), dg = upch(DIAG);
  int side = sd == 'L' ? 0 : sd == 'R' ? 1 : -1;
  int uplo = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int trans = (tr == 'N' || tr == 'R') ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  int unit = dg == 'U' ? 0 : dg == 'N' ? 1 : -1;
  int info = trsm_check(side, uplo, trans, unit, *M, *N, *ldA, *ldB);
  if (info) {
    call_xerbla("DTRMM ", info);
    return;
  }
  dtrmm_blocking(side, uplo, trans, unit, *M, *N, *alpha, A, *ldA, B, *ldB);
}

void cblas_dtrmm(enum CBLAS_ORDER order, enum CBLAS_SIDE Side, enum CBLAS_UPLO Uplo,
                 enum CBLAS_TRANSPOSE Trans, enum CBLAS_DIAG Diag, blasint m, blasint n,
                 double alpha, const double *a, blasint lda, double *b, blasint ldb) {
  int side = -1, uplo = -1, trans = -1, unit = -1, info = -1;
  int64_t M = m, N = n;
  if (order == CblasColMajor) {
    side = Side == CblasLeft ? 0 : Side == CblasRight ? 1 : -1;
    uplo = Uplo == CblasUpper ? 0 : Uplo == CblasLower ? 1 : -1;
  } else if (order == CblasRowMajor) {
    M = n;
    N = m;
    side = Side == CblasLeft ? 1 : Side == CblasRight ? 0 : -1;
    uplo = Uplo == CblasUpper ? 1 : Uplo == CblasLower ? 0 : -1;
  }
  trans = cblas_trans_code(Trans);
  unit = Diag == CblasUnit ? 0 : Diag == CblasNonUnit ? 1 : -1;
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = trsm_check(side, uplo, trans, unit, M, N, lda, ldb);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla("DTRMM ", info);
    return;
  }
  dtrmm_blocking(side, uplo, trans, unit, M, N, alpha, a, lda, b, ldb);
}

// ---------------------------------------------------------------------------
// SYR2K (interface/syr2k.c)
// ---------------------------------------------------------------------------
static int syr2k_check(int uplo, int trans, int64_t n, int64_t k, int64_t lda, int64_t ldb,
                       int64_t ldc) {
  int64_t nrowa = (trans & 1) ? k : n;
  int info = 0;
  if (ldc < (n > 1 ? n : 1)) info = 12;
  if (ldb < (nrowa > 1 ? nrowa : 1)) info = 9;
  if (lda < (nrowa > 1 ? nrowa : 1)) info = 7;
  if (k < 0) info = 4;
  if (n < 0) info = 3;
  if (trans < 0) info = 2;
  if (uplo < 0) info = 1;
  return info;
}

void dsyr2k_(const char *UPLO, const char *TRANS, const blasint *N, const blasint *K,
             const double *alpha, const double *A, const blasint *ldA, const double *B,
             const blasint *ldB, const double *beta, double *C, const blasint *ldC) {
  char up = upch(UPLO), tr = upch(TRANS);
  int uplo = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int trans = tr == 'N' ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  int info = syr2k_check(uplo, trans, *N, *K, *ldA, *ldB, *ldC);
  if (info) {
    call_xerbla("DSYR2K", info);
    return;
  }
  dsyr2k_blocking(uplo, trans, *N, *K, *alpha, A, *ldA, B, *ldB, *beta, C, *ldC);
}

void cblas_dsyr2k(enum CBLAS_ORDER order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE Trans,
                  blasint n, blasint k, double alpha, const double *a, blasint lda,
                  const double *b, blasint ldb, double beta, double *c, blasint ldc) {
  // interface/syr2k.c: row-major flips uplo and trans (the sum is symmetric in A, B)
  int uplo = -1, trans = -1, info = -1;
  if (order == CblasColMajor) {
    uplo = Uplo == CblasUpper ? 0 : Uplo == CblasLower ? 1 : -1;
    trans = cblas_trans_code(Trans);
  } else if (order == CblasRowMajor) {
    uplo = Uplo == CblasUpper ? 1 : Uplo == CblasLower ? 0 : -1;
    int t = cblas_trans_code(Trans);
    trans = t < 0 ? -1 : 1 - t;
  }
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = syr2k_check(uplo, trans, n, k, lda, ldb, ldc);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla("DSYR2K", info);
    return;
  }
  dsyr2k_blocking(uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

// ---------------------------------------------------------------------------
// GEMMT (interface/gemmt.c)
// ---------------------------------------------------------------------------
static int gemmt_check(int uplo, int ta, int tb, int64_t m, int64_t k, int64_t lda, int64_t ldb,
                       int64_t ldc) {
  const int64_t nrowa = (ta & 1) ? k : m, nrowb = (tb & 1) ? m : k;
  int info = 0;
  if (ldc < (m > 1 ? m : 1)) info = 13;
  if (ldb < (nrowb > 1 ? nrowb : 1)) info = 10;
  if (lda < (nrowa > 1 ? nrowa : 1)) info = 8;
  if (k < 0) info = 5;
  if (m < 0) info = 4;
  if (tb < 0) info = 3;
  if (ta < 0) info = 2;
  if (uplo < 0) info = 1;
  return info;
}

void dgemmt_(const char *UPLO, const char *TRANSA, const char *TRANSB, const blasint *M,
             const blasint *K, const double *alpha, const double *A, const blasint *ldA,
             const double *B, const blasint *ldB, const double *beta, double *C,
             const blasint *ldC) {
  char up = upch(UPLO);
  int uplo = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int ta = trans_code(upch(TRANSA)), tb = trans_code(upch(TRANSB));
  int info = gemmt_check(uplo, ta, tb, *M, *K, *ldA, *ldB, *ldC);
  if (info) {
    call_xerbla("DGEMMT ", info);
    return;
  }
  dgemmt_blocking(uplo, ta, tb, *M, *K, *alpha, A, *ldA, B, *ldB, *beta, C, *ldC);
}

void cblas_dgemmt(enum CBLAS_ORDER order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE TransA,
                  enum CBLAS_TRANSPOSE TransB, blasint m, blasint k, double alpha,
                  const double *a, blasint lda, const double *b, blasint ldb, double beta,
                  double *c, blasint ldc) {
  // interface/gemmt.c: row-major swaps the operands, flips uplo and the roles
  // of the two transposes
  int uplo = -1, ta = -1, tb = -1, info = -1;
  const double *pa = a, *pb = b;
  blasint la = lda, lb = ldb;
  if (order == CblasColMajor) {
    uplo = Uplo == CblasUpper ? 0 : Uplo == CblasLower ? 1 : -1;
    ta = cblas_trans_code(TransA);
    tb = cblas_trans_code(TransB);
  } else if (order == CblasRowMajor) {
    uplo = Uplo == CblasUpper ? 1 : Uplo == CblasLower ? 0 : -1;
    ta = cblas_trans_code(TransB);
    tb = cblas_trans_code(TransA);
    pa = b;
    pb = a;
    la = ldb;
    lb = lda;
  }
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = gemmt_check(uplo, ta, tb, m, k, la, lb, ldc);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla("DGEMMT ", info);
    return;
  }
  dgemmt_blocking(uplo, ta, tb, m, k, alpha, pa, la, pb, lb, beta, c, ldc);
}

// ---------------------------------------------------------------------------
// grouped batch (interface/gemm_batch.c:117-372)
// ---------------------------------------------------------------------------

void cblas_dgemm_batch(enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE *transa_array,
                       const enum CBLAS_TRANSPOSE *transb_array, const blasint *m_array,
                       const blasint *n_array, const blasint *k_array,
                       const double *alpha_array, const double **a_array,
                       const blasint *lda_array, const double **b_array,
                       const blasint *ldb_array, const double *beta_array, double **c_array,
                       const blasint *ldc_array, blasint group_count,
                       const blasint *group_size) {
  // validate every group first, exactly as the reference does before it
  // runs anything (gemm_batch.c:195-283)
  std::vector<int> ta(group_count > 0 ? group_count : 1), tb(ta.size());
  for (blasint g = 0; g < group_count; ++g) {
    int64_t M, N, la, lb;
    int a_code, b_code;
    if (order == CblasColMajor) {
      M = m_array[g];
      N = n_array[g];
      la = lda_array[g];
      lb = ldb_array[g];
      a_code = cblas_trans_code(transa_array[g]);
      b_code = cblas_trans_code(transb_array[g]);
    } else if (order == CblasRowMajor) {
      M = n_array[g];
      N = m_array[g];
      la = ldb_array[g];
      lb = lda_array[g];
      a_code = cblas_trans_code(transb_array[g]);
      b_code = cblas_trans_code(transa_array[g]);
    } else {
      call_xerbla("DGEMM_BATCH ", 0);  // gemm_batch.c:44, info 0 for a bad order
      return;
    }
    int info = gemm_check(a_code, b_code, M, N, k_array[g], la, lb, ldc_array[g]);
    if (info) {
      call_xerbla("DGEMM_BATCH ", info);
      return;
    }
    ta[g] = a_code;
    tb[g] = b_code;
  }
  gb_dgemm_batch_grouped(order, ta.data(), tb.data(), m_array, n_array, k_array, alpha_array,
                         a_array, lda_array, b_array, ldb_array, beta_array, c_array, ldc_array,
                         group_count, group_size);
}

// ---------------------------------------------------------------------------
// device-pointer API
// ---------------------------------------------------------------------------
static int dev_gemm_args(char transa, char transb, int64_t m, int64_t n, int64_t k, int64_t lda,
                         int64_t ldb, int64_t ldc, int *ta, int *tb, const char *name) {
  *ta = trans_code(transa);
  *tb = trans_code(transb);
  int info = gemm_check(*ta, *tb, m, n, k, lda, ldb, ldc);
  if (info) {
    call_xerbla(name, info);
    return GB_ERR_INVALID_VALUE;
  }
  return ensure_init();
}

int gb_dgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                 const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                 double *C, int64_t ldc) {
  int ta, tb;
  int st = dev_gemm_args(transa, transb, m, n, k, lda, ldb, ldc, &ta, &tb, "DGEMM ");
  if (st) return st;
  return dgemm_dispatch(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream());
}

int gb_dgemm_native_dev(char transa, char transb, int64_t m, int64_t n, int64_t k, double alpha,
                        const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                        double *C, int64_t ldc) {
  int ta, tb;
  int st = dev_gemm_args(transa, transb, m, n, k, lda, ldb, ldc, &ta, &tb, "DGEMM ");
  if (st) return st;
  return dgemm_native(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream());
}

int gb_dgemm_emulated_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                          double alpha, const double *A, int64_t lda, const double *B,
                          int64_t ldb, double beta, double *C, int64_t ldc, int slices) {
  int ta, tb;
  int st = dev_gemm_args(transa, transb, m, n, k, lda, ldb, ldc, &ta, &tb, "DGEMM ");
  if (st) return st;
  if (m == 0 || n == 0) return GB_SUCCESS;
  if (k == 0 || alpha == 0.0) {
    launch_dgemm_beta(m, n, beta, C, ldc, stream());
    return check_cuda(cudaGetLastError(), "dgemm_beta launch");
  }
  return dgemm_emulated(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                        slices > 0 ? slices : ozaki_caller_slices(), stream());
}

int gb_sgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k, float alpha,
                 const float *A, int64_t lda, const float *B, int64_t ldb, float beta, float *C,
                 int64_t ldc) {
  int ta, tb;
  int st = dev_gemm_args(transa, transb, m, n, k, lda, ldb, ldc, &ta, &tb, "SGEMM ");
  if (st) return st;
  if (m == 0 || n == 0) return GB_SUCCESS;
  if (k == 0 || alpha == 0.0f) {
    launch_sgemm_beta(m, n, beta, C, ldc, stream());
    return check_cuda(cudaGetLastError(), "sgemm launch");
  }
  return sgemm_dispatch(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream());
}

int gb_dgemmt_dev(char uplo, char transa, char transb, int64_t m, int64_t k, double alpha,
                  const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                  double *C, int64_t ldc) {
  const char u = upch(uplo);
  const int up = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  const int ta = trans_code(upch(transa)), tb = trans_code(upch(transb));
  const int info = gemmt_check(up, ta, tb, m, k, lda, ldb, ldc);
  if (info) {
    call_xerbla("DGEMMT ", info);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return dgemmt_device(up, ta, tb, m, k, alpha, A, lda, B, ldb, beta, C, ldc, stream());
}

int gb_dsyr2k_dev(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *A,
                  int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                  int64_t ldc) {
  const char u = upch(uplo), t = upch(trans);
  const int up = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  const int tr = t == 'N' ? 0 : (t == 'T' || t == 'C') ? 1 : -1;
  const int info = syr2k_check(up, tr, n, k, lda, ldb, ldc);
  if (info) {
    call_xerbla("DSYR2K", info);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return dsyr2k_device(up, tr, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream());
}

int gb_dtrmm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n,
                 double alpha, const double *A, int64_t lda, double *B, int64_t ldb) {
  const char sd = upch(side), up = upch(uplo), tr = upch(transa), dg = upch(diag);
  const int s_ = sd == 'L' ? 0 : sd == 'R' ? 1 : -1;
  const int u_ = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  const int t_ = (tr == 'N' || tr == 'R') ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  const int d_ = dg == 'U' ? 0 : dg == 'N' ? 1 : -1;
  const int info = trsm_check(s_, u_, t_, d_, m, n, lda, ldb);
  if (info) {
    call_xerbla("DTRMM ", info);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return dtrmm_device(s_, u_, t_, d_, m, n, alpha, A, lda, B, ldb, stream());
}

int gb_dtrsm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n,
                 double alpha, const double *A, int64_t lda, double *B, int64_t ldb) {
  char sd = upch(side), up = upch(uplo), tr = upch(transa), dg = upch(diag);
  int is = sd == 'L' ? 0 : sd == 'R' ? 1 : -1;
  int iu = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int it = (tr == 'N' || tr == 'R') ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  int id = dg == 'U' ? 0 : dg == 'N' ? 1 : -1;
  int info = trsm_check(is, iu, it, id, m, n, lda, ldb);
  if (info) {
    call_xerbla("DTRSM ", info);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  if (m == 0 || n == 0) return GB_SUCCESS;
  return dtrsm_select(is, iu, it, id, m, n, alpha, A, lda, B, ldb, stream());
}

int gb_dsyrk_dev(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *A,
                 int64_t lda, double beta, double *C, int64_t ldc) {
  char up = upch(uplo), tr = upch(trans);
  int iu = up == 'U' ? 0 : up == 'L' ? 1 : -1;
  int it = tr == 'N' ? 0 : (tr == 'T' || tr == 'C') ? 1 : -1;
  int info = syrk_check(iu, it, n, k, lda, ldc);
  if (info) {
    call_xerbla("DSYRK ", info);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  if (n == 0) return GB_SUCCESS;
  return dsyrk_device(iu, it, n, k, alpha, A, lda, beta, C, ldc, stream());
}

}  // extern "C"
