// FP32 GEMM on the bf16 tensor cores: C = alpha*op(A)*op(B) + beta*C.
//
// Every FP32 operand element x is split into three bf16 terms, x1 = bf16(x),
// x2 = bf16(x - x1), x3 = bf16(x - x1 - x2); each residual is exact in FP32.
// For |x| >= 2^-110 the split is exact, x = x1 + x2 + x3, with
// |x2| <= 2^-8 |x| and |x3| <= 2^-17 |x| (|x2| <= 2^-7 |x| for the values
// next to FLT_MAX whose x1 rounds toward zero).  The product keeps the six terms
// A_i B_j with i + j <= 4 (1-based).  The three dropped terms together are
// at most (2^-24 + 2^-34) |a b| (2^-8 * 2^-17 twice, plus 2^-17 * 2^-17),
// about FP32's unit roundoff.  Every bf16 x bf16
// product is exact in FP32, and the six products are accumulated in FP32 in
// TMEM.  So the result has the accuracy of an FP32 GEMM (errors of order
// K * 2^-24 * sum|a||b|), at six bf16 MMA passes instead of one FP32 FMA
// pass: the FP32 SIMT rate is 128 FMA/clk/SM, the bf16 tensor rate 4096
// MAC/clk/SM.
//
// Below 2^-110, x2 and x3 fall into bf16's subnormal range, which keeps
// fewer bits than FP32's.  The split then loses bits: the relative error is
// about 2^-23 at 2^-111 and doubles with each binade below, to 2^-8 at
// 2^-126, and values below 2^-133 are lost.  This is harmless for an
// element next to larger ones in its row or column.  But a product whose
// operands are all that small loses accuracy in this form; the SIMT form
// (GB_SGEMM_MODE=simt) has none of this limit.
//
// Serves the trailing updates of the FP32 LU of the mixed solver (sgemm
// semantics of interface/gemm.c; kernel/generic/gemm_beta.c for beta).
//
// Kernel layout: persistent, one CTA per SM, warp-specialised.  Per
// 64-wide K block, warp 0 loads the three A slices of the 128-row tile into
// one of two A stages (48 KB) and streams the three B slices of the 256-row
// tile through a 3-slot ring (32 KB each), so each A and B tile is fetched
// once per K block for all six products.  Warp 1 issues tcgen05.mma (M=128,
// N=256, K=16) into one of two TMEM accumulators; warps 2..9 drain the other
// accumulator into C.  All waits are bounded: a role that times out raises
// an abort flag and the kernel winds down with an error status.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"
#include "lapack_internal.h"
#include "sm100_primitives.cuh"
#include "tma_host.h"

namespace gb {
namespace s3 {

constexpr int BM = 128, BN = 256, BK = 64;
constexpr int A_BYTES = BM * BK * 2;   // one slice tile of A: 16 KB
constexpr int B_BYTES = BN * BK * 2;   // one slice tile of B: 32 KB
constexpr int A_STAGES = 2;            // each stage holds the 3 slices of A
constexpr int B_SLOTS = 3;
constexpr int NUM_THREADS = 320;
constexpr int TMEM_COLS = 512;
constexpr int SMEM_BYTES = A_STAGES * 3 * A_BYTES + B_SLOTS * B_BYTES + 1024 + 256;
constexpr uint64_t WAIT_LIMIT_NS = 4000000000ull;
constexpr int GROUP_M = 8;  // m-tiles per group of the tile order

struct Params {
  int m_tiles, n_tiles, kblocks;
  int m_pad, n_pad;
  int64_t m, n, ldc;
  float alpha, beta;
  float *C;
  const int *rflag;  // rows of op(A) holding Inf/NaN: left to the fixup kernel
  const int *cflag;  // columns of op(B) holding Inf/NaN
  int tri;           // 0 all of C; 1 only i >= j; 2 only i <= j
  const int *skip;   // device flag: when nonzero C is left unchanged
  int *status;
};

__device__ __forceinline__ void tile_coords(int tile, const Params &p, int &mt, int &nt) {
  const int span = GROUP_M * p.n_tiles;
  const int first_m = (tile / span) * GROUP_M;
  const int rem = p.m_tiles - first_m;
  const int gm = rem < GROUP_M ? rem : GROUP_M;
  const int in = tile % span;
  mt = first_m + in % gm;
  nt = in / gm;
}

// A tile takes part unless it lies wholly in the triangle left alone.
template <int TRI>
__device__ __forceinline__ bool tile_active(int mt, int nt) {
  if (TRI == 1) return mt * BM + BM - 1 >= nt * BN;
  if (TRI == 2) return mt * BM <= nt * BN + BN - 1;
  return true;
}

// TRI (0 all of C, 1 lower, 2 upper) is a template parameter so that the
// full-C instance keeps the plain store loop of the epilogue.  RC (full C
// only): beta != 0, C is read -- ahead of its use, see the epilogue.
template <int TRI, bool RC>
__global__ void __launch_bounds__(NUM_THREADS, 1)
sgemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tmA,
                    const __grid_constant__ CUtensorMap tmB, const Params p) {
  using namespace sm100;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *sA = smem;                                   // [A_STAGES][3][A_BYTES]
  uint8_t *sB = smem + A_STAGES * 3 * A_BYTES;          // [B_SLOTS][B_BYTES]
  uint64_t *afull = reinterpret_cast<uint64_t *>(sB + B_SLOTS * B_BYTES);
  uint64_t *aempty = afull + A_STAGES;
  uint64_t *bfull = aempty + A_STAGES;
  uint64_t *bempty = bfull + B_SLOTS;
  uint64_t *tfull = bempty + B_SLOTS;
  uint64_t *tempty = tfull + 2;
  uint64_t *mma_done = tempty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < A_STAGES; ++i) {
      mbar_init(&afull[i], 1);
      mbar_init(&aempty[i], 1);
    }
    for (int i = 0; i < B_SLOTS; ++i) {
      mbar_init(&bfull[i], 1);
      mbar_init(&bempty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 8);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(tmem_slot, TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const int ntiles = p.m_tiles * p.n_tiles;
  auto fail = [&](int site) {
    *abort_flag = 1;
    atomicCAS(p.status, 0, GB_KERR_MBARRIER_TIMEOUT);
    atomicExch(p.status + 1, 200 + site);
  };

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      int as = 0, bs = 0;
      uint32_t aph = 0, bph = 0;
      bool a_issued[A_STAGES] = {false, false}, b_issued[B_SLOTS] = {false, false, false};
      uint32_t a_ph[A_STAGES] = {0, 0}, b_ph[B_SLOTS] = {0, 0, 0};
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        int mt, nt;
        tile_coords(tile, p, mt, nt);
        if (!tile_active<TRI>(mt, nt)) continue;
        for (int kb = 0; ok && kb < p.kblocks; ++kb) {
          if (!mbar_wait(&aempty[as], aph ^ 1u, abort_flag, WAIT_LIMIT_NS)) {
            fail(1);
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&afull[as], 3 * A_BYTES);
          for (int i = 0; i < 3; ++i)
            tma_load_2d(sA + (as * 3 + i) * A_BYTES, &tmA, &afull[as], kb * BK,
                        i * p.m_pad + mt * BM);
          a_issued[as] = true;
          a_ph[as] = aph;
          if (++as == A_STAGES) {
            as = 0;
            aph ^= 1u;
          }
          // B slices in the order the MMA issuer consumes them: 3, 2, 1
          for (int jj = 0; jj < 3; ++jj) {
            const int j = 2 - jj;
            if (!mbar_wait(&bempty[bs], bph ^ 1u, abort_flag, WAIT_LIMIT_NS)) {
              fail(2);
              ok = false;
              break;
            }
            mbar_arrive_expect_tx(&bfull[bs], B_BYTES);
            tma_load_2d(sB + bs * B_BYTES, &tmB, &bfull[bs], kb * BK, j * p.n_pad + nt * BN);
            b_issued[bs] = true;
            b_ph[bs] = bph;
            if (++bs == B_SLOTS) {
              bs = 0;
              bph ^= 1u;
            }
          }
        }
      }
      // never leave with TMA writes still landing in shared memory
      volatile int no_abort = 0;
      for (int i = 0; i < A_STAGES; ++i)
        if (a_issued[i]) mbar_wait(&afull[i], a_ph[i], &no_abort, WAIT_LIMIT_NS);
      for (int i = 0; i < B_SLOTS; ++i)
        if (b_issued[i]) mbar_wait(&bfull[i], b_ph[i], &no_abort, WAIT_LIMIT_NS);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t IDESC = idesc_bf16_f32(BM, BN);
      int as = 0, bs = 0, acc = 0;
      uint32_t aph = 0, bph = 0, acc_phase = 0;
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        int mt, nt;
        tile_coords(tile, p, mt, nt);
        if (!tile_active<TRI>(mt, nt)) continue;
        if (!mbar_wait(&tempty[acc], acc_phase ^ 1u, abort_flag, WAIT_LIMIT_NS)) {
          fail(3);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + (uint32_t)(acc * BN);
        uint32_t accumulate = 0;
        for (int kb = 0; ok && kb < p.kblocks; ++kb) {
          if (!mbar_wait(&afull[as], aph, abort_flag, WAIT_LIMIT_NS)) {
            fail(4);
            ok = false;
            break;
          }
          for (int jj = 0; jj < 3; ++jj) {
            const int j = 2 - jj;  // B slice index (0-based) in this ring slot
            if (!mbar_wait(&bfull[bs], bph, abort_flag, WAIT_LIMIT_NS)) {
              fail(5);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t bdesc = sdesc_kmajor_sw128(smem_u32(sB + bs * B_BYTES));
            // products A_i B_j with i + j <= 2 (0-based), smaller terms first
            for (int i = 2 - j; i >= 0; --i) {
              const uint64_t adesc = sdesc_kmajor_sw128(smem_u32(sA + (as * 3 + i) * A_BYTES));
#pragma unroll
              for (int k = 0; k < BK / 16; ++k) {
                mma_bf16(d_tmem, adesc + (uint64_t)(2 * k), bdesc + (uint64_t)(2 * k), IDESC,
                         accumulate);
                accumulate = 1;
              }
            }
            mma_commit(&bempty[bs]);
            if (++bs == B_SLOTS) {
              bs = 0;
              bph ^= 1u;
            }
          }
          if (!ok) break;
          mma_commit(&aempty[as]);
          if (++as == A_STAGES) {
            as = 0;
            aph ^= 1u;
          }
        }
        if (!ok) break;
        mma_commit(&tfull[acc]);
        acc ^= 1;
        if (acc == 0) acc_phase ^= 1u;
      }
      // TMEM is freed at exit: wait until every issued MMA has completed
      mma_commit(mma_done);
      volatile int no_abort = 0;
      mbar_wait(mma_done, 0, &no_abort, WAIT_LIMIT_NS);
    }
  } else {
    // ------------------------------------------------ epilogue (8 warps)
    const int q = warp & 3;            // TMEM lane quadrant this warp may access
    const int half = (warp - 2) >> 2;  // column half of the 256-wide tile
    const int row = q * 32 + lane;     // tile row owned by this thread
    int acc = 0;
    uint32_t acc_phase = 0;
    const bool read_c = p.beta != 0.f;
    const bool skipped = p.skip != nullptr && *p.skip != 0;  // drain TMEM, write nothing
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      int mt, nt;
      tile_coords(tile, p, mt, nt);
      if (!tile_active<TRI>(mt, nt)) continue;
      if constexpr (TRI == 0) {
        const int64_t grow = (int64_t)mt * BM + row;
        const int64_t col0 = (int64_t)nt * BN + half * 128;
        const bool row_ok = !skipped && grow < p.m && p.rflag[grow] == 0;
        const bool load_c = RC && row_ok;
        // C is requested ahead of its use: chunk 0 before the accumulator is
        // ready (the loads overlap the MMAs), each later chunk while the one
        // before it is drained -- the old values are not read between a
        // finished accumulator and its stores
        float nxt[32];
        auto load_chunk = [&](int c) {
          const int64_t ncol = p.n - (col0 + c * 32);
          const float *cp = p.C + grow + (col0 + c * 32) * p.ldc;
#pragma unroll
          for (int j = 0; j < 32; ++j) nxt[j] = (load_c && j < ncol) ? cp[j * p.ldc] : 0.f;
        };
        load_chunk(0);
        const bool got = mbar_wait(&tfull[acc], acc_phase, abort_flag, WAIT_LIMIT_NS);
        // the warp-wide tcgen05.ld below needs a converged warp: agree first
        if (!__all_sync(0xffffffffu, got)) {
          if (lane == 0) fail(6);
          break;
        }
        tc_fence_after();
        const uint32_t taddr =
            tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + half * 128);
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
          float old[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) old[j] = nxt[j];
          if (c < 3) load_chunk(c + 1);
          uint32_t r[32];
          tmem_ld_32x32b_x32(taddr + c * 32, r);
          tmem_ld_wait();
          // columns of this chunk that the fixup kernel owns (lane j reads column j)
          const int64_t cj = col0 + c * 32 + lane;
          const unsigned skip = __ballot_sync(0xffffffffu, cj < p.n && p.cflag[cj] != 0);
          if (row_ok) {
            float *cp = p.C + grow + (col0 + c * 32) * p.ldc;
            const int64_t ncol = p.n - (col0 + c * 32);
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (j < ncol && !((skip >> j) & 1u))
                cp[j * p.ldc] = RC ? p.alpha * __uint_as_float(r[j]) + p.beta * old[j]
                                   : p.alpha * __uint_as_float(r[j]);
          }
        }
      } else {
        const bool got = mbar_wait(&tfull[acc], acc_phase, abort_flag, WAIT_LIMIT_NS);
        // the warp-wide tcgen05.ld below needs a converged warp: agree first
        if (!__all_sync(0xffffffffu, got)) {
          if (lane == 0) fail(6);
          break;
        }
        tc_fence_after();
        const int64_t grow = (int64_t)mt * BM + row;
        const int64_t col0 = (int64_t)nt * BN + half * 128;
        const uint32_t taddr =
            tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + half * 128);
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
          uint32_t r[32];
          tmem_ld_32x32b_x32(taddr + c * 32, r);
          tmem_ld_wait();
          // columns of this chunk that the fixup kernel owns (lane j reads column j)
          const int64_t cj = col0 + c * 32 + lane;
          const unsigned skip = __ballot_sync(0xffffffffu, cj < p.n && p.cflag[cj] != 0);
          if (!skipped && grow < p.m && p.rflag[grow] == 0) {
            float *cp = p.C + grow + (col0 + c * 32) * p.ldc;
            const int64_t ncol = p.n - (col0 + c * 32);
            float old[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) old[j] = (read_c && j < ncol) ? cp[j * p.ldc] : 0.f;
            if constexpr (TRI == 0) {
#pragma unroll
              for (int j = 0; j < 32; ++j)
                if (j < ncol && !((skip >> j) & 1u))
                  cp[j * p.ldc] = p.alpha * __uint_as_float(r[j]) + p.beta * old[j];
            } else {
              // columns j of this chunk inside the triangle: one mask per row
              uint32_t wmask = ncol >= 32 ? 0xffffffffu : (ncol <= 0 ? 0u : (1u << ncol) - 1u);
              wmask &= ~skip;
              const int64_t d = grow - (col0 + c * 32);  // row minus the chunk's first column
              if (TRI == 1)  // keep col <= row: j <= d
                wmask &= d < 0 ? 0u : (d >= 31 ? 0xffffffffu : (2u << d) - 1u);
              else           // keep col >= row: j >= d
                wmask &= d <= 0 ? 0xffffffffu : (d > 31 ? 0u : ~((1u << d) - 1u));
#pragma unroll
              for (int j = 0; j < 32; ++j)
                if ((wmask >> j) & 1u)
                  cp[j * p.ldc] = p.alpha * __uint_as_float(r[j]) + p.beta * old[j];
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
      acc ^= 1;
      if (acc == 0) acc_phase ^= 1u;
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// x = x1 + x2 + x3 (+ below 2^-27 |x|); non-finite x keeps x in the first
// term so Inf and NaN propagate as in an FP32 product.
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &a, __nv_bfloat16 &b,
                                       __nv_bfloat16 &c) {
  if (!isfinite(x)) {
    a = __float2bfloat16_rn(x);
    b = c = __float2bfloat16_rn(0.f);
    return;
  }
  a = __float2bfloat16_rn(x);
  if (__hisinf(a)) a = __float2bfloat16_rz(x);  // finite x just below FLT_MAX
  float r = x - __bfloat162float(a);
  b = __float2bfloat16_rn(r);
  r -= __bfloat162float(b);
  c = __float2bfloat16_rn(r);
}

// Split the R x K op-view operand X (element (r, p) at X[p + r*ld] when
// K-contiguous, X[r + p*ld] otherwise) into three K-contiguous bf16 slices
// of Rpad x Kpad each (zero padding).  A CTA stages a 32 x 64 tile through
// shared memory so reads and 16-byte writes are both coalesced.
template <bool KCONTIG>
__global__ void __launch_bounds__(256)
split3_kernel(int64_t R, int64_t K, const float *__restrict__ X, int64_t ld, int64_t Rpad,
              int64_t Kpad, __nv_bfloat16 *__restrict__ dst, int *__restrict__ flag,
              int *__restrict__ list, int *__restrict__ count) {
  __shared__ float tile[32][65];
  const int64_t r0 = (int64_t)blockIdx.y * 32, p0 = (int64_t)blockIdx.x * 64;
  const int tid = threadIdx.x;
  for (int e = tid; e < 32 * 64; e += 256) {
    int rr, pp;
    if (KCONTIG) {
      rr = e >> 6;
      pp = e & 63;
    } else {
      rr = e & 31;
      pp = e >> 5;
    }
    const int64_t r = r0 + rr, p = p0 + pp;
    float v = 0.f;
    if (r < R && p < K) v = KCONTIG ? X[p + r * ld] : X[r + p * ld];
    // a row with Inf/NaN is listed once for the FP32 fixup
    if (!isfinite(v) && atomicExch(&flag[r], 1) == 0) list[atomicAdd(count, 1)] = (int)r;
    tile[rr][pp] = v;
  }
  __syncthreads();
  const int rr = tid >> 3, pc = (tid & 7) * 8;
  __align__(16) __nv_bfloat16 h[8], m[8], l[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) split3(tile[rr][pc + j], h[j], m[j], l[j]);
  const int64_t off = (r0 + rr) * Kpad + p0 + pc;
  const int64_t plane = Rpad * Kpad;
  *reinterpret_cast<uint4 *>(dst + off) = *reinterpret_cast<const uint4 *>(h);
  *reinterpret_cast<uint4 *>(dst + plane + off) = *reinterpret_cast<const uint4 *>(m);
  *reinterpret_cast<uint4 *>(dst + 2 * plane + off) = *reinterpret_cast<const uint4 *>(l);
}

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

void split3(bool kcontig, int64_t R, int64_t K, const float *X, int64_t ld, int64_t Rpad,
            int64_t Kpad, __nv_bfloat16 *dst, int *flag, int *list, int *count, cudaStream_t s) {
  dim3 g((unsigned)(Kpad / 64), (unsigned)(Rpad / 32));
  if (kcontig)
    split3_kernel<true><<<g, 256, 0, s>>>(R, K, X, ld, Rpad, Kpad, dst, flag, list, count);
  else
    split3_kernel<false><<<g, 256, 0, s>>>(R, K, X, ld, Rpad, Kpad, dst, flag, list, count);
  count_launch();
}

// Elements of C in a listed row of op(A) or column of op(B) (Inf/NaN
// operands) as plain FP32 dot products, so IEEE special values propagate as
// in an FP32 GEMM (a split Inf would meet the residual terms of the other
// operand with both signs).  Exits at once when nothing is listed.
__global__ void __launch_bounds__(256)
sgemm_fixup_kernel(int64_t m, int64_t n, int64_t k, float alpha, const float *__restrict__ A,
                   int64_t lda, int ta, const float *__restrict__ B, int64_t ldb, int tb,
                   float beta, float *__restrict__ C, int64_t ldc, const int *__restrict__ rflag,
                   const int *__restrict__ rlist, const int *__restrict__ rcount,
                   const int *__restrict__ clist, const int *__restrict__ ccount, int tri,
                   const int *__restrict__ skipf) {
  const int64_t nr = *rcount, nc = *ccount;
  if (nr == 0 && nc == 0) return;
  if (skipf && *skipf) return;
  const int64_t t1 = nr * n, total = t1 + nc * m;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j;
    if (e < t1) {
      i = rlist[e / n];
      j = e % n;
    } else {
      const int64_t e2 = e - t1;
      j = clist[e2 / m];
      i = e2 % m;
      if (rflag[i]) continue;  // done by the row pass
    }
    if ((tri == 1 && i < j) || (tri == 2 && i > j)) continue;  // the other triangle
    float acc = 0.f;
    for (int64_t q = 0; q < k; ++q) {
      const float a = ta ? A[q + i * lda] : A[i + q * lda];
      const float b = tb ? B[j + q * ldb] : B[q + j * ldb];
      acc = fmaf(a, b, acc);
    }
    float *c = C + i + j * ldc;
    *c = beta == 0.f ? alpha * acc : alpha * acc + beta * *c;
  }
}

}  // namespace s3

// C = alpha*op(A)*op(B) + beta*C in FP32 through the bf16x3 tensor-core
// kernel.  Assumes m, n, k > 0.
int sgemm_tc(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha, const float *A,
             int64_t lda, const float *B, int64_t ldb, float beta, float *C, int64_t ldc,
             cudaStream_t s, int tri, const int *skip) {
  using namespace s3;
  if ((m > GEMM_BLOCK_EXTENT || n > GEMM_BLOCK_EXTENT) && tri == 0 && !skip)
    return gemm_over_blocks(ta, tb, m, n, A, lda, B, ldb, C, ldc, GEMM_BLOCK_EXTENT,
                            [&](int64_t mb, int64_t nb, const float *Ai, const float *Bj,
                                float *Cij) {
                              return sgemm_tc(ta, tb, mb, nb, k, alpha, Ai, lda, Bj, ldb, beta,
                                              Cij, ldc, s, 0, nullptr);
                            });
  if (m > GEMM_BLOCK_EXTENT || n > GEMM_BLOCK_EXTENT || k > (int64_t)1 << 24)
    return set_error(GB_ERR_UNSUPPORTED, "sgemm_tc: dimension too large");
  const int64_t m_pad = round_up(m, BM), n_pad = round_up(n, BN), k_pad = round_up(k, BK);
  const size_t a_elems = 3 * (size_t)m_pad * k_pad, b_elems = 3 * (size_t)n_pad * k_pad;
  const size_t a_bytes = (a_elems * 2 + 1023) & ~size_t(1023);
  const size_t b_bytes = (b_elems * 2 + 1023) & ~size_t(1023);
  // flags and counters (zeroed) then the row/column lists
  const size_t nflag = (size_t)m_pad + n_pad + 8;
  Scratch ws(a_bytes + b_bytes + (nflag + m_pad + n_pad) * sizeof(int), s);
  if (!ws.p) return GB_ERR_ALLOC;
  char *base = static_cast<char *>(ws.p);
  __nv_bfloat16 *sa = reinterpret_cast<__nv_bfloat16 *>(base);
  __nv_bfloat16 *sb = reinterpret_cast<__nv_bfloat16 *>(base + a_bytes);
  int *rflag = reinterpret_cast<int *>(base + a_bytes + b_bytes);
  int *cflag = rflag + m_pad;
  int *counts = cflag + n_pad;
  int *rlist = rflag + nflag;
  int *clist = rlist + m_pad;
  GB_CUDA(cudaMemsetAsync(rflag, 0, nflag * sizeof(int), s));
  // op(A) rows are K-contiguous when A is transposed; op(B) columns when B is not
  split3(ta != 0, m, k, A, lda, m_pad, k_pad, sa, rflag, rlist, counts, s);
  split3(tb == 0, n, k, B, ldb, n_pad, k_pad, sb, cflag, clist, counts + 1, s);
  CUtensorMap mapA, mapB;
  int st = make_bf16_kmajor_map(&mapA, sa, 3 * m_pad, k_pad, BK, BM);
  if (st) return st;
  if ((st = make_bf16_kmajor_map(&mapB, sb, 3 * n_pad, k_pad, BK, BN))) return st;
  static PerDeviceOnce attr_once;
  st = attr_once.run(current_device(), [] {
    GB_CUDA(cudaFuncSetAttribute(sgemm_bf16x3_kernel<0, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(sgemm_bf16x3_kernel<0, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(sgemm_bf16x3_kernel<1, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(sgemm_bf16x3_kernel<2, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    return GB_SUCCESS;
  });
  if (st) return st;
  Params p;
  p.m_tiles = (int)(m_pad / BM);
  p.n_tiles = (int)(n_pad / BN);
  p.kblocks = (int)(k_pad / BK);
  p.m_pad = (int)m_pad;
  p.n_pad = (int)n_pad;
  p.m = m;
  p.n = n;
  p.ldc = ldc;
  p.alpha = alpha;
  p.beta = beta;
  p.C = C;
  p.rflag = rflag;
  p.cflag = cflag;
  p.tri = tri;
  p.skip = skip;
  p.status = ctx().d_status;
  const int ntiles = p.m_tiles * p.n_tiles;
  const int grid = ntiles < persistent_ctas() ? ntiles : persistent_ctas();
  {
    ProfileScope prof("sgemm_tc", s);
    if (tri == 1)
      sgemm_bf16x3_kernel<1, true><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(mapA, mapB, p);
    else if (tri == 2)
      sgemm_bf16x3_kernel<2, true><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(mapA, mapB, p);
    else if (beta != 0.f)
      sgemm_bf16x3_kernel<0, true><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(mapA, mapB, p);
    else
      sgemm_bf16x3_kernel<0, false><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(mapA, mapB, p);
    count_launch();
  }
  { sgemm_fixup_kernel<<<sm_count() * 4, 256, 0, s>>>(m, n, k, alpha, A, lda, ta, B, ldb, tb, beta,
                                                     C, ldc, rflag, rlist, counts, clist,
                                                     counts + 1, tri, skip); count_launch(); }
  return check_cuda(cudaGetLastError(), "sgemm_tc");
}

int sgemm_dispatch(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha, const float *A,
                   int64_t lda, const float *B, int64_t ldb, float beta, float *C, int64_t ldc,
                   cudaStream_t s) {
  const int mode = gb_get_sgemm_mode();
  // auto: the split and the 128 x 256 tile grid pay off once the tiles
  // cover the SMs and K is at least one 64-wide block
  const bool big = m >= 1024 && n >= 1024 && k >= 64;
  if (mode == 2 || (mode == 0 && big))
    return sgemm_tc(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
  launch_sgemm_fp32(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
  return check_cuda(cudaGetLastError(), "sgemm launch");
}

}  // namespace gb
