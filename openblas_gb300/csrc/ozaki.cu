// Emulated FP64 GEMM on the bf16 tensor cores (Ozaki splitting).
//
// C = alpha*op(A)*op(B) + beta*C is computed from fixed-point slices:
//   1. split: every row i of op(A) is scaled by 2^-e_i (e_i = exponent of
//      the row's max |a|), truncated to S*8 bits and cut into S signed 8-bit
//      digits A_1..A_S (|digit| <= 255: eight significant bits, exactly
//      representable in bf16); columns of op(B) likewise with exponents f_j.
//      Slices are stored K-contiguous and zero-padded to the tile grid,
//      whatever the caller's transpose and leading dimension.  S = 7 keeps
//      56 bits (FP64-level accuracy) with S(S+1)/2 = 28 products.
//   2. slice GEMM (tcgen05, kind::f16): for each output tile and each level
//      L = s+t (2..S+1, the Ozaki triangle), each product A_s*B_t^T is
//      accumulated in TMEM in FP32 over K-chunks of 256.  With |digit| <=
//      255, every partial sum of a chunk is an integer of magnitude at most
//      256 * 255^2 < 2^24, so the FP32 accumulation is exact; each chunk is
//      drained to int32 registers (exact conversion) and summed per level.
//      A level sum of up to S <= 8 products over K <= 4096 stays below 2^31
//      (8 * 4096 * 255^2 < 2^31); longer K runs as accumulated segments.
//      Level sums are written as int32 planes.
//   3. recombine (FP64): C_ij = alpha * 2^(e_i+f_j) * sum_L P_L,ij 2^(-8L)
//      + beta*C_ij.  Rows/columns holding Inf/NaN fall back to a direct FP64
//      dot product so IEEE special values propagate.
//
// Modular scheme (automatic mode, tiles whose error bound it meets; Ozaki,
// Uchino and Imamura, "Ozaki Scheme II: a GEMM-oriented emulation of
// floating-point matrix multiplication using an integer modular technique"):
//   1. split: row i of op(A) is cut to the t-bit integers
//      A'_ik = sign(a_ik) trunc(|a_ik| 2^(t - e_i)), |A'_ik| < 2^t, column j of
//      op(B) likewise, and each is stored as its symmetric residues modulo
//      14 pairwise coprime odd moduli p_l in [461, 511] (|residue| <= 255,
//      exact in bf16, the same bound as a slice digit).
//   2. residue GEMM: the same tensor-core kernel, one product per modulus
//      (A' mod p_l)(B' mod p_l)^T with exact FP32 chunks and int32 sums,
//      reduced mod p_l in the epilogue: 14 products instead of the 28 of
//      7 digit slices.
//   3. reconstruct: the Chinese remainder theorem gives C' = A'B' exactly
//      (M = prod p_l ~ 2^125.06 > 2 k 2^2t: t = 56 for K segments of 4096),
//      then C_ij = alpha 2^(e_i + f_j - 2t) C'_ij + beta C_ij, rounded once.
//   No product is dropped: the only error is the cut of the operands, so the
//   bound is 2^-t (2^e_i ||b_j||_1 + 2^f_j ||a_i||_1 + 2^-t k 2^(e_i + f_j)).
//
// The slice GEMM is a persistent warp-specialised kernel, one CTA per SM:
// warp 0 issues TMA loads of 128x64 (A) and 256x64 (B) bf16 tiles into a
// 4-stage shared-memory ring, warp 1 issues tcgen05.mma (M=128, N=256,
// K=16) into one of two 256-column TMEM accumulators, and warps 2..9 drain
// the other accumulator (tcgen05.ld), so MMA and drain overlap.  All waits
// are bounded: a role that times out raises an abort flag and the kernel
// winds down, reporting an error status instead of hanging.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "gb_internal.h"
#include "lapack_internal.h"
#include "ozaki_digits.cuh"
#include "sm100_primitives.cuh"
#include "tma_host.h"

namespace gb {

namespace oz {

constexpr int BM = 128, BN = 256, BK = 64;
constexpr int STAGES = 4;
constexpr int DIGIT_BITS = ozd::DIGIT_BITS;  // bits of one slice digit, |digit| <= 255
constexpr unsigned long long DIGIT_MASK = ozd::DIGIT_MASK;
constexpr int KC_BLOCKS = 4;   // K chunk of one exact FP32 accumulation: 256
constexpr int A_BYTES = BM * BK * 2;
constexpr int B_BYTES = BN * BK * 2;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int NUM_THREADS = 320;
constexpr int TMEM_COLS = 512;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int MAX_SLICES = 8;
constexpr int64_t MAX_K_SEGMENT = EMU_K_SEGMENT;   // keeps a level sum below 2^31
// K segment of the automatic mode when the modular scheme is allowed: one
// residue product's int32 sum stays below 2^29; digit-slice tiles run the
// segment as sub-segments of MAX_K_SEGMENT.
constexpr int64_t MOD_K_SEGMENT = 2 * MAX_K_SEGMENT;
static_assert(MOD_K_SEGMENT * 255 * 255 < (1LL << 29), "a residue sum fits the epilogue's reduction");
static_assert(256LL * 255 * 255 < (1LL << 24), "a 256-deep chunk of one product is exact in FP32");
static_assert(8LL * MAX_K_SEGMENT * 255 * 255 < (1LL << 31), "a level sum fits int32");
constexpr uint64_t WAIT_LIMIT_NS = 4000000000ull;
constexpr int NONFINITE = ozd::NONFINITE;  // exponent marker of a row/column with Inf/NaN

// ------------------------------------------------------------ modular scheme
constexpr int MOD_COUNT = 14;       // moduli of the modular scheme
constexpr int MOD_PAIRS = MOD_COUNT / 2;
constexpr int MOD_CHUNK_BITS = 12;  // A' is read in 12-bit chunks to form its residues
constexpr int MOD_CHUNKS = 5;       // 60 bits: t <= 60
constexpr int MOD_MAX_BITS = MOD_CHUNK_BITS * MOD_CHUNKS;
// |chunk sum| < 5 * 4096 * 255 < 2^22.33: exact in FP32, and small enough
// that the rounded quotient below is exact (see split_mod_kernel)
static_assert(4096.0 * 255 * MOD_CHUNKS < 5300000.0, "a residue's chunk sum stays below 2^22.33");

// Constants of the modular scheme for one call (kernel argument).
struct ModTable {
  int bits;                          // t: operands are cut to t-bit integers
  float pf[MOD_COUNT];               // p_l
  float pinv[MOD_COUNT];             // 1 / p_l (rounded)
  float pw[MOD_COUNT][MOD_CHUNKS];   // 2^(12 d) mod p_l, symmetric (|pw| <= (p_l - 1) / 2)
  // The reconstruction pairs the moduli, m_i = a_i b_i with a_i = p_2i,
  // b_i = p_2i+1 (M = prod m_i), and runs the CRT over the seven pairs:
  uint32_t pa[MOD_PAIRS], pb[MOD_PAIRS];
  uint32_t pinv_ab[MOD_PAIRS];       // a_i^-1 mod b_i
  uint32_t pmagic[MOD_PAIRS];        // ceil(2^32 / b_i): u / b_i = umulhi(u, pmagic) for u < 2^20
  uint32_t F[MOD_PAIRS];             // round(2^32 u_i / m_i), u_i = (M / m_i)^-1 mod m_i
  uint32_t W[MOD_PAIRS][4];          // CRT weight (M / m_i) u_i, 32-bit limbs, low first
  uint32_t M[4];                     // M = prod p_l, 32-bit limbs
};

struct GemmParams {
  int S;
  int m_tiles, n_tiles;
  int group_m;  // m-tiles per group of the tile order
  int tri;      // 0 all tiles; 1 only tiles meeting i >= j; 2 only tiles meeting i <= j
  int kblocks;
  int kblock0;  // first K block of the operands' tensor maps this launch reads
  int m_pad, n_pad;
  int b_rows;  // rows of one slice (residue) plane of the op(B) operand
  int64_t plane_stride;
  int *planes;
  int *status;
  // Digit slices: per n-tile slice count (automatic mode; 0 = a modular
  // tile, skipped), or null: S everywhere.  Modular: the tiles with
  // s_tiles[nt] == 0 (all when null) take part.
  const int *s_tiles;
  const int *run_if;   // when non-null and *run_if == 0 the launch does nothing
  // Work units: (tile, level group); a tile's levels are split into
  // level_groups consecutive ranges of about equal product counts, each
  // computed by its own CTA (more CTAs than tiles for small products: the
  // levels write separate planes).
  int level_groups;
  int mod_p[MOD_COUNT];          // moduli (modular scheme)
  uint32_t mod_magic[MOD_COUNT];  // ceil(2^40 / p_l): u / p_l = umulhi(u, magic) >> 8 for u < 2^31
};

// Products of one output tile, in levels that share an accumulation: digit
// slices have levels L = s + t = 2..S+1 (the Ozaki triangle) holding the
// pairs (s, L - s); the modular scheme has one level per modulus holding
// its residue product.  Slice indices are 0-based here.
template <bool MOD>
__device__ __forceinline__ int tile_levels(int nt, const GemmParams &p) {
  if (MOD) return (!p.s_tiles || p.s_tiles[nt] == 0) ? MOD_COUNT : 0;
  return p.s_tiles ? p.s_tiles[nt] : p.S;
}
template <bool MOD>
__device__ __forceinline__ void level_products(int l, int nl, int &lo, int &hi) {
  if (MOD) {
    lo = hi = l;
    return;
  }
  const int L = l + 2;
  lo = L - nl > 1 ? L - nl : 1;
  hi = L - 1 < nl ? L - 1 : nl;
}
template <bool MOD>
__device__ __forceinline__ void product_slices(int l, int s, int &sa, int &sb) {
  if (MOD) {
    sa = sb = l;
    return;
  }
  sa = s - 1;
  sb = l + 1 - s;  // t - 1 with t = L - s, L = l + 2
}

// Levels [l0, l1) of level group g of a tile with nl levels: equal shares
// of the moduli, or of the digit-slice products (level l has l + 1).
template <bool MOD>
__device__ __forceinline__ void group_levels(int nl, int g, int groups, int &l0, int &l1) {
  if (MOD) {
    l0 = g * nl / groups;
    l1 = (g + 1) * nl / groups;
    return;
  }
  const int total = nl * (nl + 1) / 2;
  const int t0 = (g * total + groups / 2) / groups, t1 = ((g + 1) * total + groups / 2) / groups;
  l0 = l1 = 0;
  for (int l = 0, cum = 0; l < nl; cum += ++l) {  // cum: products of the levels before l
    if (cum < t0) l0 = l + 1;
    if (cum < t1) l1 = l + 1;
  }
}

// Tile order: groups of group_m m-tiles, walked column by column inside a
// group, so the tiles resident at one time cover a near-square block of C
// and their A and B panels are shared through L2 (a plain m-fastest order
// puts every m-tile of a few columns in flight and re-reads A from HBM).
__device__ __forceinline__ void tile_coords(int tile, const GemmParams &p, int &mt, int &nt) {
  const int span = p.group_m * p.n_tiles;
  const int first_m = (tile / span) * p.group_m;
  const int rem = p.m_tiles - first_m;
  const int gm = rem < p.group_m ? rem : p.group_m;
  const int in = tile % span;
  mt = first_m + in % gm;
  nt = in / gm;
}

// A tile takes part unless it lies entirely in the triangle the caller
// leaves alone (triangular output of a SYRK-shaped update).
__device__ __forceinline__ bool tile_active(int mt, int nt, const GemmParams &p) {
  if (p.tri == 1) return mt * BM + BM - 1 >= nt * BN;  // some i >= j
  if (p.tri == 2) return mt * BM <= nt * BN + BN - 1;  // some i <= j
  return true;
}

template <bool MOD>
__global__ void __launch_bounds__(NUM_THREADS, 1)
slice_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ GemmParams p) {
  using namespace sm100;
  if (p.run_if && *p.run_if == 0) return;  // every thread reads the same word
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *sA = smem;
  uint8_t *sB = smem + STAGES * A_BYTES;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *tfull = empty + STAGES;
  uint64_t *tempty = tfull + 2;
  uint64_t *mma_done = tempty + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
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

  const int nunits = p.m_tiles * p.n_tiles * p.level_groups;
  const int nkc = (p.kblocks + KC_BLOCKS - 1) / KC_BLOCKS;
  auto fail = [&](int site) {
    *abort_flag = 1;
    atomicCAS(p.status, 0, GB_KERR_MBARRIER_TIMEOUT);
    atomicExch(p.status + 1, site);
  };

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      int stage = 0;
      uint32_t phase = 0;
      uint32_t issued_phase[STAGES];
      bool issued[STAGES];
      for (int i = 0; i < STAGES; ++i) issued[i] = false;
      bool ok = true;
      for (int w = blockIdx.x; ok && w < nunits; w += gridDim.x) {
        int mt, nt, l0, l1;
        tile_coords(w / p.level_groups, p, mt, nt);
        if (!tile_active(mt, nt, p)) continue;
        const int nl = tile_levels<MOD>(nt, p);
        group_levels<MOD>(nl, w % p.level_groups, p.level_groups, l0, l1);
        for (int l = l0; ok && l < l1; ++l) {
          int s_lo, s_hi;
          level_products<MOD>(l, nl, s_lo, s_hi);
          for (int s = s_lo; ok && s <= s_hi; ++s) {
            int sa, sb;
            product_slices<MOD>(l, s, sa, sb);
            const int rowA = sa * p.m_pad + mt * BM;
            const int rowB = sb * p.b_rows + nt * BN;
            for (int kc = 0; ok && kc < nkc; ++kc) {
              const int kb1 = min(p.kblocks, (kc + 1) * KC_BLOCKS);
              for (int kb = kc * KC_BLOCKS; kb < kb1; ++kb) {
                if (!mbar_wait(&empty[stage], phase ^ 1u, abort_flag, WAIT_LIMIT_NS)) {
                  fail(1);
                  ok = false;
                  break;
                }
                mbar_arrive_expect_tx(&full[stage], STAGE_BYTES);
                tma_load_2d(sA + stage * A_BYTES, &tmA, &full[stage], (p.kblock0 + kb) * BK, rowA);
                tma_load_2d(sB + stage * B_BYTES, &tmB, &full[stage], (p.kblock0 + kb) * BK, rowB);
                issued[stage] = true;
                issued_phase[stage] = phase;
                if (++stage == STAGES) {
                  stage = 0;
                  phase ^= 1u;
                }
              }
            }
          }
        }
      }
      // never leave with TMA writes still landing in shared memory
      volatile int no_abort = 0;
      for (int i = 0; i < STAGES; ++i)
        if (issued[i]) mbar_wait(&full[i], issued_phase[i], &no_abort, WAIT_LIMIT_NS);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t IDESC = idesc_bf16_f32(BM, BN);
      int stage = 0;
      uint32_t phase = 0;
      int acc = 0;
      uint32_t acc_phase = 0;
      bool ok = true;
      for (int w = blockIdx.x; ok && w < nunits; w += gridDim.x) {
        int mt, nt, l0, l1;
        tile_coords(w / p.level_groups, p, mt, nt);
        if (!tile_active(mt, nt, p)) continue;
        const int nl = tile_levels<MOD>(nt, p);
        group_levels<MOD>(nl, w % p.level_groups, p.level_groups, l0, l1);
        for (int l = l0; ok && l < l1; ++l) {
          int s_lo, s_hi;
          level_products<MOD>(l, nl, s_lo, s_hi);
          for (int s = s_lo; ok && s <= s_hi; ++s) {
            for (int kc = 0; ok && kc < nkc; ++kc) {
              if (!mbar_wait(&tempty[acc], acc_phase ^ 1u, abort_flag, WAIT_LIMIT_NS)) {
                fail(2);
                ok = false;
                break;
              }
              tc_fence_after();
              const uint32_t d_tmem = tmem_base + (uint32_t)(acc * BN);
              const int kb0 = kc * KC_BLOCKS, kb1 = min(p.kblocks, kb0 + KC_BLOCKS);
              for (int kb = kb0; kb < kb1; ++kb) {
                if (!mbar_wait(&full[stage], phase, abort_flag, WAIT_LIMIT_NS)) {
                  fail(3);
                  ok = false;
                  break;
                }
                tc_fence_after();
                const uint64_t adesc = sdesc_kmajor_sw128(smem_u32(sA + stage * A_BYTES));
                const uint64_t bdesc = sdesc_kmajor_sw128(smem_u32(sB + stage * B_BYTES));
#pragma unroll
                for (int k = 0; k < BK / 16; ++k) {
                  // advance 16 bf16 (32 bytes) along K inside the swizzle atom
                  mma_bf16(d_tmem, adesc + (uint64_t)(2 * k), bdesc + (uint64_t)(2 * k), IDESC,
                           (kb > kb0 || k > 0) ? 1u : 0u);
                }
                mma_commit(&empty[stage]);
                if (++stage == STAGES) {
                  stage = 0;
                  phase ^= 1u;
                }
              }
              if (!ok) break;
              mma_commit(&tfull[acc]);
              acc ^= 1;
              if (acc == 0) acc_phase ^= 1u;
            }
          }
        }
      }
      // TMEM is freed at exit: wait until every issued MMA has completed
      mma_commit(mma_done);
      volatile int no_abort = 0;
      mbar_wait(mma_done, 0, &no_abort, WAIT_LIMIT_NS);
    }
  } else {
    // ------------------------------------------------ epilogue (8 warps)
    const int q = warp & 3;             // TMEM lane quadrant this warp may access
    const int half = (warp - 2) >> 2;   // column half of the 256-wide tile
    const int row = q * 32 + lane;      // tile row owned by this thread
    int acc = 0;
    uint32_t acc_phase = 0;
    bool ok = true;
    int32_t sum[128];
    for (int w = blockIdx.x; ok && w < nunits; w += gridDim.x) {
      int mt, nt, l0, l1;
      tile_coords(w / p.level_groups, p, mt, nt);
      if (!tile_active(mt, nt, p)) continue;
      const int nl = tile_levels<MOD>(nt, p);
      group_levels<MOD>(nl, w % p.level_groups, p.level_groups, l0, l1);
      const int64_t plane_tile = (int64_t)nt * p.m_tiles + mt;
      for (int l = l0; ok && l < l1; ++l) {
#pragma unroll
        for (int c = 0; c < 128; ++c) sum[c] = 0;
        int s_lo, s_hi;
        level_products<MOD>(l, nl, s_lo, s_hi);
        for (int s = s_lo; ok && s <= s_hi; ++s) {
          for (int kc = 0; kc < nkc; ++kc) {
            const bool got = mbar_wait(&tfull[acc], acc_phase, abort_flag, WAIT_LIMIT_NS);
            // the warp-wide tcgen05.ld below needs a converged warp: agree first
            if (!__all_sync(0xffffffffu, got)) {
              if (lane == 0) fail(4);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t taddr =
                tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + half * 128);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              uint32_t r[32];
              tmem_ld_32x32b_x32(taddr + c * 32, r);
              tmem_ld_wait();
#pragma unroll
              for (int j = 0; j < 32; ++j) sum[c * 32 + j] += __float2int_rn(__uint_as_float(r[j]));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
            acc ^= 1;
            if (acc == 0) acc_phase ^= 1u;
          }
        }
        if (!ok) break;
        // level plane, tile-blocked and column-major inside the tile so a
        // warp's store of one column is contiguous
        const int64_t at = (int64_t)l * p.plane_stride + plane_tile * (BM * BN) +
                           (int64_t)(half * 128) * BM + row;
        if (MOD) {
          // residue of the product modulo p_l, in [0, p_l), as 16 bits:
          // u = sum + p_l 2^21 is positive and below 2^31 (|sum| < 2^29), and
          // with magic = ceil(2^40 / p_l) the quotient umulhi(u, magic) >> 8
          // is exact (u * (magic - 2^40 / p_l) / 2^40 < 2^-9 < 1 / p_l)
          const uint32_t pm = (uint32_t)p.mod_p[l], magic = p.mod_magic[l];
          const uint32_t off = pm << 21;
          uint16_t *dst = reinterpret_cast<uint16_t *>(p.planes) + at;
#pragma unroll
          for (int c = 0; c < 128; ++c) {
            const uint32_t u = (uint32_t)sum[c] + off;
            const uint32_t q = __umulhi(u, magic) >> 8;
            dst[c * BM] = (uint16_t)(u - q * pm);
          }
        } else {
          int *dst = p.planes + at;
#pragma unroll
          for (int c = 0; c < 128; ++c) dst[c * BM] = sum[c];
        }
      }
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

// ------------------------------------------------------------------ split
// Max |x| over each row of the op-view R x K (src(r,p)).  Bits of
// non-negative doubles order like the values, so atomicMax on the bit
// pattern is a max; any NaN wins as the largest pattern.
__global__ void rowmax_kcontig_kernel(int64_t R, int64_t K, const double *__restrict__ X,
                                      int64_t ld, unsigned long long *__restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= R) return;
  const double *x = X + r * ld;
  unsigned long long best = 0;
#pragma unroll 8
  for (int64_t pp = lane; pp < K; pp += 32) {
    unsigned long long b = __double_as_longlong(fabs(x[pp]));
    best = b > best ? b : best;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_down_sync(0xffffffffu, best, off);
    best = o > best ? o : best;
  }
  if (lane == 0) atomicMax(out + r, best);
}

__global__ void rowmax_mcontig_kernel(int64_t R, int64_t K, const double *__restrict__ X,
                                      int64_t ld, int64_t kspan,
                                      unsigned long long *__restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int64_t p0 = (int64_t)blockIdx.y * kspan;
  const int64_t p1 = p0 + kspan < K ? p0 + kspan : K;
  unsigned long long best = 0;
#pragma unroll 8
  for (int64_t pp = p0; pp < p1; ++pp) {
    unsigned long long b = __double_as_longlong(fabs(X[r + pp * ld]));
    best = b > best ? b : best;
  }
  atomicMax(out + r, best);
}

// ------------------------------------------------------------- slice choice
// Automatic slice count (caller-facing GEMMs with no fixed count).  For one
// K segment of length k, truncating row i of op(A) to S digits below 2^e_i
// and column j of op(B) below 2^f_j, and dropping the products of levels
// s + t >= S + 2, bounds the error of every C(i,j) by
//   2^-8S (2^e_i ||b_j||_1 + 2^f_j ||a_i||_1 + c k 2^(e_i + f_j)),
// c = (S - 1)(1 + 2^-7) <= 7.06 (at most S - 1 dropped pairs per level, each
// below 2^16 of the level's unit, and a geometric tail), plus the final
// roundings.  Summed over the rows of column j and set against that column's
// sum of |A||B|, w_j = sum_k alpha_k |b_kj| with alpha_k = sum_i |a_ik|, the
// ratio is 2^-8S rho_j with
//   rho_j = (T_e ||b_j||_1 + 2^f_j (T_1 + c k T_e)) / w_j,
// T_e = sum_i 2^e_i (over non-zero finite rows), T_1 = sum_k alpha_k.  Every
// 256-column tile of C gets the smallest S whose 2^-8S max rho_j + (nseg + 2)
// 2^-53 stays within the tolerance (GB_OZAKI_TOL, in units of 2^-52).  Rows and
// columns with Inf/NaN are recomputed directly and left out.  A ratio that is
// not finite (operands near the overflow or underflow threshold) gets the
// largest count.  Digits are prefix-consistent (the first S digits of an
// S'-digit split, S < S', are the S-digit split), so op(A) is split once with
// MAX_SLICES digits and every tile uses the first S of them.
constexpr double DROP_C = 7.0 * (1.0 + 1.0 / 128.0);

// The statistics run in FP32 (FP64 is the scarcest unit on this part):
// every |x| is scaled by a power of two that puts it below 1 (the largest
// row exponent of op(A) for alpha_k, the column's own exponent for op(B)),
// truncated to FP32 (|x| 2^-e below FP32's normal range counts as 0) and
// summed in FP32.  Each sum is then within 2^-12 relative of its exact value
// (24-bit truncation; at most 256 terms summed in one register, then a tree
// or an atomic reduction of at most 2^12 partial sums), less the dropped
// values, each below 2^-126 of the largest.  The choice multiplies every
// ratio by RHO_SLACK = 1 + 2^-8, which covers both.
constexpr double RHO_SLACK = 1.0 + 1.0 / 256.0;

// |x| 2^-e as FP32, truncated (|x| < 2^(e + 1) assumed), 0 below 2^-126.
__device__ __forceinline__ float scaled_abs(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  int E = (int)(b >> 52);
  unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  if (E == 0) {  // subnormal double: normalise
    if (mant == 0) return 0.0f;
    const int top = 63 - __clzll((long long)mant);  // value = 1.f 2^(top - 1074)
    mant = (mant << (52 - top)) & 0xFFFFFFFFFFFFFull;
    E = top - 51;
  }
  const int fe = E - 1023 - e + 127;
  if (fe <= 0) return 0.0f;
  return __uint_as_float(((unsigned)fe << 23) | (unsigned)(mant >> 29));
}

// alpha_k 2^-E_A in FP32, E_A = *emax (the largest row exponent of op(A)),
// summed over the finite rows r of op(A) (R x K view) of |x_rk|.  KCONTIG
// (op(A) row r is K-contiguous): a thread per k, a chunk of rows per
// blockIdx.y.  Otherwise a block per k, the rows read down the column.
template <bool KCONTIG>
__global__ void __launch_bounds__(256)
abs_colsum_kernel(int64_t R, int64_t K, const double *__restrict__ X, int64_t ld,
                  const int *__restrict__ expo, const int *__restrict__ emax, int64_t rspan,
                  float *__restrict__ alpha) {
  const int ea = *emax;
  if (KCONTIG) {
    const int64_t kk = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= K) return;
    const int64_t r0 = (int64_t)blockIdx.y * rspan;
    const int64_t r1 = r0 + rspan < R ? r0 + rspan : R;
    float s = 0.0f;
    for (int64_t r = r0; r < r1; ++r)
      if (expo[r] != NONFINITE) s += scaled_abs(X[kk + r * ld], ea);
    atomicAdd(alpha + kk, s);
  } else {
    const int64_t kk = blockIdx.x;
    const int64_t r0 = (int64_t)blockIdx.y * rspan;
    const int64_t r1 = r0 + rspan < R ? r0 + rspan : R;
    float s = 0.0f;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
      if (expo[r] != NONFINITE) s += scaled_abs(X[r + kk * ld], ea);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.0f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
      atomicAdd(alpha + kk, t);
    }
  }
}

// x 2^n, equal to ldexp(x, n): when 2^n is a normal double, one multiply by
// it (the exact product rounded once, as ldexp rounds it, overflow to Inf
// included); otherwise ldexp.  The statistics and choice kernels run short
// chains of these, where ldexp's general path was most of their latency.
__device__ __forceinline__ double scale2(double x, int n) {
  if (n >= -1022 && n <= 1023) return x * __longlong_as_double((long long)(n + 1023) << 52);
  return ldexp(x, n);
}

// totals[0] = T_e = sum of 2^e_r over the non-zero finite rows of op(A),
// totals[1] = T_1 = sum_k alpha_k, totals[2] = E_A (the scale of the FP32
// alpha_k).  One block.
__global__ void __launch_bounds__(256)
a_totals_kernel(int64_t R, int64_t K, const int *__restrict__ expo,
                const unsigned long long *__restrict__ mx, const float *__restrict__ alpha,
                const int *__restrict__ emax, double *__restrict__ totals) {
  double te = 0.0, t1 = 0.0;
  for (int64_t r = threadIdx.x; r < R; r += blockDim.x)
    if (mx[r] != 0 && expo[r] != NONFINITE) te += scale2(1.0, expo[r]);
  for (int64_t kk = threadIdx.x; kk < K; kk += blockDim.x) t1 += (double)alpha[kk];
  __shared__ double pe[256], p1[256];
  pe[threadIdx.x] = te;
  p1[threadIdx.x] = t1;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      pe[threadIdx.x] += pe[threadIdx.x + h];
      p1[threadIdx.x] += p1[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    totals[0] = pe[0];
    totals[1] = scale2(p1[0], *emax);
    totals[2] = (double)*emax;
  }
}

// op(B)'s R x K view (R = columns of op(B)), a warp per column, one read:
// the column maximum and exponent f_j, and the column sums
// s1_j 2^-f_j = sum_k |b_kj| 2^-f_j and s2_j 2^-(f_j + E_A) =
// sum_k (alpha_k 2^-E_A)(|b_kj| 2^-f_j) in FP32.  Each lane scales by the
// exponent of its own running maximum and rescales its partial sums by a
// power of two when that grows, and by 2^(f_lane - f_j) at the end; FP32
// rounding commutes with power-of-two scaling, so the sums are those of
// scaling by f_j throughout except for terms below 2^-126 of the maximum
// (counted as dropped in the error bound either way).  Rows R..Rpad-1 get
// exponent 0 and zero sums.
__device__ __forceinline__ float pow2f(int d) {  // 2^d for d <= 0; 0 below FP32's normal range
  return d < -126 ? 0.0f : __int_as_float((127 + d) << 23);
}
__global__ void col_stats_kcontig_kernel(int64_t R, int64_t Rpad, int64_t K,
                                         const double *__restrict__ X, int64_t ld,
                                         const float *__restrict__ alpha,
                                         unsigned long long *__restrict__ out,
                                         int *__restrict__ expo, float *__restrict__ s1,
                                         float *__restrict__ s2) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= Rpad) return;
  if (r >= R) {
    if (lane == 0) {
      out[r] = 0;
      expo[r] = 0;
      s1[r] = s2[r] = 0.0f;
    }
    return;
  }
  const double *x = X + r * ld;
  unsigned long long best = 0;
  int fl = 0;  // exponent of this lane's running maximum (while best != 0)
  float a1 = 0.0f, a2 = 0.0f;
#pragma unroll 4
  for (int64_t pp = lane; pp < K; pp += 32) {
    const double xv = x[pp];
    const unsigned long long b = (unsigned long long)__double_as_longlong(xv) &
                                 0x7FFFFFFFFFFFFFFFull;
    if (b > best) {
      const int fn = ozd::exponent_of_max(b);
      if (best != 0 && fn != NONFINITE && fl != NONFINITE && fn != fl) {
        const float sc = pow2f(fl - fn);
        a1 *= sc;
        a2 *= sc;
      }
      best = b;
      fl = fn;
    }
    if (fl != NONFINITE) {
      const float v = scaled_abs(xv, fl);
      a1 += v;
      a2 = fmaf(alpha[pp], v, a2);
    }
  }
  unsigned long long wbest = best;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, wbest, off);
    wbest = o > wbest ? o : wbest;
  }
  const int f = ozd::exponent_of_max(wbest);
  if (wbest != 0 && f != NONFINITE) {
    const float sc = best != 0 ? pow2f(fl - f) : 0.0f;  // fl <= f
    a1 *= sc;
    a2 *= sc;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      a1 += __shfl_down_sync(0xffffffffu, a1, off);
      a2 += __shfl_down_sync(0xffffffffu, a2, off);
    }
  } else {
    a1 = a2 = 0.0f;
  }
  if (lane == 0) {
    out[r] = wbest;
    expo[r] = f;
    s1[r] = a1;
    s2[r] = a2;
  }
}

// The same sums when op(B)'s columns are strided (B transposed): a thread per
// column and a K span per blockIdx.y, after the column exponents are known.
__global__ void col_stats_mcontig_kernel(int64_t R, int64_t K, const double *__restrict__ X,
                                         int64_t ld, int64_t kspan,
                                         const float *__restrict__ alpha,
                                         const int *__restrict__ expo, float *__restrict__ s1,
                                         float *__restrict__ s2) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int f = expo[r];
  if (f == NONFINITE) return;
  const int64_t p0 = (int64_t)blockIdx.y * kspan;
  const int64_t p1 = p0 + kspan < K ? p0 + kspan : K;
  float a1 = 0.0f, a2 = 0.0f;
#pragma unroll 4
  for (int64_t pp = p0; pp < p1; ++pp) {
    const float v = scaled_abs(X[r + pp * ld], f);
    a1 += v;
    a2 = fmaf(alpha[pp], v, a2);
  }
  atomicAdd(s1 + r, a1);
  atomicAdd(s2 + r, a2);
}

// One block per 256-column tile of C: the tile's largest rho_j (digit
// slices) and rho2_j (modular scheme, t = mod_t bits; 0: not allowed), in
//   rho2_j = (T_e ||b_j||_1 + 2^f_j (T_1 + 2^-t k T_e)) / w_j
// (no dropped products, only the cut of the operands).  The tile takes the
// modular scheme when 2^-t max rho2_j meets budget_mod (s_tiles = 0,
// counted in pass[0], the call's moduli count kept in *last_moduli), else
// the smallest slice count whose bound meets budget_dig (counted in
// pass[1], the largest count of the call kept in *last).  k is the segment:
// the digit-slice bound summed over its sub-segments is the same bound with
// k the whole segment; the budgets differ by the roundings of the segment
// and sub-segment accumulations.
__global__ void __launch_bounds__(256)
choose_slices_kernel(int64_t R, const int *__restrict__ expo,
                     const unsigned long long *__restrict__ mx, const float *__restrict__ s1f,
                     const float *__restrict__ s2f, const double *__restrict__ totals, int64_t k,
                     double budget_mod, double budget_dig, int mod_t, int *__restrict__ s_tiles,
                     int *__restrict__ last,
                     int *__restrict__ last_moduli, int *__restrict__ pass) {
  const int64_t j = (int64_t)blockIdx.x * BN + threadIdx.x;
  double rho = 0.0, rho2 = 0.0;
  if (j < R && mx[j] != 0 && expo[j] != NONFINITE && s2f[j] > 0.0f) {
    const double te = totals[0], t1 = totals[1];
    const int fj = expo[j], ea = (int)totals[2];
    const double s1 = scale2((double)s1f[j], fj), s2 = scale2((double)s2f[j], fj + ea);
    rho = RHO_SLACK * (te * s1 + scale2(t1 + DROP_C * (double)k * te, fj)) / s2;
    rho2 = RHO_SLACK * (te * s1 + scale2(t1 + scale2((double)k * te, -mod_t), fj)) / s2;
    if (!(rho <= 1e300)) rho = 1e300;  // Inf or NaN: the largest count
    if (!(rho2 <= 1e300)) rho2 = 1e300;
  } else if (j < R && mx[j] != 0 && expo[j] != NONFINITE) {
    rho = rho2 = 1e300;  // every product of the column too small for the FP32 sums
  }
  __shared__ double red[256], red2[256];
  red[threadIdx.x] = rho;
  red2[threadIdx.x] = rho2;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
      red2[threadIdx.x] = fmax(red2[threadIdx.x], red2[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (mod_t > 0 && scale2(red2[0], -mod_t) <= budget_mod) {
      s_tiles[blockIdx.x] = 0;
      atomicAdd(pass, 1);
      atomicMax(last_moduli, MOD_COUNT);
      return;
    }
    int S = MAX_SLICES;
    for (int c = 1; c < MAX_SLICES; ++c)
      if (scale2(red[0], -DIGIT_BITS * c) <= budget_dig) {
        S = c;
        break;
      }
    s_tiles[blockIdx.x] = S;
    atomicAdd(pass + 1, 1);
    atomicMax(last, S);
  }
}

// Row exponents (|x| < 2^e on the row); with emax, also their maximum over
// the non-zero finite rows (emax preset to a large negative value).
__global__ void exponent_kernel(int64_t Rpad, int64_t R, const unsigned long long *__restrict__ mx,
                                int *__restrict__ expo, int *__restrict__ emax) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= Rpad) return;
  const int e = r < R ? ozd::exponent_of_max(mx[r]) : 0;
  expo[r] = e;
  if (emax && r < R && mx[r] != 0 && e != NONFINITE) atomicMax(emax, e);
}

// Digits of a 32-row x 64-K tile.  The tile is staged through shared memory
// so both the read (in the caller's layout) and the write (K-contiguous
// slices) are coalesced.
template <bool KCONTIG>
__global__ void __launch_bounds__(256)
split_kernel(int64_t R, int64_t K, const double *__restrict__ X, int64_t ld,
             const int *__restrict__ expo, int S, int64_t Rpad, int64_t Kpad,
             __nv_bfloat16 *__restrict__ slices, const int *__restrict__ s_tiles,
             const int *__restrict__ run_if) {
  __shared__ double tile[32][65];
  if (run_if && *run_if == 0) return;
  // a grid-stride loop over the tiles (see split_grid)
  const int64_t tiles_x = Kpad / 64, ntiles = tiles_x * (Rpad / 32);
  for (int64_t tid_t = blockIdx.x; tid_t < ntiles; tid_t += gridDim.x) {
  const int64_t r0 = (tid_t / tiles_x) * 32, p0 = (tid_t % tiles_x) * 64;
  // the slice count of this 256-row tile (automatic mode); 0: a modular tile
  const int St = s_tiles ? s_tiles[r0 / BN] : S;
  if (St == 0) continue;
  const int tid = threadIdx.x;
  // all eight loads of a thread in flight before the shared-memory stores
  double vin[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int e = tid + 256 * u;
    const int rr = KCONTIG ? e / 64 : e % 32, pp = KCONTIG ? e % 64 : e / 32;
    const int64_t r = r0 + rr, pk = p0 + pp;
    vin[u] = (r < R && pk < K) ? (KCONTIG ? X[pk + r * ld] : X[r + pk * ld]) : 0.0;
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int e = tid + 256 * u;
    const int rr = KCONTIG ? e / 64 : e % 32, pp = KCONTIG ? e % 64 : e / 32;
    tile[rr][pp] = vin[u];
  }
  __syncthreads();
  // each thread: row rr = tid / 8, 8 consecutive k values.  The fixed-point
  // value trunc(|x| * 2^(8S - e)) (< 2^64 for S <= 8) is taken straight from the IEEE bits
  // (mantissa shifted by the exponent difference): integer work only, as
  // FP64 arithmetic is the scarcest unit on this part.
  const int rr = tid >> 3, pc = (tid & 7) * 8;
  const int64_t r = r0 + rr;
  const int e = (r < R) ? expo[r] : 0;
  unsigned long long mag[8];
  bool neg[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) mag[j] = ozd::digit_magnitude(tile[rr][pc + j], e, St, neg[j]);
  for (int s = 1; s <= St; ++s) {
    const int sh = DIGIT_BITS * (St - s);
    __align__(16) __nv_bfloat16 out[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int d = (int)((mag[j] >> sh) & DIGIT_MASK);
      out[j] = __float2bfloat16_rn((float)(neg[j] ? -d : d));
    }
    __nv_bfloat16 *dst = slices + ((int64_t)(s - 1) * Rpad + r) * Kpad + p0 + pc;
    *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(out);
  }
  __syncthreads();  // the tile buffer is refilled by the next iteration
  }
}

// Residues of a 32-row x 64-K tile for the modular scheme: the t-bit
// integer A' = sign(x) trunc(|x| 2^(t - e)) is read in five signed 12-bit
// chunks c_d, and x = sum_d c_d w_d with w_d = 2^(12 d) mod p_l in the
// symmetric range is formed in FP32 (|x| < 2^22.33, every partial sum an
// exact integer).  The residue is x - q p_l with q = round(x fl(1/p_l)):
// |x fl(1/p_l) - x / p_l| <= 2^22.33 2^-33 = 2^-10.67, below the distance
// 1 / (2 p_l) >= 2^-10 from x / p_l to the nearest half-integer (p_l odd),
// so q is the exact nearest quotient and the residue lies in
// [-(p_l - 1)/2, (p_l - 1)/2].  Residue planes share the slices' layout.
// For op(B) (s_tiles non-null) only the rows of modular tiles are written.
template <bool KCONTIG>
__global__ void __launch_bounds__(256)
split_mod_kernel(int64_t R, int64_t K, const double *__restrict__ X, int64_t ld,
                 const int *__restrict__ expo, int64_t Rpad, int64_t Kpad,
                 __nv_bfloat16 *__restrict__ res, const int *__restrict__ s_tiles,
                 const int *__restrict__ run_if, const __grid_constant__ ModTable tab) {
  __shared__ double tile[32][65];
  if (run_if && *run_if == 0) return;
  const int64_t r0 = (int64_t)blockIdx.y * 32, p0 = (int64_t)blockIdx.x * 64;
  if (s_tiles && s_tiles[r0 / BN] != 0) return;  // a digit-slice tile
  const int tid = threadIdx.x;
  double vin[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int e = tid + 256 * u;
    const int rr = KCONTIG ? e / 64 : e % 32, pp = KCONTIG ? e % 64 : e / 32;
    const int64_t r = r0 + rr, pk = p0 + pp;
    vin[u] = (r < R && pk < K) ? (KCONTIG ? X[pk + r * ld] : X[r + pk * ld]) : 0.0;
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int e = tid + 256 * u;
    const int rr = KCONTIG ? e / 64 : e % 32, pp = KCONTIG ? e % 64 : e / 32;
    tile[rr][pp] = vin[u];
  }
  __syncthreads();
  const int rr = tid >> 3, pc = (tid & 7) * 8;
  const int64_t r = r0 + rr;
  const int e = (r < R) ? expo[r] : 0;
  // the chunks of sign(x) |A'| as signed floats (the residue of -A' is minus
  // the residue of A': no modulus is even, so no quotient is a tie)
  float ch[8][MOD_CHUNKS];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    bool neg;
    const unsigned long long mag = ozd::fixed_magnitude(tile[rr][pc + j], e, tab.bits, neg);
    const unsigned sgn = neg ? 0x80000000u : 0u;
#pragma unroll
    for (int d = 0; d < MOD_CHUNKS; ++d) {
      // exact int -> float of a 12-bit value: 2^23 + c, less 2^23
      const unsigned c = (unsigned)(mag >> (MOD_CHUNK_BITS * d)) & ((1u << MOD_CHUNK_BITS) - 1);
      ch[j][d] = __uint_as_float(sgn ^ __float_as_uint(__uint_as_float(0x4B000000u | c) -
                                                       8388608.0f));
    }
  }
  constexpr float ROUND = 12582912.0f;  // 1.5 * 2^23: adding it rounds |y| < 2^22 to an integer
#pragma unroll 2
  for (int l = 0; l < MOD_COUNT; ++l) {
    const float pl = tab.pf[l], pinv = tab.pinv[l];
    __align__(16) __nv_bfloat162 out[4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      float v[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float x = 0.0f;
#pragma unroll
        for (int d = 0; d < MOD_CHUNKS; ++d) x = fmaf(ch[j + h][d], tab.pw[l][d], x);
        const float q = fmaf(x, pinv, ROUND) - ROUND;  // the nearest quotient, exactly
        v[h] = fmaf(-q, pl, x);  // exact: both terms are integers below 2^24
      }
      out[j >> 1] = __floats2bfloat162_rn(v[0], v[1]);
    }
    __nv_bfloat16 *dst = res + ((int64_t)l * Rpad + r) * Kpad + p0 + pc;
    *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(out);
  }
}

// ------------------------------------------------------------------ recombine
// One element of C from its exact level sum: ozd::level_value.
using ozd::level_value;

// Recombine, one CTA per 128 x 256 tile of C (the plane tile layout): every
// level plane of the tile is one contiguous 128 KB run, read with 16-byte
// loads (a lane takes 4 consecutive rows of a column), and the shifts of the
// level sum are compile-time (S is a template argument).  Rows/columns with
// Inf/NaN use a direct FP64 dot product so IEEE special values propagate.
template <int S>
__device__ __forceinline__ void
recombine_tile(int64_t m, int64_t n, int m_tiles, int64_t plane_stride,
               const int *__restrict__ planes, const int *__restrict__ ea,
               const int *__restrict__ eb, double alpha, double beta,
               double *__restrict__ C, int64_t ldc, int ta, int tb, int64_t k,
               const double *__restrict__ A, int64_t lda, const double *__restrict__ B,
               int64_t ldb, int tri) {
  const int mt = blockIdx.x, nt = blockIdx.y;
  const int64_t i0 = (int64_t)mt * BM, j0 = (int64_t)nt * BN;
  if (tri == 1 && i0 + BM - 1 < j0) return;  // tile wholly in the other triangle
  if (tri == 2 && i0 > j0 + BN - 1) return;
  const int tid = threadIdx.x;
  const int il = (tid & 31) * 4, jb = tid >> 5;
  const int *pt = planes + ((int64_t)nt * m_tiles + mt) * (BM * BN);
  int e_i[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) e_i[r] = (i0 + il + r < m) ? ea[i0 + il + r] : 0;
  // grid z splits the tile's columns into chunks (more CTAs for small C)
  const int chunk = BN / (int)gridDim.z, jz0 = (int)blockIdx.z * chunk;
  for (int jl = jz0 + jb; jl < jz0 + chunk; jl += 8) {
    const int64_t j = j0 + jl;
    if (j >= n) break;
    const int fj = eb[j];
    int4 P[S];
#pragma unroll
    for (int L = 0; L < S; ++L)
      P[L] = *reinterpret_cast<const int4 *>(pt + (int64_t)L * plane_stride + jl * BM + il);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int64_t i = i0 + il + r;
      if (i >= m) continue;
      if ((tri == 1 && i < j) || (tri == 2 && i > j)) continue;  // the other triangle
      double v;
      if (e_i[r] == NONFINITE || fj == NONFINITE) {
        double sum = 0.0;
        for (int64_t pp = 0; pp < k; ++pp) {
          const double a = ta ? A[pp + i * lda] : A[i + pp * lda];
          const double b = tb ? B[j + pp * ldb] : B[pp + j * ldb];
          sum = fma(a, b, sum);
        }
        v = alpha * sum;
      } else {
        __int128 acc = 0;
#pragma unroll
        for (int L = 0; L < S; ++L) {
          const int pv = r == 0 ? P[L].x : r == 1 ? P[L].y : r == 2 ? P[L].z : P[L].w;
          acc += (__int128)pv << (DIGIT_BITS * (S - 1 - L));  // level L+2: 2^(8(S+1-(L+2)))
        }
        v = level_value(acc, S, e_i[r], fj, alpha);
      }
      double *c = C + i + j * ldc;
      *c = (beta == 0.0) ? v : fma(beta, *c, v);
    }
  }
}

template <int S>
__global__ void __launch_bounds__(256)
recombine_tile_kernel(int64_t m, int64_t n, int m_tiles, int64_t plane_stride,
                      const int *__restrict__ planes, const int *__restrict__ ea,
                      const int *__restrict__ eb, double alpha, double beta,
                      double *__restrict__ C, int64_t ldc, int ta, int tb, int64_t k,
                      const double *__restrict__ A, int64_t lda, const double *__restrict__ B,
                      int64_t ldb, int tri, const int *__restrict__ skip) {
  if (skip && *skip) return;  // a failed factorisation step upstream: leave C as it is
  recombine_tile<S>(m, n, m_tiles, plane_stride, planes, ea, eb, alpha, beta, C, ldc, ta, tb, k,
                    A, lda, B, ldb, tri);
}

// Automatic mode: each 256-column tile has its own slice count (s_tiles).
__global__ void __launch_bounds__(256)
recombine_auto_kernel(int64_t m, int64_t n, int m_tiles, int64_t plane_stride,
                      const int *__restrict__ planes, const int *__restrict__ ea,
                      const int *__restrict__ eb, double alpha, double beta,
                      double *__restrict__ C, int64_t ldc, int ta, int tb, int64_t k,
                      const double *__restrict__ A, int64_t lda, const double *__restrict__ B,
                      int64_t ldb, int tri, const int *__restrict__ skip,
                      const int *__restrict__ s_tiles, const int *__restrict__ run_if) {
  if (skip && *skip) return;
  if (run_if && *run_if == 0) return;
  switch (s_tiles[blockIdx.y]) {  // 0: a modular tile, reconstructed elsewhere
#define GB_RECOMBINE_CASE(SS)                                                                  \
  case SS:                                                                                     \
    recombine_tile<SS>(m, n, m_tiles, plane_stride, planes, ea, eb, alpha, beta, C, ldc, ta,   \
                       tb, k, A, lda, B, ldb, tri);                                            \
    break;
    GB_RECOMBINE_CASE(1) GB_RECOMBINE_CASE(2) GB_RECOMBINE_CASE(3) GB_RECOMBINE_CASE(4)
    GB_RECOMBINE_CASE(5) GB_RECOMBINE_CASE(6) GB_RECOMBINE_CASE(7) GB_RECOMBINE_CASE(8)
#undef GB_RECOMBINE_CASE
    default: break;
  }
}

// Modular scheme: C from the residue planes, one CTA per 128 x 256 tile of C
// (tiles with s_tiles[nt] != 0 belong to the digit-slice pass).  The
// residues r of C'_ij modulo a_i and b_i (in [0, a_i), [0, b_i)) first
// combine into its residue modulo m_i = a_i b_i (32-bit arithmetic):
//   y_i = r_a + a_i ((r_b - r_a) a_i^-1 mod b_i),  0 <= y_i < m_i < 2^18.
// Then X = sum_i y_i W_i is congruent to C' mod M, and
// X / M = sum_i y_i u_i / m_i, so the quotient q = round(sum_i y_i F_i 2^-32)
// (error below 7 2^18 2^-33 < 2^-12) gives C' = X - q M: |C'| < M / (2 + 2^-5)
// by the choice of t leaves a margin of 0.007 to the rounding.  X - q M is
// formed exactly in four signed 64-bit limbs of 32 bits (every limb sum is
// below 2^53) and combined modulo 2^128, which holds C' as |C'| < 2^127.
__global__ void __launch_bounds__(256)
reconstruct_tile_kernel(int64_t m, int64_t n, int m_tiles, int64_t plane_stride,
                        const uint16_t *__restrict__ planes, const int *__restrict__ ea,
                        const int *__restrict__ eb, double alpha, double beta,
                        double *__restrict__ C, int64_t ldc, int ta, int tb, int64_t k,
                        const double *__restrict__ A, int64_t lda, const double *__restrict__ B,
                        int64_t ldb, int tri, const int *__restrict__ skip,
                        const int *__restrict__ s_tiles, const int *__restrict__ run_if,
                        const __grid_constant__ ModTable tab) {
  if (skip && *skip) return;
  if (run_if && *run_if == 0) return;
  const int mt = blockIdx.x, nt = blockIdx.y;
  if (s_tiles && s_tiles[nt] != 0) return;
  const int64_t i0 = (int64_t)mt * BM, j0 = (int64_t)nt * BN;
  if (tri == 1 && i0 + BM - 1 < j0) return;
  if (tri == 2 && i0 > j0 + BN - 1) return;
  // a thread takes two consecutive rows of a column (one 4-byte load per
  // plane), 64 threads a column; grid z splits the tile's columns into
  // chunks (more CTAs, and short last waves, for any size of C)
  const int tid = threadIdx.x;
  const int il = (tid & 63) * 2, jb = tid >> 6;
  // FP64 compares run on the FP64 pipe: decide alpha = 1 and beta = 0 once
  const bool alpha_one = alpha == 1.0, beta_zero = beta == 0.0;
  const uint16_t *pt = planes + ((int64_t)nt * m_tiles + mt) * (BM * BN);
  int e_i[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) e_i[r] = (i0 + il + r < m) ? ea[i0 + il + r] : 0;
  const int chunk = BN / (int)gridDim.z, jz0 = (int)blockIdx.z * chunk;
  const int jn_tile = (n - j0) < BN ? (int)(n - j0) : BN;
  const int jend = jn_tile < jz0 + chunk ? jn_tile : jz0 + chunk;
  for (int jl = jz0 + jb; jl < jend; jl += 4) {
    const int64_t j = j0 + jl;
    const int fj = eb[j];
    uint32_t P[MOD_COUNT];
#pragma unroll
    for (int l = 0; l < MOD_COUNT; ++l)
      P[l] = __ldg(reinterpret_cast<const unsigned int *>(pt + (int64_t)l * plane_stride +
                                                          jl * BM + il));
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int64_t i = i0 + il + r;
      if (i >= m) continue;
      if ((tri == 1 && i < j) || (tri == 2 && i > j)) continue;
      double v;
      if (e_i[r] == NONFINITE || fj == NONFINITE) {
        double sum = 0.0;
        for (int64_t pp = 0; pp < k; ++pp) {
          const double a = ta ? A[pp + i * lda] : A[i + pp * lda];
          const double b = tb ? B[j + pp * ldb] : B[pp + j * ldb];
          sum = fma(a, b, sum);
        }
        v = alpha * sum;
      } else {
        // X = sum_i y_i W_i in four 32-bit limbs (each limb sum below 2^53)
        // and the quotient estimate sum_i y_i F_i (fraction of 2^32)
        unsigned long long qa = 0, x0 = 0, x1 = 0, x2 = 0, x3 = 0;
#pragma unroll
        for (int i2 = 0; i2 < MOD_PAIRS; ++i2) {
          const uint32_t ra = r ? (P[2 * i2] >> 16) : (P[2 * i2] & 0xFFFFu);
          const uint32_t rb = r ? (P[2 * i2 + 1] >> 16) : (P[2 * i2 + 1] & 0xFFFFu);
          const uint32_t b = tab.pb[i2];
          // (r_b - r_a) a^-1 mod b: the difference made positive, < 3 b;
          // the product below 2^20, its quotient by b exact from the magic
          const uint32_t u = (rb + 2 * b - ra) * tab.pinv_ab[i2];
          const uint32_t tq = u - __umulhi(u, tab.pmagic[i2]) * b;
          const uint32_t y = ra + tab.pa[i2] * tq;  // C' mod a b, below 2^18
          qa += (unsigned long long)y * tab.F[i2];
          x0 += (unsigned long long)y * tab.W[i2][0];
          x1 += (unsigned long long)y * tab.W[i2][1];
          x2 += (unsigned long long)y * tab.W[i2][2];
          x3 += (unsigned long long)y * tab.W[i2][3];
        }
        // C' = X - q M modulo 2^128: signed limb differences (|d| < 2^54),
        // then one carry pass into two 64-bit words
        const unsigned long long q = (qa + 0x80000000ull) >> 32;
        long long d = (long long)x0 - (long long)(q * tab.M[0]);
        const unsigned long long c0 = (unsigned long long)d & 0xFFFFFFFFull;
        d = ((long long)x1 - (long long)(q * tab.M[1])) + (d >> 32);
        const unsigned long long c1 = (unsigned long long)d & 0xFFFFFFFFull;
        d = ((long long)x2 - (long long)(q * tab.M[2])) + (d >> 32);
        const unsigned long long c2 = (unsigned long long)d & 0xFFFFFFFFull;
        d = ((long long)x3 - (long long)(q * tab.M[3])) + (d >> 32);
        const unsigned long long lo = c0 | (c1 << 32);
        const unsigned long long hi = c2 | ((unsigned long long)d << 32);
        const int xs = e_i[r] + fj - 2 * tab.bits;
        bool ok;
        v = ozd::i128_scaled(hi, lo, xs, ok);
        if (!ok)
          v = ozd::scaled_value((__int128)(((unsigned __int128)hi << 64) | lo), xs, alpha);
        else if (!alpha_one)
          v *= alpha;
      }
      double *c = C + i + j * ldc;
      *c = beta_zero ? v : fma(beta, *c, v);
    }
  }
}

// Automatic mode over several column blocks: op(A)'s digit split runs once,
// for the first block with digit-slice tiles (run = count > 0 and not yet
// done).
__global__ void latch_kernel(const int *__restrict__ count, int *__restrict__ latch) {
  const int run = *count > 0 && latch[0] == 0;
  latch[1] = run;
  if (run) latch[0] = 1;
}

// ------------------------------------------------------------------ host
// The modular scheme's moduli: the 14 largest odd numbers <= 511 that are
// pairwise coprime (511 = 7 * 73, 507 = 3 * 13^2, 505 = 5 * 101,
// 493 = 17 * 29, 473 = 11 * 43, the rest prime).  M = prod p_l ~ 2^125.06.
constexpr int MODULI[MOD_COUNT] = {511, 509, 507, 505, 503, 499, 493,
                                   491, 487, 479, 473, 467, 463, 461};

static int mod_inverse(int a, int p) {  // a^-1 mod p, gcd(a, p) = 1
  int t0 = 0, t1 = 1, r0 = p, r1 = a % p;
  while (r1) {
    const int q = r0 / r1, t2 = t0 - q * t1, r2 = r0 - q * r1;
    t0 = t1;
    t1 = t2;
    r0 = r1;
    r1 = r2;
  }
  return t0 < 0 ? t0 + p : t0;
}

static unsigned __int128 mod_product() {
  unsigned __int128 M = 1;
  for (int l = 0; l < MOD_COUNT; ++l) M *= (unsigned)MODULI[l];
  return M;
}

// The table without t (computed once).
static const ModTable &mod_base() {
  static const ModTable tab = [] {
    ModTable t{};
    const unsigned __int128 M = mod_product();
    for (int q = 0; q < 4; ++q) t.M[q] = (uint32_t)(M >> (32 * q));
    for (int i = 0; i < MOD_PAIRS; ++i) {
      const unsigned a = (unsigned)MODULI[2 * i], b = (unsigned)MODULI[2 * i + 1];
      const unsigned long long mi = (unsigned long long)a * b;
      t.pa[i] = a;
      t.pb[i] = b;
      t.pinv_ab[i] = (uint32_t)mod_inverse((int)(a % b), (int)b);
      t.pmagic[i] = (uint32_t)(((1ull << 32) + b - 1) / b);
      const unsigned __int128 Mi = M / mi;
      const unsigned long long mr = (unsigned long long)(Mi % mi);
      // (M / m_i)^-1 mod m_i by the extended Euclid algorithm in 64 bits
      long long t0 = 0, t1 = 1, r0 = (long long)mi, r1 = (long long)mr;
      while (r1) {
        const long long q = r0 / r1, t2 = t0 - q * t1, r2 = r0 - q * r1;
        t0 = t1;
        t1 = t2;
        r0 = r1;
        r1 = r2;
      }
      const unsigned long long u = (unsigned long long)(t0 < 0 ? t0 + (long long)mi : t0);
      const unsigned __int128 W = Mi * u;  // < M
      for (int q = 0; q < 4; ++q) t.W[i][q] = (uint32_t)(W >> (32 * q));
      t.F[i] = (uint32_t)(((unsigned __int128)u << 32) / mi +
                          ((((unsigned __int128)u << 32) % mi) * 2 >= mi ? 1 : 0));
    }
    for (int l = 0; l < MOD_COUNT; ++l) {
      const int p = MODULI[l];
      t.pf[l] = (float)p;
      t.pinv[l] = 1.0f / (float)p;
      for (int d = 0; d < MOD_CHUNKS; ++d) {
        const int w = (int)((1ull << (MOD_CHUNK_BITS * d)) % (unsigned)p);
        t.pw[l][d] = (float)(w > p / 2 ? w - p : w);
      }
    }
    return t;
  }();
  return tab;
}

// Largest t <= 60 with M > 2 k 2^2t (1 + 2^-6): every |C'_ij| < k 2^2t then
// lies below M / 2 with room for the quotient's rounding.  t = 56 for
// k = 4096.
int mod_bits(int64_t k) {
  const unsigned __int128 M = mod_product();
  int kb = 0;
  while (kb < 63 && ((int64_t)1 << kb) < k) ++kb;  // k <= 2^kb
  for (int t = MOD_MAX_BITS; t > 0; --t) {
    if (2 * t + 1 + kb > 126) continue;
    const unsigned __int128 lhs = (unsigned __int128)k << (2 * t + 1);
    if (lhs + (lhs >> 6) < M) return t;
  }
  return 0;
}

// 2-D tensor map over `rows` x `kpad` bf16 (K innermost), box 64 x box_rows.
int make_map(CUtensorMap *map, void *base, int64_t rows, int64_t kpad, int box_rows) {
  return make_bf16_kmajor_map(map, base, rows, kpad, BK, box_rows);
}

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Blocks of the digit split's grid-stride loop over 32 x 64 tiles: one per
// tile, or, for a launch predicated on the device (the automatic mode's
// digit pass, off unless some tile needs digits), eight per SM, so that a
// launch with nothing to do costs a few CTAs.
static unsigned split_grid(int64_t Rpad, int64_t Kpad, bool predicated) {
  const int64_t ntiles = (Kpad / 64) * (Rpad / 32), cap = 8LL * sm_count();
  return (unsigned)(predicated && ntiles > cap ? cap : ntiles);
}

void launch_split(bool kcontig, int64_t R, int64_t K, const double *X, int64_t ld,
                  const int *expo, int S, int64_t Rpad, int64_t Kpad, __nv_bfloat16 *slices,
                  const int *s_tiles, const int *run_if, cudaStream_t s) {
  const unsigned g2 = split_grid(Rpad, Kpad, run_if != nullptr);
  if (kcontig)
    split_kernel<true><<<g2, 256, 0, s>>>(R, K, X, ld, expo, S, Rpad, Kpad, slices, s_tiles,
                                          run_if);
  else
    split_kernel<false><<<g2, 256, 0, s>>>(R, K, X, ld, expo, S, Rpad, Kpad, slices, s_tiles,
                                           run_if);
  count_launch();
}

// Rpad: the planes' row stride; Rgrid (default Rpad): the rows written, a
// multiple of 32 (less than Rpad for a block of rows at res + i0 Kpad).
void launch_split_mod(bool kcontig, int64_t R, int64_t K, const double *X, int64_t ld,
                      const int *expo, int64_t Rpad, int64_t Kpad, __nv_bfloat16 *res,
                      const int *s_tiles, const int *run_if, const ModTable &tab,
                      cudaStream_t s, int64_t Rgrid = 0) {
  dim3 g2((unsigned)(Kpad / 64), (unsigned)((Rgrid > 0 ? Rgrid : Rpad) / 32));
  if (kcontig)
    split_mod_kernel<true><<<g2, 256, 0, s>>>(R, K, X, ld, expo, Rpad, Kpad, res, s_tiles,
                                              run_if, tab);
  else
    split_mod_kernel<false><<<g2, 256, 0, s>>>(R, K, X, ld, expo, Rpad, Kpad, res, s_tiles,
                                               run_if, tab);
  count_launch();
}

// Row maxima and exponents of an R x K op-view operand (with emax: their
// maximum over the non-zero finite rows as well).
void operand_exponents(bool kcontig, int64_t R, int64_t K, const double *X, int64_t ld,
                       int64_t Rpad, unsigned long long *mx, int *expo, cudaStream_t s,
                       int *emax = nullptr, bool init_emax = true) {
  cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * Rpad, s);
  if (emax && init_emax) cudaMemsetAsync(emax, 0x80, sizeof(int), s);  // a large negative value
  if (kcontig) {
    { rowmax_kcontig_kernel<<<(unsigned)((R + 7) / 8), 256, 0, s>>>(R, K, X, ld, mx); count_launch(); }
  } else {
    // K spans of 16..256 columns: 8 CTAs per SM (HBM needs them), a short
    // op(A) too
    const int64_t gx = (R + 255) / 256;
    int64_t kspan = 256;
    while (kspan > 16 && gx * ((K + kspan - 1) / kspan) < 8LL * persistent_ctas()) kspan /= 2;
    dim3 g((unsigned)gx, (unsigned)((K + kspan - 1) / kspan));
    { rowmax_mcontig_kernel<<<g, 256, 0, s>>>(R, K, X, ld, kspan, mx); count_launch(); }
  }
  { exponent_kernel<<<(unsigned)((Rpad + 255) / 256), 256, 0, s>>>(Rpad, R, mx, expo, emax); count_launch(); }
}

// Split an R x K op-view operand into S K-contiguous bf16 slices + exponents.
void split_operand(bool kcontig, int64_t R, int64_t K, const double *X, int64_t ld, int S,
                   int64_t Rpad, int64_t Kpad, unsigned long long *mx, int *expo,
                   __nv_bfloat16 *slices, cudaStream_t s) {
  operand_exponents(kcontig, R, K, X, ld, Rpad, mx, expo, s);
  launch_split(kcontig, R, K, X, ld, expo, S, Rpad, Kpad, slices, nullptr, nullptr, s);
}

// Automatic choice, op(A) side (after op(A)'s exponents and their maximum
// emax are known): alpha_k 2^-E_A in FP32 and the totals T_e, T_1, E_A.
void a_side_stats(bool kcontig, int64_t R, int64_t K, const double *X, int64_t ld,
                  const int *expo, const unsigned long long *mx, const int *emax, float *alpha,
                  double *totals, cudaStream_t s) {
  cudaMemsetAsync(alpha, 0, sizeof(float) * K, s);
  // at most 256 rows summed by one thread: a thread per k over 256 rows, or
  // a block of 256 threads per k over up to 65536 rows (one block per
  // column of op(A) up to that height)
  const int64_t rspan = kcontig ? 256 : 65536;
  if (kcontig) {
    dim3 g((unsigned)((K + 255) / 256), (unsigned)((R + rspan - 1) / rspan));
    { abs_colsum_kernel<true><<<g, 256, 0, s>>>(R, K, X, ld, expo, emax, rspan, alpha); count_launch(); }
  } else {
    dim3 g((unsigned)K, (unsigned)((R + rspan - 1) / rspan));
    { abs_colsum_kernel<false><<<g, 256, 0, s>>>(R, K, X, ld, expo, emax, rspan, alpha); count_launch(); }
  }
  { a_totals_kernel<<<1, 256, 0, s>>>(R, K, expo, mx, alpha, emax, totals); count_launch(); }
}

// Automatic choice, op(B) side: exponents and FP32 column statistics of
// op(B), then the scheme (and slice count) of every 256-column tile.  With
// mx_a / ea_a (op(B) = op(A)^T over the same K segment, R rows of op(A)):
// op(B)'s column maxima and exponents are op(A)'s row ones, copied instead
// of read again from the operand.
void choose_b(bool kcontig, int64_t R, int64_t K, const double *X, int64_t ld, int64_t Rpad,
              unsigned long long *mx, int *expo, const float *alpha, const double *totals,
              float *s1, float *s2, double budget_mod, double budget_dig, int mod_t,
              int *s_tiles, int *pass, cudaStream_t s,
              const unsigned long long *mx_a = nullptr, const int *ea_a = nullptr) {
  cudaMemsetAsync(pass, 0, 2 * sizeof(int), s);
  if (kcontig) {
    { col_stats_kcontig_kernel<<<(unsigned)((Rpad + 7) / 8), 256, 0, s>>>(R, Rpad, K, X, ld, alpha,
                                                                          mx, expo, s1, s2); count_launch(); }
  } else {
    if (mx_a) {
      // the values operand_exponents gives: zero maxima and exponents past R
      cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * Rpad, s);
      cudaMemsetAsync(expo, 0, sizeof(int) * Rpad, s);
      cudaMemcpyAsync(mx, mx_a, sizeof(unsigned long long) * R, cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(expo, ea_a, sizeof(int) * R, cudaMemcpyDeviceToDevice, s);
    } else {
      operand_exponents(false, R, K, X, ld, Rpad, mx, expo, s);
    }
    cudaMemsetAsync(s1, 0, sizeof(float) * Rpad, s);
    cudaMemsetAsync(s2, 0, sizeof(float) * Rpad, s);
    const int64_t kspan = 256;
    dim3 g((unsigned)((R + 255) / 256), (unsigned)((K + kspan - 1) / kspan));
    { col_stats_mcontig_kernel<<<g, 256, 0, s>>>(R, K, X, ld, kspan, alpha, expo, s1, s2); count_launch(); }
  }
  int *status = ctx().d_status;
  { choose_slices_kernel<<<(unsigned)(Rpad / BN), 256, 0, s>>>(
        R, expo, mx, s1, s2, totals, K, budget_mod, budget_dig, mod_t, s_tiles,
        status + STATUS_LAST_SLICES,
        status + STATUS_LAST_MODULI, pass); count_launch(); }
}

// The whole emulated product.  K is cut into segments of at most
// MAX_K_SEGMENT (so every int32 level sum is exact; MOD_K_SEGMENT in
// automatic mode with the modular scheme allowed, the digit-slice tiles then
// taking each segment in sub-segments of MAX_K_SEGMENT); each segment is
// split, multiplied on the tensor cores and recombined, later segments
// accumulating into C (beta = 1).  The columns of op(B) and C are taken in blocks of `nb`
// (a multiple of BN), all segments of a block before the next block, with
// the hooks (when given) making block j of op(B) and C available on the
// device first, setting the blocks' widths (multiples of 256 columns, so the
// 256-column tiles of the automatic choice are those of the single-block
// form) and told when C's block is final.  op(A) is split once when K
// is one segment and per segment and block otherwise.  Every C(i,j) depends
// only on row i of op(A) and column j of op(B) (and their own exponents), so
// the blocked result equals the single-block one bit for bit.
//
// Automatic mode runs two passes per segment, each predicated on the device
// by the count of tiles the choice gave it (a pass with none launches
// kernels that return at once): the modular pass (residues, residue GEMM,
// reconstruction) and the digit-slice pass (slices, slice GEMM, recombine).
// They share op(B)'s buffer and the planes and write disjoint tiles of C.
int emulated_product(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                     const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                     double *C, int64_t ldc, int S, cudaStream_t s, int tri, const int *skip,
                     int64_t nb = 0, EmuBlockHooks *hooks = nullptr) {
  if (nb <= 0 || nb >= n) nb = n;
  const bool automatic = S == OZAKI_SLICES_AUTO;
  const bool fixed_mod = S == OZAKI_MODULAR_FIXED;  // every tile modular, no choice
  // slices allocated (and cut from op(A)); none in the fixed modular form
  const int Sa = automatic ? MAX_SLICES : fixed_mod ? 0 : S;
  const bool modular = fixed_mod || (automatic && ozaki_modular_enabled());
  const int64_t seg_len = modular ? MOD_K_SEGMENT : MAX_K_SEGMENT;
  const int64_t kseg = k < seg_len ? k : seg_len;
  const int64_t nseg = (k + seg_len - 1) / seg_len;
  // the modular scheme's t for the longest segment
  const int mod_t = modular ? mod_bits(kseg) : 0;
  const int64_t m_pad = round_up(m, BM), nb_pad = round_up(nb, BN), ks_pad = round_up(kseg, BK);
  // How op(A) is prepared (row maxima, exponents, statistics, splits):
  //  - one K segment: once, before the block loop (with several column
  //    blocks in automatic mode, split in both forms, as the blocks' choices
  //    are not known yet);
  //  - several segments and several blocks: each segment once, while the
  //    first block runs, kept for the later blocks (both forms);
  //  - several segments, one block: per segment, each form predicated on the
  //    choice.
  const bool a_once = nseg == 1;
  const bool a_cache = !a_once && nb < n;
  const bool a_early = a_once && (!automatic || nb < n);
  const bool a_both = a_early || a_cache;  // both forms split unpredicated
  // automatic, one segment, several blocks: op(A)'s digit slices are cut for
  // the first block whose choice has digit-slice tiles (none when every
  // tile takes the modular scheme)
  const bool a_dig_lazy = a_early && automatic;
  const int64_t a_copies = a_cache ? nseg : 1;
  const int b_planes = modular && MOD_COUNT > Sa ? MOD_COUNT : Sa;
  const size_t seg_sa = align256((size_t)Sa * m_pad * ks_pad * 2);
  const size_t seg_ra = modular ? align256((size_t)MOD_COUNT * m_pad * ks_pad * 2) : 0;
  const size_t seg_ea = align256((size_t)m_pad * 4);
  // automatic mode, op(A) side: alpha_k (FP32), the three totals and emax
  const size_t seg_st = automatic ? align256((size_t)ks_pad * 4) + 256 : 0;
  const size_t bytes_sb = align256((size_t)b_planes * nb_pad * ks_pad * 2);
  const size_t bytes_mx = align256((size_t)(m_pad + nb_pad) * 8);
  const size_t bytes_eb = align256((size_t)nb_pad * 4);
  const size_t plane_bytes = (size_t)Sa * 4 > (size_t)MOD_COUNT * 2 || !modular
                                 ? (size_t)Sa * 4 : (size_t)MOD_COUNT * 2;
  const size_t bytes_pl = align256(plane_bytes * m_pad * nb_pad);
  // automatic mode, op(B) side: its column sums, the per-tile choices, the
  // two pass counts and the latch of op(A)'s digit split
  const size_t bytes_auto =
      automatic ? align256((size_t)(2 * nb_pad) * 4 + (size_t)(nb_pad / BN + 4) * 4) : 0;
  Scratch ws((seg_sa + seg_ra + seg_ea + seg_st) * a_copies + bytes_sb + bytes_mx + bytes_eb +
                 bytes_pl + bytes_auto, s);
  if (!ws.p) return GB_ERR_ALLOC;
  char *base = ws.as<char>();
  char *a_base = base;  // per-segment op(A) data: digits, residues, exponents, statistics
  base += (seg_sa + seg_ra + seg_ea + seg_st) * a_copies;
  __nv_bfloat16 *slb = reinterpret_cast<__nv_bfloat16 *>(base);
  base += bytes_sb;
  unsigned long long *mx = reinterpret_cast<unsigned long long *>(base);
  base += bytes_mx;
  int *eb = reinterpret_cast<int *>(base);
  base += bytes_eb;
  int *planes = reinterpret_cast<int *>(base);
  base += bytes_pl;
  float *st_s1 = nullptr, *st_s2 = nullptr;
  int *s_tiles = nullptr, *pass = nullptr, *latch = nullptr;
  double budget_mod = 0.0, budget_dig = 0.0;
  if (automatic) {
    st_s1 = reinterpret_cast<float *>(base);
    st_s2 = st_s1 + nb_pad;
    s_tiles = reinterpret_cast<int *>(st_s2 + nb_pad);
    pass = s_tiles + nb_pad / BN;  // [0] modular tiles, [1] digit-slice tiles
    latch = pass + 2;              // [0] op(A)'s digits split, [1] split them now
    // the tolerance in units of 2^-52 less the roundings of the recombine
    // (one conversion, the alpha/beta step) and of the accumulation over
    // the segments (modular tiles) or the digit passes' sub-segments
    int64_t nsub = 0;
    for (int64_t k0 = 0; k0 < k; k0 += seg_len) {
      const int64_t kk = (k - k0) < seg_len ? (k - k0) : seg_len;
      nsub += (kk + MAX_K_SEGMENT - 1) / MAX_K_SEGMENT;
    }
    budget_mod = ldexp(config().ozaki_tol, -52) - ldexp((double)(nseg + 2), -53);
    budget_dig = ldexp(config().ozaki_tol, -52) - ldexp((double)(nsub + 2), -53);
  }
  struct ASeg {
    __nv_bfloat16 *dig, *res;
    int *ea;
    float *alpha;
    double *tot;
    int *emax;
  };
  auto aseg = [&](int64_t sg) {
    char *p = a_base + (a_cache ? sg : 0) * (seg_sa + seg_ra + seg_ea + seg_st);
    ASeg a;
    a.dig = reinterpret_cast<__nv_bfloat16 *>(p);
    a.res = reinterpret_cast<__nv_bfloat16 *>(p + seg_sa);
    a.ea = reinterpret_cast<int *>(p + seg_sa + seg_ra);
    char *st = p + seg_sa + seg_ra + seg_ea;
    a.alpha = automatic ? reinterpret_cast<float *>(st) : nullptr;
    a.tot = automatic ? reinterpret_cast<double *>(st + align256((size_t)ks_pad * 4)) : nullptr;
    a.emax = automatic ? reinterpret_cast<int *>(a.tot + 3) : nullptr;
    return a;
  };
  ModTable tab = mod_base();
  tab.bits = mod_t;

  static PerDeviceOnce attr_once;
  int st = attr_once.run(current_device(), [] {
    GB_CUDA(cudaFuncSetAttribute(slice_gemm_kernel<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(slice_gemm_kernel<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    return GB_SUCCESS;
  });
  if (st) return st;
  std::vector<CUtensorMap> mapA((size_t)a_copies), mapAr((size_t)a_copies);
  CUtensorMap mapB, mapBr;
  // op(A) rows: K-contiguous when A is transposed; op(B) columns: K-contiguous when B is not
  auto seg_a = [&](int64_t k0) { return ta ? A + k0 : A + k0 * lda; };
  auto prep_a = [&](int64_t sg, int64_t k0, int64_t kk) {
    const ASeg a = aseg(sg);
    operand_exponents(ta != 0, m, kk, seg_a(k0), lda, m_pad, mx, a.ea, s, a.emax);
    if (automatic)
      a_side_stats(ta != 0, m, kk, seg_a(k0), lda, a.ea, mx, a.emax, a.alpha, a.tot, s);
  };
  auto split_a = [&](int64_t sg, int64_t k0, int64_t kk, const int *run_if) -> int {
    const int64_t kp = round_up(kk, BK);
    const ASeg a = aseg(sg);
    launch_split(ta != 0, m, kk, seg_a(k0), lda, a.ea, Sa, m_pad, kp, a.dig, nullptr, run_if, s);
    return make_map(&mapA[a_cache ? sg : 0], a.dig, (int64_t)Sa * m_pad, kp, BM);
  };
  auto split_a_mod = [&](int64_t sg, int64_t k0, int64_t kk, const int *run_if) -> int {
    const int64_t kp = round_up(kk, BK);
    const ASeg a = aseg(sg);
    launch_split_mod(ta != 0, m, kk, seg_a(k0), lda, a.ea, m_pad, kp, a.res, nullptr, run_if, tab,
                     s);
    return make_map(&mapAr[a_cache ? sg : 0], a.res, (int64_t)MOD_COUNT * m_pad, kp, BM);
  };
  auto gemm = [&](bool mod, const CUtensorMap &ma, const CUtensorMap &mb, int64_t jn_pad,
                  int64_t kb0, int64_t kp, const int *run_if, int64_t b_rows) -> int {
    GemmParams gp{};
    gp.S = Sa;
    gp.m_tiles = (int)(m_pad / BM);
    gp.n_tiles = (int)(jn_pad / BN);
    gp.group_m = config().ozaki_group_m;
    // the triangle is relative to C's own indices: only the single-block
    // form (j0 = 0) is used with tri
    gp.tri = tri;
    gp.kblocks = (int)(kp / BK);
    gp.kblock0 = (int)kb0;
    gp.m_pad = (int)m_pad;
    gp.n_pad = (int)jn_pad;
    gp.b_rows = (int)b_rows;
    gp.plane_stride = m_pad * jn_pad;
    gp.planes = planes;
    gp.status = ctx().d_status;
    gp.s_tiles = s_tiles;
    gp.run_if = run_if;
    for (int l = 0; l < MOD_COUNT; ++l) {
      gp.mod_p[l] = MODULI[l];
      gp.mod_magic[l] = (uint32_t)(((1ull << 40) + MODULI[l] - 1) / MODULI[l]);
    }
    const int ntiles = gp.m_tiles * gp.n_tiles;
    // fewer tiles than CTAs: split each tile's levels over idle CTAs.  Digit
    // slices: as many groups as there are idle CTAs per tile.  Modular (14
    // equal levels): the group count with the fewest levels per CTA, units
    // beyond one wave included (32 tiles: 14 groups, 3 levels per CTA, where
    // one wave of 4 groups left 4); ties keep fewer groups.
    const int maxl = mod ? MOD_COUNT : Sa;
    const int pc = persistent_ctas();
    gp.level_groups = 1;
    if (ntiles < pc && mod) {
      int64_t best = INT64_MAX;
      for (int gc = 1; gc <= maxl; ++gc) {
        const int64_t units = (int64_t)ntiles * gc;
        const int64_t per_cta = ((units + pc - 1) / pc) * ((maxl + gc - 1) / gc);
        if (per_cta < best) {
          best = per_cta;
          gp.level_groups = gc;
        }
      }
    } else if (ntiles < pc) {
      const int spare = pc / ntiles;
      gp.level_groups = spare > maxl ? maxl : spare;
    }
    const int nunits = ntiles * gp.level_groups;
    const int grid = nunits < pc ? nunits : pc;
    if (mod) {
      ProfileScope prof("residue_gemm", s);
      slice_gemm_kernel<true><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(ma, mb, gp);
    } else {
      ProfileScope prof("slice_gemm", s);
      slice_gemm_kernel<false><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(ma, mb, gp);
    }
    count_launch();
    GB_CUDA(cudaGetLastError());
    return GB_SUCCESS;
  };
  const int64_t arb = a_early && hooks ? hooks->a_row_block() : 0;
  if (a_once && arb > 0 && arb < m) {
    // op(A) arrives in row blocks: each block's row maxima and exponents
    // (and, with the modular scheme, residues) while the next one uploads;
    // the choice statistics need every row and follow the last block.  Every
    // value is the one of the whole-operand preparation (all per row).
    const ASeg a = aseg(0);
    const int64_t kp = round_up(k, BK);
    if (a.emax) cudaMemsetAsync(a.emax, 0x80, sizeof(int), s);
    for (int64_t i0 = 0; i0 < m; i0 += arb) {
      const int64_t rb = (m - i0) < arb ? (m - i0) : arb;
      const int64_t rb_pad = i0 + rb < m ? rb : m_pad - i0;  // the last block pads to m_pad
      if ((st = hooks->a_rows(i0, rb))) return st;
      const double *Xi = ta ? A + i0 * lda : A + i0;
      operand_exponents(ta != 0, rb, k, Xi, lda, rb_pad, mx + i0, a.ea + i0, s, a.emax, false);
      if (modular)
        launch_split_mod(ta != 0, rb, k, Xi, lda, a.ea + i0, m_pad, kp, a.res + i0 * kp, nullptr,
                         nullptr, tab, s, rb_pad);
    }
    if (automatic) a_side_stats(ta != 0, m, k, A, lda, a.ea, mx, a.emax, a.alpha, a.tot, s);
    if (a_dig_lazy) cudaMemsetAsync(latch, 0, 2 * sizeof(int), s);
    if (modular && (st = make_map(&mapAr[0], a.res, (int64_t)MOD_COUNT * m_pad, kp, BM)))
      return st;
    if (Sa > 0 && !a_dig_lazy && (st = split_a(0, 0, k, nullptr))) return st;
  } else if (a_once) {
    if (hooks && (st = hooks->a_range(0, k))) return st;
    prep_a(0, 0, k);
    if (a_dig_lazy) cudaMemsetAsync(latch, 0, 2 * sizeof(int), s);
    if (a_early && Sa > 0 && !a_dig_lazy && (st = split_a(0, 0, k, nullptr))) return st;
    if (a_early && modular && (st = split_a_mod(0, 0, k, nullptr))) return st;
  }
  for (int64_t j0 = 0, jn = 0; j0 < n; j0 += jn) {
    jn = hooks ? hooks->block_cols(j0, nb) : nb;
    if (jn > nb || jn <= 0) jn = nb;
    if (jn > n - j0) jn = n - j0;
    const int64_t jn_pad = round_up(jn, BN);
    // op(B) = op(A)^T (SYRK-shaped products: the same matrix, one block):
    // op(B)'s residues and digits are op(A)'s rows, split with the same
    // exponents, so the B operand reads op(A)'s planes (whose plane stride
    // is m_pad rows; tiles past n read the next plane or TMA's zero fill,
    // only for columns that are never stored)
    const bool b_from_a = B != nullptr && B == A && ldb == lda && ta != tb && m == n && jn == n;
    const int64_t b_rows = b_from_a ? m_pad : jn_pad;
    const double *Bj = tb ? B + j0 : B + j0 * ldb;
    double *Cj = C + j0 * ldc;
    int64_t ldbj = ldb, ldcj = ldc;
    if (hooks && (st = hooks->before(j0, jn, &Bj, &ldbj, &Cj, &ldcj))) return st;
    for (int64_t sg = 0; sg < nseg; ++sg) {
      const int64_t k0 = sg * seg_len;
      const int64_t kk = (k - k0) < seg_len ? (k - k0) : seg_len;
      const int64_t kp = round_up(kk, BK);
      if (hooks && (st = hooks->segment(j0, jn, k0, kk))) return st;
      if (!a_once && (!a_cache || j0 == 0)) {
        if (hooks && (st = hooks->a_range(k0, kk))) return st;
        prep_a(sg, k0, kk);
        if (a_cache && Sa > 0 && (st = split_a(sg, k0, kk, nullptr))) return st;
        if (a_cache && modular && (st = split_a_mod(sg, k0, kk, nullptr))) return st;
      }
      const ASeg a = aseg(sg);
      const double *Ak = seg_a(k0);
      const double *Bk = tb ? Bj + k0 * ldbj : Bj + k0;
      const double bseg = sg == 0 ? beta : 1.0;  // later segments accumulate
      // recombination grid: one CTA per tile and column chunk, the tiles
      // split into up to 64 chunks (of 4 columns) until there are 16 CTAs
      // per SM (about four waves: a short last wave costs little); a small C
      // then gets a column per thread instead of a chain of several
      dim3 g((unsigned)((m + BM - 1) / BM), (unsigned)((jn + BN - 1) / BN), 1);
      while (g.z < 64 && (int64_t)g.x * g.y * g.z < 16LL * persistent_ctas()) g.z *= 2;
      const int m_tiles = (int)(m_pad / BM);
      const int64_t ps = m_pad * jn_pad;
      if (fixed_mod) {
        // every tile on the modular scheme: no statistics, no choice
        if (!a_both && (st = split_a_mod(sg, k0, kk, nullptr))) return st;
        if (b_from_a) {
          if ((st = make_map(&mapBr, a.res, (int64_t)MOD_COUNT * m_pad, kp, BN))) return st;
        } else {
          operand_exponents(tb == 0, jn, kk, Bk, ldbj, jn_pad, mx + m_pad, eb, s);
          launch_split_mod(tb == 0, jn, kk, Bk, ldbj, eb, jn_pad, kp, slb, nullptr, nullptr, tab, s);
          if ((st = make_map(&mapBr, slb, (int64_t)MOD_COUNT * jn_pad, kp, BN))) return st;
        }
        if ((st = gemm(true, mapAr[a_cache ? sg : 0], mapBr, jn_pad, 0, kp, nullptr, b_rows)))
          return st;
        reconstruct_tile_kernel<<<g, 256, 0, s>>>(
            m, jn, m_tiles, ps, reinterpret_cast<const uint16_t *>(planes), a.ea,
            b_from_a ? a.ea : eb, alpha, bseg, Cj, ldcj, ta, tb, kk, Ak, lda, Bk, ldbj, tri, skip,
            nullptr, nullptr, tab);
        count_launch();
        if ((st = check_cuda(cudaGetLastError(), "emulated dgemm"))) return st;
        continue;
      }
      if (!automatic) {
        if (!a_both && (st = split_a(sg, k0, kk, nullptr))) return st;
        if (b_from_a) {
          if ((st = make_map(&mapB, a.dig, (int64_t)Sa * m_pad, kp, BN))) return st;
        } else {
          split_operand(tb == 0, jn, kk, Bk, ldbj, S, jn_pad, kp, mx + m_pad, eb, slb, s);
          if ((st = make_map(&mapB, slb, (int64_t)Sa * jn_pad, kp, BN))) return st;
        }
        if ((st = gemm(false, mapA[a_cache ? sg : 0], mapB, jn_pad, 0, kp, nullptr, b_rows)))
          return st;
        const int *ebk = b_from_a ? a.ea : eb;
#define GB_RECOMBINE(SS)                                                                        \
  case SS:                                                                                      \
    recombine_tile_kernel<SS><<<g, 256, 0, s>>>(m, jn, m_tiles, ps, planes, a.ea, ebk, alpha,   \
                                                bseg, Cj, ldcj, ta, tb, kk, Ak, lda, Bk, ldbj,  \
                                                tri, skip);                                     \
    break;
        switch (S) {
          GB_RECOMBINE(1) GB_RECOMBINE(2) GB_RECOMBINE(3) GB_RECOMBINE(4)
          GB_RECOMBINE(5) GB_RECOMBINE(6) GB_RECOMBINE(7) GB_RECOMBINE(8)
          default: return set_error(GB_ERR_UNSUPPORTED, "emulated dgemm: %d slices", S);
        }
#undef GB_RECOMBINE
        count_launch();
        if ((st = check_cuda(cudaGetLastError(), "emulated dgemm"))) return st;
        continue;
      }
      choose_b(tb == 0, jn, kk, Bk, ldbj, jn_pad, mx + m_pad, eb, a.alpha, a.tot, st_s1, st_s2,
               budget_mod, budget_dig, mod_t, s_tiles, pass, s, b_from_a ? mx : nullptr,
               b_from_a ? a.ea : nullptr);
      if (modular) {
        // ---- modular pass (tiles with s_tiles = 0)
        if (!a_both && (st = split_a_mod(sg, k0, kk, pass))) return st;
        if (b_from_a) {
          if ((st = make_map(&mapBr, a.res, (int64_t)MOD_COUNT * m_pad, kp, BN))) return st;
        } else {
          launch_split_mod(tb == 0, jn, kk, Bk, ldbj, eb, jn_pad, kp, slb, s_tiles, pass, tab, s);
          if ((st = make_map(&mapBr, slb, (int64_t)MOD_COUNT * jn_pad, kp, BN))) return st;
        }
        if ((st = gemm(true, mapAr[a_cache ? sg : 0], mapBr, jn_pad, 0, kp, pass, b_rows)))
          return st;
        reconstruct_tile_kernel<<<g, 256, 0, s>>>(
            m, jn, m_tiles, ps, reinterpret_cast<const uint16_t *>(planes), a.ea, eb, alpha, bseg,
            Cj, ldcj, ta, tb, kk, Ak, lda, Bk, ldbj, tri, skip, s_tiles, pass, tab);
        count_launch();
        if ((st = check_cuda(cudaGetLastError(), "emulated dgemm"))) return st;
      }
      // ---- digit-slice pass (tiles with s_tiles = S > 0), over sub-segments
      // of at most MAX_K_SEGMENT (each level sum exact in int32), each
      // recombined into C in turn
      if (a_dig_lazy) {
        { latch_kernel<<<1, 1, 0, s>>>(pass + 1, latch); count_launch(); }
        if ((st = split_a(sg, k0, kk, latch + 1))) return st;
      } else if (!a_both && (st = split_a(sg, k0, kk, pass + 1))) {
        return st;
      }
      if (b_from_a) {
        if ((st = make_map(&mapB, a.dig, (int64_t)Sa * m_pad, kp, BN))) return st;
      } else {
        launch_split(tb == 0, jn, kk, Bk, ldbj, eb, MAX_SLICES, jn_pad, kp, slb, s_tiles,
                     pass + 1, s);
        if ((st = make_map(&mapB, slb, (int64_t)Sa * jn_pad, kp, BN))) return st;
      }
      for (int64_t u0 = 0; u0 < kk; u0 += MAX_K_SEGMENT) {
        const int64_t uk = (kk - u0) < MAX_K_SEGMENT ? (kk - u0) : MAX_K_SEGMENT;
        if ((st = gemm(false, mapA[a_cache ? sg : 0], mapB, jn_pad, u0 / BK, round_up(uk, BK),
                       pass + 1, b_rows)))
          return st;
        const double *Au = ta ? Ak + u0 : Ak + u0 * lda;
        const double *Bu = tb ? Bk + u0 * ldbj : Bk + u0;
        recombine_auto_kernel<<<g, 256, 0, s>>>(m, jn, m_tiles, ps, planes, a.ea, eb, alpha,
                                                u0 == 0 ? bseg : 1.0, Cj, ldcj, ta, tb, uk, Au,
                                                lda, Bu, ldbj, tri, skip, s_tiles, pass + 1);
        count_launch();
        if ((st = check_cuda(cudaGetLastError(), "emulated dgemm"))) return st;
      }
    }
    if (hooks && (st = hooks->after(j0, jn))) return st;
  }
  return GB_SUCCESS;
}

}  // namespace oz

// Form used when the caller passes 0 (the LU and Cholesky trailing updates
// and panel solves, the refinement residuals): for k >= MOD_MIN_K the
// modular scheme on every tile (t >= 55 bits, nothing dropped: a tighter
// bound than 7 digit slices with half the tensor-core work), otherwise (or
// when the thread has turned the modular scheme off) 7 slices of 8-bit
// digits.  Below k = 512 the CRT reconstruction per element of C costs more
// than the 14 products it saves (measured: the emulated DPOTRF 32768 with
// k = 256 updates took 789 ms on residues against 737 ms on digits).
constexpr int64_t MOD_MIN_K = 512;
static int ozaki_default_form(int64_t k) {
  return ozaki_modular_enabled() && k >= MOD_MIN_K ? OZAKI_MODULAR_FIXED : 7;
}

// Resolves a requested slice count: > 0 fixed (at most MAX_SLICES), 0 the
// default, OZAKI_SLICES_AUTO chosen per tile on the device (the records of
// the largest count and of the moduli chosen are reset for the new call).
static int resolve_slices(int slices, int64_t k, cudaStream_t s) {
  if (slices == OZAKI_SLICES_AUTO) {
    static_assert(STATUS_LAST_MODULI == STATUS_LAST_SLICES + 1, "adjacent status words");
    cudaMemsetAsync(ctx().d_status + STATUS_LAST_SLICES, 0, 2 * sizeof(int), s);
    return OZAKI_SLICES_AUTO;
  }
  if (slices <= 0) return ozaki_default_form(k);
  return slices > oz::MAX_SLICES ? oz::MAX_SLICES : slices;
}

int64_t emulated_k_segment(int slices) {
  const bool mod = (slices == OZAKI_SLICES_AUTO || slices == OZAKI_MODULAR_FIXED || slices == 0) &&
                   ozaki_modular_enabled();
  return mod ? oz::MOD_K_SEGMENT : oz::MAX_K_SEGMENT;
}

int dgemm_emulated_blocked(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double *A, int64_t lda, double beta, int slices, int64_t nb,
                           EmuBlockHooks *hooks, cudaStream_t s) {
  if (m <= 0 || n <= 0) return GB_SUCCESS;
  const int S = resolve_slices(slices, k, s);
  if (m > (int64_t)1 << 22 || n > (int64_t)1 << 22)
    return set_error(GB_ERR_UNSUPPORTED, "blocked emulated dgemm: dimension too large");
  nb = (nb + oz::BN - 1) / oz::BN * oz::BN;
  return oz::emulated_product(ta, tb, m, n, k, alpha, A, lda, nullptr, 0, beta, nullptr, 0, S, s,
                              0, nullptr, nb, hooks);
}

int dgemm_emulated(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                   const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                   double *C, int64_t ldc, int slices, cudaStream_t s, int tri,
                   const int *skip) {
  if (m <= 0 || n <= 0) return GB_SUCCESS;
  const int S = resolve_slices(slices, k, s);
  if ((m > GEMM_BLOCK_EXTENT || n > GEMM_BLOCK_EXTENT) && tri == 0 && !skip)
    return gemm_over_blocks(ta, tb, m, n, A, lda, B, ldb, C, ldc, GEMM_BLOCK_EXTENT,
                            [&](int64_t mb, int64_t nb, const double *Ai, const double *Bj,
                                double *Cij) {
                              return oz::emulated_product(ta, tb, mb, nb, k, alpha, Ai, lda, Bj,
                                                          ldb, beta, Cij, ldc, S, s, 0, nullptr);
                            });
  if (m > GEMM_BLOCK_EXTENT || n > GEMM_BLOCK_EXTENT)
    return set_error(GB_ERR_UNSUPPORTED, "emulated dgemm: triangular update too large");
  return oz::emulated_product(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, S, s, tri,
                              skip);
}

}  // namespace gb
