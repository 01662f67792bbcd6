// fg_ozaki.cu -- FP64 matrix products on the bf16 tensor cores (tcgen05) by digit slicing.
//
// GB300 runs FP64 at ~1 TFLOP/s (DFMA and the FP64 MMA alike) and bf16 MMAs at ~1.9
// PFLOP/s.  The dense FP64 products of the BDDC set-up are moved onto the tensor cores with
// the Ozaki scheme (K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59, 2012), in its fixed-point digit form (H. Ootomo,
// K. Ozaki, R. Yokota, "DGEMM on integer matrix multiplication unit", IJHPCA 2024), with
// bf16 digits instead of int8 ones because this part's int8 MMA rate is low:
//
//   * every row i of an operand gets a power of two 2^e_i with |x_il| 2^-e_i < 1/4 and is cut
//     into S = 7 signed digits, x_il = 2^e_i sum_s d_s 2^(-8(s+1)) (+ a tail below
//     2^(e_i-56)), |d_0| <= 64, |d_s| <= 128, so every digit is an exact bf16.  The cut is
//     integer arithmetic on the FP64 bit pattern (56 fraction bits, 54 of them below the row
//     maximum, digits rounded to nearest);
//   * the digit matrices are multiplied by tcgen05.mma kind::f16 (bf16 x bf16 -> FP32).  A
//     digit product is at most 2^14 (2^13 with a leading digit), and an accumulator sums at
//     most the equivalent of 6 full pairs (class 6: two leading-digit pairs and five others;
//     class 7: six others) over at most 170 K values: every FP32 partial sum is an integer
//     below 6 2^14 170 < 2^24, i.e. exact.  K up to 170 is one exact chunk (the Poisson
//     element matrices' K = 162 among them), longer K is cut into chunks of 160;
//   * the products of weight 2^(-8k), k = s + t = 0..7 (34 digit pairs), go to 8 FP32
//     accumulators in tensor memory (8 x 64 columns: all 512); pairs with s + t >= 8 are
//     dropped (|error| <~ K 2^-57 max_l |x_il| max_l |y_jl|).  The cut keeps 54 bits below
//     the row maximum, so a value far below it loses its low bits: overall the product is
//     within ~K 2^-52 max|x_i.| max|y_j.| of the exact one (about the FP64 dot-product bound);
//   * the epilogue converts the 8 class sums to integers, combines them exactly in int64,
//     turns the chunk's sum into FP64 with one rounding (two exact conversions by bit
//     arithmetic, one addition), adds the K chunks in FP64, applies the power of two
//     2^(e_i + f_j - 16) through the exponent field and updates C: about two FP64
//     operations per output element and chunk instead of 128.  (A rounding by integer
//     arithmetic alone measured slower: 421 vs 330 us at 4096 x 4096 x 128.)
//
// Digit layout in HBM: per operand, blocks of 128 rows x 16 columns (one MMA K step) per
// digit, 4 KB each, ordered [row tile][K step][digit]; inside a block the rows are in the
// canonical K-major, non-swizzled UMMA layout: core matrices of 8 rows x 16 bytes, the two
// 8-column halves 128 B apart (LBO), row groups 256 B apart (SBO).  An operand B tile of 64
// rows is half a block (2 KB), of 32 rows a quarter.  A CTA computes 128 x 64 (or 128 x 32)
// output tiles: warp 0's lane 0 streams the digit blocks into shared memory with
// cp.async.bulk (5 or 6 stages, mbarrier
// transaction counts) and issues the MMAs; warps 1-8 read the accumulators (tcgen05.ld, two
// warps per TMEM lane quarter, 32 columns each) and write C.  CTAs are persistent (one per SM, tiles round robin):
// the epilogue releases the accumulators before its FP64 writes, which then overlap the next
// tile's MMAs, and the stages of the next tile are loaded meanwhile.  Every wait is bounded: after ~1 s the CTA records
// FG_ERR_TIMEOUT, stops, waits (bounded) for its copies and MMAs in flight, frees its tensor
// memory and returns.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdint>

#include "fg_internal.h"

namespace fg {

namespace {

constexpr int OZ_S = 7;                       // digits per value
constexpr int OZ_NACC = 8;                    // accumulators: digit weights k = s + t = 0..7
constexpr int OZ_BM = 128, OZ_BK = 16;
constexpr int OZ_KEXACT = 170;                // K values one exact accumulation may sum
constexpr int OZ_CHUNK_STEPS = 10;            // K steps of a chunk when K > OZ_KEXACT (160 values)
constexpr uint32_t OZ_BLOCK = OZ_BM * OZ_BK * 2;           // one digit block: 4096 B
constexpr uint32_t OZ_A_BYTES = OZ_S * OZ_BLOCK;           // 28672 B per K step
constexpr uint32_t OZ_TMEM_COLS = 512;                     // all of it
constexpr long long OZ_WAIT_CYCLES = 1ll << 31;            // ~1 s at 2 GHz
constexpr int OZ_THREADS = 32 + 8 * 32;                    // MMA warp + 8 epilogue warps

// Output tiles of 128 x BN.  BN = 64: the 8 accumulators fill the tensor memory (one set);
// BN = 32: two sets, so one tile's MMAs run while the epilogue reads the previous tile.
template <int BN>
struct OzT {
  static constexpr int NSET = (int)OZ_TMEM_COLS / (OZ_NACC * BN);
  static constexpr int EPI = BN / 2;                          // columns per epilogue thread
  static constexpr int QB = OZ_BM / BN;                       // B tiles per 128-row digit block
  static constexpr uint32_t B_DIGIT = BN * OZ_BK * 2;         // one digit of a B tile per K step
  static constexpr uint32_t STAGE = OZ_A_BYTES + OZ_S * B_DIGIT;
  static constexpr int NBUF = BN == 64 ? 5 : 6;               // stages: 215040 B either way
  static constexpr uint32_t SMEM = NBUF * STAGE;
  // kind::f16: FP32 accumulator, bf16 A and B, both K-major, N = BN, M = 128
  static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                    ((uint32_t)(OZ_BM >> 4) << 24);
};
constexpr int OZ_MAXBUF = 6;

// ---- PTX wrappers -------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// global -> own shared memory, completion counted in bytes on the mbarrier
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, 128 x 64 x 16, bf16 -> FP32
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// arrive on the mbarrier once every tcgen05 operation issued so far by this thread is done
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, no swizzle; LBO = 128 B (the two 8-column
// halves of a 16-column step), SBO = 256 B (consecutive 8-row groups); version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(256u >> 4) << 32) |
         (1ull << 46);
}

// bounded wait; false (and the CTA's abort flag and the error status set) when it runs out
// after an abort: wait (bounded, ignoring the abort flag) for the copies or MMAs still in
// flight, so that nothing writes this CTA's shared or tensor memory once it is released
__device__ __forceinline__ void mbar_drain(uint32_t a, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try(a, parity)) {
    __nanosleep(64);
    if (clock64() - t0 > OZ_WAIT_CYCLES) return;
  }
}

__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile int* abort_flag, int* err) {
  const long long t0 = clock64();
  int spins = 0;
  while (!mbar_try(a, parity)) {
    if (*abort_flag) return false;
    if (++spins > 64) __nanosleep(64);
    if (clock64() - t0 > OZ_WAIT_CYCLES) {
      *abort_flag = 1;
      atomicExch(err, (int)FG_ERR_TIMEOUT);
      return false;
    }
  }
  return true;
}

}  // namespace

// ---- operands: one or more row blocks cut into digits ------------------------------------
// A split item: rows x k values, element (r, l) at x[r*rs + l*cs], cut into the digit row
// tiles rtile0 .. rtile0 + ceil(rows/128) - 1 of the workspace (exponents at 128 rtile + r).
struct OzSplit {
  const double* x;
  int64_t rs, cs;
  int rows, k;
  int rtile0;
};
struct OzSplitArgs {
  const OzSplit* items;  // device array, or nullptr: one[0 .. none-1]
  int nitems;
  OzSplit one[2];
  int none;
  int ksteps;
  int32_t* ex;
  uint4* dig;
};

__device__ __forceinline__ OzSplit split_of(const OzSplitArgs& a, int rtile) {
  if (!a.items) return (a.none > 1 && rtile >= a.one[1].rtile0) ? a.one[1] : a.one[0];
  int lo = 0, hi = a.nitems - 1;  // last item with rtile0 <= rtile
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.items[mid].rtile0 <= rtile) lo = mid;
    else hi = mid - 1;
  }
  return a.items[lo];
}

// Row exponents: e_r with max_l |x_rl| < 2^(e_r - 2), from the largest biased exponent of
// the row (an all-zero or padding row gets 0).  Blocks (digit row tile, part of 32).  Rows
// with consecutive elements (cs == 1): a warp per row, lanes along it, part p taking rows
// 4p .. 4p + 3; otherwise part 0 takes the tile, a thread per row (consecutive rows are
// consecutive in memory).
__global__ void __launch_bounds__(OZ_BM) k_oz_rowexp(OzSplitArgs a) {
  const int rtile = blockIdx.x;
  const OzSplit it = split_of(a, rtile);
  if (it.cs != 1 && blockIdx.y != 0) return;
  const int64_t r0 = (int64_t)(rtile - it.rtile0) * OZ_BM;
  auto finish = [&](int local, unsigned long long mx) {
    const int E = (int)(mx >> 52);  // biased exponent of the largest |x| (0: zero/subnormal)
    a.ex[(int64_t)rtile * OZ_BM + local] = mx == 0 ? 0 : (E == 0 ? 1 : E) - 1020;
  };
  if (it.cs == 1) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    {
      const int local = blockIdx.y * (OZ_BM / 32) + warp;
      const int64_t r = r0 + local;
      unsigned long long mx = 0;
      if (r < it.rows)
        for (int64_t l = lane; l < it.k; l += 32)
          mx = max(mx, (unsigned long long)__double_as_longlong(it.x[r * it.rs + l]) & 0x7FFFFFFFFFFFFFFFull);
#pragma unroll
      for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) finish(local, mx);
    }
  } else {
    const int64_t r = r0 + threadIdx.x;
    unsigned long long mx = 0;
    if (r < it.rows)
      for (int64_t l = 0; l < it.k; ++l)
        mx = max(mx, (unsigned long long)__double_as_longlong(it.x[r * it.rs + l * it.cs]) & 0x7FFFFFFFFFFFFFFFull);
    finish(threadIdx.x, mx);
  }
}

// Digits: block (digit row tile, K step), thread per row; 16 values, 7 digits each, written as
// the 7 digit blocks' 32-byte rows.  Rows past the item and columns >= k are zero.
__global__ void __launch_bounds__(OZ_BM) k_oz_split(OzSplitArgs a) {
  const int tid = threadIdx.x;
  const int rtile = blockIdx.x, ks = blockIdx.y;
  const OzSplit it = split_of(a, rtile);
  const int64_t r = (int64_t)(rtile - it.rtile0) * OZ_BM + tid;
  const int er = a.ex[(int64_t)rtile * OZ_BM + tid];
  uint32_t w[OZ_S][8];
#pragma unroll
  for (int c = 0; c < OZ_BK; c += 2) {
    int32_t d[2][OZ_S];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t l = (int64_t)ks * OZ_BK + c + h;
      const double v = (r < it.rows && l < it.k) ? it.x[r * it.rs + l * it.cs] : 0.0;
      const unsigned long long b = (unsigned long long)__double_as_longlong(v);
      const int E = (int)((b >> 52) & 0x7FF);
      const long long mant = (long long)(b & 0xFFFFFFFFFFFFFull) | (E ? (1ll << 52) : 0ll);
      // F = |v| 2^(56 - e_r) as an integer: v = mant 2^(max(E,1) - 1075)
      const int sh = (E ? E : 1) - 1019 - er;  // <= 1 by the choice of e_r: F < 2^54
      long long F = sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> -sh) : 0ll);
      if (b >> 63) F = -F;
#pragma unroll
      for (int s = 0; s < OZ_S - 1; ++s) {
        const int q = 48 - 8 * s;
        const long long dg = (F + (1ll << (q - 1))) >> q;  // nearest digit, in [-128, 128] ([-64, 64] for s = 0)
        F -= dg << q;
        d[h][s] = (int32_t)dg;
      }
      d[h][OZ_S - 1] = (int32_t)F;  // |F| <= 128 after six digits
    }
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) {
      // small integers are exact in bf16: the upper half of their FP32 pattern
      const uint32_t lo = __float_as_uint((float)d[0][s]) >> 16;
      const uint32_t hi = __float_as_uint((float)d[1][s]) >> 16;
      w[s][c / 2] = lo | (hi << 16);
    }
  }
  const size_t blk = ((size_t)rtile * a.ksteps + ks) * OZ_S;
  const int g = tid >> 3, r8 = tid & 7;
#pragma unroll
  for (int s = 0; s < OZ_S; ++s) {
    uint4* p = a.dig + (blk + s) * (OZ_BLOCK / 16);
    p[g * 16 + r8] = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);      // columns 0-7
    p[g * 16 + 8 + r8] = make_uint4(w[s][4], w[s][5], w[s][6], w[s][7]);  // columns 8-15
  }
}

// ---- products --------------------------------------------------------------------------
// One product of a launch: C (m x n; (i, j) at c[i*c_rs + j*c_cs]) from the digit row tiles
// arow0.. (A) and brow0.. (B); its output tiles are tile0 .. tile0 + ceil(m/128) tiles_n - 1.
struct OzItem {
  double* c;
  int64_t c_rs, c_cs;
  int m, n;
  int arow0, brow0;
  int tiles_n;
  int tile0;
};

struct OzGemmArgs {
  const uint8_t* dig;    // digit blocks [row tile][K step][digit]
  const int32_t* ex;     // row exponents [row tile][128]
  const OzItem* items;   // device array, or nullptr: `one`
  int nitems;
  OzItem one;
  int ntiles;            // output tiles of all items
  int ksteps;
  int chunk;             // K steps per exact accumulation
  double alpha, beta;
  int lower;             // write only i >= j
  int drop_stage;        // test switch (FG_OZ_TEST_DROP_STAGE): CTA 0 never issues this stage's copies
  int* err;
};

__device__ __forceinline__ OzItem item_of(const OzGemmArgs& g, int t) {
  if (!g.items) return g.one;
  int lo = 0, hi = g.nitems - 1;  // last item with tile0 <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.items[mid].tile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  return g.items[lo];
}

// x 2^off as FP64, for |x| < 2^53 (exact), by integer operations on the bit pattern (no
// FP64 operation); false if the result would leave the normal FP64 range.
__device__ __forceinline__ bool i64_to_f64(long long x, int off, double& d) {
  if (x == 0) {
    d = 0.0;
    return true;
  }
  const unsigned long long sgn = x < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
  const int lz = __clzll((long long)a);
  const int be = (63 - lz) + 1023 + off;
  if (be < 1 || be > 2046) return false;
  const unsigned long long mant = (a << (lz + 1)) >> 12;  // the bits after the leading one
  d = __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | mant));
  return true;
}

// d 2^off by adding off to the exponent field; false if d or the result is not a normal
// FP64 number (zero passes).
__device__ __forceinline__ bool scale_f64(double d, int off, double& r) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF);
  if ((b << 1) == 0) {
    r = d;
    return true;
  }
  if (e == 0 || e == 0x7FF || e + off < 1 || e + off > 2046) return false;
  r = __longlong_as_double((long long)(b + ((unsigned long long)(long long)off << 52)));
  return true;
}

// out-of-range fallback of scale_f64 (kept out of line: it costs FP64 operations)
__device__ __noinline__ double scale_slow(double d, int off) { return ldexp(d, off); }

// Persistent: CTA b takes the output tiles b, b + gridDim.x, ... of all items (tiles above
// the diagonal skipped when lower).  The accumulators are released as soon as the epilogue
// has read them, so the next tile's MMAs run while the epilogue writes C.
template <int BN>
__global__ void __launch_bounds__(OZ_THREADS, 1) k_oz_gemm(OzGemmArgs g) {
  using T = OzT<BN>;
  constexpr int OZ_NBUF = T::NBUF;
  extern __shared__ __align__(1024) uint8_t oz_smem[];
  __shared__ __align__(8) uint64_t bar_full[OZ_MAXBUF], bar_empty[OZ_MAXBUF], bar_acc_full[2], bar_acc_empty[2];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = g.ntiles;
  // tile t of item it: local tile lt = t - tile0, row tile lt / tiles_n, column tile lt % tiles_n
  auto valid = [&](int t) {
    if (!g.lower) return true;
    const OzItem it = item_of(g, t);
    const int lt = t - it.tile0;
    return (lt % it.tiles_n) * BN <= (lt / it.tiles_n) * OZ_BM + OZ_BM - 1;
  };
  auto next_tile = [&](int t) {
    for (t += gridDim.x; t < ntiles && !valid(t); t += gridDim.x) {
    }
    return t;
  };
  const int first = valid(blockIdx.x) ? (int)blockIdx.x : next_tile(blockIdx.x);
  if (first >= ntiles) return;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(OZ_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    if (lane == 0) {
      for (int i = 0; i < OZ_NBUF; ++i) {
        mbar_init(smem_u32(&bar_full[i]), 1);
        mbar_init(smem_u32(&bar_empty[i]), 1);
      }
      for (int z = 0; z < 2; ++z) {
        mbar_init(smem_u32(&bar_acc_full[z]), 1);
        mbar_init(smem_u32(&bar_acc_empty[z]), OZ_THREADS - 32);
      }
      abort_flag = 0;
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int KS = g.ksteps;
  const int nchunks = (KS + g.chunk - 1) / g.chunk;

  if (warp == 0) {
    if (lane == 0) {
      const uint32_t sbase = smem_u32(oz_smem);
      // producer cursor: tile pt (its digit rows pa, pb and half), K step pks, stage counter pgs
      int pt = first, pks = 0, pgs = 0;
      const uint8_t *pa = nullptr, *pb = nullptr;
      auto locate = [&]() {
        if (pt >= ntiles) return;
        const OzItem it = item_of(g, pt);
        const int lt = pt - it.tile0, rt = lt / it.tiles_n, ct = lt % it.tiles_n;
        pa = g.dig + (size_t)(it.arow0 + rt) * KS * OZ_A_BYTES;
        pb = g.dig + (size_t)(it.brow0 + ct / T::QB) * KS * OZ_A_BYTES + (size_t)(ct % T::QB) * T::B_DIGIT;
      };
      locate();
      auto produce = [&]() -> bool {
        if (pt >= ntiles) return true;
        const int buf = pgs % OZ_NBUF;
        if (pgs >= OZ_NBUF && !mbar_wait(smem_u32(&bar_empty[buf]), ((pgs / OZ_NBUF) - 1) & 1, &abort_flag, g.err))
          return false;
        const uint32_t full = smem_u32(&bar_full[buf]);
        const uint32_t dst = sbase + buf * T::STAGE;
        mbar_expect_tx(full, T::STAGE);
        if (!(blockIdx.x == 0 && pgs == g.drop_stage)) {
          bulk_g2s(dst, pa + (size_t)pks * OZ_A_BYTES, OZ_A_BYTES, full);
          for (int t = 0; t < OZ_S; ++t)
            bulk_g2s(dst + OZ_A_BYTES + t * T::B_DIGIT, pb + ((size_t)pks * OZ_S + t) * OZ_BLOCK, T::B_DIGIT, full);
        }
        ++pgs;
        if (++pks == KS) {
          pks = 0;
          pt = next_tile(pt);
          locate();
        }
        return true;
      };
      bool ok = true;
      for (int p = 0; p < OZ_NBUF - 1 && ok; ++p) ok = produce();
      int gs = 0, gc = 0;
      for (int t = first; t < ntiles && ok; t = next_tile(t)) {
        for (int ks = 0; ks < KS && ok; ++ks) {
          const int kin = ks % g.chunk;
          const int buf = gs % OZ_NBUF;
          const int z = gc % T::NSET;  // accumulator set of this chunk
          if (kin == 0 && gc >= T::NSET &&
              !mbar_wait(smem_u32(&bar_acc_empty[z]), ((gc / T::NSET) - 1) & 1, &abort_flag, g.err)) {
            ok = false;
            break;
          }
          if (!mbar_wait(smem_u32(&bar_full[buf]), (gs / OZ_NBUF) & 1, &abort_flag, g.err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = sbase + buf * T::STAGE, sb = sa + OZ_A_BYTES;
          const uint64_t da = smem_desc(sa), db = smem_desc(sb);
          const uint32_t tacc = tmem + z * (OZ_NACC * BN);
#pragma unroll
          for (int kk = 0; kk < OZ_NACC; ++kk)
#pragma unroll
            for (int s = (kk > OZ_S - 1 ? kk - (OZ_S - 1) : 0); s <= (kk < OZ_S - 1 ? kk : OZ_S - 1); ++s)
              // start-address field in 16-byte units; the first pair of a class starts the chunk's sum
              tc_mma(tacc + kk * BN, da + (uint64_t)(s * (OZ_BLOCK >> 4)),
                     db + (uint64_t)((kk - s) * (T::B_DIGIT >> 4)), T::IDESC,
                     (kin > 0 || s > (kk > OZ_S - 1 ? kk - (OZ_S - 1) : 0)) ? 1u : 0u);
          tc_commit(smem_u32(&bar_empty[buf]));
          if (kin == g.chunk - 1 || ks == KS - 1) {
            tc_commit(smem_u32(&bar_acc_full[z]));
            ++gc;
          }
          ++gs;
          ok = produce();
        }
      }
      if (!ok) {
        // drain: the stages whose copies were issued but not consumed, then every MMA issued
        for (int q = gs; q < pgs; ++q) mbar_drain(smem_u32(&bar_full[q % OZ_NBUF]), (q / OZ_NBUF) & 1);
        if (gs > 0) mbar_drain(smem_u32(&bar_empty[(gs - 1) % OZ_NBUF]), ((gs - 1) / OZ_NBUF) & 1);
      }
    }
    __syncwarp();
  } else {
    // epilogue: warps 1-8; warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows), columns
    // EPI h .. EPI h + EPI - 1 with h = (w - 1) / 4
    constexpr int OZ_EPI_COLS = T::EPI;
    const int quarter = warp & 3, half = (warp - 1) >> 2;
    const int row = quarter * 32 + lane;
    const uint32_t trow0 = tmem + ((uint32_t)(quarter * 32) << 16) + half * OZ_EPI_COLS;
    // alpha, beta cases as integers, decided once (an FP64 compare per element would cost as
    // much as the element's arithmetic)
    const int amode = g.alpha == -1.0 ? 0 : (g.alpha == 1.0 ? 1 : 2);
    const int bmode = g.beta == 0.0 ? 0 : (g.beta == 1.0 ? 1 : 2);
    int gc = 0;
    for (int t = first; t < ntiles; t = next_tile(t)) {
      // per column: sum over K chunks of the chunk's product / 2^(e_i + f_j - 16), in FP64
      double acc[OZ_EPI_COLS];
#pragma unroll
      for (int j = 0; j < OZ_EPI_COLS; ++j) acc[j] = 0.0;
      bool ok = true;
      for (int chunk = 0; chunk < nchunks; ++chunk, ++gc) {
        const int z = gc % T::NSET;
        if (!mbar_wait(smem_u32(&bar_acc_full[z]), (gc / T::NSET) & 1, &abort_flag, g.err)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t trow = trow0 + z * (OZ_NACC * BN);
#pragma unroll
        for (int cb = 0; cb < OZ_EPI_COLS / 8; ++cb) {
          // sum_k v_k 2^(-8k) exactly: every v_k is an integer below 2^24 held in FP32; hi in
          // units of 2^-16 (classes 0-2), lo in units of 2^-56 (classes 3-7), loaded four
          // classes at a time
          long long hi[8], lo[8];
#pragma unroll
          for (int part = 0; part < 2; ++part) {
            uint32_t v[OZ_NACC / 2][8];
#pragma unroll
            for (int q = 0; q < OZ_NACC / 2; ++q) tc_ld8(trow + (part * 4 + q) * BN + cb * 8, v[q]);
            tc_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              int a[OZ_NACC / 2];
#pragma unroll
              for (int q = 0; q < OZ_NACC / 2; ++q) a[q] = __float2int_rn(__uint_as_float(v[q][j]));
              if (part == 0) {
                hi[j] = (long long)a[0] * 65536 + (long long)a[1] * 256 + a[2];
                lo[j] = (long long)a[3] * 4294967296ll;
              } else {
                lo[j] += (long long)a[0] * 16777216 + (long long)a[1] * 65536 + (long long)a[2] * 256 + a[3];
              }
            }
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            // |hi| < 2^42 and |lo| < 2^57: move lo's bits above 2^40 into hi, then both
            // convert exactly (bit arithmetic); one FP64 rounding for the chunk
            const long long carry = lo[j] >> 40;
            double xh, xl;
            i64_to_f64(hi[j] + carry, -16, xh);
            i64_to_f64(lo[j] - carry * 1099511627776ll, -56, xl);
            acc[cb * 8 + j] = chunk == 0 ? xh + xl : acc[cb * 8 + j] + (xh + xl);
          }
        }
        tc_fence_before();
        mbar_arrive(smem_u32(&bar_acc_empty[z]));  // accumulators free: the next MMAs may start
      }
      if (!ok) break;
      const OzItem it = item_of(g, t);
      const int lt = t - it.tile0, rt = lt / it.tiles_n, ct = lt % it.tiles_n;
      const int i = rt * OZ_BM + row;
      const bool row_ok = i < it.m;
      const int ei = g.ex[(int64_t)(it.arow0 + rt) * OZ_BM + row];
      const int c0 = ct * BN + half * OZ_EPI_COLS;
      // lane j < EPI holds the exponent of column c0 + j (padding rows of the exponents are 0)
      const int ecol = g.ex[(int64_t)(it.brow0 + ct / T::QB) * OZ_BM + (ct % T::QB) * BN + half * OZ_EPI_COLS +
                            (lane < OZ_EPI_COLS ? lane : 0)];
      double* crow = it.c + (int64_t)i * it.c_rs;
#pragma unroll
      for (int j0 = 0; j0 < OZ_EPI_COLS; j0 += 8) {
        // eight columns at a time: their exponents and C values are loaded before any store
        int off[8];
        double cv[8];
        bool w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int col = c0 + j0 + j;
          w[j] = row_ok && col < it.n && !(g.lower && col > i);
          off[j] = ei + __shfl_sync(0xffffffffu, ecol, j0 + j);
          cv[j] = (w[j] && bmode != 0) ? crow[(int64_t)col * it.c_cs] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (!w[j]) continue;
          // product = 2^(e_i + f_j - 16) acc: a power of two, applied to the exponent field
          double x;
          if (!scale_f64(acc[j0 + j], off[j] - 16, x)) x = scale_slow(acc[j0 + j], off[j] - 16);
          double r;
          if (bmode == 0) {
            r = amode == 0 ? -x : (amode == 1 ? x : g.alpha * x);
          } else {
            const double base = bmode == 1 ? cv[j] : g.beta * cv[j];
            r = amode == 0 ? base - x : (amode == 1 ? base + x : fma(g.alpha, x, base));
          }
          crow[(int64_t)(c0 + j0 + j) * it.c_cs] = r;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS) : "memory");
  }
}

// k = 0: C = beta C (the product is empty).
__global__ void k_oz_scale(int64_t m, int64_t n, double beta, double* c, int64_t c_rs, int64_t c_cs, int lower) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  const int64_t i = idx % m, j = idx / m;
  if (lower && j > i) return;
  double* cp = c + i * c_rs + j * c_cs;
  *cp = beta == 0.0 ? 0.0 : beta * *cp;
}

static int64_t rtiles_of(int64_t rows) { return (rows + OZ_BM - 1) / OZ_BM; }

size_t ozaki_workspace_bytes(int64_t m, int64_t n, int64_t k, bool same) {
  const int64_t rt = rtiles_of(m) + (same ? 0 : rtiles_of(n));
  const int64_t ks = std::max<int64_t>(1, (k + OZ_BK - 1) / OZ_BK);
  return (size_t)rt * ks * OZ_A_BYTES + (size_t)rt * OZ_BM * sizeof(int32_t) + 256;
}

// output tile width: 64 (default) or 32 (FG_OZ_BN=32: two accumulator sets)
static int oz_bn() {
  static const int bn = [] {
    const char* e = std::getenv("FG_OZ_BN");
    return (e && std::atoi(e) == 32) ? 32 : 64;
  }();
  return bn;
}

template <int BN>
static fg_status oz_gemm_launch(fg_ctx* ctx, cudaStream_t st, OzGemmArgs& g, int64_t ntiles) {
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_oz_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)OzT<BN>::SMEM));
  // persistent: one CTA per SM (the shared memory allows no second), at most one per tile
  k_oz_gemm<BN><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ntiles, ctx->sm_count)), OZ_THREADS,
                  OzT<BN>::SMEM, st>>>(g);
  return FG_OK;
}

static fg_status oz_launch(fg_ctx* ctx, cudaStream_t st, OzSplitArgs& sa, int64_t rtiles, OzGemmArgs& g,
                           int64_t ntiles) {
  // test switch for the failure-detection test: a stage whose copies never arrive makes the
  // bounded wait run out (FG_ERR_TIMEOUT) without a fault
  const char* drop = std::getenv("FG_OZ_TEST_DROP_STAGE");
  g.drop_stage = drop ? std::atoi(drop) : -1;
  k_oz_rowexp<<<dim3((unsigned)rtiles, 32), OZ_BM, 0, st>>>(sa);
  k_oz_split<<<dim3((unsigned)rtiles, (unsigned)sa.ksteps), OZ_BM, 0, st>>>(sa);
  FG_TRY(oz_bn() == 32 ? oz_gemm_launch<32>(ctx, st, g, ntiles) : oz_gemm_launch<64>(ctx, st, g, ntiles));
  ctx->launches += 3;
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

// C = alpha A B^T + beta C (lower: only i >= j).  B == nullptr: B = A (same strides).
fg_status ozaki_gemm_nt(fg_ctx* ctx, cudaStream_t st, int64_t m, int64_t n, int64_t k, double alpha,
                        const double* A, int64_t a_rs, int64_t a_cs, const double* B, int64_t b_rs, int64_t b_cs,
                        double beta, double* C, int64_t c_rs, int64_t c_cs, bool lower, void* work, int* d_err) {
  if (m <= 0 || n <= 0) return FG_OK;
  if (k <= 0) {
    if (beta != 1.0) {
      k_oz_scale<<<(unsigned)((m * n + 255) / 256), 256, 0, st>>>(m, n, beta, C, c_rs, c_cs, lower ? 1 : 0);
      ctx->launches += 1;
      FG_CUDA_TRY(cudaGetLastError());
    }
    return FG_OK;
  }
  const bool same = B == nullptr;
  const int64_t ksteps = (k + OZ_BK - 1) / OZ_BK;
  const int64_t rta = rtiles_of(m), rtb = same ? 0 : rtiles_of(n);
  const int64_t tiles_n = (n + oz_bn() - 1) / oz_bn();
  if (rta * tiles_n > (1ll << 31) - 1 || rta + rtb > (1ll << 31) - 1 || ksteps > 65535) {
    set_error("ozaki_gemm_nt: %lld x %lld x %lld is too large", (long long)m, (long long)n, (long long)k);
    return FG_ERR_UNSUPPORTED;
  }
  OzSplitArgs sa;
  sa.items = nullptr;
  sa.nitems = 0;
  sa.one[0] = OzSplit{A, a_rs, a_cs, (int)m, (int)k, 0};
  sa.one[1] = OzSplit{B, b_rs, b_cs, (int)n, (int)k, (int)rta};
  sa.none = same ? 1 : 2;
  sa.ksteps = (int)ksteps;
  sa.dig = (uint4*)work;
  sa.ex = (int32_t*)((uint8_t*)work + (size_t)(rta + rtb) * ksteps * OZ_A_BYTES);
  OzGemmArgs g;
  g.dig = (const uint8_t*)work;
  g.ex = sa.ex;
  g.items = nullptr;
  g.nitems = 1;
  g.one = OzItem{C, c_rs, c_cs, (int)m, (int)n, 0, same ? 0 : (int)rta, (int)tiles_n, 0};
  g.ntiles = (int)(rta * tiles_n);
  g.ksteps = (int)ksteps;
  g.chunk = k <= OZ_KEXACT ? (int)ksteps : OZ_CHUNK_STEPS;
  g.alpha = alpha;
  g.beta = beta;
  g.lower = lower ? 1 : 0;
  g.err = d_err;
  return oz_launch(ctx, st, sa, rta + rtb, g, rta * tiles_n);
}

// Batch of lower updates C_b -= P_b P_b^T, P_b m_b x k_b (k_b <= 128), all column-major.
size_t ozaki_syrk_batch_bytes(const std::vector<OzSyrk>& b) {
  int64_t rt = 0;
  for (const auto& x : b) rt += rtiles_of(x.m);
  return (size_t)rt * (128 / OZ_BK) * OZ_A_BYTES + (size_t)rt * OZ_BM * sizeof(int32_t) +
         b.size() * (sizeof(OzSplit) + sizeof(OzItem)) + 512;
}

fg_status ozaki_syrk_batch(fg_ctx* ctx, cudaStream_t st, const std::vector<OzSyrk>& b, void* work, size_t bytes,
                           int* d_err) {
  std::vector<OzSplit> hs;
  std::vector<OzItem> hi;
  int64_t rt = 0, tiles = 0;
  for (const auto& x : b) {
    if (x.m <= 0 || x.k <= 0) continue;
    if (x.k > 128) {
      set_error("ozaki_syrk_batch: k = %d > 128", x.k);
      return FG_ERR_UNSUPPORTED;
    }
    const int64_t tn = (x.m + oz_bn() - 1) / oz_bn();
    hs.push_back(OzSplit{x.p, 1, x.ld, x.m, x.k, (int)rt});
    hi.push_back(OzItem{x.c, 1, x.ld, x.m, x.m, (int)rt, (int)rt, (int)tn, (int)tiles});
    rt += rtiles_of(x.m);
    tiles += rtiles_of(x.m) * tn;
  }
  if (hs.empty()) return FG_OK;
  if (tiles > (1ll << 31) - 1 || ozaki_syrk_batch_bytes(b) > bytes) {
    set_error("ozaki_syrk_batch: workspace too small or too many tiles");
    return FG_ERR_UNSUPPORTED;
  }
  const int ksteps = 128 / OZ_BK;
  uint8_t* w = (uint8_t*)work;
  const size_t dig_bytes = (size_t)rt * ksteps * OZ_A_BYTES;
  int32_t* ex = (int32_t*)(w + dig_bytes);
  uint8_t* tail = (uint8_t*)ex + (size_t)rt * OZ_BM * sizeof(int32_t);
  tail = (uint8_t*)(((uintptr_t)tail + 255) & ~(uintptr_t)255);
  OzSplit* ds = (OzSplit*)tail;
  OzItem* di = (OzItem*)(tail + ((hs.size() * sizeof(OzSplit) + 255) / 256) * 256);
  FG_CUDA_TRY(cudaMemcpyAsync(ds, hs.data(), hs.size() * sizeof(OzSplit), cudaMemcpyHostToDevice, st));
  FG_CUDA_TRY(cudaMemcpyAsync(di, hi.data(), hi.size() * sizeof(OzItem), cudaMemcpyHostToDevice, st));
  OzSplitArgs sa;
  sa.items = ds;
  sa.nitems = (int)hs.size();
  sa.none = 0;
  sa.ksteps = ksteps;
  sa.dig = (uint4*)w;
  sa.ex = ex;
  OzGemmArgs g;
  g.dig = w;
  g.ex = ex;
  g.items = di;
  g.nitems = (int)hi.size();
  g.ntiles = (int)tiles;
  g.ksteps = ksteps;
  g.chunk = ksteps;  // k <= 128 <= OZ_KEXACT
  g.alpha = -1.0;
  g.beta = 1.0;
  g.lower = 1;
  g.err = d_err;
  return oz_launch(ctx, st, sa, rt, g, tiles);
}

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_dense_gemm_nt(fg_ctx* ctx, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                           int64_t a_rs, int64_t a_cs, const double* B, int64_t b_rs, int64_t b_cs, double beta,
                           double* C, int64_t c_rs, int64_t c_cs, int32_t flags) {
  if (!ctx || (!A && k > 0) || !C || m < 0 || n < 0 || k < 0 || (flags & ~FG_DENSE_LOWER) ||
      (!B && n != m && k > 0)) {
    set_error("bad argument: ctx/A/C/m/n/k/flags (B = NULL needs n = m)");
    return FG_ERR_BADARG;
  }
  if (m > (1ll << 31) - 1 || n > (1ll << 31) - 1) {
    set_error("bad argument: m, n < 2^31");
    return FG_ERR_BADARG;
  }
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (m == 0 || n == 0) return FG_OK;
  void* work = nullptr;
  FG_TRY(dev_alloc(ctx, &work, ozaki_workspace_bytes(m, n, k, B == nullptr) + 16));
  int* d_err = (int*)((uint8_t*)work + ozaki_workspace_bytes(m, n, k, B == nullptr));
  fg_status s = FG_OK;
  int h_err = 0;
  cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess) {
    s = ozaki_gemm_nt(ctx, ctx->stream, m, n, k, alpha, A, a_rs, a_cs, B, b_rs, b_cs, beta, C, c_rs, c_cs,
                      (flags & FG_DENSE_LOWER) != 0, work, d_err);
    if (s == FG_OK) e = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (s == FG_OK && e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  }
  dev_free(ctx, work);
  if (s != FG_OK) return s;
  if (e != cudaSuccess) {
    set_error("fg_dense_gemm_nt: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  if (h_err) {
    set_error("fg_dense_gemm_nt: a bounded tensor-core wait ran out");
    return (fg_status)h_err;
  }
  return FG_OK;
}

}  // extern "C"
