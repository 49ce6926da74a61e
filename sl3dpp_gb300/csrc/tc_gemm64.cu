// The FP64 Legendre contraction emulated on the tcgen05 tensor cores (see
// tc_gemm.cuh): C(i, n) (+)= sum_k A(i, k) B(k, n) in FP64 from exact BF16
// slice products (the Ozaki splitting).
//
// Splitting. Row i of A has the exponent e_i with max_k |A(i, k)| < 2^{e_i},
// column n of B the exponent f_n likewise; x = A(i, k) 2^{-e_i} (|x| < 1) is
// rounded to X = round(x 2^49), an integer below 2^49 read off the double's
// bits, and X is written in balanced base-2^7 digits,
// X = sum_{p < 7} s_p 2^{7 (6 - p)}, |s_p| <= 64 for p > 0 and |s_0| <= 128:
// x = sum_p s_p 2^{-7 (p + 1)} to within 2^{-50}. Integer arithmetic only
// (the FP64 units of this part are slow); the digits are exact in BF16.
//
// Products. Level d = p + q gathers sum_k s_p(A) s_q(B) over p + q = d, at
// most (d + 3) 2^12 per k in magnitude, so below 2^24 -- exact in the FP32
// accumulator -- for K <= 455 at d = 6. The levels d < 7 are kept (28
// products per 16-deep step) and joined exactly as integers,
// H = acc_0 2^14 + acc_1 2^7 + acc_2 and L = acc_3 2^21 + acc_4 2^14 +
// acc_5 2^7 + acc_6, and C(i, n) = 2^{e_i + f_n} (2^{-28} H + 2^{-56} L) is
// rounded once to FP64 from that exact integer, by integer arithmetic.
//
// Kernel. One CTA of eight warps per (64-column tile, 128-row tile, item),
// the column tiles of a row tile adjacent in the launch so that its A panel
// is read from HBM once. One elected thread runs the K loop as the FP32
// contraction does (tc_gemm.cu): it arms a stage's "full" mbarrier, issues
// two TMA bulk copies (A's seven slices, 28 KB; B's, 14 KB), four stages in
// flight, and when they have landed issues the step's tcgen05.mma kind::f16
// into the level accumulators (tensor-memory columns 64 d .. 64 d + 63 of
// 512) and commits them to the stage's "empty" mbarrier. B's seven slices
// are stored as one 448-row operand, slice q in rows 64 q .. 64 q + 63, so
// that one MMA of N = 64 c multiplies A's slice p by c consecutive slices
// q0 .. q0 + c - 1 into the c consecutive levels p + q0 ..: the 28 products
// of a step take 10 MMAs of N up to 256 rather than 28 of N = 64 (the same
// tensor work, in fewer instructions for the one issuing thread). Every wait
// has an iteration limit. The epilogue reads the seven levels with
// tcgen05.ld, two warps per lane quarter (a column half each), joins them in
// FP64 and stores (or adds) the rows in range.
#include <cstdint>

#include "profile.cuh"
#include "tc_gemm.cuh"

namespace sl3dgpu {
namespace {

constexpr int kSlices = kTc64Slices;
constexpr int kTileN = kTc64TileN;
constexpr int kStages = 4;
constexpr int kThreads = 256;  // eight warps: two per tensor-memory lane quarter in the epilogue
constexpr int kATile = kTcTileM * kTcTileK;  // BF16 values of one slice of an A tile: 2048 (4 KB)
constexpr int kBTile = kTileN * kTcTileK;    // of a B tile: 1024 (2 KB)
constexpr int kBRows = kSlices * kTileN;     // B's slices as one operand of 448 rows
constexpr int kBSlice = kTileN * 8;          // BF16 offset of the next slice's rows (8 row groups of 64)
constexpr uint32_t kTmemColumns = 512;       // 7 levels x 64 columns, rounded up to a power of two

static_assert(kSlices * kTileN <= static_cast<int>(kTmemColumns), "the levels fit in tensor memory");

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M.
__host__ __device__ constexpr uint32_t InstrDescriptorBf16(int n, int m) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

// The BF16 bits of an integer of magnitude at most 256 (exact: its float has
// at most eight significant bits, all in the upper half).
__device__ inline uint32_t Bf16Bits(int integer) { return __float_as_uint(static_cast<float>(integer)) >> 16; }

// The exponent e with |v| < 2^e for the largest |v| of a set, from the
// largest magnitude's bits (0 for zero; subnormals count as below 2^-1022).
__device__ inline int ExponentAbove(unsigned long long magnitudeBits) {
  if (magnitudeBits == 0) return 0;
  const int biased = static_cast<int>(magnitudeBits >> 52);
  return biased == 0 ? -1022 : biased - 1022;
}

// v (|v| < 2^e) as kSlices balanced base-2^7 digits of round(v 2^{49 - e}),
// packed as BF16 bits.
__device__ inline void Split(double v, int e, uint32_t (&s)[kSlices]) {
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(v));
  const int biased = static_cast<int>((bits >> 52) & 0x7FF);
  const long long mantissa = static_cast<long long>(bits & ((1ULL << 52) - 1)) | (biased ? (1LL << 52) : 0LL);
  // v = mantissa 2^{E - 52}, E <= e - 1, so X = mantissa 2^{E - e - 3}: a
  // right shift by t >= 4, rounded to nearest
  const int E = biased ? biased - 1023 : -1022;
  const int t = e - E + 3;
  long long X = 0;
  if (t < 63) X = (mantissa + (1LL << (t - 1))) >> t;
  if (bits >> 63) X = -X;
#pragma unroll
  for (int p = kSlices - 1; p > 0; --p) {
    int r = static_cast<int>(X & 127);
    if (r >= 64) r -= 128;
    s[p] = Bf16Bits(r);
    X = (X - r) >> 7;
  }
  s[0] = Bf16Bits(static_cast<int>(X));
}

// (H 2^28 + L) 2^(scale - 56) as a double, rounded to nearest even, by
// integer arithmetic (the exact 128-bit integer's top 53 bits and its
// exponent written into the bits); values outside the normal range take the
// slow path through ldexp.
__device__ inline double JoinToDouble(long long H, long long L, int scale) {
  const __int128 T = (static_cast<__int128>(H) << 28) + L;
  if (T == 0) return 0.0;
  const bool negative = T < 0;
  const unsigned __int128 m = negative ? -static_cast<unsigned __int128>(T) : static_cast<unsigned __int128>(T);
  const unsigned long long top = static_cast<unsigned long long>(m >> 64), low = static_cast<unsigned long long>(m);
  const int bits = top ? 128 - __clzll(top) : 64 - __clzll(low);  // the integer's bit length
  const int shift = bits - 53;
  unsigned long long mantissa;
  int exponent = bits - 1 + scale - 56;
  if (shift > 0) {
    const unsigned __int128 q = m >> shift;
    const unsigned __int128 rem = m - (q << shift), half = static_cast<unsigned __int128>(1) << (shift - 1);
    mantissa = static_cast<unsigned long long>(q);
    if (rem > half || (rem == half && (mantissa & 1))) ++mantissa;
    if (mantissa >> 53) {
      mantissa >>= 1;
      ++exponent;
    }
  } else {
    mantissa = static_cast<unsigned long long>(m) << -shift;
  }
  if (exponent < -1022 || exponent > 1023) {
    const double v = ldexp(static_cast<double>(mantissa), exponent - 52);
    return negative ? -v : v;
  }
  const unsigned long long out = (negative ? (1ULL << 63) : 0ULL) |
                                 (static_cast<unsigned long long>(exponent + 1023) << 52) |
                                 (mantissa & ((1ULL << 52) - 1));
  return __longlong_as_double(static_cast<long long>(out));
}

// Offset (in BF16 values) of element (row, k) of a K-major 16-deep tile of
// `rows` rows in the core-matrix layout [k / 8][row / 8][row % 8][k % 8].
__device__ inline int Tile16Index(int row, int k, int rows) {
  return (k >> 3) * (rows * 8) + (row >> 3) * 64 + (row & 7) * 8 + (k & 7);
}

// Eight consecutive-k slices of one row (s[q][p]: value q, slice p) stored as
// one 16-byte core-matrix row per slice.
__device__ inline void StoreSlices(uint16_t* tile, int sliceStride, int at, const uint32_t (&s)[8][kSlices]) {
#pragma unroll
  for (int p = 0; p < kSlices; ++p) {
    uint4 v;
    v.x = s[0][p] | (s[1][p] << 16);
    v.y = s[2][p] | (s[3][p] << 16);
    v.z = s[4][p] | (s[5][p] << 16);
    v.w = s[6][p] | (s[7][p] << 16);
    *reinterpret_cast<uint4*>(tile + p * sliceStride + at) = v;
  }
}

// Row exponents of A, one thread per (item, row): the maximum over the
// item's depth.
__global__ void RowExpKernel(const GemmItem* items, const Tc64Item* tcItems, const double* table, int* rowExp) {
  const GemmItem g = items[blockIdx.y];
  const Tc64Item it = tcItems[blockIdx.y];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.M; i += gridDim.x * blockDim.x) {
    unsigned long long mx = 0;
    for (int k = 0; k < g.K; ++k) {
      const double v = table[g.a + static_cast<long long>(i) * g.sAi + static_cast<long long>(k) * g.sAk];
      mx = max(mx, static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7FFFFFFFFFFFFFFFULL);
    }
    rowExp[it.rowExp + i] = ExponentAbove(mx);
  }
}

// A's panel: one thread per (item, tile, 8-deep K group, row).
__global__ void PanelA64Kernel(const GemmItem* items, const Tc64Item* tcItems, const double* table,
                               const int* rowExp, uint16_t* panels) {
  const GemmItem g = items[blockIdx.y];
  const Tc64Item it = tcItems[blockIdx.y];
  const long long total = static_cast<long long>(it.mTiles) * it.kSteps * 2 * kTcTileM;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(t % kTcTileM);
    const long long rest = t / kTcTileM;
    const int kg = static_cast<int>(rest % 2);
    const long long tile = rest / 2;
    const int ks = static_cast<int>(tile % it.kSteps), mt = static_cast<int>(tile / it.kSteps);
    const int i = mt * kTcTileM + r, k0 = ks * kTcTileK + 8 * kg;
    const int e = i < g.M ? rowExp[it.rowExp + i] : 0;
    uint32_t s[8][kSlices];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = k0 + q;
      const double v = (i < g.M && k < g.K) ? table[g.a + static_cast<long long>(i) * g.sAi +
                                                    static_cast<long long>(k) * g.sAk]
                                            : 0.0;
      Split(v, e, s[q]);
    }
    StoreSlices(panels + it.aPanel + tile * kSlices * kATile, kATile, Tile16Index(r, 8 * kg, kTcTileM), s);
  }
}

// B's column exponents and packed slices, one CTA of 256 threads per
// (column tile, item): 64 columns x 4 lanes along k. The exponents first
// (each lane's maximum over its k, then over the four lanes), then the
// slices, 8-deep k groups in turn; a warp's reads of one k are 32
// consecutive columns and its stores of one slice 512 contiguous bytes.
constexpr int kPackThreads = 256, kPackLanes = kPackThreads / kTileN;

__global__ void __launch_bounds__(kPackThreads) PackB64Kernel(const Tc64Item* tcItems, const double* B, int* colExp,
                                                              uint16_t* packed) {
  const Tc64Item it = tcItems[blockIdx.y];
  const int nt = blockIdx.x;
  if (nt >= it.nTiles) return;
  __shared__ unsigned long long largest[kPackLanes][kTileN];
  const int nn = threadIdx.x % kTileN, lane = threadIdx.x / kTileN;
  const int n = nt * kTileN + nn;
  const double* col = B + it.b + n;
  unsigned long long mx = 0;
  if (n < it.N)
    for (int k = lane; k < it.K; k += kPackLanes)
      mx = max(mx, static_cast<unsigned long long>(__double_as_longlong(col[static_cast<long long>(k) * it.ldb])) &
                       0x7FFFFFFFFFFFFFFFULL);
  largest[lane][nn] = mx;
  __syncthreads();
  for (int q = 0; q < kPackLanes; ++q) mx = max(mx, largest[q][nn]);
  const int e = ExponentAbove(mx);
  if (lane == 0 && n < it.N) colExp[it.colExp + n] = e;
  uint16_t* base = packed + it.bPack + static_cast<long long>(nt) * it.kSteps * kSlices * kBTile;
  for (int group = lane; group < 2 * it.kSteps; group += kPackLanes) {
    const int ks = group / 2, kg = group % 2, k0 = 8 * group;
    uint32_t s[8][kSlices];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = k0 + q;
      const double v = (n < it.N && k < it.K) ? col[static_cast<long long>(k) * it.ldb] : 0.0;
      Split(v, e, s[q]);
    }
    StoreSlices(base + static_cast<long long>(ks) * kSlices * kBTile, kBSlice, Tile16Index(nn, 8 * kg, kBRows), s);
  }
}

__global__ void __launch_bounds__(kThreads) TcGemm64Kernel(const Tc64Item* tcItems, const uint16_t* panels,
                                                           const uint16_t* packed, const int* rowExp,
                                                           const int* colExp, double* C, bool accumulate,
                                                           int* errorFlag) {
  const Tc64Item it = tcItems[blockIdx.z];
  const int nt = blockIdx.x, mt = blockIdx.y;
  if (mt >= it.mTiles || nt >= it.nTiles) return;  // the whole CTA, before any tensor-memory work
  const int i0 = mt * kTcTileM, n0 = nt * kTileN;
  const int nCols = min(kTileN, it.N - n0);
  constexpr uint32_t aBytes = kSlices * kATile * 2, bBytes = kSlices * kBTile * 2;

  extern __shared__ __align__(128) unsigned char tc64Smem[];
  uint16_t* sA = reinterpret_cast<uint16_t*>(tc64Smem);  // kStages x kSlices x kATile
  uint16_t* sB = sA + kStages * kSlices * kATile;          // kStages x kSlices x kBTile
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + kStages * kSlices * kBTile);
  uint64_t* empty = full + kStages;
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(empty + kStages);
  __shared__ int okShared;
  __shared__ double rowsOut[kThreads / 32][32][17];  // each warp's 32 x 16 block, padded
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(tmemSlot)),
                 "r"(kTmemColumns)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(full + s)), "r"(1) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(empty + s)), "r"(1) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmemSlot;

  if (tid == 0) {
    const uint16_t* aSrc = panels + it.aPanel + static_cast<long long>(mt) * it.kSteps * kSlices * kATile;
    const uint16_t* bSrc = packed + it.bPack + static_cast<long long>(nt) * it.kSteps * kSlices * kBTile;
    uint32_t phaseFull[kStages] = {0, 0, 0, 0}, phaseEmpty[kStages] = {0, 0, 0, 0};
    bool ok = true;
    auto issue = [&](int ks) {
      const int buf = ks % kStages;
      if (ks >= kStages) {
        ok = ok && WaitParity(SmemAddr(empty + buf), phaseEmpty[buf]);
        phaseEmpty[buf] ^= 1u;
      }
      if (!ok) return;
      const uint32_t bar = SmemAddr(full + buf);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(aBytes + bBytes)
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              SmemAddr(sA + buf * kSlices * kATile)),
          "l"(aSrc + static_cast<long long>(ks) * kSlices * kATile), "r"(aBytes), "r"(bar)
          : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              SmemAddr(sB + buf * kSlices * kBTile)),
          "l"(bSrc + static_cast<long long>(ks) * kSlices * kBTile), "r"(bBytes), "r"(bar)
          : "memory");
    };
    for (int ks = 0; ks < min(kStages - 1, it.kSteps); ++ks) issue(ks);
    for (int ks = 0; ks < it.kSteps && ok; ++ks) {
      if (ks + kStages - 1 < it.kSteps) issue(ks + kStages - 1);
      if (!ok) break;
      const int buf = ks % kStages;
      ok = WaitParity(SmemAddr(full + buf), phaseFull[buf]);
      phaseFull[buf] ^= 1u;
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t aBase = SmemAddr(sA + buf * kSlices * kATile);
      const uint32_t bBase = SmemAddr(sB + buf * kSlices * kBTile);
      constexpr uint32_t aLbo = kTcTileM * 16, bLbo = kBRows * 16, sbo = 128;
      // A's slice p against B's slices q0 .. q0 + c - 1 (c <= 4, N = 64 c),
      // levels p + q0 .. p + q0 + c - 1; p = 0 writes every level first.
#pragma unroll
      for (int p = 0; p < kSlices; ++p) {
        const uint64_t dA = Descriptor(aBase + p * kATile * 2, aLbo, sbo);
        const uint32_t enable = (ks > 0 || p > 0) ? 1u : 0u;
#pragma unroll
        for (int q0 = 0; q0 < kSlices - p; q0 += 4) {
          const int c = min(4, kSlices - p - q0);
          const uint64_t dB = Descriptor(bBase + q0 * kBSlice * 2, bLbo, sbo);
          asm volatile(
              "{\n\t.reg .pred r;\n\t"
              "setp.ne.b32 r, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, r;\n\t}" ::"r"(tmem + (p + q0) * kTileN),
              "l"(dA), "l"(dB), "r"(InstrDescriptorBf16(c * kTileN, kTcTileM)), "r"(enable)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       SmemAddr(empty + buf))
                   : "memory");
    }
    // The last step's commit covers every MMA before it.
    if (ok && it.kSteps > 0) {
      const int last = (it.kSteps - 1) % kStages;
      ok = WaitParity(SmemAddr(empty + last), phaseEmpty[last]);
    }
    okShared = ok ? 1 : 0;
    if (!ok) atomicExch(errorFlag, 1);
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (okShared) {
    // Epilogue: this warp's lane quarter (32 rows) and column half, 16
    // columns at a time, the seven levels joined as integers and rounded
    // once to FP64.
    const int quarter = warp % 4, half = warp / 4;
    const int i = i0 + 32 * quarter + lane;
    const int e = i < it.M ? rowExp[it.rowExp + i] : 0;
    for (int c0 = half * (kTileN / 2); c0 < (half + 1) * (kTileN / 2); c0 += 16) {
      uint32_t r[kSlices][16];
#pragma unroll
      for (int d = 0; d < kSlices; ++d) {
        const uint32_t addr =
            tmem + (static_cast<uint32_t>(32 * quarter) << 16) + static_cast<uint32_t>(d * kTileN + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[d][0]), "=r"(r[d][1]), "=r"(r[d][2]), "=r"(r[d][3]), "=r"(r[d][4]), "=r"(r[d][5]),
              "=r"(r[d][6]), "=r"(r[d][7]), "=r"(r[d][8]), "=r"(r[d][9]), "=r"(r[d][10]), "=r"(r[d][11]),
              "=r"(r[d][12]), "=r"(r[d][13]), "=r"(r[d][14]), "=r"(r[d][15])
            : "r"(addr)
            : "memory");
      }
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      // the joined values of this lane's row, then out through shared memory
      // so that a store instruction writes two rows' 16 consecutive columns
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int n = c0 + q;
        double v = 0.0;
        if (i < it.M && n < nCols) {
          long long acc[kSlices];
#pragma unroll
          for (int d = 0; d < kSlices; ++d) acc[d] = __float2int_rn(__uint_as_float(r[d][q]));
          const long long H = (acc[0] << 14) + (acc[1] << 7) + acc[2];
          const long long L = (acc[3] << 21) + (acc[4] << 14) + (acc[5] << 7) + acc[6];
          v = JoinToDouble(H, L, e + colExp[it.colExp + n0 + n]);
        }
        rowsOut[warp][lane][q] = v;
      }
      __syncwarp();
      const int n = c0 + (lane & 15);
      // this lane's 16 rows' old values first (loads in flight together), then the stores
      double old[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int row = i0 + 32 * quarter + 2 * q + (lane >> 4);
        old[q] = (accumulate && row < it.M && n < nCols) ? C[it.c + static_cast<long long>(row) * it.ldc + n0 + n]
                                                         : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int rr = 2 * q + (lane >> 4), row = i0 + 32 * quarter + rr;
        if (row < it.M && n < nCols)
          C[it.c + static_cast<long long>(row) * it.ldc + n0 + n] = old[q] + rowsOut[warp][rr][lane & 15];
      }
      __syncwarp();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColumns) : "memory");
}

}  // namespace

void LaunchPanelA64(const GemmItem* items, const Tc64Item* tcItems, int count, int maxM, int maxATiles,
                    const double* table, int* rowExp, uint16_t* panels, cudaStream_t stream) {
  if (count == 0) return;
  RowExpKernel<<<dim3(static_cast<unsigned>((maxM + 127) / 128), count), 128, 0, stream>>>(items, tcItems, table,
                                                                                          rowExp);
  const long long perItem = static_cast<long long>(maxATiles) * 2 * kTcTileM;
  const unsigned blocks = static_cast<unsigned>(std::min<long long>((perItem + 255) / 256, 4096));
  PanelA64Kernel<<<dim3(blocks, count), 256, 0, stream>>>(items, tcItems, table, rowExp, panels);
}

void LaunchPackB64(const Tc64Item* tcItems, int count, int maxNTiles, const double* B, int* colExp,
                   uint16_t* packed, cudaStream_t stream) {
  if (count == 0 || maxNTiles == 0) return;
  PackB64Kernel<<<dim3(static_cast<unsigned>(maxNTiles), count), kPackThreads, 0, stream>>>(tcItems, B, colExp,
                                                                                           packed);
}

int RunGemm64Tc(const Tc64Item* tcItems, int count, int maxMTiles, int maxNTiles, const uint16_t* panels,
                const uint16_t* packed, const int* rowExp, const int* colExp, double* C, bool accumulate,
                int* errorFlag, cudaStream_t stream) {
  if (count == 0 || maxMTiles == 0 || maxNTiles == 0) return SL3DGPU_OK;
  constexpr size_t smem = static_cast<size_t>(kStages) * kSlices * (kATile + kBTile) * sizeof(uint16_t) +
                          2 * kStages * sizeof(uint64_t) + 16;
  static_assert(smem <= 227 * 1024, "the stages fit in shared memory");
  SL3D_CUDA(AllowDynamicSmem(TcGemm64Kernel));
  dim3 grid(static_cast<unsigned>(maxNTiles), static_cast<unsigned>(maxMTiles), static_cast<unsigned>(count));
  TcGemm64Kernel<<<grid, kThreads, smem, stream>>>(tcItems, panels, packed, rowExp, colExp, C, accumulate,
                                                   errorFlag);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu
