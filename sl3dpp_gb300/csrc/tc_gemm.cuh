// The FP32 Legendre contraction on the 5th-generation tensor cores
// (tcgen05, sm_103a): C(i, n) (+)= sum_k A(i, k) B(k, n) for a batch of
// items, as three TF32 products per K slice (A_hi B_hi + A_hi B_lo + A_lo B_hi,
// the "3xTF32" split, about FP32 accuracy) accumulated in FP32 in tensor
// memory.
//
// A (the Legendre table) reaches shared memory by TMA bulk copies of
// ready-made tiles: pre-tiled once per (spin, direction) into "panels" of
// 128 x 16 tiles in the canonical K-major core-matrix layout, high part then
// low part. B is split and packed the same way (tileN x 16 tiles) inside the
// contraction, from its source, by two warps (or, the older form, by a
// separate split-and-pack pass through HBM).
#pragma once

#include <cstdint>

#include "common.cuh"
#include "sht.cuh"

namespace sl3dgpu {

// -- tcgen05 helpers shared by the contractions ------------------------------------------

constexpr int kTcWaitLimit = 1 << 22;  // polls of an mbarrier before a wait gives up

__device__ inline uint32_t SmemAddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor, no swizzle, K-major: start address,
// leading byte offset (between core matrices along K), stride byte offset
// (between 8-row groups along M/N), descriptor version 1.
__device__ inline uint64_t Descriptor(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// Wait for an mbarrier phase, at most kTcWaitLimit polls; false if it gave up.
__device__ inline bool WaitParity(uint32_t bar, uint32_t phase) {
  for (int i = 0; i < kTcWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

constexpr int kTcTileM = 128;  // rows per tile (the MMA's M)
constexpr int kTcTileK = 16;   // K per tile (two 8-deep MMA slices)
constexpr int kTcMaxTileN = 256;

// One item of a tensor-core batch, beside its GemmItem.
struct TcItem {
  int M, N, K, mTiles;   // rows, real columns, depth; 128-row tiles
  int kSteps, nTiles, ldc, ldb;
  long long aPanel;      // floats: the item's panel, [mTile][kStep][hi 2048 | lo 2048]
  long long bPack;       // floats: the item's packed B, [nTile][kStep][hi tileN*16 | lo tileN*16]
  long long b, c;        // floats: B's source and C's offsets
};

// Fill the items' A panels from the FP64 table (A(i, k) = table[a + i sAi +
// k sAk], zero outside M x K). maxTiles: the most (mTiles x kSteps) of an item.
void LaunchPanelA(const GemmItem* items, const TcItem* tcItems, int count, int maxTiles, const double* table,
                  float* panels, cudaStream_t stream);
// Split and pack B into the items' tiles. maxTiles: the most (nTiles x kSteps).
void LaunchPackB(const TcItem* tcItems, int count, int maxTiles, int tileN, const float* B, float* packed,
                 cudaStream_t stream);
// The contraction over a tile list ({item, row tile, column tile} per
// entry), persistent CTAs, one per SM. errorFlag: a device int set non-zero
// if a completion wait gives up (the launch then leaves C unspecified and
// the caller reports it).
// rawB non-null: B is split and packed inside the kernel from its source
// (packed is then not read); null: from the packed tiles (LaunchPackB).
int RunGemmTc(const TcItem* tcItems, const int4* tiles, int tileCount, int tileN, const float* panels,
              const float* packed, const float* rawB, float* C, bool accumulate, int* errorFlag,
              cudaStream_t stream);

// -- FP64 emulated on the tensor cores (tc_gemm64.cu) ------------------------------------
//
// The FP64 contraction as exact BF16 products: A's rows and B's columns are
// scaled by powers of two to |x| < 1 and split into kTc64Slices integer
// slices of at most 7 bits, x = sum_p s_p 2^{-7 (p + 1)} (the Ozaki
// splitting); the slice products of each level d = p + q < kTc64Slices are
// accumulated in FP32 by tcgen05.mma kind::f16, exactly (integers below 2^24
// for K <= 455), and the levels are joined in FP64. About 49 bits of each
// value enter, so the result carries FP64-level accuracy relative to
// (row maximum) x (column maximum) x K.
constexpr int kTc64Slices = 7;
constexpr int kTc64TileN = 64;   // 7 accumulators of 64 columns in tensor memory
constexpr int kTc64MaxK = 448;   // the exactness bound on the depth, with margin

void LaunchPanelA64(const GemmItem* items, const Tc64Item* tcItems, int count, int maxM, int maxATiles,
                    const double* table, int* rowExp, uint16_t* panels, cudaStream_t stream);
void LaunchPackB64(const Tc64Item* tcItems, int count, int maxNTiles, const double* B, int* colExp,
                   uint16_t* packed, cudaStream_t stream);
int RunGemm64Tc(const Tc64Item* tcItems, int count, int maxMTiles, int maxNTiles, const uint16_t* panels,
                const uint16_t* packed, const int* rowExp, const int* colExp, double* C, bool accumulate,
                int* errorFlag, cudaStream_t stream);

}  // namespace sl3dgpu
