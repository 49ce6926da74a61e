// The FP32 Legendre contraction on the 5th-generation tensor cores
// (tcgen05, sm_103a): C(i, n) (+)= sum_k A(i, k) B(k, n) for a batch of
// items, as three TF32 products per K slice (A_hi B_hi + A_hi B_lo + A_lo B_hi,
// the "3xTF32" split, about FP32 accuracy) accumulated in FP32 in tensor
// memory.
//
// Both operands reach shared memory by TMA bulk copies of ready-made tiles:
// A (the Legendre table) is pre-tiled once per (spin, direction) into
// "panels" of 128 x 16 tiles in the canonical K-major core-matrix layout,
// high part then low part; B is packed per call the same way (tileN x 16
// tiles) by a split-and-pack pass.
#pragma once

#include "common.cuh"
#include "sht.cuh"

namespace sl3dgpu {

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
// The contraction: per CTA one (128-row tile, item, column tile).
// errorFlag: a device int set non-zero if a completion wait gives up (the
// launch then leaves C unspecified and the caller reports it).
int RunGemmTc(const TcItem* tcItems, int count, int maxMTiles, int maxNTiles, int tileN, const float* panels,
              const float* packed, float* C, bool accumulate, int* errorFlag, cudaStream_t stream);

}  // namespace sl3dgpu
