// The FP32 Legendre contraction on the 5th-generation tensor cores
// (tcgen05, sm_103a): C(i, n) (+)= sum_k A(i, k) B(k, n) for a batch of
// items, as three TF32 products per K step (A_hi B_hi + A_hi B_lo + A_lo B_hi,
// the "3xTF32" split, about FP32 accuracy) accumulated in FP32 in tensor
// memory. A's split is precomputed (the table); B's is made by a split pass
// before the contraction.
#pragma once

#include "common.cuh"
#include "sht.cuh"

namespace sl3dgpu {

// The largest N (real columns) one tile holds; wider items take several
// tiles along N.
constexpr int kTcTileN = 256;

// items: device array of count GemmItems (a, b, c offsets in floats);
// maxM / maxN: the largest M and N over the items (the grid's extent).
// errorFlag: a device int set non-zero if a tensor-core completion wait
// gives up (the launch then leaves C unspecified and the caller reports it).
// A and B come split (hi, lo); the shared memory is three staged steps of
// A (2 x 8 KB) and B (2 x N x 64 B), at most 147 KB.
int RunGemmTc(const GemmItem* items, int count, int maxM, int maxN, const float* aHi, const float* aLo,
              const float* bHi, const float* bLo, float* C, bool accumulate, int* errorFlag, cudaStream_t stream);

// hi = x rounded to TF32, lo = x - hi (both stored as FP32), elementwise.
void LaunchSplitTf32(long long n, const float* x, float* hi, float* lo, cudaStream_t stream);
// The split of `width` values from each of `rows` rows `ld` apart (the same
// offsets in hi and lo).
void LaunchSplitTf32Rows(long long rows, int width, long long ld, const float* x, float* hi, float* lo,
                         cudaStream_t stream);
// The same from FP64 values (the Legendre table): lo = FP32 of x - hi.
void LaunchSplitTf32(long long n, const double* x, float* hi, float* lo, cudaStream_t stream);

}  // namespace sl3dgpu
