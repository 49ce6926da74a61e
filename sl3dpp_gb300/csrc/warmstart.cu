// The learned warm start: a small network that guesses the strain
// coefficients at the end of the next step, the start the fixed point of
// Viscoelastic3D::Step iterates from (Converge's `start`, include/sl3dpp/
// Viscoelastic3D.hpp:562-569; the plain start is the previous step's strain).
// The iteration always runs to the tolerance from the guess, and a guess whose
// first residual is not the smaller is dropped (the step's own rule), so the
// network can cost passes but never accuracy.
//
// The network. For each degree l, lateral memory node p and spin block b
// (-2, -1 and the real spin 0) the recent strain changes Delta_n, Delta_n-1,
// Delta_n-2 (one per step) over the block's orders m are summarised by their
// norms and correlations; a unit (l, p) takes those of its three blocks with
// l, the node's depth in the lateral zone, its relaxation ratio dt / tau and
// the coming load increment's ratio to the last one: 16 features. A
// multilayer perceptron (16 -> 768 -> ... -> 768 -> 16, six hidden layers,
// GELU, about 3M parameters) maps them to, per block, the coefficients of a
// linear predictor: Delta_n+1 = a Delta_n + b Delta_n-1 + c Delta_n-2 for
// every order of the block at that (l, p); the guess is s_n + Delta_n+1 at
// the lateral nodes and the extrapolation s_n + Delta_n elsewhere (where the
// lateral weight vanishes, the start does not enter the next pass). The last
// layer starts at zero and its outputs are offsets from (1, 0, 0): untrained,
// the network is the extrapolation. Evaluating it costs (lmax + 1) x lateral
// nodes rows of GEMM work, a fraction of a pass, whatever the orders.
//
// Kernels. The layers' products run on the tcgen05 tensor cores in BF16 with
// FP32 accumulation in tensor memory (NetGemmKernel: operands packed into
// K-major core-matrix tiles, TMA bulk copies into a two-stage ring, one
// thread issuing kind::f16 MMAs, four warps draining the accumulator);
// activations and the master weights are FP32; Adam updates the masters.
// Training runs forward, loss, backward and update on the GPU: the loss is
// the squared error of the predicted change over every order, relative to
// the extrapolation's, and its gradient reaches the predictor coefficients
// by sums over the orders.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <random>
#include <vector>

#include "profile.cuh"
#include "systems.cuh"
#include "tc_gemm.cuh"

namespace sl3dgpu {
namespace {

constexpr int kFeatures = 16;
constexpr int kOutputs = 16;  // 9 used: (a, b, c) per spin block
constexpr int kBlocks = 3;
constexpr int kNetTileN = 64;
constexpr int kNetStages = 2;
constexpr int kNetThreads = 128;
constexpr int kATileNet = kTcTileM * kTcTileK;   // BF16 values of an A tile: 2048
constexpr int kBTileNet = kNetTileN * kTcTileK;  // of a B tile: 1024
constexpr uint32_t kNetTmemColumns = 64;

__host__ __device__ constexpr uint32_t NetInstrDescriptor(int n, int m) {
  // kind::f16: FP32 accumulator (bit 4), BF16 A (bits 7-9 = 1) and B (10-12
  // = 1), both K-major, N / 8 and M / 16
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

// Offset of element (row, k) in a 16-deep K-major tile of `rows` rows, the
// core-matrix layout [k / 8][row / 8][row % 8][k % 8] (BF16 values).
__device__ inline int NetTileIndex(int row, int k, int rows) {
  return (k >> 3) * (rows * 8) + (row >> 3) * 64 + (row & 7) * 8 + (k & 7);
}

__device__ inline uint16_t Bf16(float x) {
  // round to nearest even (finite inputs)
  const uint32_t u = __float_as_uint(x);
  return static_cast<uint16_t>((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
}

// An operand matrix (rows x K, element (r, k) at src[r * sr + k * sk]) as
// BF16 tiles [rowTile][kStep][tileRows x 16], zero beyond its extent.
__global__ void PackKernel(const float* src, long long sr, long long sk, int rows, int K, int tileRows,
                           int rowTiles, int kSteps, uint16_t* out) {
  const long long total = static_cast<long long>(rowTiles) * kSteps * tileRows * kTcTileK;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int kk = static_cast<int>(t % kTcTileK);
    const long long rest = t / kTcTileK;
    const int rr = static_cast<int>(rest % tileRows);
    const long long tile = rest / tileRows;
    const int ks = static_cast<int>(tile % kSteps), rt = static_cast<int>(tile / kSteps);
    const int r = rt * tileRows + rr, k = ks * kTcTileK + kk;
    const float v = (r < rows && k < K) ? src[r * sr + k * sk] : 0.0f;
    out[tile * tileRows * kTcTileK + NetTileIndex(rr, kk, tileRows)] = Bf16(v);
  }
}

struct NetGemm {
  int M, N, K, mTiles, nTiles, kSteps;
  const uint16_t* A;  // [mTile][kStep][128 x 16]
  const uint16_t* B;  // [nTile][kStep][64 x 16]
  float* C;           // row-major M x N, ldc
  int ldc;
  int accumulate;
};

// C (+)= A B^T: one CTA per (64-column tile, 128-row tile). Thread 0 issues
// the copies (two stages in flight) and the MMAs; the four warps drain the
// accumulator, each its 32-lane quarter. Every wait is bounded; on giving up
// the issuing thread still waits (bounded) for the copies it issued and the
// CTA writes nothing.
__global__ void __launch_bounds__(kNetThreads) NetGemmKernel(NetGemm g, int* errorFlag) {
  const int nt = blockIdx.x, mt = blockIdx.y;
  extern __shared__ __align__(128) unsigned char netSmem[];
  uint16_t* sA = reinterpret_cast<uint16_t*>(netSmem);
  uint16_t* sB = sA + kNetStages * kATileNet;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + kNetStages * kBTileNet);
  uint64_t* empty = full + kNetStages;
  uint64_t* drain = empty + kNetStages;
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ int okShared;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(tmemSlot)),
                 "r"(kNetTmemColumns)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kNetStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(full + s)), "r"(1) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(empty + s)), "r"(1) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(drain)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmemSlot;
  constexpr uint32_t aBytes = kATileNet * 2, bBytes = kBTileNet * 2;
  if (tid == 0) {
    const uint16_t* aSrc = g.A + static_cast<long long>(mt) * g.kSteps * kATileNet;
    const uint16_t* bSrc = g.B + static_cast<long long>(nt) * g.kSteps * kBTileNet;
    uint32_t phaseFull[kNetStages] = {0, 0}, phaseEmpty[kNetStages] = {0, 0};
    bool landed[kNetStages] = {true, true};  // no copy of this stage outstanding
    bool ok = true;
    auto issue = [&](int ks) {
      const int buf = ks % kNetStages;
      if (ks >= kNetStages) {
        ok = ok && WaitParity(SmemAddr(empty + buf), phaseEmpty[buf]);
        phaseEmpty[buf] ^= 1u;
      }
      if (!ok) return;
      const uint32_t bar = SmemAddr(full + buf);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(aBytes + bBytes)
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              SmemAddr(sA + buf * kATileNet)),
          "l"(aSrc + static_cast<long long>(ks) * kATileNet), "r"(aBytes), "r"(bar)
          : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              SmemAddr(sB + buf * kBTileNet)),
          "l"(bSrc + static_cast<long long>(ks) * kBTileNet), "r"(bBytes), "r"(bar)
          : "memory");
      landed[buf] = false;
    };
    issue(0);
    bool issuedMma = false;
    for (int ks = 0; ks < g.kSteps && ok; ++ks) {
      if (ks + 1 < g.kSteps) issue(ks + 1);
      if (!ok) break;
      const int buf = ks % kNetStages;
      ok = WaitParity(SmemAddr(full + buf), phaseFull[buf]);
      phaseFull[buf] ^= 1u;
      if (!ok) break;
      landed[buf] = true;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t aBase = SmemAddr(sA + buf * kATileNet), bBase = SmemAddr(sB + buf * kBTileNet);
      // one MMA of K = 16 (two 8-deep core matrices along K)
      const uint64_t dA = Descriptor(aBase, kTcTileM * 16, 128), dB = Descriptor(bBase, kNetTileN * 16, 128);
      const uint32_t enable = ks > 0 ? 1u : 0u;
      asm volatile(
          "{\n\t.reg .pred r;\n\t"
          "setp.ne.b32 r, %4, 0;\n\t"
          "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, r;\n\t}" ::"r"(tmem),
          "l"(dA), "l"(dB), "r"(NetInstrDescriptor(kNetTileN, kTcTileM)), "r"(enable)
          : "memory");
      issuedMma = true;
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       SmemAddr(empty + buf))
                   : "memory");
    }
    // every MMA issued has completed before the accumulator is read or
    // tensor memory freed (a commit arrives once all earlier MMAs are done)
    if (issuedMma) {
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       SmemAddr(drain))
                   : "memory");
      ok = WaitParity(SmemAddr(drain), 0) && ok;
    }
    if (!ok) {
      // gave up: let the copies in flight land (bounded) before the CTA ends
      for (int s = 0; s < kNetStages; ++s)
        if (!landed[s]) WaitParity(SmemAddr(full + s), phaseFull[s]);
    }
    okShared = ok ? 1 : 0;
    if (!ok) atomicExch(errorFlag, 1);
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (okShared && g.kSteps > 0) {
    const int row = mt * kTcTileM + 32 * warp + lane;
    const int n0 = nt * kNetTileN;
    for (int c0 = 0; c0 < kNetTileN; c0 += 16) {
      uint32_t r[16];
      const uint32_t addr = tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < g.M) {
        float* out = g.C + static_cast<long long>(row) * g.ldc;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int n = n0 + c0 + q;
          if (n < g.N) out[n] = (g.accumulate ? out[n] : 0.0f) + __uint_as_float(r[q]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kNetTmemColumns)
                 : "memory");
}

__device__ inline float Gelu(float x) {
  const float c = 0.7978845608028654f;  // sqrt(2 / pi)
  return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}

__device__ inline float GeluSlope(float x) {
  const float c = 0.7978845608028654f;
  const float u = c * (x + 0.044715f * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * 0.044715f * x * x);
}

// Z += bias per column; H = GELU(Z) (or H = Z for the last layer).
__global__ void BiasActivationKernel(int rows, int cols, const float* bias, float* Z, float* H, int linear) {
  const long long total = static_cast<long long>(rows) * cols;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float z = Z[t] + bias[t % cols];
    Z[t] = z;
    H[t] = linear ? z : Gelu(z);
  }
}

// dZ = dH * GELU'(Z), in place in dH.
__global__ void GeluBackKernel(long long total, const float* Z, float* dH) {
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x)
    dH[t] *= GeluSlope(Z[t]);
}

// db = column sums of dZ (one thread per column; rows are few thousand).
__global__ void ColumnSumKernel(int rows, int cols, const float* dZ, float* db) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int r = 0; r < rows; ++r) s += dZ[static_cast<long long>(r) * cols + c];
    db[c] = s;
  }
}

__global__ void AdamKernel(long long n, const float* grad, float* w, float* m, float* v, float lr, float beta1,
                           float beta2, float c1, float c2, float eps) {
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float g = grad[t];
    const float mt = beta1 * m[t] + (1.0f - beta1) * g;
    const float vt = beta2 * v[t] + (1.0f - beta2) * g * g;
    m[t] = mt;
    v[t] = vt;
    w[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  }
}

// -- the unit statistics, features, predictor and loss -------------------------------------

// A batch of pairs: per pair the changes Delta_n-2, Delta_n-1, Delta_n and
// the target Delta_n+1 as compact lateral columns [row][lateral] (FP32
// complex), the load ratio and the pair's normaliser (the extrapolation's
// squared error, summed over its rows and nodes).
struct PairBatch {
  const float2* const* d2;
  const float2* const* d1;
  const float2* const* d0;
  const float2* const* target;
  const float* ratio;
  const float* norm;
};

// The rows of each (block b, degree l), m-major device layout: list[(b, l)]
// in rows [start[b * (L + 1) + l], start[... + 1]).
struct RowLists {
  int L, lateral;
  const int* start;
  const int* rows;
  const float* depth;  // per lateral node, 0 at the lateral zone's bottom, 1 at its top
  const float* relax;  // per lateral node, log10(dt itau) / 4
};

// Per unit (pair q, l, p) and block: |D0|^2, |D1|^2, |D2|^2, Re D0 conj D1,
// Re D1 conj D2 over the block's orders; then the 16 features.
__global__ void FeaturesKernel(RowLists rl, PairBatch pb, int pairs, float* features) {
  const int units = (rl.L + 1) * rl.lateral;
  const long long total = static_cast<long long>(pairs) * units;
  for (long long u = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; u < total;
       u += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int q = static_cast<int>(u / units), rest = static_cast<int>(u % units);
    const int l = rest / rl.lateral, p = rest % rl.lateral;
    float* f = features + u * kFeatures;
    for (int b = 0; b < kBlocks; ++b) {
      double n0 = 0, n1 = 0, n2 = 0, c01 = 0, c12 = 0;
      const int list = b * (rl.L + 1) + l;
      for (int k = rl.start[list]; k < rl.start[list + 1]; ++k) {
        const long long at = static_cast<long long>(rl.rows[k]) * rl.lateral + p;
        const float2 a = pb.d0[q][at], c = pb.d1[q][at], e = pb.d2[q][at];
        n0 += a.x * a.x + a.y * a.y;
        n1 += c.x * c.x + c.y * c.y;
        n2 += e.x * e.x + e.y * e.y;
        c01 += a.x * c.x + a.y * c.y;
        c12 += c.x * e.x + c.y * e.y;
      }
      const double tiny = 1e-300;
      const float r1 = n1 > tiny ? static_cast<float>(c01 / n1) : 0.0f;
      const float r2 = n2 > tiny ? static_cast<float>(c12 / n2) : 0.0f;
      const float lr = (n0 > tiny && n1 > tiny) ? static_cast<float>(0.5 * log(n0 / n1)) : 0.0f;
      f[4 * b + 0] = fminf(fmaxf(r1, -4.0f), 4.0f);
      f[4 * b + 1] = fminf(fmaxf(r2, -4.0f), 4.0f);
      f[4 * b + 2] = fminf(fmaxf(lr, -8.0f), 8.0f) * 0.25f;
      f[4 * b + 3] = n0 > tiny ? 1.0f : 0.0f;
    }
    f[12] = static_cast<float>(l) / (l + 10.0f);
    f[13] = rl.depth[p];
    f[14] = rl.relax[p];
    f[15] = pb.ratio[q];
  }
}

// The predictor's coefficients of block b at a unit from the network's
// outputs (offsets from the extrapolation's 1, 0, 0).
__device__ inline void Coefficients(const float* out, int b, float& a, float& bb, float& c) {
  a = 1.0f + out[3 * b];
  bb = out[3 * b + 1];
  c = out[3 * b + 2];
}

// Per unit and block: the squared error of the predicted change over the
// block's orders (into loss, relative to the pair's normaliser, averaged
// over the pairs) and its gradient with respect to the three coefficients.
__global__ void LossGradKernel(RowLists rl, PairBatch pb, int pairs, const float* outputs, float* dOut,
                               float* lossPartial) {
  const int units = (rl.L + 1) * rl.lateral;
  const long long total = static_cast<long long>(pairs) * units;
  __shared__ float blockLoss[256];
  float mine = 0.0f;
  for (long long u = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; u < total;
       u += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int q = static_cast<int>(u / units), rest = static_cast<int>(u % units);
    const int l = rest / rl.lateral, p = rest % rl.lateral;
    const float scale = 1.0f / (pb.norm[q] * pairs);
    float* g = dOut + u * kOutputs;
    for (int k = 0; k < kOutputs; ++k) g[k] = 0.0f;
    for (int b = 0; b < kBlocks; ++b) {
      float a, bb, c;
      Coefficients(outputs + u * kOutputs, b, a, bb, c);
      double se = 0, ga = 0, gb = 0, gc = 0;
      const int list = b * (rl.L + 1) + l;
      for (int k = rl.start[list]; k < rl.start[list + 1]; ++k) {
        const long long at = static_cast<long long>(rl.rows[k]) * rl.lateral + p;
        const float2 x0 = pb.d0[q][at], x1 = pb.d1[q][at], x2 = pb.d2[q][at], t = pb.target[q][at];
        const float rx = a * x0.x + bb * x1.x + c * x2.x - t.x;
        const float ry = a * x0.y + bb * x1.y + c * x2.y - t.y;
        se += rx * rx + ry * ry;
        ga += 2.0 * (rx * x0.x + ry * x0.y);
        gb += 2.0 * (rx * x1.x + ry * x1.y);
        gc += 2.0 * (rx * x2.x + ry * x2.y);
      }
      mine += static_cast<float>(se) * scale;
      g[3 * b] = static_cast<float>(ga) * scale;
      g[3 * b + 1] = static_cast<float>(gb) * scale;
      g[3 * b + 2] = static_cast<float>(gc) * scale;
    }
  }
  blockLoss[threadIdx.x] = mine;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) blockLoss[threadIdx.x] += blockLoss[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) lossPartial[blockIdx.x] = blockLoss[0];
}

// The guess over every node in the device layout ([spin block rows][P]
// complex, node fastest): s_n + predicted change at the lateral nodes
// [p0, p0 + lateral), s_n + Delta_n elsewhere.
__global__ void GuessKernel(long long rows, int P, int p0, int lateral, const int* rowUnitBase, const float* outputs,
                            const double2* s0, const double2* s1, const double2* s2, const double2* s3,
                            double2* guess) {
  const long long total = rows * P;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long r = t / P;
    const int p = static_cast<int>(t % P);
    const double2 a = s0[t], b = s1[t], c = s2[t], d = s3[t];
    const double2 d0 = make_double2(a.x - b.x, a.y - b.y);
    double2 out = make_double2(a.x + d0.x, a.y + d0.y);
    if (p >= p0 && p < p0 + lateral) {
      const int code = rowUnitBase[r];  // (block, l) of the row
      const int blk = code & 3, l = code >> 2;
      float ca, cb, cc;
      Coefficients(outputs + (static_cast<long long>(l) * lateral + (p - p0)) * kOutputs, blk, ca, cb, cc);
      const double2 d1 = make_double2(b.x - c.x, b.y - c.y), d2 = make_double2(c.x - d.x, c.y - d.y);
      out = make_double2(a.x + ca * d0.x + cb * d1.x + cc * d2.x, a.y + ca * d0.y + cb * d1.y + cc * d2.y);
    }
    guess[t] = out;
  }
}

// The same statistics at inference, straight from four consecutive FP64
// snapshots in the device layout (changes formed on the fly).
__global__ void FeaturesFromStatesKernel(RowLists rl, int P, int p0, const double2* s0, const double2* s1,
                                         const double2* s2, const double2* s3, float ratio, float* features) {
  const int units = (rl.L + 1) * rl.lateral;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < units; u += gridDim.x * blockDim.x) {
    const int l = u / rl.lateral, p = u % rl.lateral;
    float* f = features + static_cast<long long>(u) * kFeatures;
    for (int b = 0; b < kBlocks; ++b) {
      double n0 = 0, n1 = 0, n2 = 0, c01 = 0, c12 = 0;
      const int list = b * (rl.L + 1) + l;
      for (int k = rl.start[list]; k < rl.start[list + 1]; ++k) {
        const long long at = static_cast<long long>(rl.rows[k]) * P + p0 + p;
        const double2 a = s0[at], bb = s1[at], c = s2[at], d = s3[at];
        const double ax = a.x - bb.x, ay = a.y - bb.y, cx = bb.x - c.x, cy = bb.y - c.y;
        const double ex = c.x - d.x, ey = c.y - d.y;
        n0 += ax * ax + ay * ay;
        n1 += cx * cx + cy * cy;
        n2 += ex * ex + ey * ey;
        c01 += ax * cx + ay * cy;
        c12 += cx * ex + cy * ey;
      }
      const double tiny = 1e-300;
      const float r1 = n1 > tiny ? static_cast<float>(c01 / n1) : 0.0f;
      const float r2 = n2 > tiny ? static_cast<float>(c12 / n2) : 0.0f;
      const float lr = (n0 > tiny && n1 > tiny) ? static_cast<float>(0.5 * log(n0 / n1)) : 0.0f;
      f[4 * b + 0] = fminf(fmaxf(r1, -4.0f), 4.0f);
      f[4 * b + 1] = fminf(fmaxf(r2, -4.0f), 4.0f);
      f[4 * b + 2] = fminf(fmaxf(lr, -8.0f), 8.0f) * 0.25f;
      f[4 * b + 3] = n0 > tiny ? 1.0f : 0.0f;
    }
    f[12] = static_cast<float>(l) / (l + 10.0f);
    f[13] = rl.depth[p];
    f[14] = rl.relax[p];
    f[15] = ratio;
  }
}

unsigned Grid1(long long n) { return static_cast<unsigned>(std::min<long long>((n + 255) / 256, 4096)); }

}  // namespace
}  // namespace sl3dgpu

using namespace sl3dgpu;

// -- the network object ---------------------------------------------------------------------

struct sl3dgpu_wsnet {
  int hidden = 768, depth = 6;          // hidden width, hidden layers
  std::vector<int> in, out;              // per layer
  std::vector<long long> wOff, bOff;     // offsets into the parameter vector
  long long count = 0;
  Dev<float> params, grads, m, v;        // FP32 master parameters, gradient, Adam moments
  long long step = 0;
  Dev<int> error;
  // the bound layout
  int L = -1, lateral = 0;
  long long rows = 0;
  Dev<int> start, rowList, rowUnit;
  Dev<float> nodeDepth, nodeRelax;
  // work buffers (grown on demand)
  int capacity = 0, widest = 0;
  std::vector<Dev<float>> Z, H;          // per layer: pre-activation and output (H[0] the features)
  Dev<float> dA, dB;                     // backward ping-pong
  Dev<uint16_t> packA, packB;
  Dev<float> lossPartial;
  Dev<float> ratio, norm;
  Dev<const float2*> ptrs;               // the batch's pair pointers, 4 x pairs
  cudaStream_t stream = nullptr;

  int Layers() const { return depth + 1; }
};

namespace {

int EnsureCapacity(sl3dgpu_wsnet& n, int units) {
  if (units <= n.capacity) return SL3DGPU_OK;
  size_t widest = kFeatures;
  for (int i = 0; i < n.Layers(); ++i) widest = std::max<size_t>(widest, n.out[i]);
  // at least the widest layer, so that the packed weights (widest x widest)
  // fit the operand buffers whatever the batch
  const int cap = std::max({units, 2 * n.capacity, static_cast<int>(widest)});
  n.Z.resize(n.Layers());
  n.H.resize(n.Layers() + 1);
  SL3D_CUDA(n.H[0].Alloc(static_cast<size_t>(cap) * kFeatures));
  for (int i = 0; i < n.Layers(); ++i) {
    SL3D_CUDA(n.Z[i].Alloc(static_cast<size_t>(cap) * n.out[i]));
    SL3D_CUDA(n.H[i + 1].Alloc(static_cast<size_t>(cap) * n.out[i]));
  }
  SL3D_CUDA(n.dA.Alloc(static_cast<size_t>(cap) * widest));
  SL3D_CUDA(n.dB.Alloc(static_cast<size_t>(cap) * widest));
  // A packs at most (cap + 127) x (widest + 15) values (a batch's rows by a
  // layer's width) or (widest + 127) x (cap + 15) (a weight gradient's),
  // B likewise with 64-row tiles; the weights themselves, (widest + 127) x
  // (widest + 15), fit the first form since cap >= widest
  SL3D_CUDA(n.packA.Alloc(static_cast<size_t>(cap + kTcTileM) * (widest + kTcTileK) +
                          static_cast<size_t>(widest + kTcTileM) * (cap + kTcTileK)));
  SL3D_CUDA(n.packB.Alloc(static_cast<size_t>(cap + kNetTileN) * (widest + kTcTileK) +
                          static_cast<size_t>(widest + kNetTileN) * (cap + kTcTileK)));
  n.capacity = cap;
  n.widest = static_cast<int>(widest);
  return SL3DGPU_OK;
}

template <class T>
cudaError_t Grow(Dev<T>& d, size_t count) {
  return d.n >= count ? cudaSuccess : d.Alloc(count);
}

int Pack(const float* src, long long sr, long long sk, int rows, int K, int tileRows, uint16_t* out, cudaStream_t s) {
  const int rowTiles = (rows + tileRows - 1) / tileRows, kSteps = (K + kTcTileK - 1) / kTcTileK;
  const long long total = static_cast<long long>(rowTiles) * kSteps * tileRows * kTcTileK;
  PackKernel<<<Grid1(total), 256, 0, s>>>(src, sr, sk, rows, K, tileRows, rowTiles, kSteps, out);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// C (M x N, ldc) (+)= A B^T with A (M x K) and B (N x K) given by strides.
int Gemm(sl3dgpu_wsnet& n, const float* A, long long aR, long long aK, const float* B, long long bR, long long bK,
         int M, int N, int K, float* C, int ldc, bool accumulate) {
  if (M == 0 || N == 0) return SL3DGPU_OK;
  SL3D_TRY(Pack(A, aR, aK, M, K, kTcTileM, n.packA.p, n.stream));
  SL3D_TRY(Pack(B, bR, bK, N, K, kNetTileN, n.packB.p, n.stream));
  NetGemm g{};
  g.M = M;
  g.N = N;
  g.K = K;
  g.mTiles = (M + kTcTileM - 1) / kTcTileM;
  g.nTiles = (N + kNetTileN - 1) / kNetTileN;
  g.kSteps = (K + kTcTileK - 1) / kTcTileK;
  g.A = n.packA.p;
  g.B = n.packB.p;
  g.C = C;
  g.ldc = ldc;
  g.accumulate = accumulate ? 1 : 0;
  // the stages need 12 KB; asking 29 KB keeps at most seven CTAs on an SM,
  // whose 64 tensor-memory columns each then never exceed the SM's 512
  constexpr size_t smem = 29 * 1024;
  static_assert(kNetStages * (kATileNet + kBTileNet) * sizeof(uint16_t) + (2 * kNetStages + 1) * 8 + 16 <= smem,
                "the stages fit");
  prof::Scope scope(prof::kOther, n.stream);
  NetGemmKernel<<<dim3(g.nTiles, g.mTiles), kNetThreads, smem, n.stream>>>(g, n.error.p);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// Forward over `units` rows of H[0] (the features): Z and H per layer, the
// outputs in H[Layers()].
int Forward(sl3dgpu_wsnet& n, int units) {
  for (int i = 0; i < n.Layers(); ++i) {
    const float* W = n.params.p + n.wOff[i];
    SL3D_TRY(Gemm(n, n.H[i].p, n.in[i], 1, W, n.in[i], 1, units, n.out[i], n.in[i], n.Z[i].p, n.out[i], false));
    const long long total = static_cast<long long>(units) * n.out[i];
    BiasActivationKernel<<<Grid1(total), 256, 0, n.stream>>>(units, n.out[i], n.params.p + n.bOff[i], n.Z[i].p,
                                                             n.H[i + 1].p, i == n.Layers() - 1 ? 1 : 0);
    SL3D_CHECK_LAUNCH();
  }
  return SL3DGPU_OK;
}

// Backward from dOut (units x kOutputs, in n.dA) into n.grads.
int Backward(sl3dgpu_wsnet& n, int units) {
  float* dZ = n.dA.p;
  float* other = n.dB.p;
  for (int i = n.Layers() - 1; i >= 0; --i) {
    // dW = dZ^T H_i: A = dZ^T (out x units), B = H_i^T (in x units)
    SL3D_TRY(Gemm(n, dZ, 1, n.out[i], n.H[i].p, 1, n.in[i], n.out[i], n.in[i], units, n.grads.p + n.wOff[i],
                  n.in[i], false));
    ColumnSumKernel<<<Grid1(n.out[i]), 256, 0, n.stream>>>(units, n.out[i], dZ, n.grads.p + n.bOff[i]);
    SL3D_CHECK_LAUNCH();
    if (i == 0) break;
    // dH_i = dZ W: A = dZ (units x out), B = W^T (in x out)
    const float* W = n.params.p + n.wOff[i];
    SL3D_TRY(Gemm(n, dZ, n.out[i], 1, W, 1, n.in[i], units, n.in[i], n.out[i], other, n.in[i], false));
    const long long total = static_cast<long long>(units) * n.in[i];
    GeluBackKernel<<<Grid1(total), 256, 0, n.stream>>>(total, n.Z[i - 1].p, other);
    SL3D_CHECK_LAUNCH();
    std::swap(dZ, other);
  }
  return SL3DGPU_OK;
}

int CheckWaits(sl3dgpu_wsnet& n) {
  int flag = 0;
  SL3D_CUDA(cudaMemcpyAsync(&flag, n.error.p, sizeof(int), cudaMemcpyDeviceToHost, n.stream));
  SL3D_CUDA(cudaStreamSynchronize(n.stream));
  if (flag) {
    SL3D_CUDA(cudaMemsetAsync(n.error.p, 0, sizeof(int), n.stream));
    SetError("wsnet: a tensor-core wait ran out of its budget");
    return SL3DGPU_ERR_WAIT;
  }
  return SL3DGPU_OK;
}

RowLists ListsOf(const sl3dgpu_wsnet& n) {
  return RowLists{n.L, n.lateral, n.start.p, n.rowList.p, n.nodeDepth.p, n.nodeRelax.p};
}

// Features, forward, loss and gradient of a batch (the gradient in grads).
int BatchGradient(sl3dgpu_wsnet& n, int pairs, const float2* const* d2, const float2* const* d1,
                  const float2* const* d0, const float2* const* target, const float* ratio, const float* norm,
                  float* loss) {
  if (n.L < 0) {
    SetError("wsnet: bind a layout first");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const int units = pairs * (n.L + 1) * n.lateral;
  SL3D_TRY(EnsureCapacity(n, units));
  std::vector<const float2*> hp;
  for (auto* list : {d2, d1, d0, target}) hp.insert(hp.end(), list, list + pairs);
  SL3D_CUDA(Grow(n.ptrs, hp.size()));
  SL3D_CUDA(cudaMemcpyAsync(n.ptrs.p, hp.data(), hp.size() * sizeof(void*), cudaMemcpyHostToDevice, n.stream));
  SL3D_CUDA(Grow(n.ratio, pairs));
  SL3D_CUDA(Grow(n.norm, pairs));
  SL3D_CUDA(cudaMemcpyAsync(n.ratio.p, ratio, pairs * sizeof(float), cudaMemcpyHostToDevice, n.stream));
  SL3D_CUDA(cudaMemcpyAsync(n.norm.p, norm, pairs * sizeof(float), cudaMemcpyHostToDevice, n.stream));
  const PairBatch pb{n.ptrs.p, n.ptrs.p + pairs, n.ptrs.p + 2 * pairs, n.ptrs.p + 3 * pairs, n.ratio.p, n.norm.p};
  FeaturesKernel<<<Grid1(units), 256, 0, n.stream>>>(ListsOf(n), pb, pairs, n.H[0].p);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(Forward(n, units));
  const unsigned blocks = Grid1(units);
  SL3D_CUDA(Grow(n.lossPartial, blocks));
  LossGradKernel<<<blocks, 256, 0, n.stream>>>(ListsOf(n), pb, pairs, n.H[n.Layers()].p, n.dA.p, n.lossPartial.p);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(Backward(n, units));
  std::vector<float> partial(blocks);
  SL3D_CUDA(cudaMemcpyAsync(partial.data(), n.lossPartial.p, blocks * sizeof(float), cudaMemcpyDeviceToHost,
                            n.stream));
  SL3D_TRY(CheckWaits(n));
  double total = 0;
  for (float v : partial) total += v;
  *loss = static_cast<float>(total);
  return SL3DGPU_OK;
}

}  // namespace

extern "C" int sl3dgpu_wsnet_create(int hidden, int depth, unsigned long long seed, sl3dgpu_wsnet** out) {
  if (out == nullptr || hidden < 16 || hidden % 16 != 0 || depth < 1 || depth > 16) {
    SetError("wsnet: hidden a multiple of 16 (>= 16), 1..16 hidden layers");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto n = std::make_unique<sl3dgpu_wsnet>();
  n->hidden = hidden;
  n->depth = depth;
  for (int i = 0; i <= depth; ++i) {
    n->in.push_back(i == 0 ? kFeatures : hidden);
    n->out.push_back(i == depth ? kOutputs : hidden);
  }
  std::vector<float> host;
  std::mt19937_64 rng(seed);
  for (int i = 0; i <= depth; ++i) {
    n->wOff.push_back(static_cast<long long>(host.size()));
    // He-style initialisation for the hidden layers; the output layer starts
    // at zero, so the untrained network is the extrapolation
    std::normal_distribution<float> normal(0.0f, std::sqrt(2.0f / n->in[i]));
    for (long long k = 0; k < static_cast<long long>(n->in[i]) * n->out[i]; ++k)
      host.push_back(i == depth ? 0.0f : normal(rng));
    n->bOff.push_back(static_cast<long long>(host.size()));
    host.insert(host.end(), n->out[i], 0.0f);
  }
  n->count = static_cast<long long>(host.size());
  SL3D_CUDA(n->params.Upload(host));
  SL3D_CUDA(n->grads.Alloc(n->count));
  SL3D_CUDA(n->m.Upload(std::vector<float>(n->count, 0.0f)));
  SL3D_CUDA(n->v.Upload(std::vector<float>(n->count, 0.0f)));
  SL3D_CUDA(n->error.Upload(std::vector<int>{0}));
  SL3D_CUDA(cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking));
  SL3D_CUDA(AllowDynamicSmem(NetGemmKernel));
  *out = n.release();
  return SL3DGPU_OK;
}

extern "C" void sl3dgpu_wsnet_destroy(sl3dgpu_wsnet* n) {
  if (n == nullptr) return;
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
}

extern "C" long long sl3dgpu_wsnet_parameter_count(const sl3dgpu_wsnet* n) { return n ? n->count : -1; }

extern "C" int sl3dgpu_wsnet_parameters(const sl3dgpu_wsnet* n, float* out) {
  if (n == nullptr || out == nullptr) {
    SetError("wsnet: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaMemcpyAsync(out, n->params.p, n->count * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
  SL3D_CUDA(cudaStreamSynchronize(n->stream));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_wsnet_set_parameters(sl3dgpu_wsnet* n, const float* in) {
  if (n == nullptr || in == nullptr) {
    SetError("wsnet: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaMemcpyAsync(n->params.p, in, n->count * sizeof(float), cudaMemcpyHostToDevice, n->stream));
  SL3D_CUDA(cudaStreamSynchronize(n->stream));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_wsnet_bind(sl3dgpu_wsnet* n, int lmax, int lateral, const double* depth,
                                  const double* relax) {
  if (n == nullptr || lmax < 2 || lateral < 1 || depth == nullptr || relax == nullptr) {
    SetError("wsnet: lmax >= 2, lateral nodes >= 1, depth and relaxation per lateral node");
    return SL3DGPU_ERR_ARGUMENT;
  }
  // The m-major device rows of the three blocks (spin -2, -1 with every
  // order, the real spin 0 with m >= 0): row RowOffset(m) + (l - l0(m)).
  const int L = lmax;
  std::vector<std::vector<int>> lists(static_cast<size_t>(kBlocks) * (L + 1));
  std::vector<int> rowCode;
  long long base = 0;
  for (int b = 0; b < kBlocks; ++b) {
    const int N = b == 0 ? -2 : b == 1 ? -1 : 0;
    const int mFirst = b == 2 ? 0 : -L;
    for (int m = mFirst; m <= L; ++m) {
      const int l0 = std::max(std::abs(m), std::abs(N));
      for (int l = l0; l <= L; ++l) {
        lists[static_cast<size_t>(b) * (L + 1) + l].push_back(static_cast<int>(base));
        rowCode.push_back((l << 2) | b);
        ++base;
      }
    }
  }
  std::vector<int> start{0}, rowList;
  for (const auto& list : lists) {
    rowList.insert(rowList.end(), list.begin(), list.end());
    start.push_back(static_cast<int>(rowList.size()));
  }
  SL3D_CUDA(n->start.Upload(start));
  SL3D_CUDA(n->rowList.Upload(rowList));
  SL3D_CUDA(n->rowUnit.Upload(rowCode));
  SL3D_CUDA(n->nodeDepth.Upload(std::vector<float>(depth, depth + lateral)));
  SL3D_CUDA(n->nodeRelax.Upload(std::vector<float>(relax, relax + lateral)));
  n->L = L;
  n->lateral = lateral;
  n->rows = base;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_wsnet_gradient(sl3dgpu_wsnet* n, int pairs, const void* const* d2, const void* const* d1,
                                      const void* const* d0, const void* const* target, const float* ratio,
                                      const float* norm, float* grad, float* loss) {
  if (n == nullptr || pairs < 1 || loss == nullptr) {
    SetError("wsnet: null network, no pairs or no loss");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_TRY(BatchGradient(*n, pairs, reinterpret_cast<const float2* const*>(d2),
                         reinterpret_cast<const float2* const*>(d1), reinterpret_cast<const float2* const*>(d0),
                         reinterpret_cast<const float2* const*>(target), ratio, norm, loss));
  if (grad != nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(grad, n->grads.p, n->count * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    SL3D_CUDA(cudaStreamSynchronize(n->stream));
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_wsnet_train_step(sl3dgpu_wsnet* n, int pairs, const void* const* d2, const void* const* d1,
                                        const void* const* d0, const void* const* target, const float* ratio,
                                        const float* norm, float lr, float* loss) {
  SL3D_TRY(sl3dgpu_wsnet_gradient(n, pairs, d2, d1, d0, target, ratio, norm, nullptr, loss));
  ++n->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - std::pow(b1, static_cast<float>(n->step)), c2 = 1.0f - std::pow(b2, static_cast<float>(n->step));
  AdamKernel<<<Grid1(n->count), 256, 0, n->stream>>>(n->count, n->grads.p, n->params.p, n->m.p, n->v.p, lr, b1, b2,
                                                     c1, c2, 1e-8f);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_wsnet_predict(sl3dgpu_wsnet* n, int P, int lateral_first, const double* s_n,
                                     const double* s_nm1, const double* s_nm2, const double* s_nm3, double ratio,
                                     double* guess, void* stream) {
  if (n == nullptr || n->L < 0 || s_n == nullptr || s_nm1 == nullptr || s_nm2 == nullptr || s_nm3 == nullptr ||
      guess == nullptr || lateral_first < 0 || lateral_first + n->lateral > P) {
    SetError("wsnet: a bound network, four snapshots, a guess buffer and the lateral range inside the nodes");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const int units = (n->L + 1) * n->lateral;
  SL3D_TRY(EnsureCapacity(*n, units));
  const cudaStream_t s = AsStream(stream);
  // the caller's stream orders the snapshots; the network's stream follows it
  cudaEvent_t ready;
  SL3D_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  SL3D_CUDA(cudaEventRecord(ready, s));
  SL3D_CUDA(cudaStreamWaitEvent(n->stream, ready, 0));
  const auto* a = reinterpret_cast<const double2*>(s_n);
  const auto* b = reinterpret_cast<const double2*>(s_nm1);
  const auto* c = reinterpret_cast<const double2*>(s_nm2);
  const auto* d = reinterpret_cast<const double2*>(s_nm3);
  FeaturesFromStatesKernel<<<Grid1(units), 256, 0, n->stream>>>(ListsOf(*n), P, lateral_first, a, b, c, d,
                                                                static_cast<float>(ratio), n->H[0].p);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(Forward(*n, units));
  GuessKernel<<<Grid1(n->rows * P), 256, 0, n->stream>>>(n->rows, P, lateral_first, n->lateral, n->rowUnit.p,
                                                         n->H[n->Layers()].p, a, b, c, d,
                                                         reinterpret_cast<double2*>(guess));
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaEventRecord(ready, n->stream));
  SL3D_CUDA(cudaStreamWaitEvent(s, ready, 0));
  SL3D_CUDA(cudaEventDestroy(ready));
  return CheckWaits(*n);
}

// The network's products alone, for checking: C = A B^T for FP32 row-major
// A (M x K) and B (N x K) on the tensor cores in BF16 (device pointers).
extern "C" int sl3dgpu_wsnet_gemm(sl3dgpu_wsnet* n, const float* A, const float* B, int M, int N, int K, float* C) {
  if (n == nullptr || A == nullptr || B == nullptr || C == nullptr || M < 0 || N < 0 || K < 1) {
    SetError("wsnet: null argument or negative size");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_TRY(EnsureCapacity(*n, std::max(M, N)));
  if (K > n->widest) {
    SetError("wsnet: K beyond the network's widest layer (the packing buffers' depth)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_TRY(Gemm(*n, A, K, 1, B, K, 1, M, N, K, C, N, false));
  return CheckWaits(*n);
}
