// The FP32 Legendre contraction on the tcgen05 tensor cores (see tc_gemm.cuh).
//
// One CTA of four warps per (item, 128-row tile, column tile). K runs in
// steps of 16, three in flight: the CTA copies a step's A and B high and low
// parts into shared memory (cp.async, the canonical no-swizzle K-major layout
// of 8-row x 16-byte core matrices) two steps ahead of its use; one elected
// thread issues the step's six tcgen05.mma (two 8-deep slices x three
// products) into the FP32 accumulator in tensor memory and commits them to
// the step buffer's mbarrier, which the CTA waits on (with an iteration
// limit) before refilling that buffer. The epilogue reads the accumulator
// back with tcgen05.ld, one TMEM lane quarter per warp, and stores (or adds)
// the rows in range.
#include <cstdint>

#include "profile.cuh"
#include "tc_gemm.cuh"

namespace sl3dgpu {
namespace {

constexpr int kTM = 128;      // rows per tile (the MMA's M)
constexpr int kTK = 16;       // K per staged step (two 8-deep MMA slices)
constexpr int kStages = 3;    // staged steps in flight
constexpr int kThreads = 128;
constexpr int kWaitLimit = 1 << 22;

constexpr int kAFloats = kTM * kTK;  // one part of A's tile

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

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B,
// both K-major, N and M.
__host__ __device__ constexpr uint32_t InstrDescriptor(int n, int m) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ inline float RoundTf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Index (in floats) of element (row, k) of a K-major tile of `rows` rows in
// the core-matrix layout [k / 4][row / 8][row % 8][k % 4].
__device__ inline int TileIndex(int row, int k, int rows) {
  return (k >> 2) * (rows * 4) + (row >> 3) * 32 + (row & 7) * 4 + (k & 3);
}

__device__ inline void CopyAsync4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(SmemAddr(dst)), "l"(src) : "memory");
}

__device__ inline bool WaitParity(uint32_t bar, uint32_t phase) {
  for (int i = 0; i < kWaitLimit; ++i) {
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

// Tensor-memory columns for an accumulator of n columns: a power of two, at
// least 32.
__host__ __device__ constexpr uint32_t TmemColumns(int n) {
  uint32_t c = 32;
  while (c < static_cast<uint32_t>(n)) c *= 2;
  return c;
}

// The kernel: per CTA one (item, 128-row tile, column tile of tileN).
// Shared memory: kStages x {A hi, A lo, B hi, B lo} tiles, then the
// mbarriers and the tensor-memory address.
__global__ void __launch_bounds__(kThreads) TcGemmKernel(const GemmItem* items, const float* aHi, const float* aLo,
                                                         const float* bHi, const float* bLo, float* C,
                                                         bool accumulate, int tileN, int* errorFlag) {
  const GemmItem it = items[blockIdx.y];
  const int i0 = blockIdx.x * kTM, n0 = blockIdx.z * tileN;
  if (i0 >= it.M || n0 >= it.N) return;  // the whole CTA, before any tensor-memory work
  const int nCols = min(tileN, it.N - n0);
  const int nMma = (nCols + 15) / 16 * 16;  // the MMA's N: a multiple of 16
  const int bFloats = tileN * kTK;
  const uint32_t tmemColumns = TmemColumns(tileN);

  extern __shared__ __align__(128) unsigned char tcSmem[];
  float* stage0 = reinterpret_cast<float*>(tcSmem);
  const int stageFloats = 2 * kAFloats + 2 * bFloats;
  uint64_t* bar = reinterpret_cast<uint64_t*>(stage0 + kStages * stageFloats);
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(bar + kStages);
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(tmemSlot)),
                 "r"(tmemColumns)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(bar + s)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmemSlot;

  const float* ah = aHi + it.a;
  const float* al = aLo + it.a;
  const float* bh = bHi + it.b;
  const float* bl = bLo + it.b;
  const uint32_t idesc = InstrDescriptor(nMma, kTM);
  const int steps = (it.K + kTK - 1) / kTK;

  // Stage step `step` into buffer `buf`: cp.async of every element in range,
  // plain zero stores outside, one copy group per thread.
  auto stage = [&](int step, int buf) {
    float* sAh = stage0 + buf * stageFloats;
    float* sAl = sAh + kAFloats;
    float* sBh = sAl + kAFloats;
    float* sBl = sBh + bFloats;
    const int k0 = step * kTK;
    if (it.sAk == 1) {
      for (int e = tid; e < kTM * kTK; e += kThreads) {
        const int kk = e % kTK, ii = e / kTK;
        const int i = i0 + ii, k = k0 + kk;
        const int at = TileIndex(ii, kk, kTM);
        if (i < it.M && k < it.K) {
          const long long g = static_cast<long long>(i) * it.sAi + k;
          CopyAsync4(sAh + at, ah + g);
          CopyAsync4(sAl + at, al + g);
        } else {
          sAh[at] = 0.0f;
          sAl[at] = 0.0f;
        }
      }
    } else {
      for (int e = tid; e < kTM * kTK; e += kThreads) {
        const int ii = e % kTM, kk = e / kTM;
        const int i = i0 + ii, k = k0 + kk;
        const int at = TileIndex(ii, kk, kTM);
        if (i < it.M && k < it.K) {
          const long long g = static_cast<long long>(i) * it.sAi + static_cast<long long>(k) * it.sAk;
          CopyAsync4(sAh + at, ah + g);
          CopyAsync4(sAl + at, al + g);
        } else {
          sAh[at] = 0.0f;
          sAl[at] = 0.0f;
        }
      }
    }
    for (int e = tid; e < nMma * kTK; e += kThreads) {
      const int nn = e % nMma, kk = e / nMma;
      const int n = n0 + nn, k = k0 + kk;
      const int at = TileIndex(nn, kk, tileN);
      if (nn < nCols && k < it.K) {
        const long long g = static_cast<long long>(k) * it.ldb + n;
        CopyAsync4(sBh + at, bh + g);
        CopyAsync4(sBl + at, bl + g);
      } else {
        sBh[at] = 0.0f;
        sBl[at] = 0.0f;
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };

  uint32_t phase[kStages] = {0, 0, 0};
  bool used[kStages] = {false, false, false};
  bool ok = true;
  for (int s = 0; s < min(kStages - 1, steps); ++s) stage(s, s);
  for (int s = 0; s < steps && ok; ++s) {
    const int buf = s % kStages;
    // the step two ahead, into the buffer the previous step's MMAs read
    const int ahead = s + kStages - 1;
    if (ahead < steps) {
      const int nb = ahead % kStages;
      if (used[nb]) {
        ok = WaitParity(SmemAddr(bar + nb), phase[nb]);
        phase[nb] ^= 1u;
        used[nb] = false;
        if (!ok) break;
      }
      stage(ahead, nb);
      asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 1) : "memory");
    } else if (s + 1 < steps) {
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    // this step's copies (and zero stores) visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const float* sAh = stage0 + buf * stageFloats;
      const float* sAl = sAh + kAFloats;
      const float* sBh = sAl + kAFloats;
      const float* sBl = sBh + bFloats;
      const uint32_t aLbo = kTM * 16, bLbo = tileN * 16, sbo = 128;
#pragma unroll
      for (int q = 0; q < kTK / 8; ++q) {
        const uint32_t aOff = q * 2 * aLbo, bOff = q * 2 * bLbo;
        const uint64_t dAh = Descriptor(SmemAddr(sAh) + aOff, aLbo, sbo);
        const uint64_t dAl = Descriptor(SmemAddr(sAl) + aOff, aLbo, sbo);
        const uint64_t dBh = Descriptor(SmemAddr(sBh) + bOff, bLbo, sbo);
        const uint64_t dBl = Descriptor(SmemAddr(sBl) + bOff, bLbo, sbo);
        const uint64_t as[3] = {dAh, dAh, dAl};
        const uint64_t bs[3] = {dBh, dBl, dBh};
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const uint32_t enable = (s > 0 || q > 0 || p > 0) ? 1u : 0u;
          asm volatile(
              "{\n\t.reg .pred r;\n\t"
              "setp.ne.b32 r, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, r;\n\t}" ::"r"(tmem),
              "l"(as[p]), "l"(bs[p]), "r"(idesc), "r"(enable)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       SmemAddr(bar + buf))
                   : "memory");
    }
    used[buf] = true;
  }
  // The last step's commit covers every MMA before it.
  if (ok && steps > 0) {
    const int last = (steps - 1) % kStages;
    ok = WaitParity(SmemAddr(bar + last), phase[last]);
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!ok) {
    if (tid == 0) atomicExch(errorFlag, 1);
  } else {
    // Epilogue: this warp's TMEM lane quarter, 16 columns at a time.
    const int i = i0 + 32 * warp + lane;
    float* c = C + it.c + static_cast<long long>(i) * it.ldc + n0;
    for (int c0 = 0; c0 < nMma; c0 += 16) {
      uint32_t r[16];
      const uint32_t addr = tmem + (static_cast<uint32_t>(32 * warp) << 16) + static_cast<uint32_t>(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (i < it.M) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int n = c0 + q;
          if (n < nCols) {
            const float v = __uint_as_float(r[q]);
            c[n] = accumulate ? c[n] + v : v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmemColumns) : "memory");
}

__global__ void SplitTf32Kernel(long long n, const float* x, float* hi, float* lo) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride) {
    const float v = x[i];
    const float h = RoundTf32(v);
    hi[i] = h;
    lo[i] = v - h;
  }
}

__global__ void SplitTf32FromDoubleKernel(long long n, const double* x, float* hi, float* lo) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride) {
    const double v = x[i];
    const float h = RoundTf32(static_cast<float>(v));
    hi[i] = h;
    lo[i] = static_cast<float>(v - static_cast<double>(h));
  }
}

}  // namespace

int RunGemmTc(const GemmItem* items, int count, int maxM, int maxN, const float* aHi, const float* aLo,
              const float* bHi, const float* bLo, float* C, bool accumulate, int* errorFlag, cudaStream_t stream) {
  if (count == 0 || maxM == 0 || maxN == 0) return SL3DGPU_OK;
  // One column tile when N fits (the common case), else tiles of kTcTileN.
  const int tileN = maxN <= kTcTileN ? (maxN + 15) / 16 * 16 : kTcTileN;
  const size_t smem = static_cast<size_t>(kStages) * (2 * kAFloats + 2 * tileN * kTK) * sizeof(float) +
                      kStages * sizeof(uint64_t) + 16;
  SL3D_CUDA(cudaFuncSetAttribute(TcGemmKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  dim3 grid((maxM + kTM - 1) / kTM, static_cast<unsigned>(count), (maxN + tileN - 1) / tileN);
  TcGemmKernel<<<grid, kThreads, smem, stream>>>(items, aHi, aLo, bHi, bLo, C, accumulate, tileN, errorFlag);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

namespace {
__global__ void SplitRowsKernel(long long rows, int width, long long ld, const float* x, float* hi, float* lo) {
  const long long total = rows * width;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total; t += stride) {
    const long long at = (t / width) * ld + t % width;
    const float v = x[at];
    const float h = RoundTf32(v);
    hi[at] = h;
    lo[at] = v - h;
  }
}
}  // namespace

void LaunchSplitTf32Rows(long long rows, int width, long long ld, const float* x, float* hi, float* lo,
                         cudaStream_t stream) {
  const long long blocks = std::min<long long>((rows * width + 255) / 256, 152LL * 32);
  SplitRowsKernel<<<static_cast<unsigned>(std::max<long long>(blocks, 1)), 256, 0, stream>>>(rows, width, ld, x, hi,
                                                                                             lo);
}

void LaunchSplitTf32(long long n, const float* x, float* hi, float* lo, cudaStream_t stream) {
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 32);
  SplitTf32Kernel<<<static_cast<unsigned>(std::max<long long>(blocks, 1)), 256, 0, stream>>>(n, x, hi, lo);
}

}  // namespace sl3dgpu

namespace sl3dgpu {
void LaunchSplitTf32(long long n, const double* x, float* hi, float* lo, cudaStream_t stream) {
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 32);
  SplitTf32FromDoubleKernel<<<static_cast<unsigned>(std::max<long long>(blocks, 1)), 256, 0, stream>>>(n, x, hi,
                                                                                                        lo);
}
}  // namespace sl3dgpu
