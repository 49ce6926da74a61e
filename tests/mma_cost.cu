// Micro-benchmark: cycles per tcgen05.mma (cta_group::1, M = 128) as a
// function of N, for kind::f16 (BF16, K = 16) and kind::tf32 (K = 8), with
// zero operands resident in shared memory (no-swizzle K-major layout) and R
// accumulators used in turn. One CTA per SM (120 KB of shared memory each),
// one thread issuing back to back, clock64 from the first issue to the
// commit's mbarrier; every wait is bounded and reported. The contractions
// (tc_gemm.cu, tc_gemm64.cu) choose their MMA widths from this cost model.
// Build: nvcc -gencode arch=compute_103a,code=sm_103a -O2 -std=c++17 mma_cost.cu
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>

__device__ inline uint32_t SmemAddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ inline uint64_t Desc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(layout & 7u) << 61;
  return d;
}

__host__ __device__ constexpr uint32_t IdescBf16(int n, int m) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}
__host__ __device__ constexpr uint32_t IdescTf32(int n, int m) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

// kind: 0 f16 (bf16), 1 tf32. layout: 0 none, 6 SW32, 2 SW128.
template <int R, int COLS>
__global__ void Probe(int kind, int n, int layout, int iters, long long* cycles, int* err) {
  extern __shared__ __align__(1024) unsigned char raw[];
  // A: 128 rows x 128 B (16 KB), B: 256 rows x 128 B (32 KB): room for every
  // layout, from a 1 KB boundary of the shared window
  unsigned char* smem = raw + ((1024u - (SmemAddr(raw) & 1023u)) & 1023u);
  unsigned char* A = smem;
  unsigned char* B = smem + 16384;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t slot;
  for (int i = threadIdx.x; i < 49152 / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(smem)[i] = 0u;
  const int warp = threadIdx.x / 32;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(&slot)), "r"(COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(&bar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = slot;
  if (threadIdx.x == 0) {
    uint32_t aLbo, bLbo, sbo;
    if (layout == 0) {           // core matrices 8 x 16 B; k-group stride = rows x 16 B
      aLbo = 128 * 16; bLbo = n * 16; sbo = 128;
    } else if (layout == 6) {    // 32-byte rows, 8-row atoms of 256 B
      aLbo = 16; bLbo = 16; sbo = 256;
    } else {                     // 128-byte rows, 8-row atoms of 1 KB
      aLbo = 16; bLbo = 16; sbo = 1024;
    }
    const uint64_t dA = Desc(SmemAddr(A), aLbo, sbo, layout);
    const uint64_t dB = Desc(SmemAddr(B), bLbo, sbo, layout);
    const uint32_t idesc = kind == 0 ? IdescBf16(n, 128) : IdescTf32(n, 128);
    const long long t0 = clock64();
    for (int i = 0; i < iters; i += R) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const uint32_t en = i > 0 ? 1u : 0u;
        const uint32_t d = tmem + static_cast<uint32_t>(r * n);
        if (kind == 0)
          asm volatile("{\n\t.reg .pred r;\n\tsetp.ne.b32 r, %4, 0;\n\t"
                       "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, r;\n\t}" ::"r"(d),
                       "l"(dA), "l"(dB), "r"(idesc), "r"(en)
                       : "memory");
        else
          asm volatile("{\n\t.reg .pred r;\n\tsetp.ne.b32 r, %4, 0;\n\t"
                       "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, r;\n\t}" ::"r"(d),
                       "l"(dA), "l"(dB), "r"(idesc), "r"(en)
                       : "memory");
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(SmemAddr(&bar))
                 : "memory");
    bool ok = false;
    for (int k = 0; k < (1 << 26) && !ok; ++k) {
      uint32_t done;
      asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(done)
                   : "r"(SmemAddr(&bar)), "r"(0u)
                   : "memory");
      ok = done != 0;
    }
    const long long t1 = clock64();
    cycles[blockIdx.x] = t1 - t0;
    if (!ok) atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS) : "memory");
}

int main() {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  long long* cyc;
  int* err;
  cudaMalloc(&cyc, sms * sizeof(long long));
  cudaMalloc(&err, sizeof(int));
  cudaMemset(err, 0, sizeof(int));
  const int iters = 4096;
  auto run = [&](auto kernel, int kind, int n, int smemBytes, const char* name) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes);
    for (int rep = 0; rep < 2; ++rep) kernel<<<sms, 128, smemBytes>>>(kind, n, 0, iters, cyc, err);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { printf("%s: %s\n", name, cudaGetErrorString(e)); exit(1); }
    long long h[256];
    cudaMemcpy(h, cyc, sms * sizeof(long long), cudaMemcpyDeviceToHost);
    int he = 0;
    cudaMemcpy(&he, err, sizeof(int), cudaMemcpyDeviceToHost);
    long long mx = 0, mn = 1LL << 62, sum = 0;
    for (int i = 0; i < sms; ++i) { mx = h[i] > mx ? h[i] : mx; mn = h[i] < mn ? h[i] : mn; sum += h[i]; }
    const double per = static_cast<double>(sum) / sms / iters;
    const double macs = 128.0 * n * (kind == 0 ? 16 : 8);
    printf("%s cycles %.1f macs_per_clock %.0f err %d\n", name, per, macs / per, he);
  };
  const int big = 120 * 1024;
  run(Probe<1, 256>, 0, 64, big, "f16 N64 R1");
  run(Probe<1, 256>, 0, 128, big, "f16 N128 R1");
  run(Probe<1, 256>, 0, 256, big, "f16 N256 R1");
  run(Probe<4, 512>, 0, 64, big, "f16 N64 R4");
  run(Probe<1, 256>, 1, 128, big, "tf32 N128 R1");
  run(Probe<1, 256>, 1, 256, big, "tf32 N256 R1");
  return 0;
}
