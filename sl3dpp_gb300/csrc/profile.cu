// Launch accounting and per-kind event timing (see profile.cuh), and the
// FP64 FMA throughput probe the benchmark's FP64 roofline is measured against.
#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "profile.cuh"

namespace sl3dgpu::prof {
namespace {

struct Record {
  cudaEvent_t start, stop;
  int kind;
  double flops, bytes;
};

std::atomic<long long> launches{0};
std::atomic<bool> timing{false};
std::mutex lock;
std::vector<Record> records;
std::vector<cudaEvent_t> pool;
// The open start event of each kind, per host thread: threads driving
// operators on their own streams (sl3dgpu_v3d_run_many) each pair their own
// starts and stops.
thread_local cudaEvent_t open[kKinds];
double totalMs[kKinds], totalFlops[kKinds], totalBytes[kKinds];
long long counts[kKinds];

cudaEvent_t Take() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Folds the finished records into the totals (the caller synchronised).
void Drain() {
  for (auto& r : records) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) totalMs[r.kind] += ms;
    totalFlops[r.kind] += r.flops;
    totalBytes[r.kind] += r.bytes;
    counts[r.kind] += 1;
    pool.push_back(r.start);
    pool.push_back(r.stop);
  }
  records.clear();
}

}  // namespace

void Begin(int kind, cudaStream_t stream) {
  launches.fetch_add(1, std::memory_order_relaxed);
  if (!timing.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> g(lock);
  open[kind] = Take();
  cudaEventRecord(open[kind], stream);
}

void End(int kind, cudaStream_t stream, double flops, double bytes) {
  if (!timing.load(std::memory_order_relaxed)) return;
  std::lock_guard<std::mutex> g(lock);
  cudaEvent_t stop = Take();
  cudaEventRecord(stop, stream);
  records.push_back({open[kind], stop, kind, flops, bytes});
  if (records.size() > 20000) {
    cudaEventSynchronize(stop);
    Drain();
  }
}

bool TimingOn() { return timing.load(std::memory_order_relaxed); }
long long Launches() { return launches.load(std::memory_order_relaxed); }
void AddLaunches(long long n) { launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace sl3dgpu::prof

using namespace sl3dgpu;

extern "C" long long sl3dgpu_launch_count(void) { return prof::launches.load(); }

extern "C" int sl3dgpu_profile_enable(int on) {
  std::lock_guard<std::mutex> g(prof::lock);
  prof::timing.store(on != 0);
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_profile_reset(void) {
  std::lock_guard<std::mutex> g(prof::lock);
  SL3D_CUDA(cudaDeviceSynchronize());
  prof::Drain();
  for (int k = 0; k < prof::kKinds; ++k) {
    prof::totalMs[k] = prof::totalFlops[k] = prof::totalBytes[k] = 0.0;
    prof::counts[k] = 0;
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_profile_read(int kind, double* ms, long long* launches, double* flops, double* bytes) {
  if (kind < 0 || kind >= prof::kKinds) {
    SetError("profile: no such kernel kind");
    return SL3DGPU_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(prof::lock);
  SL3D_CUDA(cudaDeviceSynchronize());
  prof::Drain();
  if (ms) *ms = prof::totalMs[kind];
  if (launches) *launches = prof::counts[kind];
  if (flops) *flops = prof::totalFlops[kind];
  if (bytes) *bytes = prof::totalBytes[kind];
  return SL3DGPU_OK;
}

namespace {

// Eight independent FMA chains per thread.
template <class T>
__global__ void FmaKernel(T* out, int iters, T a, T b) {
  T x[8];
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x + i;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  T s = 0;
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
int FmaPeak(double* gflops, int iters) {
  int sms = 0;
  SL3D_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  const int blocks = sms * 16, threads = 256;
  T* out = nullptr;
  SL3D_CUDA(cudaMalloc(&out, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  FmaKernel<T><<<blocks, threads>>>(out, 16, T(0.999), T(0.001));
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    FmaKernel<T><<<blocks, threads>>>(out, iters, T(0.999), T(0.001));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) {
    SetError(cudaGetErrorString(err));
    return SL3DGPU_ERR_CUDA;
  }
  *gflops = 2.0 * 8 * iters * static_cast<double>(blocks) * threads / best / 1e6;
  return SL3DGPU_OK;
}

}  // namespace

extern "C" int sl3dgpu_fp64_fma_peak(double* gflops) { return FmaPeak<double>(gflops, 4096); }
extern "C" int sl3dgpu_fp32_fma_peak(double* gflops) { return FmaPeak<float>(gflops, 32768); }
