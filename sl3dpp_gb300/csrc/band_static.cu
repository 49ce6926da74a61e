// A banded Cholesky solve that allocates no device memory.
//
// Who needs it: callers whose device memory belongs to another allocator --
// a framework's caching allocator, or a fixed arena reserved at start-up --
// and that must therefore not have the solver call cudaMalloc or cudaFree,
// and callers on a time-critical loop where a driver allocation, which can
// synchronise the device, is not acceptable. They pass the factor and the
// right-hand sides in device memory they own; the solve's own scratch (the
// system descriptor, the work items and the row-major copy of the right-hand
// sides the batched kernel coalesces on) lives in one file-scope device
// array of fixed size, kStaticDoubles doubles (4 MiB), which every GPU that
// loads the library holds until the process exits.
//
// The array is shared by every call: a call overwrites all of it that it
// reads, so nothing needs clearing, and it keeps the last call's contents.
// Calls that overlap on the GPU (on different streams, or from different
// host threads) race on it and must be serialised by the caller.
#include <mutex>
#include <vector>

#include "common.cuh"

namespace sl3dgpu {

int BandSolveBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                   const int2* devItems, int itemCount, const double* bands, const int* pivots, double* rhs,
                   const double* scales, int lu, cudaStream_t stream);

namespace {

// 2^19 doubles: the descriptor and work items first, then the right-hand
// sides from a 256-byte boundary.
constexpr long long kStaticDoubles = 1LL << 19;
constexpr long long kItemsAt = 8;  // doubles reserved for the descriptor (56 bytes)
constexpr int kSolveColumns = 64;  // right-hand sides per work item of the batched solve

static __device__ __align__(256) double gSolveScratch[kStaticDoubles];

// The scratch's device address, found once per device (with that device
// current) by cudaGetSymbolAddress: in host code the array's name is only a
// host-side stand-in, not a device address.
std::mutex gAddressLock;
std::vector<double*> gAddress;

int ScratchAddress(double** out) {
  int device = 0;
  SL3D_CUDA(cudaGetDevice(&device));
  std::lock_guard<std::mutex> guard(gAddressLock);
  if (static_cast<int>(gAddress.size()) <= device) gAddress.resize(device + 1, nullptr);
  if (gAddress[device] == nullptr) {
    void* ptr = nullptr;
    SL3D_CUDA(cudaGetSymbolAddress(&ptr, gSolveScratch));
    gAddress[device] = static_cast<double*>(ptr);
  }
  *out = gAddress[device];
  return SL3DGPU_OK;
}

__global__ void DescribeKernel(double* base, int n, int kd, int nrhs, long long rhsAt, int items) {
  if (threadIdx.x == 0) {
    auto* s = reinterpret_cast<sl3dgpu_band_system*>(base);
    s->n = n;
    s->kl = kd;
    s->ku = kd;
    s->nrhs = nrhs;
    s->band = 0;
    s->pivots = 0;
    s->rhs = rhsAt;
    s->scale = -1;
    s->pinned0 = -1;
    s->pinned1 = -1;
  }
  auto* item = reinterpret_cast<int2*>(base + kItemsAt);
  for (int i = threadIdx.x; i < items; i += blockDim.x) item[i] = make_int2(0, kSolveColumns * i);
}

// Column-major (n x nrhs) to row-major and back.
__global__ void ToRowsKernel(const double* b, int n, int nrhs, double* rows) {
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<long long>(n) * nrhs) return;
  const long long i = t / nrhs, k = t % nrhs;
  rows[t] = b[k * n + i];
}

__global__ void ToColumnsKernel(const double* rows, int n, int nrhs, double* b) {
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<long long>(n) * nrhs) return;
  const long long i = t / nrhs, k = t % nrhs;
  b[k * n + i] = rows[t];
}

}  // namespace
}  // namespace sl3dgpu

using namespace sl3dgpu;

extern "C" int sl3dgpu_band_cholesky_solve_noalloc(const double* ab, int n, int kd, double* b, int nrhs,
                                                   void* stream) {
  if (n < 0 || kd < 0 || nrhs < 0) {
    SetError("negative order, bandwidth or column count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (n == 0 || nrhs == 0) return SL3DGPU_OK;
  if (ab == nullptr || b == nullptr) {
    SetError("null band or right-hand sides");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const int items = (nrhs + kSolveColumns - 1) / kSolveColumns;
  const long long rhsAt = ((kItemsAt + items + 31) / 32) * 32;
  const long long need = rhsAt + static_cast<long long>(n) * nrhs;
  if (need > kStaticDoubles) {
    SetError("the right-hand sides (n x nrhs = " + std::to_string(static_cast<long long>(n) * nrhs) +
             " values with the descriptor) exceed the static scratch of " + std::to_string(kStaticDoubles) +
             " doubles: split the columns over several calls");
    return SL3DGPU_ERR_ARGUMENT;
  }
  double* base = nullptr;
  if (int st = ScratchAddress(&base); st != SL3DGPU_OK) return st;
  const cudaStream_t s = AsStream(stream);
  sl3dgpu_band_system host{};
  host.n = n;
  host.kl = kd;
  host.ku = kd;
  host.nrhs = nrhs;
  host.rhs = rhsAt;
  host.scale = -1;
  host.pinned0 = host.pinned1 = -1;
  const long long total = static_cast<long long>(n) * nrhs;
  const unsigned blocks = static_cast<unsigned>((total + 255) / 256);
  DescribeKernel<<<1, 128, 0, s>>>(base, n, kd, nrhs, rhsAt, items);
  SL3D_CHECK_LAUNCH();
  ToRowsKernel<<<blocks, 256, 0, s>>>(b, n, nrhs, base + rhsAt);
  SL3D_CHECK_LAUNCH();
  if (int st = BandSolveBatch(reinterpret_cast<const sl3dgpu_band_system*>(base), &host, 1,
                              reinterpret_cast<const int2*>(base + kItemsAt), items, ab, nullptr, base, nullptr, 0,
                              s);
      st != SL3DGPU_OK)
    return st;
  ToColumnsKernel<<<blocks, 256, 0, s>>>(base + rhsAt, n, nrhs, b);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}
