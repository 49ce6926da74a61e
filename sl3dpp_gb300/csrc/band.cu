// Batched banded factorisations and solves on the device: every degree's
// spheroidal and toroidal system in one launch.
//
// The arithmetic is LAPACK's unblocked band algorithms as the reference
// restates them (src/BandSolvers.cpp:23-139; dpbtf2/dpbtrs, dgbtf2/dgbtrs)
// in the same band storage, with the same pivot choices, so factors agree
// with the reference's to rounding and failure indices exactly.
//
// GB300 layout:
//  - factorisation: one CTA per system; the band's active window (the kd+1
//    columns a rank-1 step touches, 2kl+ku+1 rows deep for LU) is staged in
//    shared memory as a ring and streamed column by column, so each band
//    value is read from and written to HBM once;
//  - solves: one warp per (system, 32 right-hand sides). Right-hand sides
//    are stored row-major (dof-major, the columns fastest), so a warp's load
//    of one dof across its 32 columns is one coalesced 256-byte access; a
//    degree's 2(l+1) real columns (its orders m >= 0, real and imaginary
//    parts) are its coalesced right-hand-side vectors. The recent solution
//    values live in a per-warp shared-memory ring; the band values are
//    broadcast reads. Optional diagonal scaling and pinned dofs are fused
//    in (DegreeOperator::BeginSolve/FinishSolve, src/DegreeOperator.cpp:861-901).
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "profile.cuh"

namespace sl3dgpu {
namespace {

constexpr int kRing = 64;  // solve ring depth: kd, kl + ku below this

__device__ inline double& WinAt(double* win, int ld, int window, int col, int row) {
  return win[(col % window) * ld + row];
}

// -- Cholesky factor -----------------------------------------------------------

__global__ void CholeskyFactorKernel(const sl3dgpu_band_system* systems, double* bands,
                                     int* info) {
  const sl3dgpu_band_system s = systems[blockIdx.x];
  const int n = s.n, kd = s.ku, ld = kd + 1, window = kd + 1;
  double* ab = bands + s.band;
  extern __shared__ double win[];  // window x ld
  __shared__ int failed;
  if (threadIdx.x == 0) failed = 0;
  for (int c = 0; c < min(window, n); ++c)
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      WinAt(win, ld, window, c, r) = ab[static_cast<long long>(c) * ld + r];
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const double d = WinAt(win, ld, window, j, kd);
    if (!(d > 0.0)) {
      if (threadIdx.x == 0) failed = j + 1;
      break;
    }
    const double ujj = sqrt(d);
    const double inverse = 1.0 / ujj;
    const int kn = min(kd, n - 1 - j);
    __syncthreads();  // every thread has read d before it is overwritten
    if (threadIdx.x == 0) WinAt(win, ld, window, j, kd) = ujj;
    for (int c = 1 + threadIdx.x; c <= kn; c += blockDim.x)
      WinAt(win, ld, window, j + c, kd - c) *= inverse;
    __syncthreads();
    // A(j + r, j + c) -= U(j, j + r) U(j, j + c), 1 <= r <= c <= kn.
    const int pairs = kn * (kn + 1) / 2;
    for (int t = threadIdx.x; t < pairs; t += blockDim.x) {
      int c = static_cast<int>((sqrt(8.0 * t + 1.0) - 1.0) * 0.5) + 1;
      while (c * (c - 1) / 2 > t) --c;
      while (c * (c + 1) / 2 <= t) ++c;
      const int r = t - c * (c - 1) / 2 + 1;
      const double ur = WinAt(win, ld, window, j + r, kd - r);
      const double uc = WinAt(win, ld, window, j + c, kd - c);
      WinAt(win, ld, window, j + c, kd + r - c) -= ur * uc;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      ab[static_cast<long long>(j) * ld + r] = WinAt(win, ld, window, j, r);
    __syncthreads();
    if (j + window < n)
      for (int r = threadIdx.x; r < ld; r += blockDim.x)
        WinAt(win, ld, window, j + window, r) =
            ab[static_cast<long long>(j + window) * ld + r];
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) info[blockIdx.x] = failed;
}

// -- LU factor (partial pivoting) --------------------------------------------------

__global__ void LuFactorKernel(const sl3dgpu_band_system* systems, double* bands,
                               int* pivotsAll, int* info) {
  const sl3dgpu_band_system s = systems[blockIdx.x];
  const int n = s.n, kl = s.kl, ku = s.ku, kv = kl + ku, ld = 2 * kl + ku + 1;
  const int window = kv + 1;
  double* ab = bands + s.band;
  int* pivots = pivotsAll + s.pivots;
  extern __shared__ double win[];
  __shared__ int pivot;
  auto at = [&](int i, int j) -> double& { return WinAt(win, ld, window, j, kv + i - j); };
  for (int c = 0; c < min(kv, n); ++c)
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      WinAt(win, ld, window, c, r) = ab[static_cast<long long>(c) * ld + r];
  __syncthreads();
  // The fill-in places of the first kv columns start zero (dgbtf2).
  for (int j = ku + 1; j < min(kv, n); ++j)
    for (int i = threadIdx.x; i < j - ku; i += blockDim.x) at(i, j) = 0.0;
  int infoValue = 0, ju = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (j + kv < n) {
      for (int r = threadIdx.x; r < ld; r += blockDim.x)
        WinAt(win, ld, window, j + kv, r) = ab[static_cast<long long>(j + kv) * ld + r];
      __syncthreads();
      for (int i = j + threadIdx.x; i < j + kl; i += blockDim.x) at(i, j + kv) = 0.0;
      __syncthreads();
    }
    const int km = min(kl, n - 1 - j);
    if (threadIdx.x == 0) {
      int p = j;
      for (int i = j + 1; i <= j + km; ++i)
        if (fabs(at(i, j)) > fabs(at(p, j))) p = i;
      pivot = p;
      pivots[j] = p;
    }
    __syncthreads();
    const int p = pivot;
    const bool zero = at(p, j) == 0.0;
    if (zero) {
      if (infoValue == 0) infoValue = j + 1;
    } else {
      ju = max(ju, min(p + ku, n - 1));
      if (p != j) {
        for (int c = j + threadIdx.x; c <= ju; c += blockDim.x) {
          const double t = at(p, c);
          at(p, c) = at(j, c);
          at(j, c) = t;
        }
      }
      __syncthreads();
      if (km > 0) {
        const double inverse = 1.0 / at(j, j);
        for (int i = j + 1 + threadIdx.x; i <= j + km; i += blockDim.x) at(i, j) *= inverse;
        __syncthreads();
        const int width = ju - j;
        for (int t = threadIdx.x; t < width * km; t += blockDim.x) {
          const int c = j + 1 + t / km;
          const int i = j + 1 + t % km;
          at(i, c) -= at(i, j) * at(j, c);
        }
      }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      ab[static_cast<long long>(j) * ld + r] = WinAt(win, ld, window, j, r);
    __syncthreads();
  }
  if (threadIdx.x == 0) info[blockIdx.x] = infoValue;
}

// -- solves --------------------------------------------------------------------------

struct WorkItem {
  int system;
  int column;
};

template <class T>
__device__ inline T LoadRhs(const sl3dgpu_band_system& s, const T* rhs, const T* scales, int j, int col) {
  if (j == s.pinned0 || j == s.pinned1) return T(0);
  T b = rhs[s.rhs + static_cast<long long>(j) * s.nrhs + col];
  if (s.scale >= 0) b *= scales[s.scale + j];
  return b;
}

template <class T>
__global__ void CholeskySolveKernel(const sl3dgpu_band_system* systems, const WorkItem* items, int itemCount,
                                    const T* bands, T* rhs, const T* scales) {
  const int warp = blockIdx.x * (blockDim.x / kWarp) + threadIdx.x / kWarp;
  const int lane = threadIdx.x % kWarp;
  extern __shared__ __align__(16) unsigned char ringBytes[];
  T* ring = reinterpret_cast<T*>(ringBytes) + (threadIdx.x / kWarp) * kRing * kWarp;
  if (warp >= itemCount) return;
  const WorkItem item = items[warp];
  const sl3dgpu_band_system s = systems[item.system];
  const int col = item.column + lane;
  const bool live = col < s.nrhs;
  const int n = s.n, kd = s.ku, ld = kd + 1;
  const T* ab = bands + s.band;
  T* x = rhs + s.rhs;
  // U^T y = b, forward.
  for (int j = 0; j < n; ++j) {
    T sum = live ? LoadRhs(s, rhs, scales, j, col) : T(0);
    const T* column = ab + static_cast<long long>(j) * ld + kd - j;  // column[i] = U(i, j)
    for (int i = max(0, j - kd); i < j; ++i) sum -= __ldg(column + i) * ring[(i % kRing) * kWarp + lane];
    const T y = sum / __ldg(column + j);
    ring[(j % kRing) * kWarp + lane] = y;
    if (live) x[static_cast<long long>(j) * s.nrhs + col] = y;
  }
  // U x = y, backward: row i takes its updates from j = i + kd down to i + 1.
  for (int i = n - 1; i >= 0; --i) {
    T v = live ? x[static_cast<long long>(i) * s.nrhs + col] : T(0);
    for (int j = min(n - 1, i + kd); j > i; --j)
      v -= __ldg(ab + static_cast<long long>(j) * ld + kd + i - j) * ring[(j % kRing) * kWarp + lane];
    v /= __ldg(ab + static_cast<long long>(i) * ld + kd);
    ring[(i % kRing) * kWarp + lane] = v;
    if (live) {
      T out = v;
      if (s.scale >= 0) out *= scales[s.scale + i];
      x[static_cast<long long>(i) * s.nrhs + col] = out;
    }
  }
}

template <class T>
__global__ void LuSolveKernel(const sl3dgpu_band_system* systems, const WorkItem* items, int itemCount,
                              const T* bands, const int* pivotsAll, T* rhs, const T* scales) {
  const int warp = blockIdx.x * (blockDim.x / kWarp) + threadIdx.x / kWarp;
  const int lane = threadIdx.x % kWarp;
  extern __shared__ __align__(16) unsigned char ringBytes[];
  T* ring = reinterpret_cast<T*>(ringBytes) + (threadIdx.x / kWarp) * kRing * kWarp;
  if (warp >= itemCount) return;
  const WorkItem item = items[warp];
  const sl3dgpu_band_system s = systems[item.system];
  const int col = item.column + lane;
  const bool live = col < s.nrhs;
  const int n = s.n, kl = s.kl, ku = s.ku, kv = kl + ku, ld = 2 * kl + ku + 1;
  const T* ab = bands + s.band;
  const int* pivots = pivotsAll + s.pivots;
  T* x = rhs + s.rhs;
  auto at = [&](int i, int j) { return __ldg(ab + static_cast<long long>(j) * ld + kv + i - j); };
  auto slot = [&](int i) -> T& { return ring[(i % kRing) * kWarp + lane]; };
  // L y = P^T b: the window x_j .. x_{j+kl} in the ring, interchanges and
  // eliminations in turn.
  for (int i = 0; i < min(kl, n); ++i) slot(i) = live ? LoadRhs(s, rhs, scales, i, col) : T(0);
  for (int j = 0; j < n; ++j) {
    if (j + kl < n) slot(j + kl) = live ? LoadRhs(s, rhs, scales, j + kl, col) : T(0);
    if (j + 1 < n) {
      const int p = pivots[j];
      if (p != j) {
        const T t = slot(p);
        slot(p) = slot(j);
        slot(j) = t;
      }
      const T xj = slot(j);
      const int lm = min(kl, n - 1 - j);
      for (int i = j + 1; i <= j + lm; ++i) slot(i) -= at(i, j) * xj;
    }
    if (live) x[static_cast<long long>(j) * s.nrhs + col] = slot(j);
  }
  // U x = y with kl + ku superdiagonals, backward.
  for (int i = n - 1; i >= 0; --i) {
    T v = live ? x[static_cast<long long>(i) * s.nrhs + col] : T(0);
    for (int j = min(n - 1, i + kv); j > i; --j) v -= at(i, j) * slot(j);
    v /= at(i, i);
    slot(i) = v;
    if (live) {
      T out = v;
      if (s.scale >= 0) out *= scales[s.scale + i];
      x[static_cast<long long>(i) * s.nrhs + col] = out;
    }
  }
}

int Validate(const sl3dgpu_band_system* hostSystems, int count, bool lu) {
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    if (s.n < 0 || s.kl < 0 || s.ku < 0 || s.nrhs < 0) {
      SetError("band system " + std::to_string(i) + ": negative size");
      return SL3DGPU_ERR_ARGUMENT;
    }
    const int reach = lu ? s.kl + s.ku : s.ku;
    if (reach >= kRing || (lu && s.kl >= kRing)) {
      SetError("band system " + std::to_string(i) + ": bandwidth beyond the solver's ring");
      return SL3DGPU_ERR_ARGUMENT;
    }
  }
  return SL3DGPU_OK;
}

}  // namespace

int BandFactorBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems,
                    int count, double* bands, int* pivots, int* info, int lu, cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  if (int st = Validate(hostSystems, count, lu != 0); st != SL3DGPU_OK) return st;
  int maxWindow = 0;
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    const int window = lu ? (s.kl + s.ku + 1) * (2 * s.kl + s.ku + 1) : (s.ku + 1) * (s.ku + 1);
    maxWindow = std::max(maxWindow, window);
  }
  const size_t smem = static_cast<size_t>(maxWindow) * sizeof(double);
  if (smem > 200 * 1024) {
    SetError("band factor window exceeds shared memory");
    return SL3DGPU_ERR_ARGUMENT;
  }
  prof::Scope scope(prof::kOther, stream);
  if (lu) {
    SL3D_CUDA(cudaFuncSetAttribute(LuFactorKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    LuFactorKernel<<<count, 128, smem, stream>>>(devSystems, bands, pivots, info);
  } else {
    SL3D_CUDA(cudaFuncSetAttribute(CholeskyFactorKernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    CholeskyFactorKernel<<<count, 128, smem, stream>>>(devSystems, bands, info);
  }
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// The work items of a batch: one per (system, 32 right-hand sides).
std::vector<int2> BandWorkItems(const sl3dgpu_band_system* hostSystems, int count) {
  std::vector<int2> items;
  for (int i = 0; i < count; ++i)
    for (int c = 0; c < hostSystems[i].nrhs; c += kWarp) items.push_back(make_int2(i, c));
  return items;
}

namespace {
template <class T>
int SolveBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
               const int2* devItems, int itemCount, const T* bands, const int* pivots, T* rhs, const T* scales,
               int lu, cudaStream_t stream) {
  if (itemCount == 0) return SL3DGPU_OK;
  if (int st = Validate(hostSystems, count, lu != 0); st != SL3DGPU_OK) return st;
  constexpr int warpsPerBlock = 4;
  const size_t smem = static_cast<size_t>(warpsPerBlock) * kRing * kWarp * sizeof(T);
  const int blocks = (itemCount + warpsPerBlock - 1) / warpsPerBlock;
  const auto* items = reinterpret_cast<const WorkItem*>(devItems);
  double flops = 0.0, bytes = 0.0;
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    const double n = s.n, r = s.nrhs;
    flops += lu ? r * (2.0 * n * s.kl + 2.0 * n * (s.kl + s.ku) + n) : r * (4.0 * n * s.ku + 2.0 * n);
    bytes += 4.0 * sizeof(T) * n * r + sizeof(T) * n * (lu ? 2 * s.kl + s.ku + 1 : s.ku + 1);
  }
  prof::Scope scope(sizeof(T) == sizeof(float) ? prof::kBandSolve32 : prof::kBandSolve, stream, flops, bytes);
  if (lu) {
    SL3D_CUDA(cudaFuncSetAttribute(LuSolveKernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    LuSolveKernel<T><<<blocks, warpsPerBlock * kWarp, smem, stream>>>(devSystems, items, itemCount, bands, pivots,
                                                                     rhs, scales);
  } else {
    SL3D_CUDA(cudaFuncSetAttribute(CholeskySolveKernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
    CholeskySolveKernel<T><<<blocks, warpsPerBlock * kWarp, smem, stream>>>(devSystems, items, itemCount, bands,
                                                                           rhs, scales);
  }
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}
}  // namespace

int BandSolveBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                   const int2* devItems, int itemCount, const double* bands, const int* pivots, double* rhs,
                   const double* scales, int lu, cudaStream_t stream) {
  return SolveBatch<double>(devSystems, hostSystems, count, devItems, itemCount, bands, pivots, rhs, scales, lu,
                            stream);
}

// The same solves in FP32 (the mixed form's correction passes).
int BandSolveBatchF(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                    const int2* devItems, int itemCount, const float* bands, const int* pivots, float* rhs,
                    const float* scales, int lu, cudaStream_t stream) {
  return SolveBatch<float>(devSystems, hostSystems, count, devItems, itemCount, bands, pivots, rhs, scales, lu,
                           stream);
}

}  // namespace sl3dgpu

// -- the C ABI -------------------------------------------------------------------------

using namespace sl3dgpu;

namespace {

// One host-resident system through the batched kernels (the drop-in form of
// detail::BandCholeskyFactor and friends): copies in, one launch, copies out.
struct DeviceScratch {
  std::vector<void*> owned;
  ~DeviceScratch() {
    for (void* p : owned) cudaFree(p);
  }
  template <class T>
  T* Alloc(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    owned.push_back(p);
    return static_cast<T*>(p);
  }
};

}  // namespace

extern "C" int sl3dgpu_band_cholesky_factor(double* ab, int n, int kd) {
  if (n < 0 || kd < 0) {
    SetError("negative order or bandwidth");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (n == 0) return 0;
  DeviceScratch scratch;
  const size_t size = static_cast<size_t>(kd + 1) * n;
  auto* band = scratch.Alloc<double>(size);
  auto* sys = scratch.Alloc<sl3dgpu_band_system>(1);
  auto* info = scratch.Alloc<int>(1);
  if (!band || !sys || !info) {
    SetError("device allocation failed");
    return SL3DGPU_ERR_CUDA;
  }
  sl3dgpu_band_system s{};
  s.n = n;
  s.kl = kd;
  s.ku = kd;
  s.scale = -1;
  s.pinned0 = s.pinned1 = -1;
  SL3D_CUDA(cudaMemcpy(band, ab, size * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(sys, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (int st = BandFactorBatch(sys, &s, 1, band, nullptr, info, 0, nullptr); st != SL3DGPU_OK)
    return st;
  int result = 0;
  SL3D_CUDA(cudaMemcpy(&result, info, sizeof(int), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(ab, band, size * sizeof(double), cudaMemcpyDeviceToHost));
  return result;
}

namespace {

// Column-major (n x nrhs) host right-hand sides through the row-major device
// solve, and back.
int SolveHost(const double* ab, size_t bandSize, const int* pivots, int n, int kl, int ku,
              double* b, int nrhs, int lu) {
  if (n == 0 || nrhs == 0) return SL3DGPU_OK;
  DeviceScratch scratch;
  auto* band = scratch.Alloc<double>(bandSize);
  auto* rhs = scratch.Alloc<double>(static_cast<size_t>(n) * nrhs);
  auto* sys = scratch.Alloc<sl3dgpu_band_system>(1);
  auto* piv = scratch.Alloc<int>(static_cast<size_t>(n));
  const auto hostItems = BandWorkItems(nullptr, 0);
  sl3dgpu_band_system s{};
  s.n = n;
  s.kl = kl;
  s.ku = ku;
  s.nrhs = nrhs;
  s.scale = -1;
  s.pinned0 = s.pinned1 = -1;
  auto items = BandWorkItems(&s, 1);
  auto* devItems = scratch.Alloc<int2>(items.size());
  if (!band || !rhs || !sys || !piv || !devItems) {
    SetError("device allocation failed");
    return SL3DGPU_ERR_CUDA;
  }
  std::vector<double> rowMajor(static_cast<size_t>(n) * nrhs);
  for (int k = 0; k < nrhs; ++k)
    for (int i = 0; i < n; ++i) rowMajor[static_cast<size_t>(i) * nrhs + k] = b[static_cast<size_t>(k) * n + i];
  SL3D_CUDA(cudaMemcpy(band, ab, bandSize * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(rhs, rowMajor.data(), rowMajor.size() * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(sys, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (lu) SL3D_CUDA(cudaMemcpy(piv, pivots, static_cast<size_t>(n) * sizeof(int), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(devItems, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
  if (int st = BandSolveBatch(sys, &s, 1, devItems, static_cast<int>(items.size()), band, piv, rhs,
                              nullptr, lu, nullptr);
      st != SL3DGPU_OK)
    return st;
  SL3D_CUDA(cudaMemcpy(rowMajor.data(), rhs, rowMajor.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int k = 0; k < nrhs; ++k)
    for (int i = 0; i < n; ++i) b[static_cast<size_t>(k) * n + i] = rowMajor[static_cast<size_t>(i) * nrhs + k];
  return SL3DGPU_OK;
}

}  // namespace

extern "C" int sl3dgpu_band_cholesky_solve(const double* ab, int n, int kd, double* b, int nrhs) {
  if (n < 0 || kd < 0 || nrhs < 0) {
    SetError("negative order, bandwidth or column count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return SolveHost(ab, static_cast<size_t>(kd + 1) * n, nullptr, n, kd, kd, b, nrhs, 0);
}

extern "C" int sl3dgpu_band_lu_factor(double* ab, int n, int kl, int ku, int* pivots) {
  if (n < 0 || kl < 0 || ku < 0) {
    SetError("negative order or bandwidth");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (n == 0) return 0;
  DeviceScratch scratch;
  const size_t size = static_cast<size_t>(2 * kl + ku + 1) * n;
  auto* band = scratch.Alloc<double>(size);
  auto* sys = scratch.Alloc<sl3dgpu_band_system>(1);
  auto* info = scratch.Alloc<int>(1);
  auto* piv = scratch.Alloc<int>(static_cast<size_t>(n));
  if (!band || !sys || !info || !piv) {
    SetError("device allocation failed");
    return SL3DGPU_ERR_CUDA;
  }
  sl3dgpu_band_system s{};
  s.n = n;
  s.kl = kl;
  s.ku = ku;
  s.scale = -1;
  s.pinned0 = s.pinned1 = -1;
  SL3D_CUDA(cudaMemcpy(band, ab, size * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(sys, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (int st = BandFactorBatch(sys, &s, 1, band, piv, info, 1, nullptr); st != SL3DGPU_OK) return st;
  int result = 0;
  SL3D_CUDA(cudaMemcpy(&result, info, sizeof(int), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(ab, band, size * sizeof(double), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(pivots, piv, static_cast<size_t>(n) * sizeof(int), cudaMemcpyDeviceToHost));
  return result;
}

extern "C" int sl3dgpu_band_lu_solve(const double* ab, int n, int kl, int ku, const int* pivots,
                                     double* b, int nrhs) {
  if (n < 0 || kl < 0 || ku < 0 || nrhs < 0) {
    SetError("negative order, bandwidth or column count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return SolveHost(ab, static_cast<size_t>(2 * kl + ku + 1) * n, pivots, n, kl, ku, b, nrhs, 1);
}

extern "C" int sl3dgpu_band_factor_batch(const sl3dgpu_band_system* dev_systems,
                                         const sl3dgpu_band_system* host_systems, int count,
                                         double* bands, int* pivots, int* info, int lu,
                                         void* stream) {
  return BandFactorBatch(dev_systems, host_systems, count, bands, pivots, info, lu,
                         AsStream(stream));
}

extern "C" int sl3dgpu_band_solve_batch(const sl3dgpu_band_system* dev_systems,
                                        const sl3dgpu_band_system* host_systems, int count,
                                        const int* dev_items, int item_count, const double* bands,
                                        const int* pivots, double* rhs, const double* scales,
                                        int lu, void* stream) {
  return BandSolveBatch(dev_systems, host_systems, count, reinterpret_cast<const int2*>(dev_items),
                        item_count, bands, pivots, rhs, scales, lu, AsStream(stream));
}

extern "C" int sl3dgpu_band_work_items(const sl3dgpu_band_system* host_systems, int count,
                                       int* items, int capacity) {
  const auto list = BandWorkItems(host_systems, count);
  if (items != nullptr) {
    if (capacity < static_cast<int>(list.size())) {
      SetError("work item buffer too small");
      return SL3DGPU_ERR_ARGUMENT;
    }
    for (size_t i = 0; i < list.size(); ++i) {
      items[2 * i] = list[i].x;
      items[2 * i + 1] = list[i].y;
    }
  }
  return static_cast<int>(list.size());
}
