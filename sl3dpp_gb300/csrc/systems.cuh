// The degree systems of one operator flavour on the device: every degree's
// spheroidal and toroidal band assembled and scaled on the GPU (assemble.cu),
// their batched factorisation (Cholesky, LU with partial pivoting where the
// Cholesky fails or a diagonal is not positive, src/DegreeOperator.cpp:
// 775-852), the work items of the batched solves, the load units
// K^-1 Load, and on request the assembled bands for K x and FP32 copies.
#pragma once

#include <vector>

#include "common.cuh"
#include "host/earth.hpp"
#include "step_kernels.cuh"

namespace sl3dgpu {

int BandFactorBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                    double* bands, int* pivots, int* info, int lu, cudaStream_t stream);
int BandSolveBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                   const int2* devItems, int itemCount, const double* bands, const int* pivots, double* rhs,
                   const double* scales, int lu, cudaStream_t stream);
int BandSolveBatchF(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                    const int2* devItems, int itemCount, const float* bands, const int* pivots, float* rhs,
                    const float* scales, int lu, cudaStream_t stream);
// The FP32 Cholesky solves over row windows (windows[system] = {lo, hi}, the
// right-hand side zero outside [lo, hi]): the substitutions' rows lo .. n - 1,
// or (completion) the backward substitution's rows 0 .. lo - 1 after them.
int BandSolveWindowF(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                     const int2* devItems, int itemCount, const float* bands, float* rhs, const float* scales,
                     const int2* windows, bool completion, cudaStream_t stream);
// Rows [lo, hi] of the systems' right-hand sides (up to three lists, each
// with its own right-hand-side array) set to zero.
void LaunchZeroRows(const sl3dgpu_band_system* s0, const int2* w0, int n0, float* rhs0,
                    const sl3dgpu_band_system* s1, const int2* w1, int n1, float* rhs1,
                    const sl3dgpu_band_system* s2, const int2* w2, int n2, float* rhs2, cudaStream_t stream);
std::vector<int2> BandWorkItems(const sl3dgpu_band_system* hostSystems, int count);

// A device allocation owned by value.
template <class T>
struct Dev {
  T* p = nullptr;
  size_t n = 0;
  Dev() = default;
  Dev(const Dev&) = delete;
  Dev& operator=(const Dev&) = delete;
  Dev(Dev&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  Dev& operator=(Dev&& o) noexcept {
    std::swap(p, o.p);
    std::swap(n, o.n);
    return *this;
  }
  ~Dev() { cudaFree(p); }
  cudaError_t Alloc(size_t count) {
    cudaFree(p);
    p = nullptr;
    n = count;
    return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
  }
  cudaError_t Upload(const std::vector<T>& v) {
    if (cudaError_t e = Alloc(v.size()); e != cudaSuccess) return e;
    return CopyIn(p, v.data(), v.size() * sizeof(T));
  }
};

#define SL3D_TRY(expr)                            \
  do {                                            \
    if (int _st = (expr); _st != SL3DGPU_OK) return _st; \
  } while (0)

// One flavour (scheme, dt): the factorised systems and the load units.
struct Flavour {
  int scheme = 0;
  double dt = 0.0;
  long long id = 0;  // unique per flavour built (a graph captured on it is keyed by it)
  Dev<double> bands, scales, units;
  // the tide channel's units K^-1 Tide per degree (the same offsets as units)
  // and, for conjugate gradients, the unsolved vectors
  Dev<double> tideUnits, tideForces;
  Dev<float> bands32, scales32;  // the mixed form's FP32 copies
  // the assembled (unscaled) bands in assembly-plan order, kept for K x;
  // for conjugate gradients their systems and the unsolved load force
  // vectors (DegreeOperator::Load)
  Dev<double> applyBands, loadForces;
  Dev<sl3dgpu_band_system> dSphApply, dTorApply;
  int nSphApply = 0, nTorApply = 0, maxApplyRows = 0;
  Dev<int> pivots;
  Dev<long long> unitOffset;
  std::vector<sl3dgpu_band_system> sphChol, sphLu, torChol;
  Dev<sl3dgpu_band_system> dSphChol, dSphLu, dTorChol;
  Dev<int2> iSphChol, iSphLu, iTorChol;
  int nSphChol = 0, nSphLu = 0, nTorChol = 0;
  // The FP32 correction's row windows per system ({lo, hi}: the rows its
  // lateral forces reach), for the lateral node range [windowFirst, windowEnd).
  mutable int windowFirst = -1, windowEnd = -1;
  mutable Dev<int2> wSphChol, wSphLu, wTorChol;
  // The flavour's effective Love numbers for the sea-level closure, built on
  // first use: h, k, l, ht, kt, lt per degree (lmax + 1 each), then h_c,
  // k_c, the load's inertia-trace number m and the centrifugal one m_c.
  std::vector<double> effectiveLove;
};


struct DeviceMaterial;
struct AssemblyPlan;

// What a flavour is built from: the operator's material on the device and
// its degrees' assembly plan (spheroidal degrees 0..lmax, then toroidal
// 1..lmax), the spheroidal layouts (load and tide vectors), the flavour's
// point shear (null for the plain elastic operators of the static problem)
// and the degrees' right-hand-side layout.
struct SystemsInput {
  const DeviceMaterial* material = nullptr;
  const AssemblyPlan* plan = nullptr;
  const std::vector<host::SpheroidalLayout>* sph = nullptr;
  const host::PointShear* shear = nullptr;
  int lmax = 0;
  const std::vector<DegreeInfo>* degrees = nullptr;
  long long rhsSphComplex = 0;  // where the toroidal columns start in a combined vector
  bool apply = false;           // keep the assembled bands and load vectors (K x, conjugate gradients)
  bool fp32 = false;            // FP32 copies of the factors (the mixed form)
  cudaStream_t stream = nullptr;
};
int BuildSystems(const SystemsInput& in, Flavour& f);

}  // namespace sl3dgpu
