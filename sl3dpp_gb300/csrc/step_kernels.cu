// Device kernels of the 3D step (see step_kernels.cuh).
//
// The degree <-> spin maps restate include/sl3dpp/SpinComponents.hpp:53-145
// and src/GridCoupling.cpp:595-809: one CTA per (degree l, order m >= 0), its
// threads over the memory nodes (coalesced on the [row][node] spectral
// layout) and then over the global mesh nodes of the degree's elements, with
// the per-node values staged in shared memory so that every dof is written by
// exactly one thread (no atomics, a fixed summation order).
#include <cmath>
#include <type_traits>

#include "host/lstsq.hpp"
#include "profile.cuh"
#include "step_kernels.cuh"

namespace sl3dgpu {
namespace {

template <class T2>
struct Scalar;
template <>
struct Scalar<double2> {
  using type = double;
};
template <>
struct Scalar<float2> {
  using type = float;
};

template <class T2>
__device__ inline T2 Cx(typename Scalar<T2>::type x, typename Scalar<T2>::type y) {
  T2 v;
  v.x = x;
  v.y = y;
  return v;
}
__device__ inline double2 C(double x, double y) { return make_double2(x, y); }
template <class T2>
__device__ inline T2 CAdd(T2 a, T2 b) {
  return Cx<T2>(a.x + b.x, a.y + b.y);
}
template <class T2>
__device__ inline T2 CSub(T2 a, T2 b) {
  return Cx<T2>(a.x - b.x, a.y - b.y);
}
template <class T2>
__device__ inline T2 CScale(typename Scalar<T2>::type s, T2 a) {
  return Cx<T2>(s * a.x, s * a.y);
}
template <class T2>
__device__ inline T2 CConj(T2 a) {
  return Cx<T2>(a.x, -a.y);
}
template <class T2>
__device__ inline T2 CI(T2 a) {  // i a
  return Cx<T2>(-a.y, a.x);
}

__device__ inline void DecodeLm(int lm, int& l, int& m) {
  l = static_cast<int>((sqrtf(8.0f * lm + 1.0f) - 1.0f) * 0.5f);  // a guess; the loops settle it
  while (l * (l + 1) / 2 > lm) --l;
  while ((l + 1) * (l + 2) / 2 <= lm) ++l;
  m = lm - l * (l + 1) / 2;
}

__device__ inline long long Row0(const Geometry& g, int l, int m) {
  return g.rowOff0[m + g.lmax] + (l - max(abs(m), 2));
}
__device__ inline long long Row1(const Geometry& g, int l, int m) {
  return g.rowOff1[m + g.lmax] + (l - max(abs(m), 1));
}
__device__ inline long long RowR(const Geometry& g, int l, int m) {
  return g.rowOffR[m + g.lmax] - g.rowOffR[g.lmax] + (l - m);
}

template <class T>
__device__ inline const T* Coef(const Geometry& g, int which);
template <>
__device__ inline const double* Coef<double>(const Geometry& g, int which) {
  return g.coef64[which];
}
template <>
__device__ inline const float* Coef<float>(const Geometry& g, int which) {
  return g.coef32[which];
}

template <class T2>
struct Rows {
  T2 u, v, w, du, dv, dw;
};

// ForceRowsFromComponents (SpinComponents.hpp:129-145).
template <class T2>
__device__ Rows<T2> ForceRows(int l, const T2 A[5], typename Scalar<T2>::type r) {
  using T = typename Scalar<T2>::type;
  const T zeta2 = l * (l + T(1)), zeta = sqrt(zeta2);
  const T root = sqrt(fmax(zeta2 - T(2), T(0)));
  const T s2 = T(1.41421356237309504880);
  const T2 s13 = CAdd(A[1], A[3]), d13 = CSub(A[1], A[3]);
  const T2 s04 = CAdd(A[0], A[4]), d04 = CSub(A[0], A[4]);
  Rows<T2> rows;
  rows.u = CSub(CScale(s2 * zeta, s13), CScale(T(4), A[2]));
  rows.v = CSub(CAdd(CScale(zeta * root, s04), CScale(T(2) * zeta2, A[2])), CScale(s2 * zeta, s13));
  rows.w = CI(CSub(CScale(zeta * root, d04), CScale(s2 * zeta, d13)));
  rows.du = CScale(T(4) * r, A[2]);
  rows.dv = CScale(s2 * zeta * r, s13);
  rows.dw = CI(CScale(s2 * zeta * r, d13));
  return rows;
}

// -- the force and strain maps over chunks of MC orders ------------------------------------------
//
// One block per (degree l, MC consecutive orders m0 .. m0 + MC - 1 <= l),
// the orders of a chunk side by side, so that the degree systems' right-hand
// sides and solutions, stored [dof][m] (m fastest), are read and written in
// runs of MC consecutive values, and the spectral rows [row][node] in runs
// of nodes. Every value is written by exactly one thread (no atomics, a fixed
// summation order); the sums per value are those of the reference's
// per-(l, m) loops.

// Blocks before degree l: sum over l' < l of (floor(l' / MC) + 1).
template <int MC>
__device__ inline int ChunksBefore(int l) {
  const int q = l / MC;
  return l + MC * q * (q - 1) / 2 + q * (l - q * MC);
}
template <int MC>
__device__ inline void DecodeChunk(int b, int lmax, int& l, int& m0) {
  int lo = 0, hi = lmax;  // the largest l with ChunksBefore(l) <= b
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (ChunksBefore<MC>(mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  l = lo;
  m0 = (b - ChunksBefore<MC>(l)) * MC;
}

// The memory force of an analysed (mu-weighted) tensor into the degree
// systems' right-hand sides (GridCoupling::SpheroidalForce/ToroidalForce,
// src/GridCoupling.cpp:613-809): per memory node the six force rows of the
// order's spin components, then per global node of the degree's carrying
// elements the quadrature over its elements' points.
template <class T2, int MC>
__global__ void ForceChunkKernel(Geometry g, const T2* spectral, T2* rhsSph, T2* rhsTor) {
  using T = typename Scalar<T2>::type;
  int l, m0;
  DecodeChunk<MC>(blockIdx.x, g.lmax, l, m0);
  const int mc = min(MC, l + 1 - m0);  // orders in this chunk
  const DegreeInfo d = g.degrees[l];
  if (d.firstNode >= g.P) return;
  const int np = g.P - d.firstNode;
  const int pPad = np | 1;  // odd row length: the epilogue's reads across orders miss no bank twice
  extern __shared__ __align__(16) unsigned char forceChunkSmem[];
  T2* rowsS = reinterpret_cast<T2*>(forceChunkSmem);  // [6][MC][pPad]
  const T2* c0 = spectral;
  const T2* c1 = spectral + g.rows0 * g.P;
  const T2* cr = spectral + (g.rows0 + g.rows1) * g.P;
  for (int t = threadIdx.x; t < mc * np; t += blockDim.x) {
    const int mi = t / np, p = d.firstNode + t % np, m = m0 + mi;
    const T sign = (m % 2 == 0) ? T(1) : T(-1);
    T2 A[5] = {Cx<T2>(0, 0), Cx<T2>(0, 0), Cx<T2>(0, 0), Cx<T2>(0, 0), Cx<T2>(0, 0)};
    A[2] = cr[RowR(g, l, m) * g.P + p];
    if (l >= 1) {
      A[1] = c1[Row1(g, l, m) * g.P + p];
      A[3] = CScale(sign, CConj(c1[Row1(g, l, -m) * g.P + p]));
    }
    if (l >= 2) {
      A[0] = c0[Row0(g, l, m) * g.P + p];
      A[4] = CScale(sign, CConj(c0[Row0(g, l, -m) * g.P + p]));
    }
    const Rows<T2> rows = ForceRows<T2>(l, A, static_cast<T>(g.nodeR[p]));
    T2* s = rowsS + static_cast<long long>(mi) * pPad + (p - d.firstNode);
    const long long k = static_cast<long long>(MC) * pPad;
    s[0] = rows.u;
    s[k] = rows.v;
    s[2 * k] = rows.w;
    s[3 * k] = rows.du;
    s[4 * k] = rows.dv;
    s[5 * k] = rows.dw;
  }
  __syncthreads();
  const int n = g.ngll, cols = l + 1;
  const int globals = d.lastGlobal - d.firstGlobal + 1;
  const T* fValue = Coef<T>(g, kForceValue);
  const T* fDeriv = Coef<T>(g, kForceDeriv);
  for (int t = threadIdx.x; t < globals * mc; t += blockDim.x) {
    const int mi = t % mc, gn = d.firstGlobal + t / mc;
    T2 bU = Cx<T2>(0, 0), bV = Cx<T2>(0, 0), bW = Cx<T2>(0, 0);
    const int eHi = min(gn / (n - 1), g.elements - 1);
    const int iHi = gn - eHi * (n - 1);
    const int eLo = (iHi == 0 && eHi > 0) ? eHi - 1 : eHi;
    for (int e = eLo; e <= eHi; ++e) {
      const int fn = g.elemFirstNode[e];
      if (fn < 0 || fn < d.firstNode) continue;
      const int i = e == eHi ? iHi : n - 1;
      for (int q = 0; q < g.np; ++q) {
        const int p = fn + q;
        const T2* s = rowsS + static_cast<long long>(mi) * pPad + (p - d.firstNode);
        const long long k = static_cast<long long>(MC) * pPad;
        const T v = fValue[p * n + i];
        const T deriv = fDeriv[p * n + i];
        bU = CAdd(bU, CScale(v, s[0]));
        bV = CAdd(bV, CScale(v, s[k]));
        bU = CAdd(bU, CScale(deriv, s[3 * k]));
        bV = CAdd(bV, CScale(deriv, s[4 * k]));
        bW = CAdd(bW, CScale(v, s[2 * k]));
        bW = CAdd(bW, CScale(deriv, s[5 * k]));
      }
    }
    const int m = m0 + mi;
    const int dU = g.sphMap[d.sphMap + 2LL * gn], dV = g.sphMap[d.sphMap + 2LL * gn + 1];
    if (dU >= 0) rhsSph[d.sphRhs + static_cast<long long>(dU) * cols + m] = bU;
    if (dV >= 0) rhsSph[d.sphRhs + static_cast<long long>(dV) * cols + m] = bV;
    if (l >= 1) {
      const int dW = g.torMap[d.torMap + gn];
      if (dW >= 0) rhsTor[d.torRhs + static_cast<long long>(dW) * cols + m] = bW;
    }
  }
}

// StrainOf (AddStrainOfSolution + DeviatoricComponents, SpinComponents.hpp:
// 53-72, + Scatter with the -m twins from the derived components): the
// degree's U, V, W at the carrying elements' GLL nodes, then per memory node
// the five deviatoric components; `add` (the same layout), when given, added.
template <class T2, int MC>
__global__ void StrainChunkKernel(Geometry g, const T2* solSph, const T2* solTor, T2* spectral, const T2* add) {
  using T = typename Scalar<T2>::type;
  int l, m0;
  DecodeChunk<MC>(blockIdx.x, g.lmax, l, m0);
  const int mc = min(MC, l + 1 - m0);
  const DegreeInfo d = g.degrees[l];
  extern __shared__ __align__(16) unsigned char strainChunkSmem[];
  T2* vals = reinterpret_cast<T2*>(strainChunkSmem);  // [global node][3 MC + 1]
  constexpr int kRow = 3 * MC + 1;                    // odd: reads across nodes miss no bank twice
  T2* c0 = spectral;
  T2* c1 = spectral + g.rows0 * g.P;
  T2* cr = spectral + (g.rows0 + g.rows1) * g.P;
  const int cols = l + 1;
  const bool any = d.firstNode < g.P;
  if (any) {
    const int globals = d.lastGlobal - d.firstGlobal + 1;
    for (int t = threadIdx.x; t < globals * mc; t += blockDim.x) {
      const int mi = t % mc, gn = d.firstGlobal + t / mc, m = m0 + mi;
      const int dU = g.sphMap[d.sphMap + 2LL * gn], dV = g.sphMap[d.sphMap + 2LL * gn + 1];
      T2* v = vals + static_cast<long long>(gn - d.firstGlobal) * kRow + mi;
      v[0] = dU >= 0 ? solSph[d.sphRhs + static_cast<long long>(dU) * cols + m] : Cx<T2>(0, 0);
      v[MC] = dV >= 0 ? solSph[d.sphRhs + static_cast<long long>(dV) * cols + m] : Cx<T2>(0, 0);
      T2 W = Cx<T2>(0, 0);
      if (l >= 1) {
        const int dW = g.torMap[d.torMap + gn];
        if (dW >= 0) W = solTor[d.torRhs + static_cast<long long>(dW) * cols + m];
      }
      v[2 * MC] = W;
    }
  }
  __syncthreads();
  const int n = g.ngll;
  const T zeta2 = l * (l + T(1)), zeta = sqrt(zeta2);
  const T s2 = T(1.41421356237309504880);
  auto put = [&](T2* base, long long at, T2 v) {
    const long long i = (base - spectral) + at;
    spectral[i] = add != nullptr ? CAdd(v, add[i]) : v;
  };
  for (int t = threadIdx.x; t < mc * g.P; t += blockDim.x) {
    const int mi = t / g.P, p = t % g.P, m = m0 + mi;
    const T sign = (m % 2 == 0) ? T(1) : T(-1);
    T2 A[5] = {Cx<T2>(0, 0), Cx<T2>(0, 0), Cx<T2>(0, 0), Cx<T2>(0, 0), Cx<T2>(0, 0)};
    if (any && p >= d.firstNode) {
      const int e = g.nodeElement[p];
      const T r = static_cast<T>(g.nodeR[p]);
      const T* sValue = Coef<T>(g, kStrainValue) + p * n;
      const T* sDeriv = Coef<T>(g, kStrainDeriv) + p * n;
      T2 U = Cx<T2>(0, 0), V = Cx<T2>(0, 0), W = Cx<T2>(0, 0), rdU = Cx<T2>(0, 0), rdV = Cx<T2>(0, 0),
         rdW = Cx<T2>(0, 0);
      for (int i = 0; i < n; ++i) {
        const T2* v = vals + static_cast<long long>(e * (n - 1) + i - d.firstGlobal) * kRow + mi;
        const T val = sValue[i];
        U = CAdd(U, CScale(val, v[0]));
        V = CAdd(V, CScale(val, v[MC]));
        W = CAdd(W, CScale(val, v[2 * MC]));
        const T b = sDeriv[i];
        rdU = CAdd(rdU, CScale(b, v[0]));
        rdV = CAdd(rdV, CScale(b, v[MC]));
        rdW = CAdd(rdW, CScale(b, v[2 * MC]));
      }
      const T2 t2 = CAdd(CSub(rdU, U), CScale(T(0.5) * zeta2, V));
      A[2] = Cx<T2>(t2.x / (T(3) * r), t2.y / (T(3) * r));
      if (l >= 1) {
        const T2 tangential = CAdd(CSub(rdV, V), U);
        const T2 twist = CSub(W, rdW);
        const T den = T(2) * s2 * r;
        const T2 a1 = CScale(zeta, CAdd(tangential, CI(twist)));
        const T2 a3 = CScale(zeta, CSub(tangential, CI(twist)));
        A[1] = Cx<T2>(a1.x / den, a1.y / den);
        A[3] = Cx<T2>(a3.x / den, a3.y / den);
      }
      if (l >= 2) {
        const T factor = T(0.5) * zeta * sqrt(zeta2 - T(2)) / r;
        A[0] = CScale(factor, CSub(V, CI(W)));
        A[4] = CScale(factor, CAdd(V, CI(W)));
      }
    }
    if (l >= 2) {
      put(c0, Row0(g, l, m) * g.P + p, A[0]);
      if (m > 0) put(c0, Row0(g, l, -m) * g.P + p, CScale(sign, CConj(A[4])));
    }
    if (l >= 1) {
      put(c1, Row1(g, l, m) * g.P + p, A[1]);
      if (m > 0) put(c1, Row1(g, l, -m) * g.P + p, CScale(sign, CConj(A[3])));
    }
    put(cr, RowR(g, l, m) * g.P + p, A[2]);
  }
}

// One block per (l, m >= 0): the degree's U, V at its
// carrying elements' GLL nodes in shared memory, then per memory node the
// dilatation rdU + 2 U - l(l+1) V.
__global__ void DilatationKernel(Geometry g, const double2* solSph, double2* scalar) {
  int l, m;
  DecodeLm(blockIdx.x, l, m);
  const DegreeInfo d = g.degrees[l];
  extern __shared__ __align__(16) unsigned char dilSmem[];
  double2* vals = reinterpret_cast<double2*>(dilSmem);  // (lastGlobal - firstGlobal + 1) x 2
  const int cols = l + 1;
  const bool any = d.firstNode < g.P;
  if (any)
    for (int gn = d.firstGlobal + threadIdx.x; gn <= d.lastGlobal; gn += blockDim.x) {
      const int dU = g.sphMap[d.sphMap + 2LL * gn], dV = g.sphMap[d.sphMap + 2LL * gn + 1];
      double2* v = vals + static_cast<long long>(gn - d.firstGlobal) * 2;
      v[0] = dU >= 0 ? solSph[d.sphRhs + static_cast<long long>(dU) * cols + m] : C(0, 0);
      v[1] = dV >= 0 ? solSph[d.sphRhs + static_cast<long long>(dV) * cols + m] : C(0, 0);
    }
  __syncthreads();
  const int n = g.ngll;
  const double k2 = l * (l + 1.0);
  for (int p = threadIdx.x; p < g.P; p += blockDim.x) {
    double2 D = C(0, 0);
    if (any && p >= d.firstNode) {
      const int e = g.nodeElement[p], q = g.nodeQ[p];
      const double r = g.nodeR[p], jac = g.elemJac[e];
      double2 U = C(0, 0), V = C(0, 0), rdU = C(0, 0);
      for (int i = 0; i < n; ++i) {
        const double2* v = vals + static_cast<long long>(e * (n - 1) + i - d.firstGlobal) * 2;
        const double val = g.pValue[q * n + i];
        U = CAdd(U, CScale(val, v[0]));
        V = CAdd(V, CScale(val, v[1]));
        rdU = CAdd(rdU, CScale(r * g.pDeriv[q * n + i] / jac, v[0]));
      }
      D = CSub(CAdd(rdU, CScale(2.0, U)), CScale(k2, V));
    }
    scalar[RowR(g, l, m) * g.P + p] = D;
  }
}

// One block per (l, m >= 0): per global node of the degree's
// range, the quadrature over its elements' memory points of
// 2 w jac D Value (U), -l(l+1) w jac D Value (V) and w Deriv r D (U),
// added onto the right-hand side.
__global__ void DilatationForceKernel(Geometry g, const double2* scalar, double2* rhsSph) {
  int l, m;
  DecodeLm(blockIdx.x, l, m);
  const DegreeInfo d = g.degrees[l];
  if (d.firstNode >= g.P) return;
  extern __shared__ __align__(16) unsigned char dfSmem[];
  double2* Ds = reinterpret_cast<double2*>(dfSmem);  // (P - first)
  for (int p = d.firstNode + threadIdx.x; p < g.P; p += blockDim.x) Ds[p - d.firstNode] = scalar[RowR(g, l, m) * g.P + p];
  __syncthreads();
  const int n = g.ngll, cols = l + 1;
  const double k2 = l * (l + 1.0);
  for (int gn = d.firstGlobal + threadIdx.x; gn <= d.lastGlobal; gn += blockDim.x) {
    double2 bU = C(0, 0), bV = C(0, 0);
    const int eHi = min(gn / (n - 1), g.elements - 1);
    const int iHi = gn - eHi * (n - 1);
    const int eLo = (iHi == 0 && eHi > 0) ? eHi - 1 : eHi;
    for (int e = eLo; e <= eHi; ++e) {
      const int fn = g.elemFirstNode[e];
      if (fn < 0 || fn < d.firstNode) continue;
      const int i = e == eHi ? iHi : n - 1;
      const double jac = g.elemJac[e];
      for (int q = 0; q < g.np; ++q) {
        const int p = fn + q;
        const double2 D = Ds[p - d.firstNode];
        const double point = jac * g.pWeight[q] * g.pValue[q * n + i];
        bU = CAdd(bU, CScale(2.0 * point, D));
        bV = CSub(bV, CScale(k2 * point, D));
        bU = CAdd(bU, CScale(g.pWeight[q] * g.pDeriv[q * n + i] * g.nodeR[p], D));
      }
    }
    const int dU = g.sphMap[d.sphMap + 2LL * gn], dV = g.sphMap[d.sphMap + 2LL * gn + 1];
    if (dU >= 0) {
      double2& x = rhsSph[d.sphRhs + static_cast<long long>(dU) * cols + m];
      x = CAdd(x, bU);
    }
    if (dV >= 0) {
      double2& x = rhsSph[d.sphRhs + static_cast<long long>(dV) * cols + m];
      x = CAdd(x, bV);
    }
  }
}

// x += sigma_lm units_l (+ tide_lm tideUnits_l): AddUnitChannels
// (Viscoelastic3D.cpp:1029-1073), the load column then the tide's; either
// coefficient array may be null.
__global__ void AddLoadKernel(Geometry g, const double2* sigma, const double* units, const double2* tide,
                              const double* tideUnits, const long long* unitOffset, double2* sol) {
  const int l = blockIdx.x;
  const DegreeInfo d = g.degrees[l];
  const int cols = l + 1;
  const long long total = static_cast<long long>(d.sphNdof) * cols;
  for (long long t = threadIdx.x; t < total; t += blockDim.x) {
    const int dof = static_cast<int>(t / cols), m = static_cast<int>(t % cols);
    double2& x = sol[d.sphRhs + t];
    if (sigma != nullptr) {
      const double2 a = sigma[l * (l + 1) / 2 + m];
      if (a.x != 0.0 || a.y != 0.0) x = CAdd(x, CScale(units[unitOffset[l] + dof], a));
    }
    if (tide != nullptr) {
      const double2 a = tide[l * (l + 1) / 2 + m];
      if (a.x != 0.0 || a.y != 0.0) x = CAdd(x, CScale(tideUnits[unitOffset[l] + dof], a));
    }
  }
}

__global__ void SurfaceKernel(Geometry g, const double2* sol, const double2* solTor, int component, double2* out) {
  const int lm = blockIdx.x * blockDim.x + threadIdx.x;
  const int count = (g.lmax + 1) * (g.lmax + 2) / 2;
  if (lm >= count) return;
  int l, m;
  DecodeLm(lm, l, m);
  const DegreeInfo d = g.degrees[l];
  if (component == 3) {  // SurfaceToroidal: W
    out[lm] = d.surfaceW >= 0 ? solTor[d.torRhs + static_cast<long long>(d.surfaceW) * (l + 1) + m] : C(0, 0);
    return;
  }
  const int dof = component == 0 ? d.surfaceU : component == 1 ? d.surfaceV : d.surfacePhi;
  out[lm] = dof >= 0 ? sol[d.sphRhs + static_cast<long long>(dof) * (l + 1) + m] : C(0, 0);
}

// -- streaming kernels -----------------------------------------------------------------------

__device__ inline double Phi1(double h, double e) {
  if (fabs(h) < 1e-3) return 1.0 - h / 2.0 + h * h / 6.0 - h * h * h / 24.0 + h * h * h * h / 120.0;
  return (1.0 - e) / h;
}

// A stage's weights at one grid value of step h = dt itau: the decay e, the
// start strain's share alpha and the end strain's share beta
// (ExponentialTrapezoidWeights or BackwardEulerWeight).
__device__ inline void StageWeights(int scheme, double h, double& e, double& alpha, double& beta) {
  if (scheme == 1) {
    const double wbe = 1.0 / (1.0 + h);
    e = wbe;
    alpha = 0.0;
    beta = 1.0 - wbe;
  } else {
    const double ex = exp(-h);
    const double phi1 = Phi1(h, ex);
    e = ex;
    alpha = phi1 - ex;
    beta = 1.0 - phi1;
  }
}

__global__ void WeightsKernel(WeightsArgs a) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const int P = static_cast<int>(a.values / a.fieldSize);
  for (long long x = a.begin + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < a.end;
       x += stride) {
    const int node = static_cast<int>(x / a.fieldSize);
    double w = 0.0;
    double2 f0 = C(0, 0), f1 = C(0, 0);
    double fr = 0.0;
    for (int k = 0; k < a.branches; ++k) {
      const double itauRef = a.itauRef[static_cast<long long>(k) * P + node];
      const double mu = a.muBranch[static_cast<long long>(k) * P + node];
      const double h0 = a.dt * itauRef;
      double refBeta;
      if (a.scheme == 1) {
        refBeta = 1.0 - 1.0 / (1.0 + h0);
      } else {
        const double e0 = exp(-h0);
        refBeta = 1.0 - Phi1(h0, e0);
      }
      const double h = a.dt * (itauRef * a.factor[x]);
      double ew, aw, bw;
      if (a.scheme == 1) {
        const double wbe = 1.0 / (1.0 + h);
        ew = wbe;
        aw = 0.0;
        bw = 1.0 - wbe;
      } else {
        const double e = exp(-h);
        const double phi1 = Phi1(h, e);
        ew = e;
        aw = phi1 - e;
        bw = 1.0 - phi1;
      }
      a.beta[k][x] = bw;
      const double2 m0 = a.m0[k][x], m1 = a.m1[k][x];
      const double mr = a.mr[k][x];
      const double2 o0 = C(ew * m0.x + aw * a.d0c0[x].x, ew * m0.y + aw * a.d0c0[x].y);
      const double2 o1 = C(ew * m1.x + aw * a.d0c1[x].x, ew * m1.y + aw * a.d0c1[x].y);
      const double orr = ew * mr + aw * a.d0r[x];
      a.out0[k][x] = o0;
      a.out1[k][x] = o1;
      a.outr[k][x] = orr;
      if (k == 0) {
        w = 0.0 + mu * (bw - refBeta);
        f0 = C(0.0 + mu * o0.x, 0.0 + mu * o0.y);
        f1 = C(0.0 + mu * o1.x, 0.0 + mu * o1.y);
        fr = 0.0 + mu * orr;
        continue;
      }
      if (mu == 0.0) continue;
      w += mu * (bw - refBeta);
      f0 = C(f0.x + mu * o0.x, f0.y + mu * o0.y);
      f1 = C(f1.x + mu * o1.x, f1.y + mu * o1.y);
      fr += mu * orr;
    }
    a.weight[x] = w;
    a.fixed0[x] = f0;
    a.fixed1[x] = f1;
    a.fixedr[x] = fr;
  }
}

__global__ void AdvanceKernel(long long values, const double* beta, const double2* d0, const double2* d1,
                              const double* dr, double2* m0, double2* m1, double* mr) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long x = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < values; x += stride) {
    const double b = beta[x];
    m0[x] = C(m0[x].x + b * d0[x].x, m0[x].y + b * d0[x].y);
    m1[x] = C(m1[x].x + b * d1[x].x, m1[x].y + b * d1[x].y);
    mr[x] += b * dr[x];
  }
}

__global__ void StageCombineKernel(long long values, double r, const double2* a0, const double2* a1,
                                   const double* ar, double2* o0, double2* o1, double* orr) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const double s = 1.0 - r;
  for (long long x = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < values; x += stride) {
    o0[x] = C((0.0 + s * a0[x].x) + r * o0[x].x, (0.0 + s * a0[x].y) + r * o0[x].y);
    o1[x] = C((0.0 + s * a1[x].x) + r * o1[x].x, (0.0 + s * a1[x].y) + r * o1[x].y);
    orr[x] = (0.0 + s * ar[x]) + r * orr[x];
  }
}

__global__ void CombineKernel(long long values, long long fieldSize, const double* mu, bool first,
                              const double2* m0, const double2* m1, const double* mr, double2* o0,
                              double2* o1, double* orr) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long x = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < values; x += stride) {
    const double u = mu[x / fieldSize];
    if (first) {
      if (u == 0.0) {
        o0[x] = C(0, 0);
        o1[x] = C(0, 0);
        orr[x] = 0.0;
      } else {
        o0[x] = C(0.0 + u * m0[x].x, 0.0 + u * m0[x].y);
        o1[x] = C(0.0 + u * m1[x].x, 0.0 + u * m1[x].y);
        orr[x] = 0.0 + u * mr[x];
      }
    } else if (u != 0.0) {
      o0[x] = C(o0[x].x + u * m0[x].x, o0[x].y + u * m0[x].y);
      o1[x] = C(o1[x].x + u * m1[x].x, o1[x].y + u * m1[x].y);
      orr[x] += u * mr[x];
    }
  }
}

// -- the convergence measure ------------------------------------------------------------------

// Per block: max |next|^2, max |next - now|^2 and finiteness, in the data's
// precision (a maximum of squares loses nothing to the order). Both iterates
// must be finite: the reference tests `next` alone, where a non-finite `now`
// can only come from its previous pass; here `now` may be a caller's or an
// extrapolated guess, and a NaN in it would otherwise vanish from the
// maxima (a NaN with its sign bit set is the largest bit pattern, and fmax
// drops NaNs), under-reporting the change.
template <class T2>
__global__ void RelativeChangeKernel(const T2* next, const T2* now, long long n, double* partial) {
  using T = typename Scalar<T2>::type;
  __shared__ double s0[256], s1[256], s2[256];
  T scale = 0, diff = 0;
  bool finite = true;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  if constexpr (sizeof(T) == sizeof(double)) {
    // FP64: the finiteness test and the maxima on the bits (a square is
    // never negative, and non-negative doubles order as their bit patterns),
    // so that only the squares and differences use GB300's small FP64 unit
    unsigned long long scaleBits = 0, diffBits = 0, nonFinite = 0;
    constexpr unsigned long long kExp = 0x7ff0000000000000ull;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride) {
      const T2 a = next[i], b = now[i];
      const unsigned long long ax = __double_as_longlong(a.x), ay = __double_as_longlong(a.y);
      const unsigned long long bx = __double_as_longlong(b.x), by = __double_as_longlong(b.y);
      nonFinite |= static_cast<unsigned long long>((ax & kExp) == kExp) | static_cast<unsigned long long>((ay & kExp) == kExp) |
                   static_cast<unsigned long long>((bx & kExp) == kExp) | static_cast<unsigned long long>((by & kExp) == kExp);
      const double dx = a.x - b.x, dy = a.y - b.y;
      scaleBits = max(scaleBits, static_cast<unsigned long long>(__double_as_longlong(a.x * a.x + a.y * a.y)));
      diffBits = max(diffBits, static_cast<unsigned long long>(__double_as_longlong(dx * dx + dy * dy)));
    }
    scale = __longlong_as_double(static_cast<long long>(scaleBits));
    diff = __longlong_as_double(static_cast<long long>(diffBits));
    finite = nonFinite == 0;
  } else {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride) {
      const T2 a = next[i], b = now[i];
      finite = finite && (a.x - a.x == T(0)) && (a.y - a.y == T(0)) && (b.x - b.x == T(0)) && (b.y - b.y == T(0));
      scale = fmax(scale, a.x * a.x + a.y * a.y);
      const T dx = a.x - b.x, dy = a.y - b.y;
      diff = fmax(diff, dx * dx + dy * dy);
    }
  }
  s0[threadIdx.x] = static_cast<double>(scale);
  s1[threadIdx.x] = static_cast<double>(diff);
  s2[threadIdx.x] = finite ? 1.0 : 0.0;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) {
      s0[threadIdx.x] = fmax(s0[threadIdx.x], s0[threadIdx.x + w]);
      s1[threadIdx.x] = fmax(s1[threadIdx.x], s1[threadIdx.x + w]);
      s2[threadIdx.x] = fmin(s2[threadIdx.x], s2[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[blockIdx.x * 3 + 0] = s0[0];
    partial[blockIdx.x * 3 + 1] = s1[0];
    partial[blockIdx.x * 3 + 2] = s2[0];
  }
}

__global__ void ReduceMaxKernel(const double* partial, int count, double* result) {
  __shared__ double s0[256], s1[256], s2[256];
  double a = 0.0, b = 0.0, c = 1.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) {
    a = fmax(a, partial[3 * i]);
    b = fmax(b, partial[3 * i + 1]);
    c = fmin(c, partial[3 * i + 2]);
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  s2[threadIdx.x] = c;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) {
      s0[threadIdx.x] = fmax(s0[threadIdx.x], s0[threadIdx.x + w]);
      s1[threadIdx.x] = fmax(s1[threadIdx.x], s1[threadIdx.x + w]);
      s2[threadIdx.x] = fmin(s2[threadIdx.x], s2[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    result[0] = s0[0];
    result[1] = s1[0];
    result[2] = s2[0];
  }
}

// -- the Anderson mixer ---------------------------------------------------------------------------

template <class T>
__global__ void MixerFirstKernel(long long n, T* x, const T* gx, T* xPrev, T* fPrev, const int* live) {
  if (live != nullptr && live[0] != kLiveFirst) return;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride) {
    xPrev[i] = x[i];
    fPrev[i] = gx[i] - x[i];
    x[i] = gx[i];
  }
}

constexpr int kMixThreads = 256;
constexpr int kMaxMemory = kMixMaxMemory;

// The accumulation type of the mixer's per-thread sums: FP64 for the FP64
// form, FP32 for the correction (a thread sums about a hundred products; the
// warp and block sums and the Gram solve are FP64 in both).
template <class T>
struct MixAcc {
  using type = double;
};
template <>
struct MixAcc<float> {
  using type = float;
};

// A history value stored and read back (identity for the FP64 form).
__device__ inline double ToHistory(double v, double*) { return v; }
__device__ inline __nv_bfloat16 ToHistory(float v, __nv_bfloat16*) { return __float2bfloat16_rn(v); }
__device__ inline double FromHistory(double v) { return v; }
__device__ inline float FromHistory(__nv_bfloat16 v) { return __bfloat162float(v); }

// The sweep and mix kernels take the history count M as a template
// argument, so that their per-column arrays (pointers, sums, gamma) stay in
// registers; LaunchForMemory picks the instance for a.m.

// A block's partial Gram column and right-hand side: warp shuffle trees,
// then the warps in turn, written to partial[block][0..M) and
// [kMaxMemory..kMaxMemory + M).
template <int M, class A>
__device__ inline void MixerBlockPartials(const A (&col)[M + 1], const A (&gam)[M + 1], double* partial) {
  __shared__ double red[kMixThreads / 32][2 * kMaxMemory];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
#pragma unroll
  for (int i = 0; i < M; ++i) {
    A c = col[i], g = gam[i];
    for (int off = 16; off > 0; off /= 2) {
      c += __shfl_down_sync(0xffffffffu, c, off);
      g += __shfl_down_sync(0xffffffffu, g, off);
    }
    if (lane == 0) {
      red[warp][i] = static_cast<double>(c);
      red[warp][kMaxMemory + i] = static_cast<double>(g);
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kMaxMemory) {
    const int i = threadIdx.x;
    if (i % kMaxMemory < M) {
      double v = 0.0;
      for (int w = 0; w < kMixThreads / 32; ++w) v += red[w][i];
      partial[static_cast<long long>(blockIdx.x) * 2 * kMaxMemory + i] = v;
    }
  }
}

// One block per fixed chunk of the vector (fixed by n alone): the new
// differences, the stored iterate and residual, and the block's partial Gram
// column and right-hand side, summed in a fixed order.
template <class T, int M>
__global__ void MixerSweepKernel(MixerArgsT<T> a) {
  using A = typename MixAcc<T>::type;
  using H = typename MixerArgsT<T>::H;
  int m = M, slot = a.slot;
  if (a.live != nullptr) {
    if (a.live[0] != kLiveUpdate) return;
    m = a.live[1];
    slot = a.live[2];
  }
  const long long begin = a.n * blockIdx.x / a.blocks, end = a.n * (blockIdx.x + 1) / a.blocks;
  A col[M + 1], gam[M + 1];
#pragma unroll
  for (int i = 0; i <= M; ++i) col[i] = gam[i] = A(0);
  H* dFs = a.dF[slot];
  H* dGs = a.dG[slot];
  const H* dF[M + 1];
#pragma unroll
  for (int i = 0; i < M; ++i) dF[i] = a.dF[i];
  for (long long at = begin + threadIdx.x; at < end; at += blockDim.x) {
    const T xs = a.x[at], gs = a.gx[at];
    const T f = gs - xs;
    const T dx = xs - a.xPrev[at];
    const H dfStored = ToHistory(f - a.fPrev[at], dFs);
    dFs[at] = dfStored;
    dGs[at] = ToHistory(dx + (f - a.fPrev[at]), dGs);
    a.xPrev[at] = xs;
    a.fPrev[at] = f;
    // the new column as stored, so that the Gram matrix is the stored vectors'
    const A df = static_cast<A>(FromHistory(dfStored));
#pragma unroll
    for (int i = 0; i < M; ++i) {
      if (i >= m) break;
      const A di = i == slot ? df : static_cast<A>(FromHistory(dF[i][at]));
      col[i] += di * df;
      gam[i] += di * static_cast<A>(f);
    }
  }
  MixerBlockPartials<M>(col, gam, a.partial);
}

// Two values a thread (FP32 iterate, BF16 history): the same sweep as
// MixerSweepKernel<float, M> with 8-byte and 4-byte accesses.
template <int M>
__global__ void MixerSweepPairsKernel(MixerArgsT<float> a) {
  int m = M, slot = a.slot;
  if (a.live != nullptr) {
    if (a.live[0] != kLiveUpdate) return;
    m = a.live[1];
    slot = a.live[2];
  }
  const long long pairs = a.n / 2;
  const long long begin = pairs * blockIdx.x / a.blocks, end = pairs * (blockIdx.x + 1) / a.blocks;
  float col[M + 1], gam[M + 1];
#pragma unroll
  for (int i = 0; i <= M; ++i) col[i] = gam[i] = 0.0f;
  auto* x = reinterpret_cast<const float2*>(a.x);
  auto* gx = reinterpret_cast<const float2*>(a.gx);
  auto* xPrev = reinterpret_cast<float2*>(a.xPrev);
  auto* fPrev = reinterpret_cast<float2*>(a.fPrev);
  auto* dFs = reinterpret_cast<__nv_bfloat162*>(a.dF[slot]);
  auto* dGs = reinterpret_cast<__nv_bfloat162*>(a.dG[slot]);
  const __nv_bfloat162* dF[M + 1];
#pragma unroll
  for (int i = 0; i < M; ++i) dF[i] = reinterpret_cast<const __nv_bfloat162*>(a.dF[i]);
  for (long long at = begin + threadIdx.x; at < end; at += blockDim.x) {
    const float2 xs = x[at], gs = gx[at], xp = xPrev[at], fp = fPrev[at];
    const float2 f = make_float2(gs.x - xs.x, gs.y - xs.y);
    const float2 dfRaw = make_float2(f.x - fp.x, f.y - fp.y);
    const __nv_bfloat162 dfStored = __floats2bfloat162_rn(dfRaw.x, dfRaw.y);
    dFs[at] = dfStored;
    dGs[at] = __floats2bfloat162_rn(xs.x - xp.x + dfRaw.x, xs.y - xp.y + dfRaw.y);
    xPrev[at] = xs;
    fPrev[at] = f;
    const float2 df = __bfloat1622float2(dfStored);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      if (i >= m) break;
      const float2 di = i == slot ? df : __bfloat1622float2(dF[i][at]);
      col[i] += di.x * df.x + di.y * df.y;
      gam[i] += di.x * f.x + di.y * f.y;
    }
  }
  MixerBlockPartials<M>(col, gam, a.partial);
}

// The sweep's block partial sums reduced to the new Gram column (m values)
// and the right-hand side (m values, from index kMaxMemory), a warp each, in
// a fixed order (lanes over the blocks, then a fixed shuffle tree).
__global__ void MixerReduceKernel(int m, int blocks, const double* partial, double* sums, const int* live) {
  if (live != nullptr) {
    if (live[0] != kLiveUpdate) return;
    m = live[1];
  }
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (warp >= 2 * m) return;
  const int i = warp < m ? warp : kMaxMemory + (warp - m);
  double v = 0.0;
  for (int b = lane; b < blocks; b += 32) v += partial[static_cast<long long>(b) * 2 * kMaxMemory + i];
  for (int off = 16; off > 0; off /= 2) v += __shfl_down_sync(0xffffffffu, v, off);
  if (lane == 0) sums[i] = v;
}

template <class T, int M>
__global__ void MixerMixKernel(MixerArgsT<T> a) {
  using A = typename MixAcc<T>::type;
  int m = M;
  if (a.live != nullptr) {
    if (a.live[0] != kLiveUpdate) return;
    m = a.live[1];
  }
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const bool ok = a.gamma[m] != 0.0;
  A g[M + 1];
  const typename MixerArgsT<T>::H* dG[M + 1];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    g[i] = i < m ? static_cast<A>(a.gamma[i]) : A(0);
    dG[i] = a.dG[i];
  }
  for (long long at = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; at < a.n; at += stride) {
    A value = a.gx[at];
    if (ok)
#pragma unroll
      for (int i = 0; i < M; ++i) {
        if (i >= m) break;
        value -= g[i] * static_cast<A>(FromHistory(dG[i][at]));
      }
    a.x[at] = static_cast<T>(value);
  }
}

template <int M>
__global__ void MixerMixPairsKernel(MixerArgsT<float> a) {
  int m = M;
  if (a.live != nullptr) {
    if (a.live[0] != kLiveUpdate) return;
    m = a.live[1];
  }
  const long long pairs = a.n / 2;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const bool ok = a.gamma[m] != 0.0;
  float g[M + 1];
  const __nv_bfloat162* dG[M + 1];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    g[i] = i < m ? static_cast<float>(a.gamma[i]) : 0.0f;
    dG[i] = reinterpret_cast<const __nv_bfloat162*>(a.dG[i]);
  }
  auto* x = reinterpret_cast<float2*>(a.x);
  auto* gx = reinterpret_cast<const float2*>(a.gx);
  for (long long at = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; at < pairs; at += stride) {
    float2 v = gx[at];
    if (ok)
#pragma unroll
      for (int i = 0; i < M; ++i) {
        if (i >= m) break;
        const float2 d = __bfloat1622float2(dG[i][at]);
        v.x -= g[i] * d.x;
        v.y -= g[i] * d.y;
      }
    x[at] = v;
  }
}

// Calls f(std::integral_constant<int, M>{}) for M = m (0 <= m <= kMaxMemory).
template <int M = 0, class F>
void ForMemory(int m, F&& f) {
  if constexpr (M <= kMaxMemory) {
    if (m == M) {
      f(std::integral_constant<int, M>{});
      return;
    }
    ForMemory<M + 1>(m, f);
  }
}

// -- the memory at the non-lateral nodes, spectrally ----------------------------------------------

__device__ inline bool NonLateral(int p, int pLat0, int pLat1) { return p < pLat0 || p >= pLat1; }

__global__ void SpectralStartKernel(SpectralMemoryArgs a) {
  const long long total = a.rows * a.P;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total; i += stride) {
    const int p = static_cast<int>(i % a.P);
    if (!NonLateral(p, a.pLat0, a.pLat1)) continue;
    const double2 s0 = a.s[i];
    double2 fixed = C(0, 0);
    for (int k = 0; k < a.branches; ++k) {
      double e, alpha, beta;
      StageWeights(a.scheme, a.dt * a.itauRef[static_cast<long long>(k) * a.P + p], e, alpha, beta);
      const double2 m = a.in[k][i];
      const double2 o = C(e * m.x + alpha * s0.x, e * m.y + alpha * s0.y);
      a.out[k][i] = o;
      const double mu = a.muBranch[static_cast<long long>(k) * a.P + p];
      fixed = C(fixed.x + mu * o.x, fixed.y + mu * o.y);
    }
    a.fixedS[i] = fixed;
  }
}

__global__ void SpectralAdvanceKernel(SpectralMemoryArgs a) {
  const long long total = a.rows * a.P;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total; i += stride) {
    const int p = static_cast<int>(i % a.P);
    if (!NonLateral(p, a.pLat0, a.pLat1)) continue;
    const double2 s1 = a.s[i];
    for (int k = 0; k < a.branches; ++k) {
      double e, alpha, beta;
      StageWeights(a.scheme, a.dt * a.itauRef[static_cast<long long>(k) * a.P + p], e, alpha, beta);
      const double2 m = a.out[k][i];
      a.out[k][i] = C(m.x + beta * s1.x, m.y + beta * s1.y);
    }
  }
}

__global__ void SpectralSumKernel(SpectralMemoryArgs a) {
  const long long total = a.rows * a.P;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total; i += stride) {
    const int p = static_cast<int>(i % a.P);
    if (!NonLateral(p, a.pLat0, a.pLat1)) continue;
    double2 fixed = C(0, 0);
    for (int k = 0; k < a.branches; ++k) {
      const double mu = a.muBranch[static_cast<long long>(k) * a.P + p];
      const double2 m = a.in[k][i];
      fixed = C(fixed.x + mu * m.x, fixed.y + mu * m.y);
    }
    a.fixedS[i] = fixed;
  }
}

__global__ void SpectralCombineKernel(long long rows, int P, int pLat0, int pLat1, double r, const double2* a,
                                      double2* out) {
  const long long total = rows * P;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total; i += stride) {
    const int p = static_cast<int>(i % P);
    if (!NonLateral(p, pLat0, pLat1)) continue;
    const double2 x = a[i], y = out[i];
    out[i] = C((1.0 - r) * x.x + r * y.x, (1.0 - r) * x.y + r * y.y);
  }
}

// -- conjugate gradients -----------------------------------------------------------------------

// Warp per (system, row), lanes over the row's columns: the band entries of
// the row are broadcast reads, the x rows coalesced (and L1/L2 hits for the
// neighbouring rows' warps).
__global__ void BandApplyKernel(const sl3dgpu_band_system* systems, const double* bands, const double* x, double* y,
                                double keep) {
  const sl3dgpu_band_system s = systems[blockIdx.y];
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x % 32;
  if (row >= s.n) return;
  const int kd = s.ku, ld = kd + 1, cols = s.nrhs;
  const double* band = bands + s.band;
  const double* xs = x + s.rhs;
  double* ys = y + s.rhs + static_cast<long long>(row) * cols;
  const int j0 = max(0, row - kd), j1 = min(s.n - 1, row + kd);
  for (int c = lane; c < cols; c += 32) {
    double sum = 0.0;
    for (int j = j0; j <= j1; ++j) {
      const int lo = min(row, j), hi = max(row, j);
      sum += band[static_cast<long long>(hi) * ld + kd + lo - hi] * xs[static_cast<long long>(j) * cols + c];
    }
    ys[c] = keep == 0.0 ? sum : sum + keep * ys[c];
  }
}

__global__ void PairKernel(const double2* a, const double2* b, const PairChunk* chunks, double* partial) {
  __shared__ double red[256];
  const PairChunk c = chunks[blockIdx.x];
  double sum = 0.0;
  for (long long k = c.start + threadIdx.x; k < c.end; k += blockDim.x) {
    const int m = static_cast<int>((k - c.degreeStart) % c.cols);
    const double2 u = a[k], v = b[k];
    sum += (m == 0 ? 1.0 : 2.0) * (u.x * v.x + u.y * v.y);
  }
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void SumKernel(const double* partial, int count, double* result) {
  __shared__ double red[256];
  double sum = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) sum += partial[i];
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) result[0] = red[0];
}

__global__ void AxpyKernel(long long n, double alpha, const double* x, double* y) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    y[i] += alpha * x[i];
}

__global__ void XpbyKernel(long long n, const double* x, double beta, double* y) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    y[i] = x[i] + beta * y[i];
}

__global__ void SubKernel(long long n, const double* a, const double* b, double* out) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    out[i] = a[i] - b[i];
}

// -- the mixed form's refinement glue ----------------------------------------------------------

__global__ void Residual32Kernel(long long n, const double* next, const double* now, float* r) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    r[i] = static_cast<float>(next[i] - now[i]);
}

__global__ void AddCorrectionKernel(long long n, const float* e, double* s) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    s[i] += static_cast<double>(e[i]);
}

__global__ void AddInPlaceKernel(long long n, const float* r, float* e) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    e[i] += r[i];
}

__global__ void CastKernel(long long n, const double* in, float* out) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    out[i] = static_cast<float>(in[i]);
}

__global__ void BlendKernel(long long n, double gamma, const double2* a, const double2* b, double2* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const double2 x = a ? a[i] : C(0, 0), y = b ? b[i] : C(0, 0);
  out[i] = C((1.0 - gamma) * x.x + gamma * y.x, (1.0 - gamma) * x.y + gamma * y.y);
}

int StreamBlocks(long long values) {
  const long long b = (values + 255) / 256;
  return static_cast<int>(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace

namespace {
// Orders a block of the chunked maps takes: the most (up to 32) whose
// shared-memory rows fit a budget that leaves room for two blocks an SM.
constexpr size_t kChunkSmemBudget = 110 * 1024;
inline int ChunkOrders(size_t bytesPerOrder, size_t fixedBytes) {
  int mc = 32;
  while (mc > 1 && fixedBytes + bytesPerOrder * mc > kChunkSmemBudget) mc /= 2;
  return mc;
}
inline int ChunkBlocks(int lmax, int mc) {  // sum over l <= lmax of (floor(l / mc) + 1)
  long long blocks = 0;
  for (int l = 0; l <= lmax; ++l) blocks += l / mc + 1;
  return static_cast<int>(blocks);
}

template <class T2, int MC>
void ForcesWith(const Geometry& g, const T2* spectral, T2* rhsSph, T2* rhsTor, cudaStream_t stream) {
  const size_t smem = static_cast<size_t>(6) * MC * (g.P | 1) * sizeof(T2);
  AllowDynamicSmem(ForceChunkKernel<T2, MC>);
  ForceChunkKernel<T2, MC><<<ChunkBlocks(g.lmax, MC), 256, smem, stream>>>(g, spectral, rhsSph, rhsTor);
}

template <class T2, int MC>
void StrainWith(const Geometry& g, const T2* solSph, const T2* solTor, T2* spectral, const T2* add,
                cudaStream_t stream) {
  const size_t smem = static_cast<size_t>(std::max(g.maxGlobals, 1)) * (3 * MC + 1) * sizeof(T2);
  AllowDynamicSmem(StrainChunkKernel<T2, MC>);
  StrainChunkKernel<T2, MC><<<ChunkBlocks(g.lmax, MC), 256, smem, stream>>>(g, solSph, solTor, spectral, add);
}

template <class T2>
void Forces(const Geometry& g, const T2* spectral, T2* rhsSph, T2* rhsTor, cudaStream_t stream) {
  prof::Scope scope(prof::kForce, stream);
  switch (ChunkOrders(static_cast<size_t>(6) * (g.P | 1) * sizeof(T2), 0)) {
    case 32: return ForcesWith<T2, 32>(g, spectral, rhsSph, rhsTor, stream);
    case 16: return ForcesWith<T2, 16>(g, spectral, rhsSph, rhsTor, stream);
    case 8: return ForcesWith<T2, 8>(g, spectral, rhsSph, rhsTor, stream);
    case 4: return ForcesWith<T2, 4>(g, spectral, rhsSph, rhsTor, stream);
    case 2: return ForcesWith<T2, 2>(g, spectral, rhsSph, rhsTor, stream);
    default: return ForcesWith<T2, 1>(g, spectral, rhsSph, rhsTor, stream);
  }
}

template <class T2>
void Strain(const Geometry& g, const T2* solSph, const T2* solTor, T2* spectral, const T2* add,
            cudaStream_t stream) {
  prof::Scope scope(prof::kStrain, stream);
  const size_t globals = static_cast<size_t>(std::max(g.maxGlobals, 1));
  switch (ChunkOrders(globals * 3 * sizeof(T2), globals * sizeof(T2))) {
    case 32: return StrainWith<T2, 32>(g, solSph, solTor, spectral, add, stream);
    case 16: return StrainWith<T2, 16>(g, solSph, solTor, spectral, add, stream);
    case 8: return StrainWith<T2, 8>(g, solSph, solTor, spectral, add, stream);
    case 4: return StrainWith<T2, 4>(g, solSph, solTor, spectral, add, stream);
    case 2: return StrainWith<T2, 2>(g, solSph, solTor, spectral, add, stream);
    default: return StrainWith<T2, 1>(g, solSph, solTor, spectral, add, stream);
  }
}
}  // namespace

void LaunchForces(const Geometry& g, const double2* spectral, double2* rhsSph, double2* rhsTor,
                  cudaStream_t stream) {
  Forces(g, spectral, rhsSph, rhsTor, stream);
}
void LaunchForces(const Geometry& g, const float2* spectral, float2* rhsSph, float2* rhsTor, cudaStream_t stream) {
  Forces(g, spectral, rhsSph, rhsTor, stream);
}
void LaunchStrain(const Geometry& g, const double2* solSph, const double2* solTor, double2* spectral,
                  cudaStream_t stream, const double2* add) {
  Strain(g, solSph, solTor, spectral, add, stream);
}
void LaunchStrain(const Geometry& g, const float2* solSph, const float2* solTor, float2* spectral,
                  cudaStream_t stream, const float2* add) {
  Strain(g, solSph, solTor, spectral, add, stream);
}

void LaunchDilatation(const Geometry& g, const double2* solSph, double2* scalar, cudaStream_t stream) {
  const int count = (g.lmax + 1) * (g.lmax + 2) / 2;
  const size_t smem = static_cast<size_t>(g.elements * (g.ngll - 1) + 1) * 2 * sizeof(double2);
  AllowDynamicSmem(DilatationKernel);
  prof::Scope scope(prof::kStrain, stream);
  DilatationKernel<<<count, 128, smem, stream>>>(g, solSph, scalar);
}

void LaunchDilatationForce(const Geometry& g, const double2* scalar, double2* rhsSph, cudaStream_t stream) {
  const int count = (g.lmax + 1) * (g.lmax + 2) / 2;
  const size_t smem = static_cast<size_t>(g.P) * sizeof(double2);
  AllowDynamicSmem(DilatationForceKernel);
  prof::Scope scope(prof::kForce, stream);
  DilatationForceKernel<<<count, 128, smem, stream>>>(g, scalar, rhsSph);
}

void LaunchAddLoad(const Geometry& g, const double2* sigma, const double* units, const long long* unitOffset,
                   double2* solSph, cudaStream_t stream, const double2* tide, const double* tideUnits) {
  if (sigma == nullptr && tide == nullptr) return;
  prof::Scope scope(prof::kOther, stream);
  AddLoadKernel<<<g.lmax + 1, 256, 0, stream>>>(g, sigma, units, tide, tideUnits, unitOffset, solSph);
}

void LaunchSurface(const Geometry& g, const double2* solSph, const double2* solTor, int component, double2* out,
                   cudaStream_t stream) {
  const int count = (g.lmax + 1) * (g.lmax + 2) / 2;
  prof::Scope scope(prof::kOther, stream);
  SurfaceKernel<<<(count + 127) / 128, 128, 0, stream>>>(g, solSph, solTor, component, out);
}

void LaunchWeights(const WeightsArgs& a, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, (a.end - a.begin) * (8.0 + a.branches * 96.0 + 40.0 + 48.0));
  if (a.end <= a.begin) return;
  WeightsKernel<<<StreamBlocks(a.end - a.begin), 256, 0, stream>>>(a);
}

void LaunchSpectralStart(const SpectralMemoryArgs& a, cudaStream_t stream) {
  const long long n = a.rows * a.P;
  prof::Scope scope(prof::kStream, stream, 0.0, n * (16.0 + a.branches * 32.0 + 16.0));
  SpectralStartKernel<<<StreamBlocks(n), 256, 0, stream>>>(a);
}
void LaunchSpectralAdvance(const SpectralMemoryArgs& a, cudaStream_t stream) {
  const long long n = a.rows * a.P;
  prof::Scope scope(prof::kStream, stream, 0.0, n * (16.0 + a.branches * 32.0));
  SpectralAdvanceKernel<<<StreamBlocks(n), 256, 0, stream>>>(a);
}
void LaunchSpectralSum(const SpectralMemoryArgs& a, cudaStream_t stream) {
  const long long n = a.rows * a.P;
  prof::Scope scope(prof::kStream, stream, 0.0, n * (a.branches * 16.0 + 16.0));
  SpectralSumKernel<<<StreamBlocks(n), 256, 0, stream>>>(a);
}
void LaunchSpectralCombine(long long rows, int P, int pLat0, int pLat1, double r, const double2* a, double2* out,
                           cudaStream_t stream) {
  const long long n = rows * P;
  prof::Scope scope(prof::kStream, stream, 0.0, n * 48.0);
  SpectralCombineKernel<<<StreamBlocks(n), 256, 0, stream>>>(rows, P, pLat0, pLat1, r, a, out);
}

void LaunchAdvance(long long values, const double* beta, const double2* d0, const double2* d1, const double* dr,
                   double2* m0, double2* m1, double* mr, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, values * 128.0);
  AdvanceKernel<<<StreamBlocks(values), 256, 0, stream>>>(values, beta, d0, d1, dr, m0, m1, mr);
}

void LaunchStageCombine(long long values, double r, const double2* a0, const double2* a1, const double* ar,
                        double2* o0, double2* o1, double* orr, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, values * 120.0);
  StageCombineKernel<<<StreamBlocks(values), 256, 0, stream>>>(values, r, a0, a1, ar, o0, o1, orr);
}

void LaunchCombine(long long values, long long fieldSize, const double* mu, bool first, const double2* m0,
                   const double2* m1, const double* mr, double2* o0, double2* o1, double* orr,
                   cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, values * 88.0);
  CombineKernel<<<StreamBlocks(values), 256, 0, stream>>>(values, fieldSize, mu, first, m0, m1, mr, o0, o1, orr);
}

void LaunchBlend(long long n, double gamma, const double2* a, const double2* b, double2* out, cudaStream_t stream) {
  prof::Scope scope(prof::kOther, stream);
  BlendKernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(n, gamma, a, b, out);
}

namespace {
template <class T2>
void RelChange(const T2* next, const T2* now, long long n, double* partial, int partialCount, double* result,
               cudaStream_t stream) {
  {
    prof::Scope scope(prof::kOther, stream, 0.0, n * 2.0 * sizeof(T2));
    RelativeChangeKernel<T2><<<partialCount, 256, 0, stream>>>(next, now, n, partial);
  }
  prof::Scope scope(prof::kOther, stream);
  ReduceMaxKernel<<<1, 256, 0, stream>>>(partial, partialCount, result);
}

template <class T>
void MixerFirst(const MixerArgsT<T>& a, cudaStream_t stream) {
  prof::Scope scope(prof::kMixer, stream, 0.0, a.n * 5.0 * sizeof(T));
  MixerFirstKernel<T><<<StreamBlocks(a.n), 256, 0, stream>>>(a.n, a.x, a.gx, a.xPrev, a.fPrev, a.live);
}

template <class T>
void MixerSweep(const MixerArgsT<T>& a, double* sums, cudaStream_t stream) {
  {
    using H = typename MixerArgsT<T>::H;
    prof::Scope scope(prof::kMixer, stream, 0.0, a.n * (6.0 * sizeof(T) + (a.m + 1.0) * sizeof(H)));
    ForMemory(a.m, [&](auto M) {
      if constexpr (std::is_same_v<T, float>)
        MixerSweepPairsKernel<M()><<<a.blocks, kMixThreads, 0, stream>>>(a);
      else
        MixerSweepKernel<T, M()><<<a.blocks, kMixThreads, 0, stream>>>(a);
    });
  }
  prof::Scope scope(prof::kOther, stream);
  MixerReduceKernel<<<1, 32 * 2 * kMaxMemory, 0, stream>>>(a.m, a.blocks, a.partial, sums, a.live);
}

template <class T>
void MixerMix(const MixerArgsT<T>& a, cudaStream_t stream) {
  prof::Scope scope(prof::kMixer, stream, 0.0,
                    a.n * (2.0 * sizeof(T) + a.m * sizeof(typename MixerArgsT<T>::H)));
  ForMemory(a.m, [&](auto M) {
    if constexpr (std::is_same_v<T, float>)
      MixerMixPairsKernel<M()><<<StreamBlocks(a.n / 2), 256, 0, stream>>>(a);
    else
      MixerMixKernel<T, M()><<<StreamBlocks(a.n), 256, 0, stream>>>(a);
  });
}
}  // namespace

void LaunchRelativeChange(const double* next, const double* now, long long n, double* partial, int partialCount,
                          double* result, cudaStream_t stream) {
  RelChange(reinterpret_cast<const double2*>(next), reinterpret_cast<const double2*>(now), n / 2, partial,
            partialCount, result, stream);
}
void LaunchRelativeChange(const float* next, const float* now, long long n, double* partial, int partialCount,
                          double* result, cudaStream_t stream) {
  RelChange(reinterpret_cast<const float2*>(next), reinterpret_cast<const float2*>(now), n / 2, partial,
            partialCount, result, stream);
}

void LaunchMixerFirst(const MixerArgsT<double>& a, cudaStream_t stream) { MixerFirst(a, stream); }
void LaunchMixerSweep(const MixerArgsT<double>& a, double* sums, cudaStream_t stream) { MixerSweep(a, sums, stream); }
void LaunchMixerMix(const MixerArgsT<double>& a, cudaStream_t stream) { MixerMix(a, stream); }
void LaunchMixerFirst(const MixerArgsT<float>& a, cudaStream_t stream) { MixerFirst(a, stream); }
void LaunchMixerSweep(const MixerArgsT<float>& a, double* sums, cudaStream_t stream) { MixerSweep(a, sums, stream); }
void LaunchMixerMix(const MixerArgsT<float>& a, cudaStream_t stream) { MixerMix(a, stream); }

void LaunchBandApply(const sl3dgpu_band_system* devSystems, int count, int maxRows, const double* bands,
                     const double* x, double* y, double keep, cudaStream_t stream) {
  if (count == 0 || maxRows == 0) return;
  constexpr int kRowsPerBlock = 8;
  prof::Scope scope(prof::kBandSolve, stream);
  BandApplyKernel<<<dim3((maxRows + kRowsPerBlock - 1) / kRowsPerBlock, count), kRowsPerBlock * 32, 0, stream>>>(
      devSystems, bands, x, y, keep);
}

void LaunchPair(const double2* a, const double2* b, const PairChunk* chunks, int count, double* partial,
                double* result, cudaStream_t stream) {
  {
    prof::Scope scope(prof::kOther, stream);
    PairKernel<<<count, 256, 0, stream>>>(a, b, chunks, partial);
  }
  prof::Scope scope(prof::kOther, stream);
  SumKernel<<<1, 256, 0, stream>>>(partial, count, result);
}

void LaunchAxpy(long long n, double alpha, const double* x, double* y, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 24.0);
  AxpyKernel<<<StreamBlocks(n), 256, 0, stream>>>(n, alpha, x, y);
}
void LaunchXpby(long long n, const double* x, double beta, double* y, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 24.0);
  XpbyKernel<<<StreamBlocks(n), 256, 0, stream>>>(n, x, beta, y);
}
void LaunchSub(long long n, const double* a, const double* b, double* out, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 24.0);
  SubKernel<<<StreamBlocks(n), 256, 0, stream>>>(n, a, b, out);
}

void LaunchResidual32(long long n, const double* next, const double* now, float* r, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 20.0);
  Residual32Kernel<<<StreamBlocks(n), 256, 0, stream>>>(n, next, now, r);
}
void LaunchAddCorrection(long long n, const float* e, double* s, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 20.0);
  AddCorrectionKernel<<<StreamBlocks(n), 256, 0, stream>>>(n, e, s);
}
void LaunchAddInPlace(long long n, const float* r, float* e, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 12.0);
  AddInPlaceKernel<<<StreamBlocks(n), 256, 0, stream>>>(n, r, e);
}
namespace {
__global__ void GatherColumnsKernel(long long rows, int P, int p0, int count, const float2* in, float2* out) {
  const long long total = rows * count;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total; t += stride) {
    const long long row = t / count;
    out[t] = in[row * P + p0 + t % count];
  }
}
}  // namespace

void LaunchGatherColumns(long long rows, int P, int p0, int count, const float2* in, float2* out,
                         cudaStream_t stream) {
  if (rows * count == 0) return;
  prof::Scope scope(prof::kStream, stream, 0.0, rows * count * 16.0);
  GatherColumnsKernel<<<StreamBlocks(rows * count), 256, 0, stream>>>(rows, P, p0, count, in, out);
}

void LaunchCast(long long n, const double* in, float* out, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 12.0);
  CastKernel<<<StreamBlocks(n), 256, 0, stream>>>(n, in, out);
}

}  // namespace sl3dgpu

namespace sl3dgpu {
std::vector<double> NodeCoefficients(int P, int ngll, const std::vector<int>& nodeElement,
                                     const std::vector<int>& nodeQ, const std::vector<double>& nodeR,
                                     const std::vector<double>& elemJac, const std::vector<double>& value,
                                     const std::vector<double>& deriv, const std::vector<double>& weight) {
  const size_t plane = static_cast<size_t>(P) * ngll;
  std::vector<double> out(4 * plane);
  for (int p = 0; p < P; ++p) {
    const int e = nodeElement[p], q = nodeQ[p];
    const double r = nodeR[p], jac = elemJac[e];
    for (int i = 0; i < ngll; ++i) {
      const size_t at = static_cast<size_t>(p) * ngll + i;
      out[kStrainValue * plane + at] = value[q * ngll + i];
      out[kStrainDeriv * plane + at] = r * deriv[q * ngll + i] / jac;
      out[kForceValue * plane + at] = jac * weight[q] * r * value[q * ngll + i];
      out[kForceDeriv * plane + at] = weight[q] * deriv[q * ngll + i] * r;
    }
  }
  return out;
}
}  // namespace sl3dgpu

namespace sl3dgpu {
namespace {

// The Anderson update's least squares on the device, one FP64 warp: the
// Gram matrix's slot column and row from the sweep's sums, then gamma =
// argmin |G gamma - b| by a Jacobi eigen-decomposition of the symmetric G
// with eigenvalues at or below machine epsilon times the largest dropped --
// the minimum-norm solution of LAPACK's dgelss with rcond < 0, the
// reference's call (include/sl3dpp/detail/AndersonMixer.hpp:186-211).
// Parallel Jacobi in the round-robin order (Brent and Luk): each round
// rotates m/2 disjoint index pairs at once -- their angles on as many
// lanes, then the row and column updates one lane per (pair, index) -- so
// that a sweep is m - 1 rounds of one rotation's latency rather than
// m (m - 1) / 2 (the FP64 divisions and square roots on GB300's slow FP64
// pipe set the pace). Sweeps until the off-diagonal mass is below 1e-32 of
// the diagonal's, as the host's SymmetricLstsq (host/lstsq.hpp).
//
// With `cholesky` (the FP32 correction's mixer, called every pass) the
// system is first solved by a Cholesky factorisation, a column a step:
// when every pivot is above 1e-13 of the largest diagonal value the Gram
// matrix is far from the eigenvalue cut, the minimum-norm solution is its
// solution, and the factorisation's m square roots replace the Jacobi
// sweeps' rotations; otherwise (a numerically singular Gram) the
// eigen-decomposition decides.
__global__ void __launch_bounds__(32) MixerGramKernel(double* gram, int m, int slot, int memory,
                                                      const double* sums, double* gamma, const int* live,
                                                      bool cholesky) {
  if (live != nullptr) {
    if (live[0] != kLiveUpdate) return;
    m = live[1];
    slot = live[2];
  }
  constexpr int M = kMixMaxMemory;
  __shared__ double a[M][M + 1], v[M][M + 1];
  __shared__ double rotC[M / 2], rotS[M / 2];
  __shared__ int rotP[M / 2], rotQ[M / 2];
  const int lane = threadIdx.x;
  if (lane < m) {
    gram[slot * memory + lane] = sums[lane];
    gram[lane * memory + slot] = sums[lane];
  }
  __syncwarp();
  __threadfence_block();
  for (int j = 0; j < m; ++j)
    if (lane < m) {
      a[lane][j] = 0.5 * (gram[lane * memory + j] + gram[j * memory + lane]);
      v[lane][j] = lane == j ? 1.0 : 0.0;
    }
  __syncwarp();
  if (cholesky) {
    // L L^T = G in v's lower triangle, lane i the row i
    __shared__ double inv[M], rhs[M];
    double dmax = 0.0;
    for (int i = 0; i < m; ++i) dmax = fmax(dmax, a[i][i]);
    bool regular = true;
    for (int k = 0; k < m; ++k) {
      double sk = 0.0;
      if (lane >= k && lane < m) {
        sk = a[lane][k];
        for (int j = 0; j < k; ++j) sk -= v[lane][j] * v[k][j];
      }
      const double d = __shfl_sync(0xffffffffu, sk, k);  // the pivot, on every lane
      if (!(d > 1e-13 * dmax)) {
        regular = false;
        break;
      }
      const double r = sqrt(d), ir = 1.0 / r;
      if (lane == k) {
        v[k][k] = r;
        inv[k] = ir;
      }
      if (lane > k && lane < m) v[lane][k] = sk * ir;
      __syncwarp();
    }
    __syncwarp();
    if (regular) {
      // L y = b, then L^T x = y, a column at a time
      const double* bsum = sums + kMixMaxMemory;
      if (lane < m) rhs[lane] = bsum[lane];
      __syncwarp();
      for (int k = 0; k < m; ++k) {
        const double yk = rhs[k] * inv[k];
        __syncwarp();
        if (lane == k) rhs[k] = yk;
        if (lane > k && lane < m) rhs[lane] -= v[lane][k] * yk;
        __syncwarp();
      }
      for (int k = m - 1; k >= 0; --k) {
        const double xk = rhs[k] * inv[k];
        __syncwarp();
        if (lane == k) rhs[k] = xk;
        if (lane < k) rhs[lane] -= v[k][lane] * xk;
        __syncwarp();
      }
      if (lane < m) gamma[lane] = rhs[lane];
      __syncwarp();
      if (lane == 0) {
        bool finite = true;
        for (int i = 0; i < m; ++i)
          if (!(rhs[i] - rhs[i] == 0.0)) finite = false;
        gamma[m] = finite ? 1.0 : 0.0;
      }
      return;
    }
    // a numerically singular Gram: the eigen-decomposition from the identity
    for (int j = 0; j < m; ++j)
      if (lane < m) v[lane][j] = lane == j ? 1.0 : 0.0;
    __syncwarp();
  }
  const int even = m + (m & 1);  // a padding index m when m is odd (it rotates nothing)
  const int pairs = even / 2;
  for (int sweep = 0; sweep < 60 && m > 1; ++sweep) {
    // the off-diagonal and diagonal masses, a lane a row
    double off = 0.0, diag = 0.0;
    if (lane < m)
      for (int j = 0; j < m; ++j) (lane == j ? diag : off) += a[lane][j] * a[lane][j];
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      diag += __shfl_xor_sync(0xffffffffu, diag, o);
    }
    if (off <= 1e-32 * diag || off == 0.0) break;
    for (int round = 0; round < even - 1; ++round) {
      // the round's pairs: position 0 fixed, the others turned by `round`
      if (lane < pairs) {
        auto at = [&](int pos) { return pos == 0 ? 0 : 1 + (pos - 1 + round) % (even - 1); };
        int p = at(lane), q = at(even - 1 - lane);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, sn = 0.0;
        if (q < m && a[p][q] != 0.0) {
          const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
          const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          c = 1.0 / sqrt(t * t + 1.0);
          sn = t * c;
        }
        rotC[lane] = c;
        rotS[lane] = sn;
        rotP[lane] = p;
        rotQ[lane] = q < m ? q : -1;
      }
      __syncwarp();
      // A <- A J (columns p, q), then A <- J^T A (rows p, q) and V <- V J
      for (int e = lane; e < pairs * m; e += 32) {
        const int i = e / m, k = e % m, p = rotP[i], q = rotQ[i];
        if (q < 0 || rotS[i] == 0.0) continue;
        const double c = rotC[i], sn = rotS[i];
        const double akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - sn * akq;
        a[k][q] = sn * akp + c * akq;
      }
      __syncwarp();
      for (int e = lane; e < pairs * m; e += 32) {
        const int i = e / m, k = e % m, p = rotP[i], q = rotQ[i];
        if (q < 0 || rotS[i] == 0.0) continue;
        const double c = rotC[i], sn = rotS[i];
        const double apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - sn * aqk;
        a[q][k] = sn * apk + c * aqk;
        const double vkp = v[k][p], vkq = v[k][q];
        v[k][p] = c * vkp - sn * vkq;
        v[k][q] = sn * vkp + c * vkq;
      }
      __syncwarp();
    }
  }
  // the solve: projections of b on the kept eigenvectors
  __shared__ double proj[M], y[M];
  __shared__ double cut;
  if (lane == 0) {
    double largest = 0.0;
    for (int i = 0; i < m; ++i) largest = fmax(largest, fabs(a[i][i]));
    cut = 2.220446049250313e-16 * largest;
  }
  __syncwarp();
  const double* b = sums + kMixMaxMemory;
  if (lane < m) {
    double pr = 0.0;
    for (int i = 0; i < m; ++i) pr += v[i][lane] * b[i];
    proj[lane] = pr;
  }
  __syncwarp();
  if (lane < m) {
    double yi = 0.0;
    for (int k = 0; k < m; ++k) {
      const double lambda = a[k][k];
      if (!(fabs(lambda) > cut)) continue;
      yi += v[lane][k] * proj[k] / lambda;
    }
    y[lane] = yi;
    gamma[lane] = yi;
  }
  __syncwarp();
  if (lane == 0) {
    bool finite = true;
    for (int i = 0; i < m; ++i)
      if (!(y[i] - y[i] == 0.0)) finite = false;
    gamma[m] = finite ? 1.0 : 0.0;
  }
}

}  // namespace

void LaunchMixerGram(double* gram, int m, int slot, int memory, const double* sums, double* gamma,
                     cudaStream_t stream, const int* live, bool cholesky) {
  prof::Scope scope(prof::kMixer, stream);
  MixerGramKernel<<<1, 32, 0, stream>>>(gram, m, slot, memory, sums, gamma, live, cholesky);
}

// -- the FP32 correction's loop on the device ------------------------------------------------------

namespace {

// The host loop's decisions (Viscoelastic3DGpu::Correct) made on the device:
// the same tests, in the same order, on the same numbers.
__global__ void CorrectionControlKernel(CorrectionControl* c, const double* r, cudaGraphConditionalHandle handle) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (r[2] == 0.0) {  // the iterate left the finite range
    c->status = 1;
    c->action = kLiveStop;
    cudaGraphSetConditional(handle, 0);
    return;
  }
  const double change = r[0] > 0.0 ? sqrt(r[1]) / sqrt(r[0]) : 0.0;
  if (c->historyCount < kCorrectionHistory) c->history[c->historyCount] = change;
  ++c->historyCount;
  const int iteration = c->iteration;
  c->iteration = iteration + 1;
  if (change <= c->tolerance) {
    c->action = kLiveCopy;
    c->fresh = 1;
    cudaGraphSetConditional(handle, 0);
    return;
  }
  if (c->rate > 0.0 && !c->mixing && c->memory > 0 && iteration > c->first && change > c->rate * c->previous) {
    c->mixing = 1;
    c->firstMix = 1;
    c->count = 0;
    c->slot = 0;
    c->resetGram = 1;
  }
  c->previous = change;
  if (c->mixing) {
    if (c->firstMix) {
      c->action = kLiveFirst;
      c->firstMix = 0;
    } else {
      c->action = kLiveUpdate;
      c->m = min(c->count + 1, c->memory);
    }
  } else {
    c->action = kLiveCopy;
  }
  cudaGraphSetConditional(handle, c->iteration < c->maxIterations ? 1u : 0u);
}

__global__ void CopyIfPlainKernel(const CorrectionControl* c, const float2* from, float2* to, long long n) {
  if (c->action != kLiveCopy) return;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
    to[i] = from[i];
}

__global__ void GramResetIfKernel(CorrectionControl* c, double* gram, int count) {
  if (!c->resetGram) return;
  for (int i = threadIdx.x; i < count; i += blockDim.x) gram[i] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) c->resetGram = 0;
}

__global__ void MixerAdvanceIfKernel(CorrectionControl* c) {
  if (threadIdx.x != 0 || c->action != kLiveUpdate) return;
  c->count = c->m;
  c->slot = (c->slot + 1) % c->memory;
}

}  // namespace

void LaunchCorrectionControl(CorrectionControl* c, const double* result, cudaGraphConditionalHandle handle,
                             cudaStream_t stream) {
  prof::Scope scope(prof::kOther, stream);
  CorrectionControlKernel<<<1, 32, 0, stream>>>(c, result, handle);
}

void LaunchCopyIfPlain(const CorrectionControl* c, const float2* from, float2* to, long long n, cudaStream_t stream) {
  prof::Scope scope(prof::kMixer, stream);
  CopyIfPlainKernel<<<StreamBlocks(n), 256, 0, stream>>>(c, from, to, n);
}

void LaunchGramResetIf(CorrectionControl* c, double* gram, int memory, cudaStream_t stream) {
  prof::Scope scope(prof::kOther, stream);
  GramResetIfKernel<<<1, 256, 0, stream>>>(c, gram, memory * memory);
}

void LaunchMixerAdvanceIf(CorrectionControl* c, cudaStream_t stream) {
  prof::Scope scope(prof::kOther, stream);
  MixerAdvanceIfKernel<<<1, 32, 0, stream>>>(c);
}

bool MixerSolve(double* gram, int m, int slot, int memory, const double* sums, double* gamma) {
  for (int i = 0; i < m; ++i) {
    gram[slot * memory + i] = sums[i];
    gram[i * memory + slot] = sums[i];
  }
  double A[kMixMaxMemory * kMixMaxMemory], x[kMixMaxMemory];
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) A[i * m + j] = gram[i * memory + j];
  const bool ok = SymmetricLstsq(m, A, sums + kMixMaxMemory, x);
  for (int i = 0; i < m; ++i) gamma[i] = x[i];
  gamma[m] = ok ? 1.0 : 0.0;
  return ok;
}
}  // namespace sl3dgpu
