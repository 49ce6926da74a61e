// Device kernels of the step's discrete adjoint (AdjointSolver3D's
// transposed sweep, src/AdjointDiscrete3D.cpp): the transposes of the
// surface reads and of the load channel, the end strain's dual, and the
// pointwise transposes of the stage's memory recursion with the
// log-viscosity gradient they carry. The pairings are those of
// step_kernels.cuh's adjoint section.

#include <cmath>

#include "profile.cuh"
#include "step_kernels.cuh"

namespace sl3dgpu {
namespace {

__device__ inline void LmOf(int lm, int& l, int& m) {
  l = static_cast<int>((sqrt(8.0 * lm + 1.0) - 1.0) * 0.5);
  while (l * (l + 1) / 2 > lm) --l;
  while ((l + 1) * (l + 2) / 2 <= lm) ++l;
  m = lm - l * (l + 1) / 2;
}

__global__ void SurfaceDualKernel(Geometry g, const double2* u, const double2* phi, double2* sol) {
  const int lm = blockIdx.x * blockDim.x + threadIdx.x;
  if (lm >= (g.lmax + 1) * (g.lmax + 2) / 2) return;
  int l, m;
  LmOf(lm, l, m);
  const DegreeInfo d = g.degrees[l];
  if (u != nullptr && d.surfaceU >= 0) {
    double2& x = sol[d.sphRhs + static_cast<long long>(d.surfaceU) * (l + 1) + m];
    x = make_double2(x.x + u[lm].x, x.y + u[lm].y);
  }
  if (phi != nullptr && d.surfacePhi >= 0) {
    double2& x = sol[d.sphRhs + static_cast<long long>(d.surfacePhi) * (l + 1) + m];
    x = make_double2(x.x + phi[lm].x, x.y + phi[lm].y);
  }
}

// One warp per (l, m): the lanes stride the degree's dofs, a shuffle sum.
__global__ void LoadDualKernel(Geometry g, const double* units, const long long* unitOffset, const double2* rhs,
                               double2* out) {
  const int lm = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (lm >= (g.lmax + 1) * (g.lmax + 2) / 2) return;
  int l, m;
  LmOf(lm, l, m);
  const DegreeInfo d = g.degrees[l];
  const double* u = units + unitOffset[l];
  double re = 0.0, im = 0.0;
  for (int dof = lane; dof < d.sphNdof; dof += 32) {
    const double2 y = rhs[d.sphRhs + static_cast<long long>(dof) * (l + 1) + m];
    re += u[dof] * y.x;
    im += u[dof] * y.y;
  }
  for (int o = 16; o > 0; o /= 2) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  if (lane == 0) out[lm] = make_double2(re, im);
}

// The stage weights of the step kernels (ExponentialTrapezoidWeights or
// BackwardEulerWeight) and their derivatives in h.
__device__ inline void WeightsAndSlopes(int scheme, double h, double& e, double& alpha, double& beta, double& de,
                                        double& dalpha, double& dbeta) {
  if (scheme == 1) {
    const double wbe = 1.0 / (1.0 + h);
    e = wbe;
    alpha = 0.0;
    beta = 1.0 - wbe;
    de = -wbe * wbe;
    dalpha = 0.0;
    dbeta = wbe * wbe;
    return;
  }
  const double ex = exp(-h);
  double phi1, dphi1;
  if (fabs(h) < 1e-3) {
    // the five-term series the step takes there, and its derivative
    phi1 = 1.0 - h / 2.0 + h * h / 6.0 - h * h * h / 24.0 + h * h * h * h / 120.0;
    dphi1 = -0.5 + h / 3.0 - h * h / 8.0 + h * h * h / 30.0;
  } else {
    phi1 = (1.0 - ex) / h;
    dphi1 = (ex - phi1) / h;
  }
  e = ex;
  alpha = phi1 - ex;
  beta = 1.0 - phi1;
  de = -ex;
  dalpha = dphi1 + ex;
  dbeta = -dphi1;
}

__global__ void AdjointStrainKernel(AdjointStrainArgs a) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const int P = static_cast<int>(a.values / a.fieldSize);
  for (long long x = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < a.values; x += stride) {
    const int node = static_cast<int>(x / a.fieldSize);
    double2 o0 = a.d0[x], o1 = a.d1[x];
    double orr = a.dr[x];
    for (int k = 0; k < a.branches; ++k) {
      const double h = a.dt * (a.itauRef[static_cast<long long>(k) * P + node] * a.factor[x]);
      double e, alpha, b, de, dalpha, dbeta;
      WeightsAndSlopes(a.scheme, h, e, alpha, b, de, dalpha, dbeta);
      const double2 m0 = a.m0[k][x], m1 = a.m1[k][x];
      o0 = make_double2(o0.x + b * m0.x, o0.y + b * m0.y);
      o1 = make_double2(o1.x + b * m1.x, o1.y + b * m1.y);
      orr += b * a.mr[k][x];
    }
    a.o0[x] = o0;
    a.o1[x] = o1;
    a.orr[x] = orr;
  }
}

__device__ inline double Energy(double2 a0, double2 a1, double ar, double2 b0, double2 b1, double br) {
  return 4.0 * (a0.x * b0.x + a0.y * b0.y) + 8.0 * (a1.x * b1.x + a1.y * b1.y) + 12.0 * ar * br;
}

__global__ void AdjointMemoryKernel(AdjointMemoryArgs a) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const int P = static_cast<int>(a.values / a.fieldSize);
  for (long long x = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < a.values; x += stride) {
    const int node = static_cast<int>(x / a.fieldSize);
    const int j = static_cast<int>((x % a.fieldSize) / a.nphi);
    const double2 z0 = a.z0[x], z1 = a.z1[x];
    const double zr = a.zr[x];
    const double2 st0 = a.a0[x], st1 = a.a1[x], en0 = a.b0[x], en1 = a.b1[x];
    const double str = a.ar[x], enr = a.br[x];
    double2 p0 = make_double2(0.0, 0.0), p1 = make_double2(0.0, 0.0);
    double pr = 0.0, g = 0.0;
    for (int k = 0; k < a.branches; ++k) {
      const double mu = a.muBranch[static_cast<long long>(k) * P + node];
      const double h = a.dt * (a.itauRef[static_cast<long long>(k) * P + node] * a.factor[x]);
      double e, alpha, beta, de, dalpha, dbeta;
      WeightsAndSlopes(a.scheme, h, e, alpha, beta, de, dalpha, dbeta);
      const double2 M0 = make_double2(a.m0[k][x].x + mu * z0.x, a.m0[k][x].y + mu * z0.y);
      const double2 M1 = make_double2(a.m1[k][x].x + mu * z1.x, a.m1[k][x].y + mu * z1.y);
      const double Mr = a.mr[k][x] + mu * zr;
      const double pe = Energy(M0, M1, Mr, a.s0[k][x], a.s1[k][x], a.sr[k][x]);
      const double pa = Energy(M0, M1, Mr, st0, st1, str);
      const double pb = Energy(M0, M1, Mr, en0, en1, enr);
      g -= h * (de * pe + dalpha * pa + dbeta * pb);
      a.m0[k][x] = make_double2(e * M0.x, e * M0.y);
      a.m1[k][x] = make_double2(e * M1.x, e * M1.y);
      a.mr[k][x] = e * Mr;
      p0 = make_double2(p0.x + alpha * M0.x, p0.y + alpha * M0.y);
      p1 = make_double2(p1.x + alpha * M1.x, p1.y + alpha * M1.y);
      pr += alpha * Mr;
    }
    a.d0[x] = p0;
    a.d1[x] = p1;
    a.dr[x] = pr;
    a.grad[x] += a.nodeVolume[node] * a.colWeight[j] * g;
  }
}

__global__ void TangentKernel(TangentArgs a) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const int P = static_cast<int>(a.values / a.fieldSize);
  for (long long x = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; x < a.values; x += stride) {
    const int node = static_cast<int>(x / a.fieldSize);
    const double p = a.direction != nullptr ? a.direction[x] : 0.0;
    const double2 t0 = a.t0[x], t1 = a.t1[x], b0 = a.b0[x], b1 = a.b1[x];
    const double tr = a.tr[x], br = a.br[x];
    double2 f0 = make_double2(0.0, 0.0), f1 = make_double2(0.0, 0.0);
    double fr = 0.0, wdot = 0.0;
    for (int k = 0; k < a.branches; ++k) {
      const double mu = a.muBranch[static_cast<long long>(k) * P + node];
      const double h = a.dt * (a.itauRef[static_cast<long long>(k) * P + node] * a.factor[x]);
      double e, alpha, beta, de, dalpha, dbeta;
      WeightsAndSlopes(a.scheme, h, e, alpha, beta, de, dalpha, dbeta);
      const double hdot = -h * p;
      if (a.finish) {
        const double bd = dbeta * hdot;
        a.m0[k][x] = make_double2(a.m0[k][x].x + beta * t0.x + bd * b0.x, a.m0[k][x].y + beta * t0.y + bd * b0.y);
        a.m1[k][x] = make_double2(a.m1[k][x].x + beta * t1.x + bd * b1.x, a.m1[k][x].y + beta * t1.y + bd * b1.y);
        a.mr[k][x] += beta * tr + bd * br;
        continue;
      }
      const double ed = de * hdot, ad = dalpha * hdot;
      const double2 s0 = a.s0[k][x], s1 = a.s1[k][x], a0 = a.a0[x], a1 = a.a1[x];
      const double sr = a.sr[k][x], ar = a.ar[x];
      const double2 m0 = make_double2(e * a.m0[k][x].x + alpha * t0.x + ed * s0.x + ad * a0.x,
                                      e * a.m0[k][x].y + alpha * t0.y + ed * s0.y + ad * a0.y);
      const double2 m1 = make_double2(e * a.m1[k][x].x + alpha * t1.x + ed * s1.x + ad * a1.x,
                                      e * a.m1[k][x].y + alpha * t1.y + ed * s1.y + ad * a1.y);
      const double mr = e * a.mr[k][x] + alpha * tr + ed * sr + ad * ar;
      a.m0[k][x] = m0;
      a.m1[k][x] = m1;
      a.mr[k][x] = mr;
      f0 = make_double2(f0.x + mu * m0.x, f0.y + mu * m0.y);
      f1 = make_double2(f1.x + mu * m1.x, f1.y + mu * m1.y);
      fr += mu * mr;
      wdot += mu * dbeta * hdot;
    }
    if (!a.finish) {
      a.f0[x] = make_double2(f0.x + wdot * b0.x, f0.y + wdot * b0.y);
      a.f1[x] = make_double2(f1.x + wdot * b1.x, f1.y + wdot * b1.y);
      a.fr[x] = fr + wdot * br;
    }
  }
}

__global__ void ScaleKernel(long long n, double s, double* y) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride) y[i] *= s;
}

int Blocks(long long values) {
  const long long b = (values + 255) / 256;
  return static_cast<int>(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

}  // namespace

void LaunchSurfaceDual(const Geometry& g, const double2* u, const double2* phi, double2* solSph,
                       cudaStream_t stream) {
  if (u == nullptr && phi == nullptr) return;
  const int count = (g.lmax + 1) * (g.lmax + 2) / 2;
  prof::Scope scope(prof::kOther, stream);
  SurfaceDualKernel<<<(count + 127) / 128, 128, 0, stream>>>(g, u, phi, solSph);
}

void LaunchLoadDual(const Geometry& g, const double* units, const long long* unitOffset, const double2* rhsSph,
                    double2* out, cudaStream_t stream) {
  const int count = (g.lmax + 1) * (g.lmax + 2) / 2;
  prof::Scope scope(prof::kOther, stream);
  LoadDualKernel<<<(count + 7) / 8, 256, 0, stream>>>(g, units, unitOffset, rhsSph, out);
}

void LaunchAdjointStrainDual(const AdjointStrainArgs& a, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, a.values * (a.branches * 48.0 + 80.0));
  AdjointStrainKernel<<<Blocks(a.values), 256, 0, stream>>>(a);
}

void LaunchAdjointMemory(const AdjointMemoryArgs& a, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, a.values * (a.branches * 120.0 + 136.0));
  AdjointMemoryKernel<<<Blocks(a.values), 256, 0, stream>>>(a);
}

void LaunchTangent(const TangentArgs& a, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, a.values * (a.branches * (a.finish ? 80.0 : 120.0) + 120.0));
  TangentKernel<<<Blocks(a.values), 256, 0, stream>>>(a);
}

void LaunchScale(long long n, double a, double* y, cudaStream_t stream) {
  prof::Scope scope(prof::kStream, stream, 0.0, n * 16.0);
  ScaleKernel<<<Blocks(n), 256, 0, stream>>>(n, a, y);
}

}  // namespace sl3dgpu
