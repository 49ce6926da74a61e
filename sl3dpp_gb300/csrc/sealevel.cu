// The sea-level equation's load fixed point on the GPU: GRDSolver::
// SolveGeneralised (src/SeaLevel.cpp:397-736) with rotational feedback None,
// Axial or Full, in the solver's non-dimensional units, for GeneralisedForcing's
// channels: the direct load in and outside the water budget, a layer on the
// solid surface, a prescribed tide, the displacement and potential loads and
// the tangential traction (each through its own Love numbers), and the ready
// displacement, potential and tangential responses of the coupled Evolution3D
// closure (src/Evolution3D.cpp:320-333).
//
// With per-degree load Love numbers h_l, k_l (l_l tangential), tidal ones,
// surface gravity g, water density rho_w, the sea-floor radius a, an ocean
// function C and the direct load sigma_d on the surface grid:
//
//   static  D_s = R_u + h^t T + sum_c h^c E_c,  G_s = R_phi + k^t T + sum_c k^c E_c,
//           V_s = R_v + l^t T + sum_c l^c E_c  (E_c a load channel's expansion)
//           S_s = -(D_s + G_s / g) - T / g - Expand(layer)      (:453-545, :586-600)
//   A       = a^2 int C dOmega, 1/A (0 without an ocean)       (:570-574)
//   s_mean  = -a^2 int sigma_d dOmega / (A rho_w)                (:577-581)
//   sigma   = sigma_d + sigma_outside                             (:582-587)
//   L_0     = Expand(sigma + rho_w C s_mean)                     (:672-676)
//   repeat  S    = Synthesise(-(h_l + k_l / g) L_lm + S_s)       (:625-634)
//           (rotating: its degree-2 and degree-0 coefficients from the
//           rotation block of the load, :625-640)
//           S   += s_mean - a^2 int C S dOmega / A               (:655-661)
//           stop when max|C S - C S_prev| <= rtol max|C S|       (:683-692)
//           L   <- Anderson(L, Expand(sigma + rho_w C S))        (:694-699)
//   then the displacement, potential and tangential potential as
//   Synthesise(h_l L + D_s), Synthesise(k_l L + G_s), Synthesise(l_l L + V_s)
//   (:702-720), the toroidal response carried as Synthesise(R_w).
//
// The transforms are the grid's (sht.cu), the mixer the Anderson sweeps of
// the 3D step (step_kernels.cu) with the reference's memory and plain start;
// the integrals sum each ring in a fixed tree and the rings in order (the
// grid's Integrate, SurfaceGrid.hpp:257-267); the stopping test's maxima are
// order-free. The rotation block (RotationPatchKernel) and the conservation's
// shift (ShiftKernel) are formed on the device; an iteration brings one
// thing to the host, the stopping test's maxima. A workspace (SleWorkspace)
// keeps the buffers between solves on one grid, so that the coupled closure's
// solve in every pass of a step allocates nothing.
//
// GRDSolver::SolveNonlinear (src/SeaLevel.cpp:970-1289), migrating
// shorelines, shares the static terms and the rotation patch: a plain fixed
// point from a state (ice I0, sea level SL0, ocean function C0), each
// iteration the load of the grounded ice's and the water's changes at the
// current ocean function C and change dS (BudgetLoadKernel), its sea level
// change synthesised, the water budget closed by a uniform shift over the
// current ocean (BudgetRingKernel, BudgetShiftKernel) and C re-derived by
// flotation, rho_w (SL0 + dS) - rho_i (I0 + dI) > 0 off the land held
// (BudgetUpdateKernel).
#include <algorithm>
#include <array>
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "profile.cuh"
#include "sl3dgpu.h"
#include "step_kernels.cuh"
#include "systems.cuh"
#include "sealevel.cuh"

namespace sl3dgpu {
namespace {

constexpr int kRingThreads = 256;

// partial[j] = w_j sum_k a(j, k) [b(j, k)]: one block per ring, a fixed tree.
__global__ void RingSumKernel(int nphi, const double* weights, const double* a, const double* b, double* partial) {
  __shared__ double red[kRingThreads];
  const int j = blockIdx.x;
  const double* ra = a + static_cast<long long>(j) * nphi;
  const double* rb = b ? b + static_cast<long long>(j) * nphi : nullptr;
  double v = 0.0;
  for (int k = threadIdx.x; k < nphi; k += blockDim.x) v += rb ? ra[k] * rb[k] : ra[k];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[j] = weights[j] * red[0];
}

// out[x] = f[l] in[x] + c add[x] over the (l, m >= 0) coefficients,
// Index(l, m) = l(l+1)/2 + m (add may be null).
__global__ void ScaleDegreesKernel(int lmax, const double* f, const double2* in, const double2* add, double c,
                                   double2* out) {
  const long long count = static_cast<long long>(lmax + 1) * (lmax + 2) / 2;
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  int l = static_cast<int>((sqrt(8.0 * static_cast<double>(i) + 1.0) - 1.0) * 0.5);
  while (static_cast<long long>(l) * (l + 1) / 2 > i) --l;
  while (static_cast<long long>(l + 1) * (l + 2) / 2 <= i) ++l;
  const double2 v = in[i];
  double2 o = make_double2(f[l] * v.x, f[l] * v.y);
  if (add != nullptr) {
    o.x += c * add[i].x;
    o.y += c * add[i].y;
  }
  out[i] = o;
}

// out[x] = a[x] + c b[x] over complex coefficients
__global__ void AxpyKernel(long long count, const double2* a, const double2* b, double c, double2* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < count) out[i] = make_double2(a[i].x + c * b[i].x, a[i].y + c * b[i].y);
}

// out[x] = a[x] + b[x] over a field
__global__ void AddFieldKernel(long long n, const double* a, const double* b, double* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}

// seeded[x] = sigma_d[x] + rho_w C[x] s_mean
__global__ void SeedKernel(long long n, const double* direct, const double* ocean, double rhoMean, double* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = direct[i] + rhoMean * ocean[i];
}

// S += shift; C S; the next load sigma_d + rho_w C S; per block the largest
// |C S - C S_prev| and |C S| (blockIdx-ordered partials), C S kept for the next test.
__global__ void ShiftAndLoadKernel(long long n, const double* shiftPtr, double rho, const double* direct,
                                   const double* ocean, double* slc, double* oceanSlc, double* newLoad, bool havePrev,
                                   double* maxima) {
  __shared__ double red[2][kRingThreads];
  const double shift = *shiftPtr;
  double dmax = 0.0, smax = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double s = slc[i] + shift;
    slc[i] = s;
    const double cs = ocean[i] * s;
    if (havePrev) dmax = fmax(dmax, fabs(cs - oceanSlc[i]));
    smax = fmax(smax, fabs(cs));
    oceanSlc[i] = cs;
    newLoad[i] = direct[i] + rho * cs;
  }
  red[0][threadIdx.x] = dmax;
  red[1][threadIdx.x] = smax;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if (threadIdx.x < s) {
      red[0][threadIdx.x] = fmax(red[0][threadIdx.x], red[0][threadIdx.x + s]);
      red[1][threadIdx.x] = fmax(red[1][threadIdx.x], red[1][threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    maxima[2 * blockIdx.x] = red[0][0];
    maxima[2 * blockIdx.x + 1] = red[1][0];
  }
}

// per block the largest |a|
__global__ void MaxAbsKernel(long long n, const double* a, double* maxima) {
  __shared__ double red[kRingThreads];
  double v = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    v = fmax(v, fabs(a[i]));
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) maxima[2 * blockIdx.x + 1] = red[0];
}

constexpr int kMaxBlocks = 304;  // two a multiprocessor for the pointwise pass

struct SleRun {
  sl3dgpu_grid* grid;
  cudaStream_t stream;
  int lmax = 0, ntheta = 0, nphi = 0;
  long long fieldSize = 0, coefCount = 0;
  double r2 = 0.0, dphi = 0.0;
  Dev<double> weights, ringPartial, maxima, loadLm, newLoadLm, scaledLm, factors;
  Dev<double> seeded, slc, oceanSlc, newLoad;
  std::vector<double> hostRing, hostMaxima;

  // a^2 int a (b) dOmega, the rings in order
  int Integrate(const double* a, const double* b, double* out) {
    RingSumKernel<<<ntheta, kRingThreads, 0, stream>>>(nphi, weights.p, a, b, ringPartial.p);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemcpyAsync(hostRing.data(), ringPartial.p, ntheta * sizeof(double), cudaMemcpyDeviceToHost,
                              stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    double sum = 0.0;
    for (int j = 0; j < ntheta; ++j) sum += hostRing[j];
    *out = r2 * sum * dphi;
    return SL3DGPU_OK;
  }

  // out = f_l coefficients + c add (add may be null)
  int ScaleDegrees(const double* f, const double* coeffs, const double* add, double c, double* out) {
    SL3D_CUDA(cudaMemcpyAsync(factors.p, f, (lmax + 1) * sizeof(double), cudaMemcpyHostToDevice, stream));
    const unsigned blocks = static_cast<unsigned>((coefCount + 255) / 256);
    ScaleDegreesKernel<<<blocks, 256, 0, stream>>>(lmax, factors.p, reinterpret_cast<const double2*>(coeffs),
                                                   reinterpret_cast<const double2*>(add), c,
                                                   reinterpret_cast<double2*>(out));
    SL3D_CHECK_LAUNCH();
    return SL3DGPU_OK;
  }
  // field = Synthesise(f_l coefficients + add)
  int SynthesiseScaled(const double* f, const double* coeffs, double* field, const double* add = nullptr) {
    SL3D_TRY(ScaleDegrees(f, coeffs, add, 1.0, scaledLm.p));
    return sl3dgpu_synthesise_batch(grid, scaledLm.p, 1, field, stream);
  }
  // out = a + c b (complex coefficients)
  int Axpy(const double* a, const double* b, double c, double* out) {
    AxpyKernel<<<static_cast<unsigned>((coefCount + 255) / 256), 256, 0, stream>>>(
        coefCount, reinterpret_cast<const double2*>(a), reinterpret_cast<const double2*>(b), c,
        reinterpret_cast<double2*>(out));
    SL3D_CHECK_LAUNCH();
    return SL3DGPU_OK;
  }
  // the largest |a| over n values (field or coefficients viewed as reals)
  int MaxAbs(const double* a, long long n, double* out) {
    const int b = static_cast<int>(std::min<long long>(kMaxBlocks, (n + 255) / 256));
    MaxAbsKernel<<<b, kRingThreads, 0, stream>>>(n, a, maxima.p);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemcpyAsync(hostMaxima.data(), maxima.p, 2 * b * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    double m = 0.0;
    for (int i = 0; i < b; ++i) m = std::max(m, hostMaxima[2 * i + 1]);
    *out = m;
    return SL3DGPU_OK;
  }
};

// The conservation's uniform shift on the device: a^2 dphi sum_rings of the
// ring partials of C S, in order (the host's Integrate), then s_mean minus
// it over the ocean's area (src/SeaLevel.cpp:655-661).
__global__ void ShiftKernel(const double* ringPartial, int ntheta, double scale, double meanSlc, double perOceanArea,
                            double* shift) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double sum = 0.0;
  for (int j = 0; j < ntheta; ++j) sum += ringPartial[j];
  shift[0] = meanSlc - scale * sum * perOceanArea;
}

// GRDSolver::Rotation's inputs that do not change within a solve: the
// factors of the constructor (src/SeaLevel.cpp:220-247), the static blocks
// and scalars of the forcing. Blocks as {(2,0), cos(2,1), 0, sin(2,1)}.
struct RotationInputs {
  int transverse;
  double h2, k2, ht2, kt2, hc, kc, mu, mphi, mc, g, lt2;
  double rotation, inertia, axialRotation, uniformRotation, axialInertia, inverseInertiaDifference,
      inversePolarInertia, trace, shell, rotationDenominator, axialRotationDenominator;
  double staticDisp2[4], staticGrav2[4], tide2[4], layer2[4];
  double displacementLoad0, potentialLoad0, inertiaMoment, angularMomentum[3];
};

// The rotation block of the load's (2, 0), (2, 1) and (0, 0) coefficients
// (GRDSolver::Rotation, src/SeaLevel.cpp:348-392), and the patch of a
// scaled coefficient vector's degree-0/2 entries, on the device: mode 0 the
// sea level change's (and the angular velocity out), 1 the displacement's,
// 2 the potential's, 3 the tangential potential's (src/SeaLevel.cpp:625-640,
// 714-724). One thread; the host solve's arithmetic in its order.
__global__ void RotationPatchKernel(const RotationInputs* p, const double* load, double* out, double* omegaOut,
                                    int mode) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double r2 = sqrt(2.0);
  // BlockOf of the load: (2,0) re, -sqrt2 re (2,1), sqrt2 im (2,1)
  const double l00 = load[6], l01 = -r2 * load[8], l11 = r2 * load[9];
  const double load0 = load[0];
  const double grav00 = p->k2 * l00 + p->staticGrav2[0], grav01 = p->k2 * l01 + p->staticGrav2[1],
               grav11 = p->k2 * l11 + p->staticGrav2[3];
  const double disp00 = p->h2 * l00 + p->staticDisp2[0], disp01 = p->h2 * l01 + p->staticDisp2[1],
               disp11 = p->h2 * l11 + p->staticDisp2[3];
  double transverse0 = p->inertia * grav01, transverse1 = p->inertia * grav11;
  double axial = -p->axialInertia * grav00 -
                 p->trace * ((p->mu + p->mphi) * load0 + p->mu * p->displacementLoad0 + p->mphi * p->potentialLoad0 +
                             p->inertiaMoment) -
                 p->shell * (load0 + p->potentialLoad0);
  transverse0 -= p->inverseInertiaDifference * p->angularMomentum[0];
  transverse1 -= p->inverseInertiaDifference * p->angularMomentum[1];
  axial += p->inversePolarInertia * p->angularMomentum[2];
  double omega0 = 0.0, omega1 = 0.0;
  if (p->transverse) {
    omega0 = transverse0 / p->rotationDenominator;
    omega1 = transverse1 / p->rotationDenominator;
  }
  const double omega2 = axial / p->axialRotationDenominator;
  const double c00 = p->axialRotation * omega2, c01 = p->rotation * omega0, c11 = p->rotation * omega1;
  const double centrifugal0 = p->uniformRotation * omega2;
  const double d00 = disp00 + p->ht2 * c00, d01 = disp01 + p->ht2 * c01, d11 = disp11 + p->ht2 * c11;
  const double g00 = grav00 + p->kt2 * c00, g01 = grav01 + p->kt2 * c01, g11 = grav11 + p->kt2 * c11;
  // FromBlock into out[6..9]: (2,0) = b00, (2,1) = (-b01 / sqrt2, b11 / sqrt2)
  auto put = [&](double b00, double b01, double b11) {
    out[6] = b00;
    out[7] = 0.0;
    out[8] = -b01 / r2;
    out[9] = b11 / r2;
  };
  const double ig = 1.0 / p->g;
  if (mode == 0) {
    omegaOut[0] = omega0;
    omegaOut[1] = omega1;
    omegaOut[2] = omega2;
    const double s00 = -((d00 + ((g00 + c00) + p->tide2[0]) * ig) + p->layer2[0]);
    const double s01 = -((d01 + ((g01 + c01) + p->tide2[1]) * ig) + p->layer2[1]);
    const double s11 = -((d11 + ((g11 + c11) + p->tide2[3]) * ig) + p->layer2[3]);
    put(s00, s01, s11);
    out[0] -= (p->hc + (p->kc + 1.0) / p->g) * centrifugal0;
  } else if (mode == 1) {
    put(d00, d01, d11);
    out[0] += p->hc * centrifugal0;
  } else if (mode == 2) {
    put(g00, g01, g11);
    out[0] += p->kc * centrifugal0;
  } else {
    out[6] += p->lt2 * c00;
    out[8] += -(p->lt2 * c01) / r2;
    out[9] += (p->lt2 * c11) / r2;
  }
}

// The Anderson mixer of the load coefficients (AndersonMixer::Update, the
// reference's plain form: the first call the image, then memory columns).
struct LoadMixer {
  int memory = 0, count = 0, slot = 0;
  bool first = true;
  std::vector<Dev<double>> dG, dF;
  Dev<double*> dGPtr, dFPtr;
  Dev<double> xPrev, fPrev, partial, sums, gamma, gram;  // the Gram matrix on the device

  int Init(int m, long long n) {
    memory = m;
    if (memory <= 0) return SL3DGPU_OK;
    dG.resize(memory);
    dF.resize(memory);
    std::vector<double*> gp(memory), fp(memory);
    for (int i = 0; i < memory; ++i) {
      SL3D_CUDA(dG[i].Alloc(n));
      SL3D_CUDA(dF[i].Alloc(n));
      gp[i] = dG[i].p;
      fp[i] = dF[i].p;
    }
    SL3D_CUDA(dGPtr.Upload(gp));
    SL3D_CUDA(dFPtr.Upload(fp));
    SL3D_CUDA(xPrev.Alloc(n));
    SL3D_CUDA(fPrev.Alloc(n));
    SL3D_CUDA(partial.Alloc(static_cast<size_t>(1024) * 2 * kMixMaxMemory));
    SL3D_CUDA(sums.Alloc(2 * kMixMaxMemory));
    SL3D_CUDA(gamma.Alloc(kMixMaxMemory + 1));
    SL3D_CUDA(gram.Alloc(static_cast<size_t>(memory) * memory));
    SL3D_CUDA(ZeroIn(gram.p, static_cast<size_t>(memory) * memory * sizeof(double)));
    return SL3DGPU_OK;
  }

  // x <- the mixed iterate from x and its image gx
  int Update(double* x, const double* gx, long long n, cudaStream_t stream) {
    if (memory <= 0) {
      SL3D_CUDA(cudaMemcpyAsync(x, gx, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
      return SL3DGPU_OK;
    }
    MixerArgs a{};
    a.n = n;
    a.memory = memory;
    a.x = x;
    a.gx = gx;
    a.xPrev = xPrev.p;
    a.fPrev = fPrev.p;
    a.dG = dGPtr.p;
    a.dF = dFPtr.p;
    a.partial = partial.p;
    a.blocks = static_cast<int>(std::min<long long>(1024, n));
    a.gamma = gamma.p;
    if (first) {
      LaunchMixerFirst(a, stream);
      SL3D_CHECK_LAUNCH();
      first = false;
      return SL3DGPU_OK;
    }
    a.slot = slot;
    a.m = std::min(count + 1, memory);
    LaunchMixerSweep(a, sums.p, stream);
    SL3D_CHECK_LAUNCH();
    LaunchMixerGram(gram.p, a.m, a.slot, a.memory, sums.p, gamma.p, stream);  // one FP64 warp, no host round trip
    SL3D_CHECK_LAUNCH();
    LaunchMixerMix(a, stream);
    SL3D_CHECK_LAUNCH();
    count = a.m;
    slot = (slot + 1) % memory;
    return SL3DGPU_OK;
  }
};

// -- the degree-2 / degree-0 rotational feedback (GRDSolver::Rotation,
// src/SeaLevel.cpp:340-395), on the host: a handful of coefficients an
// iteration, in the real (cos, sin) pairs of the (2, 1) coefficient
// (ShConventions.hpp:40-54) ---------------------------------------------------

using Block2 = std::array<std::array<double, 2>, 2>;  // [0][0] (2,0); [0][1], [1][1] (2,1) cos, sin

Block2 Scaled(const Block2& b, double c) { return {{{c * b[0][0], c * b[0][1]}, {c * b[1][0], c * b[1][1]}}}; }
Block2 Plus(const Block2& a, const Block2& b) {
  return {{{a[0][0] + b[0][0], a[0][1] + b[0][1]}, {a[1][0] + b[1][0], a[1][1] + b[1][1]}}};
}
// BlockOf: from the (2, 0) and (2, 1) coefficients (re, im pairs)
Block2 BlockOf(const double* c20, const double* c21) {
  const double r2 = std::sqrt(2.0);
  return {{{c20[0], -r2 * c21[0]}, {0.0, r2 * c21[1]}}};
}
// SetBlock's (2, 0) and (2, 1) coefficients from a block
void FromBlock(const Block2& b, double* c20, double* c21) {
  const double r2 = std::sqrt(2.0);
  c20[0] = b[0][0];
  c20[1] = 0.0;
  c21[0] = -b[0][1] / r2;
  c21[1] = b[1][1] / r2;
}

struct RotationFactors {
  bool on = false, transverse = false;
  double h2, k2, ht2, kt2, hc, kc, mu, mphi, mc;
  double rotation, inertia, axialRotation, uniformRotation, axialInertia, inverseInertiaDifference,
      inversePolarInertia, trace, shell, rotationDenominator, axialRotationDenominator;
  // the constructor's factors (src/SeaLevel.cpp:220-247)
  void Init(const sl3dgpu_sle_body& b) {
    on = b.rotation != 0;
    transverse = b.rotation == 2;
    if (!on) return;
    const double pi = 3.14159265358979323846, a = b.radius, w = b.omega, G = b.gravitational_constant;
    const double C = b.polar_moment, A = b.equatorial_moment;
    h2 = b.h[2];
    k2 = b.k[2];
    ht2 = b.ht[2];
    kt2 = b.kt[2];
    hc = b.hc;
    kc = b.kc;
    mu = b.m_u;
    mphi = b.m_phi;
    mc = b.m_c;
    rotation = std::sqrt(4.0 * pi / 15.0) * w * a * a;
    inertia = std::sqrt(5.0 / (12.0 * pi)) * w * a * a * a / (G * (C - A));
    axialRotation = std::sqrt(16.0 * pi / 45.0) * w * a * a;
    uniformRotation = -std::sqrt(16.0 * pi / 9.0) * w * a * a;
    axialInertia = std::sqrt(5.0 / (9.0 * pi)) * w * a * a * a / (G * C);
    inverseInertiaDifference = 1.0 / (C - A);
    inversePolarInertia = 1.0 / C;
    trace = (4.0 / 3.0) * w / C;
    shell = (2.0 / 3.0) * w * std::pow(a, 4) * std::sqrt(4.0 * pi) / C;
    rotationDenominator = 1.0 - inertia * kt2 * rotation;
    axialRotationDenominator = 1.0 + axialInertia * kt2 * axialRotation + trace * mc * uniformRotation;
  }
};

}  // namespace

// The workspace one solver keeps between solves on one grid: the run's
// buffers, the mixer and the static terms.
struct SleWorkspace {
  sl3dgpu_grid* grid = nullptr;
  SleRun run;
  LoadMixer mixer;
  int mixerMemory = -1;
  Dev<double> staticDisp, staticGrav, staticTan, staticSlc, scratch, directData;
  Dev<double> shift, omega, slcFactor;  // the conservation's shift, the angular velocity, -(h + k / g) per degree
  Dev<RotationInputs> rotation;
  std::vector<double> theta;
  // the nonlinear solve's iterates: the ocean function, the sea level change
  // from the state, the sea level change's last value and the local one,
  // and the water budget's ring partials
  Dev<double> nlOcean, nlChange, nlSlc, nlLocal, nlRingUnbalanced, nlRingOcean;

  // the grid's sizes, quadrature and buffers (once per grid)
  int Prepare(sl3dgpu_grid* g) {
    if (grid == g) return SL3DGPU_OK;
    grid = nullptr;
    run.grid = g;
    int ntheta = 0, nphi = 0;
    SL3D_TRY(sl3dgpu_grid_shape(g, &ntheta, &nphi));
    run.lmax = sl3dgpu_grid_lmax(g);
    if (run.lmax < 0) return SL3DGPU_ERR_ARGUMENT;
    run.ntheta = ntheta;
    run.nphi = nphi;
    run.fieldSize = static_cast<long long>(ntheta) * nphi;
    run.coefCount = static_cast<long long>(run.lmax + 1) * (run.lmax + 2) / 2;
    run.dphi = 2.0 * 3.14159265358979323846 / nphi;
    std::vector<double> w(ntheta);
    theta.assign(ntheta, 0.0);
    SL3D_TRY(sl3dgpu_grid_colatitudes(g, theta.data(), w.data()));
    SL3D_CUDA(run.weights.Upload(w));
    SL3D_CUDA(run.ringPartial.Alloc(ntheta));
    run.hostRing.assign(ntheta, 0.0);
    SL3D_CUDA(run.maxima.Alloc(2 * kMaxBlocks));
    run.hostMaxima.assign(2 * kMaxBlocks, 0.0);
    const long long nc = 2 * run.coefCount;
    for (auto* d : {&run.loadLm, &run.newLoadLm, &run.scaledLm}) SL3D_CUDA(d->Alloc(nc));
    SL3D_CUDA(run.factors.Alloc(run.lmax + 1));
    for (auto* d : {&run.seeded, &run.slc, &run.oceanSlc, &run.newLoad}) SL3D_CUDA(d->Alloc(run.fieldSize));
    for (auto* d : {&staticDisp, &staticGrav, &staticTan, &staticSlc, &scratch}) SL3D_CUDA(d->Alloc(nc));
    SL3D_CUDA(directData.Alloc(run.fieldSize));
    SL3D_CUDA(shift.Alloc(1));
    SL3D_CUDA(omega.Alloc(3));
    SL3D_CUDA(slcFactor.Alloc(run.lmax + 1));
    SL3D_CUDA(rotation.Alloc(1));
    for (auto* d : {&nlOcean, &nlChange, &nlSlc, &nlLocal, &nlRingUnbalanced, &nlRingOcean}) *d = Dev<double>();
    mixerMemory = -1;
    grid = g;
    return SL3DGPU_OK;
  }
  // the nonlinear solve's buffers (on its first use on the grid)
  int PrepareNonlinear() {
    if (nlOcean.p != nullptr) return SL3DGPU_OK;
    for (auto* d : {&nlOcean, &nlChange, &nlSlc, &nlLocal}) SL3D_CUDA(d->Alloc(run.fieldSize));
    SL3D_CUDA(nlRingUnbalanced.Alloc(run.ntheta));
    SL3D_CUDA(nlRingOcean.Alloc(run.ntheta));
    return SL3DGPU_OK;
  }
  // the mixer at its plain start, with `memory` columns
  int ResetMixer(int memory, cudaStream_t s) {
    if (mixerMemory != memory) {
      mixer = LoadMixer{};
      SL3D_TRY(mixer.Init(memory, 2 * run.coefCount));
      mixerMemory = memory;
      return SL3DGPU_OK;
    }
    mixer.first = true;
    mixer.count = mixer.slot = 0;
    if (memory > 0)
      SL3D_CUDA(cudaMemsetAsync(mixer.gram.p, 0, static_cast<size_t>(memory) * memory * sizeof(double), s));
    return SL3DGPU_OK;
  }
};

SleWorkspace* NewSleWorkspace() { return new SleWorkspace; }
void FreeSleWorkspace(SleWorkspace* ws) { delete ws; }

int CentrifugalCoefficients(const sl3dgpu_sle_body& body, const double omega[3], double out[6]) {
  RotationFactors rf;
  rf.Init(body);
  for (int i = 0; i < 6; ++i) out[i] = 0.0;
  if (!rf.on) return SL3DGPU_OK;
  // (0, 0), (2, 0) and (2, 1) of CentrifugalCoefficients (src/SeaLevel.cpp:249-258);
  // the (2, 1) pair as the complex coefficient (ShConventions.hpp:40-45)
  out[0] = rf.uniformRotation * omega[2];
  out[2] = rf.axialRotation * omega[2];
  out[4] = -rf.rotation * omega[0] / std::sqrt(2.0);
  out[5] = rf.rotation * omega[1] / std::sqrt(2.0);
  return SL3DGPU_OK;
}

namespace {

// What a solve's forcing carries (the reference's MaxAbs > 0 tests) and
// whether it rotates: the generalised and the nonlinear solves share it.
struct SleSetup {
  bool hasDirect = false, hasOutside = false, hasLayer = false, hasDisp = false, hasPot = false, hasTan = false,
       hasTide = false, hasLoadChannel = false;
  bool anyStatic = false, anyStaticTan = false, rotating = false;
  std::vector<double> tangential;  // the load's l per degree, degree 0 zero
};

// The body's checks, the grid's workspace, -(h + k / g) on the device, the
// static coefficient terms (src/SeaLevel.cpp:453-545, :586-600: D_s, G_s,
// V_s, S_s) and the rotation's fixed inputs (:604-608) on the device; the
// angular velocity and the shift zeroed.
int PrepareSolve(SleWorkspace& ws, sl3dgpu_grid* grid, const sl3dgpu_sle_body* body,
                 const sl3dgpu_sle_forcing* forcing, cudaStream_t s, SleSetup* su) {
  const double g = body->g, water_density = body->water_density, radius = body->radius;
  if (!(g > 0.0) || !(water_density > 0.0) || !(radius > 0.0)) {
    SetError("sle: g, water_density and radius > 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if ((forcing->displacement_load != nullptr && (body->h_u == nullptr || body->k_u == nullptr)) ||
      (forcing->potential_load != nullptr && (body->h_phi == nullptr || body->k_phi == nullptr)) ||
      (forcing->tangential_traction != nullptr && (body->h_v == nullptr || body->k_v == nullptr))) {
    SetError("sle: a displacement load needs h_u and k_u, a potential load h_phi and k_phi, a tangential traction "
             "h_v and k_v");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (forcing->tide != nullptr && (body->ht == nullptr || body->kt == nullptr)) {
    SetError("sle: a tide needs the tidal Love numbers ht and kt");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (body->rotation < 0 || body->rotation > 2 ||
      (body->rotation != 0 && (body->ht == nullptr || body->kt == nullptr || !(body->polar_moment > 0.0) ||
                               !(body->polar_moment != body->equatorial_moment) ||
                               !(body->gravitational_constant > 0.0)))) {
    SetError("sle: rotation 0 (none), 1 (axial) or 2 (full); with feedback, the tidal ht and kt, the moments of "
             "inertia (polar > 0, unequal) and the gravitational constant");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_TRY(ws.Prepare(grid));
  SleRun& run = ws.run;
  run.stream = s;
  run.r2 = radius * radius;
  if (body->rotation != 0 && run.lmax < 2) {
    SetError("sle: rotational feedback needs degree 2 on the grid");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const int L = run.lmax;
  const long long nc = 2 * run.coefCount;  // coefficients as reals
  std::vector<double> slcFactor(L + 1);
  for (int l = 0; l <= L; ++l) slcFactor[l] = -(body->h[l] + body->k[l] / g);
  SL3D_CUDA(cudaMemcpyAsync(ws.slcFactor.p, slcFactor.data(), (L + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
  su->tangential.assign(L + 1, 0.0);
  if (body->l != nullptr)
    for (int l = 1; l <= L; ++l) su->tangential[l] = body->l[l];  // a degree-0 field has no tangential part

  auto nonzero = [&](const double* a, long long n, bool* out) -> int {
    double m = 0.0;
    if (a != nullptr) SL3D_TRY(run.MaxAbs(a, n, &m));
    *out = m > 0.0;
    return SL3DGPU_OK;
  };
  bool hasDispLoad, hasPotLoad, hasTraction;
  SL3D_TRY(nonzero(forcing->direct_load, run.fieldSize, &su->hasDirect));
  SL3D_TRY(nonzero(forcing->direct_load_outside, run.fieldSize, &su->hasOutside));
  SL3D_TRY(nonzero(forcing->solid_surface_change, run.fieldSize, &su->hasLayer));
  SL3D_TRY(nonzero(forcing->displacement_response, nc, &su->hasDisp));
  SL3D_TRY(nonzero(forcing->potential_response, nc, &su->hasPot));
  SL3D_TRY(nonzero(forcing->tangential_response, nc, &su->hasTan));
  SL3D_TRY(nonzero(forcing->tide, nc, &su->hasTide));
  SL3D_TRY(nonzero(forcing->displacement_load, run.fieldSize, &hasDispLoad));
  SL3D_TRY(nonzero(forcing->potential_load, run.fieldSize, &hasPotLoad));
  SL3D_TRY(nonzero(forcing->tangential_traction, run.fieldSize, &hasTraction));
  su->hasLoadChannel = hasDispLoad || hasPotLoad || hasTraction;
  const bool hasTide = su->hasTide, hasLayer = su->hasLayer;
  if (hasTide) {
    // RequireTideDegrees (src/SeaLevel.cpp:83-96): no degree-0 or degree-1 part
    std::vector<double> low(6);
    SL3D_CUDA(cudaMemcpyAsync(low.data(), forcing->tide, 6 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SL3D_CUDA(cudaStreamSynchronize(s));
    for (double v : low)
      if (v != 0.0) {
        SetError("sle: the tide has no degree-0 or degree-1 part: tides are taken relative to the centre of mass, "
                 "degree 2 and up");
        return SL3DGPU_ERR_ARGUMENT;
      }
  }

  // The static (load-independent) coefficient terms.
  su->anyStatic = su->hasDisp || su->hasPot || hasTide || hasLayer || su->hasLoadChannel;
  su->anyStaticTan = su->hasDisp || su->hasPot || su->hasTan || hasTide || su->hasLoadChannel;
  double displacementLoad0 = 0.0, potentialLoad0 = 0.0;
  Dev<double>&staticDisp = ws.staticDisp, &staticGrav = ws.staticGrav, &staticTan = ws.staticTan,
             &staticSlc = ws.staticSlc, &scratch = ws.scratch;
  const std::vector<double> zeros(L + 1, 0.0);
  if (su->anyStatic || su->anyStaticTan) {
    for (auto* d : {&staticDisp, &staticGrav, &staticTan, &staticSlc, &scratch})
      SL3D_CUDA(cudaMemsetAsync(d->p, 0, nc * sizeof(double), s));
    if (su->hasDisp) SL3D_TRY(run.Axpy(staticDisp.p, forcing->displacement_response, 1.0, staticDisp.p));
    if (su->hasPot) SL3D_TRY(run.Axpy(staticGrav.p, forcing->potential_response, 1.0, staticGrav.p));
    if (su->hasTan) SL3D_TRY(run.Axpy(staticTan.p, forcing->tangential_response, 1.0, staticTan.p));
    if (hasTide) {
      // the body's answer to the prescribed potential (:533-545)
      std::vector<double> ht(body->ht, body->ht + L + 1), kt(body->kt, body->kt + L + 1), lt(L + 1, 0.0);
      if (body->lt != nullptr)
        for (int l = 1; l <= L; ++l) lt[l] = body->lt[l];
      ht[0] = kt[0] = 0.0;
      SL3D_TRY(run.ScaleDegrees(ht.data(), forcing->tide, staticDisp.p, 1.0, staticDisp.p));
      SL3D_TRY(run.ScaleDegrees(kt.data(), forcing->tide, staticGrav.p, 1.0, staticGrav.p));
      SL3D_TRY(run.ScaleDegrees(lt.data(), forcing->tide, staticTan.p, 1.0, staticTan.p));
    }
    // the load channels through their own numbers (:453-502): D_s += h_c L,
    // G_s += k_c L, T_s += l_c L with L the channel's expansion; a traction
    // from degree 1, the l's without degree 0
    auto channel = [&](const double* field, const double* hc, const double* kc, const double* lc, int first,
                       double* degree0) -> int {
      SL3D_TRY(sl3dgpu_expand_batch(grid, field, 1, scratch.p, s));
      std::vector<double> hf(L + 1, 0.0), kf(L + 1, 0.0), lf(L + 1, 0.0);
      for (int l = first; l <= L; ++l) {
        hf[l] = hc[l];
        kf[l] = kc[l];
        if (lc != nullptr && l >= 1) lf[l] = lc[l];
      }
      SL3D_TRY(run.ScaleDegrees(hf.data(), scratch.p, staticDisp.p, 1.0, staticDisp.p));
      SL3D_TRY(run.ScaleDegrees(kf.data(), scratch.p, staticGrav.p, 1.0, staticGrav.p));
      SL3D_TRY(run.ScaleDegrees(lf.data(), scratch.p, staticTan.p, 1.0, staticTan.p));
      if (degree0 != nullptr) {
        SL3D_CUDA(cudaMemcpyAsync(degree0, scratch.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        SL3D_CUDA(cudaStreamSynchronize(s));
      }
      return SL3DGPU_OK;
    };
    if (hasDispLoad)
      SL3D_TRY(channel(forcing->displacement_load, body->h_u, body->k_u, body->l_u, 0, &displacementLoad0));
    if (hasPotLoad)
      SL3D_TRY(channel(forcing->potential_load, body->h_phi, body->k_phi, body->l_phi, 0, &potentialLoad0));
    if (hasTraction) SL3D_TRY(channel(forcing->tangential_traction, body->h_v, body->k_v, body->l_v, 1, nullptr));
    // S_s = -(D_s + G_s / g) - T / g - Expand(layer) (:590-600)
    SL3D_TRY(run.Axpy(staticDisp.p, staticGrav.p, 1.0 / g, staticSlc.p));
    SL3D_TRY(run.ScaleDegrees(zeros.data(), staticSlc.p, staticSlc.p, -1.0, staticSlc.p));
    if (hasTide) SL3D_TRY(run.Axpy(staticSlc.p, forcing->tide, -1.0 / g, staticSlc.p));
    if (hasLayer) {
      SL3D_TRY(sl3dgpu_expand_batch(grid, forcing->solid_surface_change, 1, scratch.p, s));
      SL3D_TRY(run.Axpy(staticSlc.p, scratch.p, -1.0, staticSlc.p));
    }
  }

  // The rotational feedback's fixed blocks (src/SeaLevel.cpp:604-608), read
  // back once, and the rotation's inputs on the device, so that each
  // iteration's patch needs no host round trip.
  RotationFactors rf;
  rf.Init(*body);
  su->rotating = rf.on;
  if (rf.on) {
    Block2 staticDisp2{}, staticGrav2{}, tide2{}, layer2{};
    auto headOf = [&](const double* coeffs, double* head) -> int {  // coefficients 0 .. 4 as (re, im)
      SL3D_CUDA(cudaMemcpyAsync(head, coeffs, 10 * sizeof(double), cudaMemcpyDeviceToHost, s));
      SL3D_CUDA(cudaStreamSynchronize(s));
      return SL3DGPU_OK;
    };
    double head[10];
    if (su->anyStatic || su->anyStaticTan) {
      SL3D_TRY(headOf(staticDisp.p, head));
      staticDisp2 = BlockOf(head + 6, head + 8);
      SL3D_TRY(headOf(staticGrav.p, head));
      staticGrav2 = BlockOf(head + 6, head + 8);
    }
    if (hasTide) {
      SL3D_TRY(headOf(forcing->tide, head));
      tide2 = BlockOf(head + 6, head + 8);
    }
    if (hasLayer) {
      SL3D_TRY(headOf(scratch.p, head));  // the layer's expansion
      layer2 = BlockOf(head + 6, head + 8);
    }
    RotationInputs in{};
    in.transverse = rf.transverse ? 1 : 0;
    in.h2 = rf.h2;
    in.k2 = rf.k2;
    in.ht2 = rf.ht2;
    in.kt2 = rf.kt2;
    in.hc = rf.hc;
    in.kc = rf.kc;
    in.mu = rf.mu;
    in.mphi = rf.mphi;
    in.mc = rf.mc;
    in.g = g;
    in.lt2 = body->lt != nullptr ? body->lt[2] : 0.0;
    in.rotation = rf.rotation;
    in.inertia = rf.inertia;
    in.axialRotation = rf.axialRotation;
    in.uniformRotation = rf.uniformRotation;
    in.axialInertia = rf.axialInertia;
    in.inverseInertiaDifference = rf.inverseInertiaDifference;
    in.inversePolarInertia = rf.inversePolarInertia;
    in.trace = rf.trace;
    in.shell = rf.shell;
    in.rotationDenominator = rf.rotationDenominator;
    in.axialRotationDenominator = rf.axialRotationDenominator;
    auto flat = [](const Block2& b, double* out) {
      out[0] = b[0][0];
      out[1] = b[0][1];
      out[2] = b[1][0];
      out[3] = b[1][1];
    };
    flat(staticDisp2, in.staticDisp2);
    flat(staticGrav2, in.staticGrav2);
    flat(tide2, in.tide2);
    flat(layer2, in.layer2);
    in.displacementLoad0 = displacementLoad0;
    in.potentialLoad0 = potentialLoad0;
    in.inertiaMoment = forcing->inertia_moment_change;
    for (int i = 0; i < 3; ++i) in.angularMomentum[i] = forcing->angular_momentum_change[i];
    SL3D_CUDA(cudaMemcpyAsync(ws.rotation.p, &in, sizeof(in), cudaMemcpyHostToDevice, s));
  }
  SL3D_CUDA(cudaMemsetAsync(ws.omega.p, 0, 3 * sizeof(double), s));
  SL3D_CUDA(cudaMemsetAsync(ws.shift.p, 0, sizeof(double), s));
  return SL3DGPU_OK;
}

// field = Synthesise(f_l L + add) of the run's load L (f on the device or the
// host), its degree-0/2 coefficients patched first by the rotation of L when
// `patch` (mode: RotationPatchKernel's).
int SynthesisePatched(SleWorkspace& ws, bool patch, const double* f, bool factorsOnDevice, const double* add,
                      double* field, int mode) {
  SleRun& run = ws.run;
  const cudaStream_t s = run.stream;
  if (factorsOnDevice) {
    ScaleDegreesKernel<<<static_cast<unsigned>((run.coefCount + 255) / 256), 256, 0, s>>>(
        run.lmax, f, reinterpret_cast<const double2*>(run.loadLm.p), reinterpret_cast<const double2*>(add), 1.0,
        reinterpret_cast<double2*>(run.scaledLm.p));
    SL3D_CHECK_LAUNCH();
  } else {
    SL3D_TRY(run.ScaleDegrees(f, run.loadLm.p, add, 1.0, run.scaledLm.p));
  }
  if (patch) {
    RotationPatchKernel<<<1, 32, 0, s>>>(ws.rotation.p, run.loadLm.p, run.scaledLm.p, ws.omega.p, mode);
    SL3D_CHECK_LAUNCH();
  }
  return sl3dgpu_synthesise_batch(run.grid, run.scaledLm.p, 1, field, s);
}

// -- the nonlinear solve's pointwise work (src/SeaLevel.cpp:1098-1217) ----------------------------------

// The changes of grounded ice and of ocean water per unit area from the
// state, at ocean function c and sea level change `change`
// (groundedIceChangeAt, waterChangeAt: :1100-1110).
struct Budget {
  double rhoI, rhoW;
  const double *dice, *ice0, *ocean0, *sea0;
  __device__ double Grounded(long long i, double c) const {
    const double di = dice ? dice[i] : 0.0;
    return rhoI * ((1.0 - c) * di - (c - ocean0[i]) * ice0[i]);
  }
  __device__ double Water(long long i, double c, double change) const {
    return rhoW * (c * change + (c - ocean0[i]) * sea0[i]);
  }
};

// out = grounded + water (+ direct): the total load (:1131-1136) and the
// carried one (:1277-1283)
__global__ void BudgetLoadKernel(long long n, Budget b, const double* ocean, const double* change, const double* direct,
                                 double* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  double v = b.Grounded(i, ocean[i]) + b.Water(i, ocean[i], change[i]);
  if (direct) v += direct[i];
  out[i] = v;
}

// Per ring, w_j sum_k of what the water holds before the shift
// (unbalanced, :1167-1171, with the local change plus the dynamic one) and of
// the ocean function: one block a ring, a fixed tree (the grid's Integrate).
__global__ void BudgetRingKernel(int nphi, const double* weights, Budget b, const double* ocean, const double* local,
                                 const double* dynamic, double* unbalancedPartial, double* oceanPartial) {
  __shared__ double red[2][kRingThreads];
  const int j = blockIdx.x;
  const long long base = static_cast<long long>(j) * nphi;
  double u = 0.0, c = 0.0;
  for (int k = threadIdx.x; k < nphi; k += blockDim.x) {
    const long long i = base + k;
    const double raw = dynamic ? local[i] + dynamic[i] : local[i];
    u += b.Grounded(i, ocean[i]) + b.Water(i, ocean[i], raw);
    c += ocean[i];
  }
  red[0][threadIdx.x] = u;
  red[1][threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if (threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    unbalancedPartial[j] = weights[j] * red[0][0];
    oceanPartial[j] = weights[j] * red[1][0];
  }
}

// The eustatic shift (:1172-1176): what the water must lose, over the
// current ocean's water mass per unit height; the rings in order.
__global__ void BudgetShiftKernel(const double* unbalancedPartial, const double* oceanPartial, int ntheta, double scale,
                                  double rhoW, double directMass, double* shift) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double su = 0.0, sc = 0.0;
  for (int j = 0; j < ntheta; ++j) {
    su += unbalancedPartial[j];
    sc += oceanPartial[j];
  }
  const double oceanDensityArea = rhoW * (scale * sc);
  shift[0] = -(scale * su + directMass) / oceanDensityArea;
}

// The iterate's update (:1178-1217): the shifted sea level changes, the
// ocean function by flotation (not where land is held), and per block the
// largest |new - previous|, |previous|, |local| and |new| of the sea level
// change (blockIdx-ordered partials).
__global__ void BudgetUpdateKernel(long long n, const double* shiftPtr, Budget b, const double* local,
                                   const double* dynamic, const unsigned char* held, double* slc, double* change,
                                   double* ocean, double* maxima) {
  __shared__ double red[4][kRingThreads];
  const double shift = *shiftPtr;
  double m[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double raw = dynamic ? local[i] + dynamic[i] : local[i];
    const double newSlc = local[i] + shift, newChange = raw + shift;
    const double newIce = b.dice ? b.ice0[i] + b.dice[i] : b.ice0[i];
    const double newBathy = b.sea0[i] + newChange;
    const bool land = held != nullptr && held[i] != 0;
    const double previous = slc[i];
    m[0] = fmax(m[0], fabs(newSlc - previous));
    m[1] = fmax(m[1], fabs(previous));
    m[2] = fmax(m[2], fabs(local[i]));
    m[3] = fmax(m[3], fabs(newSlc));
    slc[i] = newSlc;
    change[i] = newChange;
    ocean[i] = !land && b.rhoW * newBathy - b.rhoI * newIce > 0.0 ? 1.0 : 0.0;
  }
  for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = m[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s /= 2) {
    if (threadIdx.x < s)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = fmax(red[q][threadIdx.x], red[q][threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) maxima[4 * blockIdx.x + q] = red[q][0];
}

// MakeState's ocean function (src/SeaLevel.cpp:279-300)
__global__ void FlotationKernel(long long n, double rhoW, double rhoI, const double* ice, const double* sea,
                                const unsigned char* held, double* ocean) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const bool floats = rhoW * sea[i] - rhoI * ice[i] > 0.0;
  const bool land = held != nullptr && held[i] != 0;
  ocean[i] = floats && !land ? 1.0 : 0.0;
}

}  // namespace

int SeaLevelSolve(SleWorkspace& ws, sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, const double* ocean,
                  const sl3dgpu_sle_forcing* forcing, double rtol, int max_iterations, int anderson_memory,
                  double* sea_level_change, double* displacement, double* potential, double* tangential_potential,
                  double* toroidal_potential, double* total_load, sl3dgpu_sle_result* result, cudaStream_t stream) {
  if (grid == nullptr || body == nullptr || body->h == nullptr || body->k == nullptr || ocean == nullptr ||
      forcing == nullptr || sea_level_change == nullptr || result == nullptr) {
    SetError("sle: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (!(rtol >= 0.0) || max_iterations < 0 || anderson_memory < 0 || anderson_memory > kMixMaxMemory) {
    SetError("sle: rtol >= 0, max_iterations >= 0, anderson_memory in [0, 16]");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SleSetup su;
  SL3D_TRY(PrepareSolve(ws, grid, body, forcing, stream, &su));
  SleRun& run = ws.run;
  const double water_density = body->water_density;
  const int blocks = static_cast<int>(std::min<long long>(kMaxBlocks, (run.fieldSize + 255) / 256));
  const cudaStream_t s = stream;
  const long long nc = 2 * run.coefCount;  // coefficients as reals
  auto zero = [&](double* f) -> int {
    if (f) SL3D_CUDA(cudaMemsetAsync(f, 0, run.fieldSize * sizeof(double), s));
    return SL3DGPU_OK;
  };
  *result = sl3dgpu_sle_result{0.0, 0.0, 0, 1, {0.0, 0.0, 0.0}};
  // the toroidal potential is carried, whatever else is solved (:561-563)
  if (toroidal_potential != nullptr) {
    if (forcing->toroidal_response != nullptr)
      SL3D_TRY(sl3dgpu_synthesise_batch(grid, forcing->toroidal_response, 1, toroidal_potential, s));
    else
      SL3D_TRY(zero(toroidal_potential));
  }
  const bool anyForcing = su.hasDirect || su.hasOutside || su.anyStatic || su.anyStaticTan;
  if (!anyForcing) {
    SL3D_TRY(zero(sea_level_change));
    SL3D_TRY(zero(displacement));
    SL3D_TRY(zero(potential));
    SL3D_TRY(zero(tangential_potential));
    if (total_load != nullptr) SL3D_CUDA(cudaMemsetAsync(total_load, 0, nc * sizeof(double), s));
    SL3D_CUDA(cudaStreamSynchronize(s));
    return SL3DGPU_OK;
  }
  const double* slcAdd = su.anyStatic ? ws.staticSlc.p : nullptr;

  double oceanArea = 0.0;
  SL3D_TRY(run.Integrate(ocean, nullptr, &oceanArea));
  const double perOceanArea = oceanArea > 0.0 ? 1.0 / oceanArea : 0.0;
  // the direct load in the water budget sets the mean; one outside it loads
  // the body and moves no water (:577-587)
  double meanSlc = 0.0;
  Dev<double>& directData = ws.directData;
  SL3D_CUDA(cudaMemsetAsync(directData.p, 0, run.fieldSize * sizeof(double), s));
  const unsigned fb = static_cast<unsigned>((run.fieldSize + 255) / 256);
  if (forcing->direct_load != nullptr) {
    double loadIntegral = 0.0;
    SL3D_TRY(run.Integrate(forcing->direct_load, nullptr, &loadIntegral));
    meanSlc = -loadIntegral * perOceanArea / water_density;
    SL3D_CUDA(cudaMemcpyAsync(directData.p, forcing->direct_load, run.fieldSize * sizeof(double),
                              cudaMemcpyDeviceToDevice, s));
  }
  if (forcing->direct_load_outside != nullptr) {
    AddFieldKernel<<<fb, 256, 0, s>>>(run.fieldSize, directData.p, forcing->direct_load_outside, directData.p);
    SL3D_CHECK_LAUNCH();
  }
  // the seed: sigma + rho_w C s_mean, expanded
  SeedKernel<<<fb, 256, 0, s>>>(run.fieldSize, directData.p, ocean, water_density * meanSlc, run.seeded.p);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(sl3dgpu_expand_batch(grid, run.seeded.p, 1, run.loadLm.p, s));

  SL3D_TRY(ws.ResetMixer(anderson_memory, s));
  LoadMixer& mixer = ws.mixer;
  double err = INFINITY;
  bool converged = false, havePrev = false;
  int count = 0;
  while (count < max_iterations) {
    // the sea level change of the load, its uniform part by conservation:
    // one host round trip an iteration, the stopping test's maxima
    SL3D_TRY(SynthesisePatched(ws, su.rotating, ws.slcFactor.p, true, slcAdd, run.slc.p, 0));
    RingSumKernel<<<run.ntheta, kRingThreads, 0, s>>>(run.nphi, run.weights.p, ocean, run.slc.p, run.ringPartial.p);
    SL3D_CHECK_LAUNCH();
    ShiftKernel<<<1, 32, 0, s>>>(run.ringPartial.p, run.ntheta, run.r2 * run.dphi, meanSlc, perOceanArea,
                                 ws.shift.p);
    SL3D_CHECK_LAUNCH();
    ShiftAndLoadKernel<<<blocks, kRingThreads, 0, s>>>(run.fieldSize, ws.shift.p, water_density, directData.p, ocean,
                                                       run.slc.p, run.oceanSlc.p, run.newLoad.p, havePrev,
                                                       run.maxima.p);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemcpyAsync(run.hostMaxima.data(), run.maxima.p, 2 * blocks * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    SL3D_CUDA(cudaStreamSynchronize(s));
    if (havePrev) {
      double diff = 0.0, scale = 0.0;
      for (int b = 0; b < blocks; ++b) {
        diff = std::max(diff, run.hostMaxima[2 * b]);
        scale = std::max(scale, run.hostMaxima[2 * b + 1]);
      }
      err = scale > 0.0 ? diff / scale : 0.0;
      if (err <= rtol) {
        converged = true;
        break;
      }
    }
    havePrev = true;
    SL3D_TRY(sl3dgpu_expand_batch(grid, run.newLoad.p, 1, run.newLoadLm.p, s));
    SL3D_TRY(mixer.Update(run.loadLm.p, run.newLoadLm.p, nc, s));
    ++count;
  }
  // the sea level change is the last one formed; the other fields from the
  // load it came from, with the static terms (:702-720)
  SL3D_CUDA(cudaMemcpyAsync(sea_level_change, run.slc.p, run.fieldSize * sizeof(double), cudaMemcpyDeviceToDevice,
                            s));
  const bool withStatic = su.anyStatic || su.anyStaticTan;
  if (displacement)
    SL3D_TRY(SynthesisePatched(ws, su.rotating, body->h, false, withStatic ? ws.staticDisp.p : nullptr, displacement,
                               1));
  if (potential)
    SL3D_TRY(SynthesisePatched(ws, su.rotating, body->k, false, withStatic ? ws.staticGrav.p : nullptr, potential, 2));
  if (tangential_potential)
    SL3D_TRY(SynthesisePatched(ws, su.rotating, su.tangential.data(), false, withStatic ? ws.staticTan.p : nullptr,
                               tangential_potential, 3));
  // TotalLoadCoefficients (src/Evolution3D.cpp:237-249): the direct loads and
  // the ocean's, rho_w C S of the last sea level change
  if (total_load != nullptr) SL3D_TRY(sl3dgpu_expand_batch(grid, run.newLoad.p, 1, total_load, s));
  double tail[4];
  SL3D_CUDA(cudaMemcpyAsync(tail, ws.shift.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  SL3D_CUDA(cudaMemcpyAsync(tail + 1, ws.omega.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  SL3D_CUDA(cudaStreamSynchronize(s));
  *result = sl3dgpu_sle_result{tail[0], err, count, converged ? 1 : 0, {tail[1], tail[2], tail[3]}};
  return SL3DGPU_OK;
}

// GRDSolver::SolveNonlinear (src/SeaLevel.cpp:970-1289): a plain fixed point
// from the state given, each iteration the total load of the current ocean
// function and sea level change expanded, its sea level change (the
// generalised solve's factors, static terms and rotation patch) synthesised,
// the water budget closed by a uniform shift over the current ocean, the
// ocean function re-derived by flotation. One host round trip an
// iteration: the stopping test's maxima.
int SeaLevelSolveNonlinear(SleWorkspace& ws, sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, double ice_density,
                           const sl3dgpu_sle_state* state, const sl3dgpu_sle_nonlinear_forcing* forcing, double rtol,
                           int max_iterations, double* sea_level_change, double* displacement, double* potential,
                           double* tangential_potential, double* toroidal_potential, double* final_sea_level,
                           double* final_ocean_function, double* load_coefficients, sl3dgpu_sle_result* result,
                           cudaStream_t stream) {
  if (grid == nullptr || body == nullptr || body->h == nullptr || body->k == nullptr || state == nullptr ||
      state->ice_thickness == nullptr || state->sea_level == nullptr || state->ocean_function == nullptr ||
      forcing == nullptr || result == nullptr) {
    SetError("sle: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (!(ice_density > 0.0) || !(rtol >= 0.0) || max_iterations < 0) {
    SetError("sle: ice_density > 0, rtol >= 0, max_iterations >= 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  // the channels the nonlinear solve shares with the generalised one
  sl3dgpu_sle_forcing shared{};
  shared.solid_surface_change = forcing->solid_surface_change;
  shared.displacement_response = forcing->displacement_response;
  shared.potential_response = forcing->potential_response;
  shared.tangential_response = forcing->tangential_response;
  shared.toroidal_response = forcing->toroidal_response;
  shared.tide = forcing->tide;
  shared.inertia_moment_change = forcing->inertia_moment_change;
  SleSetup su;
  SL3D_TRY(PrepareSolve(ws, grid, body, &shared, stream, &su));
  SL3D_TRY(ws.PrepareNonlinear());
  SleRun& run = ws.run;
  const cudaStream_t s = stream;
  const long long n = run.fieldSize, nc = 2 * run.coefCount;
  const size_t bytes = n * sizeof(double);
  const unsigned fb = static_cast<unsigned>((n + 255) / 256);
  const int blocks = static_cast<int>(std::min<long long>(kMaxBlocks / 2, (n + 255) / 256));
  double oceanArea = 0.0;
  SL3D_TRY(run.Integrate(state->ocean_function, nullptr, &oceanArea));
  if (!(oceanArea > 0.0)) {
    SetError("sle: the nonlinear sea level solve needs a state with an ocean: the shorelines of a body without one "
             "do not migrate");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const unsigned char* held = forcing->hold_land ? forcing->forced_land : state->forced_land;
  // the direct loads: the one inside the water budget takes its mass from
  // the ocean, the one outside it moves no water (:1085-1096)
  const double* direct = nullptr;
  double directMass = 0.0;
  if (forcing->direct_load != nullptr) {
    SL3D_TRY(run.Integrate(forcing->direct_load, nullptr, &directMass));
    SL3D_CUDA(cudaMemcpyAsync(ws.directData.p, forcing->direct_load, bytes, cudaMemcpyDeviceToDevice, s));
    direct = ws.directData.p;
  }
  if (forcing->direct_load_outside != nullptr) {
    if (direct == nullptr) SL3D_CUDA(cudaMemsetAsync(ws.directData.p, 0, bytes, s));
    AddFieldKernel<<<fb, 256, 0, s>>>(n, ws.directData.p, forcing->direct_load_outside, ws.directData.p);
    SL3D_CHECK_LAUNCH();
    direct = ws.directData.p;
  }
  const Budget budget{ice_density,           body->water_density, forcing->ice_thickness_change,
                      state->ice_thickness,  state->ocean_function, state->sea_level};
  const double* dynamic = forcing->dynamic_sea_level_change;
  const double* slcAdd = su.anyStatic ? ws.staticSlc.p : nullptr;
  SL3D_CUDA(cudaMemcpyAsync(ws.nlOcean.p, state->ocean_function, bytes, cudaMemcpyDeviceToDevice, s));
  SL3D_CUDA(cudaMemsetAsync(ws.nlChange.p, 0, bytes, s));
  SL3D_CUDA(cudaMemsetAsync(ws.nlSlc.p, 0, bytes, s));
  SL3D_CUDA(cudaMemsetAsync(run.loadLm.p, 0, nc * sizeof(double), s));
  *result = sl3dgpu_sle_result{0.0, INFINITY, 0, 0, {0.0, 0.0, 0.0}};
  double err = INFINITY;
  bool converged = false;
  int count = 0;
  while (count < max_iterations) {
    BudgetLoadKernel<<<fb, 256, 0, s>>>(n, budget, ws.nlOcean.p, ws.nlChange.p, direct, run.newLoad.p);
    SL3D_CHECK_LAUNCH();
    SL3D_TRY(sl3dgpu_expand_batch(grid, run.newLoad.p, 1, run.loadLm.p, s));
    SL3D_TRY(SynthesisePatched(ws, su.rotating, ws.slcFactor.p, true, slcAdd, ws.nlLocal.p, 0));
    BudgetRingKernel<<<run.ntheta, kRingThreads, 0, s>>>(run.nphi, run.weights.p, budget, ws.nlOcean.p,
                                                         ws.nlLocal.p, dynamic, ws.nlRingUnbalanced.p,
                                                         ws.nlRingOcean.p);
    SL3D_CHECK_LAUNCH();
    BudgetShiftKernel<<<1, 32, 0, s>>>(ws.nlRingUnbalanced.p, ws.nlRingOcean.p, run.ntheta, run.r2 * run.dphi,
                                       body->water_density, directMass, ws.shift.p);
    SL3D_CHECK_LAUNCH();
    BudgetUpdateKernel<<<blocks, kRingThreads, 0, s>>>(n, ws.shift.p, budget, ws.nlLocal.p, dynamic, held, ws.nlSlc.p,
                                                       ws.nlChange.p, ws.nlOcean.p, run.maxima.p);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemcpyAsync(run.hostMaxima.data(), run.maxima.p, 4 * blocks * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    SL3D_CUDA(cudaStreamSynchronize(s));
    double m[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < blocks; ++b)
      for (int q = 0; q < 4; ++q) m[q] = std::max(m[q], run.hostMaxima[4 * b + q]);
    // the change against the size of the change, before the shift as well
    // as after (:1196-1208)
    const double top = std::max(m[1], count > 0 ? m[2] : 0.0);
    err = top > 0.0 ? m[0] / top : (m[3] == 0.0 ? 0.0 : 1.0);
    ++count;
    if (err <= rtol) {
      converged = true;
      break;
    }
  }
  if (sea_level_change) SL3D_CUDA(cudaMemcpyAsync(sea_level_change, ws.nlSlc.p, bytes, cudaMemcpyDeviceToDevice, s));
  // the responses of the last load, with the static terms (:1221-1262)
  const bool withStatic = su.anyStatic || su.anyStaticTan;
  const bool patch = su.rotating && count > 0;
  if (displacement)
    SL3D_TRY(SynthesisePatched(ws, patch, body->h, false, withStatic ? ws.staticDisp.p : nullptr, displacement, 1));
  if (potential)
    SL3D_TRY(SynthesisePatched(ws, patch, body->k, false, withStatic ? ws.staticGrav.p : nullptr, potential, 2));
  if (tangential_potential)
    SL3D_TRY(SynthesisePatched(ws, patch, su.tangential.data(), false, withStatic ? ws.staticTan.p : nullptr,
                               tangential_potential, 3));
  if (toroidal_potential) {
    if (forcing->toroidal_response != nullptr)
      SL3D_TRY(sl3dgpu_synthesise_batch(grid, forcing->toroidal_response, 1, toroidal_potential, s));
    else
      SL3D_CUDA(cudaMemsetAsync(toroidal_potential, 0, bytes, s));
  }
  // the final state (:1264-1271) and the load it carries (:1276-1284)
  if (final_sea_level) {
    AddFieldKernel<<<fb, 256, 0, s>>>(n, state->sea_level, ws.nlChange.p, final_sea_level);
    SL3D_CHECK_LAUNCH();
  }
  if (final_ocean_function)
    SL3D_CUDA(cudaMemcpyAsync(final_ocean_function, ws.nlOcean.p, bytes, cudaMemcpyDeviceToDevice, s));
  if (load_coefficients) {
    BudgetLoadKernel<<<fb, 256, 0, s>>>(n, budget, ws.nlOcean.p, ws.nlChange.p, direct, run.newLoad.p);
    SL3D_CHECK_LAUNCH();
    SL3D_TRY(sl3dgpu_expand_batch(grid, run.newLoad.p, 1, load_coefficients, s));
  }
  double tail[4];
  SL3D_CUDA(cudaMemcpyAsync(tail, ws.shift.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  SL3D_CUDA(cudaMemcpyAsync(tail + 1, ws.omega.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  SL3D_CUDA(cudaStreamSynchronize(s));
  *result = sl3dgpu_sle_result{tail[0], err, count, converged ? 1 : 0, {tail[1], tail[2], tail[3]}};
  return SL3DGPU_OK;
}

int Flotation(long long n, double water_density, double ice_density, const double* ice, const double* sea_level,
              const unsigned char* forced_land, double* ocean_function, cudaStream_t stream) {
  if (n < 0 || ice == nullptr || sea_level == nullptr || ocean_function == nullptr || !(water_density > 0.0) ||
      !(ice_density > 0.0)) {
    SetError("sle: flotation needs the ice and sea level fields, the output and densities > 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (n == 0) return SL3DGPU_OK;
  FlotationKernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(n, water_density, ice_density, ice,
                                                                                sea_level, forced_land, ocean_function);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu

using namespace sl3dgpu;

extern "C" int sl3dgpu_sle_solve(sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, const double* ocean,
                                 const sl3dgpu_sle_forcing* forcing, double rtol, int max_iterations,
                                 int anderson_memory, double* sea_level_change, double* displacement,
                                 double* potential, double* tangential_potential, double* toroidal_potential,
                                 sl3dgpu_sle_result* result, void* stream) {
  SleWorkspace ws;
  return SeaLevelSolve(ws, grid, body, ocean, forcing, rtol, max_iterations, anderson_memory, sea_level_change,
                       displacement, potential, tangential_potential, toroidal_potential, nullptr, result,
                       AsStream(stream));
}

extern "C" int sl3dgpu_sle_solve_nonlinear(sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, double ice_density,
                                           const sl3dgpu_sle_state* state,
                                           const sl3dgpu_sle_nonlinear_forcing* forcing, double rtol,
                                           int max_iterations, double* sea_level_change, double* displacement,
                                           double* potential, double* tangential_potential,
                                           double* toroidal_potential, double* final_sea_level,
                                           double* final_ocean_function, double* load_coefficients,
                                           sl3dgpu_sle_result* result, void* stream) {
  SleWorkspace ws;
  return SeaLevelSolveNonlinear(ws, grid, body, ice_density, state, forcing, rtol, max_iterations, sea_level_change,
                                displacement, potential, tangential_potential, toroidal_potential, final_sea_level,
                                final_ocean_function, load_coefficients, result, AsStream(stream));
}

extern "C" int sl3dgpu_sle_flotation(long long n, double water_density, double ice_density, const double* ice,
                                     const double* sea_level, const unsigned char* forced_land,
                                     double* ocean_function, void* stream) {
  return Flotation(n, water_density, ice_density, ice, sea_level, forced_land, ocean_function, AsStream(stream));
}
