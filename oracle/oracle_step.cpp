// ORACLE — test infrastructure only (see oracle_core.cpp's header).
//
// A CPU FP64 restatement of the reference's 3D quasi-static step: the grid
// coupling and the within-step fixed point of Viscoelastic3D, on the Gauss
// memory points, one node block, the fixed-point solver (Picard, adaptive
// Anderson). It follows:
//  - include/sl3dpp/SpinComponents.hpp:53-145 (DeviatoricComponents,
//    ForceRowsFromComponents);
//  - src/GridCoupling.cpp:56-161 (memory nodes), 263-314 (Synthesise,
//    Analyse), 497-509 (Multiply), 595-689 (Scatter, Gather,
//    AddStrainOfSolution), 691-809 (SpheroidalForce, ToroidalForce);
//  - src/Viscoelastic3D.cpp:169-356 (itau sampling), 433-492 (StageState),
//    876-1073 (SolveForces, SolveElastic, AddUnitChannels), 1223-1424
//    (StartStep, Respond), 1758-1786 (StrainOf), 1636-1669 (RelativeChange),
//    1885-1974 (Finish, Converge), 1982-2030 (Step, Sdirk2 by recipe),
//    2032-2079 (Surface);
//  - include/sl3dpp/detail/AndersonMixer.hpp:65-219 (the mixer, its Gram
//    least squares by the SVD minimum-norm solve of oracle_lstsq.hpp in
//    place of LAPACK's dgelss);
//  - include/sl3dpp/StepRecipe.hpp, src/StepRecipe.cpp (Sdirk2's stages).
// The radial setup (mesh, material, rheology, degree systems) is the
// oracle's own (oracle_radial.cpp), independent of the library's GPU
// assembly; the factorisations, solves, transforms and every per-pass
// operation are restated here on the CPU.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <optional>
#include <vector>

#include <omp.h>

#include "../include/sl3dgpu.h"
#include "oracle_lstsq.hpp"
#include "oracle.h"
#include "oracle_radial.hpp"

// The ocean closure's callback (Evolution3D's Coupled::Closure,
// src/Evolution3D.cpp:296-339): given the stage's end time, the flavour's
// effective Love numbers (h, k, l, h_t, k_t, l_t per degree, then h_c, k_c,
// the load's inertia number and the centrifugal one), the surface U, V and
// phi of a pass's degree solves and their inertia moment, it writes the
// pass's load and tide channels ((l, m >= 0) complex coefficients).
extern "C" typedef void (*oracle_closure_fn)(void* user, double t, const double* love, int love_count,
                                            const double* u, const double* v, const double* phi, double inertia,
                                            double* sigma, double* psi);

namespace oracle {

using C = std::complex<double>;
using namespace orc;

// -- FFT (recursive mixed radix 2, 3, 5) --------------------------------------------------------

void FftRec(const C* in, int stride, C* out, int n, int sign) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  int p = 2;
  for (int f : {2, 3, 5})
    if (n % f == 0) {
      p = f;
      break;
    }
  const int m = n / p;
  for (int s = 0; s < p; ++s) FftRec(in + s * stride, stride * p, out + s * m, m, sign);
  std::vector<C> tmp(n);
  for (int k = 0; k < m; ++k)
    for (int q = 0; q < p; ++q) {
      C sum{};
      const int idx = k + q * m;
      for (int s = 0; s < p; ++s) {
        const double ang = sign * 2.0 * kPi * static_cast<double>((static_cast<long long>(s) * idx) % n) / n;
        sum += C(std::cos(ang), std::sin(ang)) * out[s * m + k];
      }
      tmp[idx] = sum;
    }
  std::copy(tmp.begin(), tmp.end(), out);
}

// -- the grid --------------------------------------------------------------------------------------

struct OGrid {
  int lmax = 0, ntheta = 0, nphi = 0;
  std::vector<double> theta, w;
  std::map<int, std::vector<std::vector<double>>> tables;

  OGrid(int lmax_, double oversampling) : lmax(lmax_) {
    const int band = static_cast<int>(std::ceil(oversampling * lmax - 1e-12));
    ntheta = band + 1;
    int n = 2 * band + 1;
    for (;; ++n) {
      int r = n;
      for (int p : {2, 3, 5})
        while (r % p == 0) r /= p;
      if (r == 1) break;
    }
    nphi = n;
    std::vector<double> x(ntheta);
    w.resize(ntheta);
    oracle_gauss_legendre(ntheta, x.data(), w.data());
    theta.resize(ntheta);
    for (int j = 0; j < ntheta; ++j) theta[j] = std::acos(x[j]);
    for (int N : {-2, -1, 0}) {
      auto& t = tables[N];
      t.resize(2 * lmax + 1);
      for (int m = -lmax; m <= lmax; ++m) {
        const int l0 = std::max(std::abs(m), std::abs(N));
        if (l0 > lmax) continue;
        t[m + lmax].resize(static_cast<std::size_t>(lmax - l0 + 1) * ntheta);
        oracle_wigner_column(lmax, N, m, ntheta, theta.data(), t[m + lmax].data());
      }
    }
  }
  std::size_t FieldSize() const { return static_cast<std::size_t>(ntheta) * nphi; }
  std::size_t SpinSize(int N) const { return static_cast<std::size_t>(lmax + 1) * (lmax + 1) - N * N; }
  std::size_t RealSize() const { return static_cast<std::size_t>(lmax + 1) * (lmax + 2) / 2; }
  static std::size_t SpinIndex(int N, int l, int m) { return static_cast<std::size_t>(l) * l - N * N + (m + l); }
  static std::size_t Index(int l, int m) { return static_cast<std::size_t>(l) * (l + 1) / 2 + m; }

  void SynthSpin(int N, const C* c, C* f) const {
    const auto& t = tables.at(N);
    std::vector<C> ring(nphi), out(nphi);
    for (int j = 0; j < ntheta; ++j) {
      std::fill(ring.begin(), ring.end(), C{});
      for (int m = -lmax; m <= lmax; ++m) {
        const int l0 = std::max(std::abs(m), std::abs(N));
        if (l0 > lmax) continue;
        const auto& col = t[m + lmax];
        C sum{};
        for (int l = l0; l <= lmax; ++l) sum += col[static_cast<std::size_t>(l - l0) * ntheta + j] * c[SpinIndex(N, l, m)];
        ring[((m % nphi) + nphi) % nphi] = sum;
      }
      FftRec(ring.data(), 1, out.data(), nphi, +1);
      std::copy(out.begin(), out.end(), f + static_cast<std::size_t>(j) * nphi);
    }
  }
  void ExpandSpin(int N, const C* f, C* c) const {
    const auto& t = tables.at(N);
    std::vector<C> G(static_cast<std::size_t>(2 * lmax + 1) * ntheta), out(nphi);
    for (int j = 0; j < ntheta; ++j) {
      FftRec(f + static_cast<std::size_t>(j) * nphi, 1, out.data(), nphi, -1);
      const double s = 2.0 * kPi / nphi * w[j];
      for (int m = -lmax; m <= lmax; ++m) G[static_cast<std::size_t>(m + lmax) * ntheta + j] = out[((m % nphi) + nphi) % nphi] * s;
    }
    for (int m = -lmax; m <= lmax; ++m) {
      const int l0 = std::max(std::abs(m), std::abs(N));
      if (l0 > lmax) continue;
      const auto& col = t[m + lmax];
      for (int l = l0; l <= lmax; ++l) {
        C sum{};
        for (int j = 0; j < ntheta; ++j) sum += col[static_cast<std::size_t>(l - l0) * ntheta + j] * G[static_cast<std::size_t>(m + lmax) * ntheta + j];
        c[SpinIndex(N, l, m)] = sum;
      }
    }
  }
  void SynthReal(const C* c, double* f) const {
    const auto& t = tables.at(0);
    std::vector<C> ring(nphi), out(nphi);
    for (int j = 0; j < ntheta; ++j) {
      std::fill(ring.begin(), ring.end(), C{});
      for (int m = 0; m <= lmax; ++m) {
        const auto& col = t[m + lmax];
        C sum{};
        for (int l = m; l <= lmax; ++l) sum += col[static_cast<std::size_t>(l - m) * ntheta + j] * c[Index(l, m)];
        if (m == 0) {
          ring[0] = C(sum.real(), 0.0);
        } else {
          ring[m] = sum;
          ring[nphi - m] = std::conj(sum);
        }
      }
      FftRec(ring.data(), 1, out.data(), nphi, +1);
      for (int k = 0; k < nphi; ++k) f[static_cast<std::size_t>(j) * nphi + k] = out[k].real();
    }
  }
  void ExpandReal(const double* f, C* c) const {
    const auto& t = tables.at(0);
    std::vector<C> G(static_cast<std::size_t>(lmax + 1) * ntheta), ring(nphi), out(nphi);
    for (int j = 0; j < ntheta; ++j) {
      for (int k = 0; k < nphi; ++k) ring[k] = C(f[static_cast<std::size_t>(j) * nphi + k], 0.0);
      FftRec(ring.data(), 1, out.data(), nphi, -1);
      const double s = 2.0 * kPi / nphi * w[j];
      for (int m = 0; m <= lmax; ++m) G[static_cast<std::size_t>(m) * ntheta + j] = out[m] * s;
    }
    for (int m = 0; m <= lmax; ++m) {
      const auto& col = t[m + lmax];
      for (int l = m; l <= lmax; ++l) {
        C sum{};
        for (int j = 0; j < ntheta; ++j) sum += col[static_cast<std::size_t>(l - m) * ntheta + j] * G[static_cast<std::size_t>(m) * ntheta + j];
        c[Index(l, m)] = sum;
      }
    }
  }
};

// -- spin components (SpinComponents.hpp:53-145) ------------------------------------------------

struct NodeValues {
  C U, V, W, rdU, rdV, rdW;
};

std::array<C, 5> DeviatoricComponents(int l, const NodeValues& v, double r) {
  const C i(0.0, 1.0);
  const double zeta2 = l * (l + 1.0), zeta = std::sqrt(zeta2);
  std::array<C, 5> A{};
  A[2] = (v.rdU - v.U + 0.5 * zeta2 * v.V) / (3.0 * r);
  if (l >= 1) {
    const C tangential = v.rdV - v.V + v.U;
    const C twist = v.W - v.rdW;
    A[1] = zeta * (tangential + i * twist) / (2.0 * std::sqrt(2.0) * r);
    A[3] = zeta * (tangential - i * twist) / (2.0 * std::sqrt(2.0) * r);
  }
  if (l >= 2) {
    const double factor = 0.5 * zeta * std::sqrt(zeta2 - 2.0) / r;
    A[0] = factor * (v.V - i * v.W);
    A[4] = factor * (v.V + i * v.W);
  }
  return A;
}

struct Rows {
  C u, v, w, du, dv, dw;
};

Rows ForceRows(int l, const std::array<C, 5>& A, double r) {
  const C i(0.0, 1.0);
  const double zeta2 = l * (l + 1.0), zeta = std::sqrt(zeta2);
  const double root = std::sqrt(std::max(zeta2 - 2.0, 0.0));
  const double s2 = std::sqrt(2.0);
  Rows rows;
  rows.u = s2 * zeta * (A[1] + A[3]) - 4.0 * A[2];
  rows.v = zeta * root * (A[0] + A[4]) + 2.0 * zeta2 * A[2] - s2 * zeta * (A[1] + A[3]);
  rows.w = i * (zeta * root * (A[0] - A[4]) - s2 * zeta * (A[1] - A[3]));
  rows.du = 4.0 * r * A[2];
  rows.dv = s2 * zeta * r * (A[1] + A[3]);
  rows.dw = i * s2 * zeta * r * (A[1] - A[3]);
  return rows;
}

// -- tensors ----------------------------------------------------------------------------------------

struct Spectral {
  std::vector<C> c0, c1, r;  // spin -2, spin -1 (full m), spin 0 (m >= 0); node-major
};
struct Tensor {
  std::vector<C> c0, c1;
  std::vector<double> r;
};

struct Factor {
  bool cholesky = true;
  int n = 0, kd = 0;
  std::vector<double> band;
  std::vector<int> pivots, pinned;
  std::vector<double> scale;
};

Factor FactorSpheroidal(const DegreeOperator& op) {
  Factor f;
  f.n = op.DofCount();
  f.kd = op.Bandwidth();
  f.scale = op.Scale();
  if (op.PositiveDiagonal()) {
    f.band = op.ScaledCholeskyBand();
    if (oracle_band_cholesky_factor(f.band.data(), f.n, f.kd) == 0) return f;
  }
  f.cholesky = false;
  f.band = op.ScaledLuBand();
  f.pivots.resize(f.n);
  if (oracle_band_lu_factor(f.band.data(), f.n, f.kd, f.kd, f.pivots.data()) != 0)
    throw std::runtime_error("the banded LU factorisation failed");
  return f;
}

Factor FactorToroidal(const ToroidalOperator& op) {
  Factor f;
  f.n = op.DofCount();
  f.kd = op.Bandwidth();
  f.scale = op.Scale();
  f.pinned = op.Pinned();
  f.band = op.ScaledCholeskyBand();
  if (oracle_band_cholesky_factor(f.band.data(), f.n, f.kd) != 0)
    throw std::runtime_error("toroidal Cholesky failed");
  return f;
}

// x with A x = b for complex columns (ndof x cols, column-major), as
// SolveForces' begin/finish: real and imaginary parts as real columns.
std::vector<C> SolveComplex(const Factor& f, const std::vector<C>& b, int cols) {
  const int n = f.n;
  std::vector<double> x(static_cast<std::size_t>(n) * 2 * cols);
  for (int c = 0; c < cols; ++c)
    for (int d = 0; d < n; ++d) {
      x[static_cast<std::size_t>(c) * n + d] = b[static_cast<std::size_t>(c) * n + d].real();
      x[static_cast<std::size_t>(cols + c) * n + d] = b[static_cast<std::size_t>(c) * n + d].imag();
    }
  for (int k = 0; k < 2 * cols; ++k) {
    for (int j = 0; j < n; ++j) x[static_cast<std::size_t>(k) * n + j] *= f.scale[j];
    for (int p : f.pinned) x[static_cast<std::size_t>(k) * n + p] = 0.0;
  }
  if (f.cholesky)
    oracle_band_cholesky_solve(f.band.data(), n, f.kd, x.data(), 2 * cols);
  else
    oracle_band_lu_solve(f.band.data(), n, f.kd, f.kd, f.pivots.data(), x.data(), 2 * cols);
  for (int k = 0; k < 2 * cols; ++k)
    for (int j = 0; j < n; ++j) x[static_cast<std::size_t>(k) * n + j] *= f.scale[j];
  std::vector<C> out(static_cast<std::size_t>(n) * cols);
  for (int c = 0; c < cols; ++c)
    for (int d = 0; d < n; ++d)
      out[static_cast<std::size_t>(c) * n + d] = C(x[static_cast<std::size_t>(c) * n + d], x[static_cast<std::size_t>(cols + c) * n + d]);
  return out;
}

struct Flavour {
  std::vector<std::unique_ptr<DegreeOperator>> sph;
  std::vector<std::unique_ptr<ToroidalOperator>> tor;
  std::vector<Factor> sphF, torF;
  std::vector<std::vector<double>> units;      // K^-1 Load per degree
  std::vector<std::vector<double>> tideUnits;  // K^-1 Tide per degree (degree 0 with power 2)
  PointShear shear;
};

struct Solutions {
  std::vector<std::vector<C>> sph, tor;  // per degree, (ndof x (l + 1)) column-major
};

struct State {
  double t = 0.0;
  std::vector<Tensor> m;
  std::optional<Tensor> strain;
  std::optional<Spectral> strainCoefficients;
};

struct Info {
  int iterations = 0;
  double residual = 0.0;
  bool converged = false;
  int mixedPasses = 0;
  int solveIterations = 0;
};

// -- the Anderson mixer (AndersonMixer.hpp:65-219) ----------------------------------------------

class Mixer {
 public:
  explicit Mixer(int memory) : memory_(memory) {}
  // x (in/out) and gx as flat real vectors.
  void Update(std::vector<double*> xs, std::vector<const double*> gs, std::vector<std::size_t> sizes) {
    std::size_t n = 0;
    for (auto s : sizes) n += s;
    auto sweep = [&](auto&& body) {
      std::size_t at = 0;
      for (std::size_t s = 0; s < xs.size(); ++s)
        for (std::size_t j = 0; j < sizes[s]; ++j, ++at) body(s, j, at);
    };
    if (xPrev_.empty()) {
      dG_.assign(memory_, std::vector<double>(n));
      dF_.assign(memory_, std::vector<double>(n));
      gram_.assign(static_cast<std::size_t>(memory_) * memory_, 0.0);
      xPrev_.resize(n);
      fPrev_.resize(n);
      sweep([&](std::size_t s, std::size_t j, std::size_t at) {
        xPrev_[at] = xs[s][j];
        fPrev_[at] = gs[s][j] - xs[s][j];
        xs[s][j] = gs[s][j];
      });
      return;
    }
    const int slot = slot_;
    const int m = std::min(count_ + 1, memory_);
    std::vector<double> column(m, 0.0), gamma(m, 0.0);
    sweep([&](std::size_t s, std::size_t j, std::size_t at) {
      const double f = gs[s][j] - xs[s][j];
      const double dx = xs[s][j] - xPrev_[at];
      dF_[slot][at] = f - fPrev_[at];
      dG_[slot][at] = dx + dF_[slot][at];
      xPrev_[at] = xs[s][j];
      fPrev_[at] = f;
      for (int i = 0; i < m; ++i) {
        column[i] += dF_[i][at] * dF_[slot][at];
        gamma[i] += dF_[i][at] * f;
      }
    });
    count_ = m;
    slot_ = (slot + 1) % memory_;
    for (int i = 0; i < m; ++i) {
      gram_[static_cast<std::size_t>(slot) * memory_ + i] = column[i];
      gram_[static_cast<std::size_t>(i) * memory_ + slot] = column[i];
    }
    std::vector<double> a(static_cast<std::size_t>(m) * m), g(m);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) a[static_cast<std::size_t>(i) * m + j] = gram_[static_cast<std::size_t>(i) * memory_ + j];
    if (!orc::SvdLstsq(m, a.data(), gamma.data(), g.data())) {
      sweep([&](std::size_t s, std::size_t j, std::size_t) { xs[s][j] = gs[s][j]; });
      return;
    }
    sweep([&](std::size_t s, std::size_t j, std::size_t at) {
      double value = gs[s][j];
      for (int i = 0; i < m; ++i) value -= g[i] * dG_[i][at];
      xs[s][j] = value;
    });
  }

 private:
  int memory_, count_ = 0, slot_ = 0;
  std::vector<double> xPrev_, fPrev_, gram_;
  std::vector<std::vector<double>> dG_, dF_;
};

// -- the 3D operator --------------------------------------------------------------------------------

struct Node {
  int element, q;
  double r;
};

class Viscoelastic3D {
 public:
  // staticPerturbation: ElasticPerturbation3D's coupling instead of the
  // step's (src/ElasticPerturbation3D.cpp:46-73): the GLL nodes of every
  // solid element above the one holding the centre, the unrelaxed material,
  // the elastic operators without point shear.
  Viscoelastic3D(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options& options,
                 bool staticPerturbation = false)
      : options_(options),
        static_(staticPerturbation),
        earth_(ToLayers(layers, nlayers), Scales::Geophysical(layers[nlayers - 1].r1)),
        mesh_(RadialMesh::Create(earth_, options.ngll)),
        material_(Material::Create(earth_, mesh_)),
        rheology_(Rheology::FromEarth(earth_, material_)),
        reference_(rheology_),
        grid_(options.lmax, options.oversampling),
        gll_(MemoryPoints::Of(false, mesh_)) {
    points_ = static_ ? &gll_ : &reference_.points;
    nodal_ = static_ ? &material_ : &reference_.nodal;
    const auto& mesh = nodal_->mesh;
    const int n = mesh.NGll();
    const auto& pts = *points_;
    for (int e = 0; e < mesh.ElementCount(); ++e) {
      bool carries = false;
      if (static_) {
        carries = !material_.IsFluid(e) && !(e == 0 && mesh.Left(0) == 0.0);
      } else {
        for (int i = 0; i < n; ++i) carries = carries || rheology_.IsActive(static_cast<std::size_t>(e) * n + i);
      }
      if (!carries) continue;
      for (int p = 0; p < pts.count; ++p) nodes_.push_back({e, p, pts.RadiusAt(mesh, e, p)});
    }
    const int L = options.lmax;
    firstNode_.resize(L + 1);
    for (int l = 0; l <= L; ++l) {
      const int fe = l > 0 ? mesh.StartElement(l, options.eps) : 0;
      int first = static_cast<int>(nodes_.size());
      for (std::size_t p = 0; p < nodes_.size(); ++p)
        if (nodes_[p].element >= fe) {
          first = static_cast<int>(p);
          break;
        }
      firstNode_[l] = first;
    }
    factor_.assign(static_cast<std::size_t>(NodeCount()) * grid_.FieldSize(), 1.0);
    // the elastic (unrelaxed) operators
    elastic_ = BuildFlavour(static_ ? nullptr : &reference_.elastic);
  }

  static std::vector<Layer> ToLayers(const sl3dgpu_layer* layers, int n) {
    std::vector<Layer> out(n);
    for (int i = 0; i < n; ++i) {
      const auto& s = layers[i];
      out[i] = Layer{s.r0, s.r1, s.fluid != 0, s.rho0, s.rho1, s.kappa0, s.kappa1, s.mu0, s.mu1,
                     s.viscosity, s.kelvin_fraction, s.kelvin_viscosity, s.elements};
    }
    return out;
  }

  int NodeCount() const { return static_cast<int>(nodes_.size()); }
  const OGrid& Grid() const { return grid_; }
  const std::vector<Node>& Nodes() const { return nodes_; }
  const Scales& ModelScales() const { return earth_.scales(); }
  double SurfaceRadius() const { return material_.radius; }
  double SurfaceGravity() const { return material_.surfaceGravity; }
  double GravitationalConstant() const { return material_.G; }
  int Lmax() const { return options_.lmax; }

  void SetDelta(const double* samples) {
    for (std::size_t i = 0; i < factor_.size(); ++i) factor_[i] = std::exp(-samples[i]);
  }

  State ZeroState() const {
    State s;
    for (std::size_t k = 0; k < rheology_.branches.size(); ++k) s.m.push_back(ZeroTensor());
    return s;
  }

  Tensor ZeroTensor() const {
    const auto size = static_cast<std::size_t>(NodeCount()) * grid_.FieldSize();
    return Tensor{std::vector<C>(size), std::vector<C>(size), std::vector<double>(size)};
  }
  Spectral ZeroSpectral() const {
    const auto P = static_cast<std::size_t>(NodeCount());
    return Spectral{std::vector<C>(P * grid_.SpinSize(-2)), std::vector<C>(P * grid_.SpinSize(-1)),
                    std::vector<C>(P * grid_.RealSize())};
  }

  // GridCoupling::Synthesise / Analyse
  void Synthesise(const Spectral& s, Tensor& t) const {
    const int P = NodeCount();
    const auto fs = grid_.FieldSize();
#pragma omp parallel for schedule(dynamic)
    for (int p = 0; p < P; ++p) {
      grid_.SynthSpin(-2, s.c0.data() + p * grid_.SpinSize(-2), t.c0.data() + p * fs);
      grid_.SynthSpin(-1, s.c1.data() + p * grid_.SpinSize(-1), t.c1.data() + p * fs);
      grid_.SynthReal(s.r.data() + p * grid_.RealSize(), t.r.data() + p * fs);
    }
  }
  void Analyse(const Tensor& t, Spectral& s) const {
    const int P = NodeCount();
    const auto fs = grid_.FieldSize();
#pragma omp parallel for schedule(dynamic)
    for (int p = 0; p < P; ++p) {
      grid_.ExpandSpin(-2, t.c0.data() + p * fs, s.c0.data() + p * grid_.SpinSize(-2));
      grid_.ExpandSpin(-1, t.c1.data() + p * fs, s.c1.data() + p * grid_.SpinSize(-1));
      grid_.ExpandReal(t.r.data() + p * fs, s.r.data() + p * grid_.RealSize());
    }
  }

  void Scatter(Spectral& s, int node, int l, int m, const std::array<C, 5>& A) const {
    const double sign = (m % 2 == 0) ? 1.0 : -1.0;
    const int spins[2] = {-2, -1};
    for (int c = 0; c < 2; ++c) {
      if (l < std::abs(spins[c])) continue;
      auto& block = c == 0 ? s.c0 : s.c1;
      C* b = block.data() + static_cast<std::size_t>(node) * grid_.SpinSize(spins[c]);
      b[OGrid::SpinIndex(spins[c], l, m)] += A[c];
      if (m > 0) b[OGrid::SpinIndex(spins[c], l, -m)] += sign * std::conj(A[4 - c]);
    }
    s.r[static_cast<std::size_t>(node) * grid_.RealSize() + OGrid::Index(l, m)] += A[2];
  }

  std::array<C, 5> Gather(const Spectral& s, int node, int l, int m) const {
    const double sign = (m % 2 == 0) ? 1.0 : -1.0;
    std::array<C, 5> A{};
    A[2] = s.r[static_cast<std::size_t>(node) * grid_.RealSize() + OGrid::Index(l, m)];
    if (l >= 1) {
      const C* b = s.c1.data() + static_cast<std::size_t>(node) * grid_.SpinSize(-1);
      A[1] = b[OGrid::SpinIndex(-1, l, m)];
      A[3] = sign * std::conj(b[OGrid::SpinIndex(-1, l, -m)]);
    }
    if (l >= 2) {
      const C* b = s.c0.data() + static_cast<std::size_t>(node) * grid_.SpinSize(-2);
      A[0] = b[OGrid::SpinIndex(-2, l, m)];
      A[4] = sign * std::conj(b[OGrid::SpinIndex(-2, l, -m)]);
    }
    return A;
  }

  // StrainOf: every degree's solution into a fresh spectral tensor.
  Spectral StrainOf(const Solutions& x, const Flavour& f) const {
    Spectral s = ZeroSpectral();
    const auto& mesh = nodal_->mesh;
    const auto& pts = *points_;
    const int n = mesh.NGll();
    const int L = options_.lmax;
#pragma omp parallel for schedule(dynamic)
    for (int l = L; l >= 0; --l) {
      const auto& sph = *f.sph[l];
      const ToroidalOperator* tor = l >= 1 ? f.tor[l].get() : nullptr;
      const int ndof = sph.DofCount();
      const auto& xs = x.sph[l];
      for (int node = firstNode_[l]; node < NodeCount(); ++node) {
        const int e = nodes_[node].element, q = nodes_[node].q;
        const double r = nodes_[node].r, jac = mesh.Jacobian(e);
        for (int m = 0; m <= l; ++m) {
          NodeValues v{};
          for (int i = 0; i < n; ++i) {
            const int g = mesh.GlobalIndex(e, i);
            const int dU = sph.Dof(g, kU), dV = sph.Dof(g, kV);
            const C U = dU >= 0 ? xs[static_cast<std::size_t>(m) * ndof + dU] : C{};
            const C V = dV >= 0 ? xs[static_cast<std::size_t>(m) * ndof + dV] : C{};
            C W{};
            if (tor != nullptr) {
              const int dW = tor->Dof(g);
              if (dW >= 0) W = x.tor[l][static_cast<std::size_t>(m) * tor->DofCount() + dW];
            }
            const double val = pts.Value(q, i);
            v.U += val * U;
            v.V += val * V;
            v.W += val * W;
            const double b = r * pts.Derivative(q, i) / jac;
            v.rdU += b * U;
            v.rdV += b * V;
            v.rdW += b * W;
          }
          Scatter(s, node, l, m, DeviatoricComponents(l, v, r));
        }
      }
    }
    return s;
  }

  // SpheroidalForce + ToroidalForce.
  void Forces(const Spectral& w, const Flavour& f, std::vector<std::vector<C>>& sph,
              std::vector<std::vector<C>>& tor) const {
    const auto& mesh = nodal_->mesh;
    const auto& pts = *points_;
    const int n = mesh.NGll();
    const int L = options_.lmax;
    sph.assign(L + 1, {});
    tor.assign(L + 1, {});
#pragma omp parallel for schedule(dynamic)
    for (int l = L; l >= 0; --l) {
      const auto& op = *f.sph[l];
      const ToroidalOperator* top = l >= 1 ? f.tor[l].get() : nullptr;
      const int cols = l + 1;
      std::vector<C> b(static_cast<std::size_t>(op.DofCount()) * cols);
      std::vector<C> bt(top ? static_cast<std::size_t>(top->DofCount()) * cols : 0);
      for (int node = firstNode_[l]; node < NodeCount(); ++node) {
        const int e = nodes_[node].element, q = nodes_[node].q;
        const double r = nodes_[node].r, jac = mesh.Jacobian(e);
        for (int m = 0; m < cols; ++m) {
          const auto rows = ForceRows(l, Gather(w, node, l, m), r);
          const double point = jac * pts.weight[q] * r;
          for (int i = 0; i < n; ++i) {
            const int g = mesh.GlobalIndex(e, i);
            const double v = point * pts.Value(q, i);
            const double deriv = pts.weight[q] * pts.Derivative(q, i) * r;
            const int iU = op.Dof(g, kU), iV = op.Dof(g, kV);
            if (iU >= 0) b[static_cast<std::size_t>(m) * op.DofCount() + iU] += v * rows.u;
            if (iV >= 0) b[static_cast<std::size_t>(m) * op.DofCount() + iV] += v * rows.v;
            if (iU >= 0) b[static_cast<std::size_t>(m) * op.DofCount() + iU] += deriv * rows.du;
            if (iV >= 0) b[static_cast<std::size_t>(m) * op.DofCount() + iV] += deriv * rows.dv;
            if (top != nullptr) {
              const int iW = top->Dof(g);
              if (iW >= 0) {
                bt[static_cast<std::size_t>(m) * top->DofCount() + iW] += v * rows.w;
                bt[static_cast<std::size_t>(m) * top->DofCount() + iW] += deriv * rows.dw;
              }
            }
          }
        }
      }
      sph[l] = std::move(b);
      tor[l] = std::move(bt);
    }
  }

  Solutions SolveForces(const std::vector<std::vector<C>>& sphF, const std::vector<std::vector<C>>& torF,
                        const Flavour& f) const {
    const int L = options_.lmax;
    Solutions x;
    x.sph.assign(L + 1, {});
    x.tor.assign(L + 1, {});
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < 2 * L + 1; ++t) {
      if (t <= L) {
        const int l = L - t;
        x.sph[l] = SolveComplex(f.sphF[l], sphF[l], l + 1);
      } else {
        const int l = 2 * L + 1 - t;
        x.tor[l] = SolveComplex(f.torF[l], torF[l], l + 1);
      }
    }
    return x;
  }

  Solutions SolveAll(const Spectral& analysed, const Flavour& f) const {
    std::vector<std::vector<C>> sph, tor;
    Forces(analysed, f, sph, tor);
    return SolveForces(sph, tor, f);
  }

  // x += sigma_lm K^-1 Load + tide_lm K^-1 Tide (AddUnitChannels,
  // Viscoelastic3D.cpp:1029-1073: the load column, then the tide's).
  void AddLoad(Solutions& x, const Flavour& f, const C* load, const C* tide = nullptr) const {
    for (int which = 0; which < 2; ++which) {
      const C* columns = which == 0 ? load : tide;
      if (columns == nullptr) continue;
      const auto& units = which == 0 ? f.units : f.tideUnits;
      for (int l = 0; l <= options_.lmax; ++l) {
        const int ndof = f.sph[l]->DofCount();
        for (int m = 0; m <= l; ++m) {
          const C a = columns[OGrid::Index(l, m)];
          if (a == C{}) continue;
          for (int d = 0; d < ndof; ++d) x.sph[l][static_cast<std::size_t>(m) * ndof + d] += a * units[l][d];
        }
      }
    }
  }
  // the running stage's tide at its start and end (null: none)
  const C* tideStart_ = nullptr;
  const C* tideEnd_ = nullptr;

  std::unique_ptr<Flavour> BuildFlavour(const PointShear* shear) const {
    auto f = std::make_unique<Flavour>();
    if (shear != nullptr) f->shear = *shear;
    const PointShear* use = shear != nullptr ? &f->shear : nullptr;
    const int L = options_.lmax;
    f->sph.resize(L + 1);
    f->tor.resize(L + 1);
    f->sphF.resize(L + 1);
    f->torF.resize(L + 1);
    f->units.resize(L + 1);
    f->tideUnits.resize(L + 1);
#pragma omp parallel for schedule(dynamic)
    for (int l = 0; l <= L; ++l) {
      f->sph[l] = std::make_unique<DegreeOperator>(*nodal_, l, options_.eps, use);
      f->sphF[l] = FactorSpheroidal(*f->sph[l]);
      const auto load = f->sph[l]->Load();
      std::vector<C> b(load.begin(), load.end());
      const auto x = SolveComplex(f->sphF[l], b, 1);
      f->units[l].resize(x.size());
      for (std::size_t i = 0; i < x.size(); ++i) f->units[l][i] = x[i].real();
      const auto tide = f->sph[l]->Tide(l == 0 ? 2 : -1);
      std::vector<C> bt(tide.begin(), tide.end());
      const auto xt = SolveComplex(f->sphF[l], bt, 1);
      f->tideUnits[l].resize(xt.size());
      for (std::size_t i = 0; i < xt.size(); ++i) f->tideUnits[l][i] = xt[i].real();
      if (l >= 1) {
        f->tor[l] = std::make_unique<ToroidalOperator>(*nodal_, l, options_.eps, use);
        f->torF[l] = FactorToroidal(*f->tor[l]);
      }
    }
    return f;
  }

  const Flavour& FlavourOf(Scheme scheme, double dt) {
    for (auto& [key, f] : flavours_)
      if (key.first == static_cast<int>(scheme) && key.second == dt) return *f;
    const auto shear = reference_.StepShear(scheme, dt);
    flavours_.emplace_back(std::make_pair(static_cast<int>(scheme), dt), BuildFlavour(&shear));
    return *flavours_.back().second;
  }

  static double RelativeChange(const Spectral& next, const Spectral& now) {
    double scale = 0.0, diff = 0.0;
    bool finite = true;
    for (int b = 0; b < 3; ++b) {
      const auto& nv = b == 0 ? next.c0 : b == 1 ? next.c1 : next.r;
      const auto& ov = b == 0 ? now.c0 : b == 1 ? now.c1 : now.r;
      for (std::size_t i = 0; i < nv.size(); ++i) {
        finite = finite && std::isfinite(nv[i].real()) && std::isfinite(nv[i].imag());
        scale = std::max(scale, std::norm(nv[i]));
        diff = std::max(diff, std::norm(nv[i] - ov[i]));
      }
    }
    if (!finite) return std::numeric_limits<double>::quiet_NaN();
    return scale > 0.0 ? std::sqrt(diff) / std::sqrt(scale) : 0.0;
  }

  // SolveElastic + StrainCoefficients: the start strain under the memory and
  // the load channel at the state's time, through the unrelaxed operators.
  Spectral ElasticStrainCoefficients(const State& state, const C* load) {
    Tensor combined = ZeroTensor();
    const auto fs = grid_.FieldSize();
    for (std::size_t k = 0; k < state.m.size(); ++k) {
      for (int node = 0; node < NodeCount(); ++node) {
        const double mu = MuBranch(k, node);
        if (mu == 0.0) continue;
        for (std::size_t i = node * fs; i < (node + 1) * fs; ++i) {
          combined.c0[i] += mu * state.m[k].c0[i];
          combined.c1[i] += mu * state.m[k].c1[i];
          combined.r[i] += mu * state.m[k].r[i];
        }
      }
    }
    Spectral weighted = ZeroSpectral();
    Analyse(combined, weighted);
    auto solutions = SolveAll(weighted, *elastic_);
    if (closure_ != nullptr) {
      Close(solutions, *elastic_, state.t);
      AddLoad(solutions, *elastic_, closureSigma_.data(), closurePsi_.data());
    } else {
      AddLoad(solutions, *elastic_, load, tideStart_);
    }
    return StrainOf(solutions, *elastic_);
  }

  // -- the ocean closure ---------------------------------------------------------------------------

  void SetClosure(oracle_closure_fn fn, void* user) {
    closure_ = fn;
    closureUser_ = user;
    closureSigma_.assign(grid_.RealSize(), C{});
    closurePsi_.assign(grid_.RealSize(), C{});
  }

  // sqrt(4 pi) sum w_q J_e rho r^3 x_U over degree 0's U dofs (the moment
  // of a degree-0 solution column x, its real part)
  template <class T>
  double MomentOf(const T* x) const {
    const auto& op = *elastic_->sph[0];
    const auto& mesh = nodal_->mesh;
    const int n = mesh.NGll();
    double sum = 0.0;
    for (int e = 0; e < mesh.ElementCount(); ++e)
      for (int q = 0; q < n; ++q) {
        const int dof = op.Dof(mesh.GlobalIndex(e, q), kU);
        if (dof < 0) continue;
        const double r = mesh.Radius(e, q);
        sum += mesh.Weights()[q] * mesh.Jacobian(e) * nodal_->rho[static_cast<std::size_t>(e) * n + q] * r * r * r *
               std::real(x[dof]);
      }
    return std::sqrt(4.0 * 3.14159265358979323846) * sum;
  }

  // ComputeLoveNumbers (src/LoveNumbers.cpp:92-176) on a flavour's solid,
  // from its unit channels: the surface U, phi and V of K^-1 Load and
  // K^-1 Tide per degree, degree 0's centrifugal column, and the moments.
  std::vector<double> EffectiveLove(const Flavour& f) const {
    const int L = options_.lmax;
    std::vector<double> out(6 * (L + 1) + 4, 0.0);
    auto value = [](const std::vector<double>& x, int dof) { return dof >= 0 ? x[dof] : 0.0; };
    for (int l = 0; l <= L; ++l) {
      const auto& op = *f.sph[l];
      const int iU = op.SurfaceDof(kU), iV = op.SurfaceDof(kV), iP = op.SurfaceDof(kPhi);
      out[l] = value(f.units[l], iU);
      out[(L + 1) + l] = value(f.units[l], iP);
      out[2 * (L + 1) + l] = l >= 1 ? value(f.units[l], iV) : 0.0;
      if (l >= 2) {
        out[3 * (L + 1) + l] = value(f.tideUnits[l], iU);
        out[4 * (L + 1) + l] = value(f.tideUnits[l], iP);
        out[5 * (L + 1) + l] = value(f.tideUnits[l], iV);
      }
    }
    const auto& op0 = *f.sph[0];
    out[6 * (L + 1)] = value(f.tideUnits[0], op0.SurfaceDof(kU));
    out[6 * (L + 1) + 1] = value(f.tideUnits[0], op0.SurfaceDof(kPhi));
    out[6 * (L + 1) + 2] = MomentOf(f.units[0].data());
    out[6 * (L + 1) + 3] = MomentOf(f.tideUnits[0].data());
    return out;
  }
  std::vector<double> EffectiveLoveOf(Scheme scheme, double dt) { return EffectiveLove(FlavourOf(scheme, dt)); }

  // One pass's closure: the responses' surface and moment to the callback,
  // its channels into closureSigma_ / closurePsi_.
  void Close(const Solutions& x, const Flavour& f, double t) {
    const auto love = EffectiveLove(f);
    const auto size = grid_.RealSize();
    std::vector<C> u(size), v(size), phi(size);
    SurfaceOf(x, 0, u.data());
    SurfaceOf(x, 1, v.data());
    SurfaceOf(x, 2, phi.data());
    const double inertia = x.sph.empty() ? 0.0 : MomentOf(x.sph[0].data());
    closure_(closureUser_, t, love.data(), static_cast<int>(love.size()), reinterpret_cast<const double*>(u.data()),
             reinterpret_cast<const double*>(v.data()), reinterpret_cast<const double*>(phi.data()), inertia,
             reinterpret_cast<double*>(closureSigma_.data()), reinterpret_cast<double*>(closurePsi_.data()));
  }
  oracle_closure_fn closure_ = nullptr;
  void* closureUser_ = nullptr;
  std::vector<C> closureSigma_, closurePsi_;

  double MuBranch(std::size_t k, int node) const {
    const auto& nd = nodes_[node];
    return reference_.pointMu[k][static_cast<std::size_t>(nd.element) * reference_.points.count + nd.q];
  }
  double ItauRef(std::size_t k, int node) const {
    const auto& nd = nodes_[node];
    return reference_.pointItau[k][static_cast<std::size_t>(nd.element) * reference_.points.count + nd.q];
  }

  // LateralPair (detail/LateralSolve.hpp:80-101): the m >= 0 columns of
  // every degree, m > 0 weighted twice, Re(a conj b) summed.
  static double Pair(const Solutions& a, const Solutions& b) {
    double total = 0.0;
    auto pair = [&](const std::vector<std::vector<C>>& x, const std::vector<std::vector<C>>& y) {
      for (std::size_t l = 0; l < x.size() && l < y.size(); ++l) {
        if (x[l].empty() || y[l].empty()) continue;
        const std::size_t ndof = x[l].size() / (l + 1);
        for (std::size_t m = 0; m <= l; ++m) {
          const double w = m == 0 ? 1.0 : 2.0;
          for (std::size_t d = 0; d < ndof; ++d)
            total += w * (x[l][m * ndof + d] * std::conj(y[l][m * ndof + d])).real();
        }
      }
    };
    pair(a.sph, b.sph);
    pair(a.tor, b.tor);
    return total;
  }

  // y = K x + keep y per degree (ApplyLateralOperator, Viscoelastic3D.cpp:
  // 626-728, keep -1; ElasticPerturbation3D::Apply, keep +1): the complex
  // columns as real pairs through the assembled bands.
  void AddKx(const Solutions& x, const Flavour& f, Solutions& y, double keep) const {
    const int L = options_.lmax;
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < 2 * L + 1; ++t) {
      const bool tor = t > L;
      const int l = tor ? t - L : t;
      const auto& xl = tor ? x.tor[l] : x.sph[l];
      auto& yl = tor ? y.tor[l] : y.sph[l];
      if (xl.empty()) continue;
      const int cols = l + 1;
      const int ndof = static_cast<int>(xl.size()) / cols;
      std::vector<double> real(static_cast<std::size_t>(ndof) * 2 * cols);
      for (int c = 0; c < cols; ++c)
        for (int d = 0; d < ndof; ++d) {
          real[static_cast<std::size_t>(c) * ndof + d] = xl[static_cast<std::size_t>(c) * ndof + d].real();
          real[static_cast<std::size_t>(cols + c) * ndof + d] = xl[static_cast<std::size_t>(c) * ndof + d].imag();
        }
      const auto k = tor ? ApplySymmetricBand(f.tor[l]->Band(), ndof, f.tor[l]->Bandwidth(), real, 2 * cols)
                         : ApplySymmetricBand(f.sph[l]->Band(), ndof, f.sph[l]->Bandwidth(), real, 2 * cols);
      for (int c = 0; c < cols; ++c)
        for (int d = 0; d < ndof; ++d) {
          const std::size_t at = static_cast<std::size_t>(c) * ndof + d;
          yl[at] = C(k[at], k[static_cast<std::size_t>(cols + c) * ndof + d]) + keep * yl[at];
        }
    }
  }

  static void Axpy(Solutions& y, double a, const Solutions& x) {
    for (int kind = 0; kind < 2; ++kind) {
      auto& Y = kind ? y.tor : y.sph;
      const auto& X = kind ? x.tor : x.sph;
      for (std::size_t l = 0; l < Y.size(); ++l)
        for (std::size_t i = 0; i < Y[l].size(); ++i) Y[l][i] += a * X[l][i];
    }
  }

  // The step closed by preconditioned conjugate gradients (Viscoelastic3D.cpp
  // :2008-2015 through OpenStep::Forces/Solve, LateralConjugateGradients at
  // detail/LateralSolve.hpp:112-181 with reduction 0 and no start): the
  // reference solve as the preconditioner, K x minus the lateral force as
  // the operator.
  Solutions ConjugateGradients(const Spectral& fixedS, const Flavour& flavour, const std::vector<double>& weight,
                               const C* load, bool lateral, Info& info) {
    const int L = options_.lmax;
    Solutions f;
    Forces(fixedS, flavour, f.sph, f.tor);
    for (int which = 0; which < 2; ++which) {
      const C* columns = which == 0 ? load : tideEnd_;
      if (columns == nullptr) continue;
      for (int l = 0; l <= L; ++l) {
        const auto vec = which == 0 ? flavour.sph[l]->Load() : flavour.sph[l]->Tide(l == 0 ? 2 : -1);
        const int ndof = flavour.sph[l]->DofCount();
        for (int m = 0; m <= l; ++m) {
          const C a = columns[OGrid::Index(l, m)];
          if (a == C{}) continue;
          for (int d = 0; d < ndof; ++d) f.sph[l][static_cast<std::size_t>(m) * ndof + d] += a * vec[d];
        }
      }
    }
    Tensor grid = ZeroTensor();
    Spectral analysed = ZeroSpectral();
    auto apply = [&](const Solutions& x) {
      Spectral e = StrainOf(x, flavour);
      Synthesise(e, grid);
      for (std::size_t i = 0; i < weight.size(); ++i) {
        grid.c0[i] *= weight[i];
        grid.c1[i] *= weight[i];
        grid.r[i] *= weight[i];
      }
      Analyse(grid, analysed);
      Solutions y;
      Forces(analysed, flavour, y.sph, y.tor);
      AddKx(x, flavour, y, -1.0);
      return y;
    };
    auto solve = [&](const Solutions& b) { return SolveForces(b.sph, b.tor, flavour); };
    return LateralCG(f, apply, solve, options_.solve_rtol, options_.solve_max_iterations, lateral, info);
  }

  // LateralConjugateGradients (detail/LateralSolve.hpp:112-181; no start,
  // reduction 0): from the reference response x = M^-1 f, the relative
  // residual in the preconditioned energy norm, one history entry per
  // iteration and the first.
  template <class Apply, class Solve>
  Solutions LateralCG(const Solutions& f, Apply&& apply, Solve&& solve, double rtol, int maxIterations, bool lateral,
                      Info& info) {
    Solutions x = solve(f);
    const double energy = Pair(x, f);
    auto relative = [&](double v) { return energy > 0.0 ? std::sqrt(std::abs(v) / energy) : std::sqrt(std::abs(v)); };
    info = Info{};
    if (!lateral) {
      info.converged = true;
      info.residual = 0.0;
      history_.push_back(0.0);
      return x;
    }
    Solutions r = apply(x);
    Axpy(r, -1.0, f);
    Axpy(r, -2.0, r);  // r = f - A x
    Solutions z = solve(r);
    double rz = Pair(z, r);
    info.residual = relative(rz);
    history_.push_back(info.residual);
    const double target = rtol;
    Solutions p = z;
    for (int iteration = 0; iteration < maxIterations; ++iteration) {
      if (info.residual <= target) break;
      const Solutions ap = apply(p);
      const double curvature = Pair(p, ap);
      const double alpha = rz / curvature;
      Axpy(x, alpha, p);
      Axpy(r, -alpha, ap);
      z = solve(r);
      const double next = Pair(z, r);
      const double beta = next / rz;
      rz = next;
      for (int kind = 0; kind < 2; ++kind) {
        auto& P = kind ? p.tor : p.sph;
        const auto& Z = kind ? z.tor : z.sph;
        for (std::size_t l = 0; l < P.size(); ++l)
          for (std::size_t i = 0; i < P[l].size(); ++i) P[l][i] = Z[l][i] + beta * P[l][i];
      }
      info.solveIterations = iteration + 1;
      info.residual = relative(rz);
      history_.push_back(info.residual);
    }
    info.converged = info.residual <= target;
    info.iterations = info.solveIterations;
    return x;
  }

  // -- the static perturbation problem (ElasticPerturbation3D) ---------------------------------

  void SetModuli(const double* dMu, const double* dKappa) {
    const std::size_t values = static_cast<std::size_t>(NodeCount()) * grid_.FieldSize();
    dMu_.assign(dMu ? dMu : nullptr, dMu ? dMu + values : nullptr);
    dKappa_.assign(dKappa ? dKappa : nullptr, dKappa ? dKappa + values : nullptr);
  }

  // AddDilatationOfSolution (src/GridCoupling.cpp:359-398): per node the
  // real spin-0 coefficients r dU/dr + 2 U - l(l+1) V.
  std::vector<C> DilatationOf(const Solutions& x) const {
    const auto& mesh = nodal_->mesh;
    const auto& pts = *points_;
    const int n = mesh.NGll(), L = options_.lmax;
    std::vector<C> scalar(static_cast<std::size_t>(NodeCount()) * grid_.RealSize());
#pragma omp parallel for schedule(dynamic)
    for (int l = L; l >= 0; --l) {
      const auto& op = *elastic_->sph[l];
      const int ndof = op.DofCount();
      const double k2 = l * (l + 1.0);
      for (int node = firstNode_[l]; node < NodeCount(); ++node) {
        const int e = nodes_[node].element, q = nodes_[node].q;
        const double r = nodes_[node].r, jac = mesh.Jacobian(e);
        for (int m = 0; m <= l; ++m) {
          C U{}, V{}, rdU{};
          for (int i = 0; i < n; ++i) {
            const int g = mesh.GlobalIndex(e, i);
            const int dU = op.Dof(g, kU), dV = op.Dof(g, kV);
            const C Ui = dU >= 0 ? x.sph[l][static_cast<std::size_t>(m) * ndof + dU] : C{};
            const C Vi = dV >= 0 ? x.sph[l][static_cast<std::size_t>(m) * ndof + dV] : C{};
            U += pts.Value(q, i) * Ui;
            V += pts.Value(q, i) * Vi;
            rdU += r * pts.Derivative(q, i) / jac * Ui;
          }
          scalar[static_cast<std::size_t>(node) * grid_.RealSize() + OGrid::Index(l, m)] = rdU + 2.0 * U - k2 * V;
        }
      }
    }
    return scalar;
  }

  // DilatationForce (src/GridCoupling.cpp:433-495), added onto sph.
  void AddDilatationForce(const std::vector<C>& weighted, std::vector<std::vector<C>>& sph) const {
    const auto& mesh = nodal_->mesh;
    const auto& pts = *points_;
    const int n = mesh.NGll(), L = options_.lmax;
#pragma omp parallel for schedule(dynamic)
    for (int l = L; l >= 0; --l) {
      const auto& op = *elastic_->sph[l];
      const int ndof = op.DofCount();
      const double k2 = l * (l + 1.0);
      auto& b = sph[l];
      for (int node = firstNode_[l]; node < NodeCount(); ++node) {
        const int e = nodes_[node].element, q = nodes_[node].q;
        const double r = nodes_[node].r, jac = mesh.Jacobian(e);
        for (int m = 0; m <= l; ++m) {
          const C D = weighted[static_cast<std::size_t>(node) * grid_.RealSize() + OGrid::Index(l, m)];
          const double point = jac * pts.weight[q];
          for (int i = 0; i < n; ++i) {
            const int g = mesh.GlobalIndex(e, i);
            const int iU = op.Dof(g, kU), iV = op.Dof(g, kV);
            const double v = point * pts.Value(q, i);
            if (iU >= 0) b[static_cast<std::size_t>(m) * ndof + iU] += 2.0 * v * D;
            if (iV >= 0) b[static_cast<std::size_t>(m) * ndof + iV] -= k2 * v * D;
          }
          for (int j = 0; j < n; ++j) {
            const int jU = op.Dof(mesh.GlobalIndex(e, j), kU);
            if (jU >= 0) b[static_cast<std::size_t>(m) * ndof + jU] += pts.weight[q] * pts.Derivative(q, j) * r * D;
          }
        }
      }
    }
  }

  // (dK) x (ElasticPerturbation3D::Force, src/ElasticPerturbation3D.cpp:140-226).
  Solutions PerturbationForce(const Solutions& x) const {
    const int L = options_.lmax;
    Solutions out;
    out.sph.assign(L + 1, {});
    out.tor.assign(L + 1, {});
    for (int l = 0; l <= L; ++l) {
      out.sph[l].assign(static_cast<std::size_t>(elastic_->sph[l]->DofCount()) * (l + 1), C{});
      if (l >= 1) out.tor[l].assign(static_cast<std::size_t>(elastic_->tor[l]->DofCount()) * (l + 1), C{});
    }
    if (!dMu_.empty()) {
      Spectral e = StrainOf(x, *elastic_);
      Tensor grid = ZeroTensor();
      Synthesise(e, grid);
      for (std::size_t i = 0; i < dMu_.size(); ++i) {
        grid.c0[i] *= dMu_[i];
        grid.c1[i] *= dMu_[i];
        grid.r[i] *= dMu_[i];
      }
      Spectral weighted = ZeroSpectral();
      Analyse(grid, weighted);
      std::vector<std::vector<C>> fs, ft;
      Forces(weighted, *elastic_, fs, ft);
      out.sph = std::move(fs);
      out.tor = std::move(ft);
    }
    if (!dKappa_.empty()) {
      auto scalar = DilatationOf(x);
      const auto fs = grid_.FieldSize();
      std::vector<double> field(static_cast<std::size_t>(NodeCount()) * fs);
#pragma omp parallel for schedule(dynamic)
      for (int p = 0; p < NodeCount(); ++p) {
        grid_.SynthReal(scalar.data() + static_cast<std::size_t>(p) * grid_.RealSize(), field.data() + p * fs);
        for (std::size_t i = p * fs; i < (p + 1) * fs; ++i) field[i] *= dKappa_[i];
        grid_.ExpandReal(field.data() + p * fs, scalar.data() + static_cast<std::size_t>(p) * grid_.RealSize());
      }
      AddDilatationForce(scalar, out.sph);
    }
    return out;
  }

  // SolveLoad (:98-126): the unit load responses times the coefficients.
  void SolveLoad(const C* load) {
    const int L = options_.lmax;
    Solutions x;
    x.sph.assign(L + 1, {});
    x.tor.assign(L + 1, {});
    for (int l = 0; l <= L; ++l) {
      const int ndof = elastic_->sph[l]->DofCount();
      x.sph[l].assign(static_cast<std::size_t>(ndof) * (l + 1), C{});
      if (l >= 1) x.tor[l].assign(static_cast<std::size_t>(elastic_->tor[l]->DofCount()) * (l + 1), C{});
      for (int m = 0; m <= l; ++m)
        for (int d = 0; d < ndof; ++d)
          x.sph[l][static_cast<std::size_t>(m) * ndof + d] = load[OGrid::Index(l, m)] * elastic_->units[l][d];
    }
    last_ = std::move(x);
  }

  // Respond (:474-479): -K^-1 (dK) x of the held solution.
  void Respond() {
    Solutions f = PerturbationForce(last_);
    Axpy(f, -2.0, f);
    last_ = SolveForces(f.sph, f.tor, *elastic_);
  }

  // SolveLateral for a load (:367-430): (K_ref + dK) x = LoadForces.
  void SolveLateral(const C* load, double rtol, int maxIterations, Info& info) {
    const int L = options_.lmax;
    history_.clear();
    Solutions f;
    f.sph.assign(L + 1, {});
    f.tor.assign(L + 1, {});
    for (int l = 0; l <= L; ++l) {
      const auto vec = elastic_->sph[l]->Load();
      const int ndof = elastic_->sph[l]->DofCount();
      f.sph[l].assign(static_cast<std::size_t>(ndof) * (l + 1), C{});
      if (l >= 1) f.tor[l].assign(static_cast<std::size_t>(elastic_->tor[l]->DofCount()) * (l + 1), C{});
      for (int m = 0; m <= l; ++m)
        for (int d = 0; d < ndof; ++d) f.sph[l][static_cast<std::size_t>(m) * ndof + d] = load[OGrid::Index(l, m)] * vec[d];
    }
    auto apply = [&](const Solutions& x) {
      Solutions y = PerturbationForce(x);
      AddKx(x, *elastic_, y, 1.0);
      return y;
    };
    auto solve = [&](const Solutions& b) { return SolveForces(b.sph, b.tor, *elastic_); };
    last_ = LateralCG(f, apply, solve, rtol, maxIterations, !(dMu_.empty() && dKappa_.empty()), info);
  }

  // One stage: StartStep, Converge(Respond + AddChannels + StrainOf), Finish.
  // With `samplePasses` >= 0: the bounded timing sample of a stage -- the
  // start (StartStep) and exactly that many passes, timed into tStart and
  // tPasses (seconds), the state returned unchanged.
  State StepOnce(const State& state, double dt, Scheme scheme, const C* loadStart, const C* loadEnd,
                 Info& info, Solutions& solutionsOut, int samplePasses = -1, double* tStart = nullptr,
                 double* tPasses = nullptr) {
    const double clock0 = omp_get_wtime();
    const auto& flavour = FlavourOf(scheme, dt);
    const auto fs = grid_.FieldSize();
    const std::size_t K = state.m.size();
    // The start strain.
    Spectral s0;
    if (state.strainCoefficients.has_value()) {
      s0 = *state.strainCoefficients;
    } else if (state.strain.has_value()) {
      s0 = ZeroSpectral();
      Analyse(*state.strain, s0);
    } else {
      s0 = ElasticStrainCoefficients(state, loadStart);
    }
    Tensor made;
    if (!state.strain.has_value()) {
      made = ZeroTensor();
      Synthesise(s0, made);
    }
    const Tensor& d0 = state.strain.has_value() ? *state.strain : made;
    // Weights, decayed memory, lateral weight and the fixed memory force.
    std::vector<Tensor> memory(K, ZeroTensor());
    std::vector<std::vector<double>> beta(K, std::vector<double>(d0.r.size()));
    std::vector<double> weight(d0.r.size(), 0.0);
    Tensor fixed = ZeroTensor();
    for (std::size_t k = 0; k < K; ++k) {
      for (int node = 0; node < NodeCount(); ++node) {
        const double itauRef = ItauRef(k, node);
        const double refBeta = scheme == Scheme::BackwardEuler ? 1.0 - BackwardEulerWeight(dt * itauRef)
                                                               : ExponentialTrapezoidWeights(dt * itauRef).beta;
        const double mu = MuBranch(k, node);
        for (std::size_t at = node * fs; at < (node + 1) * fs; ++at) {
          const double h = dt * (itauRef * factor_[at]);
          double e_w, a_w, b_w;
          if (scheme == Scheme::BackwardEuler) {
            const double wbe = BackwardEulerWeight(h);
            e_w = wbe;
            a_w = 0.0;
            b_w = 1.0 - wbe;
          } else {
            const auto tw = ExponentialTrapezoidWeights(h);
            e_w = tw.e;
            a_w = tw.alpha;
            b_w = tw.beta;
          }
          beta[k][at] = b_w;
          memory[k].c0[at] = e_w * state.m[k].c0[at] + a_w * d0.c0[at];
          memory[k].c1[at] = e_w * state.m[k].c1[at] + a_w * d0.c1[at];
          memory[k].r[at] = e_w * state.m[k].r[at] + a_w * d0.r[at];
          if (k == 0) {
            weight[at] = 0.0 + mu * (b_w - refBeta);
            fixed.c0[at] = C{} + mu * memory[k].c0[at];
            fixed.c1[at] = C{} + mu * memory[k].c1[at];
            fixed.r[at] = 0.0 + mu * memory[k].r[at];
            continue;
          }
          if (mu == 0.0) continue;
          weight[at] += mu * (b_w - refBeta);
          fixed.c0[at] += mu * memory[k].c0[at];
          fixed.c1[at] += mu * memory[k].c1[at];
          fixed.r[at] += mu * memory[k].r[at];
        }
      }
    }
    Spectral fixedS = ZeroSpectral();
    Analyse(fixed, fixedS);
    Spectral s;
    Solutions solutions;
    if (options_.solver == 1 && samplePasses < 0) {
      // the reference iterates whether or not the weight vanishes
      // (OpenStep::Solve passes lateral = true)
      solutions = ConjugateGradients(fixedS, flavour, weight, loadEnd, true, info);
      s = StrainOf(solutions, flavour);
    } else {
      s = s0;
    }
    // Respond: synthesise, weight, analyse, add the fixed force, solve.
    Tensor grid = ZeroTensor();
    Spectral analysed = ZeroSpectral();
    auto respond = [&](const Spectral& strain) {
      Synthesise(strain, grid);
      for (std::size_t i = 0; i < weight.size(); ++i) {
        grid.c0[i] *= weight[i];
        grid.c1[i] *= weight[i];
        grid.r[i] *= weight[i];
      }
      Analyse(grid, analysed);
      for (std::size_t i = 0; i < analysed.c0.size(); ++i) analysed.c0[i] += fixedS.c0[i];
      for (std::size_t i = 0; i < analysed.c1.size(); ++i) analysed.c1[i] += fixedS.c1[i];
      for (std::size_t i = 0; i < analysed.r.size(); ++i) analysed.r[i] += fixedS.r[i];
      return SolveAll(analysed, flavour);
    };
    // The load channel at the stage's end time.
    auto pass = [&](const Spectral& s) {
      solutions = respond(s);
      if (closure_ != nullptr) {
        Close(solutions, flavour, state.t + dt);
        AddLoad(solutions, flavour, closureSigma_.data(), closurePsi_.data());
      } else {
        AddLoad(solutions, flavour, loadEnd, tideEnd_);
      }
      return StrainOf(solutions, flavour);
    };
    if (samplePasses >= 0) {
      if (tStart) *tStart = omp_get_wtime() - clock0;
      Spectral it = s0;
      for (int k = 0; k < samplePasses; ++k) {
        const double clock1 = omp_get_wtime();
        Spectral next = pass(it);
        info.residual = RelativeChange(next, it);
        it = std::move(next);
        if (tPasses) tPasses[k] = omp_get_wtime() - clock1;  // each pass's seconds
      }
      solutionsOut = std::move(solutions);
      return state;
    }
    // Converge (Viscoelastic3D.cpp:1916-1974).
    if (options_.solver != 1) {
    info = Info{};
    const bool adaptive = options_.anderson_rate > 0.0;
    std::optional<Mixer> mixer;
    if (options_.anderson_memory > 0 && !adaptive) mixer.emplace(options_.anderson_memory);
    double previous = 0.0;
    for (int iteration = 0; iteration < options_.max_iterations; ++iteration) {
      Spectral next = pass(s);
      info.iterations = iteration + 1;
      info.residual = RelativeChange(next, s);
      history_.push_back(info.residual);
      if (!std::isfinite(info.residual)) break;
      if (info.residual <= options_.rtol) {
        info.converged = true;
        s = std::move(next);
        break;
      }
      if (options_.damping != 1.0) {
        auto damp = [&](std::vector<C>& nv, const std::vector<C>& ov) {
          for (std::size_t i = 0; i < nv.size(); ++i) nv[i] = ov[i] + options_.damping * (nv[i] - ov[i]);
        };
        damp(next.c0, s.c0);
        damp(next.c1, s.c1);
        damp(next.r, s.r);
      }
      if (adaptive && !mixer && options_.anderson_memory > 0 && iteration > 0 &&
          info.residual > options_.anderson_rate * previous)
        mixer.emplace(options_.anderson_memory);
      previous = info.residual;
      if (mixer) {
        mixer->Update({reinterpret_cast<double*>(s.c0.data()), reinterpret_cast<double*>(s.c1.data()),
                       reinterpret_cast<double*>(s.r.data())},
                      {reinterpret_cast<const double*>(next.c0.data()), reinterpret_cast<const double*>(next.c1.data()),
                       reinterpret_cast<const double*>(next.r.data())},
                      {2 * s.c0.size(), 2 * s.c1.size(), 2 * s.r.size()});
        ++info.mixedPasses;
      } else {
        s = std::move(next);
      }
    }
    }
    // Finish: synthesise the strain and advance the memory.
    State out;
    out.t = state.t + dt;
    Tensor d = ZeroTensor();
    Synthesise(s, d);
    for (std::size_t k = 0; k < K; ++k) {
      auto& mk = memory[k];
      for (std::size_t i = 0; i < mk.r.size(); ++i) {
        mk.c0[i] += beta[k][i] * d.c0[i];
        mk.c1[i] += beta[k][i] * d.c1[i];
        mk.r[i] += beta[k][i] * d.r[i];
      }
      out.m.push_back(std::move(mk));
    }
    out.strain = std::move(d);
    out.strainCoefficients = std::move(s);
    solutionsOut = std::move(solutions);
    return out;
  }

  // Step (Viscoelastic3D.cpp:1982-2030): one stage, or Sdirk2's two backward
  // Euler stages of gamma dt, the second from (1 - r) m_n + r Y_1.
  State Step(const State& state, double dt, Scheme scheme, const C* load0, const C* load1, Info& info,
             const C* tide0 = nullptr, const C* tide1 = nullptr) {
    history_.clear();
    struct Reset {
      Viscoelastic3D* self;
      ~Reset() { self->tideStart_ = self->tideEnd_ = nullptr; }
    } reset{this};
    tideStart_ = tide0;
    tideEnd_ = tide1;
    if (scheme != Scheme::Sdirk2 || dt == 0.0) {
      const Scheme one = scheme == Scheme::Sdirk2 ? Scheme::BackwardEuler : scheme;
      return StepOnce(state, dt, one, load0, load1, info, last_);
    }
    const double gamma = kSdirk2Gamma;
    const double h = gamma * dt;
    const auto size = grid_.RealSize();
    std::vector<C> loadMid;
    const C* mid = nullptr;
    if (load0 != nullptr || load1 != nullptr) {
      loadMid.assign(size, C{});
      for (std::size_t i = 0; i < size; ++i)
        loadMid[i] = (1.0 - gamma) * (load0 ? load0[i] : C{}) + gamma * (load1 ? load1[i] : C{});
      mid = loadMid.data();
    }
    std::vector<C> tideMid;
    const C* tmid = nullptr;
    if (tide0 != nullptr || tide1 != nullptr) {
      tideMid.assign(size, C{});
      for (std::size_t i = 0; i < size; ++i)
        tideMid[i] = (1.0 - gamma) * (tide0 ? tide0[i] : C{}) + gamma * (tide1 ? tide1[i] : C{});
      tmid = tideMid.data();
    }
    tideEnd_ = tmid;
    Info i1, i2;
    State y1 = StepOnce(state, h, Scheme::BackwardEuler, load0, mid, i1, last_);
    const double r = (1.0 - gamma) / gamma;
    State from;
    from.t = state.t + (1.0 - gamma) * dt;
    for (std::size_t k = 0; k < state.m.size(); ++k) {
      Tensor t = ZeroTensor();
      for (std::size_t i = 0; i < t.r.size(); ++i) {
        t.c0[i] = C{} + (1.0 - r) * state.m[k].c0[i];
        t.c0[i] += r * y1.m[k].c0[i];
        t.c1[i] = C{} + (1.0 - r) * state.m[k].c1[i];
        t.c1[i] += r * y1.m[k].c1[i];
        t.r[i] = 0.0 + (1.0 - r) * state.m[k].r[i];
        t.r[i] += r * y1.m[k].r[i];
      }
      from.m.push_back(std::move(t));
    }
    from.strain = y1.strain;
    from.strainCoefficients = y1.strainCoefficients;
    tideStart_ = tmid;
    tideEnd_ = tide1;
    State out = StepOnce(from, h, Scheme::BackwardEuler, mid, load1, i2, last_);
    out.t = state.t + dt;
    info.iterations = i1.iterations + i2.iterations;
    info.mixedPasses = i1.mixedPasses + i2.mixedPasses;
    info.solveIterations = i1.solveIterations + i2.solveIterations;
    info.residual = i2.residual;
    info.converged = i1.converged && i2.converged;
    return out;
  }

  // A stage's weights at h (ExponentialTrapezoidWeights or
  // BackwardEulerWeight) and their derivatives in h.
  static void StageWeightSlopes(Scheme sch, double h, double& e, double& a, double& b, double& de, double& da,
                                double& db) {
    if (sch == Scheme::BackwardEuler) {
      e = BackwardEulerWeight(h);
      a = 0.0;
      b = 1.0 - e;
      de = -e * e;
      da = 0.0;
      db = e * e;
      return;
    }
    const auto tw = ExponentialTrapezoidWeights(h);
    const double phi1 = tw.alpha + tw.e;
    const double dphi1 = std::abs(h) < 1e-3 ? -0.5 + h / 3.0 - h * h / 8.0 + h * h * h / 30.0 : (tw.e - phi1) / h;
    e = tw.e;
    a = tw.alpha;
    b = tw.beta;
    de = -tw.e;
    da = dphi1 + tw.e;
    db = -dphi1;
  }

  // The tangent-linear run beside the run from a zero state
  // (TangentLinearSolver3D's discrete run, src/TangentLinear3D.cpp): the
  // derivative of U and phi at every node along a log-viscosity direction p
  // (per grid sample, nullable) and load directions (nullable), stage by
  // stage beside the forward stage; each tangent solve is this step's own
  // iteration with the tangent's fixed force and load channel.
  void TangentRun(const double* times, int nodes, Scheme scheme, const C* loads, const double* p,
                  const C* loadDirections, C* uOut, C* phiOut) {
    const std::size_t lm = grid_.RealSize(), fs = grid_.FieldSize();
    State cur = ZeroState();
    cur.strain = ZeroTensor();
    const std::size_t K = cur.m.size();
    std::vector<Tensor> tm(K, ZeroTensor());
    Tensor td = ZeroTensor();
    const double gamma = kSdirk2Gamma, r = (1.0 - gamma) / gamma;
    // one tangent stage beside the forward stage in -> out
    auto stage = [&](const State& in, const State& out, double dt, Scheme sch, const C* loadDot) {
      const auto& f = FlavourOf(sch, dt);
      const Tensor start = in.strain.has_value() ? *in.strain : ZeroTensor();
      const Tensor& dEnd = *out.strain;
      std::vector<double> W(tm[0].r.size(), 0.0), hdot(W.size(), 0.0);
      Tensor fixed = ZeroTensor();
      std::vector<std::vector<double>> bdot(K, std::vector<double>(W.size())), beta(K, std::vector<double>(W.size()));
      for (std::size_t k = 0; k < K; ++k)
        for (int node = 0; node < NodeCount(); ++node) {
          const double itau = ItauRef(k, node), mu = MuBranch(k, node);
          double e0, a0, b0, de0, da0, db0;
          StageWeightSlopes(sch, dt * itau, e0, a0, b0, de0, da0, db0);
          for (std::size_t at = node * fs; at < (node + 1) * fs; ++at) {
            const double h = dt * (itau * factor_[at]), hd = -h * (p ? p[at] : 0.0);
            double e, a, b, de, da, db;
            StageWeightSlopes(sch, h, e, a, b, de, da, db);
            W[at] += mu * (b - b0);
            beta[k][at] = b;
            bdot[k][at] = db * hd;
            tm[k].c0[at] = e * tm[k].c0[at] + a * td.c0[at] + de * hd * in.m[k].c0[at] + da * hd * start.c0[at];
            tm[k].c1[at] = e * tm[k].c1[at] + a * td.c1[at] + de * hd * in.m[k].c1[at] + da * hd * start.c1[at];
            tm[k].r[at] = e * tm[k].r[at] + a * td.r[at] + de * hd * in.m[k].r[at] + da * hd * start.r[at];
            fixed.c0[at] += mu * tm[k].c0[at] + mu * db * hd * dEnd.c0[at];
            fixed.c1[at] += mu * tm[k].c1[at] + mu * db * hd * dEnd.c1[at];
            fixed.r[at] += mu * tm[k].r[at] + mu * db * hd * dEnd.r[at];
          }
        }
      Spectral fixedS = ZeroSpectral();
      Analyse(fixed, fixedS);
      Tensor g = ZeroTensor();
      Spectral analysed = ZeroSpectral();
      Solutions x;
      auto pass = [&](const Spectral& t) {
        Synthesise(t, g);
        for (std::size_t i = 0; i < W.size(); ++i) {
          g.c0[i] *= W[i];
          g.c1[i] *= W[i];
          g.r[i] *= W[i];
        }
        Analyse(g, analysed);
        for (std::size_t i = 0; i < analysed.c0.size(); ++i) analysed.c0[i] += fixedS.c0[i];
        for (std::size_t i = 0; i < analysed.c1.size(); ++i) analysed.c1[i] += fixedS.c1[i];
        for (std::size_t i = 0; i < analysed.r.size(); ++i) analysed.r[i] += fixedS.r[i];
        x = SolveAll(analysed, f);
        AddLoad(x, f, loadDot);
        return StrainOf(x, f);
      };
      Spectral t = ZeroSpectral();
      std::optional<Mixer> mixer;
      double previous = 0.0;
      bool converged = false;
      for (int iteration = 0; iteration < options_.max_iterations; ++iteration) {
        Spectral next = pass(t);
        const double residual = RelativeChange(next, t);
        if (!std::isfinite(residual)) break;
        if (residual <= options_.rtol) {
          t = std::move(next);
          converged = true;
          break;
        }
        if (!mixer && options_.anderson_memory > 0 && iteration > 0 && residual > options_.anderson_rate * previous)
          mixer.emplace(options_.anderson_memory);
        previous = residual;
        if (mixer) {
          mixer->Update({reinterpret_cast<double*>(t.c0.data()), reinterpret_cast<double*>(t.c1.data()),
                         reinterpret_cast<double*>(t.r.data())},
                        {reinterpret_cast<const double*>(next.c0.data()),
                         reinterpret_cast<const double*>(next.c1.data()), reinterpret_cast<const double*>(next.r.data())},
                        {2 * t.c0.size(), 2 * t.c1.size(), 2 * t.r.size()});
        } else {
          t = std::move(next);
        }
      }
      if (!converged) throw std::runtime_error("oracle tangent: a tangent stage did not converge");
      Synthesise(t, td);
      for (std::size_t k = 0; k < K; ++k)
        for (std::size_t i = 0; i < W.size(); ++i) {
          tm[k].c0[i] += beta[k][i] * td.c0[i] + bdot[k][i] * dEnd.c0[i];
          tm[k].c1[i] += beta[k][i] * td.c1[i] + bdot[k][i] * dEnd.c1[i];
          tm[k].r[i] += beta[k][i] * td.r[i] + bdot[k][i] * dEnd.r[i];
        }
      return x;
    };
    std::vector<C> mid(lm), dmid(lm);
    for (int k = 0; k < nodes; ++k) {
      const C* l1 = loads + lm * k;
      const C* l0 = k > 0 ? loads + lm * (k - 1) : l1;
      const C* t1 = loadDirections ? loadDirections + lm * k : nullptr;
      const C* t0 = loadDirections ? (k > 0 ? loadDirections + lm * (k - 1) : t1) : nullptr;
      const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
      Info info;
      Solutions sol, x;
      if (scheme != Scheme::Sdirk2 || dt == 0.0) {
        const Scheme one = scheme == Scheme::Sdirk2 ? Scheme::BackwardEuler : scheme;
        const State out = StepOnce(cur, dt, one, l0, l1, info, sol);
        x = stage(cur, out, dt, one, t1);
        cur = out;
      } else {
        for (std::size_t i = 0; i < lm; ++i) {
          mid[i] = (1.0 - gamma) * l0[i] + gamma * l1[i];
          if (t0) dmid[i] = (1.0 - gamma) * t0[i] + gamma * t1[i];
        }
        const State y1 = StepOnce(cur, gamma * dt, Scheme::BackwardEuler, l0, mid.data(), info, sol);
        const std::vector<Tensor> held = tm;
        stage(cur, y1, gamma * dt, Scheme::BackwardEuler, t0 ? dmid.data() : nullptr);
        State from;
        for (std::size_t b = 0; b < K; ++b) {
          Tensor c = ZeroTensor();
          for (std::size_t i = 0; i < c.r.size(); ++i) {
            c.c0[i] = (1.0 - r) * cur.m[b].c0[i] + r * y1.m[b].c0[i];
            c.c1[i] = (1.0 - r) * cur.m[b].c1[i] + r * y1.m[b].c1[i];
            c.r[i] = (1.0 - r) * cur.m[b].r[i] + r * y1.m[b].r[i];
            tm[b].c0[i] = (1.0 - r) * held[b].c0[i] + r * tm[b].c0[i];
            tm[b].c1[i] = (1.0 - r) * held[b].c1[i] + r * tm[b].c1[i];
            tm[b].r[i] = (1.0 - r) * held[b].r[i] + r * tm[b].r[i];
          }
          from.m.push_back(std::move(c));
        }
        from.strain = y1.strain;
        from.strainCoefficients = y1.strainCoefficients;
        const State out = StepOnce(from, gamma * dt, Scheme::BackwardEuler, mid.data(), l1, info, sol);
        x = stage(from, out, gamma * dt, Scheme::BackwardEuler, t1);
        cur = out;
      }
      if (!info.converged) throw std::runtime_error("oracle tangent: a forward stage did not converge");
      if (uOut) SurfaceOf(x, 0, uOut + lm * k);
      if (phiOut) SurfaceOf(x, 2, phiOut + lm * k);
    }
  }

  // The discrete adjoint of the run from a zero state (AdjointSolver3D
  // under AdjointMethod::Discrete, src/AdjointDiscrete3D.cpp; the transpose
  // of this restatement's own step): J = sum_n <u_n, U_n> + <phi_n, phi_n>
  // (surface pairing, m > 0 twice); out: the load kernels per node and
  // dJ/d delta per grid sample; returns J. Every state is kept and the
  // memory is on the grid at every node; each stage's transposed fixed
  // point is solved with this step's plain and Anderson iteration.
  double AdjointRun(const double* times, int nodes, Scheme scheme, const C* loads, const C* uDual, const C* phiDual,
                    C* loadKernels, double* grad, C* tideKernels = nullptr) {
    const std::size_t lm = grid_.RealSize(), fs = grid_.FieldSize();
    const std::size_t K = ZeroState().m.size();
    const int L = options_.lmax;
    auto pairSurface = [&](const C* a, const C* b) {
      double sum = 0.0;
      for (int l = 0; l <= L; ++l)
        for (int m = 0; m <= l; ++m) {
          const std::size_t i = OGrid::Index(l, m);
          sum += (m == 0 ? 1.0 : 2.0) * (std::conj(a[i]) * b[i]).real();
        }
      return sum;
    };
    // the forward run, every node (and Sdirk2's first stage) kept
    std::vector<State> states(nodes), firsts(nodes);
    State cur = ZeroState();
    double J = 0.0;
    std::vector<C> surface(lm), mid(lm);
    const double gamma = kSdirk2Gamma, r = (1.0 - gamma) / gamma;
    auto combine = [&](const State& a, const State& y1) {
      State from;
      for (std::size_t k = 0; k < K; ++k) {
        Tensor t = ZeroTensor();
        for (std::size_t i = 0; i < t.r.size(); ++i) {
          t.c0[i] = (1.0 - r) * a.m[k].c0[i] + r * y1.m[k].c0[i];
          t.c1[i] = (1.0 - r) * a.m[k].c1[i] + r * y1.m[k].c1[i];
          t.r[i] = (1.0 - r) * a.m[k].r[i] + r * y1.m[k].r[i];
        }
        from.m.push_back(std::move(t));
      }
      from.strain = y1.strain;
      from.strainCoefficients = y1.strainCoefficients;
      return from;
    };
    for (int k = 0; k < nodes; ++k) {
      const C* l1 = loads + lm * k;
      const C* l0 = k > 0 ? loads + lm * (k - 1) : l1;
      const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
      Info info;
      Solutions sol;
      if (scheme != Scheme::Sdirk2 || dt == 0.0) {
        cur = StepOnce(cur, dt, scheme == Scheme::Sdirk2 ? Scheme::BackwardEuler : scheme, l0, l1, info, sol);
      } else {
        for (std::size_t i = 0; i < lm; ++i) mid[i] = (1.0 - gamma) * l0[i] + gamma * l1[i];
        firsts[k] = StepOnce(cur, gamma * dt, Scheme::BackwardEuler, l0, mid.data(), info, sol);
        cur = StepOnce(combine(cur, firsts[k]), gamma * dt, Scheme::BackwardEuler, mid.data(), l1, info, sol);
      }
      if (uDual) {
        SurfaceOf(sol, 0, surface.data());
        J += pairSurface(uDual + lm * k, surface.data());
      }
      if (phiDual) {
        SurfaceOf(sol, 2, surface.data());
        J += pairSurface(phiDual + lm * k, surface.data());
      }
      states[k] = cur;
    }
    // the transposed sweep
    std::vector<Tensor> mD(K, ZeroTensor());
    Tensor dD = ZeroTensor();
    std::vector<double> gradient(static_cast<std::size_t>(NodeCount()) * fs, 0.0);
    std::fill(loadKernels, loadKernels + lm * nodes, C{});
    const State zero = [&] {
      State z = ZeroState();
      z.strain = ZeroTensor();
      return z;
    }();
    const auto& mesh = nodal_->mesh;
    const auto& pts = *points_;
    auto energy = [](C a0, C a1, double ar, C b0, C b1, double br) {
      return 4.0 * (std::conj(a0) * b0).real() + 8.0 * (std::conj(a1) * b1).real() + 12.0 * ar * br;
    };
    // one stage (in -> its end strain) transposed; the load's dual into sigma
    auto stage = [&](const State& in, const Tensor& dEnd, double dt, Scheme sch, const C* gU, const C* gPhi,
                     std::vector<C>& sigma, std::vector<C>& tide) {
      const auto& f = FlavourOf(sch, dt);
      auto weights = [&](double h, double& e, double& a, double& b, double& de, double& da, double& db) {
        StageWeightSlopes(sch, h, e, a, b, de, da, db);
      };
      // the lateral weight and the end strain's dual d-bar
      std::vector<double> W(gradient.size(), 0.0);
      Tensor bar = dD;
      for (std::size_t k = 0; k < K; ++k)
        for (int node = 0; node < NodeCount(); ++node) {
          const double itau = ItauRef(k, node), mu = MuBranch(k, node);
          double e0, a0, b0, de0, da0, db0;
          weights(dt * itau, e0, a0, b0, de0, da0, db0);
          for (std::size_t at = node * fs; at < (node + 1) * fs; ++at) {
            double e, a, b, de, da, db;
            weights(dt * (itau * factor_[at]), e, a, b, de, da, db);
            W[at] += mu * (b - b0);
            bar.c0[at] += b * mD[k].c0[at];
            bar.c1[at] += b * mD[k].c1[at];
            bar.r[at] += b * mD[k].r[at];
          }
        }
      Spectral fixedS = ZeroSpectral();
      Analyse(bar, fixedS);
      // S^T g at the surface dofs, and K^-1 of it
      auto surfaceForces = [&](std::vector<std::vector<C>>& sph) {
        for (int l = 0; l <= L; ++l) {
          const auto& op = *f.sph[l];
          const int iU = op.SurfaceDof(kU), iP = op.SurfaceDof(kPhi);
          for (int m = 0; m <= l; ++m) {
            const std::size_t i = OGrid::Index(l, m);
            if (gU && iU >= 0) sph[l][static_cast<std::size_t>(m) * op.DofCount() + iU] += gU[i];
            if (gPhi && iP >= 0) sph[l][static_cast<std::size_t>(m) * op.DofCount() + iP] += gPhi[i];
          }
        }
      };
      std::vector<std::vector<C>> gs(L + 1), gt(L + 1);
      for (int l = 0; l <= L; ++l) {
        gs[l].assign(static_cast<std::size_t>(f.sph[l]->DofCount()) * (l + 1), C{});
        if (l >= 1) gt[l].assign(static_cast<std::size_t>(f.tor[l]->DofCount()) * (l + 1), C{});
      }
      surfaceForces(gs);
      const Solutions q = SolveForces(gs, gt, f);
      // the fixed point t = Str(K^-1 F(An(W Syn t) + An(d-bar)) + q)
      Tensor g = ZeroTensor();
      Spectral analysed = ZeroSpectral();
      Solutions z;
      auto pass = [&](const Spectral& t) {
        Synthesise(t, g);
        for (std::size_t i = 0; i < W.size(); ++i) {
          g.c0[i] *= W[i];
          g.c1[i] *= W[i];
          g.r[i] *= W[i];
        }
        Analyse(g, analysed);
        for (std::size_t i = 0; i < analysed.c0.size(); ++i) analysed.c0[i] += fixedS.c0[i];
        for (std::size_t i = 0; i < analysed.c1.size(); ++i) analysed.c1[i] += fixedS.c1[i];
        for (std::size_t i = 0; i < analysed.r.size(); ++i) analysed.r[i] += fixedS.r[i];
        z = SolveAll(analysed, f);
        Axpy(z, 1.0, q);
        return StrainOf(z, f);
      };
      Spectral t = ZeroSpectral();
      std::optional<Mixer> mixer;
      double previous = 0.0;
      bool converged = false;
      for (int iteration = 0; iteration < options_.max_iterations; ++iteration) {
        Spectral next = pass(t);
        const double residual = RelativeChange(next, t);
        if (!std::isfinite(residual)) break;
        if (residual <= options_.rtol) {  // a zero dual converges at once (zero change of zero)
          t = std::move(next);
          converged = true;
          break;
        }
        if (!mixer && options_.anderson_memory > 0 && iteration > 0 && residual > options_.anderson_rate * previous)
          mixer.emplace(options_.anderson_memory);
        previous = residual;
        if (mixer) {
          mixer->Update({reinterpret_cast<double*>(t.c0.data()), reinterpret_cast<double*>(t.c1.data()),
                         reinterpret_cast<double*>(t.r.data())},
                        {reinterpret_cast<const double*>(next.c0.data()),
                         reinterpret_cast<const double*>(next.c1.data()), reinterpret_cast<const double*>(next.r.data())},
                        {2 * t.c0.size(), 2 * t.c1.size(), 2 * t.r.size()});
        } else {
          t = std::move(next);
        }
      }
      if (!converged) throw std::runtime_error("oracle adjoint: a transposed stage did not converge");
      Tensor zeta = ZeroTensor();
      Synthesise(t, zeta);
      // the load's dual u^T (F An(d-bar + W zeta) + S^T g)
      Tensor y = bar;
      for (std::size_t i = 0; i < W.size(); ++i) {
        y.c0[i] += W[i] * zeta.c0[i];
        y.c1[i] += W[i] * zeta.c1[i];
        y.r[i] += W[i] * zeta.r[i];
      }
      Spectral ys = ZeroSpectral();
      Analyse(y, ys);
      std::vector<std::vector<C>> fsph, ftor;
      Forces(ys, f, fsph, ftor);
      surfaceForces(fsph);
      sigma.assign(lm, C{});
      tide.assign(lm, C{});
      for (int l = 0; l <= L; ++l) {
        const int ndof = f.sph[l]->DofCount();
        for (int m = 0; m <= l; ++m) {
          C sum{}, tsum{};
          for (int d = 0; d < ndof; ++d) {
            sum += f.units[l][d] * fsph[l][static_cast<std::size_t>(m) * ndof + d];
            tsum += f.tideUnits[l][d] * fsph[l][static_cast<std::size_t>(m) * ndof + d];
          }
          sigma[OGrid::Index(l, m)] = sum;
          if (l != 1) tide[OGrid::Index(l, m)] = tsum;  // no degree-1 tide
        }
      }
      // the start's duals and the gradient
      Tensor start = in.strain.has_value() ? *in.strain : ZeroTensor();
      Tensor nextD = ZeroTensor();
      for (int node = 0; node < NodeCount(); ++node) {
        const auto& nd = nodes_[node];
        const double volume = mesh.Jacobian(nd.element) * pts.weight[nd.q] * nd.r * nd.r;
        for (std::size_t at = node * fs; at < (node + 1) * fs; ++at) {
          const double omega = volume * grid_.w[(at % fs) / grid_.nphi] * 2.0 * kPi / grid_.nphi;
          double sum = 0.0;
          for (std::size_t k = 0; k < K; ++k) {
            const double mu = MuBranch(k, node), h = dt * (ItauRef(k, node) * factor_[at]);
            double e, a, b, de, da, db;
            weights(h, e, a, b, de, da, db);
            const C M0 = mD[k].c0[at] + mu * zeta.c0[at], M1 = mD[k].c1[at] + mu * zeta.c1[at];
            const double Mr = mD[k].r[at] + mu * zeta.r[at];
            sum -= h * (de * energy(M0, M1, Mr, in.m[k].c0[at], in.m[k].c1[at], in.m[k].r[at]) +
                        da * energy(M0, M1, Mr, start.c0[at], start.c1[at], start.r[at]) +
                        db * energy(M0, M1, Mr, dEnd.c0[at], dEnd.c1[at], dEnd.r[at]));
            mD[k].c0[at] = e * M0;
            mD[k].c1[at] = e * M1;
            mD[k].r[at] = e * Mr;
            nextD.c0[at] += a * M0;
            nextD.c1[at] += a * M1;
            nextD.r[at] += a * Mr;
          }
          gradient[at] += omega * sum;
        }
      }
      dD = std::move(nextD);
    };
    std::vector<C> sigma, tide;
    if (tideKernels) std::fill(tideKernels, tideKernels + lm * nodes, C{});
    for (int n = nodes - 1; n >= 0; --n) {
      const State& prev = n > 0 ? states[n - 1] : zero;
      const double dt = n > 0 ? times[n] - times[n - 1] : 0.0;
      const C* gU = uDual ? uDual + lm * n : nullptr;
      const C* gPhi = phiDual ? phiDual + lm * n : nullptr;
      auto add = [&](int node, double c) {
        for (std::size_t i = 0; i < lm; ++i) loadKernels[lm * node + i] += c * sigma[i];
        if (tideKernels)
          for (std::size_t i = 0; i < lm; ++i) tideKernels[lm * node + i] += c * tide[i];
      };
      if (scheme != Scheme::Sdirk2 || dt == 0.0) {
        stage(prev, *states[n].strain, dt, scheme == Scheme::Sdirk2 ? Scheme::BackwardEuler : scheme, gU, gPhi,
              sigma, tide);
        add(n, 1.0);
        continue;
      }
      const State from = combine(prev, firsts[n]);
      stage(from, *states[n].strain, gamma * dt, Scheme::BackwardEuler, gU, gPhi, sigma, tide);
      add(n, 1.0);
      std::vector<Tensor> held(K, ZeroTensor());
      for (std::size_t k = 0; k < K; ++k)
        for (std::size_t i = 0; i < mD[k].r.size(); ++i) {
          held[k].c0[i] = (1.0 - r) * mD[k].c0[i];
          held[k].c1[i] = (1.0 - r) * mD[k].c1[i];
          held[k].r[i] = (1.0 - r) * mD[k].r[i];
          mD[k].c0[i] *= r;
          mD[k].c1[i] *= r;
          mD[k].r[i] *= r;
        }
      stage(prev, *firsts[n].strain, gamma * dt, Scheme::BackwardEuler, nullptr, nullptr, sigma, tide);
      add(n - 1, 1.0 - gamma);
      add(n, gamma);
      for (std::size_t k = 0; k < K; ++k)
        for (std::size_t i = 0; i < mD[k].r.size(); ++i) {
          mD[k].c0[i] += held[k].c0[i];
          mD[k].c1[i] += held[k].c1[i];
          mD[k].r[i] += held[k].r[i];
        }
    }
    if (grad) std::copy(gradient.begin(), gradient.end(), grad);
    return J;
  }

  // Surface (Viscoelastic3D.cpp:2032-2051): U, V or phi at the surface node.
  // InertiaMoment (Viscoelastic3D.cpp:2032-2048 with the degree-0 moment row
  // of detail/ViscoelasticDegree.hpp:142-161): sqrt(4 pi) sum over the
  // degree's elements and their GLL nodes of w_q J_e rho r^3 times the real
  // part of the last solutions' degree-0 U at that node's dof.
  double InertiaMoment() const {
    if (last_.sph.empty()) return 0.0;
    const auto& op = *elastic_->sph[0];
    const auto& mesh = nodal_->mesh;
    const int n = mesh.NGll();
    double sum = 0.0;
    for (int e = 0; e < mesh.ElementCount(); ++e)
      for (int q = 0; q < n; ++q) {
        const int dof = op.Dof(mesh.GlobalIndex(e, q), kU);
        if (dof < 0) continue;
        const double r = mesh.Radius(e, q);
        sum += mesh.Weights()[q] * mesh.Jacobian(e) * nodal_->rho[static_cast<std::size_t>(e) * n + q] * r * r * r *
               last_.sph[0][dof].real();
      }
    return std::sqrt(4.0 * 3.14159265358979323846) * sum;
  }

  // Surface (component 0 U, 1 V, 2 phi) and SurfaceToroidal (component 3,
  // W): Viscoelastic3D.cpp:2050-2112, the surface dof of each degree's
  // last solutions, zero where the degree has none.
  void Surface(int component, C* out) const { SurfaceOf(last_, component, out); }
  void SurfaceOf(const Solutions& x, int component, C* out) const {
    const auto& last_ = x;
    const int L = options_.lmax;
    if (component == 3) {
      for (int l = 0; l <= L; ++l) {
        const ToroidalOperator* op = l >= 1 ? elastic_->tor[l].get() : nullptr;
        const int dof = op != nullptr ? op->SurfaceDof() : -1;
        for (int m = 0; m <= l; ++m)
          out[OGrid::Index(l, m)] = dof >= 0 && !last_.tor.empty()
                                        ? last_.tor[l][static_cast<std::size_t>(m) * op->DofCount() + dof]
                                        : C{};
      }
      return;
    }
    for (int l = 0; l <= L; ++l) {
      const auto& op = *elastic_->sph[l];
      const int dof = op.SurfaceDof(component);
      for (int m = 0; m <= l; ++m)
        out[OGrid::Index(l, m)] = dof >= 0 && !last_.sph.empty() ? last_.sph[l][static_cast<std::size_t>(m) * op.DofCount() + dof] : C{};
    }
  }

  const Solutions& Last() const { return last_; }
  // The bounded timing sample of one backward Euler stage (see StepOnce).
  void Sample(const State& state, double dt, const C* load0, const C* load1, int passes, double* tStart,
              double* tPasses) {
    Info info;
    StepOnce(state, dt, Scheme::BackwardEuler, load0, load1, info, last_, passes, tStart, tPasses);
  }
  const std::vector<double>& History() const { return history_; }

 private:
  sl3dgpu_v3d_options options_;
  LayeredEarth earth_;
  RadialMesh mesh_;
  Material material_;
  Rheology rheology_;
  bool static_ = false;
  ReferenceRheology reference_;
  OGrid grid_;
  MemoryPoints gll_;
  const MemoryPoints* points_ = nullptr;
  const Material* nodal_ = nullptr;
  std::vector<double> dMu_, dKappa_;  // static problem: the moduli directions (empty for none)
  std::vector<Node> nodes_;
  std::vector<int> firstNode_;
  std::vector<double> factor_;  // exp(-delta) per grid value
  std::unique_ptr<Flavour> elastic_;
  std::vector<std::pair<std::pair<int, double>, std::unique_ptr<Flavour>>> flavours_;
  Solutions last_;
  std::vector<double> history_;
};

}  // namespace oracle

// -- the C interface -----------------------------------------------------------------------------------

using oracle::C;

struct oracle_v3d {
  std::unique_ptr<oracle::Viscoelastic3D> op;
};
struct oracle_state {
  oracle::State s;
};

extern "C" {

oracle_v3d* oracle_v3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options* options) {
  auto h = new oracle_v3d;
  h->op = std::make_unique<oracle::Viscoelastic3D>(layers, nlayers, *options);
  return h;
}

void oracle_v3d_destroy(oracle_v3d* h) { delete h; }

int oracle_v3d_node_count(const oracle_v3d* h) { return h->op->NodeCount(); }

void oracle_v3d_nodes(const oracle_v3d* h, double* radius, int* element) {
  const auto& nodes = h->op->Nodes();
  for (std::size_t i = 0; i < nodes.size(); ++i) {
    if (radius) radius[i] = nodes[i].r;
    if (element) element[i] = nodes[i].element;
  }
}

void oracle_v3d_grid(const oracle_v3d* h, int* ntheta, int* nphi, double* theta, double* weights) {
  const auto& g = h->op->Grid();
  if (ntheta) *ntheta = g.ntheta;
  if (nphi) *nphi = g.nphi;
  if (theta) std::memcpy(theta, g.theta.data(), g.theta.size() * sizeof(double));
  if (weights) std::memcpy(weights, g.w.data(), g.w.size() * sizeof(double));
}

double oracle_v3d_time_scale(const oracle_v3d* h) { return h->op->ModelScales().time; }
double oracle_v3d_surface_density_scale(const oracle_v3d* h) { return h->op->ModelScales().SurfaceDensity(); }

void oracle_v3d_set_delta(oracle_v3d* h, const double* samples) { h->op->SetDelta(samples); }

oracle_state* oracle_v3d_zero_state(const oracle_v3d* h) {
  auto s = new oracle_state;
  s->s = h->op->ZeroState();
  return s;
}

void oracle_v3d_free_state(oracle_state* s) { delete s; }

int oracle_v3d_step(oracle_v3d* h, oracle_state* state, double dt, int scheme, const double* load0,
                    const double* load1, sl3dgpu_step_info* info) {
  oracle::Info i;
  try {
    state->s = h->op->Step(state->s, dt, static_cast<orc::Scheme>(scheme),
                           reinterpret_cast<const C*>(load0), reinterpret_cast<const C*>(load1), i);
  } catch (const std::exception&) {
    return -3;
  }
  if (info) {
    info->iterations = i.iterations;
    info->residual = i.residual;
    info->converged = i.converged ? 1 : 0;
    info->mixed_passes = i.mixedPasses;
    info->correction_passes = 0;
    info->solve_iterations = i.solveIterations;
  }
  return 0;
}

int oracle_v3d_step_tide(oracle_v3d* h, oracle_state* state, double dt, int scheme, const double* load0,
                         const double* load1, const double* tide0, const double* tide1, sl3dgpu_step_info* info) {
  oracle::Info i;
  try {
    state->s = h->op->Step(state->s, dt, static_cast<orc::Scheme>(scheme),
                           reinterpret_cast<const C*>(load0), reinterpret_cast<const C*>(load1), i,
                           reinterpret_cast<const C*>(tide0), reinterpret_cast<const C*>(tide1));
  } catch (const std::exception&) {
    return -3;
  }
  if (info) {
    info->iterations = i.iterations;
    info->residual = i.residual;
    info->converged = i.converged ? 1 : 0;
    info->mixed_passes = i.mixedPasses;
    info->correction_passes = 0;
    info->solve_iterations = i.solveIterations;
  }
  return 0;
}

int oracle_v3d_residual_history(const oracle_v3d* h, double* out, int capacity) {
  const auto& v = h->op->History();
  if (out != nullptr)
    for (int i = 0; i < capacity && i < static_cast<int>(v.size()); ++i) out[i] = v[i];
  return static_cast<int>(v.size());
}

int oracle_v3d_sample(oracle_v3d* h, oracle_state* state, double dt, const double* load0, const double* load1,
                      int passes, double* start_seconds, double* pass_seconds) {
  try {
    h->op->Sample(state->s, dt, reinterpret_cast<const C*>(load0), reinterpret_cast<const C*>(load1), passes,
                  start_seconds, pass_seconds);
  } catch (const std::exception&) {
    return -3;
  }
  return 0;
}

int oracle_threads(void) { return omp_get_max_threads(); }

// The tangent-linear run beside the run from a zero state (the
// restatement's own derivative): U and phi derivatives per node along a
// log-viscosity direction (per grid sample, nullable) and load directions
// (nullable); status -1 when a stage did not converge.
int oracle_v3d_tangent_run(oracle_v3d* h, const double* times, int nodes, int scheme, const double* loads,
                           const double* direction, const double* load_directions, double* u, double* phi) {
  try {
    h->op->TangentRun(times, nodes, static_cast<orc::Scheme>(scheme), reinterpret_cast<const C*>(loads), direction,
                      reinterpret_cast<const C*>(load_directions), reinterpret_cast<C*>(u), reinterpret_cast<C*>(phi));
  } catch (const std::exception&) {
    return -1;
  }
  return 0;
}

// The discrete adjoint of the run from a zero state (the restatement's own
// transpose): the load kernels per node ((l, m >= 0) complex), dJ/d delta per
// grid sample (nullable), J and the tide kernels (nullable, none at degree
// 1); status -1 when a transposed stage did not converge.
int oracle_v3d_adjoint_run(oracle_v3d* h, const double* times, int nodes, int scheme, const double* loads,
                           const double* u_dual, const double* phi_dual, double* load_kernels, double* grad,
                           double* objective, double* tide_kernels) {
  try {
    *objective = h->op->AdjointRun(times, nodes, static_cast<orc::Scheme>(scheme), reinterpret_cast<const C*>(loads),
                                   reinterpret_cast<const C*>(u_dual), reinterpret_cast<const C*>(phi_dual),
                                   reinterpret_cast<C*>(load_kernels), grad, reinterpret_cast<C*>(tide_kernels));
  } catch (const std::exception&) {
    return -1;
  }
  return 0;
}

// The ocean closure: each pass's load and tide channels from the callback
// (NULL: the plain load channel again).
void oracle_v3d_set_closure(oracle_v3d* h, oracle_closure_fn fn, void* user) { h->op->SetClosure(fn, user); }

// A one-stage flavour's effective Love numbers (6 (lmax + 1) + 4 doubles).
void oracle_v3d_effective_love(oracle_v3d* h, int scheme, double dt, double* out) {
  const auto love = h->op->EffectiveLoveOf(static_cast<orc::Scheme>(scheme), dt);
  std::copy(love.begin(), love.end(), out);
}

// The body's surface radius and gravity, G (model units), and the scales
// (SI per unit of length, mass and time).
void oracle_v3d_body(const oracle_v3d* h, double* out) {
  const auto& sc = h->op->ModelScales();
  out[0] = h->op->SurfaceRadius();
  out[1] = h->op->SurfaceGravity();
  out[2] = h->op->GravitationalConstant();
  out[3] = sc.length;
  out[4] = sc.mass;
  out[5] = sc.time;
}

double oracle_v3d_inertia_moment(const oracle_v3d* h) { return h->op->InertiaMoment(); }

void oracle_v3d_surface(const oracle_v3d* h, int component, double* out) {
  h->op->Surface(component, reinterpret_cast<C*>(out));
}

// The state's strain coefficients (reference layouts, node-major): spin -2,
// spin -1, real spin 0 blocks end to end.
int oracle_v3d_state_strain(const oracle_state* s, double* out) {
  if (!s->s.strainCoefficients) return -1;
  const auto& sc = *s->s.strainCoefficients;
  C* o = reinterpret_cast<C*>(out);
  o = std::copy(sc.c0.begin(), sc.c0.end(), o);
  o = std::copy(sc.c1.begin(), sc.c1.end(), o);
  std::copy(sc.r.begin(), sc.r.end(), o);
  return 0;
}

}  // extern "C"

// The static perturbation problem through the same handle.
extern "C" oracle_v3d* oracle_ep3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_ep3d_options* o) {
  sl3dgpu_v3d_options options{};
  options.lmax = o->lmax;
  options.ngll = o->ngll;
  options.eps = o->eps;
  options.oversampling = o->oversampling;
  options.max_iterations = 1;
  options.rtol = 1e-10;
  options.damping = 1.0;
  options.solver = 1;
  auto h = new oracle_v3d;
  h->op = std::make_unique<oracle::Viscoelastic3D>(layers, nlayers, options, true);
  return h;
}
extern "C" double oracle_v3d_modulus_scale(const oracle_v3d* h) { return h->op->ModelScales().Modulus(); }
extern "C" void oracle_ep3d_set_moduli(oracle_v3d* h, const double* d_mu, const double* d_kappa) {
  h->op->SetModuli(d_mu, d_kappa);
}
extern "C" void oracle_ep3d_solve_load(oracle_v3d* h, const double* load) {
  h->op->SolveLoad(reinterpret_cast<const C*>(load));
}
extern "C" void oracle_ep3d_respond(oracle_v3d* h) { h->op->Respond(); }
extern "C" int oracle_ep3d_solve_lateral(oracle_v3d* h, const double* load, double rtol, int max_iterations,
                                         sl3dgpu_step_info* info) {
  oracle::Info i;
  h->op->SolveLateral(reinterpret_cast<const C*>(load), rtol, max_iterations, i);
  if (info) {
    *info = sl3dgpu_step_info{};
    info->iterations = i.iterations;
    info->residual = i.residual;
    info->converged = i.converged ? 1 : 0;
    info->solve_iterations = i.solveIterations;
  }
  return 0;
}

extern "C" int oracle_standard_earth(int elements, double kelvin_fraction, double kelvin_div,
                                     sl3dgpu_layer* out) {
  const auto layers = orc::StandardEarthLayers(elements, kelvin_fraction, kelvin_div);
  for (std::size_t i = 0; i < layers.size(); ++i) {
    const auto& L = layers[i];
    out[i] = sl3dgpu_layer{L.r0, L.r1, L.fluid ? 1 : 0, L.elements, L.rho0, L.rho1, L.kappa0, L.kappa1,
                           L.mu0, L.mu1, L.viscosity, L.kelvin_fraction, L.kelvin_viscosity};
  }
  return static_cast<int>(layers.size());
}
