// Host-side radial setup (see radial.hpp for what each part restates).
#include "radial.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace sl3dgpu::host {

// -- scales and the layered Earth ------------------------------------------------------------

Scales Scales::Geophysical(double length, double density) {
  Scales s;
  s.mass = density * length * length * length;
  s.length = length;
  s.time = 1.0 / std::sqrt(kGravitationalConstantSI * density);
  return s;
}

double Scales::Factor(int m, int l, int t) const {
  auto power = [](double x, int n) {
    double r = 1.0;
    const bool inv = n < 0;
    for (int k = 0; k < std::abs(n); ++k) r *= x;
    return inv ? 1.0 / r : r;
  };
  return power(mass, m) * power(length, l) * power(time, t);
}

LayeredEarth::LayeredEarth(std::vector<Layer> layers, Scales scales)
    : layers_(std::move(layers)), scales_(scales) {
  if (layers_.empty()) throw std::invalid_argument("a layered Earth needs a layer");
  double below = 0.0;
  for (std::size_t i = 0; i < layers_.size(); ++i) {
    const auto& L = layers_[i];
    if (!(L.r1 > L.r0) || (i > 0 && L.r0 != layers_[i - 1].r1))
      throw std::invalid_argument("layers must be contiguous and increasing");
    r0_.push_back(L.r0 / scales_.length);
    r1_.push_back(L.r1 / scales_.length);
  }
  massBelow_.resize(layers_.size());
  for (std::size_t i = 0; i < layers_.size(); ++i) {
    massBelow_[i] = below;
    const double a0 = r0_[i], a1 = r1_[i];
    const double d0 = layers_[i].rho0 / scales_.Density(), d1 = layers_[i].rho1 / scales_.Density();
    const double b = (d1 - d0) / (a1 - a0), a = d0 - b * a0;
    below += 4.0 * kPi * (a * (a1 * a1 * a1 - a0 * a0 * a0) / 3.0 +
                          b * (a1 * a1 * a1 * a1 - a0 * a0 * a0 * a0) / 4.0);
  }
}

double LayeredEarth::Linear(double a, double b, int layer, double r) const {
  const double t = (r - r0_[layer]) / (r1_[layer] - r0_[layer]);
  return a + (b - a) * t;
}

double LayeredEarth::Rho(int layer, double r, int nu) const {
  const auto& L = layers_[layer];
  const double a = L.rho0 / scales_.Density(), b = L.rho1 / scales_.Density();
  if (nu == 1) return (b - a) / (r1_[layer] - r0_[layer]);
  return Linear(a, b, layer, r);
}

double LayeredEarth::Kappa(int layer, double r) const {
  const auto& L = layers_[layer];
  return Linear(L.kappa0 / scales_.Modulus(), L.kappa1 / scales_.Modulus(), layer, r);
}

double LayeredEarth::Mu(int layer, double r) const {
  const auto& L = layers_[layer];
  if (L.fluid) return 0.0;
  return Linear(L.mu0 / scales_.Modulus(), L.mu1 / scales_.Modulus(), layer, r);
}

double LayeredEarth::Gravity(double r) const {
  if (r <= 0.0) return 0.0;
  int i = 0;
  while (i + 1 < LayerCount() && r > r1_[i]) ++i;
  const double a0 = r0_[i];
  const double d0 = Rho(i, a0), b = Rho(i, a0, 1), a = d0 - b * a0;
  const double rr = std::min(r, r1_[i]);
  const double M = massBelow_[i] + 4.0 * kPi * (a * (rr * rr * rr - a0 * a0 * a0) / 3.0 +
                                               b * (rr * rr * rr * rr - a0 * a0 * a0 * a0) / 4.0);
  const double G = kGravitationalConstantSI / scales_.Factor(-1, 3, -2);
  return G * M / (r * r);
}

// -- GLL and Gauss rules ------------------------------------------------------------------------

namespace {

void LegendreAt(int N, double x, double& pN, double& pNm1) {
  double p0 = 1.0, p1 = x;
  if (N == 0) {
    pN = 1.0;
    pNm1 = 0.0;
    return;
  }
  for (int k = 2; k <= N; ++k) {
    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  pN = p1;
  pNm1 = p0;
}

// Gauss-Lobatto-Legendre nodes on [-1, 1] (increasing) and weights
// 2 / (N (N + 1) P_N^2).
void GaussLobatto(int n, std::vector<double>& x, std::vector<double>& w) {
  const int N = n - 1;
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = -std::cos(kPi * i / N);
    for (int it = 0; it < 100; ++it) {
      double pN, pNm1;
      LegendreAt(N, z, pN, pNm1);
      const double dz = (z * pN - pNm1) / ((N + 1) * pN);
      z -= dz;
      if (std::abs(dz) < 1e-16) break;
    }
    x[i] = z;
  }
  x[0] = -1.0;
  x[N] = 1.0;
  for (int i = 0; i < n; ++i) {
    double pN, pNm1;
    LegendreAt(N, x[i], pN, pNm1);
    w[i] = 2.0 / (N * (N + 1.0) * pN * pN);
  }
}

// Gauss-Legendre nodes on [-1, 1] (increasing) and weights.
void GaussLegendreRule(int n, std::vector<double>& x, std::vector<double>& w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = -std::cos(kPi * (i + 0.75) / (n + 0.5));
    double pN = 0.0, pNm1 = 0.0, dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      LegendreAt(n, z, pN, pNm1);
      dp = n * (z * pN - pNm1) / (z * z - 1.0);
      const double dz = pN / dp;
      z -= dz;
      if (std::abs(dz) < 1e-16) break;
    }
    LegendreAt(n, z, pN, pNm1);
    dp = n * (z * pN - pNm1) / (z * z - 1.0);
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace

// -- the mesh ---------------------------------------------------------------------------------------

RadialMesh RadialMesh::Create(const LayeredEarth& earth, int ngll) {
  if (ngll < 2) throw std::invalid_argument("ngll must be at least 2");
  RadialMesh mesh;
  mesh.ngll_ = ngll;
  for (int s = 0; s < earth.LayerCount(); ++s) {
    const double lo = earth.Bottom(s), hi = earth.Top(s);
    const int nel = std::max(1, earth.LayerSI(s).elements);
    for (int e = 0; e < nel; ++e) {
      const double a = std::lerp(lo, hi, static_cast<double>(e) / nel);
      const double b = e + 1 == nel ? hi : std::lerp(lo, hi, static_cast<double>(e + 1) / nel);
      mesh.left_.push_back(a);
      mesh.right_.push_back(b);
      mesh.jac_.push_back(0.5 * (b - a));
      mesh.layer_.push_back(s);
    }
  }
  GaussLobatto(ngll, mesh.xi_, mesh.weights_);
  const int n = ngll, N = n - 1;
  std::vector<double> P(n);
  for (int i = 0; i < n; ++i) {
    double pN, pNm1;
    LegendreAt(N, mesh.xi_[i], pN, pNm1);
    P[i] = pN;
  }
  mesh.deriv_.assign(static_cast<std::size_t>(n) * n, 0.0);
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < n; ++i)
      if (k != i) mesh.deriv_[static_cast<std::size_t>(k) * n + i] = P[k] / (P[i] * (mesh.xi_[k] - mesh.xi_[i]));
  mesh.deriv_[0] = -0.25 * N * (N + 1);
  mesh.deriv_[static_cast<std::size_t>(n) * n - 1] = 0.25 * N * (N + 1);
  mesh.radius_.resize(mesh.left_.size() * static_cast<std::size_t>(n));
  for (std::size_t e = 0; e < mesh.left_.size(); ++e) {
    for (int i = 0; i < n; ++i) mesh.radius_[e * n + i] = mesh.left_[e] + (mesh.xi_[i] + 1.0) * mesh.jac_[e];
    mesh.radius_[e * n] = mesh.left_[e];
    mesh.radius_[e * n + N] = mesh.right_[e];
  }
  return mesh;
}

int RadialMesh::ElementOf(double r) const {
  auto it = std::upper_bound(left_.begin(), left_.end(), r);
  const auto i = static_cast<long>(it - left_.begin()) - 1;
  return static_cast<int>(std::clamp<long>(i, 0, static_cast<long>(left_.size()) - 1));
}

double RadialMesh::TruncationRadius(int l, double eps) const {
  const double rmax = right_.back();
  const double r = rmax * std::pow(eps, 1.0 / (l + 1));
  return std::clamp(r, left_.front(), rmax);
}

// -- material -----------------------------------------------------------------------------------

NodalModuli NodalModuli::Isotropic(const std::vector<double>& kappa, const std::vector<double>& mu) {
  NodalModuli m;
  const auto n = kappa.size();
  m.A.resize(n);
  m.C.resize(n);
  m.F.resize(n);
  m.L = mu;
  m.N = mu;
  for (std::size_t i = 0; i < n; ++i) {
    m.A[i] = kappa[i] + 4.0 * mu[i] / 3.0;
    m.C[i] = m.A[i];
    m.F[i] = kappa[i] - 2.0 * mu[i] / 3.0;
  }
  return m;
}

void NodalModuli::KappaMu(std::vector<double>& kappa, std::vector<double>& mu) const {
  const auto n = A.size();
  kappa.resize(n);
  mu.resize(n);
  for (std::size_t i = 0; i < n; ++i) {
    kappa[i] = (4.0 * A[i] + C[i] + 4.0 * F[i] - 4.0 * N[i]) / 9.0;
    mu[i] = (A[i] + C[i] - 2.0 * F[i] + 5.0 * N[i] + 6.0 * L[i]) / 15.0;
  }
}

Material Material::Create(const LayeredEarth& earth, const RadialMesh& mesh) {
  Material m{mesh};
  const int n = mesh.NGll();
  const auto size = static_cast<std::size_t>(mesh.ElementCount()) * n;
  m.rho.resize(size);
  m.drho.resize(size);
  m.g.resize(size);
  std::vector<double> kappa(size), mu(size);
  m.fluid.resize(mesh.ElementCount());
  for (int e = 0; e < mesh.ElementCount(); ++e) {
    const int layer = mesh.LayerOf(e);
    m.fluid[e] = earth.LayerSI(layer).fluid ? 1 : 0;
    for (int i = 0; i < n; ++i) {
      const auto at = static_cast<std::size_t>(e) * n + i;
      const double r = mesh.Radius(e, i);
      m.rho[at] = earth.Rho(layer, r);
      m.drho[at] = earth.Rho(layer, r, 1);
      m.g[at] = earth.Gravity(r);
      kappa[at] = earth.Kappa(layer, r);
      mu[at] = earth.Mu(layer, r);
    }
  }
  if (m.fluid.back()) throw std::invalid_argument("the surface of the model is fluid");
  m.moduli = NodalModuli::Isotropic(kappa, mu);
  m.G = kGravitationalConstantSI / earth.scales().Factor(-1, 3, -2);
  m.radius = mesh.Right(mesh.ElementCount() - 1);
  m.surfaceGravity = m.g.back();
  return m;
}

// -- rheology -----------------------------------------------------------------------------------

std::array<PronyTerm, 2> BurgersPronyTerms(double mu, double eta, double kelvinModulus,
                                           double kelvinViscosity) {
  for (double v : {mu, eta, kelvinModulus, kelvinViscosity})
    if (!std::isfinite(v) || !(v > 0.0))
      throw std::invalid_argument("a Burgers body's moduli and viscosities are positive and finite");
  const double a = mu / eta, b = mu / kelvinViscosity, c = kelvinModulus / kelvinViscosity;
  const double gap = std::sqrt((a - c) * (a - c) + b * b + 2.0 * b * (a + c));
  const double fast = 0.5 * (a + b + c + gap);
  const double slow = a * c / fast;
  auto plus = [&](double s, double product) { return s >= 0.0 ? gap + s : 4.0 * product / (gap - s); };
  const double aboveSlow = c * 0.5 * plus(b + c - a, a * b) / fast;
  const double belowFast = 0.5 * plus(a + b - c, b * c);
  return {PronyTerm{mu * aboveSlow / gap, slow}, PronyTerm{mu * belowFast / gap, fast}};
}

Rheology Rheology::FromEarth(const LayeredEarth& earth, const Material& material) {
  Rheology rh{material};
  const auto& mesh = material.mesh;
  const int n = mesh.NGll();
  const auto size = material.rho.size();
  std::vector<double> kappa, mu;
  material.moduli.KappaMu(kappa, mu);
  bool burgers = false;
  for (int s = 0; s < earth.LayerCount(); ++s)
    if (earth.LayerSI(s).viscosity > 0.0 && earth.LayerSI(s).kelvin_fraction > 0.0) burgers = true;
  Branch slow{std::vector<double>(size, 0.0), std::vector<double>(size, 0.0)};
  Branch fast = slow;
  const double viscosityScale = earth.scales().Viscosity();
  for (int e = 0; e < mesh.ElementCount(); ++e) {
    const auto& L = earth.LayerSI(mesh.LayerOf(e));
    if (!(L.viscosity > 0.0)) continue;
    if (material.IsFluid(e)) throw std::invalid_argument("a fluid layer cannot relax");
    const double eta = L.viscosity / viscosityScale;
    for (int i = 0; i < n; ++i) {
      const auto node = static_cast<std::size_t>(e) * n + i;
      if (L.kelvin_fraction > 0.0) {
        const auto terms = BurgersPronyTerms(mu[node], eta, L.kelvin_fraction * mu[node],
                                             L.kelvin_viscosity / viscosityScale);
        slow.mu[node] = terms[0].mu;
        slow.itau[node] = terms[0].itau;
        fast.mu[node] = terms[1].mu;
        fast.itau[node] = terms[1].itau;
      } else {
        slow.mu[node] = mu[node];
        slow.itau[node] = mu[node] / eta;
      }
    }
  }
  rh.branches.push_back(std::move(slow));
  if (burgers) rh.branches.push_back(std::move(fast));
  rh.kappa = kappa;
  rh.muUnrelaxed = mu;
  rh.muLongTerm = mu;
  rh.active.assign(size, 0);
  double scale = 0.0;
  for (double v : mu) scale = std::max(scale, v);
  for (const auto& b : rh.branches)
    for (std::size_t i = 0; i < size; ++i) {
      rh.muLongTerm[i] -= b.mu[i];
      if (b.mu[i] > 0.0) rh.active[i] = 1;
    }
  for (auto& v : rh.muLongTerm) {
    if (v < -1e-10 * scale) throw std::invalid_argument("branch moduli exceed the shear modulus");
    v = std::max(v, 0.0);
  }
  return rh;
}

Material Rheology::LongTermMaterial() const {
  Material out = material;
  for (const auto& b : branches) {
    for (std::size_t i = 0; i < b.mu.size(); ++i) {
      const double delta = -b.mu[i];
      out.moduli.A[i] += (4.0 / 3.0) * delta;
      out.moduli.C[i] += (4.0 / 3.0) * delta;
      out.moduli.F[i] -= (2.0 / 3.0) * delta;
      out.moduli.L[i] += delta;
      out.moduli.N[i] += delta;
    }
  }
  return out;
}

// -- memory points ------------------------------------------------------------------------------

MemoryPoints MemoryPoints::Of(bool gauss, const RadialMesh& mesh) {
  MemoryPoints out;
  out.gauss = gauss;
  out.ngll = mesh.NGll();
  const int n = out.ngll;
  const auto& nodes = mesh.Points();
  if (!gauss) {
    out.count = n;
    out.xi = nodes;
    out.weight = mesh.Weights();
    out.value.assign(static_cast<std::size_t>(n) * n, 0.0);
    out.derivative.resize(static_cast<std::size_t>(n) * n);
    for (int p = 0; p < n; ++p) {
      out.value[static_cast<std::size_t>(p) * n + p] = 1.0;
      for (int i = 0; i < n; ++i) out.derivative[static_cast<std::size_t>(p) * n + i] = mesh.Derivative(p, i);
    }
    return out;
  }
  out.count = n - 1;
  GaussLegendreRule(out.count, out.xi, out.weight);
  out.value.resize(static_cast<std::size_t>(out.count) * n);
  out.derivative.resize(static_cast<std::size_t>(out.count) * n);
  for (int p = 0; p < out.count; ++p) {
    const double x = out.xi[p];
    for (int i = 0; i < n; ++i) {
      double value = 1.0, slope = 0.0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        const double scale = 1.0 / (nodes[i] - nodes[j]);
        slope = slope * (x - nodes[j]) * scale + value * scale;
        value *= (x - nodes[j]) * scale;
      }
      out.value[static_cast<std::size_t>(p) * n + i] = value;
      out.derivative[static_cast<std::size_t>(p) * n + i] = slope;
    }
  }
  return out;
}

double MemoryPoints::RadiusAt(const RadialMesh& mesh, int e, int p) const {
  if (!gauss) return mesh.Radius(e, p);
  double r = 0.0;
  for (int i = 0; i < ngll; ++i) r += Value(p, i) * mesh.Radius(e, i);
  return r;
}

std::vector<double> MemoryPoints::Interpolate(const std::vector<double>& nodal) const {
  const auto elements = nodal.size() / ngll;
  std::vector<double> out(elements * count, 0.0);
  for (std::size_t e = 0; e < elements; ++e)
    for (int p = 0; p < count; ++p) {
      double sum = 0.0;
      for (int i = 0; i < ngll; ++i) sum += Value(p, i) * nodal[e * ngll + i];
      out[e * count + p] = sum;
    }
  return out;
}

// -- step weights (StepWeights.hpp:102-144) -------------------------------------------------

double Phi1(double h, double e) {
  if (std::abs(h) < 1e-3) return 1.0 - h / 2.0 + h * h / 6.0 - h * h * h / 24.0 + h * h * h * h / 120.0;
  return (1.0 - e) / h;
}

TrapezoidWeights ExponentialTrapezoidWeights(double h) {
  if (h < 0.0) throw std::invalid_argument("h = dt / tau must be >= 0");
  const double e = std::exp(-h);
  const double phi1 = Phi1(h, e);
  return {e, phi1 - e, 1.0 - phi1};
}

double BackwardEulerWeight(double h) {
  if (h < 0.0) throw std::invalid_argument("h = dt / tau must be >= 0");
  return 1.0 / (1.0 + h);
}

// -- the reference operator's point moduli ---------------------------------------------------

ReferenceRheology::ReferenceRheology(const Rheology& rh, bool gaussPoints)
    : rheology(rh), points(MemoryPoints::Of(gaussPoints, rh.material.mesh)), nodal(rh.material) {
  if (!gaussPoints) throw std::invalid_argument("the 3D step here keeps its memory at the Gauss points");
  auto sample = [&](const std::vector<double>& a) {
    auto out = points.Interpolate(a);
    for (auto& v : out) v = std::max(v, 0.0);
    return out;
  };
  for (const auto& b : rh.branches) {
    pointMu.push_back(sample(b.mu));
    pointItau.push_back(sample(b.itau));
  }
  nodal = rh.LongTermMaterial();
  elastic.points = &points;
  elastic.modulus.assign(pointMu.empty() ? 0 : pointMu[0].size(), 0.0);
  for (const auto& mu : pointMu)
    for (std::size_t i = 0; i < mu.size(); ++i) elastic.modulus[i] += mu[i];
}

PointShear ReferenceRheology::StepShear(Scheme scheme, double dt) const {
  if (dt == 0.0) return elastic;
  PointShear s;
  s.points = &points;
  s.modulus.assign(elastic.modulus.size(), 0.0);
  for (std::size_t k = 0; k < pointMu.size(); ++k)
    for (std::size_t i = 0; i < s.modulus.size(); ++i) {
      const double h = dt * pointItau[k][i];
      const double unrelaxed = scheme == Scheme::BackwardEuler ? BackwardEulerWeight(h)
                                                               : 1.0 - ExponentialTrapezoidWeights(h).beta;
      s.modulus[i] += pointMu[k][i] * unrelaxed;
    }
  return s;
}

// -- the spheroidal degree system ---------------------------------------------------------------

namespace {
double Stratification(double r, double drho, double g) { return g > 0.0 ? r * r * drho / g : 0.0; }
}  // namespace

DegreeOperator::DegreeOperator(const Material& material, int l, double eps,
                               const PointShear* pointShear)
    : material_(&material), l_(l) {
  if (l < 0) throw std::invalid_argument("degree must be non-negative");
  const auto& mesh = material.mesh;
  firstElement_ = l > 0 ? mesh.StartElement(l, eps) : 0;
  kd_ = 3 * (mesh.NGll() - 1) + 2;
  BuildDofMap();
  Assemble(pointShear);
  const int n = ndof_, ld = kd_ + 1;
  scale_.resize(n);
  positive_ = true;
  for (int j = 0; j < n; ++j) {
    const double d = band_[static_cast<std::size_t>(j) * ld + kd_];
    positive_ = positive_ && d > 0.0;
    scale_[j] = 1.0 / std::sqrt(std::abs(d) > 0.0 ? std::abs(d) : 1.0);
  }
}

void DegreeOperator::BuildDofMap() {
  const auto& mesh = material_->mesh;
  const int n = mesh.NGll(), nglob = mesh.NodeCount();
  const int g0 = mesh.GlobalIndex(firstElement_, 0);
  std::vector<char> solid(nglob, 0);
  for (int e = firstElement_; e < mesh.ElementCount(); ++e)
    if (l_ == 0 || !material_->IsFluid(e))
      for (int i = 0; i < n; ++i) solid[mesh.GlobalIndex(e, i)] = 1;
  dof_.assign(static_cast<std::size_t>(nglob) * 3, -1);
  ndof_ = 0;
  for (int gn = g0; gn < nglob; ++gn) {
    if (solid[gn]) {
      if (l_ == 0) {
        dof_[gn * 3 + 0] = ndof_++;
        dof_[gn * 3 + 2] = ndof_++;
      } else {
        for (int c = 0; c < 3; ++c) dof_[gn * 3 + c] = ndof_++;
      }
    } else {
      dof_[gn * 3 + 2] = ndof_++;
    }
  }
  auto drop = [&](std::size_t position) {
    const int removed = dof_[position];
    dof_[position] = -1;
    for (auto& d : dof_)
      if (d > removed) --d;
    --ndof_;
  };
  if (l_ == 1) drop(static_cast<std::size_t>(nglob - 1) * 3 + 2);  // centre-of-mass frame
  if (l_ == 0 && mesh.Left(firstElement_) == 0.0) drop(static_cast<std::size_t>(g0) * 3 + 0);
}

void DegreeOperator::Assemble(const PointShear* pointShear) {
  const auto& mesh = material_->mesh;
  const auto& mat = *material_;
  const int n = mesh.NGll(), n3 = 3 * n;
  const double k2 = l_ * (l_ + 1.0);
  const double G = mat.G;
  const double ifpg = 1.0 / (4.0 * kPi * G);
  const auto& w = mesh.Weights();
  const auto& M = mat.moduli;
  band_.assign(static_cast<std::size_t>(kd_ + 1) * ndof_, 0.0);
  std::vector<double> local(static_cast<std::size_t>(n3) * n3), B(static_cast<std::size_t>(n) * n);
  std::vector<double> X(n3), Y(n3), S(n3), dM(n3), dR(n3), dS(n3);
  auto at = [n3](std::vector<double>& m, int a, int b) -> double& { return m[static_cast<std::size_t>(a) * n3 + b]; };
  auto bandAt = [&](int i, int j) -> double& {
    return band_[static_cast<std::size_t>(j) * (kd_ + 1) + (kd_ + i - j)];
  };
  for (int e = firstElement_; e < mesh.ElementCount(); ++e) {
    std::fill(local.begin(), local.end(), 0.0);
    const auto base = static_cast<std::size_t>(e) * n;
    const double jac = mesh.Jacobian(e);
    const bool fluid = mat.IsFluid(e) && l_ > 0;
    for (int q = 0; q < n; ++q)
      for (int i = 0; i < n; ++i) B[q * n + i] = mesh.Radius(e, q) * mesh.Derivative(q, i) / jac;
    // int r^2 phi' psi' dr / 4 pi G
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double kp = 0.0;
        for (int q = 0; q < n; ++q) {
          const double rq = mesh.Radius(e, q);
          kp += mesh.Derivative(q, i) * w[q] * rq * rq * mesh.Derivative(q, j);
        }
        at(local, 3 * i + 2, 3 * j + 2) += ifpg * kp / jac;
      }
    for (int q = 0; q < n; ++q) {
      const double Wq = w[q] * jac;
      const double rq = mesh.Radius(e, q);
      at(local, 3 * q + 2, 3 * q + 2) += ifpg * k2 * Wq;
      if (fluid) {
        at(local, 3 * q + 2, 3 * q + 2) += Stratification(rq, mat.drho[base + q], mat.g[base + q]) * Wq;
        continue;
      }
      std::fill(X.begin(), X.end(), 0.0);
      std::fill(Y.begin(), Y.end(), 0.0);
      std::fill(S.begin(), S.end(), 0.0);
      for (int i = 0; i < n; ++i) {
        const double b = B[q * n + i];
        X[3 * i] = b;
        S[3 * i + 1] = b;
      }
      Y[3 * q] = 2.0;
      S[3 * q] = 1.0;
      Y[3 * q + 1] = -k2;
      S[3 * q + 1] -= 1.0;
      const double cC = M.C[base + q], cAN = M.A[base + q] - M.N[base + q], cF = M.F[base + q],
                   cL = M.L[base + q];
      for (int a = 0; a < n3; ++a) {
        const double xa = X[a], ya = Y[a], sa = S[a];
        if (xa == 0.0 && ya == 0.0 && sa == 0.0) continue;
        for (int b = 0; b < n3; ++b)
          at(local, a, b) += Wq * (cC * xa * X[b] + cAN * ya * Y[b] + cF * (xa * Y[b] + ya * X[b]) +
                                   k2 * cL * sa * S[b]);
      }
      at(local, 3 * q + 1, 3 * q + 1) += k2 * (k2 - 2.0) * M.N[base + q] * Wq;
      const double rho = mat.rho[base + q], g = mat.g[base + q];
      at(local, 3 * q, 3 * q) += 4.0 * rho * (kPi * G * rho * rq - g) * rq * Wq;
      const double cUV = k2 * rho * g * rq * Wq;
      at(local, 3 * q, 3 * q + 1) += cUV;
      at(local, 3 * q + 1, 3 * q) += cUV;
      const double cVP = k2 * rho * rq * Wq;
      at(local, 3 * q + 1, 3 * q + 2) += cVP;
      at(local, 3 * q + 2, 3 * q + 1) += cVP;
    }
    if (!fluid) {
      for (int i = 0; i < n; ++i) {
        const double ri = mesh.Radius(e, i);
        const double mi = mat.rho[base + i] * ri * ri * w[i];
        for (int j = 0; j < n; ++j) {
          const double m = mi * mesh.Derivative(i, j);
          at(local, 3 * i, 3 * j + 2) += m;
          at(local, 3 * j + 2, 3 * i) += m;
        }
      }
    }
    if (pointShear != nullptr && !fluid && !pointShear->bulk.empty()) {
      const auto& pts = *pointShear->points;
      for (int p = 0; p < pts.count; ++p) {
        const double kappa = pointShear->bulk[static_cast<std::size_t>(e) * pts.count + p];
        if (kappa == 0.0) continue;
        double rp = 0.0;
        for (int i = 0; i < n; ++i) rp += pts.Value(p, i) * mesh.Radius(e, i);
        std::fill(dR.begin(), dR.end(), 0.0);
        for (int i = 0; i < n; ++i) {
          const double v = pts.Value(p, i);
          dR[3 * i] = rp * pts.Derivative(p, i) / jac + 2.0 * v;
          dR[3 * i + 1] = -k2 * v;
        }
        const double weight = pts.weight[p] * jac * kappa;
        for (int a = 0; a < n3; ++a) {
          if (dR[a] == 0.0) continue;
          for (int b = 0; b < n3; ++b) at(local, a, b) += weight * dR[a] * dR[b];
        }
      }
    }
    if (pointShear != nullptr && !fluid) {
      const auto& pts = *pointShear->points;
      for (int p = 0; p < pts.count; ++p) {
        const double s = pointShear->modulus[static_cast<std::size_t>(e) * pts.count + p];
        if (s == 0.0) continue;
        double rp = 0.0;
        for (int i = 0; i < n; ++i) rp += pts.Value(p, i) * mesh.Radius(e, i);
        std::fill(dM.begin(), dM.end(), 0.0);
        std::fill(dR.begin(), dR.end(), 0.0);
        std::fill(dS.begin(), dS.end(), 0.0);
        for (int i = 0; i < n; ++i) {
          const double v = pts.Value(p, i);
          const double b = rp * pts.Derivative(p, i) / jac;
          dR[3 * i] = b - v;
          dR[3 * i + 1] = 0.5 * k2 * v;
          dS[3 * i] = v;
          dS[3 * i + 1] = b - v;
          dM[3 * i + 1] = v;
        }
        const double weight = pts.weight[p] * jac * s;
        for (int a = 0; a < n3; ++a) {
          if (dM[a] == 0.0 && dR[a] == 0.0 && dS[a] == 0.0) continue;
          for (int b = 0; b < n3; ++b)
            at(local, a, b) += weight * (k2 * (k2 - 2.0) * dM[a] * dM[b] + (4.0 / 3.0) * dR[a] * dR[b] +
                                         k2 * dS[a] * dS[b]);
        }
      }
    }
    for (int a = 0; a < n3; ++a) {
      const int ga = Dof(mesh.GlobalIndex(e, a / 3), a % 3);
      if (ga < 0) continue;
      for (int b = 0; b < n3; ++b) {
        const int gb = Dof(mesh.GlobalIndex(e, b / 3), b % 3);
        if (gb < ga) continue;
        const double value = at(local, a, b);
        if (value != 0.0) bandAt(ga, gb) += value;
      }
    }
  }
  auto point = [&](int i, int j, double value) {
    if (i < 0 || j < 0) return;
    if (i > j) std::swap(i, j);
    bandAt(i, j) += value;
  };
  // Fluid-solid interfaces (l > 0): +/- rho_f (g U U' + phi U' + U phi') r^2.
  if (l_ > 0) {
    for (int e = firstElement_; e + 1 < mesh.ElementCount(); ++e) {
      if (mat.IsFluid(e) == mat.IsFluid(e + 1)) continue;
      const int gn = mesh.GlobalIndex(e, n - 1);
      const double rt = mesh.Radius(e, n - 1);
      const double gt = mat.g[static_cast<std::size_t>(e) * n + (n - 1)];
      double rhoF, sign;
      if (mat.IsFluid(e)) {
        rhoF = mat.rho[static_cast<std::size_t>(e) * n + (n - 1)];
        sign = +1.0;
      } else {
        rhoF = mat.rho[static_cast<std::size_t>(e + 1) * n];
        sign = -1.0;
      }
      const int iU = Dof(gn, kU), iP = Dof(gn, kPhi);
      point(iU, iU, sign * rhoF * gt * rt * rt);
      point(iU, iP, sign * rhoF * rt * rt);
    }
  }
  // Dirichlet-to-Neumann closures.
  const int top = mesh.GlobalIndex(mesh.ElementCount() - 1, n - 1);
  if (l_ != 1) point(Dof(top, kPhi), Dof(top, kPhi), (l_ + 1) * mat.radius * ifpg);
  if (mesh.Left(firstElement_) > 0.0) {
    const int bottom = mesh.GlobalIndex(firstElement_, 0);
    point(Dof(bottom, kPhi), Dof(bottom, kPhi), l_ * mesh.Left(firstElement_) * ifpg);
  }
}

std::vector<double> DegreeOperator::ScaledCholeskyBand() const {
  const int n = ndof_, ld = kd_ + 1;
  std::vector<double> out(static_cast<std::size_t>(ld) * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - kd_); i <= j; ++i)
      out[static_cast<std::size_t>(j) * ld + (kd_ + i - j)] =
          band_[static_cast<std::size_t>(j) * ld + (kd_ + i - j)] * scale_[i] * scale_[j];
  return out;
}

std::vector<double> DegreeOperator::ScaledLuBand() const {
  const int n = ndof_, ld = kd_ + 1, ldlu = 3 * kd_ + 1;
  std::vector<double> out(static_cast<std::size_t>(ldlu) * n, 0.0);
  auto scaled = [&](int i, int j) {
    return band_[static_cast<std::size_t>(j) * ld + (kd_ + i - j)] * scale_[i] * scale_[j];
  };
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - kd_); i <= std::min(n - 1, j + kd_); ++i)
      out[static_cast<std::size_t>(j) * ldlu + (2 * kd_ + i - j)] = i <= j ? scaled(i, j) : scaled(j, i);
  return out;
}

int DegreeOperator::SurfaceDof(int c) const {
  const auto& mesh = material_->mesh;
  return Dof(mesh.GlobalIndex(mesh.ElementCount() - 1, mesh.NGll() - 1), c);
}

std::vector<double> DegreeOperator::Load() const {
  std::vector<double> b(ndof_, 0.0);
  const double a = material_->radius;
  b[SurfaceDof(kU)] = -material_->surfaceGravity * a * a;
  if (SurfaceDof(kPhi) >= 0) b[SurfaceDof(kPhi)] = -a * a;
  return b;
}

std::vector<double> DegreeOperator::Tide(int power) const {
  const int p = power < 0 ? l_ : power;
  std::vector<double> b(ndof_, 0.0);
  if (p == 0) return b;
  const auto& mesh = material_->mesh;
  const auto& mat = *material_;
  const int n = mesh.NGll();
  const double a = mat.radius, k2 = l_ * (l_ + 1.0);
  const auto& w = mesh.Weights();
  for (int e = firstElement_; e < mesh.ElementCount(); ++e) {
    const auto base = static_cast<std::size_t>(e) * n;
    const double jac = mesh.Jacobian(e);
    const bool fluid = mat.IsFluid(e) && l_ > 0;
    for (int q = 0; q < n; ++q) {
      const double Wq = w[q] * jac, rq = mesh.Radius(e, q);
      const double psi = std::pow(rq / a, p);
      const int gn = mesh.GlobalIndex(e, q);
      if (fluid) {
        b[Dof(gn, kPhi)] -= Wq * Stratification(rq, mat.drho[base + q], mat.g[base + q]) * psi;
        continue;
      }
      const double dpsi = (p / a) * std::pow(rq / a, p - 1);
      const int iU = Dof(gn, kU);
      if (iU >= 0) b[iU] -= Wq * mat.rho[base + q] * rq * rq * dpsi;
      if (l_ > 0) b[Dof(gn, kV)] -= k2 * Wq * mat.rho[base + q] * rq * psi;
    }
  }
  if (l_ > 0) {
    for (int e = firstElement_; e + 1 < mesh.ElementCount(); ++e) {
      if (mat.IsFluid(e) == mat.IsFluid(e + 1)) continue;
      const int gn = mesh.GlobalIndex(e, n - 1);
      const double rt = mesh.Radius(e, n - 1);
      const double rhoF = mat.IsFluid(e) ? mat.rho[static_cast<std::size_t>(e) * n + (n - 1)]
                                          : mat.rho[static_cast<std::size_t>(e + 1) * n];
      const double sign = mat.IsFluid(e) ? 1.0 : -1.0;
      b[Dof(gn, kU)] -= sign * rhoF * rt * rt * std::pow(rt / a, p);
    }
  }
  return b;
}

std::vector<double> DegreeOperator::Apply(const std::vector<double>& x, int nrhs) const {
  const int n = ndof_, ld = kd_ + 1;
  std::vector<double> y(x.size(), 0.0);
  for (int k = 0; k < nrhs; ++k) {
    const double* xk = x.data() + static_cast<std::size_t>(k) * n;
    double* yk = y.data() + static_cast<std::size_t>(k) * n;
    for (int j = 0; j < n; ++j)
      for (int i = std::max(0, j - kd_); i <= j; ++i) {
        const double a = band_[static_cast<std::size_t>(j) * ld + (kd_ + i - j)];
        yk[i] += a * xk[j];
        if (i != j) yk[j] += a * xk[i];
      }
  }
  return y;
}

// -- the toroidal degree system -----------------------------------------------------------------

ToroidalOperator::ToroidalOperator(const Material& material, int l, double eps,
                                   const PointShear* pointShear, double pinFraction)
    : material_(&material), l_(l) {
  if (l < 1) throw std::invalid_argument("the toroidal system exists for degrees one and above");
  const auto& mesh = material.mesh;
  const int n = mesh.NGll();
  firstElement_ = mesh.StartElement(l, eps);
  kd_ = n - 1;
  dof_.assign(mesh.NodeCount(), -1);
  bool inRegion = false;
  for (int e = firstElement_; e < mesh.ElementCount(); ++e) {
    if (material.IsFluid(e)) {
      if (inRegion) regions_.back().second = ndof_;
      inRegion = false;
      continue;
    }
    if (!inRegion) regions_.push_back({ndof_, ndof_});
    inRegion = true;
    for (int i = 0; i < n; ++i) {
      const int gn = mesh.GlobalIndex(e, i);
      if (dof_[gn] < 0) dof_[gn] = ndof_++;
    }
  }
  if (inRegion) regions_.back().second = ndof_;
  if (ndof_ == 0) throw std::invalid_argument("the degree's element subset holds no solid element");
  if (l == 1)
    for (const auto& [first, end] : regions_) {
      const int below = static_cast<int>(std::floor(pinFraction * static_cast<double>(end - first - 1)));
      pinned_.push_back(end - 1 - below);
    }
  // Assembly: k^2 L (r d_r W - W)^2 + k^2 (k^2 - 2) N W^2, plus the point shear.
  const double k2 = l * (l + 1.0);
  const auto& M = material.moduli;
  const auto& w = mesh.Weights();
  band_.assign(static_cast<std::size_t>(kd_ + 1) * ndof_, 0.0);
  auto bandAt = [&](int i, int j) -> double& {
    return band_[static_cast<std::size_t>(j) * (kd_ + 1) + (kd_ + i - j)];
  };
  for (int e = firstElement_; e < mesh.ElementCount(); ++e) {
    if (material.IsFluid(e)) continue;
    const auto base = static_cast<std::size_t>(e) * n;
    const double jac = mesh.Jacobian(e);
    for (int i = 0; i < n; ++i) {
      const int gi = dof_[mesh.GlobalIndex(e, i)];
      for (int j = i; j < n; ++j) {
        const int gj = dof_[mesh.GlobalIndex(e, j)];
        double value = 0.0;
        for (int q = 0; q < n; ++q) {
          const double rq = mesh.Radius(e, q);
          const double si = rq * mesh.Derivative(q, i) / jac - (q == i ? 1.0 : 0.0);
          const double sj = rq * mesh.Derivative(q, j) / jac - (q == j ? 1.0 : 0.0);
          value += w[q] * jac * k2 * M.L[base + q] * si * sj;
        }
        if (i == j) value += w[i] * jac * k2 * (k2 - 2.0) * M.N[base + i];
        bandAt(std::min(gi, gj), std::max(gi, gj)) += value;
      }
    }
  }
  if (pointShear != nullptr) {
    const auto& pts = *pointShear->points;
    for (int e = firstElement_; e < mesh.ElementCount(); ++e) {
      if (material.IsFluid(e)) continue;
      const double jac = mesh.Jacobian(e);
      for (int p = 0; p < pts.count; ++p) {
        const double s = pointShear->modulus[static_cast<std::size_t>(e) * pts.count + p];
        if (s == 0.0) continue;
        double rp = 0.0;
        for (int i = 0; i < n; ++i) rp += pts.Value(p, i) * mesh.Radius(e, i);
        const double weight = pts.weight[p] * jac * s;
        for (int i = 0; i < n; ++i) {
          const int gi = dof_[mesh.GlobalIndex(e, i)];
          const double ti = rp * pts.Derivative(p, i) / jac - pts.Value(p, i);
          const double wi = pts.Value(p, i);
          for (int j = i; j < n; ++j) {
            const int gj = dof_[mesh.GlobalIndex(e, j)];
            const double tj = rp * pts.Derivative(p, j) / jac - pts.Value(p, j);
            const double wj = pts.Value(p, j);
            const double value = weight * (k2 * ti * tj + k2 * (k2 - 2.0) * wi * wj);
            if (value == 0.0) continue;
            bandAt(std::min(gi, gj), std::max(gi, gj)) += value;
          }
        }
      }
    }
  }
  const int ld = kd_ + 1;
  scale_.resize(ndof_);
  for (int j = 0; j < ndof_; ++j) {
    const double d = band_[static_cast<std::size_t>(j) * ld + kd_];
    if (!(d > 0.0)) throw std::runtime_error("toroidal degree " + std::to_string(l) + ": a non-positive diagonal");
    scale_[j] = 1.0 / std::sqrt(d);
  }
}

std::vector<double> ToroidalOperator::ScaledCholeskyBand() const {
  const int n = ndof_, ld = kd_ + 1;
  std::vector<double> out(static_cast<std::size_t>(ld) * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - kd_); i <= j; ++i)
      out[static_cast<std::size_t>(j) * ld + (kd_ + i - j)] =
          band_[static_cast<std::size_t>(j) * ld + (kd_ + i - j)] * scale_[i] * scale_[j];
  for (const int p : pinned_)
    for (int j = std::max(0, p - kd_); j <= std::min(n - 1, p + kd_); ++j) {
      const int i = std::min(p, j), k = std::max(p, j);
      out[static_cast<std::size_t>(k) * ld + (kd_ + i - k)] = i == k ? 1.0 : 0.0;
    }
  return out;
}

int ToroidalOperator::SurfaceDof() const {
  const auto& mesh = material_->mesh;
  return dof_[mesh.GlobalIndex(mesh.ElementCount() - 1, mesh.NGll() - 1)];
}

std::vector<double> ToroidalOperator::Apply(const std::vector<double>& x, int nrhs) const {
  const int n = ndof_, ld = kd_ + 1;
  std::vector<double> y(x.size(), 0.0);
  for (int k = 0; k < nrhs; ++k) {
    const double* xk = x.data() + static_cast<std::size_t>(k) * n;
    double* yk = y.data() + static_cast<std::size_t>(k) * n;
    for (int j = 0; j < n; ++j)
      for (int i = std::max(0, j - kd_); i <= j; ++i) {
        const double a = band_[static_cast<std::size_t>(j) * ld + (kd_ + i - j)];
        yk[i] += a * xk[j];
        if (i != j) yk[j] += a * xk[i];
      }
  }
  return y;
}

// -- the configurations' Earth -----------------------------------------------------------------

std::vector<Layer> StandardEarthLayers(int elements, double kelvin_fraction, double kelvin_div) {
  const double a = 6371e3, cmb = 3480e3, r670 = 5701e3, lid = 6271e3;
  auto lin = [&](double v0, double v1, double r) { return v0 + (v1 - v0) * (r - cmb) / (a - cmb); };
  const double bounds[5] = {0.0, cmb, r670, lid, a};
  std::vector<Layer> layers(4);
  for (int i = 0; i < 4; ++i) {
    auto& L = layers[i];
    L.r0 = bounds[i];
    L.r1 = bounds[i + 1];
    if (i == 0) {
      L.fluid = true;
      L.rho0 = L.rho1 = 10900.0;
      L.kappa0 = L.kappa1 = 1.3e12;  // the core's bulk modulus (acts at degree 0 alone)
      continue;
    }
    L.rho0 = lin(5500.0, 3300.0, L.r0);
    L.rho1 = lin(5500.0, 3300.0, L.r1);
    L.mu0 = lin(2.9e11, 0.7e11, L.r0);
    L.mu1 = lin(2.9e11, 0.7e11, L.r1);
    L.kappa0 = lin(6.5e11, 1.3e11, L.r0);
    L.kappa1 = lin(6.5e11, 1.3e11, L.r1);
    if (i == 1) L.viscosity = 5e21;
    if (i == 2) L.viscosity = 5e20;
    if (L.viscosity > 0.0 && kelvin_fraction > 0.0) {
      L.kelvin_fraction = kelvin_fraction;
      L.kelvin_viscosity = L.viscosity / kelvin_div;
    }
  }
  // Elements in proportion to thickness, largest remainder, one at least.
  std::vector<double> share(4);
  std::vector<int> count(4);
  int total = 0;
  for (int i = 0; i < 4; ++i) {
    share[i] = elements * (bounds[i + 1] - bounds[i]) / a;
    count[i] = std::max(1, static_cast<int>(std::floor(share[i])));
    total += count[i];
  }
  while (total < elements) {
    int best = 0;
    double rem = -1.0;
    for (int i = 0; i < 4; ++i) {
      const double r = share[i] - count[i];
      if (r > rem) {
        rem = r;
        best = i;
      }
    }
    ++count[best];
    ++total;
  }
  for (int i = 0; i < 4; ++i) layers[i].elements = count[i];
  return layers;
}

}  // namespace sl3dgpu::host
