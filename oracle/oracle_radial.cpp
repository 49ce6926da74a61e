// The oracle's radial setup and degree systems (see oracle_radial.hpp).
// Test infrastructure only: loaded by tests/, __graft_entry__.smoke() and
// bench.py's CPU baseline, never by the library.
#include "oracle_radial.hpp"

#include <algorithm>
#include <cmath>
#include <memory>

namespace orc {

// -- scales and the body ---------------------------------------------------------------------

Scales Scales::Geophysical(double length, double density) {
  Scales s;
  s.length = length;
  s.mass = density * std::pow(length, 3);
  s.time = std::pow(kG_SI * density, -0.5);
  return s;
}

double Scales::Factor(int m, int l, int t) const { return std::pow(mass, m) * std::pow(length, l) * std::pow(time, t); }

LayeredEarth::LayeredEarth(std::vector<Layer> layers, Scales scales) : layers_(std::move(layers)), scales_(scales) {
  if (layers_.empty()) throw std::invalid_argument("no layers");
  for (std::size_t i = 0; i < layers_.size(); ++i)
    if (!(layers_[i].r1 > layers_[i].r0) || (i > 0 && layers_[i].r0 != layers_[i - 1].r1))
      throw std::invalid_argument("layers must be contiguous and increasing");
}

double LayeredEarth::Value(int i, double atBottom, double atTop, double r) const {
  const double t = (r - Bottom(i)) / (Top(i) - Bottom(i));
  return atBottom + t * (atTop - atBottom);
}

double LayeredEarth::Gravity(double r) const {
  // m(r) = 4 pi int_0^r rho s^2 ds: three Gauss points a layer integrate the
  // cubic rho(s) s^2 exactly
  if (r <= 0.0) return 0.0;
  const double x[3] = {-std::sqrt(0.6), 0.0, std::sqrt(0.6)}, w[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  double mass = 0.0;
  for (int i = 0; i < LayerCount(); ++i) {
    const double a = Bottom(i);
    if (a >= r && i > 0) break;
    const double b = std::min(Top(i), r);
    const double mid = 0.5 * (a + b), half = 0.5 * (b - a);
    for (int k = 0; k < 3; ++k) {
      const double s = mid + half * x[k];
      const double rho = Value(i, layers_[i].rho0, layers_[i].rho1, s) / scales_.Density();
      mass += 4.0 * kPi * w[k] * half * rho * s * s;
    }
    if (Top(i) >= r) break;
  }
  return mass / (r * r);  // G = 1 in these units
}

// -- the element rule -------------------------------------------------------------------------

namespace {

void LegendrePair(int N, double x, double& pN, double& pNm1) {
  double a = 1.0, b = x;
  if (N == 0) {
    pN = 1.0;
    pNm1 = 0.0;
    return;
  }
  for (int k = 2; k <= N; ++k) {
    const double c = ((2.0 * k - 1.0) * x * b - (k - 1.0) * a) / k;
    a = b;
    b = c;
  }
  pN = b;
  pNm1 = a;
}

}  // namespace

RadialMesh RadialMesh::Create(const LayeredEarth& earth, int ngll) {
  if (ngll < 2) throw std::invalid_argument("ngll >= 2");
  RadialMesh m;
  m.n_ = ngll;
  const int N = ngll - 1;
  // GLL nodes: Newton on (x P_N - P_{N-1}) from the Chebyshev-Lobatto points
  m.xi_.resize(ngll);
  for (int i = 0; i < ngll; ++i) {
    double z = -std::cos(kPi * i / N);
    for (int it = 0; it < 100 && i > 0 && i < N; ++it) {
      double pN, pNm1;
      LegendrePair(N, z, pN, pNm1);
      const double dz = (z * pN - pNm1) / ((N + 1) * pN);
      z -= dz;
      if (std::abs(dz) < 1e-16) break;
    }
    m.xi_[i] = z;
  }
  m.xi_[0] = -1.0;
  m.xi_[N] = 1.0;
  m.w_.resize(ngll);
  for (int i = 0; i < ngll; ++i) {
    double pN, pNm1;
    LegendrePair(N, m.xi_[i], pN, pNm1);
    m.w_[i] = 2.0 / (N * (N + 1.0) * pN * pN);
  }
  // differentiation matrix from the barycentric weights
  std::vector<double> bw(ngll, 1.0);
  for (int i = 0; i < ngll; ++i)
    for (int j = 0; j < ngll; ++j)
      if (j != i) bw[i] /= (m.xi_[i] - m.xi_[j]);
  m.d_.assign(static_cast<std::size_t>(ngll) * ngll, 0.0);
  for (int q = 0; q < ngll; ++q) {
    double diag = 0.0;
    for (int i = 0; i < ngll; ++i) {
      if (i == q) continue;
      const double v = (bw[i] / bw[q]) / (m.xi_[q] - m.xi_[i]);
      m.d_[static_cast<std::size_t>(q) * ngll + i] = v;
      diag -= v;
    }
    m.d_[static_cast<std::size_t>(q) * ngll + q] = diag;
  }
  for (int s = 0; s < earth.LayerCount(); ++s) {
    const int count = std::max(1, earth.LayerSI(s).elements);
    for (int e = 0; e < count; ++e) {
      const double a = std::lerp(earth.Bottom(s), earth.Top(s), static_cast<double>(e) / count);
      const double b = e + 1 == count ? earth.Top(s) : std::lerp(earth.Bottom(s), earth.Top(s), (e + 1.0) / count);
      m.left_.push_back(a);
      m.right_.push_back(b);
      m.layer_.push_back(s);
    }
  }
  m.radius_.resize(m.left_.size() * ngll);
  for (std::size_t e = 0; e < m.left_.size(); ++e) {
    const double h = 0.5 * (m.right_[e] - m.left_[e]);
    for (int i = 0; i < ngll; ++i) m.radius_[e * ngll + i] = m.left_[e] + (m.xi_[i] + 1.0) * h;
    m.radius_[e * ngll] = m.left_[e];
    m.radius_[e * ngll + N] = m.right_[e];
  }
  return m;
}

int RadialMesh::ElementOf(double r) const {
  const auto it = std::upper_bound(left_.begin(), left_.end(), r);
  return std::clamp(static_cast<int>(it - left_.begin()) - 1, 0, ElementCount() - 1);
}

double RadialMesh::TruncationRadius(int l, double eps) const {
  const double top = right_.back();
  return std::clamp(top * std::pow(eps, 1.0 / (l + 1)), left_.front(), top);
}

// -- material and rheology ---------------------------------------------------------------------

Material Material::Create(const LayeredEarth& earth, const RadialMesh& mesh) {
  Material m{mesh};
  const int n = mesh.NGll(), E = mesh.ElementCount();
  const auto& sc = earth.scales();
  m.fluid.resize(E);
  for (auto* v : {&m.rho, &m.drho, &m.g, &m.moduli.A, &m.moduli.C, &m.moduli.F, &m.moduli.L, &m.moduli.N})
    v->resize(static_cast<std::size_t>(E) * n);
  for (int e = 0; e < E; ++e) {
    const int s = mesh.LayerOf(e);
    const Layer& L = earth.LayerSI(s);
    m.fluid[e] = L.fluid;
    for (int i = 0; i < n; ++i) {
      const std::size_t k = static_cast<std::size_t>(e) * n + i;
      const double r = mesh.Radius(e, i);
      m.rho[k] = earth.Value(s, L.rho0, L.rho1, r) / sc.Density();
      m.drho[k] = (L.rho1 - L.rho0) / sc.Density() / (earth.Top(s) - earth.Bottom(s));
      m.g[k] = earth.Gravity(r);
      const double kappa = earth.Value(s, L.kappa0, L.kappa1, r) / sc.Modulus();
      const double mu = L.fluid ? 0.0 : earth.Value(s, L.mu0, L.mu1, r) / sc.Modulus();
      m.moduli.A[k] = m.moduli.C[k] = kappa + 4.0 * mu / 3.0;
      m.moduli.F[k] = kappa - 2.0 * mu / 3.0;
      m.moduli.L[k] = m.moduli.N[k] = mu;
    }
  }
  if (m.fluid.back()) throw std::invalid_argument("the surface of the model is fluid");
  m.G = 1.0;
  m.radius = mesh.Right(E - 1);
  m.surfaceGravity = m.g.back();
  return m;
}

namespace {

// The two Prony terms of a Burgers body: relaxation rates s1 < s2, the
// roots of s^2 - (a + b + c) s + a c, and the residues of
// mu (s + c) / ((s + s1)(s + s2)).
std::array<std::array<double, 2>, 2> Burgers(double mu, double eta, double muK, double etaK) {
  const double a = mu / eta, b = mu / etaK, c = muK / etaK;
  const double sum = a + b + c, disc = std::sqrt(sum * sum - 4.0 * a * c);
  const double s2 = 0.5 * (sum + disc), s1 = a * c / s2;
  return {{{mu * (c - s1) / (s2 - s1), s1}, {mu * (s2 - c) / (s2 - s1), s2}}};
}

}  // namespace

Rheology Rheology::FromEarth(const LayeredEarth& earth, const Material& material) {
  Rheology rh{material};
  const auto& mesh = material.mesh;
  const int n = mesh.NGll();
  const std::size_t size = material.rho.size();
  bool burgers = false;
  for (int s = 0; s < earth.LayerCount(); ++s)
    burgers = burgers || (earth.LayerSI(s).viscosity > 0.0 && earth.LayerSI(s).kelvin_fraction > 0.0);
  rh.branches.assign(burgers ? 2 : 1, Branch{std::vector<double>(size, 0.0), std::vector<double>(size, 0.0)});
  const double etaScale = earth.scales().Viscosity();
  for (int e = 0; e < mesh.ElementCount(); ++e) {
    const Layer& L = earth.LayerSI(mesh.LayerOf(e));
    if (!(L.viscosity > 0.0)) continue;
    for (int i = 0; i < n; ++i) {
      const std::size_t k = static_cast<std::size_t>(e) * n + i;
      const double mu = material.moduli.N[k];  // isotropic: N = mu
      if (L.kelvin_fraction > 0.0) {
        const auto t = Burgers(mu, L.viscosity / etaScale, L.kelvin_fraction * mu, L.kelvin_viscosity / etaScale);
        for (int b = 0; b < 2; ++b) {
          rh.branches[b].mu[k] = t[b][0];
          rh.branches[b].itau[k] = t[b][1];
        }
      } else {
        rh.branches[0].mu[k] = mu;
        rh.branches[0].itau[k] = mu / (L.viscosity / etaScale);
      }
    }
  }
  rh.active.assign(size, 0);
  for (const auto& b : rh.branches)
    for (std::size_t k = 0; k < size; ++k)
      if (b.mu[k] > 0.0) rh.active[k] = 1;
  return rh;
}

MemoryPoints MemoryPoints::Of(bool gauss, const RadialMesh& mesh) {
  MemoryPoints mp;
  mp.gauss = gauss;
  mp.ngll = mesh.NGll();
  const int n = mp.ngll;
  const auto& x = mesh.Points();
  if (!gauss) {
    mp.count = n;
    mp.xi = x;
    mp.weight = mesh.Weights();
  } else {
    // Gauss-Legendre points of order n - 1 by Newton on P_{n-1}
    const int g = n - 1;
    mp.count = g;
    mp.xi.resize(g);
    mp.weight.resize(g);
    for (int k = 0; k < g; ++k) {
      double z = std::cos(kPi * (g - k - 0.25) / (g + 0.5));
      double dp = 1.0;
      for (int it = 0; it < 100; ++it) {
        double pN, pNm1;
        LegendrePair(g, z, pN, pNm1);
        dp = g * (z * pN - pNm1) / (z * z - 1.0);
        const double dz = pN / dp;
        z -= dz;
        if (std::abs(dz) < 1e-16) break;
      }
      double pN, pNm1;
      LegendrePair(g, z, pN, pNm1);
      dp = g * (z * pN - pNm1) / (z * z - 1.0);
      mp.xi[k] = z;
      mp.weight[k] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
  }
  // Lagrange basis values and derivatives at the points, by the barycentric
  // form (the identity and the nodal derivative at the nodes)
  mp.value.assign(static_cast<std::size_t>(mp.count) * n, 0.0);
  mp.derivative.assign(static_cast<std::size_t>(mp.count) * n, 0.0);
  for (int p = 0; p < mp.count; ++p) {
    const double z = mp.xi[p];
    for (int i = 0; i < n; ++i) {
      if (!gauss) {
        mp.value[static_cast<std::size_t>(p) * n + i] = p == i ? 1.0 : 0.0;
        mp.derivative[static_cast<std::size_t>(p) * n + i] = mesh.Derivative(p, i);
        continue;
      }
      double v = 1.0;
      for (int j = 0; j < n; ++j)
        if (j != i) v *= (z - x[j]) / (x[i] - x[j]);
      double dv = 0.0;
      for (int k = 0; k < n; ++k) {
        if (k == i) continue;
        double term = 1.0 / (x[i] - x[k]);
        for (int j = 0; j < n; ++j)
          if (j != i && j != k) term *= (z - x[j]) / (x[i] - x[j]);
        dv += term;
      }
      mp.value[static_cast<std::size_t>(p) * n + i] = v;
      mp.derivative[static_cast<std::size_t>(p) * n + i] = dv;
    }
  }
  return mp;
}

double MemoryPoints::RadiusAt(const RadialMesh& mesh, int e, int p) const {
  if (!gauss) return mesh.Radius(e, p);
  return mesh.Left(e) + (xi[p] + 1.0) * mesh.Jacobian(e);  // the element map is affine
}

TrapezoidWeights ExponentialTrapezoidWeights(double h) {
  if (h < 0.0) throw std::invalid_argument("h >= 0");
  TrapezoidWeights t;
  t.e = std::exp(-h);
  // (1 - e^-h) / h, the alternating series below h = 1e-3 (StepWeights.hpp:98-107)
  const double phi1 = std::abs(h) < 1e-3 ? 1.0 - h / 2.0 + h * h / 6.0 - h * h * h / 24.0 + h * h * h * h / 120.0
                                          : (1.0 - t.e) / h;
  t.alpha = phi1 - t.e;
  t.beta = 1.0 - phi1;
  return t;
}

double BackwardEulerWeight(double h) {
  if (h < 0.0) throw std::invalid_argument("h >= 0");
  return 1.0 / (1.0 + h);
}

ReferenceRheology::ReferenceRheology(const Rheology& rh)
    : rheology(rh), points(MemoryPoints::Of(true, rh.material.mesh)), nodal(rh.material) {
  const int n = points.ngll;
  const std::size_t E = rh.material.rho.size() / n;
  for (const auto& b : rh.branches) {
    std::vector<double> mu(E * points.count), itau(E * points.count);
    for (std::size_t e = 0; e < E; ++e)
      for (int p = 0; p < points.count; ++p) {
        double a = 0.0, t = 0.0;
        for (int i = 0; i < n; ++i) {
          a += points.Value(p, i) * b.mu[e * n + i];
          t += points.Value(p, i) * b.itau[e * n + i];
        }
        mu[e * points.count + p] = std::max(a, 0.0);
        itau[e * points.count + p] = std::max(t, 0.0);
      }
    pointMu.push_back(std::move(mu));
    pointItau.push_back(std::move(itau));
    // the long-term material: the branch's shear taken out of the moduli
    for (std::size_t k = 0; k < b.mu.size(); ++k) {
      nodal.moduli.A[k] -= 4.0 * b.mu[k] / 3.0;
      nodal.moduli.C[k] -= 4.0 * b.mu[k] / 3.0;
      nodal.moduli.F[k] += 2.0 * b.mu[k] / 3.0;
      nodal.moduli.L[k] -= b.mu[k];
      nodal.moduli.N[k] -= b.mu[k];
    }
  }
  elastic.points = &points;
  elastic.modulus.assign(E * points.count, 0.0);
  for (const auto& mu : pointMu)
    for (std::size_t k = 0; k < mu.size(); ++k) elastic.modulus[k] += mu[k];
}

PointShear ReferenceRheology::StepShear(Scheme scheme, double dt) const {
  if (dt == 0.0) return elastic;
  PointShear s{&points, std::vector<double>(elastic.modulus.size(), 0.0)};
  for (std::size_t b = 0; b < pointMu.size(); ++b)
    for (std::size_t k = 0; k < s.modulus.size(); ++k) {
      const double h = dt * pointItau[b][k];
      const double keep = scheme == Scheme::BackwardEuler ? BackwardEulerWeight(h)
                                                          : 1.0 - ExponentialTrapezoidWeights(h).beta;
      s.modulus[k] += pointMu[b][k] * keep;
    }
  return s;
}

// -- assembly: element matrices as sums of F^T M F -----------------------------------------------

namespace {

// One quadrature point's contribution: rows F (nf x dim, row-major), the
// symmetric nf x nf matrix M, a weight; K (dim x dim) += weight F^T M F.
void AddForm(std::vector<double>& K, int dim, const std::vector<double>& F, const std::vector<double>& M, int nf,
             double weight) {
  std::vector<double> MF(static_cast<std::size_t>(nf) * dim, 0.0);
  for (int a = 0; a < nf; ++a)
    for (int b = 0; b < nf; ++b) {
      const double m = M[static_cast<std::size_t>(a) * nf + b];
      if (m == 0.0) continue;
      for (int k = 0; k < dim; ++k) MF[static_cast<std::size_t>(a) * dim + k] += m * F[static_cast<std::size_t>(b) * dim + k];
    }
  for (int a = 0; a < nf; ++a)
    for (int i = 0; i < dim; ++i) {
      const double f = F[static_cast<std::size_t>(a) * dim + i];
      if (f == 0.0) continue;
      for (int j = 0; j < dim; ++j) K[static_cast<std::size_t>(i) * dim + j] += weight * f * MF[static_cast<std::size_t>(a) * dim + j];
    }
}

std::vector<double> UpperBandScaled(const std::vector<double>& band, const std::vector<double>& scale, int n, int kd) {
  std::vector<double> out(band.size());
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - kd); i <= j; ++i) {
      const std::size_t at = static_cast<std::size_t>(j) * (kd + 1) + (kd + i - j);
      out[at] = band[at] * scale[i] * scale[j];
    }
  return out;
}

}  // namespace

DegreeOperator::DegreeOperator(const Material& material, int l, double eps, const PointShear* shear)
    : material_(&material), l_(l) {
  const auto& mesh = material.mesh;
  const int n = mesh.NGll(), E = mesh.ElementCount(), nodes = mesh.NodeCount();
  first_ = l > 0 ? mesh.StartElement(l, eps) : 0;
  kd_ = 3 * (n - 1) + 2;
  // unknowns per node: U, V, phi on solid nodes (U, phi at l = 0), phi on
  // fluid ones; U at the centre, and the surface phi at l = 1, left out
  std::vector<int> kind(nodes, 0);  // 0 none, 1 fluid, 2 solid
  for (int e = first_; e < E; ++e)
    for (int i = 0; i < n; ++i) {
      const int g = mesh.GlobalIndex(e, i);
      kind[g] = std::max(kind[g], (l == 0 || !material.IsFluid(e)) ? 2 : 1);
    }
  dof_.assign(static_cast<std::size_t>(nodes) * 3, -1);
  const int base = mesh.GlobalIndex(first_, 0);
  for (int g = 0; g < nodes; ++g) {
    if (kind[g] == 0) continue;
    if (kind[g] == 2 && !(l == 0 && g == base && mesh.Left(first_) == 0.0)) dof_[g * 3 + kU] = ndof_++;
    if (kind[g] == 2 && l > 0) dof_[g * 3 + kV] = ndof_++;
    if (!(l == 1 && g == nodes - 1)) dof_[g * 3 + kPhi] = ndof_++;
  }
  band_.assign(static_cast<std::size_t>(kd_ + 1) * ndof_, 0.0);
  auto add = [&](int i, int j, double v) {
    if (i < 0 || j < 0) return;
    if (i > j) std::swap(i, j);
    band_[static_cast<std::size_t>(j) * (kd_ + 1) + (kd_ + i - j)] += v;
  };
  const double k2 = l * (l + 1.0), ifpg = 1.0 / (4.0 * kPi * material.G);
  const int dim = 3 * n;
  for (int e = first_; e < E; ++e) {
    std::vector<double> K(static_cast<std::size_t>(dim) * dim, 0.0);
    const double jac = mesh.Jacobian(e);
    const bool fluid = l > 0 && material.IsFluid(e);
    for (int q = 0; q < n; ++q) {
      const std::size_t k = static_cast<std::size_t>(e) * n + q;
      const double r = mesh.Radius(e, q), Wq = mesh.Weights()[q] * jac;
      const double rho = material.rho[k], g = material.g[k];
      if (fluid) {
        // phi, dphi/dr
        std::vector<double> F(2 * dim, 0.0), M(4, 0.0);
        F[3 * q + kPhi] = 1.0;
        for (int i = 0; i < n; ++i) F[dim + 3 * i + kPhi] = mesh.Derivative(q, i) / jac;
        M[0] = ifpg * k2 + (g > 0.0 ? r * r * material.drho[k] / g : 0.0);
        M[3] = ifpg * r * r;
        AddForm(K, dim, F, M, 2, Wq);
        continue;
      }
      // r dU/dr, 2U - k^2 V, r dV/dr + U - V, V, U, V, phi, dphi/dr
      const int nf = 8;
      std::vector<double> F(static_cast<std::size_t>(nf) * dim, 0.0), M(nf * nf, 0.0);
      for (int i = 0; i < n; ++i) {
        const double t = r * mesh.Derivative(q, i) / jac;
        F[0 * dim + 3 * i + kU] = t;
        F[2 * dim + 3 * i + kV] = t;
        F[7 * dim + 3 * i + kPhi] = mesh.Derivative(q, i) / jac;
      }
      F[1 * dim + 3 * q + kU] = 2.0;
      F[1 * dim + 3 * q + kV] = -k2;
      F[2 * dim + 3 * q + kU] += 1.0;
      F[2 * dim + 3 * q + kV] -= 1.0;
      F[3 * dim + 3 * q + kV] = 1.0;
      F[4 * dim + 3 * q + kU] = 1.0;
      F[5 * dim + 3 * q + kV] = 1.0;
      F[6 * dim + 3 * q + kPhi] = 1.0;
      auto set = [&](int a, int b, double v) { M[a * nf + b] = M[b * nf + a] = v; };
      const auto& md = material.moduli;
      set(0, 0, md.C[k]);
      set(1, 1, md.A[k] - md.N[k]);
      set(0, 1, md.F[k]);
      set(2, 2, k2 * md.L[k]);
      set(3, 3, k2 * (k2 - 2.0) * md.N[k]);
      set(4, 4, 4.0 * rho * (kPi * material.G * rho * r - g) * r);
      set(4, 5, k2 * rho * g * r);
      set(5, 6, k2 * rho * r);
      set(4, 7, rho * r * r);
      set(6, 6, ifpg * k2);
      set(7, 7, ifpg * r * r);
      AddForm(K, dim, F, M, nf, Wq);
    }
    if (shear != nullptr && !fluid) {
      const auto& pts = *shear->points;
      for (int p = 0; p < pts.count; ++p) {
        const double s = shear->modulus[static_cast<std::size_t>(e) * pts.count + p];
        if (s == 0.0) continue;
        const double rp = pts.RadiusAt(mesh, e, p);
        std::vector<double> F(3 * static_cast<std::size_t>(dim), 0.0), M(9, 0.0);
        for (int i = 0; i < n; ++i) {
          const double v = pts.Value(p, i), t = rp * pts.Derivative(p, i) / jac;
          F[0 * dim + 3 * i + kU] = t - v;
          F[0 * dim + 3 * i + kV] = 0.5 * k2 * v;
          F[1 * dim + 3 * i + kU] = v;
          F[1 * dim + 3 * i + kV] = t - v;
          F[2 * dim + 3 * i + kV] = v;
        }
        M[0] = 4.0 / 3.0;
        M[4] = k2;
        M[8] = k2 * (k2 - 2.0);
        AddForm(K, dim, F, M, 3, pts.weight[p] * jac * s);
      }
    }
    for (int a = 0; a < dim; ++a)
      for (int b = a; b < dim; ++b) {
        const double v = K[static_cast<std::size_t>(a) * dim + b];
        if (v != 0.0) add(Dof(mesh.GlobalIndex(e, a / 3), a % 3), Dof(mesh.GlobalIndex(e, b / 3), b % 3), v);
      }
  }
  if (l > 0)
    for (int e = first_; e + 1 < E; ++e) {
      if (material.IsFluid(e) == material.IsFluid(e + 1)) continue;
      const bool below = material.IsFluid(e);
      const int g = mesh.GlobalIndex(e, n - 1);
      const double r = mesh.Right(e), gt = material.g[static_cast<std::size_t>(e) * n + n - 1];
      const double rhoF = below ? material.rho[static_cast<std::size_t>(e) * n + n - 1]
                                : material.rho[static_cast<std::size_t>(e + 1) * n];
      const double sign = below ? 1.0 : -1.0;
      add(Dof(g, kU), Dof(g, kU), sign * rhoF * gt * r * r);
      add(Dof(g, kU), Dof(g, kPhi), sign * rhoF * r * r);
    }
  if (l != 1) add(Dof(nodes - 1, kPhi), Dof(nodes - 1, kPhi), (l + 1.0) * material.radius * ifpg);
  if (mesh.Left(first_) > 0.0) {
    const int g = mesh.GlobalIndex(first_, 0);
    add(Dof(g, kPhi), Dof(g, kPhi), l * mesh.Left(first_) * ifpg);
  }
  scale_.resize(ndof_);
  for (int j = 0; j < ndof_; ++j) {
    const double d = band_[static_cast<std::size_t>(j) * (kd_ + 1) + kd_];
    positive_ = positive_ && d > 0.0;
    scale_[j] = d != 0.0 ? 1.0 / std::sqrt(std::abs(d)) : 1.0;
  }
}

std::vector<double> DegreeOperator::ScaledCholeskyBand() const { return UpperBandScaled(band_, scale_, ndof_, kd_); }

std::vector<double> DegreeOperator::ScaledLuBand() const {
  const int n = ndof_, kd = kd_, ld = 3 * kd + 1;
  const auto up = UpperBandScaled(band_, scale_, n, kd);
  std::vector<double> out(static_cast<std::size_t>(ld) * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - kd); i <= std::min(n - 1, j + kd); ++i) {
      const int lo = std::min(i, j), hi = std::max(i, j);
      out[static_cast<std::size_t>(j) * ld + (2 * kd + i - j)] = up[static_cast<std::size_t>(hi) * (kd + 1) + (kd + lo - hi)];
    }
  return out;
}

std::vector<double> DegreeOperator::Load() const {
  std::vector<double> f(ndof_, 0.0);
  const double a = material_->radius;
  f[SurfaceDof(kU)] = -material_->surfaceGravity * a * a;
  if (SurfaceDof(kPhi) >= 0) f[SurfaceDof(kPhi)] = -a * a;
  return f;
}

std::vector<double> DegreeOperator::Tide(int power) const {
  const int p = power < 0 ? l_ : power;
  std::vector<double> f(ndof_, 0.0);
  if (p == 0) return f;
  const auto& m = *material_;
  const auto& mesh = m.mesh;
  const int n = mesh.NGll();
  const double a = m.radius, k2 = l_ * (l_ + 1.0);
  for (int e = first_; e < mesh.ElementCount(); ++e)
    for (int q = 0; q < n; ++q) {
      const std::size_t k = static_cast<std::size_t>(e) * n + q;
      const double r = mesh.Radius(e, q), W = mesh.Weights()[q] * mesh.Jacobian(e);
      const int g = mesh.GlobalIndex(e, q);
      const double psi = std::pow(r / a, p), dpsi = p * std::pow(r / a, p - 1) / a;
      if (l_ > 0 && m.IsFluid(e)) {
        if (m.g[k] > 0.0) f[Dof(g, kPhi)] -= W * r * r * m.drho[k] / m.g[k] * psi;
        continue;
      }
      if (Dof(g, kU) >= 0) f[Dof(g, kU)] -= W * m.rho[k] * r * r * dpsi;
      if (l_ > 0) f[Dof(g, kV)] -= W * k2 * m.rho[k] * r * psi;
    }
  if (l_ > 0)
    for (int e = first_; e + 1 < mesh.ElementCount(); ++e) {
      if (m.IsFluid(e) == m.IsFluid(e + 1)) continue;
      const bool below = m.IsFluid(e);
      const double r = mesh.Right(e);
      const double rhoF = below ? m.rho[static_cast<std::size_t>(e) * n + n - 1] : m.rho[static_cast<std::size_t>(e + 1) * n];
      f[Dof(mesh.GlobalIndex(e, n - 1), kU)] -= (below ? 1.0 : -1.0) * rhoF * r * r * std::pow(r / a, p);
    }
  return f;
}

ToroidalOperator::ToroidalOperator(const Material& material, int l, double eps, const PointShear* shear)
    : material_(&material), l_(l) {
  if (l < 1) throw std::invalid_argument("toroidal degrees start at one");
  const auto& mesh = material.mesh;
  const int n = mesh.NGll(), E = mesh.ElementCount();
  const int first = mesh.StartElement(l, eps);
  kd_ = n - 1;
  dof_.assign(mesh.NodeCount(), -1);
  for (int e = first; e < E; ++e) {
    if (material.IsFluid(e)) continue;
    for (int i = 0; i < n; ++i)
      if (dof_[mesh.GlobalIndex(e, i)] < 0) dof_[mesh.GlobalIndex(e, i)] = ndof_++;
    // the top of a solid region (the next element fluid or none): the gauge row at l = 1
    if (l == 1 && (e + 1 == E || material.IsFluid(e + 1))) pinned_.push_back(dof_[mesh.GlobalIndex(e, n - 1)]);
  }
  if (ndof_ == 0) throw std::invalid_argument("no solid element above the truncation radius");
  band_.assign(static_cast<std::size_t>(kd_ + 1) * ndof_, 0.0);
  const double k2 = l * (l + 1.0);
  for (int e = first; e < E; ++e) {
    if (material.IsFluid(e)) continue;
    const double jac = mesh.Jacobian(e);
    std::vector<double> K(static_cast<std::size_t>(n) * n, 0.0);
    for (int q = 0; q < n; ++q) {
      const std::size_t k = static_cast<std::size_t>(e) * n + q;
      const double r = mesh.Radius(e, q);
      std::vector<double> F(2 * static_cast<std::size_t>(n), 0.0), M(4, 0.0);
      for (int i = 0; i < n; ++i) F[i] = r * mesh.Derivative(q, i) / jac;
      F[q] -= 1.0;
      F[n + q] = 1.0;
      M[0] = k2 * material.moduli.L[k];
      M[3] = k2 * (k2 - 2.0) * material.moduli.N[k];
      AddForm(K, n, F, M, 2, mesh.Weights()[q] * jac);
    }
    if (shear != nullptr) {
      const auto& pts = *shear->points;
      for (int p = 0; p < pts.count; ++p) {
        const double s = shear->modulus[static_cast<std::size_t>(e) * pts.count + p];
        if (s == 0.0) continue;
        const double rp = pts.RadiusAt(mesh, e, p);
        std::vector<double> F(2 * static_cast<std::size_t>(n), 0.0), M(4, 0.0);
        for (int i = 0; i < n; ++i) {
          F[i] = rp * pts.Derivative(p, i) / jac - pts.Value(p, i);
          F[n + i] = pts.Value(p, i);
        }
        M[0] = k2;
        M[3] = k2 * (k2 - 2.0);
        AddForm(K, n, F, M, 2, pts.weight[p] * jac * s);
      }
    }
    for (int a = 0; a < n; ++a)
      for (int b = a; b < n; ++b) {
        const int i = dof_[mesh.GlobalIndex(e, a)], j = dof_[mesh.GlobalIndex(e, b)];
        band_[static_cast<std::size_t>(std::max(i, j)) * (kd_ + 1) + (kd_ + std::min(i, j) - std::max(i, j))] +=
            K[static_cast<std::size_t>(a) * n + b];
      }
  }
  scale_.resize(ndof_);
  for (int j = 0; j < ndof_; ++j) {
    const double d = band_[static_cast<std::size_t>(j) * (kd_ + 1) + kd_];
    if (!(d > 0.0)) throw std::runtime_error("toroidal degree " + std::to_string(l) + ": non-positive diagonal");
    scale_[j] = 1.0 / std::sqrt(d);
  }
}

std::vector<double> ToroidalOperator::ScaledCholeskyBand() const {
  auto out = UpperBandScaled(band_, scale_, ndof_, kd_);
  for (int p : pinned_)
    for (int j = std::max(0, p - kd_); j <= std::min(ndof_ - 1, p + kd_); ++j) {
      const int lo = std::min(p, j), hi = std::max(p, j);
      out[static_cast<std::size_t>(hi) * (kd_ + 1) + (kd_ + lo - hi)] = lo == hi ? 1.0 : 0.0;
    }
  return out;
}

std::vector<double> ApplySymmetricBand(const std::vector<double>& band, int n, int kd, const std::vector<double>& x,
                                       int nrhs) {
  std::vector<double> y(x.size(), 0.0);
  for (int c = 0; c < nrhs; ++c)
    for (int i = 0; i < n; ++i) {
      // row i: the stored column i above the diagonal, row i of later columns
      double sum = 0.0;
      for (int k = std::max(0, i - kd); k <= std::min(n - 1, i + kd); ++k) {
        const int lo = std::min(i, k), hi = std::max(i, k);
        sum += band[static_cast<std::size_t>(hi) * (kd + 1) + (kd + lo - hi)] * x[static_cast<std::size_t>(c) * n + k];
      }
      y[static_cast<std::size_t>(c) * n + i] = sum;
    }
  return y;
}

std::vector<Layer> StandardEarthLayers(int elements, double kelvin_fraction, double kelvin_div) {
  const double a = 6371e3, cmb = 3480e3;
  const double r[5] = {0.0, cmb, 5701e3, 6271e3, a};
  auto mantle = [&](double top, double bottom, double x) { return top + (bottom - top) * (x - cmb) / (a - cmb); };
  std::vector<Layer> ls(4);
  for (int i = 0; i < 4; ++i) {
    ls[i].r0 = r[i];
    ls[i].r1 = r[i + 1];
  }
  ls[0].fluid = true;
  ls[0].rho0 = ls[0].rho1 = 10900.0;
  ls[0].kappa0 = ls[0].kappa1 = 1.3e12;
  for (int i = 1; i < 4; ++i) {
    ls[i].rho0 = mantle(5500.0, 3300.0, r[i]);
    ls[i].rho1 = mantle(5500.0, 3300.0, r[i + 1]);
    ls[i].mu0 = mantle(2.9e11, 0.7e11, r[i]);
    ls[i].mu1 = mantle(2.9e11, 0.7e11, r[i + 1]);
    ls[i].kappa0 = mantle(6.5e11, 1.3e11, r[i]);
    ls[i].kappa1 = mantle(6.5e11, 1.3e11, r[i + 1]);
  }
  ls[1].viscosity = 5e21;
  ls[2].viscosity = 5e20;
  for (int i = 1; i <= 2; ++i)
    if (kelvin_fraction > 0.0) {
      ls[i].kelvin_fraction = kelvin_fraction;
      ls[i].kelvin_viscosity = ls[i].viscosity / kelvin_div;
    }
  // thickness-proportional shares, floors then largest remainders
  std::vector<double> share(4);
  int total = 0;
  for (int i = 0; i < 4; ++i) {
    share[i] = elements * (r[i + 1] - r[i]) / a;
    ls[i].elements = std::max(1, static_cast<int>(share[i]));
    total += ls[i].elements;
  }
  while (total++ < elements) {
    int best = 0;
    for (int i = 1; i < 4; ++i)
      if (share[i] - ls[i].elements > share[best] - ls[best].elements) best = i;
    ++ls[best].elements;
  }
  return ls;
}

}  // namespace orc

// -- the C interface of the degree systems (for tests) --------------------------------------------

#include "../include/sl3dgpu.h"

extern "C" int oracle_degree_band(const sl3dgpu_layer* layers, int nlayers, int ngll, double eps, int relaxed,
                                  int scheme, double dt, int toroidal, int l, double* out, int* n, int* kd) {
  // relaxed = 1: the 3D step's flavour systems (the long-term material and
  // the point shear a step of this scheme and length leaves, dt = 0 the
  // elastic one); relaxed = 0: the unrelaxed material without point shear
  try {
    std::vector<orc::Layer> ls(nlayers);
    for (int i = 0; i < nlayers; ++i) {
      const auto& s = layers[i];
      ls[i] = orc::Layer{s.r0, s.r1, s.fluid != 0, s.rho0, s.rho1, s.kappa0, s.kappa1, s.mu0, s.mu1,
                         s.viscosity, s.kelvin_fraction, s.kelvin_viscosity, s.elements};
    }
    const orc::LayeredEarth earth(ls, orc::Scales::Geophysical(layers[nlayers - 1].r1));
    const auto mesh = orc::RadialMesh::Create(earth, ngll);
    const auto material = orc::Material::Create(earth, mesh);
    std::unique_ptr<orc::ReferenceRheology> ref;
    orc::PointShear shear;
    const orc::Material* nodal = &material;
    if (relaxed) {
      ref = std::make_unique<orc::ReferenceRheology>(orc::Rheology::FromEarth(earth, material));
      shear = ref->StepShear(static_cast<orc::Scheme>(scheme), dt);
      nodal = &ref->nodal;
    }
    const orc::PointShear* use = relaxed ? &shear : nullptr;
    std::vector<double> band;
    if (toroidal) {
      const orc::ToroidalOperator op(*nodal, l, eps, use);
      *n = op.DofCount();
      *kd = op.Bandwidth();
      band = op.Band();
    } else {
      const orc::DegreeOperator op(*nodal, l, eps, use);
      *n = op.DofCount();
      *kd = op.Bandwidth();
      band = op.Band();
    }
    if (out) std::copy(band.begin(), band.end(), out);
    return 0;
  } catch (const std::exception&) {
    return -1;
  }
}
