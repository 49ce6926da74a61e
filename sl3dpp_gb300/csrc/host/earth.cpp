// Host-side radial setup of the 3D operators (what each part stands for is
// listed in earth.hpp).
#include "earth.hpp"

#include <algorithm>
#include <cmath>

namespace sl3dgpu::host {

// -- scales ----------------------------------------------------------------------------------------

Scales Scales::Geophysical(double length, double density) {
  Scales s;
  s.length = length;
  s.mass = density * length * length * length;
  s.time = 1.0 / std::sqrt(kGravitationalConstantSI * density);
  return s;
}

double Scales::Factor(int m, int l, int t) const {
  auto raise = [](double base, int power) {
    double out = 1.0;
    for (int k = 0; k < std::abs(power); ++k) out *= base;
    return power < 0 ? 1.0 / out : out;
  };
  return raise(mass, m) * raise(length, l) * raise(time, t);
}

// -- the layered body --------------------------------------------------------------------------------

double LayeredBody::Span::MassBetween(double a, double b) const {
  // rho(s) = c0 + c1 s on the span; 4 pi int s^2 (c0 + c1 s) ds
  const double c1 = rhoSlope, c0 = rhoAt0 - rhoSlope * r0;
  const double cube = (b * b * b - a * a * a) / 3.0, quart = (b * b * b * b - a * a * a * a) / 4.0;
  return 4.0 * kPi * (c0 * cube + c1 * quart);
}

LayeredBody::LayeredBody(const std::vector<Layer>& layers, const Scales& scales) : source_(layers), scales_(scales) {
  if (layers.empty()) throw std::invalid_argument("a layered body needs at least one layer");
  const double rhoU = scales.Density(), modU = scales.Modulus(), lenU = scales.length;
  double mass = 0.0;
  for (std::size_t s = 0; s < layers.size(); ++s) {
    const Layer& in = layers[s];
    if (!(in.r1 > in.r0)) throw std::invalid_argument("every layer needs r1 > r0");
    if (s > 0 && in.r0 != layers[s - 1].r1) throw std::invalid_argument("layers must join end to end");
    Span sp{};
    sp.r0 = in.r0 / lenU;
    sp.r1 = in.r1 / lenU;
    const double h = sp.r1 - sp.r0;
    sp.rhoAt0 = in.rho0 / rhoU;
    sp.rhoSlope = (in.rho1 - in.rho0) / rhoU / h;
    sp.kappaAt0 = in.kappa0 / modU;
    sp.kappaSlope = (in.kappa1 - in.kappa0) / modU / h;
    sp.muAt0 = in.fluid ? 0.0 : in.mu0 / modU;
    sp.muSlope = in.fluid ? 0.0 : (in.mu1 - in.mu0) / modU / h;
    massBelow_.push_back(mass);
    mass += sp.MassBetween(sp.r0, sp.r1);
    spans_.push_back(sp);
  }
}

double LayeredBody::Bulk(int s, double r) const { return spans_[s].kappaAt0 + spans_[s].kappaSlope * (r - spans_[s].r0); }

double LayeredBody::Shear(int s, double r) const { return spans_[s].muAt0 + spans_[s].muSlope * (r - spans_[s].r0); }

double LayeredBody::Gravity(double r) const {
  if (r <= 0.0) return 0.0;
  std::size_t s = 0;
  while (s + 1 < spans_.size() && r > spans_[s].r1) ++s;
  const double top = std::min(r, spans_[s].r1);
  const double inside = massBelow_[s] + spans_[s].MassBetween(spans_[s].r0, top);
  return G() * inside / (r * r);
}

// -- the reference element ---------------------------------------------------------------------------

namespace {

// P_N(x) and its first two derivatives by the three-term recurrence.
void Legendre(int N, double x, double& p, double& dp, double& d2p) {
  double pm1 = 1.0, pk = x, dpm1 = 0.0, dpk = 1.0;
  if (N == 0) {
    p = 1.0;
    dp = d2p = 0.0;
    return;
  }
  for (int k = 1; k < N; ++k) {
    const double next = ((2.0 * k + 1.0) * x * pk - k * pm1) / (k + 1.0);
    const double dnext = dpm1 + (2.0 * k + 1.0) * pk;  // P'_{k+1} = P'_{k-1} + (2k+1) P_k
    pm1 = pk;
    pk = next;
    dpm1 = dpk;
    dpk = dnext;
  }
  p = pk;
  dp = dpk;
  // Legendre's equation: (1 - x^2) P'' = 2 x P' - N (N + 1) P
  d2p = std::abs(1.0 - x * x) > 0.0 ? (2.0 * x * dp - N * (N + 1.0) * p) / (1.0 - x * x) : 0.0;
}

// Gauss-Legendre points and weights on [-1, 1], increasing.
void GaussRule(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int k = 0; k < n; ++k) {
    double z = -std::cos(kPi * (k + 0.75) / (n + 0.5));
    double p = 0.0, dp = 0.0, d2p = 0.0;
    for (int it = 0; it < 60; ++it) {
      Legendre(n, z, p, dp, d2p);
      const double step = p / dp;
      z -= step;
      if (std::abs(step) <= 1e-16 * std::max(1.0, std::abs(z))) break;
    }
    Legendre(n, z, p, dp, d2p);
    x[k] = z;
    w[k] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace

GllRule GllRule::Of(int n) {
  if (n < 2) throw std::invalid_argument("an element needs at least two GLL nodes");
  GllRule g;
  g.n = n;
  const int N = n - 1;
  g.x.assign(n, 0.0);
  g.w.assign(n, 0.0);
  g.x[0] = -1.0;
  g.x[N] = 1.0;
  // interior nodes: the roots of P'_N, by Newton from the Chebyshev-Lobatto points
  for (int k = 1; k < N; ++k) {
    double z = -std::cos(kPi * k / N);
    for (int it = 0; it < 60; ++it) {
      double p, dp, d2p;
      Legendre(N, z, p, dp, d2p);
      const double step = dp / d2p;
      z -= step;
      if (std::abs(step) <= 1e-16) break;
    }
    g.x[k] = z;
  }
  std::vector<double> pn(n);
  for (int k = 0; k < n; ++k) {
    double p, dp, d2p;
    Legendre(N, g.x[k], p, dp, d2p);
    pn[k] = p;
    g.w[k] = 2.0 / (N * (N + 1.0) * p * p);
  }
  // l_i'(x_q): P_N(x_q) / (P_N(x_i) (x_q - x_i)) off the diagonal; the
  // diagonal vanishes but at the two ends, -+N (N + 1) / 4
  g.d.assign(static_cast<std::size_t>(n) * n, 0.0);
  for (int q = 0; q < n; ++q)
    for (int i = 0; i < n; ++i)
      if (q != i) g.d[static_cast<std::size_t>(q) * n + i] = pn[q] / (pn[i] * (g.x[q] - g.x[i]));
  g.d[0] = -0.25 * N * (N + 1.0);
  g.d[static_cast<std::size_t>(n) * n - 1] = 0.25 * N * (N + 1.0);
  return g;
}

// -- the mesh -----------------------------------------------------------------------------------------

RadialMesh RadialMesh::Create(const LayeredBody& body, int ngll) {
  RadialMesh m;
  m.rule_ = GllRule::Of(ngll);
  for (int s = 0; s < body.Layers(); ++s) {
    const int count = std::max(1, body.Source(s).elements);
    const double lo = body.Bottom(s), hi = body.Top(s);
    for (int k = 0; k < count; ++k) {
      const double a = lo + (hi - lo) * k / count;
      const double b = k + 1 == count ? hi : lo + (hi - lo) * (k + 1) / count;
      m.elems_.push_back({a, b, s});
    }
  }
  const int n = ngll;
  m.nodes_.resize(m.elems_.size() * n);
  for (std::size_t e = 0; e < m.elems_.size(); ++e) {
    const auto& el = m.elems_[e];
    const double half = 0.5 * (el.right - el.left);
    for (int i = 0; i < n; ++i) m.nodes_[e * n + i] = el.left + (m.rule_.x[i] + 1.0) * half;
    m.nodes_[e * n] = el.left;  // the ends exactly
    m.nodes_[e * n + n - 1] = el.right;
  }
  return m;
}

int RadialMesh::ElementOf(double r) const {
  // the last element whose left end is at or below r
  int lo = 0, hi = ElementCount() - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (elems_[mid].left <= r)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

double RadialMesh::TruncationRadius(int l, double eps) const {
  const double top = elems_.back().right;
  return std::clamp(top * std::pow(eps, 1.0 / (l + 1.0)), elems_.front().left, top);
}

// -- material -------------------------------------------------------------------------------------------

NodalModuli NodalModuli::Isotropic(const std::vector<double>& kappa, const std::vector<double>& mu) {
  NodalModuli out;
  const std::size_t n = kappa.size();
  out.A.resize(n);
  out.F.resize(n);
  for (std::size_t i = 0; i < n; ++i) {
    out.A[i] = kappa[i] + (4.0 / 3.0) * mu[i];
    out.F[i] = kappa[i] - (2.0 / 3.0) * mu[i];
  }
  out.C = out.A;
  out.L = mu;
  out.N = mu;
  return out;
}

Material Material::Create(const LayeredBody& body, const RadialMesh& mesh) {
  Material out{mesh};
  const int E = mesh.ElementCount(), n = mesh.NGll();
  const std::size_t size = static_cast<std::size_t>(E) * n;
  out.rho.resize(size);
  out.drho.resize(size);
  out.g.resize(size);
  out.fluid.resize(E);
  std::vector<double> kappa(size), mu(size);
  for (int e = 0; e < E; ++e) {
    const int s = mesh.LayerOf(e);
    out.fluid[e] = body.Source(s).fluid ? 1 : 0;
    for (int i = 0; i < n; ++i) {
      const std::size_t k = static_cast<std::size_t>(e) * n + i;
      const double r = mesh.Radius(e, i);
      out.rho[k] = body.Density(s, r);
      out.drho[k] = body.DensitySlope(s);
      out.g[k] = body.Gravity(r);
      kappa[k] = body.Bulk(s, r);
      mu[k] = body.Shear(s, r);
    }
  }
  if (out.fluid.back()) throw std::invalid_argument("the body's outermost layer must be solid");
  out.moduli = NodalModuli::Isotropic(kappa, mu);
  out.G = body.G();
  out.radius = mesh.Right(E - 1);
  out.surfaceGravity = out.g.back();
  return out;
}

Material Material::WithoutShear(const std::vector<double>& removed) const {
  Material out = *this;
  for (std::size_t i = 0; i < removed.size(); ++i) {
    const double d = removed[i];
    out.moduli.A[i] -= (4.0 / 3.0) * d;
    out.moduli.C[i] -= (4.0 / 3.0) * d;
    out.moduli.F[i] += (2.0 / 3.0) * d;
    out.moduli.L[i] -= d;
    out.moduli.N[i] -= d;
  }
  return out;
}

// -- rheology -------------------------------------------------------------------------------------------

std::array<PronyTerm, 2> BurgersPronyTerms(double mu, double eta, double kelvinModulus, double kelvinViscosity) {
  for (double v : {mu, eta, kelvinModulus, kelvinViscosity})
    if (!(v > 0.0) || !std::isfinite(v))
      throw std::invalid_argument("a Burgers body needs positive, finite moduli and viscosities");
  // The relaxation modulus mu s (s + c) / (s^2 + (a + b + c) s + a c) with
  // a = mu / eta, b = mu / etaK, c = muK / etaK has poles at -slow, -fast;
  // its residues mu (c - slow) / (fast - slow) and mu (fast - c) / (fast - slow)
  // are the Prony moduli.
  const double a = mu / eta, b = mu / kelvinViscosity, c = kelvinModulus / kelvinViscosity;
  const double sum = a + b + c;
  const double spread = std::sqrt((a - c) * (a - c) + b * (b + 2.0 * (a + c)));  // sqrt(sum^2 - 4 a c)
  const double fast = 0.5 * (sum + spread);
  const double slow = a * c / fast;
  // fast - a = (spread + (b + c - a)) / 2 and fast - c = (spread + (a + b - c)) / 2,
  // each written without cancellation when its bracket is negative
  auto halfPlus = [spread](double t, double product) {
    return t >= 0.0 ? 0.5 * (spread + t) : 2.0 * product / (spread - t);
  };
  const double fastMinusA = halfPlus(b + c - a, a * b);
  const double fastMinusC = halfPlus(a + b - c, b * c);
  const double cMinusSlow = c * fastMinusA / fast;  // c - a c / fast
  return {PronyTerm{mu * cMinusSlow / spread, slow}, PronyTerm{mu * fastMinusC / spread, fast}};
}

Rheology Rheology::FromBody(const LayeredBody& body, const Material& material) {
  Rheology out{material};
  const RadialMesh& mesh = material.mesh;
  const int E = mesh.ElementCount(), n = mesh.NGll();
  const std::size_t size = material.rho.size();
  out.kappa.resize(size);
  out.muUnrelaxed.resize(size);
  for (std::size_t i = 0; i < size; ++i) {
    out.kappa[i] = material.moduli.Kappa(i);
    out.muUnrelaxed[i] = material.moduli.Mu(i);
  }
  bool twoTerms = false;
  for (int s = 0; s < body.Layers(); ++s)
    twoTerms = twoTerms || (body.Source(s).viscosity > 0.0 && body.Source(s).kelvin_fraction > 0.0);
  std::vector<Branch> branches(twoTerms ? 2 : 1, Branch{std::vector<double>(size, 0.0), std::vector<double>(size, 0.0)});
  const double etaU = body.scales().Viscosity();
  for (int e = 0; e < E; ++e) {
    const Layer& src = body.Source(mesh.LayerOf(e));
    if (!(src.viscosity > 0.0)) continue;
    if (material.IsFluid(e)) throw std::invalid_argument("a fluid layer cannot carry a viscosity");
    const double eta = src.viscosity / etaU;
    for (int i = 0; i < n; ++i) {
      const std::size_t k = static_cast<std::size_t>(e) * n + i;
      const double mu = out.muUnrelaxed[k];
      if (src.kelvin_fraction > 0.0) {
        const auto terms = BurgersPronyTerms(mu, eta, src.kelvin_fraction * mu, src.kelvin_viscosity / etaU);
        for (int t = 0; t < 2; ++t) {
          branches[t].mu[k] = terms[t].mu;
          branches[t].itau[k] = terms[t].itau;
        }
      } else {  // Maxwell: the whole modulus relaxes at mu / eta
        branches[0].mu[k] = mu;
        branches[0].itau[k] = mu / eta;
      }
    }
  }
  out.branches = std::move(branches);
  out.active.assign(size, 0);
  out.muLongTerm = out.muUnrelaxed;
  double largest = 0.0;
  for (double v : out.muUnrelaxed) largest = std::max(largest, v);
  for (const Branch& b : out.branches)
    for (std::size_t i = 0; i < size; ++i) {
      out.muLongTerm[i] -= b.mu[i];
      out.active[i] = out.active[i] || b.mu[i] > 0.0;
    }
  for (double& v : out.muLongTerm) {
    if (v < -1e-10 * largest) throw std::invalid_argument("the branches' moduli exceed the shear modulus");
    v = std::max(v, 0.0);
  }
  return out;
}

Material Rheology::LongTermMaterial() const {
  std::vector<double> removed(material.rho.size(), 0.0);
  for (const Branch& b : branches)
    for (std::size_t i = 0; i < removed.size(); ++i) removed[i] += b.mu[i];
  return material.WithoutShear(removed);
}

// -- memory points ------------------------------------------------------------------------------------------

MemoryPoints MemoryPoints::Of(bool gauss, const RadialMesh& mesh) {
  MemoryPoints out;
  out.gauss = gauss;
  out.ngll = mesh.NGll();
  const int n = out.ngll;
  const GllRule& rule = mesh.Rule();
  if (gauss) {
    out.count = n - 1;
    GaussRule(out.count, out.xi, out.weight);
  } else {
    out.count = n;
    out.xi = rule.x;
    out.weight = rule.w;
  }
  out.value.assign(static_cast<std::size_t>(out.count) * n, 0.0);
  out.derivative.assign(static_cast<std::size_t>(out.count) * n, 0.0);
  for (int p = 0; p < out.count; ++p) {
    if (!gauss) {  // the nodes themselves: the basis is the identity there
      out.value[static_cast<std::size_t>(p) * n + p] = 1.0;
      for (int i = 0; i < n; ++i) out.derivative[static_cast<std::size_t>(p) * n + i] = rule.Slope(p, i);
      continue;
    }
    const double x = out.xi[p];
    for (int i = 0; i < n; ++i) {
      // l_i(x) = prod_{j != i} (x - x_j) / (x_i - x_j) and its derivative by
      // the product rule, accumulated factor by factor
      double value = 1.0, slope = 0.0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        const double inv = 1.0 / (rule.x[i] - rule.x[j]);
        slope = slope * (x - rule.x[j]) * inv + value * inv;
        value *= (x - rule.x[j]) * inv;
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
  const std::size_t E = nodal.size() / ngll;
  std::vector<double> out(E * count);
  for (std::size_t e = 0; e < E; ++e)
    for (int p = 0; p < count; ++p) {
      double v = 0.0;
      for (int i = 0; i < ngll; ++i) v += Value(p, i) * nodal[e * ngll + i];
      out[e * count + p] = v;
    }
  return out;
}

// -- step weights -----------------------------------------------------------------------------------------------

double Phi1(double h, double e) {
  if (std::abs(h) < 1e-3) return 1.0 + h * (-1.0 / 2.0 + h * (1.0 / 6.0 + h * (-1.0 / 24.0 + h / 120.0)));
  return (1.0 - e) / h;
}

TrapezoidWeights ExponentialTrapezoidWeights(double h) {
  if (h < 0.0) throw std::invalid_argument("a step's h = dt / tau is never negative");
  TrapezoidWeights t;
  t.e = std::exp(-h);
  const double phi1 = Phi1(h, t.e);
  t.alpha = phi1 - t.e;
  t.beta = 1.0 - phi1;
  return t;
}

double BackwardEulerWeight(double h) {
  if (h < 0.0) throw std::invalid_argument("a step's h = dt / tau is never negative");
  return 1.0 / (1.0 + h);
}

// -- the relaxing body ---------------------------------------------------------------------------------------------

RelaxingBody::RelaxingBody(const Rheology& rh)
    : rheology(rh), points(MemoryPoints::Of(true, rh.material.mesh)), nodal(rh.LongTermMaterial()) {
  for (const Branch& b : rh.branches) {
    auto mu = points.Interpolate(b.mu);
    auto itau = points.Interpolate(b.itau);
    for (double& v : mu) v = std::max(v, 0.0);  // interpolation cannot make a modulus negative
    for (double& v : itau) v = std::max(v, 0.0);
    pointMu.push_back(std::move(mu));
    pointItau.push_back(std::move(itau));
  }
  elastic.points = &points;
  elastic.modulus.assign(pointMu.empty() ? 0 : pointMu[0].size(), 0.0);
  for (const auto& mu : pointMu)
    for (std::size_t i = 0; i < mu.size(); ++i) elastic.modulus[i] += mu[i];
}

PointShear RelaxingBody::StepShear(Scheme scheme, double dt) const {
  if (dt == 0.0) return elastic;
  PointShear out;
  out.points = &points;
  out.modulus.assign(elastic.modulus.size(), 0.0);
  for (std::size_t k = 0; k < pointMu.size(); ++k)
    for (std::size_t i = 0; i < out.modulus.size(); ++i) {
      const double h = dt * pointItau[k][i];
      const double kept =
          scheme == Scheme::BackwardEuler ? BackwardEulerWeight(h) : 1.0 - ExponentialTrapezoidWeights(h).beta;
      out.modulus[i] += pointMu[k][i] * kept;
    }
  return out;
}

// -- degree layouts ---------------------------------------------------------------------------------------------------

SpheroidalLayout::SpheroidalLayout(const Material& material, int l, double eps)
    : material_(&material), mesh_(&material.mesh), l_(l) {
  if (l < 0) throw std::invalid_argument("a degree is never negative");
  const RadialMesh& mesh = material.mesh;
  const int n = mesh.NGll(), E = mesh.ElementCount(), nodes = mesh.NodeCount();
  first_ = l > 0 ? mesh.StartElement(l, eps) : 0;
  // which unknowns each node carries
  std::vector<char> solidNode(nodes, 0), anyNode(nodes, 0);
  for (int e = first_; e < E; ++e)
    for (int i = 0; i < n; ++i) {
      anyNode[mesh.GlobalIndex(e, i)] = 1;
      if (l == 0 || !material.IsFluid(e)) solidNode[mesh.GlobalIndex(e, i)] = 1;
    }
  const int bottom = mesh.GlobalIndex(first_, 0), top = nodes - 1;
  const bool fromCentre = mesh.Left(first_) == 0.0;
  map_.assign(static_cast<std::size_t>(nodes) * 3, -1);
  for (int g = 0; g < nodes; ++g) {
    if (!anyNode[g]) continue;
    for (int c = 0; c < 3; ++c) {
      bool carried = c == kPhi || solidNode[g];
      if (c == kV && l == 0) carried = false;                      // no tangential motion at degree 0
      if (c == kU && l == 0 && g == bottom && fromCentre) carried = false;  // U(0) = 0 at the centre
      if (c == kPhi && l == 1 && g == top) carried = false;       // the centre-of-mass frame
      if (!carried) continue;
      map_[static_cast<std::size_t>(g) * 3 + c] = static_cast<int>(node_.size());
      node_.push_back(g);
      comp_.push_back(c);
    }
  }
}

std::vector<double> SpheroidalLayout::Load() const {
  std::vector<double> f(DofCount(), 0.0);
  const double a = material_->radius;
  f[SurfaceDof(kU)] = -material_->surfaceGravity * a * a;
  if (SurfaceDof(kPhi) >= 0) f[SurfaceDof(kPhi)] = -a * a;
  return f;
}

std::vector<double> SpheroidalLayout::Tide(int power) const {
  // Minus the weak-form work of the external potential psi = (r / a)^p on
  // each unknown: rho r^2 psi' on U and k^2 rho r psi on V in solids, the
  // stratification r^2 rho' / g psi on phi in fluids, and the fluid-solid
  // boundaries' rho_f r^2 psi jump on U.
  const int p = power < 0 ? l_ : power;
  std::vector<double> f(DofCount(), 0.0);
  if (p == 0) return f;
  const Material& mat = *material_;
  const RadialMesh& mesh = *mesh_;
  const int n = mesh.NGll(), E = mesh.ElementCount();
  const double a = mat.radius, k2 = l_ * (l_ + 1.0);
  for (int e = first_; e < E; ++e) {
    const double jac = mesh.Jacobian(e);
    const bool fluidHere = l_ > 0 && mat.IsFluid(e);
    for (int q = 0; q < n; ++q) {
      const std::size_t k = static_cast<std::size_t>(e) * n + q;
      const double r = mesh.Radius(e, q), wq = mesh.Weights()[q] * jac;
      const double psi = std::pow(r / a, p);
      const int g = mesh.GlobalIndex(e, q);
      if (fluidHere) {
        const double strat = mat.g[k] > 0.0 ? r * r * mat.drho[k] / mat.g[k] : 0.0;
        f[Dof(g, kPhi)] -= wq * strat * psi;
        continue;
      }
      const double dpsi = (p / a) * std::pow(r / a, p - 1);
      if (Dof(g, kU) >= 0) f[Dof(g, kU)] -= wq * mat.rho[k] * r * r * dpsi;
      if (l_ > 0) f[Dof(g, kV)] -= wq * k2 * mat.rho[k] * r * psi;
    }
  }
  if (l_ > 0)
    for (int e = first_; e + 1 < E; ++e) {
      if (mat.IsFluid(e) == mat.IsFluid(e + 1)) continue;
      const double r = mesh.Right(e);
      const bool fluidBelow = mat.IsFluid(e);
      const double rhoF = fluidBelow ? mat.rho[static_cast<std::size_t>(e) * n + n - 1]
                                     : mat.rho[static_cast<std::size_t>(e + 1) * n];
      f[Dof(mesh.GlobalIndex(e, n - 1), kU)] -= (fluidBelow ? 1.0 : -1.0) * rhoF * r * r * std::pow(r / a, p);
    }
  return f;
}

ToroidalLayout::ToroidalLayout(const Material& material, int l, double eps) : mesh_(&material.mesh), l_(l) {
  if (l < 1) throw std::invalid_argument("toroidal unknowns start at degree one");
  const RadialMesh& mesh = material.mesh;
  const int n = mesh.NGll(), E = mesh.ElementCount();
  first_ = mesh.StartElement(l, eps);
  map_.assign(mesh.NodeCount(), -1);
  int regionTop = -1;
  for (int e = first_; e < E; ++e) {
    if (material.IsFluid(e)) {
      if (regionTop >= 0 && l == 1) pinned_.push_back(regionTop);
      regionTop = -1;
      continue;
    }
    for (int i = 0; i < n; ++i) {
      const int g = mesh.GlobalIndex(e, i);
      if (map_[g] >= 0) continue;
      map_[g] = static_cast<int>(node_.size());
      node_.push_back(g);
    }
    regionTop = map_[mesh.GlobalIndex(e, n - 1)];
  }
  if (regionTop >= 0 && l == 1) pinned_.push_back(regionTop);
  if (node_.empty()) throw std::invalid_argument("degree " + std::to_string(l) + " reaches no solid element");
}

// -- the configurations' body ---------------------------------------------------------------------------------------------

std::vector<Layer> StandardEarthLayers(int elements, double kelvin_fraction, double kelvin_div) {
  const double surface = 6371e3, cmb = 3480e3;
  const double edges[5] = {0.0, cmb, 5701e3, 6271e3, surface};
  const double viscosity[4] = {0.0, 5e21, 5e20, 0.0};
  auto mantle = [&](double top, double bottom, double r) { return top + (bottom - top) * (r - cmb) / (surface - cmb); };
  std::vector<Layer> out(4);
  for (int s = 0; s < 4; ++s) {
    Layer& L = out[s];
    L.r0 = edges[s];
    L.r1 = edges[s + 1];
    if (s == 0) {  // the fluid core; its bulk modulus acts at degree 0 alone
      L.fluid = true;
      L.rho0 = L.rho1 = 10900.0;
      L.kappa0 = L.kappa1 = 1.3e12;
      continue;
    }
    L.rho0 = mantle(5500.0, 3300.0, L.r0);
    L.rho1 = mantle(5500.0, 3300.0, L.r1);
    L.mu0 = mantle(2.9e11, 0.7e11, L.r0);
    L.mu1 = mantle(2.9e11, 0.7e11, L.r1);
    L.kappa0 = mantle(6.5e11, 1.3e11, L.r0);
    L.kappa1 = mantle(6.5e11, 1.3e11, L.r1);
    L.viscosity = viscosity[s];
    if (L.viscosity > 0.0 && kelvin_fraction > 0.0) {
      L.kelvin_fraction = kelvin_fraction;
      L.kelvin_viscosity = L.viscosity / kelvin_div;
    }
  }
  // elements in proportion to thickness: the floors (one at least), then the
  // largest remainders
  double want[4];
  int given = 0;
  for (int s = 0; s < 4; ++s) {
    want[s] = elements * (edges[s + 1] - edges[s]) / surface;
    out[s].elements = std::max(1, static_cast<int>(std::floor(want[s])));
    given += out[s].elements;
  }
  for (; given < elements; ++given) {
    int pick = 0;
    for (int s = 1; s < 4; ++s)
      if (want[s] - out[s].elements > want[pick] - out[pick].elements) pick = s;
    ++out[pick].elements;
  }
  return out;
}

}  // namespace sl3dgpu::host
