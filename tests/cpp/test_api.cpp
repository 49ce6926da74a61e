// The C++ library API (include/sl3dgpu.hpp) used the way the reference's
// C++ callers use theirs, checked against the oracle (linked beside the
// library as the checker).
//
//   test_api host   argument checks and error mapping, no GPU call
//   test_api gpu    one degree's system, the band solvers, three Sdirk2
//                   steps of the 3D operator and one lateral static solve,
//                   each against the oracle on the same inputs; a driver's
//                   own iteration through OpenStep against the operator's
//                   step, the GridCoupling maps' identities, the static
//                   problem's Force / Apply / LoadForces, GRDSolver's
//                   identities and Evolution3D's migrating and frozen runs
//
// Prints one line per check and exits non-zero on the first failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <optional>
#include <span>
#include <random>
#include <string>
#include <vector>

#include "sl3dgpu.hpp"

extern "C" {
struct oracle_v3d;
struct oracle_state;
int oracle_standard_earth(int elements, double kelvin_fraction, double kelvin_div, sl3dgpu_layer* out);
int oracle_degree_band(const sl3dgpu_layer* layers, int nlayers, int ngll, double eps, int relaxed, int scheme,
                       double dt, int toroidal, int l, double* out, int* n, int* kd);
int oracle_band_cholesky_factor(double* ab, int n, int kd);
void oracle_band_cholesky_solve(const double* ab, int n, int kd, double* b, int nrhs);
int oracle_band_lu_factor(double* ab, int n, int kl, int ku, int* pivots);
void oracle_band_lu_solve(const double* ab, int n, int kl, int ku, const int* pivots, double* b, int nrhs);
oracle_v3d* oracle_v3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options* options);
void oracle_v3d_destroy(oracle_v3d* h);
int oracle_v3d_node_count(const oracle_v3d* h);
void oracle_v3d_nodes(const oracle_v3d* h, double* radius, int* element);
void oracle_v3d_grid(const oracle_v3d* h, int* ntheta, int* nphi, double* theta, double* weights);
void oracle_v3d_set_delta(oracle_v3d* h, const double* samples);
oracle_state* oracle_v3d_zero_state(const oracle_v3d* h);
void oracle_v3d_free_state(oracle_state* s);
int oracle_v3d_step(oracle_v3d* h, oracle_state* state, double dt, int scheme, const double* load0,
                    const double* load1, sl3dgpu_step_info* info);
void oracle_v3d_surface(const oracle_v3d* h, int component, double* out);
oracle_v3d* oracle_ep3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_ep3d_options* o);
void oracle_ep3d_set_moduli(oracle_v3d* h, const double* d_mu, const double* d_kappa);
int oracle_ep3d_solve_lateral(oracle_v3d* h, const double* load, double rtol, int max_iterations,
                              sl3dgpu_step_info* info);
int oracle_v3d_residual_history(const oracle_v3d* h, double* out, int capacity);
}

namespace {

using sl3dpp::Complex;
int failures = 0;

void Expect(bool ok, const std::string& what) {
  std::printf("%s %s\n", ok ? "ok  " : "FAIL", what.c_str());
  if (!ok) ++failures;
}

template <class E, class F>
void ExpectThrow(F&& f, const std::string& what) {
  try {
    f();
  } catch (const E&) {
    Expect(true, what);
    return;
  } catch (const std::exception& e) {
    Expect(false, what + " (threw another exception: " + e.what() + ")");
    return;
  }
  Expect(false, what + " (nothing thrown)");
}

double Rel(std::span<const double> a, std::span<const double> b) {
  double diff = 0.0, size = 0.0;
  for (std::size_t i = 0; i < a.size(); ++i) {
    diff = std::max(diff, std::abs(a[i] - b[i]));
    size = std::max(size, std::abs(b[i]));
  }
  return diff / std::max(size, 1e-300);
}

double Rel(std::span<const Complex> a, std::span<const Complex> b) {
  double diff = 0.0, size = 0.0;
  for (std::size_t i = 0; i < a.size(); ++i) {
    diff = std::max(diff, std::abs(a[i] - b[i]));
    size = std::max(size, std::abs(b[i]));
  }
  return a.size() == b.size() ? diff / std::max(size, 1e-300) : 1.0;
}

double Rel(const std::map<int, std::vector<Complex>>& a, std::span<const Complex> flat) {
  double diff = 0.0, size = 0.0;
  for (const auto& [l, col] : a)
    for (int m = 0; m <= l; ++m) {
      diff = std::max(diff, std::abs(col[m] - flat[l * (l + 1) / 2 + m]));
      size = std::max(size, std::abs(flat[l * (l + 1) / 2 + m]));
    }
  return diff / std::max(size, 1e-300);
}

bool SameLayers(const std::vector<sl3dgpu_layer>& a, const std::vector<sl3dgpu_layer>& b) {
  if (a.size() != b.size()) return false;
  for (std::size_t i = 0; i < a.size(); ++i)
    if (std::memcmp(&a[i], &b[i], sizeof(sl3dgpu_layer)) != 0) return false;
  return true;
}

// -- no GPU call ------------------------------------------------------------------------------------

void Host() {
  const auto body = sl3dpp::Rheology::Standard(20);
  std::vector<sl3dgpu_layer> want(4);
  want.resize(oracle_standard_earth(20, 0.0, 10.0, want.data()));
  Expect(SameLayers(body.layers, want), "Rheology::Standard has the oracle's layers");

  ExpectThrow<std::invalid_argument>([] { sl3dpp::gpu::Check(SL3DGPU_ERR_ARGUMENT); },
                                     "an argument status throws std::invalid_argument");
  for (int status : {SL3DGPU_ERR_CUDA, SL3DGPU_ERR_RUNTIME, SL3DGPU_ERR_UNCONVERGED, SL3DGPU_ERR_WAIT})
    ExpectThrow<std::runtime_error>([status] { sl3dpp::gpu::Check(status); },
                                    "status " + std::to_string(status) + " throws std::runtime_error");
  ExpectThrow<std::invalid_argument>([&] { sl3dpp::DegreeOperator op(body, -1); },
                                     "DegreeOperator refuses a negative degree");
  ExpectThrow<std::invalid_argument>([&] { sl3dpp::ToroidalOperator op(body, 0); },
                                     "ToroidalOperator refuses degree 0");
  ExpectThrow<std::invalid_argument>([] { sl3dpp::Rheology::Standard(2); },
                                     "the standard Earth needs four elements");
  std::vector<double> ab(10);
  ExpectThrow<std::invalid_argument>([&] { sl3dpp::detail::BandCholeskyFactor(ab, 10, 3); },
                                     "a band span shorter than (kd + 1) n is refused");

  auto load = [](int l, double t) -> std::optional<std::vector<Complex>> {
    if (l > 3) return std::nullopt;
    std::vector<Complex> c(l + 1);
    for (int m = 0; m <= l; ++m) c[m] = Complex(t * (l + 1), m);
    return c;
  };
  const auto flat = sl3dpp::gpu::Flatten(load, 5, 2.0);
  const auto cols = sl3dpp::gpu::Columns(flat, 5);
  Expect(flat.size() == 21 && flat[3 * 4 / 2 + 2] == Complex(8.0, 2.0) && flat[4 * 5 / 2] == Complex{} &&
             cols.at(3)[2] == Complex(8.0, 2.0) && cols.at(5).size() == 6,
         "load callables flatten to the (l, m >= 0) layout and back");
  auto wrong = [](int l, double) -> std::optional<std::vector<Complex>> { return std::vector<Complex>(l + 2); };
  ExpectThrow<std::invalid_argument>([&] { (void)sl3dpp::gpu::Flatten(wrong, 4, 0.0); },
                                     "a load callable with the wrong column count is refused");
}

// -- on the GPU -----------------------------------------------------------------------------------

void Bands() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  const int n = 300, kd = 9, nrhs = 3;
  std::vector<double> ab(static_cast<std::size_t>(kd + 1) * n);
  for (int j = 0; j < n; ++j)
    for (int t = 0; t <= kd; ++t) ab[j * (kd + 1) + t] = t == kd ? 4.0 * kd : u(rng);
  std::vector<double> b(static_cast<std::size_t>(n) * nrhs);
  for (auto& x : b) x = u(rng);
  auto ab1 = ab, ab2 = ab;
  auto b1 = b, b2 = b;
  Expect(sl3dpp::detail::BandCholeskyFactor(ab1, n, kd) == 0 && oracle_band_cholesky_factor(ab2.data(), n, kd) == 0,
         "BandCholeskyFactor succeeds on an SPD band");
  sl3dpp::detail::BandCholeskySolve(ab1, n, kd, b1, nrhs);
  oracle_band_cholesky_solve(ab2.data(), n, kd, b2.data(), nrhs);
  Expect(Rel(b1, b2) < 1e-12, "BandCholeskySolve matches the oracle");

  const int kl = 4, ku = 5, ld = 2 * kl + ku + 1;
  std::vector<double> lu(static_cast<std::size_t>(ld) * n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - ku); i <= std::min(n - 1, j + kl); ++i) lu[j * ld + kl + ku + i - j] = u(rng);
  auto lu1 = lu, lu2 = lu;
  std::vector<int> p1(n), p2(n);
  b1 = b;
  b2 = b;
  const int i1 = sl3dpp::detail::BandLuFactor(lu1, n, kl, ku, p1);
  const int i2 = oracle_band_lu_factor(lu2.data(), n, kl, ku, p2.data());
  Expect(i1 == 0 && i2 == 0 && p1 == p2, "BandLuFactor pivots as the oracle");
  sl3dpp::detail::BandLuSolve(lu1, n, kl, ku, p1, b1, nrhs);
  oracle_band_lu_solve(lu2.data(), n, kl, ku, p2.data(), b2.data(), nrhs);
  Expect(Rel(b1, b2) < 1e-11, "BandLuSolve matches the oracle");
}

template <class Op>
void CheckDegree(const sl3dpp::Rheology& body, const Op& op, int l, int toroidal, const std::string& name) {
  int n = 0, kd = 0;
  const int layers = static_cast<int>(body.layers.size());
  oracle_degree_band(body.layers.data(), layers, body.ngll, 1e-8, 0, 1, 0.0, toroidal, l, nullptr, &n, &kd);
  std::vector<double> want(static_cast<std::size_t>(kd + 1) * n);
  oracle_degree_band(body.layers.data(), layers, body.ngll, 1e-8, 0, 1, 0.0, toroidal, l, want.data(), &n, &kd);
  Expect(op.DofCount() == n && op.Bandwidth() == kd && Rel(op.Band(), want) < 1e-13,
         name + " l=" + std::to_string(l) + " band matches the oracle");
  std::mt19937_64 rng(l);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::vector<double> b(2 * static_cast<std::size_t>(n));
  for (auto& x : b) x = u(rng);
  if (toroidal && l == 1) return;  // the rigid rotation's gauge row is pinned: K Solve(b) = b off it only
  Expect(Rel(op.Apply(op.Solve(b, 2), 2), b) < 1e-9, name + " l=" + std::to_string(l) + " K Solve(b) = b");
}

void Degree(const sl3dpp::Rheology& body) {
  for (int l : {0, 1, 3, 12}) CheckDegree(body, sl3dpp::DegreeOperator(body, l), l, 0, "DegreeOperator");
  for (int l : {1, 4}) CheckDegree(body, sl3dpp::ToroidalOperator(body, l), l, 1, "ToroidalOperator");
  const sl3dpp::DegreeOperator op(body, 2);
  Expect(op.SurfaceDof(sl3dpp::Component::U) == op.Dof(20 * (body.ngll - 1), sl3dpp::Component::U),
         "DegreeOperator's surface U is the top node's");
}

// delta(r, theta, phi): a lateral pattern below the lid, as a reference caller writes it
double Delta(double r, double theta, double phi) {
  const double depth = 1.0 - r;
  const double radial = depth > 0.016 ? std::exp(-depth / 0.2) : 0.0;
  return 0.6 * radial *
         (std::sin(theta) * std::cos(theta) * std::cos(phi) + 0.4 * std::pow(std::sin(theta), 2) * std::sin(2 * phi));
}

void Step(const sl3dpp::Rheology& body) {
  const int lmax = 12;
  sl3dpp::Viscoelastic3D::Options options;
  options.rtol = 1e-10;
  options.max_iterations = 60;
  sl3dpp::Viscoelastic3D op(body, lmax, Delta, options);

  sl3dgpu_v3d_options o{};
  o.lmax = lmax;
  o.ngll = body.ngll;
  o.eps = options.eps;
  o.oversampling = options.oversampling;
  o.max_iterations = options.max_iterations;
  o.rtol = options.rtol;
  o.damping = options.damping;
  o.anderson_memory = options.anderson_memory;
  o.anderson_rate = options.anderson_rate;
  o.solve_rtol = options.solve_rtol;
  o.solve_max_iterations = options.solve_max_iterations;
  oracle_v3d* ref = oracle_v3d_create(body.layers.data(), static_cast<int>(body.layers.size()), &o);
  const int P = oracle_v3d_node_count(ref);
  int nt = 0, np = 0;
  oracle_v3d_grid(ref, &nt, &np, nullptr, nullptr);
  std::vector<double> radius(P), theta(nt);
  oracle_v3d_nodes(ref, radius.data(), nullptr);
  oracle_v3d_grid(ref, nullptr, nullptr, theta.data(), nullptr);
  Expect(P == op.NodeCount() && Rel(op.Radii(), radius) < 1e-14, "Viscoelastic3D has the oracle's memory nodes");
  std::vector<double> samples;
  samples.reserve(static_cast<std::size_t>(P) * nt * np);
  for (int p = 0; p < P; ++p)
    for (int j = 0; j < nt; ++j)
      for (int k = 0; k < np; ++k) samples.push_back(Delta(radius[p], theta[j], 6.283185307179586476925286766559 * k / np));
  oracle_v3d_set_delta(ref, samples.data());

  // a zonal load growing linearly to 1000 kg m^-2 at degree 2 over 1500 yr,
  // with a smaller sectoral part
  const double year = 3.15576e7 / op.TimeScale();
  const double sigma = 1e3 / op.SurfaceDensityScale();
  auto load = [&](int l, double t) -> std::optional<std::vector<Complex>> {
    if (l < 2 || l > 6) return std::nullopt;
    std::vector<Complex> c(l + 1);
    c[0] = sigma * t / (1500.0 * year) / l;
    c[2] = Complex(0.2, -0.1) * c[0];
    return c;
  };
  auto state = op.ZeroState();
  oracle_state* rs = oracle_v3d_zero_state(ref);
  const double dt = 500.0 * year;
  for (int n = 0; n < 3; ++n) {
    const auto l0 = sl3dpp::gpu::Flatten(load, lmax, state.t), l1 = sl3dpp::gpu::Flatten(load, lmax, state.t + dt);
    sl3dgpu_step_info ri{};
    oracle_v3d_step(ref, rs, dt, 2, reinterpret_cast<const double*>(l0.data()),
                    reinterpret_cast<const double*>(l1.data()), &ri);
    const auto info = op.Step(state, dt, sl3dpp::Scheme::Sdirk2, load);
    Expect(info.converged && ri.converged && std::abs(info.iterations - ri.iterations) <= 1,
           "step " + std::to_string(n) + " converges in the oracle's passes (" + std::to_string(info.iterations) +
               " / " + std::to_string(ri.iterations) + ")");
    for (auto [c, name] : {std::pair{sl3dpp::Component::U, "U"}, std::pair{sl3dpp::Component::Phi, "phi"}}) {
      std::vector<Complex> want(static_cast<std::size_t>(lmax + 1) * (lmax + 2) / 2);
      oracle_v3d_surface(ref, static_cast<int>(c), reinterpret_cast<double*>(want.data()));
      const double err = Rel(op.Surface(c), want);
      Expect(err < 1e-10, "step " + std::to_string(n) + " surface " + name + " matches the oracle (" +
                              std::to_string(err) + ")");
    }
  }
  Expect(std::abs(state.t - 3 * dt) < 1e-12 * dt, "the state's time advanced by the steps");
  oracle_v3d_free_state(rs);
  oracle_v3d_destroy(ref);
}

void Static(const sl3dpp::Rheology& body) {
  const int lmax = 8;
  sl3dpp::ElasticPerturbation3D op(body, lmax);
  const sl3dgpu_ep3d_options o{lmax, body.ngll, 1e-8, 1.5};
  oracle_v3d* ref = oracle_ep3d_create(body.layers.data(), static_cast<int>(body.layers.size()), &o);
  const auto radius = op.Radii();
  const auto theta = op.CoLatitudes();
  const int np = op.NumberOfLongitudes();
  std::vector<double> dMu, dKappa;
  for (double r : radius)
    for (double t : theta)
      for (int k = 0; k < np; ++k) {
        const double p = 6.283185307179586476925286766559 * k / np;
        dMu.push_back(0.02 * (0.5 + r * r) * (std::sin(t) * std::cos(t) * std::cos(p) + 0.3 * std::cos(2 * p)));
        dKappa.push_back(0.02 * (1.0 - 0.5 * r) * (std::cos(t) * std::sin(p) + 0.2));
      }
  std::vector<Complex> load(static_cast<std::size_t>(lmax + 1) * (lmax + 2) / 2);
  for (int l = 0; l <= lmax; ++l)
    for (int m = 0; m <= l; ++m) load[l * (l + 1) / 2 + m] = 1e-4 * Complex(1.0 / (1.0 + l), m == 0 ? 0.0 : 0.3 * m);
  const auto info = op.SolveLateral(load, dMu, dKappa, {.rtol = 1e-12, .max_iterations = 200});
  oracle_ep3d_set_moduli(ref, dMu.data(), dKappa.data());
  sl3dgpu_step_info ri{};
  oracle_ep3d_solve_lateral(ref, reinterpret_cast<const double*>(load.data()), 1e-12, 200, &ri);
  std::vector<double> history(oracle_v3d_residual_history(ref, nullptr, 0));
  oracle_v3d_residual_history(ref, history.data(), static_cast<int>(history.size()));
  bool same = info.residuals.size() == history.size();
  for (std::size_t i = 0; same && i < history.size(); ++i)
    same = history[i] < 1e-9 || std::abs(info.residuals[i] - history[i]) < 1e-6 * history[i];
  Expect(info.converged && ri.converged && std::abs(info.iterations - ri.iterations) <= 1,
         "SolveLateral converges in the oracle's iterations (" + std::to_string(info.iterations) + " / " +
             std::to_string(ri.iterations) + ")");
  Expect(same, "SolveLateral's residuals are the oracle's (" + std::to_string(info.residuals.size()) + " / " +
                   std::to_string(history.size()) + ")");
  for (auto c : {sl3dpp::Component::U, sl3dpp::Component::V, sl3dpp::Component::Phi}) {
    std::vector<Complex> want(load.size());
    oracle_v3d_surface(ref, static_cast<int>(c), reinterpret_cast<double*>(want.data()));
    const double err = Rel(op.Surface(c), want);
    Expect(err < 1e-9, "SolveLateral surface " + std::to_string(static_cast<int>(c)) + " matches the oracle (" +
                           std::to_string(err) + ")");
  }
  ExpectThrow<std::invalid_argument>([&] { op.Respond(std::span<const double>(dMu).first(5), {}); },
                                     "a moduli direction off the nodes' grids is refused");
  oracle_v3d_destroy(ref);
}

// A driver's own within-step iteration through OpenStep -- StartStep,
// then Respond / AddChannels / StrainOf / RelativeChange until the change is
// under the tolerance, then Finish -- is the operator's own plain fixed
// point step for step (the same passes in the same order); the
// GridCoupling maps keep their identities.
void OpenStepAndCoupling(const sl3dpp::Rheology& body) {
  const int lmax = 10;
  sl3dpp::Viscoelastic3D::Options options;
  options.rtol = 1e-11;
  options.max_iterations = 80;
  options.anderson_memory = 0;
  sl3dpp::Viscoelastic3D driver(body, lmax, Delta, options), plain(body, lmax, Delta, options);
  const double year = 3.15576e7 / plain.TimeScale();
  const double sigma = 1e3 / plain.SurfaceDensityScale();
  auto load = [&](int l, double t) -> std::optional<std::vector<Complex>> {
    if (l < 2 || l > 6) return std::nullopt;
    std::vector<Complex> c(l + 1);
    c[0] = sigma * (1.0 + t / (1500.0 * year)) / l;
    c[1] = Complex(0.1, 0.3) * c[0];
    return c;
  };
  const double h = 300.0 * year;
  auto sd = driver.ZeroState(), sp = plain.ZeroState();
  std::vector<Complex> converged;
  for (int n = 0; n < 2; ++n) {
    const auto l0 = sl3dpp::gpu::Flatten(load, lmax, sd.t), l1 = sl3dpp::gpu::Flatten(load, lmax, sd.t + h);
    const auto info = plain.Step(sp, h, sl3dpp::Scheme::BackwardEuler, load);
    auto step = driver.StartStep(sd, h, sl3dpp::Scheme::BackwardEuler, l0);
    auto s = step.StartStrain();
    int passes = 0;
    for (bool first = true;; first = false) {
      step.Respond(first ? std::span<const Complex>{} : std::span<const Complex>(s));
      step.AddChannels(l1);
      auto next = step.StrainOf();
      const double change = step.RelativeChange(next, s);
      ++passes;
      s = std::move(next);
      if (change <= options.rtol || passes >= options.max_iterations) break;
    }
    converged = s;
    step.Finish(s);
    Expect(info.converged && passes == info.iterations,
           "open step " + std::to_string(n) + " takes the operator's passes (" + std::to_string(passes) + " / " +
               std::to_string(info.iterations) + ")");
    for (auto c : {sl3dpp::Component::U, sl3dpp::Component::Phi}) {
      const auto a = driver.Surface(c), b = plain.Surface(c);
      double diff = 0.0;
      for (const auto& [l, col] : a)
        for (std::size_t m = 0; m < col.size(); ++m) diff = std::max(diff, std::abs(col[m] - b.at(l)[m]));
      Expect(diff == 0.0, "open step " + std::to_string(n) + " surface " + std::to_string(static_cast<int>(c)) +
                              " is the operator's step bit for bit");
    }
  }
  Expect(std::abs(sd.t - sp.t) == 0.0, "Finish advanced the state's time as Step did");
  // GridCoupling: Analyse(Synthesise(s)) = s for band-limited s (the grid
  // oversampled); the degree forces linear; the strain of zero solutions zero
  const auto layout = driver.GetLayout();
  Expect(static_cast<long long>(converged.size()) == layout.spectral, "a strain has the layout's spectral size");
  const auto back = driver.Analyse(driver.Synthesise(converged));
  double top = 0.0, err = 0.0;
  for (std::size_t i = 0; i < converged.size(); ++i) {
    top = std::max(top, std::abs(converged[i]));
    err = std::max(err, std::abs(back[i] - converged[i]));
  }
  Expect(err < 1e-12 * top, "GridCoupling Analyse(Synthesise(s)) = s (" + std::to_string(err / top) + ")");
  std::vector<Complex> scaled(converged);
  for (auto& v : scaled) v *= 2.5;
  const auto [f1s, f1t] = driver.DegreeForces(converged);
  const auto [f2s, f2t] = driver.DegreeForces(scaled);
  double ftop = 0.0, ferr = 0.0;
  for (std::size_t i = 0; i < f1s.size(); ++i) {
    ftop = std::max(ftop, std::abs(f2s[i]));
    ferr = std::max(ferr, std::abs(f2s[i] - 2.5 * f1s[i]));
  }
  Expect(ferr <= 1e-14 * ftop && static_cast<long long>(f1t.size()) == layout.toroidal,
         "GridCoupling degree forces are linear");
  const auto zero = driver.StrainOfSolutions(std::vector<Complex>(layout.spheroidal),
                                             std::vector<Complex>(layout.toroidal));
  double zmax = 0.0;
  for (const auto& v : zero) zmax = std::max(zmax, std::abs(v));
  Expect(zmax == 0.0, "the strain of zero solutions is zero");
  ExpectThrow<std::invalid_argument>([&] { (void)driver.Synthesise(std::vector<Complex>(3)); },
                                     "a strain off the layout is refused");
}

// ElasticPerturbation3D's Force, Apply and LoadForces on the lateral
// solution: Apply(y) = LoadForces(load) to the solve's tolerance, Force linear.
void StaticForceApply(const sl3dpp::Rheology& body) {
  const int lmax = 8;
  sl3dpp::ElasticPerturbation3D op(body, lmax);
  const auto radius = op.Radii();
  const auto theta = op.CoLatitudes();
  const int np = op.NumberOfLongitudes();
  std::vector<double> dMu, dKappa;
  for (double r : radius)
    for (double t : theta)
      for (int k = 0; k < np; ++k) {
        const double p = 6.283185307179586476925286766559 * k / np;
        dMu.push_back(0.03 * r * (std::sin(t) * std::cos(p) + 0.2));
        dKappa.push_back(0.01 * (std::cos(t) + 0.5));
      }
  std::vector<Complex> load(static_cast<std::size_t>(lmax + 1) * (lmax + 2) / 2);
  for (int l = 1; l <= lmax; ++l)
    for (int m = 0; m <= l; ++m) load[l * (l + 1) / 2 + m] = 1e-4 * Complex(1.0 / (1.0 + l), m == 0 ? 0.0 : 0.2);
  const auto info = op.SolveLateral(load, dMu, dKappa, {.rtol = 1e-12, .max_iterations = 300});
  const auto y = op.Solution();
  const auto applied = op.Apply(y), forces = op.LoadForces(load);
  double top = 0.0, err = 0.0;
  for (std::size_t i = 0; i < y.size(); ++i) {
    top = std::max(top, std::abs(forces[i]));
    err = std::max(err, std::abs(applied[i] - forces[i]));
  }
  Expect(info.converged && err < 1e-9 * top,
         "ElasticPerturbation3D Apply(y) = LoadForces for SolveLateral's y (" + std::to_string(err / top) + ")");
  std::vector<Complex> twice(y);
  for (auto& v : twice) v *= 2.0;
  const auto f1 = op.Force(y), f2 = op.Force(twice);
  double ftop = 0.0, ferr = 0.0;
  for (std::size_t i = 0; i < f1.size(); ++i) {
    ftop = std::max(ftop, std::abs(f2[i]));
    ferr = std::max(ferr, std::abs(f2[i] - 2.0 * f1[i]));
  }
  Expect(ftop > 0.0 && ferr <= 1e-14 * ftop, "ElasticPerturbation3D Force is linear");
}

// GRDSolver on the GPU through the class API: the rigid-earth eustatic
// limit and the ocean gaining the mass the load lost (the generalised solve,
// tests/TestSeaLevel.cpp:135-206's identities); the nonlinear solve's
// flotation, its carried load without mass, and where no shoreline moves the
// linear solve under the grounded ice change.
void SeaLevel() {
  const int lmax = 14;  // at 16 the 5% thinning below floats a coastal cell
  sl3dpp::GRDSolver::Body body;
  for (int l = 0; l <= lmax; ++l) {
    body.h.push_back(l > 0 ? -1.2 / (l + 1.0) : 0.0);
    body.k.push_back(l > 0 ? -0.5 / (l + 1.0) : 0.0);
    body.l.push_back(l > 0 ? 0.3 / (l + 1.0) : 0.0);
  }
  sl3dpp::GRDSolver solver(lmax, body);
  const auto theta = solver.Grid().CoLatitudes();
  const int np = solver.Grid().NumberOfLongitudes();
  const std::size_t n = solver.FieldSize();
  std::vector<double> sea(n), ice(n), load(n);
  for (std::size_t j = 0; j < theta.size(); ++j)
    for (int k = 0; k < np; ++k) {
      const double t = theta[j], p = 6.283185307179586476925286766559 * k / np;
      sea[j * np + k] = 0.3 * (0.5 * std::cos(2 * t) + 0.3 + 0.3 * std::sin(2 * p) * std::sin(t));
      ice[j * np + k] = 0.75 * std::exp(-std::pow(t / 0.5, 4));
      load[j * np + k] = -0.2 * std::exp(-std::pow((t - 0.3) / 0.2, 2));
    }
  const auto state = solver.MakeState(ice, sea);
  bool flotation = true;
  for (std::size_t i = 0; i < n; ++i)
    flotation = flotation && state.oceanFunction[i] == (1.0 * sea[i] - 0.917 * ice[i] > 0.0 ? 1.0 : 0.0);
  Expect(flotation && state.oceanArea > 0.0, "GRDSolver MakeState takes flotation's ocean function");
  // the ocean gains what the load lost
  std::vector<double> land(n);
  for (std::size_t i = 0; i < n; ++i) land[i] = load[i] * (1.0 - state.oceanFunction[i]);
  sl3dpp::GRDSolver::GeneralisedForcing forcing;
  forcing.directLoad = land;
  const auto r = solver.SolveGeneralised(state, forcing, {.rtol = 1e-12, .max_iterations = 300, .anderson_memory = 5});
  std::vector<double> gained(n);
  for (std::size_t i = 0; i < n; ++i) gained[i] = state.oceanFunction[i] * r.relativeSeaLevelChange[i];
  const double lost = solver.IntegrateSurface(land), got = solver.IntegrateSurface(gained);
  Expect(r.converged && std::abs(got + lost) < 1e-10 * std::abs(lost),
         "GRDSolver SolveGeneralised: the ocean gains what the load lost");
  // a thinning marine cap floats; the carried load has no mass; the final
  // state is flotation's
  sl3dpp::GRDSolver::NonlinearForcing melt;
  melt.iceThicknessChange.resize(n);
  for (std::size_t i = 0; i < n; ++i) melt.iceThicknessChange[i] = -0.6 * ice[i];
  const auto nl = solver.SolveNonlinear(state, melt, {.rtol = 1e-12, .max_iterations = 200, .anderson_memory = 0});
  std::size_t floated = 0;
  bool final = true;
  for (std::size_t i = 0; i < n; ++i) {
    floated += state.oceanFunction[i] == 0.0 && nl.finalState.oceanFunction[i] == 1.0;
    final = final && nl.finalState.oceanFunction[i] ==
                         (1.0 * nl.finalState.seaLevel[i] - 0.917 * nl.finalState.iceThickness[i] > 0.0 ? 1.0 : 0.0);
  }
  double top = 0.0;
  for (const auto& c : nl.loadCoefficients) top = std::max(top, std::abs(c));
  Expect(nl.response.converged && floated > 0 && final,
         "GRDSolver SolveNonlinear: the thinning cap floats (" + std::to_string(floated) +
             " cells) and the final state is flotation's");
  Expect(std::abs(nl.loadCoefficients[0]) < 1e-10 * top, "GRDSolver SolveNonlinear: the carried load has no mass");
  // a thinning that floats nothing: the linear solve under rho_i (1 - C) dI
  sl3dpp::GRDSolver::NonlinearForcing thin;
  thin.iceThicknessChange.resize(n);
  std::vector<double> grounded(n);
  for (std::size_t i = 0; i < n; ++i) {
    thin.iceThicknessChange[i] = -0.05 * ice[i];
    grounded[i] = 0.917 * (1.0 - state.oceanFunction[i]) * thin.iceThicknessChange[i];
  }
  const auto still = solver.SolveNonlinear(state, thin, {.rtol = 1e-13, .max_iterations = 400, .anderson_memory = 0});
  sl3dpp::GRDSolver::GeneralisedForcing lin;
  lin.directLoad = grounded;
  const auto linear = solver.SolveGeneralised(state, lin, {.rtol = 1e-13, .max_iterations = 400, .anderson_memory = 5});
  Expect(still.finalState.oceanFunction == state.oceanFunction &&
             Rel(still.response.relativeSeaLevelChange, linear.relativeSeaLevelChange) < 1e-10,
         "GRDSolver SolveNonlinear without a moving shoreline is the linear solve");
  ExpectThrow<std::invalid_argument>([&] { (void)solver.MakeState(std::vector<double>(3), sea); },
                                     "a state off the grid is refused");
}

// Evolution3D through the class API: under ice that does not change and a
// direct load that moves no shoreline, the migrating run is the frozen one
// (tests/TestEvolution3D.cpp:486-507's check, at its 1e-7).
void Evolution(const sl3dpp::Rheology& body) {
  const int lmax = 8;
  sl3dpp::Viscoelastic3D::Options options;
  options.rtol = 1e-12;
  options.max_iterations = 80;
  sl3dpp::Viscoelastic3D a(body, lmax, Delta, options), b(body, lmax, Delta, options);
  sl3dpp::Evolution3D moving(a), frozen(b);
  const std::size_t n = moving.OceanFieldSize();
  sl3dpp::SurfaceGrid grid(lmax, 0, 1.0);
  const auto theta = grid.CoLatitudes();
  const int np = grid.NumberOfLongitudes();
  std::vector<double> sea(n), ice(n), cap(n);
  const double length = a.LengthScale();
  for (std::size_t j = 0; j < theta.size(); ++j)
    for (int k = 0; k < np; ++k) {
      const double t = theta[j], p = 6.283185307179586476925286766559 * k / np;
      double f = 0.5 * std::cos(2 * t) + 0.3 + 0.3 * std::sin(2 * p) * std::sin(t);
      if (std::abs(f) < 0.05) f = f < 0.0 ? -0.05 : 0.05;
      sea[j * np + k] = 1500.0 * f / length;
      ice[j * np + k] = 2500.0 * std::exp(-std::pow(t / 0.45, 4)) / length;
      cap[j * np + k] = t < 0.26 ? 20.0 * 917.0 / a.SurfaceDensityScale() : 0.0;
    }
  sl3dpp::Evolution3D::Ocean c;
  c.rtol = 1e-12;
  c.max_iterations = 400;
  c.max_nonlinear_iterations = 400;
  moving.SetMigrating(ice, sea, {}, c);
  std::vector<double> ocean(n);
  for (std::size_t i = 0; i < n; ++i) ocean[i] = 1000.0 * sea[i] - 917.0 * ice[i] > 0.0 ? 1.0 : 0.0;
  frozen.SetOcean(ocean, c);
  const double year = 3.15576e7 / a.TimeScale();
  std::vector<double> times;
  for (int k = 0; k < 4; ++k) times.push_back(500.0 * year * k);
  auto loadAt = [&](double t) {
    std::vector<double> out(cap);
    for (auto& v : out) v *= t / (1500.0 * year);
    return out;
  };
  const auto m = moving.RunMigrating(times, [&](double) { return ice; }, loadAt);
  const auto f = frozen.RunOcean(times, loadAt);
  bool same = m.size() == f.size();
  double worst = 0.0;
  for (std::size_t k = 0; same && k < m.size(); ++k) {
    same = m[k].oceanFunction == ocean;
    worst = std::max({worst, Rel(m[k].U, f[k].U), Rel(m[k].seaLevel, f[k].seaLevel)});
  }
  Expect(same && worst < 1e-7, "Evolution3D RunMigrating under still ice is RunOcean's frozen run (" +
                                   std::to_string(worst) + ")");
}

// AdjointSolver3D: the load kernels pair with the loads to the objective of
// the forward run (Evolution3D::Run) under them; the kernel in delta is a
// finite density wherever the gradient is.
void Adjoint(const sl3dpp::Rheology& body) {
  const int lmax = 8;
  sl3dpp::Viscoelastic3D::Options options;
  options.rtol = 1e-12;
  options.max_iterations = 80;
  sl3dpp::Viscoelastic3D op(body, lmax, Delta, options);
  sl3dpp::Evolution3D evolution(op);
  const double year = 3.15576e7 / op.TimeScale();
  std::vector<double> times;
  for (int k = 0; k < 4; ++k) times.push_back(500.0 * year * k);
  auto load = [&](int l, double t) -> std::optional<std::vector<Complex>> {
    std::vector<Complex> c(l + 1);
    for (int m = 0; m <= l; ++m)
      c[m] = Complex(std::cos(1.0 + l + 0.3 * m + t / year), m == 0 ? 0.0 : std::sin(2.0 * l - m)) / (1.0 + l * l);
    return c;
  };
  const std::size_t lm = static_cast<std::size_t>(lmax + 1) * (lmax + 2) / 2;
  std::map<std::size_t, sl3dpp::Measurement3D> measurements;
  for (std::size_t node : {std::size_t{1}, std::size_t{3}}) {
    auto& m = measurements[node];
    m.displacementDual.resize(lm);
    m.potentialDual.resize(lm);
    for (std::size_t i = 0; i < lm; ++i) {
      m.displacementDual[i] = Complex(std::sin(0.7 * static_cast<double>(i + node)), 0.0);
      m.potentialDual[i] = Complex(std::cos(0.3 * static_cast<double>(i) - static_cast<double>(node)), 0.0);
    }
  }
  const auto kernels = sl3dpp::AdjointSolver3D(evolution).FirstOrderKernels(times, load, measurements);
  const auto run = evolution.Run(times, load);
  auto pair = [&](const std::vector<Complex>& a, const std::vector<Complex>& b) {
    double sum = 0.0;
    for (int l = 0, i = 0; l <= lmax; ++l)
      for (int m = 0; m <= l; ++m, ++i) sum += (m == 0 ? 1.0 : 2.0) * (a[i] * std::conj(b[i])).real();
    return sum;
  };
  double objective = 0.0, paired = 0.0;
  for (const auto& [node, m] : measurements)
    objective += pair(m.displacementDual, run[node].U) + pair(m.potentialDual, run[node].phi);
  for (std::size_t k = 0; k < times.size(); ++k) {
    std::vector<Complex> flat;
    for (int l = 0; l <= lmax; ++l) {
      const auto c = *load(l, times[k]);
      flat.insert(flat.end(), c.begin(), c.end());
    }
    paired += pair(kernels.directLoadKernels[k], flat);
  }
  bool finite = kernels.logViscosityKernel3D.size() == op.GridValues();
  double largest = 0.0;
  for (double v : kernels.logViscosityKernel3D) {
    finite = finite && std::isfinite(v);
    largest = std::max(largest, std::abs(v));
  }
  Expect(std::abs(kernels.objective - objective) < 1e-10 * std::abs(objective) &&
             std::abs(paired - objective) < 1e-8 * std::abs(objective) && finite && largest > 0.0,
         "AdjointSolver3D load kernels pair with the loads to the forward run's objective (" +
             std::to_string(std::abs(paired - objective) / std::abs(objective)) + ")");
  // TangentLinearSolver3D along a log-viscosity direction: the objective's
  // derivative is the gradient paired with it
  std::vector<double> direction(op.GridValues());
  for (std::size_t x = 0; x < direction.size(); ++x) direction[x] = std::sin(0.37 * static_cast<double>(x % 977));
  const auto tangent = sl3dpp::TangentLinearSolver3D(evolution).Run(times, load, direction);
  double derivative = 0.0, predicted = 0.0;
  for (const auto& [node, m] : measurements)
    derivative += pair(m.displacementDual, tangent.U[node]) + pair(m.potentialDual, tangent.phi[node]);
  for (std::size_t x = 0; x < direction.size(); ++x) predicted += kernels.deltaGradient[x] * direction[x];
  Expect(std::abs(derivative - predicted) < 1e-8 * std::max(std::abs(derivative), std::abs(predicted)),
         "TangentLinearSolver3D pairs with AdjointSolver3D's gradient (" +
             std::to_string(std::abs(derivative - predicted) / std::abs(predicted)) + ")");
}

}  // namespace

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "host";
  try {
    Host();
    if (mode == "gpu") {
      const auto body = sl3dpp::Rheology::Standard(20);
      Bands();
      Degree(body);
      Step(body);
      Static(body);
      OpenStepAndCoupling(body);
      StaticForceApply(body);
      SeaLevel();
      Evolution(body);
      Adjoint(body);
    }
  } catch (const std::exception& e) {
    std::printf("FAIL uncaught %s\n", e.what());
    return 2;
  }
  std::printf("%d failures\n", failures);
  return failures == 0 ? 0 : 1;
}
