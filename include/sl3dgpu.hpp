// sl3dgpu.hpp -- the reference's C++ library API (namespace sl3dpp) over the
// C ABI of sl3dgpu.h, for callers of sl3dpp's 3D viscoelastic hot path.
//
// C++23, header only: every class holds a C handle and every call goes
// through the C ABI (libsl3dgpu.so, CUDA underneath). Names, argument
// meanings and error behaviour follow the reference's headers:
//   detail::BandCholeskyFactor/Solve, BandLuFactor/Solve
//                          include/sl3dpp/detail/BandSolvers.hpp:24-49
//   DegreeOperator, ToroidalOperator
//                          include/sl3dpp/DegreeOperator.hpp:94-384
//   SurfaceGrid            include/sl3dpp/SurfaceGrid.hpp:58-287
//   Viscoelastic3D         include/sl3dpp/Viscoelastic3D.hpp:79-837
//   ElasticPerturbation3D  include/sl3dpp/ElasticPerturbation3D.hpp:77-225
// Errors: a bad argument throws std::invalid_argument, anything else that
// fails std::runtime_error, with the library's text (the reference's
// DegreeOperator.hpp:132-137); a step that does not converge is reported in
// StepInfo, not thrown (Viscoelastic3D.hpp:357-375); the band factorisations
// return LAPACK-style info.
//
// Where the GPU build differs from the reference, said at the member:
//  - the body is a Rheology of linear layers (sl3dgpu_layer) rather than the
//    reference's EarthModel / Material / Rheology chain;
//  - a Step advances its State in place and keeps the end-time solutions in
//    the operator (Surface reads them), where the reference returns a new
//    State and the Solutions;
//  - the load and tide callables are evaluated at the step's start and end
//    times, the Sdirk2 stages taking the linear interpolation between them;
//  - Options carries the GPU forms (mixed precision, warm starts,
//    tensor-core FP64 contractions) beside the reference's fields, and
//    refuses the reference's options this build does not implement.
#pragma once

#include <complex>
#include <functional>
#include <map>
#include <memory>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

#include "sl3dgpu.h"

namespace sl3dpp {

using Complex = std::complex<double>;

enum class Component { U = 0, V = 1, Phi = 2 };
enum class Scheme { ExponentialTrapezoid = 0, BackwardEuler = 1, Sdirk2 = 2 };

namespace gpu {

// A status of the C ABI as the reference's exception.
inline void Check(int status) {
  if (status == SL3DGPU_OK) return;
  const std::string text = sl3dgpu_last_error();
  if (status == SL3DGPU_ERR_ARGUMENT) throw std::invalid_argument(text);
  throw std::runtime_error(text);
}

template <class T, void (*Destroy)(T*)>
struct Deleter {
  void operator()(T* p) const {
    if (p) Destroy(p);
  }
};

// (l, m >= 0) coefficients in the l(l+1)/2 + m layout as the reference's
// per-degree columns.
inline std::map<int, std::vector<Complex>> Columns(std::span<const Complex> flat, int lmax) {
  std::map<int, std::vector<Complex>> out;
  for (int l = 0; l <= lmax; ++l)
    out[l] = std::vector<Complex>(flat.begin() + l * (l + 1) / 2, flat.begin() + l * (l + 1) / 2 + l + 1);
  return out;
}

// A load or tide callable at time t as the flat (l, m >= 0) coefficients
// (degrees it leaves empty are zero).
template <class F>
std::vector<Complex> Flatten(const F& callable, int lmax, double t) {
  std::vector<Complex> out(static_cast<std::size_t>(lmax + 1) * (lmax + 2) / 2, Complex{});
  for (int l = 0; l <= lmax; ++l) {
    const auto columns = callable(l, t);
    if (!columns) continue;
    if (static_cast<int>(columns->size()) != l + 1)
      throw std::invalid_argument("a load callable gives l + 1 columns (m = 0 .. l) per degree");
    for (int m = 0; m <= l; ++m) out[l * (l + 1) / 2 + m] = (*columns)[m];
  }
  return out;
}

}  // namespace gpu

// The body the GPU operators build on: layers with fields linear in radius
// (SI), each split into `elements` spectral elements, and the GLL order.
struct Rheology {
  std::vector<sl3dgpu_layer> layers;
  int ngll = 5;
  // The measured configurations' Earth (sl3dgpu_standard_earth).
  static Rheology Standard(int elements, int ngll = 5, double kelvinFraction = 0.0, double kelvinDiv = 10.0) {
    Rheology r;
    r.layers.resize(4);
    const int count = sl3dgpu_standard_earth(elements, kelvinFraction, kelvinDiv, r.layers.data());
    if (count < 0) gpu::Check(count);
    r.layers.resize(count);
    r.ngll = ngll;
    return r;
  }
};

// -- band solvers --------------------------------------------------------------------------------

namespace detail {

inline int BandCholeskyFactor(std::span<double> ab, int n, int kd) {
  if (ab.size() < static_cast<std::size_t>(kd + 1) * n) throw std::invalid_argument("ab holds (kd + 1) n values");
  const int info = sl3dgpu_band_cholesky_factor(ab.data(), n, kd);
  if (info < 0) gpu::Check(info);
  return info;
}

inline void BandCholeskySolve(std::span<const double> ab, int n, int kd, std::span<double> b, int nrhs) {
  if (b.size() < static_cast<std::size_t>(n) * nrhs) throw std::invalid_argument("b holds n nrhs values");
  gpu::Check(sl3dgpu_band_cholesky_solve(ab.data(), n, kd, b.data(), nrhs));
}

inline int BandLuFactor(std::span<double> ab, int n, int kl, int ku, std::span<int> pivots) {
  if (ab.size() < static_cast<std::size_t>(2 * kl + ku + 1) * n || pivots.size() < static_cast<std::size_t>(n))
    throw std::invalid_argument("ab holds (2 kl + ku + 1) n values, pivots n");
  const int info = sl3dgpu_band_lu_factor(ab.data(), n, kl, ku, pivots.data());
  if (info < 0) gpu::Check(info);
  return info;
}

inline void BandLuSolve(std::span<const double> ab, int n, int kl, int ku, std::span<const int> pivots,
                        std::span<double> b, int nrhs) {
  if (b.size() < static_cast<std::size_t>(n) * nrhs) throw std::invalid_argument("b holds n nrhs values");
  gpu::Check(sl3dgpu_band_lu_solve(ab.data(), n, kl, ku, pivots.data(), b.data(), nrhs));
}

}  // namespace detail

// -- one degree's systems ---------------------------------------------------------------------------

// DegreeOperator on the unrelaxed material of the body (the reference takes
// a Material): the degree's unknowns, load and tide vectors, K x and K^-1 b.
class DegreeOperator {
 public:
  struct Options {
    double eps = 1e-8;
  };
  DegreeOperator(const Rheology& body, int l) : DegreeOperator(body, l, Options{}) {}
  DegreeOperator(const Rheology& body, int l, Options options) : l_(l) {
    sl3dgpu_degree* h = nullptr;
    gpu::Check(sl3dgpu_degree_create(body.layers.data(), static_cast<int>(body.layers.size()), body.ngll, l,
                                     options.eps, 0, &h));
    h_.reset(h);
  }
  [[nodiscard]] int Degree() const { return l_; }
  [[nodiscard]] int DofCount() const { return sl3dgpu_degree_dof_count(h_.get()); }
  [[nodiscard]] int Bandwidth() const { return sl3dgpu_degree_bandwidth(h_.get()); }
  [[nodiscard]] int Dof(int node, Component c) const {
    const int d = sl3dgpu_degree_dof(h_.get(), node, static_cast<int>(c));
    if (d < -1) gpu::Check(d);
    return d;
  }
  [[nodiscard]] int SurfaceDof(Component c) const { return sl3dgpu_degree_surface_dof(h_.get(), static_cast<int>(c)); }
  [[nodiscard]] bool UsedCholesky() const { return sl3dgpu_degree_used_cholesky(h_.get()) == 1; }
  [[nodiscard]] std::vector<double> Load() const {
    std::vector<double> out(DofCount());
    gpu::Check(sl3dgpu_degree_load(h_.get(), out.data()));
    return out;
  }
  [[nodiscard]] std::vector<double> Tide(int power = -1) const {
    std::vector<double> out(DofCount());
    gpu::Check(sl3dgpu_degree_tide(h_.get(), power, out.data()));
    return out;
  }
  // x with K x = b for nrhs columns of DofCount() values, column-major.
  [[nodiscard]] std::vector<double> Solve(std::span<const double> b, int nrhs = 1) const {
    if (b.size() != static_cast<std::size_t>(DofCount()) * nrhs)
      throw std::invalid_argument("b holds DofCount() nrhs values");
    std::vector<double> x(b.begin(), b.end());
    gpu::Check(sl3dgpu_degree_solve(h_.get(), x.data(), nrhs));
    return x;
  }
  [[nodiscard]] std::vector<double> Apply(std::span<const double> x, int nrhs = 1) const {
    if (x.size() != static_cast<std::size_t>(DofCount()) * nrhs)
      throw std::invalid_argument("x holds DofCount() nrhs values");
    std::vector<double> y(x.size());
    gpu::Check(sl3dgpu_degree_apply(h_.get(), x.data(), nrhs, y.data()));
    return y;
  }
  // The assembled, unscaled upper band ((kd + 1) x DofCount(), LAPACK storage).
  [[nodiscard]] std::vector<double> Band() const {
    std::vector<double> out(static_cast<std::size_t>(Bandwidth() + 1) * DofCount());
    gpu::Check(sl3dgpu_degree_band(h_.get(), out.data()));
    return out;
  }

 protected:
  DegreeOperator(const Rheology& body, int l, double eps, int toroidal) : l_(l) {
    sl3dgpu_degree* h = nullptr;
    gpu::Check(sl3dgpu_degree_create(body.layers.data(), static_cast<int>(body.layers.size()), body.ngll, l, eps,
                                     toroidal, &h));
    h_.reset(h);
  }
  int l_;
  std::unique_ptr<sl3dgpu_degree, gpu::Deleter<sl3dgpu_degree, sl3dgpu_degree_destroy>> h_;
};

// ToroidalOperator (l >= 1): W on the solid elements; Dof ignores the component.
class ToroidalOperator : public DegreeOperator {
 public:
  ToroidalOperator(const Rheology& body, int l) : ToroidalOperator(body, l, Options{}) {}
  ToroidalOperator(const Rheology& body, int l, Options options) : DegreeOperator(body, l, options.eps, 1) {}
  [[nodiscard]] int Dof(int node) const { return DegreeOperator::Dof(node, Component::U); }
  [[nodiscard]] int SurfaceDof() const { return DegreeOperator::SurfaceDof(Component::U); }
};

// -- the surface grid -------------------------------------------------------------------------------

// SurfaceGrid's batched transforms on device buffers (reference layouts,
// complex values as (re, im) pairs); `stream` a cudaStream_t or null.
class SurfaceGrid {
 public:
  SurfaceGrid(int lmax, int nmax = 2, double oversampling = 1.0) {
    sl3dgpu_grid* h = nullptr;
    gpu::Check(sl3dgpu_grid_create(lmax, nmax, oversampling, &h));
    h_.reset(h);
    gpu::Check(sl3dgpu_grid_shape(h, &ntheta_, &nphi_));
  }
  [[nodiscard]] int LMax() const { return sl3dgpu_grid_lmax(h_.get()); }
  [[nodiscard]] int NumberOfCoLatitudes() const { return ntheta_; }
  [[nodiscard]] int NumberOfLongitudes() const { return nphi_; }
  [[nodiscard]] std::vector<double> CoLatitudes() const {
    std::vector<double> theta(ntheta_), w(ntheta_);
    gpu::Check(sl3dgpu_grid_colatitudes(h_.get(), theta.data(), w.data()));
    return theta;
  }
  void SynthesiseSpinBatch(int N, const double* coeffs, int count, double* fields, void* stream = nullptr) {
    gpu::Check(sl3dgpu_synthesise_spin_batch(h_.get(), N, coeffs, count, fields, stream));
  }
  void ExpandSpinBatch(int N, const double* fields, int count, double* coeffs, void* stream = nullptr) {
    gpu::Check(sl3dgpu_expand_spin_batch(h_.get(), N, fields, count, coeffs, stream));
  }
  void SynthesiseBatch(const double* coeffs, int count, double* fields, void* stream = nullptr) {
    gpu::Check(sl3dgpu_synthesise_batch(h_.get(), coeffs, count, fields, stream));
  }
  void ExpandBatch(const double* fields, int count, double* coeffs, void* stream = nullptr) {
    gpu::Check(sl3dgpu_expand_batch(h_.get(), fields, count, coeffs, stream));
  }
  [[nodiscard]] sl3dgpu_grid* Handle() const { return h_.get(); }

 private:
  std::unique_ptr<sl3dgpu_grid, gpu::Deleter<sl3dgpu_grid, sl3dgpu_grid_destroy>> h_;
  int ntheta_ = 0, nphi_ = 0;
};

// -- the 3D step ----------------------------------------------------------------------------------------

class Viscoelastic3D {
 public:
  using LoadCallable3D = std::function<std::optional<std::vector<Complex>>(int l, double t)>;
  using DeltaFunction = std::function<double(double r, double theta, double phi)>;

  struct Options {
    // the reference's fields (Viscoelastic3D.hpp:89-187)
    double eps = 1e-8;
    double oversampling = 1.5;
    int max_iterations = 40;
    double rtol = 1e-11;
    double damping = 1.0;
    int anderson_memory = 5;
    double anderson_rate = 0.5;
    enum class StepSolver { FixedPoint, ConjugateGradients };
    StepSolver solver = StepSolver::FixedPoint;
    double solve_rtol = 1e-11;
    int solve_max_iterations = 200;
    // the GPU forms (no counterpart in the reference): 1 the mixed form;
    // the FP32 correction's finest relative change and Anderson history; the
    // extrapolated warm start; FP64 contractions emulated on the tensor cores
    int precision = 0;
    double correction_rtol = 1e-5;
    int correction_memory = 0;
    int warm_start = 0;
    int fp64_emulation = 0;
  };

  struct StepInfo {
    int iterations = 0;
    double residual = 0.0;
    bool converged = true;
    int mixedPasses = 0;
    int solveIterations = 0;
    int correctionPasses = 0;  // the mixed form's FP32 passes
  };

  // The memory state on the GPU, with its time.
  class State {
   public:
    double t = 0.0;
    [[nodiscard]] sl3dgpu_v3d_state* Handle() const { return h_.get(); }

   private:
    friend class Viscoelastic3D;
    std::unique_ptr<sl3dgpu_v3d_state, gpu::Deleter<sl3dgpu_v3d_state, sl3dgpu_v3d_free_state>> h_;
  };

  // delta(r, theta, phi), r in the model's length unit (the Earth's radius,
  // 6371 km), is sampled at every memory node over the operator's grid, as the
  // reference's constructor samples it (Viscoelastic3D.cpp:250-287).
  Viscoelastic3D(const Rheology& body, int lmax, const DeltaFunction& delta)
      : Viscoelastic3D(body, lmax, delta, Options{}) {}
  Viscoelastic3D(const Rheology& body, int lmax, const DeltaFunction& delta, Options options) : lmax_(lmax) {
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
    o.precision = options.precision;
    o.correction_rtol = options.correction_rtol;
    o.solver = options.solver == Options::StepSolver::ConjugateGradients ? 1 : 0;
    o.solve_rtol = options.solve_rtol;
    o.solve_max_iterations = options.solve_max_iterations;
    o.warm_start = options.warm_start;
    o.fp64_emulation = options.fp64_emulation;
    o.correction_memory = options.correction_memory;
    sl3dgpu_v3d* h = nullptr;
    gpu::Check(sl3dgpu_v3d_create(body.layers.data(), static_cast<int>(body.layers.size()), &o, &h));
    h_.reset(h);
    gpu::Check(sl3dgpu_v3d_shape(h, &nodes_, &ntheta_, &nphi_));
    radius_.resize(nodes_);
    gpu::Check(sl3dgpu_v3d_nodes(h, radius_.data(), nullptr));
    theta_.resize(ntheta_);
    std::vector<double> w(ntheta_);
    gpu::Check(sl3dgpu_v3d_colatitudes(h, theta_.data(), w.data()));
    gpu::Check(sl3dgpu_v3d_scales(h, &length_, &time_, &sigma_));
    if (delta) {
      std::vector<double> samples(static_cast<std::size_t>(nodes_) * ntheta_ * nphi_);
      const double twoPi = 6.283185307179586476925286766559;
      std::size_t at = 0;
      for (int p = 0; p < nodes_; ++p)
        for (int j = 0; j < ntheta_; ++j)
          for (int k = 0; k < nphi_; ++k) samples[at++] = delta(radius_[p], theta_[j], twoPi * k / nphi_);
      gpu::Check(sl3dgpu_v3d_set_delta(h, samples.data(), 0));
    }
  }

  [[nodiscard]] int LMax() const { return lmax_; }
  [[nodiscard]] int NodeCount() const { return nodes_; }
  [[nodiscard]] const std::vector<double>& Radii() const { return radius_; }
  // SI per model unit
  [[nodiscard]] double LengthScale() const { return length_; }
  [[nodiscard]] double TimeScale() const { return time_; }
  [[nodiscard]] double SurfaceDensityScale() const { return sigma_; }

  [[nodiscard]] State ZeroState() const {
    State s;
    sl3dgpu_v3d_state* h = nullptr;
    gpu::Check(sl3dgpu_v3d_zero_state(h_.get(), &h));
    s.h_.reset(h);
    return s;
  }

  // One step of length dt (model units) under the load and tide channels;
  // the state advances in place and its time by dt.
  StepInfo Step(State& state, double dt, Scheme scheme = Scheme::Sdirk2, const LoadCallable3D& load = {},
                const LoadCallable3D& tide = {}) {
    sl3dgpu_step_info info{};
    std::vector<Complex> l0, l1, t0, t1;
    if (load) {
      l0 = gpu::Flatten(load, lmax_, state.t);
      l1 = gpu::Flatten(load, lmax_, state.t + dt);
    }
    if (tide) {
      t0 = gpu::Flatten(tide, lmax_, state.t);
      t1 = gpu::Flatten(tide, lmax_, state.t + dt);
    }
    auto raw = [](const std::vector<Complex>& v) {
      return v.empty() ? nullptr : reinterpret_cast<const double*>(v.data());
    };
    gpu::Check(sl3dgpu_v3d_step_tide(h_.get(), state.Handle(), dt, static_cast<int>(scheme), raw(l0), raw(l1),
                                     raw(t0), raw(t1), 0, &info));
    state.t += dt;
    return StepInfo{info.iterations, info.residual, info.converged != 0, info.mixed_passes, info.solve_iterations,
                    info.correction_passes};
  }

  // The last step's end-time surface values per degree, complex m >= 0 columns.
  [[nodiscard]] std::map<int, std::vector<Complex>> Surface(Component component) const {
    return SurfaceOf(static_cast<int>(component));
  }
  [[nodiscard]] std::map<int, std::vector<Complex>> SurfaceToroidal() const { return SurfaceOf(3); }
  [[nodiscard]] double InertiaMoment() const {
    double out = 0.0;
    gpu::Check(sl3dgpu_v3d_inertia_moment(h_.get(), &out));
    return out;
  }
  // The next step's start (Converge's start argument, Viscoelastic3D.hpp:
  // 562-569): strain coefficients in the device layout of a state's
  // coefficients (host memory); kept only if its first residual is the smaller.
  void SetStart(std::span<const double> coefficients) {
    gpu::Check(sl3dgpu_v3d_set_start(h_.get(), coefficients.data(), 0));
  }
  [[nodiscard]] std::vector<double> ResidualHistory() const {
    const int n = sl3dgpu_v3d_residual_history(h_.get(), nullptr, 0);
    std::vector<double> out(n > 0 ? n : 0);
    if (n > 0) sl3dgpu_v3d_residual_history(h_.get(), out.data(), n);
    return out;
  }
  [[nodiscard]] sl3dgpu_v3d* Handle() const { return h_.get(); }

 private:
  std::map<int, std::vector<Complex>> SurfaceOf(int component) const {
    std::vector<Complex> flat(static_cast<std::size_t>(lmax_ + 1) * (lmax_ + 2) / 2);
    gpu::Check(sl3dgpu_v3d_surface(h_.get(), component, reinterpret_cast<double*>(flat.data())));
    return gpu::Columns(flat, lmax_);
  }
  int lmax_;
  std::unique_ptr<sl3dgpu_v3d, gpu::Deleter<sl3dgpu_v3d, sl3dgpu_v3d_destroy>> h_;
  int nodes_ = 0, ntheta_ = 0, nphi_ = 0;
  std::vector<double> radius_, theta_;
  double length_ = 1.0, time_ = 1.0, sigma_ = 1.0;
};

// -- the static 3D solve ----------------------------------------------------------------------------------

class ElasticPerturbation3D {
 public:
  struct Options {
    double eps = 1e-8;
    double oversampling = 1.5;
  };
  struct SolveOptions {
    double rtol = 1e-10;
    int max_iterations = 200;
  };
  struct SolveInfo {
    int iterations = 0;
    double residual = 0.0;
    bool converged = false;
    std::vector<double> residuals;
  };

  ElasticPerturbation3D(const Rheology& body, int lmax) : ElasticPerturbation3D(body, lmax, Options{}) {}
  ElasticPerturbation3D(const Rheology& body, int lmax, Options options) : lmax_(lmax) {
    sl3dgpu_ep3d_options o{lmax, body.ngll, options.eps, options.oversampling};
    sl3dgpu_ep3d* h = nullptr;
    gpu::Check(sl3dgpu_ep3d_create(body.layers.data(), static_cast<int>(body.layers.size()), &o, &h));
    h_.reset(h);
    gpu::Check(sl3dgpu_ep3d_shape(h, &nodes_, &ntheta_, &nphi_));
  }
  [[nodiscard]] int LMax() const { return lmax_; }
  // GridCoupling's nodes and grid the moduli directions live on
  // (node-major, colatitude, longitude).
  [[nodiscard]] int NodeCount() const { return nodes_; }
  [[nodiscard]] std::size_t FieldValues() const { return static_cast<std::size_t>(nodes_) * ntheta_ * nphi_; }
  [[nodiscard]] std::vector<double> Radii() const {
    std::vector<double> r(nodes_);
    gpu::Check(sl3dgpu_ep3d_nodes(h_.get(), r.data(), nullptr));
    return r;
  }
  [[nodiscard]] std::vector<double> CoLatitudes() const {
    std::vector<double> theta(ntheta_), w(ntheta_);
    gpu::Check(sl3dgpu_ep3d_colatitudes(h_.get(), theta.data(), w.data()));
    return theta;
  }
  [[nodiscard]] int NumberOfLongitudes() const { return nphi_; }

  // SolveLateral: (K_ref + dK) x = the load's forces by preconditioned
  // conjugate gradients from the reference response; dMu / dKappa over the
  // nodes' grids (empty for none), non-dimensional; the solution is kept
  // for Surface.
  SolveInfo SolveLateral(std::span<const Complex> load, std::span<const double> dMu,
                         std::span<const double> dKappa) {
    return SolveLateral(load, dMu, dKappa, SolveOptions{});
  }
  SolveInfo SolveLateral(std::span<const Complex> load, std::span<const double> dMu,
                         std::span<const double> dKappa, SolveOptions options) {
    SetModuli(dMu, dKappa);
    sl3dgpu_step_info info{};
    gpu::Check(sl3dgpu_ep3d_solve_lateral(h_.get(), reinterpret_cast<const double*>(load.data()), options.rtol,
                                          options.max_iterations, &info));
    SolveInfo out{info.iterations, info.residual, info.converged != 0, {}};
    const int n = sl3dgpu_ep3d_residual_history(h_.get(), nullptr, 0);
    out.residuals.resize(n > 0 ? n : 0);
    if (n > 0) sl3dgpu_ep3d_residual_history(h_.get(), out.residuals.data(), n);
    return out;
  }
  // SolveLoad: the reference response (kept for Surface).
  void SolveLoad(std::span<const Complex> load) {
    gpu::Check(sl3dgpu_ep3d_solve_load(h_.get(), reinterpret_cast<const double*>(load.data())));
  }
  // Respond: the kept solution x replaced by -K^-1 (dK) x (the Born response).
  void Respond(std::span<const double> dMu, std::span<const double> dKappa) {
    SetModuli(dMu, dKappa);
    gpu::Check(sl3dgpu_ep3d_respond(h_.get()));
  }
  [[nodiscard]] std::map<int, std::vector<Complex>> Surface(Component component) const {
    std::vector<Complex> flat(static_cast<std::size_t>(lmax_ + 1) * (lmax_ + 2) / 2);
    gpu::Check(sl3dgpu_ep3d_surface(h_.get(), static_cast<int>(component), reinterpret_cast<double*>(flat.data())));
    return gpu::Columns(flat, lmax_);
  }

 private:
  void SetModuli(std::span<const double> dMu, std::span<const double> dKappa) {
    for (auto s : {dMu, dKappa})
      if (!s.empty() && s.size() != FieldValues())
        throw std::invalid_argument("a moduli direction covers every node's grid (or is empty)");
    gpu::Check(sl3dgpu_ep3d_set_moduli(h_.get(), dMu.empty() ? nullptr : dMu.data(),
                                       dKappa.empty() ? nullptr : dKappa.data(), 0));
  }
  int lmax_;
  std::unique_ptr<sl3dgpu_ep3d, gpu::Deleter<sl3dgpu_ep3d, sl3dgpu_ep3d_destroy>> h_;
  int nodes_ = 0, ntheta_ = 0, nphi_ = 0;
};

}  // namespace sl3dpp
