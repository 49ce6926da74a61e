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
//   GRDSolver              include/sl3dpp/SeaLevel.hpp:206-481 (SolveGeneralised,
//                          SolveNonlinear, MakeState)
//   Viscoelastic3D         include/sl3dpp/Viscoelastic3D.hpp:79-837, with
//                          its OpenStep (:440-640) and the GridCoupling maps
//                          (include/sl3dpp/GridCoupling.hpp:82-428)
//   Evolution3D            include/sl3dpp/Evolution3D.hpp (Run, RunMigrating;
//                          frozen and migrating shorelines)
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
//    refuses the reference's options this build does not implement;
//  - the open step's spectral tensors and the degree systems' solutions are
//    flat complex vectors in the GPU's layouts (Viscoelastic3D::Layout), the
//    library's device arrays copied in and out by the classes.
#pragma once

#include <array>
#include <complex>
#include <cstddef>
#include <functional>
#include <map>
#include <memory>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>
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

// n values of T in device memory (the library's allocator), freed with the
// object; host vectors go in and out by copy.
template <class T>
class DeviceVector {
 public:
  DeviceVector() = default;
  explicit DeviceVector(std::size_t n) : n_(n) {
    void* p = nullptr;
    Check(sl3dgpu_device_alloc(static_cast<long long>(n * sizeof(T)), &p));
    p_.reset(static_cast<T*>(p));
  }
  explicit DeviceVector(std::span<const T> host) : DeviceVector(host.size()) { Upload(host); }
  void Upload(std::span<const T> host) {
    if (host.size() != n_) throw std::invalid_argument("a device vector is copied whole");
    Check(sl3dgpu_device_copy(p_.get(), host.data(), static_cast<long long>(n_ * sizeof(T))));
  }
  [[nodiscard]] std::vector<T> Download() const {
    std::vector<T> out(n_);
    Check(sl3dgpu_device_copy(out.data(), p_.get(), static_cast<long long>(n_ * sizeof(T))));
    return out;
  }
  [[nodiscard]] T* data() const { return p_.get(); }
  [[nodiscard]] double* doubles() const { return reinterpret_cast<double*>(p_.get()); }
  [[nodiscard]] std::size_t size() const { return n_; }

 private:
  struct Free {
    void operator()(T* p) const { sl3dgpu_device_free(p); }
  };
  std::unique_ptr<T, Free> p_;
  std::size_t n_ = 0;
};

// A host coefficient vector for the C ABI (empty: none).
inline const double* Raw(std::span<const Complex> v) {
  return v.empty() ? nullptr : reinterpret_cast<const double*>(v.data());
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


// -- the sea-level equation (include/sl3dpp/SeaLevel.hpp) ---------------------------------------------

enum class RotationalFeedback { None = 0, Axial = 1, Full = 2 };

// GRDSolver on its own grid (lmax, spin 0, oversampling 1), non-dimensional:
// SolveGeneralised (SeaLevel.hpp:228-330) and SolveNonlinear (:418-481)
// with MakeState (:206). Fields are host vectors over the grid
// (colatitude-major), coefficients (l, m >= 0) complex; an empty vector is
// an absent channel. Where the GPU build differs: the body's Love numbers
// and constants are given as a Body (the reference converts its LoveNumbers
// and SeaLevelParameters in the constructor), the ice density beside them.
class GRDSolver {
 public:
  struct Body {
    std::vector<double> h, k, l, ht, kt, lt;  // per degree 0 .. lmax (l, ht, kt, lt may be empty)
    double g = 1.0, waterDensity = 1.0, radius = 1.0, iceDensity = 0.917;
    RotationalFeedback rotation = RotationalFeedback::None;
    double omega = 0.0, polarMoment = 0.0, equatorialMoment = 0.0, gravitationalConstant = 0.0;
    double hc = 0.0, kc = 0.0, mU = 0.0, mPhi = 0.0, mC = 0.0;
  };
  struct Options {
    double rtol = 1e-9;
    int max_iterations = 1000;
    int anderson_memory = 5;
  };
  struct State {
    std::vector<double> iceThickness, seaLevel, oceanFunction;
    double oceanArea = 0.0;
    std::vector<char> forcedLand;
  };
  struct GeneralisedForcing {
    std::vector<double> directLoad, directLoadOutsideWaterBudget, solidSurfaceChange;
    std::vector<Complex> displacementResponse, potentialResponse, tangentialResponse, toroidalResponse, tide;
    double inertiaMomentChange = 0.0;
    std::array<double, 3> angularMomentumChange{0.0, 0.0, 0.0};
  };
  struct Response {
    std::vector<double> relativeSeaLevelChange, displacement, potential, tangentialPotential, toroidalPotential;
    std::array<double, 3> angularVelocity{0.0, 0.0, 0.0};
    double uniformShift = 0.0;
    int iterations = 0;
    double error = 0.0;
    bool converged = true;
  };
  struct NonlinearForcing {
    std::vector<double> iceThicknessChange, directLoad, directLoadOutsideWaterBudget, solidSurfaceChange,
        dynamicSeaLevelChange;
    std::vector<Complex> displacementResponse, potentialResponse, tangentialResponse, toroidalResponse, tide;
    double inertiaMomentChange = 0.0;
    std::optional<std::vector<char>> forcedLand;  // absent: the state's
  };
  struct NonlinearResponse {
    State finalState;
    Response response;
    std::vector<Complex> loadCoefficients;
  };

  GRDSolver(int lmax, Body body) : grid_(lmax, 0, 1.0), body_(std::move(body)), lmax_(lmax) {
    for (const auto* v : {&body_.h, &body_.k})
      if (static_cast<int>(v->size()) < lmax + 1) throw std::invalid_argument("h and k reach degree lmax");
    size_ = static_cast<std::size_t>(grid_.NumberOfCoLatitudes()) * grid_.NumberOfLongitudes();
    weights_.resize(grid_.NumberOfCoLatitudes());
    std::vector<double> theta(weights_.size());
    gpu::Check(sl3dgpu_grid_colatitudes(grid_.Handle(), theta.data(), weights_.data()));
  }
  [[nodiscard]] std::size_t FieldSize() const { return size_; }
  [[nodiscard]] std::size_t CoefficientSize() const { return static_cast<std::size_t>(lmax_ + 1) * (lmax_ + 2) / 2; }
  [[nodiscard]] const SurfaceGrid& Grid() const { return grid_; }

  // int f dS over the sphere of the solver's radius
  [[nodiscard]] double IntegrateSurface(std::span<const double> field) const {
    const int nphi = grid_.NumberOfLongitudes();
    double sum = 0.0;
    for (std::size_t j = 0; j < weights_.size(); ++j) {
      double ring = 0.0;
      for (int k = 0; k < nphi; ++k) ring += field[j * nphi + k];
      sum += weights_[j] * ring;
    }
    return body_.radius * body_.radius * sum * 6.283185307179586476925286766559 / nphi;
  }

  [[nodiscard]] State MakeState(std::vector<double> iceThickness, std::vector<double> seaLevel,
                                std::span<const char> forcedLand = {}) const {
    if (iceThickness.size() != size_ || seaLevel.size() != size_ || (!forcedLand.empty() && forcedLand.size() != size_))
      throw std::invalid_argument("state fields must live on the grid");
    gpu::DeviceVector<double> ice{std::span<const double>(iceThickness)}, sea{std::span<const double>(seaLevel)},
        ocean(size_);
    gpu::DeviceVector<unsigned char> land(forcedLand.size());
    if (!forcedLand.empty()) land.Upload(std::span(reinterpret_cast<const unsigned char*>(forcedLand.data()), size_));
    gpu::Check(sl3dgpu_sle_flotation(static_cast<long long>(size_), body_.waterDensity, body_.iceDensity, ice.data(),
                                     sea.data(), forcedLand.empty() ? nullptr : land.data(), ocean.data(), nullptr));
    State st;
    st.oceanFunction = ocean.Download();
    st.iceThickness = std::move(iceThickness);
    st.seaLevel = std::move(seaLevel);
    st.oceanArea = IntegrateSurface(st.oceanFunction);
    st.forcedLand.assign(forcedLand.begin(), forcedLand.end());
    return st;
  }

  [[nodiscard]] Response SolveGeneralised(const State& state, const GeneralisedForcing& forcing) const {
    return SolveGeneralised(state, forcing, Options{});
  }
  [[nodiscard]] Response SolveGeneralised(const State& state, const GeneralisedForcing& forcing,
                                          Options options) const {
    Fields f(*this);
    const double* ocean = f.Field(state.oceanFunction, "the ocean function", true);
    sl3dgpu_sle_forcing c{};
    c.direct_load = f.Field(forcing.directLoad, "the direct load");
    c.direct_load_outside = f.Field(forcing.directLoadOutsideWaterBudget, "the direct load outside the budget");
    c.solid_surface_change = f.Field(forcing.solidSurfaceChange, "the solid surface change");
    c.displacement_response = f.Coeffs(forcing.displacementResponse);
    c.potential_response = f.Coeffs(forcing.potentialResponse);
    c.tangential_response = f.Coeffs(forcing.tangentialResponse);
    c.toroidal_response = f.Coeffs(forcing.toroidalResponse);
    c.tide = f.Coeffs(forcing.tide);
    c.inertia_moment_change = forcing.inertiaMomentChange;
    for (int i = 0; i < 3; ++i) c.angular_momentum_change[i] = forcing.angularMomentumChange[i];
    Outputs out(size_);
    const auto b = RawBody();
    sl3dgpu_sle_result r{};
    gpu::Check(sl3dgpu_sle_solve(grid_.Handle(), &b, ocean, &c, options.rtol, options.max_iterations,
                                 options.anderson_memory, out.slc.data(), out.disp.data(), out.pot.data(),
                                 out.tan.data(), out.tor.data(), &r, nullptr));
    return out.Collect(r, !forcing.toroidalResponse.empty());
  }

  // the reference's default budget for the nonlinear solve: 50 iterations
  [[nodiscard]] NonlinearResponse SolveNonlinear(const State& state, const NonlinearForcing& forcing) const {
    Options options;
    options.max_iterations = 50;
    return SolveNonlinear(state, forcing, options);
  }
  [[nodiscard]] NonlinearResponse SolveNonlinear(const State& state, const NonlinearForcing& forcing,
                                                 Options options) const {
    Fields f(*this);
    sl3dgpu_sle_state st{f.Field(state.iceThickness, "the ice thickness", true),
                         f.Field(state.seaLevel, "the sea level", true),
                         f.Field(state.oceanFunction, "the ocean function", true), f.Mask(state.forcedLand)};
    sl3dgpu_sle_nonlinear_forcing c{};
    c.ice_thickness_change = f.Field(forcing.iceThicknessChange, "the ice thickness change");
    c.direct_load = f.Field(forcing.directLoad, "the direct load");
    c.direct_load_outside = f.Field(forcing.directLoadOutsideWaterBudget, "the direct load outside the budget");
    c.solid_surface_change = f.Field(forcing.solidSurfaceChange, "the solid surface change");
    c.dynamic_sea_level_change = f.Field(forcing.dynamicSeaLevelChange, "the dynamic sea level change");
    c.displacement_response = f.Coeffs(forcing.displacementResponse);
    c.potential_response = f.Coeffs(forcing.potentialResponse);
    c.tangential_response = f.Coeffs(forcing.tangentialResponse);
    c.toroidal_response = f.Coeffs(forcing.toroidalResponse);
    c.tide = f.Coeffs(forcing.tide);
    c.inertia_moment_change = forcing.inertiaMomentChange;
    if (forcing.forcedLand) {
      c.hold_land = 1;
      c.forced_land = f.Mask(*forcing.forcedLand);
    }
    Outputs out(size_);
    gpu::DeviceVector<double> sea(size_), ocean(size_);
    gpu::DeviceVector<Complex> load(CoefficientSize());
    const auto b = RawBody();
    sl3dgpu_sle_result r{};
    gpu::Check(sl3dgpu_sle_solve_nonlinear(grid_.Handle(), &b, body_.iceDensity, &st, &c, options.rtol,
                                           options.max_iterations, out.slc.data(), out.disp.data(), out.pot.data(),
                                           out.tan.data(), out.tor.data(), sea.data(), ocean.data(), load.doubles(),
                                           &r, nullptr));
    NonlinearResponse nr;
    nr.response = out.Collect(r, !forcing.toroidalResponse.empty());
    nr.finalState.iceThickness = state.iceThickness;
    if (!forcing.iceThicknessChange.empty())
      for (std::size_t i = 0; i < size_; ++i) nr.finalState.iceThickness[i] += forcing.iceThicknessChange[i];
    nr.finalState.seaLevel = sea.Download();
    nr.finalState.oceanFunction = ocean.Download();
    nr.finalState.oceanArea = IntegrateSurface(nr.finalState.oceanFunction);
    nr.finalState.forcedLand = forcing.forcedLand ? *forcing.forcedLand : state.forcedLand;
    nr.loadCoefficients = load.Download();
    return nr;
  }

 private:
  // the forcing's device copies, alive for one call
  struct Fields {
    explicit Fields(const GRDSolver& s) : solver(s) {}
    const double* Field(const std::vector<double>& v, const char* what, bool required = false) {
      if (v.empty()) {
        if (required) throw std::invalid_argument(std::string(what) + " is required");
        return nullptr;
      }
      if (v.size() != solver.size_) throw std::invalid_argument(std::string(what) + " is not a field on the grid");
      return fields.emplace_back(std::span<const double>(v)).data();
    }
    const double* Coeffs(const std::vector<Complex>& v) {
      if (v.empty()) return nullptr;
      if (v.size() != solver.CoefficientSize())
        throw std::invalid_argument("a response or tide is not a coefficient vector of the grid");
      return coeffs.emplace_back(std::span<const Complex>(v)).doubles();
    }
    const unsigned char* Mask(const std::vector<char>& m) {
      if (m.empty()) return nullptr;
      if (m.size() != solver.size_) throw std::invalid_argument("the land held is not a mask on the grid");
      return masks.emplace_back(std::span(reinterpret_cast<const unsigned char*>(m.data()), m.size())).data();
    }
    const GRDSolver& solver;
    std::vector<gpu::DeviceVector<double>> fields;
    std::vector<gpu::DeviceVector<Complex>> coeffs;
    std::vector<gpu::DeviceVector<unsigned char>> masks;
  };
  struct Outputs {
    explicit Outputs(std::size_t n) : slc(n), disp(n), pot(n), tan(n), tor(n) {}
    GRDSolver::Response Collect(const sl3dgpu_sle_result& r, bool toroidal) const {
      GRDSolver::Response out;
      out.relativeSeaLevelChange = slc.Download();
      out.displacement = disp.Download();
      out.potential = pot.Download();
      out.tangentialPotential = tan.Download();
      if (toroidal) out.toroidalPotential = tor.Download();
      for (int i = 0; i < 3; ++i) out.angularVelocity[i] = r.angular_velocity[i];
      out.uniformShift = r.uniform_shift;
      out.iterations = r.iterations;
      out.error = r.error;
      out.converged = r.converged != 0;
      return out;
    }
    gpu::DeviceVector<double> slc, disp, pot, tan, tor;
  };
  [[nodiscard]] sl3dgpu_sle_body RawBody() const {
    auto ptr = [](const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); };
    sl3dgpu_sle_body b{};
    b.h = ptr(body_.h);
    b.k = ptr(body_.k);
    b.l = ptr(body_.l);
    b.ht = ptr(body_.ht);
    b.kt = ptr(body_.kt);
    b.lt = ptr(body_.lt);
    b.g = body_.g;
    b.water_density = body_.waterDensity;
    b.radius = body_.radius;
    b.rotation = static_cast<int>(body_.rotation);
    b.omega = body_.omega;
    b.polar_moment = body_.polarMoment;
    b.equatorial_moment = body_.equatorialMoment;
    b.gravitational_constant = body_.gravitationalConstant;
    b.hc = body_.hc;
    b.kc = body_.kc;
    b.m_u = body_.mU;
    b.m_phi = body_.mPhi;
    b.m_c = body_.mC;
    return b;
  }
  SurfaceGrid grid_;
  Body body_;
  int lmax_;
  std::size_t size_ = 0;
  std::vector<double> weights_;
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
  // grid values over every node: delta's samples, the kernels' layout
  [[nodiscard]] std::size_t GridValues() const { return static_cast<std::size_t>(nodes_) * ntheta_ * nphi_; }
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

  // -- GridCoupling (include/sl3dpp/GridCoupling.hpp:82-428) ------------------------------------------

  // The sizes of the GPU layouts: complex spectral coefficients of a tensor
  // over every node, grid values at every node, and the spheroidal and
  // toroidal systems' complex solution values.
  struct Layout {
    long long spectral = 0, gridValues = 0, spheroidal = 0, toroidal = 0;
  };
  [[nodiscard]] Layout GetLayout() const {
    Layout l;
    gpu::Check(sl3dgpu_v3d_layout(h_.get(), &l.spectral, &l.gridValues, &l.spheroidal, &l.toroidal));
    return l;
  }
  // A tensor field on every node's grid: its spin -2 and spin -1 components
  // (complex) and its spin 0 component (real), node-major.
  struct TensorField {
    std::vector<Complex> c0, c1;
    std::vector<double> r;
  };
  // Synthesise / Analyse of a spectral tensor (GridCoupling::Synthesise,
  // Analyse).
  [[nodiscard]] TensorField Synthesise(std::span<const Complex> spectral) const {
    const auto l = GetLayout();
    Expect(spectral.size(), l.spectral, "a spectral tensor");
    gpu::DeviceVector<Complex> in(spectral), c0(l.gridValues), c1(l.gridValues);
    gpu::DeviceVector<double> r(l.gridValues);
    gpu::Check(sl3dgpu_v3d_synthesise_tensor(h_.get(), in.doubles(), c0.doubles(), c1.doubles(), r.data()));
    return TensorField{c0.Download(), c1.Download(), r.Download()};
  }
  [[nodiscard]] std::vector<Complex> Analyse(const TensorField& field) const {
    const auto l = GetLayout();
    Expect(field.c0.size(), l.gridValues, "a tensor field's spin -2 component");
    Expect(field.c1.size(), l.gridValues, "a tensor field's spin -1 component");
    Expect(field.r.size(), l.gridValues, "a tensor field's spin 0 component");
    gpu::DeviceVector<Complex> c0{std::span<const Complex>(field.c0)}, c1{std::span<const Complex>(field.c1)},
        out(l.spectral);
    gpu::DeviceVector<double> r{std::span<const double>(field.r)};
    gpu::Check(sl3dgpu_v3d_analyse_tensor(h_.get(), c0.doubles(), c1.doubles(), r.data(), out.doubles()));
    return out.Download();
  }
  // SpheroidalForce / ToroidalForce of an analysed tensor: the degree
  // systems' right-hand sides, spheroidal then toroidal.
  [[nodiscard]] std::pair<std::vector<Complex>, std::vector<Complex>> DegreeForces(
      std::span<const Complex> spectral) const {
    const auto l = GetLayout();
    Expect(spectral.size(), l.spectral, "a spectral tensor");
    gpu::DeviceVector<Complex> in(spectral), sph(l.spheroidal), tor(l.toroidal);
    gpu::Check(sl3dgpu_v3d_degree_forces(h_.get(), in.doubles(), sph.doubles(), tor.doubles()));
    return {sph.Download(), tor.Download()};
  }
  // AddStrainOfSolution: the strain coefficients of the systems' solutions.
  [[nodiscard]] std::vector<Complex> StrainOfSolutions(std::span<const Complex> spheroidal,
                                                       std::span<const Complex> toroidal) const {
    const auto l = GetLayout();
    Expect(spheroidal.size(), l.spheroidal, "the spheroidal solutions");
    Expect(toroidal.size(), l.toroidal, "the toroidal solutions");
    gpu::DeviceVector<Complex> sph(spheroidal), tor(toroidal), out(l.spectral);
    gpu::Check(sl3dgpu_v3d_strain_of_solutions(h_.get(), sph.doubles(), tor.doubles(), out.doubles()));
    return out.Download();
  }

  // -- OpenStep (Viscoelastic3D.hpp:440-640) ------------------------------------------------------------

  // One stage opened on the operator's buffers for a driver's own
  // within-step iteration (one open step per operator at a time); strains
  // are spectral tensors in the GPU layout, the solutions stay in the
  // operator (Surface and InertiaMoment read them).
  class OpenStep {
   public:
    // the start strain of the stage
    [[nodiscard]] std::vector<Complex> StartStrain() {
      gpu::Check(sl3dgpu_v3d_step_start_strain(op_->h_.get(), strain_.doubles()));
      return strain_.Download();
    }
    // Respond: the solutions of the memory and lateral force of a strain
    // (empty: the start strain), no channels.
    void Respond(std::span<const Complex> strain = {}) {
      if (!strain.empty()) Put(strain);
      gpu::Check(sl3dgpu_v3d_step_respond(op_->h_.get(), strain.empty() ? nullptr : strain_.doubles()));
    }
    // AddChannels: the load and tide channels' responses added (host
    // (l, m >= 0) coefficients, either empty).
    void AddChannels(std::span<const Complex> load, std::span<const Complex> tide = {}) {
      gpu::Check(sl3dgpu_v3d_step_add_channels(op_->h_.get(), gpu::Raw(load), gpu::Raw(tide)));
    }
    // StrainOf: the strain coefficients of the solutions.
    [[nodiscard]] std::vector<Complex> StrainOf() {
      gpu::Check(sl3dgpu_v3d_step_strain_of(op_->h_.get(), strain_.doubles()));
      return strain_.Download();
    }
    // Converge's measure between two strains.
    [[nodiscard]] double RelativeChange(std::span<const Complex> next, std::span<const Complex> now) {
      Put(next);
      gpu::DeviceVector<Complex> b(now);
      double out = 0.0;
      gpu::Check(sl3dgpu_v3d_relative_change(op_->h_.get(), strain_.doubles(), b.doubles(), &out));
      return out;
    }
    // Close under known channels: the operator's own fixed point (or
    // conjugate gradients, or the mixed form, as its options say) from the
    // start strain; the converged strain and the iteration's info.
    [[nodiscard]] std::pair<std::vector<Complex>, StepInfo> Close(std::span<const Complex> load,
                                                                 std::span<const Complex> tide = {}) {
      sl3dgpu_step_info info{};
      gpu::Check(sl3dgpu_v3d_step_converge(op_->h_.get(), gpu::Raw(load), gpu::Raw(tide), strain_.doubles(), &info));
      return {strain_.Download(), Info(info)};
    }
    // Finish with a strain (empty: the converged one): the state advances
    // in place and the step closes.
    void Finish(std::span<const Complex> strain = {}) {
      if (!strain.empty()) Put(strain);
      gpu::Check(sl3dgpu_v3d_step_finish(op_->h_.get(), strain.empty() ? nullptr : strain_.doubles()));
      state_->t += dt_;
    }
    // The conjugate-gradient close's pieces (Forces, Apply, Solve): degree
    // systems' values, spheroidal then toroidal.
    [[nodiscard]] std::vector<Complex> Forces(std::span<const Complex> load, std::span<const Complex> tide = {}) {
      gpu::Check(sl3dgpu_v3d_step_forces(op_->h_.get(), gpu::Raw(load), gpu::Raw(tide), solutions_.doubles()));
      return solutions_.Download();
    }
    [[nodiscard]] std::vector<Complex> Apply(std::span<const Complex> x) {
      Expect(x.size(), solutions_.size(), "the degree systems' values");
      gpu::DeviceVector<Complex> in(x);
      gpu::Check(sl3dgpu_v3d_step_apply(op_->h_.get(), in.doubles(), solutions_.doubles()));
      return solutions_.Download();
    }
    [[nodiscard]] std::pair<std::vector<Complex>, StepInfo> Solve(std::span<const Complex> forces) {
      Expect(forces.size(), solutions_.size(), "the degree systems' values");
      gpu::DeviceVector<Complex> in(forces);
      sl3dgpu_step_info info{};
      gpu::Check(sl3dgpu_v3d_step_solve(op_->h_.get(), in.doubles(), solutions_.doubles(), &info));
      return {solutions_.Download(), Info(info)};
    }

   private:
    friend class Viscoelastic3D;
    OpenStep(Viscoelastic3D* op, State* state, double dt)
        : op_(op), state_(state), dt_(dt), strain_(static_cast<std::size_t>(op->GetLayout().spectral)),
          solutions_(static_cast<std::size_t>(op->GetLayout().spheroidal + op->GetLayout().toroidal)) {}
    void Put(std::span<const Complex> strain) {
      Expect(strain.size(), strain_.size(), "a spectral tensor");
      strain_.Upload(strain);
    }
    Viscoelastic3D* op_;
    State* state_;
    double dt_;
    gpu::DeviceVector<Complex> strain_, solutions_;
  };
  // StartStep: one stage of length dt (a one-stage family: backward Euler
  // or the exponential trapezoid) opened from the state; load0 the load at
  // the state's time where the state carries no strain (empty: none).
  [[nodiscard]] OpenStep StartStep(State& state, double dt, Scheme family, std::span<const Complex> load0 = {}) {
    if (family == Scheme::Sdirk2)
      throw std::invalid_argument("StartStep opens one stage: backward Euler or the exponential trapezoid");
    gpu::Check(sl3dgpu_v3d_start_step(h_.get(), state.Handle(), dt, static_cast<int>(family), gpu::Raw(load0)));
    return OpenStep(this, &state, dt);
  }

 private:
  std::map<int, std::vector<Complex>> SurfaceOf(int component) const {
    std::vector<Complex> flat(static_cast<std::size_t>(lmax_ + 1) * (lmax_ + 2) / 2);
    gpu::Check(sl3dgpu_v3d_surface(h_.get(), component, reinterpret_cast<double*>(flat.data())));
    return gpu::Columns(flat, lmax_);
  }
  static void Expect(std::size_t got, long long want, const char* what) {
    if (static_cast<long long>(got) != want) throw std::invalid_argument(std::string(what) + " has the layout's size");
  }
  static StepInfo Info(const sl3dgpu_step_info& info) {
    return StepInfo{info.iterations, info.residual, info.converged != 0, info.mixed_passes, info.solve_iterations,
                    info.correction_passes};
  }
  int lmax_;
  std::unique_ptr<sl3dgpu_v3d, gpu::Deleter<sl3dgpu_v3d, sl3dgpu_v3d_destroy>> h_;
  int nodes_ = 0, ntheta_ = 0, nphi_ = 0;
  std::vector<double> radius_, theta_;
  double length_ = 1.0, time_ = 1.0, sigma_ = 1.0;
};


// -- the run through time (include/sl3dpp/Evolution3D.hpp) ---------------------------------------------

// Evolution3D::Run and RunMigrating (src/Evolution3D.cpp:93-133, March
// :540-821) on a Viscoelastic3D operator: without an ocean (NoOceanState, the
// loads as coefficient callables), under an ocean with frozen shorelines
// (SetOcean; the direct loads as fields on the sea-level grid), or with
// migrating ones (SetMigrating; the ice thickness history as fields). Where
// the GPU build differs: the ocean is set on the operator rather than given
// as the GRDSolver and State of the reference's constructor, its constants
// SI as SeaLevelParameters gives them; fields are in the model's units.
class Evolution3D {
 public:
  using FieldCallable = std::function<std::vector<double>(double t)>;
  struct Snapshot {
    double t = 0.0;
    std::vector<Complex> U, phi, seaLevel;  // (l, m >= 0) coefficients
    std::array<double, 3> angularVelocity{0.0, 0.0, 0.0};
    std::vector<double> oceanFunction;      // migrating shorelines: the node's
    Viscoelastic3D::StepInfo info;
  };
  // The ocean's constants (SeaLevelParameters, include/sl3dpp/SeaLevel.hpp:54-68, SI).
  struct Ocean {
    RotationalFeedback rotation = RotationalFeedback::Axial;
    double waterDensity = 1000.0, iceDensity = 917.0;
    double rotationFrequency = 7.27220521664304e-05, polarMoment = 8.0359e37, equatorialMoment = 8.0096e37;
    double rtol = 1e-10;
    int max_iterations = 200, anderson_memory = 5, max_nonlinear_iterations = 50;
  };

  explicit Evolution3D(Viscoelastic3D& op, Scheme scheme = Scheme::Sdirk2) : op_(&op), scheme_(scheme) {}

  // The sea-level grid (the operator's lmax, oversampling 1): fields on it are colatitude-major.
  [[nodiscard]] std::size_t OceanFieldSize() const {
    int nt = 0, np = 0;
    gpu::Check(sl3dgpu_v3d_ocean_grid(op_->Handle(), &nt, &np, nullptr, nullptr));
    return static_cast<std::size_t>(nt) * np;
  }
  // Frozen shorelines over an ocean function.
  void SetOcean(std::span<const double> oceanFunction, const Ocean& c) {
    if (oceanFunction.size() != OceanFieldSize()) throw std::invalid_argument("the ocean function lives on the sea-level grid");
    sl3dgpu_v3d_ocean o = Raw(c);
    o.ocean_function = oceanFunction.data();
    gpu::Check(sl3dgpu_v3d_set_ocean(op_->Handle(), &o));
    migrating_ = false;
  }
  // Migrating shorelines from a background state (model length; the land
  // held, empty for none): its ocean function is flotation's.
  void SetMigrating(std::span<const double> iceThickness, std::span<const double> seaLevel,
                    std::span<const char> forcedLand, const Ocean& c) {
    const std::size_t n = OceanFieldSize();
    if (iceThickness.size() != n || seaLevel.size() != n || (!forcedLand.empty() && forcedLand.size() != n))
      throw std::invalid_argument("the background's fields live on the sea-level grid");
    sl3dgpu_v3d_ocean o = Raw(c);
    o.migrating = 1;
    o.ice_thickness = iceThickness.data();
    o.sea_level = seaLevel.data();
    o.forced_land = forcedLand.empty() ? nullptr : reinterpret_cast<const unsigned char*>(forcedLand.data());
    gpu::Check(sl3dgpu_v3d_set_ocean(op_->Handle(), &o));
    migrating_ = true;
  }
  void RemoveOcean() { gpu::Check(sl3dgpu_v3d_set_ocean(op_->Handle(), nullptr)); }

  // Run without an ocean: node 0 the instantaneous response, a step a node.
  [[nodiscard]] std::vector<Snapshot> Run(std::span<const double> times, const Viscoelastic3D::LoadCallable3D& load) {
    const int n = static_cast<int>(times.size());
    const std::size_t lm = Coefficients();
    std::vector<Complex> loads(lm * n);
    for (int k = 0; k < n; ++k) {
      const auto flat = gpu::Flatten(load, op_->LMax(), times[k]);
      std::copy(flat.begin(), flat.end(), loads.begin() + lm * k);
    }
    std::vector<Complex> U(lm * n), phi(lm * n);
    std::vector<sl3dgpu_step_info> infos(std::max(n, 1));
    auto state = op_->ZeroState();
    gpu::Check(sl3dgpu_v3d_run(op_->Handle(), state.Handle(), times.data(), n, static_cast<int>(scheme_),
                               reinterpret_cast<const double*>(loads.data()), reinterpret_cast<double*>(U.data()),
                               reinterpret_cast<double*>(phi.data()), infos.data()));
    return Snapshots(times, U, phi, {}, {}, {}, infos);
  }
  // Run under the frozen ocean: the direct (ice) load's fields per node.
  [[nodiscard]] std::vector<Snapshot> RunOcean(std::span<const double> times, const FieldCallable& directLoad) {
    const auto loads = Sample(times, directLoad, "a direct load");
    const int n = static_cast<int>(times.size());
    const std::size_t lm = Coefficients();
    std::vector<Complex> U(lm * n), phi(lm * n), slc(lm * n);
    std::vector<double> omega(3 * n);
    std::vector<sl3dgpu_step_info> infos(std::max(n, 1));
    auto state = op_->ZeroState();
    gpu::Check(sl3dgpu_v3d_run_ocean(op_->Handle(), state.Handle(), times.data(), n, static_cast<int>(scheme_),
                                     loads.data(), reinterpret_cast<double*>(U.data()),
                                     reinterpret_cast<double*>(phi.data()), reinterpret_cast<double*>(slc.data()),
                                     omega.data(), infos.data()));
    return Snapshots(times, U, phi, slc, omega, {}, infos);
  }
  // RunMigrating: the ice thickness per node (the first the background's
  // unless direct loads are given), the direct loads beside it (empty: none).
  [[nodiscard]] std::vector<Snapshot> RunMigrating(std::span<const double> times, const FieldCallable& iceThickness,
                                                   const FieldCallable& directLoad = {}) {
    if (!migrating_) throw std::invalid_argument("RunMigrating needs SetMigrating");
    const auto ice = Sample(times, iceThickness, "an ice thickness");
    std::vector<double> loads;
    if (directLoad) loads = Sample(times, directLoad, "a direct load");
    const int n = static_cast<int>(times.size());
    const std::size_t lm = Coefficients(), size = OceanFieldSize();
    std::vector<Complex> U(lm * n), phi(lm * n), slc(lm * n);
    std::vector<double> omega(3 * n), oceans(size * n);
    std::vector<sl3dgpu_step_info> infos(std::max(n, 1));
    auto state = op_->ZeroState();
    gpu::Check(sl3dgpu_v3d_run_migrating(op_->Handle(), state.Handle(), times.data(), n, static_cast<int>(scheme_),
                                         ice.data(), loads.empty() ? nullptr : loads.data(),
                                         reinterpret_cast<double*>(U.data()), reinterpret_cast<double*>(phi.data()),
                                         reinterpret_cast<double*>(slc.data()), omega.data(), oceans.data(),
                                         infos.data()));
    return Snapshots(times, U, phi, slc, omega, oceans, infos);
  }

 private:
  [[nodiscard]] std::size_t Coefficients() const {
    return static_cast<std::size_t>(op_->LMax() + 1) * (op_->LMax() + 2) / 2;
  }
  static sl3dgpu_v3d_ocean Raw(const Ocean& c) {
    sl3dgpu_v3d_ocean o{};
    o.rotation = static_cast<int>(c.rotation);
    o.water_density = c.waterDensity;
    o.rotation_frequency = c.rotationFrequency;
    o.polar_moment = c.polarMoment;
    o.equatorial_moment = c.equatorialMoment;
    o.rtol = c.rtol;
    o.max_iterations = c.max_iterations;
    o.anderson_memory = c.anderson_memory;
    o.ice_density = c.iceDensity;
    o.max_nonlinear_iterations = c.max_nonlinear_iterations;
    return o;
  }
  std::vector<double> Sample(std::span<const double> times, const FieldCallable& f, const char* what) const {
    const std::size_t size = OceanFieldSize();
    std::vector<double> out;
    out.reserve(size * times.size());
    for (double t : times) {
      const auto v = f(t);
      if (v.size() != size) throw std::invalid_argument(std::string(what) + " lives on the sea-level grid");
      out.insert(out.end(), v.begin(), v.end());
    }
    return out;
  }
  std::vector<Snapshot> Snapshots(std::span<const double> times, const std::vector<Complex>& U,
                                  const std::vector<Complex>& phi, const std::vector<Complex>& slc,
                                  const std::vector<double>& omega, const std::vector<double>& oceans,
                                  const std::vector<sl3dgpu_step_info>& infos) const {
    const std::size_t lm = Coefficients(), size = OceanFieldSize();
    std::vector<Snapshot> out(times.size());
    for (std::size_t k = 0; k < times.size(); ++k) {
      auto& s = out[k];
      s.t = times[k];
      s.U.assign(U.begin() + lm * k, U.begin() + lm * (k + 1));
      s.phi.assign(phi.begin() + lm * k, phi.begin() + lm * (k + 1));
      if (!slc.empty()) s.seaLevel.assign(slc.begin() + lm * k, slc.begin() + lm * (k + 1));
      if (!omega.empty())
        for (int i = 0; i < 3; ++i) s.angularVelocity[i] = omega[3 * k + i];
      if (!oceans.empty()) s.oceanFunction.assign(oceans.begin() + size * k, oceans.begin() + size * (k + 1));
      const auto& i = infos[k];
      s.info = Viscoelastic3D::StepInfo{i.iterations, i.residual, i.converged != 0, i.mixed_passes,
                                        i.solve_iterations, i.correction_passes};
    }
    return out;
  }
  Viscoelastic3D* op_;
  Scheme scheme_;
  bool migrating_ = false;
  friend class AdjointSolver3D;
  friend class TangentLinearSolver3D;
};

// -- the discrete 3D adjoint -----------------------------------------------------------------------------

// What an objective reads at one node (Adjoint.hpp's Measurement): the
// duals of the surface U and phi coefficients (l, m >= 0, either empty),
// paired by the surface integral of real fields (m > 0 twice).
struct Measurement3D {
  std::vector<Complex> displacementDual, potentialDual;
};
// The first-order kernels (Kernels3D, include/sl3dpp/Adjoint3D.hpp:104-140):
// per node the direct-load and tide kernels (dJ = sum_n <kernel_n, dL_n>); dJ/d delta
// per grid sample and its density per unit volume (logViscosityKernel3D,
// the gradient over the samples' volumes); the objective of the forward run.
struct Kernels3D {
  std::vector<std::vector<Complex>> directLoadKernels, tideKernels;
  std::vector<double> deltaGradient, logViscosityKernel3D;
  double objective = 0.0;
};

// AdjointSolver3D under AdjointMethod::Discrete (include/sl3dpp/Adjoint3D.hpp:
// 241-322, src/AdjointDiscrete3D.cpp) for the evolution without an ocean:
// the exact transpose of the time-stepped map, swept back over a forward
// run the solver records itself from a zero state under the loads.
class AdjointSolver3D {
 public:
  struct Options {
    int record_stride = 1;  // the forward run's states kept every stride-th node (Evolution3D::Options::record_stride)
  };
  explicit AdjointSolver3D(const Evolution3D& evolution) : AdjointSolver3D(evolution, Options{}) {}
  AdjointSolver3D(const Evolution3D& evolution, Options options) : evolution_(&evolution), options_(options) {}

  [[nodiscard]] Kernels3D FirstOrderKernels(std::span<const double> times, const Viscoelastic3D::LoadCallable3D& load,
                                            const std::map<std::size_t, Measurement3D>& measurements) const {
    Viscoelastic3D& op = *evolution_->op_;
    const int n = static_cast<int>(times.size());
    const std::size_t lm = evolution_->Coefficients();
    std::vector<Complex> loads(lm * n), u(lm * n), phi(lm * n);
    for (int k = 0; k < n; ++k) {
      const auto flat = gpu::Flatten(load, op.LMax(), times[k]);
      std::copy(flat.begin(), flat.end(), loads.begin() + lm * k);
    }
    bool anyU = false, anyPhi = false;
    for (const auto& [node, m] : measurements) {
      if (node >= static_cast<std::size_t>(n)) throw std::invalid_argument("a measurement past the last node");
      for (const auto* dual : {&m.displacementDual, &m.potentialDual}) {
        if (dual->empty()) continue;
        if (dual->size() != lm) throw std::invalid_argument("a dual has l(l+1)/2 + m coefficients");
        auto& into = dual == &m.displacementDual ? u : phi;
        std::copy(dual->begin(), dual->end(), into.begin() + lm * node);
        (dual == &m.displacementDual ? anyU : anyPhi) = true;
      }
    }
    Kernels3D out;
    std::vector<Complex> kernels(lm * n), tides(lm * n);
    const std::size_t values = op.GridValues();
    out.deltaGradient.resize(values);
    gpu::Check(sl3dgpu_v3d_adjoint_run(op.Handle(), times.data(), n, static_cast<int>(evolution_->scheme_),
                                       options_.record_stride,
                                       reinterpret_cast<const double*>(loads.data()),
                                       anyU ? reinterpret_cast<const double*>(u.data()) : nullptr,
                                       anyPhi ? reinterpret_cast<const double*>(phi.data()) : nullptr,
                                       reinterpret_cast<double*>(kernels.data()),
                                       reinterpret_cast<double*>(tides.data()), out.deltaGradient.data(),
                                       &out.objective, nullptr));
    out.directLoadKernels.resize(n);
    out.tideKernels.resize(n);
    for (int k = 0; k < n; ++k) {
      out.directLoadKernels[k].assign(kernels.begin() + lm * k, kernels.begin() + lm * (k + 1));
      out.tideKernels[k].assign(tides.begin() + lm * k, tides.begin() + lm * (k + 1));
    }
    std::vector<double> volume(values);
    gpu::Check(sl3dgpu_v3d_sample_volumes(op.Handle(), volume.data()));
    out.logViscosityKernel3D.resize(values);
    for (std::size_t x = 0; x < values; ++x) out.logViscosityKernel3D[x] = out.deltaGradient[x] / volume[x];
    return out;
  }

 private:
  const Evolution3D* evolution_;
  Options options_;
};

// TangentLinearSolver3D's discrete run (src/TangentLinear3D.cpp) for the
// evolution without an ocean: the derivative of the surface U and phi at
// every node along a log-viscosity direction over every grid sample
// (empty: none) and along a load direction (empty callable: none), beside
// the forward run from a zero state under the loads.
class TangentLinearSolver3D {
 public:
  struct Derivative {
    std::vector<std::vector<Complex>> U, phi;  // per node, (l, m >= 0)
  };
  explicit TangentLinearSolver3D(const Evolution3D& evolution) : evolution_(&evolution) {}

  [[nodiscard]] Derivative Run(std::span<const double> times, const Viscoelastic3D::LoadCallable3D& load,
                               std::span<const double> deltaDirection,
                               const Viscoelastic3D::LoadCallable3D& loadDirection = {}) const {
    Viscoelastic3D& op = *evolution_->op_;
    const int n = static_cast<int>(times.size());
    const std::size_t lm = evolution_->Coefficients();
    if (!deltaDirection.empty() && deltaDirection.size() != op.GridValues())
      throw std::invalid_argument("the direction has one value per grid sample");
    std::vector<Complex> loads(lm * n), directions(loadDirection ? lm * n : 0), U(lm * n), phi(lm * n);
    for (int k = 0; k < n; ++k) {
      const auto flat = gpu::Flatten(load, op.LMax(), times[k]);
      std::copy(flat.begin(), flat.end(), loads.begin() + lm * k);
      if (loadDirection) {
        const auto d = gpu::Flatten(loadDirection, op.LMax(), times[k]);
        std::copy(d.begin(), d.end(), directions.begin() + lm * k);
      }
    }
    gpu::Check(sl3dgpu_v3d_tangent_run(op.Handle(), times.data(), n, static_cast<int>(evolution_->scheme_),
                                       reinterpret_cast<const double*>(loads.data()),
                                       deltaDirection.empty() ? nullptr : deltaDirection.data(),
                                       loadDirection ? reinterpret_cast<const double*>(directions.data()) : nullptr,
                                       reinterpret_cast<double*>(U.data()), reinterpret_cast<double*>(phi.data()),
                                       nullptr));
    Derivative out;
    out.U.resize(n);
    out.phi.resize(n);
    for (int k = 0; k < n; ++k) {
      out.U[k].assign(U.begin() + lm * k, U.begin() + lm * (k + 1));
      out.phi[k].assign(phi.begin() + lm * k, phi.begin() + lm * (k + 1));
    }
    return out;
  }

 private:
  const Evolution3D* evolution_;
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
  // The degree systems' complex values (spheroidal then toroidal), the
  // layout of Force, Apply, LoadForces and Solution.
  [[nodiscard]] std::size_t SolutionValues() const {
    long long sph = 0, tor = 0;
    gpu::Check(sl3dgpu_ep3d_layout(h_.get(), &sph, &tor));
    return static_cast<std::size_t>(sph + tor);
  }
  // Force: (dK) x under the moduli last set (ElasticPerturbation3D.hpp:98-112).
  [[nodiscard]] std::vector<Complex> Force(std::span<const Complex> x) { return Map(x, sl3dgpu_ep3d_force); }
  // Apply: (K_ref + dK) x (:114-130).
  [[nodiscard]] std::vector<Complex> Apply(std::span<const Complex> x) { return Map(x, sl3dgpu_ep3d_apply); }
  // LoadForces: the unit load vectors times a load's coefficients.
  [[nodiscard]] std::vector<Complex> LoadForces(std::span<const Complex> load) {
    gpu::DeviceVector<Complex> out(SolutionValues());
    gpu::Check(sl3dgpu_ep3d_load_forces(h_.get(), reinterpret_cast<const double*>(load.data()), out.doubles()));
    return out.Download();
  }
  // The held solution (SolveLoad's, SolveLateral's or Respond's).
  [[nodiscard]] std::vector<Complex> Solution() {
    gpu::DeviceVector<Complex> out(SolutionValues());
    gpu::Check(sl3dgpu_ep3d_solution(h_.get(), out.doubles()));
    return out.Download();
  }

 private:
  std::vector<Complex> Map(std::span<const Complex> x, int (*fn)(sl3dgpu_ep3d*, const double*, double*)) {
    if (x.size() != SolutionValues()) throw std::invalid_argument("x covers the degree systems' values");
    gpu::DeviceVector<Complex> in(x), out(x.size());
    gpu::Check(fn(h_.get(), in.doubles(), out.doubles()));
    return out.Download();
  }
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
