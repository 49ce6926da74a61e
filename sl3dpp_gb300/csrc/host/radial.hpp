// Host-side radial setup of the 3D step: the layered Earth, its GLL mesh,
// nodal material, Prony rheology, memory points, and the per-degree
// spheroidal and toroidal band systems. Non-dimensional throughout (the
// reference's geophysical scales: the surface radius and the Earth's mean
// density, G = 1).
//
// Restates, for layered Earths whose fields are linear in radius within each
// layer (the configurations this library is measured on), the reference's
// include/sl3dpp/Scales.hpp, EarthModel.hpp (gravity, segment-exact),
// RadialMesh.hpp/src/RadialMesh.cpp (GLL element, truncation rule),
// Material.hpp/src/Material.cpp, Rheology.hpp/src/Rheology.cpp (Maxwell,
// Burgers), MemoryPoints.hpp/src/MemoryPoints.cpp, the reference operator's
// point moduli (src/Viscoelastic.cpp:120-170, 324-347) and the degree
// systems of src/DegreeOperator.cpp:24-474, 775-1038 and
// src/ToroidalOperator.cpp. Plain C++; it runs once per operator, as the
// reference's construction does. Used by the library and by the oracle.
#pragma once

#include <array>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

namespace sl3dgpu::host {

inline constexpr double kGravitationalConstantSI = 6.6743e-11;
inline constexpr double kEarthMeanDensitySI = 5515.0;
inline constexpr double kEarthRadiusSI = 6.371e6;
inline constexpr double kSecondsPerYear = 3.15576e7;  // Julian year
inline constexpr double kPi = 3.14159265358979323846;

// Scales.hpp: Geophysical(length, density) makes G one.
struct Scales {
  double mass = 1.0, length = 1.0, time = 1.0;
  static Scales Geophysical(double length = kEarthRadiusSI, double density = kEarthMeanDensitySI);
  double Factor(int m, int l, int t) const;
  double Density() const { return Factor(1, -3, 0); }
  double Modulus() const { return Factor(1, -1, -2); }
  double Viscosity() const { return Factor(1, -1, -1); }
  double Acceleration() const { return Factor(0, 1, -2); }
  double Potential() const { return Factor(0, 2, -2); }
  double SurfaceDensity() const { return Factor(1, -2, 0); }
};

// One layer of a layered Earth, SI, its fields linear in radius between r0
// and r1 (a constant when both ends agree).
struct Layer {
  double r0 = 0.0, r1 = 0.0;  // metres
  bool fluid = false;
  double rho0 = 0.0, rho1 = 0.0;      // kg m^-3
  double kappa0 = 0.0, kappa1 = 0.0;  // Pa
  double mu0 = 0.0, mu1 = 0.0;        // Pa
  double viscosity = 0.0;             // Pa s; 0 = elastic
  double kelvin_fraction = 0.0;       // Burgers: Kelvin modulus / mu (0 = Maxwell)
  double kelvin_viscosity = 0.0;      // Burgers: Kelvin viscosity, Pa s
  int elements = 1;                   // radial elements in this layer
};

// The layered Earth, non-dimensional (EarthModel::Dimensionless).
class LayeredEarth {
 public:
  LayeredEarth(std::vector<Layer> layers, Scales scales);
  const Scales& scales() const { return scales_; }
  int LayerCount() const { return static_cast<int>(layers_.size()); }
  const Layer& LayerSI(int i) const { return layers_[i]; }
  double Bottom(int i) const { return r0_[i]; }
  double Top(int i) const { return r1_[i]; }
  double SurfaceRadius() const { return r1_.back(); }
  // Non-dimensional fields in a layer at radius r (nu = 1: the derivative).
  double Rho(int layer, double r, int nu = 0) const;
  double Kappa(int layer, double r) const;
  double Mu(int layer, double r) const;
  double Gravity(double r) const;  // G M(r) / r^2, segment-exact

 private:
  std::vector<Layer> layers_;
  Scales scales_;
  std::vector<double> r0_, r1_;
  std::vector<double> massBelow_;  // 4 pi int_0^{r0_i} rho s^2 ds
  double Linear(double a, double b, int layer, double r) const;
};

// RadialMesh: uniform elements per layer, ngll GLL nodes per element.
class RadialMesh {
 public:
  static RadialMesh Create(const LayeredEarth& earth, int ngll);
  int ElementCount() const { return static_cast<int>(left_.size()); }
  int NGll() const { return ngll_; }
  int NodeCount() const { return ElementCount() * (ngll_ - 1) + 1; }
  double Left(int e) const { return left_[e]; }
  double Right(int e) const { return right_[e]; }
  double Jacobian(int e) const { return jac_[e]; }
  double Radius(int e, int i) const { return radius_[static_cast<std::size_t>(e) * ngll_ + i]; }
  const std::vector<double>& Radii() const { return radius_; }
  int GlobalIndex(int e, int i) const { return e * (ngll_ - 1) + i; }
  int LayerOf(int e) const { return layer_[e]; }
  int ElementOf(double r) const;
  const std::vector<double>& Points() const { return xi_; }
  const std::vector<double>& Weights() const { return weights_; }
  double Derivative(int k, int i) const { return deriv_[static_cast<std::size_t>(k) * ngll_ + i]; }
  // The graded truncation rule r_l = rmax eps^(1/(l+1)) (RadialMesh.cpp).
  double TruncationRadius(int l, double eps) const;
  int StartElement(int l, double eps) const { return ElementOf(TruncationRadius(l, eps)); }

 private:
  int ngll_ = 0;
  std::vector<double> left_, right_, jac_, radius_, xi_, weights_, deriv_;
  std::vector<int> layer_;
};

// Material: the nodal arrays a degree system assembles from.
struct NodalModuli {
  std::vector<double> A, C, F, L, N;
  static NodalModuli Isotropic(const std::vector<double>& kappa, const std::vector<double>& mu);
  void KappaMu(std::vector<double>& kappa, std::vector<double>& mu) const;
};

struct Material {
  RadialMesh mesh;
  std::vector<double> rho, drho, g;
  std::vector<char> fluid;  // per element
  NodalModuli moduli;
  double G = 1.0, radius = 1.0, surfaceGravity = 1.0;
  bool IsFluid(int e) const { return fluid[e] != 0; }
  static Material Create(const LayeredEarth& earth, const RadialMesh& mesh);
};

// Rheology: Prony branches on the nodes (unrelaxed material's moduli).
struct Branch {
  std::vector<double> mu, itau;
};

struct PronyTerm {
  double mu = 0.0, itau = 0.0;
};
// Rheology.hpp:59-77: a Burgers body as two exact Prony terms, slower first.
std::array<PronyTerm, 2> BurgersPronyTerms(double mu, double eta, double kelvinModulus,
                                           double kelvinViscosity);

struct Rheology {
  Material material;
  std::vector<Branch> branches;
  std::vector<double> kappa, muUnrelaxed, muLongTerm;
  std::vector<char> active;
  // Maxwell per viscous layer, Burgers where the layer has a Kelvin element
  // (Rheology::Maxwell / Rheology::Burgers).
  static Rheology FromEarth(const LayeredEarth& earth, const Material& material);
  Material LongTermMaterial() const;
  bool IsActive(std::size_t node) const { return active[node] != 0; }
};

// MemoryPoints: Gauss (default) or GLL points, with the GLL Lagrange basis.
struct MemoryPoints {
  bool gauss = true;
  int count = 0, ngll = 0;
  std::vector<double> xi, weight, value, derivative;  // value/derivative: (count, ngll)
  static MemoryPoints Of(bool gauss, const RadialMesh& mesh);
  double Value(int p, int i) const { return value[static_cast<std::size_t>(p) * ngll + i]; }
  double Derivative(int p, int i) const { return derivative[static_cast<std::size_t>(p) * ngll + i]; }
  double RadiusAt(const RadialMesh& mesh, int e, int p) const;
  std::vector<double> Interpolate(const std::vector<double>& nodal) const;
};

// A shear (and optionally bulk) modulus held at the memory points.
struct PointShear {
  const MemoryPoints* points = nullptr;
  std::vector<double> modulus;  // (element, point)
  std::vector<double> bulk;     // (element, point), or empty
};

enum class Scheme { ExponentialTrapezoid = 0, BackwardEuler = 1, Sdirk2 = 2 };

// The reference operator's point moduli (Viscoelastic.cpp:120-170, 324-347):
// branch moduli and inverse times at the memory points, the long-term nodal
// material, and a step's point shear.
struct ReferenceRheology {
  Rheology rheology;
  MemoryPoints points;
  Material nodal;  // long-term material (Gauss) or the unrelaxed one (GLL)
  std::vector<std::vector<double>> pointMu, pointItau;
  PointShear elastic;
  ReferenceRheology(const Rheology& rh, bool gaussPoints);
  // Sum_k mu_k (1 - beta_k) (trapezoid) or mu_k e_k (backward Euler).
  PointShear StepShear(Scheme scheme, double dt) const;
};

double Phi1(double h, double e);
struct TrapezoidWeights {
  double e = 1.0, alpha = 0.0, beta = 0.0;
};
TrapezoidWeights ExponentialTrapezoidWeights(double h);
double BackwardEulerWeight(double h);
inline constexpr double kSdirk2Gamma = 0.29289321881345247560;

enum Component { kU = 0, kV = 1, kPhi = 2 };

// DegreeOperator: the degree-l spheroidal system with gravity.
class DegreeOperator {
 public:
  DegreeOperator(const Material& material, int l, double eps, const PointShear* pointShear);
  int Degree() const { return l_; }
  int FirstElement() const { return firstElement_; }
  int DofCount() const { return ndof_; }
  int Bandwidth() const { return kd_; }
  int Dof(int node, int c) const { return dof_[static_cast<std::size_t>(node) * 3 + c]; }
  int SurfaceDof(int c) const;
  const std::vector<double>& Band() const { return band_; }  // unscaled upper band
  // The symmetric diagonal scaling, whether every diagonal is positive, and
  // the scaled upper band (Cholesky storage) / the full scaled band in LU
  // storage (3 kd + 1 rows).
  const std::vector<double>& Scale() const { return scale_; }
  bool PositiveDiagonal() const { return positive_; }
  std::vector<double> ScaledCholeskyBand() const;
  std::vector<double> ScaledLuBand() const;
  std::vector<double> Load() const;
  std::vector<double> Tide(int power = -1) const;
  std::vector<double> Apply(const std::vector<double>& x, int nrhs) const;

 private:
  void BuildDofMap();
  void Assemble(const PointShear* pointShear);
  const Material* material_;
  int l_;
  int firstElement_ = 0, kd_ = 0, ndof_ = 0;
  bool positive_ = true;
  std::vector<int> dof_;
  std::vector<double> band_, scale_;
};

// ToroidalOperator: the degree-l (l >= 1) toroidal system.
class ToroidalOperator {
 public:
  ToroidalOperator(const Material& material, int l, double eps, const PointShear* pointShear,
                   double pinFraction = 0.0);
  int Degree() const { return l_; }
  int FirstElement() const { return firstElement_; }
  int DofCount() const { return ndof_; }
  int Bandwidth() const { return kd_; }
  int Dof(int node) const { return dof_[node]; }
  int SurfaceDof() const;
  const std::vector<int>& Pinned() const { return pinned_; }
  const std::vector<double>& Band() const { return band_; }  // unscaled upper band
  const std::vector<double>& Scale() const { return scale_; }
  std::vector<double> ScaledCholeskyBand() const;  // pinned rows/cols the identity's
  std::vector<double> Apply(const std::vector<double>& x, int nrhs) const;

 private:
  const Material* material_;
  int l_;
  int firstElement_ = 0, kd_ = 0, ndof_ = 0;
  std::vector<int> dof_, pinned_;
  std::vector<std::pair<int, int>> regions_;
  std::vector<double> band_, scale_;
};

// The BASELINE configurations' Earth: fluid core to 3480 km (10900 kg/m^3),
// mantle density 5500 -> 3300, mu 2.9e11 -> 0.7e11, kappa 6.5e11 -> 1.3e11 Pa
// (linear over the mantle), 100 km elastic lid, viscosity 5e21 below 670 km
// depth and 5e20 above, elements spread over the layers in proportion to
// thickness (largest remainder). kelvin_fraction > 0 makes the viscous
// layers Burgers bodies with that modulus fraction and viscosity / kelvin_div.
std::vector<Layer> StandardEarthLayers(int elements, double kelvin_fraction = 0.0,
                                       double kelvin_div = 10.0);

}  // namespace sl3dgpu::host
