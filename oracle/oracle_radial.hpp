// The oracle's radial setup (test infrastructure only): the layered body,
// its spectral-element mesh, material, rheology and memory points, and each
// degree's spheroidal and toroidal system, assembled on the CPU in FP64.
//
// This is the checker's own restatement, kept apart from the library's (the
// library assembles its bands on the GPU, one thread per stored entry;
// here each element's matrix is the quadrature sum of F^T M F over a list of
// strain-like functionals F of the element's unknowns and a small symmetric
// material matrix M at each quadrature point, then scattered into the band),
// so that an error in either shows up as a disagreement. It follows the
// reference's weak form (Al-Attar & Tromp 2014 eq. D76 for the spheroidal
// system, src/DegreeOperator.cpp:24-474 and 775-1038; the toroidal system of
// src/ToroidalOperator.cpp), mesh (src/RadialMesh.cpp: uniform elements per
// layer, GLL nodes, graded truncation), material (include/sl3dpp/
// Material.hpp), rheology (include/sl3dpp/Rheology.hpp:59-77), memory
// points (include/sl3dpp/MemoryPoints.hpp) and the reference operator's
// point moduli (src/Viscoelastic.cpp:120-170, 324-347).
#pragma once

#include <array>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

inline constexpr double kG_SI = 6.6743e-11;
inline constexpr double kRhoEarth = 5515.0;
inline constexpr double kPi = 3.14159265358979323846;
inline constexpr double kSdirk2Gamma = 0.29289321881345247560;

struct Scales {
  double mass = 1.0, length = 1.0, time = 1.0;
  static Scales Geophysical(double length, double density = kRhoEarth);
  double Factor(int m, int l, int t) const;
  double Density() const { return Factor(1, -3, 0); }
  double Modulus() const { return Factor(1, -1, -2); }
  double Viscosity() const { return Factor(1, -1, -1); }
  double Potential() const { return Factor(0, 2, -2); }
  double SurfaceDensity() const { return Factor(1, -2, 0); }
};

struct Layer {
  double r0 = 0.0, r1 = 0.0;
  bool fluid = false;
  double rho0 = 0.0, rho1 = 0.0, kappa0 = 0.0, kappa1 = 0.0, mu0 = 0.0, mu1 = 0.0;
  double viscosity = 0.0, kelvin_fraction = 0.0, kelvin_viscosity = 0.0;
  int elements = 1;
};

class LayeredEarth {
 public:
  LayeredEarth(std::vector<Layer> layers, Scales scales);
  const Scales& scales() const { return scales_; }
  int LayerCount() const { return static_cast<int>(layers_.size()); }
  const Layer& LayerSI(int i) const { return layers_[i]; }
  double Bottom(int i) const { return layers_[i].r0 / scales_.length; }
  double Top(int i) const { return layers_[i].r1 / scales_.length; }
  double Value(int i, double atBottom, double atTop, double r) const;  // SI ends, model radius
  double Gravity(double r) const;

 private:
  std::vector<Layer> layers_;
  Scales scales_;
};

class RadialMesh {
 public:
  static RadialMesh Create(const LayeredEarth& earth, int ngll);
  int ElementCount() const { return static_cast<int>(left_.size()); }
  int NGll() const { return n_; }
  int NodeCount() const { return ElementCount() * (n_ - 1) + 1; }
  double Left(int e) const { return left_[e]; }
  double Right(int e) const { return right_[e]; }
  double Jacobian(int e) const { return 0.5 * (right_[e] - left_[e]); }
  double Radius(int e, int i) const { return radius_[static_cast<std::size_t>(e) * n_ + i]; }
  int GlobalIndex(int e, int i) const { return e * (n_ - 1) + i; }
  int LayerOf(int e) const { return layer_[e]; }
  int ElementOf(double r) const;
  const std::vector<double>& Points() const { return xi_; }
  const std::vector<double>& Weights() const { return w_; }
  double Derivative(int q, int i) const { return d_[static_cast<std::size_t>(q) * n_ + i]; }
  double TruncationRadius(int l, double eps) const;
  int StartElement(int l, double eps) const { return ElementOf(TruncationRadius(l, eps)); }

 private:
  int n_ = 0;
  std::vector<double> left_, right_, radius_, xi_, w_, d_;
  std::vector<int> layer_;
};

struct NodalModuli {
  std::vector<double> A, C, F, L, N;
};

struct Material {
  RadialMesh mesh;
  std::vector<double> rho, drho, g;
  std::vector<char> fluid;
  NodalModuli moduli;
  double G = 1.0, radius = 1.0, surfaceGravity = 1.0;
  bool IsFluid(int e) const { return fluid[e] != 0; }
  static Material Create(const LayeredEarth& earth, const RadialMesh& mesh);
};

struct Branch {
  std::vector<double> mu, itau;
};

struct Rheology {
  Material material;
  std::vector<Branch> branches;
  std::vector<char> active;
  static Rheology FromEarth(const LayeredEarth& earth, const Material& material);
  bool IsActive(std::size_t node) const { return active[node] != 0; }
};

struct MemoryPoints {
  bool gauss = true;
  int count = 0, ngll = 0;
  std::vector<double> xi, weight, value, derivative;
  static MemoryPoints Of(bool gauss, const RadialMesh& mesh);
  double Value(int p, int i) const { return value[static_cast<std::size_t>(p) * ngll + i]; }
  double Derivative(int p, int i) const { return derivative[static_cast<std::size_t>(p) * ngll + i]; }
  double RadiusAt(const RadialMesh& mesh, int e, int p) const;
};

struct PointShear {
  const MemoryPoints* points = nullptr;
  std::vector<double> modulus;  // (element, point)
};

enum class Scheme { ExponentialTrapezoid = 0, BackwardEuler = 1, Sdirk2 = 2 };

struct TrapezoidWeights {
  double e = 1.0, alpha = 0.0, beta = 0.0;
};
TrapezoidWeights ExponentialTrapezoidWeights(double h);
double BackwardEulerWeight(double h);

struct ReferenceRheology {
  Rheology rheology;
  MemoryPoints points;
  Material nodal;  // the long-term material
  std::vector<std::vector<double>> pointMu, pointItau;
  PointShear elastic;
  explicit ReferenceRheology(const Rheology& rh);
  PointShear StepShear(Scheme scheme, double dt) const;
};

enum Component { kU = 0, kV = 1, kPhi = 2 };

class DegreeOperator {
 public:
  DegreeOperator(const Material& material, int l, double eps, const PointShear* shear);
  int DofCount() const { return ndof_; }
  int Bandwidth() const { return kd_; }
  int FirstElement() const { return first_; }
  int Dof(int node, int c) const { return dof_[static_cast<std::size_t>(node) * 3 + c]; }
  int SurfaceDof(int c) const { return Dof(material_->mesh.NodeCount() - 1, c); }
  const std::vector<double>& Band() const { return band_; }
  const std::vector<double>& Scale() const { return scale_; }
  bool PositiveDiagonal() const { return positive_; }
  std::vector<double> ScaledCholeskyBand() const;
  std::vector<double> ScaledLuBand() const;
  std::vector<double> Load() const;
  std::vector<double> Tide(int power = -1) const;

 private:
  const Material* material_;
  int l_, first_ = 0, kd_ = 0, ndof_ = 0;
  bool positive_ = true;
  std::vector<int> dof_;
  std::vector<double> band_, scale_;
};

class ToroidalOperator {
 public:
  ToroidalOperator(const Material& material, int l, double eps, const PointShear* shear);
  int DofCount() const { return ndof_; }
  int Bandwidth() const { return kd_; }
  int Dof(int node) const { return dof_[node]; }
  int SurfaceDof() const { return dof_[material_->mesh.NodeCount() - 1]; }
  const std::vector<int>& Pinned() const { return pinned_; }
  const std::vector<double>& Band() const { return band_; }
  const std::vector<double>& Scale() const { return scale_; }
  std::vector<double> ScaledCholeskyBand() const;

 private:
  const Material* material_;
  int l_, kd_ = 0, ndof_ = 0;
  std::vector<int> dof_, pinned_;
  std::vector<double> band_, scale_;
};

// y = K x for a symmetric K stored as an upper band ((kd + 1) x n, LAPACK),
// nrhs columns of n end to end.
std::vector<double> ApplySymmetricBand(const std::vector<double>& band, int n, int kd, const std::vector<double>& x,
                                       int nrhs);

std::vector<Layer> StandardEarthLayers(int elements, double kelvin_fraction = 0.0, double kelvin_div = 10.0);

}  // namespace orc
