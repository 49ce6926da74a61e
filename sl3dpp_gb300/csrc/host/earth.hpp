// Host-side radial setup of the 3D operators: the layered body and its
// non-dimensional scales, the spectral-element mesh, the nodal material,
// the Prony rheology with its memory points, and each degree's degree-of-
// freedom layout. Everything here runs once per operator (the reference does
// the same work in its constructors); the degree systems themselves are
// assembled on the GPU (assemble.cu).
//
// What each part stands for in the reference (sl3dpp):
//   Scales             include/sl3dpp/Scales.hpp (geophysical scales, G = 1)
//   LayeredBody        EarthModel (segment-exact gravity), for bodies whose
//                      fields are linear in radius within each layer
//   RadialMesh         include/sl3dpp/RadialMesh.hpp, src/RadialMesh.cpp
//                      (uniform elements per span, GLL nodes, the graded
//                      truncation r_l = a eps^(1/(l+1)))
//   Material           include/sl3dpp/Material.hpp (nodal TI moduli, density,
//                      its slope and gravity per element node)
//   Rheology           include/sl3dpp/Rheology.hpp:59-77, 125 (Maxwell and
//                      Burgers bodies as Prony terms)
//   MemoryPoints       include/sl3dpp/MemoryPoints.hpp (Gauss or GLL points)
//   RelaxingBody       src/Viscoelastic.cpp:120-170, 324-347 (branch moduli at
//                      the memory points, the long-term material, a step's
//                      point shear)
//   SpheroidalLayout   DegreeOperator's dof map, surface dofs, load and tide
//                      vectors (src/DegreeOperator.cpp:24-152, 905-1038)
//   ToroidalLayout     ToroidalOperator's dof map and gauge rows
//                      (src/ToroidalOperator.cpp)
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
inline constexpr double kSdirk2Gamma = 0.29289321881345247560;

// Units in which the gravitational constant is one: a length L, a density
// rho, mass rho L^3 and time (G rho)^-1/2.
struct Scales {
  double mass = 1.0, length = 1.0, time = 1.0;
  static Scales Geophysical(double length = kEarthRadiusSI, double density = kEarthMeanDensitySI);
  // The SI size of one model unit of mass^m length^l time^t.
  double Factor(int m, int l, int t) const;
  double Density() const { return Factor(1, -3, 0); }
  double Modulus() const { return Factor(1, -1, -2); }
  double Viscosity() const { return Factor(1, -1, -1); }
  double Potential() const { return Factor(0, 2, -2); }
  double SurfaceDensity() const { return Factor(1, -2, 0); }
};

// One layer, SI, its fields linear in radius from r0 to r1.
struct Layer {
  double r0 = 0.0, r1 = 0.0;  // metres
  bool fluid = false;
  double rho0 = 0.0, rho1 = 0.0;      // kg m^-3
  double kappa0 = 0.0, kappa1 = 0.0;  // Pa
  double mu0 = 0.0, mu1 = 0.0;        // Pa
  double viscosity = 0.0;             // Pa s; 0: elastic
  double kelvin_fraction = 0.0;       // Burgers: Kelvin modulus over mu (0: Maxwell)
  double kelvin_viscosity = 0.0;      // Burgers: Kelvin viscosity, Pa s
  int elements = 1;                   // spectral elements across the layer
};

// The layered body in model units.
class LayeredBody {
 public:
  LayeredBody(const std::vector<Layer>& layers, const Scales& scales);
  const Scales& scales() const { return scales_; }
  int Layers() const { return static_cast<int>(spans_.size()); }
  const Layer& Source(int s) const { return source_[s]; }
  double Bottom(int s) const { return spans_[s].r0; }
  double Top(int s) const { return spans_[s].r1; }
  double Surface() const { return spans_.back().r1; }
  double Density(int s, double r) const { return spans_[s].Rho(r); }
  double DensitySlope(int s) const { return spans_[s].rhoSlope; }
  double Bulk(int s, double r) const;
  double Shear(int s, double r) const;
  // G m(r) / r^2, m(r) the mass inside r, integrated exactly layer by layer.
  double Gravity(double r) const;
  double G() const { return 1.0; }

 private:
  struct Span {
    double r0, r1, rhoAt0, rhoSlope, kappaAt0, kappaSlope, muAt0, muSlope;
    double Rho(double r) const { return rhoAt0 + rhoSlope * (r - r0); }
    double MassBetween(double a, double b) const;  // 4 pi int_a^b rho s^2 ds
  };
  std::vector<Layer> source_;
  std::vector<Span> spans_;
  std::vector<double> massBelow_;
  Scales scales_;
};

// The reference element: n GLL nodes on [-1, 1], their weights, and the
// derivative of each Lagrange basis function at each node.
struct GllRule {
  int n = 0;
  std::vector<double> x, w;
  std::vector<double> d;  // d[q * n + i] = l_i'(x_q)
  static GllRule Of(int n);
  double Slope(int q, int i) const { return d[static_cast<std::size_t>(q) * n + i]; }
};

// Elements spanning each layer uniformly; every layer boundary is an element
// boundary. Global node g = e (n - 1) + i is shared by the elements it ends
// and starts.
class RadialMesh {
 public:
  static RadialMesh Create(const LayeredBody& body, int ngll);
  int ElementCount() const { return static_cast<int>(elems_.size()); }
  int NGll() const { return rule_.n; }
  int NodeCount() const { return ElementCount() * (NGll() - 1) + 1; }
  double Left(int e) const { return elems_[e].left; }
  double Right(int e) const { return elems_[e].right; }
  double Jacobian(int e) const { return 0.5 * (elems_[e].right - elems_[e].left); }
  double Radius(int e, int i) const { return nodes_[static_cast<std::size_t>(e) * NGll() + i]; }
  const std::vector<double>& Radii() const { return nodes_; }  // (element, node)
  int GlobalIndex(int e, int i) const { return e * (NGll() - 1) + i; }
  int LayerOf(int e) const { return elems_[e].layer; }
  int ElementOf(double r) const;
  const GllRule& Rule() const { return rule_; }
  const std::vector<double>& Points() const { return rule_.x; }
  const std::vector<double>& Weights() const { return rule_.w; }
  double Derivative(int q, int i) const { return rule_.Slope(q, i); }
  double TruncationRadius(int l, double eps) const;
  int StartElement(int l, double eps) const { return ElementOf(TruncationRadius(l, eps)); }

 private:
  struct Element {
    double left, right;
    int layer;
  };
  GllRule rule_;
  std::vector<Element> elems_;
  std::vector<double> nodes_;
};

// Nodal elastic moduli, transversely isotropic form (isotropic here).
struct NodalModuli {
  std::vector<double> A, C, F, L, N;
  static NodalModuli Isotropic(const std::vector<double>& kappa, const std::vector<double>& mu);
  double Kappa(std::size_t i) const { return (4.0 * A[i] + C[i] + 4.0 * F[i] - 4.0 * N[i]) / 9.0; }
  double Mu(std::size_t i) const { return (A[i] + C[i] - 2.0 * F[i] + 5.0 * N[i] + 6.0 * L[i]) / 15.0; }
};

// The material on the mesh's element nodes.
struct Material {
  RadialMesh mesh;
  std::vector<double> rho, drho, g;  // (element, node)
  std::vector<char> fluid;           // per element
  NodalModuli moduli;
  double G = 1.0, radius = 1.0, surfaceGravity = 1.0;
  bool IsFluid(int e) const { return fluid[e] != 0; }
  static Material Create(const LayeredBody& body, const RadialMesh& mesh);
  // The same material with shear modulus removed at every node (the shear a
  // relaxing branch carries, taken out of the long-term moduli).
  Material WithoutShear(const std::vector<double>& removed) const;
};

// A relaxing branch on the element nodes: shear modulus and inverse time.
struct Branch {
  std::vector<double> mu, itau;
};

struct PronyTerm {
  double mu = 0.0, itau = 0.0;
};
// A Burgers body (Maxwell mu, eta in series with Kelvin muK, etaK) as its
// two exact Prony terms, slower first.
std::array<PronyTerm, 2> BurgersPronyTerms(double mu, double eta, double kelvinModulus, double kelvinViscosity);

struct Rheology {
  Material material;
  std::vector<Branch> branches;
  std::vector<double> kappa, muUnrelaxed, muLongTerm;
  std::vector<char> active;
  // One Maxwell branch per viscous layer, two Prony branches where the layer
  // has a Kelvin element.
  static Rheology FromBody(const LayeredBody& body, const Material& material);
  Material LongTermMaterial() const;
  bool IsActive(std::size_t node) const { return active[node] != 0; }
};

// Points at which the memory lives inside each element, with the Lagrange
// basis of the element's GLL nodes evaluated there.
struct MemoryPoints {
  bool gauss = true;
  int count = 0, ngll = 0;
  std::vector<double> xi, weight, value, derivative;  // value / derivative: (count, ngll)
  static MemoryPoints Of(bool gauss, const RadialMesh& mesh);
  double Value(int p, int i) const { return value[static_cast<std::size_t>(p) * ngll + i]; }
  double Derivative(int p, int i) const { return derivative[static_cast<std::size_t>(p) * ngll + i]; }
  double RadiusAt(const RadialMesh& mesh, int e, int p) const;
  std::vector<double> Interpolate(const std::vector<double>& nodal) const;
};

// A shear modulus held at the memory points, (element, point).
struct PointShear {
  const MemoryPoints* points = nullptr;
  std::vector<double> modulus;
};

enum class Scheme { ExponentialTrapezoid = 0, BackwardEuler = 1, Sdirk2 = 2 };

// phi_1(h) = (1 - e^-h) / h (a series below |h| = 1e-3), e = e^-h.
double Phi1(double h, double e);
struct TrapezoidWeights {
  double e = 1.0, alpha = 0.0, beta = 0.0;
};
TrapezoidWeights ExponentialTrapezoidWeights(double h);
double BackwardEulerWeight(double h);

// The relaxing body as the 3D step sees it: each branch's modulus and
// inverse time at the Gauss memory points, the long-term nodal material the
// degree systems are assembled on, and a step's point shear.
struct RelaxingBody {
  Rheology rheology;
  MemoryPoints points;
  Material nodal;
  std::vector<std::vector<double>> pointMu, pointItau;
  PointShear elastic;  // sum of the branch moduli: the unrelaxed step
  explicit RelaxingBody(const Rheology& rh);
  // The modulus a step of this scheme and length leaves unrelaxed:
  // sum_k mu_k (1 - beta_k) (exponential trapezoid) or mu_k / (1 + h_k).
  PointShear StepShear(Scheme scheme, double dt) const;
};

enum Component { kU = 0, kV = 1, kPhi = 2 };

// Degree l's spheroidal unknowns: U, V, phi on the nodes of solid elements
// above the truncation radius (U and phi alone at l = 0), phi alone inside
// fluid elements; U at the centre and, at l = 1, the surface phi (the
// centre-of-mass frame) are not unknowns. Numbered node by node upwards.
class SpheroidalLayout {
 public:
  SpheroidalLayout(const Material& material, int l, double eps);
  int Degree() const { return l_; }
  int FirstElement() const { return first_; }
  int DofCount() const { return static_cast<int>(node_.size()); }
  int Bandwidth() const { return 3 * (mesh_->NGll() - 1) + 2; }
  int Dof(int node, int c) const { return map_[static_cast<std::size_t>(node) * 3 + c]; }
  int SurfaceDof(int c) const { return Dof(mesh_->NodeCount() - 1, c); }
  // dof -> (global node, component)
  const std::vector<int>& DofNodes() const { return node_; }
  const std::vector<int>& DofComponents() const { return comp_; }
  // The unit surface load's force (Viscoelastic3D's load channel).
  std::vector<double> Load() const;
  // The force of a degree-l tidal potential (r/a)^power (power < 0: l).
  std::vector<double> Tide(int power = -1) const;

 private:
  const Material* material_;
  const RadialMesh* mesh_;
  int l_, first_;
  std::vector<int> map_, node_, comp_;
};

// Degree l's toroidal unknown W on the nodes of solid elements above the
// truncation radius, numbered upwards; at l = 1 the top row of every solid
// region is held at zero (the rigid rotation's gauge).
class ToroidalLayout {
 public:
  ToroidalLayout(const Material& material, int l, double eps);
  int Degree() const { return l_; }
  int FirstElement() const { return first_; }
  int DofCount() const { return static_cast<int>(node_.size()); }
  int Bandwidth() const { return mesh_->NGll() - 1; }
  int Dof(int node) const { return map_[node]; }
  int SurfaceDof() const { return map_[mesh_->NodeCount() - 1]; }
  const std::vector<int>& DofNodes() const { return node_; }
  const std::vector<int>& Pinned() const { return pinned_; }

 private:
  const RadialMesh* mesh_;
  int l_, first_;
  std::vector<int> map_, node_, pinned_;
};

// The configurations' body: a fluid core to 3480 km (10900 kg/m^3), mantle
// density 5500 -> 3300, mu 2.9e11 -> 0.7e11, kappa 6.5e11 -> 1.3e11 Pa
// (linear over the mantle), a 100 km elastic lid, viscosity 5e21 below 670 km
// depth and 5e20 above, elements in proportion to thickness (largest
// remainder). kelvin_fraction > 0 makes the viscous layers Burgers bodies
// with that modulus fraction and viscosity / kelvin_div.
std::vector<Layer> StandardEarthLayers(int elements, double kelvin_fraction = 0.0, double kelvin_div = 10.0);

}  // namespace sl3dgpu::host
