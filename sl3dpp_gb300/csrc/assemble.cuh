// The degree systems assembled on the GPU, every degree of a flavour in one
// launch.
//
// The reference assembles each degree's band on the host, element by element
// (src/DegreeOperator.cpp:253-474 for the spheroidal system of the weak form
// of Al-Attar & Tromp 2014 eq. D76, src/ToroidalOperator.cpp for the
// toroidal one). Here one thread computes one stored entry of one degree's
// upper band directly: it finds the element(s) holding both of its unknowns
// and evaluates the weak form's bilinear terms for that pair of basis
// functions by the elements' GLL quadrature and memory-point sums. No
// element matrix is formed and nothing is scattered; every entry is written
// once, so the result does not depend on thread order. Scaling (the
// symmetric diagonal scaling of DegreeOperator::Factorise,
// src/DegreeOperator.cpp:775-852), the positivity test that picks Cholesky
// and the LU storage of a fallback follow as separate batched kernels.
#pragma once

#include <vector>

#include "common.cuh"
#include "host/earth.hpp"
#include "systems.cuh"

namespace sl3dgpu {

// One system to assemble: the degree, which family, its element subset,
// size and bandwidth, where its band goes and where its unknowns' (node,
// component) lists start.
struct AssemblySystem {
  int l;
  int toroidal;   // 0 spheroidal (U, V, phi), 1 toroidal (W)
  int first;      // first element of the degree's subset
  int ndof, kd;
  long long band;  // offset (doubles) of its (kd + 1) x ndof upper band
  long long dofs;  // offset of its unknowns in the node / component lists
  int pinned0, pinned1;  // toroidal gauge rows, -1 none
};

// The mesh and material on the device, made once per operator: node radii,
// element half-widths and fluid flags, the nodal density, its slope,
// gravity and the five moduli, the GLL rule and the memory points.
struct DeviceMaterial {
  int elements = 0, ngll = 0, points = 0;
  double radius = 1.0, fourPiGInverse = 0.0;
  Dev<double> r, jac, rho, drho, g, A, C, F, L, N;
  Dev<unsigned char> fluid;
  Dev<double> w, d, pw, pv, pd;
  std::vector<char> hostFluid;
  std::vector<double> hostLeft;
  int Upload(const host::Material& material, const host::MemoryPoints& points);
};

// Unknown lists of a set of layouts: for each system, its unknowns' global
// nodes and components (0 U, 1 V, 2 phi; toroidal 0), end to end.
struct AssemblyPlan {
  std::vector<AssemblySystem> systems;
  std::vector<int> dofNode;
  std::vector<signed char> dofComp;
  long long bandDoubles = 0;
  void Add(const host::SpheroidalLayout& s);
  void Add(const host::ToroidalLayout& t);
};

// Assemble the plan's raw bands into `bands` (plan.bandDoubles values) with
// the point shear `shear` ((element, point) values, device; null: none).
// Then the symmetric scaling s = 1 / sqrt|diag| into `scales` (one per
// unknown, end to end in plan order; `scaleOffsets` receives each system's
// start), the scaled bands into `scaled` (toroidal gauge rows the identity's)
// and, per system, whether every diagonal was positive. Synchronises.
struct AssembledSystems {
  Dev<double> raw, scaled, scales;
  std::vector<long long> scaleOffset;
  std::vector<int> positive;
  Dev<AssemblySystem> dSystems;
};
int AssembleAndScale(const DeviceMaterial& mat, const AssemblyPlan& plan, const double* shear,
                     AssembledSystems& out, cudaStream_t stream);

// LU storage (2 kd + kd + 1 rows, the fill-in rows zero) of the scaled
// symmetric band of each listed system, built on the device from the raw
// band and the scales; `offsets` gives each output band's start in `out`.
int LuBands(const AssembledSystems& in, const std::vector<int>& which, const AssemblyPlan& plan,
            const std::vector<long long>& offsets, double* out, cudaStream_t stream);

}  // namespace sl3dgpu
