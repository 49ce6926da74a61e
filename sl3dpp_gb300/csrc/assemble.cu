// The degree systems assembled on the GPU (see assemble.cuh).
#include <algorithm>
#include <cmath>

#include "assemble.cuh"
#include "profile.cuh"

namespace sl3dgpu {
namespace {

constexpr int kU = 0, kV = 1, kPhi = 2;
constexpr double kPiD = 3.14159265358979323846;

// The view of a DeviceMaterial a kernel takes by value.
struct MaterialView {
  int E, n, np;
  double radius, ifpg;
  const double *r, *jac, *rho, *drho, *g, *A, *C, *F, *L, *N;
  const unsigned char* fluid;
  const double *w, *d, *pw, *pv, *pd;
};

// The spheroidal pair (a, ca), (b, cb) of element e's local nodes: the
// element's share of the stored entry. The weak form's terms, per GLL
// quadrature node q (weight W = w_q jac, radius r, rb_a = r dl_a/dr there):
//   elastic, with x = r dU/dr, y = 2U - k^2 V, s = r dV/dr + U - V:
//     W [C x x + (A - N) y y + F (x y + y x) + k^2 L s s + k^2 (k^2 - 2) N V V]
//   self-gravitation: W [4 rho (pi G rho r - g) r U U + k^2 rho g r (U V + V U)
//     + k^2 rho r (V phi + phi V)] + rho r^2 (U dphi/dr + dphi/dr U) r-weighted
//   potential: (1 / 4 pi G) [r^2 dphi/dr dpsi/dr + k^2 phi psi]
// fluid elements (l > 0) keep the potential and the stratification
// r^2 rho' / g phi psi; the relaxing branches add, at each memory point p
// (weight w_p jac times the step's unrelaxed shear), with v the basis value
// and t = r_p dl/dr:
//   k^2 (k^2 - 2) V V + 4/3 (t U - U + k^2 V / 2)^2 + k^2 (U + t V - V)^2.
__host__ __device__ double SpheroidalElement(const MaterialView& m, const double* shear, int l, int e, int a, int ca, int b,
                                    int cb) {
  const int n = m.n;
  const double k2 = l * (l + 1.0);
  const double jac = m.jac[e];
  const int base = e * n;
  double value = 0.0;
  if (ca == kPhi && cb == kPhi) {
    double grad = 0.0;
    for (int q = 0; q < n; ++q) {
      const double rq = m.r[base + q];
      grad += m.d[q * n + a] * m.d[q * n + b] * m.w[q] * rq * rq;
    }
    value += m.ifpg * grad / jac;
    if (a == b) value += m.ifpg * k2 * m.w[a] * jac;
  }
  const bool fluid = l > 0 && m.fluid[e];
  if (fluid) {
    if (ca == kPhi && cb == kPhi && a == b && m.g[base + a] > 0.0) {
      const double ra = m.r[base + a];
      value += ra * ra * m.drho[base + a] / m.g[base + a] * m.w[a] * jac;
    }
    return value;
  }
  if (ca == kPhi && cb == kPhi) return value;  // the solid's elastic and point terms hold no phi
  // elastic quadrature over the element's nodes
  if (ca != kPhi && cb != kPhi) {
    for (int q = 0; q < n; ++q) {
      const double rq = m.r[base + q];
      const double ta = rq * m.d[q * n + a] / jac, tb = rq * m.d[q * n + b] / jac;
      const double da = a == q ? 1.0 : 0.0, db = b == q ? 1.0 : 0.0;
      const double xa = ca == kU ? ta : 0.0, xb = cb == kU ? tb : 0.0;
      const double ya = ca == kU ? 2.0 * da : -k2 * da, yb = cb == kU ? 2.0 * db : -k2 * db;
      const double sa = ca == kU ? da : ta - da, sb = cb == kU ? db : tb - db;
      const int k = base + q;
      const double Wq = m.w[q] * jac;
      double t = m.C[k] * xa * xb + (m.A[k] - m.N[k]) * ya * yb + m.F[k] * (xa * yb + ya * xb) + k2 * m.L[k] * sa * sb;
      if (ca == kV && cb == kV && a == q && b == q) t += k2 * (k2 - 2.0) * m.N[k];
      value += Wq * t;
    }
  }
  // self-gravitation at the nodes (GLL collocation)
  if (a == b) {
    const int k = base + a;
    const double r = m.r[k], rho = m.rho[k], g = m.g[k], Wq = m.w[a] * jac;
    const double piG = 0.25 / m.ifpg;
    if (ca == kU && cb == kU) value += 4.0 * rho * (piG * rho * r - g) * r * Wq;
    if ((ca == kU && cb == kV) || (ca == kV && cb == kU)) value += k2 * rho * g * r * Wq;
    if ((ca == kV && cb == kPhi) || (ca == kPhi && cb == kV)) value += k2 * rho * r * Wq;
  }
  if (ca == kU && cb == kPhi) {
    const double r = m.r[base + a];
    value += m.rho[base + a] * r * r * m.w[a] * m.d[a * n + b];
  } else if (ca == kPhi && cb == kU) {
    const double r = m.r[base + b];
    value += m.rho[base + b] * r * r * m.w[b] * m.d[b * n + a];
  }
  // the relaxing branches' shear at the memory points
  if (shear != nullptr && ca != kPhi && cb != kPhi) {
    for (int p = 0; p < m.np; ++p) {
      const double s = shear[e * m.np + p];
      if (s == 0.0) continue;
      double rp = 0.0;
      for (int i = 0; i < n; ++i) rp += m.pv[p * n + i] * m.r[base + i];
      const double va = m.pv[p * n + a], vb = m.pv[p * n + b];
      const double ta = rp * m.pd[p * n + a] / jac, tb = rp * m.pd[p * n + b] / jac;
      const double ra = ca == kU ? ta - va : 0.5 * k2 * va, rb = cb == kU ? tb - vb : 0.5 * k2 * vb;
      const double sa = ca == kU ? va : ta - va, sb = cb == kU ? vb : tb - vb;
      const double ma = ca == kV ? va : 0.0, mb = cb == kV ? vb : 0.0;
      value += m.pw[p] * jac * s * (k2 * (k2 - 2.0) * ma * mb + (4.0 / 3.0) * ra * rb + k2 * sa * sb);
    }
  }
  return value;
}

// The toroidal pair (a, b) of solid element e: W [k^2 L t t + k^2 (k^2 - 2) N w w]
// with t = r dW/dr - W, and the branches' shear at the memory points.
__host__ __device__ double ToroidalElement(const MaterialView& m, const double* shear, int l, int e, int a, int b) {
  const int n = m.n;
  const double k2 = l * (l + 1.0);
  const double jac = m.jac[e];
  const int base = e * n;
  double value = 0.0;
  for (int q = 0; q < n; ++q) {
    const double rq = m.r[base + q];
    const double ta = rq * m.d[q * n + a] / jac - (a == q ? 1.0 : 0.0);
    const double tb = rq * m.d[q * n + b] / jac - (b == q ? 1.0 : 0.0);
    value += m.w[q] * jac * k2 * m.L[base + q] * ta * tb;
  }
  if (a == b) value += m.w[a] * jac * k2 * (k2 - 2.0) * m.N[base + a];
  if (shear != nullptr)
    for (int p = 0; p < m.np; ++p) {
      const double s = shear[e * m.np + p];
      if (s == 0.0) continue;
      double rp = 0.0;
      for (int i = 0; i < n; ++i) rp += m.pv[p * n + i] * m.r[base + i];
      const double va = m.pv[p * n + a], vb = m.pv[p * n + b];
      const double ta = rp * m.pd[p * n + a] / jac - va, tb = rp * m.pd[p * n + b] / jac - vb;
      value += m.pw[p] * jac * s * (k2 * ta * tb + k2 * (k2 - 2.0) * va * vb);
    }
  return value;
}

// Entry (i, j), i <= j, of one system's band: the elements holding both
// unknowns' nodes (at most two, when both are one node shared by
// neighbours), then the point terms of the fluid-solid boundaries and the
// exterior closures.
__host__ __device__ double BandEntry(const MaterialView& m, const AssemblySystem& s, const int* dofNode,
                                     const signed char* dofComp, const double* shear, int i, int j) {
  const int n1 = m.n - 1;
  const int gi = dofNode[s.dofs + i], gj = dofNode[s.dofs + j];
  if (gj - gi > n1) return 0.0;
  const int ci = s.toroidal ? 0 : dofComp[s.dofs + i], cj = s.toroidal ? 0 : dofComp[s.dofs + j];
  const int lowest = (gj + n1 - 1) / n1 - 1, highest = gi / n1;
  const int eLo = lowest > s.first ? lowest : s.first, eHi = highest < m.E - 1 ? highest : m.E - 1;
  double value = 0.0;
  for (int e = eLo; e <= eHi; ++e) {
    const int a = gi - e * n1, b = gj - e * n1;
    if (s.toroidal) {
      if (!m.fluid[e]) value += ToroidalElement(m, shear, s.l, e, a, b);
    } else {
      value += SpheroidalElement(m, shear, s.l, e, a, ci, b, cj);
    }
  }
  if (!s.toroidal && gi == gj) {
    // fluid-solid boundaries (l > 0): the fluid's weight and its potential
    // acting on the boundary's normal motion
    const int eBelow = gi / n1 - 1;
    if (s.l > 0 && gi % n1 == 0 && eBelow >= s.first && eBelow + 1 < m.E && m.fluid[eBelow] != m.fluid[eBelow + 1] &&
        ci == kU) {
      const bool fluidBelow = m.fluid[eBelow] != 0;
      const int kTop = eBelow * m.n + n1;
      const double rt = m.r[kTop], gt = m.g[kTop];
      const double rhoF = fluidBelow ? m.rho[kTop] : m.rho[(eBelow + 1) * m.n];
      const double sign = fluidBelow ? 1.0 : -1.0;
      if (cj == kU) value += sign * rhoF * gt * rt * rt;
      if (cj == kPhi) value += sign * rhoF * rt * rt;
    }
    // the exterior (Dirichlet-to-Neumann) closures of the potential
    if (ci == kPhi && cj == kPhi) {
      if (gi == m.E * n1 && s.l != 1) value += (s.l + 1.0) * m.radius * m.ifpg;
      const double bottom = m.r[s.first * m.n];
      if (gi == s.first * n1 && bottom > 0.0) value += s.l * bottom * m.ifpg;
    }
  }
  return value;
}

// One thread per stored entry (row i = j - kd + t of column j) of one
// system's upper band, blockIdx.y the system.
__global__ void AssembleKernel(MaterialView m, const AssemblySystem* systems, const int* dofNode,
                               const signed char* dofComp, const double* shear, double* bands) {
  const AssemblySystem s = systems[blockIdx.y];
  const int ld = s.kd + 1;
  const long long entries = static_cast<long long>(ld) * s.ndof;
  for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < entries;
       idx += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int j = static_cast<int>(idx / ld);
    const int i = j - s.kd + static_cast<int>(idx % ld);
    bands[s.band + idx] = i >= 0 ? BandEntry(m, s, dofNode, dofComp, shear, i, j) : 0.0;
  }
}

// Per unknown: s = 1 / sqrt|diag| (1 where the diagonal vanishes) and the
// positivity flag of its system (cleared by any non-positive diagonal).
__global__ void ScalesKernel(const AssemblySystem* systems, const long long* scaleOffset, const double* raw,
                             double* scales, int* positive) {
  const AssemblySystem s = systems[blockIdx.y];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < s.ndof; j += gridDim.x * blockDim.x) {
    const double d = raw[s.band + static_cast<long long>(j) * (s.kd + 1) + s.kd];
    scales[scaleOffset[blockIdx.y] + j] = 1.0 / sqrt(fabs(d) > 0.0 ? fabs(d) : 1.0);
    if (!(d > 0.0)) positive[blockIdx.y] = 0;
  }
}

// The scaled upper band; a toroidal gauge row and column become the
// identity's.
__global__ void ScaledBandKernel(const AssemblySystem* systems, const long long* scaleOffset, const double* raw,
                                 const double* scales, double* scaled) {
  const AssemblySystem s = systems[blockIdx.y];
  const int ld = s.kd + 1;
  const long long entries = static_cast<long long>(ld) * s.ndof;
  const double* sc = scales + scaleOffset[blockIdx.y];
  for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < entries;
       idx += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int j = static_cast<int>(idx / ld), i = j - s.kd + static_cast<int>(idx % ld);
    double v = 0.0;
    if (i >= 0) {
      v = raw[s.band + idx] * sc[i] * sc[j];
      const bool gauge = i == s.pinned0 || j == s.pinned0 || i == s.pinned1 || j == s.pinned1;
      if (gauge) v = i == j ? 1.0 : 0.0;
    }
    scaled[s.band + idx] = v;
  }
}

// LU storage of a scaled symmetric band: row 2 kd + i - j of column j holds
// entry (i, j) for |i - j| <= kd; rows above are the factorisation's fill-in.
__global__ void LuBandKernel(const AssemblySystem* systems, const int* which, const long long* outOffset,
                             const long long* scaleOffset, const double* raw, const double* scales, double* out) {
  const int sys = which[blockIdx.y];
  const AssemblySystem s = systems[sys];
  const int ldu = s.kd + 1, ldlu = 3 * s.kd + 1;
  const long long entries = static_cast<long long>(ldlu) * s.ndof;
  const double* sc = scales + scaleOffset[sys];
  for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < entries;
       idx += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int j = static_cast<int>(idx / ldlu), row = static_cast<int>(idx % ldlu);
    const int i = j + row - 2 * s.kd;
    double v = 0.0;
    if (row >= s.kd && i >= 0 && i < s.ndof) {
      const int lo = min(i, j), hi = max(i, j);
      v = raw[s.band + static_cast<long long>(hi) * ldu + (s.kd + lo - hi)] * sc[i] * sc[j];
    }
    out[outOffset[blockIdx.y] + idx] = v;
  }
}

unsigned BlocksFor(long long entries) {
  return static_cast<unsigned>(std::clamp<long long>((entries + 255) / 256, 1, 1024));
}

}  // namespace

int DeviceMaterial::Upload(const host::Material& material, const host::MemoryPoints& pts) {
  const host::RadialMesh& mesh = material.mesh;
  elements = mesh.ElementCount();
  ngll = mesh.NGll();
  points = pts.count;
  radius = material.radius;
  fourPiGInverse = 1.0 / (4.0 * kPiD * material.G);
  std::vector<double> jacs(elements);
  hostLeft.resize(elements);
  for (int e = 0; e < elements; ++e) {
    jacs[e] = mesh.Jacobian(e);
    hostLeft[e] = mesh.Left(e);
  }
  hostFluid.assign(material.fluid.begin(), material.fluid.end());
  std::vector<unsigned char> fl(material.fluid.begin(), material.fluid.end());
  SL3D_CUDA(r.Upload(mesh.Radii()));
  SL3D_CUDA(jac.Upload(jacs));
  SL3D_CUDA(fluid.Upload(fl));
  SL3D_CUDA(rho.Upload(material.rho));
  SL3D_CUDA(drho.Upload(material.drho));
  SL3D_CUDA(g.Upload(material.g));
  SL3D_CUDA(A.Upload(material.moduli.A));
  SL3D_CUDA(C.Upload(material.moduli.C));
  SL3D_CUDA(F.Upload(material.moduli.F));
  SL3D_CUDA(L.Upload(material.moduli.L));
  SL3D_CUDA(N.Upload(material.moduli.N));
  SL3D_CUDA(w.Upload(mesh.Weights()));
  SL3D_CUDA(d.Upload(mesh.Rule().d));
  SL3D_CUDA(pw.Upload(pts.weight));
  SL3D_CUDA(pv.Upload(pts.value));
  SL3D_CUDA(pd.Upload(pts.derivative));
  return SL3DGPU_OK;
}

void AssemblyPlan::Add(const host::SpheroidalLayout& s) {
  AssemblySystem a{};
  a.l = s.Degree();
  a.toroidal = 0;
  a.first = s.FirstElement();
  a.ndof = s.DofCount();
  a.kd = s.Bandwidth();
  a.band = bandDoubles;
  a.dofs = static_cast<long long>(dofNode.size());
  a.pinned0 = a.pinned1 = -1;
  dofNode.insert(dofNode.end(), s.DofNodes().begin(), s.DofNodes().end());
  for (int c : s.DofComponents()) dofComp.push_back(static_cast<signed char>(c));
  bandDoubles += static_cast<long long>(a.kd + 1) * a.ndof;
  systems.push_back(a);
}

void AssemblyPlan::Add(const host::ToroidalLayout& t) {
  AssemblySystem a{};
  a.l = t.Degree();
  a.toroidal = 1;
  a.first = t.FirstElement();
  a.ndof = t.DofCount();
  a.kd = t.Bandwidth();
  a.band = bandDoubles;
  a.dofs = static_cast<long long>(dofNode.size());
  a.pinned0 = t.Pinned().size() > 0 ? t.Pinned()[0] : -1;
  a.pinned1 = t.Pinned().size() > 1 ? t.Pinned()[1] : -1;
  dofNode.insert(dofNode.end(), t.DofNodes().begin(), t.DofNodes().end());
  dofComp.insert(dofComp.end(), t.DofNodes().size(), 0);
  bandDoubles += static_cast<long long>(a.kd + 1) * a.ndof;
  systems.push_back(a);
}

int AssembleAndScale(const DeviceMaterial& mat, const AssemblyPlan& plan, const double* shear,
                     AssembledSystems& out, cudaStream_t stream) {
  const int count = static_cast<int>(plan.systems.size());
  if (count == 0) return SL3DGPU_OK;
  for (const auto& s : plan.systems)
    if ((s.pinned0 >= 0 || s.pinned1 >= 0) && s.toroidal == 0) {
      SetError("assembly: gauge rows belong to toroidal systems");
      return SL3DGPU_ERR_ARGUMENT;
    }
  Dev<int> dofNode;
  Dev<signed char> dofComp;
  Dev<long long> scaleOffsets;
  Dev<int> positive;
  SL3D_CUDA(dofNode.Upload(plan.dofNode));
  SL3D_CUDA(dofComp.Upload(plan.dofComp));
  SL3D_CUDA(out.dSystems.Upload(plan.systems));
  out.scaleOffset.assign(count, 0);
  long long unknowns = 0, largest = 0;
  for (int k = 0; k < count; ++k) {
    out.scaleOffset[k] = unknowns;
    unknowns += plan.systems[k].ndof;
    largest = std::max(largest, static_cast<long long>(plan.systems[k].kd + 1) * plan.systems[k].ndof);
  }
  SL3D_CUDA(scaleOffsets.Upload(out.scaleOffset));
  SL3D_CUDA(positive.Upload(std::vector<int>(count, 1)));
  SL3D_CUDA(out.raw.Alloc(plan.bandDoubles));
  SL3D_CUDA(out.scaled.Alloc(plan.bandDoubles));
  SL3D_CUDA(out.scales.Alloc(unknowns));
  const MaterialView view{mat.elements, mat.ngll, mat.points, mat.radius, mat.fourPiGInverse, mat.r.p, mat.jac.p,
                          mat.rho.p, mat.drho.p, mat.g.p, mat.A.p, mat.C.p, mat.F.p, mat.L.p, mat.N.p, mat.fluid.p,
                          mat.w.p, mat.d.p, mat.pw.p, mat.pv.p, mat.pd.p};
  const dim3 grid(BlocksFor(largest), static_cast<unsigned>(count));
  {
    prof::Scope scope(prof::kOther, stream);
    AssembleKernel<<<grid, 256, 0, stream>>>(view, out.dSystems.p, dofNode.p, dofComp.p, shear, out.raw.p);
    SL3D_CHECK_LAUNCH();
  }
  {
    prof::Scope scope(prof::kOther, stream);
    ScalesKernel<<<dim3(8, count), 256, 0, stream>>>(out.dSystems.p, scaleOffsets.p, out.raw.p, out.scales.p,
                                                     positive.p);
    SL3D_CHECK_LAUNCH();
  }
  {
    prof::Scope scope(prof::kOther, stream);
    ScaledBandKernel<<<grid, 256, 0, stream>>>(out.dSystems.p, scaleOffsets.p, out.raw.p, out.scales.p,
                                               out.scaled.p);
    SL3D_CHECK_LAUNCH();
  }
  out.positive.assign(count, 0);
  SL3D_CUDA(cudaMemcpyAsync(out.positive.data(), positive.p, count * sizeof(int), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));  // the lists above are freed on return
  return SL3DGPU_OK;
}

int LuBands(const AssembledSystems& in, const std::vector<int>& which, const AssemblyPlan& plan,
            const std::vector<long long>& offsets, double* out, cudaStream_t stream) {
  if (which.empty()) return SL3DGPU_OK;
  Dev<int> dWhich;
  Dev<long long> dOffsets, scaleOffsets;
  SL3D_CUDA(dWhich.Upload(which));
  SL3D_CUDA(dOffsets.Upload(offsets));
  SL3D_CUDA(scaleOffsets.Upload(in.scaleOffset));
  long long largest = 0;
  for (int k : which)
    largest = std::max(largest, static_cast<long long>(3 * plan.systems[k].kd + 1) * plan.systems[k].ndof);
  {
    prof::Scope scope(prof::kOther, stream);
    LuBandKernel<<<dim3(BlocksFor(largest), static_cast<unsigned>(which.size())), 256, 0, stream>>>(
        in.dSystems.p, dWhich.p, dOffsets.p, scaleOffsets.p, in.raw.p, in.scales.p, out);
    SL3D_CHECK_LAUNCH();
  }
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu
