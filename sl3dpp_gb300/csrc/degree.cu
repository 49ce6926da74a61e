// The degree systems through the C ABI: DegreeOperator and ToroidalOperator
// (include/sl3dpp/DegreeOperator.hpp:94-384, src/DegreeOperator.cpp:24-505,
// src/ToroidalOperator.cpp) of one degree on the unrelaxed material of a
// layered earth -- its dof map, load and tide vectors and product on the
// host, its band assembled and scaled on the GPU (assemble.cu) and its
// solves on the GPU through the band drop-ins (the scaled band factorised
// once, Cholesky where every diagonal is positive, LU otherwise, as
// DegreeOperator::Factorise chooses).
#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "assemble.cuh"
#include "common.cuh"
#include "host/earth.hpp"

using namespace sl3dgpu;

struct sl3dgpu_degree {
  std::unique_ptr<host::LayeredBody> earth;
  std::unique_ptr<host::RadialMesh> mesh;
  std::unique_ptr<host::Material> material;
  std::unique_ptr<host::SpheroidalLayout> sph;
  std::unique_ptr<host::ToroidalLayout> tor;
  std::vector<double> band;    // the assembled (unscaled) upper band
  std::vector<double> factor;  // the factorised scaled band
  std::vector<int> pivots;     // LU only
  std::vector<double> scale;
  std::vector<int> pinned;     // toroidal rows held at zero
  int n = 0, kd = 0;
  bool cholesky = true;
};

namespace {

// The degree's band assembled and scaled on the GPU, copied to the host:
// raw band, scales, and the scaled band in Cholesky or LU storage.
int AssembleOne(sl3dgpu_degree& h, bool& positive, std::vector<double>& luBand) {
  AssemblyPlan plan;
  if (h.tor)
    plan.Add(*h.tor);
  else
    plan.Add(*h.sph);
  const auto points = host::MemoryPoints::Of(true, *h.mesh);
  DeviceMaterial mat;
  SL3D_TRY(mat.Upload(*h.material, points));
  AssembledSystems a;
  SL3D_TRY(AssembleAndScale(mat, plan, nullptr, a, nullptr));
  positive = a.positive[0] != 0;
  const size_t size = static_cast<size_t>(h.kd + 1) * h.n;
  h.band.resize(size);
  h.factor.resize(size);
  h.scale.resize(h.n);
  SL3D_CUDA(cudaMemcpy(h.band.data(), a.raw.p, size * sizeof(double), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(h.factor.data(), a.scaled.p, size * sizeof(double), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(h.scale.data(), a.scales.p, h.n * sizeof(double), cudaMemcpyDeviceToHost));
  if (h.sph) {
    Dev<double> lu;
    const long long luSize = static_cast<long long>(3 * h.kd + 1) * h.n;
    SL3D_CUDA(lu.Alloc(luSize));
    SL3D_TRY(LuBands(a, {0}, plan, {0}, lu.p, nullptr));
    luBand.resize(luSize);
    SL3D_CUDA(cudaMemcpy(luBand.data(), lu.p, luSize * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return SL3DGPU_OK;
}

}  // namespace

extern "C" int sl3dgpu_degree_create(const sl3dgpu_layer* layers, int nlayers, int ngll, int l, double eps,
                                     int toroidal, sl3dgpu_degree** out) {
  if (layers == nullptr || nlayers <= 0 || out == nullptr || ngll < 2 || l < 0 || (toroidal && l < 1) ||
      !(eps > 0.0)) {
    SetError("degree: layers, ngll >= 2, l >= 0 (>= 1 toroidal) and eps > 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto h = std::make_unique<sl3dgpu_degree>();
  try {
    std::vector<host::Layer> ls(nlayers);
    for (int i = 0; i < nlayers; ++i) {
      const auto& s = layers[i];
      ls[i] = host::Layer{s.r0, s.r1, s.fluid != 0, s.rho0, s.rho1, s.kappa0, s.kappa1, s.mu0, s.mu1,
                          s.viscosity, s.kelvin_fraction, s.kelvin_viscosity, s.elements};
    }
    h->earth = std::make_unique<host::LayeredBody>(ls, host::Scales::Geophysical(layers[nlayers - 1].r1));
    h->mesh = std::make_unique<host::RadialMesh>(host::RadialMesh::Create(*h->earth, ngll));
    h->material = std::make_unique<host::Material>(host::Material::Create(*h->earth, *h->mesh));
    if (toroidal) {
      h->tor = std::make_unique<host::ToroidalLayout>(*h->material, l, eps);
      h->n = h->tor->DofCount();
      h->kd = h->tor->Bandwidth();
      h->pinned = h->tor->Pinned();
    } else {
      h->sph = std::make_unique<host::SpheroidalLayout>(*h->material, l, eps);
      h->n = h->sph->DofCount();
      h->kd = h->sph->Bandwidth();
    }
  } catch (const std::exception& e) {
    SetError(std::string("degree: ") + e.what());
    return SL3DGPU_ERR_ARGUMENT;
  }
  bool positive = true;
  std::vector<double> luBand;
  SL3D_TRY(AssembleOne(*h, positive, luBand));
  if (h->tor && !positive) {
    SetError("degree: toroidal degree " + std::to_string(l) + ": a non-positive diagonal");
    return SL3DGPU_ERR_RUNTIME;
  }
  h->cholesky = positive;
  int info = 0;
  if (positive) {
    info = sl3dgpu_band_cholesky_factor(h->factor.data(), h->n, h->kd);
    if (info > 0) {
      // DegreeOperator::Factorise falls back to LU when Cholesky meets a
      // non-positive pivot
      if (h->tor) {
        SetError("degree: the toroidal system is not positive definite");
        return SL3DGPU_ERR_RUNTIME;
      }
      h->cholesky = false;
    }
  }
  if (!h->cholesky) {
    h->factor = luBand;
    h->pivots.assign(static_cast<size_t>(h->n), 0);
    info = sl3dgpu_band_lu_factor(h->factor.data(), h->n, h->kd, h->kd, h->pivots.data());
  }
  if (info < 0) return info;
  if (info > 0) {
    SetError("degree: the factorisation failed at row " + std::to_string(info));
    return SL3DGPU_ERR_RUNTIME;
  }
  *out = h.release();
  return SL3DGPU_OK;
}

extern "C" void sl3dgpu_degree_destroy(sl3dgpu_degree* h) { delete h; }

extern "C" int sl3dgpu_degree_dof_count(const sl3dgpu_degree* h) { return h ? h->n : SL3DGPU_ERR_ARGUMENT; }

extern "C" int sl3dgpu_degree_bandwidth(const sl3dgpu_degree* h) { return h ? h->kd : SL3DGPU_ERR_ARGUMENT; }

extern "C" int sl3dgpu_degree_used_cholesky(const sl3dgpu_degree* h) {
  return h ? (h->cholesky ? 1 : 0) : SL3DGPU_ERR_ARGUMENT;
}

extern "C" int sl3dgpu_degree_dof(const sl3dgpu_degree* h, int node, int component) {
  if (h == nullptr || node < 0 || node >= h->mesh->NodeCount() || component < 0 || component > 2) {
    SetError("degree: a node of the mesh and component 0 (U), 1 (V) or 2 (phi)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (h->tor) return h->tor->Dof(node);
  return h->sph->Dof(node, component);
}

extern "C" int sl3dgpu_degree_surface_dof(const sl3dgpu_degree* h, int component) {
  if (h == nullptr || component < 0 || component > 2) {
    SetError("degree: component 0 (U), 1 (V) or 2 (phi)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->tor ? h->tor->SurfaceDof() : h->sph->SurfaceDof(component);
}

extern "C" int sl3dgpu_degree_load(const sl3dgpu_degree* h, double* out) {
  if (h == nullptr || out == nullptr || !h->sph) {
    SetError("degree: the load vector is the spheroidal system's");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto v = h->sph->Load();
  std::copy(v.begin(), v.end(), out);
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_degree_tide(const sl3dgpu_degree* h, int power, double* out) {
  if (h == nullptr || out == nullptr || !h->sph) {
    SetError("degree: the tide vector is the spheroidal system's");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto v = h->sph->Tide(power);
  std::copy(v.begin(), v.end(), out);
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_degree_band(const sl3dgpu_degree* h, double* out) {
  if (h == nullptr || out == nullptr) {
    SetError("degree: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  std::copy(h->band.begin(), h->band.end(), out);
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_degree_apply(const sl3dgpu_degree* h, const double* x, int nrhs, double* y) {
  if (h == nullptr || x == nullptr || y == nullptr || nrhs < 0) {
    SetError("degree: null argument or negative nrhs");
    return SL3DGPU_ERR_ARGUMENT;
  }
  // the symmetric band's product, column by column
  const int n = h->n, kd = h->kd, ld = kd + 1;
  std::fill(y, y + static_cast<size_t>(n) * nrhs, 0.0);
  for (int c = 0; c < nrhs; ++c) {
    const double* xc = x + static_cast<size_t>(c) * n;
    double* yc = y + static_cast<size_t>(c) * n;
    for (int j = 0; j < n; ++j) {
      yc[j] += h->band[static_cast<size_t>(j) * ld + kd] * xc[j];
      for (int i = std::max(0, j - kd); i < j; ++i) {
        const double v = h->band[static_cast<size_t>(j) * ld + (kd + i - j)];
        yc[i] += v * xc[j];
        yc[j] += v * xc[i];
      }
    }
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_degree_solve(const sl3dgpu_degree* h, double* b, int nrhs) {
  if (h == nullptr || b == nullptr || nrhs < 0) {
    SetError("degree: null argument or negative nrhs");
    return SL3DGPU_ERR_ARGUMENT;
  }
  // K x = b as D (D K D)^-1 D b with the symmetric scaling D; pinned rows
  // (the toroidal rigid rotation) held at zero
  const int n = h->n;
  for (int c = 0; c < nrhs; ++c) {
    double* col = b + static_cast<size_t>(c) * n;
    for (int i = 0; i < n; ++i) col[i] *= h->scale[i];
    for (int p : h->pinned)
      if (p >= 0 && p < n) col[p] = 0.0;
  }
  const int st = h->cholesky ? sl3dgpu_band_cholesky_solve(h->factor.data(), n, h->kd, b, nrhs)
                             : sl3dgpu_band_lu_solve(h->factor.data(), n, h->kd, h->kd, h->pivots.data(), b, nrhs);
  if (st != SL3DGPU_OK) return st;
  for (int c = 0; c < nrhs; ++c) {
    double* col = b + static_cast<size_t>(c) * n;
    for (int i = 0; i < n; ++i) col[i] *= h->scale[i];
  }
  return SL3DGPU_OK;
}
