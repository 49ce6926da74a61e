// The degree systems through the C ABI: DegreeOperator and ToroidalOperator
// (include/sl3dpp/DegreeOperator.hpp:94-384, src/DegreeOperator.cpp:24-505,
// src/ToroidalOperator.cpp) of one degree on the unrelaxed material of a
// layered earth -- its dof map, load and tide vectors and product on the
// host, its solves on the GPU through the band drop-ins (the scaled band
// factorised once, Cholesky where every diagonal is positive, LU otherwise,
// as DegreeOperator::Factorise chooses).
#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "host/radial.hpp"

using namespace sl3dgpu;

struct sl3dgpu_degree {
  std::unique_ptr<host::LayeredEarth> earth;
  std::unique_ptr<host::RadialMesh> mesh;
  std::unique_ptr<host::Material> material;
  std::unique_ptr<host::DegreeOperator> sph;
  std::unique_ptr<host::ToroidalOperator> tor;
  std::vector<double> factor;  // the factorised scaled band
  std::vector<int> pivots;     // LU only
  std::vector<double> scale;
  std::vector<int> pinned;     // toroidal rows held at zero
  int n = 0, kd = 0;
  bool cholesky = true;
};

extern "C" int sl3dgpu_degree_create(const sl3dgpu_layer* layers, int nlayers, int ngll, int l, double eps,
                                     int toroidal, sl3dgpu_degree** out) {
  if (layers == nullptr || nlayers <= 0 || out == nullptr || ngll < 2 || l < 0 || (toroidal && l < 1) ||
      !(eps > 0.0)) {
    SetError("degree: layers, ngll >= 2, l >= 0 (>= 1 toroidal) and eps > 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  try {
    auto h = std::make_unique<sl3dgpu_degree>();
    std::vector<host::Layer> ls(nlayers);
    for (int i = 0; i < nlayers; ++i) {
      const auto& s = layers[i];
      ls[i] = host::Layer{s.r0, s.r1, s.fluid != 0, s.rho0, s.rho1, s.kappa0, s.kappa1, s.mu0, s.mu1,
                          s.viscosity, s.kelvin_fraction, s.kelvin_viscosity, s.elements};
    }
    h->earth = std::make_unique<host::LayeredEarth>(ls, host::Scales::Geophysical(layers[nlayers - 1].r1));
    h->mesh = std::make_unique<host::RadialMesh>(host::RadialMesh::Create(*h->earth, ngll));
    h->material = std::make_unique<host::Material>(host::Material::Create(*h->earth, *h->mesh));
    bool positive = true;
    if (toroidal) {
      h->tor = std::make_unique<host::ToroidalOperator>(*h->material, l, eps, nullptr);
      h->n = h->tor->DofCount();
      h->kd = h->tor->Bandwidth();
      h->scale = h->tor->Scale();
      h->pinned = h->tor->Pinned();
      h->factor = h->tor->ScaledCholeskyBand();
    } else {
      h->sph = std::make_unique<host::DegreeOperator>(*h->material, l, eps, nullptr);
      h->n = h->sph->DofCount();
      h->kd = h->sph->Bandwidth();
      h->scale = h->sph->Scale();
      positive = h->sph->PositiveDiagonal();
      h->factor = positive ? h->sph->ScaledCholeskyBand() : h->sph->ScaledLuBand();
    }
    h->cholesky = positive;
    int info = 0;
    if (positive) {
      info = sl3dgpu_band_cholesky_factor(h->factor.data(), h->n, h->kd);
      if (info > 0) {
        // DegreeOperator::Factorise falls back to LU when Cholesky meets a
        // non-positive pivot
        h->cholesky = false;
        h->factor = h->sph ? h->sph->ScaledLuBand() : std::vector<double>{};
        if (h->factor.empty()) {
          SetError("degree: the toroidal system is not positive definite");
          return SL3DGPU_ERR_RUNTIME;
        }
      }
    }
    if (!h->cholesky) {
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
  } catch (const std::exception& e) {
    SetError(std::string("degree: ") + e.what());
    return SL3DGPU_ERR_ARGUMENT;
  }
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

extern "C" int sl3dgpu_degree_apply(const sl3dgpu_degree* h, const double* x, int nrhs, double* y) {
  if (h == nullptr || x == nullptr || y == nullptr || nrhs < 0) {
    SetError("degree: null argument or negative nrhs");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const std::vector<double> in(x, x + static_cast<size_t>(h->n) * nrhs);
  const auto out = h->tor ? h->tor->Apply(in, nrhs) : h->sph->Apply(in, nrhs);
  std::copy(out.begin(), out.end(), y);
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
