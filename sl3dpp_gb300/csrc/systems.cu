// The degree systems of an operator flavour, assembled on the host and
// factorised on the device (see systems.cuh).
#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "systems.cuh"

namespace sl3dgpu {

int BuildSystems(const SystemsInput& in, Flavour& f) {
  const int L = in.lmax;
  const auto& nodal = *in.nodal;
  const auto& degrees = *in.degrees;
  const long long rhsSphComplex = in.rhsSphComplex;
  const cudaStream_t stream = in.stream;
  std::vector<std::unique_ptr<host::DegreeOperator>> sph(L + 1);
  std::vector<std::unique_ptr<host::ToroidalOperator>> tor(L + 1);
  std::string failure;
  {
    const int threads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    std::mutex lock;
    for (int t = 0; t < threads; ++t)
      pool.emplace_back([&, t] {
        for (int l = L - t; l >= 0; l -= threads) {
          try {
            sph[l] = std::make_unique<host::DegreeOperator>(nodal, l, in.eps, in.shear);
            if (l >= 1) tor[l] = std::make_unique<host::ToroidalOperator>(nodal, l, in.eps, in.shear);
          } catch (const std::exception& e) {
            std::lock_guard<std::mutex> g(lock);
            failure = e.what();
          }
        }
      });
    for (auto& th : pool) th.join();
  }
  if (!failure.empty()) {
    SetError("v3d: " + failure);
    return SL3DGPU_ERR_RUNTIME;
  }
  // Bands, scales, systems: spheroidal degrees 0..L, toroidal 1..L.
  std::vector<double> bands, scales;
  std::vector<sl3dgpu_band_system> chol;  // all Cholesky candidates, sph then tor
  std::vector<int> cholDegree, cholKind;  // degree, 0 sph 1 tor
  std::vector<sl3dgpu_band_system> lu;
  std::vector<int> luDegree;
  std::vector<long long> sphScale(L + 1), torScale(L + 1);
  for (int l = 0; l <= L; ++l) {
    sphScale[l] = static_cast<long long>(scales.size());
    scales.insert(scales.end(), sph[l]->Scale().begin(), sph[l]->Scale().end());
  }
  for (int l = 1; l <= L; ++l) {
    torScale[l] = static_cast<long long>(scales.size());
    scales.insert(scales.end(), tor[l]->Scale().begin(), tor[l]->Scale().end());
  }
  auto system = [](int n, int kd, long long band, long long rhs, int nrhs, long long scale) {
    sl3dgpu_band_system s{};
    s.n = n;
    s.kl = kd;
    s.ku = kd;
    s.nrhs = nrhs;
    s.band = band;
    s.pivots = 0;
    s.rhs = rhs;
    s.scale = scale;
    s.pinned0 = s.pinned1 = -1;
    return s;
  };
  for (int l = 0; l <= L; ++l) {
    const auto& op = *sph[l];
    if (op.PositiveDiagonal()) {
      const auto b = op.ScaledCholeskyBand();
      chol.push_back(system(op.DofCount(), op.Bandwidth(), static_cast<long long>(bands.size()),
                            2 * degrees[l].sphRhs, 2 * (l + 1), sphScale[l]));
      bands.insert(bands.end(), b.begin(), b.end());
      cholDegree.push_back(l);
      cholKind.push_back(0);
    } else {
      luDegree.push_back(l);
    }
  }
  for (int l = 1; l <= L; ++l) {
    const auto& op = *tor[l];
    const auto b = op.ScaledCholeskyBand();
    auto s = system(op.DofCount(), op.Bandwidth(), static_cast<long long>(bands.size()), 2 * degrees[l].torRhs,
                    2 * (l + 1), torScale[l]);
    if (!op.Pinned().empty()) s.pinned0 = op.Pinned()[0];
    if (op.Pinned().size() > 1) s.pinned1 = op.Pinned()[1];
    if (op.Pinned().size() > 2) {
      SetError("v3d: more than two solid regions");
      return SL3DGPU_ERR_ARGUMENT;
    }
    chol.push_back(s);
    bands.insert(bands.end(), b.begin(), b.end());
    cholDegree.push_back(l);
    cholKind.push_back(1);
  }
  if (in.apply) {
    // K x for conjugate gradients: the assembled upper bands, spheroidal
    // degrees then toroidal, with their systems (right-hand sides in the
    // combined spheroidal-then-toroidal columns).
    std::vector<double> applyBands;
    std::vector<sl3dgpu_band_system> sphApply, torApply;
    int rows = 0;
    for (int l = 0; l <= L; ++l) {
      const auto& op = *sph[l];
      sphApply.push_back(system(op.DofCount(), op.Bandwidth(), static_cast<long long>(applyBands.size()),
                                2 * degrees[l].sphRhs, 2 * (l + 1), -1));
      applyBands.insert(applyBands.end(), op.Band().begin(), op.Band().end());
      rows = std::max(rows, op.DofCount());
    }
    for (int l = 1; l <= L; ++l) {
      const auto& op = *tor[l];
      torApply.push_back(system(op.DofCount(), op.Bandwidth(), static_cast<long long>(applyBands.size()),
                                2 * (rhsSphComplex + degrees[l].torRhs), 2 * (l + 1), -1));
      applyBands.insert(applyBands.end(), op.Band().begin(), op.Band().end());
      rows = std::max(rows, op.DofCount());
    }
    SL3D_CUDA(f.applyBands.Upload(applyBands));
    SL3D_CUDA(f.dSphApply.Upload(sphApply));
    SL3D_CUDA(f.dTorApply.Upload(torApply));
    f.nSphApply = static_cast<int>(sphApply.size());
    f.nTorApply = static_cast<int>(torApply.size());
    f.maxApplyRows = rows;
  }
  // Factor the Cholesky candidates; the spheroidal failures fall back to LU.
  Dev<double> dBands;
  SL3D_CUDA(dBands.Upload(bands));
  Dev<sl3dgpu_band_system> dChol;
  SL3D_CUDA(dChol.Upload(chol));
  Dev<int> info;
  SL3D_CUDA(info.Alloc(chol.size()));
  SL3D_TRY(BandFactorBatch(dChol.p, chol.data(), static_cast<int>(chol.size()), dBands.p, nullptr, info.p, 0, stream));
  std::vector<int> hInfo(chol.size());
  SL3D_CUDA(cudaMemcpyAsync(hInfo.data(), info.p, hInfo.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  std::vector<double> hostBands(bands.size());
  SL3D_CUDA(cudaMemcpy(hostBands.data(), dBands.p, bands.size() * sizeof(double), cudaMemcpyDeviceToHost));
  std::vector<double> finalBands;
  f.sphChol.clear();
  f.sphLu.clear();
  f.torChol.clear();
  for (size_t i = 0; i < chol.size(); ++i) {
    if (hInfo[i] != 0) {
      if (cholKind[i] == 1) {
        SetError("v3d: toroidal degree " + std::to_string(cholDegree[i]) + ": Cholesky failed");
        return SL3DGPU_ERR_RUNTIME;
      }
      luDegree.push_back(cholDegree[i]);
      continue;
    }
    auto s = chol[i];
    const size_t len = static_cast<size_t>(s.ku + 1) * s.n;
    const long long at = static_cast<long long>(finalBands.size());
    finalBands.insert(finalBands.end(), hostBands.begin() + s.band, hostBands.begin() + s.band + len);
    s.band = at;
    (cholKind[i] == 0 ? f.sphChol : f.torChol).push_back(s);
  }
  std::sort(luDegree.begin(), luDegree.end());
  std::vector<int> pivots;
  if (!luDegree.empty()) {
    std::vector<double> luBands;
    std::vector<sl3dgpu_band_system> luSys;
    for (int l : luDegree) {
      const auto& op = *sph[l];
      auto s = system(op.DofCount(), op.Bandwidth(), static_cast<long long>(luBands.size()), 2 * degrees[l].sphRhs,
                      2 * (l + 1), sphScale[l]);
      s.pivots = static_cast<long long>(pivots.size());
      pivots.resize(pivots.size() + op.DofCount());
      const auto b = op.ScaledLuBand();
      luBands.insert(luBands.end(), b.begin(), b.end());
      luSys.push_back(s);
    }
    Dev<double> dLu;
    SL3D_CUDA(dLu.Upload(luBands));
    Dev<sl3dgpu_band_system> dLuSys;
    SL3D_CUDA(dLuSys.Upload(luSys));
    Dev<int> dPiv, luInfo;
    SL3D_CUDA(dPiv.Alloc(pivots.size()));
    SL3D_CUDA(luInfo.Alloc(luSys.size()));
    SL3D_TRY(BandFactorBatch(dLuSys.p, luSys.data(), static_cast<int>(luSys.size()), dLu.p, dPiv.p, luInfo.p, 1, stream));
    // the copies below run on the legacy stream, which does not wait for
    // this non-blocking one: the factors and pivots must be complete first
    SL3D_CUDA(cudaStreamSynchronize(stream));
    std::vector<int> hLuInfo(luSys.size());
    SL3D_CUDA(cudaMemcpy(hLuInfo.data(), luInfo.p, hLuInfo.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < luSys.size(); ++i)
      if (hLuInfo[i] != 0) {
        SetError("v3d: degree " + std::to_string(luDegree[i]) + ": the banded LU factorisation failed (info = " +
                 std::to_string(hLuInfo[i]) + ")");
        return SL3DGPU_ERR_RUNTIME;
      }
    SL3D_CUDA(cudaMemcpy(luBands.data(), dLu.p, luBands.size() * sizeof(double), cudaMemcpyDeviceToHost));
    SL3D_CUDA(cudaMemcpy(pivots.data(), dPiv.p, pivots.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (auto s : luSys) {
      const size_t len = static_cast<size_t>(3 * s.ku + 1) * s.n;
      const long long at = static_cast<long long>(finalBands.size());
      finalBands.insert(finalBands.end(), luBands.begin() + s.band, luBands.begin() + s.band + len);
      s.band = at;
      f.sphLu.push_back(s);
    }
  }
  SL3D_CUDA(f.bands.Upload(finalBands));
  SL3D_CUDA(f.scales.Upload(scales));
  SL3D_CUDA(f.pivots.Upload(pivots.empty() ? std::vector<int>{0} : pivots));
  auto upload = [&](const std::vector<sl3dgpu_band_system>& sys, Dev<sl3dgpu_band_system>& d, Dev<int2>& items,
                    int& count) -> int {
    SL3D_CUDA(d.Upload(sys));
    const auto list = BandWorkItems(sys.data(), static_cast<int>(sys.size()));
    SL3D_CUDA(items.Upload(list));
    count = static_cast<int>(list.size());
    return SL3DGPU_OK;
  };
  SL3D_TRY(upload(f.sphChol, f.dSphChol, f.iSphChol, f.nSphChol));
  SL3D_TRY(upload(f.sphLu, f.dSphLu, f.iSphLu, f.nSphLu));
  SL3D_TRY(upload(f.torChol, f.dTorChol, f.iTorChol, f.nTorChol));
  // The load units K^-1 Load per degree (AddUnitChannels' cached responses).
  // The tide channel's, K^-1 Tide with the degree's power (degree 0 the
  // spherical mean of a centrifugal change, power 2: Viscoelastic3D.cpp:1049).
  std::vector<double> units, tides;
  std::vector<long long> unitOffset(L + 1);
  for (int l = 0; l <= L; ++l) {
    unitOffset[l] = static_cast<long long>(units.size());
    const auto load = sph[l]->Load();
    units.insert(units.end(), load.begin(), load.end());
    const auto tide = sph[l]->Tide(l == 0 ? 2 : -1);
    tides.insert(tides.end(), tide.begin(), tide.end());
  }
  SL3D_CUDA(f.units.Upload(units));
  SL3D_CUDA(f.tideUnits.Upload(tides));
  SL3D_CUDA(f.unitOffset.Upload(unitOffset));
  if (in.apply) {  // before the solve turns them into responses
    SL3D_CUDA(f.loadForces.Upload(units));
    SL3D_CUDA(f.tideForces.Upload(tides));
  }
  auto unitSystems = [&](const std::vector<sl3dgpu_band_system>& src) {
    std::vector<sl3dgpu_band_system> out;
    for (auto s : src) {
      // the system's degree from its right-hand-side offset
      int l = 0;
      while (l < L && 2 * degrees[l + 1].sphRhs <= s.rhs) ++l;
      s.rhs = unitOffset[l];
      s.nrhs = 1;
      out.push_back(s);
    }
    return out;
  };
  for (int lu = 0; lu < 2; ++lu) {
    const auto sys = unitSystems(lu ? f.sphLu : f.sphChol);
    if (sys.empty()) continue;
    Dev<sl3dgpu_band_system> d;
    Dev<int2> items;
    int count = 0;
    SL3D_TRY(upload(sys, d, items, count));
    SL3D_TRY(BandSolveBatch(d.p, sys.data(), static_cast<int>(sys.size()), items.p, count, f.bands.p, f.pivots.p,
                            f.units.p, f.scales.p, lu, stream));
    SL3D_TRY(BandSolveBatch(d.p, sys.data(), static_cast<int>(sys.size()), items.p, count, f.bands.p, f.pivots.p,
                            f.tideUnits.p, f.scales.p, lu, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
  }
  if (in.fp32) {
    // The FP64 factors and scales rounded to FP32 for the correction passes.
    SL3D_CUDA(f.bands32.Alloc(f.bands.n));
    SL3D_CUDA(f.scales32.Alloc(f.scales.n));
    LaunchCast(static_cast<long long>(f.bands.n), f.bands.p, f.bands32.p, stream);
    SL3D_CHECK_LAUNCH();
    LaunchCast(static_cast<long long>(f.scales.n), f.scales.p, f.scales32.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaStreamSynchronize(stream));
  }
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu
