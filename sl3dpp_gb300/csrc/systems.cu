// The degree systems of an operator flavour, assembled, scaled and
// factorised on the device (see systems.cuh).
#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "assemble.cuh"
#include "systems.cuh"

namespace sl3dgpu {

int BuildSystems(const SystemsInput& in, Flavour& f) {
  const int L = in.lmax;
  const auto& degrees = *in.degrees;
  const auto& plan = *in.plan;
  const long long rhsSphComplex = in.rhsSphComplex;
  const cudaStream_t stream = in.stream;
  // Every degree's raw band, its scales and scaled band, on the device.
  Dev<double> shear;
  if (in.shear != nullptr) SL3D_CUDA(shear.Upload(in.shear->modulus));
  AssembledSystems a;
  SL3D_TRY(AssembleAndScale(*in.material, plan, in.shear != nullptr ? shear.p : nullptr, a, stream));
  // plan order: spheroidal l at index l, toroidal l at L + l
  auto systemOf = [&](int index, long long rhs, int nrhs) {
    const AssemblySystem& p = plan.systems[index];
    sl3dgpu_band_system s{};
    s.n = p.ndof;
    s.kl = s.ku = p.kd;
    s.nrhs = nrhs;
    s.band = p.band;
    s.rhs = rhs;
    s.scale = a.scaleOffset[index];
    s.pinned0 = p.pinned0;
    s.pinned1 = p.pinned1;
    return s;
  };
  for (int l = 1; l <= L; ++l)
    if (!a.positive[L + l]) {
      SetError("v3d: toroidal degree " + std::to_string(l) + ": a non-positive diagonal");
      return SL3DGPU_ERR_RUNTIME;
    }
  if (in.apply) {
    // K x for conjugate gradients: the raw bands, right-hand sides in the
    // combined spheroidal-then-toroidal columns
    std::vector<sl3dgpu_band_system> sphApply, torApply;
    int rows = 0;
    for (int l = 0; l <= L; ++l) {
      auto s = systemOf(l, 2 * degrees[l].sphRhs, 2 * (l + 1));
      s.scale = -1;
      sphApply.push_back(s);
      rows = std::max(rows, s.n);
    }
    for (int l = 1; l <= L; ++l) {
      auto s = systemOf(L + l, 2 * (rhsSphComplex + degrees[l].torRhs), 2 * (l + 1));
      s.scale = -1;
      s.pinned0 = s.pinned1 = -1;
      torApply.push_back(s);
      rows = std::max(rows, s.n);
    }
    SL3D_CUDA(f.dSphApply.Upload(sphApply));
    SL3D_CUDA(f.dTorApply.Upload(torApply));
    f.nSphApply = static_cast<int>(sphApply.size());
    f.nTorApply = static_cast<int>(torApply.size());
    f.maxApplyRows = rows;
  }
  // Cholesky on every toroidal system and the spheroidal ones whose
  // diagonal is positive, in place on the scaled bands.
  std::vector<sl3dgpu_band_system> chol;
  std::vector<int> cholIndex, luDegree;
  for (int l = 0; l <= L; ++l) {
    if (!a.positive[l]) {
      luDegree.push_back(l);
      continue;
    }
    chol.push_back(systemOf(l, 2 * degrees[l].sphRhs, 2 * (l + 1)));
    cholIndex.push_back(l);
  }
  for (int l = 1; l <= L; ++l) {
    chol.push_back(systemOf(L + l, 2 * degrees[l].torRhs, 2 * (l + 1)));
    cholIndex.push_back(L + l);
  }
  Dev<sl3dgpu_band_system> dChol;
  SL3D_CUDA(dChol.Upload(chol));
  Dev<int> info;
  SL3D_CUDA(info.Alloc(chol.size()));
  SL3D_TRY(BandFactorBatch(dChol.p, chol.data(), static_cast<int>(chol.size()), a.scaled.p, nullptr, info.p, 0,
                           stream));
  std::vector<int> hInfo(chol.size());
  SL3D_CUDA(cudaMemcpyAsync(hInfo.data(), info.p, hInfo.size() * sizeof(int), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  f.sphChol.clear();
  f.sphLu.clear();
  f.torChol.clear();
  for (size_t i = 0; i < chol.size(); ++i) {
    const int index = cholIndex[i];
    if (hInfo[i] != 0) {
      if (index > L) {
        SetError("v3d: toroidal degree " + std::to_string(index - L) + ": Cholesky failed");
        return SL3DGPU_ERR_RUNTIME;
      }
      luDegree.push_back(index);  // DegreeOperator::Factorise's LU fallback
      continue;
    }
    (index <= L ? f.sphChol : f.torChol).push_back(chol[i]);
  }
  std::sort(luDegree.begin(), luDegree.end());
  std::vector<int> pivots{0};
  if (luDegree.empty()) {
    f.bands = std::move(a.scaled);
  } else {
    // LU storage of the fallback degrees after the scaled bands, built on
    // the device from the raw bands and scales, factorised in place
    std::vector<long long> offsets;
    std::vector<sl3dgpu_band_system> luSys;
    long long total = plan.bandDoubles, pivotCount = 0;
    for (int l : luDegree) {
      auto s = systemOf(l, 2 * degrees[l].sphRhs, 2 * (l + 1));
      s.band = total;
      s.pivots = pivotCount;
      offsets.push_back(total);
      total += static_cast<long long>(3 * s.ku + 1) * s.n;
      pivotCount += s.n;
      luSys.push_back(s);
    }
    SL3D_CUDA(f.bands.Alloc(total));
    SL3D_CUDA(cudaMemcpyAsync(f.bands.p, a.scaled.p, plan.bandDoubles * sizeof(double), cudaMemcpyDeviceToDevice,
                              stream));
    SL3D_TRY(LuBands(a, luDegree, plan, offsets, f.bands.p, stream));
    Dev<sl3dgpu_band_system> dLuSys;
    SL3D_CUDA(dLuSys.Upload(luSys));
    Dev<int> luInfo;
    SL3D_CUDA(f.pivots.Alloc(pivotCount));
    SL3D_CUDA(luInfo.Alloc(luSys.size()));
    SL3D_TRY(BandFactorBatch(dLuSys.p, luSys.data(), static_cast<int>(luSys.size()), f.bands.p, f.pivots.p, luInfo.p,
                             1, stream));
    std::vector<int> hLuInfo(luSys.size());
    SL3D_CUDA(cudaMemcpyAsync(hLuInfo.data(), luInfo.p, hLuInfo.size() * sizeof(int), cudaMemcpyDeviceToHost,
                              stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < luSys.size(); ++i)
      if (hLuInfo[i] != 0) {
        SetError("v3d: degree " + std::to_string(luDegree[i]) + ": the banded LU factorisation failed (info = " +
                 std::to_string(hLuInfo[i]) + ")");
        return SL3DGPU_ERR_RUNTIME;
      }
    f.sphLu = luSys;
    pivots.clear();
  }
  f.scales = std::move(a.scales);
  if (pivots.size() == 1) SL3D_CUDA(f.pivots.Upload(pivots));
  f.applyBands = std::move(a.raw);  // K x (conjugate gradients, the static problem) and inspection
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
    const auto load = (*in.sph)[l].Load();
    units.insert(units.end(), load.begin(), load.end());
    const auto tide = (*in.sph)[l].Tide(l == 0 ? 2 : -1);
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
