// sl3d -- the front end of the 3D quasi-static run (the reference's
// `sl3d solve` for a run through time under a lateral viscosity,
// apps/SolveCommand.cpp:1747-1795, with its disk checkpoints, :239-290),
// over the library's C ABI on one GPU.
//
//   sl3d check CONFIG.json   the config read and checked, its run hash and
//                            shape printed (no GPU used)
//   sl3d solve CONFIG.json   the run: node 0 the instantaneous response,
//                            then a step per node; a checkpoint every
//                            `stride` nodes; the surface table at the end
//   sl3d kernel CONFIG.json  the kernels of the config's measurements (the
//                            reference's `sl3d kernel` under the discrete
//                            method, for a run without an ocean): per
//                            measurement one transposed sweep of the run
//
// The config (JSON; members other than these are refused):
//   model       {"earth": "standard", "elements": N, "kelvin_fraction": f,
//               "kelvin_div": d} -- the configurations' Earth
//               (sl3dgpu_standard_earth) -- or {"layers": [{"r0", "r1",
//               "fluid", "elements", "rho": [at r0, at r1], "kappa": [..],
//               "mu": [..], "viscosity", "kelvin_fraction",
//               "kelvin_viscosity"}, ...]} in SI
//   mesh        {"lmax", "ngll" (5), "eps" (1e-8), "oversampling" (1.5)}
//   lateral     {"viscosity": {"seed", "degree", "rms", "top_km" (100),
//               "bottom_km" (670)}} a seeded log-viscosity field, power
//               (l + 1)^-2 to the degree, scaled to the RMS, between the two
//               depths; or {"viscosity": {"coefficients": FILE, "top_km",
//               "bottom_km"}} its (l, m >= 0) complex coefficients as raw
//               little-endian doubles (re, im), (lmax + 1)(lmax + 2) / 2 of them
//   forcing     {"ice": {"cap_degrees", "thickness_m", "ramp_nodes"}} a polar
//               cap of ice (917 kg m^-3) growing linearly to its thickness
//               over the first ramp_nodes nodes, then held
//   ocean       (optional) {"land_fraction" (0.3), "seed" (11), "rotation":
//               "none" | "axial" | "full", "shorelines": "frozen" |
//               "migrating", "depth_m" (1500)} frozen shorelines over a land
//               mask thresholded from a seeded smooth field, each pass closed
//               by the sea-level equation (sl3dgpu_v3d_set_ocean); or
//               migrating ones (Evolution3D::RunMigrating): a background sea
//               level from the same field (ocean depth up to depth_m, land
//               where the field is above the threshold) with no ice, the cap
//               as an ice thickness history, each pass closed by the
//               nonlinear sea-level equation and flotation
//   time        {"step_yr", "nodes"} or {"times_yr": [...]} on the run's clock
//   solve       {"scheme": "sdirk2" | "exponential_trapezoid" |
//               "backward_euler", "step_solver": "fixed_point" |
//               "conjugate_gradients", "precision": "fp64" | "mixed", "rtol"
//               (1e-10), "max_iterations" (60), "anderson_memory" (5),
//               "warm_start" (false)}
//   checkpoint  (optional) {"directory", "stride"}
//   restart     (optional) true: continue from the newest whole checkpoint
//               of this run in the directory (another run's is refused)
//   stop_after_node (optional) the run stops after that node's checkpoint
//   output      {"file"}: the surface table, a row per node and (l, m >= 0):
//               node, time (yr), l, m, U (m, re im), phi (m^2 s^-2, re im)
//               and, with an ocean, the relative sea level change (m, re im)
////   kernels     (the kernel command) {"method": "discrete", "parameters":
//               ["load", "tide", "viscosity"], "measurements": [{"type":
//               "displacement_point" | "displacement_cap" | "potential_point"
//               | "potential_cap", "name", "latitude", "longitude",
//               "width_deg" (a cap's Gaussian width), "time" (a node's, on the
//               run's clock; the last node by default)}], "output": DIR,
//               "record_stride" (1)}; per measurement NAME_summary.txt (its
//               value in SI), NAME_load_kernels.txt (the load kernel's (l, m
//               >= 0) coefficients per node, per kg m^-2 per m^2 of the
//               run's sphere), NAME_tide_kernels.txt ("tide": per tidal
//               potential coefficient, m^2 s^-2) and NAME_viscosity_kernels.bin with
//               NAME_viscosity_grid.txt (dJ/d delta per m^3 on every memory
//               node's grid). Kernels under an ocean, the continuous method
//               and the other parameters are refused as not built.
//
// Checkpoints (the reference's scheme: a whole file written as
// `.node_NNNNNN.partial` and renamed to `node_NNNNNN.ckpt`, the newest two
// kept): a magic with the format's version, the run hash (FNV-1a of the
// canonical text of the members that decide the computation: model, mesh,
// lateral, forcing, ocean, time and solve -- not checkpoint, restart,
// stop_after_node or output), the node, the state's bytes
// (sl3dgpu_v3d_state_save) and the finished nodes' surface history. A
// restart from a checkpoint continues the run bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "json.hpp"
#include "sl3dgpu.h"

namespace {

using sl3d::json::Object;
using sl3d::json::Value;
using Complex = std::complex<double>;
namespace fs = std::filesystem;

constexpr double kPi = 3.14159265358979323846;
constexpr double kYear = 3.15576e7;
constexpr double kIceDensity = 917.0;
constexpr double kEarthRadius = 6371e3;
constexpr uint64_t kMagic = 0x53334447434b3031ull;  // "10KCGD3S": the format's version in the low bytes

// -- the config ---------------------------------------------------------------------------------

const Value* Find(const Object& o, const std::string& key) {
  auto it = o.find(key);
  return it == o.end() ? nullptr : &it->second;
}
double NumberOr(const Object& o, const std::string& key, double fallback) {
  const Value* v = Find(o, key);
  return v ? v->Number(key) : fallback;
}
void OnlyKeys(const Object& o, const std::vector<std::string>& allowed, const std::string& where) {
  for (const auto& [k, v] : o)
    if (std::find(allowed.begin(), allowed.end(), k) == allowed.end())
      throw std::invalid_argument(where + ": unknown member \"" + k + "\"");
}

struct Config {
  std::vector<sl3dgpu_layer> layers;
  sl3dgpu_v3d_options options{};
  // lateral viscosity
  bool seeded = true;
  uint64_t deltaSeed = 1;
  int deltaDegree = 0;
  double deltaRms = 0.0, topKm = 100.0, bottomKm = 670.0;
  std::string coefficientsFile;
  // forcing
  double capDegrees = 15.0, thicknessM = 2000.0;
  int rampNodes = 10;
  // ocean
  bool ocean = false, migrating = false;
  double landFraction = 0.3, depthM = 1500.0;
  uint64_t oceanSeed = 11;
  int rotation = 0;
  // time and scheme
  std::vector<double> timesYr;
  int scheme = 2;
  // steering
  std::string checkpointDir;
  int stride = 0;
  bool restart = false;
  long long stopAfter = -1;
  std::string output;
  uint64_t hash = 0;
  // kernels (the `kernel` command)
  struct Measurement {
    std::string name, type;  // displacement_point | displacement_cap | potential_point | potential_cap
    double latitude = 0.0, longitude = 0.0, widthDeg = 0.0;
    size_t node = 0;
  };
  bool kernels = false, loadKernels = false, tideKernels = false, viscosityKernels = false;
  std::vector<Measurement> measurements;
  std::string kernelDir;
  int recordStride = 1;
};

uint64_t Fnv1a(const std::string& text) {
  uint64_t h = 1469598103934665603ull;
  for (unsigned char c : text) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

Config ReadConfig(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw std::invalid_argument("cannot read " + path);
  std::stringstream text;
  text << in.rdbuf();
  const Value doc = sl3d::json::Parse(text.str());
  const Object& root = doc.Members("the config");
  OnlyKeys(root, {"model", "mesh", "lateral", "forcing", "ocean", "time", "solve", "checkpoint", "restart",
                  "stop_after_node", "output", "kernels"},
           "config");
  Config c;
  // the members that decide the computation, for the run hash
  std::string decided;
  for (const char* key : {"model", "mesh", "lateral", "forcing", "ocean", "time", "solve"})
    if (const Value* v = Find(root, key)) decided += std::string(key) + "=" + sl3d::json::Canonical(*v) + ";";
  c.hash = Fnv1a(decided);

  // model
  const Value* model = Find(root, "model");
  if (!model) throw std::invalid_argument("config: a model is required");
  const Object& m = model->Members("model");
  if (const Value* earth = Find(m, "earth")) {
    OnlyKeys(m, {"earth", "elements", "kelvin_fraction", "kelvin_div"}, "model");
    if (earth->String("model.earth") != "standard") throw std::invalid_argument("model.earth: \"standard\" only");
    c.layers.resize(4);
    const int n = sl3dgpu_standard_earth(static_cast<int>(NumberOr(m, "elements", 40)), NumberOr(m, "kelvin_fraction", 0.0),
                                         NumberOr(m, "kelvin_div", 10.0), c.layers.data());
    if (n < 0) throw std::invalid_argument(std::string("model: ") + sl3dgpu_last_error());
    c.layers.resize(n);
  } else {
    OnlyKeys(m, {"layers"}, "model");
    const Value* layers = Find(m, "layers");
    if (!layers) throw std::invalid_argument("model: \"earth\" or \"layers\" is required");
    for (const Value& lv : layers->Items("model.layers")) {
      const Object& L = lv.Members("a layer");
      OnlyKeys(L, {"r0", "r1", "fluid", "elements", "rho", "kappa", "mu", "viscosity", "kelvin_fraction",
                   "kelvin_viscosity"},
               "a layer");
      auto pair = [&](const char* key) {
        const Value* v = Find(L, key);
        if (!v) throw std::invalid_argument(std::string("a layer needs ") + key);
        const auto& a = v->Items(key);
        if (a.size() != 2) throw std::invalid_argument(std::string(key) + ": [at r0, at r1]");
        return std::pair{a[0].Number(key), a[1].Number(key)};
      };
      sl3dgpu_layer layer{};
      layer.r0 = NumberOr(L, "r0", -1.0);
      layer.r1 = NumberOr(L, "r1", -1.0);
      layer.fluid = Find(L, "fluid") && Find(L, "fluid")->Bool("fluid") ? 1 : 0;
      layer.elements = static_cast<int>(NumberOr(L, "elements", 1));
      std::tie(layer.rho0, layer.rho1) = pair("rho");
      std::tie(layer.kappa0, layer.kappa1) = pair("kappa");
      std::tie(layer.mu0, layer.mu1) = pair("mu");
      layer.viscosity = NumberOr(L, "viscosity", 0.0);
      layer.kelvin_fraction = NumberOr(L, "kelvin_fraction", 0.0);
      layer.kelvin_viscosity = NumberOr(L, "kelvin_viscosity", 0.0);
      c.layers.push_back(layer);
    }
    if (c.layers.empty()) throw std::invalid_argument("model.layers: at least one layer");
  }

  // mesh
  const Value* mesh = Find(root, "mesh");
  if (!mesh) throw std::invalid_argument("config: a mesh is required");
  const Object& me = mesh->Members("mesh");
  OnlyKeys(me, {"lmax", "ngll", "eps", "oversampling"}, "mesh");
  c.options.lmax = static_cast<int>(NumberOr(me, "lmax", -1));
  c.options.ngll = static_cast<int>(NumberOr(me, "ngll", 5));
  c.options.eps = NumberOr(me, "eps", 1e-8);
  c.options.oversampling = NumberOr(me, "oversampling", 1.5);
  if (c.options.lmax < 2) throw std::invalid_argument("mesh.lmax: at least 2");

  // solve
  c.options.max_iterations = 60;
  c.options.rtol = 1e-10;
  c.options.damping = 1.0;
  c.options.anderson_memory = 5;
  c.options.anderson_rate = 0.5;
  c.options.correction_rtol = 3e-6;
  c.options.correction_memory = 10;
  c.options.solve_rtol = 1e-11;
  c.options.solve_max_iterations = 200;
  if (const Value* solve = Find(root, "solve")) {
    const Object& s = solve->Members("solve");
    OnlyKeys(s, {"scheme", "step_solver", "precision", "rtol", "max_iterations", "anderson_memory", "warm_start"},
             "solve");
    if (const Value* v = Find(s, "scheme")) {
      const std::string& name = v->String("solve.scheme");
      c.scheme = name == "exponential_trapezoid" ? 0 : name == "backward_euler" ? 1 : name == "sdirk2" ? 2 : -1;
      if (c.scheme < 0) throw std::invalid_argument("solve.scheme: sdirk2, exponential_trapezoid or backward_euler");
    }
    if (const Value* v = Find(s, "step_solver")) {
      const std::string& name = v->String("solve.step_solver");
      if (name != "fixed_point" && name != "conjugate_gradients")
        throw std::invalid_argument("solve.step_solver: fixed_point or conjugate_gradients");
      c.options.solver = name == "conjugate_gradients" ? 1 : 0;
    }
    if (const Value* v = Find(s, "precision")) {
      const std::string& name = v->String("solve.precision");
      if (name != "fp64" && name != "mixed") throw std::invalid_argument("solve.precision: fp64 or mixed");
      c.options.precision = name == "mixed" ? 1 : 0;
      c.options.fp64_emulation = c.options.precision;
    }
    c.options.rtol = NumberOr(s, "rtol", c.options.rtol);
    c.options.max_iterations = static_cast<int>(NumberOr(s, "max_iterations", c.options.max_iterations));
    c.options.anderson_memory = static_cast<int>(NumberOr(s, "anderson_memory", c.options.anderson_memory));
    if (const Value* v = Find(s, "warm_start")) c.options.warm_start = v->Bool("solve.warm_start") ? 1 : 0;
  }

  // lateral viscosity
  if (const Value* lateral = Find(root, "lateral")) {
    const Object& la = lateral->Members("lateral");
    OnlyKeys(la, {"viscosity"}, "lateral");
    const Object& v = Find(la, "viscosity") ? Find(la, "viscosity")->Members("lateral.viscosity")
                                            : throw std::invalid_argument("lateral: a viscosity is required");
    OnlyKeys(v, {"seed", "degree", "rms", "coefficients", "top_km", "bottom_km"}, "lateral.viscosity");
    c.topKm = NumberOr(v, "top_km", 100.0);
    c.bottomKm = NumberOr(v, "bottom_km", 670.0);
    if (const Value* f = Find(v, "coefficients")) {
      c.seeded = false;
      c.coefficientsFile = f->String("lateral.viscosity.coefficients");
    } else {
      c.deltaSeed = static_cast<uint64_t>(NumberOr(v, "seed", 1));
      c.deltaDegree = static_cast<int>(NumberOr(v, "degree", 0));
      c.deltaRms = NumberOr(v, "rms", 0.0);
    }
  }

  // forcing
  if (const Value* forcing = Find(root, "forcing")) {
    const Object& f = forcing->Members("forcing");
    OnlyKeys(f, {"ice"}, "forcing");
    if (const Value* ice = Find(f, "ice")) {
      const Object& i = ice->Members("forcing.ice");
      OnlyKeys(i, {"cap_degrees", "thickness_m", "ramp_nodes"}, "forcing.ice");
      c.capDegrees = NumberOr(i, "cap_degrees", 15.0);
      c.thicknessM = NumberOr(i, "thickness_m", 2000.0);
      c.rampNodes = std::max(1, static_cast<int>(NumberOr(i, "ramp_nodes", 10)));
    }
  }

  // ocean
  if (const Value* ocean = Find(root, "ocean")) {
    const Object& o = ocean->Members("ocean");
    OnlyKeys(o, {"land_fraction", "seed", "rotation", "shorelines", "depth_m"}, "ocean");
    c.ocean = true;
    c.landFraction = NumberOr(o, "land_fraction", 0.3);
    c.depthM = NumberOr(o, "depth_m", 1500.0);
    if (const Value* sh = Find(o, "shorelines")) {
      const std::string& name = sh->String("ocean.shorelines");
      if (name != "frozen" && name != "migrating") throw std::invalid_argument("ocean.shorelines: frozen or migrating");
      c.migrating = name == "migrating";
    }
    if (!(c.depthM > 0.0)) throw std::invalid_argument("ocean.depth_m > 0");
    c.oceanSeed = static_cast<uint64_t>(NumberOr(o, "seed", 11));
    if (const Value* r = Find(o, "rotation")) {
      const std::string& name = r->String("ocean.rotation");
      c.rotation = name == "none" ? 0 : name == "axial" ? 1 : name == "full" ? 2 : -1;
      if (c.rotation < 0) throw std::invalid_argument("ocean.rotation: none, axial or full");
    }
    if (!(c.landFraction >= 0.0 && c.landFraction < 1.0)) throw std::invalid_argument("ocean.land_fraction: [0, 1)");
  }

  // time
  const Value* time = Find(root, "time");
  if (!time) throw std::invalid_argument("config: a time block is required");
  const Object& t = time->Members("time");
  OnlyKeys(t, {"step_yr", "nodes", "times_yr"}, "time");
  if (const Value* times = Find(t, "times_yr")) {
    for (const Value& v : times->Items("time.times_yr")) c.timesYr.push_back(v.Number("time.times_yr"));
  } else {
    const double step = NumberOr(t, "step_yr", -1.0);
    const int nodes = static_cast<int>(NumberOr(t, "nodes", 0));
    if (!(step > 0.0) || nodes < 1) throw std::invalid_argument("time: step_yr > 0 and nodes >= 1, or times_yr");
    for (int k = 0; k < nodes; ++k) c.timesYr.push_back(step * k);
  }
  if (c.timesYr.empty()) throw std::invalid_argument("time: at least one node");
  for (size_t k = 1; k < c.timesYr.size(); ++k)
    if (!(c.timesYr[k] > c.timesYr[k - 1])) throw std::invalid_argument("time: node times must increase");

  // steering
  if (const Value* ck = Find(root, "checkpoint")) {
    const Object& k = ck->Members("checkpoint");
    OnlyKeys(k, {"directory", "stride"}, "checkpoint");
    c.checkpointDir = Find(k, "directory") ? Find(k, "directory")->String("checkpoint.directory") : "";
    c.stride = static_cast<int>(NumberOr(k, "stride", 1));
    if (c.checkpointDir.empty() || c.stride < 1) throw std::invalid_argument("checkpoint: a directory and stride >= 1");
  }
  if (const Value* r = Find(root, "restart")) c.restart = r->Bool("restart");
  if (const Value* s = Find(root, "stop_after_node")) c.stopAfter = static_cast<long long>(s->Number("stop_after_node"));
  if (c.restart && c.checkpointDir.empty()) throw std::invalid_argument("restart: a checkpoint directory is required");
  const Value* out = Find(root, "output");
  if (!out) throw std::invalid_argument("config: an output is required");
  const Object& o = out->Members("output");
  OnlyKeys(o, {"file"}, "output");
  c.output = Find(o, "file") ? Find(o, "file")->String("output.file") : "";
  if (c.output.empty()) throw std::invalid_argument("output: a file is required");

  // kernels
  if (const Value* kv = Find(root, "kernels")) {
    const Object& k = kv->Members("kernels");
    OnlyKeys(k, {"method", "parameters", "measurements", "output", "record_stride"}, "kernels");
    c.kernels = true;
    if (c.ocean)
      throw std::invalid_argument("kernels: the kernels of a run under an ocean are not built (the sweep is the run "
                                  "without an ocean's)");
    if (const Value* m = Find(k, "method")) {
      const std::string& name = m->String("kernels.method");
      if (name == "continuous") throw std::invalid_argument("kernels.method: \"continuous\" is not built; \"discrete\"");
      if (name != "discrete") throw std::invalid_argument("kernels.method: \"discrete\"");
    }
    const Value* params = Find(k, "parameters");
    if (!params) throw std::invalid_argument("kernels.parameters is required: \"load\", \"tide\", \"viscosity\"");
    for (const Value& v : params->Items("kernels.parameters")) {
      const std::string& word = v.String("kernels.parameters");
      bool& flag = word == "load" ? c.loadKernels : word == "tide" ? c.tideKernels : c.viscosityKernels;
      if (word != "load" && word != "tide" && word != "viscosity") {
        if (word == "ice") throw std::invalid_argument("kernels.parameters: \"ice\" needs an ocean");
        throw std::invalid_argument("kernels.parameters: \"" + word +
                                    "\" is not built; \"load\", \"tide\", \"viscosity\"");
      }
      if (flag) throw std::invalid_argument("kernels.parameters: \"" + word + "\" named twice");
      flag = true;
    }
    if (!c.loadKernels && !c.tideKernels && !c.viscosityKernels)
      throw std::invalid_argument("kernels.parameters: at least one");
    const Value* dir = Find(k, "output");
    c.kernelDir = dir ? dir->String("kernels.output") : "";
    if (c.kernelDir.empty()) throw std::invalid_argument("kernels.output: a directory is required");
    c.recordStride = static_cast<int>(NumberOr(k, "record_stride", 1));
    if (c.recordStride < 1) throw std::invalid_argument("kernels.record_stride: at least 1");
    const Value* ms = Find(k, "measurements");
    if (!ms) throw std::invalid_argument("kernels.measurements is required");
    const double span = c.timesYr.back() - c.timesYr.front();
    for (const Value& mv : ms->Items("kernels.measurements")) {
      const Object& mo = mv.Members("a measurement");
      OnlyKeys(mo, {"type", "name", "latitude", "longitude", "width_deg", "time"}, "a measurement");
      Config::Measurement m;
      m.name = Find(mo, "name") ? Find(mo, "name")->String("measurement.name")
                                : "measurement_" + std::to_string(c.measurements.size());
      const bool plain = !m.name.empty() && m.name[0] != '.' &&
                         std::all_of(m.name.begin(), m.name.end(), [](char ch) {
                           return std::isalnum(static_cast<unsigned char>(ch)) || ch == '_' || ch == '-' || ch == '.';
                         });
      if (!plain) throw std::invalid_argument("measurement.name: letters, digits, _, - and ., not starting with .");
      for (const auto& other : c.measurements)
        if (other.name == m.name) throw std::invalid_argument("measurement.name: \"" + m.name + "\" named twice");
      m.type = Find(mo, "type") ? Find(mo, "type")->String("measurement.type") : "";
      const bool cap = m.type == "displacement_cap" || m.type == "potential_cap";
      const bool point = m.type == "displacement_point" || m.type == "potential_point";
      if (m.type.rfind("relative_sea_level", 0) == 0 || m.type == "decay_time")
        throw std::invalid_argument("measurement.type: \"" + m.type + "\" needs an ocean");
      if (!cap && !point)
        throw std::invalid_argument("measurement.type: displacement_point, displacement_cap, potential_point or "
                                    "potential_cap");
      if (!Find(mo, "latitude") || !Find(mo, "longitude"))
        throw std::invalid_argument("measurement " + m.name + ": latitude and longitude are required");
      m.latitude = Find(mo, "latitude")->Number("measurement.latitude");
      m.longitude = Find(mo, "longitude")->Number("measurement.longitude");
      if (!(m.latitude >= -90.0 && m.latitude <= 90.0))
        throw std::invalid_argument("measurement " + m.name + ": latitude in [-90, 90]");
      if (cap) {
        m.widthDeg = NumberOr(mo, "width_deg", -1.0);
        if (!(m.widthDeg > 0.0)) throw std::invalid_argument("measurement " + m.name + ": width_deg > 0");
      } else if (Find(mo, "width_deg")) {
        throw std::invalid_argument("measurement " + m.name + ": width_deg is a cap's");
      }
      m.node = c.timesYr.size() - 1;
      if (const Value* tv = Find(mo, "time")) {
        const double t = tv->Number("measurement.time");
        bool found = false;
        for (size_t n = 0; n < c.timesYr.size() && !found; ++n)
          if (std::abs(c.timesYr[n] - t) <= 1e-9 * std::max(span, 1.0)) {
            m.node = n;
            found = true;
          }
        if (!found) throw std::invalid_argument("measurement " + m.name + ": time is not a node of the run");
      }
      c.measurements.push_back(m);
    }
    if (c.measurements.empty()) throw std::invalid_argument("kernels.measurements: at least one");
  }
  return c;
}

// -- seeded fields (the front end's own generator: splitmix64 and Box-Muller) ---------------------

struct Rng {
  uint64_t state;
  explicit Rng(uint64_t seed) : state(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
  uint64_t Next() {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double Uniform() { return ((Next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double Normal() { return std::sqrt(-2.0 * std::log(Uniform())) * std::cos(2.0 * kPi * Uniform()); }
};

size_t Index(int l, int m) { return static_cast<size_t>(l) * (l + 1) / 2 + m; }

// power (l + 1)^-2 to the degree, scaled to the RMS over the sphere
std::vector<Complex> SeededField(int lmax, int degree, double rms, uint64_t seed, int lowest) {
  Rng rng(seed);
  std::vector<Complex> c(Index(lmax, lmax) + 1, Complex{});
  for (int l = lowest; l <= std::min(degree, lmax); ++l) {
    const double s = 1.0 / (l + 1);
    c[Index(l, 0)] = s * rng.Normal();
    for (int m = 1; m <= l; ++m) c[Index(l, m)] = Complex(rng.Normal(), rng.Normal()) * (s / std::sqrt(2.0));
  }
  if (rms <= 0.0) return c;
  double ms = 0.0;
  for (int l = 0; l <= lmax; ++l) {
    ms += std::norm(c[Index(l, 0)]);
    for (int m = 1; m <= l; ++m) ms += 2.0 * std::norm(c[Index(l, m)]);
  }
  ms /= 4.0 * kPi;
  if (ms > 0.0)
    for (auto& v : c) v *= rms / std::sqrt(ms);
  return c;
}

void Check(int status, const char* what) {
  if (status < 0) throw std::runtime_error(std::string(what) + ": " + sl3dgpu_last_error());
}
void CheckCuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
struct DeviceArray {
  T* p = nullptr;
  explicit DeviceArray(size_t n) { CheckCuda(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc"); }
  ~DeviceArray() { cudaFree(p); }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
};

// A grid's values of real spin-0 coefficients (host in, host out).
std::vector<double> Synthesise(sl3dgpu_grid* grid, const std::vector<Complex>& coeffs) {
  int nt = 0, np = 0;
  Check(sl3dgpu_grid_shape(grid, &nt, &np), "grid");
  DeviceArray<Complex> c(coeffs.size());
  DeviceArray<double> f(static_cast<size_t>(nt) * np);
  CheckCuda(cudaMemcpy(c.p, coeffs.data(), coeffs.size() * sizeof(Complex), cudaMemcpyHostToDevice), "copy");
  Check(sl3dgpu_synthesise_batch(grid, reinterpret_cast<const double*>(c.p), 1, f.p, nullptr), "synthesis");
  std::vector<double> out(static_cast<size_t>(nt) * np);
  CheckCuda(cudaMemcpy(out.data(), f.p, out.size() * sizeof(double), cudaMemcpyDeviceToHost), "copy");
  return out;
}
std::vector<Complex> Expand(sl3dgpu_grid* grid, const std::vector<double>& field, size_t coefficients) {
  DeviceArray<double> f(field.size());
  DeviceArray<Complex> c(coefficients);
  CheckCuda(cudaMemcpy(f.p, field.data(), field.size() * sizeof(double), cudaMemcpyHostToDevice), "copy");
  Check(sl3dgpu_expand_batch(grid, f.p, 1, reinterpret_cast<double*>(c.p), nullptr), "expansion");
  std::vector<Complex> out(coefficients);
  CheckCuda(cudaMemcpy(out.data(), c.p, coefficients * sizeof(Complex), cudaMemcpyDeviceToHost), "copy");
  return out;
}

// -- the run ----------------------------------------------------------------------------------------

struct NodeRecord {
  uint64_t node = 0;
  double tYr = 0.0;
  int iterations = 0, converged = 0;
  double residual = 0.0;
  std::vector<Complex> U, phi, seaLevel;
};

template <class T>
void Put(std::ofstream& out, const T& v) {
  out.write(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <class T>
void Get(std::ifstream& in, T& v) {
  in.read(reinterpret_cast<char*>(&v), sizeof(T));
  if (!in) throw std::runtime_error("a checkpoint ended early");
}
void PutVec(std::ofstream& out, const std::vector<Complex>& v) {
  Put(out, static_cast<uint64_t>(v.size()));
  out.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(Complex)));
}
void GetVec(std::ifstream& in, std::vector<Complex>& v) {
  uint64_t n = 0;
  Get(in, n);
  v.resize(n);
  in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(Complex)));
  if (!in) throw std::runtime_error("a checkpoint ended early");
}

std::vector<fs::path> Checkpoints(const fs::path& dir) {
  std::vector<fs::path> out;
  if (!fs::exists(dir)) return out;
  for (const auto& e : fs::directory_iterator(dir))
    if (e.path().extension() == ".ckpt" && e.path().filename().string().rfind("node_", 0) == 0) out.push_back(e.path());
  std::sort(out.begin(), out.end());
  return out;
}

void WriteCheckpoint(const Config& c, sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, uint64_t node,
                     const std::vector<NodeRecord>& history) {
  const fs::path dir(c.checkpointDir);
  fs::create_directories(dir);
  char name[64], partial[64];
  std::snprintf(name, sizeof(name), "node_%06llu.ckpt", static_cast<unsigned long long>(node));
  std::snprintf(partial, sizeof(partial), ".node_%06llu.partial", static_cast<unsigned long long>(node));
  const long long bytes = sl3dgpu_v3d_state_bytes(op, state);
  Check(static_cast<int>(std::min<long long>(bytes, 0)), "state size");
  std::vector<char> buffer(static_cast<size_t>(bytes));
  Check(sl3dgpu_v3d_state_save(op, state, buffer.data(), bytes), "state save");
  {
    std::ofstream out(dir / partial, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + (dir / partial).string());
    Put(out, kMagic);
    Put(out, c.hash);
    Put(out, node);
    Put(out, static_cast<uint64_t>(bytes));
    out.write(buffer.data(), bytes);
    Put(out, static_cast<uint64_t>(history.size()));
    for (const auto& h : history) {
      Put(out, h.node);
      Put(out, h.tYr);
      Put(out, h.iterations);
      Put(out, h.converged);
      Put(out, h.residual);
      PutVec(out, h.U);
      PutVec(out, h.phi);
      PutVec(out, h.seaLevel);
    }
    if (!out) throw std::runtime_error("cannot write " + (dir / partial).string());
  }
  fs::rename(dir / partial, dir / name);
  auto kept = Checkpoints(dir);
  while (kept.size() > 2) {
    fs::remove(kept.front());
    kept.erase(kept.begin());
  }
}

// The newest whole checkpoint of this run: the state restored, the history
// and the node returned; none: -1. Another run's checkpoint is refused.
long long ReadCheckpoint(const Config& c, sl3dgpu_v3d* op, sl3dgpu_v3d_state* state,
                         std::vector<NodeRecord>& history) {
  const auto found = Checkpoints(c.checkpointDir);
  if (found.empty()) return -1;
  std::ifstream in(found.back(), std::ios::binary);
  uint64_t magic = 0, hash = 0, node = 0, bytes = 0, count = 0;
  Get(in, magic);
  if (magic != kMagic) throw std::runtime_error(found.back().string() + " is not a checkpoint of this format");
  Get(in, hash);
  if (hash != c.hash)
    throw std::runtime_error(found.back().string() + " belongs to another run (its config or inputs differ)");
  Get(in, node);
  Get(in, bytes);
  std::vector<char> buffer(bytes);
  in.read(buffer.data(), static_cast<std::streamsize>(bytes));
  if (!in) throw std::runtime_error("a checkpoint ended early");
  Check(sl3dgpu_v3d_state_load(op, state, buffer.data(), static_cast<long long>(bytes)), "state load");
  Get(in, count);
  history.assign(count, NodeRecord{});
  for (auto& h : history) {
    Get(in, h.node);
    Get(in, h.tYr);
    Get(in, h.iterations);
    Get(in, h.converged);
    Get(in, h.residual);
    GetVec(in, h.U);
    GetVec(in, h.phi);
    GetVec(in, h.seaLevel);
  }
  return static_cast<long long>(node);
}

// The lateral viscosity on every node's grid: the seeded (or read) pattern
// between the two depths.
void SetLateral(const Config& c, sl3dgpu_v3d* op) {
  const int lmax = c.options.lmax;
  const size_t lm = Index(lmax, lmax) + 1;
  int P = 0, nt = 0, np = 0;
  Check(sl3dgpu_v3d_shape(op, &P, &nt, &np), "shape");
  std::vector<double> radius(P);
  Check(sl3dgpu_v3d_nodes(op, radius.data(), nullptr), "nodes");
  double length = 1.0, time = 1.0, sigma = 1.0;
  Check(sl3dgpu_v3d_scales(op, &length, &time, &sigma), "scales");
  if (c.deltaRms > 0.0 || !c.coefficientsFile.empty()) {
    std::vector<Complex> coeffs;
    if (c.seeded) {
      coeffs = SeededField(lmax, c.deltaDegree, c.deltaRms, c.deltaSeed, 1);
    } else {
      std::ifstream in(c.coefficientsFile, std::ios::binary);
      coeffs.resize(lm);
      in.read(reinterpret_cast<char*>(coeffs.data()), static_cast<std::streamsize>(lm * sizeof(Complex)));
      if (!in) throw std::runtime_error(c.coefficientsFile + ": not " + std::to_string(lm) + " complex coefficients");
    }
    sl3dgpu_grid* grid = nullptr;
    Check(sl3dgpu_grid_create(lmax, 0, c.options.oversampling, &grid), "grid");
    const auto pattern = Synthesise(grid, coeffs);
    sl3dgpu_grid_destroy(grid);
    if (pattern.size() != static_cast<size_t>(nt) * np) throw std::runtime_error("the delta grid's shape");
    std::vector<double> samples(static_cast<size_t>(P) * nt * np, 0.0);
    for (int p = 0; p < P; ++p) {
      const double r = radius[p] * length;
      if (!(r > kEarthRadius - c.bottomKm * 1e3 && r < kEarthRadius - c.topKm * 1e3)) continue;
      std::copy(pattern.begin(), pattern.end(), samples.begin() + static_cast<size_t>(p) * nt * np);
    }
    Check(sl3dgpu_v3d_set_delta(op, samples.data(), 0), "delta");
  }
}

int Solve(const Config& c) {
  const int lmax = c.options.lmax;
  const size_t lm = Index(lmax, lmax) + 1;
  sl3dgpu_v3d* op = nullptr;
  Check(sl3dgpu_v3d_create(c.layers.data(), static_cast<int>(c.layers.size()), &c.options, &op), "operator");
  struct Guard {
    sl3dgpu_v3d* op;
    sl3dgpu_v3d_state* state = nullptr;
    ~Guard() {
      if (state) sl3dgpu_v3d_free_state(state);
      sl3dgpu_v3d_destroy(op);
    }
  } guard{op};
  double length = 1.0, time = 1.0, sigma = 1.0;
  Check(sl3dgpu_v3d_scales(op, &length, &time, &sigma), "scales");
  SetLateral(c, op);

  // the ice cap, on the sea-level grid (the ocean closure's) or as coefficients
  std::vector<double> seaLevel, backgroundIce, oceanWeights;
  int oceanNphi = 0;
  sl3dgpu_grid* exact = nullptr;
  Check(sl3dgpu_grid_create(lmax, 0, 1.0, &exact), "grid");
  int et = 0, ep = 0;
  Check(sl3dgpu_grid_shape(exact, &et, &ep), "grid");
  std::vector<double> theta(et), weights(et);
  Check(sl3dgpu_grid_colatitudes(exact, theta.data(), weights.data()), "grid");
  std::vector<double> cap(static_cast<size_t>(et) * ep, 0.0);
  for (int j = 0; j < et; ++j)
    if (theta[j] < c.capDegrees * kPi / 180.0)
      for (int k = 0; k < ep; ++k) cap[static_cast<size_t>(j) * ep + k] = kIceDensity * c.thicknessM / sigma;
  const std::vector<Complex> capCoeffs = Expand(exact, cap, lm);
  if (c.ocean) {
    // land where a seeded smooth field is highest, over the land fraction of the area
    const auto field = Synthesise(exact, SeededField(lmax, 12, 0.0, c.oceanSeed, 1));
    std::vector<size_t> order(field.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return field[a] > field[b]; });
    double total = 0.0;
    for (int j = 0; j < et; ++j) total += weights[j] * ep;
    std::vector<double> oceanFunction(field.size(), 1.0);
    double covered = 0.0;
    size_t landCount = 0;
    for (size_t i : order) {
      covered += weights[i / ep];
      if (covered / total > c.landFraction) break;
      oceanFunction[i] = 0.0;
      ++landCount;
    }
    sl3dgpu_v3d_ocean o{oceanFunction.data(), c.rotation, 1000.0, 7.27220521664304e-05, 8.0359e37, 8.0096e37,
                        c.options.rtol, 200, c.options.anderson_memory};
    if (c.migrating) {
      // the background: ocean depth below the threshold value, land height
      // above it, up to depth_m; no ice (the history's first node)
      const double threshold = landCount < order.size() ? field[order[landCount]] : field[order.back()];
      double span = 0.0;
      for (double v : field) span = std::max(span, std::abs(threshold - v));
      seaLevel.resize(field.size());
      for (size_t i = 0; i < field.size(); ++i)
        seaLevel[i] = c.depthM * (threshold - field[i]) / std::max(span, 1e-300) / length;
      backgroundIce.assign(field.size(), 0.0);
      o.ocean_function = nullptr;
      o.migrating = 1;
      o.ice_density = kIceDensity;
      o.ice_thickness = backgroundIce.data();
      o.sea_level = seaLevel.data();
      o.max_nonlinear_iterations = 200;
      oceanWeights = weights;
      oceanNphi = ep;
    }
    Check(sl3dgpu_v3d_set_ocean(op, &o), "ocean");
  }
  sl3dgpu_grid_destroy(exact);
  auto ramp = [&](size_t node) { return std::min<double>(static_cast<double>(node), c.rampNodes) / c.rampNodes; };

  sl3dgpu_v3d_state* state = nullptr;
  Check(sl3dgpu_v3d_zero_state(op, &state), "state");
  guard.state = state;
  std::vector<NodeRecord> history;
  long long first = 0;
  if (c.restart) {
    const long long done = ReadCheckpoint(c, op, state, history);
    if (done >= 0) {
      first = done + 1;
      std::printf("sl3d: resumed after node %lld\n", done);
    }
  }
  const size_t nodes = c.timesYr.size();
  std::vector<double> load0, load1;
  std::vector<Complex> sigma0, sigma1;
  for (size_t node = static_cast<size_t>(first); node < nodes; ++node) {
    const size_t before = node > 0 ? node - 1 : 0;
    const double dt = node > 0 ? (c.timesYr[node] - c.timesYr[node - 1]) * kYear / time : 0.0;
    sl3dgpu_step_info info{};
    NodeRecord rec;
    if (c.migrating && node == 0) {
      // undisturbed at the background (the history's first ice is none)
      info.converged = 1;
      rec.seaLevel.assign(lm, Complex{});
    } else if (c.migrating) {
      // the cap's thickness at the step's two ends (model length)
      load0.assign(cap.size(), 0.0);
      load1.assign(cap.size(), 0.0);
      const double toThickness = sigma / (kIceDensity * length);
      for (size_t i = 0; i < cap.size(); ++i) {
        load0[i] = ramp(before) * cap[i] * toThickness;
        load1[i] = ramp(node) * cap[i] * toThickness;
      }
      Check(sl3dgpu_v3d_step_migrating(op, state, dt, c.scheme, load0.data(), load1.data(), nullptr, nullptr, &info),
            "step");
      rec.seaLevel.resize(lm);
      Check(sl3dgpu_v3d_sea_level(op, reinterpret_cast<double*>(rec.seaLevel.data()), nullptr, nullptr),
            "sea level");
      for (auto& v : rec.seaLevel) v *= length;
      // the ocean's share of the area under the node's shorelines
      std::vector<double> function(cap.size());
      Check(sl3dgpu_v3d_ocean_function(op, function.data()), "ocean function");
      double wet = 0.0, all = 0.0;
      for (size_t i = 0; i < function.size(); ++i) {
        wet += oceanWeights[i / oceanNphi] * function[i];
        all += oceanWeights[i / oceanNphi];
      }
      std::printf("sl3d: node %zu ocean fraction %.9f\n", node, wet / all);
    } else if (c.ocean) {
      load0.assign(cap.size(), 0.0);
      load1.assign(cap.size(), 0.0);
      for (size_t i = 0; i < cap.size(); ++i) {
        load0[i] = ramp(before) * cap[i];
        load1[i] = ramp(node) * cap[i];
      }
      Check(sl3dgpu_v3d_step_ocean(op, state, dt, c.scheme, load0.data(), load1.data(), &info), "step");
      rec.seaLevel.resize(lm);
      Check(sl3dgpu_v3d_sea_level(op, reinterpret_cast<double*>(rec.seaLevel.data()), nullptr, nullptr),
            "sea level");
      for (auto& v : rec.seaLevel) v *= length;
    } else {
      sigma0.assign(lm, Complex{});
      sigma1.assign(lm, Complex{});
      for (size_t i = 0; i < lm; ++i) {
        sigma0[i] = ramp(before) * capCoeffs[i];
        sigma1[i] = ramp(node) * capCoeffs[i];
      }
      Check(sl3dgpu_v3d_step(op, state, dt, c.scheme, reinterpret_cast<const double*>(sigma0.data()),
                             reinterpret_cast<const double*>(sigma1.data()), &info),
            "step");
    }
    rec.node = node;
    rec.tYr = c.timesYr[node];
    rec.iterations = info.iterations;
    rec.converged = info.converged;
    rec.residual = info.residual;
    rec.U.assign(lm, Complex{});
    rec.phi.assign(lm, Complex{});
    if (!(c.migrating && node == 0)) {
      Check(sl3dgpu_v3d_surface(op, 0, reinterpret_cast<double*>(rec.U.data())), "surface");
      Check(sl3dgpu_v3d_surface(op, 2, reinterpret_cast<double*>(rec.phi.data())), "surface");
    }
    const double potential = length * length / (time * time);
    for (auto& v : rec.U) v *= length;
    for (auto& v : rec.phi) v *= potential;
    std::printf("sl3d: node %zu t %.6g yr: %d passes%s\n", node, rec.tYr, info.iterations,
                info.converged ? "" : " (not converged)");
    history.push_back(std::move(rec));
    const bool last = node + 1 == nodes;
    if (c.stride > 0 && (node % static_cast<size_t>(c.stride) == 0 || last))
      WriteCheckpoint(c, op, state, node, history);
    if (c.stopAfter >= 0 && static_cast<long long>(node) >= c.stopAfter && !last) {
      std::printf("sl3d: stopped after node %zu (restart continues the run)\n", node);
      return 0;
    }
  }

  std::ofstream out(c.output);
  if (!out) throw std::runtime_error("cannot write " + c.output);
  out << "# sl3d surface table: node t_yr l m U_re U_im phi_re phi_im" << (c.ocean ? " sea_level_re sea_level_im" : "")
      << " (SI: m, m^2 s^-2)\n";
  char row[512];
  for (const auto& h : history)
    for (int l = 0; l <= lmax; ++l)
      for (int m = 0; m <= l; ++m) {
        const size_t i = Index(l, m);
        int n = std::snprintf(row, sizeof(row), "%llu %.17g %d %d %.17g %.17g %.17g %.17g",
                              static_cast<unsigned long long>(h.node), h.tYr, l, m, h.U[i].real(), h.U[i].imag(),
                              h.phi[i].real(), h.phi[i].imag());
        if (c.ocean)
          n += std::snprintf(row + n, sizeof(row) - n, " %.17g %.17g", h.seaLevel[i].real(), h.seaLevel[i].imag());
        out << row << '\n';
      }
  std::printf("sl3d: wrote %s (%zu nodes)\n", c.output.c_str(), history.size());
  return 0;
}


// -- kernel: the discrete adjoint of the run -----------------------------------------------------------

// Orthonormal spherical harmonics Y_lm(theta, phi), m >= 0, with the
// Condon-Shortley phase (the library's basis), by the standard recurrences
// of the normalised associated Legendre functions; (l, m) at l(l+1)/2 + m.
std::vector<Complex> Harmonics(int lmax, double theta, double phi) {
  const double x = std::cos(theta), s = std::sin(theta);
  std::vector<double> P(Index(lmax, lmax) + 1, 0.0);
  P[0] = std::sqrt(1.0 / (4.0 * kPi));
  for (int m = 1; m <= lmax; ++m) P[Index(m, m)] = -std::sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * P[Index(m - 1, m - 1)];
  for (int m = 0; m < lmax; ++m) P[Index(m + 1, m)] = std::sqrt(2.0 * m + 3.0) * x * P[Index(m, m)];
  for (int m = 0; m <= lmax; ++m)
    for (int l = m + 2; l <= lmax; ++l) {
      const double a = std::sqrt((4.0 * l * l - 1.0) / (static_cast<double>(l) * l - static_cast<double>(m) * m));
      const double b = std::sqrt(((l - 1.0) * (l - 1.0) - static_cast<double>(m) * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
      P[Index(l, m)] = a * (x * P[Index(l - 1, m)] - b * P[Index(l - 2, m)]);
    }
  std::vector<Complex> Y(P.size());
  for (int l = 0; l <= lmax; ++l)
    for (int m = 0; m <= l; ++m) Y[Index(l, m)] = P[Index(l, m)] * std::polar(1.0, m * phi);
  return Y;
}

// A Gaussian cap's degree weights: b_l = 2 pi int cap(d) P_l(cos d) sin d dd
// for the cap exp(-d^2 / (2 w^2)) normalised to a unit integral over the
// sphere (composite Simpson in d).
std::vector<double> CapWeights(int lmax, double widthDeg) {
  const double w = widthDeg * kPi / 180.0;
  const int n = 20000;
  const double h = kPi / n;
  std::vector<double> b(lmax + 1, 0.0);
  double area = 0.0;
  std::vector<double> Pl(lmax + 1);
  for (int i = 0; i <= n; ++i) {
    const double d = i * h, x = std::cos(d);
    const double weight = (i == 0 || i == n) ? 1.0 : (i % 2 ? 4.0 : 2.0);
    const double f = std::exp(-d * d / (2.0 * w * w)) * std::sin(d) * weight;
    Pl[0] = 1.0;
    if (lmax > 0) Pl[1] = x;
    for (int l = 2; l <= lmax; ++l) Pl[l] = ((2.0 * l - 1.0) * x * Pl[l - 1] - (l - 1.0) * Pl[l - 2]) / l;
    area += f;
    for (int l = 0; l <= lmax; ++l) b[l] += f * Pl[l];
  }
  for (double& v : b) v /= area;  // 2 pi and h / 3 cancel in the normalisation
  return b;
}

// `sl3d kernel CONFIG`: the run of `solve` (without an ocean) and, for each
// measurement, one transposed sweep (sl3dgpu_v3d_adjoint_run) giving the
// load kernels and the log-viscosity kernel, written in SI.
int Kernel(const Config& c) {
  const int lmax = c.options.lmax;
  const size_t lm = Index(lmax, lmax) + 1;
  sl3dgpu_v3d* op = nullptr;
  Check(sl3dgpu_v3d_create(c.layers.data(), static_cast<int>(c.layers.size()), &c.options, &op), "operator");
  struct Guard {
    sl3dgpu_v3d* op;
    ~Guard() { sl3dgpu_v3d_destroy(op); }
  } guard{op};
  int P = 0, nt = 0, np = 0;
  Check(sl3dgpu_v3d_shape(op, &P, &nt, &np), "shape");
  std::vector<double> radius(P), theta(nt), thetaWeights(nt);
  Check(sl3dgpu_v3d_nodes(op, radius.data(), nullptr), "nodes");
  Check(sl3dgpu_v3d_colatitudes(op, theta.data(), thetaWeights.data()), "colatitudes");
  double length = 1.0, time = 1.0, sigma = 1.0;
  Check(sl3dgpu_v3d_scales(op, &length, &time, &sigma), "scales");
  SetLateral(c, op);
  double surface = 0.0;  // the run's sphere (m)
  for (const auto& layer : c.layers) surface = std::max(surface, layer.r1);

  // the node loads: the cap's coefficients ramped
  sl3dgpu_grid* exact = nullptr;
  Check(sl3dgpu_grid_create(lmax, 0, 1.0, &exact), "grid");
  int et = 0, ep = 0;
  Check(sl3dgpu_grid_shape(exact, &et, &ep), "grid");
  std::vector<double> capTheta(et), capWeights(et);
  Check(sl3dgpu_grid_colatitudes(exact, capTheta.data(), capWeights.data()), "grid");
  std::vector<double> cap(static_cast<size_t>(et) * ep, 0.0);
  for (int j = 0; j < et; ++j)
    if (capTheta[j] < c.capDegrees * kPi / 180.0)
      for (int k = 0; k < ep; ++k) cap[static_cast<size_t>(j) * ep + k] = kIceDensity * c.thicknessM / sigma;
  const std::vector<Complex> capCoeffs = Expand(exact, cap, lm);
  sl3dgpu_grid_destroy(exact);
  const size_t nodes = c.timesYr.size();
  std::vector<Complex> loads(lm * nodes);
  std::vector<double> times(nodes);
  for (size_t n = 0; n < nodes; ++n) {
    const double ramp = std::min<double>(static_cast<double>(n), c.rampNodes) / c.rampNodes;
    for (size_t i = 0; i < lm; ++i) loads[lm * n + i] = ramp * capCoeffs[i];
    times[n] = c.timesYr[n] * kYear / time;
  }
  const size_t values = static_cast<size_t>(P) * nt * np;
  std::vector<double> volume(values);
  Check(sl3dgpu_v3d_sample_volumes(op, volume.data()), "volumes");
  fs::create_directories(c.kernelDir);

  for (const auto& m : c.measurements) {
    const bool displacement = m.type.rfind("displacement", 0) == 0;
    const bool isCap = m.type.size() > 4 && m.type.substr(m.type.size() - 4) == "_cap";
    const double scale = displacement ? length : length * length / (time * time);  // SI per model unit of J
    const char* unit = displacement ? "m" : "m^2 s^-2";
    // J = sum_{m >= 0} w_m Re(g* X) at the node: g = b_l conj(Y_lm(x0)), b_l = 1 at a point
    const auto Y = Harmonics(lmax, (90.0 - m.latitude) * kPi / 180.0, m.longitude * kPi / 180.0);
    const std::vector<double> b = isCap ? CapWeights(lmax, m.widthDeg) : std::vector<double>(lmax + 1, 1.0);
    std::vector<Complex> dual(lm * nodes);
    for (int l = 0; l <= lmax; ++l)
      for (int k = 0; k <= l; ++k) dual[lm * m.node + Index(l, k)] = b[l] * std::conj(Y[Index(l, k)]);
    std::vector<Complex> kernels(lm * nodes), tides(c.tideKernels ? lm * nodes : 0);
    std::vector<double> gradient(c.viscosityKernels ? values : 0);
    double objective = 0.0;
    Check(sl3dgpu_v3d_adjoint_run(op, times.data(), static_cast<int>(nodes), c.scheme, c.recordStride,
                                  reinterpret_cast<const double*>(loads.data()),
                                  displacement ? reinterpret_cast<const double*>(dual.data()) : nullptr,
                                  displacement ? nullptr : reinterpret_cast<const double*>(dual.data()),
                                  reinterpret_cast<double*>(kernels.data()),
                                  c.tideKernels ? reinterpret_cast<double*>(tides.data()) : nullptr,
                                  c.viscosityKernels ? gradient.data() : nullptr, &objective, nullptr),
          "adjoint");
    const double value = scale * objective;
    const fs::path dir(c.kernelDir);
    {
      std::ofstream out(dir / (m.name + "_summary.txt"));
      char line[512];
      std::snprintf(line, sizeof(line),
                    "measurement %s\ntype %s\nlatitude %.17g\nlongitude %.17g\nwidth_deg %.17g\nnode %zu\nt_yr "
                    "%.17g\nvalue %.17g %s\nmethod discrete\nrun_hash %016llx\n",
                    m.name.c_str(), m.type.c_str(), m.latitude, m.longitude, m.widthDeg, m.node, c.timesYr[m.node],
                    value, unit, static_cast<unsigned long long>(c.hash));
      out << line;
      if (!out) throw std::runtime_error("cannot write the summary of " + m.name);
    }
    if (c.loadKernels) {
      // K_n(x) = sum_{m >= 0} w_m Re(K_lm Y_lm(x)) per kg m^-2 per m^2 of the run's sphere
      const double toSi = scale / (sigma * surface * surface);
      std::ofstream out(dir / (m.name + "_load_kernels.txt"));
      out << "# sl3d load kernels of " << m.name << " (" << m.type << ", " << unit
          << "): node t_yr l m K_re K_im, the coefficients of K_n(x) = sum_{m >= 0} w_m Re(K_lm Y_lm(x)) "
             "(w_m = 1 at m = 0, 2 above; Y orthonormal, Condon-Shortley phase), dJ = sum_n int K_n dsigma_n dS "
             "over the sphere of radius "
          << surface << " m, per kg m^-2 per m^2\n";
      char row[256];
      for (size_t n = 0; n < nodes; ++n)
        for (int l = 0; l <= lmax; ++l)
          for (int k = 0; k <= l; ++k) {
            const Complex v = toSi * kernels[lm * n + Index(l, k)];
            std::snprintf(row, sizeof(row), "%zu %.17g %d %d %.17g %.17g\n", n, c.timesYr[n], l, k, v.real(),
                          v.imag());
            out << row;
          }
      if (!out) throw std::runtime_error("cannot write the load kernels of " + m.name);
    }
    if (c.tideKernels) {
      // per (l, m >= 0) coefficient of a tidal potential (m^2 s^-2), the
      // coefficient pairing of real fields (m > 0 twice); degree 1 none
      const double toSi = scale * time * time / (length * length);
      std::ofstream out(dir / (m.name + "_tide_kernels.txt"));
      out << "# sl3d tide kernels of " << m.name << " (" << m.type << ", " << unit
          << "): node t_yr l m K_re K_im, dJ = sum_n sum_{l, m >= 0} w_m Re(K_lm* dpsi_lm) for a tidal potential's "
             "coefficients dpsi (m^2 s^-2; w_m = 1 at m = 0, 2 above; no degree-1 tide)\n";
      char row[256];
      for (size_t n = 0; n < nodes; ++n)
        for (int l = 0; l <= lmax; ++l)
          for (int k = 0; k <= l; ++k) {
            const Complex v = toSi * tides[lm * n + Index(l, k)];
            std::snprintf(row, sizeof(row), "%zu %.17g %d %d %.17g %.17g\n", n, c.timesYr[n], l, k, v.real(),
                          v.imag());
            out << row;
          }
      if (!out) throw std::runtime_error("cannot write the tide kernels of " + m.name);
    }
    if (c.viscosityKernels) {
      // dJ / d delta per unit volume (SI): the gradient over the samples' volumes
      const double toSi = scale / (length * length * length);
      std::vector<double> density(values);
      for (size_t x = 0; x < values; ++x) density[x] = toSi * gradient[x] / volume[x];
      std::ofstream bin(dir / (m.name + "_viscosity_kernels.bin"), std::ios::binary);
      bin.write(reinterpret_cast<const char*>(density.data()), static_cast<std::streamsize>(values * sizeof(double)));
      std::ofstream grid(dir / (m.name + "_viscosity_grid.txt"));
      grid << "# " << m.name << "_viscosity_kernels.bin: the log-viscosity kernel dJ / d delta (" << unit
           << " per m^3; eta = eta_ref exp(delta)), float64 little-endian, node-major [node][colatitude][longitude], "
           << P << " x " << nt << " x " << np << "; dJ = sum K d delta dV\n# nodes (radius m)\n";
      char row[64];
      for (int p = 0; p < P; ++p) {
        std::snprintf(row, sizeof(row), "%.17g\n", radius[p] * length);
        grid << row;
      }
      grid << "# colatitudes (rad)\n";
      for (int j = 0; j < nt; ++j) {
        std::snprintf(row, sizeof(row), "%.17g\n", theta[j]);
        grid << row;
      }
      grid << "# longitudes: " << np << ", 2 pi k / " << np << "\n";
      if (!bin || !grid) throw std::runtime_error("cannot write the viscosity kernels of " + m.name);
    }
    std::printf("sl3d: measurement %s (node %zu) = %.17g %s; kernels in %s\n", m.name.c_str(), m.node, value, unit,
                c.kernelDir.c_str());
  }
  return 0;
}
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3 || (std::strcmp(argv[1], "check") != 0 && std::strcmp(argv[1], "solve") != 0 &&
                    std::strcmp(argv[1], "kernel") != 0)) {
    std::fprintf(stderr, "usage: sl3d check|solve|kernel CONFIG.json\n");
    return 2;
  }
  try {
    const Config c = ReadConfig(argv[2]);
    if (std::strcmp(argv[1], "check") == 0) {
      std::printf("sl3d: config ok: run hash %016llx, lmax %d, %zu layers, %zu nodes%s%s\n",
                  static_cast<unsigned long long>(c.hash), c.options.lmax, c.layers.size(), c.timesYr.size(),
                  c.ocean ? ", ocean" : "",
                  c.kernels ? (", kernels of " + std::to_string(c.measurements.size()) + " measurement(s)").c_str()
                            : "");
      return 0;
    }
    if (std::strcmp(argv[1], "kernel") == 0) {
      if (!c.kernels) throw std::invalid_argument("kernel: the config needs a kernels block");
      return Kernel(c);
    }
    return Solve(c);
  } catch (const std::invalid_argument& e) {
    std::fprintf(stderr, "sl3d: %s\n", e.what());
    return 2;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "sl3d: %s\n", e.what());
    return 1;
  }
}
