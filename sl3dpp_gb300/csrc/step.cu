// The GB300 3D quasi-static step: Viscoelastic3D's fixed-point step
// (src/Viscoelastic3D.cpp:1223-2030) with every per-pass operation on the
// device and the host only steering the iteration.
//
// A pass (Respond + AddChannels + StrainOf): the lateral force W d of the
// iterate strain, transformed only at the memory nodes where W is not
// identically zero (elsewhere the reference's Analyse(0) is exactly zero) --
// Legendre synthesis, the ring FFTs with the pointwise weight fused in shared
// memory, Legendre analysis accumulated onto the stage's fixed memory force;
// the force assembly onto every degree's spheroidal and toroidal right-hand
// sides; one batched band solve over every system; the load channel; the
// strain recovery into the next iterate. The convergence measure and the
// Anderson mixer (Gram least squares in FP64 on the device) close the loop;
// the host reads three numbers per pass.
//
// The mixed form (precision 1) keeps that loop's FP64 passes and its stopping
// rule, and between two of them solves for the correction in FP32: with
// G(s) = B s + c the pass and r = G(s) - s its residual, the fixed point is
// s + e with e = B e + r, and e is iterated (with the same Anderson
// acceleration) through FP32 passes -- the FP32 table, ring FFTs, band solves
// with the FP64 factors rounded to FP32, force and strain maps -- to a loose
// relative change; s += e in FP64 and the next FP64 pass measures the true
// residual. B has neither the fixed memory force nor the load, so the
// correction passes need neither.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "assemble.cuh"
#include "host/earth.hpp"
#include "profile.cuh"
#include "sealevel.cuh"
#include "sht.cuh"
#include "step_kernels.cuh"
#include "systems.cuh"

namespace sl3dgpu {


namespace {

using host::Scheme;

// A grid tensor: the spin -2 and -1 components complex, spin 0 real.
struct GridTensor {
  Dev<double2> c0, c1;
  Dev<double> r;
  cudaError_t Alloc(size_t values) {
    if (auto e = c0.Alloc(values); e != cudaSuccess) return e;
    if (auto e = c1.Alloc(values); e != cudaSuccess) return e;
    return r.Alloc(values);
  }
};

}  // namespace

// A state: the memory tensors and the strain on the grid at the lateral
// nodes [latFirst, latEnd), the memory as spectral coefficients at the
// others (mSpec, the same [row][node] layout as the strain coefficients),
// and the strain coefficients at every node.
struct V3dState {
  std::vector<GridTensor> m;
  std::vector<Dev<double2>> mSpec;
  GridTensor strain;
  Dev<double2> coeffs;
  Dev<double2> prev;  // the step before's coefficients (warm_start 1)
  bool hasStrain = false;
  bool hasCoeffs = false;
  bool hasPrev = false;
  int latFirst = 0, latEnd = 0;  // the lateral range the state is laid out for
};

class Viscoelastic3DGpu {
 public:
  sl3dgpu_v3d_options options{};
  std::unique_ptr<host::LayeredBody> earth;
  std::unique_ptr<host::RadialMesh> mesh;
  std::unique_ptr<host::Material> material;
  std::unique_ptr<host::Rheology> rheology;
  std::unique_ptr<host::RelaxingBody> reference;
  // The degrees' unknowns and the flavours' assembly: every degree's layout,
  // the plan of their bands and the nodal material on the device.
  std::vector<host::SpheroidalLayout> sphLayouts;
  std::vector<host::ToroidalLayout> torLayouts;
  AssemblyPlan plan;
  DeviceMaterial deviceMaterial;
  std::unique_ptr<Grid> grid;
  cudaStream_t stream = nullptr;

  // memory nodes
  std::vector<int> nodeElement, nodeQ, elemFirstNode, firstNode;
  std::vector<double> nodeR;
  int P = 0, K = 0;
  long long fieldSize = 0, values = 0;
  long long rows0 = 0, rows1 = 0, rowsR = 0, spectralComplex = 0;
  int lateralFirst = 0, lateralEnd = 0;  // nodes [first, end) where the lateral weight may be non-zero

  // device geometry
  Geometry geo{};
  Dev<int> dNodeElement, dNodeQ, dElemFirstNode, dSphMap, dTorMap;
  Dev<double> dNodeR, dElemJac, dValue, dDeriv, dWeight;
  Dev<double> dCoef64;  // the node coefficient tables (Geometry::coef64/coef32)
  Dev<float> dCoef32;
  Dev<DegreeInfo> dDegrees;
  std::vector<DegreeInfo> degrees;
  long long rhsSphComplex = 0, rhsTorComplex = 0;

  // per-operator device data
  Dev<double> factor, muBranch, itauRef;
  std::vector<std::unique_ptr<Flavour>> flavours;  // most recent first
  std::unique_ptr<Flavour> elastic;

  // workspaces
  Dev<double2> rhsSph, rhsTor;
  Dev<double2> s, sNext, fixedS, analysed, analysedStart;
  Dev<double2> spectraA, spectraB;
  GridTensor fixedGrid, dGrid;
  Dev<double> weight;
  std::vector<Dev<double>> beta;
  Dev<double2> sigma0, sigmaMid, sigma1, surfaceOut;
  Dev<double> changePartial, changeResult;
  double* hostResult = nullptr;  // pinned
  static constexpr int kChangeBlocks = 1024;

  // mixer
  int mixerMemory = 0;
  Dev<double> xPrev, fPrev, gammaOut, mixPartial, mixSums;
  // the Anderson least squares runs on the host: each mixer's Gram matrix,
  // and pinned room for an update's sums (16) and gamma (9)
  // the mixers' Gram matrices (memory x memory), on the device
  Dev<double> gram64, gram32;
  double* hostMix = nullptr;
  int MixerDeviceSolve(Dev<double>& gram, int m, int slot, int memory);
  std::vector<Dev<double>> dG, dF;
  Dev<double*> dGPtr, dFPtr;
  static constexpr int kMixBlocks = 1024;
  static constexpr int kMixBlocks32 = 1216;  // 8 a multiprocessor; FP32 sums of about a hundred products a thread
  static constexpr double kWarmKeep = 0.3;   // the largest first change a kept warm start may show

  // the mixed form's FP32 correction: iterate, next iterate, residual,
  // analysed force, right-hand sides, spectra, weight and its own mixer
  Dev<float2> e32, r32, rhsSph32, rhsTor32;  // every node
  // the correction's iterate, next iterate, residual and analysed force at
  // the lateral nodes only, compact [row][lateral node]; the geometry seen
  // from those nodes (renumbered from 0)
  Dev<float2> eL, eNextL, rL, analysedL;
  long long compactComplex = 0;
  Geometry geoL{};
  Dev<int> dElemFirstNodeL;
  Dev<DegreeInfo> dDegreesL;
  int geoLFirst = -1, geoLEnd = -1;
  // the dof maps (host copies) and, per degree, the rows {lo, hi} the
  // lateral nodes' forces reach in its spheroidal and toroidal systems
  std::vector<int> hostSphMap, hostTorMap;
  std::vector<int2> sphWindow, torWindow;
  int SolveWindows(const Flavour& f);
  size_t mixer32Size = 0;
  Dev<float> spectra32A, spectra32B, weight32;
  int mixer32Memory = 0;
  Dev<float> xPrev32, fPrev32;
  std::vector<Dev<__nv_bfloat16>> dG32, dF32;  // the correction's history, BF16
  Dev<__nv_bfloat16*> dG32Ptr, dF32Ptr;
  std::vector<double> correctionHistory;  // the last step's FP32 pass changes
  // The FP32 correction's loop as a CUDA graph: a while node over one pass,
  // its relative change, the device-side decision (CorrectionControl) and
  // the mixer's kernels, rebuilt when anything it captured moved (keyed by
  // the flavour, the lateral range and every buffer it reads or writes).
  struct CorrectionGraph {
    std::vector<long long> key;
    cudaGraphExec_t exec = nullptr;
    long long launchesPerPass = 0;
  };
  std::vector<CorrectionGraph> correctionGraphs;
  Dev<CorrectionControl> correctionControl;
  bool useGraphs = true;  // SL3DGPU_NO_GRAPHS=1 keeps the loop on the host
  std::vector<long long> CorrectionKey(const Flavour& f) const;
  int CorrectionGraphFor(const Flavour& f, CorrectionGraph** out);
  int CaptureCorrectionBody(const Flavour& f, cudaGraphConditionalHandle handle);

  // conjugate gradients (solver 1): forces, iterate, residual, preconditioned
  // residual, direction and product, each the spheroidal then the toroidal
  // right-hand sides; the pairing's chunks and partial sums
  Dev<double2> cgF, cgX, cgR, cgZ, cgP, cgAp;
  Dev<PairChunk> pairChunks;
  int pairChunkCount = 0;
  Dev<double> pairPartial, pairResult;

  // The static perturbation problem (ElasticPerturbation3D): GLL nodes of the
  // solid elements, the elastic systems, dMu as the tensor weight and dKappa
  // on the dilatation companion.
  bool staticMode = false;
  std::unique_ptr<host::MemoryPoints> gllPoints;
  Dev<double> kappaWeight;
  Dev<double2> scalarD, scalarW;
  bool hasMu = false, hasKappa = false;

  // The warm-start hook (Converge's start argument): a caller's guess of the
  // strain coefficients at the end of the next step, tried against the plain
  // start (the previous strain) on the step's last stage and kept only if its
  // first residual is the smaller.
  Dev<double2> guess, guessNext, guessMid;
  bool guessArmed = false;
  const double2* stageGuess = nullptr;  // the guess the running stage may take
  int guessTaken = 0;  // the last step: 1 when the guess was kept

  V3dState scratch;  // the second buffer set a step writes into
  std::vector<double> history;  // the last step's pass residuals, stages in turn

  // The ocean closure (Evolution3D's Coupled::Closure, src/Evolution3D.cpp:
  // 296-339, frozen shorelines): in every pass the surface responses of the
  // degree solves (before the channels) close the sea-level equation on the
  // flavour's effective Love numbers, on the sea-level grid, and its total
  // load and centrifugal potential become the pass's load and tide channels.
  struct Ocean {
    bool on = false;
    sl3dgpu_grid* grid = nullptr;  // the sea-level grid (lmax, spin 0, oversampling 1)
    SleWorkspace* ws = nullptr;
    sl3dgpu_sle_body body{};       // the constants, model units; the Love arrays per flavour
    double rtol = 1e-10;
    int maxIterations = 200, memory = 5;
    long long fieldSize = 0;
    Dev<double> function, load0, load1, stageLoad, slc;
    Dev<double2> U, V, Phi, sigma, psi;
    double cStart = 0.0, cEnd = 1.0;  // the running stage's start and end as fractions of the step
    sl3dgpu_sle_result last{};        // the last closure's solve
    bool solved = false;
    // Migrating shorelines (Coupled::Closure's nonlinear branch,
    // src/Evolution3D.cpp:308-319): the background state (ice, sea level,
    // flotation's ocean function in `function`, the land held), the ice at
    // the running step's two ends and the stage's change from the
    // background, and the last closure's ocean function.
    bool migrating = false, hasLand = false, hasLoads = false;
    double iceDensity = 0.0;
    int maxNonlinear = 50;
    Dev<double> ice, seaLevel, ice0, ice1, stageIceChange, current;
    Dev<unsigned char> land;
    ~Ocean() {
      if (ws) FreeSleWorkspace(ws);
      if (grid) sl3dgpu_grid_destroy(grid);
    }
  } ocean;
  int SetOcean(const sl3dgpu_v3d_ocean* o);
  int StageLoad(double c);
  int EffectiveLove(const Flavour& f, const std::vector<double>** out);
  int EffectiveLoveOf(int scheme, double dt, const std::vector<double>** out);
  int Closure(const Flavour& f);
  int StepOcean(V3dState& st, double dt, int scheme, const double* load0, const double* load1,
                sl3dgpu_step_info* info);
  int RunOcean(V3dState& st, const double* times, int nodes, int scheme, const double* loads, double* u, double* phi,
               double* slc, double* omega, sl3dgpu_step_info* infos);
  int SeaLevel(double* coefficients, double* omega, sl3dgpu_sle_result* result);
  int StepMigrating(V3dState& st, double dt, int scheme, const double* ice0, const double* ice1, const double* load0,
                    const double* load1, sl3dgpu_step_info* info);
  int RunMigrating(V3dState& st, const double* times, int nodes, int scheme, const double* ice, const double* loads,
                   double* u, double* phi, double* slc, double* omega, double* oceans, sl3dgpu_step_info* infos);
  int OceanFunction(double* out);

  // The discrete adjoint of Run without an ocean (AdjointSolver3D under
  // AdjointMethod::Discrete, src/AdjointDiscrete3D.cpp): the forward run
  // recorded (every stride-th node kept), then the transposed sweep node by
  // node. With no ocean the step's system (K - F An W Syn Str) x = F phi +
  // C sigma is symmetric, so each stage's transposed fixed point is the
  // step's own iteration, over the operator's lateral range, with a dual
  // right-hand side. The memory and strain duals are grid tensors at every
  // node (at the nodes where W is zero they stay band-limited, the exact
  // image of the forward's coefficient memory there), so that the
  // log-viscosity gradient is formed at every node.
  Dev<double> nodeVolume, colWeight;  // rho_p r_p^2 per memory node; w_theta 2 pi / nphi per colatitude
  const double2* passAddSph = nullptr;  // solutions a pass adds after its solve (the dual's K^-1 S^T g)
  const double2* passAddTor = nullptr;
  struct AdjointBuffers {
    std::vector<GridTensor> m, hold;  // memory duals per branch; Sdirk2's held share
    GridTensor d, bar;                // the strain dual; the end strain's total dual
    std::vector<GridTensor> startM;   // the stage's start memory on the grid at every node
    GridTensor startD, endD;          // its start and end strain on the grid at every node
    Dev<double2> qSph, qTor, gU, gPhi, sigma, tide;
    Dev<double> grad;
    V3dState scratch, stage;          // StartStage's output; Sdirk2's recomputed first stage
    // the last two converged dual strains per stage kind (one-stage, Sdirk2's
    // first, its second): the next transposed solve's extrapolated start
    Dev<double2> last[3], before[3];
    int count[3] = {0, 0, 0};
    bool ready = false;
  } adj;
  // The tangent-linear run (TangentLinearSolver3D's discrete run) beside
  // its forward run, stage by stage: the tangent memory and strain on the
  // grid at every node, each stage's tangent solve the step's own iteration
  // with the tangent's fixed force and load channel.
  struct TangentBuffers {
    std::vector<GridTensor> m, hold;  // tangent memory per branch; Sdirk2's held start
    GridTensor d, fixed;              // the tangent strain; a stage's fixed force
    Dev<double> direction;            // p per grid value
    Dev<double2> load0, load1, loadMid;
    V3dState prev, first, end;        // the forward's start, first stage and end states
    bool ready = false;
  } tan;
  int AllocAdjoint();
  int ForwardFields(const V3dState& in, const V3dState& end);
  int TangentStage(V3dState& in, const V3dState& end, double dt, int scheme, const double2* loadDot,
                   sl3dgpu_step_info& info);
  int TangentRun(const double* times, int nodes, int scheme, const double* loads, const double* direction,
                 const double* loadDirections, double* u, double* phi, sl3dgpu_step_info* infos);
  int CopyState(const V3dState& from, V3dState& to);
  int StageAdjoint(V3dState& in, const V3dState& end, double dt, int scheme, bool measured, int kind,
                   sl3dgpu_step_info& info);
  int ArmGuess(const double2* a, const double2* b, double c);
  int AdjointRun(const double* times, int nodes, int scheme, int stride, const double* loads, const double* uDual,
                 const double* phiDual, double* loadKernels, double* tideKernels, double* deltaGradient,
                 double* objective, sl3dgpu_step_info* infos);
  int AdjointSweep(const double* times, int nodes, int scheme, int stride, const double* loads, const double* uDual,
                   const double* phiDual, double* loadKernels, double* tideKernels, double* deltaGradient,
                   double* objective, sl3dgpu_step_info* infos);

  ~Viscoelastic3DGpu() {
    for (auto& g : correctionGraphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    if (hostResult) cudaFreeHost(hostResult);
    if (hostMix) cudaFreeHost(hostMix);
    if (stream) cudaStreamDestroy(stream);
  }

  int Create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options& opt, bool staticPerturbation = false);
  // ElasticPerturbation3D: the moduli directions (either may be null), the
  // reference load response, the Born response of the held solution, the
  // full solve by conjugate gradients.
  int SetModuli(const double* dMu, const double* dKappa, bool onDevice);
  int SolveLoad(const double* load);
  int Respond();
  int SolveLateral(const double* load, double rtol, int maxIterations, sl3dgpu_step_info* info);
  // The warm start of the next step (device layout of a state's coefficients).
  int SetStart(const double* coefficients, bool onDevice);
  // Evolution3D::Run without ocean or rotation: the march over the node times.
  int Run(V3dState& st, const double* times, int nodes, int scheme, const double* loads, double* u, double* phi,
          sl3dgpu_step_info* infos);
  int SetDelta(const double* samples, bool onDevice);
  int ZeroState(V3dState& st);
  int Step(V3dState& st, double dt, int scheme, const double* load0, const double* load1, sl3dgpu_step_info* info,
           bool onDevice = false, const double* tide0 = nullptr, const double* tide1 = nullptr);
  Dev<double2> tideDev0, tideDev1, tideDevMid;
  int Surface(int component, double* out, bool deviceOut = false);
  int InertiaMoment(double* out);
  std::vector<double> momentRow;  // the degree-0 inertia-moment row over its dofs
  int StrainReference(const V3dState& st, double* out);
  // The assembled (unscaled) upper band of degree l's spheroidal or
  // toroidal system in the flavour (scheme, dt); dt = 0 the elastic one.
  int AssembledBand(int scheme, double dt, int toroidal, int l, double* out, long long capacity, int* n, int* kd);

 private:
  int AllocState(V3dState& st);
  int BuildFlavour(const host::PointShear& shear, Flavour& f);
  int FlavourOf(int scheme, double dt, Flavour** out);
  int Synthesise(const double2* spectral, GridTensor& out);
  // Over the nodes [p0, p0 + count) only (the spectral arrays keep their
  // every-node layout; the grid fields their node-major one).
  int SynthesiseRange(const double2* spectral, GridTensor& out, int p0, int count);
  int AnalyseRange(const GridTensor& in, double2* spectral, int p0, int count);
  // A state laid out for another lateral range moved to the current one.
  int AdaptState(V3dState& st);
  SpectralMemoryArgs SpectralArgs(int scheme, double dt, const V3dState& in, V3dState& out, const double2* strain,
                                  double2* fixed) const;
  int Analyse(const GridTensor& in, double2* spectral);
  int AnalyseWeighted(const GridTensor& in, const double* w, double2* spectral);  // accumulate, lateral nodes
  int WeightedPass(const double2* strain, double2* out);                           // accumulate, lateral nodes
  int Solve(const Flavour& f);
  int Respond(const Flavour& f, const double2* strain, bool useStart);
  int Pass(const Flavour& f, const double2* strain, bool useStart, const double2* sigma, const double2* tide,
           double2* next);
  // the running stage's tide coefficients at its start and end (null: none)
  const double2* tideStart = nullptr;
  const double2* tideEnd = nullptr;
  int RelativeChange(const double2* next, const double2* now, double* residual);
  int MixerReset();
  int MixerUpdate(int& count, int& slot, bool& first);
  int PrepareLateral();
  int WeightedPass32(const float2* strain, float2* out);  // compact lateral arrays
  int Pass32(const Flavour& f, const float2* e, float2* next);
  int Mixer32Reset();
  // the FP32 correction's Anderson history (correction_memory, else anderson_memory)
  int CorrectionMemory() const { return options.correction_memory > 0 ? options.correction_memory : options.anderson_memory; }
  int Mixer32Update(int& count, int& slot, bool& first);
  int Correct(const Flavour& f, double tolerance, sl3dgpu_step_info& info, const double2* warm);
  int SolveColumns(const Flavour& f, double2* sph, double2* tor);
  int LateralForce(const double2* x, double2* out);
  int ApplyOperator(const Flavour& f, const double2* x, double2* out);
  int PairOf(const double2* a, const double2* b, double* out);
  int ConvergeConjugateGradients(const Flavour& f, const double2* sigmaEnd, sl3dgpu_step_info& info);
  int ConjugateGradients(const Flavour& f, bool lateral, double rtol, int maxIterations, sl3dgpu_step_info& info);
  int FirstPass(const Flavour& f, const double2* sigmaEnd, double* residual);
  int PerturbationForce(const double2* x, double2* out);
  int ApplyPerturbed(const Flavour& f, const double2* x, double2* out);
  int HoldSolution(const double2* x);
  long long Columns() const { return rhsSphComplex + std::max<long long>(rhsTorComplex, 1); }
  int Converge(const Flavour& f, const double2* sigmaEnd, sl3dgpu_step_info& info);
  int ConvergeMixed(const Flavour& f, const double2* sigmaEnd, sl3dgpu_step_info& info);
  int ElasticStrain(const V3dState& st, const double2* sigma);
  int StepOnce(V3dState& in, V3dState& out, double dt, int scheme, const double2* sigmaStart,
               const double2* sigmaEnd, sl3dgpu_step_info& info);
  int StartStage(V3dState& in, V3dState& out, double dt, int scheme, const double2* sigmaStart, Flavour** f);
  int FinishStage(V3dState& out, double dt, int scheme);
  int Adopt(V3dState& st);

 public:
  // The open step: one stage opened on the operator's buffers (s holds the
  // start strain; rhsSph / rhsTor the last Respond's solutions).
  struct OpenStage {
    bool open = false;
    V3dState* st = nullptr;
    Flavour* f = nullptr;
    int scheme = 0;
    double dt = 0.0;
  } opened;
  int OpenStart(V3dState& st, double dt, int scheme, const double* load0);
  int OpenCheck() const;
  int OpenChannels(const double* load, const double* tide);
  int OpenConverge(const double* load, const double* tide, sl3dgpu_step_info* info);
  int OpenFinish(const double2* strain);
  // OpenStep::Forces / Apply / Solve (the conjugate-gradient close, under
  // Options::solver = ConjugateGradients): the step's degree forces (the
  // fixed memory force's and the channels'), (K_eff - P^T W S) x, and the
  // solutions for given forces from the reference response.
  int OpenForces(const double* load, const double* tide, double2* out);
  int OpenApply(const double2* x, double2* out);
  int OpenSolve(const double2* forces, double2* out, sl3dgpu_step_info* info);
  int OpenRespond(const double2* strain) {
    SL3D_TRY(OpenCheck());
    SL3D_TRY(Respond(*opened.f, strain, strain == nullptr));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    return SL3DGPU_OK;
  }
  // GridCoupling's maps on the operator's nodes and grid (device arrays in
  // the device layouts): Synthesise / Analyse of a tensor field, the degree
  // forces of an analysed tensor, the strain of solutions.
  int TensorSynthesise(const double2* spectral, double2* c0, double2* c1, double* r);
  int TensorAnalyse(const double2* c0, const double2* c1, const double* r, double2* spectral);
  int DegreeForces(const double2* spectral, double2* sph, double2* tor);
  int StrainOfSolutions(const double2* sph, const double2* tor, double2* spectral);
  // A state as bytes (checkpoints): a header, each branch's memory on the
  // grid at the lateral nodes and as coefficients, the strain likewise, the
  // coefficients (and the step before's under warm_start 1).
  long long StateBytes(const V3dState& st) const;
  int SaveState(const V3dState& st, char* out, long long capacity);
  int LoadState(V3dState& st, const char* in, long long bytes);
  // ElasticPerturbation3D::Force / Apply / LoadForces on device solutions
  // in the [spheroidal | toroidal] layout, and the held solution.
  int StaticForce(const double2* x, double2* out) {
    SL3D_TRY(PerturbationForce(x, out));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    return SL3DGPU_OK;
  }
  int StaticApply(const double2* x, double2* out) {
    SL3D_TRY(ApplyPerturbed(*elastic, x, out));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    return SL3DGPU_OK;
  }
  int StaticLoadForces(const double* load, double2* out) {
    const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
    SL3D_CUDA(cudaMemcpyAsync(sigma0.p, load, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    SL3D_CUDA(cudaMemsetAsync(out, 0, Columns() * sizeof(double2), stream));
    LaunchAddLoad(geo, sigma0.p, elastic->loadForces.p, elastic->unitOffset.p, out, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaStreamSynchronize(stream));
    return SL3DGPU_OK;
  }
  int StaticSolution(double2* out) {
    SL3D_CUDA(cudaMemcpyAsync(out, rhsSph.p, rhsSphComplex * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
    if (rhsTorComplex > 0)
      SL3D_CUDA(cudaMemcpyAsync(out + rhsSphComplex, rhsTor.p, rhsTorComplex * sizeof(double2),
                                cudaMemcpyDeviceToDevice, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    return SL3DGPU_OK;
  }
  int Change(const double2* next, const double2* now, double* out) {
    SL3D_TRY(RelativeChange(next, now, out));
    return SL3DGPU_OK;
  }
  double2* Block(double2* base, int spin) const {
    return base + (spin == -2 ? 0 : spin == -1 ? rows0 * P : (rows0 + rows1) * P);
  }
};

// -- construction ----------------------------------------------------------------------------------

int Viscoelastic3DGpu::Create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options& opt,
                              bool staticPerturbation) {
  if (const char* off = std::getenv("SL3DGPU_NO_GRAPHS"); off != nullptr && off[0] == '1') useGraphs = false;
  options = opt;
  staticMode = staticPerturbation;
  if (opt.lmax < 2 || opt.ngll < 2 || !(opt.oversampling >= 1.0) || opt.anderson_memory > 8 ||
      opt.anderson_memory < 0 || nlayers < 1) {
    SetError("v3d: lmax >= 2, ngll >= 2, oversampling >= 1, anderson_memory in [0, 8]");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.precision != 0 && opt.precision != 1) {
    SetError("v3d: precision 0 (FP64) or 1 (mixed)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.solver != 0 && opt.solver != 1) {
    SetError("v3d: solver 0 (fixed point) or 1 (conjugate gradients)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.solver == 1 && (opt.precision != 0 || !(opt.solve_rtol > 0.0) || opt.solve_max_iterations < 0)) {
    SetError("v3d: conjugate gradients run in FP64 (precision 0) with solve_rtol > 0 and solve_max_iterations >= 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.warm_start != 0 && opt.warm_start != 1) {
    SetError("v3d: warm_start 0 (the previous step's strain) or 1 (the extrapolation of the last two)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.fp64_emulation != 0 && opt.fp64_emulation != 1) {
    SetError("v3d: fp64_emulation 0 (the FP64 units) or 1 (the tensor cores)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.correction_memory < 0 || opt.correction_memory > kMixMaxMemory) {
    SetError("v3d: correction_memory in [0, 16] (0: anderson_memory)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (opt.precision == 1 && !(opt.correction_rtol > 0.0 && opt.correction_rtol < 1.0)) {
    SetError("v3d: the mixed form needs 0 < correction_rtol < 1");
    return SL3DGPU_ERR_ARGUMENT;
  }
  try {
    std::vector<host::Layer> ls(nlayers);
    for (int i = 0; i < nlayers; ++i) {
      const auto& s = layers[i];
      ls[i] = host::Layer{s.r0, s.r1, s.fluid != 0, s.rho0, s.rho1, s.kappa0, s.kappa1, s.mu0, s.mu1,
                          s.viscosity, s.kelvin_fraction, s.kelvin_viscosity, s.elements};
    }
    earth = std::make_unique<host::LayeredBody>(ls, host::Scales::Geophysical(layers[nlayers - 1].r1));
    mesh = std::make_unique<host::RadialMesh>(host::RadialMesh::Create(*earth, opt.ngll));
    material = std::make_unique<host::Material>(host::Material::Create(*earth, *mesh));
    rheology = std::make_unique<host::Rheology>(host::Rheology::FromBody(*earth, *material));
    reference = std::make_unique<host::RelaxingBody>(*rheology);
  } catch (const std::exception& e) {
    SetError(std::string("v3d: ") + e.what());
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (rheology->branches.size() > 2) {
    SetError("v3d: at most two Prony branches");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  SL3D_CUDA(cudaMallocHost(&hostResult, 8 * sizeof(double)));
  SL3D_CUDA(cudaMallocHost(&hostMix, 4 * kMixMaxMemory * sizeof(double)));  // sums, then gamma
  SL3D_CUDA(mixSums.Alloc(2 * kMixMaxMemory));
  SL3D_TRY(Grid::Create(opt.lmax, 2, opt.oversampling, grid));
  grid->emulateFp64 = opt.fp64_emulation == 1;
  // The step: the long-term material, the Gauss memory points of every
  // element where a branch relaxes. The static perturbation problem: the
  // unrelaxed material and the GLL nodes of every solid element above the
  // one holding the centre (ElasticPerturbation3D's coupling, src/
  // ElasticPerturbation3D.cpp:46-73).
  if (staticMode) gllPoints = std::make_unique<host::MemoryPoints>(host::MemoryPoints::Of(false, *mesh));
  const auto& nodal = staticMode ? *material : reference->nodal;
  const auto& msh = nodal.mesh;
  const auto& pts = staticMode ? *gllPoints : reference->points;
  const int n = msh.NGll(), E = msh.ElementCount(), L = opt.lmax;
  K = staticMode ? 0 : static_cast<int>(rheology->branches.size());
  elemFirstNode.assign(E, -1);
  for (int e = 0; e < E; ++e) {
    bool carries = false;
    if (staticMode) {
      carries = !material->IsFluid(e) && !(e == 0 && msh.Left(0) == 0.0);
    } else {
      for (int i = 0; i < n; ++i) carries = carries || rheology->IsActive(static_cast<size_t>(e) * n + i);
    }
    if (!carries) continue;
    elemFirstNode[e] = static_cast<int>(nodeElement.size());
    for (int p = 0; p < pts.count; ++p) {
      nodeElement.push_back(e);
      nodeQ.push_back(p);
      nodeR.push_back(pts.RadiusAt(msh, e, p));
    }
  }
  P = static_cast<int>(nodeElement.size());
  if (P == 0) {
    SetError("v3d: the rheology has no active branch anywhere");
    return SL3DGPU_ERR_ARGUMENT;
  }
  firstNode.assign(L + 1, P);
  for (int l = 0; l <= L; ++l) {
    const int fe = l > 0 ? msh.StartElement(l, opt.eps) : 0;
    for (int p = 0; p < P; ++p)
      if (nodeElement[p] >= fe) {
        firstNode[l] = p;
        break;
      }
  }
  fieldSize = static_cast<long long>(grid->ntheta) * grid->nphi;
  values = fieldSize * P;
  rows0 = grid->SpinRows(-2);
  rows1 = grid->SpinRows(-1);
  rowsR = grid->RealRows();
  spectralComplex = (rows0 + rows1 + rowsR) * P;
  lateralFirst = 0;
  lateralEnd = P;

  // The elastic operators: the dof maps and right-hand-side layout, shared by
  // every flavour (they depend on the mesh and the degree alone).
  elastic = std::make_unique<Flavour>();
  const int nglob = msh.NodeCount();
  std::vector<int> sphMap(static_cast<size_t>(L + 1) * nglob * 2, -1), torMap(static_cast<size_t>(L + 1) * nglob, -1);
  degrees.resize(L + 1);
  long long sphOff = 0, torOff = 0;
  try {
    for (int l = 0; l <= L; ++l) sphLayouts.emplace_back(nodal, l, opt.eps);
    for (int l = 1; l <= L; ++l) torLayouts.emplace_back(nodal, l, opt.eps);
  } catch (const std::exception& e) {
    SetError(std::string("v3d: ") + e.what());
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (const auto& layout : sphLayouts) plan.Add(layout);
  for (const auto& layout : torLayouts) plan.Add(layout);
  SL3D_TRY(deviceMaterial.Upload(nodal, pts));
  for (int l = 0; l <= L; ++l) {
    const host::SpheroidalLayout& op = sphLayouts[l];
    auto& d = degrees[l];
    d.firstNode = firstNode[l];
    d.firstGlobal = d.firstNode < P ? msh.GlobalIndex(nodeElement[d.firstNode], 0) : 0;
    d.lastGlobal = d.firstNode < P ? msh.GlobalIndex(nodeElement[P - 1], n - 1) : -1;
    d.sphNdof = op.DofCount();
    if (l == 0) {
      // sqrt(4 pi) w_q J_e rho r^3 at each GLL node's U dof, over the whole
      // mesh (detail/ViscoelasticDegree.hpp:142-161)
      momentRow.assign(static_cast<size_t>(d.sphNdof), 0.0);
      const int ng = msh.NGll();
      for (int e = 0; e < msh.ElementCount(); ++e)
        for (int q = 0; q < ng; ++q) {
          const int dof = op.Dof(msh.GlobalIndex(e, q), host::kU);
          if (dof < 0) continue;
          const double r = msh.Radius(e, q);
          momentRow[dof] += std::sqrt(4.0 * 3.14159265358979323846) * msh.Weights()[q] * msh.Jacobian(e) *
                            nodal.rho[static_cast<size_t>(e) * ng + q] * r * r * r;
        }
    }
    d.surfaceU = op.SurfaceDof(host::kU);
    d.surfaceV = op.SurfaceDof(host::kV);
    d.surfacePhi = op.SurfaceDof(host::kPhi);
    d.sphMap = static_cast<long long>(l) * nglob * 2;
    d.torMap = static_cast<long long>(l) * nglob;
    d.sphRhs = sphOff;
    sphOff += static_cast<long long>(d.sphNdof) * (l + 1);
    for (int gn = 0; gn < nglob; ++gn) {
      sphMap[d.sphMap + 2 * gn] = op.Dof(gn, host::kU);
      sphMap[d.sphMap + 2 * gn + 1] = op.Dof(gn, host::kV);
    }
    d.torNdof = 0;
    d.torRhs = torOff;
    d.surfaceW = -1;
    if (l >= 1) {
      const host::ToroidalLayout& top = torLayouts[l - 1];
      d.torNdof = top.DofCount();
      d.surfaceW = top.SurfaceDof();
      torOff += static_cast<long long>(d.torNdof) * (l + 1);
      for (int gn = 0; gn < nglob; ++gn) torMap[d.torMap + gn] = top.Dof(gn);
    }
  }
  rhsSphComplex = sphOff;
  rhsTorComplex = torOff;
  hostSphMap = sphMap;
  hostTorMap = torMap;

  std::vector<double> elemJac(E);
  for (int e = 0; e < E; ++e) elemJac[e] = msh.Jacobian(e);
  SL3D_CUDA(dNodeElement.Upload(nodeElement));
  SL3D_CUDA(dNodeQ.Upload(nodeQ));
  SL3D_CUDA(dNodeR.Upload(nodeR));
  SL3D_CUDA(dElemFirstNode.Upload(elemFirstNode));
  SL3D_CUDA(dElemJac.Upload(elemJac));
  SL3D_CUDA(dValue.Upload(pts.value));
  SL3D_CUDA(dDeriv.Upload(pts.derivative));
  SL3D_CUDA(dWeight.Upload(pts.weight));
  SL3D_CUDA(dDegrees.Upload(degrees));
  SL3D_CUDA(dSphMap.Upload(sphMap));
  SL3D_CUDA(dTorMap.Upload(torMap));
  const SpinTable *t0 = nullptr, *t1 = nullptr, *tr = nullptr;
  SL3D_TRY(grid->Table(-2, &t0));
  SL3D_TRY(grid->Table(-1, &t1));
  SL3D_TRY(grid->Table(0, &tr));
  geo = Geometry{L, P, n, pts.count, E, dNodeElement.p, dNodeQ.p, dNodeR.p, dElemFirstNode.p, dElemJac.p,
                 dValue.p, dDeriv.p, dWeight.p, t0->dRowOffset, t1->dRowOffset, tr->dRowOffset,
                 rows0, rows1, rowsR, dDegrees.p, dSphMap.p, dTorMap.p, {}, {}, 0};
  for (const auto& d : degrees) geo.maxGlobals = std::max(geo.maxGlobals, d.lastGlobal - d.firstGlobal + 1);
  {
    const auto coef = NodeCoefficients(P, n, nodeElement, nodeQ, nodeR, elemJac, pts.value, pts.derivative,
                                       pts.weight);
    SL3D_CUDA(dCoef64.Upload(coef));
    SL3D_CUDA(dCoef32.Upload(std::vector<float>(coef.begin(), coef.end())));
    const size_t plane = static_cast<size_t>(P) * n;
    for (int w = 0; w < 4; ++w) {
      geo.coef64[w] = dCoef64.p + w * plane;
      geo.coef32[w] = dCoef32.p + w * plane;
    }
  }

  {
    std::vector<double> volume(P), colw(grid->ntheta);
    for (int p = 0; p < P; ++p)
      volume[p] = elemJac[nodeElement[p]] * pts.weight[nodeQ[p]] * nodeR[p] * nodeR[p];
    for (int j = 0; j < grid->ntheta; ++j) colw[j] = grid->weights[j] * 2.0 * 3.14159265358979323846 / grid->nphi;
    SL3D_CUDA(nodeVolume.Upload(volume));
    SL3D_CUDA(colWeight.Upload(colw));
  }

  // Branch moduli and reference inverse times at the nodes; exp(-delta) = 1.
  std::vector<double> mu(static_cast<size_t>(K) * P), itau(static_cast<size_t>(K) * P);
  for (int k = 0; k < K; ++k)
    for (int p = 0; p < P; ++p) {
      const size_t at = static_cast<size_t>(nodeElement[p]) * pts.count + nodeQ[p];
      mu[static_cast<size_t>(k) * P + p] = reference->pointMu[k][at];
      itau[static_cast<size_t>(k) * P + p] = reference->pointItau[k][at];
    }
  SL3D_CUDA(muBranch.Upload(mu));
  SL3D_CUDA(itauRef.Upload(itau));
  std::vector<double> ones(values, 1.0);
  SL3D_CUDA(factor.Upload(ones));
  lateralFirst = lateralEnd = 0;  // no lateral variation until delta is set

  // workspaces
  SL3D_CUDA(rhsSph.Alloc(rhsSphComplex));
  SL3D_CUDA(rhsTor.Alloc(std::max<long long>(rhsTorComplex, 1)));
  for (auto* b : {&s, &sNext, &fixedS, &analysed, &analysedStart}) SL3D_CUDA(b->Alloc(spectralComplex));
  const size_t spectra = static_cast<size_t>(2 * L + 1) * grid->ntheta * P;
  SL3D_CUDA(spectraA.Alloc(spectra));
  SL3D_CUDA(spectraB.Alloc(spectra));
  if (!staticMode) {
    SL3D_CUDA(fixedGrid.Alloc(values));
    SL3D_CUDA(dGrid.Alloc(values));
  } else {
    SL3D_CUDA(kappaWeight.Alloc(values));
    SL3D_CUDA(scalarD.Alloc(rowsR * P));
    SL3D_CUDA(scalarW.Alloc(rowsR * P));
  }
  SL3D_CUDA(weight.Alloc(values));
  beta.resize(K);
  for (auto& b : beta) SL3D_CUDA(b.Alloc(values));
  const size_t lm = static_cast<size_t>(L + 1) * (L + 2) / 2;
  for (auto* b : {&sigma0, &sigmaMid, &sigma1, &surfaceOut}) SL3D_CUDA(b->Alloc(lm));
  SL3D_CUDA(changePartial.Alloc(3 * kChangeBlocks));
  SL3D_CUDA(changeResult.Alloc(3));
  SL3D_CUDA(gammaOut.Alloc(kMixMaxMemory + 1));
  SL3D_CUDA(mixPartial.Alloc(static_cast<size_t>(kMixBlocks32) * 2 * kMixMaxMemory));
  if (options.solver == 1) {
    for (auto* b : {&cgF, &cgX, &cgR, &cgZ, &cgP, &cgAp}) {
      SL3D_CUDA(b->Alloc(Columns()));
      SL3D_CUDA(cudaMemsetAsync(b->p, 0, Columns() * sizeof(double2), stream));
    }
    // The pairing's chunks: every degree's spheroidal then toroidal block in
    // spans of at most 16384 values.
    std::vector<PairChunk> chunks;
    auto add = [&](long long start, long long size, int cols) {
      for (long long at = 0; at < size; at += 16384) {
        PairChunk c{};
        c.start = start + at;
        c.end = start + std::min(size, at + 16384);
        c.degreeStart = start;
        c.cols = cols;
        chunks.push_back(c);
      }
    };
    for (int l = 0; l <= L; ++l) add(degrees[l].sphRhs, static_cast<long long>(degrees[l].sphNdof) * (l + 1), l + 1);
    for (int l = 1; l <= L; ++l)
      add(rhsSphComplex + degrees[l].torRhs, static_cast<long long>(degrees[l].torNdof) * (l + 1), l + 1);
    pairChunkCount = static_cast<int>(chunks.size());
    SL3D_CUDA(pairChunks.Upload(chunks));
    SL3D_CUDA(pairPartial.Alloc(chunks.size()));
    SL3D_CUDA(pairResult.Alloc(4));
  }
  if (options.precision == 1) {
    for (auto* b : {&e32, &r32}) SL3D_CUDA(b->Alloc(spectralComplex));
    SL3D_CUDA(rhsSph32.Alloc(rhsSphComplex));
    SL3D_CUDA(rhsTor32.Alloc(std::max<long long>(rhsTorComplex, 1)));
    SL3D_CUDA(spectra32A.Alloc(2 * spectra));
    SL3D_CUDA(spectra32B.Alloc(2 * spectra));
    SL3D_CUDA(weight32.Alloc(values));
  }
  if (!staticMode) SL3D_TRY(AllocState(scratch));
  SL3D_TRY(BuildFlavour(reference->elastic, *elastic));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::AllocState(V3dState& st) {
  st.m.resize(K);
  for (auto& t : st.m) SL3D_CUDA(t.Alloc(values));
  st.mSpec.resize(K);
  for (auto& c : st.mSpec) SL3D_CUDA(c.Alloc(spectralComplex));
  SL3D_CUDA(st.strain.Alloc(values));
  SL3D_CUDA(st.coeffs.Alloc(spectralComplex));
  if (options.warm_start == 1) SL3D_CUDA(st.prev.Alloc(spectralComplex));
  st.hasStrain = st.hasCoeffs = st.hasPrev = false;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::ZeroState(V3dState& st) {
  SL3D_TRY(AllocState(st));
  for (auto& t : st.m) {
    SL3D_CUDA(cudaMemsetAsync(t.c0.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(t.c1.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(t.r.p, 0, values * sizeof(double), stream));
  }
  for (auto& c : st.mSpec) SL3D_CUDA(cudaMemsetAsync(c.p, 0, spectralComplex * sizeof(double2), stream));
  st.latFirst = lateralFirst;
  st.latEnd = lateralEnd;
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::SetDelta(const double* samples, bool onDevice) {
  std::vector<double> host(values);
  if (onDevice)
    SL3D_CUDA(cudaMemcpy(host.data(), samples, values * sizeof(double), cudaMemcpyDeviceToHost));
  else
    std::memcpy(host.data(), samples, values * sizeof(double));
  // exp(-delta) per value (as Viscoelastic3D's constructor samples it), and
  // the nodes where it departs from one: only there can W be non-zero.
  int first = P, last = -1;
  for (int p = 0; p < P; ++p) {
    bool lateral = false;
    for (long long x = p * fieldSize; x < (p + 1) * fieldSize; ++x) {
      host[x] = std::exp(-host[x]);
      lateral = lateral || host[x] != 1.0;
    }
    if (lateral) {
      first = std::min(first, p);
      last = std::max(last, p);
    }
  }
  // whole elements: the range starts at its first node's element's first
  // node and ends at its last node's element's last
  lateralFirst = last >= 0 ? elemFirstNode[nodeElement[first]] : 0;
  lateralEnd = last >= 0 ? elemFirstNode[nodeElement[last]] + geo.np : 0;
  SL3D_CUDA(cudaStreamSynchronize(stream));  // no earlier kernel of the operator still reads it
  SL3D_CUDA(CopyIn(factor.p, host.data(), values * sizeof(double)));
  return SL3DGPU_OK;
}

// -- flavours: assembly on the host (once), factorisation on the device ----------------------------

int Viscoelastic3DGpu::BuildFlavour(const host::PointShear& shear, Flavour& f) {
  static std::atomic<long long> built{0};
  f.id = ++built;
  SystemsInput in;
  in.material = &deviceMaterial;
  in.plan = &plan;
  in.sph = &sphLayouts;
  in.shear = staticMode ? nullptr : &shear;
  in.lmax = options.lmax;
  in.degrees = &degrees;
  in.rhsSphComplex = rhsSphComplex;
  const bool stepFlavour = &f != elastic.get();
  in.apply = (options.solver == 1 && stepFlavour) || staticMode;
  in.fp32 = options.precision == 1 && stepFlavour;
  in.stream = stream;
  return BuildSystems(in, f);
}

int Viscoelastic3DGpu::FlavourOf(int scheme, double dt, Flavour** out) {
  for (size_t i = 0; i < flavours.size(); ++i)
    if (flavours[i]->scheme == scheme && flavours[i]->dt == dt) {
      std::rotate(flavours.begin(), flavours.begin() + i, flavours.begin() + i + 1);
      *out = flavours.front().get();
      return SL3DGPU_OK;
    }
  constexpr size_t kFlavourCache = 4;  // the reference's LRU (Viscoelastic3D.cpp:535-558)
  while (flavours.size() >= kFlavourCache) flavours.pop_back();
  auto f = std::make_unique<Flavour>();
  f->scheme = scheme;
  f->dt = dt;
  SL3D_TRY(BuildFlavour(reference->StepShear(static_cast<Scheme>(scheme), dt), *f));
  flavours.insert(flavours.begin(), std::move(f));
  *out = flavours.front().get();
  return SL3DGPU_OK;
}

// -- transforms over the nodes ----------------------------------------------------------------------

int Viscoelastic3DGpu::Synthesise(const double2* spectral, GridTensor& out) {
  const auto* base = reinterpret_cast<const double*>(spectral);
  auto* spectra = reinterpret_cast<double*>(spectraA.p);
  SL3D_TRY(grid->LegendreSynthesis(-2, false, base, P, 0, P, spectra, stream));
  SL3D_TRY(grid->RingSynthesis(false, spectra, P, reinterpret_cast<double*>(out.c0.p), stream));
  SL3D_TRY(grid->LegendreSynthesis(-1, false, base + 2 * rows0 * P, P, 0, P, spectra, stream));
  SL3D_TRY(grid->RingSynthesis(false, spectra, P, reinterpret_cast<double*>(out.c1.p), stream));
  SL3D_TRY(grid->LegendreSynthesis(0, true, base + 2 * (rows0 + rows1) * P, P, 0, P, spectra, stream));
  return grid->RingSynthesis(true, spectra, P, out.r.p, stream);
}

int Viscoelastic3DGpu::Analyse(const GridTensor& in, double2* spectral) {
  auto* base = reinterpret_cast<double*>(spectral);
  auto* spectra = reinterpret_cast<double*>(spectraA.p);
  SL3D_TRY(grid->RingAnalysis(false, reinterpret_cast<const double*>(in.c0.p), P, spectra, stream));
  SL3D_TRY(grid->LegendreAnalysis(-2, false, spectra, P, 0, P, base, false, stream));
  SL3D_TRY(grid->RingAnalysis(false, reinterpret_cast<const double*>(in.c1.p), P, spectra, stream));
  SL3D_TRY(grid->LegendreAnalysis(-1, false, spectra, P, 0, P, base + 2 * rows0 * P, false, stream));
  SL3D_TRY(grid->RingAnalysis(true, in.r.p, P, spectra, stream));
  return grid->LegendreAnalysis(0, true, spectra, P, 0, P, base + 2 * (rows0 + rows1) * P, false, stream);
}

int Viscoelastic3DGpu::SynthesiseRange(const double2* spectral, GridTensor& out, int p0, int count) {
  if (count <= 0) return SL3DGPU_OK;
  const auto* base = reinterpret_cast<const double*>(spectral);
  auto* spectra = reinterpret_cast<double*>(spectraA.p);
  const long long off = p0 * fieldSize;
  SL3D_TRY(grid->LegendreSynthesis(-2, false, base, P, p0, count, spectra, stream));
  SL3D_TRY(grid->RingSynthesis(false, spectra, count, reinterpret_cast<double*>(out.c0.p + off), stream));
  SL3D_TRY(grid->LegendreSynthesis(-1, false, base + 2 * rows0 * P, P, p0, count, spectra, stream));
  SL3D_TRY(grid->RingSynthesis(false, spectra, count, reinterpret_cast<double*>(out.c1.p + off), stream));
  SL3D_TRY(grid->LegendreSynthesis(0, true, base + 2 * (rows0 + rows1) * P, P, p0, count, spectra, stream));
  return grid->RingSynthesis(true, spectra, count, out.r.p + off, stream);
}

int Viscoelastic3DGpu::AnalyseRange(const GridTensor& in, double2* spectral, int p0, int count) {
  if (count <= 0) return SL3DGPU_OK;
  auto* base = reinterpret_cast<double*>(spectral);
  auto* spectra = reinterpret_cast<double*>(spectraA.p);
  const long long off = p0 * fieldSize;
  SL3D_TRY(grid->RingAnalysis(false, reinterpret_cast<const double*>(in.c0.p + off), count, spectra, stream));
  SL3D_TRY(grid->LegendreAnalysis(-2, false, spectra, P, p0, count, base, false, stream));
  SL3D_TRY(grid->RingAnalysis(false, reinterpret_cast<const double*>(in.c1.p + off), count, spectra, stream));
  SL3D_TRY(grid->LegendreAnalysis(-1, false, spectra, P, p0, count, base + 2 * rows0 * P, false, stream));
  SL3D_TRY(grid->RingAnalysis(true, in.r.p + off, count, spectra, stream));
  return grid->LegendreAnalysis(0, true, spectra, P, p0, count, base + 2 * (rows0 + rows1) * P, false, stream);
}

// The nodes a state holds on the grid follow the operator's lateral range;
// after set_delta moved it, the nodes that became lateral get their grid
// memory and strain by synthesis, those that left it their coefficients by
// analysis (exact for these band-limited fields, to rounding).
int Viscoelastic3DGpu::AdaptState(V3dState& st) {
  if (st.latFirst == lateralFirst && st.latEnd == lateralEnd) return SL3DGPU_OK;
  auto pieces = [](int a0, int a1, int b0, int b1) {
    // [a0, a1) minus [b0, b1), at most two intervals
    std::vector<std::pair<int, int>> out;
    if (a1 <= a0) return out;
    if (b1 <= b0 || b1 <= a0 || b0 >= a1) {
      out.emplace_back(a0, a1);
      return out;
    }
    if (a0 < b0) out.emplace_back(a0, b0);
    if (b1 < a1) out.emplace_back(b1, a1);
    return out;
  };
  for (auto [p0, p1] : pieces(lateralFirst, lateralEnd, st.latFirst, st.latEnd)) {
    for (int k = 0; k < K; ++k) SL3D_TRY(SynthesiseRange(st.mSpec[k].p, st.m[k], p0, p1 - p0));
    if (st.hasCoeffs) SL3D_TRY(SynthesiseRange(st.coeffs.p, st.strain, p0, p1 - p0));
  }
  for (auto [p0, p1] : pieces(st.latFirst, st.latEnd, lateralFirst, lateralEnd))
    for (int k = 0; k < K; ++k) SL3D_TRY(AnalyseRange(st.m[k], st.mSpec[k].p, p0, p1 - p0));
  st.latFirst = lateralFirst;
  st.latEnd = lateralEnd;
  return SL3DGPU_OK;
}

SpectralMemoryArgs Viscoelastic3DGpu::SpectralArgs(int scheme, double dt, const V3dState& in, V3dState& out,
                                                   const double2* strain, double2* fixed) const {
  SpectralMemoryArgs a{};
  a.branches = K;
  a.scheme = scheme == static_cast<int>(Scheme::BackwardEuler) ? 1 : 0;
  a.dt = dt;
  a.rows = rows0 + rows1 + rowsR;
  a.P = P;
  a.pLat0 = lateralFirst;
  a.pLat1 = lateralEnd;
  a.muBranch = muBranch.p;
  a.itauRef = itauRef.p;
  for (int k = 0; k < K; ++k) {
    a.in[k] = in.mSpec[k].p;
    a.out[k] = out.mSpec[k].p;
  }
  a.s = strain;
  a.fixedS = fixed;
  return a;
}

// Analyse(w f) over the lateral nodes, added to what the spectral tensor holds.
int Viscoelastic3DGpu::AnalyseWeighted(const GridTensor& in, const double* w, double2* spectral) {
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  if (count <= 0) return SL3DGPU_OK;
  auto* base = reinterpret_cast<double*>(spectral);
  auto* spectra = reinterpret_cast<double*>(spectraA.p);
  const long long off = p0 * fieldSize;
  SL3D_TRY(grid->RingAnalysis(false, reinterpret_cast<const double*>(in.c0.p + off), count, spectra, stream, w + off));
  SL3D_TRY(grid->LegendreAnalysis(-2, false, spectra, P, p0, count, base, true, stream));
  SL3D_TRY(grid->RingAnalysis(false, reinterpret_cast<const double*>(in.c1.p + off), count, spectra, stream, w + off));
  SL3D_TRY(grid->LegendreAnalysis(-1, false, spectra, P, p0, count, base + 2 * rows0 * P, true, stream));
  SL3D_TRY(grid->RingAnalysis(true, in.r.p + off, count, spectra, stream, w + off));
  return grid->LegendreAnalysis(0, true, spectra, P, p0, count, base + 2 * (rows0 + rows1) * P, true, stream);
}

// Analyse(W Synthesise(strain)) over the lateral nodes, added onto out.
int Viscoelastic3DGpu::WeightedPass(const double2* strain, double2* out) {
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  if (count <= 0) return SL3DGPU_OK;
  const auto* in = reinterpret_cast<const double*>(strain);
  auto* o = reinterpret_cast<double*>(out);
  auto* a = reinterpret_cast<double*>(spectraA.p);
  auto* b = reinterpret_cast<double*>(spectraB.p);
  const double* w = weight.p + p0 * fieldSize;
  const long long offs[3] = {0, 2 * rows0 * P, 2 * (rows0 + rows1) * P};
  const int spins[3] = {-2, -1, 0};
  for (int c = 0; c < 3; ++c) {
    const bool real = c == 2;
    SL3D_TRY(grid->LegendreSynthesis(spins[c], real, in + offs[c], P, p0, count, a, stream));
    SL3D_TRY(grid->RingWeighted(real, a, count, w, b, stream));
    SL3D_TRY(grid->LegendreAnalysis(spins[c], real, b, P, p0, count, o + offs[c], true, stream));
  }
  return SL3DGPU_OK;
}

// -- a pass --------------------------------------------------------------------------------------------

int Viscoelastic3DGpu::Solve(const Flavour& f) { return SolveColumns(f, rhsSph.p, rhsTor.p); }

int Viscoelastic3DGpu::SolveColumns(const Flavour& f, double2* sph, double2* tor) {
  auto* sphD = reinterpret_cast<double*>(sph);
  auto* torD = reinterpret_cast<double*>(tor);
  SL3D_TRY(BandSolveBatch(f.dSphChol.p, f.sphChol.data(), static_cast<int>(f.sphChol.size()), f.iSphChol.p,
                          f.nSphChol, f.bands.p, f.pivots.p, sphD, f.scales.p, 0, stream));
  SL3D_TRY(BandSolveBatch(f.dSphLu.p, f.sphLu.data(), static_cast<int>(f.sphLu.size()), f.iSphLu.p, f.nSphLu,
                          f.bands.p, f.pivots.p, sphD, f.scales.p, 1, stream));
  return BandSolveBatch(f.dTorChol.p, f.torChol.data(), static_cast<int>(f.torChol.size()), f.iTorChol.p,
                        f.nTorChol, f.bands.p, f.pivots.p, torD, f.scales.p, 0, stream);
}

// Respond (Viscoelastic3D.hpp OpenStep::Respond): the solutions of the
// memory and lateral force of a strain (the start strain's force, already
// analysed, when useStart) through the flavour's systems, no channels.
int Viscoelastic3DGpu::Respond(const Flavour& f, const double2* strain, bool useStart) {
  const double2* force = analysedStart.p;
  if (!useStart) {
    SL3D_CUDA(cudaMemcpyAsync(analysed.p, fixedS.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                              stream));
    SL3D_TRY(WeightedPass(strain, analysed.p));
    force = analysed.p;
  }
  SL3D_CUDA(cudaMemsetAsync(rhsSph.p, 0, rhsSphComplex * sizeof(double2), stream));
  SL3D_CUDA(cudaMemsetAsync(rhsTor.p, 0, std::max<long long>(rhsTorComplex, 1) * sizeof(double2), stream));
  LaunchForces(geo, force, rhsSph.p, rhsTor.p, stream);
  SL3D_CHECK_LAUNCH();
  return Solve(f);
}

int Viscoelastic3DGpu::Pass(const Flavour& f, const double2* strain, bool useStart, const double2* sigma,
                            const double2* tide,
                            double2* next) {
  SL3D_TRY(Respond(f, strain, useStart));
  if (ocean.on) {
    // the pass's closure sets its load and tide channels
    SL3D_TRY(Closure(f));
    sigma = ocean.sigma.p;
    tide = ocean.psi.p;
  }
  if (sigma != nullptr || tide != nullptr) {
    LaunchAddLoad(geo, sigma, f.units.p, f.unitOffset.p, rhsSph.p, stream, tide, f.tideUnits.p);
    SL3D_CHECK_LAUNCH();
  }
  if (passAddSph != nullptr) {
    LaunchAxpy(2 * rhsSphComplex, 1.0, reinterpret_cast<const double*>(passAddSph),
               reinterpret_cast<double*>(rhsSph.p), stream);
    SL3D_CHECK_LAUNCH();
    if (rhsTorComplex > 0) {
      LaunchAxpy(2 * rhsTorComplex, 1.0, reinterpret_cast<const double*>(passAddTor),
                 reinterpret_cast<double*>(rhsTor.p), stream);
      SL3D_CHECK_LAUNCH();
    }
  }
  LaunchStrain(geo, rhsSph.p, rhsTor.p, next, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::RelativeChange(const double2* next, const double2* now, double* residual) {
  LaunchRelativeChange(reinterpret_cast<const double*>(next), reinterpret_cast<const double*>(now),
                       2 * spectralComplex, changePartial.p, kChangeBlocks, changeResult.p, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaMemcpyAsync(hostResult, changeResult.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  const double scale = hostResult[0], diff = hostResult[1];
  if (hostResult[2] == 0.0) {
    *residual = std::numeric_limits<double>::quiet_NaN();
  } else {
    *residual = scale > 0.0 ? std::sqrt(diff) / std::sqrt(scale) : 0.0;
  }
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::MixerReset() {
  const int memory = options.anderson_memory;
  if (memory <= 0) return SL3DGPU_OK;
  if (mixerMemory != memory) {
    const size_t n = 2 * spectralComplex;
    dG.resize(memory);
    dF.resize(memory);
    std::vector<double*> gp(memory), fp(memory);
    for (int i = 0; i < memory; ++i) {
      SL3D_CUDA(dG[i].Alloc(n));
      SL3D_CUDA(dF[i].Alloc(n));
      gp[i] = dG[i].p;
      fp[i] = dF[i].p;
    }
    SL3D_CUDA(dGPtr.Upload(gp));
    SL3D_CUDA(dFPtr.Upload(fp));
    SL3D_CUDA(xPrev.Alloc(n));
    SL3D_CUDA(fPrev.Alloc(n));
    mixerMemory = memory;
  }
  if (gram64.n < static_cast<size_t>(memory) * memory) SL3D_CUDA(gram64.Alloc(static_cast<size_t>(memory) * memory));
  SL3D_CUDA(cudaMemsetAsync(gram64.p, 0, static_cast<size_t>(memory) * memory * sizeof(double), stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::MixerUpdate(int& count, int& slot, bool& first) {
  MixerArgs a{};
  a.n = 2 * spectralComplex;
  a.memory = options.anderson_memory;
  a.x = reinterpret_cast<double*>(s.p);
  a.gx = reinterpret_cast<const double*>(sNext.p);
  a.xPrev = xPrev.p;
  a.fPrev = fPrev.p;
  a.dG = dGPtr.p;
  a.dF = dFPtr.p;
  a.partial = mixPartial.p;
  a.blocks = static_cast<int>(std::min<long long>(kMixBlocks, a.n));
  a.gamma = gammaOut.p;
  if (first) {
    LaunchMixerFirst(a, stream);
    SL3D_CHECK_LAUNCH();
    first = false;
    return SL3DGPU_OK;
  }
  a.slot = slot;
  a.m = std::min(count + 1, a.memory);
  LaunchMixerSweep(a, mixSums.p, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(MixerDeviceSolve(gram64, a.m, a.slot, a.memory));
  LaunchMixerMix(a, stream);
  SL3D_CHECK_LAUNCH();
  count = a.m;
  slot = (slot + 1) % a.memory;
  return SL3DGPU_OK;
}

// SolveElastic + StrainCoefficients into s: the memory force sum_k mu_k m_k,
// the unrelaxed systems, the load channel at the state's time.
int Viscoelastic3DGpu::ElasticStrain(const V3dState& st, const double2* sigma) {
  // the memory force: on the grid at the lateral nodes, analysed; from the
  // coefficients at the others
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  const long long off = p0 * fieldSize, n = static_cast<long long>(count) * fieldSize;
  for (int k = 0; k < K && count > 0; ++k) {
    LaunchCombine(n, fieldSize, muBranch.p + static_cast<long long>(k) * P + p0, k == 0, st.m[k].c0.p + off,
                  st.m[k].c1.p + off, st.m[k].r.p + off, fixedGrid.c0.p + off, fixedGrid.c1.p + off,
                  fixedGrid.r.p + off, stream);
    SL3D_CHECK_LAUNCH();
  }
  if (count > 0 && K == 0) {
    SL3D_CUDA(cudaMemsetAsync(fixedGrid.c0.p + off, 0, n * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(fixedGrid.c1.p + off, 0, n * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(fixedGrid.r.p + off, 0, n * sizeof(double), stream));
  }
  SL3D_TRY(AnalyseRange(fixedGrid, analysedStart.p, p0, count));
  V3dState& mutableSt = const_cast<V3dState&>(st);
  LaunchSpectralSum(SpectralArgs(0, 0.0, st, mutableSt, nullptr, analysedStart.p), stream);
  SL3D_CHECK_LAUNCH();
  return Pass(*elastic, nullptr, true, sigma, tideStart, s.p);
}

// StartStep (Viscoelastic3D.cpp:1223-1378): the stage's flavour, the start
// strain in s, the weights, the decayed memory (into `out`), the lateral
// weight and the fixed force, analysed; the first pass's force in
// analysedStart.
int Viscoelastic3DGpu::StartStage(V3dState& in, V3dState& out, double dt, int scheme, const double2* sigmaStart,
                                  Flavour** flavourOut) {
  Flavour* f = nullptr;
  SL3D_TRY(FlavourOf(scheme, dt, &f));
  *flavourOut = f;
  SL3D_TRY(AdaptState(in));
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  const long long begin = p0 * fieldSize, end = static_cast<long long>(lateralEnd) * fieldSize;
  // The start strain: the cached coefficients, else a consistent unrelaxed
  // solve (a state's grid strain is kept only beside its coefficients).
  if (in.hasCoeffs) {
    SL3D_CUDA(cudaMemcpyAsync(s.p, in.coeffs.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  } else {
    if (ocean.on) SL3D_TRY(StageLoad(ocean.cStart));  // the start's closure under the load at the state's time
    SL3D_TRY(ElasticStrain(in, sigmaStart));
  }
  if (ocean.on) SL3D_TRY(StageLoad(ocean.cEnd));
  // The start strain on the grid, needed at the lateral nodes only.
  const GridTensor* d0 = &in.strain;
  if (!in.hasStrain) {
    SL3D_TRY(SynthesiseRange(s.p, dGrid, p0, count));
    d0 = &dGrid;
  }
  // Weights, decayed memory (into the output state's memory), lateral
  // weight and fixed force; the fixed force analysed once.
  WeightsArgs w{};
  w.branches = K;
  w.scheme = scheme == static_cast<int>(Scheme::BackwardEuler) ? 1 : 0;
  w.dt = dt;
  w.values = values;
  w.begin = begin;
  w.end = end;
  w.fieldSize = fieldSize;
  w.factor = factor.p;
  w.muBranch = muBranch.p;
  w.itauRef = itauRef.p;
  for (int k = 0; k < K; ++k) {
    w.m0[k] = in.m[k].c0.p;
    w.m1[k] = in.m[k].c1.p;
    w.mr[k] = in.m[k].r.p;
    w.out0[k] = out.m[k].c0.p;
    w.out1[k] = out.m[k].c1.p;
    w.outr[k] = out.m[k].r.p;
    w.beta[k] = beta[k].p;
  }
  w.d0c0 = d0->c0.p;
  w.d0c1 = d0->c1.p;
  w.d0r = d0->r.p;
  w.weight = weight.p;
  w.fixed0 = fixedGrid.c0.p;
  w.fixed1 = fixedGrid.c1.p;
  w.fixedr = fixedGrid.r.p;
  LaunchWeights(w, stream);
  SL3D_CHECK_LAUNCH();
  // The fixed force: analysed at the lateral nodes, from the coefficients
  // (decayed in place into the output state) at the others.
  SL3D_TRY(AnalyseRange(fixedGrid, fixedS.p, p0, count));
  LaunchSpectralStart(SpectralArgs(scheme, dt, in, out, s.p, fixedS.p), stream);
  SL3D_CHECK_LAUNCH();
  // The first pass's force from the grid strain in hand: Analyse(W d0) + fixed.
  SL3D_CUDA(cudaMemcpyAsync(analysedStart.p, fixedS.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  SL3D_TRY(AnalyseWeighted(*d0, weight.p, analysedStart.p));
  return SL3DGPU_OK;
}

// Finish (Viscoelastic3D.cpp:1885-1914) for the strain coefficients in s:
// the strain on the grid and the memory advanced at the lateral nodes, the
// coefficients advanced at the others, the state's coefficients cached.
int Viscoelastic3DGpu::FinishStage(V3dState& out, double dt, int scheme) {
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  const long long begin = p0 * fieldSize, end = static_cast<long long>(lateralEnd) * fieldSize;
  SL3D_TRY(SynthesiseRange(s.p, out.strain, p0, count));
  for (int k = 0; k < K && count > 0; ++k) {
    LaunchAdvance(end - begin, beta[k].p + begin, out.strain.c0.p + begin, out.strain.c1.p + begin,
                  out.strain.r.p + begin, out.m[k].c0.p + begin, out.m[k].c1.p + begin, out.m[k].r.p + begin,
                  stream);
    SL3D_CHECK_LAUNCH();
  }
  LaunchSpectralAdvance(SpectralArgs(scheme, dt, out, out, s.p, nullptr), stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaMemcpyAsync(out.coeffs.p, s.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  // a tensor-core contraction that gave up waiting leaves its output
  // unspecified: the step fails rather than return it
  if (grid->emulateFp64) SL3D_TRY(grid->TensorCoreStatus(stream));
  out.hasStrain = out.hasCoeffs = true;
  out.latFirst = lateralFirst;
  out.latEnd = lateralEnd;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::StepOnce(V3dState& in, V3dState& out, double dt, int scheme, const double2* sigmaStart,
                                const double2* sigmaEnd, sl3dgpu_step_info& info) {
  Flavour* f = nullptr;
  SL3D_TRY(StartStage(in, out, dt, scheme, sigmaStart, &f));
  info = sl3dgpu_step_info{};
  if (options.solver == 1) {
    SL3D_TRY(ConvergeConjugateGradients(*f, sigmaEnd, info));
  } else if (options.precision == 1) {
    LaunchCast(values, weight.p, weight32.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_TRY(ConvergeMixed(*f, sigmaEnd, info));
  } else {
    SL3D_TRY(Converge(*f, sigmaEnd, info));
  }
  return FinishStage(out, dt, scheme);
}

// Converge (Viscoelastic3D.cpp:1916-1974): FP64 passes from the start
// strain, plain until the residual ratio exceeds the Anderson rate, mixed
// from then on.
int Viscoelastic3DGpu::Converge(const Flavour& f, const double2* sigmaEnd, sl3dgpu_step_info& info) {
  const bool adaptive = options.anderson_rate > 0.0;
  bool mixing = options.anderson_memory > 0 && !adaptive;
  bool firstMix = true;
  int count = 0, slot = 0;
  if (mixing) SL3D_TRY(MixerReset());
  double previous = 0.0;
  for (int iteration = 0; iteration < options.max_iterations; ++iteration) {
    double residual = 0.0;
    if (iteration == 0) {
      SL3D_TRY(FirstPass(f, sigmaEnd, &residual));
    } else {
      SL3D_TRY(Pass(f, s.p, false, sigmaEnd, tideEnd, sNext.p));
      SL3D_TRY(RelativeChange(sNext.p, s.p, &residual));
    }
    history.push_back(residual);
    info.iterations = iteration + 1;
    info.residual = residual;
    if (!std::isfinite(residual)) break;
    if (residual <= options.rtol) {
      info.converged = 1;
      std::swap(s, sNext);
      break;
    }
    if (options.damping != 1.0) {
      SetError("v3d: damping other than 1 is not built");
      return SL3DGPU_ERR_ARGUMENT;
    }
    if (adaptive && !mixing && options.anderson_memory > 0 && iteration > 0 &&
        residual > options.anderson_rate * previous) {
      mixing = true;
      firstMix = true;
      count = slot = 0;
      SL3D_TRY(MixerReset());
    }
    previous = residual;
    if (mixing) {
      SL3D_TRY(MixerUpdate(count, slot, firstMix));
      ++info.mixed_passes;
    } else {
      std::swap(s, sNext);
    }
  }
  return SL3DGPU_OK;
}

// The mixed form's loop: the same FP64 passes and stopping rule, each FP64
// pass that does not meet the tolerance followed by an FP32 correction.
int Viscoelastic3DGpu::ConvergeMixed(const Flavour& f, const double2* sigmaEnd, sl3dgpu_step_info& info) {
  if (options.damping != 1.0) {
    SetError("v3d: damping other than 1 is not built");
    return SL3DGPU_ERR_ARGUMENT;
  }
  // A guess of the stage's end strain (the caller's, or the extrapolation of
  // warm_start 1) starts the first correction: e = guess - s.
  const double2* warm = stageGuess;
  stageGuess = nullptr;
  for (int iteration = 0; iteration < options.max_iterations; ++iteration) {
    double residual = 0.0;
    SL3D_TRY(Pass(f, s.p, iteration == 0, sigmaEnd, tideEnd, sNext.p));
    SL3D_TRY(RelativeChange(sNext.p, s.p, &residual));
    history.push_back(residual);
    info.iterations = iteration + 1;
    info.residual = residual;
    if (!std::isfinite(residual)) break;
    if (residual <= options.rtol) {
      info.converged = 1;
      std::swap(s, sNext);
      break;
    }
    // r = G(s) - s in FP32, e = B e + r, s += e.
    LaunchResidual32(2 * spectralComplex, reinterpret_cast<const double*>(sNext.p),
                     reinterpret_cast<const double*>(s.p), reinterpret_cast<float*>(r32.p), stream);
    SL3D_CHECK_LAUNCH();
    // The correction needs only the accuracy that brings the next FP64
    // residual under rtol: r' is about (its relative change) x (residual),
    // with a factor 10 to spare, and never finer than correction_rtol.
    SL3D_TRY(Correct(f, std::max(options.correction_rtol, std::min(0.1, 0.1 * options.rtol / residual)), info,
                     warm));
    warm = nullptr;
    SL3D_TRY(grid->TensorCoreStatus(stream));
    LaunchAddCorrection(2 * spectralComplex, reinterpret_cast<const float*>(e32.p), reinterpret_cast<double*>(s.p),
                        stream);
    SL3D_CHECK_LAUNCH();
  }
  return SL3DGPU_OK;
}

// The first pass of a stage: from the plain start (the force of the grid
// strain in hand), and when a warm start is armed for this stage, also from
// the guess; the iteration continues from whichever left the smaller
// relative change (the guess discarded otherwise), its next iterate in sNext.
int Viscoelastic3DGpu::FirstPass(const Flavour& f, const double2* sigmaEnd, double* residual) {
  SL3D_TRY(Pass(f, s.p, true, sigmaEnd, tideEnd, sNext.p));
  double plain = 0.0;
  SL3D_TRY(RelativeChange(sNext.p, s.p, &plain));
  *residual = plain;
  if (stageGuess == nullptr) return SL3DGPU_OK;
  stageGuess = nullptr;
  SL3D_TRY(Pass(f, guess.p, false, sigmaEnd, tideEnd, guessNext.p));
  double tried = 0.0;
  SL3D_TRY(RelativeChange(guessNext.p, guess.p, &tried));
  if (std::isfinite(tried) && tried < plain) {
    std::swap(s, guess);
    std::swap(sNext, guessNext);
    *residual = tried;
    guessTaken = 1;
  } else if (plain <= options.rtol) {
    // the plain start converges at once: its solutions back for Surface
    SL3D_TRY(Pass(f, s.p, true, sigmaEnd, tideEnd, sNext.p));
  }
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::SetStart(const double* coefficients, bool onDevice) {
  if (staticMode || options.solver == 1) {
    SetError("v3d: the warm start applies to the fixed-point step");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (coefficients == nullptr) {
    guessArmed = false;
    return SL3DGPU_OK;
  }
  if (guess.n != static_cast<size_t>(spectralComplex)) {
    SL3D_CUDA(guess.Alloc(spectralComplex));
    SL3D_CUDA(guessNext.Alloc(spectralComplex));
  }
  SL3D_CUDA(cudaMemcpyAsync(guess.p, coefficients, spectralComplex * sizeof(double2),
                            onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  guessArmed = true;
  return SL3DGPU_OK;
}

// Evolution3D::Run with no ocean and no rotation (GRDSolver::NoOceanState,
// RotationalFeedback::None): the direct load is the whole load, so each node
// is one step under the loads at its ends; node 0 is the instantaneous
// (elastic, dt = 0) response to its load (Evolution3D::Instantaneous). Per
// node the surface U and phi coefficients (l, m >= 0) and the step's info.
int Viscoelastic3DGpu::Run(V3dState& st, const double* times, int nodes, int scheme, const double* loads, double* u,
                           double* phi, sl3dgpu_step_info* infos) {
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  for (int k = 0; k < nodes; ++k) {
    const double* l1 = loads + 2 * lm * k;
    const double* l0 = k > 0 ? loads + 2 * lm * (k - 1) : l1;
    const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
    if (!(dt >= 0.0)) {
      SetError("v3d: node times must not decrease");
      return SL3DGPU_ERR_ARGUMENT;
    }
    sl3dgpu_step_info info{};
    SL3D_TRY(Step(st, dt, scheme, l0, l1, &info));
    if (infos) infos[k] = info;
    if (u) SL3D_TRY(Surface(0, u + 2 * lm * k));
    if (phi) SL3D_TRY(Surface(2, phi + 2 * lm * k));
  }
  return SL3DGPU_OK;
}

// -- the ocean closure ---------------------------------------------------------------------------------

namespace {
// out = (1 - c) a + c b over a field
__global__ void BlendFieldKernel(long long n, double c, const double* a, const double* b, double* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = (1.0 - c) * a[i] + c * b[i];
}
// out = ((1 - c) a + c b) - background over a field
__global__ void StageChangeKernel(long long n, double c, const double* a, const double* b, const double* background,
                                  double* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = ((1.0 - c) * a[i] + c * b[i]) - background[i];
}
}  // namespace

// The sea-level body of the operator's Earth in its model units: the
// surface gravity and radius (the sea floor at the surface), water density,
// rotation and moments of inertia (SeaLevelParameters, include/sl3dpp/
// SeaLevel.hpp:54-68, SI on input), G = 1 in the geophysical scales.
int Viscoelastic3DGpu::SetOcean(const sl3dgpu_v3d_ocean* o) {
  if (o == nullptr) {
    ocean.on = false;
    return SL3DGPU_OK;
  }
  if (staticMode || options.solver != 0) {
    SetError("v3d: the ocean closure is built for the fixed point (solver 0), FP64 or mixed");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if ((o->ocean_function == nullptr && !o->migrating) || o->rotation < 0 || o->rotation > 2 ||
      !(o->water_density > 0.0) ||
      !(o->rtol > 0.0) || o->max_iterations < 1 || o->anderson_memory < 0 || o->anderson_memory > 16 ||
      (o->rotation != 0 && (!(o->rotation_frequency > 0.0) || !(o->polar_moment > 0.0) ||
                            !(o->polar_moment != o->equatorial_moment)))) {
    SetError("v3d: an ocean needs its function, rotation 0, 1 or 2 (with a rotation frequency and unequal "
             "moments of inertia), water density > 0, rtol > 0, max_iterations >= 1 and anderson_memory in "
             "[0, 16]");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (o->migrating && (o->ice_thickness == nullptr || o->sea_level == nullptr || !(o->ice_density > 0.0) ||
                       o->max_nonlinear_iterations < 1)) {
    SetError("v3d: migrating shorelines need the background's ice thickness and sea level, an ice density > 0 and "
             "max_nonlinear_iterations >= 1");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (ocean.grid == nullptr) {
    SL3D_TRY(sl3dgpu_grid_create(options.lmax, 0, 1.0, &ocean.grid));
    ocean.ws = NewSleWorkspace();
  }
  int nt = 0, np = 0;
  SL3D_TRY(sl3dgpu_grid_shape(ocean.grid, &nt, &np));
  ocean.fieldSize = static_cast<long long>(nt) * np;
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  const auto& scales = earth->scales();
  ocean.migrating = o->migrating != 0;
  if (ocean.migrating) {
    // the background state, its ocean function by flotation
    // (CheckMigratingStart, src/Shorelines.cpp:9-35: a prescribed one must
    // be flotation's)
    const size_t n = static_cast<size_t>(ocean.fieldSize);
    SL3D_CUDA(ocean.ice.Upload(std::vector<double>(o->ice_thickness, o->ice_thickness + n)));
    SL3D_CUDA(ocean.seaLevel.Upload(std::vector<double>(o->sea_level, o->sea_level + n)));
    ocean.hasLand = o->forced_land != nullptr;
    if (ocean.hasLand)
      SL3D_CUDA(ocean.land.Upload(std::vector<unsigned char>(o->forced_land, o->forced_land + n)));
    ocean.iceDensity = o->ice_density / scales.Density();
    ocean.maxNonlinear = o->max_nonlinear_iterations;
    SL3D_CUDA(ocean.function.Alloc(n));
    SL3D_TRY(Flotation(ocean.fieldSize, o->water_density / scales.Density(), ocean.iceDensity, ocean.ice.p,
                       ocean.seaLevel.p, ocean.hasLand ? ocean.land.p : nullptr, ocean.function.p, stream));
    if (o->ocean_function != nullptr) {
      std::vector<double> got(n);
      SL3D_CUDA(cudaMemcpyAsync(got.data(), ocean.function.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
      SL3D_CUDA(cudaStreamSynchronize(stream));
      for (size_t i = 0; i < n; ++i)
        if (got[i] != o->ocean_function[i]) {
          SetError("v3d: migrating shorelines follow the flotation condition from the first node, so the "
                   "background state must not prescribe its ocean function");
          return SL3DGPU_ERR_ARGUMENT;
        }
    }
    for (auto* d : {&ocean.ice0, &ocean.ice1, &ocean.stageIceChange, &ocean.current}) SL3D_CUDA(d->Alloc(n));
    SL3D_CUDA(cudaMemcpyAsync(ocean.current.p, ocean.function.p, n * sizeof(double), cudaMemcpyDeviceToDevice,
                              stream));
    SL3D_CUDA(cudaMemcpyAsync(ocean.ice0.p, ocean.ice.p, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    SL3D_CUDA(cudaMemcpyAsync(ocean.ice1.p, ocean.ice.p, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  } else {
    std::vector<double> function(o->ocean_function, o->ocean_function + ocean.fieldSize);
    SL3D_CUDA(ocean.function.Upload(function));
  }
  for (auto* d : {&ocean.load0, &ocean.load1, &ocean.stageLoad, &ocean.slc}) SL3D_CUDA(d->Alloc(ocean.fieldSize));
  for (auto* d : {&ocean.U, &ocean.V, &ocean.Phi, &ocean.sigma, &ocean.psi}) SL3D_CUDA(d->Alloc(lm));
  SL3D_CUDA(ZeroIn(ocean.psi.p, lm * sizeof(double2)));
  SL3D_CUDA(ZeroIn(ocean.load0.p, ocean.fieldSize * sizeof(double)));
  SL3D_CUDA(ZeroIn(ocean.load1.p, ocean.fieldSize * sizeof(double)));
  ocean.hasLoads = false;
  const auto& sc = scales;
  sl3dgpu_sle_body& b = ocean.body;
  b = sl3dgpu_sle_body{};
  b.g = material->surfaceGravity;
  b.radius = material->radius;
  b.water_density = o->water_density / sc.Density();
  b.rotation = o->rotation;
  b.omega = o->rotation_frequency * sc.time;
  b.polar_moment = o->polar_moment / sc.Factor(1, 2, 0);
  b.equatorial_moment = o->equatorial_moment / sc.Factor(1, 2, 0);
  b.gravitational_constant = material->G;
  ocean.rtol = o->rtol;
  ocean.maxIterations = o->max_iterations;
  ocean.memory = o->anderson_memory;
  ocean.solved = false;
  ocean.on = true;
  return SL3DGPU_OK;
}

// The running stage's direct load: (1 - c) of the step's start load and c of its end's.
int Viscoelastic3DGpu::StageLoad(double c) {
  const unsigned blocks = static_cast<unsigned>((ocean.fieldSize + 255) / 256);
  BlendFieldKernel<<<blocks, 256, 0, stream>>>(ocean.fieldSize, c, ocean.load0.p, ocean.load1.p, ocean.stageLoad.p);
  SL3D_CHECK_LAUNCH();
  if (ocean.migrating) {
    // the stage's ice less the background's (src/Evolution3D.cpp:717-722)
    StageChangeKernel<<<blocks, 256, 0, stream>>>(ocean.fieldSize, c, ocean.ice0.p, ocean.ice1.p, ocean.ice.p,
                                                  ocean.stageIceChange.p);
    SL3D_CHECK_LAUNCH();
  }
  return SL3DGPU_OK;
}

// A flavour's effective Love numbers (ComputeLoveNumbers, src/LoveNumbers.cpp:
// 92-176, on the flavour's solid): the surface U, V and phi of its unit
// channels K^-1 Load and K^-1 Tide per degree, degree 0's centrifugal column
// for h_c, k_c, and the inertia moments of degree 0's load and centrifugal
// solutions (the moment row of InertiaMoment).
int Viscoelastic3DGpu::EffectiveLove(const Flavour& f, const std::vector<double>** out) {
  Flavour& mf = const_cast<Flavour&>(f);
  if (mf.effectiveLove.empty()) {
    const int L = options.lmax;
    std::vector<double> units(f.units.n), tides(f.tideUnits.n);
    std::vector<long long> offset(L + 1);
    SL3D_CUDA(cudaMemcpyAsync(units.data(), f.units.p, units.size() * sizeof(double), cudaMemcpyDeviceToHost,
                              stream));
    SL3D_CUDA(cudaMemcpyAsync(tides.data(), f.tideUnits.p, tides.size() * sizeof(double), cudaMemcpyDeviceToHost,
                              stream));
    SL3D_CUDA(cudaMemcpyAsync(offset.data(), f.unitOffset.p, offset.size() * sizeof(long long),
                              cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    std::vector<double> love(6 * (L + 1) + 4, 0.0);
    auto at = [&](const std::vector<double>& v, int l, int dof) { return dof >= 0 ? v[offset[l] + dof] : 0.0; };
    for (int l = 0; l <= L; ++l) {
      const DegreeInfo& d = degrees[l];
      love[l] = at(units, l, d.surfaceU);
      love[(L + 1) + l] = at(units, l, d.surfacePhi);
      love[2 * (L + 1) + l] = l >= 1 ? at(units, l, d.surfaceV) : 0.0;
      if (l >= 2) {  // the tidal numbers from degree 2 (degree 0 carries the centrifugal column)
        love[3 * (L + 1) + l] = at(tides, l, d.surfaceU);
        love[4 * (L + 1) + l] = at(tides, l, d.surfacePhi);
        love[5 * (L + 1) + l] = at(tides, l, d.surfaceV);
      }
    }
    double m = 0.0, mc = 0.0;
    for (int dof = 0; dof < degrees[0].sphNdof; ++dof) {
      m += momentRow[dof] * units[offset[0] + dof];
      mc += momentRow[dof] * tides[offset[0] + dof];
    }
    love[6 * (L + 1)] = at(tides, 0, degrees[0].surfaceU);
    love[6 * (L + 1) + 1] = at(tides, 0, degrees[0].surfacePhi);
    love[6 * (L + 1) + 2] = m;
    love[6 * (L + 1) + 3] = mc;
    mf.effectiveLove = std::move(love);
  }
  *out = &mf.effectiveLove;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::EffectiveLoveOf(int scheme, double dt, const std::vector<double>** out) {
  Flavour* f = nullptr;
  SL3D_TRY(FlavourOf(scheme, dt, &f));
  return EffectiveLove(*f, out);
}

// Closure (src/Evolution3D.cpp:296-339, frozen shorelines): the surface
// responses of the pass's degree solves and their inertia moment close the
// sea-level equation on the flavour's effective numbers under the stage's
// direct load; its total load and the centrifugal potential of its angular
// velocity are the pass's load and tide channels.
int Viscoelastic3DGpu::Closure(const Flavour& f) {
  const std::vector<double>* love = nullptr;
  SL3D_TRY(EffectiveLove(f, &love));
  const int L = options.lmax;
  LaunchSurface(geo, rhsSph.p, rhsTor.p, 0, ocean.U.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchSurface(geo, rhsSph.p, rhsTor.p, 1, ocean.V.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchSurface(geo, rhsSph.p, rhsTor.p, 2, ocean.Phi.p, stream);
  SL3D_CHECK_LAUNCH();
  double moment = 0.0;
  SL3D_TRY(InertiaMoment(&moment));
  sl3dgpu_sle_body b = ocean.body;
  const double* v = love->data();
  b.h = v;
  b.k = v + (L + 1);
  b.l = v + 2 * (L + 1);
  b.ht = v + 3 * (L + 1);
  b.kt = v + 4 * (L + 1);
  b.lt = v + 5 * (L + 1);
  b.hc = v[6 * (L + 1)];
  b.kc = v[6 * (L + 1) + 1];
  b.m_u = v[6 * (L + 1) + 2];  // the load's whole trace number (no displacement or potential load channel)
  b.m_phi = 0.0;
  b.m_c = v[6 * (L + 1) + 3];
  if (ocean.migrating) {
    // the nonlinear equation from the background under the stage's ice
    // change (and direct load, where given), the responses as ready channels
    const sl3dgpu_sle_state state{ocean.ice.p, ocean.seaLevel.p, ocean.function.p,
                                  ocean.hasLand ? ocean.land.p : nullptr};
    sl3dgpu_sle_nonlinear_forcing moving{};
    moving.ice_thickness_change = ocean.stageIceChange.p;
    moving.direct_load = ocean.hasLoads ? ocean.stageLoad.p : nullptr;
    moving.displacement_response = reinterpret_cast<const double*>(ocean.U.p);
    moving.potential_response = reinterpret_cast<const double*>(ocean.Phi.p);
    moving.tangential_response = reinterpret_cast<const double*>(ocean.V.p);
    moving.inertia_moment_change = moment;
    SL3D_TRY(SeaLevelSolveNonlinear(*ocean.ws, ocean.grid, &b, ocean.iceDensity, &state, &moving, ocean.rtol,
                                    ocean.maxNonlinear, ocean.slc.p, nullptr, nullptr, nullptr, nullptr, nullptr,
                                    ocean.current.p, reinterpret_cast<double*>(ocean.sigma.p), &ocean.last,
                                    stream));
  } else {
    sl3dgpu_sle_forcing forcing{};
    forcing.direct_load = ocean.stageLoad.p;
    forcing.displacement_response = reinterpret_cast<const double*>(ocean.U.p);
    forcing.potential_response = reinterpret_cast<const double*>(ocean.Phi.p);
    forcing.tangential_response = reinterpret_cast<const double*>(ocean.V.p);
    forcing.inertia_moment_change = moment;
    SL3D_TRY(SeaLevelSolve(*ocean.ws, ocean.grid, &b, ocean.function.p, &forcing, ocean.rtol, ocean.maxIterations,
                           ocean.memory, ocean.slc.p, nullptr, nullptr, nullptr, nullptr,
                           reinterpret_cast<double*>(ocean.sigma.p), &ocean.last, stream));
  }
  double psi[6];
  SL3D_TRY(CentrifugalCoefficients(b, ocean.last.angular_velocity, psi));
  // (0, 0) at 0, (2, 0) at 3, (2, 1) at 4 of the l(l+1)/2 + m layout
  if (b.rotation != 0) {
    SL3D_CUDA(cudaMemcpyAsync(ocean.psi.p, psi, sizeof(double2), cudaMemcpyHostToDevice, stream));
    SL3D_CUDA(cudaMemcpyAsync(ocean.psi.p + 3, psi + 2, 2 * sizeof(double2), cudaMemcpyHostToDevice, stream));
  }
  ocean.solved = true;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::StepOcean(V3dState& st, double dt, int scheme, const double* load0, const double* load1,
                                 sl3dgpu_step_info* info) {
  if (!ocean.on) {
    SetError("v3d: no ocean is set (sl3dgpu_v3d_set_ocean)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (ocean.migrating) {
    SetError("v3d: the ocean's shorelines migrate: its steps take the ice (sl3dgpu_v3d_step_migrating)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const size_t bytes = ocean.fieldSize * sizeof(double);
  if (load0) SL3D_CUDA(cudaMemcpyAsync(ocean.load0.p, load0, bytes, cudaMemcpyHostToDevice, stream));
  else SL3D_CUDA(cudaMemsetAsync(ocean.load0.p, 0, bytes, stream));
  if (load1) SL3D_CUDA(cudaMemcpyAsync(ocean.load1.p, load1, bytes, cudaMemcpyHostToDevice, stream));
  else SL3D_CUDA(cudaMemsetAsync(ocean.load1.p, 0, bytes, stream));
  return Step(st, dt, scheme, nullptr, nullptr, info);
}

// Evolution3D::March for frozen shorelines (src/Evolution3D.cpp:521-821):
// node 0 the instantaneous response closed by the sea-level equation (a
// zero-length step), then one step per node, each pass closed.
int Viscoelastic3DGpu::RunOcean(V3dState& st, const double* times, int nodes, int scheme, const double* loads,
                                double* u, double* phi, double* slc, double* omega, sl3dgpu_step_info* infos) {
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  for (int k = 0; k < nodes; ++k) {
    const double* l1 = loads + ocean.fieldSize * k;
    const double* l0 = k > 0 ? loads + ocean.fieldSize * (k - 1) : l1;
    const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
    if (!(dt >= 0.0)) {
      SetError("v3d: node times must not decrease");
      return SL3DGPU_ERR_ARGUMENT;
    }
    sl3dgpu_step_info info{};
    SL3D_TRY(StepOcean(st, dt, scheme, l0, l1, &info));
    if (infos) infos[k] = info;
    if (u) SL3D_TRY(Surface(0, u + 2 * lm * k));
    if (phi) SL3D_TRY(Surface(2, phi + 2 * lm * k));
    if (slc || omega)
      SL3D_TRY(SeaLevel(slc ? slc + 2 * lm * k : nullptr, omega ? omega + 3 * k : nullptr, nullptr));
  }
  return SL3DGPU_OK;
}

// The last closure's relative sea level change as (l, m >= 0) coefficients
// (host), its angular velocity and its solve's scalars.
int Viscoelastic3DGpu::SeaLevel(double* coefficients, double* omega, sl3dgpu_sle_result* result) {
  if (!ocean.on || !ocean.solved) {
    SetError("v3d: no sea-level closure has run (an ocean and a step)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (coefficients) {
    const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
    SL3D_TRY(sl3dgpu_expand_batch(ocean.grid, ocean.slc.p, 1, reinterpret_cast<double*>(ocean.U.p), stream));
    SL3D_CUDA(cudaMemcpyAsync(coefficients, ocean.U.p, lm * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
  }
  if (omega)
    for (int i = 0; i < 3; ++i) omega[i] = ocean.last.angular_velocity[i];
  if (result) *result = ocean.last;
  return SL3DGPU_OK;
}

// One coupled step under migrating shorelines: the ice thickness at the
// step's two ends (host fields, model length), the direct loads beside it
// (NULL: none); the stages take their combinations (detail::AtStage).
int Viscoelastic3DGpu::StepMigrating(V3dState& st, double dt, int scheme, const double* ice0, const double* ice1,
                                     const double* load0, const double* load1, sl3dgpu_step_info* info) {
  if (!ocean.on || !ocean.migrating) {
    SetError("v3d: no ocean with migrating shorelines is set (sl3dgpu_v3d_set_ocean, migrating = 1)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (ice0 == nullptr || ice1 == nullptr) {
    SetError("v3d: a migrating step needs the ice thickness at both its ends");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const size_t bytes = ocean.fieldSize * sizeof(double);
  SL3D_CUDA(cudaMemcpyAsync(ocean.ice0.p, ice0, bytes, cudaMemcpyHostToDevice, stream));
  SL3D_CUDA(cudaMemcpyAsync(ocean.ice1.p, ice1, bytes, cudaMemcpyHostToDevice, stream));
  ocean.hasLoads = load0 != nullptr || load1 != nullptr;
  if (load0) SL3D_CUDA(cudaMemcpyAsync(ocean.load0.p, load0, bytes, cudaMemcpyHostToDevice, stream));
  else SL3D_CUDA(cudaMemsetAsync(ocean.load0.p, 0, bytes, stream));
  if (load1) SL3D_CUDA(cudaMemcpyAsync(ocean.load1.p, load1, bytes, cudaMemcpyHostToDevice, stream));
  else SL3D_CUDA(cudaMemsetAsync(ocean.load1.p, 0, bytes, stream));
  return Step(st, dt, scheme, nullptr, nullptr, info);
}

// Evolution3D::RunMigrating (src/Evolution3D.cpp:117-133, March :540-821):
// node 0 undisturbed at the background (its ice must be the history's
// first, CheckMigratingStart) or, with direct loads, the start's solve (a
// zero-length step, :690-700); then a step per node, every pass closed by the
// nonlinear equation. ice: nodes x field; loads: nodes x field or NULL;
// oceans (nullable): nodes x field, each node's ocean function.
int Viscoelastic3DGpu::RunMigrating(V3dState& st, const double* times, int nodes, int scheme, const double* ice,
                                    const double* loads, double* u, double* phi, double* slc, double* omega,
                                    double* oceans, sl3dgpu_step_info* infos) {
  if (!ocean.on || !ocean.migrating) {
    SetError("v3d: no ocean with migrating shorelines is set (sl3dgpu_v3d_set_ocean, migrating = 1)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  const long long n = ocean.fieldSize;
  for (int k = 0; k < nodes; ++k) {
    const double* i1 = ice + n * k;
    const double* i0 = k > 0 ? ice + n * (k - 1) : i1;
    const double* l1 = loads ? loads + n * k : nullptr;
    const double* l0 = loads ? (k > 0 ? loads + n * (k - 1) : l1) : nullptr;
    const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
    if (!(dt >= 0.0)) {
      SetError("v3d: node times must not decrease");
      return SL3DGPU_ERR_ARGUMENT;
    }
    sl3dgpu_step_info info{};
    info.converged = 1;
    if (k == 0 && loads == nullptr) {
      // the background is the state at the first node: undisturbed
      std::vector<double> background(n);
      SL3D_CUDA(cudaMemcpyAsync(background.data(), ocean.ice.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
      SL3D_CUDA(cudaStreamSynchronize(stream));
      double scale = 0.0, worst = 0.0;
      for (long long i = 0; i < n; ++i) {
        scale = std::max(scale, std::abs(i1[i]));
        worst = std::max(worst, std::abs(background[i] - i1[i]));
      }
      if (worst > 1e-6 * scale) {
        SetError("v3d: the background state's ice thickness is not the history's at the first node; build the "
                 "state at times[0]");
        return SL3DGPU_ERR_ARGUMENT;
      }
      SL3D_CUDA(cudaMemcpyAsync(ocean.current.p, ocean.function.p, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                stream));
      SL3D_CUDA(cudaMemsetAsync(ocean.sigma.p, 0, lm * sizeof(double2), stream));
      SL3D_CUDA(cudaMemsetAsync(ocean.psi.p, 0, lm * sizeof(double2), stream));
      if (u) std::fill(u, u + 2 * lm, 0.0);
      if (phi) std::fill(phi, phi + 2 * lm, 0.0);
      if (slc) std::fill(slc, slc + 2 * lm, 0.0);
      if (omega) std::fill(omega, omega + 3, 0.0);
      if (oceans) SL3D_TRY(OceanFunction(oceans));
      if (infos) infos[0] = info;
      continue;
    }
    SL3D_TRY(StepMigrating(st, dt, scheme, i0, i1, l0, l1, &info));
    if (infos) infos[k] = info;
    if (u) SL3D_TRY(Surface(0, u + 2 * lm * k));
    if (phi) SL3D_TRY(Surface(2, phi + 2 * lm * k));
    if (slc || omega)
      SL3D_TRY(SeaLevel(slc ? slc + 2 * lm * k : nullptr, omega ? omega + 3 * k : nullptr, nullptr));
    if (oceans) SL3D_TRY(OceanFunction(oceans + n * k));
  }
  return SL3DGPU_OK;
}

// The ocean function of the last closure (migrating shorelines; the fixed
// one otherwise), a host field on the sea-level grid.
int Viscoelastic3DGpu::OceanFunction(double* out) {
  if (!ocean.on) {
    SetError("v3d: no ocean is set (sl3dgpu_v3d_set_ocean)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const double* src = ocean.migrating ? ocean.current.p : ocean.function.p;
  SL3D_CUDA(cudaMemcpyAsync(out, src, ocean.fieldSize * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// -- the mixed form's FP32 correction ---------------------------------------------------------------

// The correction's view of the lateral nodes: the geometry with the nodes
// [lateralFirst, lateralEnd) renumbered from 0 (whole elements), and the
// compact buffers, rebuilt when the range moves.
int Viscoelastic3DGpu::PrepareLateral() {
  if (geoLFirst == lateralFirst && geoLEnd == lateralEnd) return SL3DGPU_OK;
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  std::vector<int> efn(elemFirstNode.size(), -1);
  for (size_t e = 0; e < elemFirstNode.size(); ++e) {
    const int fn = elemFirstNode[e];
    if (fn >= p0 && fn < lateralEnd) efn[e] = fn - p0;
  }
  // The global nodes of the lateral elements; each degree's force and
  // strain stay within them, and so do the rows its forces reach.
  const int n = geo.ngll;
  const int g0 = count > 0 ? nodeElement[p0] * (n - 1) : 0;
  const int g1 = count > 0 ? nodeElement[lateralEnd - 1] * (n - 1) + n - 1 : -1;
  std::vector<DegreeInfo> dl = degrees;
  sphWindow.assign(degrees.size(), make_int2(1 << 30, -1));
  torWindow.assign(degrees.size(), make_int2(1 << 30, -1));
  for (size_t l = 0; l < dl.size(); ++l) {
    auto& d = dl[l];
    d.firstNode = std::min(std::max(d.firstNode - p0, 0), count);
    d.firstGlobal = std::max(d.firstGlobal, g0);
    d.lastGlobal = std::min(d.lastGlobal, g1);
    if (d.firstNode >= count || d.firstGlobal > d.lastGlobal) {
      d.firstNode = count;
      d.firstGlobal = 0;
      d.lastGlobal = -1;
      continue;
    }
    auto widen = [](int2& w, int dof) {
      if (dof < 0) return;
      w.x = std::min(w.x, dof);
      w.y = std::max(w.y, dof);
    };
    for (int gn = d.firstGlobal; gn <= d.lastGlobal; ++gn) {
      widen(sphWindow[l], hostSphMap[d.sphMap + 2LL * gn]);
      widen(sphWindow[l], hostSphMap[d.sphMap + 2LL * gn + 1]);
      if (l >= 1) widen(torWindow[l], hostTorMap[d.torMap + gn]);
    }
  }
  SL3D_CUDA(dElemFirstNodeL.Upload(efn));
  SL3D_CUDA(dDegreesL.Upload(dl));
  geoL = geo;
  geoL.P = count;
  geoL.nodeElement = dNodeElement.p + p0;
  geoL.nodeQ = dNodeQ.p + p0;
  geoL.nodeR = dNodeR.p + p0;
  for (int w = 0; w < 4; ++w) {
    geoL.coef64[w] = geo.coef64[w] + static_cast<long long>(p0) * geo.ngll;
    geoL.coef32[w] = geo.coef32[w] + static_cast<long long>(p0) * geo.ngll;
  }
  geoL.elemFirstNode = dElemFirstNodeL.p;
  geoL.degrees = dDegreesL.p;
  geoL.maxGlobals = 0;
  for (const auto& d : dl) geoL.maxGlobals = std::max(geoL.maxGlobals, d.lastGlobal - d.firstGlobal + 1);
  compactComplex = (rows0 + rows1 + rowsR) * count;
  for (auto* b : {&eL, &eNextL, &rL, &analysedL}) SL3D_CUDA(b->Alloc(std::max<long long>(compactComplex, 1)));
  geoLFirst = lateralFirst;
  geoLEnd = lateralEnd;
  return SL3DGPU_OK;
}

// Analyse(W Synthesise(e)) of a compact lateral iterate into a compact
// lateral force.
int Viscoelastic3DGpu::WeightedPass32(const float2* strain, float2* out) {
  const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
  if (count <= 0) return SL3DGPU_OK;
  const auto* in = reinterpret_cast<const float*>(strain);
  auto* o = reinterpret_cast<float*>(out);
  const float* w = weight32.p + p0 * fieldSize;
  const long long offs[3] = {0, 2 * rows0 * count, 2 * (rows0 + rows1) * count};
  const int spins[3] = {-2, -1, 0};
  for (int c = 0; c < 3; ++c) {
    const bool real = c == 2;
    SL3D_TRY(grid->LegendreSynthesisF(spins[c], real, in + offs[c], count, 0, count, spectra32A.p, stream));
    SL3D_TRY(grid->RingWeightedF(real, spectra32A.p, count, w, spectra32B.p, stream));
    SL3D_TRY(grid->LegendreAnalysisF(spins[c], real, spectra32B.p, count, 0, count, o + offs[c], false, stream));
  }
  return SL3DGPU_OK;
}

// The flavour's per-system row windows for the current lateral range: a
// Cholesky system's from its degree (its right-hand sides are the degree's
// 2 (l + 1) real columns), an LU system's every row (solved whole).
int Viscoelastic3DGpu::SolveWindows(const Flavour& f) {
  if (f.windowFirst == geoLFirst && f.windowEnd == geoLEnd) return SL3DGPU_OK;
  auto build = [](const std::vector<sl3dgpu_band_system>& systems, const std::vector<int2>* perDegree,
                  Dev<int2>& out) -> int {
    std::vector<int2> w;
    w.reserve(systems.size());
    for (const auto& s : systems) {
      const int l = s.nrhs / 2 - 1;
      w.push_back(perDegree ? (*perDegree)[l] : make_int2(0, s.n - 1));
    }
    SL3D_CUDA(out.Upload(w));
    return SL3DGPU_OK;
  };
  SL3D_TRY(build(f.sphChol, &sphWindow, f.wSphChol));
  SL3D_TRY(build(f.sphLu, nullptr, f.wSphLu));
  SL3D_TRY(build(f.torChol, &torWindow, f.wTorChol));
  f.windowFirst = geoLFirst;
  f.windowEnd = geoLEnd;
  return SL3DGPU_OK;
}

// next = B e + r on the lateral nodes: the lateral force of e alone through
// the FP32 solves. The forces reach only the lateral rows of each system, so
// the substitutions run over those rows and above (row windows); their
// solutions are complete from the lowest lateral row up, and the end of
// Correct finishes the rows below for the last pass.
int Viscoelastic3DGpu::Pass32(const Flavour& f, const float2* e, float2* next) {
  SL3D_TRY(WeightedPass32(e, analysedL.p));
  SL3D_TRY(SolveWindows(f));
  auto* sph = reinterpret_cast<float*>(rhsSph32.p);
  auto* tor = reinterpret_cast<float*>(rhsTor32.p);
  LaunchZeroRows(f.dSphChol.p, f.wSphChol.p, static_cast<int>(f.sphChol.size()), sph, f.dSphLu.p, f.wSphLu.p,
                 static_cast<int>(f.sphLu.size()), sph, f.dTorChol.p, f.wTorChol.p,
                 static_cast<int>(f.torChol.size()), tor, stream);
  SL3D_CHECK_LAUNCH();
  LaunchForces(geoL, analysedL.p, rhsSph32.p, rhsTor32.p, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(BandSolveWindowF(f.dSphChol.p, f.sphChol.data(), static_cast<int>(f.sphChol.size()), f.iSphChol.p,
                            f.nSphChol, f.bands32.p, sph, f.scales32.p, f.wSphChol.p, false, stream));
  SL3D_TRY(BandSolveBatchF(f.dSphLu.p, f.sphLu.data(), static_cast<int>(f.sphLu.size()), f.iSphLu.p, f.nSphLu,
                           f.bands32.p, f.pivots.p, sph, f.scales32.p, 1, stream));
  SL3D_TRY(BandSolveWindowF(f.dTorChol.p, f.torChol.data(), static_cast<int>(f.torChol.size()), f.iTorChol.p,
                            f.nTorChol, f.bands32.p, tor, f.scales32.p, f.wTorChol.p, false, stream));
  LaunchStrain(geoL, rhsSph32.p, rhsTor32.p, next, stream, rL.p);  // B e + r
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::Mixer32Reset() {
  const int memory = CorrectionMemory();
  if (memory <= 0) return SL3DGPU_OK;
  const size_t n = 2 * compactComplex;
  if (mixer32Memory != memory || mixer32Size != n) {
    dG32.resize(memory);
    dF32.resize(memory);
    std::vector<__nv_bfloat16*> gp(memory), fp(memory);
    for (int i = 0; i < memory; ++i) {
      SL3D_CUDA(dG32[i].Alloc(n));
      SL3D_CUDA(dF32[i].Alloc(n));
      gp[i] = dG32[i].p;
      fp[i] = dF32[i].p;
    }
    SL3D_CUDA(dG32Ptr.Upload(gp));
    SL3D_CUDA(dF32Ptr.Upload(fp));
    SL3D_CUDA(xPrev32.Alloc(n));
    SL3D_CUDA(fPrev32.Alloc(n));
    mixer32Memory = memory;
    mixer32Size = n;
  }
  if (gram32.n < static_cast<size_t>(memory) * memory) SL3D_CUDA(gram32.Alloc(static_cast<size_t>(memory) * memory));
  SL3D_CUDA(cudaMemsetAsync(gram32.p, 0, static_cast<size_t>(memory) * memory * sizeof(double), stream));
  return SL3DGPU_OK;
}

// An update's least squares on the device: the sweep's sums, the Gram
// column and gamma by one FP64 warp (LaunchMixerGram), ordered on the
// stream before the mix -- no host round trip.
int Viscoelastic3DGpu::MixerDeviceSolve(Dev<double>& gram, int m, int slot, int memory) {
  LaunchMixerGram(gram.p, m, slot, memory, mixSums.p, gammaOut.p, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::Mixer32Update(int& count, int& slot, bool& first) {
  MixerArgsT<float> a{};
  a.n = 2 * compactComplex;
  a.memory = CorrectionMemory();
  a.x = reinterpret_cast<float*>(eL.p);
  a.gx = reinterpret_cast<const float*>(eNextL.p);
  a.xPrev = xPrev32.p;
  a.fPrev = fPrev32.p;
  a.dG = dG32Ptr.p;
  a.dF = dF32Ptr.p;
  a.partial = mixPartial.p;
  a.blocks = static_cast<int>(std::min<long long>(kMixBlocks32, a.n));
  a.gamma = gammaOut.p;
  if (first) {
    LaunchMixerFirst(a, stream);
    SL3D_CHECK_LAUNCH();
    first = false;
    return SL3DGPU_OK;
  }
  a.slot = slot;
  a.m = std::min(count + 1, a.memory);
  LaunchMixerSweep(a, mixSums.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchMixerGram(gram32.p, a.m, a.slot, a.memory, mixSums.p, gammaOut.p, stream, nullptr, true);
  SL3D_CHECK_LAUNCH();
  LaunchMixerMix(a, stream);
  SL3D_CHECK_LAUNCH();
  count = a.m;
  slot = (slot + 1) % a.memory;
  return SL3DGPU_OK;
}

// e = B e + r from e = r, with the FP64 loop's Anderson schedule, until the
// relative change is at most the tolerance (or max_iterations passes). B
// reads e at the lateral nodes only, so the iteration runs on their compact
// columns; e at every node is B e + r of the last pass's solutions, left in
// e32 for s += e.
// What a captured correction loop depends on: the flavour, the lateral
// range, the mixer's memory and every buffer its kernels were given.
std::vector<long long> Viscoelastic3DGpu::CorrectionKey(const Flavour& f) const {
  auto at = [](const void* p) { return static_cast<long long>(reinterpret_cast<uintptr_t>(p)); };
  return {f.id, f.windowFirst, f.windowEnd, lateralFirst, lateralEnd, compactComplex, CorrectionMemory(),
          mixer32Memory, at(eL.p), at(eNextL.p), at(rL.p), at(analysedL.p), at(rhsSph32.p), at(rhsTor32.p),
          at(spectra32A.p), at(spectra32B.p), at(weight32.p), at(xPrev32.p), at(fPrev32.p), at(dG32Ptr.p),
          at(dF32Ptr.p), at(gram32.p), at(mixPartial.p), at(mixSums.p), at(gammaOut.p), at(changePartial.p),
          at(changeResult.p), at(correctionControl.p), at(dDegreesL.p), at(dElemFirstNodeL.p),
          at(f.wSphChol.p), at(f.wSphLu.p), at(f.wTorChol.p)};
}

// One pass of the loop and its decision, enqueued on the capturing stream.
int Viscoelastic3DGpu::CaptureCorrectionBody(const Flavour& f, cudaGraphConditionalHandle handle) {
  SL3D_TRY(Pass32(f, eL.p, eNextL.p));
  LaunchRelativeChange(reinterpret_cast<const float*>(eNextL.p), reinterpret_cast<const float*>(eL.p),
                       2 * compactComplex, changePartial.p, kChangeBlocks, changeResult.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchCorrectionControl(correctionControl.p, changeResult.p, handle, stream);
  SL3D_CHECK_LAUNCH();
  LaunchCopyIfPlain(correctionControl.p, eNextL.p, eL.p, compactComplex, stream);
  SL3D_CHECK_LAUNCH();
  const int memory = CorrectionMemory();
  if (memory <= 0) return SL3DGPU_OK;
  LaunchGramResetIf(correctionControl.p, gram32.p, memory, stream);
  SL3D_CHECK_LAUNCH();
  MixerArgsT<float> a{};
  a.n = 2 * compactComplex;
  a.memory = memory;
  a.m = memory;  // the kernels' instance; the runtime m comes from the control
  a.slot = 0;
  a.x = reinterpret_cast<float*>(eL.p);
  a.gx = reinterpret_cast<const float*>(eNextL.p);
  a.xPrev = xPrev32.p;
  a.fPrev = fPrev32.p;
  a.dG = dG32Ptr.p;
  a.dF = dF32Ptr.p;
  a.partial = mixPartial.p;
  a.blocks = static_cast<int>(std::min<long long>(kMixBlocks32, a.n));
  a.gamma = gammaOut.p;
  a.live = reinterpret_cast<const int*>(correctionControl.p);
  LaunchMixerFirst(a, stream);
  SL3D_CHECK_LAUNCH();
  LaunchMixerSweep(a, mixSums.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchMixerGram(gram32.p, memory, 0, memory, mixSums.p, gammaOut.p, stream, a.live, true);
  SL3D_CHECK_LAUNCH();
  LaunchMixerMix(a, stream);
  SL3D_CHECK_LAUNCH();
  LaunchMixerAdvanceIf(correctionControl.p, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// The loop's graph for the flavour: found by key, else captured (a while
// node whose body is one pass and its decision) and instantiated.
int Viscoelastic3DGpu::CorrectionGraphFor(const Flavour& f, CorrectionGraph** out) {
  if (CorrectionMemory() > kMixMaxMemory) return SL3DGPU_ERR_ARGUMENT;
  if (correctionControl.n == 0) SL3D_CUDA(correctionControl.Alloc(1));
  if (CorrectionMemory() > 0 && (mixer32Memory != CorrectionMemory() || mixer32Size != 2 * compactComplex))
    SL3D_TRY(Mixer32Reset());  // the history buffers the graph will hold
  const auto key = CorrectionKey(f);
  for (auto& g : correctionGraphs)
    if (g.key == key) {
      *out = &g;
      return SL3DGPU_OK;
    }
  cudaGraph_t graph = nullptr;
  SL3D_CUDA(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle handle;
  cudaGraphNodeParams params{};
  cudaGraphNode_t node;
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;
  auto fail = [&](int status) {
    cudaGraphDestroy(graph);
    cudaGetLastError();
    return status;
  };
  if (cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault) != cudaSuccess)
    return fail(SL3DGPU_ERR_CUDA);
  params.type = cudaGraphNodeTypeConditional;
  params.conditional.handle = handle;
  params.conditional.type = cudaGraphCondTypeWhile;
  params.conditional.size = 1;
  if (cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &params) != cudaSuccess) return fail(SL3DGPU_ERR_CUDA);
  cudaGraph_t body = params.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess)
    return fail(SL3DGPU_ERR_CUDA);
  const long long before = prof::Launches();
  const int st = CaptureCorrectionBody(f, handle);
  launches = prof::Launches() - before;
  prof::AddLaunches(-launches);  // captured, not launched
  cudaGraph_t captured = nullptr;
  const cudaError_t ended = cudaStreamEndCapture(stream, &captured);
  if (st != SL3DGPU_OK || ended != cudaSuccess) return fail(SL3DGPU_ERR_CUDA);
  if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) return fail(SL3DGPU_ERR_CUDA);
  cudaGraphDestroy(graph);
  if (correctionGraphs.size() >= 4) {
    cudaGraphExecDestroy(correctionGraphs.front().exec);
    correctionGraphs.erase(correctionGraphs.begin());
  }
  correctionGraphs.push_back(CorrectionGraph{key, exec, launches});
  *out = &correctionGraphs.back();
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::Correct(const Flavour& f, double tolerance, sl3dgpu_step_info& info, const double2* warm) {
  SL3D_TRY(PrepareLateral());
  const long long rows = rows0 + rows1 + rowsR;
  const int p0 = lateralFirst, lateral = lateralEnd - lateralFirst;
  LaunchGatherColumns(rows, P, p0, lateral, r32.p, rL.p, stream);
  SL3D_CHECK_LAUNCH();
  if (warm != nullptr) {
    // the guess's correction e = guess - s (FP32), its lateral columns
    LaunchResidual32(2 * spectralComplex, reinterpret_cast<const double*>(warm), reinterpret_cast<const double*>(s.p),
                     reinterpret_cast<float*>(e32.p), stream);
    SL3D_CHECK_LAUNCH();
    LaunchGatherColumns(rows, P, p0, lateral, e32.p, eL.p, stream);
    SL3D_CHECK_LAUNCH();
  } else {
    SL3D_CUDA(cudaMemcpyAsync(eL.p, rL.p, compactComplex * sizeof(float2), cudaMemcpyDeviceToDevice, stream));
  }
  const bool adaptive = options.anderson_rate > 0.0;
  bool mixing = CorrectionMemory() > 0 && !adaptive;
  bool firstMix = true;
  int count = 0, slot = 0;
  if (mixing) SL3D_TRY(Mixer32Reset());
  double previous = 0.0;
  int first = 0;       // the iteration the plain start's sequence begins at
  bool fresh = false;  // the solutions in rhs*32 are the pass of the final e
  bool triedGraph = false;
  CorrectionGraph* graph = nullptr;
  int iteration = 0;
  for (; iteration < options.max_iterations; ++iteration) {
    // after the first pass (and the warm start's decision) the loop runs on
    // the device, as a CUDA graph, when it can
    if (iteration >= 1 && !triedGraph && useGraphs && !prof::TimingOn()) {
      triedGraph = true;
      if (CorrectionGraphFor(f, &graph) == SL3DGPU_OK) break;
      graph = nullptr;
      useGraphs = false;  // the capture was refused: the host loop carries on
      cudaGetLastError();
    }
    SL3D_TRY(Pass32(f, eL.p, eNextL.p));
    ++info.correction_passes;
    LaunchRelativeChange(reinterpret_cast<const float*>(eNextL.p), reinterpret_cast<const float*>(eL.p),
                         2 * compactComplex, changePartial.p, kChangeBlocks, changeResult.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemcpyAsync(hostResult, changeResult.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    if (hostResult[2] == 0.0) {
      SetError("v3d: the FP32 correction left the finite range");
      return SL3DGPU_ERR_RUNTIME;
    }
    const double change = hostResult[0] > 0.0 ? std::sqrt(hostResult[1]) / std::sqrt(hostResult[0]) : 0.0;
    correctionHistory.push_back(change);
    if (warm != nullptr && iteration == 0) {
      // A guess whose first change is not well below the plain start's
      // (about rho / (1 + rho), near a half) is dropped: restart from e = r.
      warm = nullptr;
      if (change > kWarmKeep) {
        SL3D_CUDA(cudaMemcpyAsync(eL.p, rL.p, compactComplex * sizeof(float2), cudaMemcpyDeviceToDevice, stream));
        first = iteration + 1;
        continue;
      }
      guessTaken = 1;
    }
    if (change <= tolerance) {
      std::swap(eL, eNextL);
      fresh = true;
      break;
    }
    if (adaptive && !mixing && CorrectionMemory() > 0 && iteration > first &&
        change > options.anderson_rate * previous) {
      mixing = true;
      firstMix = true;
      count = slot = 0;
      SL3D_TRY(Mixer32Reset());
    }
    previous = change;
    if (mixing) {
      SL3D_TRY(Mixer32Update(count, slot, firstMix));
    } else {
      std::swap(eL, eNextL);
    }
  }
  if (graph != nullptr) {
    // the same loop from this iteration on the device: the host state in, the
    // graph's while node over the passes, the outcome out
    CorrectionControl c{};
    c.slot = slot;
    c.iteration = iteration;
    c.first = first;
    c.mixing = mixing ? 1 : 0;
    c.firstMix = firstMix ? 1 : 0;
    c.count = count;
    c.memory = CorrectionMemory();
    c.maxIterations = options.max_iterations;
    c.tolerance = tolerance;
    c.rate = adaptive ? options.anderson_rate : 0.0;
    c.previous = previous;
    const size_t head = offsetof(CorrectionControl, history);
    SL3D_CUDA(cudaMemcpyAsync(correctionControl.p, &c, head, cudaMemcpyHostToDevice, stream));
    SL3D_CUDA(cudaGraphLaunch(graph->exec, stream));
    SL3D_CUDA(cudaMemcpyAsync(&c, correctionControl.p, sizeof(CorrectionControl), cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    const int passes = c.historyCount;
    prof::AddLaunches(graph->launchesPerPass * passes);
    info.correction_passes += passes;
    for (int i = 0; i < std::min(passes, kCorrectionHistory); ++i) correctionHistory.push_back(c.history[i]);
    if (c.status != 0) {
      SetError("v3d: the FP32 correction left the finite range");
      return SL3DGPU_ERR_RUNTIME;
    }
    fresh = c.fresh != 0;
  }
  if (!fresh) {
    // out of passes on a mixed iterate: one more pass for its solutions
    SL3D_TRY(Pass32(f, eL.p, eNextL.p));
    ++info.correction_passes;
  }
  // the last pass's solutions below the lateral rows (y = 0 there), then
  // e at every node: the strain of those solutions, plus r
  auto* sph = reinterpret_cast<float*>(rhsSph32.p);
  auto* tor = reinterpret_cast<float*>(rhsTor32.p);
  SL3D_TRY(BandSolveWindowF(f.dSphChol.p, f.sphChol.data(), static_cast<int>(f.sphChol.size()), f.iSphChol.p,
                            f.nSphChol, f.bands32.p, sph, f.scales32.p, f.wSphChol.p, true, stream));
  SL3D_TRY(BandSolveWindowF(f.dTorChol.p, f.torChol.data(), static_cast<int>(f.torChol.size()), f.iTorChol.p,
                            f.nTorChol, f.bands32.p, tor, f.scales32.p, f.wTorChol.p, true, stream));
  LaunchStrain(geo, rhsSph32.p, rhsTor32.p, e32.p, stream, r32.p);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// -- conjugate gradients (Options::solver = ConjugateGradients) ---------------------------------------

// LateralForce (OpenStep::LateralForce): the strain of solutions x, its
// laterally weighted grid analysed over the lateral nodes, and the force of
// that on every degree's columns.
int Viscoelastic3DGpu::LateralForce(const double2* x, double2* out) {
  LaunchStrain(geo, x, x + rhsSphComplex, sNext.p, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaMemsetAsync(analysed.p, 0, spectralComplex * sizeof(double2), stream));
  SL3D_TRY(WeightedPass(sNext.p, analysed.p));
  SL3D_CUDA(cudaMemsetAsync(out, 0, Columns() * sizeof(double2), stream));
  LaunchForces(geo, analysed.p, out, out + rhsSphComplex, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// ApplyLateralOperator (Viscoelastic3D.cpp:626-728): K x - LateralForce(x).
int Viscoelastic3DGpu::ApplyOperator(const Flavour& f, const double2* x, double2* out) {
  SL3D_TRY(LateralForce(x, out));
  const auto* xd = reinterpret_cast<const double*>(x);
  auto* od = reinterpret_cast<double*>(out);
  LaunchBandApply(f.dSphApply.p, f.nSphApply, f.maxApplyRows, f.applyBands.p, xd, od, -1.0, stream);
  SL3D_CHECK_LAUNCH();
  LaunchBandApply(f.dTorApply.p, f.nTorApply, f.maxApplyRows, f.applyBands.p, xd, od, -1.0, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// LateralPair over every degree's m >= 0 columns, read back to the host.
int Viscoelastic3DGpu::PairOf(const double2* a, const double2* b, double* out) {
  LaunchPair(a, b, pairChunks.p, pairChunkCount, pairPartial.p, pairResult.p, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaMemcpyAsync(hostResult, pairResult.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  *out = hostResult[0];
  return SL3DGPU_OK;
}

// Preconditioned conjugate gradients (detail/LateralSolve.hpp:112-181, no
// start, reduction 0) on the forces in cgF into cgX: the reference response
// first, then the iteration on K x - LateralForce(x) (the step) or
// K x + (dK) x (the static perturbation problem), the reference solves as
// the preconditioner. `lateral` false stops at the reference response.
int Viscoelastic3DGpu::ConjugateGradients(const Flavour& f, bool lateral, double rtol, int maxIterations,
                                          sl3dgpu_step_info& info) {
  const long long n = 2 * Columns();
  auto* F = reinterpret_cast<double*>(cgF.p);
  auto* X = reinterpret_cast<double*>(cgX.p);
  auto* R = reinterpret_cast<double*>(cgR.p);
  auto* Z = reinterpret_cast<double*>(cgZ.p);
  auto* Pd = reinterpret_cast<double*>(cgP.p);
  auto* AP = reinterpret_cast<double*>(cgAp.p);
  auto apply = [&](const double2* x, double2* out) {
    return staticMode ? ApplyPerturbed(f, x, out) : ApplyOperator(f, x, out);
  };
  // x = K^-1 f, the reference response; energy = <x, f>.
  SL3D_CUDA(cudaMemcpyAsync(cgX.p, cgF.p, Columns() * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_TRY(SolveColumns(f, cgX.p, cgX.p + rhsSphComplex));
  double energy = 0.0;
  SL3D_TRY(PairOf(cgX.p, cgF.p, &energy));
  auto relative = [&](double value) {
    return energy > 0.0 ? std::sqrt(std::abs(value) / energy) : std::sqrt(std::abs(value));
  };
  info.converged = 0;
  info.solve_iterations = 0;
  if (!lateral) {
    info.converged = 1;
    info.residual = 0.0;
    history.push_back(0.0);
    return SL3DGPU_OK;
  }
  // r = f - A x, z = M^-1 r, p = z.
  SL3D_TRY(apply(cgX.p, cgAp.p));
  LaunchSub(n, F, AP, R, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaMemcpyAsync(cgZ.p, cgR.p, Columns() * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_TRY(SolveColumns(f, cgZ.p, cgZ.p + rhsSphComplex));
  double rz = 0.0;
  SL3D_TRY(PairOf(cgZ.p, cgR.p, &rz));
  info.residual = relative(rz);
  history.push_back(info.residual);
  SL3D_CUDA(cudaMemcpyAsync(cgP.p, cgZ.p, Columns() * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  for (int iteration = 0; iteration < maxIterations; ++iteration) {
    if (info.residual <= rtol) break;
    SL3D_TRY(apply(cgP.p, cgAp.p));
    double curvature = 0.0;
    SL3D_TRY(PairOf(cgP.p, cgAp.p, &curvature));
    const double alpha = rz / curvature;
    LaunchAxpy(n, alpha, Pd, X, stream);
    LaunchAxpy(n, -alpha, AP, R, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemcpyAsync(cgZ.p, cgR.p, Columns() * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
    SL3D_TRY(SolveColumns(f, cgZ.p, cgZ.p + rhsSphComplex));
    double next = 0.0;
    SL3D_TRY(PairOf(cgZ.p, cgR.p, &next));
    const double beta = next / rz;
    rz = next;
    LaunchXpby(n, Z, beta, Pd, stream);
    SL3D_CHECK_LAUNCH();
    info.solve_iterations = iteration + 1;
    info.residual = relative(rz);
    history.push_back(info.residual);
  }
  if (info.residual <= rtol) info.converged = 1;
  return SL3DGPU_OK;
}

// The solutions x (combined columns) as the operator's held solution, the
// one Surface reads.
int Viscoelastic3DGpu::HoldSolution(const double2* x) {
  SL3D_CUDA(cudaMemcpyAsync(rhsSph.p, x, rhsSphComplex * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  if (rhsTorComplex > 0)
    SL3D_CUDA(cudaMemcpyAsync(rhsTor.p, x + rhsSphComplex, rhsTorComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                              stream));
  return SL3DGPU_OK;
}

// The step closed by preconditioned conjugate gradients (Viscoelastic3D.cpp
// :2008-2015): forces of the fixed memory and the load channel
// (OpenStep::Forces), the solve (OpenStep::Solve, lateral always), the
// strain of the solution.
int Viscoelastic3DGpu::ConvergeConjugateGradients(const Flavour& f, const double2* sigmaEnd,
                                                  sl3dgpu_step_info& info) {
  SL3D_CUDA(cudaMemsetAsync(cgF.p, 0, Columns() * sizeof(double2), stream));
  LaunchForces(geo, fixedS.p, cgF.p, cgF.p + rhsSphComplex, stream);
  SL3D_CHECK_LAUNCH();
  if (sigmaEnd != nullptr || tideEnd != nullptr) {
    LaunchAddLoad(geo, sigmaEnd, f.loadForces.p, f.unitOffset.p, cgF.p, stream, tideEnd, f.tideForces.p);
    SL3D_CHECK_LAUNCH();
  }
  SL3D_TRY(ConjugateGradients(f, true, options.solve_rtol, options.solve_max_iterations, info));
  info.iterations = info.solve_iterations;
  SL3D_TRY(HoldSolution(cgX.p));
  LaunchStrain(geo, rhsSph.p, rhsTor.p, s.p, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::AssembledBand(int scheme, double dt, int toroidal, int l, double* out, long long capacity,
                                     int* n, int* kd) {
  const int L = options.lmax;
  if (l < (toroidal ? 1 : 0) || l > L || scheme < 0 || scheme > 1 || !(dt >= 0.0)) {
    SetError("v3d: a degree in range (toroidal from 1), scheme 0 (exponential trapezoid) or 1 (backward Euler) "
             "and dt >= 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  Flavour* f = elastic.get();
  if (dt > 0.0) SL3D_TRY(FlavourOf(scheme, dt, &f));
  const AssemblySystem& sys = plan.systems[toroidal ? L + l : l];
  const long long size = static_cast<long long>(sys.kd + 1) * sys.ndof;
  if (n) *n = sys.ndof;
  if (kd) *kd = sys.kd;
  if (out == nullptr) return SL3DGPU_OK;
  if (capacity < size) {
    SetError("v3d: the band needs " + std::to_string(size) + " values");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaMemcpyAsync(out, f->applyBands.p + sys.band, size * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// -- the static perturbation problem (ElasticPerturbation3D) ----------------------------------------

// The moduli directions over the grid values (node-major, colatitude,
// longitude), either null; the transforms then run over the nodes where
// one of them is non-zero.
int Viscoelastic3DGpu::SetModuli(const double* dMu, const double* dKappa, bool onDevice) {
  if (!staticMode) {
    SetError("ep3d: not a static perturbation operator");
    return SL3DGPU_ERR_ARGUMENT;
  }
  hasMu = dMu != nullptr;
  hasKappa = dKappa != nullptr;
  std::vector<double> host(values);
  std::vector<char> lateral(P, 0);
  auto take = [&](const double* src, Dev<double>& dst) -> int {
    if (src == nullptr) {
      SL3D_CUDA(ZeroIn(dst.p, values * sizeof(double)));
      return SL3DGPU_OK;
    }
    if (onDevice) {
      SL3D_CUDA(cudaMemcpy(host.data(), src, values * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
      std::memcpy(host.data(), src, values * sizeof(double));
    }
    for (int p = 0; p < P; ++p)
      for (long long x = p * fieldSize; x < (p + 1) * fieldSize && !lateral[p]; ++x) lateral[p] = host[x] != 0.0;
    SL3D_CUDA(cudaStreamSynchronize(stream));  // no earlier kernel of the operator still reads it
    SL3D_CUDA(CopyIn(dst.p, host.data(), values * sizeof(double)));
    return SL3DGPU_OK;
  };
  SL3D_TRY(take(dMu, weight));
  SL3D_TRY(take(dKappa, kappaWeight));
  int first = P, last = -1;
  for (int p = 0; p < P; ++p)
    if (lateral[p]) {
      first = std::min(first, p);
      last = std::max(last, p);
    }
  lateralFirst = last >= 0 ? first : 0;
  lateralEnd = last >= 0 ? last + 1 : 0;
  return SL3DGPU_OK;
}

// (dK) x (ElasticPerturbation3D::Force, src/ElasticPerturbation3D.cpp:140-
// 226): the deviatoric strain weighted by dMu back as force, plus the
// dilatation weighted by dKappa back as force.
int Viscoelastic3DGpu::PerturbationForce(const double2* x, double2* out) {
  SL3D_CUDA(cudaMemsetAsync(out, 0, Columns() * sizeof(double2), stream));
  if (hasMu) {
    LaunchStrain(geo, x, x + rhsSphComplex, sNext.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemsetAsync(analysed.p, 0, spectralComplex * sizeof(double2), stream));
    SL3D_TRY(WeightedPass(sNext.p, analysed.p));
    LaunchForces(geo, analysed.p, out, out + rhsSphComplex, stream);
    SL3D_CHECK_LAUNCH();
  }
  if (hasKappa) {
    LaunchDilatation(geo, x, scalarD.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaMemsetAsync(scalarW.p, 0, rowsR * P * sizeof(double2), stream));
    const int p0 = lateralFirst, count = lateralEnd - lateralFirst;
    if (count > 0) {
      auto* a = reinterpret_cast<double*>(spectraA.p);
      auto* b = reinterpret_cast<double*>(spectraB.p);
      SL3D_TRY(grid->LegendreSynthesis(0, true, reinterpret_cast<const double*>(scalarD.p), P, p0, count, a, stream));
      SL3D_TRY(grid->RingWeighted(true, a, count, kappaWeight.p + p0 * fieldSize, b, stream));
      SL3D_TRY(grid->LegendreAnalysis(0, true, b, P, p0, count, reinterpret_cast<double*>(scalarW.p), false, stream));
    }
    LaunchDilatationForce(geo, scalarW.p, out, stream);
    SL3D_CHECK_LAUNCH();
  }
  return SL3DGPU_OK;
}

// (K_ref + dK) x (ElasticPerturbation3D::Apply, :305-338).
int Viscoelastic3DGpu::ApplyPerturbed(const Flavour& f, const double2* x, double2* out) {
  SL3D_TRY(PerturbationForce(x, out));
  const auto* xd = reinterpret_cast<const double*>(x);
  auto* od = reinterpret_cast<double*>(out);
  LaunchBandApply(f.dSphApply.p, f.nSphApply, f.maxApplyRows, f.applyBands.p, xd, od, 1.0, stream);
  SL3D_CHECK_LAUNCH();
  LaunchBandApply(f.dTorApply.p, f.nTorApply, f.maxApplyRows, f.applyBands.p, xd, od, 1.0, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// SolveLoad (:98-126): per degree the unit load response times the load's
// coefficients, held as the solution.
int Viscoelastic3DGpu::SolveLoad(const double* load) {
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  SL3D_CUDA(cudaMemcpyAsync(sigma0.p, load, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
  SL3D_CUDA(cudaMemsetAsync(cgX.p, 0, Columns() * sizeof(double2), stream));
  LaunchAddLoad(geo, sigma0.p, elastic->units.p, elastic->unitOffset.p, cgX.p, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(HoldSolution(cgX.p));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// Respond (:474-479): the held solution x replaced by its first-order change
// -K^-1 (dK) x.
int Viscoelastic3DGpu::Respond() {
  SL3D_TRY(PerturbationForce(cgX.p, cgF.p));
  SL3D_TRY(SolveColumns(*elastic, cgF.p, cgF.p + rhsSphComplex));
  SL3D_CUDA(cudaMemsetAsync(cgX.p, 0, Columns() * sizeof(double2), stream));
  LaunchAxpy(2 * Columns(), -1.0, reinterpret_cast<const double*>(cgF.p), reinterpret_cast<double*>(cgX.p), stream);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(HoldSolution(cgX.p));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// SolveLateral for a load (:367-372, :374-430): (K_ref + dK) x = LoadForces,
// conjugate gradients from the reference response; lateral unless neither
// direction was given.
int Viscoelastic3DGpu::SolveLateral(const double* load, double rtol, int maxIterations, sl3dgpu_step_info* out) {
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  history.clear();
  SL3D_CUDA(cudaMemcpyAsync(sigma0.p, load, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
  SL3D_CUDA(cudaMemsetAsync(cgF.p, 0, Columns() * sizeof(double2), stream));
  LaunchAddLoad(geo, sigma0.p, elastic->loadForces.p, elastic->unitOffset.p, cgF.p, stream);
  SL3D_CHECK_LAUNCH();
  sl3dgpu_step_info info{};
  SL3D_TRY(ConjugateGradients(*elastic, hasMu || hasKappa, rtol, maxIterations, info));
  info.iterations = info.solve_iterations;
  SL3D_TRY(HoldSolution(cgX.p));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  if (out) *out = info;
  return SL3DGPU_OK;
}

// Step (Viscoelastic3D.cpp:1982-2030): one stage, or Sdirk2's two backward
// Euler stages of gamma dt, the second from (1 - r) m_n + r Y_1.
int Viscoelastic3DGpu::Step(V3dState& st, double dt, int scheme, const double* load0, const double* load1,
                            sl3dgpu_step_info* infoOut, bool onDevice, const double* tide0, const double* tide1) {
  if (!(dt >= 0.0) || scheme < 0 || scheme > 2) {
    SetError("v3d: dt >= 0 and a scheme of 0 (trapezoid), 1 (backward Euler) or 2 (Sdirk2)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  // The tide channel (TideColumns, Viscoelastic3D.cpp:137-154): its degree-1
  // columns must vanish, a tide being taken relative to the centre of mass.
  const double2* t0 = nullptr;
  const double2* t1 = nullptr;
  for (int end = 0; end < 2; ++end) {
    const double* tide = end ? tide1 : tide0;
    if (tide == nullptr) continue;
    Dev<double2>& dev = end ? tideDev1 : tideDev0;
    if (dev.n != lm) SL3D_CUDA(dev.Alloc(lm));
    SL3D_CUDA(cudaMemcpyAsync(dev.p, tide, lm * sizeof(double2),
                              onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
    double2 degreeOne[2];
    SL3D_CUDA(cudaMemcpyAsync(degreeOne, dev.p + 1, 2 * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    for (const auto& v : degreeOne)
      if (v.x != 0.0 || v.y != 0.0) {
        SetError("v3d: a tide channel has no degree-1 part: tides are taken relative to the centre of mass, its "
                 "degree-1 columns must vanish");
        return SL3DGPU_ERR_ARGUMENT;
      }
    (end ? t1 : t0) = dev.p;
  }
  const double2* s0 = nullptr;
  const double2* s1 = nullptr;
  const cudaMemcpyKind kind = onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (load0) {
    SL3D_CUDA(cudaMemcpyAsync(sigma0.p, load0, lm * sizeof(double2), kind, stream));
    s0 = sigma0.p;
  }
  if (load1) {
    SL3D_CUDA(cudaMemcpyAsync(sigma1.p, load1, lm * sizeof(double2), kind, stream));
    s1 = sigma1.p;
  }
  sl3dgpu_step_info info{};
  history.clear();
  correctionHistory.clear();
  guessTaken = 0;
  // The guess of the step's end strain: the caller's, else (warm_start 1)
  // the linear extrapolation 2 s_n - s_{n-1} of the last two steps.
  bool haveGuess = guessArmed;
  if (!haveGuess && options.warm_start == 1 && st.hasCoeffs && st.hasPrev && dt > 0.0) {
    if (guess.n != static_cast<size_t>(spectralComplex)) {
      SL3D_CUDA(guess.Alloc(spectralComplex));
      SL3D_CUDA(guessNext.Alloc(spectralComplex));
    }
    LaunchBlend(spectralComplex, 2.0, st.prev.p, st.coeffs.p, guess.p, stream);
    SL3D_CHECK_LAUNCH();
    haveGuess = true;
  }
  tideStart = t0;
  tideEnd = t1;
  if (scheme != 2 || dt == 0.0) {
    const int one = scheme == 2 ? 1 : scheme;
    stageGuess = haveGuess ? guess.p : nullptr;
    ocean.cStart = 0.0;
    ocean.cEnd = 1.0;
    SL3D_TRY(StepOnce(st, scratch, dt, one, s0, s1, info));
  } else {
    const double gamma = host::kSdirk2Gamma;
    const double h = gamma * dt;
    const double2* mid = nullptr;
    if (load0 || load1) {
      // the first stage's end: (1 - gamma) of the start load and gamma of the end's
      LaunchBlend(static_cast<long long>(lm), gamma, s0, s1, sigmaMid.p, stream);
      SL3D_CHECK_LAUNCH();
      mid = sigmaMid.p;
    }
    const double2* tmid = nullptr;
    if (t0 || t1) {
      if (tideDevMid.n != lm) SL3D_CUDA(tideDevMid.Alloc(lm));
      LaunchBlend(static_cast<long long>(lm), gamma, t0, t1, tideDevMid.p, stream);
      SL3D_CHECK_LAUNCH();
      tmid = tideDevMid.p;
    }
    tideEnd = tmid;
    sl3dgpu_step_info i1{}, i2{};
    // the first stage's guess (the mixed form, which takes it at no FP64
    // cost): (1 - gamma) s_n + gamma guess
    stageGuess = nullptr;
    if (haveGuess && options.precision == 1 && st.hasCoeffs) {
      if (guessMid.n != static_cast<size_t>(spectralComplex)) SL3D_CUDA(guessMid.Alloc(spectralComplex));
      LaunchBlend(spectralComplex, gamma, st.coeffs.p, guess.p, guessMid.p, stream);
      SL3D_CHECK_LAUNCH();
      stageGuess = guessMid.p;
    }
    ocean.cStart = 0.0;
    ocean.cEnd = gamma;
    SL3D_TRY(StepOnce(st, scratch, h, 1, s0, mid, i1));
    // the second stage's memory (1 - r) m_n + r Y_1, formed in place in Y_1
    const double r = (1.0 - gamma) / gamma;
    const long long begin = lateralFirst * fieldSize, end = static_cast<long long>(lateralEnd) * fieldSize;
    for (int k = 0; k < K; ++k) {
      if (end > begin) {
        LaunchStageCombine(end - begin, r, st.m[k].c0.p + begin, st.m[k].c1.p + begin, st.m[k].r.p + begin,
                           scratch.m[k].c0.p + begin, scratch.m[k].c1.p + begin, scratch.m[k].r.p + begin, stream);
        SL3D_CHECK_LAUNCH();
      }
      LaunchSpectralCombine(rows0 + rows1 + rowsR, P, lateralFirst, lateralEnd, r, st.mSpec[k].p,
                            scratch.mSpec[k].p, stream);
      SL3D_CHECK_LAUNCH();
    }
    stageGuess = haveGuess ? guess.p : nullptr;
    tideStart = tmid;
    tideEnd = t1;
    ocean.cStart = gamma;
    ocean.cEnd = 1.0;
    SL3D_TRY(StepOnce(scratch, scratch, h, 1, mid, s1, i2));
    info.iterations = i1.iterations + i2.iterations;
    info.mixed_passes = i1.mixed_passes + i2.mixed_passes;
    info.correction_passes = i1.correction_passes + i2.correction_passes;
    info.solve_iterations = i1.solve_iterations + i2.solve_iterations;
    info.residual = i2.residual;
    info.converged = i1.converged && i2.converged;
  }
  guessArmed = false;  // a warm start serves one step
  stageGuess = nullptr;
  tideStart = tideEnd = nullptr;
  SL3D_TRY(Adopt(st));
  if (infoOut) *infoOut = info;
  return SL3DGPU_OK;
}

// The state takes the finished stage's buffers (the scratch set), keeping
// its coefficients as the step before's under warm_start 1.
int Viscoelastic3DGpu::Adopt(V3dState& st) {
  if (options.warm_start == 1 && st.hasCoeffs) {
    SL3D_CUDA(cudaMemcpyAsync(st.prev.p, st.coeffs.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                              stream));
    st.hasPrev = true;
  }
  std::swap(st.m, scratch.m);
  std::swap(st.mSpec, scratch.mSpec);
  std::swap(st.strain, scratch.strain);
  std::swap(st.coeffs, scratch.coeffs);
  std::swap(st.latFirst, scratch.latFirst);
  std::swap(st.latEnd, scratch.latEnd);
  st.hasStrain = st.hasCoeffs = true;
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// -- a state as bytes -----------------------------------------------------------------------------------

namespace {
struct StateHeader {
  char magic[8];  // "SL3DGST1"
  long long K, values, spectralComplex, fieldSize;
  int latFirst, latEnd, hasStrain, hasCoeffs, hasPrev, pad;
};
constexpr char kStateMagic[8] = {'S', 'L', '3', 'D', 'G', 'S', 'T', '1'};
}  // namespace

long long Viscoelastic3DGpu::StateBytes(const V3dState& st) const {
  const long long lateral = static_cast<long long>(st.latEnd - st.latFirst) * fieldSize;
  const long long grid = lateral * static_cast<long long>(2 * sizeof(double2) + sizeof(double));
  const long long spec = spectralComplex * static_cast<long long>(sizeof(double2));
  return static_cast<long long>(sizeof(StateHeader)) + K * (grid + spec) + (st.hasStrain ? grid : 0) +
         (st.hasCoeffs ? spec : 0) + (st.hasPrev ? spec : 0);
}

int Viscoelastic3DGpu::SaveState(const V3dState& st, char* out, long long capacity) {
  if (capacity < StateBytes(st)) {
    SetError("v3d: the buffer is smaller than the state (sl3dgpu_v3d_state_bytes)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  StateHeader h{};
  std::memcpy(h.magic, kStateMagic, 8);
  h.K = K;
  h.values = values;
  h.spectralComplex = spectralComplex;
  h.fieldSize = fieldSize;
  h.latFirst = st.latFirst;
  h.latEnd = st.latEnd;
  h.hasStrain = st.hasStrain;
  h.hasCoeffs = st.hasCoeffs;
  h.hasPrev = st.hasPrev;
  std::memcpy(out, &h, sizeof(h));
  char* at = out + sizeof(h);
  const long long begin = static_cast<long long>(st.latFirst) * fieldSize;
  const long long lateral = static_cast<long long>(st.latEnd - st.latFirst) * fieldSize;
  auto take = [&](const void* device, size_t bytes) -> int {
    if (bytes > 0) SL3D_CUDA(cudaMemcpyAsync(at, device, bytes, cudaMemcpyDeviceToHost, stream));
    at += bytes;
    return SL3DGPU_OK;
  };
  auto grid = [&](const GridTensor& g) -> int {
    SL3D_TRY(take(g.c0.p + begin, lateral * sizeof(double2)));
    SL3D_TRY(take(g.c1.p + begin, lateral * sizeof(double2)));
    return take(g.r.p + begin, lateral * sizeof(double));
  };
  for (int k = 0; k < K; ++k) {
    SL3D_TRY(grid(st.m[k]));
    SL3D_TRY(take(st.mSpec[k].p, spectralComplex * sizeof(double2)));
  }
  if (st.hasStrain) SL3D_TRY(grid(st.strain));
  if (st.hasCoeffs) SL3D_TRY(take(st.coeffs.p, spectralComplex * sizeof(double2)));
  if (st.hasPrev) SL3D_TRY(take(st.prev.p, spectralComplex * sizeof(double2)));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::LoadState(V3dState& st, const char* in, long long bytes) {
  StateHeader h{};
  if (bytes < static_cast<long long>(sizeof(h))) {
    SetError("v3d: not a state (too short)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  std::memcpy(&h, in, sizeof(h));
  if (std::memcmp(h.magic, kStateMagic, 8) != 0 || h.K != K || h.values != values ||
      h.spectralComplex != spectralComplex || h.fieldSize != fieldSize || h.latFirst < 0 || h.latEnd > P ||
      h.latFirst > h.latEnd || (h.hasPrev && options.warm_start != 1)) {
    SetError("v3d: the state was not saved by an operator of this shape");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_TRY(AllocState(st));
  st.latFirst = h.latFirst;
  st.latEnd = h.latEnd;
  st.hasStrain = h.hasStrain != 0;
  st.hasCoeffs = h.hasCoeffs != 0;
  st.hasPrev = h.hasPrev != 0;
  if (bytes != StateBytes(st)) {
    SetError("v3d: the state's size does not match its header");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const char* at = in + sizeof(h);
  const long long begin = static_cast<long long>(st.latFirst) * fieldSize;
  const long long lateral = static_cast<long long>(st.latEnd - st.latFirst) * fieldSize;
  auto give = [&](void* device, size_t n) -> int {
    if (n > 0) SL3D_CUDA(cudaMemcpyAsync(device, at, n, cudaMemcpyHostToDevice, stream));
    at += n;
    return SL3DGPU_OK;
  };
  auto grid = [&](GridTensor& g) -> int {
    SL3D_TRY(give(g.c0.p + begin, lateral * sizeof(double2)));
    SL3D_TRY(give(g.c1.p + begin, lateral * sizeof(double2)));
    return give(g.r.p + begin, lateral * sizeof(double));
  };
  for (int k = 0; k < K; ++k) {
    SL3D_TRY(grid(st.m[k]));
    SL3D_TRY(give(st.mSpec[k].p, spectralComplex * sizeof(double2)));
  }
  if (st.hasStrain) SL3D_TRY(grid(st.strain));
  if (st.hasCoeffs) SL3D_TRY(give(st.coeffs.p, spectralComplex * sizeof(double2)));
  if (st.hasPrev) SL3D_TRY(give(st.prev.p, spectralComplex * sizeof(double2)));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// -- GridCoupling's maps (include/sl3dpp/GridCoupling.hpp:82-428) ---------------------------------------

int Viscoelastic3DGpu::TensorSynthesise(const double2* spectral, double2* c0, double2* c1, double* r) {
  SL3D_TRY(Synthesise(spectral, dGrid));
  SL3D_CUDA(cudaMemcpyAsync(c0, dGrid.c0.p, values * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_CUDA(cudaMemcpyAsync(c1, dGrid.c1.p, values * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_CUDA(cudaMemcpyAsync(r, dGrid.r.p, values * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::TensorAnalyse(const double2* c0, const double2* c1, const double* r, double2* spectral) {
  SL3D_CUDA(cudaMemcpyAsync(dGrid.c0.p, c0, values * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_CUDA(cudaMemcpyAsync(dGrid.c1.p, c1, values * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_CUDA(cudaMemcpyAsync(dGrid.r.p, r, values * sizeof(double), cudaMemcpyDeviceToDevice, stream));
  SL3D_TRY(Analyse(dGrid, spectral));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::DegreeForces(const double2* spectral, double2* sph, double2* tor) {
  SL3D_CUDA(cudaMemsetAsync(sph, 0, rhsSphComplex * sizeof(double2), stream));
  if (rhsTorComplex > 0) SL3D_CUDA(cudaMemsetAsync(tor, 0, rhsTorComplex * sizeof(double2), stream));
  LaunchForces(geo, spectral, sph, tor, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::StrainOfSolutions(const double2* sph, const double2* tor, double2* spectral) {
  LaunchStrain(geo, sph, tor, spectral, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// -- the open step (Viscoelastic3D::OpenStep, include/sl3dpp/Viscoelastic3D.hpp:440-640) ------------

int Viscoelastic3DGpu::OpenStart(V3dState& st, double dt, int scheme, const double* load0) {
  if (opened.open) {
    SetError("v3d: a step is open on this operator: finish it first (one open step per operator)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (!(dt >= 0.0) || scheme < 0 || scheme > 1 || staticMode || ocean.on) {
    SetError("v3d: an open step is one stage (scheme 0 or 1, dt >= 0) of the step operator without an ocean");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  const double2* s0 = nullptr;
  if (load0 != nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(sigma0.p, load0, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    s0 = sigma0.p;
  }
  history.clear();
  tideStart = tideEnd = nullptr;
  ocean.cStart = 0.0;
  ocean.cEnd = 1.0;
  Flavour* f = nullptr;
  SL3D_TRY(StartStage(st, scratch, dt, scheme, s0, &f));
  opened = OpenStage{true, &st, f, scheme, dt};
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenCheck() const {
  if (!opened.open) {
    SetError("v3d: no open step (sl3dgpu_v3d_start_step)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenChannels(const double* load, const double* tide) {
  SL3D_TRY(OpenCheck());
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  const double2* sigma = nullptr;
  const double2* psi = nullptr;
  if (load != nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(sigma1.p, load, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    sigma = sigma1.p;
  }
  if (tide != nullptr) {
    const double2* t = reinterpret_cast<const double2*>(tide);
    if (t[1].x != 0.0 || t[1].y != 0.0 || t[2].x != 0.0 || t[2].y != 0.0) {
      SetError("v3d: a tide channel has no degree-1 part: tides are taken relative to the centre of mass");
      return SL3DGPU_ERR_ARGUMENT;
    }
    if (tideDev1.n != lm) SL3D_CUDA(tideDev1.Alloc(lm));
    SL3D_CUDA(cudaMemcpyAsync(tideDev1.p, tide, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    psi = tideDev1.p;
  }
  if (sigma != nullptr || psi != nullptr) {
    LaunchAddLoad(geo, sigma, opened.f->units.p, opened.f->unitOffset.p, rhsSph.p, stream, psi,
                  opened.f->tideUnits.p);
    SL3D_CHECK_LAUNCH();
  }
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenConverge(const double* load, const double* tide, sl3dgpu_step_info* infoOut) {
  SL3D_TRY(OpenCheck());
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  const double2* sigma = nullptr;
  if (load != nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(sigma1.p, load, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    sigma = sigma1.p;
  }
  tideEnd = nullptr;
  if (tide != nullptr) {
    if (tideDev1.n != lm) SL3D_CUDA(tideDev1.Alloc(lm));
    SL3D_CUDA(cudaMemcpyAsync(tideDev1.p, tide, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    tideEnd = tideDev1.p;
  }
  sl3dgpu_step_info info{};
  history.clear();
  const Flavour& f = *opened.f;
  if (options.solver == 1) {
    SL3D_TRY(ConvergeConjugateGradients(f, sigma, info));
  } else if (options.precision == 1) {
    LaunchCast(values, weight.p, weight32.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_TRY(ConvergeMixed(f, sigma, info));
  } else {
    SL3D_TRY(Converge(f, sigma, info));
  }
  tideEnd = nullptr;
  SL3D_CUDA(cudaStreamSynchronize(stream));
  if (infoOut) *infoOut = info;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenForces(const double* load, const double* tide, double2* out) {
  SL3D_TRY(OpenCheck());
  if (options.solver != 1) {
    SetError("v3d: the open step's forces and operator are the conjugate-gradient close's (solver 1)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  const Flavour& f = *opened.f;
  SL3D_CUDA(cudaMemsetAsync(out, 0, Columns() * sizeof(double2), stream));
  LaunchForces(geo, fixedS.p, out, out + rhsSphComplex, stream);
  SL3D_CHECK_LAUNCH();
  const double2* sigma = nullptr;
  const double2* psi = nullptr;
  if (load != nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(sigma1.p, load, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    sigma = sigma1.p;
  }
  if (tide != nullptr) {
    if (tideDev1.n != lm) SL3D_CUDA(tideDev1.Alloc(lm));
    SL3D_CUDA(cudaMemcpyAsync(tideDev1.p, tide, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    psi = tideDev1.p;
  }
  if (sigma != nullptr || psi != nullptr) {
    LaunchAddLoad(geo, sigma, f.loadForces.p, f.unitOffset.p, out, stream, psi, f.tideForces.p);
    SL3D_CHECK_LAUNCH();
  }
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenApply(const double2* x, double2* out) {
  SL3D_TRY(OpenCheck());
  if (options.solver != 1) {
    SetError("v3d: the open step's forces and operator are the conjugate-gradient close's (solver 1)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_TRY(ApplyOperator(*opened.f, x, out));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenSolve(const double2* forces, double2* out, sl3dgpu_step_info* infoOut) {
  SL3D_TRY(OpenCheck());
  if (options.solver != 1) {
    SetError("v3d: the open step's forces and operator are the conjugate-gradient close's (solver 1)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaMemcpyAsync(cgF.p, forces, Columns() * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  sl3dgpu_step_info info{};
  history.clear();
  SL3D_TRY(ConjugateGradients(*opened.f, true, options.solve_rtol, options.solve_max_iterations, info));
  info.iterations = info.solve_iterations;
  SL3D_TRY(HoldSolution(cgX.p));
  if (out != nullptr)
    SL3D_CUDA(cudaMemcpyAsync(out, cgX.p, Columns() * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  if (infoOut) *infoOut = info;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::OpenFinish(const double2* strain) {
  SL3D_TRY(OpenCheck());
  if (strain != nullptr)
    SL3D_CUDA(cudaMemcpyAsync(s.p, strain, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  SL3D_TRY(FinishStage(scratch, opened.dt, opened.scheme));
  V3dState& st = *opened.st;
  opened = OpenStage{};
  return Adopt(st);
}

int Viscoelastic3DGpu::Surface(int component, double* out, bool deviceOut) {
  if (component < 0 || component > 3) {
    SetError("v3d: component 0 (U), 1 (V), 2 (phi) or 3 (W, toroidal)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (deviceOut) {  // stream-ordered into the caller's device buffer, no wait
    LaunchSurface(geo, rhsSph.p, rhsTor.p, component, reinterpret_cast<double2*>(out), stream);
    SL3D_CHECK_LAUNCH();
    return SL3DGPU_OK;
  }
  LaunchSurface(geo, rhsSph.p, rhsTor.p, component, surfaceOut.p, stream);
  SL3D_CHECK_LAUNCH();
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  SL3D_CUDA(cudaMemcpyAsync(out, surfaceOut.p, lm * sizeof(double2), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// InertiaMoment (Viscoelastic3D.cpp:2032-2048): the degree-0 moment row
// (detail/ViscoelasticDegree.hpp:142-161) against the real part of the last
// solutions' degree-0 column.
int Viscoelastic3DGpu::InertiaMoment(double* out) {
  const int ndof = degrees[0].sphNdof;
  std::vector<double2> x(static_cast<size_t>(ndof));
  SL3D_CUDA(cudaMemcpyAsync(x.data(), rhsSph.p + degrees[0].sphRhs, ndof * sizeof(double2), cudaMemcpyDeviceToHost,
                            stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  double sum = 0.0;
  for (int d = 0; d < ndof; ++d) sum += momentRow[d] * x[d].x;
  *out = sum;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::StrainReference(const V3dState& st, double* out) {
  if (!st.hasCoeffs) {
    SetError("v3d: the state carries no strain coefficients");
    return SL3DGPU_ERR_ARGUMENT;
  }
  Dev<double> ref;
  SL3D_CUDA(ref.Alloc(2 * spectralComplex));
  const auto* base = reinterpret_cast<const double*>(st.coeffs.p);
  SL3D_TRY(grid->FromDevice(-2, false, base, P, ref.p, stream));
  SL3D_TRY(grid->FromDevice(-1, false, base + 2 * rows0 * P, P, ref.p + 2 * rows0 * P, stream));
  SL3D_TRY(grid->FromDevice(0, true, base + 2 * (rows0 + rows1) * P, P, ref.p + 2 * (rows0 + rows1) * P, stream));
  SL3D_CUDA(cudaMemcpyAsync(out, ref.p, 2 * spectralComplex * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

// -- the discrete adjoint -------------------------------------------------------------------------------

int Viscoelastic3DGpu::CopyState(const V3dState& from, V3dState& to) {
  for (int k = 0; k < K; ++k) {
    SL3D_CUDA(cudaMemcpyAsync(to.m[k].c0.p, from.m[k].c0.p, values * sizeof(double2), cudaMemcpyDeviceToDevice,
                              stream));
    SL3D_CUDA(cudaMemcpyAsync(to.m[k].c1.p, from.m[k].c1.p, values * sizeof(double2), cudaMemcpyDeviceToDevice,
                              stream));
    SL3D_CUDA(cudaMemcpyAsync(to.m[k].r.p, from.m[k].r.p, values * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    SL3D_CUDA(cudaMemcpyAsync(to.mSpec[k].p, from.mSpec[k].p, spectralComplex * sizeof(double2),
                              cudaMemcpyDeviceToDevice, stream));
  }
  SL3D_CUDA(cudaMemcpyAsync(to.strain.c0.p, from.strain.c0.p, values * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  SL3D_CUDA(cudaMemcpyAsync(to.strain.c1.p, from.strain.c1.p, values * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  SL3D_CUDA(cudaMemcpyAsync(to.strain.r.p, from.strain.r.p, values * sizeof(double), cudaMemcpyDeviceToDevice,
                            stream));
  SL3D_CUDA(cudaMemcpyAsync(to.coeffs.p, from.coeffs.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  to.hasStrain = from.hasStrain;
  to.hasCoeffs = from.hasCoeffs;
  to.hasPrev = false;
  to.latFirst = from.latFirst;
  to.latEnd = from.latEnd;
  return SL3DGPU_OK;
}

// One stage transposed. Forward (StartStage, the converged fixed point,
// FinishStage): m~_k = e_k m_k + alpha_k d_start; phi = An(sum_k mu_k m~_k);
// (K - F An W Syn Str) x = F phi + K u sigma; d_end = Syn Str x; m'_k = m~_k +
// beta_k d_end; the surface reads S x. Given the duals of m'_k and d_end (the
// sweep's buffers) and of the surface reads (measured), the system's
// symmetry makes its dual solve z = (K - F An W Syn Str)^-1 (F An d-bar +
// S^T g), d-bar = dD + sum_k beta_k mD_k, the step's own iteration from a
// zero strain with fixed force An(d-bar) and K^-1 S^T g added after every
// solve; then zeta = Syn Str z gives the memory duals M_k = mD_k + mu_k zeta,
// the start's duals e_k M_k and sum_k alpha_k M_k, the load's dual u^T K z
// = u^T (F An(d-bar + W zeta) + S^T g) and the gradient in delta through
// e, alpha, beta (W's share folded into M). The stage's weights are
// StartStage's own, recomputed from the start state.
// The stage's forward fields on the grid at every node (adj.startM,
// startD, endD): the memory as the state holds it at the lateral nodes and
// synthesised from its coefficients elsewhere, the strains from their
// coefficients.
int Viscoelastic3DGpu::ForwardFields(const V3dState& in, const V3dState& end) {
  const int p0 = lateralFirst, p1 = lateralEnd;
  const long long begin = p0 * fieldSize, span = static_cast<long long>(p1 - p0) * fieldSize;
  for (int k = 0; k < K; ++k) {
    if (span > 0) {
      SL3D_CUDA(cudaMemcpyAsync(adj.startM[k].c0.p + begin, in.m[k].c0.p + begin, span * sizeof(double2),
                                cudaMemcpyDeviceToDevice, stream));
      SL3D_CUDA(cudaMemcpyAsync(adj.startM[k].c1.p + begin, in.m[k].c1.p + begin, span * sizeof(double2),
                                cudaMemcpyDeviceToDevice, stream));
      SL3D_CUDA(cudaMemcpyAsync(adj.startM[k].r.p + begin, in.m[k].r.p + begin, span * sizeof(double),
                                cudaMemcpyDeviceToDevice, stream));
    }
    if (p0 > 0) SL3D_TRY(SynthesiseRange(in.mSpec[k].p, adj.startM[k], 0, p0));
    if (p1 < P) SL3D_TRY(SynthesiseRange(in.mSpec[k].p, adj.startM[k], p1, P - p1));
  }
  if (in.hasCoeffs) {
    SL3D_TRY(SynthesiseRange(in.coeffs.p, adj.startD, 0, P));
  } else {
    SL3D_CUDA(cudaMemsetAsync(adj.startD.c0.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(adj.startD.c1.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(adj.startD.r.p, 0, values * sizeof(double), stream));
  }
  SL3D_TRY(SynthesiseRange(end.coeffs.p, adj.endD, 0, P));
  return SL3DGPU_OK;
}

// The next stage's start guess (1 - c) a + c b in the warm-start buffer
// (b null: a itself), armed for the stage.
int Viscoelastic3DGpu::ArmGuess(const double2* a, const double2* b, double c) {
  if (guess.n != static_cast<size_t>(spectralComplex)) {
    SL3D_CUDA(guess.Alloc(spectralComplex));
    SL3D_CUDA(guessNext.Alloc(spectralComplex));
  }
  if (b == nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(guess.p, a, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
  } else {
    LaunchBlend(spectralComplex, c, a, b, guess.p, stream);
    SL3D_CHECK_LAUNCH();
  }
  stageGuess = guess.p;
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::StageAdjoint(V3dState& in, const V3dState& end, double dt, int scheme, bool measured,
                                    int kind, sl3dgpu_step_info& info) {
  Flavour* f = nullptr;
  SL3D_TRY(StartStage(in, adj.scratch, dt, scheme, nullptr, &f));
  const int bw = scheme == static_cast<int>(Scheme::BackwardEuler) ? 1 : 0;
  AdjointStrainArgs sa{};
  sa.values = values;
  sa.fieldSize = fieldSize;
  sa.branches = K;
  sa.scheme = bw;
  sa.dt = dt;
  sa.itauRef = itauRef.p;
  sa.factor = factor.p;
  for (int k = 0; k < K; ++k) {
    sa.m0[k] = adj.m[k].c0.p;
    sa.m1[k] = adj.m[k].c1.p;
    sa.mr[k] = adj.m[k].r.p;
  }
  sa.d0 = adj.d.c0.p;
  sa.d1 = adj.d.c1.p;
  sa.dr = adj.d.r.p;
  sa.o0 = adj.bar.c0.p;
  sa.o1 = adj.bar.c1.p;
  sa.orr = adj.bar.r.p;
  LaunchAdjointStrainDual(sa, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(AnalyseRange(adj.bar, fixedS.p, 0, P));
  SL3D_CUDA(cudaMemcpyAsync(analysedStart.p, fixedS.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  const double2* gU = measured ? adj.gU.p : nullptr;
  const double2* gPhi = measured ? adj.gPhi.p : nullptr;
  if (measured) {
    SL3D_CUDA(cudaMemsetAsync(rhsSph.p, 0, rhsSphComplex * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(rhsTor.p, 0, std::max<long long>(rhsTorComplex, 1) * sizeof(double2), stream));
    LaunchSurfaceDual(geo, gU, gPhi, rhsSph.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_TRY(SolveColumns(*f, rhsSph.p, rhsTor.p));
    SL3D_CUDA(cudaMemcpyAsync(adj.qSph.p, rhsSph.p, rhsSphComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                              stream));
    if (rhsTorComplex > 0)
      SL3D_CUDA(cudaMemcpyAsync(adj.qTor.p, rhsTor.p, rhsTorComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                                stream));
    passAddSph = adj.qSph.p;
    passAddTor = adj.qTor.p;
  }
  SL3D_CUDA(cudaMemsetAsync(s.p, 0, spectralComplex * sizeof(double2), stream));
  // the start: zero, and the extrapolation of this kind's last two dual
  // strains when the sweep has them (kept only if its first pass is better)
  stageGuess = nullptr;
  if (adj.count[kind] >= 2) SL3D_TRY(ArmGuess(adj.before[kind].p, adj.last[kind].p, 2.0));
  else if (adj.count[kind] == 1) SL3D_TRY(ArmGuess(adj.last[kind].p, nullptr, 0.0));
  info = sl3dgpu_step_info{};
  int rc = SL3DGPU_OK;
  if (options.precision == 1) {
    LaunchCast(values, weight.p, weight32.p, stream);
    SL3D_CHECK_LAUNCH();
    rc = ConvergeMixed(*f, nullptr, info);
  } else {
    rc = Converge(*f, nullptr, info);
  }
  passAddSph = passAddTor = nullptr;
  SL3D_TRY(rc);
  if (grid->emulateFp64) SL3D_TRY(grid->TensorCoreStatus(stream));
  if (!info.converged) {
    SetError("v3d adjoint: a stage's transposed fixed point did not converge");
    return SL3DGPU_ERR_UNCONVERGED;
  }
  std::swap(adj.before[kind], adj.last[kind]);
  SL3D_CUDA(cudaMemcpyAsync(adj.last[kind].p, s.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  ++adj.count[kind];
  // zeta = Syn Str z, the converged iterate's synthesis
  SL3D_TRY(SynthesiseRange(s.p, dGrid, 0, P));
  // the load's dual: u^T (F An(d-bar + W zeta) + S^T g)
  SL3D_CUDA(cudaMemcpyAsync(analysed.p, fixedS.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  SL3D_TRY(AnalyseWeighted(dGrid, weight.p, analysed.p));
  SL3D_CUDA(cudaMemsetAsync(rhsSph.p, 0, rhsSphComplex * sizeof(double2), stream));
  SL3D_CUDA(cudaMemsetAsync(rhsTor.p, 0, std::max<long long>(rhsTorComplex, 1) * sizeof(double2), stream));
  LaunchForces(geo, analysed.p, rhsSph.p, rhsTor.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchSurfaceDual(geo, gU, gPhi, rhsSph.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchLoadDual(geo, f->units.p, f->unitOffset.p, rhsSph.p, adj.sigma.p, stream);
  SL3D_CHECK_LAUNCH();
  LaunchLoadDual(geo, f->tideUnits.p, f->unitOffset.p, rhsSph.p, adj.tide.p, stream);  // the tide channel's
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(ForwardFields(in, end));
  // the start's memory and strain duals, the gradient
  AdjointMemoryArgs ma{};
  ma.values = values;
  ma.fieldSize = fieldSize;
  ma.nphi = grid->nphi;
  ma.branches = K;
  ma.scheme = bw;
  ma.dt = dt;
  ma.muBranch = muBranch.p;
  ma.itauRef = itauRef.p;
  ma.factor = factor.p;
  ma.nodeVolume = nodeVolume.p;
  ma.colWeight = colWeight.p;
  for (int k = 0; k < K; ++k) {
    ma.m0[k] = adj.m[k].c0.p;
    ma.m1[k] = adj.m[k].c1.p;
    ma.mr[k] = adj.m[k].r.p;
    ma.s0[k] = adj.startM[k].c0.p;
    ma.s1[k] = adj.startM[k].c1.p;
    ma.sr[k] = adj.startM[k].r.p;
  }
  ma.d0 = adj.d.c0.p;
  ma.d1 = adj.d.c1.p;
  ma.dr = adj.d.r.p;
  ma.z0 = dGrid.c0.p;
  ma.z1 = dGrid.c1.p;
  ma.zr = dGrid.r.p;
  ma.a0 = adj.startD.c0.p;
  ma.a1 = adj.startD.c1.p;
  ma.ar = adj.startD.r.p;
  ma.b0 = adj.endD.c0.p;
  ma.b1 = adj.endD.c1.p;
  ma.br = adj.endD.r.p;
  ma.grad = adj.grad.p;
  LaunchAdjointMemory(ma, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// One tangent-linear stage beside its forward stage (in -> end, already
// stepped): the tangent memory's decay and the fixed force of it and of W'
// d_end, the tangent solve (the step's own iteration from a zero strain,
// the tangent load in the load channel), the tangent end strain and the
// memory's advance.
int Viscoelastic3DGpu::TangentStage(V3dState& in, const V3dState& end, double dt, int scheme,
                                    const double2* loadDot, sl3dgpu_step_info& info) {
  Flavour* f = nullptr;
  SL3D_TRY(StartStage(in, adj.scratch, dt, scheme, nullptr, &f));
  SL3D_TRY(ForwardFields(in, end));
  TangentArgs ta{};
  ta.values = values;
  ta.fieldSize = fieldSize;
  ta.branches = K;
  ta.scheme = scheme == static_cast<int>(Scheme::BackwardEuler) ? 1 : 0;
  ta.dt = dt;
  ta.muBranch = muBranch.p;
  ta.itauRef = itauRef.p;
  ta.factor = factor.p;
  ta.direction = tan.direction.p;
  for (int k = 0; k < K; ++k) {
    ta.m0[k] = tan.m[k].c0.p;
    ta.m1[k] = tan.m[k].c1.p;
    ta.mr[k] = tan.m[k].r.p;
    ta.s0[k] = adj.startM[k].c0.p;
    ta.s1[k] = adj.startM[k].c1.p;
    ta.sr[k] = adj.startM[k].r.p;
  }
  ta.t0 = tan.d.c0.p;
  ta.t1 = tan.d.c1.p;
  ta.tr = tan.d.r.p;
  ta.a0 = adj.startD.c0.p;
  ta.a1 = adj.startD.c1.p;
  ta.ar = adj.startD.r.p;
  ta.b0 = adj.endD.c0.p;
  ta.b1 = adj.endD.c1.p;
  ta.br = adj.endD.r.p;
  ta.f0 = tan.fixed.c0.p;
  ta.f1 = tan.fixed.c1.p;
  ta.fr = tan.fixed.r.p;
  LaunchTangent(ta, stream);
  SL3D_CHECK_LAUNCH();
  SL3D_TRY(AnalyseRange(tan.fixed, fixedS.p, 0, P));
  SL3D_CUDA(cudaMemcpyAsync(analysedStart.p, fixedS.p, spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            stream));
  SL3D_CUDA(cudaMemsetAsync(s.p, 0, spectralComplex * sizeof(double2), stream));
  stageGuess = nullptr;
  info = sl3dgpu_step_info{};
  if (options.precision == 1) {
    LaunchCast(values, weight.p, weight32.p, stream);
    SL3D_CHECK_LAUNCH();
    SL3D_TRY(ConvergeMixed(*f, loadDot, info));
  } else {
    SL3D_TRY(Converge(*f, loadDot, info));
  }
  if (grid->emulateFp64) SL3D_TRY(grid->TensorCoreStatus(stream));
  if (!info.converged) {
    SetError("v3d tangent: a stage's tangent solve did not converge");
    return SL3DGPU_ERR_UNCONVERGED;
  }
  SL3D_TRY(SynthesiseRange(s.p, tan.d, 0, P));
  ta.finish = true;
  LaunchTangent(ta, stream);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::TangentRun(const double* times, int nodes, int scheme, const double* loads,
                                  const double* direction, const double* loadDirections, double* u, double* phi,
                                  sl3dgpu_step_info* infos) {
  if (staticMode || ocean.on || options.solver != 0) {
    SetError("v3d tangent: built for the fixed-point step (solver 0, FP64 or mixed) without an ocean");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (nodes < 1 || times == nullptr || loads == nullptr || scheme < 0 || scheme > 2) {
    SetError("v3d tangent: at least one node, times, loads and a scheme of 0, 1 or 2");
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (int k = 1; k < nodes; ++k)
    if (!(times[k] >= times[k - 1])) {
      SetError("v3d: node times must not decrease");
      return SL3DGPU_ERR_ARGUMENT;
    }
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  SL3D_TRY(AllocAdjoint());
  if (!tan.ready) {
    tan.m.resize(K);
    tan.hold.resize(K);
    for (int k = 0; k < K; ++k) {
      SL3D_CUDA(tan.m[k].Alloc(values));
      SL3D_CUDA(tan.hold[k].Alloc(values));
    }
    SL3D_CUDA(tan.d.Alloc(values));
    SL3D_CUDA(tan.fixed.Alloc(values));
    SL3D_CUDA(tan.direction.Alloc(values));
    SL3D_CUDA(tan.load0.Alloc(lm));
    SL3D_CUDA(tan.load1.Alloc(lm));
    SL3D_CUDA(tan.loadMid.Alloc(lm));
    SL3D_TRY(AllocState(tan.first));
    SL3D_TRY(AllocState(tan.end));
    tan.ready = true;
  }
  if (direction)
    SL3D_CUDA(cudaMemcpyAsync(tan.direction.p, direction, values * sizeof(double), cudaMemcpyHostToDevice, stream));
  else
    SL3D_CUDA(cudaMemsetAsync(tan.direction.p, 0, values * sizeof(double), stream));
  auto zeroTensor = [&](GridTensor& t) -> int {
    SL3D_CUDA(cudaMemsetAsync(t.c0.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(t.c1.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(t.r.p, 0, values * sizeof(double), stream));
    return SL3DGPU_OK;
  };
  for (int k = 0; k < K; ++k) SL3D_TRY(zeroTensor(tan.m[k]));
  SL3D_TRY(zeroTensor(tan.d));
  SL3D_TRY(ZeroState(tan.prev));
  SL3D_TRY(zeroTensor(tan.prev.strain));
  for (int k = 0; k < nodes; ++k) {
    const double* l1 = loads + 2 * lm * k;
    const double* l0 = k > 0 ? loads + 2 * lm * (k - 1) : l1;
    const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
    SL3D_CUDA(cudaMemcpyAsync(sigma0.p, l0, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    SL3D_CUDA(cudaMemcpyAsync(sigma1.p, l1, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    const double2* dot0 = nullptr;
    const double2* dot1 = nullptr;
    if (loadDirections) {
      const double* t1 = loadDirections + 2 * lm * k;
      const double* t0 = k > 0 ? loadDirections + 2 * lm * (k - 1) : t1;
      SL3D_CUDA(cudaMemcpyAsync(tan.load0.p, t0, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
      SL3D_CUDA(cudaMemcpyAsync(tan.load1.p, t1, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
      dot0 = tan.load0.p;
      dot1 = tan.load1.p;
    }
    sl3dgpu_step_info info{}, tangent{};
    stageGuess = nullptr;
    if (scheme != 2 || dt == 0.0) {
      const int one = scheme == 2 ? 1 : scheme;
      SL3D_TRY(StepOnce(tan.prev, tan.end, dt, one, sigma0.p, sigma1.p, info));
      SL3D_TRY(TangentStage(tan.prev, tan.end, dt, one, dot1, tangent));
    } else {
      const double gamma = host::kSdirk2Gamma, h = gamma * dt, r = (1.0 - gamma) / gamma;
      LaunchBlend(static_cast<long long>(lm), gamma, sigma0.p, sigma1.p, sigmaMid.p, stream);
      SL3D_CHECK_LAUNCH();
      const double2* dotMid = nullptr;
      if (dot0) {
        LaunchBlend(static_cast<long long>(lm), gamma, dot0, dot1, tan.loadMid.p, stream);
        SL3D_CHECK_LAUNCH();
        dotMid = tan.loadMid.p;
      }
      sl3dgpu_step_info i1{};
      SL3D_TRY(StepOnce(tan.prev, tan.first, h, 1, sigma0.p, sigmaMid.p, i1));
      for (int b = 0; b < K; ++b) {
        SL3D_CUDA(cudaMemcpyAsync(tan.hold[b].c0.p, tan.m[b].c0.p, values * sizeof(double2), cudaMemcpyDeviceToDevice,
                                  stream));
        SL3D_CUDA(cudaMemcpyAsync(tan.hold[b].c1.p, tan.m[b].c1.p, values * sizeof(double2), cudaMemcpyDeviceToDevice,
                                  stream));
        SL3D_CUDA(cudaMemcpyAsync(tan.hold[b].r.p, tan.m[b].r.p, values * sizeof(double), cudaMemcpyDeviceToDevice,
                                  stream));
      }
      SL3D_TRY(TangentStage(tan.prev, tan.first, h, 1, dotMid, tangent));
      // the second stage's memory (1 - r) m_n + r Y1, forward and tangent
      const long long begin = lateralFirst * fieldSize, stop = static_cast<long long>(lateralEnd) * fieldSize;
      for (int b = 0; b < K; ++b) {
        if (stop > begin) {
          LaunchStageCombine(stop - begin, r, tan.prev.m[b].c0.p + begin, tan.prev.m[b].c1.p + begin,
                             tan.prev.m[b].r.p + begin, tan.first.m[b].c0.p + begin, tan.first.m[b].c1.p + begin,
                             tan.first.m[b].r.p + begin, stream);
          SL3D_CHECK_LAUNCH();
        }
        LaunchSpectralCombine(rows0 + rows1 + rowsR, P, lateralFirst, lateralEnd, r, tan.prev.mSpec[b].p,
                              tan.first.mSpec[b].p, stream);
        SL3D_CHECK_LAUNCH();
        LaunchStageCombine(values, r, tan.hold[b].c0.p, tan.hold[b].c1.p, tan.hold[b].r.p, tan.m[b].c0.p,
                           tan.m[b].c1.p, tan.m[b].r.p, stream);
        SL3D_CHECK_LAUNCH();
      }
      sl3dgpu_step_info t1{};
      SL3D_TRY(StepOnce(tan.first, tan.end, h, 1, sigmaMid.p, sigma1.p, info));
      SL3D_TRY(TangentStage(tan.first, tan.end, h, 1, dot1, t1));
      info.converged = info.converged && i1.converged;
    }
    if (infos) infos[k] = info;
    if (!info.converged) {
      SetError("v3d tangent: a step of the forward run did not converge");
      return SL3DGPU_ERR_UNCONVERGED;
    }
    if (u) SL3D_TRY(Surface(0, u + 2 * lm * k));
    if (phi) SL3D_TRY(Surface(2, phi + 2 * lm * k));
    std::swap(tan.prev, tan.end);
  }
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::AllocAdjoint() {
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  if (!adj.ready) {
    adj.m.resize(K);
    adj.hold.resize(K);
    adj.startM.resize(K);
    for (int k = 0; k < K; ++k) {
      SL3D_CUDA(adj.m[k].Alloc(values));
      SL3D_CUDA(adj.hold[k].Alloc(values));
      SL3D_CUDA(adj.startM[k].Alloc(values));
    }
    SL3D_CUDA(adj.startD.Alloc(values));
    SL3D_CUDA(adj.endD.Alloc(values));
    SL3D_CUDA(adj.d.Alloc(values));
    SL3D_CUDA(adj.bar.Alloc(values));
    SL3D_CUDA(adj.qSph.Alloc(rhsSphComplex));
    SL3D_CUDA(adj.qTor.Alloc(std::max<long long>(rhsTorComplex, 1)));
    SL3D_CUDA(adj.gU.Alloc(lm));
    SL3D_CUDA(adj.gPhi.Alloc(lm));
    SL3D_CUDA(adj.sigma.Alloc(lm));
    SL3D_CUDA(adj.tide.Alloc(lm));
    SL3D_CUDA(adj.grad.Alloc(values));
    SL3D_TRY(AllocState(adj.scratch));
    SL3D_TRY(AllocState(adj.stage));
    for (int i = 0; i < 3; ++i) {
      SL3D_CUDA(adj.last[i].Alloc(spectralComplex));
      SL3D_CUDA(adj.before[i].Alloc(spectralComplex));
    }
    adj.ready = true;
  }
  return SL3DGPU_OK;
}

int Viscoelastic3DGpu::AdjointRun(const double* times, int nodes, int scheme, int stride, const double* loads,
                                  const double* uDual, const double* phiDual, double* loadKernels,
                                  double* tideKernels, double* deltaGradient, double* objective,
                                  sl3dgpu_step_info* infos) {
  if (staticMode || ocean.on || options.solver != 0) {
    SetError("v3d adjoint: built for the fixed-point step (solver 0, FP64 or mixed) without an ocean");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (nodes < 1 || times == nullptr || loads == nullptr || loadKernels == nullptr || scheme < 0 || scheme > 2 ||
      stride < 1) {
    SetError("v3d adjoint: at least one node, times, loads, the load kernels' buffer, a scheme of 0, 1 or 2 and a "
             "record stride of at least 1");
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (int k = 1; k < nodes; ++k)
    if (!(times[k] >= times[k - 1])) {
      SetError("v3d: node times must not decrease");
      return SL3DGPU_ERR_ARGUMENT;
    }
  const int rc = AdjointSweep(times, nodes, scheme, stride, loads, uDual, phiDual, loadKernels, tideKernels,
                              deltaGradient, objective, infos);
  passAddSph = passAddTor = nullptr;
  stageGuess = nullptr;
  return rc;
}

int Viscoelastic3DGpu::AdjointSweep(const double* times, int nodes, int scheme, int stride, const double* loads,
                                    const double* uDual, const double* phiDual, double* loadKernels,
                                    double* tideKernels, double* deltaGradient, double* objective,
                                    sl3dgpu_step_info* infos) {
  const size_t lm = static_cast<size_t>(options.lmax + 1) * (options.lmax + 2) / 2;
  SL3D_TRY(AllocAdjoint());
  auto zeroTensor = [&](GridTensor& t) -> int {
    SL3D_CUDA(cudaMemsetAsync(t.c0.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(t.c1.p, 0, values * sizeof(double2), stream));
    SL3D_CUDA(cudaMemsetAsync(t.r.p, 0, values * sizeof(double), stream));
    return SL3DGPU_OK;
  };
  // the surface pairing of two coefficient arrays (l, m >= 0), m > 0 twice
  auto pair = [&](const double* a, const double* b) {
    double sum = 0.0;
    for (int l = 0; l <= options.lmax; ++l)
      for (int m = 0; m <= l; ++m) {
        const size_t i = static_cast<size_t>(l) * (l + 1) / 2 + m;
        sum += (m == 0 ? 1.0 : 2.0) * (a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1]);
      }
    return sum;
  };

  // The forward run, every node's state kept (Evolution3D::Run: node 0 the
  // instantaneous response, each later node one step under its two loads).
  std::vector<V3dState> trajectory(nodes);
  V3dState cur, zero;
  SL3D_TRY(ZeroState(cur));
  SL3D_TRY(ZeroState(zero));
  SL3D_TRY(zeroTensor(zero.strain));
  std::vector<double> surface(2 * lm);
  double objectiveSum = 0.0;
  for (int k = 0; k < nodes; ++k) {
    const double* l1 = loads + 2 * lm * k;
    const double* l0 = k > 0 ? loads + 2 * lm * (k - 1) : l1;
    const double dt = k > 0 ? times[k] - times[k - 1] : 0.0;
    sl3dgpu_step_info info{};
    SL3D_TRY(Step(cur, dt, scheme, l0, l1, &info));
    if (infos) infos[k] = info;
    if (!info.converged) {
      SetError("v3d adjoint: a step of the forward run did not converge");
      return SL3DGPU_ERR_UNCONVERGED;
    }
    if (uDual) {
      SL3D_TRY(Surface(0, surface.data()));
      objectiveSum += pair(uDual + 2 * lm * k, surface.data());
    }
    if (phiDual) {
      SL3D_TRY(Surface(2, surface.data()));
      objectiveSum += pair(phiDual + 2 * lm * k, surface.data());
    }
    if (k % stride == 0) {
      SL3D_TRY(AllocState(trajectory[k]));
      SL3D_TRY(CopyState(cur, trajectory[k]));
    }
  }
  if (objective) *objective = objectiveSum;

  // The states of a gap between two kept nodes, rebuilt by the run's own
  // steps from the kept state below when the sweep first needs one of them
  // (ForwardTrajectory3D's record stride): the kept states and one gap's
  // are held, about nodes / stride + stride states.
  std::vector<V3dState> gap(stride > 1 ? stride : 0);
  int gapBase = -1;
  auto stateAt = [&](int k, V3dState** out) -> int {
    if (k % stride == 0) {
      *out = &trajectory[k];
      return SL3DGPU_OK;
    }
    const int base = k - k % stride;
    if (base != gapBase) {
      SL3D_TRY(CopyState(trajectory[base], cur));
      for (int j = base + 1; j < std::min(base + stride, nodes); ++j) {
        sl3dgpu_step_info info{};
        SL3D_TRY(Step(cur, times[j] - times[j - 1], scheme, loads + 2 * lm * (j - 1), loads + 2 * lm * j, &info));
        if (!info.converged) {
          SetError("v3d adjoint: a step of the forward run did not converge when repeated");
          return SL3DGPU_ERR_UNCONVERGED;
        }
        V3dState& slot = gap[j - base];
        if (slot.m.empty()) SL3D_TRY(AllocState(slot));
        SL3D_TRY(CopyState(cur, slot));
      }
      gapBase = base;
    }
    *out = &gap[k - base];
    return SL3DGPU_OK;
  };

  // The transposed sweep, node by node from the last.
  for (int& c : adj.count) c = 0;
  for (int k = 0; k < K; ++k) SL3D_TRY(zeroTensor(adj.m[k]));
  SL3D_TRY(zeroTensor(adj.d));
  SL3D_CUDA(cudaMemsetAsync(adj.grad.p, 0, values * sizeof(double), stream));
  std::vector<double> kernels(2 * lm * nodes, 0.0), tides(tideKernels ? 2 * lm * nodes : 0, 0.0), sigma(2 * lm),
      tide(2 * lm);
  // a stage's load and tide duals, c of them to the node (its end load's
  // share of the stage's)
  auto addSigma = [&](int node, double c) -> int {
    SL3D_CUDA(cudaMemcpyAsync(sigma.data(), adj.sigma.p, lm * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    if (tideKernels)
      SL3D_CUDA(cudaMemcpyAsync(tide.data(), adj.tide.p, lm * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    SL3D_CUDA(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < 2 * lm; ++i) kernels[2 * lm * node + i] += c * sigma[i];
    if (tideKernels)
      for (size_t i = 0; i < 2 * lm; ++i) tides[2 * lm * node + i] += c * tide[i];
    return SL3DGPU_OK;
  };
  const bool measured = uDual != nullptr || phiDual != nullptr;
  for (int n = nodes - 1; n >= 0; --n) {
    V3dState* prevState = &zero;
    V3dState* endState = nullptr;
    if (n > 0) SL3D_TRY(stateAt(n - 1, &prevState));
    SL3D_TRY(stateAt(n, &endState));
    V3dState& prev = *prevState;
    V3dState& endAt = *endState;
    const double dt = n > 0 ? times[n] - times[n - 1] : 0.0;
    if (uDual)
      SL3D_CUDA(cudaMemcpyAsync(adj.gU.p, uDual + 2 * lm * n, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    if (phiDual)
      SL3D_CUDA(cudaMemcpyAsync(adj.gPhi.p, phiDual + 2 * lm * n, lm * sizeof(double2), cudaMemcpyHostToDevice,
                                stream));
    if (uDual == nullptr) SL3D_CUDA(cudaMemsetAsync(adj.gU.p, 0, lm * sizeof(double2), stream));
    if (phiDual == nullptr) SL3D_CUDA(cudaMemsetAsync(adj.gPhi.p, 0, lm * sizeof(double2), stream));
    sl3dgpu_step_info info{};
    if (scheme != 2 || dt == 0.0) {
      SL3D_TRY(StageAdjoint(prev, endAt, dt, scheme == 2 ? 1 : scheme, measured, 0, info));
      SL3D_TRY(addSigma(n, 1.0));
      continue;
    }
    // Sdirk2: the first stage again from the node below, under the blend
    // (1 - gamma) L_{n-1} + gamma L_n; the second stage's memory
    // M2 = (1 - r) m_{n-1} + r Y1 formed in its place.
    const double gamma = host::kSdirk2Gamma, h = gamma * dt, r = (1.0 - gamma) / gamma;
    SL3D_CUDA(cudaMemcpyAsync(sigma0.p, loads + 2 * lm * (n - 1), lm * sizeof(double2), cudaMemcpyHostToDevice,
                              stream));
    SL3D_CUDA(cudaMemcpyAsync(sigma1.p, loads + 2 * lm * n, lm * sizeof(double2), cudaMemcpyHostToDevice, stream));
    LaunchBlend(static_cast<long long>(lm), gamma, sigma0.p, sigma1.p, sigmaMid.p, stream);
    SL3D_CHECK_LAUNCH();
    // its start guess the forward's: (1 - gamma) s_{n-1} + gamma s_n
    SL3D_TRY(ArmGuess(prev.coeffs.p, endAt.coeffs.p, gamma));
    sl3dgpu_step_info first{};
    SL3D_TRY(StepOnce(prev, adj.stage, h, 1, sigma0.p, sigmaMid.p, first));
    stageGuess = nullptr;
    if (!first.converged) {
      SetError("v3d adjoint: the first stage of a forward step did not converge when repeated");
      return SL3DGPU_ERR_UNCONVERGED;
    }
    const long long begin = lateralFirst * fieldSize, end = static_cast<long long>(lateralEnd) * fieldSize;
    for (int k = 0; k < K; ++k) {
      if (end > begin) {
        LaunchStageCombine(end - begin, r, prev.m[k].c0.p + begin, prev.m[k].c1.p + begin, prev.m[k].r.p + begin,
                           adj.stage.m[k].c0.p + begin, adj.stage.m[k].c1.p + begin, adj.stage.m[k].r.p + begin,
                           stream);
        SL3D_CHECK_LAUNCH();
      }
      LaunchSpectralCombine(rows0 + rows1 + rowsR, P, lateralFirst, lateralEnd, r, prev.mSpec[k].p,
                            adj.stage.mSpec[k].p, stream);
      SL3D_CHECK_LAUNCH();
    }
    SL3D_TRY(StageAdjoint(adj.stage, endAt, h, 1, measured, 2, info));
    SL3D_TRY(addSigma(n, 1.0));
    // the combination transposed: (1 - r) of M2's dual held for m_{n-1}, r of it Y1's
    for (int k = 0; k < K; ++k) {
      for (auto [from, to, count] : {std::tuple{reinterpret_cast<double*>(adj.m[k].c0.p),
                                                reinterpret_cast<double*>(adj.hold[k].c0.p), 2 * values},
                                     std::tuple{reinterpret_cast<double*>(adj.m[k].c1.p),
                                                reinterpret_cast<double*>(adj.hold[k].c1.p), 2 * values},
                                     std::tuple{adj.m[k].r.p, adj.hold[k].r.p, values}}) {
        SL3D_CUDA(cudaMemcpyAsync(to, from, count * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        LaunchScale(count, 1.0 - r, to, stream);
        SL3D_CHECK_LAUNCH();
        LaunchScale(count, r, from, stream);
        SL3D_CHECK_LAUNCH();
      }
    }
    SL3D_TRY(StageAdjoint(prev, adj.stage, h, 1, false, 1, info));
    SL3D_TRY(addSigma(n - 1, 1.0 - gamma));
    SL3D_TRY(addSigma(n, gamma));
    for (int k = 0; k < K; ++k) {
      LaunchAxpy(2 * values, 1.0, reinterpret_cast<const double*>(adj.hold[k].c0.p),
                 reinterpret_cast<double*>(adj.m[k].c0.p), stream);
      LaunchAxpy(2 * values, 1.0, reinterpret_cast<const double*>(adj.hold[k].c1.p),
                 reinterpret_cast<double*>(adj.m[k].c1.p), stream);
      LaunchAxpy(values, 1.0, adj.hold[k].r.p, adj.m[k].r.p, stream);
      SL3D_CHECK_LAUNCH();
    }
  }
  std::copy(kernels.begin(), kernels.end(), loadKernels);
  if (tideKernels) {
    // a tide has no degree-1 part (the channel refuses one): its kernel there is none
    if (options.lmax >= 1)
      for (int n = 0; n < nodes; ++n)
        for (size_t i = 2; i < 6; ++i) tides[2 * lm * n + i] = 0.0;
    std::copy(tides.begin(), tides.end(), tideKernels);
  }
  if (deltaGradient)
    SL3D_CUDA(cudaMemcpyAsync(deltaGradient, adj.grad.p, values * sizeof(double), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu

// -- the C ABI -------------------------------------------------------------------------------------------

using namespace sl3dgpu;

struct sl3dgpu_v3d {
  Viscoelastic3DGpu op;
};
struct sl3dgpu_v3d_state {
  V3dState st;
};

extern "C" int sl3dgpu_v3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options* options,
                                  sl3dgpu_v3d** out) {
  if (layers == nullptr || options == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto h = std::make_unique<sl3dgpu_v3d>();
  SL3D_TRY(h->op.Create(layers, nlayers, *options));
  *out = h.release();
  return SL3DGPU_OK;
}

extern "C" void sl3dgpu_v3d_destroy(sl3dgpu_v3d* h) { delete h; }

extern "C" int sl3dgpu_v3d_shape(const sl3dgpu_v3d* h, int* nodes, int* ntheta, int* nphi) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (nodes) *nodes = h->op.P;
  if (ntheta) *ntheta = h->op.grid->ntheta;
  if (nphi) *nphi = h->op.grid->nphi;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_nodes(const sl3dgpu_v3d* h, double* radius, int* element) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (int p = 0; p < h->op.P; ++p) {
    if (radius) radius[p] = h->op.nodeR[p];
    if (element) element[p] = h->op.nodeElement[p];
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_lateral_range(const sl3dgpu_v3d* h, int* first, int* end) {
  if (h == nullptr || first == nullptr || end == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  *first = h->op.lateralFirst;
  *end = h->op.lateralEnd;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_node_relaxation(const sl3dgpu_v3d* h, double* itau) {
  if (h == nullptr || itau == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  // the slowest branch's reference inverse relaxation time at each node
  const auto& ref = *h->op.reference;
  for (int p = 0; p < h->op.P; ++p) {
    const size_t at = static_cast<size_t>(h->op.nodeElement[p]) * ref.points.count + h->op.nodeQ[p];
    itau[p] = ref.pointItau.empty() ? 0.0 : ref.pointItau[0][at];
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_colatitudes(const sl3dgpu_v3d* h, double* theta, double* weights) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& g = *h->op.grid;
  if (theta) std::memcpy(theta, g.theta.data(), g.theta.size() * sizeof(double));
  if (weights) std::memcpy(weights, g.weights.data(), g.weights.size() * sizeof(double));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_scales(const sl3dgpu_v3d* h, double* length, double* time, double* surface_density) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& sc = h->op.earth->scales();
  if (length) *length = sc.length;
  if (time) *time = sc.time;
  if (surface_density) *surface_density = sc.SurfaceDensity();
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_set_delta(sl3dgpu_v3d* h, const double* samples, int on_device) {
  if (h == nullptr || samples == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SetDelta(samples, on_device != 0);
}

extern "C" int sl3dgpu_v3d_zero_state(sl3dgpu_v3d* h, sl3dgpu_v3d_state** out) {
  if (h == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto s = std::make_unique<sl3dgpu_v3d_state>();
  SL3D_TRY(h->op.ZeroState(s->st));
  *out = s.release();
  return SL3DGPU_OK;
}

extern "C" void sl3dgpu_v3d_free_state(sl3dgpu_v3d_state* s) { delete s; }

extern "C" int sl3dgpu_v3d_step(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, double dt, int scheme, const double* load0,
                                const double* load1, sl3dgpu_step_info* info) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Step(state->st, dt, scheme, load0, load1, info);
}

extern "C" int sl3dgpu_v3d_step_device(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, double dt, int scheme,
                                       const double* load0, const double* load1, sl3dgpu_step_info* info) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Step(state->st, dt, scheme, load0, load1, info, true);
}

extern "C" int sl3dgpu_v3d_step_tide(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, double dt, int scheme,
                                     const double* load0, const double* load1, const double* tide0,
                                     const double* tide1, int on_device, sl3dgpu_step_info* info) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Step(state->st, dt, scheme, load0, load1, info, on_device != 0, tide0, tide1);
}

extern "C" int sl3dgpu_v3d_set_start(sl3dgpu_v3d* h, const double* coefficients, int on_device) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SetStart(coefficients, on_device != 0);
}

extern "C" int sl3dgpu_v3d_start_taken(const sl3dgpu_v3d* h) { return h == nullptr ? 0 : h->op.guessTaken; }

extern "C" int sl3dgpu_v3d_state_coefficients(const sl3dgpu_v3d* h, const sl3dgpu_v3d_state* state,
                                              const double** device, long long* count) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (device) *device = state->st.hasCoeffs ? reinterpret_cast<const double*>(state->st.coeffs.p) : nullptr;
  if (count) *count = 2 * h->op.spectralComplex;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_state_coefficients_copy(const sl3dgpu_v3d* h, const sl3dgpu_v3d_state* state,
                                                   double* device_out) {
  if (h == nullptr || state == nullptr || device_out == nullptr || !state->st.hasCoeffs) {
    SetError("v3d: null argument or a state without strain coefficients");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaMemcpyAsync(device_out, state->st.coeffs.p, h->op.spectralComplex * sizeof(double2),
                            cudaMemcpyDeviceToDevice, h->op.stream));
  SL3D_CUDA(cudaStreamSynchronize(h->op.stream));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_state_coefficients_host(const sl3dgpu_v3d* h, const sl3dgpu_v3d_state* state, double* out) {
  if (h == nullptr || state == nullptr || out == nullptr || !state->st.hasCoeffs) {
    SetError("v3d: null argument or a state without strain coefficients");
    return SL3DGPU_ERR_ARGUMENT;
  }
  SL3D_CUDA(cudaStreamSynchronize(h->op.stream));  // the legacy-stream copy does not wait for it
  SL3D_CUDA(cudaMemcpy(out, state->st.coeffs.p, h->op.spectralComplex * sizeof(double2), cudaMemcpyDeviceToHost));
  return SL3DGPU_OK;
}

// -- the open step and the grid coupling --------------------------------------------------------------

namespace {
int NeedStepOperator(const sl3dgpu_v3d* h) {
  if (h == nullptr || h->op.staticMode) {
    SetError("v3d: a step operator (not the static problem's) is required");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return SL3DGPU_OK;
}
}  // namespace

extern "C" int sl3dgpu_v3d_start_step(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, double dt, int scheme,
                                      const double* load0) {
  SL3D_TRY(NeedStepOperator(h));
  if (state == nullptr) {
    SetError("v3d: null state");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.OpenStart(state->st, dt, scheme, load0);
}

extern "C" int sl3dgpu_v3d_step_start_strain(sl3dgpu_v3d* h, double* device_out) {
  SL3D_TRY(NeedStepOperator(h));
  SL3D_TRY(h->op.OpenCheck());
  if (device_out == nullptr) {
    SetError("v3d: null output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto& op = h->op;
  SL3D_CUDA(cudaMemcpyAsync(device_out, op.s.p, op.spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                            op.stream));
  SL3D_CUDA(cudaStreamSynchronize(op.stream));
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_step_respond(sl3dgpu_v3d* h, const double* strain) {
  SL3D_TRY(NeedStepOperator(h));
  return h->op.OpenRespond(reinterpret_cast<const double2*>(strain));
}

extern "C" int sl3dgpu_v3d_step_add_channels(sl3dgpu_v3d* h, const double* load, const double* tide) {
  SL3D_TRY(NeedStepOperator(h));
  return h->op.OpenChannels(load, tide);
}

extern "C" int sl3dgpu_v3d_step_strain_of(sl3dgpu_v3d* h, double* device_out) {
  SL3D_TRY(NeedStepOperator(h));
  SL3D_TRY(h->op.OpenCheck());
  if (device_out == nullptr) {
    SetError("v3d: null output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto& op = h->op;
  return op.StrainOfSolutions(op.rhsSph.p, op.rhsTor.p, reinterpret_cast<double2*>(device_out));
}

extern "C" int sl3dgpu_v3d_step_converge(sl3dgpu_v3d* h, const double* load, const double* tide,
                                         double* device_strain, sl3dgpu_step_info* info) {
  SL3D_TRY(NeedStepOperator(h));
  auto& op = h->op;
  SL3D_TRY(op.OpenConverge(load, tide, info));
  if (device_strain != nullptr) {
    SL3D_CUDA(cudaMemcpyAsync(device_strain, op.s.p, op.spectralComplex * sizeof(double2), cudaMemcpyDeviceToDevice,
                              op.stream));
    SL3D_CUDA(cudaStreamSynchronize(op.stream));
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_step_forces(sl3dgpu_v3d* h, const double* load, const double* tide, double* out) {
  SL3D_TRY(NeedStepOperator(h));
  if (out == nullptr) {
    SetError("v3d: null output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.OpenForces(load, tide, reinterpret_cast<double2*>(out));
}

extern "C" int sl3dgpu_v3d_step_apply(sl3dgpu_v3d* h, const double* x, double* out) {
  SL3D_TRY(NeedStepOperator(h));
  if (x == nullptr || out == nullptr || x == out) {
    SetError("v3d: distinct device solutions and output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.OpenApply(reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(out));
}

extern "C" int sl3dgpu_v3d_step_solve(sl3dgpu_v3d* h, const double* forces, double* out, sl3dgpu_step_info* info) {
  SL3D_TRY(NeedStepOperator(h));
  if (forces == nullptr) {
    SetError("v3d: null forces");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.OpenSolve(reinterpret_cast<const double2*>(forces), reinterpret_cast<double2*>(out), info);
}

extern "C" int sl3dgpu_v3d_step_finish(sl3dgpu_v3d* h, const double* strain) {
  SL3D_TRY(NeedStepOperator(h));
  return h->op.OpenFinish(reinterpret_cast<const double2*>(strain));
}

extern "C" int sl3dgpu_v3d_relative_change(sl3dgpu_v3d* h, const double* next, const double* now, double* out) {
  SL3D_TRY(NeedStepOperator(h));
  if (next == nullptr || now == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Change(reinterpret_cast<const double2*>(next), reinterpret_cast<const double2*>(now), out);
}

extern "C" int sl3dgpu_v3d_layout(const sl3dgpu_v3d* h, long long* spectral, long long* grid_values,
                                  long long* spheroidal, long long* toroidal) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& op = h->op;
  if (spectral) *spectral = op.spectralComplex;
  if (grid_values) *grid_values = op.values;
  if (spheroidal) *spheroidal = op.rhsSphComplex;
  if (toroidal) *toroidal = op.rhsTorComplex;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_solution_layout(const sl3dgpu_v3d* h, int l, long long* sph_offset, int* sph_dofs,
                                           long long* tor_offset, int* tor_dofs) {
  if (h == nullptr || l < 0 || l > h->op.options.lmax) {
    SetError("v3d: a handle and 0 <= l <= lmax");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& d = h->op.degrees[l];
  if (sph_offset) *sph_offset = d.sphRhs;
  if (sph_dofs) *sph_dofs = d.sphNdof;
  if (tor_offset) *tor_offset = d.torRhs;
  if (tor_dofs) *tor_dofs = d.torNdof;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_synthesise_tensor(sl3dgpu_v3d* h, const double* spectral, double* c0, double* c1,
                                             double* r) {
  SL3D_TRY(NeedStepOperator(h));
  if (spectral == nullptr || c0 == nullptr || c1 == nullptr || r == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.TensorSynthesise(reinterpret_cast<const double2*>(spectral), reinterpret_cast<double2*>(c0),
                                reinterpret_cast<double2*>(c1), r);
}

extern "C" int sl3dgpu_v3d_analyse_tensor(sl3dgpu_v3d* h, const double* c0, const double* c1, const double* r,
                                          double* spectral) {
  SL3D_TRY(NeedStepOperator(h));
  if (spectral == nullptr || c0 == nullptr || c1 == nullptr || r == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.TensorAnalyse(reinterpret_cast<const double2*>(c0), reinterpret_cast<const double2*>(c1), r,
                             reinterpret_cast<double2*>(spectral));
}

extern "C" int sl3dgpu_v3d_degree_forces(sl3dgpu_v3d* h, const double* spectral, double* spheroidal,
                                         double* toroidal) {
  SL3D_TRY(NeedStepOperator(h));
  if (spectral == nullptr || spheroidal == nullptr || (toroidal == nullptr && h->op.rhsTorComplex > 0)) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.DegreeForces(reinterpret_cast<const double2*>(spectral), reinterpret_cast<double2*>(spheroidal),
                            reinterpret_cast<double2*>(toroidal));
}

extern "C" int sl3dgpu_v3d_strain_of_solutions(sl3dgpu_v3d* h, const double* spheroidal, const double* toroidal,
                                               double* spectral) {
  SL3D_TRY(NeedStepOperator(h));
  if (spectral == nullptr || spheroidal == nullptr || (toroidal == nullptr && h->op.rhsTorComplex > 0)) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StrainOfSolutions(reinterpret_cast<const double2*>(spheroidal),
                                 reinterpret_cast<const double2*>(toroidal), reinterpret_cast<double2*>(spectral));
}

extern "C" long long sl3dgpu_v3d_state_bytes(const sl3dgpu_v3d* h, const sl3dgpu_v3d_state* state) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null handle or state");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StateBytes(state->st);
}

extern "C" int sl3dgpu_v3d_state_save(sl3dgpu_v3d* h, const sl3dgpu_v3d_state* state, void* out, long long capacity) {
  if (h == nullptr || state == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SaveState(state->st, static_cast<char*>(out), capacity);
}

extern "C" int sl3dgpu_v3d_state_load(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, const void* in, long long bytes) {
  if (h == nullptr || state == nullptr || in == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.LoadState(state->st, static_cast<const char*>(in), bytes);
}

extern "C" int sl3dgpu_v3d_set_ocean(sl3dgpu_v3d* h, const sl3dgpu_v3d_ocean* ocean) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SetOcean(ocean);
}

extern "C" int sl3dgpu_v3d_ocean_grid(sl3dgpu_v3d* h, int* ntheta, int* nphi, double* theta, double* weights) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto& op = h->op;
  if (op.ocean.grid == nullptr) {
    SL3D_TRY(sl3dgpu_grid_create(op.options.lmax, 0, 1.0, &op.ocean.grid));
    op.ocean.ws = NewSleWorkspace();
  }
  int nt = 0, np = 0;
  SL3D_TRY(sl3dgpu_grid_shape(op.ocean.grid, &nt, &np));
  if (ntheta) *ntheta = nt;
  if (nphi) *nphi = np;
  if (theta != nullptr || weights != nullptr) {
    std::vector<double> th(nt), w(nt);
    SL3D_TRY(sl3dgpu_grid_colatitudes(op.ocean.grid, th.data(), w.data()));
    if (theta) std::copy(th.begin(), th.end(), theta);
    if (weights) std::copy(w.begin(), w.end(), weights);
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_step_ocean(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, double dt, int scheme,
                                      const double* load0, const double* load1, sl3dgpu_step_info* info) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null handle or state");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StepOcean(state->st, dt, scheme, load0, load1, info);
}

extern "C" int sl3dgpu_v3d_run_ocean(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, const double* times, int nodes,
                                     int scheme, const double* loads, double* u, double* phi, double* sea_level,
                                     double* angular_velocity, sl3dgpu_step_info* infos) {
  if (h == nullptr || state == nullptr || times == nullptr || loads == nullptr || nodes < 0) {
    SetError("v3d: null argument or negative node count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (!h->op.ocean.on) {
    SetError("v3d: no ocean is set (sl3dgpu_v3d_set_ocean)");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.RunOcean(state->st, times, nodes, scheme, loads, u, phi, sea_level, angular_velocity, infos);
}

extern "C" int sl3dgpu_v3d_step_migrating(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, double dt, int scheme,
                                          const double* ice0, const double* ice1, const double* load0,
                                          const double* load1, sl3dgpu_step_info* info) {
  if (h == nullptr || state == nullptr) {
    SetError("v3d: null handle or state");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StepMigrating(state->st, dt, scheme, ice0, ice1, load0, load1, info);
}

extern "C" int sl3dgpu_v3d_run_migrating(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, const double* times, int nodes,
                                         int scheme, const double* ice, const double* loads, double* u, double* phi,
                                         double* sea_level, double* angular_velocity, double* ocean_functions,
                                         sl3dgpu_step_info* infos) {
  if (h == nullptr || state == nullptr || times == nullptr || ice == nullptr || nodes < 0) {
    SetError("v3d: null argument or negative node count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.RunMigrating(state->st, times, nodes, scheme, ice, loads, u, phi, sea_level, angular_velocity,
                            ocean_functions, infos);
}

extern "C" int sl3dgpu_v3d_ocean_function(sl3dgpu_v3d* h, double* out) {
  if (h == nullptr || out == nullptr) {
    SetError("v3d: null handle or output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.OceanFunction(out);
}

extern "C" int sl3dgpu_v3d_sea_level(sl3dgpu_v3d* h, double* coefficients, double* angular_velocity,
                                     sl3dgpu_sle_result* result) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SeaLevel(coefficients, angular_velocity, result);
}

extern "C" int sl3dgpu_v3d_effective_love(sl3dgpu_v3d* h, int scheme, double dt, double* out) {
  if (h == nullptr || out == nullptr || scheme < 0 || scheme > 1 || !(dt >= 0.0) || h->op.staticMode) {
    SetError("v3d: effective Love numbers of a one-stage flavour (scheme 0 or 1, dt >= 0) of the step operator");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const std::vector<double>* love = nullptr;
  SL3D_TRY(h->op.EffectiveLoveOf(scheme, dt, &love));
  std::copy(love->begin(), love->end(), out);
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_run(sl3dgpu_v3d* h, sl3dgpu_v3d_state* state, const double* times, int nodes, int scheme,
                               const double* loads, double* u, double* phi, sl3dgpu_step_info* infos) {
  if (h == nullptr || state == nullptr || times == nullptr || loads == nullptr || nodes < 0) {
    SetError("v3d: null argument or negative node count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Run(state->st, times, nodes, scheme, loads, u, phi, infos);
}

extern "C" int sl3dgpu_v3d_adjoint_run(sl3dgpu_v3d* h, const double* times, int nodes, int scheme, int stride,
                                       const double* loads, const double* u_dual, const double* phi_dual,
                                       double* load_kernels, double* tide_kernels, double* delta_gradient,
                                       double* objective, sl3dgpu_step_info* infos) {
  if (h == nullptr) {
    SetError("v3d adjoint: null operator");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.AdjointRun(times, nodes, scheme, stride, loads, u_dual, phi_dual, load_kernels, tide_kernels,
                          delta_gradient, objective, infos);
}

extern "C" int sl3dgpu_v3d_tangent_run(sl3dgpu_v3d* h, const double* times, int nodes, int scheme,
                                       const double* loads, const double* delta_direction,
                                       const double* load_directions, double* u, double* phi,
                                       sl3dgpu_step_info* infos) {
  if (h == nullptr) {
    SetError("v3d tangent: null operator");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.TangentRun(times, nodes, scheme, loads, delta_direction, load_directions, u, phi, infos);
}

extern "C" int sl3dgpu_v3d_sample_volumes(const sl3dgpu_v3d* h, double* out) {
  if (h == nullptr || out == nullptr || h->op.staticMode) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& op = h->op;
  std::vector<double> volume(op.P), colw(op.grid->ntheta);
  SL3D_CUDA(cudaMemcpy(volume.data(), op.nodeVolume.p, op.P * sizeof(double), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(colw.data(), op.colWeight.p, colw.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int p = 0; p < op.P; ++p)
    for (int j = 0; j < op.grid->ntheta; ++j)
      for (int i = 0; i < op.grid->nphi; ++i)
        out[(static_cast<long long>(p) * op.grid->ntheta + j) * op.grid->nphi + i] = volume[p] * colw[j];
  return SL3DGPU_OK;
}

// Independent runs driven by a pool of host threads, one run at a time per
// thread; each operator's kernels stay on its own stream, so the runs'
// kernels overlap on the GPU. A worker's error text is kept per run and the
// first failure's text becomes the caller's.
extern "C" int sl3dgpu_v3d_run_many(int count, sl3dgpu_v3d* const* ops, sl3dgpu_v3d_state* const* states,
                                    const double* const* times, const int* nodes, int scheme,
                                    const double* const* loads, double* const* u, double* const* phi,
                                    sl3dgpu_step_info* const* infos, int threads, int* statuses) {
  if (count < 0 || (count > 0 && (ops == nullptr || states == nullptr || times == nullptr || nodes == nullptr ||
                                  loads == nullptr || statuses == nullptr))) {
    SetError("v3d: run_many needs the operators, states, times, node counts, loads and statuses");
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (int i = 0; i < count; ++i)
    for (int j = 0; j < i; ++j)
      if (ops[i] == ops[j] || states[i] == states[j]) {
        SetError("v3d: run_many's runs need distinct operators and states");
        return SL3DGPU_ERR_ARGUMENT;
      }
  int device = 0;
  SL3D_CUDA(cudaGetDevice(&device));
  const int cores = std::max(1, static_cast<int>(std::thread::hardware_concurrency()));
  const int workers = std::max(1, std::min(count, threads > 0 ? threads : cores));
  std::vector<std::string> errors(count);
  std::atomic<int> next{0};
  auto work = [&] {
    cudaSetDevice(device);
    for (int i = next.fetch_add(1); i < count; i = next.fetch_add(1)) {
      statuses[i] = sl3dgpu_v3d_run(ops[i], states[i], times[i], nodes[i], scheme, loads[i], u ? u[i] : nullptr,
                                    phi ? phi[i] : nullptr, infos ? infos[i] : nullptr);
      if (statuses[i] != SL3DGPU_OK) errors[i] = sl3dgpu_last_error();
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < workers; ++w) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  for (int i = 0; i < count; ++i)
    if (statuses[i] != SL3DGPU_OK) {
      SetError("v3d: run " + std::to_string(i) + ": " + errors[i]);
      return statuses[i];
    }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_v3d_assembled_band(sl3dgpu_v3d* h, int scheme, double dt, int toroidal, int l, double* out,
                                          long long capacity, int* n, int* kd) {
  if (h == nullptr) {
    SetError("v3d: null operator");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.AssembledBand(scheme, dt, toroidal, l, out, capacity, n, kd);
}

extern "C" int sl3dgpu_v3d_inertia_moment(sl3dgpu_v3d* h, double* out) {
  if (h == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.InertiaMoment(out);
}

extern "C" int sl3dgpu_v3d_surface(sl3dgpu_v3d* h, int component, double* out) {
  if (h == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Surface(component, out);
}

extern "C" int sl3dgpu_v3d_surface_device(sl3dgpu_v3d* h, int component, double* device_out) {
  if (h == nullptr || device_out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Surface(component, device_out, true);
}

extern "C" int sl3dgpu_v3d_state_strain(sl3dgpu_v3d* h, const sl3dgpu_v3d_state* state, double* out) {
  if (h == nullptr || state == nullptr || out == nullptr) {
    SetError("v3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StrainReference(state->st, out);
}

extern "C" void* sl3dgpu_v3d_stream(const sl3dgpu_v3d* h) { return h ? h->op.stream : nullptr; }

extern "C" int sl3dgpu_v3d_residual_history(const sl3dgpu_v3d* h, double* out, int capacity) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& v = h->op.history;
  if (out != nullptr)
    for (int i = 0; i < capacity && i < static_cast<int>(v.size()); ++i) out[i] = v[i];
  return static_cast<int>(v.size());
}

extern "C" int sl3dgpu_v3d_correction_history(const sl3dgpu_v3d* h, double* out, int capacity) {
  if (h == nullptr) {
    SetError("v3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& v = h->op.correctionHistory;
  if (out != nullptr)
    for (int i = 0; i < capacity && i < static_cast<int>(v.size()); ++i) out[i] = v[i];
  return static_cast<int>(v.size());
}

extern "C" int sl3dgpu_standard_earth(int elements, double kelvin_fraction, double kelvin_div, sl3dgpu_layer* out) {
  if (out == nullptr || elements < 4) {
    SetError("standard earth: at least four elements and an output of four layers");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto layers = host::StandardEarthLayers(elements, kelvin_fraction, kelvin_div);
  for (size_t i = 0; i < layers.size(); ++i) {
    const auto& L = layers[i];
    out[i] = sl3dgpu_layer{L.r0, L.r1, L.fluid ? 1 : 0, L.elements, L.rho0, L.rho1, L.kappa0, L.kappa1,
                           L.mu0, L.mu1, L.viscosity, L.kelvin_fraction, L.kelvin_viscosity};
  }
  return static_cast<int>(layers.size());
}

// -- the C ABI of the static perturbation problem ---------------------------------------------------

struct sl3dgpu_ep3d {
  Viscoelastic3DGpu op;
};

extern "C" int sl3dgpu_ep3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_ep3d_options* options,
                                   sl3dgpu_ep3d** out) {
  if (layers == nullptr || options == nullptr || out == nullptr) {
    SetError("ep3d: null layers, options or output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  sl3dgpu_v3d_options o{};
  o.lmax = options->lmax;
  o.ngll = options->ngll;
  o.eps = options->eps;
  o.oversampling = options->oversampling;
  o.max_iterations = 1;
  o.rtol = 1e-10;
  o.damping = 1.0;
  o.solver = 1;
  o.solve_rtol = 1e-10;
  o.solve_max_iterations = 200;
  auto h = std::make_unique<sl3dgpu_ep3d>();
  if (int st = h->op.Create(layers, nlayers, o, true); st != SL3DGPU_OK) return st;
  *out = h.release();
  return SL3DGPU_OK;
}

extern "C" void sl3dgpu_ep3d_destroy(sl3dgpu_ep3d* h) { delete h; }

extern "C" int sl3dgpu_ep3d_shape(const sl3dgpu_ep3d* h, int* nodes, int* ntheta, int* nphi) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (nodes) *nodes = h->op.P;
  if (ntheta) *ntheta = h->op.grid->ntheta;
  if (nphi) *nphi = h->op.grid->nphi;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_ep3d_nodes(const sl3dgpu_ep3d* h, double* radius, int* element) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (int p = 0; p < h->op.P; ++p) {
    if (radius) radius[p] = h->op.nodeR[p];
    if (element) element[p] = h->op.nodeElement[p];
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_ep3d_colatitudes(const sl3dgpu_ep3d* h, double* theta, double* weights) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  for (int j = 0; j < h->op.grid->ntheta; ++j) {
    if (theta) theta[j] = h->op.grid->theta[j];
    if (weights) weights[j] = h->op.grid->weights[j];
  }
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_ep3d_scales(const sl3dgpu_ep3d* h, double* length, double* modulus, double* surface_density) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& sc = h->op.earth->scales();
  if (length) *length = sc.length;
  if (modulus) *modulus = sc.Modulus();
  if (surface_density) *surface_density = sc.SurfaceDensity();
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_ep3d_set_moduli(sl3dgpu_ep3d* h, const double* d_mu, const double* d_kappa, int on_device) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SetModuli(d_mu, d_kappa, on_device != 0);
}

extern "C" int sl3dgpu_ep3d_solve_load(sl3dgpu_ep3d* h, const double* load) {
  if (h == nullptr || load == nullptr) {
    SetError("ep3d: null handle or load");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SolveLoad(load);
}

extern "C" int sl3dgpu_ep3d_respond(sl3dgpu_ep3d* h) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Respond();
}

extern "C" int sl3dgpu_ep3d_layout(const sl3dgpu_ep3d* h, long long* spheroidal, long long* toroidal) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (spheroidal) *spheroidal = h->op.rhsSphComplex;
  if (toroidal) *toroidal = h->op.rhsTorComplex;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_ep3d_force(sl3dgpu_ep3d* h, const double* x, double* out) {
  if (h == nullptr || x == nullptr || out == nullptr || x == out) {
    SetError("ep3d: a handle and distinct device solutions and output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StaticForce(reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(out));
}

extern "C" int sl3dgpu_ep3d_apply(sl3dgpu_ep3d* h, const double* x, double* out) {
  if (h == nullptr || x == nullptr || out == nullptr || x == out) {
    SetError("ep3d: a handle and distinct device solutions and output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StaticApply(reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(out));
}

extern "C" int sl3dgpu_ep3d_load_forces(sl3dgpu_ep3d* h, const double* load, double* out) {
  if (h == nullptr || load == nullptr || out == nullptr) {
    SetError("ep3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StaticLoadForces(load, reinterpret_cast<double2*>(out));
}

extern "C" int sl3dgpu_ep3d_solution(sl3dgpu_ep3d* h, double* out) {
  if (h == nullptr || out == nullptr) {
    SetError("ep3d: null argument");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.StaticSolution(reinterpret_cast<double2*>(out));
}

extern "C" int sl3dgpu_ep3d_solve_lateral(sl3dgpu_ep3d* h, const double* load, double rtol, int max_iterations,
                                          sl3dgpu_step_info* info) {
  if (h == nullptr || load == nullptr || !(rtol > 0.0) || max_iterations < 0) {
    SetError("ep3d: null handle or load, rtol > 0, max_iterations >= 0");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.SolveLateral(load, rtol, max_iterations, info);
}

extern "C" int sl3dgpu_ep3d_surface(sl3dgpu_ep3d* h, int component, double* out) {
  if (h == nullptr || out == nullptr) {
    SetError("ep3d: null handle or output");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return h->op.Surface(component, out);
}

extern "C" int sl3dgpu_ep3d_residual_history(const sl3dgpu_ep3d* h, double* out, int capacity) {
  if (h == nullptr) {
    SetError("ep3d: null handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& v = h->op.history;
  if (out != nullptr)
    for (int i = 0; i < capacity && i < static_cast<int>(v.size()); ++i) out[i] = v[i];
  return static_cast<int>(v.size());
}
