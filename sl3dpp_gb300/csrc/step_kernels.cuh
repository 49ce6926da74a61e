// Device kernels of the 3D step: the degree <-> spin-component maps (strain
// recovery and memory-force assembly), the streaming step-weight and memory
// kernels, the load channel, the convergence measure and the Anderson mixer.
// The maps, the measure and the mixer come in FP64 and FP32 (the mixed
// form's correction passes); the FP32 mixer keeps its Gram sums in FP64.
#pragma once

#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace sl3dgpu {

// Per degree l, what the maps need: its first memory node, the global node
// range its memory nodes' elements span, and where its dof maps and its
// right-hand sides / solutions start.
struct DegreeInfo {
  int firstNode;      // first memory node of the degree's element subset
  int firstGlobal;    // global node range of the carrying elements from it
  int lastGlobal;
  int sphNdof, torNdof;
  int surfaceU, surfaceV, surfacePhi, surfaceW;  // -1: none
  long long sphMap, torMap;  // offsets into the dof maps
  long long sphRhs, torRhs;  // complex offsets of the degree's [dof][l+1] blocks
};

// Constant geometry of the coupling.
struct Geometry {
  int lmax, P, ngll, np;     // degrees, memory nodes, GLL nodes, points per element
  int elements;
  const int* nodeElement;    // per memory node
  const int* nodeQ;
  const double* nodeR;
  const int* elemFirstNode;  // per element, -1 when not carrying
  const double* elemJac;
  const double* pValue;      // (np, ngll) Lagrange values at the points
  const double* pDeriv;      // (np, ngll) their xi-derivatives
  const double* pWeight;     // (np)
  const int* rowOff0;        // spin -2 row offsets (2 lmax + 2)
  const int* rowOff1;        // spin -1
  const int* rowOffR;        // spin 0 (full m range; real rows from m = 0)
  long long rows0, rows1, rowsR;
  const DegreeInfo* degrees;
  const int* sphMap;         // (g, {U, V}) per degree
  const int* torMap;         // g per degree
  // Per memory node p and GLL node i (p-major, ngll a row), in FP64 and FP32:
  // [kStrainValue] Value(q_p, i); [kStrainDeriv] r_p Deriv(q_p, i) / jac;
  // [kForceValue] jac w_q r_p Value(q_p, i); [kForceDeriv] w_q Deriv(q_p, i) r_p.
  const double* coef64[4];
  const float* coef32[4];
  int maxGlobals;  // the most global nodes a degree's carrying elements span (shared-memory sizing)
};
enum NodeCoefficient { kStrainValue = 0, kStrainDeriv = 1, kForceValue = 2, kForceDeriv = 3 };
// The node coefficient tables of a geometry, host FP64 (4 x P x ngll).
std::vector<double> NodeCoefficients(int P, int ngll, const std::vector<int>& nodeElement,
                                     const std::vector<int>& nodeQ, const std::vector<double>& nodeR,
                                     const std::vector<double>& elemJac, const std::vector<double>& value,
                                     const std::vector<double>& deriv, const std::vector<double>& weight);

// The memory force of an analysed (mu-weighted) tensor into the degree
// systems' right-hand sides (GridCoupling::SpheroidalForce/ToroidalForce).
void LaunchForces(const Geometry& g, const double2* spectral, double2* rhsSph, double2* rhsTor,
                  cudaStream_t stream);
void LaunchForces(const Geometry& g, const float2* spectral, float2* rhsSph, float2* rhsTor, cudaStream_t stream);
// The deviatoric strain of every degree's solutions into a spectral tensor
// (StrainOf: AddStrainOfSolution + DeviatoricComponents + Scatter), plus
// `add` (a tensor of the same layout) when given.
void LaunchStrain(const Geometry& g, const double2* solSph, const double2* solTor, double2* spectral,
                  cudaStream_t stream, const double2* add = nullptr);
void LaunchStrain(const Geometry& g, const float2* solSph, const float2* solTor, float2* spectral,
                  cudaStream_t stream, const float2* add = nullptr);
// The dilatation companion (GridCoupling::AddDilatationOfSolution,
// src/GridCoupling.cpp:359-398): D_lm = r dU/dr + 2 U - l(l+1) V per memory
// node into a real spin-0 spectral block (rowsR x P), every (l, m >= 0).
void LaunchDilatation(const Geometry& g, const double2* solSph, double2* scalar, cudaStream_t stream);
// GridCoupling::DilatationForce (:433-495): a weighted dilatation's force
// added onto every degree's spheroidal right-hand sides.
void LaunchDilatationForce(const Geometry& g, const double2* scalar, double2* rhsSph, cudaStream_t stream);
// x += sigma_lm K^-1 Load (+ tide_lm K^-1 Tide) for every degree
// (AddUnitChannels); sigma or tide may be null.
void LaunchAddLoad(const Geometry& g, const double2* sigma, const double* units,
                   const long long* unitOffset, double2* solSph, cudaStream_t stream,
                   const double2* tide = nullptr, const double* tideUnits = nullptr);
// Surface values of a component (0 U, 1 V, 2 phi from the spheroidal
// solutions; 3 W from the toroidal ones) for every (l, m >= 0).
void LaunchSurface(const Geometry& g, const double2* solSph, const double2* solTor, int component, double2* out,
                   cudaStream_t stream);

// The step weights, decayed memory, lateral weight and fixed force
// (StartStep's loop, src/Viscoelastic3D.cpp:1283-1354).
struct WeightsArgs {
  int branches;
  int scheme;  // 0 trapezoid, 1 backward Euler
  double dt;
  long long begin, end;  // the grid values worked on (the lateral nodes')
  long long values, fieldSize;
  const double* factor;     // exp(-delta)
  const double* muBranch;   // [k][P]
  const double* itauRef;    // [k][P]
  const double2* m0[2];     // state memory per branch: spin -2, spin -1, spin 0
  const double2* m1[2];
  const double* mr[2];
  double2* out0[2];         // decayed memory per branch (may alias the state's)
  double2* out1[2];
  double* outr[2];
  const double2* d0c0;      // start strain grid
  const double2* d0c1;
  const double* d0r;
  double* beta[2];
  double* weight;
  double2* fixed0;
  double2* fixed1;
  double* fixedr;
};
void LaunchWeights(const WeightsArgs& a, cudaStream_t stream);

// m += beta d (AdvanceMemory), per branch.
void LaunchAdvance(long long values, const double* beta, const double2* d0, const double2* d1,
                   const double* dr, double2* m0, double2* m1, double* mr, cudaStream_t stream);
// out = (1 - r) a + r out, per grid value (Sdirk2's second-stage memory).
void LaunchStageCombine(long long values, double r, const double2* a0, const double2* a1,
                        const double* ar, double2* o0, double2* o1, double* orr, cudaStream_t stream);
// out (+)= mu_k(node) m (SolveElastic's combined memory), first branch assigns.
void LaunchCombine(long long values, long long fieldSize, const double* mu, bool first,
                   const double2* m0, const double2* m1, const double* mr, double2* o0, double2* o1,
                   double* orr, cudaStream_t stream);
// The memory at the nodes outside [pLat0, pLat1) carried as spectral
// coefficients ([row][node], the three components' rows together): there
// exp(-delta) = 1, the step weights are one per node, and StartStep's decay
// and fixed force, Finish's advance and Sdirk2's stage combination act on the
// coefficients themselves (a transform of a node's grid values is exact for
// these band-limited fields, so the results are the grid route's to rounding).
struct SpectralMemoryArgs {
  int branches, scheme;
  double dt;
  long long rows;
  int P, pLat0, pLat1;
  const double* muBranch;  // [k][P]
  const double* itauRef;   // [k][P]
  const double2* in[2];    // memory coefficients per branch
  double2* out[2];         // (may alias in)
  const double2* s;        // strain coefficients: the start's, or the end's for the advance
  double2* fixedS;         // StartStep: sum_k mu_k of the decayed memory
};
// out_k = e_k in_k + alpha_k s; fixedS = sum_k mu_k out_k.
void LaunchSpectralStart(const SpectralMemoryArgs& a, cudaStream_t stream);
// out_k += beta_k s.
void LaunchSpectralAdvance(const SpectralMemoryArgs& a, cudaStream_t stream);
// fixedS = sum_k mu_k in_k (the unrelaxed solve's memory force).
void LaunchSpectralSum(const SpectralMemoryArgs& a, cudaStream_t stream);
// out = (1 - r) a + r out at the non-lateral columns.
void LaunchSpectralCombine(long long rows, int P, int pLat0, int pLat1, double r, const double2* a, double2* out,
                           cudaStream_t stream);
// out = (1 - gamma) a + gamma b over complex values, a or b null for zero.
void LaunchBlend(long long n, double gamma, const double2* a, const double2* b, double2* out, cudaStream_t stream);

// RelativeChange: max |n|^2, max |n - o|^2 and finiteness over n reals
// (complex pairs), into result[3] (FP64) on the device.
void LaunchRelativeChange(const double* next, const double* now, long long n, double* partial,
                          int partialCount, double* result, cudaStream_t stream);
void LaunchRelativeChange(const float* next, const float* now, long long n, double* partial, int partialCount,
                          double* result, cudaStream_t stream);

// Refinement glue over n reals: r = next - now rounded to FP32; s += e;
// e += r; out = FP32 of in.
void LaunchResidual32(long long n, const double* next, const double* now, float* r, cudaStream_t stream);
void LaunchAddCorrection(long long n, const float* e, double* s, cudaStream_t stream);
void LaunchAddInPlace(long long n, const float* r, float* e, cudaStream_t stream);
void LaunchCast(long long n, const double* in, float* out, cudaStream_t stream);
// out[row][c] = in[row][p0 + c] for c < count: the lateral columns of an
// every-node [row][P] array, compact.
void LaunchGatherColumns(long long rows, int P, int p0, int count, const float2* in, float2* out,
                         cudaStream_t stream);

// -- conjugate gradients (detail/LateralSolve.hpp:71-181) --------------------------------------

// y = A x for a batch of symmetric band systems (upper storage, kd + 1 rows,
// DegreeOperator::ApplyBand) on row-major right-hand sides: y = A x +
// keep y (keep 0, or -1 / +1 to take or add a force). systems[i].band and
// .rhs are element offsets.
void LaunchBandApply(const sl3dgpu_band_system* devSystems, int count, int maxRows, const double* bands,
                     const double* x, double* y, double keep, cudaStream_t stream);

// A span of one degree's [dof][l + 1] complex block for the weighted pairing.
struct PairChunk {
  long long start, end;  // complex offsets of the span
  long long degreeStart; // the degree block's first value
  int cols;              // l + 1
  int pad;
};
// LateralPair: sum over the chunks of w_m Re(a conj b), w_m = 1 at m = 0 and
// 2 above, into result[0] (FP64, fixed order). partial holds count doubles.
void LaunchPair(const double2* a, const double2* b, const PairChunk* chunks, int count, double* partial,
                double* result, cudaStream_t stream);
// y += alpha x; y = x + beta y; out = a - b (n reals).
void LaunchAxpy(long long n, double alpha, const double* x, double* y, cudaStream_t stream);
void LaunchXpby(long long n, const double* x, double beta, double* y, cudaStream_t stream);
void LaunchSub(long long n, const double* a, const double* b, double* out, cudaStream_t stream);

// The Anderson mixer's sweeps (AndersonMixer.hpp:65-219), on vectors of
// reals T with the Gram sums in FP64. The history columns (the differences
// dF, dG) are stored as MixHistory<T>: FP64 for the FP64 form; BF16 for the
// FP32 correction, whose least squares then runs on the rounded columns
// (the Gram matrix is that of the stored vectors, the mix uses the same
// ones) -- the pass's own residual stays FP32 and decides convergence.
template <class T>
struct MixHistory {
  using type = T;
};
template <>
struct MixHistory<float> {
  using type = __nv_bfloat16;
};

template <class T>
struct MixerArgsT {
  using H = typename MixHistory<T>::type;
  long long n;
  int m, slot, memory;
  T* x;
  const T* gx;
  T* xPrev;
  T* fPrev;
  H** dG;  // device array of memory pointers
  H** dF;
  double* partial;  // blocks x 2 x 8
  int blocks;
  double* gram;     // memory x memory
  double* gamma;    // m (+1 status)
  // Under a CUDA graph the pass's mixer work is decided on the device: live
  // points at a CorrectionControl's {action, m, slot}, the kernels taking
  // m and slot from it and doing nothing unless the action is theirs (the
  // template history count is then the mixer's memory, the runtime m <= it).
  const int* live = nullptr;
};
using MixerArgs = MixerArgsT<double>;
constexpr int kMixMaxMemory = 16;  // the most history columns; sums hold 2 x this
void LaunchMixerFirst(const MixerArgsT<double>& a, cudaStream_t stream);
void LaunchMixerFirst(const MixerArgsT<float>& a, cudaStream_t stream);
// An update's device part: the history sweep and its reduction to the new
// Gram column (sums[0..m)) and right-hand side (sums[8..8+m)); then, after
// the host's MixerSolve has put gamma (m values and a status) in a.gamma,
// the mix.
void LaunchMixerSweep(const MixerArgsT<double>& a, double* sums, cudaStream_t stream);
void LaunchMixerMix(const MixerArgsT<double>& a, cudaStream_t stream);
void LaunchMixerSweep(const MixerArgsT<float>& a, double* sums, cudaStream_t stream);
void LaunchMixerMix(const MixerArgsT<float>& a, cudaStream_t stream);
// The update's small least-squares solve on the host (FP64): the Gram
// matrix's slot column from the sums, then gamma by SymmetricLstsq
// (gamma[m] = 1 on success, 0 when it failed and the mix takes the plain
// step). gram: memory x memory, kept by the caller.
bool MixerSolve(double* gram, int m, int slot, int memory, const double* sums, double* gamma);
// The same on the device, one FP64 warp, ordered on the stream: gram
// (memory x memory, device) updated from sums (device), gamma (m values and
// the status) written for the mix. No host round trip.
void LaunchMixerGram(double* gram, int m, int slot, int memory, const double* sums, double* gamma,
                     cudaStream_t stream, const int* live = nullptr, bool cholesky = false);

// -- the FP32 correction's loop on the device (a CUDA graph's while node) -------------------------

// What a pass's mixer kernels do: nothing (the loop stops), the plain step
// (the next iterate copied over the iterate), the mixer's first call, an update.
constexpr int kLiveStop = 0, kLiveCopy = 1, kLiveFirst = 2, kLiveUpdate = 3;
constexpr int kCorrectionHistory = 1024;
// The loop's state in device memory: the correction loop of the mixed form
// (its host form in step.cu, Viscoelastic3DGpu::Correct) decided pass by
// pass by CorrectionControlKernel. The first three ints are the mixer
// kernels' `live` view.
struct CorrectionControl {
  int action, m, slot;
  int iteration, first, mixing, firstMix, count, memory, maxIterations;
  int fresh, status, resetGram, historyCount;
  double tolerance, rate, previous;
  double history[kCorrectionHistory];
};
// After a pass's relative change (result: scale, diff, finite flag): the
// change recorded, the stopping test, the switch to mixing, the pass's
// mixer action, and the while node's condition (continue while not
// converged, finite and within the pass budget).
void LaunchCorrectionControl(CorrectionControl* c, const double* result, cudaGraphConditionalHandle handle,
                             cudaStream_t stream);
// to = from where the pass's action is the plain step.
void LaunchCopyIfPlain(const CorrectionControl* c, const float2* from, float2* to, long long n, cudaStream_t stream);
// The mixer's Gram matrix zeroed when the loop switched to mixing.
void LaunchGramResetIf(CorrectionControl* c, double* gram, int memory, cudaStream_t stream);
// The mixer's count and slot moved on after an update.
void LaunchMixerAdvanceIf(CorrectionControl* c, cudaStream_t stream);

// -- the discrete adjoint of the step (adjoint_kernels.cu) ---------------------------------------
//
// Duals are carried in the pairings under which the force assembly of an
// analysed tensor is the transpose of the strain synthesis of a solution:
// grid tensors in the energy pairing sum_p rho_p r_p^2 sum_x w_x [4 Re(a0 b0*)
// + 8 Re(a1 b1*) + 12 ar br] (rho_p the radial quadrature weight jac w_q of
// memory node p, w_x the colatitude weight times 2 pi / nphi, spins -2, -1, 0),
// solution columns in sum w_m Re(a b*) with w_m = 1 at m = 0 and 2 above,
// surface coefficients likewise (the L2 pairing of real fields on the unit
// sphere).

// sol[surface U dof] += u_lm and sol[surface phi dof] += phi_lm (S^T of the
// surface reads); either array may be null.
void LaunchSurfaceDual(const Geometry& g, const double2* u, const double2* phi, double2* solSph,
                       cudaStream_t stream);
// out_lm = sum over the spheroidal dofs of units_l[dof] rhs[dof][m] (the
// transpose of the load channel x += sigma_lm units_l).
void LaunchLoadDual(const Geometry& g, const double* units, const long long* unitOffset, const double2* rhsSph,
                    double2* out, cudaStream_t stream);
// out = dD + sum_k beta_k mD_k over a grid tensor (the end strain's dual:
// its own and the memory advance's), beta_k the stage's weight at every
// grid value.
struct AdjointStrainArgs {
  long long values, fieldSize;
  int branches, scheme;
  double dt;
  const double* itauRef;    // [k][P]
  const double* factor;     // exp(-delta) per grid value
  const double2* m0[2];
  const double2* m1[2];
  const double* mr[2];
  const double2 *d0, *d1;
  const double* dr;
  double2 *o0, *o1;
  double* orr;
};
void LaunchAdjointStrainDual(const AdjointStrainArgs& a, cudaStream_t stream);
// Per grid value, the stage's memory duals and the log-viscosity gradient:
// M_k = mD_k + mu_k zeta; mD_k = e_k M_k (the start memory's dual); dD =
// sum_k alpha_k M_k (the start strain's dual); grad += rho r^2 w_x sum_k
// -h_k [e_k' <M_k, m_k> + alpha_k' <M_k, d_start> + beta_k' <M_k, d_end>]
// (h_k = dt itau_ref exp(-delta), primes d/dh, <,> the energy metric).
struct AdjointMemoryArgs {
  long long values, fieldSize;
  int nphi, branches, scheme;
  double dt;
  const double* muBranch;   // [k][P]
  const double* itauRef;    // [k][P]
  const double* factor;     // exp(-delta) per grid value
  const double* nodeVolume; // rho_p r_p^2 per memory node
  const double* colWeight;  // w_theta 2 pi / nphi per colatitude
  double2* m0[2];           // memory duals per branch, updated in place
  double2* m1[2];
  double* mr[2];
  double2 *d0, *d1;         // the strain dual, overwritten
  double* dr;
  const double2 *z0, *z1;   // zeta: the strain synthesis of the stage's dual solution
  const double* zr;
  const double2* s0[2];     // the stage's start memory per branch
  const double2* s1[2];
  const double* sr[2];
  const double2 *a0, *a1;   // the start strain
  const double* ar;
  const double2 *b0, *b1;   // the end strain
  const double* br;
  double* grad;             // dJ / d delta per grid value, accumulated
};
void LaunchAdjointMemory(const AdjointMemoryArgs& a, cudaStream_t stream);
// y *= a (n reals).
void LaunchScale(long long n, double a, double* y, cudaStream_t stream);

// The tangent-linear stage (TangentLinearSolver3D's discrete run) along a
// log-viscosity direction p: h' = -h p, e.g. e' = (de/dh) h'. Start: the
// tangent memory's decay tm~_k = e_k tm_k + alpha_k td_start + e'_k m_k +
// alpha'_k d_start, in place, and its fixed force sum_k mu_k tm~_k + W' d_end
// (W' = sum_k mu_k beta'_k) into `fixed`. Finish (finish = true): tm_k =
// tm~_k + beta_k td_end + beta'_k d_end, in place.
struct TangentArgs {
  long long values, fieldSize;
  int branches, scheme;
  double dt;
  bool finish;
  const double* muBranch;   // [k][P]
  const double* itauRef;    // [k][P]
  const double* factor;     // exp(-delta)
  const double* direction;  // p per grid value
  double2* m0[2];           // tangent memory per branch, in place
  double2* m1[2];
  double* mr[2];
  const double2 *t0, *t1;   // the tangent strain: the start's (start) or the end's (finish)
  const double* tr;
  const double2* s0[2];     // the stage's start memory
  const double2* s1[2];
  const double* sr[2];
  const double2 *a0, *a1;   // the start strain
  const double* ar;
  const double2 *b0, *b1;   // the end strain
  const double* br;
  double2 *f0, *f1;         // the fixed force (start)
  double* fr;
};
void LaunchTangent(const TangentArgs& a, cudaStream_t stream);

}  // namespace sl3dgpu
