/*
 * sl3dgpu — the C ABI of the GB300-native 3D viscoelastic hot path of sl3dpp.
 *
 * Plain C: opaque handles, pointers and sizes, int status codes, a CUDA stream
 * passed as void*. Every entry point names the reference interface it replaces
 * (file:line within the sl3dpp source tree). Status codes: SL3DGPU_OK (0);
 * a positive LAPACK-style info for a failed factorisation; negative codes for
 * errors, whose text sl3dgpu_last_error() returns (per thread).
 *
 * Layouts. "Reference layout" is the reference's own: band storage as
 * LAPACK's (include/sl3dpp/detail/BandSolvers.hpp:24-49), right-hand sides
 * column-major; spin-N coefficients at l^2 - N^2 + (m + l), real spin-0 ones
 * at l(l+1)/2 + m (include/sl3dpp/SurfaceGrid.hpp:110-118, 191-200); grid
 * values colatitude-major. Batched device calls keep right-hand sides
 * row-major (dof-major, columns fastest), the layout the kernels coalesce on.
 */
#ifndef SL3DGPU_H
#define SL3DGPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SL3DGPU_OK = 0,
  SL3DGPU_ERR_ARGUMENT = -1,   /* std::invalid_argument in the reference */
  SL3DGPU_ERR_CUDA = -2,       /* a CUDA call failed */
  SL3DGPU_ERR_RUNTIME = -3,    /* std::runtime_error in the reference */
  SL3DGPU_ERR_UNCONVERGED = -4, /* an iteration ended without converging */
  SL3DGPU_ERR_WAIT = -5        /* a device-side wait ran out of its budget */
};

/* The last error's text on this thread. */
const char* sl3dgpu_last_error(void);
/* Library version string. */
const char* sl3dgpu_version(void);

/* Device memory for callers without a CUDA toolchain of their own (the C++
 * classes' device buffers): allocate (*out NULL for 0 bytes), free, and a
 * synchronous copy between any two of host and device memory. */
int sl3dgpu_device_alloc(long long bytes, void** out);
int sl3dgpu_device_free(void* p);
int sl3dgpu_device_copy(void* dst, const void* src, long long bytes);

/* ---- band solvers (include/sl3dpp/detail/BandSolvers.hpp:24-49) -----------
 * Host-pointer drop-ins of detail::BandCholeskyFactor / BandCholeskySolve /
 * BandLuFactor / BandLuSolve (src/BandSolvers.cpp:23-139): the same storage,
 * pivots (zero-based) and info returns, computed on the GPU. */
int sl3dgpu_band_cholesky_factor(double* ab, int n, int kd);
int sl3dgpu_band_cholesky_solve(const double* ab, int n, int kd, double* b, int nrhs);
int sl3dgpu_band_lu_factor(double* ab, int n, int kl, int ku, int* pivots);
int sl3dgpu_band_lu_solve(const double* ab, int n, int kl, int ku, const int* pivots,
                          double* b, int nrhs);

/* One system of a device batch: every degree's system solved in one launch
 * (DegreeOperator::BeginSolve/FinishSolve, src/DegreeOperator.cpp:861-901;
 * ToroidalOperator::BeginSolve/FinishSolve, src/ToroidalOperator.cpp). */
typedef struct sl3dgpu_band_system {
  int n;            /* order */
  int kl, ku;       /* sub- and superdiagonals; Cholesky reads ku as kd */
  int nrhs;         /* right-hand sides of a solve */
  long long band;   /* offset (doubles) of the band in the batch's band array */
  long long pivots; /* offset (ints) of the LU pivots */
  long long rhs;    /* offset (doubles) of the n x nrhs right-hand sides, row-major */
  long long scale;  /* offset (doubles) of the symmetric diagonal scaling, -1 none */
  int pinned0, pinned1; /* dofs pinned to zero (identity rows), -1 none */
} sl3dgpu_band_system;

/* Factorise a batch in place (device pointers), Cholesky (lu = 0) or LU with
 * partial pivoting (lu = 1); info[i] receives system i's LAPACK-style info. */
int sl3dgpu_band_factor_batch(const sl3dgpu_band_system* dev_systems,
                              const sl3dgpu_band_system* host_systems, int count,
                              double* bands, int* pivots, int* info, int lu, void* stream);
/* The work items of a batch solve: (system, first column) pairs, one per 64
 * right-hand sides; returns their count (items may be NULL to ask). */
int sl3dgpu_band_work_items(const sl3dgpu_band_system* host_systems, int count, int* items,
                            int capacity);
/* Solve a factorised batch in place on row-major right-hand sides. */
int sl3dgpu_band_solve_batch(const sl3dgpu_band_system* dev_systems,
                             const sl3dgpu_band_system* host_systems, int count,
                             const int* dev_items, int item_count, const double* bands,
                             const int* pivots, double* rhs, const double* scales, int lu,
                             void* stream);
/* The same Cholesky solves in FP32 (float bands, right-hand sides and
 * scales; the systems' offsets count floats), optionally over row windows:
 * dev_windows holds {lo, hi} per system, the right-hand side being zero
 * outside rows lo..hi. mode 0: every row (dev_windows NULL); 1: both
 * substitutions over rows lo..n-1 only (rows below lo are left as they
 * are); 2: the backward substitution's rows 0..lo-1, after a mode-1 solve,
 * from the solution at rows lo..lo+kd-1. Modes 1 then 2 give mode 0's
 * solution. (The mixed-precision step's correction passes, whose forces reach
 * a band of rows; no reference counterpart: LAPACK dpbtrs solves every row.) */
int sl3dgpu_band_solve_batch_f32(const sl3dgpu_band_system* dev_systems,
                                 const sl3dgpu_band_system* host_systems, int count,
                                 const int* dev_items, int item_count, const float* bands,
                                 float* rhs, const float* scales, const int* dev_windows,
                                 int mode, void* stream);

/* A banded Cholesky solve (the factor from sl3dgpu_band_cholesky_factor,
 * LAPACK upper storage, and n x nrhs column-major right-hand sides,
 * overwritten by the solution) on DEVICE pointers that allocates no device
 * memory: its scratch is a fixed 2^19-double (4 MiB) array in the library,
 * held by every GPU that loads it. No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc (their device memory is owned by
 * another allocator or a fixed arena, or a driver allocation is not
 * acceptable on their loop). Larger n x nrhs is refused
 * (SL3DGPU_ERR_ARGUMENT); the first call on a device looks the array's
 * address up and should come before any stream capture; calls that overlap
 * on the GPU race on the shared array. */
int sl3dgpu_band_cholesky_solve_noalloc(const double* ab, int n, int kd, double* b, int nrhs,
                                        void* stream);

/* ---- the surface grid (include/sl3dpp/SurfaceGrid.hpp:58-287) ---------------
 * A Gauss-Legendre grid for degrees to lmax and spins to nmax, oversampled
 * by `oversampling` (band L' = ceil(oversampling lmax): L' + 1 colatitudes,
 * the smallest 2^a 3^b 5^c >= 2 L' + 1 longitudes from zero). */
typedef struct sl3dgpu_grid sl3dgpu_grid;
int sl3dgpu_grid_create(int lmax, int nmax, double oversampling, sl3dgpu_grid** out);
void sl3dgpu_grid_destroy(sl3dgpu_grid* grid);
int sl3dgpu_grid_shape(const sl3dgpu_grid* grid, int* ntheta, int* nphi);
/* SurfaceGrid::LMax (SurfaceGrid.hpp): the grid's degree bound, -1 for a null grid. */
int sl3dgpu_grid_lmax(const sl3dgpu_grid* grid);
/* The grid's FP64 Legendre contractions: 0 on the FP64 units, 1 emulated on
 * the tensor cores (seven BF16 slices a value under a power-of-two scale per
 * row and column, exact FP32 products, levels joined in FP64: about 49 bits
 * of each operand; depths beyond 448 stay on the FP64 units). */
int sl3dgpu_grid_set_fp64_emulation(sl3dgpu_grid* grid, int on);
/* Host copies of the colatitudes and their Gauss-Legendre weights. */
int sl3dgpu_grid_colatitudes(const sl3dgpu_grid* grid, double* theta, double* weights);
/* SurfaceGrid::SynthesiseSpinBatch / ExpandSpinBatch (SurfaceGrid.hpp:217-253):
 * `count` spin-N fields end to end, device pointers, complex values as
 * (re, im) pairs, reference layouts. */
int sl3dgpu_synthesise_spin_batch(sl3dgpu_grid* grid, int N, const double* coeffs, int count,
                                  double* fields, void* stream);
int sl3dgpu_expand_spin_batch(sl3dgpu_grid* grid, int N, const double* fields, int count,
                              double* coeffs, void* stream);
/* The Legendre stage alone of SurfaceGrid's transforms (SurfaceGrid.hpp:217-253,
 * the contraction inside Synthesise/Expand), in the device layouts: spin-N
 * coefficients [row][count] complex (rows in (m, l) order, m from -lmax, or
 * m >= 0 for a real spin-0 field) <-> spectra [m][colatitude][count]
 * complex. fp32 = 0: FP64 (the FP64 units, or the tensor-core emulation the
 * grid is set to); 1: FP32 buffers through the 3xTF32 tensor-core
 * contraction of the mixed form's correction passes. */
int sl3dgpu_legendre_device(sl3dgpu_grid* grid, int N, int real, int analysis, int fp32, const void* in,
                            int count, void* out, void* stream);
/* SurfaceGrid::SynthesiseBatch / ExpandBatch (SurfaceGrid.hpp:164-185): real
 * spin-0 fields from and to m >= 0 coefficients. */
int sl3dgpu_synthesise_batch(sl3dgpu_grid* grid, const double* coeffs, int count,
                             double* fields, void* stream);
int sl3dgpu_expand_batch(sl3dgpu_grid* grid, const double* fields, int count, double* coeffs,
                         void* stream);

/* ---- the sea-level equation (include/sl3dpp/SeaLevel.hpp, src/SeaLevel.cpp) -----
 * GRDSolver::SolveGeneralised (src/SeaLevel.cpp:397-736) with rotational
 * feedback None, Axial or Full, in the solver's non-dimensional units, for
 * GeneralisedForcing's channels (those of the coupled Evolution3D closure,
 * src/Evolution3D.cpp:320-333, and the load channels beside them). The body: per-degree load Love numbers h, k
 * (lmax + 1 each: the sums h_u + h_phi and k_u + k_phi the reference's
 * constructor forms, src/SeaLevel.cpp:163-171), the tangential l (may be
 * null), the tidal ht, kt, lt (may be null without a tide), surface gravity,
 * water density and the sea-floor radius; host arrays. The forcing:
 * GeneralisedForcing's channels as device arrays, each may be null -- fields
 * on the grid (directLoad, directLoadOutsideWaterBudget, solidSurfaceChange,
 * displacementLoad, potentialLoad, tangentialTraction) or (l, m >= 0)
 * complex coefficients as (re, im) pairs (the ready
 * displacement, potential, tangential and toroidal responses, the tide,
 * degrees 2 and up). The load's fixed point runs under Anderson mixing of
 * its coefficients (anderson_memory columns, 0 for plain iteration) until the
 * largest change of the ocean's sea level is at most rtol of its largest
 * value (or max_iterations). Outputs are device fields; all but
 * sea_level_change may be null. */
typedef struct sl3dgpu_sle_body {
  const double* h;
  const double* k;
  const double* l;
  const double* ht;
  const double* kt;
  const double* lt;
  double g, water_density, radius;
  /* rotational feedback (RotationalFeedback: 0 None, 1 Axial, 2 Full; the
   * tidal ht and kt required with it) and its constants, non-dimensional:
   * the rotation frequency, the polar and equatorial moments of inertia,
   * the gravitational constant, the centrifugal Love numbers h_c, k_c and
   * the inertia-trace numbers m_u, m_phi, m_c (src/SeaLevel.cpp:194-247) */
  int rotation;
  double omega, polar_moment, equatorial_moment, gravitational_constant;
  double hc, kc, m_u, m_phi, m_c;
  /* the channels' own numbers (lmax + 1 each; null where the channel is
   * unused): h_u, k_u, l_u answer a displacement load, h_phi, k_phi, l_phi a
   * potential load, h_v, k_v, l_v a tangential traction (LoveNumbers'
   * columns, src/SeaLevel.cpp:163-193; degree 0 of the l's and of the v's is
   * not read) */
  const double *h_u, *k_u, *l_u;
  const double *h_phi, *k_phi, *l_phi;
  const double *h_v, *k_v, *l_v;
} sl3dgpu_sle_body;
typedef struct sl3dgpu_sle_forcing {
  const double* direct_load;            /* field: in the water budget */
  const double* direct_load_outside;    /* field: outside it */
  const double* solid_surface_change;   /* field: a layer on the solid surface */
  const double* displacement_response;  /* coefficients */
  const double* potential_response;
  const double* tangential_response;
  const double* toroidal_response;      /* carried to the response alone */
  const double* tide;                   /* coefficients, degrees >= 2 */
  double inertia_moment_change;         /* GeneralisedForcing::inertiaMomentChange */
  double angular_momentum_change[3];    /* GeneralisedForcing::angularMomentumChange */
  const double* displacement_load;      /* field: a surface load seen through h_u, k_u, l_u */
  const double* potential_load;         /* field: one seen through h_phi, k_phi, l_phi */
  const double* tangential_traction;    /* field: a traction seen through h_v, k_v, l_v (degrees >= 1) */
} sl3dgpu_sle_forcing;
typedef struct sl3dgpu_sle_result {
  double uniform_shift; /* Response::uniformShift: the conservation's uniform part, last formed */
  double error;         /* Response::error: the last relative change of the ocean's sea level */
  int iterations;       /* Response::iterations */
  int converged;        /* Response::converged */
  double angular_velocity[3]; /* Response::angularVelocity (zero without rotational feedback) */
} sl3dgpu_sle_result;
int sl3dgpu_sle_solve(sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, const double* ocean,
                      const sl3dgpu_sle_forcing* forcing, double rtol, int max_iterations, int anderson_memory,
                      double* sea_level_change, double* displacement, double* potential,
                      double* tangential_potential, double* toroidal_potential, sl3dgpu_sle_result* result,
                      void* stream);

/* ---- the nonlinear sea-level solve: migrating shorelines
 * (GRDSolver::SolveNonlinear, include/sl3dpp/SeaLevel.hpp:418-481,
 * src/SeaLevel.cpp:970-1289) ------------------------------------------------
 * A plain fixed point from a state: each iteration the load of the current
 * ocean function and sea level change, its sea level change (the
 * generalised solve's Love numbers, static terms and rotational feedback),
 * the water budget closed by a uniform shift, and the ocean function
 * re-derived by flotation, rho_w SL - rho_i I > 0 where no land is held.
 * Fields on the grid, device pointers, non-dimensional like the body. */
typedef struct sl3dgpu_sle_state {  /* GRDSolver::State */
  const double* ice_thickness;
  const double* sea_level;            /* the sea surface over the solid surface (ocean depth) */
  const double* ocean_function;       /* 1 ocean, 0 land; flotation's for a migrating run */
  const unsigned char* forced_land;   /* nonzero: held at C = 0 (NULL: none) */
} sl3dgpu_sle_state;
typedef struct sl3dgpu_sle_nonlinear_forcing {  /* GRDSolver::NonlinearForcing; NULL: absent */
  const double* ice_thickness_change;   /* field: its grounded part loads the body from the water budget */
  const double* direct_load;            /* field: in the water budget */
  const double* direct_load_outside;    /* field: outside it */
  const double* solid_surface_change;   /* field: a layer on the solid surface */
  const double* dynamic_sea_level_change; /* field: a given change of the sea surface over the oceans */
  const double* displacement_response;  /* coefficients: ready responses */
  const double* potential_response;
  const double* tangential_response;
  const double* toroidal_response;      /* carried to the response alone */
  const double* tide;                   /* coefficients, degrees >= 2 */
  double inertia_moment_change;         /* NonlinearForcing::inertiaMomentChange */
  int hold_land;                        /* 0: the state's forced_land; 1: forced_land below (NULL: none held) */
  const unsigned char* forced_land;
} sl3dgpu_sle_nonlinear_forcing;
/* The solve (max_iterations: the reference's default 50). Outputs, any NULL:
 * the relative sea level change, displacement, potential, tangential and
 * toroidal potentials (fields); the final state's sea level and ocean
 * function (fields); the load the final state carries relative to the one
 * given, (l, m >= 0) complex coefficients (NonlinearResponse::
 * loadCoefficients). result: the last shift, error, iterations, whether it
 * converged and the angular velocity. A state without ocean is refused. */
int sl3dgpu_sle_solve_nonlinear(sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, double ice_density,
                                const sl3dgpu_sle_state* state, const sl3dgpu_sle_nonlinear_forcing* forcing,
                                double rtol, int max_iterations, double* sea_level_change, double* displacement,
                                double* potential, double* tangential_potential, double* toroidal_potential,
                                double* final_sea_level, double* final_ocean_function, double* load_coefficients,
                                sl3dgpu_sle_result* result, void* stream);
/* GRDSolver::MakeState's ocean function (src/SeaLevel.cpp:279-300) over n
 * points: 1 where rho_w sea_level - rho_i ice > 0 and no land is held. */
int sl3dgpu_sle_flotation(long long n, double water_density, double ice_density, const double* ice,
                          const double* sea_level, const unsigned char* forced_land, double* ocean_function,
                          void* stream);

/* ---- the 3D viscoelastic step (include/sl3dpp/Viscoelastic3D.hpp:79-837) -----
 * A layered Earth (SI), each field linear in radius within its layer: the
 * host-side counterpart of the reference's EarthModel + RadialMesh + Material
 * + Rheology (Maxwell, or Burgers where kelvin_fraction > 0). */
typedef struct sl3dgpu_layer {
  double r0, r1;           /* metres */
  int fluid;               /* 1: a fluid layer (mu = 0) */
  int elements;            /* radial spectral elements in the layer */
  double rho0, rho1;       /* density at r0, r1 (kg m^-3) */
  double kappa0, kappa1;   /* bulk modulus (Pa) */
  double mu0, mu1;         /* shear modulus (Pa) */
  double viscosity;        /* Pa s; 0: elastic */
  double kelvin_fraction;  /* Burgers: Kelvin modulus over mu; 0: Maxwell */
  double kelvin_viscosity; /* Burgers: Kelvin viscosity (Pa s) */
} sl3dgpu_layer;

/* Viscoelastic3D::Options (Viscoelastic3D.hpp:89-187) for the fixed-point step. */
typedef struct sl3dgpu_v3d_options {
  int lmax;
  int ngll;              /* GLL nodes per element (order + 1) */
  double eps;            /* truncation level, 1e-8 */
  double oversampling;   /* 1.5 */
  int max_iterations;    /* 40 */
  double rtol;           /* 1e-11 */
  double damping;        /* 1.0 */
  int anderson_memory;   /* 5 */
  double anderson_rate;  /* 0.5 */
  int precision;         /* 0: FP64 throughout; 1: mixed (see sl3dgpu_v3d_create) */
  double correction_rtol; /* mixed form: the finest relative change an FP32 correction iterates to, 1e-5 */
  int solver;             /* Options::StepSolver: 0 the fixed point, 1 conjugate gradients */
  double solve_rtol;      /* conjugate gradients: relative residual (preconditioned energy norm), 1e-11 */
  int solve_max_iterations; /* conjugate gradients: iteration budget, 200 */
  int warm_start;           /* 0: each step starts from the previous strain (the reference's start);
                               1: also guesses 2 s_n - s_{n-1}, the mixed form's FP32 correction
                               starting from it (the FP64 form tries it as a first pass) */
  int fp64_emulation;       /* 0: the FP64 Legendre contractions on the FP64 units; 1: emulated on
                               the tensor cores (sl3dgpu_grid_set_fp64_emulation) */
  int correction_memory;    /* mixed form: the FP32 correction's Anderson history, 0..16; 0 takes
                               anderson_memory */
} sl3dgpu_v3d_options;

/* Viscoelastic3D::StepInfo (Viscoelastic3D.hpp:357-375). */
typedef struct sl3dgpu_step_info {
  int iterations;
  double residual;
  int converged;
  int mixed_passes;
  int correction_passes; /* mixed form: FP32 correction passes (not counted in iterations) */
  int solve_iterations;  /* conjugate gradients: iterations (StepInfo::solveIterations) */
} sl3dgpu_step_info;

/* ElasticPerturbation3D (include/sl3dpp/ElasticPerturbation3D.hpp:77-225): the
 * static gravitating elastic problem under lateral perturbations dMu, dKappa
 * of the shear and bulk moduli. The coupling's nodes are the GLL nodes of
 * every solid element above the one holding the centre; the reference systems
 * are the elastic degree operators of the layered Earth. Moduli directions
 * live on the grid values (node-major, colatitude, longitude) in the model's
 * modulus unit (sl3dgpu_ep3d_scales); loads are non-dimensional surface
 * densities in the real layout l(l+1)/2 + m. The operator holds one solution:
 * SolveLoad's, Respond's or SolveLateral's, which Surface reads. */
typedef struct sl3dgpu_ep3d sl3dgpu_ep3d;
typedef struct sl3dgpu_ep3d_options {
  int lmax;
  int ngll;             /* GLL nodes per element */
  double eps;           /* truncation level, 1e-8 */
  double oversampling;  /* 1.5 */
} sl3dgpu_ep3d_options;
int sl3dgpu_ep3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_ep3d_options* options,
                        sl3dgpu_ep3d** out);
void sl3dgpu_ep3d_destroy(sl3dgpu_ep3d* op);
int sl3dgpu_ep3d_shape(const sl3dgpu_ep3d* op, int* nodes, int* ntheta, int* nphi);
int sl3dgpu_ep3d_nodes(const sl3dgpu_ep3d* op, double* radius, int* element);
int sl3dgpu_ep3d_colatitudes(const sl3dgpu_ep3d* op, double* theta, double* weights);
/* SI per model unit: length, modulus, surface density. */
int sl3dgpu_ep3d_scales(const sl3dgpu_ep3d* op, double* length, double* modulus, double* surface_density);
/* The directions (host or device arrays, either NULL for none). */
int sl3dgpu_ep3d_set_moduli(sl3dgpu_ep3d* op, const double* d_mu, const double* d_kappa, int on_device);
/* SolveLoad: the reference response to a load (host coefficients). */
int sl3dgpu_ep3d_solve_load(sl3dgpu_ep3d* op, const double* load);
/* Respond: the held solution x replaced by -K^-1 (dK) x (the Born response). */
int sl3dgpu_ep3d_respond(sl3dgpu_ep3d* op);
/* SolveLateral: (K_ref + dK) x = the load's forces by preconditioned
 * conjugate gradients from the reference response (iterations, residual and
 * convergence in info; the residuals after each iteration in the history). */
int sl3dgpu_ep3d_solve_lateral(sl3dgpu_ep3d* op, const double* load, double rtol, int max_iterations,
                               sl3dgpu_step_info* info);
/* Surface U (0), V (1) or phi (2) of the held solution, (l, m >= 0). */
int sl3dgpu_ep3d_surface(sl3dgpu_ep3d* op, int component, double* out);
int sl3dgpu_ep3d_residual_history(const sl3dgpu_ep3d* op, double* out, int capacity);
/* Force and Apply (ElasticPerturbation3D.hpp:98-130) on solutions held in
 * device memory: the spheroidal then the toroidal systems' complex values
 * (sl3dgpu_ep3d_layout's counts; degree l's block [dof][l + 1] at
 * sl3dgpu_v3d_solution_layout's offsets of the same shape), x and out
 * distinct. force: (dK) x under the set directions; apply: (K_ref + dK) x;
 * load_forces: LoadForces, the unit load vectors times a load's host
 * coefficients (spheroidal; toroidal zero); solution: the held solution
 * copied out. */
int sl3dgpu_ep3d_layout(const sl3dgpu_ep3d* op, long long* spheroidal, long long* toroidal);
int sl3dgpu_ep3d_force(sl3dgpu_ep3d* op, const double* x, double* out);
int sl3dgpu_ep3d_apply(sl3dgpu_ep3d* op, const double* x, double* out);
int sl3dgpu_ep3d_load_forces(sl3dgpu_ep3d* op, const double* load, double* out);
int sl3dgpu_ep3d_solution(sl3dgpu_ep3d* op, double* out);

/* ---- one degree's system (include/sl3dpp/DegreeOperator.hpp:94-384) -------
 * DegreeOperator (toroidal = 0) or ToroidalOperator (toroidal = 1, l >= 1) of
 * degree l on the unrelaxed material of a layered earth meshed with ngll GLL
 * nodes an element, truncated at eps (src/DegreeOperator.cpp:24-505,
 * src/ToroidalOperator.cpp): the symmetric-scaled band factorised at
 * creation on the GPU (Cholesky, or LU when a diagonal is not positive or
 * Cholesky meets a non-positive pivot: UsedCholesky). Dof(node, component)
 * over the mesh's global GLL nodes (-1: no dof), SurfaceDof, the Load and
 * Tide(power) vectors (spheroidal), Apply (K x, host), and Solve (K^-1 b in
 * place on the GPU, pinned rows zero); vectors are ndof long, nrhs columns
 * of ndof end to end. */
typedef struct sl3dgpu_degree sl3dgpu_degree;
int sl3dgpu_degree_create(const sl3dgpu_layer* layers, int nlayers, int ngll, int l, double eps, int toroidal,
                          sl3dgpu_degree** out);
void sl3dgpu_degree_destroy(sl3dgpu_degree* op);
int sl3dgpu_degree_dof_count(const sl3dgpu_degree* op);
int sl3dgpu_degree_bandwidth(const sl3dgpu_degree* op);
int sl3dgpu_degree_used_cholesky(const sl3dgpu_degree* op);
int sl3dgpu_degree_dof(const sl3dgpu_degree* op, int node, int component);
int sl3dgpu_degree_surface_dof(const sl3dgpu_degree* op, int component);
int sl3dgpu_degree_load(const sl3dgpu_degree* op, double* out);
int sl3dgpu_degree_tide(const sl3dgpu_degree* op, int power, double* out);
int sl3dgpu_degree_apply(const sl3dgpu_degree* op, const double* x, int nrhs, double* y);
/* The assembled, unscaled upper band ((kd + 1) x ndof, LAPACK storage): the
 * matrix DegreeOperator / ToroidalOperator hold before Factorise scales it
 * (src/DegreeOperator.cpp:253-474, src/ToroidalOperator.cpp), assembled on
 * the GPU. */
int sl3dgpu_degree_band(const sl3dgpu_degree* op, double* out);
int sl3dgpu_degree_solve(const sl3dgpu_degree* op, double* b, int nrhs);

/* The configurations' Earth (radius 6371 km, fluid core to 3480 km, linear
 * mantle, 100 km elastic lid, 5e21 / 5e20 Pa s below / above 670 km), the
 * given element count spread over its four layers in proportion to
 * thickness; kelvin_fraction > 0 makes the viscous layers Burgers bodies
 * (Kelvin viscosity = viscosity / kelvin_div). Fills layers[0..3]. */
int sl3dgpu_standard_earth(int elements, double kelvin_fraction, double kelvin_div,
                           sl3dgpu_layer* layers);

/* The 3D operator: Viscoelastic3D's constructor (src/Viscoelastic3D.cpp:169-356)
 * over the layered Earth, at the Gauss memory points. The degree systems
 * are assembled and factorised on the GPU; delta is zero until
 * sl3dgpu_v3d_set_delta.
 *
 * precision 1 (the mixed form) keeps the FP64 passes and the stopping rule
 * (relative change <= rtol on an FP64 pass, whose result is the step's) and
 * replaces the iterations between FP64 passes by a correction solved in
 * FP32 (transforms, band solves with FP32 copies of the FP64 factors, force
 * and strain maps, Anderson mixing with FP64 Gram sums), iterated until its
 * relative change is at most max(correction_rtol, 0.1 rtol / residual), the
 * accuracy that brings the next FP64 residual under rtol. No counterpart in
 * the reference, whose Converge is FP64 throughout. */
typedef struct sl3dgpu_v3d sl3dgpu_v3d;
typedef struct sl3dgpu_v3d_state sl3dgpu_v3d_state;
int sl3dgpu_v3d_create(const sl3dgpu_layer* layers, int nlayers, const sl3dgpu_v3d_options* options,
                       sl3dgpu_v3d** out);
void sl3dgpu_v3d_destroy(sl3dgpu_v3d* op);
/* Memory nodes, and the grid every node's values sit on (GridCoupling's one
 * block: NodeCount, Grid().NumberOfCoLatitudes/NumberOfLongitudes). */
int sl3dgpu_v3d_shape(const sl3dgpu_v3d* op, int* nodes, int* ntheta, int* nphi);
/* GridCoupling::RadiusOfNode / ElementOfNode, non-dimensional radii. */
int sl3dgpu_v3d_nodes(const sl3dgpu_v3d* op, double* radius, int* element);
int sl3dgpu_v3d_colatitudes(const sl3dgpu_v3d* op, double* theta, double* weights);
/* The model's scales (SI per unit): length, time, surface density. */
int sl3dgpu_v3d_scales(const sl3dgpu_v3d* op, double* length, double* time, double* surface_density);
/* The log-viscosity perturbation delta(r, theta, phi) sampled over every
 * memory node's grid (node-major, colatitude, longitude): the samples the
 * reference's delta callback gives (Viscoelastic3D.cpp:250-287); host or
 * device pointer. */
int sl3dgpu_v3d_set_delta(sl3dgpu_v3d* op, const double* samples, int on_device);
/* Viscoelastic3D::ZeroState (Viscoelastic3D.hpp, State). */
int sl3dgpu_v3d_zero_state(sl3dgpu_v3d* op, sl3dgpu_v3d_state** out);
void sl3dgpu_v3d_free_state(sl3dgpu_v3d_state* state);
/* Viscoelastic3D::Step (Viscoelastic3D.cpp:1982-2030): scheme 0
 * ExponentialTrapezoid, 1 BackwardEuler, 2 Sdirk2; the load channel's
 * coefficients (host, complex pairs, real spin-0 layout l(l+1)/2 + m,
 * non-dimensional surface density) at the step's start and end, the stages
 * taking the linear interpolation between them; NULL for none. The state
 * advances in place. */
int sl3dgpu_v3d_step(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, double dt, int scheme,
                     const double* load0, const double* load1, sl3dgpu_step_info* info);
/* The same step with the tide channel beside the load (Viscoelastic3D::Step's
 * tide, AddUnitChannels at Viscoelastic3D.cpp:1029-1073: the tide's (l, m >= 0)
 * coefficients at the step's start and end times times each degree's
 * K^-1 Tide, degree 0 with power 2); either pair may be null, all four are
 * host or (on_device) device pointers. A tide with degree-1 coefficients is
 * refused (TideColumns, Viscoelastic3D.cpp:137-154). */
int sl3dgpu_v3d_step_tide(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, double dt, int scheme,
                          const double* load0, const double* load1, const double* tide0, const double* tide1,
                          int on_device, sl3dgpu_step_info* info);
/* The same step with the load coefficients in device memory. */
int sl3dgpu_v3d_step_device(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, double dt, int scheme,
                            const double* load0, const double* load1, sl3dgpu_step_info* info);
/* Viscoelastic3D::Surface (Viscoelastic3D.cpp:2050-2081) of the last step's
 * solutions: component 0 U, 1 V, 2 phi; component 3 W is SurfaceToroidal
 * (:2083-2112, zero at degree 0); complex m >= 0 columns per degree in the
 * l(l+1)/2 + m layout, into host memory. */
int sl3dgpu_v3d_surface(sl3dgpu_v3d* op, int component, double* out);
/* The same surface coefficients written into a device buffer of
 * (lmax + 1)(lmax + 2) / 2 complex values, stream-ordered on the operator's
 * stream (sl3dgpu_v3d_stream) with no host wait: a driver collecting every
 * step's surface keeps the steps back to back. */
int sl3dgpu_v3d_surface_device(sl3dgpu_v3d* op, int component, double* device_out);
/* The memory nodes [first, end) where the lateral weight may be non-zero
 * (whole elements; empty until delta is set): Analyse(W d) vanishes
 * outside, so only these nodes' strain enters the next pass. */
int sl3dgpu_v3d_lateral_range(const sl3dgpu_v3d* op, int* first, int* end);
/* Per memory node, the slowest Prony branch's reference inverse relaxation
 * time (model units): PointItau of the radial reference (Viscoelastic.hpp:
 * 367-372). */
int sl3dgpu_v3d_node_relaxation(const sl3dgpu_v3d* op, double* itau);

/* ---- the learned warm start (Converge's start, Viscoelastic3D.hpp:562-569) ----
 * No counterpart in the reference, which starts each step from the previous
 * step's strain. A network (16 features -> `depth` hidden layers of `hidden`
 * GELU units -> 16 outputs; BF16 tensor-core products, FP32 masters and
 * accumulation) predicts, per degree, lateral memory node and spin block, the
 * coefficients (a, b, c) of Delta_n+1 = a Delta_n + b Delta_n-1 +
 * c Delta_n-2 from statistics of the last three strain changes over the
 * block's orders; the guess for sl3dgpu_v3d_set_start is s_n + Delta_n+1 at
 * the lateral nodes and s_n + Delta_n elsewhere. Trained on the GPU on pairs
 * the plain iteration produced; the step takes a guess only when its first
 * residual beats the plain start's. */
typedef struct sl3dgpu_wsnet sl3dgpu_wsnet;
int sl3dgpu_wsnet_create(int hidden, int depth, unsigned long long seed, sl3dgpu_wsnet** out);
void sl3dgpu_wsnet_destroy(sl3dgpu_wsnet* net);
long long sl3dgpu_wsnet_parameter_count(const sl3dgpu_wsnet* net);
/* The FP32 master parameters (per layer: weights out x in row-major, then biases). */
int sl3dgpu_wsnet_parameters(const sl3dgpu_wsnet* net, float* out);
int sl3dgpu_wsnet_set_parameters(sl3dgpu_wsnet* net, const float* in);
/* The operator layout the network reads: lmax, the lateral node count and
 * per lateral node its depth fraction in the lateral zone and log10(dt itau) / 4. */
int sl3dgpu_wsnet_bind(sl3dgpu_wsnet* net, int lmax, int lateral, const double* depth, const double* relax);
/* A batch of training pairs: per pair device pointers to the changes
 * Delta_n-2, Delta_n-1, Delta_n and the target Delta_n+1 as compact lateral
 * columns ([row][lateral] FP32 complex, rows in the bound layout's order),
 * host arrays of the load ratios and of the normalisers (the extrapolation's
 * squared error of each pair). The loss is the pairs' mean squared error of
 * the predicted change over the extrapolation's. gradient: the loss and the
 * FP32 gradient (grad may be NULL); train_step: one Adam step at rate lr. */
int sl3dgpu_wsnet_gradient(sl3dgpu_wsnet* net, int pairs, const void* const* d2, const void* const* d1,
                           const void* const* d0, const void* const* target, const float* ratio,
                           const float* norm, float* grad, float* loss);
int sl3dgpu_wsnet_train_step(sl3dgpu_wsnet* net, int pairs, const void* const* d2, const void* const* d1,
                             const void* const* d0, const void* const* target, const float* ratio,
                             const float* norm, float lr, float* loss);
/* The guess of the next step's end strain from the last four snapshots of a
 * state's strain coefficients (device layout of sl3dgpu_v3d_state_coefficients,
 * P nodes), the lateral range's first node, and the load ratio; ordered on
 * `stream` (device pointers). */
int sl3dgpu_wsnet_predict(sl3dgpu_wsnet* net, int P, int lateral_first, const double* s_n, const double* s_nm1,
                          const double* s_nm2, const double* s_nm3, double ratio, double* guess, void* stream);
/* The network's tensor-core product alone: C = A B^T, FP32 row-major A (M x K),
 * B (N x K), C (M x N), device pointers, operands rounded to BF16, FP32 sums. */
int sl3dgpu_wsnet_gemm(sl3dgpu_wsnet* net, const float* A, const float* B, int M, int N, int K, float* C);
/* Viscoelastic3D::InertiaMoment (Viscoelastic3D.cpp:2032-2048) of the last
 * step's solutions: sqrt(4 pi) int rho U r^3 dr of their degree-0 radial
 * displacement (the degree-0 moment row of detail/ViscoelasticDegree.hpp:
 * 142-161), in the operator's non-dimensional units. */
int sl3dgpu_v3d_inertia_moment(sl3dgpu_v3d* op, double* out);
/* The assembled, unscaled upper band of degree l's spheroidal (toroidal = 0)
 * or toroidal (1, l >= 1) system in the flavour of one scheme (0 exponential
 * trapezoid, 1 backward Euler; Sdirk2's stages are backward Euler flavours)
 * and step length dt (0: the elastic flavour) -- the reference's flavour
 * systems (Viscoelastic3D.cpp:535-558, DegreeOperator.cpp:253-474) with the
 * flavour's point shear, assembled on the GPU. out NULL asks the order n and
 * bandwidth kd; capacity counts doubles. */
int sl3dgpu_v3d_assembled_band(sl3dgpu_v3d* op, int scheme, double dt, int toroidal, int l, double* out,
                               long long capacity, int* n, int* kd);
/* The warm-start hook (OpenStep::Converge's start, Viscoelastic3D.hpp:562-569):
 * a guess of the strain coefficients at the end of the NEXT step, in the
 * device layout a state's coefficients have (sl3dgpu_v3d_state_coefficients;
 * 2 x spectral-size doubles, host or device). The step's last stage runs its
 * first pass from both the plain start (the previous strain) and the guess
 * and continues from the one with the smaller relative change, so a guess can
 * cost a pass but never accuracy. NULL disarms; a guess serves one step. No
 * reference counterpart for the choice (the reference takes the start as
 * given). */
int sl3dgpu_v3d_set_start(sl3dgpu_v3d* op, const double* coefficients, int on_device);
/* Whether the last step kept its warm start (1) or discarded it (0). */
int sl3dgpu_v3d_start_taken(const sl3dgpu_v3d* op);
/* A state's strain coefficients in the device layout: their device address
 * (NULL before a step) and their count of doubles. */
int sl3dgpu_v3d_state_coefficients(const sl3dgpu_v3d* op, const sl3dgpu_v3d_state* state, const double** device,
                                   long long* count);
/* The same coefficients copied to a host array (count doubles). */
int sl3dgpu_v3d_state_coefficients_host(const sl3dgpu_v3d* op, const sl3dgpu_v3d_state* state, double* out);
/* The same coefficients copied into a caller's device buffer (device
 * layout, 2 x count doubles), ordered on the operator's stream, which it
 * waits for. */
int sl3dgpu_v3d_state_coefficients_copy(const sl3dgpu_v3d* op, const sl3dgpu_v3d_state* state, double* device_out);
/* Evolution3D::Run (src/Evolution3D.cpp:184-394) for a body without an ocean
 * and without rotational feedback (GRDSolver::NoOceanState): node 0 the
 * instantaneous elastic response to loads[0] (a dt = 0 step), then one step
 * per node under the loads at its two ends. loads: nodes x (l(l+1)/2 + m)
 * complex host coefficients; u, phi (nullable): the surface U and phi per
 * node in the same layout; infos (nullable): each node's step info. */
int sl3dgpu_v3d_run(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, const double* times, int nodes, int scheme,
                    const double* loads, double* u, double* phi, sl3dgpu_step_info* infos);
/* The discrete adjoint of that run (AdjointSolver3D::FirstOrderKernels under
 * AdjointMethod::Discrete, include/sl3dpp/Adjoint3D.hpp:241-322,
 * src/AdjointDiscrete3D.cpp): the run from a zero state, every node's state
 * kept, then the exact transpose of its time-stepped map swept back node by
 * node (Sdirk2's first stage repeated from the node below). stride
 * (ForwardTrajectory3D's record stride, at least 1): the states of every
 * stride-th node are kept, a gap's rebuilt by the run's own steps when the
 * sweep reaches it -- about nodes / stride + stride states held, fewest near
 * sqrt(nodes). The objective
 * J = sum_n <u_dual_n, U_n> + <phi_dual_n, phi_n>, <a, b> = sum_{l, m >= 0}
 * w_m Re(a b*) with w_m = 1 at m = 0 and 2 above (the surface integral of
 * the two real fields over the unit sphere); u_dual, phi_dual: nodes x
 * (l(l+1)/2 + m) complex host coefficients (nullable, m = 0 parts real).
 * Out: load_kernels (required, the same layout), the load kernels
 * (Kernels::directLoadKernels): dJ = sum_n <load_kernels_n, dL_n>;
 * tide_kernels (nullable, the same layout; Kernels::tideKernels): dJ =
 * sum_n <tide_kernels_n, dpsi_n> for a tidal potential added to the run's
 * tide channel (degree 1 none);
 * delta_gradient (nullable, one double per grid value, node-major as
 * set_delta's samples): dJ/d delta at each sample, dJ = sum_x
 * delta_gradient_x d delta_x -- divided by sl3dgpu_v3d_sample_volumes it
 * is the reference's logViscosityKernel3D, a density per unit volume;
 * objective (nullable): J of the forward run; infos (nullable): the forward
 * steps' infos. Without an ocean and for the fixed-point step (solver 0,
 * FP64 or mixed); the transposed solves take the operator's rtol. */
int sl3dgpu_v3d_adjoint_run(sl3dgpu_v3d* op, const double* times, int nodes, int scheme, int stride,
                            const double* loads, const double* u_dual, const double* phi_dual, double* load_kernels,
                            double* tide_kernels, double* delta_gradient, double* objective,
                            sl3dgpu_step_info* infos);
/* The discrete tangent-linear run beside the same run
 * (TangentLinearSolver3D, src/TangentLinear3D.cpp, its discrete method): the
 * derivative of the surface U and phi at every node along a log-viscosity
 * direction (delta_direction: one double per grid value, node-major as
 * set_delta's samples, nullable) and along load directions (nodes x
 * (l(l+1)/2 + m) complex host coefficients, nullable), each stage's tangent
 * solve the step's own iteration. u, phi (nullable): the derivatives per
 * node, the run's layout; infos: the forward steps'. Without an ocean, the
 * fixed-point step (FP64 or mixed). With the adjoint:
 * sum_n <u_dual_n, u_n> + <phi_dual_n, phi_n> = delta_gradient . direction
 * + sum_n <load_kernels_n, load_direction_n>. */
int sl3dgpu_v3d_tangent_run(sl3dgpu_v3d* op, const double* times, int nodes, int scheme, const double* loads,
                            const double* delta_direction, const double* load_directions, double* u, double* phi,
                            sl3dgpu_step_info* infos);
/* The volume each grid sample stands for (GridCoupling's volume weight:
 * the radial quadrature weight jac w_q r^2 of its memory node times its
 * colatitude's weight 2 pi w_theta / nphi), one double per grid value. */
int sl3dgpu_v3d_sample_volumes(const sl3dgpu_v3d* op, double* out);
/* Many independent runs at once (an ensemble: the reference's calibration and
 * line-search workloads run Evolution3D per member): run i is
 * sl3dgpu_v3d_run(ops[i], states[i], times[i], nodes[i], scheme, loads[i],
 * u[i], phi[i], infos[i]) (u, phi, infos nullable as arrays). `threads` host
 * threads (0: one per run up to the host's cores) drive the runs; each
 * operator keeps its own stream, so the runs' kernels overlap on the GPU.
 * statuses[i] receives run i's status; the call returns the first failure's
 * (its text in sl3dgpu_last_error) or 0. Operators and states must be
 * distinct. No reference counterpart (the reference runs members one by one
 * or in separate processes). */
int sl3dgpu_v3d_run_many(int count, sl3dgpu_v3d* const* ops, sl3dgpu_v3d_state* const* states,
                         const double* const* times, const int* nodes, int scheme,
                         const double* const* loads, double* const* u, double* const* phi,
                         sl3dgpu_step_info* const* infos, int threads, int* statuses);
/* A state as bytes, for checkpoints (Evolution3D::Checkpoint's memory and
 * strain, src/Evolution3D.cpp:146-167): the byte count, the state copied to
 * a host buffer of that size, and a state (from sl3dgpu_v3d_zero_state)
 * replaced by saved bytes -- refused unless an operator of the same shape
 * saved them. A run resumed from saved bytes continues bit for bit. */
long long sl3dgpu_v3d_state_bytes(const sl3dgpu_v3d* op, const sl3dgpu_v3d_state* state);
int sl3dgpu_v3d_state_save(sl3dgpu_v3d* op, const sl3dgpu_v3d_state* state, void* out, long long capacity);
int sl3dgpu_v3d_state_load(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, const void* in, long long bytes);

/* ---- the open step (Viscoelastic3D::OpenStep, include/sl3dpp/Viscoelastic3D.hpp:440-640) ----
 * One stage opened on the operator's own buffers, for a driver's own
 * within-step iteration (one open step per operator at a time). Strain
 * coefficients are device arrays in the device layout
 * (sl3dgpu_v3d_layout's `spectral` complex values); solutions live in the
 * operator and are read by sl3dgpu_v3d_surface / sl3dgpu_v3d_inertia_moment.
 * start_step: StartStep of one stage (scheme 0 or 1, length dt) from the
 * state; load0 (host coefficients, nullable) the load at the state's time
 * when the state carries no strain. step_respond: Respond, the solutions of
 * the memory and lateral force of a strain (NULL: the start strain), no
 * channels. step_add_channels: AddChannels (host (l, m >= 0) coefficients,
 * either nullable; a tide's degree-1 part refused). step_strain_of:
 * StrainOf of the solutions. step_converge: Close under known channels, the
 * operator's own fixed point (or conjugate gradients / the mixed form, as its
 * options say) from the start strain; the strain (nullable device out).
 * step_finish: Finish with a strain (NULL: the converged one), the state
 * advanced in place; the step closes. relative_change: Converge's measure
 * between two strains. */
int sl3dgpu_v3d_start_step(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, double dt, int scheme, const double* load0);
int sl3dgpu_v3d_step_start_strain(sl3dgpu_v3d* op, double* device_out);
int sl3dgpu_v3d_step_respond(sl3dgpu_v3d* op, const double* strain);
int sl3dgpu_v3d_step_add_channels(sl3dgpu_v3d* op, const double* load, const double* tide);
int sl3dgpu_v3d_step_strain_of(sl3dgpu_v3d* op, double* device_out);
int sl3dgpu_v3d_step_converge(sl3dgpu_v3d* op, const double* load, const double* tide, double* device_strain,
                              sl3dgpu_step_info* info);
int sl3dgpu_v3d_step_finish(sl3dgpu_v3d* op, const double* strain);
/* The conjugate-gradient close's pieces (options.solver = 1): step_forces,
 * OpenStep::Forces -- the degree forces of the fixed memory force and of
 * the channels (host coefficients, nullable) into device solutions laid out
 * spheroidal then toroidal (sl3dgpu_v3d_layout's counts); step_apply,
 * OpenStep::Apply -- (K_eff - P^T W S) x; step_solve, OpenStep::Solve -- the
 * solutions for given forces by preconditioned conjugate gradients from the
 * reference response (out nullable; the solutions are also held, so
 * step_strain_of and the surface read them). */
int sl3dgpu_v3d_step_forces(sl3dgpu_v3d* op, const double* load, const double* tide, double* out);
int sl3dgpu_v3d_step_apply(sl3dgpu_v3d* op, const double* x, double* out);
int sl3dgpu_v3d_step_solve(sl3dgpu_v3d* op, const double* forces, double* out, sl3dgpu_step_info* info);
int sl3dgpu_v3d_relative_change(sl3dgpu_v3d* op, const double* next, const double* now, double* out);

/* ---- the grid coupling (GridCoupling, include/sl3dpp/GridCoupling.hpp:82-428) ----
 * The maps between the operator's tensor fields and the degree systems, on
 * device arrays: sizes (complex spectral coefficients, grid values at every
 * node, spheroidal and toroidal solution values) from sl3dgpu_v3d_layout;
 * degree l's solutions are [dof][l + 1] blocks at sl3dgpu_v3d_solution_layout's
 * offsets. synthesise_tensor / analyse_tensor: Synthesise / Analyse of the
 * spin -2, spin -1 (complex) and spin 0 (real) components at every node;
 * degree_forces: SpheroidalForce / ToroidalForce of an analysed tensor into
 * the systems' right-hand sides; strain_of_solutions: AddStrainOfSolution
 * with the deviatoric components, the strain coefficients of solutions. */
int sl3dgpu_v3d_layout(const sl3dgpu_v3d* op, long long* spectral, long long* grid_values, long long* spheroidal,
                       long long* toroidal);
int sl3dgpu_v3d_solution_layout(const sl3dgpu_v3d* op, int l, long long* sph_offset, int* sph_dofs,
                                long long* tor_offset, int* tor_dofs);
int sl3dgpu_v3d_synthesise_tensor(sl3dgpu_v3d* op, const double* spectral, double* c0, double* c1, double* r);
int sl3dgpu_v3d_analyse_tensor(sl3dgpu_v3d* op, const double* c0, const double* c1, const double* r,
                               double* spectral);
int sl3dgpu_v3d_degree_forces(sl3dgpu_v3d* op, const double* spectral, double* spheroidal, double* toroidal);
int sl3dgpu_v3d_strain_of_solutions(sl3dgpu_v3d* op, const double* spheroidal, const double* toroidal,
                                    double* spectral);

/* ---- the ocean closure (Evolution3D, src/Evolution3D.cpp:184-394) ----------
 * The coupled fixed point of a step under an ocean with frozen shorelines:
 * in every pass the surface responses of the degree solves (before the load
 * and tide channels) and their inertia moment close the sea-level equation
 * (GRDSolver::SolveGeneralised) on the pass flavour's effective Love numbers,
 * under the stage's direct load; its total load (the direct load and the
 * ocean's) and the centrifugal potential of its angular velocity are the
 * pass's load and tide channels (Coupled::Closure, :296-339). The sea-level
 * grid is the operator's lmax at oversampling 1 (sl3dgpu_v3d_ocean_grid);
 * fields on it are colatitude-major. Built for the FP64 fixed point
 * (precision 0, solver 0); no prescribed tide beside it. */
typedef struct sl3dgpu_v3d_ocean {
  const double* ocean_function; /* host field on the sea-level grid (1 ocean, 0 land) */
  int rotation;                 /* RotationalFeedback: 0 None, 1 Axial, 2 Full */
  double water_density;         /* kg m^-3 (SeaLevelParameters: 1000) */
  double rotation_frequency;    /* s^-1 (7.27220521664304e-05) */
  double polar_moment;          /* kg m^2 (8.0359e37) */
  double equatorial_moment;     /* kg m^2 (8.0096e37) */
  double rtol;                  /* the sea-level solve's (Evolution3D::Options::rtol) */
  int max_iterations;           /* its budget */
  int anderson_memory;          /* its mixer's columns, 0..16 */
  /* migrating shorelines (Evolution3D::RunMigrating, src/Evolution3D.cpp:
   * 117-133; Coupled::Closure's nonlinear branch :308-319): every pass
   * solves GRDSolver::SolveNonlinear from the background state below under
   * the stage's ice. ocean_function may then be NULL (flotation's is taken;
   * one given must equal it). Fields are host fields on the sea-level grid
   * in the model's length unit. */
  int migrating;                      /* 0: frozen shorelines, 1: migrating */
  double ice_density;                 /* kg m^-3 (SeaLevelParameters: 917) */
  const double* ice_thickness;        /* the background's ice thickness */
  const double* sea_level;            /* its sea level (the sea surface over the solid surface) */
  const unsigned char* forced_land;   /* the land held at C = 0 (NULL: none) */
  int max_nonlinear_iterations;       /* Evolution3D::Options::max_nonlinear_iterations */
} sl3dgpu_v3d_ocean;
/* Sets (NULL: removes) the ocean of the operator's steps. */
int sl3dgpu_v3d_set_ocean(sl3dgpu_v3d* op, const sl3dgpu_v3d_ocean* ocean);
/* The sea-level grid: its shape, colatitudes and quadrature weights (either nullable). */
int sl3dgpu_v3d_ocean_grid(sl3dgpu_v3d* op, int* ntheta, int* nphi, double* theta, double* weights);
/* One coupled step: the direct (non-ocean) load at the step's start and end
 * as host fields on the sea-level grid, non-dimensional surface density
 * (NULL: zero); the stages take their linear combination (detail::AtStage).
 * A dt = 0 step is Evolution3D::Start's instantaneous response to load1. */
int sl3dgpu_v3d_step_ocean(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, double dt, int scheme, const double* load0,
                           const double* load1, sl3dgpu_step_info* info);
/* Evolution3D::Run with the ocean: node 0 the instantaneous response, then a
 * step per node. loads: nodes x the sea-level grid's field; u, phi,
 * sea_level (nullable): nodes x (l(l+1)/2 + m) complex coefficients of the
 * surface U, phi and the relative sea level change; angular_velocity
 * (nullable): nodes x 3; infos (nullable). */
int sl3dgpu_v3d_run_ocean(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, const double* times, int nodes, int scheme,
                          const double* loads, double* u, double* phi, double* sea_level, double* angular_velocity,
                          sl3dgpu_step_info* infos);
/* One coupled step under migrating shorelines: the ice thickness at the
 * step's start and end (host fields, model length) and the direct loads
 * beside it (NULL: none); a dt = 0 step is the start's solve
 * (src/Evolution3D.cpp:690-700). */
int sl3dgpu_v3d_step_migrating(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, double dt, int scheme, const double* ice0,
                               const double* ice1, const double* load0, const double* load1,
                               sl3dgpu_step_info* info);
/* Evolution3D::RunMigrating: ice (nodes x field), loads (nodes x field;
 * NULL: none, node 0 then undisturbed at the background, whose ice must be
 * the first node's), the outputs of sl3dgpu_v3d_run_ocean and each node's
 * ocean function (ocean_functions: nodes x field, nullable). */
int sl3dgpu_v3d_run_migrating(sl3dgpu_v3d* op, sl3dgpu_v3d_state* state, const double* times, int nodes, int scheme,
                              const double* ice, const double* loads, double* u, double* phi, double* sea_level,
                              double* angular_velocity, double* ocean_functions, sl3dgpu_step_info* infos);
/* The last closure's ocean function (the fixed one under frozen
 * shorelines), a host field on the sea-level grid. */
int sl3dgpu_v3d_ocean_function(sl3dgpu_v3d* op, double* out);
/* The last closure's relative sea level change, (l, m >= 0) complex host
 * coefficients in the model's length unit (nullable), its angular velocity
 * (3, nullable) and its solve's scalars (nullable). */
int sl3dgpu_v3d_sea_level(sl3dgpu_v3d* op, double* coefficients, double* angular_velocity,
                          sl3dgpu_sle_result* result);
/* The effective Love numbers of a one-stage flavour (scheme 0 or 1, step
 * length dt, 0 the elastic solid; ComputeLoveNumbers on the flavour's solid,
 * src/LoveNumbers.cpp:92-176): h, k, l, h_t, k_t, l_t per degree (lmax + 1
 * each, the tidal ones from degree 2), then h_c, k_c, the load's inertia
 * number m_u + m_phi and m_c; 6 (lmax + 1) + 4 doubles. */
int sl3dgpu_v3d_effective_love(sl3dgpu_v3d* op, int scheme, double dt, double* out);
/* The CUDA stream the operator's kernels run on. */
void* sl3dgpu_v3d_stream(const sl3dgpu_v3d* op);
/* The last step's pass residuals (RelativeChange per pass, the stages in
 * turn): returns their count, copying at most `capacity` into out. */
int sl3dgpu_v3d_residual_history(const sl3dgpu_v3d* op, double* out, int capacity);
/* The mixed form's last step: the relative change of every FP32 correction
 * pass in turn (empty in the FP64 form). No reference counterpart. */
int sl3dgpu_v3d_correction_history(const sl3dgpu_v3d* op, double* out, int capacity);
/* A state's strain coefficients in the reference layouts, node-major blocks:
 * spin -2, spin -1, real spin 0 (GridCoupling::SpectralTensor). Host out. */
int sl3dgpu_v3d_state_strain(sl3dgpu_v3d* op, const sl3dgpu_v3d_state* state, double* out);

/* ---- measurement ------------------------------------------------------------
 * Kernel launches the library has made since it was loaded. */
long long sl3dgpu_launch_count(void);
/* Per-kernel-kind CUDA-event timing of every launch (on its own stream) and
 * its algorithmic work: kinds 0 Legendre synthesis, 1 Legendre analysis,
 * 2 ring FFTs, 3 force assembly, 4 strain recovery, 5 band solves,
 * 6 streaming weights/memory, 7 Anderson sweeps, 8 other, and the mixed
 * form's FP32 passes: 9 Legendre contractions, 10 ring FFTs, 11 band solves;
 * 12 the FP64 Legendre contractions emulated on the tensor cores. */
int sl3dgpu_profile_enable(int on);
int sl3dgpu_profile_reset(void);
int sl3dgpu_profile_read(int kind, double* ms, long long* launches, double* flops, double* bytes);
/* The FP64 FMA throughput of the device (GFLOP/s), measured by a short
 * register-resident kernel: the FP64 path's compute roofline. */
int sl3dgpu_fp64_fma_peak(double* gflops);
/* The same for FP32 FMA (the mixed form's correction passes). */
int sl3dgpu_fp32_fma_peak(double* gflops);

#ifdef __cplusplus
}
#endif

#endif /* SL3DGPU_H */
