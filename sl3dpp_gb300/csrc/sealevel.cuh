// The sea-level solves as the coupled step calls them (sealevel.cu): a
// workspace kept between solves on one grid, the generalised solve (the C
// ABI's sl3dgpu_sle_solve with the total load's coefficients as an extra
// output), the nonlinear one with migrating shorelines, flotation, and the
// centrifugal potential of an angular velocity.
#pragma once

#include <cuda_runtime.h>

#include "sl3dgpu.h"

namespace sl3dgpu {

struct SleWorkspace;
SleWorkspace* NewSleWorkspace();
void FreeSleWorkspace(SleWorkspace* ws);

// GRDSolver::SolveGeneralised on `grid`; total_load (nullable, device,
// (l, m >= 0) complex coefficients) receives Expand(sigma_d + sigma_outside +
// rho_w C S) of the last sea level change S, TotalLoadCoefficients
// (src/Evolution3D.cpp:237-249). Every field and coefficient pointer is a
// device pointer, ordered on `stream`, which the call waits for.
int SeaLevelSolve(SleWorkspace& ws, sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, const double* ocean,
                  const sl3dgpu_sle_forcing* forcing, double rtol, int max_iterations, int anderson_memory,
                  double* sea_level_change, double* displacement, double* potential, double* tangential_potential,
                  double* toroidal_potential, double* total_load, sl3dgpu_sle_result* result, cudaStream_t stream);

// GRDSolver::SolveNonlinear (the C ABI's sl3dgpu_sle_solve_nonlinear) on the
// workspace; device pointers ordered on `stream`, which the call waits for.
int SeaLevelSolveNonlinear(SleWorkspace& ws, sl3dgpu_grid* grid, const sl3dgpu_sle_body* body, double ice_density,
                           const sl3dgpu_sle_state* state, const sl3dgpu_sle_nonlinear_forcing* forcing, double rtol,
                           int max_iterations, double* sea_level_change, double* displacement, double* potential,
                           double* tangential_potential, double* toroidal_potential, double* final_sea_level,
                           double* final_ocean_function, double* load_coefficients, sl3dgpu_sle_result* result,
                           cudaStream_t stream);

// MakeState's ocean function by flotation, ordered on `stream`.
int Flotation(long long n, double water_density, double ice_density, const double* ice, const double* sea_level,
              const unsigned char* forced_land, double* ocean_function, cudaStream_t stream);

// GRDSolver::CentrifugalCoefficients (src/SeaLevel.cpp:249-258): the (0, 0),
// (2, 0) and (2, 1) complex coefficients, as (re, im) pairs, of the
// centrifugal potential of the angular velocity change omega (zero without
// rotational feedback).
int CentrifugalCoefficients(const sl3dgpu_sle_body& body, const double omega[3], double out[6]);

}  // namespace sl3dgpu
