// The device spherical-harmonic grid: Gauss-Legendre colatitudes, uniform
// longitudes, the stored spin-N Legendre (Wigner-d) tables and the FFT plan,
// with the batched transforms between coefficients and grid values.
//
// Basis (docs/design.md:245-250 of the reference): Y^N_lm =
// sqrt((2l+1)/4pi) d^l_{Nm}(theta) e^{i m phi}, d^l_{0m} the Condon-Shortley
// associated Legendre function; forward transform the integral of conj(Y) f.
// Reference index layouts (include/sl3dpp/SurfaceGrid.hpp:110-118, 191-200):
// spin N complex, l^2 - N^2 + (m + l) over l = |N|..lmax and every m; real
// spin 0, l(l+1)/2 + m over m >= 0. Grid values colatitude-major, longitude
// k at 2 pi k / nphi.
//
// Device ("m-major") layouts, what the kernels read and write: a batch of
// `count` fields keeps, per spin, the coefficients of order m and degree l at
// row RowOffset(m) + (l - l0(m)) of a [row][count] complex array (the node
// fastest), so that one order's degrees over the batch are one dense matrix;
// ring spectra are [m][j][count] complex.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <vector>

#include "common.cuh"

namespace sl3dgpu {

struct FftPlan {
  int n = 0;
  int stages = 0;
  int radix[16] = {};
};

// One spin's table: for each order m in [-lmax, lmax] (index m + lmax) a
// block of (lmax - l0 + 1) rows of ntheta values, rows = degrees.
struct SpinTable {
  int N = 0;
  std::vector<int> rowOffset;  // 2 lmax + 2 entries, cumulative rows by m index
  double* values = nullptr;    // device
  int* dRowOffset = nullptr;   // device copy of rowOffset
  int Rows(int m, int lmax) const { return rowOffset[m + lmax + 1] - rowOffset[m + lmax]; }
};

struct GemmItem {
  int M, N, K, pad;
  long long a, b, c;
  int sAi, sAk, ldb, ldc;
};

// One item of the FP64 contraction emulated on the tensor cores: 128-row
// tiles of A, 64-column tiles of B, 16-deep steps.
struct Tc64Item {
  int M, N, K, mTiles;
  int kSteps, nTiles, ldc, ldb;
  long long aPanel;  // BF16 values: the item's panel, [mTile][kStep][slice][128 x 16]
  long long bPack;   // BF16 values: its packed B, [nTile][kStep][slice][64 x 16]
  long long b, c;    // FP64 offsets of B's source and of C
  long long rowExp;  // ints: the power-of-two exponents of its M rows of A
  long long colExp;  // ints: those of its N columns of B (per call)
};

// A tensor-core item's host description (mirrors TcItem in tc_gemm.cuh).
struct TcItemHost {
  int M, N, K, mTiles;
  int kSteps, nTiles, ldc, ldb;
  long long aPanel, bPack;
  long long b, c;
};

class Grid {
 public:
  static int Create(int lmax, int nmax, double oversampling, std::unique_ptr<Grid>& out);
  ~Grid();

  int lmax = 0, nmax = 0, band = 0, ntheta = 0, nphi = 0;
  // The FP64 contractions emulated on the tensor cores (tc_gemm64.cu)
  // rather than run on the FP64 units; batches deeper than the emulation's
  // exactness bound keep the FP64 units.
  bool emulateFp64 = false;
  std::vector<double> theta, weights;  // host copies
  double* dTheta = nullptr;
  double* dWeights = nullptr;
  double2* dTwiddle = nullptr;
  float2* dTwiddle32 = nullptr;
  FftPlan plan;

  // The table of spin N, built on first use (device kernel).
  int Table(int N, const SpinTable** out);
  // Rows of one spin's coefficients per field (its (l, m) count).
  long long SpinRows(int N) const { return static_cast<long long>(lmax + 1) * (lmax + 1) - N * N; }
  // Rows of a real spin-0 field (m >= 0).
  long long RealRows() const { return static_cast<long long>(lmax + 1) * (lmax + 2) / 2; }

  // -- transforms in the device layouts -------------------------------------------
  // Spin N: coefficients [row][P] complex (columns p0 .. p0 + count of them
  // taking part) -> spectra [m][j][count] -> fields [count][j][k] complex;
  // and back. Real spin 0 likewise with m >= 0 rows. The analysis may add its
  // result to what the coefficients hold (the memory force's fixed part).
  int LegendreSynthesis(int N, bool real, const double* coeffs, int P, int p0, int count,
                        double* spectra, cudaStream_t stream);
  int LegendreAnalysis(int N, bool real, const double* spectra, int P, int p0, int count,
                       double* coeffs, bool accumulate, cudaStream_t stream);
  int LegendreSynthesis(int N, bool real, const double* coeffs, int count, double* spectra,
                        cudaStream_t stream) {
    return LegendreSynthesis(N, real, coeffs, count, 0, count, spectra, stream);
  }
  int LegendreAnalysis(int N, bool real, const double* spectra, int count, double* coeffs,
                       cudaStream_t stream) {
    return LegendreAnalysis(N, real, spectra, count, 0, count, coeffs, false, stream);
  }
  int RingSynthesis(bool real, const double* spectra, int count, double* fields, cudaStream_t stream);
  // Optional pointwise weight (a real field over the same values) applied
  // before the analysis.
  int RingAnalysis(bool real, const double* fields, int count, double* spectra, cudaStream_t stream,
                   const double* weight = nullptr);
  // Synthesis, the pointwise weight and the analysis of each ring in one
  // pass through shared memory: the grid values never reach HBM.
  int RingWeighted(bool real, const double* spectraIn, int count, const double* weight,
                   double* spectraOut, cudaStream_t stream);

  // The same contraction and ring passes in FP32 (the mixed form's
  // correction passes): FP32 copies of the table and twiddles, made once.
  int LegendreSynthesisF(int N, bool real, const float* coeffs, int P, int p0, int count, float* spectra,
                         cudaStream_t stream);
  // Whether a tensor-core contraction gave up waiting since the last call
  // (reads and clears the device flag; synchronises the stream).
  int TensorCoreStatus(cudaStream_t stream);
  int LegendreAnalysisF(int N, bool real, const float* spectra, int P, int p0, int count, float* coeffs,
                        bool accumulate, cudaStream_t stream);
  int RingWeightedF(bool real, const float* spectraIn, int count, const float* weight, float* spectraOut,
                    cudaStream_t stream);

  // Reference layout <-> device layout permutations.
  int ToDevice(int N, bool real, const double* ref, int count, double* dev, cudaStream_t stream);
  int FromDevice(int N, bool real, const double* dev, int count, double* ref, cudaStream_t stream);

  // Scratch owned by the grid for the reference-layout batch calls.
  int Scratch(size_t spectraDoubles, size_t coeffDoubles, double** spectra, double** coeffs);

 private:
  std::map<int, SpinTable> tables_;
  struct Batch {
    GemmItem* items = nullptr;
    int count = 0, maxM = 0, maxN = 0;
    bool analysis = false;
    double flops = 0.0;    // 2 M N K summed over the items
    double outputs = 0.0;  // M N summed over the items
    // the tensor-core form (FP32): its items, tile width and extents, the
    // packed B (made on first use) and the key of its table panel
    std::vector<TcItemHost> tcHost;
    void* tcItems = nullptr;
    int tileN = 0, maxMTiles = 0, maxNTiles = 0, maxATiles = 0, maxBTiles = 0;
    long long panelFloats = 0, packedFloats = 0;
    float* packed = nullptr;
    std::vector<int4> tcTiles;  // {item, row tile, column tile}, column tiles of a row tile adjacent
    int4* dTcTiles = nullptr;
    int maxK = 0;
    // the FP64 emulation's form: items, extents, packed B and column
    // exponents (made on first use)
    std::vector<Tc64Item> tc64Host;
    Tc64Item* tc64Items = nullptr;
    int maxNTiles64 = 0, maxBTiles64 = 0;
    long long panel64 = 0, packed64Count = 0, rowExps = 0, colExps = 0;
    uint16_t* packed64 = nullptr;
    int* colExp = nullptr;
  };
  // The table split for the FP64 emulation per (spin, real, direction): its
  // slice panels and row exponents.
  struct Panel64 {
    uint16_t* slices = nullptr;
    int* rowExp = nullptr;
  };
  std::map<std::array<int, 3>, Panel64> panels64_;
  int RunGemm64(int N, bool real, Batch& b, const double* B, double* C, bool accumulate, cudaStream_t stream);
  // The table pre-tiled for the tensor cores per (spin, real, direction).
  std::map<std::array<int, 3>, float*> panels_;
  std::map<std::array<long long, 6>, Batch> batches_;
  int BatchFor(int N, bool real, bool analysis, int P, int p0, int count, const Batch** out);
  Batch* MutableBatch(int N, bool real, bool analysis, int P, int p0, int count);
  double* scratchSpectra_ = nullptr;
  size_t scratchSpectraSize_ = 0;
  double* scratchCoeffs_ = nullptr;
  size_t scratchCoeffsSize_ = 0;
  int RunGemm(const Batch& b, const double* A, const double* B, double* C, bool accumulate,
              cudaStream_t stream);
  // The FP32 contraction on the tensor cores (tc_gemm.cu): the spin's table
  // panel (made on first use), B packed, the contraction.
  int RunGemmF(int N, bool real, Batch& b, const float* B, float* C, bool accumulate, cudaStream_t stream);
  int* dTcError_ = nullptr;  // set by a tensor-core wait that gave up
  int Table32(int N, const SpinTable** out);
};

// Smallest 2^a 3^b 5^c at or above n.
int FftFriendly(int n);

}  // namespace sl3dgpu
