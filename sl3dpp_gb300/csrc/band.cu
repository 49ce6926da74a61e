// Batched banded factorisations and solves on the device: every degree's
// spheroidal and toroidal system in one launch.
//
// The arithmetic is LAPACK's unblocked band algorithms as the reference
// restates them (src/BandSolvers.cpp:23-139; dpbtf2/dpbtrs, dgbtf2/dgbtrs)
// in the same band storage, with the same pivot choices, so factors agree
// with the reference's to rounding and failure indices exactly.
//
// GB300 layout:
//  - factorisation: one CTA per system; the band's active window (the kd+1
//    columns a rank-1 step touches, 2kl+ku+1 rows deep for LU) is staged in
//    shared memory as a ring and streamed column by column, so each band
//    value is read from and written to HBM once;
//  - solves: one warp per (system, 64 right-hand sides), two adjacent
//    columns a lane (an order's real and imaginary parts). Right-hand sides
//    are stored row-major (dof-major, the columns fastest), so a warp's rows
//    are coalesced; a degree's 2(l+1) real columns (its orders m >= 0) are
//    its right-hand-side vectors. Each substitution runs in chunks of rows:
//    the next chunk's band columns and right-hand-side rows are copied into
//    shared memory (cp.async) while the current one is solved, the recent
//    solution values live in a per-warp shared-memory ring, and a band value
//    read serves two columns. Optional diagonal scaling and pinned dofs are fused
//    in (DegreeOperator::BeginSolve/FinishSolve, src/DegreeOperator.cpp:861-901);
//  - FP32 Cholesky solves may run over row windows: a right-hand side that is
//    zero below row lo has y = 0 there, so the substitutions cover rows
//    lo .. n - 1, and a completion launch finishes the rows below.
#include <algorithm>
#include <utility>
#include <vector>

#include "common.cuh"
#include "profile.cuh"

namespace sl3dgpu {
namespace {

constexpr int kRing = 64;  // solve ring depth: kd, kl + ku below this

__device__ inline double& WinAt(double* win, int ld, int window, int col, int row) {
  return win[(col % window) * ld + row];
}

// -- Cholesky factor -----------------------------------------------------------

__global__ void CholeskyFactorKernel(const sl3dgpu_band_system* systems, double* bands,
                                     int* info) {
  const sl3dgpu_band_system s = systems[blockIdx.x];
  const int n = s.n, kd = s.ku, ld = kd + 1, window = kd + 1;
  double* ab = bands + s.band;
  extern __shared__ double win[];  // window x ld
  __shared__ int failed;
  if (threadIdx.x == 0) failed = 0;
  for (int c = 0; c < min(window, n); ++c)
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      WinAt(win, ld, window, c, r) = ab[static_cast<long long>(c) * ld + r];
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const double d = WinAt(win, ld, window, j, kd);
    if (!(d > 0.0)) {
      if (threadIdx.x == 0) failed = j + 1;
      break;
    }
    const double ujj = sqrt(d);
    const double inverse = 1.0 / ujj;
    const int kn = min(kd, n - 1 - j);
    __syncthreads();  // every thread has read d before it is overwritten
    if (threadIdx.x == 0) WinAt(win, ld, window, j, kd) = ujj;
    for (int c = 1 + threadIdx.x; c <= kn; c += blockDim.x)
      WinAt(win, ld, window, j + c, kd - c) *= inverse;
    __syncthreads();
    // A(j + r, j + c) -= U(j, j + r) U(j, j + c), 1 <= r <= c <= kn.
    const int pairs = kn * (kn + 1) / 2;
    for (int t = threadIdx.x; t < pairs; t += blockDim.x) {
      int c = static_cast<int>((sqrt(8.0 * t + 1.0) - 1.0) * 0.5) + 1;
      while (c * (c - 1) / 2 > t) --c;
      while (c * (c + 1) / 2 <= t) ++c;
      const int r = t - c * (c - 1) / 2 + 1;
      const double ur = WinAt(win, ld, window, j + r, kd - r);
      const double uc = WinAt(win, ld, window, j + c, kd - c);
      WinAt(win, ld, window, j + c, kd + r - c) -= ur * uc;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      ab[static_cast<long long>(j) * ld + r] = WinAt(win, ld, window, j, r);
    __syncthreads();
    if (j + window < n)
      for (int r = threadIdx.x; r < ld; r += blockDim.x)
        WinAt(win, ld, window, j + window, r) =
            ab[static_cast<long long>(j + window) * ld + r];
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) info[blockIdx.x] = failed;
}

// -- LU factor (partial pivoting) --------------------------------------------------

__global__ void LuFactorKernel(const sl3dgpu_band_system* systems, double* bands,
                               int* pivotsAll, int* info) {
  const sl3dgpu_band_system s = systems[blockIdx.x];
  const int n = s.n, kl = s.kl, ku = s.ku, kv = kl + ku, ld = 2 * kl + ku + 1;
  const int window = kv + 1;
  double* ab = bands + s.band;
  int* pivots = pivotsAll + s.pivots;
  extern __shared__ double win[];
  __shared__ int pivot;
  auto at = [&](int i, int j) -> double& { return WinAt(win, ld, window, j, kv + i - j); };
  for (int c = 0; c < min(kv, n); ++c)
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      WinAt(win, ld, window, c, r) = ab[static_cast<long long>(c) * ld + r];
  __syncthreads();
  // The fill-in places of the first kv columns start zero (dgbtf2).
  for (int j = ku + 1; j < min(kv, n); ++j)
    for (int i = threadIdx.x; i < j - ku; i += blockDim.x) at(i, j) = 0.0;
  int infoValue = 0, ju = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (j + kv < n) {
      for (int r = threadIdx.x; r < ld; r += blockDim.x)
        WinAt(win, ld, window, j + kv, r) = ab[static_cast<long long>(j + kv) * ld + r];
      __syncthreads();
      for (int i = j + threadIdx.x; i < j + kl; i += blockDim.x) at(i, j + kv) = 0.0;
      __syncthreads();
    }
    const int km = min(kl, n - 1 - j);
    if (threadIdx.x == 0) {
      int p = j;
      for (int i = j + 1; i <= j + km; ++i)
        if (fabs(at(i, j)) > fabs(at(p, j))) p = i;
      pivot = p;
      pivots[j] = p;
    }
    __syncthreads();
    const int p = pivot;
    const bool zero = at(p, j) == 0.0;
    if (zero) {
      if (infoValue == 0) infoValue = j + 1;
    } else {
      ju = max(ju, min(p + ku, n - 1));
      if (p != j) {
        for (int c = j + threadIdx.x; c <= ju; c += blockDim.x) {
          const double t = at(p, c);
          at(p, c) = at(j, c);
          at(j, c) = t;
        }
      }
      __syncthreads();
      if (km > 0) {
        const double inverse = 1.0 / at(j, j);
        for (int i = j + 1 + threadIdx.x; i <= j + km; i += blockDim.x) at(i, j) *= inverse;
        __syncthreads();
        const int width = ju - j;
        for (int t = threadIdx.x; t < width * km; t += blockDim.x) {
          const int c = j + 1 + t / km;
          const int i = j + 1 + t % km;
          at(i, c) -= at(i, j) * at(j, c);
        }
      }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < ld; r += blockDim.x)
      ab[static_cast<long long>(j) * ld + r] = WinAt(win, ld, window, j, r);
    __syncthreads();
  }
  if (threadIdx.x == 0) info[blockIdx.x] = infoValue;
}

// -- solves --------------------------------------------------------------------------

struct WorkItem {
  int system;
  int column;
};

constexpr int kSolveCols = 2 * kWarp;  // right-hand sides per warp: two adjacent columns a lane
constexpr int kChunk = 16;             // rows staged per step
constexpr int kBuffers = 3;            // staged chunks: the current one and two ahead

template <class T>
struct PairOf;
template <>
struct PairOf<float> {
  using type = float2;
};
template <>
struct PairOf<double> {
  using type = double2;
};

// Asynchronous global -> shared copies of 4, 8 or 16 bytes, and their groups.
template <class T>
__device__ inline void CpAsync(T* dst, const T* src) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16, "copy size");
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
  else if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ inline void CpCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ inline void CpWaitAll() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ inline void CpWaitOne() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// The solution ring's slots: in FP64 twice the depth, the Cholesky
// substitution keeping a mirror of every slot at slot + depth so that its
// reads need no wrap (fewer integer instructions beside the FP64 ones, which
// bound it); in FP32 the wrapped ring alone (the mirror's larger staging cost
// the windowed FP32 solves more than the wrap did).
template <class T>
__host__ __device__ constexpr int RingSlots(int depth) {
  return sizeof(T) == sizeof(double) ? 2 * depth : depth;
}

// A solve launch's per-warp shared-memory plan.
struct SolvePlan {
  int depth;    // ring slots: the solve's reach + 1
  int bandCap;  // band values one staged chunk holds
  template <class T>
  __host__ __device__ long long Bytes() const {
    const long long pairs = static_cast<long long>(RingSlots<T>(depth)) * kWarp +
                            static_cast<long long>(kBuffers) * kChunk * kWarp;
    const long long b = pairs * 2 * sizeof(T) + static_cast<long long>(kBuffers) * (bandCap + kChunk) * sizeof(T) +
                        static_cast<long long>(kBuffers) * kChunk * sizeof(int);
    return (b + 15) / 16 * 16;
  }
};

// One warp's staging: the solution ring (RingSlots x 32 lane pairs, each
// lane's own columns; in FP64 slots depth.. mirror slots 0..), and kBuffers of band columns, right-hand-side rows (lane
// pairs), row scales and pivots.
template <class T>
struct Stage {
  using T2 = typename PairOf<T>::type;
  T2* ring;
  T2* rhs;      // [buffer][kChunk][32]
  T* band;      // [buffer][bandCap]
  T* scale;     // [buffer][kChunk]
  int* pivot;   // [buffer][kChunk]
  int bandCap;
  __device__ Stage(unsigned char* base, const SolvePlan& plan) : bandCap(plan.bandCap) {
    ring = reinterpret_cast<T2*>(base);
    rhs = ring + static_cast<long long>(RingSlots<T>(plan.depth)) * kWarp;
    band = reinterpret_cast<T*>(rhs + static_cast<long long>(kBuffers) * kChunk * kWarp);
    scale = band + static_cast<long long>(kBuffers) * plan.bandCap;
    pivot = reinterpret_cast<int*>(scale + kBuffers * kChunk);
  }
  __device__ T2* Rhs(int buf, int r) const { return rhs + (buf * kChunk + r) * kWarp; }
  __device__ T* Band(int buf) const { return band + static_cast<long long>(buf) * bandCap; }
  __device__ T Scale(int buf, int r) const { return scale[buf * kChunk + r]; }
  __device__ int Pivot(int buf, int r) const { return pivot[buf * kChunk + r]; }
};

// The solve's view of one work item: the system, this lane's two columns.
template <class T>
struct Lane {
  using T2 = typename PairOf<T>::type;
  sl3dgpu_band_system s;
  T* x;
  int col;      // the lane's first column
  bool live0, live1;
  bool paired;  // both columns live and the pair 2 sizeof(T)-aligned
  __device__ T2 Load(int row) const {
    const T* at = x + static_cast<long long>(row) * s.nrhs + col;
    if (paired) return *reinterpret_cast<const T2*>(at);
    T2 v;
    v.x = live0 ? at[0] : T(0);
    v.y = live1 ? at[1] : T(0);
    return v;
  }
  __device__ void Store(int row, T2 v) const {
    T* at = x + static_cast<long long>(row) * s.nrhs + col;
    if (paired) {
      *reinterpret_cast<T2*>(at) = v;
    } else {
      if (live0) at[0] = v.x;
      if (live1) at[1] = v.y;
    }
  }
};

// Stage band columns [c0, c1) (ld values each, contiguous), right-hand-side
// rows [r0, min(r1, rhsEnd)) of this lane's columns, the scales of rows
// [r0, r1) and (pivots != null) pivots [p0, p1) into buffer `buf`, as one
// copy group.
template <class T>
__device__ inline void StageChunk(const Stage<T>& st, int buf, const T* ab, int ld, int c0, int c1,
                                  const Lane<T>& ln, int r0, int r1, const T* scales, const int* pivots, int p0,
                                  int p1, int lane, int rhsEnd = 0x7fffffff) {
  using T2 = typename PairOf<T>::type;
  const T* src = ab + static_cast<long long>(c0) * ld;
  T* band = st.Band(buf);
  const int count = (c1 - c0) * ld;
  for (int e = lane; e < count; e += kWarp) CpAsync(band + e, src + e);
  for (int r = r0; r < min(r1, rhsEnd); ++r) {
    T2* dst = st.Rhs(buf, r - r0) + lane;
    const T* at = ln.x + static_cast<long long>(r) * ln.s.nrhs + ln.col;
    if (ln.paired) {
      CpAsync(dst, reinterpret_cast<const T2*>(at));
    } else {
      if (ln.live0) CpAsync(reinterpret_cast<T*>(dst), at);
      if (ln.live1) CpAsync(reinterpret_cast<T*>(dst) + 1, at + 1);
    }
  }
  if (ln.s.scale >= 0)
    for (int r = r0 + lane; r < r1; r += kWarp) CpAsync(st.scale + buf * kChunk + (r - r0), scales + ln.s.scale + r);
  if (pivots != nullptr)
    for (int r = p0 + lane; r < p1; r += kWarp) CpAsync(st.pivot + buf * kChunk + (r - p0), pivots + r);
  CpCommit();
}

// The chunks of one substitution through the staging buffers: chunk c is
// staged two chunks ahead of its use, into buffer c % kBuffers.
template <class StageFn, class SolveFn>
__device__ inline void Pipeline(int chunks, StageFn stage, SolveFn solve) {
  if (chunks > 0) stage(0);
  if (chunks > 1) stage(1);
  for (int c = 0; c < chunks; ++c) {
    if (c + 1 < chunks)
      CpWaitOne();
    else
      CpWaitAll();
    __syncwarp();
    if (c + 2 < chunks) stage(c + 2);  // its buffer held chunk c - 1, done
    solve(c, c % kBuffers);
    __syncwarp();
  }
}

template <class T>
__device__ inline typename PairOf<T>::type Scaled(typename PairOf<T>::type v, T f) {
  v.x *= f;
  v.y *= f;
  return v;
}

// A right-hand side's value as the solve starts from it: zero at a pinned
// dof, scaled by the row's factor otherwise.
template <class T>
__device__ inline typename PairOf<T>::type Start(const Lane<T>& ln, const Stage<T>& st, int buf, int r, int row,
                                                 int lane) {
  using T2 = typename PairOf<T>::type;
  if (row == ln.s.pinned0 || row == ln.s.pinned1) {
    T2 z;
    z.x = z.y = T(0);
    return z;
  }
  T2 b = st.Rhs(buf, r)[lane];
  if (ln.s.scale >= 0) b = Scaled(b, st.Scale(buf, r));
  return b;
}

template <class T>
__device__ inline Lane<T> LaneOf(const sl3dgpu_band_system& s, T* rhs, int column, int lane) {
  using T2 = typename PairOf<T>::type;
  Lane<T> ln;
  ln.s = s;
  ln.x = rhs + s.rhs;
  ln.col = column + 2 * lane;
  ln.live0 = ln.col < s.nrhs;
  ln.live1 = ln.col + 1 < s.nrhs;
  ln.paired = ln.live1 && (reinterpret_cast<unsigned long long>(ln.x + ln.col) % sizeof(T2) == 0) &&
              (s.nrhs % 2 == 0);
  return ln;
}

// The ring slot of row j given the slot of row j0 (rows within depth of it).
__device__ inline int SlotBack(int slot, int t, int depth) {
  const int k = slot - t;
  return k < 0 ? k + depth : k;
}
__device__ inline int SlotAhead(int slot, int t, int depth) {
  const int k = slot + t;
  return k >= depth ? k - depth : k;
}

// Which rows a Cholesky solve covers (per system, windows[system] = {lo, hi}:
// the right-hand side is zero outside rows [lo, hi]).
enum SolveMode {
  kSolveAll = 0,         // every row (no windows)
  kSolveWindow = 1,      // rows lo .. n - 1 of both substitutions: y = 0 below lo
  kSolveCompletion = 2,  // the backward substitution's rows 0 .. lo - 1 after a
                         // windowed solve, from x at rows lo .. lo + kd - 1
};

// U^T U x = b, warp per (system, 64 right-hand sides): the forward and the
// backward substitution in chunks of rows whose band columns and
// right-hand-side rows are staged in shared memory two chunks ahead; each
// lane carries two columns (a band value read serves both), two independent
// partial sums per column, and the diagonal's reciprocal formed off the
// dependence chain.
//
// With windows, a right-hand side that is zero below row lo has y = 0 there,
// so the forward substitution starts at lo; the backward one stops at lo
// (kSolveWindow), and a later completion launch finishes rows below lo from
// the stored x (unscaled again) with y = 0.
// The substitutions with a lane's recent solutions in registers (bandwidth
// KD a compile-time constant; the FP32 solves use it): a chunk of kChunk = 16
// rows writes cur[0..15], and old[d] holds the row d + 1 before the chunk's
// first, so that every index is a constant and one unrolled chunk serves
// every chunk; after the chunk old shifts by 16 (2 KD moves at most). The
// solve is bound by instructions per row at a few warps an SM; this drops
// the shared-memory ring's loads and its wrap arithmetic, reads the band at
// constant offsets, and sums the terms t >= 2 before the one that waits on
// the row just solved.
template <class T2, int KD>
struct Window {
  T2 cur[kChunk];
  T2 old[KD];
  // row k - t of the chunk (k - t < 0: before it)
  template <int K, int TT>
  __device__ __forceinline__ const T2& At() const {
    if constexpr (K - TT >= 0)
      return cur[K - TT];
    else
      return old[TT - K - 1];
  }
  __device__ __forceinline__ void Shift() {
#pragma unroll
    for (int d = KD - 1; d >= kChunk; --d) old[d] = old[d - kChunk];
#pragma unroll
    for (int d = 0; d < (KD < kChunk ? KD : kChunk); ++d) old[d] = cur[kChunk - 1 - d];
  }
};

template <class T, int KD, bool FORWARD, int K>
__device__ __forceinline__ void WindowRow(const Lane<T>& ln, const Stage<T>& st, int buf, int rowBase, int rows,
                                          int hi, bool rhsLive, Window<typename PairOf<T>::type, KD>& w, T laneInv,
                                          int lane) {
  using T2 = typename PairOf<T>::type;
  constexpr int LD = KD + 1;
  // forward: row j = rowBase + K, U(j - t, j) = at[-t];
  // backward: row i = rowBase - K, U(i, i + t) = at[t (LD - 1)]
  const int row = FORWARD ? rowBase + K : rowBase - K;
  const int r = FORWARD ? K : rows - 1 - K;
  const T* at = st.Band(buf) + r * LD + KD;
  T2 zero;
  zero.x = zero.y = T(0);
  T2 acc0, acc1 = zero, acc2 = zero, acc3 = zero;
  if (FORWARD)
    acc0 = row <= hi ? Start(ln, st, buf, r, row, lane) : zero;
  else
    acc0 = rhsLive ? st.Rhs(buf, r)[lane] : zero;
  [&]<int... TS>(std::integer_sequence<int, TS...>) {
    // t = KD .. 2 into the sums by t % 4
    (
        [&] {
          constexpr int t = KD - TS;
          const T u = FORWARD ? at[-t] : at[t * (LD - 1)];
          const T2 y = w.template At<K, t>();
          T2& acc = (t & 3) == 0 ? acc0 : (t & 3) == 1 ? acc1 : (t & 3) == 2 ? acc2 : acc3;
          acc.x -= u * y.x;
          acc.y -= u * y.y;
        }(),
        ...);
  }(std::make_integer_sequence<int, KD - 1>{});
  T2 sum;
  sum.x = (acc0.x + acc1.x) + (acc2.x + acc3.x);
  sum.y = (acc0.y + acc1.y) + (acc2.y + acc3.y);
  const T u1 = FORWARD ? at[-1] : at[LD - 1];
  const T2 y1 = w.template At<K, 1>();
  sum.x -= u1 * y1.x;
  sum.y -= u1 * y1.y;
  const T inv = __shfl_sync(0xffffffffu, laneInv, K);  // 1 / U(row, row), from lane K
  T2 v;
  v.x = sum.x * inv;
  v.y = sum.y * inv;
  w.cur[K] = v;
  if (!FORWARD && ln.s.scale >= 0) v = Scaled(v, st.Scale(buf, r));
  ln.Store(row, v);
}

template <class T, int KD, bool FORWARD>
__device__ __forceinline__ void WindowChunk(const Lane<T>& ln, const Stage<T>& st, int buf, int rowBase, int rows,
                                            int hi, bool rhsLive, Window<typename PairOf<T>::type, KD>& w,
                                            int lane) {
  // the chunk's reciprocal diagonals, row k's in lane k, computed together
  // off the substitution's dependency chain
  T laneInv = T(1);
  if (lane < rows) laneInv = T(1) / st.Band(buf)[(FORWARD ? lane : rows - 1 - lane) * (KD + 1) + KD];
  [&]<int... KS>(std::integer_sequence<int, KS...>) {
    ((KS < rows ? WindowRow<T, KD, FORWARD, KS>(ln, st, buf, rowBase, rows, hi, rhsLive, w, laneInv, lane)
                : void()),
     ...);
  }(std::make_integer_sequence<int, kChunk>{});
  w.Shift();
}

// The FP32 ring form's row sum in the register form's order, so that a row
// comes out the same whichever form solves it: the terms t = reach .. 2 into
// four sums by t % 4 (descending t), the sums paired, then the t = 1 term.
// `at` points at the row's diagonal (forward: U(j - t, j) = at[-t];
// backward: U(i, i + t) = at[t (ld - 1)]); the ring holds row j - t (i + t)
// at SlotBack (SlotAhead) of `slot`.
template <bool FORWARD>
__device__ __forceinline__ float2 RowSum32(float2 start, const float* at, int ld, int reach, const float2* ring,
                                           int slot, int depth) {
  float2 a0 = start, a1 = make_float2(0.0f, 0.0f), a2 = a1, a3 = a1;
  for (int t = reach; t >= 2; --t) {
    const float u = FORWARD ? at[-t] : at[t * (ld - 1)];
    const float2 y = ring[(FORWARD ? SlotBack(slot, t, depth) : SlotAhead(slot, t, depth)) * kWarp];
    switch (t & 3) {
      case 0: a0.x -= u * y.x; a0.y -= u * y.y; break;
      case 1: a1.x -= u * y.x; a1.y -= u * y.y; break;
      case 2: a2.x -= u * y.x; a2.y -= u * y.y; break;
      default: a3.x -= u * y.x; a3.y -= u * y.y; break;
    }
  }
  float2 sum = make_float2((a0.x + a1.x) + (a2.x + a3.x), (a0.y + a1.y) + (a2.y + a3.y));
  if (reach >= 1) {
    const float u1 = FORWARD ? at[-1] : at[ld - 1];
    const float2 y1 = ring[(FORWARD ? SlotBack(slot, 1, depth) : SlotAhead(slot, 1, depth)) * kWarp];
    sum.x -= u1 * y1.x;
    sum.y -= u1 * y1.y;
  }
  return sum;
}

// old[0 .. KD - 1] from the wrapped ring: the KD rows before a
// substitution's third chunk, row first + 31 - d (forward) or first - 31 + d
// (backward) at old[d]; the ring holds row i at slot i % depth.
template <class T2, int KD, bool FORWARD>
__device__ __forceinline__ void WindowLoad(const T2* ring, int first, int depth, Window<T2, KD>& w) {
#pragma unroll
  for (int d = 0; d < KD; ++d) {
    const int row = FORWARD ? first + 2 * kChunk - 1 - d : first - 2 * kChunk + 1 + d;
    w.old[d] = ring[(row % depth) * kWarp];
  }
}

// The register form for chunk c >= 2 of a substitution, when the bandwidth
// is one it is built for (the operators' 3 (ngll - 1) + 2 and ngll - 1 for
// ngll 5 and 6); false: the ring form solves the chunk. The windows of the
// four bandwidths share the kernel's registers (a union: one is live).
template <class T2>
union WindowSet {
  Window<T2, 4> w4;
  Window<T2, 5> w5;
  Window<T2, 14> w14;
  Window<T2, 17> w17;
  __device__ WindowSet() {}
};

template <class T, bool FORWARD>
__device__ __forceinline__ bool WindowSolve(int kd, int c, const Lane<T>& ln, const Stage<T>& st, int buf,
                                            const typename PairOf<T>::type* ring, int first, int depth, int rowBase,
                                            int rows, int hi, bool rhsLive, WindowSet<typename PairOf<T>::type>& ws,
                                            int lane) {
  using T2 = typename PairOf<T>::type;
#define SL3D_WINDOW_CASE(KD)                                                             \
  case KD:                                                                               \
    if (c == 2) WindowLoad<T2, KD, FORWARD>(ring, first, depth, ws.w##KD);               \
    WindowChunk<T, KD, FORWARD>(ln, st, buf, rowBase, rows, hi, rhsLive, ws.w##KD, lane); \
    return true;
  switch (kd) {
    SL3D_WINDOW_CASE(4)
    SL3D_WINDOW_CASE(5)
    SL3D_WINDOW_CASE(14)
    SL3D_WINDOW_CASE(17)
    default: return false;
  }
#undef SL3D_WINDOW_CASE
}

template <class T>
__global__ void CholeskySolveKernel(const sl3dgpu_band_system* systems, const WorkItem* items, int itemCount,
                                    const T* bands, T* rhs, const T* scales, SolvePlan plan, const int2* windows,
                                    int mode) {
  using T2 = typename PairOf<T>::type;
  extern __shared__ __align__(16) unsigned char solveSmem[];
  const int warpInBlock = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const int warp = blockIdx.x * (blockDim.x / kWarp) + warpInBlock;
  if (warp >= itemCount) return;
  const Stage<T> st(solveSmem + warpInBlock * plan.Bytes<T>(), plan);
  const WorkItem item = items[warp];
  const Lane<T> ln = LaneOf(systems[item.system], rhs, item.column, lane);
  const int n = ln.s.n, kd = ln.s.ku, ld = kd + 1, depth = plan.depth;
  constexpr bool kMirror = RingSlots<T>(1) == 2;
  const T* ab = bands + ln.s.band;
  T2* ring = st.ring + lane;
  int lo = 0, hi = n - 1;
  if (mode != kSolveAll) {
    const int2 w = windows[item.system];
    lo = min(max(w.x, 0), n);
    hi = min(w.y, n - 1);
  }
  T2 zero;
  zero.x = zero.y = T(0);
  // The register form in FP32 only: FP64's solves are bound by its FP64
  // unit, and its window's 128 registers slowed them (the mirrored ring
  // serves them better).
  constexpr bool kWindowForm = sizeof(T) == sizeof(float);
  WindowSet<T2> window;  // the register form's recent solutions
  if (mode == kSolveCompletion) {
    // x at rows lo .. lo + kd - 1 (stored scaled) seeds the ring
    for (int r = lo; r < min(n, lo + kd); ++r) {
      T2 v = ln.Load(r);
      if (ln.s.scale >= 0) {
        const T f = scales[ln.s.scale + r];
        v.x /= f;
        v.y /= f;
      }
      ring[(r % depth) * kWarp] = v;
      if constexpr (kMirror) ring[(r % depth + depth) * kWarp] = v;
    }
  } else {
    // U^T y = b, forward: chunk c holds rows [lo + c kChunk, ...) and their
    // columns; right-hand-side rows above hi are zero and not read.
    const int chunks = (n - lo + kChunk - 1) / kChunk;
    int slot = lo % depth;  // the ring slot of the current row (row mod depth)
    Pipeline(
        chunks,
        [&](int c) {
          const int j0 = lo + c * kChunk, j1 = min(n, j0 + kChunk);
          StageChunk(st, c % kBuffers, ab, ld, j0, j1, ln, j0, min(j1, hi + 1), scales, nullptr, 0, 0, lane);
        },
        [&](int c, int buf) {
          const int j0 = lo + c * kChunk, j1 = min(n, j0 + kChunk);
          if (kWindowForm && c >= 2 &&
              WindowSolve<T, true>(kd, c, ln, st, buf, ring, lo, depth, j0, j1 - j0, hi, true, window, lane))
            return;
          const T* band = st.Band(buf);
          // the chunk's reciprocal diagonals, row j0 + k's in lane k: one
          // division a lane instead of one a row on every lane
          const T laneInv = lane < j1 - j0 ? T(1) / band[lane * ld + kd] : T(1);
          for (int j = j0; j < j1; ++j) {
            const T* column = band + (j - j0) * ld + kd;  // column[-t] = U(j - t, j)
            const T inv = __shfl_sync(0xffffffffu, laneInv, j - j0);
            T2 a = j <= hi ? Start(ln, st, buf, j - j0, j, lane) : zero;
            T2 b = zero;
            const int reach = min(kd, j - lo);
            if constexpr (sizeof(T) == sizeof(float)) {
              const float2 sum = RowSum32<true>(a, column, ld, reach, ring, slot, depth);
              const T2 y = make_float2(sum.x * inv, sum.y * inv);
              ring[slot * kWarp] = y;
              ln.Store(j, y);
              slot = SlotAhead(slot, 1, depth);
              continue;
            }
            // row j - t: slot + depth - t of the mirrored ring, else wrapped
            const T2* back = ring + (slot + depth) * kWarp;
            int t = 1;
            for (; t + 1 <= reach; t += 2) {
              const T u0 = column[-t], u1 = column[-t - 1];
              const T2 y0 = kMirror ? back[-t * kWarp] : ring[SlotBack(slot, t, depth) * kWarp];
              const T2 y1 = kMirror ? back[-(t + 1) * kWarp] : ring[SlotBack(slot, t + 1, depth) * kWarp];
              a.x -= u0 * y0.x;
              a.y -= u0 * y0.y;
              b.x -= u1 * y1.x;
              b.y -= u1 * y1.y;
            }
            if (t <= reach) {
              const T u0 = column[-t];
              const T2 y0 = kMirror ? back[-t * kWarp] : ring[SlotBack(slot, t, depth) * kWarp];
              a.x -= u0 * y0.x;
              a.y -= u0 * y0.y;
            }
            T2 y;
            y.x = (a.x + b.x) * inv;
            y.y = (a.y + b.y) * inv;
            ring[slot * kWarp] = y;
            if constexpr (kMirror) ring[(slot + depth) * kWarp] = y;
            ln.Store(j, y);
            slot = SlotAhead(slot, 1, depth);
          }
        });
  }
  // U x = y, backward over rows [bottom, top): chunk c holds rows [i0, i1)
  // counted from the top and the columns [i0, i1 + kd) their updates come
  // from; below lo (completion) y = 0 and is not read.
  const int top = mode == kSolveCompletion ? lo : n, bottom = mode == kSolveCompletion ? 0 : lo;
  const int rhsEnd = mode == kSolveCompletion ? 0 : n;
  const int chunks = (top - bottom + kChunk - 1) / kChunk;
  int slot = ((top - 1) % depth + depth) % depth;
  Pipeline(
      chunks,
      [&](int c) {
        const int i1 = top - c * kChunk, i0 = max(bottom, i1 - kChunk);
        StageChunk(st, c % kBuffers, ab, ld, i0, min(n, i1 + kd), ln, i0, i1, scales, nullptr, 0, 0, lane, rhsEnd);
      },
      [&](int c, int buf) {
        const int i1 = top - c * kChunk, i0 = max(bottom, i1 - kChunk);
        if (kWindowForm && c >= 2 &&
            WindowSolve<T, false>(kd, c, ln, st, buf, ring, top - 1, depth, i1 - 1, i1 - i0, 0, rhsEnd > 0, window, lane))
          return;
        const T* band = st.Band(buf);
        const T laneInv = lane < i1 - i0 ? T(1) / band[lane * ld + kd] : T(1);  // row i0 + k's in lane k
        for (int i = i1 - 1; i >= i0; --i) {
          const int r = i - i0;
          const T inv = __shfl_sync(0xffffffffu, laneInv, r);
          T2 a = rhsEnd > 0 ? st.Rhs(buf, r)[lane] : zero;
          T2 b = zero;
          const int reach = min(kd, n - 1 - i);
          if constexpr (sizeof(T) == sizeof(float)) {
            const float2 sum = RowSum32<false>(a, band + r * ld + kd, ld, reach, ring, slot, depth);
            T2 v = make_float2(sum.x * inv, sum.y * inv);
            ring[slot * kWarp] = v;
            if (ln.s.scale >= 0) v = Scaled(v, st.Scale(buf, r));
            ln.Store(i, v);
            slot = SlotBack(slot, 1, depth);
            continue;
          }
          // row i + t: slot + t of the mirrored ring, else wrapped
          const T2* ahead = ring + slot * kWarp;
          int t = 1;
          for (; t + 1 <= reach; t += 2) {
            const T u0 = band[(r + t) * ld + kd - t];  // U(i, i + t)
            const T u1 = band[(r + t + 1) * ld + kd - t - 1];
            const T2 y0 = kMirror ? ahead[t * kWarp] : ring[SlotAhead(slot, t, depth) * kWarp];
            const T2 y1 = kMirror ? ahead[(t + 1) * kWarp] : ring[SlotAhead(slot, t + 1, depth) * kWarp];
            a.x -= u0 * y0.x;
            a.y -= u0 * y0.y;
            b.x -= u1 * y1.x;
            b.y -= u1 * y1.y;
          }
          if (t <= reach) {
            const T u0 = band[(r + t) * ld + kd - t];
            const T2 y0 = kMirror ? ahead[t * kWarp] : ring[SlotAhead(slot, t, depth) * kWarp];
            a.x -= u0 * y0.x;
            a.y -= u0 * y0.y;
          }
          T2 v;
          v.x = (a.x + b.x) * inv;
          v.y = (a.y + b.y) * inv;
          ring[slot * kWarp] = v;
          if constexpr (kMirror) ring[(slot + depth) * kWarp] = v;
          if (ln.s.scale >= 0) v = Scaled(v, st.Scale(buf, r));
          ln.Store(i, v);
          slot = SlotBack(slot, 1, depth);
        }
      });
}

// P L U x = b (LAPACK dgbtrs's order), warp per (system, 64 right-hand
// sides), staged like the Cholesky solve. Forward: the window x_j .. x_{j+kl}
// in the ring, the interchanges and eliminations in turn; right-hand-side row
// j + kl enters as row j is eliminated. Backward: U with kl + ku
// superdiagonals.
template <class T>
__global__ void LuSolveKernel(const sl3dgpu_band_system* systems, const WorkItem* items, int itemCount,
                              const T* bands, const int* pivotsAll, T* rhs, const T* scales, SolvePlan plan) {
  using T2 = typename PairOf<T>::type;
  extern __shared__ __align__(16) unsigned char solveSmem[];
  const int warpInBlock = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  const int warp = blockIdx.x * (blockDim.x / kWarp) + warpInBlock;
  if (warp >= itemCount) return;
  const Stage<T> st(solveSmem + warpInBlock * plan.Bytes<T>(), plan);
  const WorkItem item = items[warp];
  const Lane<T> ln = LaneOf(systems[item.system], rhs, item.column, lane);
  const int n = ln.s.n, kl = ln.s.kl, ku = ln.s.ku, kv = kl + ku, ld = 2 * kl + ku + 1, depth = plan.depth;
  const T* ab = bands + ln.s.band;
  const int* pivots = pivotsAll + ln.s.pivots;
  T2* ring = st.ring + lane;
  const int chunks = (n + kChunk - 1) / kChunk;
  // The first kl rows of the window, before the chunks (row i in slot i).
  for (int i = 0; i < min(kl, n); ++i) {
    T2 b;
    b.x = b.y = T(0);
    if (i != ln.s.pinned0 && i != ln.s.pinned1) {
      b = ln.Load(i);
      if (ln.s.scale >= 0) b = Scaled(b, scales[ln.s.scale + i]);
    }
    ring[i * kWarp] = b;
  }
  // Forward chunk c: rows j in [j0, j1), their columns and pivots, and the
  // right-hand-side rows [j0 + kl, j1 + kl) that enter the window.
  int slot = 0;
  Pipeline(
      chunks,
      [&](int c) {
        const int j0 = c * kChunk, j1 = min(n, j0 + kChunk);
        StageChunk(st, c % kBuffers, ab, ld, j0, j1, ln, min(n, j0 + kl), min(n, j1 + kl), scales, pivots, j0, j1,
                   lane);
      },
      [&](int c, int buf) {
        const int j0 = c * kChunk, j1 = min(n, j0 + kChunk);
        const T* band = st.Band(buf);
        for (int j = j0; j < j1; ++j) {
          if (j + kl < n) ring[SlotAhead(slot, kl, depth) * kWarp] = Start(ln, st, buf, j - j0, j + kl, lane);
          T2 xj = ring[slot * kWarp];
          if (j + 1 < n) {
            // a pivot row lies within the window (dgbtrf's kl rows below);
            // one outside it is ignored rather than followed out of the ring
            const int p = st.Pivot(buf, j - j0);
            if (p > j && p - j <= kl) {
              T2* sp = ring + SlotAhead(slot, p - j, depth) * kWarp;
              const T2 t = *sp;
              *sp = xj;
              xj = t;
              ring[slot * kWarp] = xj;
            }
            const int lm = min(kl, n - 1 - j);
            const T* column = band + (j - j0) * ld + kv;  // column[t] = L(j + t, j)
            for (int t = 1; t <= lm; ++t) {
              T2* si = ring + SlotAhead(slot, t, depth) * kWarp;
              T2 v = *si;
              v.x -= column[t] * xj.x;
              v.y -= column[t] * xj.y;
              *si = v;
            }
          }
          ln.Store(j, xj);
          slot = SlotAhead(slot, 1, depth);
        }
      });
  // Backward chunk c: rows [i0, i1) from the end, columns [i0, i1 + kv).
  slot = (n - 1) % depth;
  Pipeline(
      chunks,
      [&](int c) {
        const int i1 = n - c * kChunk, i0 = max(0, i1 - kChunk);
        StageChunk(st, c % kBuffers, ab, ld, i0, min(n, i1 + kv), ln, i0, i1, scales, nullptr, 0, 0, lane);
      },
      [&](int c, int buf) {
        const int i1 = n - c * kChunk, i0 = max(0, i1 - kChunk);
        const T* band = st.Band(buf);
        for (int i = i1 - 1; i >= i0; --i) {
          const int r = i - i0;
          const T inv = T(1) / band[r * ld + kv];
          T2 a = st.Rhs(buf, r)[lane];
          T2 b;
          b.x = b.y = T(0);
          const int reach = min(kv, n - 1 - i);
          int t = 1;
          for (; t + 1 <= reach; t += 2) {
            const T u0 = band[(r + t) * ld + kv - t];  // U(i, i + t)
            const T u1 = band[(r + t + 1) * ld + kv - t - 1];
            const T2 y0 = ring[SlotAhead(slot, t, depth) * kWarp];
            const T2 y1 = ring[SlotAhead(slot, t + 1, depth) * kWarp];
            a.x -= u0 * y0.x;
            a.y -= u0 * y0.y;
            b.x -= u1 * y1.x;
            b.y -= u1 * y1.y;
          }
          if (t <= reach) {
            const T u0 = band[(r + t) * ld + kv - t];
            const T2 y0 = ring[SlotAhead(slot, t, depth) * kWarp];
            a.x -= u0 * y0.x;
            a.y -= u0 * y0.y;
          }
          T2 v;
          v.x = (a.x + b.x) * inv;
          v.y = (a.y + b.y) * inv;
          ring[slot * kWarp] = v;
          if (ln.s.scale >= 0) v = Scaled(v, st.Scale(buf, r));
          ln.Store(i, v);
          slot = SlotBack(slot, 1, depth);
        }
      });
}

int Validate(const sl3dgpu_band_system* hostSystems, int count, bool lu) {
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    if (s.n < 0 || s.kl < 0 || s.ku < 0 || s.nrhs < 0) {
      SetError("band system " + std::to_string(i) + ": negative size");
      return SL3DGPU_ERR_ARGUMENT;
    }
    const int reach = lu ? s.kl + s.ku : s.ku;
    if (reach >= kRing || (lu && s.kl >= kRing)) {
      SetError("band system " + std::to_string(i) + ": bandwidth beyond the solver's ring");
      return SL3DGPU_ERR_ARGUMENT;
    }
  }
  return SL3DGPU_OK;
}

}  // namespace

int BandFactorBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems,
                    int count, double* bands, int* pivots, int* info, int lu, cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  if (int st = Validate(hostSystems, count, lu != 0); st != SL3DGPU_OK) return st;
  int maxWindow = 0;
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    const int window = lu ? (s.kl + s.ku + 1) * (2 * s.kl + s.ku + 1) : (s.ku + 1) * (s.ku + 1);
    maxWindow = std::max(maxWindow, window);
  }
  const size_t smem = static_cast<size_t>(maxWindow) * sizeof(double);
  if (smem > 200 * 1024) {
    SetError("band factor window exceeds shared memory");
    return SL3DGPU_ERR_ARGUMENT;
  }
  prof::Scope scope(prof::kOther, stream);
  if (lu) {
    SL3D_CUDA(AllowDynamicSmem(LuFactorKernel));
    LuFactorKernel<<<count, 128, smem, stream>>>(devSystems, bands, pivots, info);
  } else {
    SL3D_CUDA(AllowDynamicSmem(CholeskyFactorKernel));
    CholeskyFactorKernel<<<count, 128, smem, stream>>>(devSystems, bands, info);
  }
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// The work items of a batch: one per (system, 64 right-hand sides).
std::vector<int2> BandWorkItems(const sl3dgpu_band_system* hostSystems, int count) {
  std::vector<int2> items;
  for (int i = 0; i < count; ++i)
    for (int c = 0; c < hostSystems[i].nrhs; c += kSolveCols) items.push_back(make_int2(i, c));
  return items;
}

namespace {
template <class T>
int SolveBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
               const int2* devItems, int itemCount, const T* bands, const int* pivots, T* rhs, const T* scales,
               int lu, cudaStream_t stream, const int2* windows = nullptr, int mode = kSolveAll) {
  if (itemCount == 0) return SL3DGPU_OK;
  if ((mode != kSolveAll) != (windows != nullptr) || (lu && mode != kSolveAll)) {
    SetError("band solve: row windows go with a windowed Cholesky solve");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (int st = Validate(hostSystems, count, lu != 0); st != SL3DGPU_OK) return st;
  // The ring spans the solve's reach (kd; kl + ku for LU); a staged chunk the
  // band columns of kChunk rows and of the reach beyond them.
  int reach = 0, ldMax = 0;
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    reach = std::max(reach, lu ? s.kl + s.ku : s.ku);
    ldMax = std::max(ldMax, lu ? 2 * s.kl + s.ku + 1 : s.ku + 1);
  }
  SolvePlan plan{};
  plan.depth = reach + 1;
  plan.bandCap = (kChunk + reach) * ldMax;
  const size_t perWarp = static_cast<size_t>(plan.Bytes<T>());
  int warpsPerBlock = 4;
  while (warpsPerBlock > 1 && perWarp * warpsPerBlock > 100 * 1024) warpsPerBlock /= 2;
  const size_t smem = perWarp * warpsPerBlock;
  if (smem > 200 * 1024) {
    SetError("band solve: the staged band exceeds shared memory");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const int blocks = (itemCount + warpsPerBlock - 1) / warpsPerBlock;
  const auto* items = reinterpret_cast<const WorkItem*>(devItems);
  double flops = 0.0, bytes = 0.0;
  for (int i = 0; i < count; ++i) {
    const auto& s = hostSystems[i];
    const double n = s.n, r = s.nrhs;
    flops += lu ? r * (2.0 * n * s.kl + 2.0 * n * (s.kl + s.ku) + n) : r * (4.0 * n * s.ku + 2.0 * n);
    bytes += 4.0 * sizeof(T) * n * r + sizeof(T) * n * (lu ? 2 * s.kl + s.ku + 1 : s.ku + 1);
  }
  prof::Scope scope(sizeof(T) == sizeof(float) ? prof::kBandSolve32 : prof::kBandSolve, stream, flops, bytes);
  if (lu) {
    SL3D_CUDA(AllowDynamicSmem(LuSolveKernel<T>));
    LuSolveKernel<T><<<blocks, warpsPerBlock * kWarp, smem, stream>>>(devSystems, items, itemCount, bands, pivots,
                                                                     rhs, scales, plan);
  } else {
    SL3D_CUDA(AllowDynamicSmem(CholeskySolveKernel<T>));
    CholeskySolveKernel<T><<<blocks, warpsPerBlock * kWarp, smem, stream>>>(devSystems, items, itemCount, bands,
                                                                           rhs, scales, plan, windows, mode);
  }
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}
}  // namespace

int BandSolveBatch(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                   const int2* devItems, int itemCount, const double* bands, const int* pivots, double* rhs,
                   const double* scales, int lu, cudaStream_t stream) {
  return SolveBatch<double>(devSystems, hostSystems, count, devItems, itemCount, bands, pivots, rhs, scales, lu,
                            stream);
}

// The same solves in FP32 (the mixed form's correction passes).
int BandSolveBatchF(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                    const int2* devItems, int itemCount, const float* bands, const int* pivots, float* rhs,
                    const float* scales, int lu, cudaStream_t stream) {
  return SolveBatch<float>(devSystems, hostSystems, count, devItems, itemCount, bands, pivots, rhs, scales, lu,
                           stream);
}

int BandSolveWindowF(const sl3dgpu_band_system* devSystems, const sl3dgpu_band_system* hostSystems, int count,
                     const int2* devItems, int itemCount, const float* bands, float* rhs, const float* scales,
                     const int2* windows, bool completion, cudaStream_t stream) {
  return SolveBatch<float>(devSystems, hostSystems, count, devItems, itemCount, bands, nullptr, rhs, scales, 0,
                           stream, windows, completion ? kSolveCompletion : kSolveWindow);
}

namespace {
// One block per system of up to three lists: rows [lo, hi] of its right-hand
// sides set to zero.
struct ZeroList {
  const sl3dgpu_band_system* systems;
  const int2* windows;
  int count;
  float* rhs;
};
__global__ void ZeroRowsKernel(ZeroList a, ZeroList b, ZeroList c) {
  int i = blockIdx.x;
  const ZeroList* list = &a;
  if (i >= a.count) {
    i -= a.count;
    list = &b;
    if (i >= b.count) {
      i -= b.count;
      list = &c;
    }
  }
  const sl3dgpu_band_system s = list->systems[i];
  const int2 w = list->windows[i];
  const int lo = max(w.x, 0), hi = min(w.y, s.n - 1);
  if (hi < lo) return;
  float* base = list->rhs + s.rhs + static_cast<long long>(lo) * s.nrhs;
  const long long count = static_cast<long long>(hi - lo + 1) * s.nrhs;
  for (long long e = threadIdx.x; e < count; e += blockDim.x) base[e] = 0.0f;
}
}  // namespace

void LaunchZeroRows(const sl3dgpu_band_system* s0, const int2* w0, int n0, float* rhs0,
                    const sl3dgpu_band_system* s1, const int2* w1, int n1, float* rhs1,
                    const sl3dgpu_band_system* s2, const int2* w2, int n2, float* rhs2, cudaStream_t stream) {
  const int blocks = n0 + n1 + n2;
  if (blocks == 0) return;
  ZeroRowsKernel<<<blocks, 256, 0, stream>>>(ZeroList{s0, w0, n0, rhs0}, ZeroList{s1, w1, n1, rhs1},
                                             ZeroList{s2, w2, n2, rhs2});
}

}  // namespace sl3dgpu

// -- the C ABI -------------------------------------------------------------------------

using namespace sl3dgpu;

namespace {

// One host-resident system through the batched kernels (the drop-in form of
// detail::BandCholeskyFactor and friends): copies in, one launch, copies out.
struct DeviceScratch {
  std::vector<void*> owned;
  ~DeviceScratch() {
    for (void* p : owned) cudaFree(p);
  }
  template <class T>
  T* Alloc(size_t count) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    owned.push_back(p);
    return static_cast<T*>(p);
  }
};

}  // namespace

extern "C" int sl3dgpu_band_cholesky_factor(double* ab, int n, int kd) {
  if (n < 0 || kd < 0) {
    SetError("negative order or bandwidth");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (n == 0) return 0;
  DeviceScratch scratch;
  const size_t size = static_cast<size_t>(kd + 1) * n;
  auto* band = scratch.Alloc<double>(size);
  auto* sys = scratch.Alloc<sl3dgpu_band_system>(1);
  auto* info = scratch.Alloc<int>(1);
  if (!band || !sys || !info) {
    SetError("device allocation failed");
    return SL3DGPU_ERR_CUDA;
  }
  sl3dgpu_band_system s{};
  s.n = n;
  s.kl = kd;
  s.ku = kd;
  s.scale = -1;
  s.pinned0 = s.pinned1 = -1;
  SL3D_CUDA(cudaMemcpy(band, ab, size * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(sys, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (int st = BandFactorBatch(sys, &s, 1, band, nullptr, info, 0, nullptr); st != SL3DGPU_OK)
    return st;
  int result = 0;
  SL3D_CUDA(cudaMemcpy(&result, info, sizeof(int), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(ab, band, size * sizeof(double), cudaMemcpyDeviceToHost));
  return result;
}

namespace {

// Column-major (n x nrhs) host right-hand sides through the row-major device
// solve, and back.
int SolveHost(const double* ab, size_t bandSize, const int* pivots, int n, int kl, int ku,
              double* b, int nrhs, int lu) {
  if (n == 0 || nrhs == 0) return SL3DGPU_OK;
  DeviceScratch scratch;
  auto* band = scratch.Alloc<double>(bandSize);
  auto* rhs = scratch.Alloc<double>(static_cast<size_t>(n) * nrhs);
  auto* sys = scratch.Alloc<sl3dgpu_band_system>(1);
  auto* piv = scratch.Alloc<int>(static_cast<size_t>(n));
  const auto hostItems = BandWorkItems(nullptr, 0);
  sl3dgpu_band_system s{};
  s.n = n;
  s.kl = kl;
  s.ku = ku;
  s.nrhs = nrhs;
  s.scale = -1;
  s.pinned0 = s.pinned1 = -1;
  auto items = BandWorkItems(&s, 1);
  auto* devItems = scratch.Alloc<int2>(items.size());
  if (!band || !rhs || !sys || !piv || !devItems) {
    SetError("device allocation failed");
    return SL3DGPU_ERR_CUDA;
  }
  std::vector<double> rowMajor(static_cast<size_t>(n) * nrhs);
  for (int k = 0; k < nrhs; ++k)
    for (int i = 0; i < n; ++i) rowMajor[static_cast<size_t>(i) * nrhs + k] = b[static_cast<size_t>(k) * n + i];
  SL3D_CUDA(cudaMemcpy(band, ab, bandSize * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(rhs, rowMajor.data(), rowMajor.size() * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(sys, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (lu) SL3D_CUDA(cudaMemcpy(piv, pivots, static_cast<size_t>(n) * sizeof(int), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(devItems, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
  if (int st = BandSolveBatch(sys, &s, 1, devItems, static_cast<int>(items.size()), band, piv, rhs,
                              nullptr, lu, nullptr);
      st != SL3DGPU_OK)
    return st;
  SL3D_CUDA(cudaMemcpy(rowMajor.data(), rhs, rowMajor.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int k = 0; k < nrhs; ++k)
    for (int i = 0; i < n; ++i) b[static_cast<size_t>(k) * n + i] = rowMajor[static_cast<size_t>(i) * nrhs + k];
  return SL3DGPU_OK;
}

}  // namespace

extern "C" int sl3dgpu_band_cholesky_solve(const double* ab, int n, int kd, double* b, int nrhs) {
  if (n < 0 || kd < 0 || nrhs < 0) {
    SetError("negative order, bandwidth or column count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return SolveHost(ab, static_cast<size_t>(kd + 1) * n, nullptr, n, kd, kd, b, nrhs, 0);
}

extern "C" int sl3dgpu_band_lu_factor(double* ab, int n, int kl, int ku, int* pivots) {
  if (n < 0 || kl < 0 || ku < 0) {
    SetError("negative order or bandwidth");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (n == 0) return 0;
  DeviceScratch scratch;
  const size_t size = static_cast<size_t>(2 * kl + ku + 1) * n;
  auto* band = scratch.Alloc<double>(size);
  auto* sys = scratch.Alloc<sl3dgpu_band_system>(1);
  auto* info = scratch.Alloc<int>(1);
  auto* piv = scratch.Alloc<int>(static_cast<size_t>(n));
  if (!band || !sys || !info || !piv) {
    SetError("device allocation failed");
    return SL3DGPU_ERR_CUDA;
  }
  sl3dgpu_band_system s{};
  s.n = n;
  s.kl = kl;
  s.ku = ku;
  s.scale = -1;
  s.pinned0 = s.pinned1 = -1;
  SL3D_CUDA(cudaMemcpy(band, ab, size * sizeof(double), cudaMemcpyHostToDevice));
  SL3D_CUDA(cudaMemcpy(sys, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (int st = BandFactorBatch(sys, &s, 1, band, piv, info, 1, nullptr); st != SL3DGPU_OK) return st;
  int result = 0;
  SL3D_CUDA(cudaMemcpy(&result, info, sizeof(int), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(ab, band, size * sizeof(double), cudaMemcpyDeviceToHost));
  SL3D_CUDA(cudaMemcpy(pivots, piv, static_cast<size_t>(n) * sizeof(int), cudaMemcpyDeviceToHost));
  return result;
}

extern "C" int sl3dgpu_band_lu_solve(const double* ab, int n, int kl, int ku, const int* pivots,
                                     double* b, int nrhs) {
  if (n < 0 || kl < 0 || ku < 0 || nrhs < 0) {
    SetError("negative order, bandwidth or column count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return SolveHost(ab, static_cast<size_t>(2 * kl + ku + 1) * n, pivots, n, kl, ku, b, nrhs, 1);
}

extern "C" int sl3dgpu_band_factor_batch(const sl3dgpu_band_system* dev_systems,
                                         const sl3dgpu_band_system* host_systems, int count,
                                         double* bands, int* pivots, int* info, int lu,
                                         void* stream) {
  return BandFactorBatch(dev_systems, host_systems, count, bands, pivots, info, lu,
                         AsStream(stream));
}

extern "C" int sl3dgpu_band_solve_batch(const sl3dgpu_band_system* dev_systems,
                                        const sl3dgpu_band_system* host_systems, int count,
                                        const int* dev_items, int item_count, const double* bands,
                                        const int* pivots, double* rhs, const double* scales,
                                        int lu, void* stream) {
  return BandSolveBatch(dev_systems, host_systems, count, reinterpret_cast<const int2*>(dev_items),
                        item_count, bands, pivots, rhs, scales, lu, AsStream(stream));
}

extern "C" int sl3dgpu_band_solve_batch_f32(const sl3dgpu_band_system* dev_systems,
                                            const sl3dgpu_band_system* host_systems, int count,
                                            const int* dev_items, int item_count, const float* bands,
                                            float* rhs, const float* scales, const int* dev_windows,
                                            int mode, void* stream) {
  const auto* items = reinterpret_cast<const int2*>(dev_items);
  const auto* windows = reinterpret_cast<const int2*>(dev_windows);
  if (mode == 0)
    return SolveBatch<float>(dev_systems, host_systems, count, items, item_count, bands, nullptr, rhs, scales, 0,
                             AsStream(stream), windows, kSolveAll);
  if (mode != 1 && mode != 2) {
    SetError("band solve: mode must be 0, 1 or 2");
    return SL3DGPU_ERR_ARGUMENT;
  }
  return BandSolveWindowF(dev_systems, host_systems, count, items, item_count, bands, rhs, scales, windows,
                          mode == 2, AsStream(stream));
}

extern "C" int sl3dgpu_band_work_items(const sl3dgpu_band_system* host_systems, int count,
                                       int* items, int capacity) {
  const auto list = BandWorkItems(host_systems, count);
  if (items != nullptr) {
    if (capacity < static_cast<int>(list.size())) {
      SetError("work item buffer too small");
      return SL3DGPU_ERR_ARGUMENT;
    }
    for (size_t i = 0; i < list.size(); ++i) {
      items[2 * i] = list[i].x;
      items[2 * i + 1] = list[i].y;
    }
  }
  return static_cast<int>(list.size());
}
