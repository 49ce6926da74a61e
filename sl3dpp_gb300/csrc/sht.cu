// Spin-weighted spherical-harmonic transforms on the device (the GSHTrans
// transforms behind SurfaceGrid's batched calls, include/sl3dpp/SurfaceGrid.hpp:164-253).
//
// A transform factors into the Legendre contraction over degrees at every
// (order, colatitude) and a longitude FFT per colatitude ring:
//  - synthesis: H_m(theta_j) = sum_l Lambda^N_lm(theta_j) c_lm, then
//    f(theta_j, phi_k) = sum_m H_m(theta_j) e^{i m phi_k};
//  - analysis: G_m(theta_j) = (2 pi / nphi) w_j sum_k f e^{-i m phi_k}, then
//    c_lm = sum_j Lambda^N_lm(theta_j) G_m(theta_j).
// The contraction is one dense matrix product per (spin, order) with the
// batch's fields as columns, run here as a batched FP64 register-tiled GEMM;
// the FFT is a mixed-radix (2, 3, 4, 5) Stockham transform in shared memory,
// one warp per ring (warp-synchronous stages), several rings per CTA.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <numeric>

#include "profile.cuh"
#include "sht.cuh"
#include "tc_gemm.cuh"

namespace sl3dgpu {

int FftFriendly(int n) {
  for (int m = std::max(n, 1);; ++m) {
    int r = m;
    for (int p : {2, 3, 5})
      while (r % p == 0) r /= p;
    if (r == 1) return m;
  }
}

namespace {

// -- Wigner table --------------------------------------------------------------------

// The closed form at l0 = max(|m|, |N|) for N <= 0 (see the host oracle's
// restatement of the same algorithm): a product recursion in |m|.
__device__ double WignerStart(int N, int m, double c, double s) {
  const int M = abs(m), A = -N;
  if (M >= A) {
    double v = 1.0;
    for (int k = 0; k < 2 * A; ++k) v *= (m >= 0 ? s : c);
    for (int k = A; k < M; ++k)
      v *= sqrt((2.0 * k + 2.0) * (2.0 * k + 1.0) / ((k + 1.0 + N) * (k + 1.0 - N))) * c * s;
    if (m >= 0 && ((M - N) % 2 != 0)) v = -v;
    return v;
  }
  const int l = A;
  const double fact[5] = {1.0, 1.0, 2.0, 6.0, 24.0};
  double v = sqrt(fact[2 * l] / (fact[l + m] * fact[l - m]));
  for (int k = 0; k < l - m; ++k) v *= c;
  for (int k = 0; k < l + m; ++k) v *= s;
  if ((l + m) % 2 != 0) v = -v;
  return v;
}

// One thread per (order, colatitude): the three-term recurrence in l.
__global__ void WignerTableKernel(int lmax, int N, int ntheta, const double* theta,
                                  const int* rowOffset, double* table) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = static_cast<int>(blockIdx.y) - lmax;
  if (j >= ntheta) return;
  const double pi = 3.14159265358979323846;
  const int l0 = max(abs(m), abs(N));
  if (l0 > lmax) return;
  const bool mirrored = N > 0;
  const int Nr = mirrored ? -N : N;
  const double t = mirrored ? pi - theta[j] : theta[j];
  const double c = cos(0.5 * t), s = sin(0.5 * t);
  double* out = table + static_cast<long long>(rowOffset[m + lmax]) * ntheta + j;
  double dprev = 0.0, d = WignerStart(Nr, m, c, s);
  const double ct = cos(t);
  for (int l = l0; l <= lmax; ++l) {
    const double sign = mirrored && ((l + m) % 2 != 0) ? -1.0 : 1.0;
    out[static_cast<long long>(l - l0) * ntheta] = sign * sqrt((2.0 * l + 1.0) / (4.0 * pi)) * d;
    if (l == lmax) break;
    double next;
    if (l == 0) {
      next = ct;
    } else {
      const double a = (l + 1.0) * (2.0 * l + 1.0) /
                       sqrt(((l + 1.0) * (l + 1.0) - 1.0 * m * m) * ((l + 1.0) * (l + 1.0) - 1.0 * Nr * Nr));
      const double b = 1.0 * m * Nr / (l * (l + 1.0));
      const double e = sqrt((1.0 * l * l - 1.0 * m * m) * (1.0 * l * l - 1.0 * Nr * Nr)) / (l * (2.0 * l + 1.0));
      next = a * ((ct - b) * d - e * dprev);
    }
    dprev = d;
    d = next;
  }
}

// -- batched FP64 GEMM: C(i, n) = sum_k A(i, k) B(k, n) --------------------------------

constexpr int kBM = 64, kBN = 64, kBK = 16;

template <class T>
__global__ void __launch_bounds__(256) GemmKernel(const GemmItem* items, const T* A, const T* B, T* C,
                                                  bool accumulate) {
  const GemmItem it = items[blockIdx.z];
  const int i0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  if (i0 >= it.M || n0 >= it.N) return;
  __shared__ T As[kBK][kBM + 1];
  __shared__ T Bs[kBK][kBN];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const T* a = A + it.a;
  const T* b = B + it.b;
  T acc[4][4] = {};
  for (int k0 = 0; k0 < it.K; k0 += kBK) {
    if (it.sAk == 1) {
      for (int e = tid; e < kBM * kBK; e += 256) {
        const int kk = e % kBK, ii = e / kBK;
        const int i = i0 + ii, k = k0 + kk;
        As[kk][ii] = (i < it.M && k < it.K) ? a[static_cast<long long>(i) * it.sAi + k] : T(0);
      }
    } else {
      for (int e = tid; e < kBM * kBK; e += 256) {
        const int ii = e % kBM, kk = e / kBM;
        const int i = i0 + ii, k = k0 + kk;
        As[kk][ii] = (i < it.M && k < it.K)
                         ? a[static_cast<long long>(i) * it.sAi + static_cast<long long>(k) * it.sAk]
                         : T(0);
      }
    }
    for (int e = tid; e < kBK * kBN; e += 256) {
      const int nn = e % kBN, kk = e / kBN;
      const int n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = (n < it.N && k < it.K) ? b[static_cast<long long>(k) * it.ldb + n] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      T av[4], bv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) av[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int q = 0; q < 4; ++q) bv[q] = Bs[kk][tx + 16 * q];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] = fma(av[r], bv[q], acc[r][q]);
    }
    __syncthreads();
  }
  T* c = C + it.c;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty + 16 * r;
    if (i >= it.M) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int n = n0 + tx + 16 * q;
      if (n >= it.N) continue;
      T* out = c + static_cast<long long>(i) * it.ldc + n;
      *out = accumulate ? acc[r][q] + *out : acc[r][q];
    }
  }
}

// -- the same contraction for a few columns (N <= 16) --------------------------------------
//
// A batch of one to eight fields (the sea-level grid's single load, a few
// stacked channels) has N = 2 to 16 columns; the 64 x 64 tile above would
// spend 64 columns of FP64 FMAs on them, and FP64 is GB300's slow pipe. These
// kernels do only the N columns and stream the table once.

constexpr int kNarrowN = 16;

// Analysis (A row-major in k, sAk = 1): one warp per output row, the lanes
// over k (coalesced reads of the row), a shuffle sum at the end.
template <int NT>
__global__ void __launch_bounds__(256) GemmRowsNarrowKernel(const GemmItem* items, const double* A,
                                                            const double* B, double* C, bool accumulate) {
  const GemmItem it = items[blockIdx.y];
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= it.M) return;  // uniform over the warp
  const double* a = A + it.a + static_cast<long long>(i) * it.sAi;
  const double* b = B + it.b;
  double acc[NT] = {};
  for (int k = lane; k < it.K; k += 32) {
    const double av = a[k];
    const double* bk = b + static_cast<long long>(k) * it.ldb;
#pragma unroll
    for (int n = 0; n < NT; ++n)
      if (n < it.N) acc[n] = fma(av, bk[n], acc[n]);
  }
#pragma unroll
  for (int n = 0; n < NT; ++n)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc[n] += __shfl_xor_sync(0xffffffffu, acc[n], off);
  if (lane != 0) return;
  double* c = C + it.c + static_cast<long long>(i) * it.ldc;
#pragma unroll
  for (int n = 0; n < NT; ++n)
    if (n < it.N) c[n] = accumulate ? acc[n] + c[n] : acc[n];
}

// Synthesis (A column-major in i, sAi = 1): 32 output rows a block, one a
// lane (coalesced reads down the table's columns), k split over the eight
// warps and the partial sums added in shared memory.
template <int NT>
__global__ void __launch_bounds__(256) GemmColsNarrowKernel(const GemmItem* items, const double* A,
                                                            const double* B, double* C, bool accumulate) {
  __shared__ double part[8][NT][32];
  const GemmItem it = items[blockIdx.y];
  const int lane = threadIdx.x & 31, group = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  if (blockIdx.x * 32 >= it.M) return;  // uniform over the block
  const double* b = B + it.b;
  double acc[NT] = {};
  if (i < it.M) {
    const double* a = A + it.a + i;
#pragma unroll 4
    for (int k = group; k < it.K; k += 8) {
      const double av = a[static_cast<long long>(k) * it.sAk];
      const double* bk = b + static_cast<long long>(k) * it.ldb;
#pragma unroll
      for (int n = 0; n < NT; ++n)
        if (n < it.N) acc[n] = fma(av, bk[n], acc[n]);
    }
  }
#pragma unroll
  for (int n = 0; n < NT; ++n) part[group][n][lane] = acc[n];
  __syncthreads();
  if (group != 0 || i >= it.M) return;
  double* c = C + it.c + static_cast<long long>(i) * it.ldc;
#pragma unroll
  for (int n = 0; n < NT; ++n) {
    if (n >= it.N) break;
    double s = part[0][n][lane];
#pragma unroll
    for (int g = 1; g < 8; ++g) s += part[g][n][lane];
    c[n] = accumulate ? s + c[n] : s;
  }
}

template <int NT>
void LaunchNarrow(bool analysis, int maxM, int count, const GemmItem* items, const double* A, const double* B,
                  double* C, bool accumulate, cudaStream_t stream) {
  if (analysis)
    GemmRowsNarrowKernel<NT><<<dim3((maxM + 7) / 8, count), 256, 0, stream>>>(items, A, B, C, accumulate);
  else
    GemmColsNarrowKernel<NT><<<dim3((maxM + 31) / 32, count), 256, 0, stream>>>(items, A, B, C, accumulate);
}

// -- FFT ---------------------------------------------------------------------------------

template <class T2>
struct Real;
template <>
struct Real<double2> {
  using type = double;
};
template <>
struct Real<float2> {
  using type = float;
};

template <class T2>
__device__ inline T2 Make(typename Real<T2>::type x, typename Real<T2>::type y) {
  T2 v;
  v.x = x;
  v.y = y;
  return v;
}
template <class T2>
__device__ inline T2 Mul(T2 a, T2 b) {
  return Make<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class T2>
__device__ inline T2 Add(T2 a, T2 b) {
  return Make<T2>(a.x + b.x, a.y + b.y);
}
template <class T2>
__device__ inline T2 Sub(T2 a, T2 b) {
  return Make<T2>(a.x - b.x, a.y - b.y);
}

// A double-float value, hi + lo with |lo| <= ulp(hi) / 2 (about 48
// significant bits): the FP64 ring transforms' arithmetic on the FP32 pipe
// when the grid emulates FP64 (the FP64 pipe is GB300's slow one). Dekker's
// and Knuth's error-free transformations -- TwoSum, FastTwoSum and the
// FMA-based TwoProduct -- in their usual double-single forms: a sum's
// error is bounded by about 2^-46 (|a| + |b|) (the "sloppy" addition, whose
// bound is normwise, which is what a transform's error analysis uses), a
// product's by about 2^-46 |a b|. The _rn intrinsics keep the compiler from
// contracting the error terms into FMAs.
struct Df {
  float hi, lo;
  __host__ __device__ constexpr Df() : hi(0.0f), lo(0.0f) {}
  __host__ __device__ constexpr Df(float h, float l) : hi(h), lo(l) {}
  // the nearest double-float of d (constant-folded for literal constants)
  __host__ __device__ constexpr Df(double d)
      : hi(static_cast<float>(d)), lo(static_cast<float>(d - static_cast<double>(static_cast<float>(d)))) {}
  __host__ __device__ constexpr Df(int i) : Df(static_cast<double>(i)) {}
  __device__ explicit operator double() const { return static_cast<double>(hi) + static_cast<double>(lo); }
  __device__ explicit operator float() const { return __fadd_rn(hi, lo); }
};
struct Df2 {
  Df x, y;
};
template <>
struct Real<Df2> {
  using type = Df;
};

// FastTwoSum of s and an error term e (|s| >= |e| or s = 0)
__device__ inline Df Renormalise(float s, float e) {
  const float h = __fadd_rn(s, e);
  return Df(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ inline Df operator+(Df a, Df b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));  // TwoSum's error
  return Renormalise(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ inline Df operator-(Df a) { return Df(-a.hi, -a.lo); }
__device__ inline Df operator-(Df a, Df b) { return a + (-b); }
__device__ inline Df operator*(Df a, Df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // TwoProduct's error
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return Renormalise(p, e);
}

// A value of the storage type in the compute type, and back.
template <class C2, class T2>
__device__ inline C2 ToCompute(T2 v) {
  if constexpr (std::is_same_v<C2, T2>)
    return v;
  else
    return Make<C2>(typename Real<C2>::type(v.x), typename Real<C2>::type(v.y));
}
template <class T, class C>
__device__ inline T ToStorage(C v) {
  if constexpr (std::is_same_v<T, C>)
    return v;
  else
    return static_cast<T>(v);
}
template <class T2, class C2>
__device__ inline T2 ToStorage2(C2 v) {
  if constexpr (std::is_same_v<T2, C2>)
    return v;
  else
    return Make<T2>(ToStorage<typename Real<T2>::type>(v.x), ToStorage<typename Real<T2>::type>(v.y));
}

// The DFT of R values in registers, y_u = sum_q v_q e^{sign 2 pi i q u / R},
// for the radices of the plans (2, 3, 4, 5), with the roots as constants.
template <class T2, int R>
__device__ inline void Butterfly(T2 (&v)[R], int sign) {
  using T = typename Real<T2>::type;
  auto I = [](T2 a) { return Make<T2>(-a.y, a.x); };  // i a
  auto S = [](T k, T2 a) { return Make<T2>(k * a.x, k * a.y); };
  const T sg = sign > 0 ? T(1) : T(-1);
  if constexpr (R == 2) {
    const T2 a = v[0], b = v[1];
    v[0] = Add(a, b);
    v[1] = Sub(a, b);
  } else if constexpr (R == 3) {
    const T2 t = Add(v[1], v[2]);
    const T2 d = S(sg * T(0.86602540378443864676), Sub(v[1], v[2]));
    const T2 a = Sub(v[0], S(T(0.5), t));
    v[0] = Add(v[0], t);
    v[1] = Add(a, I(d));
    v[2] = Sub(a, I(d));
  } else if constexpr (R == 4) {
    const T2 a0 = Add(v[0], v[2]), a1 = Sub(v[0], v[2]);
    const T2 b0 = Add(v[1], v[3]), b1 = S(sg, Sub(v[1], v[3]));
    v[0] = Add(a0, b0);
    v[1] = Add(a1, I(b1));
    v[2] = Sub(a0, b0);
    v[3] = Sub(a1, I(b1));
  } else {
    static_assert(R == 5, "radix");
    const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
    const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);
    const T2 t1 = Add(v[1], v[4]), t2 = Add(v[2], v[3]);
    const T2 d1 = Sub(v[1], v[4]), d2 = Sub(v[2], v[3]);
    const T2 a1 = Add(v[0], Add(S(c1, t1), S(c2, t2)));
    const T2 a2 = Add(v[0], Add(S(c2, t1), S(c1, t2)));
    const T2 b1 = S(sg, Add(S(s1, d1), S(s2, d2)));
    const T2 b2 = S(sg, Sub(S(s2, d1), S(s1, d2)));
    v[0] = Add(v[0], Add(t1, t2));
    v[1] = Add(a1, I(b1));
    v[4] = Sub(a1, I(b1));
    v[2] = Add(a2, I(b2));
    v[3] = Sub(a2, I(b2));
  }
}

// One Stockham stage of radix R over one ring, by one warp: butterfly idx
// takes in[idx + q m] (q < R), twiddled by e^{sign 2 pi i q k stride / n}
// (k = idx mod Ns; the exponent stays below n), and writes
// out[(idx / Ns) Ns R + k + u Ns].
template <class T2, int R>
__device__ inline void WarpStage(const T2* in, T2* out, int n, int Ns, const T2* tw, int sign, int lane) {
  const int m = n / R;
  const int stride = n / (Ns * R);
  for (int idx = lane; idx < m; idx += kWarp) {
    const int blk = idx / Ns, k = idx - blk * Ns;
    T2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = in[idx + q * m];
    if (k > 0) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        T2 w = tw[q * k * stride];
        if (sign < 0) w.y = -w.y;
        v[q] = Mul(v[q], w);
      }
    }
    Butterfly<T2, R>(v, sign);
    const int base = blk * Ns * R + k;
#pragma unroll
    for (int u = 0; u < R; ++u) out[base + u * Ns] = v[u];
  }
}

// The whole transform of one ring by one warp, ping-ponging between a and b;
// returns 0 when the result is in a, 1 in b (the same for every ring).
template <class T2>
__device__ int WarpFft(T2* a, T2* b, const FftPlan& plan, const T2* tw, int sign, int lane) {
  T2* src = a;
  T2* dst = b;
  int Ns = 1;
  for (int s = 0; s < plan.stages; ++s) {
    const int r = plan.radix[s];
    if (r == 4)
      WarpStage<T2, 4>(src, dst, plan.n, Ns, tw, sign, lane);
    else if (r == 2)
      WarpStage<T2, 2>(src, dst, plan.n, Ns, tw, sign, lane);
    else if (r == 3)
      WarpStage<T2, 3>(src, dst, plan.n, Ns, tw, sign, lane);
    else
      WarpStage<T2, 5>(src, dst, plan.n, Ns, tw, sign, lane);
    __syncwarp();
    T2* t = src;
    src = dst;
    dst = t;
    Ns *= r;
  }
  return src == a ? 0 : 1;
}

// -- two-stage ring transforms in registers -----------------------------------------------
//
// For n = R1 R2 with R1, R2 <= 32 the ring transform is two Stockham stages
// of radix R1 and R2 with one butterfly a lane: stage A (R2 butterflies)
// takes a[idx + q R2] (q < R1) and writes b[idx R1 + u]; stage B (R1
// butterflies) takes b[idx + q R1] twiddled by e^{sign 2 pi i q idx / n} and
// writes a[idx + u R1]. Each butterfly is an R-point transform held in
// registers (RegFft: the Stockham algorithm again, radices 4, 2, 3, 5, every
// index a compile-time constant). The stage-B twiddles are kept as
// twB[q R1 + idx], so a warp's loads of one q are consecutive.

// The radix of the next in-register stage of an R-point transform.
__host__ __device__ constexpr int NextRadix(int r) { return r % 4 == 0 ? 4 : r % 2 == 0 ? 2 : r % 3 == 0 ? 3 : 5; }

// Whether an R-point transform factors into the radices 2, 3, 4, 5.
__host__ __device__ constexpr bool Smooth(int r) {
  while (r > 1) {
    const int f = NextRadix(r);
    if (r % f != 0) return false;
    r /= f;
  }
  return true;
}

// The in-register stages of an R-point transform from stage width Ns on;
// tw[j] = e^{2 pi i j / n} (n a multiple of R), Sign +1 or -1.
template <class T2, int R, int Ns, int Sign, int n>
__device__ inline void RegStages(T2 (&x)[R], const T2* tw) {
  if constexpr (Ns < R) {
    constexpr int Rr = NextRadix(R / Ns);
    constexpr int m = R / Rr;
    T2 y[R];
#pragma unroll
    for (int b = 0; b < m; ++b) {
      const int k = b % Ns;
      T2 v[Rr];
#pragma unroll
      for (int q = 0; q < Rr; ++q) {
        v[q] = x[b + q * m];
        if (q > 0 && k > 0) {
          T2 w = tw[(n / (Ns * Rr)) * q * k];
          if (Sign < 0) w.y = -w.y;
          v[q] = Mul(v[q], w);
        }
      }
      Butterfly<T2, Rr>(v, Sign);
      const int base = (b / Ns) * Ns * Rr + k;
#pragma unroll
      for (int u = 0; u < Rr; ++u) y[base + u * Ns] = v[u];
    }
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = y[i];
    RegStages<T2, R, Ns * Rr, Sign, n>(x, tw);
  }
}

// The whole ring's transform in place: every lane reads its butterfly's
// values into registers before any lane writes.
template <class T2, int R1, int R2, int Sign>
__device__ inline void RingFft2(T2* a, const T2* tw, const T2* twB, int lane) {
  static_assert(R1 <= kWarp && R2 <= kWarp && Smooth(R1) && Smooth(R2), "a butterfly a lane, radices 2-5");
  constexpr int n = R1 * R2;
  {
    T2 v[R1];
    if (lane < R2) {
#pragma unroll
      for (int q = 0; q < R1; ++q) v[q] = a[lane + q * R2];
      RegStages<T2, R1, 1, Sign, n>(v, tw);
    }
    __syncwarp();
    if (lane < R2) {
#pragma unroll
      for (int u = 0; u < R1; ++u) a[lane * R1 + u] = v[u];
    }
    __syncwarp();
  }
  T2 v[R2];
  if (lane < R1) {
#pragma unroll
    for (int q = 0; q < R2; ++q) {
      v[q] = a[lane + q * R1];
      if (q > 0) {
        T2 w = twB[q * R1 + lane];
        if (Sign < 0) w.y = -w.y;
        v[q] = Mul(v[q], w);
      }
    }
    RegStages<T2, R2, 1, Sign, n>(v, tw);
  }
  __syncwarp();
  if (lane < R1) {
#pragma unroll
    for (int u = 0; u < R2; ++u) a[lane + u * R1] = v[u];
  }
  __syncwarp();
}

// A ring's transform by the kernel's form: the two-stage one (R1 > 0; the
// result back in a) or the plan's stages (the result's side returned).
template <class T2, int R1, int R2>
__device__ inline int RingTransform(T2* a, T2* b, const FftPlan& plan, const T2* tw, const T2* twB, int sign,
                                    int lane) {
  if constexpr (R1 > 0) {
    if (sign > 0)
      RingFft2<T2, R1, R2, 1>(a, tw, twB, lane);
    else
      RingFft2<T2, R1, R2, -1>(a, tw, twB, lane);
    return 0;
  } else {
    return WarpFft(a, b, plan, tw, sign, lane);
  }
}

// A hint that the line holding p will be read soon (no register waits on it).
__device__ inline void PrefetchL2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Ring modes: spectra -> fields; fields (times an optional weight) ->
// spectra; spectra -> fields -> weight -> spectra without leaving shared
// memory.
enum RingMode { kRingSynth = 0, kRingAnalyse = 1, kRingWeighted = 2 };

// Rings per CTA (one warp each) so that a CTA's shared memory (the twiddles
// and the rings' buffers: two for the planned stages, one for the two-stage
// form, which works in place) stays near 100 KB.
template <class T2>
int RingsPerCta(int n, int buffers, long long budget = 100 * 1024) {
  const long long ring = static_cast<long long>(buffers) * n * sizeof(T2);
  const long long g = (budget - 2LL * n * sizeof(T2)) / ring;
  return static_cast<int>(std::max(1LL, std::min(8LL, g)));
}

// The twiddles (two tables of n) and `buffers` rings of n per warp, one
// value of padding after each warp's.
template <class T2>
size_t RingSmem(int n, int rings, int buffers) {
  return (2ULL * n + static_cast<unsigned long long>(rings) * (static_cast<unsigned long long>(buffers) * n + 1)) *
         sizeof(T2);
}

// One CTA per (colatitude j, group of G consecutive fields p0..p0+G-1), one
// warp per ring. The spectra [m][j][p] are read and written by the whole CTA
// with the G fields of an order adjacent; the transforms run warp-synchronous.
//
// T2 is the values' type in memory, C2 the transform's arithmetic: the same
// type, or double-float (Df2) for FP64 values under FP64 emulation.
template <class T2, class C2, int R1, int R2>
__global__ void __launch_bounds__(256, (R1 > 0 && sizeof(T2) == 8) ? 3 : 1)
    RingKernel(int mode, int lmax, int ntheta, int count, bool real, FftPlan plan, const T2* twGlobal,
               const double* weights, const T2* spectraIn, const void* fieldsIn,
               const typename Real<T2>::type* pointWeight, void* fieldsOut, T2* spectraOut) {
  static_assert(sizeof(C2) == sizeof(T2), "the shared-memory layout is sized by the storage type");
  using T = typename Real<T2>::type;
  using C = typename Real<C2>::type;
  extern __shared__ __align__(16) unsigned char ringSmem[];
  const int n = R1 > 0 ? R1 * R2 : plan.n;  // a constant in the two-stage form
  constexpr int buffers = R1 > 0 ? 1 : 2;
  // a warp's rings one value apart beyond their buffers, so that the G
  // rings' values of one order fall in different banks
  const long long ringStride = static_cast<long long>(buffers) * n + 1;
  const int G = blockDim.x / kWarp;
  const int warp = threadIdx.x / kWarp, lane = threadIdx.x % kWarp;
  C2* tw = reinterpret_cast<C2*>(ringSmem);
  C2* twB = tw + n;  // the two-stage form's stage-B twiddles
  C2* bufs = twB + n;
  // A real field's ring shares one complex transform with the next field's
  // (z = x + i y; Z_m = X_m + i Y_m, X_m = (Z_m + conj Z_{n-m}) / 2,
  // Y_m = (Z_m - conj Z_{n-m}) / 2i): a warp carries two real fields.
  const int perRing = real ? 2 : 1;
  const int j = blockIdx.y;
  const int p0 = blockIdx.x * G * perRing;
  const int groups = min(G * perRing, count - p0);  // fields of this CTA
  const int rings = (groups + perRing - 1) / perRing;
  const int mcount = real ? lmax + 1 : 2 * lmax + 1;
  if (mode == kRingSynth || mode == kRingWeighted) {
    // ask L2 for this CTA's spectra (one line an order) and, weighted, for
    // the rings' point weights (read after the synthesis): their DRAM
    // latency then overlaps the twiddle loads and the transform
    for (int mi = threadIdx.x; mi < mcount; mi += blockDim.x)
      PrefetchL2(spectraIn + (static_cast<long long>(mi) * ntheta + j) * count + p0);
    if (mode == kRingWeighted) {
      const int f = p0 + perRing * (threadIdx.x / kWarp) + (threadIdx.x % 2);
      const int lines = (n * static_cast<int>(sizeof(T)) + 127) / 128;
      if (f < p0 + groups && f < count)
        for (int k = (threadIdx.x % kWarp) / 2; k < lines; k += kWarp / 2)
          PrefetchL2(pointWeight + (static_cast<long long>(f) * ntheta + j) * n + k * (128 / sizeof(T)));
    }
  }
  for (int e = threadIdx.x; e < n; e += blockDim.x) tw[e] = ToCompute<C2>(twGlobal[e]);
  if constexpr (R1 > 0)
    for (int e = threadIdx.x; e < n; e += blockDim.x) twB[e] = ToCompute<C2>(twGlobal[(e / R1) * (e % R1)]);
  C2* a = bufs + ringStride * warp;  // this warp's ring
  C2* b = buffers == 2 ? a + n : a;
  int at = 0;  // which of a, b holds the ring's current values
  // the rows of this warp's fields (the second of a real pair may not exist)
  const int f0 = p0 + perRing * warp, f1 = real ? f0 + 1 : f0;
  const bool second = real && f1 < p0 + groups;
  const long long row0 = (static_cast<long long>(f0) * ntheta + j) * n;
  const long long row1 = (static_cast<long long>(f1) * ntheta + j) * n;
  if (mode == kRingSynth || mode == kRingWeighted) {
    for (int e = threadIdx.x; e < G * n; e += blockDim.x)
      bufs[ringStride * (e / n) + e % n] = Make<C2>(0, 0);
    __syncthreads();
#pragma unroll 4
    for (int e = threadIdx.x; e < mcount * rings; e += blockDim.x) {
      const int r = e % rings, mi = e / rings;
      const int m = real ? mi : mi - lmax;
      const long long at0 = (static_cast<long long>(mi) * ntheta + j) * count + p0 + perRing * r;
      const C2 v = ToCompute<C2>(spectraIn[at0]);
      C2* ring = bufs + ringStride * r;
      if (real) {
        const C2 u = perRing * r + 1 < groups ? ToCompute<C2>(spectraIn[at0 + 1]) : Make<C2>(0, 0);
        if (m == 0) {
          ring[0] = Make<C2>(v.x, u.x);
        } else {
          ring[m] = Make<C2>(v.x - u.y, v.y + u.x);      // v + i u
          ring[n - m] = Make<C2>(v.x + u.y, u.x - v.y);  // conj(v) + i conj(u)
        }
      } else {
        ring[m < 0 ? m + n : m] = v;
      }
    }
    __syncthreads();
    if (warp < rings) {
      at = RingTransform<C2, R1, R2>(a, b, plan, tw, twB, +1, lane);
      C2* res = at ? b : a;
      if (mode == kRingSynth) {
        for (int k = lane; k < n; k += kWarp) {
          if (real) {
            static_cast<T*>(fieldsOut)[row0 + k] = ToStorage<T>(res[k].x);
            if (second) static_cast<T*>(fieldsOut)[row1 + k] = ToStorage<T>(res[k].y);
          } else {
            static_cast<T2*>(fieldsOut)[row0 + k] = ToStorage2<T2>(res[k]);
          }
        }
      } else {
        // the pointwise weights on the synthesised values
#pragma unroll 5
        for (int k = lane; k < n; k += kWarp) {
          const C w0 = C(pointWeight[row0 + k]);
          const C w1 = real ? (second ? C(pointWeight[row1 + k]) : C(0)) : w0;
          const C2 v = res[k];
          res[k] = Make<C2>(v.x * w0, v.y * w1);
        }
        __syncwarp();
      }
    }
    if (mode == kRingSynth) return;
  } else {
    __syncthreads();  // the twiddles
    if (warp < rings) {
#pragma unroll 5
      for (int k = lane; k < n; k += kWarp) {
        C2 v;
        if (real) {
          v = Make<C2>(C(static_cast<const T*>(fieldsIn)[row0 + k]),
                       second ? C(static_cast<const T*>(fieldsIn)[row1 + k]) : C(0));
        } else {
          v = ToCompute<C2>(static_cast<const T2*>(fieldsIn)[row0 + k]);
        }
        if (pointWeight != nullptr) {
          const C w0 = C(pointWeight[row0 + k]);
          const C w1 = real ? (second ? C(pointWeight[row1 + k]) : C(0)) : w0;
          v = Make<C2>(v.x * w0, v.y * w1);
        }
        a[k] = v;
      }
      __syncwarp();
    }
  }
  // the analysis transform from wherever the ring's values are; every ring
  // has the same stage count, so the result's side is the same for all: a
  // after two transforms, the stage parity's side after one
  if (warp < rings) {
    C2* x = at ? b : a;
    C2* y = at ? a : b;
    RingTransform<C2, R1, R2>(x, y, plan, tw, twB, -1, lane);
  }
  const int out = (mode == kRingWeighted || R1 > 0) ? 0 : plan.stages % 2;
  __syncthreads();
  const C scale = C(static_cast<T>(2.0 * 3.14159265358979323846 / n * weights[j]));
#pragma unroll 4
  for (int e = threadIdx.x; e < mcount * groups; e += blockDim.x) {
    const int g = e % groups, mi = e / groups;
    const int m = real ? mi : mi - lmax;
    const C2* ring = bufs + ringStride * (g / perRing) + (out ? n : 0);
    C2 v;
    if (real) {
      const C2 z = ring[m], w = ring[m == 0 ? 0 : n - m];  // Z_m and Z_{n-m}
      // X_m = (Z_m + conj Z_{n-m}) / 2, Y_m = (Z_m - conj Z_{n-m}) / 2i
      v = g % 2 == 0 ? Make<C2>(C(0.5) * (z.x + w.x), C(0.5) * (z.y - w.y))
                     : Make<C2>(C(0.5) * (z.y + w.y), C(0.5) * (w.x - z.x));
    } else {
      v = ring[m < 0 ? m + n : m];
    }
    spectraOut[(static_cast<long long>(mi) * ntheta + j) * count + p0 + g] =
        ToStorage2<T2>(Make<C2>(v.x * scale, v.y * scale));
  }
}

// The ring kernel for a ring of n longitudes: the two-stage register form
// for the sizes it is built for, else the plan's stages.
template <class T2>
using RingFn = void (*)(int, int, int, int, bool, FftPlan, const T2*, const double*, const T2*, const void*,
                        const typename Real<T2>::type*, void*, T2*);

template <class T2, class C2 = T2>
RingFn<T2> RingKernelFor(int n, int* buffers) {
  *buffers = 1;
  switch (n) {
    case 800: return RingKernel<T2, C2, 25, 32>;
    case 400: return RingKernel<T2, C2, 25, 16>;  // R1 odd: stage A's stores are bank-conflict free
    case 50: return RingKernel<T2, C2, 5, 10>;
    case 40: return RingKernel<T2, C2, 5, 8>;
    case 25: return RingKernel<T2, C2, 5, 5>;
    default: *buffers = 2; return RingKernel<T2, C2, 0, 0>;
  }
}

__global__ void CastKernel(const double* in, long long n, float* out) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = static_cast<float>(in[i]);
}

// -- layout permutations -------------------------------------------------------------------

__global__ void ToDeviceKernel(int lmax, int N, bool real, int count, const int* rowOffset,
                               const double2* ref, double2* dev) {
  const long long rows = real ? static_cast<long long>(lmax + 1) * (lmax + 2) / 2
                              : static_cast<long long>(lmax + 1) * (lmax + 1) - N * N;
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t >= rows * count) return;
  const int p = static_cast<int>(t / rows);
  const long long i = t % rows;
  int l, m;
  if (real) {
    l = static_cast<int>((sqrt(8.0 * i + 1.0) - 1.0) * 0.5);
    while (static_cast<long long>(l) * (l + 1) / 2 > i) --l;
    while (static_cast<long long>(l + 1) * (l + 2) / 2 <= i) ++l;
    m = static_cast<int>(i - static_cast<long long>(l) * (l + 1) / 2);
  } else {
    const long long q = i + N * N;
    l = static_cast<int>(sqrt(static_cast<double>(q)));
    while (static_cast<long long>(l) * l > q) --l;
    while (static_cast<long long>(l + 1) * (l + 1) <= q) ++l;
    m = static_cast<int>(q - static_cast<long long>(l) * l) - l;
  }
  const int l0 = max(abs(m), abs(N));
  const long long row = rowOffset[m + lmax] - (real ? rowOffset[lmax] : 0) + (l - l0);
  dev[row * count + p] = ref[t];
}

__global__ void FromDeviceKernel(int lmax, int N, bool real, int count, const int* rowOffset,
                                 const double2* dev, double2* ref) {
  const long long rows = real ? static_cast<long long>(lmax + 1) * (lmax + 2) / 2
                              : static_cast<long long>(lmax + 1) * (lmax + 1) - N * N;
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t >= rows * count) return;
  const int p = static_cast<int>(t / rows);
  const long long i = t % rows;
  int l, m;
  if (real) {
    l = static_cast<int>((sqrt(8.0 * i + 1.0) - 1.0) * 0.5);
    while (static_cast<long long>(l) * (l + 1) / 2 > i) --l;
    while (static_cast<long long>(l + 1) * (l + 2) / 2 <= i) ++l;
    m = static_cast<int>(i - static_cast<long long>(l) * (l + 1) / 2);
  } else {
    const long long q = i + N * N;
    l = static_cast<int>(sqrt(static_cast<double>(q)));
    while (static_cast<long long>(l) * l > q) --l;
    while (static_cast<long long>(l + 1) * (l + 1) <= q) ++l;
    m = static_cast<int>(q - static_cast<long long>(l) * l) - l;
  }
  const int l0 = max(abs(m), abs(N));
  const long long row = rowOffset[m + lmax] - (real ? rowOffset[lmax] : 0) + (l - l0);
  ref[t] = dev[row * count + p];
}

void GaussLegendre(int n, std::vector<double>& x, std::vector<double>& w) {
  const double pi = 3.14159265358979323846;
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    auto legendre = [n](double zz, double& p1, double& p0) {
      p0 = 1.0;
      p1 = zz;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * zz * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) {
        p1 = zz;
        p0 = 1.0;
      }
    };
    double p1, p0, dp;
    for (int it = 0; it < 100; ++it) {
      legendre(z, p1, p0);
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::abs(dz) < 1e-16) break;
    }
    legendre(z, p1, p0);
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace

int Grid::Create(int lmax, int nmax, double oversampling, std::unique_ptr<Grid>& out) {
  if (lmax < 0 || nmax < 0 || nmax > lmax + 1 || !(oversampling >= 1.0)) {
    SetError("grid: lmax >= 0, 0 <= nmax, oversampling >= 1");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto g = std::make_unique<Grid>();
  g->lmax = lmax;
  g->nmax = nmax;
  g->band = static_cast<int>(std::ceil(oversampling * lmax - 1e-12));
  g->ntheta = g->band + 1;
  g->nphi = FftFriendly(2 * g->band + 1);
  std::vector<double> x;
  GaussLegendre(g->ntheta, x, g->weights);
  g->theta.resize(g->ntheta);
  for (int j = 0; j < g->ntheta; ++j) g->theta[j] = std::acos(x[j]);
  // FFT plan: fours first, then twos, threes and fives.
  int r = g->nphi;
  auto& plan = g->plan;
  plan.n = g->nphi;
  while (r % 4 == 0) {
    plan.radix[plan.stages++] = 4;
    r /= 4;
  }
  for (int p : {2, 3, 5})
    while (r % p == 0) {
      plan.radix[plan.stages++] = p;
      r /= p;
    }
  std::vector<double2> tw(g->nphi);
  for (int k = 0; k < g->nphi; ++k) {
    const double a = 2.0 * 3.14159265358979323846 * k / g->nphi;
    tw[k] = make_double2(std::cos(a), std::sin(a));
  }
  SL3D_CUDA(cudaMalloc(&g->dTheta, g->ntheta * sizeof(double)));
  SL3D_CUDA(cudaMalloc(&g->dWeights, g->ntheta * sizeof(double)));
  SL3D_CUDA(cudaMalloc(&g->dTwiddle, g->nphi * sizeof(double2)));
  SL3D_CUDA(CopyIn(g->dTheta, g->theta.data(), g->ntheta * sizeof(double)));
  SL3D_CUDA(CopyIn(g->dWeights, g->weights.data(), g->ntheta * sizeof(double)));
  SL3D_CUDA(CopyIn(g->dTwiddle, tw.data(), g->nphi * sizeof(double2)));
  out = std::move(g);
  return SL3DGPU_OK;
}

Grid::~Grid() {
  cudaFree(dTcError_);
  for (auto& [key, panel] : panels_) cudaFree(panel);
  for (auto& [key, panel] : panels64_) {
    cudaFree(panel.slices);
    cudaFree(panel.rowExp);
  }
  cudaFree(dTheta);
  cudaFree(dWeights);
  cudaFree(dTwiddle);
  cudaFree(dTwiddle32);
  for (auto& [key, b] : batches_) {
    cudaFree(b.items);
    cudaFree(b.tcItems);
    cudaFree(b.packed);
    cudaFree(b.dTcTiles);
    cudaFree(b.tc64Items);
    cudaFree(b.packed64);
    cudaFree(b.colExp);
  }
  cudaFree(scratchSpectra_);
  cudaFree(scratchCoeffs_);
  for (auto& [N, t] : tables_) {
    cudaFree(t.values);

    cudaFree(t.dRowOffset);
  }
}

int Grid::Table(int N, const SpinTable** out) {
  if (std::abs(N) > nmax) {
    SetError("grid: spin " + std::to_string(N) + " beyond the grid's nmax " + std::to_string(nmax));
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto found = tables_.find(N);
  if (found == tables_.end()) {
    SpinTable t;
    t.N = N;
    t.rowOffset.assign(2 * lmax + 2, 0);
    for (int m = -lmax; m <= lmax; ++m) {
      const int l0 = std::max(std::abs(m), std::abs(N));
      t.rowOffset[m + lmax + 1] = t.rowOffset[m + lmax] + std::max(0, lmax - l0 + 1);
    }
    const size_t size = static_cast<size_t>(t.rowOffset.back()) * ntheta;
    SL3D_CUDA(cudaMalloc(&t.values, std::max<size_t>(size, 1) * sizeof(double)));
    SL3D_CUDA(cudaMalloc(&t.dRowOffset, t.rowOffset.size() * sizeof(int)));
    SL3D_CUDA(CopyIn(t.dRowOffset, t.rowOffset.data(), t.rowOffset.size() * sizeof(int)));
    dim3 grid((ntheta + 127) / 128, 2 * lmax + 1);
    prof::Scope scope(prof::kOther, nullptr);
    WignerTableKernel<<<grid, 128>>>(lmax, N, ntheta, dTheta, t.dRowOffset, t.values);
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaDeviceSynchronize());
    found = tables_.emplace(N, std::move(t)).first;
  }
  *out = &found->second;
  return SL3DGPU_OK;
}

int Grid::BatchFor(int N, bool real, bool analysis, int P, int p0, int count, const Batch** out) {
  const std::array<long long, 6> key{N, real, analysis, P, p0, count};
  auto found = batches_.find(key);
  if (found != batches_.end()) {
    *out = &found->second;
    return SL3DGPU_OK;
  }
  const SpinTable* t = nullptr;
  if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
  std::vector<GemmItem> items;
  const int mlo = real ? 0 : -lmax;
  const long long base = real ? t->rowOffset[lmax] : 0;
  Batch b;
  for (int m = mlo; m <= lmax; ++m) {
    const int rows = t->Rows(m, lmax);
    if (rows == 0) continue;
    const int mi = m - mlo;
    GemmItem it{};
    if (!analysis) {
      it.M = ntheta;
      it.N = 2 * count;
      it.K = rows;
      it.a = static_cast<long long>(t->rowOffset[m + lmax]) * ntheta;
      it.b = (t->rowOffset[m + lmax] - base) * 2LL * P + 2LL * p0;
      it.c = static_cast<long long>(mi) * ntheta * 2LL * count;
      it.sAi = 1;
      it.sAk = ntheta;
      it.ldb = 2 * P;
      it.ldc = 2 * count;
    } else {
      it.M = rows;
      it.N = 2 * count;
      it.K = ntheta;
      it.a = static_cast<long long>(t->rowOffset[m + lmax]) * ntheta;
      it.b = static_cast<long long>(mi) * ntheta * 2LL * count;
      it.c = (t->rowOffset[m + lmax] - base) * 2LL * P + 2LL * p0;
      it.sAi = ntheta;
      it.sAk = 1;
      it.ldb = 2 * count;
      it.ldc = 2 * P;
    }
    b.maxM = std::max(b.maxM, it.M);
    b.maxN = std::max(b.maxN, it.N);
    b.maxK = std::max(b.maxK, it.K);
    b.flops += 2.0 * it.M * it.N * it.K;
    b.outputs += static_cast<double>(it.M) * it.N;
    items.push_back(it);
  }
  b.count = static_cast<int>(items.size());
  b.analysis = analysis;
  if (b.count > 0) {
    SL3D_CUDA(cudaMalloc(&b.items, items.size() * sizeof(GemmItem)));
    SL3D_CUDA(CopyIn(b.items, items.data(), items.size() * sizeof(GemmItem)));
  }
  // The tensor-core form's tiles: 128-row tiles of A in the spin's panel,
  // 16-deep K steps, one column tile when N fits.
  b.tileN = b.maxN <= kTcMaxTileN ? (b.maxN + 15) / 16 * 16 : kTcMaxTileN;
  for (const auto& g : items) {
    TcItemHost h{};
    h.M = g.M;
    h.N = g.N;
    h.K = g.K;
    h.mTiles = (g.M + kTcTileM - 1) / kTcTileM;
    h.kSteps = (g.K + kTcTileK - 1) / kTcTileK;
    h.nTiles = b.tileN > 0 ? (g.N + b.tileN - 1) / b.tileN : 0;
    h.ldc = g.ldc;
    h.ldb = g.ldb;
    h.aPanel = b.panelFloats;
    h.bPack = b.packedFloats;
    h.b = g.b;
    h.c = g.c;
    b.panelFloats += static_cast<long long>(h.mTiles) * h.kSteps * 2 * kTcTileM * kTcTileK;
    b.packedFloats += static_cast<long long>(h.nTiles) * h.kSteps * 2 * b.tileN * kTcTileK;
    b.maxMTiles = std::max(b.maxMTiles, h.mTiles);
    b.maxNTiles = std::max(b.maxNTiles, h.nTiles);
    b.maxATiles = std::max(b.maxATiles, h.mTiles * h.kSteps);
    b.maxBTiles = std::max(b.maxBTiles, h.nTiles * h.kSteps);
    for (int mt = 0; mt < h.mTiles; ++mt)
      for (int nt = 0; nt < h.nTiles; ++nt)
        b.tcTiles.push_back(make_int4(static_cast<int>(b.tcHost.size()), mt, nt, 0));
    b.tcHost.push_back(h);
    // the FP64 emulation's tiles: 128 rows, 64 columns, 16 deep, seven
    // slices a tile
    Tc64Item e{};
    e.M = g.M;
    e.N = g.N;
    e.K = g.K;
    e.mTiles = h.mTiles;
    e.kSteps = h.kSteps;
    e.nTiles = (g.N + kTc64TileN - 1) / kTc64TileN;
    e.ldc = g.ldc;
    e.ldb = g.ldb;
    e.aPanel = b.panel64;
    e.bPack = b.packed64Count;
    e.b = g.b;
    e.c = g.c;
    e.rowExp = b.rowExps;
    e.colExp = b.colExps;
    b.panel64 += static_cast<long long>(e.mTiles) * e.kSteps * kTc64Slices * kTcTileM * kTcTileK;
    b.packed64Count += static_cast<long long>(e.nTiles) * e.kSteps * kTc64Slices * kTc64TileN * kTcTileK;
    b.rowExps += g.M;
    b.colExps += g.N;
    b.maxNTiles64 = std::max(b.maxNTiles64, e.nTiles);
    b.maxBTiles64 = std::max(b.maxBTiles64, e.nTiles * e.kSteps);
    b.tc64Host.push_back(e);
  }
  *out = &batches_.emplace(key, b).first->second;
  return SL3DGPU_OK;
}

int Grid::RunGemm(const Batch& b, const double* A, const double* B, double* C, bool accumulate,
                  cudaStream_t stream) {
  if (b.count == 0) return SL3DGPU_OK;
  prof::Scope scope(b.analysis ? prof::kLegendreAnalysis : prof::kLegendreSynthesis, stream, b.flops);
  // the batch's items all have the direction's layout: analysis sAk = 1,
  // synthesis sAi = 1 (BatchFor)
  if (b.maxN <= kNarrowN) {
    if (b.maxN <= 2)
      LaunchNarrow<2>(b.analysis, b.maxM, b.count, b.items, A, B, C, accumulate, stream);
    else if (b.maxN <= 4)
      LaunchNarrow<4>(b.analysis, b.maxM, b.count, b.items, A, B, C, accumulate, stream);
    else if (b.maxN <= 8)
      LaunchNarrow<8>(b.analysis, b.maxM, b.count, b.items, A, B, C, accumulate, stream);
    else
      LaunchNarrow<16>(b.analysis, b.maxM, b.count, b.items, A, B, C, accumulate, stream);
    SL3D_CHECK_LAUNCH();
    return SL3DGPU_OK;
  }
  dim3 grid((b.maxM + kBM - 1) / kBM, (b.maxN + kBN - 1) / kBN, static_cast<unsigned>(b.count));
  GemmKernel<double><<<grid, 256, 0, stream>>>(b.items, A, B, C, accumulate);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

// The FP64 contraction emulated on the tensor cores: the spin's split
// panel for this direction made on first use, the batch's items, packed-B
// buffer and column exponents on its first use; then B split and packed, and
// the contraction.
int Grid::RunGemm64(int N, bool real, Batch& b, const double* B, double* C, bool accumulate,
                    cudaStream_t stream) {
  if (b.count == 0) return SL3DGPU_OK;
  if (dTcError_ == nullptr) {
    SL3D_CUDA(cudaMalloc(&dTcError_, sizeof(int)));
    SL3D_CUDA(ZeroIn(dTcError_, sizeof(int)));
  }
  if (b.tc64Items == nullptr) {
    SL3D_CUDA(cudaMalloc(&b.tc64Items, b.tc64Host.size() * sizeof(Tc64Item)));
    SL3D_CUDA(CopyIn(b.tc64Items, b.tc64Host.data(), b.tc64Host.size() * sizeof(Tc64Item)));
    SL3D_CUDA(cudaMalloc(&b.packed64, std::max<long long>(b.packed64Count, 1) * sizeof(uint16_t)));
    SL3D_CUDA(cudaMalloc(&b.colExp, std::max<long long>(b.colExps, 1) * sizeof(int)));
  }
  const std::array<int, 3> key{N, real ? 1 : 0, b.analysis ? 1 : 0};
  auto found = panels64_.find(key);
  if (found == panels64_.end()) {
    const SpinTable* t = nullptr;
    if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
    Panel64 panel;
    SL3D_CUDA(cudaMalloc(&panel.slices, std::max<long long>(b.panel64, 1) * sizeof(uint16_t)));
    SL3D_CUDA(cudaMalloc(&panel.rowExp, std::max<long long>(b.rowExps, 1) * sizeof(int)));
    prof::Scope scope(prof::kOther, stream);
    LaunchPanelA64(b.items, b.tc64Items, b.count, b.maxM, b.maxATiles, t->values, panel.rowExp, panel.slices,
                   stream);
    SL3D_CHECK_LAUNCH();
    found = panels64_.emplace(key, panel).first;
  }
  {
    prof::Scope scope(prof::kStream, stream, 0.0, 8.0 * b.colExps + 2.0 * b.packed64Count);
    LaunchPackB64(b.tc64Items, b.count, b.maxNTiles64, B, b.colExp, b.packed64, stream);
    SL3D_CHECK_LAUNCH();
  }
  prof::Scope scope(prof::kLegendre64Tc, stream, b.flops);
  return RunGemm64Tc(b.tc64Items, b.count, b.maxMTiles, b.maxNTiles64, found->second.slices, b.packed64,
                     found->second.rowExp, b.colExp, C, accumulate, dTcError_, stream);
}

int Grid::LegendreSynthesis(int N, bool real, const double* coeffs, int P, int p0, int count,
                            double* spectra, cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  const SpinTable* t = nullptr;
  if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
  const Batch* b = nullptr;
  if (int st = BatchFor(N, real, false, P, p0, count, &b); st != SL3DGPU_OK) return st;
  // orders without degrees (|N| > lmax) leave their spectra zero
  const int mlo = real ? 0 : -lmax;
  for (int m = mlo; m <= lmax; ++m)
    if (t->Rows(m, lmax) == 0)
      SL3D_CUDA(cudaMemsetAsync(spectra + static_cast<long long>(m - mlo) * ntheta * 2LL * count, 0,
                                sizeof(double) * ntheta * 2 * count, stream));
  if (emulateFp64 && b->maxK <= kTc64MaxK)
    return RunGemm64(N, real, *MutableBatch(N, real, false, P, p0, count), coeffs, spectra, false, stream);
  return RunGemm(*b, t->values, coeffs, spectra, false, stream);
}

int Grid::LegendreAnalysis(int N, bool real, const double* spectra, int P, int p0, int count,
                           double* coeffs, bool accumulate, cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  const SpinTable* t = nullptr;
  if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
  const Batch* b = nullptr;
  if (int st = BatchFor(N, real, true, P, p0, count, &b); st != SL3DGPU_OK) return st;
  if (emulateFp64 && b->maxK <= kTc64MaxK)
    return RunGemm64(N, real, *MutableBatch(N, real, true, P, p0, count), spectra, coeffs, accumulate, stream);
  return RunGemm(*b, t->values, spectra, coeffs, accumulate, stream);
}

namespace {
// Under FP64 emulation the FP64 rings' transforms run in double-float on the
// FP32 pipe, unless SL3DGPU_FP64_RINGS=1 keeps them on the FP64 pipe.
bool DoubleFloatRings(const Grid& g) {
  static const bool fp64 = [] {
    const char* v = std::getenv("SL3DGPU_FP64_RINGS");
    return v != nullptr && v[0] == '1';
  }();
  return g.emulateFp64 && !fp64;
}

int LaunchRing(const Grid& g, int mode, bool real, int count, const double* spectraIn,
               const void* fieldsIn, const double* weight, void* fieldsOut, double* spectraOut,
               cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  int buffers = 2;
  // double-float takes the planned stages: the two-stage form's unrolled
  // register transforms would outgrow the instruction cache in it
  const bool df = DoubleFloatRings(g);
  const RingFn<double2> kernel = df ? RingKernel<double2, Df2, 0, 0> : RingKernelFor<double2>(g.nphi, &buffers);
  // the planned stages keep two rings of 16-byte values a warp: at long
  // rings the double-float kernel takes one CTA an SM with up to eight
  // rings rather than two CTAs of two
  const int rings = RingsPerCta<double2>(g.nphi, buffers, df && g.nphi > 400 ? 210 * 1024 : 100 * 1024);
  const size_t smem = RingSmem<double2>(g.nphi, rings, buffers);
  SL3D_CUDA(AllowDynamicSmem(kernel));
  const int fields = real ? 2 * rings : rings;  // real fields go two to a ring
  dim3 grid((count + fields - 1) / fields, g.ntheta);
  // algorithmic traffic: the spectra and the grid values the mode reads and writes
  const double spec = static_cast<double>(real ? g.lmax + 1 : 2 * g.lmax + 1) * g.ntheta * count * 16.0;
  const double field = static_cast<double>(g.ntheta) * g.nphi * count * (real ? 8.0 : 16.0);
  const double wbytes = weight ? static_cast<double>(g.ntheta) * g.nphi * count * 8.0 : 0.0;
  const double bytes = mode == kRingWeighted ? 2 * spec + wbytes : spec + field + wbytes;
  // a real field's transform counts half a complex one (two share a ring)
  const double ffts = static_cast<double>(g.ntheta) * count * (mode == kRingWeighted ? 2 : 1) * (real ? 0.5 : 1.0);
  prof::Scope scope(prof::kRing, stream, ffts * 5.0 * g.nphi * std::log2(static_cast<double>(g.nphi)), bytes);
  kernel<<<grid, rings * kWarp, smem, stream>>>(mode, g.lmax, g.ntheta, count, real, g.plan, g.dTwiddle,
                                          g.dWeights, reinterpret_cast<const double2*>(spectraIn),
                                          fieldsIn, weight, fieldsOut,
                                          reinterpret_cast<double2*>(spectraOut));
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}
}  // namespace

int Grid::RingSynthesis(bool real, const double* spectra, int count, double* fields,
                        cudaStream_t stream) {
  return LaunchRing(*this, kRingSynth, real, count, spectra, nullptr, nullptr, fields, nullptr, stream);
}

int Grid::RingAnalysis(bool real, const double* fields, int count, double* spectra,
                       cudaStream_t stream, const double* weight) {
  return LaunchRing(*this, kRingAnalyse, real, count, nullptr, fields, weight, nullptr, spectra, stream);
}

int Grid::RingWeighted(bool real, const double* spectraIn, int count, const double* weight,
                       double* spectraOut, cudaStream_t stream) {
  return LaunchRing(*this, kRingWeighted, real, count, spectraIn, nullptr, weight, nullptr, spectraOut,
                    stream);
}

// The spin's table (FP64; the tensor-core panels are made from it) and the
// FP32 twiddles of the correction's ring passes, made once.
int Grid::Table32(int N, const SpinTable** out) {
  if (int st = Table(N, out); st != SL3DGPU_OK) return st;
  if (dTwiddle32 == nullptr) {
    SL3D_CUDA(cudaMalloc(&dTwiddle32, nphi * sizeof(float2)));
    CastKernel<<<(2 * nphi + 255) / 256, 256>>>(reinterpret_cast<const double*>(dTwiddle), 2LL * nphi,
                                                reinterpret_cast<float*>(dTwiddle32));
    SL3D_CHECK_LAUNCH();
    SL3D_CUDA(cudaDeviceSynchronize());
  }
  return SL3DGPU_OK;
}

// The FP32 contractions run on the tensor cores (3xTF32, tc_gemm.cu): the
// spin's table panel for this direction made on first use, the batch's items
// and packed-B buffer on its first use, then B packed and the contraction.
int Grid::RunGemmF(int N, bool real, Batch& b, const float* B, float* C, bool accumulate, cudaStream_t stream) {
  if (b.count == 0) return SL3DGPU_OK;
  static_assert(sizeof(TcItemHost) == sizeof(TcItem), "host and device tensor-core items agree");
  if (dTcError_ == nullptr) {
    SL3D_CUDA(cudaMalloc(&dTcError_, sizeof(int)));
    SL3D_CUDA(ZeroIn(dTcError_, sizeof(int)));
  }
  if (b.tcItems == nullptr) {
    SL3D_CUDA(cudaMalloc(&b.tcItems, b.tcHost.size() * sizeof(TcItem)));
    SL3D_CUDA(CopyIn(b.tcItems, b.tcHost.data(), b.tcHost.size() * sizeof(TcItem)));
    SL3D_CUDA(cudaMalloc(&b.packed, std::max<long long>(b.packedFloats, 1) * sizeof(float)));
    SL3D_CUDA(cudaMalloc(&b.dTcTiles, std::max<size_t>(b.tcTiles.size(), 1) * sizeof(int4)));
    if (!b.tcTiles.empty())
      SL3D_CUDA(CopyIn(b.dTcTiles, b.tcTiles.data(), b.tcTiles.size() * sizeof(int4)));
  }
  const auto* items = static_cast<const TcItem*>(b.tcItems);
  const std::array<int, 3> key{N, real ? 1 : 0, b.analysis ? 1 : 0};
  auto found = panels_.find(key);
  if (found == panels_.end()) {
    const SpinTable* t = nullptr;
    if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
    float* panel = nullptr;
    SL3D_CUDA(cudaMalloc(&panel, std::max<long long>(b.panelFloats, 1) * sizeof(float)));
    prof::Scope scope(prof::kOther, stream);
    LaunchPanelA(b.items, items, b.count, b.maxATiles, t->values, panel, stream);
    SL3D_CHECK_LAUNCH();
    found = panels_.emplace(key, panel).first;
  }
  // B split and packed inside the contraction (B and C never overlap here:
  // the packing warps read B while other CTAs' epilogues write C); with
  // SL3DGPU_PACKB=1 by the separate pass, through HBM
  static const bool separatePack = [] {
    const char* v = std::getenv("SL3DGPU_PACKB");
    return v != nullptr && v[0] == '1';
  }();
  if (separatePack) {
    prof::Scope scope(prof::kStream, stream, 0.0, 12.0 * b.packedFloats / 2);
    LaunchPackB(items, b.count, b.maxBTiles, b.tileN, B, b.packed, stream);
    SL3D_CHECK_LAUNCH();
  }
  // algorithmic traffic: the table panel once, B once per row tile (4 bytes
  // a value read in the contraction; 8 from the packed tiles), C once
  prof::Scope scope(prof::kLegendre32, stream, b.flops,
                    4.0 * b.panelFloats + (separatePack ? 4.0 : 2.0) * b.packedFloats * b.maxMTiles +
                        4.0 * b.outputs);
  return RunGemmTc(items, b.dTcTiles, static_cast<int>(b.tcTiles.size()), b.tileN, found->second, b.packed,
                   separatePack ? nullptr : B, C, accumulate, dTcError_, stream);
}

Grid::Batch* Grid::MutableBatch(int N, bool real, bool analysis, int P, int p0, int count) {
  const Batch* b = nullptr;
  if (BatchFor(N, real, analysis, P, p0, count, &b) != SL3DGPU_OK) return nullptr;
  return const_cast<Batch*>(b);
}

int Grid::TensorCoreStatus(cudaStream_t stream) {
  if (dTcError_ == nullptr) return SL3DGPU_OK;
  int flag = 0;
  SL3D_CUDA(cudaMemcpyAsync(&flag, dTcError_, sizeof(int), cudaMemcpyDeviceToHost, stream));
  SL3D_CUDA(cudaStreamSynchronize(stream));
  if (flag != 0) {
    SL3D_CUDA(cudaMemsetAsync(dTcError_, 0, sizeof(int), stream));
    SetError("a tensor-core contraction gave up waiting for its completion");
    return SL3DGPU_ERR_WAIT;
  }
  return SL3DGPU_OK;
}

int Grid::LegendreSynthesisF(int N, bool real, const float* coeffs, int P, int p0, int count, float* spectra,
                             cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  const SpinTable* t = nullptr;
  if (int st = Table32(N, &t); st != SL3DGPU_OK) return st;
  Batch* b = MutableBatch(N, real, false, P, p0, count);
  if (b == nullptr) return SL3DGPU_ERR_CUDA;
  const int mlo = real ? 0 : -lmax;
  for (int m = mlo; m <= lmax; ++m)
    if (t->Rows(m, lmax) == 0)
      SL3D_CUDA(cudaMemsetAsync(spectra + static_cast<long long>(m - mlo) * ntheta * 2LL * count, 0,
                                sizeof(float) * ntheta * 2 * count, stream));
  return RunGemmF(N, real, *b, coeffs, spectra, false, stream);
}

int Grid::LegendreAnalysisF(int N, bool real, const float* spectra, int P, int p0, int count, float* coeffs,
                            bool accumulate, cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  const SpinTable* t = nullptr;
  if (int st = Table32(N, &t); st != SL3DGPU_OK) return st;
  Batch* b = MutableBatch(N, real, true, P, p0, count);
  if (b == nullptr) return SL3DGPU_ERR_CUDA;
  return RunGemmF(N, real, *b, spectra, coeffs, accumulate, stream);
}

int Grid::RingWeightedF(bool real, const float* spectraIn, int count, const float* weight, float* spectraOut,
                        cudaStream_t stream) {
  if (count == 0) return SL3DGPU_OK;
  const SpinTable* t = nullptr;
  if (int st = Table32(0, &t); st != SL3DGPU_OK) return st;  // makes the FP32 twiddles
  int buffers = 2;
  const RingFn<float2> kernel = RingKernelFor<float2>(nphi, &buffers);
  const int rings = RingsPerCta<float2>(nphi, buffers);
  const size_t smem = RingSmem<float2>(nphi, rings, buffers);
  SL3D_CUDA(AllowDynamicSmem(kernel));
  const int fields = real ? 2 * rings : rings;  // real fields go two to a ring
  dim3 grid((count + fields - 1) / fields, ntheta);
  const double spec = static_cast<double>(real ? lmax + 1 : 2 * lmax + 1) * ntheta * count * 8.0;
  const double wbytes = static_cast<double>(ntheta) * nphi * count * 4.0;
  prof::Scope scope(prof::kRing32, stream,
                    (real ? 1.0 : 2.0) * ntheta * count * 5.0 * nphi * std::log2(static_cast<double>(nphi)),
                    2 * spec + wbytes);
  kernel<<<grid, rings * kWarp, smem, stream>>>(kRingWeighted, lmax, ntheta, count, real, plan, dTwiddle32,
                                                  dWeights, reinterpret_cast<const float2*>(spectraIn), nullptr,
                                                  weight, nullptr, reinterpret_cast<float2*>(spectraOut));
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Grid::ToDevice(int N, bool real, const double* ref, int count, double* dev,
                   cudaStream_t stream) {
  const SpinTable* t = nullptr;
  if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
  const long long total = (real ? RealRows() : SpinRows(N)) * count;
  if (total == 0) return SL3DGPU_OK;
  prof::Scope scope(prof::kOther, stream);
  ToDeviceKernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, stream>>>(
      lmax, N, real, count, t->dRowOffset, reinterpret_cast<const double2*>(ref),
      reinterpret_cast<double2*>(dev));
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Grid::FromDevice(int N, bool real, const double* dev, int count, double* ref,
                     cudaStream_t stream) {
  const SpinTable* t = nullptr;
  if (int st = Table(N, &t); st != SL3DGPU_OK) return st;
  const long long total = (real ? RealRows() : SpinRows(N)) * count;
  if (total == 0) return SL3DGPU_OK;
  prof::Scope scope(prof::kOther, stream);
  FromDeviceKernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, stream>>>(
      lmax, N, real, count, t->dRowOffset, reinterpret_cast<const double2*>(dev),
      reinterpret_cast<double2*>(ref));
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

int Grid::Scratch(size_t spectraDoubles, size_t coeffDoubles, double** spectra, double** coeffs) {
  if (spectraDoubles > scratchSpectraSize_) {
    cudaFree(scratchSpectra_);
    scratchSpectra_ = nullptr;
    scratchSpectraSize_ = 0;
    SL3D_CUDA(cudaMalloc(&scratchSpectra_, spectraDoubles * sizeof(double)));
    scratchSpectraSize_ = spectraDoubles;
  }
  if (coeffDoubles > scratchCoeffsSize_) {
    cudaFree(scratchCoeffs_);
    scratchCoeffs_ = nullptr;
    scratchCoeffsSize_ = 0;
    SL3D_CUDA(cudaMalloc(&scratchCoeffs_, coeffDoubles * sizeof(double)));
    scratchCoeffsSize_ = coeffDoubles;
  }
  *spectra = scratchSpectra_;
  *coeffs = scratchCoeffs_;
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu

// -- the C ABI: SurfaceGrid's batched calls on device buffers in the reference layouts -----

using namespace sl3dgpu;

struct sl3dgpu_grid {
  std::unique_ptr<Grid> grid;
};

extern "C" int sl3dgpu_grid_create(int lmax, int nmax, double oversampling, sl3dgpu_grid** out) {
  if (out == nullptr) {
    SetError("null output handle");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto handle = std::make_unique<sl3dgpu_grid>();
  if (int st = Grid::Create(lmax, nmax, oversampling, handle->grid); st != SL3DGPU_OK) return st;
  *out = handle.release();
  return SL3DGPU_OK;
}

extern "C" void sl3dgpu_grid_destroy(sl3dgpu_grid* grid) { delete grid; }

extern "C" int sl3dgpu_grid_lmax(const sl3dgpu_grid* grid) {
  if (grid == nullptr) {
    SetError("null grid");
    return -1;
  }
  return grid->grid->lmax;
}

extern "C" int sl3dgpu_grid_shape(const sl3dgpu_grid* grid, int* ntheta, int* nphi) {
  if (grid == nullptr) {
    SetError("null grid");
    return SL3DGPU_ERR_ARGUMENT;
  }
  if (ntheta) *ntheta = grid->grid->ntheta;
  if (nphi) *nphi = grid->grid->nphi;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_grid_set_fp64_emulation(sl3dgpu_grid* grid, int on) {
  if (grid == nullptr || (on != 0 && on != 1)) {
    SetError("grid: null handle, or fp64 emulation not 0 or 1");
    return SL3DGPU_ERR_ARGUMENT;
  }
  grid->grid->emulateFp64 = on != 0;
  return SL3DGPU_OK;
}

extern "C" int sl3dgpu_grid_colatitudes(const sl3dgpu_grid* grid, double* theta, double* weights) {
  if (grid == nullptr) {
    SetError("null grid");
    return SL3DGPU_ERR_ARGUMENT;
  }
  const auto& g = *grid->grid;
  if (theta) std::memcpy(theta, g.theta.data(), g.theta.size() * sizeof(double));
  if (weights) std::memcpy(weights, g.weights.data(), g.weights.size() * sizeof(double));
  return SL3DGPU_OK;
}

namespace {

int Synthesise(sl3dgpu_grid* handle, int N, bool real, const double* coeffs, int count,
               double* fields, void* stream) {
  if (handle == nullptr || count < 0) {
    SetError("null grid or negative count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto& g = *handle->grid;
  const cudaStream_t s = AsStream(stream);
  const size_t mcount = real ? g.lmax + 1 : 2 * g.lmax + 1;
  const size_t rows = real ? g.RealRows() : g.SpinRows(N);
  double *spectra = nullptr, *dev = nullptr;
  if (int st = g.Scratch(mcount * g.ntheta * 2 * std::max(count, 1), rows * 2 * std::max(count, 1),
                         &spectra, &dev);
      st != SL3DGPU_OK)
    return st;
  if (int st = g.ToDevice(N, real, coeffs, count, dev, s); st != SL3DGPU_OK) return st;
  if (int st = g.LegendreSynthesis(N, real, dev, count, spectra, s); st != SL3DGPU_OK) return st;
  return g.RingSynthesis(real, spectra, count, fields, s);
}

int Expand(sl3dgpu_grid* handle, int N, bool real, const double* fields, int count, double* coeffs,
           void* stream) {
  if (handle == nullptr || count < 0) {
    SetError("null grid or negative count");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto& g = *handle->grid;
  const cudaStream_t s = AsStream(stream);
  const size_t mcount = real ? g.lmax + 1 : 2 * g.lmax + 1;
  const size_t rows = real ? g.RealRows() : g.SpinRows(N);
  double *spectra = nullptr, *dev = nullptr;
  if (int st = g.Scratch(mcount * g.ntheta * 2 * std::max(count, 1), rows * 2 * std::max(count, 1),
                         &spectra, &dev);
      st != SL3DGPU_OK)
    return st;
  if (int st = g.RingAnalysis(real, fields, count, spectra, s); st != SL3DGPU_OK) return st;
  if (int st = g.LegendreAnalysis(N, real, spectra, count, dev, s); st != SL3DGPU_OK) return st;
  return g.FromDevice(N, real, dev, count, coeffs, s);
}

}  // namespace

extern "C" int sl3dgpu_synthesise_spin_batch(sl3dgpu_grid* grid, int N, const double* coeffs,
                                             int count, double* fields, void* stream) {
  return Synthesise(grid, N, false, coeffs, count, fields, stream);
}

extern "C" int sl3dgpu_expand_spin_batch(sl3dgpu_grid* grid, int N, const double* fields,
                                         int count, double* coeffs, void* stream) {
  return Expand(grid, N, false, fields, count, coeffs, stream);
}

extern "C" int sl3dgpu_legendre_device(sl3dgpu_grid* grid, int N, int real, int analysis, int fp32, const void* in,
                                       int count, void* out, void* stream) {
  if (grid == nullptr || count < 0 || (real && N != 0)) {
    SetError("legendre: null grid, negative count, or a real field of nonzero spin");
    return SL3DGPU_ERR_ARGUMENT;
  }
  auto& g = *grid->grid;
  const cudaStream_t s = AsStream(stream);
  if (fp32) {
    return analysis ? g.LegendreAnalysisF(N, real != 0, static_cast<const float*>(in), count, 0, count,
                                          static_cast<float*>(out), false, s)
                    : g.LegendreSynthesisF(N, real != 0, static_cast<const float*>(in), count, 0, count,
                                           static_cast<float*>(out), s);
  }
  return analysis ? g.LegendreAnalysis(N, real != 0, static_cast<const double*>(in), count,
                                       static_cast<double*>(out), s)
                  : g.LegendreSynthesis(N, real != 0, static_cast<const double*>(in), count,
                                        static_cast<double*>(out), s);
}

extern "C" int sl3dgpu_synthesise_batch(sl3dgpu_grid* grid, const double* coeffs, int count,
                                        double* fields, void* stream) {
  return Synthesise(grid, 0, true, coeffs, count, fields, stream);
}

extern "C" int sl3dgpu_expand_batch(sl3dgpu_grid* grid, const double* fields, int count,
                                    double* coeffs, void* stream) {
  return Expand(grid, 0, true, fields, count, coeffs, stream);
}
