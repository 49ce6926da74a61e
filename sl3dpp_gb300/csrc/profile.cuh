// Launch accounting and optional per-kernel-kind event timing: every kernel
// launch of the library counts; with timing on, each launch of a kind is
// bracketed by CUDA events on its own stream and its algorithmic work
// (flops, bytes) recorded, for the live roofline of the benchmark.
#pragma once

#include <cuda_runtime.h>

namespace sl3dgpu::prof {

enum Kind {
  kLegendreSynthesis = 0,
  kLegendreAnalysis = 1,
  kRing = 2,
  kForce = 3,
  kStrain = 4,
  kBandSolve = 5,
  kStream = 6,
  kMixer = 7,
  kOther = 8,
  kLegendre32 = 9,   // the mixed form's FP32 contractions (synthesis and analysis)
  kRing32 = 10,      // its FP32 ring passes
  kBandSolve32 = 11, // its FP32 band solves
  kLegendre64Tc = 12, // FP64 contractions emulated on the tensor cores (both directions)
  kKinds = 13
};

// Counts one launch; with timing on, records its start event.
void Begin(int kind, cudaStream_t stream);
// Records the end event of the launch begun last on this kind, with its work.
void End(int kind, cudaStream_t stream, double flops, double bytes);
// Whether per-kind event timing is on (a CUDA graph cannot hold its events).
bool TimingOn();
// The launch count, and launches made by a replayed graph (or a capture's,
// taken back: captured kernels do not run then).
long long Launches();
void AddLaunches(long long n);

struct Scope {
  int kind;
  cudaStream_t stream;
  double flops, bytes;
  Scope(int k, cudaStream_t s, double f = 0.0, double b = 0.0) : kind(k), stream(s), flops(f), bytes(b) {
    Begin(kind, stream);
  }
  ~Scope() { End(kind, stream, flops, bytes); }
};

}  // namespace sl3dgpu::prof
