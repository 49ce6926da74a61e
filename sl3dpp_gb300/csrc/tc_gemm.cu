// The FP32 Legendre contraction on the tcgen05 tensor cores (see tc_gemm.cuh).
//
// A persistent, warp-specialised kernel (TcGemmKernel, below): a TMA
// producer lane fills a ring of shared-memory stages (the A tile's high and
// low TF32 parts, 16 KB; B's, 2 x tileN x 64 B, split and packed there by two
// warps from B's source), an MMA lane issues each
// 16-deep step's tcgen05.mma kind::tf32 into one of two TMEM accumulators,
// and four epilogue warps drain the other. B's high and low parts form one
// operand of 2 tileN rows, so that for tileN <= 128 the products A_hi B_hi
// and A_hi B_lo are one MMA of N = 2 tileN into the accumulator's two column
// halves, and A_lo B_hi a second MMA into the first half: two MMAs per 8-deep
// slice instead of three (an M = 128 MMA costs about the same below N = 128
// as at N = 128, so the wide one is nearly free). The epilogue sums the
// halves. Every wait has an iteration limit.
#include <cstdint>

#include "profile.cuh"
#include "tc_gemm.cuh"

namespace sl3dgpu {
namespace {

constexpr int kATileFloats = kTcTileM * kTcTileK;  // one part: 2048 floats, 8 KB

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B,
// both K-major, N and M.
__host__ __device__ constexpr uint32_t InstrDescriptor(int n, int m) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ inline float RoundTf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Index (in floats) of element (row, k) of a K-major 16-deep tile of `rows`
// rows in the core-matrix layout [k / 4][row / 8][row % 8][k % 4].
__device__ inline int TileIndex(int row, int k, int rows) {
  return (k >> 2) * (rows * 4) + (row >> 3) * 32 + (row & 7) * 4 + (k & 3);
}

// Tensor-memory columns for an accumulator of n columns: a power of two, at
// least 32.
__host__ __device__ constexpr uint32_t TmemColumns(int n) {
  uint32_t c = 32;
  while (c < static_cast<uint32_t>(n)) c *= 2;
  return c;
}

__global__ void PanelAKernel(const GemmItem* items, const TcItem* tcItems, const double* table, float* panels) {
  const GemmItem g = items[blockIdx.y];
  const TcItem it = tcItems[blockIdx.y];
  const long long total = static_cast<long long>(it.mTiles) * it.kSteps * kATileFloats;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int e = static_cast<int>(t % kATileFloats);
    const long long tile = t / kATileFloats;
    const int ks = static_cast<int>(tile % it.kSteps), mt = static_cast<int>(tile / it.kSteps);
    const int r = e % kTcTileM, kk = e / kTcTileM;
    const int i = mt * kTcTileM + r, k = ks * kTcTileK + kk;
    const double v = (i < g.M && k < g.K) ? table[g.a + static_cast<long long>(i) * g.sAi +
                                                  static_cast<long long>(k) * g.sAk]
                                          : 0.0;
    const float hi = RoundTf32(static_cast<float>(v));
    float* out = panels + it.aPanel + tile * 2 * kATileFloats;
    out[TileIndex(r, kk, kTcTileM)] = hi;
    out[kATileFloats + TileIndex(r, kk, kTcTileM)] = static_cast<float>(v - static_cast<double>(hi));
  }
}

// A thread per (tile, 4-deep K group, column): four coalesced reads down
// B's column, one 16-byte store of each part (a core-matrix row).
__global__ void PackBKernel(const TcItem* tcItems, int tileN, const float* B, float* packed) {
  const TcItem it = tcItems[blockIdx.y];
  const int tileFloats = tileN * kTcTileK;
  const int groups = kTcTileK / 4;
  const long long total = static_cast<long long>(it.nTiles) * it.kSteps * groups * tileN;
  for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int nn = static_cast<int>(t % tileN);
    const long long rest = t / tileN;
    const int g = static_cast<int>(rest % groups);
    const long long tile = rest / groups;
    const int ks = static_cast<int>(tile % it.kSteps), nt = static_cast<int>(tile / it.kSteps);
    const int n = nt * tileN + nn, k0 = ks * kTcTileK + 4 * g;
    float v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      v[q] = (n < it.N && k0 + q < it.K) ? B[it.b + static_cast<long long>(k0 + q) * it.ldb + n] : 0.0f;
    float4 hi, lo;
    hi.x = RoundTf32(v[0]);
    hi.y = RoundTf32(v[1]);
    hi.z = RoundTf32(v[2]);
    hi.w = RoundTf32(v[3]);
    lo.x = v[0] - hi.x;
    lo.y = v[1] - hi.y;
    lo.z = v[2] - hi.z;
    lo.w = v[3] - hi.w;
    // one operand of 2 tileN rows: the high parts in rows 0 .. tileN - 1,
    // the low parts below them
    float* out = packed + it.bPack + tile * 2 * tileFloats;
    *reinterpret_cast<float4*>(out + TileIndex(nn, 4 * g, 2 * tileN)) = hi;
    *reinterpret_cast<float4*>(out + TileIndex(tileN + nn, 4 * g, 2 * tileN)) = lo;
  }
}

// The persistent, warp-specialised contraction: one CTA per SM walks the
// batch's tile list (tile t, t + gridDim.x, ...). Warp 0 (one lane) is the TMA
// producer, filling a ring of `stages` shared-memory stages (the A tile's
// two parts and B's) ahead of use; warp 1 (one lane) issues each step's six
// MMAs into one of two TMEM accumulators and commits them to the stage's
// "empty" barrier, and a tile's last step also to its accumulator's "full"
// barrier; warps 2-5 drain a full accumulator (each its TMEM lane quarter,
// warp % 4) to C and release it. The epilogue of one tile thus overlaps the
// main loop of the next, and the copies never wait for an epilogue. Stage g
// of the CTA's step sequence uses ring slot g % stages in use round
// g / stages; tile i uses accumulator i % 2 in round i / 2. Every wait is
// bounded: one that gives up sets the error flag and a shared abort flag that
// ends the other roles' loops; before TMEM is freed the MMA lane waits for its
// issued MMAs and the producer for its issued copies (bounded too).
//
// With rawB, B is not packed beforehand: the packing warps (6 .. 9, a step
// each in turn) read the step's 16 x tileN slice of B straight from its
// source (four coalesced reads down a column a lane, per 4-deep group),
// split it into its TF32 high and low parts and store them in the stage's B
// tile in the core-matrix layout, then fence the stores for the tensor
// cores' (async) proxy and arrive on the stage's "full" barrier beside the
// producer's A copy -- the packing pass and its round trip through HBM are
// gone, and B is read at 4 bytes a value.
constexpr int kPackWarps = 4;  // warps 6 .. 9, a step each in turn
constexpr int kPersistentThreads = 32 * (6 + kPackWarps);
constexpr int kPackChunk = 16;  // (column, group) items a lane loads before it stores (64 reads in flight)

__global__ void __launch_bounds__(kPersistentThreads, 1)
    TcGemmKernel(const TcItem* tcItems, const int4* tiles, int tileCount, int tileN, int stages,
                 const float* panels, const float* packed, const float* rawB, float* C, bool accumulate,
                 int* errorFlag) {
  const int bTileFloats = tileN * kTcTileK;
  // tileN <= 128: A_hi B_hi and A_hi B_lo in one MMA of N = 2 tileN, into
  // the accumulator's two column halves (summed by the epilogue)
  const bool fused = 2 * tileN <= 256;
  const uint32_t accColumns = TmemColumns(fused ? 2 * tileN : tileN);
  const uint32_t aBytes = 2 * kATileFloats * sizeof(float), bBytes = 2 * bTileFloats * sizeof(float);

  extern __shared__ __align__(128) unsigned char tcSmem[];
  float* sA = reinterpret_cast<float*>(tcSmem);  // stages x (hi | lo)
  float* sB = sA + stages * 2 * kATileFloats;    // stages x (hi | lo)
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + stages * 2 * bTileFloats);
  uint64_t* empty = full + stages;
  uint64_t* accFull = empty + stages;  // 2
  uint64_t* accEmpty = accFull + 2;    // 2
  uint64_t* drain = accEmpty + 2;
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ volatile int abortFlag;
  __shared__ float rowsOut[4][32][33];  // each epilogue warp's 32 x 32 block, padded
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(tmemSlot)),
                 "r"(2 * accColumns)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  const uint32_t fullCount = rawB != nullptr ? 1 + 32 : 1;  // the producer, and the packing warp of the step
  if (tid == 0) {
    abortFlag = 0;
    for (int s = 0; s < stages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(full + s)), "r"(fullCount) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(empty + s)), "r"(1) : "memory");
    }
    for (int a = 0; a < 2; ++a) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(accFull + a)), "r"(1) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(accEmpty + a)), "r"(128) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(drain)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmemSlot;
  auto giveUp = [&] {
    abortFlag = 1;
    atomicExch(errorFlag, 1);
  };

  if (warp == 0 && lane == 0) {
    // -- producer --------------------------------------------------------------
    long long g = 0;
    for (int t = blockIdx.x; t < tileCount && !abortFlag; t += gridDim.x) {
      const int4 tile = tiles[t];
      const TcItem it = tcItems[tile.x];
      const float* aSrc = panels + it.aPanel + static_cast<long long>(tile.y) * it.kSteps * 2 * kATileFloats;
      const float* bSrc = packed + it.bPack + static_cast<long long>(tile.z) * it.kSteps * 2 * bTileFloats;
      for (int ks = 0; ks < it.kSteps; ++ks, ++g) {
        const int slot = static_cast<int>(g % stages);
        const long long round = g / stages;
        if (round > 0 && !WaitParity(SmemAddr(empty + slot), static_cast<uint32_t>((round - 1) & 1))) {
          giveUp();
          break;
        }
        if (abortFlag) break;
        const uint32_t bar = SmemAddr(full + slot);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                     "r"(rawB != nullptr ? aBytes : aBytes + bBytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                SmemAddr(sA + slot * 2 * kATileFloats)),
            "l"(aSrc + static_cast<long long>(ks) * 2 * kATileFloats), "r"(aBytes), "r"(bar)
            : "memory");
        if (rawB == nullptr)
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                  SmemAddr(sB + slot * 2 * bTileFloats)),
              "l"(bSrc + static_cast<long long>(ks) * 2 * bTileFloats), "r"(bBytes), "r"(bar)
              : "memory");
      }
    }
    // the copies issued last land before the CTA can end (the MMA lane has
    // waited for all it consumed; on an abort some may be unconsumed)
    for (long long q = g > stages ? g - stages : 0; q < g; ++q)
      WaitParity(SmemAddr(full + static_cast<int>(q % stages)), static_cast<uint32_t>((q / stages) & 1));
  } else if (warp == 1 && lane == 0) {
    // -- MMA issue ---------------------------------------------------------------
    long long g = 0;
    int local = 0;
    bool issued = false;
    for (int t = blockIdx.x; t < tileCount && !abortFlag; t += gridDim.x, ++local) {
      const int4 tile = tiles[t];
      const TcItem it = tcItems[tile.x];
      const int nCols = min(tileN, it.N - tile.z * tileN);
      const uint32_t idesc = InstrDescriptor((nCols + 15) / 16 * 16, kTcTileM);
      const uint32_t idescPair = InstrDescriptor(2 * tileN, kTcTileM);
      const int acc = local & 1;
      const int use = local >> 1;
      if (use > 0 && !WaitParity(SmemAddr(accEmpty + acc), static_cast<uint32_t>((use - 1) & 1))) {
        giveUp();
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + acc * accColumns;
      bool ok = true;
      for (int ks = 0; ks < it.kSteps; ++ks, ++g) {
        const int slot = static_cast<int>(g % stages);
        if (!WaitParity(SmemAddr(full + slot), static_cast<uint32_t>((g / stages) & 1)) || abortFlag) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t aHi = SmemAddr(sA + slot * 2 * kATileFloats), aLo = aHi + kATileFloats * 4;
        const uint32_t bHi = SmemAddr(sB + slot * 2 * bTileFloats), bLo = bHi + tileN * 16;
        const uint32_t aLbo = kTcTileM * 16, bLbo = 2 * tileN * 16, sbo = 128;
#pragma unroll
        for (int q = 0; q < kTcTileK / 8; ++q) {
          const uint32_t aOff = q * 2 * aLbo, bOff = q * 2 * bLbo;
          const uint64_t dAh = Descriptor(aHi + aOff, aLbo, sbo), dAl = Descriptor(aLo + aOff, aLbo, sbo);
          const uint64_t dBh = Descriptor(bHi + bOff, bLbo, sbo), dBl = Descriptor(bLo + bOff, bLbo, sbo);
          const uint32_t enable = (ks > 0 || q > 0) ? 1u : 0u;
          if (fused) {
            // A_hi [B_hi; B_lo] into both halves, then A_lo B_hi into the first
            asm volatile(
                "{\n\t.reg .pred r;\n\t"
                "setp.ne.b32 r, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, r;\n\t}" ::"r"(d),
                "l"(dAh), "l"(dBh), "r"(idescPair), "r"(enable)
                : "memory");
            asm volatile(
                "{\n\t.reg .pred r;\n\t"
                "setp.ne.b32 r, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, r;\n\t}" ::"r"(d),
                "l"(dAl), "l"(dBh), "r"(idesc), "r"(1u)
                : "memory");
          } else {
            const uint64_t as[3] = {dAh, dAh, dAl};
            const uint64_t bs[3] = {dBh, dBl, dBh};
#pragma unroll
            for (int p = 0; p < 3; ++p) {
              const uint32_t on = (enable || p > 0) ? 1u : 0u;
              asm volatile(
                  "{\n\t.reg .pred r;\n\t"
                  "setp.ne.b32 r, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, r;\n\t}" ::"r"(d),
                  "l"(as[p]), "l"(bs[p]), "r"(idesc), "r"(on)
                  : "memory");
            }
          }
        }
        issued = true;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         SmemAddr(empty + slot))
                     : "memory");
      }
      if (!ok) {
        giveUp();
        break;
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       SmemAddr(accFull + acc))
                   : "memory");
    }
    // every MMA issued has completed before TMEM is freed
    if (issued) {
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       SmemAddr(drain))
                   : "memory");
      if (!WaitParity(SmemAddr(drain), 0)) atomicExch(errorFlag, 1);
    }
  } else if (warp >= 6) {
    // -- B's split and pack, in shared memory: packing warp p takes the
    // steps g = p, p + kPackWarps, ..., so that kPackWarps steps' reads are in
    // flight; a lane loads all its items' values before it converts and
    // stores any (its loads overlap)
    if (rawB != nullptr) {
      const int packer = warp - 6;
      const int groups = kTcTileK / 4;
      long long g = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < tileCount && !abortFlag && ok; t += gridDim.x) {
        const int4 tile = tiles[t];
        const TcItem it = tcItems[tile.x];
        const int nBase = tile.z * tileN;
        const int items = tileN * groups;
        for (int ks = 0; ks < it.kSteps; ++ks, ++g) {
          if (static_cast<int>(g % kPackWarps) != packer) continue;
          const int slot = static_cast<int>(g % stages);
          const long long round = g / stages;
          float* out = sB + slot * 2 * bTileFloats;
          // B's values are read before the slot is waited for (they go to
          // registers): their global latency overlaps the wait
          bool waited = false;
          for (int first = 0; first < items; first += 32 * kPackChunk) {
            float v[kPackChunk][4];
#pragma unroll
            for (int j = 0; j < kPackChunk; ++j) {
              const int item = first + lane + 32 * j;
              const int nn = item % tileN, grp = item / tileN;
              const int n = nBase + nn, k0 = ks * kTcTileK + 4 * grp;
              const bool in = item < items && n < it.N;
#pragma unroll
              for (int q = 0; q < 4; ++q)
                v[j][q] = (in && k0 + q < it.K) ? __ldg(rawB + it.b + static_cast<long long>(k0 + q) * it.ldb + n)
                                                : 0.0f;
            }
            if (!waited) {
              waited = true;
              if (round > 0 && !WaitParity(SmemAddr(empty + slot), static_cast<uint32_t>((round - 1) & 1))) {
                ok = false;
                break;
              }
              if (abortFlag) break;
            }
#pragma unroll
            for (int j = 0; j < kPackChunk; ++j) {
              const int item = first + lane + 32 * j;
              if (item >= items) break;
              const int nn = item % tileN, grp = item / tileN;
              float4 hi, lo;
              hi.x = RoundTf32(v[j][0]);
              hi.y = RoundTf32(v[j][1]);
              hi.z = RoundTf32(v[j][2]);
              hi.w = RoundTf32(v[j][3]);
              lo.x = v[j][0] - hi.x;
              lo.y = v[j][1] - hi.y;
              lo.z = v[j][2] - hi.z;
              lo.w = v[j][3] - hi.w;
              *reinterpret_cast<float4*>(out + TileIndex(nn, 4 * grp, 2 * tileN)) = hi;
              *reinterpret_cast<float4*>(out + TileIndex(tileN + nn, 4 * grp, 2 * tileN)) = lo;
            }
          }
          if (!ok || abortFlag) break;
          // the stores visible to the tensor cores before the stage is full
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(SmemAddr(full + slot)) : "memory");
        }
      }
      if (!ok) giveUp();
    }
  } else if (warp >= 2) {
    // -- epilogue ----------------------------------------------------------------
    const int quarter = warp % 4;
    int local = 0;
    for (int t = blockIdx.x; t < tileCount && !abortFlag; t += gridDim.x, ++local) {
      const int4 tile = tiles[t];
      const TcItem it = tcItems[tile.x];
      const int acc = local & 1;
      if (!WaitParity(SmemAddr(accFull + acc), static_cast<uint32_t>((local >> 1) & 1))) {
        giveUp();
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int n0 = tile.z * tileN;
      const int nCols = min(tileN, it.N - n0), nMma = (nCols + 15) / 16 * 16;
      // TMEM gives a lane one row; the rows go out through shared memory so
      // that each store instruction writes one row's 32 consecutive columns
      const int row0 = tile.y * kTcTileM + 32 * quarter;
      float(*block)[33] = rowsOut[warp - 2];
      for (int c0 = 0; c0 < nMma; c0 += 32) {
        uint32_t r[32];
        const uint32_t addr =
            tmem + (static_cast<uint32_t>(32 * quarter) << 16) + acc * accColumns + static_cast<uint32_t>(c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(addr)
            : "memory");
        if (c0 + 16 < nMma)
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
              "%14, %15}, [%16];"
              : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
                "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                "=r"(r[30]), "=r"(r[31])
              : "r"(addr + 16)
              : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int q = 0; q < 32; ++q) block[lane][q] = __uint_as_float(r[q]);
        if (fused) {
          // the A_hi B_lo half, tileN columns on
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
              "%14, %15}, [%16];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
              : "r"(addr + tileN)
              : "memory");
          if (c0 + 16 < nMma)
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15}, [%16];"
                : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
                  "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                  "=r"(r[30]), "=r"(r[31])
                : "r"(addr + tileN + 16)
                : "memory");
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int q = 0; q < 32; ++q) block[lane][q] += __uint_as_float(r[q]);
        }
        __syncwarp();
        const int n = c0 + lane;
        for (int rr = 0; rr < 32; ++rr) {
          const int i = row0 + rr;
          if (i < it.M && n < nCols) {
            float* c = C + it.c + static_cast<long long>(i) * it.ldc + n0 + n;
            const float v = block[rr][lane];
            *c = accumulate ? *c + v : v;
          }
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(SmemAddr(accEmpty + acc)) : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * accColumns)
                 : "memory");
}

}  // namespace

void LaunchPanelA(const GemmItem* items, const TcItem* tcItems, int count, int maxTiles, const double* table,
                  float* panels, cudaStream_t stream) {
  if (count == 0) return;
  const long long perItem = static_cast<long long>(maxTiles) * kATileFloats;
  const unsigned blocks = static_cast<unsigned>(std::min<long long>((perItem + 255) / 256, 4096));
  PanelAKernel<<<dim3(blocks, count), 256, 0, stream>>>(items, tcItems, table, panels);
}

void LaunchPackB(const TcItem* tcItems, int count, int maxTiles, int tileN, const float* B, float* packed,
                 cudaStream_t stream) {
  if (count == 0) return;
  const long long perItem = static_cast<long long>(maxTiles) * tileN * (kTcTileK / 4);
  const unsigned blocks = static_cast<unsigned>(std::min<long long>((perItem + 255) / 256, 4096));
  PackBKernel<<<dim3(blocks, count), 256, 0, stream>>>(tcItems, tileN, B, packed);
}

int RunGemmTc(const TcItem* tcItems, const int4* tiles, int tileCount, int tileN, const float* panels,
              const float* packed, const float* rawB, float* C, bool accumulate, int* errorFlag,
              cudaStream_t stream) {
  if (tileCount == 0) return SL3DGPU_OK;
  static const int sms = [] {
    int device = 0, count = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, device);
    return std::max(count, 1);
  }();
  const size_t stageBytes = 2 * (kATileFloats + static_cast<size_t>(tileN) * kTcTileK) * sizeof(float);
  const int stages = static_cast<int>(std::min<size_t>(8, std::max<size_t>(2, (200 * 1024) / stageBytes)));
  const size_t smem = stages * stageBytes + (2 * stages + 5) * sizeof(uint64_t) + 16;
  SL3D_CUDA(AllowDynamicSmem(TcGemmKernel));
  const int blocks = std::min(tileCount, sms);
  TcGemmKernel<<<blocks, kPersistentThreads, smem, stream>>>(tcItems, tiles, tileCount, tileN, stages, panels,
                                                            packed, rawB, C, accumulate, errorFlag);
  SL3D_CHECK_LAUNCH();
  return SL3DGPU_OK;
}

}  // namespace sl3dgpu
