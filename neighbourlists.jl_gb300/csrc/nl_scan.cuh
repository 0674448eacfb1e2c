// Single-pass exclusive prefix sum of int32 counts into CSR offsets, using
// decoupled look-back over tiles claimed in order from an atomic counter.
//
// Produces the 1-based offsets the reference builds with
// AcceleratedKernels.accumulate! followed by `.+= 1`
// (gpu_kernels.jl:222-237 for `first`, :262-285 for `cell_offsets`):
//   out1[0] = 1, out1[k+1] = out1[k] + in[k]      (TI, length n+1)
// and optionally the same 0-based in int32 (out0, length n+1) for internal use
// (either output may be null).
//
// Every wait on another tile's status is bounded: after kSpinLimit polls the
// tile sets kFlagTimeout in the error word and proceeds, so the kernel
// always terminates; the host turns the flag into kErrTimeout.
#pragma once
#include "nl_common.cuh"

namespace nl {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;                         // per thread
constexpr int kScanTile = kScanBlock * kScanItems;    // 2048 elements
constexpr unsigned long long kStFlagAgg = 1ull << 62;
constexpr unsigned long long kStFlagPre = 2ull << 62;
constexpr unsigned long long kStValue = (1ull << 62) - 1;
constexpr long long kSpinLimit = 1ll << 22;

__device__ __forceinline__ long long warp_incl_scan(long long v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long n = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += n;
  }
  return v;
}

__device__ __forceinline__ unsigned long long load_status(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}

inline int scan_tiles(long long n) { return int((n + kScanTile - 1) / kScanTile); }

// status[ntiles] and counter[1] must be zero before launch.
template <typename TI>
__global__ void __launch_bounds__(kScanBlock) k_scan_offsets(const int* __restrict__ in, long long n,
                                                             TI* __restrict__ out1, int* __restrict__ out0,
                                                             unsigned long long* __restrict__ status,
                                                             int* __restrict__ counter, long long* __restrict__ total,
                                                             unsigned* __restrict__ err) {
  __shared__ int s_tile;
  __shared__ long long s_warp[kScanBlock / 32];
  __shared__ long long s_prefix;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
  __syncthreads();
  const int tile = s_tile;
  const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
  int v[kScanItems];
  long long local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    long long idx = base + k;
    v[k] = idx < n ? in[idx] : 0;
    local += v[k];
  }
  long long incl = warp_incl_scan(local);
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < kScanBlock / 32 ? s_warp[lane] : 0;
    long long wi = warp_incl_scan(w);
    if (lane < kScanBlock / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
    long long agg = __shfl_sync(0xffffffffu, wi, kScanBlock / 32 - 1);
    // publish and look back
    long long prefix = 0;
    if (tile == 0) {
      if (lane == 0) atomicExch(&status[0], kStFlagPre | (unsigned long long)agg);
    } else {
      if (lane == 0) atomicExch(&status[tile], kStFlagAgg | (unsigned long long)agg);
      int pred = tile - 1;
      bool done = false;
      long long spins = 0;
      while (!done) {
        int t = pred - lane;
        unsigned long long st = t >= 0 ? load_status(&status[t]) : kStFlagPre;
        // wait until every status in the window is published
        while (__any_sync(0xffffffffu, (st >> 62) == 0)) {
          if (++spins > kSpinLimit) {
            if (lane == 0) atomicOr(err, kFlagTimeout);
            st = kStFlagPre;  // give up: treat as prefix 0
            break;
          }
          __nanosleep(64);
          if ((st >> 62) == 0) st = t >= 0 ? load_status(&status[t]) : kStFlagPre;
        }
        unsigned pre_mask = __ballot_sync(0xffffffffu, (st >> 62) == 2);
        long long val = (long long)(st & kStValue);
        if (pre_mask) {
          int first_pre = __ffs(pre_mask) - 1;  // nearest tile with an inclusive prefix
          if (lane > first_pre) val = 0;
          done = true;
        }
        // sum values of lanes 0..first_pre (or all lanes if none)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
        prefix += val;
        pred -= 32;
      }
      if (lane == 0) atomicExch(&status[tile], kStFlagPre | (unsigned long long)(prefix + agg));
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  long long run = s_prefix + s_warp[warp] + (incl - local);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    long long idx = base + k;
    if (idx < n) {
      if (out1) out1[idx] = TI(run + 1);
      if (out0) out0[idx] = int(run);
    }
    run += v[k];
  }
  // the thread owning element n-1 also writes the sentinel and the total
  if (n > 0 && base <= n - 1 && n - 1 < base + kScanItems) {
    if (out1) out1[n] = TI(run + 1);
    if (out0) out0[n] = int(run);
    if (total) *total = run;
    if (run + 1 > IndexTraits<TI>::kMax) atomicOr(err, kFlagIndexOverflow);
  }
}

}  // namespace nl
