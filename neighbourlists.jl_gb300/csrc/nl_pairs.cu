// Stages (c) count, (d) fill and (e) lazy reduction: one traversal kernel,
// specialised by mode.
//
// Replaces the reference's per-atom traversal
//   _for_each_neighbor_pair     gpu_kernels.jl:58-101
//   count_neighbours_kernel!    gpu_kernels.jl:132-152
//   fill_pairs_kernel!          gpu_kernels.jl:159-180
//   for_each_neighbour          cell_list.jl:779-801 (built-in reduction)
// and the pair vector formula _getR (cell_list.jl:525-531).
//
// Work decomposition: one warp per home cell.  All atoms of a home cell share
// the same (2n+1)^3 stencil (the reference computes it per atom from the same
// cell), so the warp stages the stencil's candidate atoms once in shared
// memory as FP32 positions relative to the home cell's corner, then screens
// every home atom against them with one candidate per lane.
//
// Precision: the screen runs in FP32 on cell-local offsets.  Geometry.lo/hi
// bracket cutoff^2 by a band that provably exceeds the FP32 error (see the
// host-side screen_band); only candidates inside the band, or involving an
// "exact" atom, are decided in FP64 with the reference arithmetic
// R = (xj - xi) + C'S, r2 = dot(R,R), r2 < cutoff^2.  The accepted pair set is
// therefore identical to the reference's.
//
// Output order: candidates are visited in the reference's order (stencil
// dz, dy, dx with dx fastest, then sorted order inside a cell) and compacted
// with ballots that preserve lane order, so each atom's pairs come out in the
// reference's order, and R is computed with the reference's operations, so
// i, j, S, R and first are bit-identical to the reference's arrays.
#include "nl_pairs.cuh"

namespace nl {

constexpr int kPairWarps = 4;   // warps per block
constexpr int kChunk = 192;     // staged candidates per warp and pass
constexpr int kQ = 64;          // pair queue per warp
constexpr int kCsR = 2;         // C'S table covers |S_k| <= kCsR
constexpr int kCsN = 2 * kCsR + 1;

struct __align__(16) WarpSmem {
  float4 cv[kChunk];        // candidate: (x, y, z) relative to home corner, w = meta bits
  int2 ci[kChunk];          // candidate: (sorted slot, packed s_loop)
  double hx[32][3];         // home batch: FP64 positions
  double hacc[32];          // home batch: lazy accumulators
  long long hbase[32];      // home batch: first[orig] - 1
  long long qslot[kQ];      // queue: output slot
  double qval[32];          // queue: lazy values
  int horig[32];            // home batch: original index (0-based)
  unsigned hmeta[32];       // home batch: meta bits
  int q[kQ];                // queue: (home atom << 16) | candidate
};

__device__ __forceinline__ unsigned lt_mask() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ int clampi(T v, int hi) {
  return v < T(0) ? 0 : (v > T(hi) ? hi : int(v));
}

__device__ __forceinline__ int pack3(int a, int b, int c) {
  return int((unsigned(a) & 0xFFu) | ((unsigned(b) & 0xFFu) << 8) | ((unsigned(c) & 0xFFu) << 16));
}
__device__ __forceinline__ int unpack3(int p, int k) { return int(int8_t((unsigned(p) >> (8 * k)) & 0xFFu)); }

// R = (xj - xi) + C'S with the reference's operation order.  For S == 0 the
// sum reduces to (xj - xi) + (+-0): that is xj - xi unless the difference is
// itself a zero, where the IEEE sign rule for adding two zeros applies.
__device__ __forceinline__ void pair_R(const Geometry& g, const double* cs_tab, const double* xi, const double* xj,
                                       int S0, int S1, int S2, double* R) {
  const double d0 = dsub(xj[0], xi[0]), d1 = dsub(xj[1], xi[1]), d2 = dsub(xj[2], xi[2]);
  if ((S0 | S1 | S2) == 0) {
    const double* z = cs_tab + 3 * ((kCsN * kCsN + kCsN + 1) * kCsR);  // entry S = (0,0,0)
    R[0] = d0 != 0.0 ? d0 : __longlong_as_double(__double_as_longlong(d0) & __double_as_longlong(z[0]));
    R[1] = d1 != 0.0 ? d1 : __longlong_as_double(__double_as_longlong(d1) & __double_as_longlong(z[1]));
    R[2] = d2 != 0.0 ? d2 : __longlong_as_double(__double_as_longlong(d2) & __double_as_longlong(z[2]));
    return;
  }
  double c0, c1, c2;
  if (abs(S0) <= kCsR && abs(S1) <= kCsR && abs(S2) <= kCsR) {
    const double* t = cs_tab + 3 * ((S0 + kCsR) + kCsN * ((S1 + kCsR) + kCsN * (S2 + kCsR)));
    c0 = t[0];
    c1 = t[1];
    c2 = t[2];
  } else {
    c0 = cts_k(g.C, S0, S1, S2, 0);
    c1 = cts_k(g.C, S0, S1, S2, 1);
    c2 = cts_k(g.C, S0, S1, S2, 2);
  }
  R[0] = dadd(d0, c0);
  R[1] = dadd(d1, c1);
  R[2] = dadd(d2, c2);
}

__device__ __forceinline__ double dot_ref(const double* R) {
  return dadd(dadd(dmul(R[0], R[0]), dmul(R[1], R[1])), dmul(R[2], R[2]));
}

// S = s_loop + wi - wj (gpu_kernels.jl:88).  Windings come from the packed
// records unless either atom is "exact", in which case they are recomputed
// from the FP64 positions.
__device__ __forceinline__ void pair_S(const Geometry& g, const double* xi, const double* xj, unsigned mi,
                                       unsigned mj, int slp, int* S) {
  if (!meta_exact(mi) && !meta_exact(mj)) {
#pragma unroll
    for (int k = 0; k < 3; ++k) S[k] = unpack3(slp, k) + meta_w(mi, k) - meta_w(mj, k);
  } else {
    Binned bi, bj;
    bin_position(g, xi[0], xi[1], xi[2], bi);
    bin_position(g, xj[0], xj[1], xj[2], bj);
#pragma unroll
    for (int k = 0; k < 3; ++k) S[k] = unpack3(slp, k) + bi.w[k] - bj.w[k];
  }
}

template <typename TI, int MODE>
__device__ __forceinline__ void flush_queue(const PairArgs<TI>& A, const double* cs_tab, WarpSmem& W, int n,
                                            int lane) {
  if (lane < n) {
    const int e = W.q[lane];
    const int a = e >> 16, f = e & 0xFFFF;
    const int slot_j = W.ci[f].x;
    const unsigned mj = __float_as_uint(W.cv[f].w), mi = W.hmeta[a];
    double xj[3];
    xj[0] = A.Xs[3LL * slot_j + 0];
    xj[1] = A.Xs[3LL * slot_j + 1];
    xj[2] = A.Xs[3LL * slot_j + 2];
    const double* xi = W.hx[a];
    int S[3];
    pair_S(A.g, xi, xj, mi, mj, W.ci[f].y, S);
    if (MODE == kModeFill) {
      const long long out = W.qslot[lane];
      if (out < A.capacity) {
        A.oi[out] = TI(W.horig[a]) + 1;
        A.oj[out] = TI(clampi(A.perm[slot_j] - 1, A.g.nat - 1)) + 1;
        A.oS[3 * out + 0] = TI(S[0]);
        A.oS[3 * out + 1] = TI(S[1]);
        A.oS[3 * out + 2] = TI(S[2]);
        if (A.oR) {
          double R[3];
          pair_R(A.g, cs_tab, xi, xj, S[0], S[1], S[2], R);
          A.oR[3 * out + 0] = R[0];
          A.oR[3 * out + 1] = R[1];
          A.oR[3 * out + 2] = R[2];
        }
      } else {
        atomicOr(A.err, kFlagCapacity);
      }
    } else {  // lazy: f(R) = 1 / ((r2*r2)*r2)
      double R[3];
      pair_R(A.g, cs_tab, xi, xj, S[0], S[1], S[2], R);
      const double r2 = dot_ref(R);
      W.qval[lane] = __ddiv_rn(1.0, dmul(dmul(r2, r2), r2));
    }
  }
  __syncwarp();
  if (MODE == kModeLazyR6) {
    // accumulate in queue order so that every atom's sum follows the
    // reference's traversal order exactly
    if (lane == 0)
      for (int e = 0; e < n; ++e) {
        const int a = W.q[e] >> 16;
        W.hacc[a] = dadd(W.hacc[a], W.qval[e]);
      }
    __syncwarp();
  }
}

template <typename TI, int MODE>
__global__ void __launch_bounds__(kPairWarps * 32) k_pairs(PairArgs<TI> A) {
  __shared__ WarpSmem sm[kPairWarps];
  __shared__ double cs_tab[3 * kCsN * kCsN * kCsN];
  const Geometry& g = A.g;
  for (int t = threadIdx.x; t < kCsN * kCsN * kCsN; t += blockDim.x) {
    const int s0 = t % kCsN - kCsR, s1 = (t / kCsN) % kCsN - kCsR, s2 = t / (kCsN * kCsN) - kCsR;
    cs_tab[3 * t + 0] = cts_k(g.C, s0, s1, s2, 0);
    cs_tab[3 * t + 1] = cts_k(g.C, s0, s1, s2, 1);
    cs_tab[3 * t + 2] = cts_k(g.C, s0, s1, s2, 2);
  }
  __syncthreads();

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpSmem& W = sm[warp];
  const int nwarps = gridDim.x * kPairWarps;
  const int sx = 2 * g.nxyz[0] + 1, sy = 2 * g.nxyz[1] + 1, sz = 2 * g.nxyz[2] + 1;
  const int nst = sx * sy * sz;
  const int center = g.nxyz[0] + sx * (g.nxyz[1] + sy * g.nxyz[2]);
  unsigned long long rechecks = 0;

  for (int h = blockIdx.x * kPairWarps + warp; h < g.ncells; h += nwarps) {
    // offsets are clamped to [0, nat] so that a malformed cell list (which the
    // prepare pass reports as inconsistent) can never index out of bounds
    const int hs = clampi(A.cell_offsets[h] - 1, g.nat), he = clampi(A.cell_offsets[h + 1] - 1, g.nat);
    if (hs >= he) continue;
    const int hc0 = h % g.ns[0] + 1, hc1 = (h / g.ns[0]) % g.ns[1] + 1, hc2 = h / (g.ns[0] * g.ns[1]) + 1;

    for (int hb = hs; hb < he; hb += 32) {
      const int nb = min(32, he - hb);
      float ux = 0.f, uy = 0.f, uz = 0.f;
      long long my_run = 0;  // pairs emitted so far by home atom hb+lane
      if (lane < nb) {
        const int s = hb + lane;
        const float4 r = A.rec[s];
        ux = r.x;
        uy = r.y;
        uz = r.z;
        W.hmeta[lane] = __float_as_uint(r.w);
        const int orig = clampi(A.perm[s] - 1, g.nat - 1);
        W.horig[lane] = orig;
        W.hx[lane][0] = A.Xs[3LL * s + 0];
        W.hx[lane][1] = A.Xs[3LL * s + 1];
        W.hx[lane][2] = A.Xs[3LL * s + 2];
        if (MODE == kModeFill) W.hbase[lane] = (long long)A.first[orig] - 1;
        if (MODE == kModeLazyR6) W.hacc[lane] = 0.0;
      }
      int qn = 0;
      __syncwarp();

      for (int gb = 0; gb < nst; gb += 32) {
        // ---- stencil cell held by this lane
        const int q = gb + lane;
        int cstart = 0, ccount = 0, slp = 0;
        float ox = 0.f, oy = 0.f, oz = 0.f;
        if (q < nst) {
          const int d0 = q % sx - g.nxyz[0], d1 = (q / sx) % sy - g.nxyz[1], d2 = q / (sx * sy) - g.nxyz[2];
          const bool inb = (g.pbc[0] || (hc0 + d0 >= 1 && hc0 + d0 <= g.ns[0])) &&
                           (g.pbc[1] || (hc1 + d1 >= 1 && hc1 + d1 <= g.ns[1])) &&
                           (g.pbc[2] || (hc2 + d2 >= 1 && hc2 + d2 <= g.ns[2]));
          if (inb) {
            int s0, s1, s2;
            const int c0 = wrap_shift(hc0 + d0, g.ns[0], g.pbc[0], s0);
            const int c1 = wrap_shift(hc1 + d1, g.ns[1], g.pbc[1], s1);
            const int c2 = wrap_shift(hc2 + d2, g.ns[2], g.pbc[2], s2);
            const int lin = linear_cell(g, c0, c1, c2);
            cstart = clampi(A.cell_offsets[lin] - 1, g.nat);
            ccount = max(clampi(A.cell_offsets[lin + 1] - 1, g.nat) - cstart, 0);
            slp = pack3(s0, s1, s2);
            const float fd0 = float(d0), fd1 = float(d1), fd2 = float(d2);
            ox = fmaf(fd2, g.b[6], fmaf(fd1, g.b[3], fd0 * g.b[0]));
            oy = fmaf(fd2, g.b[7], fmaf(fd1, g.b[4], fd0 * g.b[1]));
            oz = fmaf(fd2, g.b[8], fmaf(fd1, g.b[5], fd0 * g.b[2]));
          }
        }
        int incl = ccount;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int tg = __shfl_sync(0xffffffffu, incl, 31);
        // flattened index of the home atoms inside this group (center cell)
        const int cl = center - gb;
        const int center_excl = (cl >= 0 && cl < 32) ? __shfl_sync(0xffffffffu, incl - ccount, cl & 31) : -1;

        for (int cb = 0; cb < tg; cb += kChunk) {
          const int nch = min(kChunk, tg - cb);
          if (MODE != kModeCount && qn > 0) {
            flush_queue<TI, MODE>(A, cs_tab, W, qn, lane);
            qn = 0;
          }
          __syncwarp();
          // ---- stage the chunk
          for (int f0 = 0; f0 < nch; f0 += 32) {
            const int f = f0 + lane;
            const int gf = cb + min(f, nch - 1);
            int qq = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
              const int v = __shfl_sync(0xffffffffu, incl, qq + step - 1);
              if (v <= gf) qq += step;
            }
            const int q_incl = __shfl_sync(0xffffffffu, incl, qq);
            const int q_cnt = __shfl_sync(0xffffffffu, ccount, qq);
            const int q_start = __shfl_sync(0xffffffffu, cstart, qq);
            const int q_slp = __shfl_sync(0xffffffffu, slp, qq);
            const float qx = __shfl_sync(0xffffffffu, ox, qq);
            const float qy = __shfl_sync(0xffffffffu, oy, qq);
            const float qz = __shfl_sync(0xffffffffu, oz, qq);
            if (f < nch) {
              const int slot = q_start + (gf - (q_incl - q_cnt));
              const float4 r = A.rec[slot];
              W.cv[f] = make_float4(r.x + qx, r.y + qy, r.z + qz, r.w);
              W.ci[f] = make_int2(slot, q_slp);
            }
          }
          __syncwarp();

          // ---- screen every home atom of the batch
          for (int a = 0; a < nb; ++a) {
            const float ax = __shfl_sync(0xffffffffu, ux, a);
            const float ay = __shfl_sync(0xffffffffu, uy, a);
            const float az = __shfl_sync(0xffffffffu, uz, a);
            long long run = __shfl_sync(0xffffffffu, my_run, a);
            const unsigned mi = W.hmeta[a];
            const bool exact_i = meta_exact(mi);
            // the self candidate (j == i with zero loop shift) sits in the center cell
            const int self_f = center_excl >= 0 ? center_excl + (hb + a - hs) - cb : -1;
            for (int r0 = 0; r0 < nch; r0 += 32) {
              const int f = r0 + lane;
              bool acc = false;
              if (f < nch && f != self_f) {
                const float4 c = W.cv[f];
                const float rx = c.x - ax, ry = c.y - ay, rz = c.z - az;
                const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
                const unsigned mj = __float_as_uint(c.w);
                const bool ex = exact_i || meta_exact(mj);
                if (!ex && r2 < g.lo) {
                  acc = true;
                } else if (ex || r2 <= g.hi) {
                  // FP64 decision with the reference arithmetic
                  ++rechecks;
                  const int slot_j = W.ci[f].x;
                  double xj[3];
                  xj[0] = A.Xs[3LL * slot_j + 0];
                  xj[1] = A.Xs[3LL * slot_j + 1];
                  xj[2] = A.Xs[3LL * slot_j + 2];
                  int S[3];
                  pair_S(g, W.hx[a], xj, mi, mj, W.ci[f].y, S);
                  double R[3];
                  pair_R(g, cs_tab, W.hx[a], xj, S[0], S[1], S[2], R);
                  acc = dot_ref(R) < g.cutoff_sq;
                }
              }
              const unsigned mask = __ballot_sync(0xffffffffu, acc);
              const int np = __popc(mask);
              if (MODE != kModeCount && np) {
                const int rank = __popc(mask & lt_mask());
                if (acc) {
                  W.q[qn + rank] = (a << 16) | f;
                  if (MODE == kModeFill) W.qslot[qn + rank] = W.hbase[a] + run + rank;
                }
                qn += np;
                __syncwarp();
                if (qn >= 32) {
                  flush_queue<TI, MODE>(A, cs_tab, W, 32, lane);
                  qn -= 32;
                  // move the overflow [32, 32+qn) down to [0, qn); the ranges are disjoint
                  if (lane < qn) {
                    W.q[lane] = W.q[32 + lane];
                    W.qslot[lane] = W.qslot[32 + lane];
                  }
                  __syncwarp();
                }
              }
              run += np;
            }
            if (lane == a) my_run = run;
          }
        }
      }
      if (MODE != kModeCount && qn > 0) flush_queue<TI, MODE>(A, cs_tab, W, qn, lane);
      __syncwarp();
      if (lane < nb) {
        if (MODE == kModeCount) A.counts[W.horig[lane]] = int(my_run);
        if (MODE == kModeLazyR6) A.per_atom[W.horig[lane]] = W.hacc[lane];
      }
      __syncwarp();
    }
  }
  // statistics: number of FP64 decisions
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_xor_sync(0xffffffffu, rechecks, o);
  if (lane == 0 && rechecks) atomicAdd(A.stats, rechecks);
}

template <typename TI>
void launch_pairs(int mode, const PairArgs<TI>& a, int num_sms, cudaStream_t st) {
  if (a.g.nat <= 0 || a.g.ncells <= 0) return;
  const int per_sm = 6;  // resident blocks per SM targeted by the grid
  long long blocks = ((long long)a.g.ncells + kPairWarps - 1) / kPairWarps;
  if (blocks > (long long)num_sms * per_sm) blocks = (long long)num_sms * per_sm;
  if (blocks < 1) blocks = 1;
  switch (mode) {
    case kModeCount: k_pairs<TI, kModeCount><<<int(blocks), kPairWarps * 32, 0, st>>>(a); break;
    case kModeFill: k_pairs<TI, kModeFill><<<int(blocks), kPairWarps * 32, 0, st>>>(a); break;
    default: k_pairs<TI, kModeLazyR6><<<int(blocks), kPairWarps * 32, 0, st>>>(a); break;
  }
}

template void launch_pairs<int32_t>(int, const PairArgs<int32_t>&, int, cudaStream_t);
template void launch_pairs<int64_t>(int, const PairArgs<int64_t>&, int, cudaStream_t);

}  // namespace nl
