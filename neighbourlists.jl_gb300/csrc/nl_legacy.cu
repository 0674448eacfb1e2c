// The legacy linked-list PairList on the GPU (cell_list.jl:11-20, 185-505).
//
//   _fix_cell_        (:459-505)  k_legacy_fix + k_legacy_shift, cell update on the host
//   _celllist_        (:185-230)  the sort-based build (nl_build.cu): a linked list of a bin
//                                 holds its atoms in ascending index order, which is the
//                                 order of the stable counting sort
//   _find_neighbours_! (:301-366) k_legacy_prepare (per-atom bin-relative coordinates) and
//                                 k_legacy_pairs (screen, count, fill)
//   get_first         (:401-418)  the pair-offset scan (nl_scan.cuh)
//   sort_neigs!       (:427-446)  rank sort of each atom's (j, S) by j, ties in traversal
//                                 order (sortperm is stable), inside the fill pass
//
// Screening.  The legacy distance of a candidate is
//   dx = (D_j - D_i) + bins * xyz,   D_a = x_a - bins * (bin_trunc(c0_a) - 1),
// accepted when dot(dx, dx) < cutoff^2 (:335-352).  D is bin-relative, so an
// FP32 evaluation from D rounded to FP32 is accurate to a few ulps of the bin
// size; candidates within a rigorous band of the cutoff (derived below from
// max |D| and max |bins * xyz|) are decided again with the reference's FP64
// arithmetic, so membership is the reference's exactly.
#include <cstring>

#include "nl_legacy.cuh"
#include "nl_scan.cuh"

namespace nl {

namespace {

constexpr int kLegacyWarps = 8;      // warps per block of the pair kernels
constexpr int kLegacyStage = 256;    // pairs of one atom sorted in shared memory; more take two traversals

inline int grid_for(long long n, int block, int max_blocks) {
  long long g = (n + block - 1) / block;
  if (g > max_blocks) g = max_blocks;
  return g < 1 ? 1 : int(g);
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Julia's mod(x, 1.0) for Float64: r = rem(x, 1); r == 0 -> +0; r < 0 -> r + 1.
// rem (fmod) is exact.
__device__ __forceinline__ double julia_mod1(double x) {
  const double r = fmod(x, 1.0);
  if (r == 0.0) return 0.0;
  if (!(r > 0.0)) return dadd(r, 1.0);
  return r;
}

// bin_wrap (cell_list.jl:33-37): i mapped into [1, n] by multiples of n
__device__ __forceinline__ int bin_wrap(int i, int n) { return i - n * floordiv(i - 1, n); }

__device__ __forceinline__ int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }

// (bins * v)_r for an integer vector v (exactly converted), StaticArrays
// mat-vec order (a1*b1 + a2*b2) + a3*b3
__device__ __forceinline__ double bins_mul(const double* bins, int r, int v0, int v1, int v2) {
  return dadd(dadd(dmul(bins[r], double(v0)), dmul(bins[r + 3], double(v1))), dmul(bins[r + 6], double(v2)));
}

struct FixGeo {
  double inv[9];
  double C[9];
  int pbc[3];
};

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long n = __shfl_xor_sync(0xffffffffu, v, o);
    v = n < v ? n : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long n = __shfl_xor_sync(0xffffffffu, v, o);
    v = n > v ? n : v;
  }
  return v;
}

// _fix_cell_ per atom (cell_list.jl:467-486): lambda = inv(C)' * x; periodic
// components outside [0, 1) become mod(lambda, 1) and the position is
// rewritten as C' * lambda; open components outside [0, 1) update the
// extremes (min from 0, max from 1).
__global__ void __launch_bounds__(256) k_legacy_fix(FixGeo fg, const double* X, double* Xout, int nat,
                                                    unsigned long long* __restrict__ minmax,
                                                    unsigned* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nat; base += stride) {
    const long long a = base + lane;
    const bool valid = a < nat;
    unsigned long long kmin[3], kmax[3];
    bool open_out[3] = {false, false, false};
    if (valid) {
      const double x0 = X[3 * a + 0], x1 = X[3 * a + 1], x2 = X[3 * a + 2];
      if (!isfinite(x0) || !isfinite(x1) || !isfinite(x2)) atomicOr(err, kFlagBadPosition);
      double lam[3];
      bool upd = false;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        lam[k] = frac_k(fg.inv, x0, x1, x2, k);
        if (!(0.0 <= lam[k] && lam[k] < 1.0)) {
          if (fg.pbc[k]) {
            lam[k] = julia_mod1(lam[k]);
            upd = true;
          } else {
            open_out[k] = true;
          }
        }
        kmin[k] = open_out[k] ? legacy_key(lam[k]) : ~0ull;
        kmax[k] = open_out[k] ? legacy_key(lam[k]) : 0ull;
      }
      double y0 = x0, y1 = x1, y2 = x2;
      if (upd) {  // C' * lambda
        y0 = dadd(dadd(dmul(fg.C[0], lam[0]), dmul(fg.C[1], lam[1])), dmul(fg.C[2], lam[2]));
        y1 = dadd(dadd(dmul(fg.C[3], lam[0]), dmul(fg.C[4], lam[1])), dmul(fg.C[5], lam[2]));
        y2 = dadd(dadd(dmul(fg.C[6], lam[0]), dmul(fg.C[7], lam[1])), dmul(fg.C[8], lam[2]));
      }
      Xout[3 * a + 0] = y0;
      Xout[3 * a + 1] = y1;
      Xout[3 * a + 2] = y2;
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        kmin[k] = ~0ull;
        kmax[k] = 0ull;
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (__any_sync(0xffffffffu, open_out[k])) {
        const unsigned long long mn = warp_min_u64(kmin[k]);
        const unsigned long long mx = warp_max_u64(kmax[k]);
        if (lane == 0) {
          atomicMin(&minmax[k], mn);
          atomicMax(&minmax[3 + k], mx);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_legacy_shift(double* X, long long n3, double t0, double t1, double t2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += stride) {
    const int k = int(e % 3);
    X[e] = dadd(X[e], k == 0 ? t0 : (k == 1 ? t1 : t2));
  }
}

// Per sorted slot: c0 = floor(frac * ns + 1) (position_to_cell_index,
// cell_list.jl:66-74), D = x - bins * (bin_trunc(c0) - 1) (:321-323,
// :346-349), D in FP32, and max |D| over the atoms.
template <typename TI>
__global__ void __launch_bounds__(256) k_legacy_prepare(LegacyArgs<TI> a) {
  const LegacyGeo& g = a.g;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < g.nat; base += stride) {
    const long long s = base + (threadIdx.x & 31);
    unsigned m = 0;
    if (s < g.nat) {
      const double x[3] = {a.Xs[3 * s + 0], a.Xs[3 * s + 1], a.Xs[3 * s + 2]};
      int c0[3], ct[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double y = dmul(frac_k(g.inv, x[0], x[1], x[2], k), double(g.ns[k]));
        double yp = dadd(y, 1.0);
        if (!(fabs(yp) < kBadY)) {  // cannot be binned (also flagged by the build)
          atomicOr(a.err, kFlagBadPosition);
          yp = 1.0;
        }
        c0[k] = int(__double2ll_rd(yp));
        ct[k] = g.pbc[k] ? c0[k] : clampi(c0[k], 1, g.ns[k]);
      }
      double D[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        D[r] = dsub(x[r], bins_mul(g.bins, r, ct[0] - 1, ct[1] - 1, ct[2] - 1));
        a.D[3 * s + r] = D[r];
        const unsigned b = __float_as_uint(__double2float_ru(fabs(D[r])));
        m = b > m ? b : m;
      }
      bool inbox = true;  // then bin_trunc(c0) is the bin the atom was listed in
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (g.pbc[k] && (c0[k] < 1 || c0[k] > g.ns[k])) inbox = false;
      a.Df[s] = make_float4(__double2float_rn(D[0]), __double2float_rn(D[1]), __double2float_rn(D[2]),
                            inbox ? 1.f : 0.f);
      a.c0[s] = make_int4(c0[0], c0[1], c0[2], 0);
    }
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(a.dmax, m);
  }
}

// Per-warp shared state of one chunk of 32 stencil cells.
struct LegacyChunk {
  int incl[32];     // inclusive prefix of the candidate counts
  int start[32];    // first sorted slot of the cell
  int q[32];        // stencil index (dx fastest, then dy, dz: CartesianIndices order)
  float off[3][32]; // bins * xyz in FP32
  int S[3][32];     // (ci0 - cj + xyz) .÷ ns for the bin cj itself (S of the candidates inside the box)
};
struct LegacyStage {
  int j[kLegacyStage];     // 1-based original index of j (also the rank tile of long lists)
  int S[3][kLegacyStage];
};

// One warp per sorted slot (atom i).  The stencil is walked in the
// reference's order (xyz_range = CartesianIndices, x fastest, :272-276), each
// neighbouring bin's atoms in ascending index order, skipping bins outside
// the open axes (:315) and i itself in the home bin (:331).
//
// Count: pairs per atom.  Fill: the accepted (j, S) of atom i are ranked by
// (j, traversal position) -- sort_neigs!'s stable sortperm -- and written
// at first[i]; up to kLegacyStage pairs are ranked in shared memory, longer
// lists take a second traversal that ranks against the j written to the
// atom's range of the i array by the first.
template <typename TI, bool FILL>
__global__ void __launch_bounds__(kLegacyWarps * 32) k_legacy_pairs(LegacyArgs<TI> a) {
  __shared__ LegacyChunk chunk_all[kLegacyWarps];
  __shared__ LegacyStage stage_all[FILL ? kLegacyWarps : 1];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  LegacyChunk& W = chunk_all[wib];
  LegacyStage& T = stage_all[FILL ? wib : 0];
  const LegacyGeo& g = a.g;

  // FP32 screen band.  With u = 2^-24, M = max |D_r| and O = max |off_r|,
  // the FP32 offset (two FMAs on the FP32 bins) is within 4u O of the
  // reference's FP64 bins * xyz, and each FP32 component of dx is within
  // e = 6u (2M + O) of the exact (D_j - D_i) + off; a candidate whose FP32
  // r^2 is outside cutoff^2 -+ B, B = 2 (4u cutoff^2 + 2 sqrt(3) (cutoff + e) e
  // + 3 e^2), is decided the same way by the reference's FP64 arithmetic.
  const double u = 5.9604644775390625e-08;
  const double M = double(__uint_as_float(*a.dmax));
  const double e = 6.0 * u * (2.0 * M + g.offmax) * 1.0001;
  const double B = 2.0 * (4.0 * u * g.cutoff_sq + 3.4641016151377544 * (g.cutoff + e) * e + 3.0 * e * e);
  const float lo = __double2float_rd(g.cutoff_sq - B);
  const float hi = __double2float_ru(g.cutoff_sq + B);

  const int wx = 2 * g.nxyz[0] + 1, wy = 2 * g.nxyz[1] + 1;
  const int nst = wx * wy * (2 * g.nxyz[2] + 1);
  const int qcenter = g.nxyz[0] + wx * (g.nxyz[1] + wy * g.nxyz[2]);
  unsigned long long rechecks = 0;

  for (long long slot = (long long)blockIdx.x * kLegacyWarps + wib; slot < g.nat;
       slot += (long long)gridDim.x * kLegacyWarps) {
    const double Di0 = a.D[3 * slot + 0], Di1 = a.D[3 * slot + 1], Di2 = a.D[3 * slot + 2];
    const float4 dfi = a.Df[slot];
    const int4 c0i = a.c0[slot];
    const int ci0[3] = {c0i.x, c0i.y, c0i.z};
    int ci[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) ci[k] = g.pbc[k] ? bin_wrap(ci0[k], g.ns[k]) : clampi(ci0[k], 1, g.ns[k]);
    const TI iorig = a.perm[slot];

    long long base = 0;
    int n = 0;
    bool write_ok = false;
    if constexpr (FILL) {
      base = (long long)a.first[iorig - 1] - 1;
      n = int((long long)a.first[iorig] - 1 - base);
      write_ok = base >= 0 && n >= 0 && base + n <= a.capacity;
      if (!write_ok && lane == 0) atomicOr(a.err, kFlagCapacity);
    }
    const bool staged = n <= kLegacyStage;
    const int passes = (FILL && !staged) ? 2 : 1;
    int nacc = 0;

    for (int pass = 0; pass < passes; ++pass) {
      nacc = 0;
      for (int q0 = 0; q0 < nst; q0 += 32) {
        const int q = q0 + lane;
        bool valid = q < nst;
        const int x = q % wx - g.nxyz[0];
        const int rest = q / wx;
        const int y = rest % wy - g.nxyz[1];
        const int z = rest / wy - g.nxyz[2];
        const int xyz[3] = {x, y, z};
        int cj[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          cj[k] = g.pbc[k] ? bin_wrap(ci[k] + xyz[k], g.ns[k]) : ci[k] + xyz[k];
          valid = valid && cj[k] >= 1 && cj[k] <= g.ns[k];
        }
        int st = 0, cnt = 0;
        float o0 = 0.f, o1 = 0.f, o2 = 0.f;
        int s0 = 0, s1 = 0, s2 = 0;
        if (valid) {
          const int lin = (cj[0] - 1) + g.ns[0] * ((cj[1] - 1) + g.ns[1] * (cj[2] - 1));
          st = a.cell_start[lin];
          cnt = a.cell_start[lin + 1] - st;
          const float fx = float(x), fy = float(y), fz = float(z);
          o0 = fmaf(g.binsf[6], fz, fmaf(g.binsf[3], fy, g.binsf[0] * fx));
          o1 = fmaf(g.binsf[7], fz, fmaf(g.binsf[4], fy, g.binsf[1] * fx));
          o2 = fmaf(g.binsf[8], fz, fmaf(g.binsf[5], fy, g.binsf[2] * fx));
          s0 = (ci0[0] - cj[0] + x) / g.ns[0];
          s1 = (ci0[1] - cj[1] + y) / g.ns[1];
          s2 = (ci0[2] - cj[2] + z) / g.ns[2];
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        __syncwarp();
        W.incl[lane] = incl;
        W.start[lane] = st;
        W.q[lane] = q;
        W.off[0][lane] = o0;
        W.off[1][lane] = o1;
        W.off[2][lane] = o2;
        W.S[0][lane] = s0;
        W.S[1][lane] = s1;
        W.S[2][lane] = s2;
        __syncwarp();
        const int total = __shfl_sync(0xffffffffu, incl, 31);

        for (int p0 = 0; p0 < total; p0 += 32) {
          const int p = p0 + lane;
          bool acc = false, rechk = false, jin = false;
          int js = 0, owner = 0;
          if (p < total) {
            int lo_l = 0, hi_l = 31;  // first lane whose inclusive count exceeds p
            while (lo_l < hi_l) {
              const int mid = (lo_l + hi_l) >> 1;
              if (W.incl[mid] > p)
                hi_l = mid;
              else
                lo_l = mid + 1;
            }
            owner = lo_l;
            js = W.start[owner] + (p - (owner ? W.incl[owner - 1] : 0));
            if (!(js == slot && W.q[owner] == qcenter)) {
              const float4 dj = a.Df[js];
              jin = dj.w != 0.f;
              const float d0 = (dj.x - dfi.x) + W.off[0][owner];
              const float d1 = (dj.y - dfi.y) + W.off[1][owner];
              const float d2 = (dj.z - dfi.z) + W.off[2][owner];
              const float r2 = d0 * d0 + d1 * d1 + d2 * d2;
              if (r2 < lo) {
                acc = true;
              } else if (r2 <= hi) {  // the reference's FP64 test (:346-352)
                rechk = true;
                const int qo = W.q[owner];
                const int ox = qo % wx - g.nxyz[0], orr = qo / wx;
                const int oy = orr % wy - g.nxyz[1], oz = orr / wy - g.nxyz[2];
                const double e0 = dadd(dsub(a.D[3LL * js + 0], Di0), bins_mul(g.bins, 0, ox, oy, oz));
                const double e1 = dadd(dsub(a.D[3LL * js + 1], Di1), bins_mul(g.bins, 1, ox, oy, oz));
                const double e2 = dadd(dsub(a.D[3LL * js + 2], Di2), bins_mul(g.bins, 2, ox, oy, oz));
                const double d2x = dadd(dadd(dmul(e0, e0), dmul(e1, e1)), dmul(e2, e2));
                acc = d2x < g.cutoff_sq;
              }
            }
          }
          if constexpr (!FILL) rechecks += rechk ? 1 : 0;
          const unsigned mask = __ballot_sync(0xffffffffu, acc);
          if constexpr (FILL) {
            int jo = 0, S[3] = {0, 0, 0};
            const int pos = nacc + __popc(mask & lanemask_lt());
            if (acc) {
              jo = int(a.perm[js]);
              if (jin) {  // bin_trunc(c0_j) is the bin itself
                S[0] = W.S[0][owner];
                S[1] = W.S[1][owner];
                S[2] = W.S[2][owner];
              } else {
                const int qo = W.q[owner];
                const int oxyz[3] = {qo % wx - g.nxyz[0], (qo / wx) % wy - g.nxyz[1], (qo / wx) / wy - g.nxyz[2]};
                const int4 c0j = a.c0[js];
                const int cjp[3] = {c0j.x, c0j.y, c0j.z};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                  const int ct = g.pbc[k] ? cjp[k] : clampi(cjp[k], 1, g.ns[k]);
                  S[k] = (ci0[k] - ct + oxyz[k]) / g.ns[k];  // truncating, like Julia's div (:358)
                }
              }
            }
            if (staged) {
              if (acc && pos < kLegacyStage) {
                T.j[pos] = jo;
                T.S[0][pos] = S[0];
                T.S[1][pos] = S[1];
                T.S[2][pos] = S[2];
              }
            } else if (pass == 0) {
              if (acc && write_ok && pos < n) a.oi[base + pos] = TI(jo);
            } else {
              // rank against the traversal-order j of the first pass, in tiles
              long long rank = 0;
              for (int t0 = 0; t0 < n; t0 += kLegacyStage) {
                const int tn = min(kLegacyStage, n - t0);
                __syncwarp();
                for (int l = lane; l < tn; l += 32) T.j[l] = write_ok ? int(a.oi[base + t0 + l]) : 0;
                __syncwarp();
                if (acc) {
                  for (int l = 0; l < tn; ++l) {
                    const int j2 = T.j[l];
                    rank += (j2 < jo) | ((j2 == jo) & (t0 + l < pos));
                  }
                }
              }
              if (acc && write_ok && rank < n) {
                a.oj[base + rank] = TI(jo);
                a.oS[3 * (base + rank) + 0] = TI(S[0]);
                a.oS[3 * (base + rank) + 1] = TI(S[1]);
                a.oS[3 * (base + rank) + 2] = TI(S[2]);
              }
            }
          }
          nacc += __popc(mask);
        }
      }
      __syncwarp();  // first-pass writes of j are visible to the whole warp
    }

    if constexpr (!FILL) {
      if (lane == 0) a.counts[iorig - 1] = nacc;
    } else {
      if (nacc != n) {
        if (lane == 0) atomicOr(a.err, kFlagInconsistent);
      } else if (write_ok) {
        if (staged) {
          for (int e2 = lane; e2 < n; e2 += 32) {
            const int je = T.j[e2];
            int rank = 0;
            for (int l = 0; l < n; ++l) {
              const int j2 = T.j[l];
              rank += (j2 < je) | ((j2 == je) & (l < e2));
            }
            a.oj[base + rank] = TI(je);
            a.oS[3 * (base + rank) + 0] = TI(T.S[0][e2]);
            a.oS[3 * (base + rank) + 1] = TI(T.S[1][e2]);
            a.oS[3 * (base + rank) + 2] = TI(T.S[2][e2]);
          }
        }
        for (int e2 = lane; e2 < n; e2 += 32) a.oi[base + e2] = iorig;
      }
      __syncwarp();
    }
  }
  rechecks = __reduce_add_sync(0xffffffffu, unsigned(rechecks));
  if (lane == 0 && rechecks) atomicAdd(a.stats, rechecks);
}

}  // namespace

void launch_legacy_fix(const double* inv, const double* C, const int* pbc, const double* X, double* Xout, int nat,
                       unsigned long long* minmax, unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  FixGeo fg;
  std::memcpy(fg.inv, inv, sizeof(fg.inv));
  std::memcpy(fg.C, C, sizeof(fg.C));
  for (int k = 0; k < 3; ++k) fg.pbc[k] = pbc[k];
  k_legacy_fix<<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(fg, X, Xout, nat, minmax, err);
}

void launch_legacy_shift(double* X, int nat, const double* t, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  const long long n3 = 3LL * nat;
  k_legacy_shift<<<grid_for(n3, 256, num_sms * 8), 256, 0, st>>>(X, n3, t[0], t[1], t[2]);
}

template <typename TI>
void launch_legacy_prepare(const LegacyArgs<TI>& a, int num_sms, cudaStream_t st) {
  if (a.g.nat <= 0) return;
  k_legacy_prepare<TI><<<grid_for(a.g.nat, 256, num_sms * 8), 256, 0, st>>>(a);
}

template <typename TI>
void launch_legacy_pairs(bool fill, const LegacyArgs<TI>& a, int num_sms, cudaStream_t st) {
  if (a.g.nat <= 0) return;
  const int bps = a.blocks_per_sm > 0 ? a.blocks_per_sm : 4;
  const int grid = grid_for(a.g.nat, kLegacyWarps, num_sms * bps);
  if (fill)
    k_legacy_pairs<TI, true><<<grid, kLegacyWarps * 32, 0, st>>>(a);
  else
    k_legacy_pairs<TI, false><<<grid, kLegacyWarps * 32, 0, st>>>(a);
}

#define NL_INST(TI)                                                                          \
  template void launch_legacy_prepare<TI>(const LegacyArgs<TI>&, int, cudaStream_t);         \
  template void launch_legacy_pairs<TI>(bool, const LegacyArgs<TI>&, int, cudaStream_t);
NL_INST(int32_t)
NL_INST(int64_t)
#undef NL_INST

}  // namespace nl
