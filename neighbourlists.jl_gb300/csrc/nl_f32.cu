// Single-precision path: the reference with T = Float32.
//
//   position_to_cell_index (cell_list.jl:66-74)     bin32 / k_bin32 / k_prepare32
//   _for_each_neighbor_pair (gpu_kernels.jl:58-101) k_pairs32 (count and fill)
//
// The sort (scan, scatter, stable fix-up) is the double-precision path's
// (nl_build.cu, instantiated for float positions).  Every floating-point
// operation is an explicit round-to-nearest FP32 intrinsic, so nvcc cannot
// contract a product and a sum into one FMA: the reference rounds each
// operation separately.  No screen band is needed: the distance test itself
// is the reference's FP32 arithmetic, and FP32 is the fast pipe.
#include "nl_f32.cuh"
#include "nl_pairs.cuh"

namespace nl {

namespace {

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

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// frac_k = (inv' x)_k, StaticArrays order (a1*b1 + a2*b2) + a3*b3
__device__ __forceinline__ float frac32(const float* inv, float x0, float x1, float x2, int k) {
  return fadd(fadd(fmul(inv[3 * k + 0], x0), fmul(inv[3 * k + 1], x1)), fmul(inv[3 * k + 2], x2));
}

// (C' S)_k with S converted to Float32, as the reference promotes Int * Float32
__device__ __forceinline__ float cts32(const float* C, int s0, int s1, int s2, int k) {
  return fadd(fadd(fmul(C[3 * k + 0], float(s0)), fmul(C[3 * k + 1], float(s1))), fmul(C[3 * k + 2], float(s2)));
}

// c0 = floor(frac * n + 1) in Float32, then wrap / clamp with the winding.
// false: a position that cannot be binned (non-finite, |frac * n| >= 2^30,
// or a winding beyond the record's 10-bit field).
__device__ __forceinline__ bool bin32(const Geo32& g, float x0, float x1, float x2, int c[3], int w[3]) {
  bool ok = isfinite(x0) && isfinite(x1) && isfinite(x2);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float y = fmul(frac32(g.inv, x0, x1, x2, k), float(g.ns[k]));
    float yp = fadd(y, 1.0f);
    if (!(fabsf(yp) < 1073741824.0f)) {
      ok = false;
      yp = 1.0f;
    }
    int s;
    c[k] = wrap_shift(int(floorf(yp)), g.ns[k], g.pbc[k], s);
    if (s < -(kW32Bias - 1) || s > kW32Bias - 1) {
      ok = false;
      s = 0;
    }
    w[k] = s;
  }
  return ok;
}

__device__ __forceinline__ float4 record32(float x0, float x1, float x2, const int w[3]) {
  return make_float4(x0, x1, x2, __uint_as_float(pack10(w[0] + kW32Bias, w[1] + kW32Bias, w[2] + kW32Bias)));
}

// One thread per atom (original order): cell id, ticket, record, histogram
// (the same outputs as the double-precision binning).
__global__ void __launch_bounds__(256) k_bin32(Geo32 g, const float* __restrict__ X, int nat, int* __restrict__ cid,
                                               int* __restrict__ ticket, float4* __restrict__ rec,
                                               int* __restrict__ cell_count, unsigned* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nat; base += stride) {
    const long long i = base + lane;
    const bool valid = i < nat;
    int c = 0;
    if (valid) {
      const float x0 = X[3 * i + 0], x1 = X[3 * i + 1], x2 = X[3 * i + 2];
      int cc[3], w[3];
      if (!bin32(g, x0, x1, x2, cc, w)) atomicOr(err, kFlagBadPosition);
      c = (cc[0] - 1) + g.ns[0] * ((cc[1] - 1) + g.ns[1] * (cc[2] - 1));
      rec[i] = record32(x0, x1, x2, w);
      cid[i] = c;
    }
    const int key = valid ? c : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int b = 0;
    if (valid && lane == leader) b = atomicAdd(&cell_count[c], __popc(peers));
    b = __shfl_sync(0xffffffffu, b, leader);
    if (valid) ticket[i] = b + __popc(peers & lanemask_lt());
  }
}

template <typename TI>
__global__ void __launch_bounds__(256) k_prepare32(Geo32 g, const float* __restrict__ Xs,
                                                   const TI* __restrict__ cell_id, const TI* __restrict__ perm, int nat,
                                                   float4* __restrict__ rec_sorted, int* __restrict__ scell,
                                                   unsigned* __restrict__ err) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nat; s += (long long)gridDim.x * blockDim.x) {
    const float x0 = Xs[3 * s + 0], x1 = Xs[3 * s + 1], x2 = Xs[3 * s + 2];
    int cc[3], w[3];
    if (!bin32(g, x0, x1, x2, cc, w)) atomicOr(err, kFlagBadPosition);
    rec_sorted[s] = record32(x0, x1, x2, w);
    const int c = (cc[0] - 1) + g.ns[0] * ((cc[1] - 1) + g.ns[1] * (cc[2] - 1));
    scell[s] = c;
    if ((long long)cell_id[s] != (long long)c + 1) atomicOr(err, kFlagInconsistent);
    if ((long long)perm[s] < 1 || (long long)perm[s] > nat) atomicOr(err, kFlagInconsistent);
  }
}

// One thread per sorted slot (home atom i): the reference's traversal of
// _for_each_neighbor_pair -- stencil dz, dy, dx (dx fastest), each cell's
// atoms in sorted order, skipping i itself at zero cell shift -- with
// S = s_loop + wi - wj, R = (xj - xi) + C'S and dot(R, R) < cutoff^2 in FP32.
// C'S is formed once per stencil cell for wj = 0 and again for the rare
// candidates with a non-zero winding.  Count: pairs per atom.  Fill: i, j,
// S, R at first[i] in traversal order.
template <typename TI, bool FILL>
__global__ void __launch_bounds__(256) k_pairs32(Pairs32Args<TI> a) {
  const Geo32& g = a.g;
  const unsigned wzero = pack10(kW32Bias, kW32Bias, kW32Bias);
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < g.nat;
       s += (long long)gridDim.x * blockDim.x) {
    const float4 ri = a.rec[s];
    const unsigned mi = __float_as_uint(ri.w);
    const int wi0 = field10(mi, 0) - kW32Bias, wi1 = field10(mi, 1) - kW32Bias, wi2 = field10(mi, 2) - kW32Bias;
    const int c = a.scell[s];
    const int ci0 = c % g.ns[0] + 1, ci1 = (c / g.ns[0]) % g.ns[1] + 1, ci2 = c / (g.ns[0] * g.ns[1]) + 1;
    const TI iorig = a.perm[s];
    long long pos = 0, end = 0;
    bool write_ok = false;
    int count = 0;
    if constexpr (FILL) {
      pos = (long long)a.first[iorig - 1] - 1;
      end = (long long)a.first[iorig] - 1;
      write_ok = pos >= 0 && end >= pos && end <= a.capacity;
      if (!write_ok) atomicOr(a.err, kFlagCapacity);
    }
    for (int dz = -g.nxyz[2]; dz <= g.nxyz[2]; ++dz) {
      if (!g.pbc[2] && (ci2 + dz < 1 || ci2 + dz > g.ns[2])) continue;
      int sz;
      const int cz = wrap_shift(ci2 + dz, g.ns[2], g.pbc[2], sz);
      for (int dy = -g.nxyz[1]; dy <= g.nxyz[1]; ++dy) {
        if (!g.pbc[1] && (ci1 + dy < 1 || ci1 + dy > g.ns[1])) continue;
        int sy;
        const int cy = wrap_shift(ci1 + dy, g.ns[1], g.pbc[1], sy);
        for (int dx = -g.nxyz[0]; dx <= g.nxyz[0]; ++dx) {
          if (!g.pbc[0] && (ci0 + dx < 1 || ci0 + dx > g.ns[0])) continue;
          int sx;
          const int cx = wrap_shift(ci0 + dx, g.ns[0], g.pbc[0], sx);
          const int lin = (cx - 1) + g.ns[0] * ((cy - 1) + g.ns[1] * (cz - 1));
          const long long beg = (long long)a.cell_offsets[lin] - 1, fin = (long long)a.cell_offsets[lin + 1] - 1;
          if (beg >= fin) continue;
          const int Sb0 = sx + wi0, Sb1 = sy + wi1, Sb2 = sz + wi2;
          const float cb0 = cts32(g.C, Sb0, Sb1, Sb2, 0);
          const float cb1 = cts32(g.C, Sb0, Sb1, Sb2, 1);
          const float cb2 = cts32(g.C, Sb0, Sb1, Sb2, 2);
          const bool zero_loop = (sx | sy | sz) == 0;
          for (long long idx = beg; idx < fin; ++idx) {
            if (zero_loop && idx == s) continue;
            const float4 rj = a.rec[idx];
            const unsigned mj = __float_as_uint(rj.w);
            int S0 = Sb0, S1 = Sb1, S2 = Sb2;
            float e0 = cb0, e1 = cb1, e2 = cb2;
            if ((mj & kMetaFields) != wzero) {
              S0 -= field10(mj, 0) - kW32Bias;
              S1 -= field10(mj, 1) - kW32Bias;
              S2 -= field10(mj, 2) - kW32Bias;
              e0 = cts32(g.C, S0, S1, S2, 0);
              e1 = cts32(g.C, S0, S1, S2, 1);
              e2 = cts32(g.C, S0, S1, S2, 2);
            }
            const float R0 = fadd(fsub(rj.x, ri.x), e0);
            const float R1 = fadd(fsub(rj.y, ri.y), e1);
            const float R2 = fadd(fsub(rj.z, ri.z), e2);
            const float r2 = fadd(fadd(fmul(R0, R0), fmul(R1, R1)), fmul(R2, R2));
            if (r2 < g.cutoff_sq) {
              if constexpr (FILL) {
                if (write_ok && pos < end) {
                  a.oi[pos] = iorig;
                  a.oj[pos] = a.perm[idx];
                  a.oS[3 * pos + 0] = TI(S0);
                  a.oS[3 * pos + 1] = TI(S1);
                  a.oS[3 * pos + 2] = TI(S2);
                  if (a.oR) {
                    a.oR[3 * pos + 0] = R0;
                    a.oR[3 * pos + 1] = R1;
                    a.oR[3 * pos + 2] = R2;
                  }
                }
                ++pos;
              } else {
                ++count;
              }
            }
          }
        }
      }
    }
    if constexpr (FILL) {
      if (write_ok && pos != end) atomicOr(a.err, kFlagInconsistent);
    } else {
      a.counts[iorig - 1] = count;
    }
  }
}

}  // namespace

void launch_bin32(const Geo32& g, const float* X, int nat, int* cid, int* ticket, float4* rec, int* cell_count,
                  unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  k_bin32<<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, X, nat, cid, ticket, rec, cell_count, err);
}

template <typename TI>
void launch_prepare32(const Geo32& g, const float* Xs, const TI* cell_id, const TI* perm, int nat, float4* rec_sorted,
                      int* scell, unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  k_prepare32<TI><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, Xs, cell_id, perm, nat, rec_sorted, scell, err);
}

template <typename TI>
void launch_pairs32(bool fill, const Pairs32Args<TI>& a, int num_sms, cudaStream_t st) {
  if (a.g.nat <= 0) return;
  const int grid = grid_for(a.g.nat, 128, num_sms * 16);
  if (fill)
    k_pairs32<TI, true><<<grid, 128, 0, st>>>(a);
  else
    k_pairs32<TI, false><<<grid, 128, 0, st>>>(a);
}

#define NL_INST(TI)                                                                                                 \
  template void launch_prepare32<TI>(const Geo32&, const float*, const TI*, const TI*, int, float4*, int*,         \
                                     unsigned*, int, cudaStream_t);                                                \
  template void launch_pairs32<TI>(bool, const Pairs32Args<TI>&, int, cudaStream_t);
NL_INST(int32_t)
NL_INST(int64_t)
#undef NL_INST

}  // namespace nl
