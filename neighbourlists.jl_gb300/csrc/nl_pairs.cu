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
// home atoms against them: each lane loads one candidate and tests it against
// kGroup home atoms at once.
//
// Precision: the screen runs in FP32 on cell-local offsets.  Geometry.lo/hi
// bracket cutoff^2 by a band that provably exceeds the FP32 error (host-side
// screen_band in nl_api.cu); only candidates inside the band, or involving an
// "exact" atom, are decided in FP64 with the reference arithmetic
// R = (xj - xi) + C'S, r2 = dot(R,R), r2 < cutoff^2.  The accepted pair set is
// therefore identical to the reference's.
//
// Output order: candidates are visited in the reference's order (stencil
// dz, dy, dx with dx fastest, then sorted order inside a cell) and compacted
// with ballots that preserve lane order, so each atom's pairs come out in the
// reference's order, and R is computed with the reference's operations, so
// i, j, S, R and first are bit-identical to the reference's arrays.
#include <type_traits>

#include "nl_pairs.cuh"

namespace nl {

#ifndef NL_PAIR_MIN_BLOCKS
#define NL_PAIR_MIN_BLOCKS 7
#endif
#ifndef NL_PAIR_BATCH_MIN_BLOCKS
#define NL_PAIR_BATCH_MIN_BLOCKS NL_PAIR_MIN_BLOCKS  // the batch variant (per-system view in registers)
#endif
#ifndef NL_PAIR_GROUP
#define NL_PAIR_GROUP 2
#endif
#ifndef NL_PAIR_CHUNK
#define NL_PAIR_CHUNK 192
#endif
#ifndef NL_STAGE_UNROLL
#define NL_STAGE_UNROLL 2
#endif
constexpr int kPairWarps = 4;                    // warps per block
constexpr int kMinBlocks = NL_PAIR_MIN_BLOCKS;   // resident blocks per SM the register budget targets
constexpr int kChunk = NL_PAIR_CHUNK;            // staged candidates per warp and pass
constexpr int kGroup = NL_PAIR_GROUP;            // home atoms screened per candidate load
constexpr int kStageUnroll = NL_STAGE_UNROLL;    // staging iterations interleaved (loads in flight)
constexpr int kRing = 64;       // pair queue (ring) per warp
constexpr int kCsR = 2;         // C'S table covers |S_k| <= kCsR
constexpr int kCsN = 2 * kCsR + 1;
constexpr unsigned kExactBit = kMetaExact;

struct __align__(16) WarpSmem {
  float4 cv[kChunk];        // candidate: (x, y, z) relative to home corner; w = packed S base | exact bit
  int cslot[kChunk];        // candidate: sorted slot
  int corig[kChunk];        // candidate: original index within its system (half lists)
  double hx[32][3];         // home batch: FP64 positions
  long long hnext[32];      // home batch: next output slot (fill) / running count (count)
  double hacc[32];          // home batch: lazy accumulators
  long long rslot[kRing];   // queue: output slot
  int rent[kRing];          // queue: (home atom << 16) | candidate
  double rval[32];          // queue: lazy values
  int horig[32];            // home batch: original index (0-based)
  unsigned hmeta[32];       // home batch: packed windings | exact bit
  float box[6];             // home batch: bounding box (x lo/hi, y lo/hi, z lo/hi) of the FP32 records
  int prune;                // home batch: the box may prune candidates (no exact home atom)
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

__device__ __forceinline__ unsigned pack3(int a, int b, int c) {
  return (unsigned(a) & 0xFFu) | ((unsigned(b) & 0xFFu) << 8) | ((unsigned(c) & 0xFFu) << 16);
}
__device__ __forceinline__ int unpack3(unsigned p, int k) { return int(int8_t((p >> (8 * k)) & 0xFFu)); }

// RN(d + z) where z is +-0: d itself unless d is a zero, in which case the
// IEEE sum of two zeros is -0 only if both are -0.  Integer operations only.
__device__ __forceinline__ double add_signed_zero(double d, double z) {
  const long long bd = __double_as_longlong(d);
  return (bd << 1) != 0 ? d : __longlong_as_double(bd & __double_as_longlong(z));
}

// L2 residency of the 32-byte gather rows (XPack): the write pass gathers
// each row ~26 times from anywhere in the array while it streams the masks
// and headers in and the pair arrays out, so the gathers load with an
// evict-last L2 policy and the read-once data with evict-first (cache-
// streaming) loads.  At 1M atoms this took the write pass's DRAM reads from
// 724 to 585 MB per launch (NL_L2_HINTS=0 builds plain loads).  Storing the
// rows with the same policy in the count pass slowed the count pass down.
#ifndef NL_L2_HINTS
#define NL_L2_HINTS 1
#endif
#ifndef NL_L2_HINTS_STORE
#define NL_L2_HINTS_STORE 0  // 1: the count pass stores the rows with the same policy (slower count pass)
#endif
__device__ __forceinline__ unsigned long long l2_keep_policy() {
  unsigned long long p = 0;
#if NL_L2_HINTS
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
#endif
  return p;
}
__device__ __forceinline__ double2 ld_keep(const double2* ptr, unsigned long long pol) {
#if NL_L2_HINTS
  double2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(ptr), "l"(pol));
  return v;
#else
  return __ldg(ptr);
#endif
}
__device__ __forceinline__ int4 ld_keep(const int4* ptr, unsigned long long pol) {
#if NL_L2_HINTS
  int4 v;
  asm("ld.global.nc.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(ptr), "l"(pol));
  return v;
#else
  return __ldg(ptr);
#endif
}
__device__ __forceinline__ void st_keep(XPack* dst, const XPack& v, unsigned long long pol) {
#if NL_L2_HINTS && NL_L2_HINTS_STORE
  double2* d = reinterpret_cast<double2*>(dst);
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(d), "d"(v.x), "d"(v.y), "l"(pol));
  asm volatile("st.global.L2::cache_hint.v4.s32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(d + 1),
               "r"(__double2loint(v.z)), "r"(__double2hiint(v.z)), "r"(v.perm), "r"(int(v.meta)), "l"(pol));
#else
  *dst = v;
#endif
}
// A whole 32-byte gather row (32-byte aligned) in one 256-bit load, with the
// evict-last policy (NL_ROW_V4=0: two 16-byte loads)
#ifndef NL_ROW_V4
#define NL_ROW_V4 1
#endif
__device__ __forceinline__ void ld_row(const XPack* ptr, unsigned long long pol, double2& w0, int4& w1) {
#if NL_ROW_V4 && NL_L2_HINTS
  unsigned long long a, b, c, d;
  asm("ld.global.nc.L2::cache_hint.v4.u64 {%0, %1, %2, %3}, [%4], %5;"
      : "=l"(a), "=l"(b), "=l"(c), "=l"(d)
      : "l"(ptr), "l"(pol));
  w0 = make_double2(__longlong_as_double((long long)a), __longlong_as_double((long long)b));
  w1 = make_int4(int(unsigned(c)), int(unsigned(c >> 32)), int(unsigned(d)), int(unsigned(d >> 32)));
#else
  w0 = ld_keep(reinterpret_cast<const double2*>(ptr), pol);
  w1 = ld_keep(reinterpret_cast<const int4*>(ptr) + 1, pol);
#endif
}
// read-once data: evict first from L1 and L2
template <typename T>
__device__ __forceinline__ T ld_stream(const T* ptr) {
#if NL_L2_HINTS
  return __ldcs(ptr);
#else
  return __ldg(ptr);
#endif
}

// R = (xj - xi) + C'S with the reference's operation order.  The three sums
// with C'S are only issued when the warp holds a pair with S != 0 (for S == 0
// C'S is a vector of signed zeros and the sum is exact, see add_signed_zero).
__device__ __forceinline__ void pair_R(const Geometry& g, const double* cs_tab, const double* xi, const double* xj,
                                       int S0, int S1, int S2, bool active, double* R) {
  R[0] = dsub(xj[0], xi[0]);
  R[1] = dsub(xj[1], xi[1]);
  R[2] = dsub(xj[2], xi[2]);
  const bool nz = active && (S0 | S1 | S2) != 0;
  if (__any_sync(0xffffffffu, nz)) {
    if (nz) {
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
      R[0] = dadd(R[0], c0);
      R[1] = dadd(R[1], c1);
      R[2] = dadd(R[2], c2);
    }
  }
  if (!nz) {
    const double* z = cs_tab + 3 * ((kCsN * kCsN + kCsN + 1) * kCsR);  // C'(0,0,0): signed zeros
    R[0] = add_signed_zero(R[0], z[0]);
    R[1] = add_signed_zero(R[1], z[1]);
    R[2] = add_signed_zero(R[2], z[2]);
  }
}

__device__ __forceinline__ double dot_ref(const double* R) {
  return dadd(dadd(dmul(R[0], R[0]), dmul(R[1], R[1])), dmul(R[2], R[2]));
}

// The candidate word of stencil cell q: 10-bit fields s_loop + 640.  With
// the record's meta (fields wj + 128) the packed difference
//   cw = cand_base(q) - (meta_j & kMetaFields)   (no borrow between fields)
// holds s_loop - wj + 512 per field; for an exact candidate (whose meta
// windings are zero) it holds s_loop + 512, and the exact bit is or-ed in.
__device__ __forceinline__ unsigned cand_base(int s0, int s1, int s2) { return pack10(s0 + 640, s1 + 640, s2 + 640); }
__device__ __forceinline__ unsigned cand_word(unsigned base, unsigned mj) {
  return (base - (mj & kMetaFields)) | (mj & kMetaExact);
}

// S = s_loop + wi - wj (gpu_kernels.jl:88) from a candidate word.  Exact pairs
// recompute both windings in FP64.
__device__ __forceinline__ void pair_S(const Geometry& g, const double* xi, const double* xj, unsigned mi, unsigned cw,
                                       int* S) {
  if (!((mi | cw) & kExactBit)) {
#pragma unroll
    for (int k = 0; k < 3; ++k) S[k] = field10(cw, k) + field10(mi, k) - 640;
  } else {
    Binned bi, bj;
    bin_position(g, xi[0], xi[1], xi[2], bi);
    bin_position(g, xj[0], xj[1], xj[2], bj);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int sl = (cw & kExactBit) ? field10(cw, k) - 512 : field10(cw, k) - 512 + bj.w[k];
      S[k] = sl + bi.w[k] - bj.w[k];
    }
  }
}

// The candidate is the home atom itself with zero loop shift (the reference
// skips i == j && s_loop == 0, gpu_kernels.jl:82); the same atom seen through
// a periodic image is a neighbour.  s_loop comes back from the candidate word:
// its fields hold s_loop - w_j + 512 (w_j = w_i here) or, for an exact atom,
// s_loop + 512.
__device__ __forceinline__ bool is_self(int cand_slot, int home_slot, unsigned cw, unsigned mi) {
  if (cand_slot != home_slot) return false;
  const bool ex = (cw & kMetaExact) != 0;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (field10(cw, k) - 512 + (ex ? 0 : field10(mi, k) - 128) != 0) return false;
  return true;
}

// Half lists keep (i, j, S) when j > i, or j == i (a periodic image of the
// atom itself) and S > 0 lexicographically; of the two directions of every
// accepted pair exactly one is kept.  For j == i, S is the loop shift.
__device__ __forceinline__ bool half_keep(int oi, int oj, unsigned cw, unsigned mi) {
  if (oj != oi) return oj > oi;
  const bool ex = (cw & kMetaExact) != 0;
  int s[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) s[k] = field10(cw, k) - 512 + (ex ? 0 : field10(mi, k) - 128);
  return s[0] > 0 || (s[0] == 0 && (s[1] > 0 || (s[1] == 0 && s[2] > 0)));
}

// Full FP64 decision of one candidate pair with the reference arithmetic.
__device__ __forceinline__ bool exact_pair(const Geometry& g, const double* Xs, int slot_i, int slot_j, unsigned mi,
                                           unsigned cw) {
  double xi[3], xj[3];
  xi[0] = Xs[3LL * slot_i + 0];
  xi[1] = Xs[3LL * slot_i + 1];
  xi[2] = Xs[3LL * slot_i + 2];
  xj[0] = Xs[3LL * slot_j + 0];
  xj[1] = Xs[3LL * slot_j + 1];
  xj[2] = Xs[3LL * slot_j + 2];
  int S[3];
  pair_S(g, xi, xj, mi, cw, S);
  double R[3];
  R[0] = dadd(dsub(xj[0], xi[0]), cts_k(g.C, S[0], S[1], S[2], 0));
  R[1] = dadd(dsub(xj[1], xi[1]), cts_k(g.C, S[0], S[1], S[2], 1));
  R[2] = dadd(dsub(xj[2], xi[2]), cts_k(g.C, S[0], S[1], S[2], 2));
  return dot_ref(R) < g.cutoff_sq;
}

// Processes n <= 32 queued pairs starting at ring position head.
template <typename TI, int MODE>
__device__ __forceinline__ void flush_ring(const PairArgs<TI>& A, const Geometry& g, const double* cs_tab, WarpSmem& W,
                                           int head, int n, int lane) {
  const bool act = lane < n;
  const int rp = (head + lane) & (kRing - 1);
  const int e = act ? W.rent[rp] : 0;
  const int a = e >> 16, f = e & 0xFFFF;
  const int slot_j = W.cslot[f];
  const unsigned cw = __float_as_uint(W.cv[f].w), mi = W.hmeta[a];
  double xj[3];
  const double* xi = W.hx[a];
  int S[3] = {0, 0, 0};
  if (act) {
    xj[0] = A.Xs[3LL * slot_j + 0];
    xj[1] = A.Xs[3LL * slot_j + 1];
    xj[2] = A.Xs[3LL * slot_j + 2];
    pair_S(g, xi, xj, mi, cw, S);
  } else {
    xj[0] = xj[1] = xj[2] = 0.0;
  }
  if (MODE == kModeFill) {
    const long long out = act ? W.rslot[rp] : 0;
    const bool wr = act && out < A.capacity;
    if (act && !wr) atomicOr(A.err, kFlagCapacity);
    if (wr) {
      A.oi[out] = TI(W.horig[a]) + 1;
      A.oj[out] = TI(clampi(A.perm[slot_j] - 1, g.nat - 1)) + 1;
      A.oS[3 * out + 0] = TI(S[0]);
      A.oS[3 * out + 1] = TI(S[1]);
      A.oS[3 * out + 2] = TI(S[2]);
    }
    if (A.oR) {
      double R[3];
      pair_R(g, cs_tab, xi, xj, S[0], S[1], S[2], act, R);
      if (wr) {
        A.oR[3 * out + 0] = R[0];
        A.oR[3 * out + 1] = R[1];
        A.oR[3 * out + 2] = R[2];
      }
    }
  } else {  // lazy: f(R) = 1 / ((r2*r2)*r2)
    double R[3];
    pair_R(g, cs_tab, xi, xj, S[0], S[1], S[2], act, R);
    if (act) {
      const double r2 = dot_ref(R);
      W.rval[lane] = __ddiv_rn(1.0, dmul(dmul(r2, r2), r2));
    }
    __syncwarp();
    // accumulate in queue order: every atom's sum follows the reference's
    // traversal order exactly
    if (lane == 0)
      for (int q = 0; q < n; ++q) {
        const int aa = W.rent[(head + q) & (kRing - 1)] >> 16;
        W.hacc[aa] = dadd(W.hacc[aa], W.rval[q]);
      }
  }
  __syncwarp();
}

// C'S for |S_k| <= kCsR with the reference's operation order, built once per
// call (one block) and read by the fill / emit / lazy kernels.
__global__ void k_cs_table(Geometry g, double* __restrict__ out, const int* __restrict__ cap_rec, int list_cap,
                           unsigned* __restrict__ err) {
  // the write pass must use the lists the count pass made (same workspace size)
  if (threadIdx.x == 0 && cap_rec && *cap_rec != list_cap) atomicOr(err, kFlagInconsistent);
  for (int t = threadIdx.x; t < kCsN * kCsN * kCsN; t += blockDim.x) {
    const int s0 = t % kCsN - kCsR, s1 = (t / kCsN) % kCsN - kCsR, s2 = t / (kCsN * kCsN) - kCsR;
    out[3 * t + 0] = cts_k(g.C, s0, s1, s2, 0);
    out[3 * t + 1] = cts_k(g.C, s0, s1, s2, 1);
    out[3 * t + 2] = cts_k(g.C, s0, s1, s2, 2);
  }
}

// Batches: one block per system.
__global__ void k_cs_tables(const Geometry* __restrict__ geo, double* __restrict__ out) {
  const Geometry& g = geo[blockIdx.x];
  double* o = out + 3 * kCsN * kCsN * kCsN * (long long)blockIdx.x;
  for (int t = threadIdx.x; t < kCsN * kCsN * kCsN; t += blockDim.x) {
    const int s0 = t % kCsN - kCsR, s1 = (t / kCsN) % kCsN - kCsR, s2 = t / (kCsN * kCsN) - kCsR;
    o[3 * t + 0] = cts_k(g.C, s0, s1, s2, 0);
    o[3 * t + 1] = cts_k(g.C, s0, s1, s2, 1);
    o[3 * t + 2] = cts_k(g.C, s0, s1, s2, 2);
  }
}

// wrap_shift without a division for the common case of an index already
// inside [1, n]
__device__ __forceinline__ int wrap_shift_fast(int i, int n, int pbc, int& s) {
  if (i >= 1 && i <= n) {
    s = 0;
    return i;
  }
  return wrap_shift(i, n, pbc, s);
}

constexpr int kStencilTab = 512;  // stencil offsets tabulated per block up to this size

// Stencil cell q of home cell (hc0, hc1, hc2): its 0-based linear index (or
// -1 when it falls outside an open axis), packed loop shift and FP32 offset
// d.b of its lower corner from the home corner.
__device__ __forceinline__ int stencil_cell(const Geometry& g, const unsigned* dtab, int tabn, int sx, int sy, int hc0,
                                            int hc1, int hc2, int q, unsigned& slp, float& ox, float& oy, float& oz) {
  int d0, d1, d2;
  if (q < tabn) {
    const unsigned dq = dtab[q];
    d0 = unpack3(dq, 0);
    d1 = unpack3(dq, 1);
    d2 = unpack3(dq, 2);
  } else {
    d0 = q % sx - g.nxyz[0];
    d1 = (q / sx) % sy - g.nxyz[1];
    d2 = q / (sx * sy) - g.nxyz[2];
  }
  const bool inb = (g.pbc[0] || (hc0 + d0 >= 1 && hc0 + d0 <= g.ns[0])) &&
                   (g.pbc[1] || (hc1 + d1 >= 1 && hc1 + d1 <= g.ns[1])) &&
                   (g.pbc[2] || (hc2 + d2 >= 1 && hc2 + d2 <= g.ns[2]));
  if (!inb) return -1;
  int s0, s1, s2;
  const int c0 = wrap_shift_fast(hc0 + d0, g.ns[0], g.pbc[0], s0);
  const int c1 = wrap_shift_fast(hc1 + d1, g.ns[1], g.pbc[1], s1);
  const int c2 = wrap_shift_fast(hc2 + d2, g.ns[2], g.pbc[2], s2);
  slp = cand_base(s0, s1, s2);  // |s| <= 63: the host limits nxyz to 62
  const float fd0 = float(d0), fd1 = float(d1), fd2 = float(d2);
  ox = fmaf(fd2, g.b[6], fmaf(fd1, g.b[3], fd0 * g.b[0]));
  oy = fmaf(fd2, g.b[7], fmaf(fd1, g.b[4], fd0 * g.b[1]));
  oz = fmaf(fd2, g.b[8], fmaf(fd1, g.b[5], fd0 * g.b[2]));
  return linear_cell(g, c0, c1, c2);
}

// Per-warp view of the system that owns a home cell (batches: every warp
// copies its current system's geometry and stencil table to shared memory).
template <bool BATCH>
struct SysView {
  int s = 0;      // system index
  int abase = 0;  // first global slot / original atom of the system
  int coff = 0;   // index of the system's cell 0 in cell_offsets
  int hl = 0;     // home cell within the system
};

template <typename TI, bool BATCH>
__device__ __forceinline__ void load_system(const PairArgs<TI>& A, int s, Geometry& gw, unsigned* wtab, int lane) {
  __syncwarp();
  const int* src = reinterpret_cast<const int*>(A.geo + s);
  int* dst = reinterpret_cast<int*>(&gw);
  for (int k = lane; k < int(sizeof(Geometry) / 4); k += 32) dst[k] = src[k];
  __syncwarp();
  const int sx = 2 * gw.nxyz[0] + 1, sy = 2 * gw.nxyz[1] + 1, sz = 2 * gw.nxyz[2] + 1;
  if (lane < sx * sy * sz)
    wtab[lane] = pack3(lane % sx - gw.nxyz[0], (lane / sx) % sy - gw.nxyz[1], lane / (sx * sy) - gw.nxyz[2]);
  __syncwarp();
}

#ifndef NL_BATCH_RUN
#define NL_BATCH_RUN 1
#endif
constexpr int kBatchRun = NL_BATCH_RUN;  // consecutive cells a warp takes per counter increment (batches)

template <typename TI, int MODE, bool BATCH>
__global__ void __launch_bounds__(kPairWarps * 32, BATCH ? NL_PAIR_BATCH_MIN_BLOCKS : kMinBlocks)
    k_pairs(PairArgs<TI> A) {
  if ((MODE == kModeCount || MODE == kModeLazyR6) && !BATCH && (A.sym || A.sym_gate) && *A.sym_fail == 0)
    return;  // the symmetric pass counted (or summed)
  // the screening passes visit only listed cells: none listed, nothing to do
  // (the same value for every thread, so no block stops at a barrier alone)
  if ((MODE == kModeFill || (MODE == kModeLazyR6 && A.list_cap > 0)) && *A.n_screen_cells <= 0) return;
  __shared__ WarpSmem sm[kPairWarps];
  __shared__ double cs_blk[BATCH ? 1 : 3 * kCsN * kCsN * kCsN];
  __shared__ unsigned dtab_blk[BATCH ? 32 * kPairWarps : kStencilTab];  // packed (d0, d1, d2) of stencil cell q
  __shared__ Geometry geo_w[BATCH ? kPairWarps : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Geometry& g = BATCH ? geo_w[warp] : A.g;
  const unsigned* dtab = BATCH ? dtab_blk + 32 * warp : dtab_blk;
  constexpr int tabn = BATCH ? 32 : kStencilTab;
  if (!BATCH) {
    if (MODE != kModeCount)
      for (int t = threadIdx.x; t < 3 * kCsN * kCsN * kCsN; t += blockDim.x) cs_blk[t] = A.cs_table[t];
    const int tx = 2 * g.nxyz[0] + 1, ty = 2 * g.nxyz[1] + 1;
    const int tn = min(kStencilTab, tx * ty * (2 * g.nxyz[2] + 1));
    for (int t = threadIdx.x; t < tn; t += blockDim.x)
      dtab_blk[t] = pack3(t % tx - g.nxyz[0], (t / tx) % ty - g.nxyz[1], t / (tx * ty) - g.nxyz[2]);
    __syncthreads();
  }
  const double* cs_tab = cs_blk;

  WarpSmem& W = sm[warp];
  const int nwarps = gridDim.x * kPairWarps;
  int sx = 0, sy = 0, nst = 0, center = 0;
  float lo = 0.f, hi = 0.f;
  auto set_stencil = [&]() {
    sx = 2 * g.nxyz[0] + 1;
    sy = 2 * g.nxyz[1] + 1;
    nst = sx * sy * (2 * g.nxyz[2] + 1);
    center = g.nxyz[0] + sx * (g.nxyz[1] + sy * g.nxyz[2]);
    lo = g.lo;
    hi = g.hi;
  };
  if (!BATCH) set_stencil();
  int cur_sys = -1;
  unsigned rechecks = 0;
  const int list_cap = MODE == kModeCount ? A.list_cap : 0;
  if (MODE == kModeCount && A.cap_rec && blockIdx.x == 0 && threadIdx.x == 0) *A.cap_rec = list_cap;

  // Single systems prefetch the ranges of the next cell one cell ahead: its
  // home range and, per lane, the range of its stencil cell in the first
  // group of 32.
  // The fill pass visits only the cells whose pairs the count pass could not list
  // (k_emit writes the others); count and lazy visit every cell.
  // (so does the lazy pass when the per-atom lists cover the other cells)
  const bool listed = MODE == kModeFill || (MODE == kModeLazyR6 && A.list_cap > 0);
  // a batch's count pass after the symmetric one: only the cells of the
  // systems it did not take or that failed it
  const bool nonsym = BATCH && MODE == kModeCount && A.sym && A.nonsym_cells;
  // ... in rounds of 32 home atoms, so that a cell of many atoms (a small
  // system's only cell, a crowded one) does not hold one warp alone
  const bool split = nonsym && A.rounds;
  const bool rpass = split && A.round_pass;
  const int rcap = A.nat_total / 32 + 2;  // rounds the list holds
  const int ncell_iter = listed   ? min(*A.n_screen_cells, A.ncells_total)
                         : rpass  ? min(*A.n_rounds, rcap)
                         : nonsym ? min(A.n_nonsym_cells + *A.extra_cells, A.ncells_total)
                                  : A.ncells_total;
  auto cell_at = [&](int idx) {
    return listed ? clampi(A.screen_cells[idx], A.ncells_total - 1)
           : rpass  ? clampi(A.rounds[idx].x, A.ncells_total - 1)
           : nonsym ? clampi(A.nonsym_cells[idx], A.ncells_total - 1)
                    : idx;
  };
  // Batches: warps take their next cell (runs of kBatchRun cells) from a
  // counter as they free up, which balances the uneven cells of a batch
  // (4.69 -> 4.33 ms per 4,096-system batch against a grid stride; runs of
  // 2, 4 and 8 consecutive cells, fewer geometry loads, were slower: 4.59,
  // 5.26, 5.65 ms).  Single systems: a grid stride.
  int* work = BATCH ? (rpass ? A.round_work : A.work + (MODE == kModeCount ? 0 : 1)) : nullptr;
  int run_left = 0;
  auto next_idx = [&](int cur) -> int {
    if (!BATCH) return cur + nwarps;
    if (run_left > 1) {
      --run_left;
      return cur + 1;
    }
    int b = 0;
    if (lane == 0) b = atomicAdd(work, kBatchRun);
    run_left = kBatchRun;
    return __shfl_sync(0xffffffffu, b, 0);
  };
  int idx = BATCH ? next_idx(0) : blockIdx.x * kPairWarps + warp;
  // (0-based slot offsets, clamped to [0, nat])
  int pf_hs = 0, pf_he = 0, pf_lo = 0, pf_hi = 0;
  auto prefetch = [&](int pidx) {
    if (BATCH || pidx >= ncell_iter) return;
    const int hh = cell_at(pidx);
    pf_hs = clampi(A.cell_offsets[hh] - 1, g.nat);
    pf_he = clampi(A.cell_offsets[hh + 1] - 1, g.nat);
    const int c0 = hh % g.ns[0] + 1, c1 = (hh / g.ns[0]) % g.ns[1] + 1, c2 = hh / (g.ns[0] * g.ns[1]) + 1;
    unsigned sl;
    float a, b, c;
    const int lin = lane < nst ? stencil_cell(g, dtab, tabn, sx, sy, c0, c1, c2, lane, sl, a, b, c) : -1;
    pf_lo = lin >= 0 ? clampi(A.cell_offsets[lin] - 1, g.nat) : 0;
    pf_hi = lin >= 0 ? clampi(A.cell_offsets[lin + 1] - 1, g.nat) : 0;
  };
  prefetch(idx);
  for (; idx < ncell_iter; idx = next_idx(idx)) {
    const int h = cell_at(idx);
    // offsets are clamped to [0, nat] so that a malformed cell list (which
    // the prepare pass reports as inconsistent) never indexes out of bounds
    int hs = pf_hs, he = pf_he;
    const int g0_lo = pf_lo, g0_hi = pf_hi;
    SysView<BATCH> sv;
    sv.hl = h;
    if constexpr (BATCH) {
      sv.s = clampi(A.cell_sys[h], A.nsys - 1);
      // systems the symmetric pass counted
      if (MODE == kModeCount && A.sym && A.sys_sym[sv.s] && !A.sys_fail[sv.s]) continue;
      if (sv.s != cur_sys) {
        load_system<TI, BATCH>(A, sv.s, geo_w[warp], dtab_blk + 32 * warp, lane);
        set_stencil();
        cur_sys = sv.s;
      }
      cs_tab = A.cs_sys + 3 * kCsN * kCsN * kCsN * (long long)sv.s;
      sv.abase = A.sys_atom[sv.s];
      sv.coff = A.sys_cell[sv.s] + sv.s;
      sv.hl = h - A.sys_cell[sv.s];
      hs = clampi(A.cell_offsets[sv.coff + sv.hl] - 1 + sv.abase, A.nat_total);
      he = clampi(A.cell_offsets[sv.coff + sv.hl + 1] - 1 + sv.abase, A.nat_total);
    }
    prefetch(idx + nwarps);  // loads in flight while this cell is processed
    if (hs >= he) continue;
    const int hl = sv.hl;
    bool overflow = false;  // count: an atom of this cell has more than list_cap pairs
    const int hc0 = hl % g.ns[0] + 1, hc1 = (hl / g.ns[0]) % g.ns[1] + 1, hc2 = hl / (g.ns[0] * g.ns[1]) + 1;
    int hb0 = hs, hb1 = he;  // the home atoms this warp takes
    if (rpass) {
      hb0 = min(hs + 32 * max(A.rounds[idx].y, 0), he);
      hb1 = min(hb0 + 32, he);
    } else if (split && he - hs > 32) {  // the first 32 here, the other rounds listed
      hb1 = hs + 32;
      const int nr = ((he - hs + 31) >> 5) - 1;
      int base = 0;
      if (lane == 0) base = atomicAdd(A.n_rounds, nr);
      base = __shfl_sync(0xffffffffu, base, 0);
      for (int k = lane; k < nr; k += 32)
        if (base + k < rcap) A.rounds[base + k] = make_int2(h, k + 1);
    }

    for (int hb = hb0; hb < hb1; hb += 32) {
      const int nb = min(32, he - hb);
      float ux = 0.f, uy = 0.f, uz = 0.f;

      int head = 0, tail = 0;  // ring queue (fill / lazy)

      for (int gb = 0; gb < nst; gb += 32) {
        // ---- stencil cell held by this lane (reference order: dx fastest)
        const int q = gb + lane;
        int cstart = 0, ccount = 0;
        unsigned slp = 0;
        float ox = 0.f, oy = 0.f, oz = 0.f;
        if (q < nst) {
          const int lin = stencil_cell(g, dtab, tabn, sx, sy, hc0, hc1, hc2, q, slp, ox, oy, oz);
          if (lin >= 0) {
            const bool pre = !BATCH && gb == 0;
            cstart = pre ? g0_lo : clampi(A.cell_offsets[sv.coff + lin] - 1 + sv.abase, A.nat_total);
            const int cend = pre ? g0_hi : clampi(A.cell_offsets[sv.coff + lin + 1] - 1 + sv.abase, A.nat_total);
            ccount = max(cend - cstart, 0);
          }
        }
        int incl = ccount;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        const int tg = __shfl_sync(0xffffffffu, incl, 31);
        for (int cb = 0; cb < tg || (gb == 0 && cb == 0); cb += kChunk) {
          const int nch = min(kChunk, tg - cb);
          if (MODE != kModeCount && tail > head) {  // queued pairs refer to the previous chunk
            flush_ring<TI, MODE>(A, g, cs_tab, W, head, tail - head, lane);
            head = tail;
          }
          __syncwarp();
          if (gb == 0 && cb == 0) {
            // home batch
            if (lane < nb) {
              const int s = hb + lane;
              const float4 r = A.rec[s];  // exact atoms carry NaN coordinates
              ux = r.x;
              uy = r.y;
              uz = r.z;
              W.hmeta[lane] = __float_as_uint(r.w);
              const int orig = clampi(A.perm[s] - 1, g.nat - 1);
              W.horig[lane] = orig;
              if (MODE != kModeCount) {
                W.hx[lane][0] = A.Xs[3LL * s + 0];
                W.hx[lane][1] = A.Xs[3LL * s + 1];
                W.hx[lane][2] = A.Xs[3LL * s + 2];
              }
              W.hnext[lane] = MODE == kModeFill ? (long long)A.first[sv.abase + orig] - 1 : 0;
              if (MODE == kModeLazyR6) W.hacc[lane] = 0.0;
            }
            // bounding box of the home batch: candidates farther than the
            // screen's reject bound from it are not staged
            {
              const float inf = __int_as_float(0x7f800000);
              const bool in = lane < nb;
              float bl[3] = {in ? ux : inf, in ? uy : inf, in ? uz : inf};
              float bh[3] = {in ? ux : -inf, in ? uy : -inf, in ? uz : -inf};
#pragma unroll
              for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                  bl[d] = fminf(bl[d], __shfl_xor_sync(0xffffffffu, bl[d], o));
                  bh[d] = fmaxf(bh[d], __shfl_xor_sync(0xffffffffu, bh[d], o));
                }
              // an exact home atom (NaN record) is tested against every candidate
              const bool pr = !__any_sync(0xffffffffu, in && (W.hmeta[lane] & kExactBit) != 0);
              if (lane == 0) {
                W.box[0] = bl[0];
                W.box[1] = bh[0];
                W.box[2] = bl[1];
                W.box[3] = bh[1];
                W.box[4] = bl[2];
                W.box[5] = bh[2];
                W.prune = pr;
              }
            }
          }
          if (nch <= 0) {
            __syncwarp();
            continue;
          }
          // ---- stage the chunk: home-relative FP32 positions, packed S base;
          // exact candidates stay NaN, padding up to whole rounds is +inf.
          // Candidates whose distance from the home batch's bounding box is
          // above the reject bound are dropped; the kept ones stay in
          // traversal order.  (The box distance is computed with the screen's
          // own operations on smaller magnitudes, so by monotonicity of
          // rounding it never exceeds any home atom's screened r2.)
          int nkeep = 0;
          __syncwarp();
          const bool prune = W.prune != 0;
#pragma unroll kStageUnroll
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
            const unsigned q_slp = __shfl_sync(0xffffffffu, slp, qq);
            const float qx = __shfl_sync(0xffffffffu, ox, qq);
            const float qy = __shfl_sync(0xffffffffu, oy, qq);
            const float qz = __shfl_sync(0xffffffffu, oz, qq);
            bool keep = false;
            float4 cv;
            int slot = 0;
            if (f < nch) {
              slot = q_start + (gf - (q_incl - q_cnt));
              const float4 r = A.rec[slot];
              const unsigned mj = __float_as_uint(r.w);
              const unsigned cw = cand_word(q_slp, mj);
              const float nan = __int_as_float(0x7fc00000);
              const bool ex = (cw & kExactBit) != 0;
              cv = make_float4(ex ? nan : r.x + qx, ex ? nan : r.y + qy, ex ? nan : r.z + qz, __uint_as_float(cw));
              const float dx = fmaxf(fmaxf(W.box[0] - cv.x, cv.x - W.box[1]), 0.f);
              const float dy = fmaxf(fmaxf(W.box[2] - cv.y, cv.y - W.box[3]), 0.f);
              const float dz = fmaxf(fmaxf(W.box[4] - cv.z, cv.z - W.box[5]), 0.f);
              const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
              keep = ex || !(prune && d2 > hi);
            }
            const unsigned km = __ballot_sync(0xffffffffu, keep);
            if (keep) {
              const int pos = nkeep + __popc(km & lt_mask());
              W.cv[pos] = cv;
              W.cslot[pos] = slot;
              if (A.half) W.corig[pos] = int(A.perm[slot]) - 1;
            }
            nkeep += __popc(km);
          }
          {
            const int pos = nkeep + lane;  // padding up to a whole round
            if (pos < ((nkeep + 31) & ~31)) {
              const float inf = __int_as_float(0x7f800000);
              W.cv[pos] = make_float4(inf, inf, inf, 0.f);
            }
          }
          __syncwarp();

          // ---- screen the home batch, kGroup atoms per candidate load.
          // A test is pure FP32: accept 0 < r2 < lo, reject r2 > hi; the rest
          // (the band, r2 == 0 which includes the self candidate, and NaN from
          // exact atoms) is resolved in the warp-uniform rare branch.
          const int nround = (nkeep + 31) & ~31;
          for (int a0 = 0; a0 < nb; a0 += kGroup) {
            float ax[kGroup], ay[kGroup], az[kGroup];
            // running pair count (count) or next output slot (fill) of each atom
            using NextT = std::conditional_t<MODE == kModeFill, long long, int>;
            NextT next[kGroup];
#pragma unroll
            for (int k = 0; k < kGroup; ++k) {
              const int a = min(a0 + k, nb - 1);
              const bool use = a0 + k < nb;
              const float inf = __int_as_float(0x7f800000);
              ax[k] = use ? __shfl_sync(0xffffffffu, ux, a) : inf;
              ay[k] = use ? __shfl_sync(0xffffffffu, uy, a) : inf;
              az[k] = use ? __shfl_sync(0xffffffffu, uz, a) : inf;
              next[k] = NextT(W.hnext[a]);
            }
            for (int r0 = 0; r0 < nround; r0 += 32) {
              const int f = r0 + lane;
              const float4 c = W.cv[f];
              bool acc[kGroup], unc[kGroup];
              bool any_unc = false;
#pragma unroll
              for (int k = 0; k < kGroup; ++k) {
                const float rx = c.x - ax[k], ry = c.y - ay[k], rz = c.z - az[k];
                const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
                acc[k] = r2 < lo && r2 > 0.f;
                unc[k] = !(r2 > hi) && !acc[k];
                any_unc |= unc[k];
              }
              if (__any_sync(0xffffffffu, any_unc)) {
#pragma unroll
                for (int k = 0; k < kGroup; ++k)
                  if (unc[k]) {
                    const int a = a0 + k;
                    if (f >= nkeep || a >= nb || is_self(W.cslot[f], hb + a, __float_as_uint(c.w), W.hmeta[a])) {
                      acc[k] = false;
                    } else {
                      ++rechecks;
                      acc[k] = exact_pair(g, A.Xs, hb + a, W.cslot[f], W.hmeta[a], __float_as_uint(c.w));
                    }
                  }
              }
              if (A.half) {  // half list: keep each unordered pair once
#pragma unroll
                for (int k = 0; k < kGroup; ++k)
                  if (acc[k]) acc[k] = half_keep(W.horig[a0 + k], W.corig[f], __float_as_uint(c.w), W.hmeta[a0 + k]);
              }
              if constexpr (MODE == kModeCount) {
                unsigned m[kGroup];
#pragma unroll
                for (int k = 0; k < kGroup; ++k) m[k] = __ballot_sync(0xffffffffu, acc[k]);
                if (list_cap > 0) {
                  // list entry: (slot of j, candidate word), in traversal order
                  // (32-bit offsets: the host keeps nat * list_cap below 2^32)
                  const uint2 ent = make_uint2(unsigned(W.cslot[f]), __float_as_uint(c.w));
                  const unsigned lt = lt_mask();
#pragma unroll
                  for (int k = 0; k < kGroup; ++k) {
                    const unsigned pos = unsigned(next[k]) + unsigned(__popc(m[k] & lt));
                    if (acc[k] && pos < unsigned(list_cap))
                      A.lists[unsigned(hb + a0 + k) * unsigned(list_cap) + pos] = ent;
                  }
                }
#pragma unroll
                for (int k = 0; k < kGroup; ++k) next[k] += __popc(m[k]);
              } else {
#pragma unroll
                for (int k = 0; k < kGroup; ++k) {
                  const unsigned mask = __ballot_sync(0xffffffffu, acc[k]);
                  if (mask == 0u) continue;
                  const int np = __popc(mask);
                  const int rank = __popc(mask & lt_mask());
                  if (acc[k]) {
                    const int rp = (tail + rank) & (kRing - 1);
                    W.rent[rp] = ((a0 + k) << 16) | f;
                    W.rslot[rp] = next[k] + rank;
                  }
                  tail += np;
                  next[k] += np;
                  if (tail - head >= 32) {
                    __syncwarp();
                    flush_ring<TI, MODE>(A, g, cs_tab, W, head, 32, lane);
                    head += 32;
                  }
                }
              }
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < kGroup; ++k)
              if (lane == k && a0 + k < nb) W.hnext[a0 + k] = next[k];
            __syncwarp();
          }
        }
      }
      if (MODE != kModeCount && tail > head) flush_ring<TI, MODE>(A, g, cs_tab, W, head, tail - head, lane);
      __syncwarp();
      if (lane < nb) {
        if (MODE == kModeCount) {
          const int cnt = int(W.hnext[lane]);
          A.counts[sv.abase + W.horig[lane]] = cnt;
          if (A.lcount) {
            A.lcount[hb + lane] = cnt;
            A.sorig[hb + lane] = sv.abase + W.horig[lane];
          }
          overflow |= cnt > list_cap;
        }
        if (MODE == kModeLazyR6) A.per_atom[sv.abase + W.horig[lane]] = W.hacc[lane];
      }
      __syncwarp();
    }
    // a cell with an atom whose list overflowed (or with no lists at all) is
    // written by the screening write pass (once: its rounds may all overflow)
    if (MODE == kModeCount && __any_sync(0xffffffffu, overflow) && lane == 0 &&
        (!split || atomicExch(A.cell_flag + h, 1) == 0)) {
      const int u = atomicAdd(A.n_screen_cells, 1);
      if (u < A.ncells_total) A.screen_cells[u] = h;
    }
  }
  // statistics: number of FP64 decisions
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_xor_sync(0xffffffffu, rechecks, o);
  if (lane == 0 && rechecks) atomicAdd(A.stats, (unsigned long long)rechecks);
}

// ------------------------------------------------------------------------
// Symmetric count pass (systems whose 27-cell stencil has distinct
// cells).  The reference decides (i, j, S) and (j, i, -S) identically:
// R(j, i, -S) = -R(i, j, S) bit for bit under round-to-nearest, so dot(R, R)
// is the same.  Each unordered pair of cells (A, A + d) is therefore
// screened once, by the warp of A, for the centre and the 13 stencil offsets
// after it.  An atom's accepted neighbours in stencil cell q are a 32-bit
// mask over that cell's atoms in sorted order, stored densely (27 words per
// atom, in the list region): the warp of A writes its atoms' words for
// q >= 13 (rows) and, for every atom j of A + d, j's word for the mirrored
// cell 26 - q (column: which atoms of A accepted j); words whose mirrored
// cell is empty or outside an open axis are written as 0 by the atom's own
// warp, so every word is written exactly once.  Pair counts accumulate with
// atomics; the write pass decodes the masks in the reference's order (stencil
// order, then sorted order in each cell).  A cell of more than 32 atoms sets
// sym_fail, and the per-cell count pass with per-atom lists runs instead.
// record meta of an atom without windings that is not exact
constexpr unsigned kPlainMeta = (128u) | (128u << 10) | (128u << 20);

// ------------------------------------------------------------------------
// The symmetric count pass, candidate-parallel: each unordered pair of cells
// (A, A + d), d the centre or one of the 13 stencil offsets after it, is
// screened once, by the warp of A.
// Lanes hold the candidates -- the atoms of stencil cells q = 13..26 in
// stencil order (centre first), 32 per round -- and the warp walks the home
// atoms two at a time with packed FP32 pair arithmetic (f32x2: the same IEEE
// operations, rounded per element, so the screen's r2 is bit for bit the
// scalar fmaf(rz, rz, fmaf(ry, ry, rx * rx))).  A home atom's accepted
// candidates of one round are a ballot; its row word for stencil cell q is
// the run of ballot bits of q's candidates (a funnel shift across two
// rounds).  A candidate's column word -- the home atoms that accepted it,
// stored as its word for the mirrored cell 26 - q -- accumulates in the
// candidate lane's register from its own decisions.  Lanes beyond the round's
// candidates and atoms beyond the home cell get infinite coordinates, so the
// screen needs no masks; the home atom itself (its own candidate in the
// centre) is taken out of its row afterwards.  The next cell's stencil ranges
// are loaded one cell ahead.  The write pass finds stencil cells from
// cell_offsets (a per-cell table of them was slower there: 0.492 against
// 0.484 ms at 1M atoms), the lazy sum's pass from a 28-word table row per
// home cell (first sorted slot of its 27 cells, their loop shifts; 0.711
// against 0.762 ms); each home atom's (position, sorted slot, home cell) goes to orow,
// indexed by its original index, for the original-order write pass.  Mask
// words are kMaskStride per atom (27 used) so that they load as 16-byte
// vectors.
constexpr int kSCWarps = 4;
constexpr long long kMaskStride = 28;  // mask words per atom (27 used; 16-byte rows)
constexpr int kSCMaxRounds = 14;  // 14 stencil cells of at most 32 atoms
#ifndef NL_SC_MIN_BLOCKS
#define NL_SC_MIN_BLOCKS 7  // 72 registers: 7 resident blocks; the default grid is twice that (0.815 against 0.820 ms per 1M-atom step with 6)
#endif
#ifndef NL_SC_PACKED
#define NL_SC_PACKED 1  // packed f32x2 pair arithmetic (0: the same operations as scalar FP32)
#endif

struct __align__(16) SCSmem {
  float hx[32], hy[32], hz[32];      // home atoms: FP32 record (+inf beyond the cell's atoms)
  unsigned hmeta[32];
  int horig[32];
  int hcnt[32];                      // pairs in the rows written by this warp
  unsigned B[32][kSCMaxRounds + 1];  // ballot of home atom a in round r
};

__device__ __forceinline__ unsigned long long f2pack(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2unpack(unsigned long long v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2sub(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2mul(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// What the candidate-parallel symmetric pass produces: the neighbour masks
// (and headers and gather rows) of the write pass, only the per-atom counts
// (the lazy count), or the masks with gather rows whose positions are fixed
// point (the lazy sum of 1/r^6, k_lazy_rows).
constexpr int kSymMasks = 0, kSymCounts = 1, kSymMasksFix = 2;
// Fixed-point positions of the lazy sum: x * 2^52 as a 64-bit integer
// (|x| < 2^11 A; below 1 A the position loses bits under 2^-53 A).
constexpr double kFixScale = 4503599627370496.0;  // 2^52
constexpr double kFixMax = 2000.0;

// Double-float (unevaluated FP32 pairs, hi + lo): Dekker's and Knuth's
// error-free products and sums (about 48 significant bits).
struct dfloat {
  float hi, lo;
};
__device__ __forceinline__ dfloat df_quick(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dfloat df_sq(float h, float l) {  // (h + l)^2
  const float p = h * h;
  float e = fmaf(h, h, -p);
  e = fmaf(2.f * h, l, e);
  return df_quick(p, e);
}
__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  return df_quick(s, e);
}
__device__ __forceinline__ dfloat df_mul(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_quick(p, e);
}
__device__ __forceinline__ dfloat df_rcp(dfloat a) {  // one Newton step from the FP32 reciprocal
  const float y = __fdividef(1.0f, a.hi);
  float e = fmaf(-a.hi, y, 1.0f);
  e = fmaf(-a.lo, y, e);
  return df_quick(y, y * e);
}
// A normal float (or zero) as a double, with integer operations.
__device__ __forceinline__ double f2d_exact(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned ex = (u >> 23) & 0xFFu;
  if (ex == 0u) return __longlong_as_double((long long)(u & 0x80000000u) << 32);  // +-0 (subnormals to zero)
  const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
  return __hiloint2double(int(hi), int((u & 0x7u) << 29));
}

// BATCH (masks only): the cells of the systems flagged in sys_sym, each warp
// reading its home cell's system geometry through L1, slots and original
// indices offset to the launch's; a system with a crowded cell sets its
// sys_fail, and the per-cell pass then counts all of it.  A batch keeps an
// atom's mask words at the start of its own list region.
#ifndef NL_SC_BATCH_MIN_BLOCKS
#define NL_SC_BATCH_MIN_BLOCKS 5  // resident blocks per SM of the batch variant (no spills at 96 registers)
#endif
template <typename TI, int SM, bool BATCH = false>
__global__ void __launch_bounds__(kSCWarps * 32, BATCH ? NL_SC_BATCH_MIN_BLOCKS : NL_SC_MIN_BLOCKS)
    k_sym_count(PairArgs<TI> A) {
  constexpr bool kMask = SM == kSymMasks || SM == kSymMasksFix;  // neighbour masks written
  static_assert(!BATCH || SM == kSymMasks, "batches take the mask variant only");
  // the screen's step: four home atoms (batches: 3.36 against 3.38 ms per
  // batch) or two (single systems: 0.855 against 0.865 ms per 1M-atom step)
  constexpr bool kQuad = BATCH && NL_SC_PACKED;
  __shared__ SCSmem sm[kSCWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  SCSmem& W = sm[warp];
  // batches: the home cell's system geometry, read through L1 (copying it to
  // shared memory for every cell was slower: 3.40 against 3.38 ms per batch)
  const Geometry* gp = &A.g;
  const int nat = BATCH ? A.nat_total : A.g.nat;  // bound of sorted slots and original indices
  float lo = A.g.lo, hi = A.g.hi;
  // batches: the home cell's system, its first slot / original atom and the
  // index of its cell 0 in cell_offsets (zero for a single system)
  int sys = 0, abase = 0, coff = 0;
  const float inf = __int_as_float(0x7f800000), nan = __int_as_float(0x7fc00000);
  unsigned rechecks = 0;
  if (A.cap_rec && blockIdx.x == 0 && threadIdx.x == 0) *A.cap_rec = A.list_cap;
  unsigned* masks = reinterpret_cast<unsigned*>(A.lists);
  auto mrow = [&](long long slot) -> unsigned* {  // the mask words of a sorted slot
    return BATCH ? reinterpret_cast<unsigned*>(A.lists + slot * A.list_cap) : masks + kMaskStride * slot;
  };
  const int nwarps = gridDim.x * kSCWarps;
  // stencil cell q = lane of home cell h: sorted range, loop-shift base, FP32 corner offset
  struct St {
    int start, cnt, lin;
    unsigned slp;
    float ox, oy, oz;
  };
  auto stencil = [&](int h, St& s) {
    s.start = s.cnt = 0;
    s.lin = -1;
    s.slp = 0;
    s.ox = s.oy = s.oz = 0.f;
    if (h < A.ncells_total && lane < 27) {
      const int hl = BATCH ? h - A.sys_cell[sys] : h;
      const Geometry& g = *gp;
      const int c0 = hl % g.ns[0] + 1, c1 = (hl / g.ns[0]) % g.ns[1] + 1, c2 = hl / (g.ns[0] * g.ns[1]) + 1;
      s.lin = stencil_cell(g, nullptr, 0, 3, 3, c0, c1, c2, lane, s.slp, s.ox, s.oy, s.oz);
      if (s.lin >= 0) {
        s.start = clampi(A.cell_offsets[coff + s.lin] - 1 + abase, nat);
        s.cnt = max(clampi(A.cell_offsets[coff + s.lin + 1] - 1 + abase, nat) - s.start, 0);
      }
    }
  };
  // (batches: a grid stride as well; runs of 8 consecutive cells per warp,
  // with the next cell's ranges loaded ahead within a system, were slower:
  // 1.20 against 0.99 ms per 4,096-system batch, and so was the next cell's
  // system and ranges loaded one grid-stride step ahead: 3.56 against 3.38 ms
  // per batch with the default launch shapes)
  int h = blockIdx.x * kSCWarps + warp;
  St cur;
  if (!BATCH) stencil(h, cur);
  for (; h < A.ncells_total; h += nwarps) {
    St nxt;
    if constexpr (BATCH) {
      sys = clampi(A.cell_sys[h], A.nsys - 1);
      if (!A.sys_sym[sys]) continue;
      gp = A.geo + sys;
      abase = A.sys_atom[sys];
      coff = A.sys_cell[sys] + sys;
      lo = gp->lo;
      hi = gp->hi;
      stencil(h, cur);
    } else {
      stencil(h + nwarps, nxt);  // the next cell's ranges are loaded while this one is screened
    }
    const int hs = __shfl_sync(0xffffffffu, cur.start, 13), nb = __shfl_sync(0xffffffffu, cur.cnt, 13);
    if (nb > 32 || __any_sync(0xffffffffu, cur.cnt > 32)) {
      // a crowded cell: the per-cell pass with lists counts instead
      if constexpr (BATCH) {
        // the first warp to fail the system appends its cells and slot
        // chunks to the lists the per-cell passes walk
        int first = 0;
        if (lane == 0) first = atomicExch(A.sys_fail + sys, 1) == 0;
        if (__shfl_sync(0xffffffffu, first, 0)) {
          const int c0 = A.sys_cell[sys], nc = A.sys_cell[sys + 1] - c0;
          int base = 0;
          if (lane == 0) base = atomicAdd(A.extra_cells, nc);
          base = __shfl_sync(0xffffffffu, base, 0);
          for (int c = lane; c < nc; c += 32) A.nonsym_cells[A.n_nonsym_cells + base + c] = c0 + c;
          const int a0 = A.sys_atom[sys] & ~31, nch = (A.sys_atom[sys + 1] - a0 + 31) >> 5;
          if (lane == 0) base = atomicAdd(A.extra_chunks, nch);
          base = __shfl_sync(0xffffffffu, base, 0);
          for (int k = lane; k < nch; k += 32) A.nonsym_chunks[A.n_nonsym_chunks + base + k] = a0 + 32 * k;
        }
      } else if (lane == 0) {
        atomicOr(A.sym_fail, 1);
      }
    } else if (nb > 0) {
      if constexpr (SM == kSymMasksFix) {
        // the stencil table row of the home cell, read by the lazy sum's
        // pass (k_lazy_rows): words q < 27 the first sorted slot of stencil cell q
        // (~0 outside an open axis), word 27 the loop shift + 1 of the
        // three cells along each axis (2 bits each: x at bit 0, y at 6, z at
        // 12), taken from the cells (dx, 1, 1), (1, dy, 1), (1, 1, dz)
        const int s0 = field10(cur.slp, 0) - 640 + 1, s1 = field10(cur.slp, 1) - 640 + 1,
                  s2 = field10(cur.slp, 2) - 640 + 1;
        unsigned part = 0u;
        if (cur.lin >= 0) {
          if (lane >= 12 && lane <= 14) part |= unsigned(s0 & 3) << (2 * (lane - 12));
          if (lane == 10 || lane == 13 || lane == 16) part |= unsigned(s1 & 3) << (6 + 2 * ((lane - 10) / 3));
          if (lane == 4 || lane == 13 || lane == 22) part |= unsigned(s2 & 3) << (12 + 2 * ((lane - 4) / 9));
        }
        const unsigned shifts = __reduce_or_sync(0xffffffffu, part);
        if (lane < 28) A.stab[28LL * h + lane] = lane < 27 ? (cur.lin >= 0 ? unsigned(cur.start) : ~0u) : shifts;
      }
      // words q < 13 of the home atoms that no other warp writes: their cell is empty or outside
      const unsigned zq = kMask ? __ballot_sync(0xffffffffu, lane < 13 && (cur.lin < 0 || cur.cnt == 0)) : 0u;
      if (zq)
        for (int t = lane; t < nb * 13; t += 32) {
          const int a = t / 13, q = t - 13 * a;
          if ((zq >> q) & 1u) mrow(hs + a)[q] = 0u;
        }
      unsigned hm = kPlainMeta;
      {
        float x = inf, y = inf, z = inf;
        if (lane < nb) {
          const float4 r = A.rec[hs + lane];  // exact atoms carry NaN coordinates
          x = r.x;
          y = r.y;
          z = r.z;
          hm = __float_as_uint(r.w);
          const int o = clampi(A.perm[hs + lane] - 1 + abase, nat - 1);
          W.horig[lane] = o;
          const double X0 = A.Xs[3LL * (hs + lane) + 0], X1 = A.Xs[3LL * (hs + lane) + 1],
                       X2 = A.Xs[3LL * (hs + lane) + 2];
          if constexpr (SM == kSymMasks) {
            ORow orw;  // the write pass walks atoms in original order
            orw.x = X0;
            orw.y = X1;
            orw.z = X2;
            orw.slot = hs + lane;
            orw.cell = h;
            A.orow[o] = orw;
            XPack xp;
            xp.x = X0;
            xp.y = X1;
            xp.z = X2;
            xp.perm = o + 1 - abase;  // j of the pair (system-local in a batch)
            xp.meta = hm;
            st_keep(A.xpk + hs + lane, xp, l2_keep_policy());
            const long long nz = (long long)0x8000000000000000ULL;
            if (__double_as_longlong(X0) == nz || __double_as_longlong(X1) == nz || __double_as_longlong(X2) == nz)
              atomicOr(A.sym_wound, 2);
          }
          if constexpr (SM == kSymMasksFix) {  // the lazy sum's gather row: fixed-point position
            XPack xp;
            xp.x = __longlong_as_double(__double2ll_rn(dmul(X0, kFixScale)));
            xp.y = __longlong_as_double(__double2ll_rn(dmul(X1, kFixScale)));
            xp.z = __longlong_as_double(__double2ll_rn(dmul(X2, kFixScale)));
            xp.perm = o + 1;
            xp.meta = hm;
            st_keep(A.xpk + hs + lane, xp, l2_keep_policy());
            if (!(fabs(X0) < kFixMax && fabs(X1) < kFixMax && fabs(X2) < kFixMax) || (hm & kExactBit))
              atomicOr(A.sym_wound, 4);  // out of the fixed-point range, or exact: FP64 pairs instead
          }
        }
        W.hx[lane] = x;
        W.hy[lane] = y;
        W.hz[lane] = z;
        W.hmeta[lane] = hm;
        W.hcnt[lane] = 0;
      }
      if (kMask && __any_sync(0xffffffffu, hm != kPlainMeta) && lane == 0) atomicOr(A.sym_wound, 1);
      // candidates: stencil cells 13..26 in stencil order, flattened
      const int scnt = lane >= 13 ? cur.cnt : 0;
      int incl = scnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int T = __shfl_sync(0xffffffffu, incl, 31);
      const int nr = (T + 31) >> 5;  // <= kSCMaxRounds
      __syncwarp();
      for (int rr = 0; rr < nr; ++rr) {
        const int f = 32 * rr + lane;
        const bool valid = f < T;
        const int gf = min(f, T - 1);
        int qq = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int v = __shfl_sync(0xffffffffu, incl, qq + step - 1);
          if (v <= gf) qq += step;
        }
        const int q_incl = __shfl_sync(0xffffffffu, incl, qq);
        const int q_cnt = __shfl_sync(0xffffffffu, scnt, qq);
        const int q_start = __shfl_sync(0xffffffffu, cur.start, qq);
        const unsigned q_slp = __shfl_sync(0xffffffffu, cur.slp, qq);
        const float qx = __shfl_sync(0xffffffffu, cur.ox, qq);
        const float qy = __shfl_sync(0xffffffffu, cur.oy, qq);
        const float qz = __shfl_sync(0xffffffffu, cur.oz, qq);
        const int slot = clampi(q_start + gf - (q_incl - q_cnt), nat - 1);
        const float4 r = A.rec[slot];
        const unsigned cw = cand_word(q_slp, __float_as_uint(r.w));
        const bool ex = (cw & kExactBit) != 0;
        // exact atoms carry NaN (always rechecked); lanes beyond the candidates -inf
        // (r2 = +inf against every home atom, +inf ones included: never accepted or rechecked)
        const float cx = !valid ? -inf : ex ? nan : r.x + qx, cy = !valid ? -inf : ex ? nan : r.y + qy,
                    cz = !valid ? -inf : ex ? nan : r.z + qz;
        const int corig = clampi(A.perm[slot] - 1 + abase, nat - 1);
#if NL_SC_PACKED
        const unsigned long long px = f2pack(cx, cx), py = f2pack(cy, cy), pz = f2pack(cz, cz);
#endif
        const bool fwd = qq > 13;  // a forward cell: this warp writes the candidate's column word
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);  // the round's candidates
        unsigned col = 0u;
        if constexpr (kQuad) {
        // home atoms a .. a + 3 per step (+inf beyond the cell): two packed
        // pairs from one 16-byte load per coordinate; one vote, one ballot
        // per atom
        for (int a = 0; a < nb; a += 4) {
          const ulonglong2 hx4 = *reinterpret_cast<const ulonglong2*>(&W.hx[a]);  // a % 4 == 0: 16-byte aligned
          const ulonglong2 hy4 = *reinterpret_cast<const ulonglong2*>(&W.hy[a]);
          const ulonglong2 hz4 = *reinterpret_cast<const ulonglong2*>(&W.hz[a]);
          float r2[4];
          {
            const unsigned long long rx = f2sub(px, hx4.x), ry = f2sub(py, hy4.x), rz = f2sub(pz, hz4.x);
            f2unpack(f2fma(rz, rz, f2fma(ry, ry, f2mul(rx, rx))), r2[0], r2[1]);
          }
          {
            const unsigned long long rx = f2sub(px, hx4.y), ry = f2sub(py, hy4.y), rz = f2sub(pz, hz4.y);
            f2unpack(f2fma(rz, rz, f2fma(ry, ry, f2mul(rx, rx))), r2[2], r2[3]);
          }
          bool l[4], u[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            l[k] = r2[k] < lo;
            u[k] = !l[k] && !(r2[k] > hi);
          }
          if (__any_sync(0xffffffffu, u[0] || u[1] || u[2] || u[3])) {
            const unsigned sb = rr == 0 ? 1u << a : 0u;  // the home atom itself
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const bool v = a + k < nb && (((vmask & ~(sb << k)) >> lane) & 1u);
              if (u[k] && v) {
                ++rechecks;
                l[k] = exact_pair(*gp, A.Xs, hs + a + k, slot, W.hmeta[a + k], cw);
              }
            }
          }
          unsigned row[4];
          bool c[4];  // this lane's candidate joins the column of home atom a + k
#pragma unroll
          for (int k = 0; k < 4; ++k) row[k] = __ballot_sync(0xffffffffu, l[k]);
          if constexpr (!kMask) {  // the home atom itself is no pair
            const unsigned sb = rr == 0 ? 1u << a : 0u;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              row[k] &= ~(sb << k);
              l[k] = l[k] && ((row[k] >> lane) & 1u);
            }
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) c[k] = l[k];
          if (A.half) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const bool kk = l[k] && half_keep(W.horig[a + k], corig, cw, W.hmeta[a + k]);
              row[k] = __ballot_sync(0xffffffffu, kk);
              c[k] = l[k] && !kk;
            }
          }
          if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {  // a + k <= 31: nb <= 32 and a % 4 == 0
              if constexpr (kMask)
                W.B[a + k][rr] = row[k];
              else
                W.hcnt[a + k] += __popc(row[k]);
            }
          }
          col |= ((c[0] ? 1u : 0u) | (c[1] ? 2u : 0u) | (c[2] ? 4u : 0u) | (c[3] ? 8u : 0u)) << a;
        }
        } else {
        for (int a = 0; a < nb; a += 2) {
          // home atoms a and a + 1 (+inf beyond the cell): packed (a, a + 1) pairs
          float r20, r21;
#if NL_SC_PACKED
          const unsigned long long hx2 = *reinterpret_cast<const unsigned long long*>(&W.hx[a]);
          const unsigned long long hy2 = *reinterpret_cast<const unsigned long long*>(&W.hy[a]);
          const unsigned long long hz2 = *reinterpret_cast<const unsigned long long*>(&W.hz[a]);
          const unsigned long long rx = f2sub(px, hx2), ry = f2sub(py, hy2), rz = f2sub(pz, hz2);
          const unsigned long long r2p = f2fma(rz, rz, f2fma(ry, ry, f2mul(rx, rx)));
          f2unpack(r2p, r20, r21);
#else
          {
            const float2 hx2 = *reinterpret_cast<const float2*>(&W.hx[a]);
            const float2 hy2 = *reinterpret_cast<const float2*>(&W.hy[a]);
            const float2 hz2 = *reinterpret_cast<const float2*>(&W.hz[a]);
            const float rx0 = cx - hx2.x, ry0 = cy - hy2.x, rz0 = cz - hz2.x;
            const float rx1 = cx - hx2.y, ry1 = cy - hy2.y, rz1 = cz - hz2.y;
            r20 = fmaf(rz0, rz0, fmaf(ry0, ry0, rx0 * rx0));
            r21 = fmaf(rz1, rz1, fmaf(ry1, ry1, rx1 * rx1));
          }
#endif
          // accepted: r2 < lo; the band and NaN (exact atoms) are decided in FP64
          // with the reference's arithmetic.  The centre holds the home atom
          // itself at candidate f == a (round 0, lane a): accepted here (r2 = 0)
          // and taken out of its row word after the rounds (masks) or below.
          bool l0 = r20 < lo, l1 = r21 < lo;
          const bool u0 = !l0 && !(r20 > hi), u1 = !l1 && !(r21 > hi);
          if (__any_sync(0xffffffffu, u0 || u1)) {
            const unsigned sb = rr == 0 ? 1u << a : 0u;  // the home atom itself
            const bool v0 = ((vmask & ~sb) >> lane) & 1u;
            const bool v1 = a + 1 < nb && (((vmask & ~(sb << 1)) >> lane) & 1u);
            if (u0 && v0) {
              ++rechecks;
              l0 = exact_pair(*gp, A.Xs, hs + a, slot, W.hmeta[a], cw);
            }
            if (u1 && v1) {
              ++rechecks;
              l1 = exact_pair(*gp, A.Xs, hs + a + 1, slot, W.hmeta[a + 1], cw);
            }
          }
          unsigned acc0 = __ballot_sync(0xffffffffu, l0), acc1 = __ballot_sync(0xffffffffu, l1);
          if constexpr (!kMask) {  // the home atom itself is no pair
            const unsigned sb = rr == 0 ? 1u << a : 0u;
            acc0 &= ~sb;
            acc1 &= ~(sb << 1);
            l0 = l0 && ((acc0 >> lane) & 1u);
            l1 = l1 && ((acc1 >> lane) & 1u);
          }
          // full lists keep both directions (row and, for forward cells, column);
          // a half list keeps the one half_keep selects
          unsigned row0 = acc0, row1 = acc1;
          bool c0 = l0, c1 = l1;  // this lane's candidate joins the column of home atom a / a + 1
          if (A.half) {
            const bool k0 = l0 && half_keep(W.horig[a], corig, cw, W.hmeta[a]);
            const bool k1 = l1 && half_keep(W.horig[a + 1], corig, cw, W.hmeta[a + 1]);
            row0 = __ballot_sync(0xffffffffu, k0);
            row1 = __ballot_sync(0xffffffffu, k1);
            c0 = l0 && !k0;
            c1 = l1 && !k1;
          }
          if constexpr (kMask) {
            if (lane == 0) {
              W.B[a][rr] = row0;
              W.B[a + 1][rr] = row1;  // a + 1 <= 31: nb <= 32 and a is even
            }
          } else {
            if (lane == 0) {
              W.hcnt[a] += __popc(row0);
              W.hcnt[a + 1] += __popc(row1);
            }
          }
          col |= (c0 ? 1u << a : 0u) | (c1 ? 2u << a : 0u);
        }
        }
        if constexpr (kMask) {
          if (valid && fwd) {  // the candidate's word for its mirrored cell
            mrow(slot)[26 - qq] = col;
            if (col) atomicAdd(A.counts + corig, __popc(col));
          }
        } else {
          if (valid && fwd && col) atomicAdd(A.counts + corig, __popc(col));
        }
      }
      __syncwarp();
      if constexpr (kMask) {  // the home atom itself (round 0, candidate a) is no pair
        if (lane < nb) W.B[lane][0] &= ~(1u << lane);
        __syncwarp();
      }
      if constexpr (SM == kSymCounts) {
        if (lane < nb && W.hcnt[lane]) atomicAdd(A.counts + W.horig[lane], W.hcnt[lane]);
        __syncwarp();
      }
      if constexpr (kMask) {
      // rows: word q = 13..26 of every home atom, from its ballots
      for (int t0 = 0; t0 < nb * 14; t0 += 32) {
        const int t = t0 + lane;
        const int a = t / 14, k = t - 14 * (t / 14);
        const int off = __shfl_sync(0xffffffffu, incl - scnt, 13 + k);
        const int cnt = __shfl_sync(0xffffffffu, scnt, 13 + k);
        if (t < nb * 14) {
          unsigned w = 0u;
          if (cnt > 0) {  // then off + cnt <= 32 nr: both ballot words exist
            w = __funnelshift_r(W.B[a][off >> 5], W.B[a][(off >> 5) + 1], off & 31);
            if (cnt < 32) w &= (1u << cnt) - 1u;
          }
          mrow(hs + a)[13 + k] = w;
          if (w) atomicAdd(&W.hcnt[a], __popc(w));
        }
      }
      __syncwarp();
      if (lane < nb && W.hcnt[lane]) atomicAdd(A.counts + W.horig[lane], W.hcnt[lane]);
      __syncwarp();
      }
    }
    if constexpr (!BATCH) cur = nxt;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_xor_sync(0xffffffffu, rechecks, o);
  if (lane == 0 && rechecks) atomicAdd(A.stats, (unsigned long long)rechecks);
}

// ------------------------------------------------------------------------
// Emit: writes i, j, S, R of every atom whose pairs the count pass listed --
// no stencil, no staging and no screening.  One warp takes 32 consecutive
// sorted slots; their per-atom data go to shared memory, then the warp walks
// the atoms one at a time, lane r writing the atom's r-th pair.  The output
// slots first[i] + r are consecutive, so the stores coalesce.  Passes run as
// a three-stage pipeline (list entries, gathers, S / R / stores).
#ifndef NL_EMIT_MIN_BLOCKS
#define NL_EMIT_MIN_BLOCKS 8
#endif

constexpr int kEmitWarps = 4;
constexpr int kEmitMinBlocks = NL_EMIT_MIN_BLOCKS;  // resident blocks per SM the register budget targets

// passes of a chunk of 32 atoms of at most kListCap listed pairs each; a
// pass number within an atom is kept in 8 bits
constexpr int kChunkPasses = 32 * ((kListCap + 31) / 32);
static_assert((kListCap + 31) / 32 <= 255, "pass numbers within an atom are 8-bit");

struct __align__(16) EmitAtoms {
  long long sbuf[96];   // a pass's S, three words per pair, staged for contiguous stores
  unsigned short pass[kChunkPasses];  // the chunk's passes (32 atoms, up to kListCap / 32 each): atom << 8 | pass
  double rbuf[96];      // a pass's R, likewise
  double xi[32][3];     // FP64 position
  long long base[32];   // first output slot (0-based)
  long long ti[32];     // output value of i (system-local, 1-based)
  unsigned mi[32];      // packed windings | exact bit
  int n[32];            // listed pairs (0 when written by the screening pass)
  int sys[32];          // batch: system of the slot
};

// The atoms whose pairs the per-cell count pass listed: a single system's
// when the symmetric pass gave up (or did not apply), a batch's in the
// systems the symmetric pass did not count.  Atoms of more than list_cap
// pairs are left to the screening write pass.
#ifndef NL_EMIT_BATCH_MIN_BLOCKS
#define NL_EMIT_BATCH_MIN_BLOCKS 6  // the batch variant (4.94 -> 4.85 ms per 4,096 systems against 8)
#endif
template <typename TI, bool BATCH>
__global__ void __launch_bounds__(kEmitWarps * 32, BATCH ? NL_EMIT_BATCH_MIN_BLOCKS : kEmitMinBlocks)
    k_emit(PairArgs<TI> A) {
  // the count recorded its choice in the workspace: sym_fail == 0 after a
  // successful symmetric count (the mask write pass), non-zero otherwise
  if (!BATCH && *A.sym_fail == 0) return;
  __shared__ EmitAtoms ea[kEmitWarps];
  __shared__ double cs_blk[BATCH ? 1 : 3 * kCsN * kCsN * kCsN];
  if (!BATCH) {
    for (int t = threadIdx.x; t < 3 * kCsN * kCsN * kCsN; t += blockDim.x) cs_blk[t] = A.cs_table[t];
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  EmitAtoms& E = ea[warp];
  const int K = A.list_cap;
  const long long nwarps = (long long)gridDim.x * kEmitWarps;
  // batches: the next 32 atoms from a counter as warps free up (uneven pair
  // counts); single systems: a grid stride
  unsigned* ework = BATCH ? reinterpret_cast<unsigned*>(A.work) + 2 : nullptr;
  // with the symmetric pass, only the chunks of the systems it did not take
  // or that failed it (a chunk met twice is written twice with the same values)
  const bool nonsym = BATCH && A.sym && A.nonsym_chunks;
  const unsigned nchunks = nonsym ? unsigned(A.n_nonsym_chunks + *A.extra_chunks) : 0u;
  auto next_c0 = [&](long long cur) -> long long {
    if constexpr (!BATCH) {
      return cur + nwarps * 32;
    } else {
      unsigned b = 0;
      if (lane == 0) b = atomicAdd(ework, nonsym ? 1u : 32u);
      b = __shfl_sync(0xffffffffu, b, 0);
      if (!nonsym) return (long long)b;
      return b < nchunks ? (long long)A.nonsym_chunks[b] : A.nat_total;
    }
  };
  for (long long c0 = BATCH ? next_c0(0) : ((long long)blockIdx.x * kEmitWarps + warp) * 32; c0 < A.nat_total;
       c0 = next_c0(c0)) {
    const int na = int(min(32LL, A.nat_total - c0));
    __syncwarp();
    if (lane < na) {
      const int slot = int(c0) + lane;
      const int sys = BATCH ? clampi(A.cell_sys[clampi(A.scell[slot], A.ncells_total - 1)], A.nsys - 1) : 0;
      E.sys[lane] = sys;
      // batches: the atoms of the systems the symmetric pass did not count
      const bool own = !BATCH || !(A.sym && A.sys_sym[sys] && !A.sys_fail[sys]);
      if (!own) {
        E.n[lane] = 0;      } else {
        int n = A.lcount[slot];
        E.n[lane] = n > K ? 0 : n;  // overflowed atoms belong to the screening pass
        E.base[lane] = (long long)A.first[clampi(A.sorig[slot], A.nat_total - 1)] - 1;
      }
      E.ti[lane] = (long long)A.perm[slot];
      E.mi[lane] = __float_as_uint(A.rec[slot].w);
      E.xi[lane][0] = A.Xs[3LL * slot + 0];
      E.xi[lane][1] = A.Xs[3LL * slot + 1];
      E.xi[lane][2] = A.Xs[3LL * slot + 2];
    }
    __syncwarp();

    int pa = 0, pr = 0, pn = 0;  // the pass in stage 3
    unsigned pcw = 0;
    long long poj = 0;
    double pxj0 = 0.0, pxj1 = 0.0, pxj2 = 0.0;
    // The pass's pairs occupy output slots [out0, out0 + nact): i and j are
    // stored per lane, S and R are staged in shared memory and stored as
    // consecutive words, so every store instruction covers whole sectors.
    auto finish = [&]() {
      const bool act = pr < pn;
      const double* xi = E.xi[pa];
      const double xj[3] = {pxj0, pxj1, pxj2};
      const Geometry& g = BATCH ? A.geo[E.sys[pa]] : A.g;
      const double* cs_tab = BATCH ? A.cs_sys + 3 * kCsN * kCsN * kCsN * (long long)E.sys[pa] : cs_blk;
      int S[3];
      pair_S(g, xi, xj, E.mi[pa], pcw, S);
      const long long out0 = E.base[pa] + (pr - lane);
      const int nact = min(32, pn - (pr - lane));
      const long long out = out0 + lane;
      const bool wr = act && out < A.capacity;
      if (act && !wr) atomicOr(A.err, kFlagCapacity);
      // outputs are written once and never re-read here: streaming stores keep
      // the gathered positions and the lists in L2
      if (wr) {
        __stcs(A.oi + out, TI(E.ti[pa]));
        __stcs(A.oj + out, TI(poj));
      }
      E.sbuf[3 * lane + 0] = S[0];
      E.sbuf[3 * lane + 1] = S[1];
      E.sbuf[3 * lane + 2] = S[2];
      if (A.oR) {
        double R[3];
        pair_R(g, cs_tab, xi, xj, S[0], S[1], S[2], act, R);
        E.rbuf[3 * lane + 0] = R[0];
        E.rbuf[3 * lane + 1] = R[1];
        E.rbuf[3 * lane + 2] = R[2];
      }
      __syncwarp();
      const long long wend = 3 * min(out0 + nact, A.capacity);  // words that fit the buffers
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int t = lane + 32 * k;
        const long long wpos = 3 * out0 + t;
        if (t < 3 * nact && wpos < wend) {
          __stcs(A.oS + wpos, TI(E.sbuf[t]));
          if (A.oR) __stcs(A.oR + wpos, E.rbuf[t]);
        }
      }
      __syncwarp();
    };
    // Three stages over the chunk's passes -- list entry (pass h), gathers
    // (pass h-1), S / R / stores (pass h-2) -- with two register sets used
    // alternately, so that no value waits to be copied between stages: the
    // gathers of a pass are consumed only after another pass's stores.
    {
      const int c = lane < na ? (E.n[lane] + 31) >> 5 : 0;  // passes of atom `lane`
      int ci = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, ci, o);
        if (lane >= o) ci += v;
      }
      const int npass = __shfl_sync(0xffffffffu, ci, 31);
      for (int k = 0; k < c; ++k) E.pass[ci - c + k] = (unsigned short)((lane << 8) | k);
      __syncwarp();
      struct StE {
        uint2 e;
        int a, r;
        bool v;
      };
      struct StG {
        double x0, x1, x2;
        long long oj;
        unsigned cw;
        int a, r;
        bool v;
      };
      auto stage_e = [&](int h, StE& t) {
        t.v = h < npass;
        if (t.v) {
          const unsigned pd = E.pass[h];
          t.a = int(pd >> 8);
          t.r = 32 * int(pd & 255u) + lane;
          t.e = __ldcs(A.lists + (c0 + t.a) * K + min(t.r, E.n[t.a] - 1));  // read once
        }
      };
      auto stage_g = [&](const StE& t, StG& u) {
        u.v = t.v;
        if (u.v) {
          const uint2 e = t.e;
          const int slot_j = clampi(int(e.x), A.nat_total - 1);
          u.x0 = __ldg(A.Xs + 3LL * slot_j + 0);
          u.x1 = __ldg(A.Xs + 3LL * slot_j + 1);
          u.x2 = __ldg(A.Xs + 3LL * slot_j + 2);
          u.oj = (long long)__ldg(A.perm + slot_j);
          u.cw = e.y;
          u.a = t.a;
          u.r = t.r;
        }
      };
      auto stage_f = [&](const StG& u) {
        if (u.v) {
          pa = u.a;
          pr = u.r;
          pn = E.n[u.a];
          pcw = u.cw;
          poj = u.oj;
          pxj0 = u.x0;
          pxj1 = u.x1;
          pxj2 = u.x2;
          finish();
        }
      };
      StE e0, e1;
      StG g0, g1;
      e0.v = e1.v = false;
      g0.v = g1.v = false;
      e0.a = e0.r = e1.a = e1.r = 0;
      e0.e = e1.e = make_uint2(0u, 0u);
      for (int h = 0; h < npass + 2; h += 2) {
        stage_e(h, e0);
        stage_g(e1, g1);
        stage_f(g0);
        stage_e(h + 1, e1);
        stage_g(e0, g0);
        stage_f(g1);
      }
    }
  }
}

// ------------------------------------------------------------------------
// Write pass for the symmetric count pass's neighbour masks, in ORIGINAL atom
// order (single systems; batches below).  Atom o's pairs occupy [first[o], first[o+1]) and
// atoms follow one another in original order, so a warp that takes 32
// consecutive original atoms writes one contiguous run of every output array:
// its stores cover whole lines, and only the run's two ends share a sector
// with another warp's atoms.  (Walking atoms in cell order instead scatters
// ~26-pair runs over the arrays; the partial sectors at both ends of every
// run cost extra DRAM traffic.)  The neighbours' data are gathered from
// anywhere in the sorted arrays, so they come from L2: one 32-byte row per
// neighbour (XPack: position, perm, meta, written by the count pass), read
// as one 256-bit load.
//
// Per batch of 32 atoms, lane a holds atom o0 + a: its row by original index
// (ORow: position, sorted slot, home cell, written by the count pass; read
// coalesced) and output range, then -- loads issued together -- its 27 mask
// words (16-byte vector loads) and the sorted start of each of its 27
// stencil cells (cell_offsets; the wrapped cell and loop shift per axis
// follow from the home cell); the record meta only where some atom has
// windings or is exact.  The masks are expanded into a
// shared-memory table of 8-byte entries (slot of j; atom and the three loop
// shifts) at the pairs' output positions, in stencil order (dz, dy, dx) and
// sorted order within each stencil cell -- the reference's traversal order.
// The expansion is balanced over the warp: each lane lists its non-empty
// words (word, stencil cell start, loop-shift code) at the end of its own
// stretch of the table, then takes one set bit per step, reading the next
// listed word when a word is used up.  The warp takes as many steps as its
// busiest lane has pairs (about 37 for 26 pairs per atom) instead of, word by
// word, as many as the fullest word of any lane has bits (about 120).  A
// listed word is read before the entries reach it: when the entry at stretch
// position s is written, every unread listed word still holds a bit, so the
// unread part of the list lies beyond s.  The table holds kEOEnt entries; a
// batch with more pairs is cut at atom boundaries (an atom has at most
// 27 * 32 - 1 pairs on this path).  The warp then walks the output positions
// 32 at a time, passes aligned to multiples of 32 in the output arrays, lane
// r writing pair base + r: i, j, S (the loop shifts, or with windings
// s_loop + wi - wj) and R = (xj - xi) + C'S with the reference's operations,
// one word per lane and array in each store instruction.  The gathers of
// kEOPasses passes are in flight before the first of them is written.
#ifndef NL_EO_MIN_BLOCKS
#define NL_EO_MIN_BLOCKS 8  // resident blocks per SM the register budget targets
#endif
#ifndef NL_EO_PASSES
#define NL_EO_PASSES 2  // passes whose gathers are in flight together
#endif
constexpr int kEOWarps = 2;
constexpr int kEOEnt = 1024;  // pair entries per warp (896 with the C'S table read through L1: slower)
constexpr int kEOPasses = NL_EO_PASSES;
static_assert(kEOEnt >= 27 * 32 + 32, "a chunk holds an atom of 27 * 32 pairs from any offset");

template <typename TI>
struct __align__(16) EOSmem {
  uint2 ent[kEOEnt];           // entry: (sorted slot of j, atom | loop shift + 1 per axis << 5 + 2k);
                               // while the masks are expanded also the listed words (word, cell start)
  unsigned char code[kEOEnt];  // loop-shift code (bits 5.. of an entry's second word) of a listed word
  double xi[32][4];            // the batch's atoms: FP64 position; [3]: batches' system and i
  unsigned mi[32];             //   record meta (windings, exact bit)
};
// (shared memory per block: 8 resident blocks of 23.7 KB leave the L1 60 KB
// of the SM's 256 KB; 512 bytes more per block took it to 28 KB and the
// write pass from 0.49 to 0.74 ms at 1M atoms)

// The three cells c - 1, c, c + 1 along one axis (c 1-based): 0-based wrapped
// index, loop shift and whether the cell exists (wrap_and_shift,
// cell_list.jl:105-120; periodic axes of the symmetric path have n >= 3).
__device__ __forceinline__ void axis3(int c, int n, int pbc, int* w, int* s, bool* ok) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int i = c + d - 1, sh = 0;
    bool v = true;
    if (i < 1) {
      if (pbc) {
        i += n;
        sh = -1;
      } else {
        v = false;
      }
    } else if (i > n) {
      if (pbc) {
        i -= n;
        sh = 1;
      } else {
        v = false;
      }
    }
    w[d] = i - 1;
    s[d] = sh;
    ok[d] = v;
  }
}

// BATCH: the atoms of the systems the symmetric pass counted (sys_sym set,
// sys_fail clear), in the launch's original order; each lane looks up its
// atom's system, and each pair takes its atom's system geometry and C'S
// table; i and j are system-local.  The atoms of the other systems are left
// to the list write pass (a warp's chunks are runs of this kernel's atoms).
template <typename TI, bool BATCH = false>
__global__ void __launch_bounds__(kEOWarps * 32, NL_EO_MIN_BLOCKS) k_emit_orig(PairArgs<TI> A) {
  if (!BATCH && *A.sym_fail != 0) return;  // the count pass used lists: k_emit writes them
  __shared__ EOSmem<TI> sm[kEOWarps];
  constexpr bool kCsSmem = !BATCH;
  __shared__ double cs_blk[kCsSmem ? 3 * kCsN * kCsN * kCsN : 1];
  const Geometry& g = A.g;  // single systems
  if (kCsSmem) {
    for (int t = threadIdx.x; t < 3 * kCsN * kCsN * kCsN; t += blockDim.x) cs_blk[t] = A.cs_table[t];
    __syncthreads();
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  EOSmem<TI>& E = sm[warp];
  const int nat = BATCH ? A.nat_total : A.g.nat;  // bound of sorted slots and original indices
  const int sw = *A.sym_wound;
  const bool plain = (sw & 1) == 0;   // no atom has a winding or is exact: S = the loop shift
  const bool negzero = (sw & 2) != 0;  // a coordinate is -0: R needs the signed-zero rule for S = 0
  const unsigned* masks = reinterpret_cast<const unsigned*>(A.lists);
  const long long cap = A.capacity;
  constexpr int kZc = 3 * ((kCsN * kCsN + kCsN + 1) * kCsR);  // C'(0,0,0) in a C'S table: signed zeros
  const unsigned long long keep = l2_keep_policy();
  unsigned bad = 0;  // error flags of this lane
  const long long nwarps = (long long)gridDim.x * kEOWarps;
  for (long long o0 = ((long long)blockIdx.x * kEOWarps + warp) * 32; o0 < nat; o0 += nwarps * 32) {
    const int na = int(min(32LL, nat - o0));
    bool own = lane < na;
    int sy = 0;  // batches: the atom's system (the last one whose first atom is at or before it)
    if (BATCH && own) {
      const int o = int(o0) + lane;
      int lo_s = 0, hi_s = A.nsys - 1;
      while (lo_s < hi_s) {
        const int mid = (lo_s + hi_s + 1) >> 1;
        if (A.sys_atom[mid] <= o) lo_s = mid;
        else hi_s = mid - 1;
      }
      sy = lo_s;
      own = A.sys_sym[sy] && !A.sys_fail[sy];
    }
    // ---- lane a: atom o0 + a.  Its row (position, slot, home cell) and output range first ...
    int2 hd = make_int2(0, 0);
    long long f = 0, n = 0;
    if (own) {
      const long long o = o0 + lane;
      const double2 p01 = ld_stream(reinterpret_cast<const double2*>(A.orow + o));
      const int4 p2 = ld_stream(reinterpret_cast<const int4*>(A.orow + o) + 1);
      hd = make_int2(p2.z, p2.w);
      E.xi[lane][0] = p01.x;
      E.xi[lane][1] = p01.y;
      E.xi[lane][2] = __hiloint2double(p2.y, p2.x);
      f = (long long)A.first[o] - 1;
      n = (long long)A.first[o + 1] - 1 - f;
    }
    const int slot = clampi(hd.x, nat - 1);
    // the home cell within its system, the system's grid, its cell 0 in
    // cell_offsets and its first slot / original atom
    int ns0 = g.ns[0], ns1 = g.ns[1], ns2 = g.ns[2], pb0 = g.pbc[0], pb1 = g.pbc[1], pb2 = g.pbc[2];
    int coff = 0, abase = 0;
    if (BATCH) {
      const Geometry& gs = A.geo[sy];
      ns0 = max(gs.ns[0], 1);
      ns1 = max(gs.ns[1], 1);
      ns2 = max(gs.ns[2], 1);
      pb0 = gs.pbc[0];
      pb1 = gs.pbc[1];
      pb2 = gs.pbc[2];
      coff = A.sys_cell[sy] + sy;
      abase = A.sys_atom[sy];
    }
    const int hc = clampi(hd.y - (BATCH ? A.sys_cell[sy] : 0), ns0 * ns1 * ns2 - 1);
    const unsigned ownm = __ballot_sync(0xffffffffu, own);
    // ---- chunks of at most kEOEnt pairs, cut at atom boundaries; each chunk
    // loads, expands and writes its own atoms, so that the masks and cell
    // starts held for the expansion are dead while the chunk is written
    // (chunks are runs of consecutive lanes of this kernel's atoms: all of
    // them for a single system)
    int l0 = ownm ? __ffs(ownm) - 1 : 32;
    while (l0 < na) {
      const long long G = __shfl_sync(0xffffffffu, f, l0);
      // (entries are stored from index G mod 32: kEOEnt - 32 pairs per chunk)
      const unsigned inch = __ballot_sync(0xffffffffu, lane >= l0 && own && f + n - G <= kEOEnt - 32);
      const unsigned gap = ~(inch >> l0);
      const int l1 = gap ? l0 + __ffs(gap) - 1 : 32;
      if (l1 == l0) {  // an atom with more pairs than its masks can hold: counts and masks disagree
        bad |= kFlagInconsistent;
        break;
      }
      const int cnt = int(__shfl_sync(0xffffffffu, f + n, l1 - 1) - G);
      const bool mine = lane >= l0 && lane < l1;
      {
        int wx[3], wy[3], wz[3], sx[3], sy3[3], sz[3];
        bool okx[3], oky[3], okz[3];
        axis3(hc % ns0 + 1, ns0, pb0, wx, sx, okx);
        axis3((hc / ns0) % ns1 + 1, ns1, pb1, wy, sy3, oky);
        axis3(hc / (ns0 * ns1) + 1, ns2, pb2, wz, sz, okz);
        // masks, position, meta and the 27 stencil cell starts, all in flight together
        uint4 mv[7];
        const uint4* mrow = reinterpret_cast<const uint4*>(
            BATCH ? reinterpret_cast<const unsigned*>(A.lists + (long long)slot * A.list_cap) : masks + kMaskStride * slot);
#pragma unroll
        for (int k = 0; k < 7; ++k) mv[k] = mine ? ld_stream(mrow + k) : make_uint4(0u, 0u, 0u, 0u);
        unsigned st[27];
#pragma unroll
        for (int r = 0; r < 9; ++r) {
          const int dy = r % 3, dz = r / 3;
          const int rb = coff + ns0 * (wy[dy] + ns1 * wz[dz]);
          const bool rok = mine && oky[dy] && okz[dz];
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
            st[3 * r + dx] =
                unsigned(clampi((rok && okx[dx] ? A.cell_offsets[rb + wx[dx]] : TI(1 - abase)) - 1 + abase, nat));
        }
        if (mine) {  // record meta (windings, exact bit): only where some atom has one
          E.mi[lane] = plain ? kPlainMeta : __float_as_uint(A.rec[slot].w);
          if (BATCH) E.xi[lane][3] = __hiloint2double(sy, int(o0) + lane + 1 - abase);  // system, i
        }
        // ---- the lane's non-empty words, listed at the end of its stretch
        // [e0, e0 + nn) of the table (each holds a bit: nnz <= nn), written
        // from the last word down so that each mask word and cell start dies
        // as soon as it is listed
        const int e0 = mine ? int(f - G) + int(G & 31) : 0;  // the entry of output position p sits at p - (G - G mod 32)
        const int nn = mine ? int(n) : 0;
        int nnz = 0, tot = 0;
#pragma unroll
        for (int q = 26; q >= 0; --q) {
          unsigned mq = (&mv[q >> 2].x)[q & 3];
          if (mq && !(okx[q % 3] && oky[(q / 3) % 3] && okz[q / 9])) {  // a neighbour in a cell outside an open axis
            bad |= kFlagInconsistent;
            mq = 0u;
          }
          if (mq) {
            if (nnz < nn && e0 >= 0) {
              const int k = e0 + nn - 1 - nnz;
              E.ent[k] = make_uint2(mq, st[q]);
              E.code[k] = (unsigned char)(unsigned(sx[q % 3] + 1) | unsigned(sy3[(q / 3) % 3] + 1) << 2 |
                                          unsigned(sz[q / 9] + 1) << 4);
            }
            ++nnz;
            tot += __popc(mq);
          }
        }
        const bool lok = mine && tot == nn && e0 >= 0;
        if (mine && !lok) bad |= kFlagInconsistent;  // counts and masks disagree
        const int li = e0 + nn - nnz;  // the first listed word
        // ---- one set bit per step: entry e0 + s is the lane's pair s
        unsigned w = 0u, stq = 0u, inf = 0u;
        int kk = 0;
        if (lok && nnz > 0) {
          const uint2 it = E.ent[li];
          w = it.x;
          stq = it.y;
          inf = unsigned(lane) | unsigned(E.code[li]) << 5;
          kk = 1;
        }
        const int smax = __reduce_max_sync(0xffffffffu, lok ? nn : 0);
        for (int s = 0; s < smax; ++s) {
          const bool on = lok && s < nn;
          const unsigned bit = unsigned(__ffs(w) - 1);
          if (on) E.ent[e0 + s] = make_uint2(stq + bit, inf);
          w &= w - 1u;
          if (on && w == 0u && s + 1 < nn && kk < nnz) {  // the word is used up: the next listed one
            const int p = li + kk;
            const uint2 it = E.ent[p];
            w = it.x;
            stq = it.y;
            inf = unsigned(lane) | unsigned(E.code[p]) << 5;
            ++kk;
          }
        }
      }
      __syncwarp();
      // ---- emission: lane r of pass j writes output position p0 + 32 j + r
      // (p0 = G rounded down to a multiple of 32), entry 32 j + r: i and j as
      // one word per lane, S and R as three words per lane (each store
      // instruction covers a contiguous run of the arrays).
      const int off = int(G & 31);
      const int lim = int(max(min((long long)cnt, cap - G), 0LL));  // entries that fit the buffers
      if ((long long)cnt > cap - G && lane == l0) bad |= kFlagCapacity;
      const int hix = off + lim;  // entries [off, hix) are this chunk's pairs
      const int npass = (hix + 31) >> 5;
      const long long p0 = G - off;
      TI* __restrict__ oi = A.oi + p0;
      TI* __restrict__ oj = A.oj + p0;
      TI* __restrict__ oS = A.oS + 3 * p0;
      double* __restrict__ oR = A.oR ? A.oR + 3 * p0 : nullptr;
      const TI ti0 = TI(o0 + 1);  // i of atom a is ti0 + a
      struct Ld {
        uint2 en;
        double2 w0;
        int4 w1;
      };
      // every lane loads (entries outside [off, hix) repeat an edge entry; their stores are off)
      auto load = [&](int k, Ld& u) {
        u.en = E.ent[min(max(k, off), hix - 1)];
        ld_row(A.xpk + min(u.en.x, unsigned(nat - 1)), keep, u.w0, u.w1);
      };
      auto write = [&](int k, const Ld& u) {
        const bool act = k >= off && k < hix;
        const unsigned info = u.en.y;
        const int a = int(info & 31u);
        const double* xi = E.xi[a];
        const int ps = BATCH ? __double2hiint(xi[3]) : 0;  // batches: the pair's system
        const double* cst = BATCH ? A.cs_sys + (long long)kCsTableDoubles * ps : cs_blk;
        const double x0 = u.w0.x, x1 = u.w0.y, x2 = __hiloint2double(u.w1.y, u.w1.x);
        int S0 = int((info >> 5) & 3u) - 1, S1 = int((info >> 7) & 3u) - 1, S2 = int((info >> 9) & 3u) - 1;
        bool snz = (info & (63u << 5)) != (21u << 5);  // (S0, S1, S2) != 0: the codes are not 1, 1, 1
        if (!plain) {  // windings or exact atoms: S = s_loop + wi - wj
          const double xj[3] = {x0, x1, x2};
          int S[3];
          pair_S(BATCH ? A.geo[ps] : g, xi, xj, E.mi[a], cand_word(cand_base(S0, S1, S2), unsigned(u.w1.w)), S);
          S0 = S[0];
          S1 = S[1];
          S2 = S[2];
          snz = (S0 | S1 | S2) != 0;
        }
        if (act) {
          __stcs(oi + k, BATCH ? TI(__double2loint(xi[3])) : TI(ti0 + a));
          __stcs(oj + k, TI(u.w1.z));
          __stcs(oS + 3 * k + 0, TI(S0));
          __stcs(oS + 3 * k + 1, TI(S1));
          __stcs(oS + 3 * k + 2, TI(S2));
        }
        if (oR) {
          double R0 = dsub(x0, xi[0]), R1 = dsub(x1, xi[1]), R2 = dsub(x2, xi[2]);
          const bool nz = act && snz;
          if (__any_sync(0xffffffffu, nz)) {
            if (nz) {
              double c0, c1, c2;
              if (abs(S0) <= kCsR && abs(S1) <= kCsR && abs(S2) <= kCsR) {
                const double* tb = cst + 3 * ((S0 + kCsR) + kCsN * ((S1 + kCsR) + kCsN * (S2 + kCsR)));
                c0 = tb[0];
                c1 = tb[1];
                c2 = tb[2];
              } else {
                const double* C = BATCH ? A.geo[ps].C : g.C;
                c0 = cts_k(C, S0, S1, S2, 0);
                c1 = cts_k(C, S0, S1, S2, 1);
                c2 = cts_k(C, S0, S1, S2, 2);
              }
              R0 = dadd(R0, c0);
              R1 = dadd(R1, c1);
              R2 = dadd(R2, c2);
            }
          }
          if (negzero && !nz) {  // a -0 coordinate: RN(d + C'(0,0,0)) differs from d when d is -0
            R0 = add_signed_zero(R0, cst[kZc + 0]);
            R1 = add_signed_zero(R1, cst[kZc + 1]);
            R2 = add_signed_zero(R2, cst[kZc + 2]);
          }
          if (act) {
            __stcs(oR + 3 * k + 0, R0);
            __stcs(oR + 3 * k + 1, R1);
            __stcs(oR + 3 * k + 2, R2);
          }
        }
      };
      for (int j = 0; j < npass; j += kEOPasses) {  // kEOPasses passes' gathers in flight, then all written
        Ld u[kEOPasses];
#pragma unroll
        for (int t = 0; t < kEOPasses; ++t) load(32 * (j + t) + lane, u[t]);
#pragma unroll
        for (int t = 0; t < kEOPasses; ++t)
          if (t == 0 || j + t < npass) write(32 * (j + t) + lane, u[t]);
      }
      __syncwarp();
      const unsigned rest = l1 < 32 ? ownm & (~0u << l1) : 0u;  // the next run of this kernel's atoms
      l0 = rest ? __ffs(rest) - 1 : 32;
    }
  }
  if (bad) atomicOr(A.err, bad);
}

// ------------------------------------------------------------------------
// Lazy sum of 1/r^6 per atom (NL_REDUCE_INV_R6_FAST) from the neighbour
// masks of the symmetric count pass (k_sym_count<kSymMasksFix>, whose gather
// rows carry fixed-point positions: x * 2^52 as 64-bit integers).  One lane
// per sorted atom walks the atom's own pairs in the reference's traversal
// order (stencil order, sorted order within each stencil cell), one set bit
// per step, and sums 1/r2^3 over them.  R = Xj - Xi + C'S is exact in fixed
// point (two integer subtractions and the C'S table in fixed point), then a
// double-float; r2 and 1/r2^3 are double-float (relative error far below
// 1e-12), and so is the sum.  No FP64 instruction is issued per pair: FP64
// runs at a small fraction of the FP32 rate on this GPU.  When a position is
// outside the fixed-point range (|x| >= 2000 A) or an atom is exact, R takes
// the reference's FP64 operations (gpu_kernels.jl:88-91) from the sorted
// positions instead.  r2 below 1e-12 (1/r2^3 beyond the FP32 range:
// coincident or nearly coincident atoms) is evaluated in FP64 with the
// reference's formula.  Each lane stores its atom's sum: no atomics, no pair
// list, and the same result on every run.  A warp takes 32 consecutive sorted
// atoms -- a few neighbouring cells, so the neighbours' 32-byte gather rows
// mostly come from L1 -- keeps each lane's 27 mask words, stencil cell starts
// and loop-shift codes in shared memory (rows of 33 words: lanes reading the
// same word index hit distinct banks), and takes as many steps as its
// busiest lane has pairs, two pairs per lane per step.
constexpr int kLRWarps = 2;
constexpr int kLRRow = 33;
#ifndef NL_LR_MIN_BLOCKS
#define NL_LR_MIN_BLOCKS 10  // 96 registers, 10 resident blocks (0.659 against 0.684 ms with 8 at 128 registers)
#endif
#ifndef NL_LR_HALF
#define NL_LR_HALF 1  // each unordered pair once (0: every atom walks all its pairs, no atomics)
#endif
struct LRSmem {
  unsigned m[32 * kLRRow];       // mask word q of lane a at a * kLRRow + q
  unsigned st[32 * kLRRow];      // the sorted start of stencil cell q
  unsigned char cd[32 * kLRRow];  // loop shift + 1 per axis of stencil cell q (2 bits each)
};

// A C'S value in the positions' fixed point, modulo 2^64: the pair vector
// Xj - Xi + C'S is formed in wrapping 64-bit arithmetic and is small (|R| <
// 2^11 A), so only C'S modulo 2^12 A matters (2^12 * 2^52 = 2^64); the
// remainder is exact in FP64 and scaled into [-2^63, 2^63).
__device__ __forceinline__ unsigned long long fix_mod(double c) {
  if (fabs(c) < 2048.0) return (unsigned long long)__double2ll_rn(dmul(c, kFixScale));  // no reduction needed
  double r = remainder(c, 4096.0);  // exact, in [-2048, 2048]
  if (r >= 2048.0) r -= 4096.0;
  return (unsigned long long)__double2ll_rn(dmul(r, kFixScale));
}

// The C'S table in the fixed point (after the FP64 one in the workspace), once per call.
__global__ void k_cs_fix(const double* __restrict__ cs, unsigned long long* __restrict__ out) {
  for (int t = threadIdx.x; t < 3 * kCsN * kCsN * kCsN; t += blockDim.x) out[t] = fix_mod(cs[t]);
}

// v * 2^-52 (v a fixed-point value of magnitude below 2^63) as a double-float:
// three 24-bit chunks are exact floats; their sum is formed with an
// error-free two-sum and the smallest chunk added to the error term.
__device__ __forceinline__ dfloat fix_to_df(long long v) {
  const int a = int(v >> 48);
  const unsigned b = unsigned((unsigned long long)v >> 24) & 0xFFFFFFu;
  const unsigned c = unsigned(v) & 0xFFFFFFu;
  const float fa = float(a) * 0x1p-4f, fb = float(b) * 0x1p-28f, fc = float(c) * 0x1p-52f;
  const float s = fa + fb;
  const float bb = s - fa;
  const float e = ((fa - (s - bb)) + (fb - bb)) + fc;
  return df_quick(s, e);
}

template <typename TI>
__global__ void __launch_bounds__(kLRWarps * 32, NL_LR_MIN_BLOCKS) k_lazy_rows(PairArgs<TI> A) {
  if (*A.sym_fail != 0) return;  // a crowded cell: the per-cell passes sum instead
  __shared__ LRSmem sm[kLRWarps];
  // the FP64 C'S table (only the FP64 pairs read it) through L1, the fixed-point
  // one in shared memory (0.762 against 0.766 ms with both in shared memory)
  const double* cs_blk = A.cs_table;
  __shared__ unsigned long long cs_fix[3 * kCsN * kCsN * kCsN];
  const Geometry& g = A.g;
  const unsigned long long* cs_fix_g = reinterpret_cast<const unsigned long long*>(A.cs_table + kCsTableDoubles);
  for (int t = threadIdx.x; t < 3 * kCsN * kCsN * kCsN; t += blockDim.x) cs_fix[t] = cs_fix_g[t];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  LRSmem& W = sm[warp];
  unsigned* wm = W.m + lane * kLRRow;
  unsigned* wst = W.st + lane * kLRRow;
  unsigned char* wcd = W.cd + lane * kLRRow;
  const int nat = g.nat;
  const int sw = *A.sym_wound;
  const bool plain = (sw & 1) == 0;   // no atom has a winding or is exact: S = the loop shift
  const bool negzero = (sw & 2) != 0;  // a coordinate is -0 (FP64 pairs: the signed-zero rule for S = 0)
  const bool fixed = (sw & 4) == 0;    // every position is in the fixed-point range, no atom is exact
  const unsigned* masks = reinterpret_cast<const unsigned*>(A.lists);
  const unsigned long long keep = l2_keep_policy();
  const double* zc = cs_blk + 3 * ((kCsN * kCsN + kCsN + 1) * kCsR);  // C'(0,0,0): signed zeros
  unsigned bad = 0;
  const long long nwarps = (long long)gridDim.x * kLRWarps;
  for (long long s0 = ((long long)blockIdx.x * kLRWarps + warp) * 32; s0 < nat; s0 += nwarps * 32) {
    const bool own = s0 + lane < nat;
    const int slot = int(min(s0 + lane, (long long)nat - 1));
    const int hc = clampi(A.scell[slot], g.ncells - 1);
    int n = 0;        // the atom's pairs
    unsigned ne = 0;  // its non-empty words
    {
      // the masks and the home cell's stencil table row (first slot of each
      // stencil cell, ~0 outside an open axis; loop shifts per axis)
      uint4 mv[7], sv[7];
      const uint4* mrow = reinterpret_cast<const uint4*>(masks + kMaskStride * slot);
      const uint4* srow = reinterpret_cast<const uint4*>(A.stab + 28LL * hc);
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        mv[k] = own ? ld_stream(mrow + k) : make_uint4(0u, 0u, 0u, 0u);
        sv[k] = own ? __ldg(srow + k) : make_uint4(0u, 0u, 0u, 0u);
      }
      const unsigned shw = sv[6].w;
#pragma unroll
      for (int q = 0; q < 27; ++q) {
        wst[q] = min((&sv[q >> 2].x)[q & 3], unsigned(nat));
        wcd[q] = (unsigned char)(((shw >> (2 * (q % 3))) & 3u) | ((shw >> (6 + 2 * ((q / 3) % 3))) & 3u) << 2 |
                                 ((shw >> (12 + 2 * (q / 9))) & 3u) << 4);
      }
      const int me = slot - int(wst[13]);  // the atom's place in its own cell (bit of the centre word)
#pragma unroll
      for (int q = 0; q < 27; ++q) {
        unsigned mq = (&mv[q >> 2].x)[q & 3];
        if (mq && wst[q] == unsigned(nat)) {  // a neighbour in a cell outside an open axis
          bad |= kFlagInconsistent;
          mq = 0u;
        }
        if (NL_LR_HALF) {  // each unordered pair from one side: forward cells, and later atoms of the centre
          if (q < 13) mq = 0u;
          if (q == 13) mq &= me >= 0 && me < 32 ? ~((2u << me) - 1u) : 0u;
        }
        wm[q] = mq;
        ne |= unsigned(mq != 0u) << q;
        n += __popc(mq);
      }
    }
    const XPack xp = A.xpk[slot];
    const unsigned mi = xp.meta;
    long long xf[3];  // fixed-point position
    double xi[3];     // FP64 position (FP64 pairs)
    xf[0] = __double_as_longlong(xp.x);
    xf[1] = __double_as_longlong(xp.y);
    xf[2] = __double_as_longlong(xp.z);
    xi[0] = xi[1] = xi[2] = 0.0;
    if (!fixed) {
      xi[0] = A.Xs[3LL * slot + 0];
      xi[1] = A.Xs[3LL * slot + 1];
      xi[2] = A.Xs[3LL * slot + 2];
    }
    // the current word of the walk
    unsigned w = 0u, stq = 0u, cq = 0u;
    auto next_word = [&]() {
      const int q = __ffs(ne) - 1;
      ne &= ne - 1u;
      w = wm[q];
      stq = wst[q];
      cq = wcd[q];
    };
    if (ne) next_word();
    auto take = [&](bool on, int& j, unsigned& c) {
      j = 0;
      c = 21u;  // no loop shift
      if (on) {
        j = int(stq) + __ffs(w) - 1;
        c = cq;
        w &= w - 1u;
        if (w == 0u && ne) next_word();
      }
    };
    dfloat acc = {0.f, 0.f};
    double accd = 0.0;  // the FP64-evaluated terms
    // 1/r2^3 of the pair (atom, j) with loop-shift code c (0 when !on): a
    // double-float, or (r2 below 1e-12) an FP64 value in fr
    auto term = [&](bool on, int j, unsigned c, const double2& w0, const int4& w1, double& fr) -> dfloat {
      fr = 0.0;
      int S[3] = {int(c & 3u) - 1, int((c >> 2) & 3u) - 1, int((c >> 4) & 3u) - 1};
      dfloat r2 = {0.f, 0.f};
      double R[3];
      if (fixed) {
        if (!plain) {  // windings (no exact atoms here): S = s_loop + wi - wj
          const unsigned cw = cand_word(cand_base(S[0], S[1], S[2]), unsigned(w1.w));
#pragma unroll
          for (int k = 0; k < 3; ++k) S[k] = field10(cw, k) + field10(mi, k) - 640;
        }
        // (unsigned: the differences and sums wrap modulo 2^64, the result is exact)
        unsigned long long rf[3];
        rf[0] = (unsigned long long)__double_as_longlong(w0.x) - (unsigned long long)xf[0];
        rf[1] = (unsigned long long)__double_as_longlong(w0.y) - (unsigned long long)xf[1];
        rf[2] = (((unsigned long long)unsigned(w1.y) << 32) | unsigned(w1.x)) - (unsigned long long)xf[2];
        const bool nz = on && (S[0] | S[1] | S[2]) != 0;
        if (__any_sync(0xffffffffu, nz)) {
          if (nz) {
            if (abs(S[0]) <= kCsR && abs(S[1]) <= kCsR && abs(S[2]) <= kCsR) {
              const unsigned long long* tb = cs_fix + 3 * ((S[0] + kCsR) + kCsN * ((S[1] + kCsR) + kCsN * (S[2] + kCsR)));
              rf[0] += tb[0];
              rf[1] += tb[1];
              rf[2] += tb[2];
            } else {
#pragma unroll
              for (int k = 0; k < 3; ++k) rf[k] += fix_mod(cts_k(g.C, S[0], S[1], S[2], k));
            }
          }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const dfloat d = fix_to_df((long long)rf[k]);
          r2 = df_add(r2, df_sq(d.hi, d.lo));
        }
        if (__any_sync(0xffffffffu, on && !(r2.hi >= 1e-12f))) {  // (rare) the FP64 positions for the formula
          const double xj0 = A.Xs[3LL * min(unsigned(j), unsigned(nat - 1)) + 0];
          const double xj1 = A.Xs[3LL * min(unsigned(j), unsigned(nat - 1)) + 1];
          const double xj2 = A.Xs[3LL * min(unsigned(j), unsigned(nat - 1)) + 2];
          const double xs0 = A.Xs[3LL * slot + 0], xs1 = A.Xs[3LL * slot + 1], xs2 = A.Xs[3LL * slot + 2];
          const double xa[3] = {xs0, xs1, xs2}, xb[3] = {xj0, xj1, xj2};
          pair_R(g, cs_blk, xa, xb, S[0], S[1], S[2], on, R);
        }
      } else {
        const double xj[3] = {A.Xs[3LL * min(unsigned(j), unsigned(nat - 1)) + 0],
                              A.Xs[3LL * min(unsigned(j), unsigned(nat - 1)) + 1],
                              A.Xs[3LL * min(unsigned(j), unsigned(nat - 1)) + 2]};
        if (!plain) {  // windings or exact atoms: S = s_loop + wi - wj
          int T[3];
          pair_S(g, xi, xj, mi, cand_word(cand_base(S[0], S[1], S[2]), unsigned(w1.w)), T);
          S[0] = T[0];
          S[1] = T[1];
          S[2] = T[2];
        }
        R[0] = dsub(xj[0], xi[0]);
        R[1] = dsub(xj[1], xi[1]);
        R[2] = dsub(xj[2], xi[2]);
        const bool nz = on && (S[0] | S[1] | S[2]) != 0;
        if (__any_sync(0xffffffffu, nz)) {
          if (nz) {
            double c0, c1, c2;
            if (abs(S[0]) <= kCsR && abs(S[1]) <= kCsR && abs(S[2]) <= kCsR) {
              const double* tb = cs_blk + 3 * ((S[0] + kCsR) + kCsN * ((S[1] + kCsR) + kCsN * (S[2] + kCsR)));
              c0 = tb[0];
              c1 = tb[1];
              c2 = tb[2];
            } else {
              c0 = cts_k(g.C, S[0], S[1], S[2], 0);
              c1 = cts_k(g.C, S[0], S[1], S[2], 1);
              c2 = cts_k(g.C, S[0], S[1], S[2], 2);
            }
            R[0] = dadd(R[0], c0);
            R[1] = dadd(R[1], c1);
            R[2] = dadd(R[2], c2);
          }
        }
        if (negzero && !nz) {
          R[0] = add_signed_zero(R[0], zc[0]);
          R[1] = add_signed_zero(R[1], zc[1]);
          R[2] = add_signed_zero(R[2], zc[2]);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          float h, l, cc;
          if (!split3(R[k], h, l, cc)) {  // |R_k| outside [2^-60, 2^60]
            h = __double2float_rn(R[k]);
            l = 0.f;
          }
          r2 = df_add(r2, df_sq(h, l));
        }
      }
      dfloat f = {0.f, 0.f};
      if (!on) return f;
      if (!(r2.hi >= 1e-12f)) {
        const double r2d = dot_ref(R);
        fr = __ddiv_rn(1.0, dmul(dmul(r2d, r2d), r2d));
        return f;
      }
      const dfloat y = df_rcp(r2);
      return df_mul(df_mul(y, y), y);
    };
    const int smax = __reduce_max_sync(0xffffffffu, own ? n : 0);
    for (int s = 0; s < smax; s += 2) {  // two pairs per lane: their gathers in flight together
      int j0, j1;
      unsigned c0, c1;
      const bool on0 = own && s < n, on1 = own && s + 1 < n;
      take(on0, j0, c0);
      take(on1, j1, c1);
      const XPack* p0 = A.xpk + min(unsigned(j0), unsigned(nat - 1));
      const XPack* p1 = A.xpk + min(unsigned(j1), unsigned(nat - 1));
      double2 a0, a1;
      int4 b0, b1;
      ld_row(p0, keep, a0, b0);
      ld_row(p1, keep, a1, b1);
      double r0, r1;
      const dfloat f0 = term(on0, j0, c0, a0, b0, r0), f1 = term(on1, j1, c1, a1, b1, r1);
      acc = df_add(df_add(acc, f0), f1);
      accd += r0 + r1;
      if (NL_LR_HALF) {  // the neighbour's share of the pair
        double v0 = dadd(f2d_exact(f0.hi), f2d_exact(f0.lo)), v1 = dadd(f2d_exact(f1.hi), f2d_exact(f1.lo));
        if (__any_sync(0xffffffffu, r0 != 0.0 || r1 != 0.0)) {  // (rare) FP64-evaluated terms
          v0 = dadd(v0, r0);
          v1 = dadd(v1, r1);
        }
        if (on0) atomicAdd(A.per_atom + clampi(b0.z - 1, nat - 1), v0);
        if (on1) atomicAdd(A.per_atom + clampi(b1.z - 1, nat - 1), v1);
      }
    }
    if (own) {
      const double tot = dadd(dadd(f2d_exact(acc.hi), f2d_exact(acc.lo)), accd);
      if (NL_LR_HALF)
        atomicAdd(A.per_atom + clampi(int(xp.perm) - 1, nat - 1), tot);
      else
        A.per_atom[clampi(int(xp.perm) - 1, nat - 1)] = tot;
    }
  }
  if (bad) atomicOr(A.err, bad);
}

// ------------------------------------------------------------------------
// Count pass with one thread per home atom.  Each thread walks its own
// stencil in the reference's order (dz, dy, dx; then the cell's atoms in
// sorted order), screens every candidate with the same FP32 arithmetic as
// the cell kernel (candidate v = u_j + d.b relative to the home cell's
// corner, r2 of v - u_i; FP64 decision inside the band, for exact atoms and
// for r2 == 0), counts, and appends accepted candidates to its list.  Threads
// of one home cell walk the same candidates in lockstep (one address per
// cell per load); the warp's trip count per stencil cell is the largest of
// its home cells'.
#ifndef NL_COUNT_MIN_BLOCKS
#define NL_COUNT_MIN_BLOCKS 8
#endif
constexpr int kCountThreads = 128;

template <typename TI, bool BATCH>
__global__ void __launch_bounds__(kCountThreads, NL_COUNT_MIN_BLOCKS) k_count_atoms(PairArgs<TI> A) {
  // the symmetric pass counted (batches run this pass only without it)
  if (!BATCH && (A.sym || A.sym_gate) && *A.sym_fail == 0) return;
  __shared__ unsigned dtab_blk[BATCH ? 1 : kStencilTab];
  if (!BATCH) {
    const int tx = 2 * A.g.nxyz[0] + 1, ty = 2 * A.g.nxyz[1] + 1;
    const int tn = min(kStencilTab, tx * ty * (2 * A.g.nxyz[2] + 1));
    for (int t = threadIdx.x; t < tn; t += blockDim.x)
      dtab_blk[t] = pack3(t % tx - A.g.nxyz[0], (t / tx) % ty - A.g.nxyz[1], t / (tx * ty) - A.g.nxyz[2]);
    __syncthreads();
  }
  const int list_cap = A.list_cap;
  if (A.cap_rec && blockIdx.x == 0 && threadIdx.x == 0) *A.cap_rec = list_cap;
  unsigned rechecks = 0;
  for (long long sl = (long long)blockIdx.x * blockDim.x + threadIdx.x; sl < A.nat_total;
       sl += (long long)gridDim.x * blockDim.x) {
    const int slot = int(sl);
    const int sys = BATCH ? clampi(A.cell_sys[clampi(A.scell[slot], A.ncells_total - 1)], A.nsys - 1) : 0;
    const Geometry& g = BATCH ? A.geo[sys] : A.g;
    const int abase = BATCH ? A.sys_atom[sys] : 0;
    const int coff = BATCH ? A.sys_cell[sys] + sys : 0;
    const int hl = clampi(A.scell[slot] - (BATCH ? A.sys_cell[sys] : 0), g.ncells - 1);
    const int hc0 = hl % g.ns[0] + 1, hc1 = (hl / g.ns[0]) % g.ns[1] + 1, hc2 = hl / (g.ns[0] * g.ns[1]) + 1;
    const float4 u = A.rec[slot];
    const unsigned mi = __float_as_uint(u.w);
    const int horig = clampi(A.perm[slot] - 1, g.nat - 1);
    const float lo = g.lo, hi = g.hi;
    const int sx = 2 * g.nxyz[0] + 1, sy = 2 * g.nxyz[1] + 1;
    const int nst = sx * sy * (2 * g.nxyz[2] + 1);
    const int tabn = BATCH ? 0 : kStencilTab;
    uint2* lst = A.lists ? A.lists + (long long)slot * list_cap : nullptr;
    int cnt = 0;
    // stencil cell q+1 is resolved (and its range loaded) while q is screened
    unsigned n_slp = 0;
    float n_ox = 0.f, n_oy = 0.f, n_oz = 0.f;
    int n_cs = 0, n_ce = 0;
    auto resolve = [&](int q) {
      n_cs = n_ce = 0;
      if (q >= nst) return;
      const int lin = stencil_cell(g, dtab_blk, tabn, sx, sy, hc0, hc1, hc2, q, n_slp, n_ox, n_oy, n_oz);
      if (lin < 0) return;
      n_cs = clampi(A.cell_offsets[coff + lin] - 1 + abase, A.nat_total);
      n_ce = clampi(A.cell_offsets[coff + lin + 1] - 1 + abase, A.nat_total);
    };
    resolve(0);
    for (int q = 0; q < nst; ++q) {
      const unsigned slp = n_slp;
      const float ox = n_ox, oy = n_oy, oz = n_oz;
      const int cs = n_cs, ce = n_ce;
      resolve(q + 1);
      // four candidates per step: their loads are in flight together
      for (int j0 = cs; j0 < ce; j0 += 4) {
        float4 rr[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) rr[k] = A.rec[min(j0 + k, ce - 1)];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int j = j0 + k;
          if (j >= ce) break;
          const float4 r = rr[k];
          const unsigned cw = cand_word(slp, __float_as_uint(r.w));
          const bool ex = (cw & kExactBit) != 0;
          const float nan = __int_as_float(0x7fc00000);
          const float cx = ex ? nan : r.x + ox, cy = ex ? nan : r.y + oy, cz = ex ? nan : r.z + oz;
          const float rx = cx - u.x, ry = cy - u.y, rz = cz - u.z;
          const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
          bool acc = r2 < lo && r2 > 0.f;
          if (!(r2 > hi) && !acc) {
            if (is_self(j, slot, cw, mi)) {
              acc = false;
            } else {
              ++rechecks;
              acc = exact_pair(g, A.Xs, slot, j, mi, cw);
            }
          }
          if (acc && A.half) acc = half_keep(horig, int(A.perm[j]) - 1, cw, mi);
          if (acc) {
            if (cnt < list_cap) lst[cnt] = make_uint2(unsigned(j), cw);
            ++cnt;
          }
        }
      }
    }
    A.counts[abase + horig] = cnt;
    if (A.lcount) {
      A.lcount[slot] = cnt;
      A.sorig[slot] = abase + horig;
    }
    if (cnt > list_cap) {
      // the atom's cell goes to the screening write pass, once
      const int hg = (BATCH ? A.sys_cell[sys] : 0) + hl;
      if (atomicExch(A.cell_flag + hg, 1) == 0) {
        const int uix = atomicAdd(A.n_screen_cells, 1);
        if (uix < A.ncells_total) A.screen_cells[uix] = hg;
      }
    }
  }
  if (rechecks) atomicAdd(A.stats, (unsigned long long)rechecks);
}

// ------------------------------------------------------------------------
// Lazy reduction from the count pass's lists: one thread per sorted atom
// walks its list in the reference's traversal order and accumulates
// 1 / ((r2*r2)*r2) exactly as the traversal does (for_each_neighbour with a
// sequential per-atom sum), 32 atoms per warp in parallel.  Atoms of cells
// whose lists overflowed are summed by the screening lazy pass.
__device__ __forceinline__ void pair_R_lane(const Geometry& g, const double* cs_tab, const double* xi,
                                            const double* xj, int S0, int S1, int S2, double* R) {
  R[0] = dsub(xj[0], xi[0]);
  R[1] = dsub(xj[1], xi[1]);
  R[2] = dsub(xj[2], xi[2]);
  if ((S0 | S1 | S2) != 0) {
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
    R[0] = dadd(R[0], c0);
    R[1] = dadd(R[1], c1);
    R[2] = dadd(R[2], c2);
  } else {
    const double* z = cs_tab + 3 * ((kCsN * kCsN + kCsN + 1) * kCsR);  // C'(0,0,0): signed zeros
    R[0] = add_signed_zero(R[0], z[0]);
    R[1] = add_signed_zero(R[1], z[1]);
    R[2] = add_signed_zero(R[2], z[2]);
  }
}

template <typename TI, bool BATCH>
__global__ void __launch_bounds__(128) k_lazy_lists(PairArgs<TI> A) {
  if (!BATCH && (A.sym || A.sym_gate) && *A.sym_fail == 0) return;  // the fused symmetric pass summed
  __shared__ double cs_blk[BATCH ? 1 : 3 * kCsN * kCsN * kCsN];
  if (!BATCH) {
    for (int t = threadIdx.x; t < 3 * kCsN * kCsN * kCsN; t += blockDim.x) cs_blk[t] = A.cs_table[t];
    __syncthreads();
  }
  const int K = A.list_cap;
  for (long long slot = (long long)blockIdx.x * blockDim.x + threadIdx.x; slot < A.nat_total;
       slot += (long long)gridDim.x * blockDim.x) {
    const int n = A.lcount[slot];
    if (n > K) continue;  // the screening lazy pass sums this atom
    const int sys = BATCH ? batch_system(A.sys_atom, A.nsys, int(slot)) : 0;
    const Geometry& g = BATCH ? A.geo[sys] : A.g;
    const double* cs_tab = BATCH ? A.cs_sys + 3 * kCsN * kCsN * kCsN * (long long)sys : cs_blk;
    const double xi[3] = {A.Xs[3 * slot + 0], A.Xs[3 * slot + 1], A.Xs[3 * slot + 2]};
    const unsigned mi = __float_as_uint(A.rec[slot].w);
    const uint2* lst = A.lists + slot * K;
    double acc = 0.0;
    for (int r = 0; r < n; ++r) {
      const uint2 e = lst[r];
      const int sj = clampi(int(e.x), A.nat_total - 1);
      const double xj[3] = {A.Xs[3LL * sj + 0], A.Xs[3LL * sj + 1], A.Xs[3LL * sj + 2]};
      int S[3];
      pair_S(g, xi, xj, mi, e.y, S);
      double R[3];
      pair_R_lane(g, cs_tab, xi, xj, S[0], S[1], S[2], R);
      const double r2 = dot_ref(R);
      acc = dadd(acc, __ddiv_rn(1.0, dmul(dmul(r2, r2), r2)));
    }
    A.per_atom[clampi(A.sorig[slot], A.nat_total - 1)] = acc;
  }
}

// ------------------------------------------------------------------------
// R = (X[j] - X[i]) + C'S for an existing pair list (the reference's _getR,
// cell_list.jl:525-531, over every pair; Verlet reuse recomputes R this way
// for moved atoms), and the largest squared displacement of a set of
// positions from reference positions.
template <typename TI>
__global__ void __launch_bounds__(256) k_pair_vectors(Geometry g, const double* __restrict__ X, const TI* __restrict__ pi,
                                                      const TI* __restrict__ pj, const TI* __restrict__ pS,
                                                      long long npairs, double* __restrict__ R) {
  __shared__ double cs_blk[3 * kCsN * kCsN * kCsN];
  for (int t = threadIdx.x; t < kCsN * kCsN * kCsN; t += blockDim.x) {
    const int s0 = t % kCsN - kCsR, s1 = (t / kCsN) % kCsN - kCsR, s2 = t / (kCsN * kCsN) - kCsR;
    cs_blk[3 * t + 0] = cts_k(g.C, s0, s1, s2, 0);
    cs_blk[3 * t + 1] = cts_k(g.C, s0, s1, s2, 1);
    cs_blk[3 * t + 2] = cts_k(g.C, s0, s1, s2, 2);
  }
  __syncthreads();
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npairs;
       p += (long long)gridDim.x * blockDim.x) {
    const long long i = clampi((long long)pi[p] - 1, g.nat - 1), j = clampi((long long)pj[p] - 1, g.nat - 1);
    const double xi[3] = {X[3 * i + 0], X[3 * i + 1], X[3 * i + 2]};
    const double xj[3] = {X[3 * j + 0], X[3 * j + 1], X[3 * j + 2]};
    double r[3];
    pair_R_lane(g, cs_blk, xi, xj, int(pS[3 * p + 0]), int(pS[3 * p + 1]), int(pS[3 * p + 2]), r);
    R[3 * p + 0] = r[0];
    R[3 * p + 1] = r[1];
    R[3 * p + 2] = r[2];
  }
}

__global__ void __launch_bounds__(256) k_max_disp_sq(const double* __restrict__ X, const double* __restrict__ Xref,
                                                     long long nat, unsigned long long* __restrict__ out) {
  double m = 0.0;
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a < nat; a += (long long)gridDim.x * blockDim.x) {
    const double d0 = X[3 * a + 0] - Xref[3 * a + 0], d1 = X[3 * a + 1] - Xref[3 * a + 1],
                 d2 = X[3 * a + 2] - Xref[3 * a + 2];
    const double d = d0 * d0 + d1 * d1 + d2 * d2;
    m = (d > m || d != d) ? d : m;  // a NaN displacement forces a rebuild
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, m, o);
    m = (v > m || v != v) ? v : m;
  }
  // non-negative doubles (and NaN) order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

template <typename TI>
void launch_pair_vectors(const Geometry& g, const double* X, const TI* pi, const TI* pj, const TI* pS,
                         long long npairs, double* R, int num_sms, cudaStream_t st) {
  if (npairs <= 0) return;
  long long b = (npairs + 255) / 256;
  if (b > (long long)num_sms * 8) b = (long long)num_sms * 8;
  k_pair_vectors<TI><<<int(b), 256, 0, st>>>(g, X, pi, pj, pS, npairs, R);
}

void launch_max_disp_sq(const double* X, const double* Xref, long long nat, unsigned long long* out, int num_sms,
                        cudaStream_t st) {
  if (nat <= 0) return;
  long long b = (nat + 255) / 256;
  if (b > (long long)num_sms * 8) b = (long long)num_sms * 8;
  k_max_disp_sq<<<int(b), 256, 0, st>>>(X, Xref, nat, out);
}

template void launch_pair_vectors<int32_t>(const Geometry&, const double*, const int32_t*, const int32_t*,
                                           const int32_t*, long long, double*, int, cudaStream_t);
template void launch_pair_vectors<int64_t>(const Geometry&, const double*, const int64_t*, const int64_t*,
                                           const int64_t*, long long, double*, int, cudaStream_t);

template <typename TI, bool BATCH>
static void launch_modes(int mode, const PairArgs<TI>& a, int num_sms, cudaStream_t st) {
  if (a.nat_total <= 0 || a.ncells_total <= 0) return;
  // grids: the tuned number of blocks per SM, by default twice (count) and
  // four times (write) the resident ones, so that the tail of uneven cells
  // and atoms balances over the SMs; every kernel walks its cells / atoms in
  // a grid-stride loop
  const int pbps = a.pair_blocks_per_sm > 0 ? a.pair_blocks_per_sm : 2 * kMinBlocks;
  const int ebps = a.emit_blocks_per_sm > 0 ? a.emit_blocks_per_sm : 4 * kEmitMinBlocks;
  long long blocks = ((long long)a.ncells_total + kPairWarps - 1) / kPairWarps;
  if (blocks > (long long)num_sms * pbps) blocks = (long long)num_sms * pbps;
  if (blocks < 1) blocks = 1;
  switch (mode) {
    case kModeCount:
      if (a.sym) {  // symmetric pass; the per-cell pass below counts what it gave up (or left)
        // (default grid: twice the resident blocks; batches 14 per SM: 3.31
        // against 3.47 ms per 4,096-system batch with 10)
        const int sbps = a.pair_blocks_per_sm > 0 ? a.pair_blocks_per_sm : BATCH ? 14 : 2 * NL_SC_MIN_BLOCKS;
        long long sb = ((long long)a.ncells_total + kSCWarps - 1) / kSCWarps;
        if (sb > (long long)num_sms * sbps) sb = (long long)num_sms * sbps;
        k_sym_count<TI, kSymMasks, BATCH><<<int(sb), kSCWarps * 32, 0, st>>>(a);
      }
      if (a.count_kernel != 2) {  // default: one warp per home cell
        k_pairs<TI, kModeCount, BATCH><<<int(blocks), kPairWarps * 32, 0, st>>>(a);
        if (BATCH && a.sym && a.nonsym_cells && a.rounds) {  // the rounds the first launch listed
          PairArgs<TI> r = a;
          r.round_pass = 1;
          k_pairs<TI, kModeCount, BATCH><<<int(blocks), kPairWarps * 32, 0, st>>>(r);
        }
      } else {
        const int cbps = a.pair_blocks_per_sm > 0 ? a.pair_blocks_per_sm : NL_COUNT_MIN_BLOCKS;
        long long cb = ((long long)a.nat_total + kCountThreads - 1) / kCountThreads;
        if (cb > (long long)num_sms * cbps) cb = (long long)num_sms * cbps;
        k_count_atoms<TI, BATCH><<<int(cb), kCountThreads, 0, st>>>(a);
      }
      break;
    case kModeFill: {
      if (!BATCH) k_cs_table<<<1, 128, 0, st>>>(a.g, a.cs_table, a.cap_rec, a.list_cap, a.err);
      if (a.list_cap > 0) {
        long long eb = ((long long)a.nat_total + 32 * kEmitWarps - 1) / (32 * kEmitWarps);
        if (eb > (long long)num_sms * ebps) eb = (long long)num_sms * ebps;
        k_emit<TI, BATCH><<<int(eb), kEmitWarps * 32, 0, st>>>(a);
        if (!BATCH || a.sym) {  // masks: written in original atom order
          const int obps = a.emit_blocks_per_sm > 0 ? a.emit_blocks_per_sm : 2 * NL_EO_MIN_BLOCKS;
          long long ob = ((long long)a.nat_total + 32 * kEOWarps - 1) / (32 * kEOWarps);
          if (ob > (long long)num_sms * obps) ob = (long long)num_sms * obps;
          k_emit_orig<TI, BATCH><<<int(ob), kEOWarps * 32, 0, st>>>(a);
        }
      }
      k_pairs<TI, kModeFill, BATCH><<<int(blocks), kPairWarps * 32, 0, st>>>(a);
      break;
    }
    default:
      if (!BATCH) k_cs_table<<<1, 128, 0, st>>>(a.g, a.cs_table, nullptr, 0, a.err);
      if (a.list_cap > 0) {
        long long lb = ((long long)a.nat_total + 127) / 128;
        if (lb > (long long)num_sms * 16) lb = (long long)num_sms * 16;
        k_lazy_lists<TI, BATCH><<<int(lb), 128, 0, st>>>(a);
      }
      k_pairs<TI, kModeLazyR6, BATCH><<<int(blocks), kPairWarps * 32, 0, st>>>(a);
      break;
  }
}

template <typename TI>
void launch_sym_lazy(int what, const PairArgs<TI>& a, int num_sms, cudaStream_t st) {
  if (a.nat_total <= 0 || a.ncells_total <= 0) return;
  const int sbps = a.pair_blocks_per_sm > 0 ? a.pair_blocks_per_sm : 2 * NL_SC_MIN_BLOCKS;
  long long sb = ((long long)a.ncells_total + kSCWarps - 1) / kSCWarps;
  if (sb > (long long)num_sms * sbps) sb = (long long)num_sms * sbps;
  if (what == kLazyCounts) {
    k_sym_count<TI, kSymCounts><<<int(sb), kSCWarps * 32, 0, st>>>(a);
  } else {
    k_cs_table<<<1, 128, 0, st>>>(a.g, a.cs_table, nullptr, 0, a.err);
    k_cs_fix<<<1, 128, 0, st>>>(a.cs_table, reinterpret_cast<unsigned long long*>(a.cs_table + kCsTableDoubles));
    // the neighbour masks with fixed-point gather rows, then each atom's sum from its masks
    k_sym_count<TI, kSymMasksFix><<<int(sb), kSCWarps * 32, 0, st>>>(a);
    long long lb = ((long long)a.nat_total + 32 * kLRWarps - 1) / (32 * kLRWarps);
    if (lb > (long long)num_sms * 2 * NL_LR_MIN_BLOCKS) lb = (long long)num_sms * 2 * NL_LR_MIN_BLOCKS;
    k_lazy_rows<TI><<<int(lb), kLRWarps * 32, 0, st>>>(a);
  }
}
template void launch_sym_lazy<int32_t>(int, const PairArgs<int32_t>&, int, cudaStream_t);
template void launch_sym_lazy<int64_t>(int, const PairArgs<int64_t>&, int, cudaStream_t);

template <typename TI>
void launch_pairs(int mode, const PairArgs<TI>& a, int num_sms, cudaStream_t st) {
  if (a.nsys > 0)
    launch_modes<TI, true>(mode, a, num_sms, st);
  else
    launch_modes<TI, false>(mode, a, num_sms, st);
}

void launch_cs_tables(const Geometry* geo, int nsys, double* out, cudaStream_t st) {
  if (nsys > 0) k_cs_tables<<<nsys, 128, 0, st>>>(geo, out);
}

// Batches: the system of every cell (one block per system).
__global__ void k_cell_systems(const int* __restrict__ sys_cell, int* __restrict__ out) {
  const int s = blockIdx.x;
  for (int c = sys_cell[s] + threadIdx.x; c < sys_cell[s + 1]; c += blockDim.x) out[c] = s;
}

void launch_cell_systems(const int* sys_cell, int nsys, int* out, cudaStream_t st) {
  if (nsys > 0) k_cell_systems<<<nsys, 128, 0, st>>>(sys_cell, out);
}

template void launch_pairs<int32_t>(int, const PairArgs<int32_t>&, int, cudaStream_t);
template void launch_pairs<int64_t>(int, const PairArgs<int64_t>&, int, cudaStream_t);

}  // namespace nl
