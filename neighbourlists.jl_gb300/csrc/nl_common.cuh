// Shared definitions of the sm_103a neighbour-list engine.
//
// Geometry conventions follow NeighbourLists.jl (src/types.jl, src/cell_list.jl):
// matrices are 9 doubles in column-major order (Julia SMatrix layout),
// M[r + 3*c] is row r / column c, and the ROWS of the cell are the lattice
// vectors.  All index arrays that leave the library are 1-based, in the
// index type TI (int32 or int64) chosen by the caller.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nl {

// ---------------------------------------------------------------- status --
enum Status : int {
  kOk = 0,
  kErrArg = 1,
  kErrTooManyCells = 2,
  kErrNoMem = 3,
  kErrCuda = 4,
  kErrTimeout = 5,
  kErrBadPosition = 6,
  kErrCapacity = 7,
  kErrIndexOverflow = 8,
  kErrInconsistent = 9,
};

// bits of the device-side error word (workspace)
enum : unsigned {
  kFlagBadPosition = 1u,
  kFlagTimeout = 2u,
  kFlagCapacity = 4u,
  kFlagInconsistent = 8u,
  kFlagIndexOverflow = 16u,
  kFlagBadIndex = 32u,  // an atom index given to the call is out of range
};

// ---------------------------------------------------------------- geometry --
// Everything a kernel needs about one system, passed by value.
struct Geometry {
  double C[9];     // cell, column-major, rows = lattice vectors
  double inv[9];   // inv(cell), column-major
  double cutoff_sq;
  int ns[3];       // cells per axis
  int nxyz[3];     // stencil half-width per axis
  int pbc[3];
  int ncells;      // ns[0]*ns[1]*ns[2]
  int nat;
  float b[9];      // bin vectors: b[3k + r] = float(C[k,r] / ns[k])
  float lo, hi;    // FP32 screen: accept r2 < lo, reject r2 > hi, else FP64 recheck
  float qh[9], ql[9];  // inv[m,k]*ns[k] as a float pair, index 3k + m (fast binning)
};

// Per-atom record in cell-sorted order: float4 (u.x, u.y, u.z, meta) where
// u = sum_k t_k b_k is the FP32 position relative to the lower corner of the
// atom's (wrapped) cell and meta packs the winding numbers, each biased by
// +128 into a 10-bit field (bits 0-9, 10-19, 20-29), and the exact flag (bit
// 30).  The same 10-bit field layout carries the per-candidate S base in the
// pair kernels, so that one packed subtraction yields three small integers.
constexpr unsigned kMetaExact = 1u << 30;
constexpr unsigned kMetaFields = (1u << 30) - 1u;
__host__ __device__ inline unsigned pack10(int a, int b, int c) {
  return (unsigned(a) & 1023u) | ((unsigned(b) & 1023u) << 10) | ((unsigned(c) & 1023u) << 20);
}
__host__ __device__ inline int field10(unsigned m, int k) { return int((m >> (10 * k)) & 1023u); }
__host__ __device__ inline unsigned pack_meta(int w0, int w1, int w2, bool exact) {
  return pack10(w0 + 128, w1 + 128, w2 + 128) | (exact ? kMetaExact : 0u);
}
__host__ __device__ inline int meta_w(unsigned m, int k) { return field10(m, k) - 128; }
__host__ __device__ inline bool meta_exact(unsigned m) { return (m & kMetaExact) != 0u; }

// Atoms whose cell-local coordinate |t_k| exceeds this (open-axis atoms far
// outside the box), whose |frac*n| exceeds kMaxY, or whose winding does not
// fit in 8 bits are "exact" atoms: every candidate pair involving them is
// decided in FP64 with the reference arithmetic.
constexpr double kMaxT = 2.0;
constexpr double kMaxY = 65536.0;
// |frac*n| beyond this cannot be binned (the reference's unsafe_trunc is
// undefined there); such positions raise kErrBadPosition.
constexpr double kBadY = 1073741824.0;  // 2^30

// ----------------------------------------------------------- FP64 helpers --
// Round-to-nearest operations that nvcc never contracts into FMA: the
// reference (Julia, no @fastmath) rounds every product and sum separately.
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// frac = inv' * x  (StaticArrays unrolled mat-vec: (a1*b1 + a2*b2) + a3*b3),
// cell_list.jl:68.
__device__ __forceinline__ double frac_k(const double* inv, double x0, double x1, double x2, int k) {
  return dadd(dadd(dmul(inv[3 * k + 0], x0), dmul(inv[3 * k + 1], x1)), dmul(inv[3 * k + 2], x2));
}

// (C' * S)_k for integer S (exactly converted), left fold.
__device__ __forceinline__ double cts_k(const double* C, int s0, int s1, int s2, int k) {
  return dadd(dadd(dmul(C[3 * k + 0], double(s0)), dmul(C[3 * k + 1], double(s1))), dmul(C[3 * k + 2], double(s2)));
}

// floor division for the winding of a wrapped index (n > 0)
__device__ __forceinline__ int floordiv(int a, int n) {
  int q = a / n;
  return (a % n != 0 && ((a < 0) != (n < 0))) ? q - 1 : q;
}

// wrap_and_shift (cell_list.jl:105-120): i == wrapped + shift*n for pbc;
// clamp with zero shift otherwise.
__device__ __forceinline__ int wrap_shift(int i, int n, int pbc, int& s) {
  if (!pbc) {
    s = 0;
    return i < 1 ? 1 : (i > n ? n : i);
  }
  int w = floordiv(i - 1, n);
  s = w;
  return i - w * n;
}

// Binning of one position with the reference arithmetic (cell_list.jl:66-74,
// 126-147): y_k = frac_k*n_k, c0_k = floor(y_k + 1), (c, w) = wrap/clamp(c0).
// Also returns t_k = y_k - m_k (m_k = c_k - 1 + w_k n_k): the coordinate
// relative to the lower corner of the wrapped cell in cell units.
// Returns false for a position that cannot be binned (non-finite or |y|>2^30).
struct Binned {
  int c[3];      // 1-based wrapped/clamped cell index
  int w[3];      // winding
  float t[3];    // cell-local coordinate (cell units), rounded to FP32
  bool exact;    // route through the FP64 path
};

__device__ __forceinline__ bool bin_position(const Geometry& g, double x0, double x1, double x2, Binned& o) {
  bool ok = true, exact = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double f = frac_k(g.inv, x0, x1, x2, k);
    double y = dmul(f, double(g.ns[k]));
    double yp = dadd(y, 1.0);
    if (!(fabs(yp) < kBadY)) {  // also catches NaN
      ok = false;
      yp = 1.0;
      y = 0.0;
    }
    int c0 = int(__double2ll_rd(yp));
    int s;
    int c = wrap_shift(c0, g.ns[k], g.pbc[k], s);
    o.c[k] = c;
    o.w[k] = s;
    long long m = (long long)(c - 1) + (long long)s * (long long)g.ns[k];
    double t = dsub(y, double(m));
    o.t[k] = __double2float_rn(t);
    if (!(fabs(t) <= kMaxT) || !(fabs(y) <= kMaxY) || s > 127 || s < -127) exact = true;
  }
  o.exact = exact;
  return ok;
}

// ---------------------------------------------------------- fast binning --
// Splits a double exactly into three floats (x = a + b + c) with integer
// operations.  Returns false for zero-free values outside [2^-60, 2^60] and
// for non-finite values (the caller then bins in FP64).
__device__ __forceinline__ bool split3(double x, float& a, float& b, float& c) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  if ((bits << 1) == 0ull) {
    a = b = c = 0.f;
    return true;
  }
  const int e = int((bits >> 52) & 0x7FF);
  if (e < 1023 - 60 || e > 1023 + 60) return false;
  const unsigned sign = unsigned(bits >> 32) & 0x80000000u;
  const unsigned long long m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
  const unsigned hi24 = unsigned(m >> 29);            // top 24 bits, leading bit at 23
  const unsigned r = unsigned(m & ((1u << 29) - 1));  // remaining 29 bits
  a = __uint_as_float(sign | (unsigned(e - 896) << 23) | (hi24 & 0x7FFFFFu));
  const float rf = __uint2float_rn(r);                // r rounded to 24 bits
  const int low = int(r - __float2uint_rn(rf));       // |low| <= 16, exact
  const float scale = __uint_as_float(unsigned(e - 1075 + 127) << 23);  // 2^(e-1075)
  b = __uint_as_float(__float_as_uint(rf * scale) | sign);
  c = __uint_as_float(__float_as_uint(float(low) * scale) ^ sign);
  return true;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Cell index, winding and cell-local coordinate from a double-float
// evaluation of y_k = sum_m inv[m,k] x_m n_k on the FP32 pipe (relative error
// about 2^-44).  The cell index equals the reference's floor(frac*n + 1)
// whenever the fractional part of y + 1 is farther than `margin` from an
// integer; otherwise (and for out-of-range values) this returns false and the
// caller bins with the reference's FP64 arithmetic (bin_position).
__device__ __forceinline__ bool bin_fast(const Geometry& g, double x0, double x1, double x2, Binned& o) {
  float a[3], b[3], c[3];
  if (!split3(x0, a[0], b[0], c[0]) || !split3(x1, a[1], b[1], c[1]) || !split3(x2, a[2], b[2], c[2])) return false;
  bool exact = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float p[3], low = 0.f, mag = 0.f;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const float qh = g.qh[3 * k + m], ql = g.ql[3 * k + m];
      p[m] = qh * a[m];
      const float e = fmaf(qh, a[m], -p[m]);
      const float sm = fmaf(qh, b[m], fmaf(ql, a[m], fmaf(qh, c[m], ql * b[m])));
      low += e + sm;
      mag += fabsf(p[m]);
    }
    float s01, e01, s012, e012;
    two_sum(p[0], p[1], s01, e01);
    two_sum(s01, p[2], s012, e012);
    low += e01 + e012;
    const float yh = s012 + low;             // y = yh + yl (fast two-sum)
    const float yl = low - (yh - s012);
    if (!(fabsf(yh) < 4194304.f)) return false;  // 2^22
    const float z = yh + 1.0f;                   // exact for |yh| < 2^22
    const float fl = floorf(z);
    const float fr = (z - fl) + yl;              // fractional part of y + 1
    const float margin = fmaxf(9.5367431640625e-07f, mag * 3.637978807091713e-12f);  // 2^-20, 2^-38 * sum|terms|
    if (!(fr > margin && fr < 1.0f - margin)) return false;
    const int c0 = int(fl);
    int s;
    const int cc = wrap_shift(c0, g.ns[k], g.pbc[k], s);
    o.c[k] = cc;
    o.w[k] = s;
    const int mm = (cc - 1) + s * g.ns[k];
    const float t = (yh - float(mm)) + yl;
    o.t[k] = t;
    if (!(fabsf(t) <= float(kMaxT)) || !(fabsf(yh) <= float(kMaxY)) || s > 127 || s < -127) exact = true;
  }
  o.exact = exact;
  return true;
}

__device__ __forceinline__ float4 make_record(const Geometry& g, const Binned& bn) {
  float t0 = bn.t[0], t1 = bn.t[1], t2 = bn.t[2];
  float4 r;
  r.x = fmaf(t2, g.b[6], fmaf(t1, g.b[3], t0 * g.b[0]));
  r.y = fmaf(t2, g.b[7], fmaf(t1, g.b[4], t0 * g.b[1]));
  r.z = fmaf(t2, g.b[8], fmaf(t1, g.b[5], t0 * g.b[2]));
  bool ex = bn.exact;
  unsigned meta = pack_meta(ex ? 0 : bn.w[0], ex ? 0 : bn.w[1], ex ? 0 : bn.w[2], ex);
  r.w = __uint_as_float(meta);
  if (ex) {  // an exact atom screens as NaN: every FP32 comparison fails
    r.x = r.y = r.z = __int_as_float(0x7fc00000);
  }
  return r;
}

__device__ __forceinline__ int linear_cell(const Geometry& g, int c0, int c1, int c2) {
  // _sub2ind (cell_list.jl:83-86), 0-based result
  return (c0 - 1) + g.ns[0] * ((c1 - 1) + g.ns[1] * (c2 - 1));
}

// index type helpers
template <typename TI>
struct IndexTraits;
template <>
struct IndexTraits<int32_t> {
  static constexpr int64_t kMax = 2147483647LL;
};
template <>
struct IndexTraits<int64_t> {
  static constexpr int64_t kMax = 9223372036854775807LL;
};

}  // namespace nl
