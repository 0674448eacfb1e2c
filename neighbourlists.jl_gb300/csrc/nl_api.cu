// C ABI of the neighbour-list engine (declared in include/nlgpu.h).
//
// Host orchestration of the kernels in nl_build.cu / nl_pairs.cu, the
// restated cell analysis of the reference (analyze_cell, cell_list.jl:152-170,
// with StaticArrays' 3x3 inv/det/cross/norm operation order), and the
// rigorous half-width of the FP32 screen's FP64 recheck band.
//
// Host floating point must not be contracted into FMAs (Julia rounds every
// operation): the build passes -ffp-contract=off to the host compiler.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "nl_api_internal.h"
#include "nl_build.cuh"
#include "nl_common.cuh"
#include "nl_f32.cuh"
#include "nl_legacy.cuh"
#include "nl_pairs.cuh"
#include "nlgpu.h"

namespace {

thread_local std::string g_last_error;
thread_local nl_tuning g_tuning = {0, 0, 0};  // single-system calls of this thread


int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(NL_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// ------------------------------------------------ StaticArrays 3x3 algebra --
// T = double, or float for the single-precision path (every operation then
// rounds to Float32, as Julia's Float32 arithmetic does).
template <typename T>
void sa_cross(const T* a, const T* b, T* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename T>
T sa_dot(const T* a, const T* b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
template <typename T>
T sa_norm(const T* a) {
  return std::sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]);
}
template <typename T>
T sa_det(const T* M) {
  T c[3];
  sa_cross(M + 3, M + 6, c);
  return sa_dot(M, c);
}
// inv of a column-major 3x3: rows of the result are y0, y1, y2 with
// y0 = x1 x x2 / d, y1 = x2 x (x0/d), y2 = (x0/d) x x1, d = x0 . (x1 x x2).
template <typename T>
void sa_inv(const T* M, T* out) {
  T x0[3] = {M[0], M[1], M[2]}, x1[3] = {M[3], M[4], M[5]}, x2[3] = {M[6], M[7], M[8]};
  T y0[3], y1[3], y2[3];
  sa_cross(x1, x2, y0);
  const T d = sa_dot(x0, y0);
  for (int k = 0; k < 3; ++k) {
    x0[k] = x0[k] / d;
    y0[k] = y0[k] / d;
  }
  sa_cross(x2, x0, y1);
  sa_cross(x0, x1, y2);
  for (int c = 0; c < 3; ++c) {
    out[0 + 3 * c] = y0[c];
    out[1 + 3 * c] = y1[c];
    out[2 + 3 * c] = y2[c];
  }
}
// lengths(C) = det(C) ./ (|r2 x r3|, |r3 x r1|, |r1 x r2|), cell_list.jl:94-95
template <typename T>
void lengths(const T* C, T* lens) {
  const T r1[3] = {C[0], C[3], C[6]}, r2[3] = {C[1], C[4], C[7]}, r3[3] = {C[2], C[5], C[8]};
  const T det = sa_det(C);
  T c[3];
  sa_cross(r2, r3, c);
  lens[0] = det / sa_norm(c);
  sa_cross(r3, r1, c);
  lens[1] = det / sa_norm(c);
  sa_cross(r1, r2, c);
  lens[2] = det / sa_norm(c);
}

// ------------------------------------------------------- FP32 screen band --
// The kernel screens candidates with r2_32 = |v_j - u_i|^2 where u (per atom)
// and v = u_j + d.b (per candidate) are FP32 sums of FP64-exact cell-local
// coordinates t (|t_k| <= kMaxT for non-exact atoms) times the bin vectors b_k;
// t carries at most 2^-24 (|t| + 2) of rounding (FP32 rounding of the FP64
// value, or the double-float binning's final FP32 operations).
// Per Cartesian component r the FP32 error of R is at most
//   e_r = 2^-24 * 1.01 * ((11 T + 6) B_r + 4 O_r + |R_r|) + e64,
//   B_r = sum_k |b_kr|,  O_r = sum_k nxyz_k |b_kr|,
// where e64 = 2^-29 (1 + cond(C)) sum_k |b_k| bounds the difference between
// the reference's FP64 R and the exact R of the FP64 t values for atoms with
// |frac*n| <= kMaxY.  With |R_r| <= cutoff near the cutoff, the error of r2 is
// at most Delta = sum_r (2 rc e_r + e_r^2) + 3.03 * 2^-24 rc^2 + 2^-51 rc^2.
// The band is max(1e-5 rc^2, 2 Delta): outside it the FP32 decision equals
// the FP64 one, inside it the kernel decides in FP64.
double screen_band(const double* C, const double* inv, const int64_t* ns, const int64_t* nxyz, double rc) {
  const double eps = std::ldexp(1.0, -24);
  double b[3][3], B[3] = {0, 0, 0}, O[3] = {0, 0, 0}, bsum = 0;
  for (int k = 0; k < 3; ++k) {
    double nk = 0;
    for (int r = 0; r < 3; ++r) {
      b[k][r] = C[k + 3 * r] / double(ns[k]);
      B[r] += std::fabs(b[k][r]);
      O[r] += double(nxyz[k]) * std::fabs(b[k][r]);
      nk += b[k][r] * b[k][r];
    }
    bsum += std::sqrt(nk);
  }
  double cn = 0, in = 0;  // infinity norms
  for (int r = 0; r < 3; ++r) {
    double rc_ = 0, ri = 0;
    for (int c = 0; c < 3; ++c) {
      rc_ += std::fabs(C[r + 3 * c]);
      ri += std::fabs(inv[r + 3 * c]);
    }
    cn = std::fmax(cn, rc_);
    in = std::fmax(in, ri);
  }
  const double cond = cn * in;
  const double e64 = std::ldexp(1.0, -29) * (1.0 + cond) * bsum;
  const double T = nl::kMaxT;
  double delta = 0;
  for (int r = 0; r < 3; ++r) {
    const double e = eps * 1.01 * ((11 * T + 6) * B[r] + 4 * O[r] + rc) + e64;
    delta += 2 * rc * e + e * e;
  }
  delta += 3.03 * eps * rc * rc + std::ldexp(1.0, -51) * rc * rc;
  return std::fmax(1e-5 * rc * rc, 2 * delta);
}

int analyze(const double* cell, double cutoff, int index_bytes, nl_cell_plan* p) {
  if (!(cutoff > 0) || !std::isfinite(cutoff)) return fail(NL_ERR_ARG, "cutoff must be positive and finite");
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  sa_inv(cell, p->inv_cell);
  lengths(cell, p->lens);
  const double tmax = index_bytes == 4 ? 2147483647.0 : 9223372036854775807.0;
  long double prod = 1;
  for (int k = 0; k < 3; ++k) {
    p->lens[k] = std::fabs(p->lens[k]);
    const double t = std::floor(p->lens[k] / cutoff);
    if (!(t < tmax)) return fail(NL_ERR_TOO_MANY_CELLS, "Ratio of simulation cell size to cutoff is very large.");
    p->ncells[k] = t < 1 ? 1 : int64_t(t);
    prod *= (long double)p->ncells[k];
  }
  if (prod > (long double)tmax)
    return fail(NL_ERR_TOO_MANY_CELLS,
                "Ratio of simulation cell size to cutoff is very large. Use a larger integer type (e.g. Int64), "
                "larger cutoff, or smaller simulation cell.");
  if (prod > 2147483646.0L)
    return fail(NL_ERR_TOO_MANY_CELLS, "more than 2^31-2 cells: use a larger cutoff or a smaller simulation cell");
  p->ncells_total = p->ncells[0] * p->ncells[1] * p->ncells[2];
  for (int k = 0; k < 3; ++k) {
    const double v = std::ceil(cutoff * (double(p->ncells[k]) / p->lens[k]));
    if (!(v < 1e9)) return fail(NL_ERR_ARG, "degenerate cell: stencil half-width is not finite");
    p->nxyz[k] = int64_t(v);
  }
  p->band = screen_band(cell, p->inv_cell, p->ncells, p->nxyz, cutoff);
  return NL_OK;
}

// ------------------------------------------------------------- workspace --
constexpr size_t kAlign = 256;
size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct Layout {
  // [err 64 | stats 64] [pairs zero region: counters 64 | st_pairs | cell_flag]
  // [build zero region: counters 64 | st_cells | cell_count] [arrays...]
  size_t err, stats, pcount, st_pairs, cell_flag, pend, bcount, st_cells, cell_count, bend;
  size_t totals, cell_start, cid, ticket, rec, tmp, rec_sorted, scell, counts, lcount, sorig, orow, xpk, cs_table,
      screen_cells,
      big_list, base_end, stab, lists, end;
  bool use_lists = true;  // the workspace holds the pair lists (it reaches `end`)
};

Layout layout(int64_t nat, int64_t ncells) {
  Layout L;
  size_t o = 0;
  L.err = o;
  L.stats = o + 64;
  o += 128;
  L.pcount = o;
  o += 64;
  L.st_pairs = o;
  o += up(sizeof(unsigned long long) * size_t(nl::scan_tiles(nat > 0 ? nat : 1)));
  L.cell_flag = o;
  o += up(sizeof(int) * size_t(ncells > 0 ? ncells : 1));
  L.pend = o;
  L.bcount = o;
  o += 64;
  L.st_cells = o;
  o += up(sizeof(unsigned long long) * size_t(nl::scan_tiles(ncells > 0 ? ncells : 1)));
  L.cell_count = o;
  o += up(sizeof(int) * size_t(ncells));
  L.bend = o;
  L.totals = o;
  o += 64;
  L.cell_start = o;
  o += up(sizeof(int) * size_t(ncells + 1));
  const size_t n = size_t(nat > 0 ? nat : 1);
  L.cid = o;
  o += up(sizeof(int) * n);
  L.ticket = o;
  o += up(sizeof(int) * n);
  L.rec = o;
  o += up(sizeof(float4) * n);
  L.tmp = o;
  o += up(sizeof(int) * n);
  L.rec_sorted = o;
  o += up(sizeof(float4) * n);
  L.scell = o;
  o += up(sizeof(int) * n);
  L.counts = o;
  o += up(sizeof(int) * n);
  L.lcount = o;
  o += up(sizeof(int) * n);
  L.sorig = o;
  o += up(sizeof(int) * n);
  L.cs_table = o;  // C'S for |S_k| <= 2 in FP64, then (lazy sums) in the positions' fixed point
  o += up(sizeof(double) * 2 * 3 * 125);
  L.screen_cells = o;
  o += up(sizeof(int) * size_t(ncells > 0 ? ncells : 1));
  L.big_list = o;
  o += up(sizeof(int) * size_t(ncells < (int64_t)n ? ncells : (int64_t)n));
  // the pair lists come last: a workspace that ends before them still runs
  // every call, with the screening write pass for every cell
  L.base_end = o;
  // the symmetric passes' rows and tables (they run only with the lists):
  // per original atom its row (ORow), per sorted slot its gather row
  // (XPack), per cell the lazy sum's stencil table (28 words)
  L.orow = o;
  o += up(sizeof(nl::ORow) * n);
  L.xpk = o;
  o += up(sizeof(nl::XPack) * n);
  L.stab = o;
  o += up(sizeof(unsigned) * 28 * size_t(ncells > 0 ? ncells : 1));
  L.lists = o;
  o += up(sizeof(uint2) * size_t(nl::kListCap) * n);
  L.end = o;
  return L;
}

template <typename T>
T* at(void* ws, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

int num_sms() {
  // per device, filled on first use; concurrent first calls store the same value
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (!v) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    v = n > 0 ? n : 148;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

struct Pinned {
  long long* p = nullptr;
  Pinned() { cudaHostAlloc(reinterpret_cast<void**>(&p), 64, cudaHostAllocDefault); }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};
long long* pinned_scratch() {
  thread_local Pinned pin;
  return pin.p;
}

int check_common(int64_t nat, const int64_t* ncells, const int64_t* nxyz, int index_bytes, void* ws,
                 size_t ws_bytes, Layout& L, int64_t& ncells_total) {
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  if (nat < 0 || nat > 2147483646LL) return fail(NL_ERR_ARG, "nat must be in [0, 2^31-2]");
  long double prod = 1;
  for (int k = 0; k < 3; ++k) {
    if (ncells[k] < 1) return fail(NL_ERR_ARG, "ncells must be >= 1");
    prod *= (long double)ncells[k];
    if (nxyz && (nxyz[k] < 0 || nxyz[k] > 62))
      return fail(NL_ERR_ARG, "stencil half-width nxyz must be in [0, 62] (cutoff at most 62 cell widths)");
  }
  if (prod > 2147483646.0L) return fail(NL_ERR_TOO_MANY_CELLS, "more than 2^31-2 cells");
  if (index_bytes == 4 && prod > 2147483647.0L)
    return fail(NL_ERR_TOO_MANY_CELLS, "Ratio of simulation cell size to cutoff is very large.");
  ncells_total = int64_t(prod);
  L = layout(nat, ncells_total);
  if (!ws || ws_bytes < L.base_end) return fail(NL_ERR_NOMEM, "workspace too small (see nl_workspace_bytes)");
  // list entries are addressed with 32-bit offsets
  L.use_lists = ws_bytes >= L.end && (unsigned long long)nat * nl::kListCap < (1ull << 32);
  return NL_OK;
}

nl::Geometry make_geometry(const double* cell, const double* inv, const int64_t* ns, const int64_t* nxyz,
                           const uint8_t* pbc, double cutoff, int64_t nat) {
  nl::Geometry g;
  std::memcpy(g.C, cell, sizeof(g.C));
  std::memcpy(g.inv, inv, sizeof(g.inv));
  g.cutoff_sq = cutoff * cutoff;
  for (int k = 0; k < 3; ++k) {
    g.ns[k] = int(ns[k]);
    g.nxyz[k] = nxyz ? int(nxyz[k]) : 0;
    g.pbc[k] = pbc[k] ? 1 : 0;
    for (int r = 0; r < 3; ++r) g.b[3 * k + r] = float(cell[k + 3 * r] / double(ns[k]));
  }
  g.ncells = int(ns[0] * ns[1] * ns[2]);
  g.nat = int(nat);
  double band = 0;
  if (nxyz) {
    band = screen_band(cell, inv, ns, nxyz, cutoff);
  }
  const double lo = g.cutoff_sq - band, hi = g.cutoff_sq + band;
  float flo = float(lo), fhi = float(hi);
  if (double(flo) > lo) flo = std::nextafter(flo, -INFINITY);
  if (double(fhi) < hi) fhi = std::nextafter(fhi, INFINITY);
  g.lo = lo > 0 ? flo : -1.0f;  // lo <= 0: every candidate is rechecked
  g.hi = fhi;
  // inv[m,k] * ns[k] as a float pair for the double-float binning
  for (int k = 0; k < 3; ++k)
    for (int m = 0; m < 3; ++m) {
      const double q = inv[3 * k + m] * double(ns[k]);
      const float qh = float(q);
      g.qh[3 * k + m] = qh;
      g.ql[3 * k + m] = float(q - double(qh));
    }
  return g;
}

int status_from_flags(unsigned f) {
  if (f & nl::kFlagBadPosition)
    return fail(NL_ERR_BAD_POSITION, "non-finite position or |frac * ncells| >= 2^30 (cannot be binned)");
  if (f & nl::kFlagInconsistent) return fail(NL_ERR_INCONSISTENT, "cell list ids do not match its positions");
  if (f & nl::kFlagTimeout) return fail(NL_ERR_TIMEOUT, "a bounded device-side wait timed out");
  if (f & nl::kFlagIndexOverflow) return fail(NL_ERR_INDEX_OVERFLOW, "pair count does not fit the index type");
  if (f & nl::kFlagBadIndex) return fail(NL_ERR_ARG, "an atom index given to the call is out of range");
  if (f & nl::kFlagCapacity) return fail(NL_ERR_CAPACITY, "pair buffers are smaller than the pair count");
  return NL_OK;
}

// read err word (and optionally a total) after synchronising; clears err
int sync_read(void* ws, cudaStream_t st, const long long* d_total, int64_t* total) {
  long long* h = pinned_scratch();
  if (!h) return fail(NL_ERR_NOMEM, "cannot allocate pinned host scratch");
  cudaError_t e = cudaMemcpyAsync(h, ws, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && d_total) e = cudaMemcpyAsync(h + 1, d_total, sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws, 0, sizeof(unsigned), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "synchronise");
  unsigned flags = *reinterpret_cast<unsigned*>(h);
  if (d_total && total) *total = h[1];
  return status_from_flags(flags);
}

template <typename TI>
int build_impl(const double* X, int64_t nat, const nl::Geometry& g, TI* perm, double* Xs, TI* cell_id,
               TI* cell_offsets, void* ws, const Layout& L, cudaStream_t st) {
  const int sms = num_sms();
  cudaError_t e = cudaMemsetAsync(ws, 0, L.bend, st);  // err, stats, both zero regions
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  if (nat == 0) {
    // empty system: cell_offsets all ones (cell_list.jl:731-734) -- the scan
    // of the (zeroed) histogram produces exactly that
    nl::launch_scan<TI>(at<int>(ws, L.cell_count), g.ncells, cell_offsets, at<int>(ws, L.cell_start),
                        at<unsigned long long>(ws, L.st_cells), at<int>(ws, L.bcount), at<long long>(ws, L.totals),
                        at<unsigned>(ws, L.err), st);
    e = cudaGetLastError();
    return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch");
  }
  int* cid = at<int>(ws, L.cid);
  int* ticket = at<int>(ws, L.ticket);
  float4* rec = at<float4>(ws, L.rec);
  int* cell_count = at<int>(ws, L.cell_count);
  int* cell_start = at<int>(ws, L.cell_start);
  unsigned* err = at<unsigned>(ws, L.err);
  int* bcount = at<int>(ws, L.bcount);
  const nl::SysIndex single{nullptr, nullptr, nullptr, 0};
  nl::launch_bin(g, single, X, int(nat), cid, ticket, rec, cell_count, err, sms, st);
  nl::launch_scan<TI>(cell_count, g.ncells, cell_offsets, cell_start, at<unsigned long long>(ws, L.st_cells), bcount,
                      at<long long>(ws, L.totals), err, st);
  nl::launch_scatter(int(nat), cid, ticket, cell_start, at<int>(ws, L.tmp), sms, st);
  nl::launch_fix<TI>(single, int(nat), at<int>(ws, L.tmp), cid, cell_start, X, rec, perm, cell_id, Xs,
                     at<float4>(ws, L.rec_sorted), at<int>(ws, L.scell), at<int>(ws, L.big_list), bcount + 1, sms, st);
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch build kernels");
}

template <typename TI>
nl::PairArgs<TI> pair_args(const nl::Geometry& g, const TI* cell_offsets, const TI* perm, const double* Xs, void* ws,
                           const Layout& L) {
  nl::PairArgs<TI> a;
  std::memset(&a, 0, sizeof(a));
  a.g = g;
  a.nat_total = g.nat;
  a.ncells_total = g.ncells;
  a.cell_offsets = cell_offsets;
  a.perm = perm;
  a.Xs = Xs;
  a.rec = at<float4>(ws, L.rec_sorted);
  a.scell = at<int>(ws, L.scell);
  a.list_cap = L.use_lists ? nl::kListCap : 0;
  a.lists = L.use_lists ? at<uint2>(ws, L.lists) : nullptr;
  a.stab = L.use_lists ? at<unsigned>(ws, L.stab) : nullptr;
  a.lcount = at<int>(ws, L.lcount);
  a.sorig = at<int>(ws, L.sorig);
  a.orow = L.use_lists ? at<nl::ORow>(ws, L.orow) : nullptr;
  a.xpk = L.use_lists ? at<nl::XPack>(ws, L.xpk) : nullptr;
  a.cap_rec = at<int>(ws, L.pcount) + 2;  // the count pass's list_cap, checked by the write pass
  a.cs_table = at<double>(ws, L.cs_table);
  a.screen_cells = at<int>(ws, L.screen_cells);
  a.n_screen_cells = at<int>(ws, L.pcount) + 4;  // zeroed with the pair scan state
  a.sym_fail = at<int>(ws, L.pcount) + 6;        // likewise
  a.sym_wound = at<int>(ws, L.pcount) + 7;       // likewise
  a.cell_flag = at<int>(ws, L.cell_flag);     // likewise
  a.count_kernel = g_tuning.count_kernel;
  a.pair_blocks_per_sm = g_tuning.pair_blocks_per_sm;
  a.emit_blocks_per_sm = g_tuning.emit_blocks_per_sm;
  a.stats = at<unsigned long long>(ws, L.stats);
  a.err = at<unsigned>(ws, L.err);
  return a;
}

// The symmetric count pass and the mask write pass (nl_pairs.cu) apply to a
// full or half list of a single system with per-atom lists in the workspace
// and a 27-cell stencil of distinct cells (nxyz = 1, periodic axes of at
// least 3 cells); count_kernel 1 or 2 selects the per-cell / per-atom pass.
// The stencil is 27 distinct cells: nxyz = 1 on every axis and periodic axes
// of at least 3 cells (the symmetric passes' condition on the geometry).
bool sym_geometry(const nl::Geometry& g) {
  bool sym = true;
  for (int k = 0; k < 3; ++k) sym = sym && g.nxyz[k] == 1 && (!g.pbc[k] || g.ns[k] >= 3);
  return sym;
}

bool use_sym(const nl::Geometry& g, const Layout& L) {
  // masks (27 words per atom) and the stencil table (54 words per cell) share the list region
  const bool fits = 27.0 * g.nat + 54.0 * g.ncells <= 2.0 * nl::kListCap * g.nat;
  bool sym = L.use_lists && fits && g_tuning.count_kernel != 1 && g_tuning.count_kernel != 2;
  for (int k = 0; k < 3; ++k) sym = sym && g.nxyz[k] == 1 && (!g.pbc[k] || g.ns[k] >= 3);
  return sym;
}

template <typename TI>
int count_impl(const nl::Geometry& g, const double* Xs, const TI* perm, const TI* cell_id, const TI* cell_offsets,
               int reuse, TI* first, void* ws, const Layout& L, cudaStream_t st, int half = 0) {
  const int sms = num_sms();
  // reuse: keep err (set by the build), reset stats and the pair scan state
  const size_t z0 = reuse ? L.stats : L.err;
  cudaError_t e = cudaMemsetAsync(static_cast<char*>(ws) + z0, 0, L.pend - z0, st);
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  if (g.nat == 0) {
    // first = [1]
    static const TI one = 1;
    e = cudaMemcpyAsync(first, &one, sizeof(TI), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? NL_OK : cuda_fail(e, "empty system");
  }
  if (!reuse)
    nl::launch_prepare<TI>(g, Xs, cell_id, perm, g.nat, at<float4>(ws, L.rec_sorted), at<int>(ws, L.scell),
                           at<unsigned>(ws, L.err), sms, st);
  nl::PairArgs<TI> a = pair_args<TI>(g, cell_offsets, perm, Xs, ws, L);
  a.counts = at<int>(ws, L.counts);
  a.half = half;
  a.sym = use_sym(g, L) ? 1 : 0;
  // the symmetric pass accumulates the counts; without it, sym_fail records
  // for the write pass that the lists are to be used
  e = a.sym ? cudaMemsetAsync(a.counts, 0, sizeof(int) * size_t(g.nat), st)
            : cudaMemsetAsync(a.sym_fail, 0xFF, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "memset counts");
  nl::launch_pairs<TI>(nl::kModeCount, a, sms, st);
  nl::launch_scan<TI>(at<int>(ws, L.counts), g.nat, first, nullptr, at<unsigned long long>(ws, L.st_pairs),
                      at<int>(ws, L.pcount), at<long long>(ws, L.totals) + 1, at<unsigned>(ws, L.err), st);
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch count kernels");
}

template <typename TI>
int fill_impl(const nl::Geometry& g, const double* Xs, const TI* perm, const TI* cell_offsets, const TI* first,
              int64_t capacity, TI* oi, TI* oj, TI* oS, double* oR, void* ws, const Layout& L, cudaStream_t st,
              int half = 0) {
  if (g.nat == 0 || capacity <= 0) return NL_OK;
  nl::PairArgs<TI> a = pair_args<TI>(g, cell_offsets, perm, Xs, ws, L);
  a.half = half;
  a.first = first;
  a.oi = oi;
  a.oj = oj;
  a.oS = oS;
  a.oR = oR;
  a.capacity = capacity;
  a.vec_ok = (reinterpret_cast<uintptr_t>(oi) % 16 == 0) && (reinterpret_cast<uintptr_t>(oj) % 16 == 0) &&
             (reinterpret_cast<uintptr_t>(oS) % 16 == 0) && (reinterpret_cast<uintptr_t>(oR) % 16 == 0);
  nl::launch_pairs<TI>(nl::kModeFill, a, num_sms(), st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch fill kernel");
}

// ------------------------------------------------- single-precision path --
// analyze_cell (cell_list.jl:152-170) and nxyz (gpu_kernels.jl:315-316) with
// T = Float32: every operation rounds to Float32.
int analyze_f32(const float* cell, float cutoff, int index_bytes, nl_cell_plan_f32* p) {
  if (!(cutoff > 0) || !std::isfinite(cutoff)) return fail(NL_ERR_ARG, "cutoff must be positive and finite");
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  sa_inv(cell, p->inv_cell);
  lengths(cell, p->lens);
  // floor(TI, x) accepts x < typemax(TI) + 1 (a power of two in Float32)
  const float tmax = index_bytes == 4 ? 2147483648.0f : 9223372036854775808.0f;
  long double prod = 1;
  for (int k = 0; k < 3; ++k) {
    p->lens[k] = std::fabs(p->lens[k]);
    const float t = std::floor(p->lens[k] / cutoff);
    if (!(t < tmax)) return fail(NL_ERR_TOO_MANY_CELLS, "Ratio of simulation cell size to cutoff is very large.");
    p->ncells[k] = t < 1 ? 1 : int64_t(t);
    prod *= (long double)p->ncells[k];
  }
  if (prod > (long double)(index_bytes == 4 ? 2147483647.0 : 9223372036854775807.0))
    return fail(NL_ERR_TOO_MANY_CELLS,
                "Ratio of simulation cell size to cutoff is very large. Use a larger integer type (e.g. Int64), "
                "larger cutoff, or smaller simulation cell.");
  if (prod > 2147483646.0L)
    return fail(NL_ERR_TOO_MANY_CELLS, "more than 2^31-2 cells: use a larger cutoff or a smaller simulation cell");
  p->ncells_total = p->ncells[0] * p->ncells[1] * p->ncells[2];
  for (int k = 0; k < 3; ++k) {
    const float v = std::ceil(cutoff * (float(p->ncells[k]) / p->lens[k]));
    if (!(v < 1e9f)) return fail(NL_ERR_ARG, "degenerate cell: stencil half-width is not finite");
    p->nxyz[k] = int64_t(v);
  }
  return NL_OK;
}

nl::Geo32 make_geo32(const float* cell, const float* inv, const int64_t* ns, const int64_t* nxyz, const uint8_t* pbc,
                     float cutoff, int64_t nat) {
  nl::Geo32 g;
  std::memset(&g, 0, sizeof(g));
  std::memcpy(g.C, cell, sizeof(g.C));
  std::memcpy(g.inv, inv, sizeof(g.inv));
  g.cutoff_sq = cutoff * cutoff;  // clist.cutoff^2 in Float32
  for (int k = 0; k < 3; ++k) {
    g.ns[k] = int(ns[k]);
    g.nxyz[k] = nxyz ? int(nxyz[k]) : 0;
    g.pbc[k] = pbc[k] ? 1 : 0;
  }
  g.ncells = int(ns[0] * ns[1] * ns[2]);
  g.nat = int(nat);
  return g;
}

template <typename TI>
int build_impl32(const float* X, int64_t nat, const nl::Geo32& g, TI* perm, float* Xs, TI* cell_id, TI* cell_offsets,
                 void* ws, const Layout& L, cudaStream_t st) {
  const int sms = num_sms();
  cudaError_t e = cudaMemsetAsync(ws, 0, L.bend, st);
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  int* cell_count = at<int>(ws, L.cell_count);
  int* cell_start = at<int>(ws, L.cell_start);
  unsigned* err = at<unsigned>(ws, L.err);
  int* bcount = at<int>(ws, L.bcount);
  if (nat > 0)
    nl::launch_bin32(g, X, int(nat), at<int>(ws, L.cid), at<int>(ws, L.ticket), at<float4>(ws, L.rec), cell_count, err,
                     sms, st);
  // an empty system scans the zeroed histogram: cell_offsets all ones
  nl::launch_scan<TI>(cell_count, g.ncells, cell_offsets, cell_start, at<unsigned long long>(ws, L.st_cells), bcount,
                      at<long long>(ws, L.totals), err, st);
  if (nat > 0) {
    const nl::SysIndex single{nullptr, nullptr, nullptr, 0};
    nl::launch_scatter(int(nat), at<int>(ws, L.cid), at<int>(ws, L.ticket), cell_start, at<int>(ws, L.tmp), sms, st);
    nl::launch_fix<TI, float>(single, int(nat), at<int>(ws, L.tmp), at<int>(ws, L.cid), cell_start, X,
                              at<float4>(ws, L.rec), perm, cell_id, Xs, at<float4>(ws, L.rec_sorted),
                              at<int>(ws, L.scell), at<int>(ws, L.big_list), bcount + 1, sms, st);
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch build kernels");
}

// the symmetric count / mask write pass of the Float32 path: as use_sym
bool use_sym32(const nl::Geo32& g, const Layout& L) {
  const bool fits = 27.0 * g.nat + 54.0 * g.ncells <= 2.0 * nl::kListCap * g.nat;
  bool sym = L.use_lists && fits && g_tuning.count_kernel != 1 && g_tuning.count_kernel != 2;
  for (int k = 0; k < 3; ++k) sym = sym && g.nxyz[k] == 1 && (!g.pbc[k] || g.ns[k] >= 3);
  return sym;
}

template <typename TI>
nl::Pairs32Args<TI> pairs32_args(const nl::Geo32& g, const TI* cell_offsets, const TI* perm, void* ws,
                                 const Layout& L, int half = 0) {
  nl::Pairs32Args<TI> a;
  std::memset(&a, 0, sizeof(a));
  a.half = half;
  a.g = g;
  a.rec = at<float4>(ws, L.rec_sorted);
  a.scell = at<int>(ws, L.scell);
  a.cell_offsets = cell_offsets;
  a.perm = perm;
  a.counts = at<int>(ws, L.counts);
  a.err = at<unsigned>(ws, L.err);
  a.sym = !half && use_sym32(g, L) ? 1 : 0;  // half lists: the per-cell passes (they filter every pair)
  a.masks = reinterpret_cast<unsigned*>(at<uint2>(ws, L.lists));
  a.sym_fail = at<int>(ws, L.pcount) + 6;  // zeroed with the pair scan state
  return a;
}

template <typename TI>
int count_impl32(const nl::Geo32& g, const float* Xs, const TI* perm, const TI* cell_id, const TI* cell_offsets,
                 int reuse, TI* first, void* ws, const Layout& L, cudaStream_t st, int half = 0) {
  const int sms = num_sms();
  const size_t z0 = reuse ? L.stats : L.err;
  cudaError_t e = cudaMemsetAsync(static_cast<char*>(ws) + z0, 0, L.pend - z0, st);
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  if (g.nat == 0) {
    static const TI one = 1;
    e = cudaMemcpyAsync(first, &one, sizeof(TI), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? NL_OK : cuda_fail(e, "empty system");
  }
  if (!reuse)
    nl::launch_prepare32<TI>(g, Xs, cell_id, perm, g.nat, at<float4>(ws, L.rec_sorted), at<int>(ws, L.scell),
                             at<unsigned>(ws, L.err), sms, st);
  const nl::Pairs32Args<TI> a = pairs32_args<TI>(g, cell_offsets, perm, ws, L, half);
  // as count_impl: counts accumulated by the symmetric pass, else the record
  e = a.sym ? cudaMemsetAsync(a.counts, 0, sizeof(int) * size_t(g.nat), st)
            : cudaMemsetAsync(a.sym_fail, 0xFF, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "memset counts");
  nl::launch_pairs32<TI>(false, a, sms, st);
  nl::launch_scan<TI>(a.counts, g.nat, first, nullptr, at<unsigned long long>(ws, L.st_pairs), at<int>(ws, L.pcount),
                      at<long long>(ws, L.totals) + 1, a.err, st);
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch count kernels");
}

template <typename TI>
int fill_impl32(const nl::Geo32& g, const TI* perm, const TI* cell_offsets, const TI* first, int64_t capacity, TI* oi,
                TI* oj, TI* oS, float* oR, void* ws, const Layout& L, cudaStream_t st, int half = 0) {
  if (g.nat == 0 || capacity <= 0) return NL_OK;
  nl::Pairs32Args<TI> a = pairs32_args<TI>(g, cell_offsets, perm, ws, L, half);
  a.first = first;
  a.oi = oi;
  a.oj = oj;
  a.oS = oS;
  a.oR = oR;
  a.capacity = capacity;
  nl::launch_pairs32<TI>(true, a, num_sms(), st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch fill kernel");
}

// ------------------------------------------------- legacy linked-list path --
// The legacy path keeps its own cell list in the workspace (the reference's
// legacy PairList does not expose it), after the sort-based layout's
// list-free part, followed by the per-slot legacy records.
struct LegacyLayout {
  Layout L;
  size_t perm, Xs, cell_id, cell_offsets, D, Df, c0, end;
};

LegacyLayout legacy_layout(int64_t nat, int64_t ncells, int index_bytes) {
  LegacyLayout Q;
  Q.L = layout(nat, ncells);
  Q.L.use_lists = false;
  const size_t n = size_t(nat > 0 ? nat : 1), ib = size_t(index_bytes);
  size_t o = Q.L.base_end;
  Q.perm = o;
  o += up(ib * n);
  Q.Xs = o;
  o += up(3 * sizeof(double) * n);
  Q.cell_id = o;
  o += up(ib * n);
  Q.cell_offsets = o;
  o += up(ib * size_t(ncells + 1));
  Q.D = o;
  o += up(3 * sizeof(double) * n);
  Q.Df = o;
  o += up(sizeof(float4) * n);
  Q.c0 = o;
  o += up(sizeof(int4) * n);
  Q.end = o;
  return Q;
}

// bins = hcat(C[1,:]/n1, C[2,:]/n2, C[3,:]/n3) (cell_list.jl:258): column k is
// row k of the cell divided by ns[k]
nl::LegacyGeo legacy_geo(const double* cell, const double* inv, const int64_t* ns, const int64_t* nxyz,
                         const uint8_t* pbc, double cutoff, int64_t nat) {
  nl::LegacyGeo g;
  std::memset(&g, 0, sizeof(g));
  std::memcpy(g.inv, inv, sizeof(g.inv));
  double offmax = 0;
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < 3; ++r) {
      g.bins[r + 3 * k] = cell[k + 3 * r] / double(ns[k]);
      g.binsf[r + 3 * k] = float(g.bins[r + 3 * k]);
    }
  for (int r = 0; r < 3; ++r) {
    double m = 0;
    for (int k = 0; k < 3; ++k) m += std::fabs(g.bins[r + 3 * k]) * double(nxyz[k]);
    offmax = m > offmax ? m : offmax;
  }
  g.offmax = offmax * (1.0 + 1e-12);
  g.cutoff = cutoff;
  g.cutoff_sq = cutoff * cutoff;  // clist.cutoff^2 (:305)
  for (int k = 0; k < 3; ++k) {
    g.ns[k] = int(ns[k]);
    g.nxyz[k] = int(nxyz[k]);
    g.pbc[k] = pbc[k] ? 1 : 0;
  }
  g.ncells = int(ns[0] * ns[1] * ns[2]);
  g.nat = int(nat);
  return g;
}

template <typename TI>
nl::LegacyArgs<TI> legacy_args(const nl::LegacyGeo& lg, void* ws, const LegacyLayout& Q) {
  nl::LegacyArgs<TI> a;
  std::memset(&a, 0, sizeof(a));
  a.g = lg;
  a.Xs = at<double>(ws, Q.Xs);
  a.perm = at<TI>(ws, Q.perm);
  a.cell_start = at<int>(ws, Q.L.cell_start);
  a.D = at<double>(ws, Q.D);
  a.Df = at<float4>(ws, Q.Df);
  a.c0 = at<int4>(ws, Q.c0);
  a.dmax = at<unsigned>(ws, Q.L.pcount) + 8;  // zeroed with the build's region
  a.counts = at<int>(ws, Q.L.counts);
  a.blocks_per_sm = g_tuning.pair_blocks_per_sm;
  a.stats = at<unsigned long long>(ws, Q.L.stats);
  a.err = at<unsigned>(ws, Q.L.err);
  return a;
}

// build (the legacy cell list) + per-slot records + count + pair offsets
template <typename TI>
int legacy_count_impl(const double* X, int64_t nat, const nl::Geometry& g, const nl::LegacyGeo& lg, TI* first,
                      void* ws, const LegacyLayout& Q, cudaStream_t st) {
  int s = build_impl<TI>(X, nat, g, at<TI>(ws, Q.perm), at<double>(ws, Q.Xs), at<TI>(ws, Q.cell_id),
                         at<TI>(ws, Q.cell_offsets), ws, Q.L, st);
  if (s) return s;
  if (nat == 0) {  // first = [1] (get_first of an empty list, :416)
    static const TI one = 1;
    cudaError_t e = cudaMemcpyAsync(first, &one, sizeof(TI), cudaMemcpyHostToDevice, st);
    return e == cudaSuccess ? NL_OK : cuda_fail(e, "empty system");
  }
  const int sms = num_sms();
  nl::LegacyArgs<TI> a = legacy_args<TI>(lg, ws, Q);
  nl::launch_legacy_prepare<TI>(a, sms, st);
  nl::launch_legacy_pairs<TI>(false, a, sms, st);
  nl::launch_scan<TI>(a.counts, nat, first, nullptr, at<unsigned long long>(ws, Q.L.st_pairs), at<int>(ws, Q.L.pcount),
                      at<long long>(ws, Q.L.totals) + 1, a.err, st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch legacy count kernels");
}

template <typename TI>
int legacy_fill_impl(const nl::LegacyGeo& lg, const TI* first, int64_t capacity, TI* oi, TI* oj, TI* oS, void* ws,
                     const LegacyLayout& Q, cudaStream_t st) {
  if (lg.nat == 0 || capacity <= 0) return NL_OK;
  nl::LegacyArgs<TI> a = legacy_args<TI>(lg, ws, Q);
  a.first = first;
  a.oi = oi;
  a.oj = oj;
  a.oS = oS;
  a.capacity = capacity;
  nl::launch_legacy_pairs<TI>(true, a, num_sms(), st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch legacy fill kernel");
}

int legacy_check(int64_t nat, const int64_t* ncells, const int64_t* nxyz, int index_bytes, void* ws, size_t ws_bytes,
                 LegacyLayout& Q) {
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nxyz, index_bytes, ws, ws_bytes, L, nct);
  if (s == NL_ERR_NOMEM) return fail(NL_ERR_NOMEM, "workspace too small (see nl_legacy_workspace_bytes)");
  if (s) return s;
  Q = legacy_layout(nat, nct, index_bytes);
  if (!ws || ws_bytes < Q.end) return fail(NL_ERR_NOMEM, "workspace too small (see nl_legacy_workspace_bytes)");
  return NL_OK;
}

// --------------------------------------------------------------- batches --
struct BatchLayout {
  Layout L;  // the single-system layout for all atoms and cells of the batch
  size_t geo, atom0, cell0, cs, first_all, sys_sym, sys_fail, cell_sys, geo32, nonsym_cells, nonsym_chunks, rounds,
      end;
};

// n_chunks: the 32-slot chunks of the systems that the symmetric count pass
// does not take; the lists of cells and chunks the per-cell passes walk have
// room for every system failing the pass as well
BatchLayout batch_layout(int64_t nat, int64_t ncells, int nsys, size_t n_chunks = 0) {
  BatchLayout B;
  B.L = layout(nat, ncells);
  B.L.use_lists = (unsigned long long)nat * nl::kListCap < (1ull << 32);
  size_t o = B.L.end;
  B.geo = o;
  o += up(sizeof(nl::Geometry) * size_t(nsys));
  B.atom0 = o;
  o += up(sizeof(int) * size_t(nsys + 1));
  B.cell0 = o;
  o += up(sizeof(int) * size_t(nsys + 1));
  B.cs = o;
  o += up(sizeof(double) * size_t(nl::kCsTableDoubles) * size_t(nsys));
  B.first_all = o;
  o += up(sizeof(int64_t) * size_t(nat + 1));
  B.sys_sym = o;
  o += up(sizeof(int) * size_t(nsys));
  B.sys_fail = o;
  o += up(sizeof(int) * size_t(nsys));
  B.cell_sys = o;
  o += up(sizeof(int) * size_t(ncells > 0 ? ncells : 1));
  B.geo32 = o;  // Float32 batches: the per-system single-precision geometry
  o += up(sizeof(nl::Geo32) * size_t(nsys));
  B.nonsym_cells = o;
  o += up(sizeof(int) * size_t(ncells > 0 ? ncells : 1));
  B.nonsym_chunks = o;
  o += up(sizeof(int) * (n_chunks + size_t(nat / 32) + 2 * size_t(nsys) + 2));
  B.rounds = o;  // rounds of 32 home atoms of those cells (at most nat / 32 + 2)
  o += up(sizeof(int2) * (size_t(nat / 32) + 2));
  B.end = o;
  return B;
}

// A system of a batch takes the symmetric count pass when its 27-cell
// stencil has distinct cells (the single-system condition); its masks and
// stencil tables live in its atoms' own list regions, which hold 2 kListCap
// words each.
static_assert(2 * nl::kListCap >= 27 + 54, "a list region holds an atom's masks and its cell's stencil table");
bool batch_system_sym(const nl::Geometry& g) {
  bool sym = g.nat > 0;
  for (int k = 0; k < 3; ++k) sym = sym && g.nxyz[k] == 1 && (!g.pbc[k] || g.ns[k] >= 3);
  return sym;
}

}  // namespace

struct nl_batch {
  int nsys = 0;
  int index_bytes = 4;
  bool f32 = false;  // Float32 positions (nl_batch_create_f32): geo32 instead of geo
  int64_t nat = 0, ncells = 0;
  std::vector<nl::Geometry> geo;
  std::vector<nl::Geo32> geo32;
  std::vector<int> atom0, cell0;
  std::vector<int> sym;  // per system: the symmetric count pass applies
  bool any_sym = false;
  // the cells, and the 32-slot chunks of sorted slots, of the systems the
  // symmetric pass does not take: the per-cell count and list write passes
  // walk these and those of the systems that fail the pass
  std::vector<int> nonsym_cells, nonsym_chunks;
  BatchLayout B;
  nl_tuning tuning = {0, 0, 0};
};

namespace {

template <typename TI>
int batch_impl(const nl_batch& b, const double* X, TI* perm, double* Xs, TI* cell_id, TI* cell_offsets, TI* first,
               long long* pair_offsets, int64_t capacity, TI* oi, TI* oj, TI* oS, double* oR, void* ws,
               cudaStream_t st) {
  const Layout& L = b.B.L;
  const int sms = num_sms();
  const int na = int(b.nat), nc = int(b.ncells);
  cudaError_t e = cudaMemsetAsync(ws, 0, L.bend, st);  // err, stats, both zero regions
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  const nl::SysIndex si{at<nl::Geometry>(ws, b.B.geo), at<int>(ws, b.B.atom0), at<int>(ws, b.B.cell0), b.nsys};
  int* cid = at<int>(ws, L.cid);
  int* ticket = at<int>(ws, L.ticket);
  float4* rec = at<float4>(ws, L.rec);
  int* cell_count = at<int>(ws, L.cell_count);
  int* cell_start = at<int>(ws, L.cell_start);
  unsigned* err = at<unsigned>(ws, L.err);
  int* bcount = at<int>(ws, L.bcount);
  TI* first_all = at<TI>(ws, b.B.first_all);
  nl::Geometry g0;
  std::memset(&g0, 0, sizeof(g0));
  // stage (a)/(b): bin, sort, cell offsets
  nl::launch_bin(g0, si, X, na, cid, ticket, rec, cell_count, err, sms, st);
  nl::launch_scan<TI>(cell_count, nc, nullptr, cell_start, at<unsigned long long>(ws, L.st_cells), bcount,
                      at<long long>(ws, L.totals), err, st);
  nl::launch_scatter(na, cid, ticket, cell_start, at<int>(ws, L.tmp), sms, st);
  nl::launch_fix<TI>(si, na, at<int>(ws, L.tmp), cid, cell_start, X, rec, perm, cell_id, Xs,
                     at<float4>(ws, L.rec_sorted), at<int>(ws, L.scell), at<int>(ws, L.big_list), bcount + 1, sms, st);
  nl::launch_batch_cell_offsets<TI>(si, nc, cell_start, cell_offsets, sms, st);
  // stage (c): count and per-atom offsets
  nl::PairArgs<TI> a = pair_args<TI>(g0, cell_offsets, perm, Xs, ws, L);
  a.geo = si.geo;
  a.sys_atom = si.atom0;
  a.sys_cell = si.cell0;
  a.cell_sys = at<int>(ws, b.B.cell_sys);
  a.cs_sys = at<double>(ws, b.B.cs);
  a.work = at<int>(ws, L.pcount) + 12;  // zeroed with the workspace's first region
  a.nsys = b.nsys;
  a.nat_total = na;
  a.ncells_total = nc;
  a.counts = at<int>(ws, L.counts);
  a.pair_blocks_per_sm = b.tuning.pair_blocks_per_sm;
  a.emit_blocks_per_sm = b.tuning.emit_blocks_per_sm;
  a.count_kernel = b.tuning.count_kernel;
  // count kernel 0 (default) or 3: the symmetric pass for the systems it
  // applies to (it accumulates their counts; their pairs are written from the
  // masks in original order), the per-cell pass for the rest -- 3.87 against
  // 4.16 ms with the per-cell pass for all (count kernel 1) on 4,096 systems
  // of 8 to 4,096 atoms.
  a.sym = b.any_sym && a.list_cap > 0 && (a.count_kernel == 0 || a.count_kernel == 3) ? 1 : 0;
  a.sys_sym = at<int>(ws, b.B.sys_sym);
  a.sys_fail = at<int>(ws, b.B.sys_fail);
  a.extra_cells = at<int>(ws, L.pcount) + 9;    // zeroed with the workspace's first region
  a.extra_chunks = at<int>(ws, L.pcount) + 10;  // likewise
  a.n_rounds = at<int>(ws, L.pcount) + 3;       // likewise
  a.round_work = at<int>(ws, L.pcount) + 11;    // likewise
  a.rounds = at<int2>(ws, b.B.rounds);
  a.nonsym_cells = at<int>(ws, b.B.nonsym_cells);
  a.n_nonsym_cells = int(b.nonsym_cells.size());
  a.nonsym_chunks = at<int>(ws, b.B.nonsym_chunks);
  a.n_nonsym_chunks = int(b.nonsym_chunks.size());
  if (a.sym && na > 0) {
    e = cudaMemsetAsync(a.counts, 0, sizeof(int) * size_t(na), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.sys_fail, 0, sizeof(int) * size_t(b.nsys), st);
    if (e != cudaSuccess) return cuda_fail(e, "memset counts");
  }
  if (na > 0) {
    nl::launch_pairs<TI>(nl::kModeCount, a, sms, st);
    nl::launch_scan<TI>(at<int>(ws, L.counts), na, first_all, nullptr, at<unsigned long long>(ws, L.st_pairs),
                        at<int>(ws, L.pcount), at<long long>(ws, L.totals) + 1, err, st);
  } else {
    static const TI one = 1;
    e = cudaMemcpyAsync(first_all, &one, sizeof(TI), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "empty batch");
  }
  nl::launch_batch_first<TI>(si, na, first_all, first, pair_offsets, sms, st);
  // stage (d): pairs
  if (na > 0 && capacity > 0) {
    a.first = first_all;
    a.oi = oi;
    a.oj = oj;
    a.oS = oS;
    a.oR = oR;
    a.capacity = capacity;
    nl::launch_pairs<TI>(nl::kModeFill, a, sms, st);
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch batch kernels");
}

// A Float32 batch: the single-precision kernels over all systems at once --
// binning with each atom's system geometry, the counting sort of the launch's
// cells, then the per-cell count and fill passes, each warp taking the
// geometry of its home cell's system (no symmetric pass for batches).
template <typename TI>
int batch_impl32(const nl_batch& b, const float* X, TI* perm, float* Xs, TI* cell_id, TI* cell_offsets, TI* first,
                 long long* pair_offsets, int64_t capacity, TI* oi, TI* oj, TI* oS, float* oR, void* ws,
                 cudaStream_t st) {
  const Layout& L = b.B.L;
  const int sms = num_sms();
  const int na = int(b.nat), nc = int(b.ncells);
  cudaError_t e = cudaMemsetAsync(ws, 0, L.bend, st);
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  const nl::SysIndex si{nullptr, at<int>(ws, b.B.atom0), at<int>(ws, b.B.cell0), b.nsys};
  const nl::Geo32* geos = at<nl::Geo32>(ws, b.B.geo32);
  int* cid = at<int>(ws, L.cid);
  int* ticket = at<int>(ws, L.ticket);
  float4* rec = at<float4>(ws, L.rec);
  int* cell_count = at<int>(ws, L.cell_count);
  int* cell_start = at<int>(ws, L.cell_start);
  unsigned* err = at<unsigned>(ws, L.err);
  int* bcount = at<int>(ws, L.bcount);
  TI* first_all = at<TI>(ws, b.B.first_all);
  nl::launch_bin32_batch(geos, si.atom0, si.cell0, b.nsys, X, na, cid, ticket, rec, cell_count, err, sms, st);
  nl::launch_scan<TI>(cell_count, nc, nullptr, cell_start, at<unsigned long long>(ws, L.st_cells), bcount,
                      at<long long>(ws, L.totals), err, st);
  nl::launch_scatter(na, cid, ticket, cell_start, at<int>(ws, L.tmp), sms, st);
  nl::launch_fix<TI, float>(si, na, at<int>(ws, L.tmp), cid, cell_start, X, rec, perm, cell_id, Xs,
                            at<float4>(ws, L.rec_sorted), at<int>(ws, L.scell), at<int>(ws, L.big_list), bcount + 1,
                            sms, st);
  nl::launch_batch_cell_offsets<TI>(si, nc, cell_start, cell_offsets, sms, st);
  nl::Pairs32Args<TI> a;
  std::memset(&a, 0, sizeof(a));
  a.rec = at<float4>(ws, L.rec_sorted);
  a.scell = at<int>(ws, L.scell);
  a.cell_offsets = cell_offsets;
  a.perm = perm;
  a.counts = at<int>(ws, L.counts);
  a.err = err;
  a.sym = 0;
  a.sym_fail = at<int>(ws, L.pcount) + 6;  // set: the per-cell fill writes every pair
  a.geos = geos;
  a.sys_atom = si.atom0;
  a.sys_cell = si.cell0;
  a.cell_sys = at<int>(ws, b.B.cell_sys);
  a.work = at<int>(ws, L.pcount) + 12;  // zeroed with the workspace's first region
  a.rounds = at<int2>(ws, b.B.rounds);
  a.n_rounds = at<int>(ws, L.pcount) + 3;    // likewise
  a.round_work = at<int>(ws, L.pcount) + 9;  // likewise (two counters)
  a.nsys = b.nsys;
  a.nat_total = na;
  a.ncells_total = nc;
  e = cudaMemsetAsync(a.sym_fail, 0xFF, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  if (na > 0) {
    nl::launch_pairs32<TI>(false, a, sms, st);
    nl::launch_scan<TI>(a.counts, na, first_all, nullptr, at<unsigned long long>(ws, L.st_pairs),
                        at<int>(ws, L.pcount), at<long long>(ws, L.totals) + 1, err, st);
  } else {
    static const TI one = 1;
    e = cudaMemcpyAsync(first_all, &one, sizeof(TI), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "empty batch");
  }
  nl::launch_batch_first<TI>(si, na, first_all, first, pair_offsets, sms, st);
  if (na > 0 && capacity > 0) {
    a.first = first_all;
    a.oi = oi;
    a.oj = oj;
    a.oS = oS;
    a.oR = oR;
    a.capacity = capacity;
    nl::launch_pairs32<TI>(true, a, sms, st);
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch batch kernels");
}

}  // namespace

namespace nl {
int report(int status, const std::string& msg) { return fail(status, msg); }
int status_from_device_flags(unsigned flags) { return status_from_flags(flags); }
size_t workspace_min_bytes(int64_t nat, int64_t ncells_total) {
  if (nat < 0 || ncells_total < 1) return 0;
  return layout(nat, ncells_total).base_end;
}
Geometry geometry_for(const double* cell, const double* inv, const int64_t* ns, const int64_t* nxyz,
                      const uint8_t* pbc, double cutoff, int64_t nat) {
  return make_geometry(cell, inv, ns, nxyz, pbc, cutoff, nat);
}
size_t workspace_total_offset(int64_t nat, int64_t ncells_total) {
  return layout(nat, ncells_total).totals + sizeof(long long);
}
}  // namespace nl

// ======================================================================
extern "C" {

int nl_version(void) { return 1; }

const char* nl_last_error(void) { return g_last_error.c_str(); }

const char* nl_status_string(int s) {
  switch (s) {
    case NL_OK: return "ok";
    case NL_ERR_ARG: return "invalid argument";
    case NL_ERR_TOO_MANY_CELLS: return "too many cells";
    case NL_ERR_NOMEM: return "out of memory";
    case NL_ERR_CUDA: return "CUDA error";
    case NL_ERR_TIMEOUT: return "device wait timed out";
    case NL_ERR_BAD_POSITION: return "position cannot be binned";
    case NL_ERR_CAPACITY: return "pair buffer capacity exceeded";
    case NL_ERR_INDEX_OVERFLOW: return "index type overflow";
    case NL_ERR_INCONSISTENT: return "inconsistent cell list";
    default: return "unknown status";
  }
}

int nl_analyze_cell(const double cell[9], double cutoff, int index_bytes, nl_cell_plan* plan) {
  if (!cell || !plan) return fail(NL_ERR_ARG, "null argument");
  return analyze(cell, cutoff, index_bytes, plan);
}

size_t nl_workspace_bytes(int64_t nat, int64_t ncells_total) {
  if (nat < 0 || ncells_total < 1) return 0;
  return layout(nat, ncells_total).end;
}

size_t nl_workspace_min_bytes(int64_t nat, int64_t ncells_total) { return nl::workspace_min_bytes(nat, ncells_total); }

int nl_build_cell_list(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                       const int64_t ncells[3], const uint8_t pbc[3], double cutoff, int index_bytes, void* d_perm,
                       double* d_X_sorted, void* d_cell_id, void* d_cell_offsets, void* d_workspace,
                       size_t workspace_bytes, void* stream) {
  if (!cell || !inv_cell || !ncells || !pbc || !d_cell_offsets || (nat > 0 && (!d_X || !d_perm || !d_X_sorted || !d_cell_id)))
    return fail(NL_ERR_ARG, "null argument");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nullptr, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  const nl::Geometry g = make_geometry(cell, inv_cell, ncells, nullptr, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    return build_impl<int32_t>(d_X, nat, g, static_cast<int32_t*>(d_perm), d_X_sorted, static_cast<int32_t*>(d_cell_id),
                               static_cast<int32_t*>(d_cell_offsets), d_workspace, L, st);
  return build_impl<int64_t>(d_X, nat, g, static_cast<int64_t*>(d_perm), d_X_sorted, static_cast<int64_t*>(d_cell_id),
                             static_cast<int64_t*>(d_cell_offsets), d_workspace, L, st);
}

static int count_pairs_entry(const double* d_X_sorted, const void* d_perm, const void* d_cell_id,
                             const void* d_cell_offsets, int64_t nat, const double cell[9], const double inv_cell[9],
                             const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                             int index_bytes, int reuse_records, void* d_first, int64_t* total_pairs, void* d_workspace,
                             size_t workspace_bytes, void* stream, int half) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_first || !d_cell_offsets ||
      (nat > 0 && (!d_X_sorted || !d_perm || !d_cell_id)))
    return fail(NL_ERR_ARG, "null argument");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  const nl::Geometry g = make_geometry(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    s = count_impl<int32_t>(g, d_X_sorted, static_cast<const int32_t*>(d_perm), static_cast<const int32_t*>(d_cell_id),
                            static_cast<const int32_t*>(d_cell_offsets), reuse_records, static_cast<int32_t*>(d_first),
                            d_workspace, L, st, half);
  else
    s = count_impl<int64_t>(g, d_X_sorted, static_cast<const int64_t*>(d_perm), static_cast<const int64_t*>(d_cell_id),
                            static_cast<const int64_t*>(d_cell_offsets), reuse_records, static_cast<int64_t*>(d_first),
                            d_workspace, L, st, half);
  if (s) return s;
  if (total_pairs) {
    if (nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    return sync_read(d_workspace, st, at<long long>(d_workspace, L.totals) + 1, total_pairs);
  }
  return NL_OK;
}

int nl_count_pairs(const double* d_X_sorted, const void* d_perm, const void* d_cell_id, const void* d_cell_offsets,
                   int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                   const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes, int reuse_records,
                   void* d_first, int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream) {
  return count_pairs_entry(d_X_sorted, d_perm, d_cell_id, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff,
                           index_bytes, reuse_records, d_first, total_pairs, d_workspace, workspace_bytes, stream, 0);
}

static int fill_pairs_entry(const double* d_X_sorted, const void* d_perm, const void* d_cell_offsets, int64_t nat,
                            const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                            const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes,
                            const void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                            void* d_workspace, size_t workspace_bytes, void* stream, int half) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_first || !d_cell_offsets)
    return fail(NL_ERR_ARG, "null argument");
  // an empty system writes no pairs: its (empty) arrays may be null
  if (capacity > 0 && nat > 0 && (!d_i || !d_j || !d_S || !d_X_sorted || !d_perm))
    return fail(NL_ERR_ARG, "null argument");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  const nl::Geometry g = make_geometry(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    return fill_impl<int32_t>(g, d_X_sorted, static_cast<const int32_t*>(d_perm), static_cast<const int32_t*>(d_cell_offsets),
                              static_cast<const int32_t*>(d_first), capacity, static_cast<int32_t*>(d_i),
                              static_cast<int32_t*>(d_j), static_cast<int32_t*>(d_S), d_R, d_workspace, L, st, half);
  return fill_impl<int64_t>(g, d_X_sorted, static_cast<const int64_t*>(d_perm), static_cast<const int64_t*>(d_cell_offsets),
                            static_cast<const int64_t*>(d_first), capacity, static_cast<int64_t*>(d_i),
                            static_cast<int64_t*>(d_j), static_cast<int64_t*>(d_S), d_R, d_workspace, L, st, half);
}

int nl_fill_pairs(const double* d_X_sorted, const void* d_perm, const void* d_cell_offsets, int64_t nat,
                  const double cell[9], const double inv_cell[9], const int64_t ncells[3], const int64_t nxyz[3],
                  const uint8_t pbc[3], double cutoff, int index_bytes, const void* d_first, int64_t capacity,
                  void* d_i, void* d_j, void* d_S, double* d_R, void* d_workspace, size_t workspace_bytes,
                  void* stream) {
  return fill_pairs_entry(d_X_sorted, d_perm, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff,
                          index_bytes, d_first, capacity, d_i, d_j, d_S, d_R, d_workspace, workspace_bytes, stream, 0);
}

static int neighbour_list_entry(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                                const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                                int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id,
                                void* d_cell_offsets, void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S,
                                double* d_R, int64_t* total_pairs, void* d_workspace, size_t workspace_bytes,
                                void* stream, int half);

int nl_neighbour_list(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                      const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                      int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                      void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                      int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream) {
  return neighbour_list_entry(d_X, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff, index_bytes, d_perm, d_X_sorted,
                              d_cell_id, d_cell_offsets, d_first, capacity, d_i, d_j, d_S, d_R, total_pairs,
                              d_workspace, workspace_bytes, stream, 0);
}

int nl_neighbour_list_half(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                           const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                           int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                           void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                           int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream) {
  return neighbour_list_entry(d_X, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff, index_bytes, d_perm, d_X_sorted,
                              d_cell_id, d_cell_offsets, d_first, capacity, d_i, d_j, d_S, d_R, total_pairs,
                              d_workspace, workspace_bytes, stream, 1);
}

static int neighbour_list_entry(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                                const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                                int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id,
                                void* d_cell_offsets, void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S,
                                double* d_R, int64_t* total_pairs, void* d_workspace, size_t workspace_bytes,
                                void* stream, int half) {
  int s = nl_build_cell_list(d_X, nat, cell, inv_cell, ncells, pbc, cutoff, index_bytes, d_perm, d_X_sorted, d_cell_id,
                             d_cell_offsets, d_workspace, workspace_bytes, stream);
  if (s) return s;
  s = count_pairs_entry(d_X_sorted, d_perm, d_cell_id, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff,
                        index_bytes, 1, d_first, nullptr, d_workspace, workspace_bytes, stream, half);
  if (s) return s;
  s = fill_pairs_entry(d_X_sorted, d_perm, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff, index_bytes,
                       d_first, capacity, d_i, d_j, d_S, d_R, d_workspace, workspace_bytes, stream, half);
  if (s) return s;
  if (total_pairs) {
    Layout L = layout(nat, ncells[0] * ncells[1] * ncells[2]);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    s = sync_read(d_workspace, st, at<long long>(d_workspace, L.totals) + 1, total_pairs);
    if (s == NL_OK && *total_pairs > capacity) return fail(NL_ERR_CAPACITY, "pair buffers are smaller than the pair count");
    return s;
  }
  return NL_OK;
}

int nl_lazy_reduce(const double* d_X_sorted, const void* d_perm, const void* d_cell_id, const void* d_cell_offsets,
                   int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                   const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes, int reuse_records,
                   int op, void* d_out, void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_cell_offsets ||
      (nat > 0 && (!d_X_sorted || !d_perm || !d_cell_id || !d_out)))
    return fail(NL_ERR_ARG, "null argument");
  if (op != NL_REDUCE_COUNT && op != NL_REDUCE_INV_R6 && op != NL_REDUCE_INV_R6_FAST)
    return fail(NL_ERR_ARG, "unknown reduction");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  if (nat == 0) return NL_OK;
  const nl::Geometry g = make_geometry(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (!reuse_records) e = cudaMemsetAsync(d_workspace, 0, 128, st);
  // the count kernel appends the cells left to the screening pass to a list counted in pcount
  if (e == cudaSuccess) e = cudaMemsetAsync(static_cast<char*>(d_workspace) + L.pcount, 0, L.pend - L.pcount, st);
  if (e != cudaSuccess) return cuda_fail(e, "memset workspace");
  const int sms = num_sms();
  auto run = [&](auto tag) {
    using TI = decltype(tag);
    if (!reuse_records)
      nl::launch_prepare<TI>(g, d_X_sorted, static_cast<const TI*>(d_cell_id), static_cast<const TI*>(d_perm), g.nat,
                             at<float4>(d_workspace, L.rec_sorted), at<int>(d_workspace, L.scell),
                             at<unsigned>(d_workspace, L.err), sms, st);
    nl::PairArgs<TI> a =
        pair_args<TI>(g, static_cast<const TI*>(d_cell_offsets), static_cast<const TI*>(d_perm), d_X_sorted, d_workspace, L);
    a.cap_rec = nullptr;  // a later nl_fill_pairs must not take these lists for its own
    // the fused symmetric passes where the stencil is 27 distinct cells; the
    // per-cell passes below are gated on their success and redo the whole
    // reduction when a cell holds more than 32 atoms
    // (sym_gate, not sym: the count launcher reads sym as "launch the mask pass")
    // (the fast sum reads the neighbour masks, which need the list region)
    a.sym = 0;
    a.sym_gate = (op == NL_REDUCE_COUNT && sym_geometry(g)) ||
                         (op == NL_REDUCE_INV_R6_FAST && sym_geometry(g) && use_sym(g, L))
                     ? 1
                     : 0;
    if (a.sym_gate) {
      const size_t bytes = op == NL_REDUCE_COUNT ? sizeof(int) : sizeof(double);
      cudaError_t me = cudaMemsetAsync(d_out, 0, bytes * size_t(g.nat), st);
      if (me != cudaSuccess) e = me;
      if (op == NL_REDUCE_COUNT) {
        a.counts = static_cast<int*>(d_out);
      } else {
        a.per_atom = static_cast<double*>(d_out);
        a.counts = at<int>(d_workspace, L.counts);  // the mask pass's counts (not the result)
        me = cudaMemsetAsync(a.counts, 0, sizeof(int) * size_t(g.nat), st);
        if (me != cudaSuccess) e = me;
      }
      nl::launch_sym_lazy<TI>(op == NL_REDUCE_COUNT ? nl::kLazyCounts : nl::kLazyInvR6, a, sms, st);
    }
    if (op == NL_REDUCE_COUNT) {
      a.list_cap = 0;  // the counts are the result: no lists
      a.lists = nullptr;
      a.lcount = nullptr;
      a.counts = static_cast<int*>(d_out);
      nl::launch_pairs<TI>(nl::kModeCount, a, sms, st);
    } else {
      // with room for the lists: count pass with lists, each atom's sum from
      // its list, screening pass only for overflowed cells; else one
      // screening traversal
      if (a.list_cap > 0) {
        a.counts = at<int>(d_workspace, L.counts);
        nl::launch_pairs<TI>(nl::kModeCount, a, sms, st);
      }
      a.per_atom = static_cast<double*>(d_out);
      nl::launch_pairs<TI>(nl::kModeLazyR6, a, sms, st);
    }
  };
  if (index_bytes == 4)
    run(int32_t(0));
  else
    run(int64_t(0));
  if (e != cudaSuccess) return cuda_fail(e, "memset lazy output");
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch lazy kernel");
}

int nl_batch_create(const nl_system* systems, int nsys, int index_bytes, nl_batch** batch) {
  if (!batch || (nsys > 0 && !systems)) return fail(NL_ERR_ARG, "null argument");
  *batch = nullptr;
  if (nsys < 1) return fail(NL_ERR_ARG, "a batch needs at least one system");
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  nl_batch* b = new (std::nothrow) nl_batch;
  if (!b) return fail(NL_ERR_NOMEM, "cannot allocate the batch plan");
  b->nsys = nsys;
  b->index_bytes = index_bytes;
  b->geo.resize(size_t(nsys));
  b->atom0.resize(size_t(nsys) + 1);
  b->cell0.resize(size_t(nsys) + 1);
  int64_t na = 0, nc = 0;
  for (int s = 0; s < nsys; ++s) {
    const nl_system& y = systems[s];
    Layout Ls;
    int64_t nct;
    // per-system checks of the single-system calls (a dummy workspace size)
    int st = check_common(y.nat, y.ncells, y.nxyz, index_bytes, reinterpret_cast<void*>(1), ~size_t(0), Ls, nct);
    if (st == NL_OK && (!(y.cutoff > 0) || !std::isfinite(y.cutoff))) st = fail(NL_ERR_ARG, "cutoff must be positive");
    if (st) {
      g_last_error = "system " + std::to_string(s) + ": " + g_last_error;
      delete b;
      return st;
    }
    b->atom0[size_t(s)] = int(na);
    b->cell0[size_t(s)] = int(nc);
    b->geo[size_t(s)] = make_geometry(y.cell, y.inv_cell, y.ncells, y.nxyz, y.pbc, y.cutoff, y.nat);
    b->sym.push_back(batch_system_sym(b->geo[size_t(s)]) ? 1 : 0);
    b->any_sym = b->any_sym || b->sym.back();
    na += y.nat;
    nc += nct;
    if (na > 2147483646LL || nc + nsys > 2147483646LL) {
      delete b;
      return fail(NL_ERR_ARG, "a batch holds at most 2^31-2 atoms and 2^31-2 cells");
    }
  }
  b->atom0[size_t(nsys)] = int(na);
  b->cell0[size_t(nsys)] = int(nc);
  b->nat = na;
  b->ncells = nc;
  for (int s = 0; s < nsys; ++s) {
    if (b->sym[size_t(s)]) continue;
    for (int c = b->cell0[size_t(s)]; c < b->cell0[size_t(s) + 1]; ++c) b->nonsym_cells.push_back(c);
    for (int c0 = b->atom0[size_t(s)] & ~31; c0 < b->atom0[size_t(s) + 1]; c0 += 32)
      if (b->nonsym_chunks.empty() || b->nonsym_chunks.back() != c0) b->nonsym_chunks.push_back(c0);
  }
  b->B = batch_layout(na, nc, nsys, b->nonsym_chunks.size());
  *batch = b;
  return NL_OK;
}

int nl_batch_create_auto(const double* cells, const double* cutoffs, const uint8_t* pbc, const int64_t* nat, int nsys,
                         int index_bytes, nl_batch** batch) {
  if (!batch || (nsys > 0 && (!cells || !cutoffs || !pbc || !nat))) return fail(NL_ERR_ARG, "null argument");
  if (nsys < 1) return fail(NL_ERR_ARG, "a batch needs at least one system");
  std::vector<nl_system> sys(static_cast<size_t>(nsys));
  for (int s = 0; s < nsys; ++s) {
    nl_system& y = sys[size_t(s)];
    nl_cell_plan p;
    if (int st = analyze(cells + 9 * size_t(s), cutoffs[s], index_bytes, &p)) {
      g_last_error = "system " + std::to_string(s) + ": " + g_last_error;
      return st;
    }
    y.nat = nat[s];
    std::memcpy(y.cell, cells + 9 * size_t(s), sizeof(y.cell));
    std::memcpy(y.inv_cell, p.inv_cell, sizeof(y.inv_cell));
    for (int k = 0; k < 3; ++k) {
      y.ncells[k] = p.ncells[k];
      y.nxyz[k] = p.nxyz[k];
      y.pbc[k] = pbc[3 * size_t(s) + k] ? 1 : 0;
    }
    y.cutoff = cutoffs[s];
  }
  return nl_batch_create(sys.data(), nsys, index_bytes, batch);
}

int nl_batch_create_f32(const nl_system_f32* systems, int nsys, int index_bytes, nl_batch** batch) {
  if (!batch || (nsys > 0 && !systems)) return fail(NL_ERR_ARG, "null argument");
  *batch = nullptr;
  if (nsys < 1) return fail(NL_ERR_ARG, "a batch needs at least one system");
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  nl_batch* b = new (std::nothrow) nl_batch;
  if (!b) return fail(NL_ERR_NOMEM, "cannot allocate the batch plan");
  b->nsys = nsys;
  b->index_bytes = index_bytes;
  b->f32 = true;
  b->geo32.resize(size_t(nsys));
  b->atom0.resize(size_t(nsys) + 1);
  b->cell0.resize(size_t(nsys) + 1);
  b->sym.assign(size_t(nsys), 0);
  int64_t na = 0, nc = 0;
  for (int s = 0; s < nsys; ++s) {
    const nl_system_f32& y = systems[s];
    Layout Ls;
    int64_t nct;
    int st = check_common(y.nat, y.ncells, y.nxyz, index_bytes, reinterpret_cast<void*>(1), ~size_t(0), Ls, nct);
    if (st == NL_OK && (!(y.cutoff > 0) || !std::isfinite(y.cutoff))) st = fail(NL_ERR_ARG, "cutoff must be positive");
    if (st) {
      g_last_error = "system " + std::to_string(s) + ": " + g_last_error;
      delete b;
      return st;
    }
    b->atom0[size_t(s)] = int(na);
    b->cell0[size_t(s)] = int(nc);
    b->geo32[size_t(s)] = make_geo32(y.cell, y.inv_cell, y.ncells, y.nxyz, y.pbc, y.cutoff, y.nat);
    na += y.nat;
    nc += nct;
    if (na > 2147483646LL || nc + nsys > 2147483646LL) {
      delete b;
      return fail(NL_ERR_ARG, "a batch holds at most 2^31-2 atoms and 2^31-2 cells");
    }
  }
  b->atom0[size_t(nsys)] = int(na);
  b->cell0[size_t(nsys)] = int(nc);
  b->nat = na;
  b->ncells = nc;
  b->B = batch_layout(na, nc, nsys);
  *batch = b;
  return NL_OK;
}

int nl_batch_create_auto_f32(const float* cells, const float* cutoffs, const uint8_t* pbc, const int64_t* nat,
                             int nsys, int index_bytes, nl_batch** batch) {
  if (!batch || (nsys > 0 && (!cells || !cutoffs || !pbc || !nat))) return fail(NL_ERR_ARG, "null argument");
  if (nsys < 1) return fail(NL_ERR_ARG, "a batch needs at least one system");
  std::vector<nl_system_f32> sys(static_cast<size_t>(nsys));
  for (int s = 0; s < nsys; ++s) {
    nl_system_f32& y = sys[size_t(s)];
    nl_cell_plan_f32 p;
    if (int st = analyze_f32(cells + 9 * size_t(s), cutoffs[s], index_bytes, &p)) {
      g_last_error = "system " + std::to_string(s) + ": " + g_last_error;
      return st;
    }
    y.nat = nat[s];
    std::memcpy(y.cell, cells + 9 * size_t(s), sizeof(y.cell));
    std::memcpy(y.inv_cell, p.inv_cell, sizeof(y.inv_cell));
    for (int k = 0; k < 3; ++k) {
      y.ncells[k] = p.ncells[k];
      y.nxyz[k] = p.nxyz[k];
      y.pbc[k] = pbc[3 * size_t(s) + k] ? 1 : 0;
    }
    y.cutoff = cutoffs[s];
  }
  return nl_batch_create_f32(sys.data(), nsys, index_bytes, batch);
}

void nl_batch_destroy(nl_batch* batch) { delete batch; }

size_t nl_batch_workspace_bytes(const nl_batch* batch) { return batch ? batch->B.end : 0; }

int nl_batch_sizes(const nl_batch* batch, int64_t* total_atoms, int64_t* total_cells) {
  if (!batch) return fail(NL_ERR_ARG, "null batch");
  if (total_atoms) *total_atoms = batch->nat;
  if (total_cells) *total_cells = batch->ncells;
  return NL_OK;
}

int nl_batch_upload(const nl_batch* batch, void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!batch || !d_workspace) return fail(NL_ERR_ARG, "null argument");
  if (workspace_bytes < batch->B.end) return fail(NL_ERR_NOMEM, "workspace too small (see nl_batch_workspace_bytes)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const BatchLayout& B = batch->B;
  // pageable sources: each copy returns once its source has been consumed
  cudaError_t e = batch->f32 ? cudaMemcpyAsync(at<char>(d_workspace, B.geo32), batch->geo32.data(),
                                               sizeof(nl::Geo32) * batch->geo32.size(), cudaMemcpyHostToDevice, st)
                             : cudaMemcpyAsync(at<char>(d_workspace, B.geo), batch->geo.data(),
                                               sizeof(nl::Geometry) * batch->geo.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(at<char>(d_workspace, B.atom0), batch->atom0.data(), sizeof(int) * batch->atom0.size(),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(at<char>(d_workspace, B.cell0), batch->cell0.data(), sizeof(int) * batch->cell0.size(),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(at<char>(d_workspace, B.sys_sym), batch->sym.data(), sizeof(int) * batch->sym.size(),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !batch->nonsym_cells.empty())
    e = cudaMemcpyAsync(at<char>(d_workspace, B.nonsym_cells), batch->nonsym_cells.data(),
                        sizeof(int) * batch->nonsym_cells.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !batch->nonsym_chunks.empty())
    e = cudaMemcpyAsync(at<char>(d_workspace, B.nonsym_chunks), batch->nonsym_chunks.data(),
                        sizeof(int) * batch->nonsym_chunks.size(), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "upload batch tables");
  if (!batch->f32) nl::launch_cs_tables(at<nl::Geometry>(d_workspace, B.geo), batch->nsys, at<double>(d_workspace, B.cs), st);
  nl::launch_cell_systems(at<int>(d_workspace, B.cell0), batch->nsys, at<int>(d_workspace, B.cell_sys), st);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "upload batch tables");
}

int nl_batch_neighbour_list(const nl_batch* batch, const double* d_X, void* d_perm, double* d_X_sorted,
                            void* d_cell_id, void* d_cell_offsets, void* d_first, int64_t* d_pair_offsets,
                            int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R, int64_t* total_pairs,
                            void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!batch || !d_cell_offsets || !d_first || !d_pair_offsets || !d_workspace) return fail(NL_ERR_ARG, "null argument");
  if (batch->f32) return fail(NL_ERR_ARG, "a Float32 batch runs through nl_batch_neighbour_list_f32");
  if (batch->nat > 0 && (!d_X || !d_perm || !d_X_sorted || !d_cell_id)) return fail(NL_ERR_ARG, "null argument");
  if (capacity > 0 && (!d_i || !d_j || !d_S)) return fail(NL_ERR_ARG, "null argument");
  if (workspace_bytes < batch->B.end) return fail(NL_ERR_NOMEM, "workspace too small (see nl_batch_workspace_bytes)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int s;
  if (batch->index_bytes == 4)
    s = batch_impl<int32_t>(*batch, d_X, static_cast<int32_t*>(d_perm), d_X_sorted, static_cast<int32_t*>(d_cell_id),
                            static_cast<int32_t*>(d_cell_offsets), static_cast<int32_t*>(d_first),
                            reinterpret_cast<long long*>(d_pair_offsets), capacity, static_cast<int32_t*>(d_i),
                            static_cast<int32_t*>(d_j), static_cast<int32_t*>(d_S), d_R, d_workspace, st);
  else
    s = batch_impl<int64_t>(*batch, d_X, static_cast<int64_t*>(d_perm), d_X_sorted, static_cast<int64_t*>(d_cell_id),
                            static_cast<int64_t*>(d_cell_offsets), static_cast<int64_t*>(d_first),
                            reinterpret_cast<long long*>(d_pair_offsets), capacity, static_cast<int64_t*>(d_i),
                            static_cast<int64_t*>(d_j), static_cast<int64_t*>(d_S), d_R, d_workspace, st);
  if (s) return s;
  if (total_pairs) {
    if (batch->nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    s = sync_read(d_workspace, st, at<long long>(d_workspace, batch->B.L.totals) + 1, total_pairs);
    if (s == NL_OK && *total_pairs > capacity) return fail(NL_ERR_CAPACITY, "pair buffers are smaller than the pair count");
    return s;
  }
  return NL_OK;
}

int nl_batch_neighbour_list_f32(const nl_batch* batch, const float* d_X, void* d_perm, float* d_X_sorted,
                                void* d_cell_id, void* d_cell_offsets, void* d_first, int64_t* d_pair_offsets,
                                int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R, int64_t* total_pairs,
                                void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!batch || !d_cell_offsets || !d_first || !d_pair_offsets || !d_workspace) return fail(NL_ERR_ARG, "null argument");
  if (!batch->f32) return fail(NL_ERR_ARG, "a Float64 batch runs through nl_batch_neighbour_list");
  if (batch->nat > 0 && (!d_X || !d_perm || !d_X_sorted || !d_cell_id)) return fail(NL_ERR_ARG, "null argument");
  if (capacity > 0 && (!d_i || !d_j || !d_S)) return fail(NL_ERR_ARG, "null argument");
  if (workspace_bytes < batch->B.end) return fail(NL_ERR_NOMEM, "workspace too small (see nl_batch_workspace_bytes)");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int s;
  if (batch->index_bytes == 4)
    s = batch_impl32<int32_t>(*batch, d_X, static_cast<int32_t*>(d_perm), d_X_sorted, static_cast<int32_t*>(d_cell_id),
                              static_cast<int32_t*>(d_cell_offsets), static_cast<int32_t*>(d_first),
                              reinterpret_cast<long long*>(d_pair_offsets), capacity, static_cast<int32_t*>(d_i),
                              static_cast<int32_t*>(d_j), static_cast<int32_t*>(d_S), d_R, d_workspace, st);
  else
    s = batch_impl32<int64_t>(*batch, d_X, static_cast<int64_t*>(d_perm), d_X_sorted, static_cast<int64_t*>(d_cell_id),
                              static_cast<int64_t*>(d_cell_offsets), static_cast<int64_t*>(d_first),
                              reinterpret_cast<long long*>(d_pair_offsets), capacity, static_cast<int64_t*>(d_i),
                              static_cast<int64_t*>(d_j), static_cast<int64_t*>(d_S), d_R, d_workspace, st);
  if (s) return s;
  if (total_pairs) {
    if (batch->nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    s = sync_read(d_workspace, st, at<long long>(d_workspace, batch->B.L.totals) + 1, total_pairs);
    if (s == NL_OK && *total_pairs > capacity) return fail(NL_ERR_CAPACITY, "pair buffers are smaller than the pair count");
    return s;
  }
  return NL_OK;
}

static int check_tuning(const nl_tuning* t) {
  if (t && (t->pair_blocks_per_sm < 0 || t->pair_blocks_per_sm > 256 || t->emit_blocks_per_sm < 0 ||
            t->emit_blocks_per_sm > 256 || t->count_kernel < 0 || t->count_kernel > 3))
    return fail(NL_ERR_ARG, "tuning out of range (0..256 blocks per SM, count kernel 0..3)");
  return NL_OK;
}

int nl_set_tuning(const nl_tuning* tuning) {
  if (int s = check_tuning(tuning)) return s;
  g_tuning = tuning ? *tuning : nl_tuning{0, 0, 0};
  return NL_OK;
}

int nl_batch_set_tuning(nl_batch* batch, const nl_tuning* tuning) {
  if (!batch) return fail(NL_ERR_ARG, "null batch");
  if (int s = check_tuning(tuning)) return s;
  batch->tuning = tuning ? *tuning : nl_tuning{0, 0, 0};
  return NL_OK;
}

int nl_pair_vectors(const double* d_X, int64_t nat, const double cell[9], int index_bytes, const void* d_i,
                    const void* d_j, const void* d_S, int64_t npairs, double* d_R, void* stream) {
  if (!cell || npairs < 0 || nat < 0) return fail(NL_ERR_ARG, "invalid argument");
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  if (npairs == 0) return NL_OK;
  if (!d_X || !d_i || !d_j || !d_S || !d_R || nat == 0) return fail(NL_ERR_ARG, "null argument");
  if (nat > 2147483646LL) return fail(NL_ERR_ARG, "nat must be in [0, 2^31-2]");
  nl::Geometry g;
  std::memset(&g, 0, sizeof(g));
  std::memcpy(g.C, cell, sizeof(g.C));
  g.nat = int(nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    nl::launch_pair_vectors<int32_t>(g, d_X, static_cast<const int32_t*>(d_i), static_cast<const int32_t*>(d_j),
                                     static_cast<const int32_t*>(d_S), npairs, d_R, num_sms(), st);
  else
    nl::launch_pair_vectors<int64_t>(g, d_X, static_cast<const int64_t*>(d_i), static_cast<const int64_t*>(d_j),
                                     static_cast<const int64_t*>(d_S), npairs, d_R, num_sms(), st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch pair vectors");
}

int nl_max_displacement_sq(const double* d_X, const double* d_Xref, int64_t nat, double* d_out, void* stream) {
  if (!d_out || nat < 0 || (nat > 0 && (!d_X || !d_Xref))) return fail(NL_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(double), st);
  if (e != cudaSuccess) return cuda_fail(e, "memset");
  nl::launch_max_disp_sq(d_X, d_Xref, nat, reinterpret_cast<unsigned long long*>(d_out), num_sms(), st);
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch max displacement");
}

int nl_pair_vectors_f32(const float* d_X, int64_t nat, const float cell[9], int index_bytes, const void* d_i,
                        const void* d_j, const void* d_S, int64_t npairs, float* d_R, void* stream) {
  if (!cell || npairs < 0 || nat < 0) return fail(NL_ERR_ARG, "invalid argument");
  if (index_bytes != 4 && index_bytes != 8) return fail(NL_ERR_ARG, "index_bytes must be 4 or 8");
  if (npairs == 0) return NL_OK;
  if (!d_X || !d_i || !d_j || !d_S || !d_R || nat == 0) return fail(NL_ERR_ARG, "null argument");
  if (nat > 2147483646LL) return fail(NL_ERR_ARG, "nat must be in [0, 2^31-2]");
  nl::Geo32 g;
  std::memset(&g, 0, sizeof(g));
  std::memcpy(g.C, cell, sizeof(g.C));
  g.nat = int(nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    nl::launch_pair_vectors32<int32_t>(g, d_X, static_cast<const int32_t*>(d_i), static_cast<const int32_t*>(d_j),
                                       static_cast<const int32_t*>(d_S), npairs, d_R, num_sms(), st);
  else
    nl::launch_pair_vectors32<int64_t>(g, d_X, static_cast<const int64_t*>(d_i), static_cast<const int64_t*>(d_j),
                                       static_cast<const int64_t*>(d_S), npairs, d_R, num_sms(), st);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch pair vectors");
}

int nl_max_displacement_sq_f32(const float* d_X, const float* d_Xref, int64_t nat, float* d_out, void* stream) {
  if (!d_out || nat < 0 || (nat > 0 && (!d_X || !d_Xref))) return fail(NL_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(float), st);
  if (e != cudaSuccess) return cuda_fail(e, "memset");
  nl::launch_max_disp_sq32(d_X, d_Xref, nat, reinterpret_cast<unsigned*>(d_out), num_sms(), st);
  e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : cuda_fail(e, "launch max displacement");
}

int nl_analyze_cell_f32(const float cell[9], float cutoff, int index_bytes, nl_cell_plan_f32* plan) {
  if (!cell || !plan) return fail(NL_ERR_ARG, "null argument");
  return analyze_f32(cell, cutoff, index_bytes, plan);
}

int nl_build_cell_list_f32(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                           const int64_t ncells[3], const uint8_t pbc[3], float cutoff, int index_bytes, void* d_perm,
                           float* d_X_sorted, void* d_cell_id, void* d_cell_offsets, void* d_workspace,
                           size_t workspace_bytes, void* stream) {
  if (!cell || !inv_cell || !ncells || !pbc || !d_cell_offsets || (nat > 0 && (!d_X || !d_perm || !d_X_sorted || !d_cell_id)))
    return fail(NL_ERR_ARG, "null argument");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nullptr, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  const nl::Geo32 g = make_geo32(cell, inv_cell, ncells, nullptr, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    return build_impl32<int32_t>(d_X, nat, g, static_cast<int32_t*>(d_perm), d_X_sorted,
                                 static_cast<int32_t*>(d_cell_id), static_cast<int32_t*>(d_cell_offsets), d_workspace, L,
                                 st);
  return build_impl32<int64_t>(d_X, nat, g, static_cast<int64_t*>(d_perm), d_X_sorted, static_cast<int64_t*>(d_cell_id),
                               static_cast<int64_t*>(d_cell_offsets), d_workspace, L, st);
}

static int count_pairs_f32_entry(const float* d_X_sorted, const void* d_perm, const void* d_cell_id,
                                 const void* d_cell_offsets, int64_t nat, const float cell[9], const float inv_cell[9],
                                 const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], float cutoff,
                                 int index_bytes, int reuse_records, void* d_first, int64_t* total_pairs,
                                 void* d_workspace, size_t workspace_bytes, void* stream, int half) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_first || !d_cell_offsets ||
      (nat > 0 && (!d_X_sorted || !d_perm || !d_cell_id)))
    return fail(NL_ERR_ARG, "null argument");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  const nl::Geo32 g = make_geo32(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    s = count_impl32<int32_t>(g, d_X_sorted, static_cast<const int32_t*>(d_perm),
                              static_cast<const int32_t*>(d_cell_id), static_cast<const int32_t*>(d_cell_offsets),
                              reuse_records, static_cast<int32_t*>(d_first), d_workspace, L, st, half);
  else
    s = count_impl32<int64_t>(g, d_X_sorted, static_cast<const int64_t*>(d_perm),
                              static_cast<const int64_t*>(d_cell_id), static_cast<const int64_t*>(d_cell_offsets),
                              reuse_records, static_cast<int64_t*>(d_first), d_workspace, L, st, half);
  if (s) return s;
  if (total_pairs) {
    if (nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    return sync_read(d_workspace, st, at<long long>(d_workspace, L.totals) + 1, total_pairs);
  }
  return NL_OK;
}

int nl_count_pairs_f32(const float* d_X_sorted, const void* d_perm, const void* d_cell_id, const void* d_cell_offsets,
                       int64_t nat, const float cell[9], const float inv_cell[9], const int64_t ncells[3],
                       const int64_t nxyz[3], const uint8_t pbc[3], float cutoff, int index_bytes, int reuse_records,
                       void* d_first, int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream) {
  return count_pairs_f32_entry(d_X_sorted, d_perm, d_cell_id, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc,
                               cutoff, index_bytes, reuse_records, d_first, total_pairs, d_workspace, workspace_bytes,
                               stream, 0);
}

static int fill_pairs_f32_entry(const float* d_X_sorted, const void* d_perm, const void* d_cell_offsets, int64_t nat,
                                const float cell[9], const float inv_cell[9], const int64_t ncells[3],
                                const int64_t nxyz[3], const uint8_t pbc[3], float cutoff, int index_bytes,
                                const void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R,
                                void* d_workspace, size_t workspace_bytes, void* stream, int half) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_first || !d_cell_offsets)
    return fail(NL_ERR_ARG, "null argument");
  if (capacity > 0 && nat > 0 && (!d_i || !d_j || !d_S || !d_X_sorted || !d_perm))
    return fail(NL_ERR_ARG, "null argument");
  Layout L;
  int64_t nct;
  int s = check_common(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, L, nct);
  if (s) return s;
  const nl::Geo32 g = make_geo32(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    return fill_impl32<int32_t>(g, static_cast<const int32_t*>(d_perm), static_cast<const int32_t*>(d_cell_offsets),
                                static_cast<const int32_t*>(d_first), capacity, static_cast<int32_t*>(d_i),
                                static_cast<int32_t*>(d_j), static_cast<int32_t*>(d_S), d_R, d_workspace, L, st, half);
  return fill_impl32<int64_t>(g, static_cast<const int64_t*>(d_perm), static_cast<const int64_t*>(d_cell_offsets),
                              static_cast<const int64_t*>(d_first), capacity, static_cast<int64_t*>(d_i),
                              static_cast<int64_t*>(d_j), static_cast<int64_t*>(d_S), d_R, d_workspace, L, st, half);
}

int nl_fill_pairs_f32(const float* d_X_sorted, const void* d_perm, const void* d_cell_offsets, int64_t nat,
                      const float cell[9], const float inv_cell[9], const int64_t ncells[3], const int64_t nxyz[3],
                      const uint8_t pbc[3], float cutoff, int index_bytes, const void* d_first, int64_t capacity,
                      void* d_i, void* d_j, void* d_S, float* d_R, void* d_workspace, size_t workspace_bytes,
                      void* stream) {
  return fill_pairs_f32_entry(d_X_sorted, d_perm, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff,
                              index_bytes, d_first, capacity, d_i, d_j, d_S, d_R, d_workspace, workspace_bytes, stream,
                              0);
}

static int neighbour_list_f32_entry(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                                    const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3],
                                    float cutoff, int index_bytes, void* d_perm, float* d_X_sorted, void* d_cell_id,
                                    void* d_cell_offsets, void* d_first, int64_t capacity, void* d_i, void* d_j,
                                    void* d_S, float* d_R, int64_t* total_pairs, void* d_workspace,
                                    size_t workspace_bytes, void* stream, int half) {
  int s = nl_build_cell_list_f32(d_X, nat, cell, inv_cell, ncells, pbc, cutoff, index_bytes, d_perm, d_X_sorted,
                                 d_cell_id, d_cell_offsets, d_workspace, workspace_bytes, stream);
  if (s) return s;
  s = count_pairs_f32_entry(d_X_sorted, d_perm, d_cell_id, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc,
                            cutoff, index_bytes, 1, d_first, nullptr, d_workspace, workspace_bytes, stream, half);
  if (s) return s;
  s = fill_pairs_f32_entry(d_X_sorted, d_perm, d_cell_offsets, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff,
                           index_bytes, d_first, capacity, d_i, d_j, d_S, d_R, d_workspace, workspace_bytes, stream,
                           half);
  if (s) return s;
  if (total_pairs) {
    Layout L = layout(nat, ncells[0] * ncells[1] * ncells[2]);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    s = sync_read(d_workspace, st, at<long long>(d_workspace, L.totals) + 1, total_pairs);
    if (s == NL_OK && *total_pairs > capacity) return fail(NL_ERR_CAPACITY, "pair buffers are smaller than the pair count");
    return s;
  }
  return NL_OK;
}

int nl_neighbour_list_f32(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                          const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], float cutoff,
                          int index_bytes, void* d_perm, float* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                          void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R,
                          int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream) {
  return neighbour_list_f32_entry(d_X, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff, index_bytes, d_perm, d_X_sorted,
                                  d_cell_id, d_cell_offsets, d_first, capacity, d_i, d_j, d_S, d_R, total_pairs,
                                  d_workspace, workspace_bytes, stream, 0);
}

int nl_neighbour_list_half_f32(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                               const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], float cutoff,
                               int index_bytes, void* d_perm, float* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                               void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R,
                               int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream) {
  return neighbour_list_f32_entry(d_X, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff, index_bytes, d_perm, d_X_sorted,
                                  d_cell_id, d_cell_offsets, d_first, capacity, d_i, d_j, d_S, d_R, total_pairs,
                                  d_workspace, workspace_bytes, stream, 1);
}

size_t nl_legacy_workspace_bytes(int64_t nat, int64_t ncells_total, int index_bytes) {
  if (nat < 0 || ncells_total < 1 || (index_bytes != 4 && index_bytes != 8)) return 0;
  return legacy_layout(nat, ncells_total, index_bytes).end;
}

int nl_legacy_fix_cell(const double* d_X, int64_t nat, const double cell[9], const uint8_t pbc[3], double* d_X_fixed,
                       double cell_fixed[9], void* d_workspace, size_t workspace_bytes, void* stream) {
  if (!cell || !pbc || !cell_fixed || !d_workspace) return fail(NL_ERR_ARG, "null argument");
  if (nat < 0 || nat > 2147483646LL) return fail(NL_ERR_ARG, "nat must be in [0, 2^31-2]");
  if (nat > 0 && (!d_X || !d_X_fixed)) return fail(NL_ERR_ARG, "null argument");
  if (workspace_bytes < NL_LEGACY_FIX_WORKSPACE_BYTES) return fail(NL_ERR_NOMEM, "workspace too small for the cell fix");
  double C[9];
  std::memcpy(C, cell, sizeof(C));
  std::memcpy(cell_fixed, C, sizeof(C));
  if (nat == 0) return NL_OK;  // no atom moves, the cell stays
  double inv[9];
  sa_inv(C, inv);  // invCt = inv(C)' (:460)
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // error word at 0; open-axis extremes at 64: min from 0.0, max from 1.0 (:462-463)
  unsigned long long init[6];
  for (int k = 0; k < 3; ++k) {
    init[k] = nl::legacy_key(0.0);
    init[3 + k] = nl::legacy_key(1.0);
  }
  cudaError_t e = cudaMemsetAsync(d_workspace, 0, 64, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(at<char>(d_workspace, 64), init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "initialise cell fix");
  const int pb[3] = {pbc[0] ? 1 : 0, pbc[1] ? 1 : 0, pbc[2] ? 1 : 0};
  nl::launch_legacy_fix(inv, C, pb, d_X, d_X_fixed, int(nat), at<unsigned long long>(d_workspace, 64),
                        at<unsigned>(d_workspace, 0), num_sms(), st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "launch cell fix");
  long long* h = pinned_scratch();
  if (!h) return fail(NL_ERR_NOMEM, "cannot allocate pinned host scratch");
  e = cudaMemcpyAsync(h, d_workspace, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h + 1, at<char>(d_workspace, 64), 6 * sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "read cell fix");
  if (int s = status_from_flags(*reinterpret_cast<unsigned*>(h))) return s;
  double min_lam[3], max_lam[3];
  for (int k = 0; k < 3; ++k) {
    min_lam[k] = nl::legacy_unkey((unsigned long long)h[1 + k]);
    max_lam[k] = nl::legacy_unkey((unsigned long long)h[4 + k]);
  }
  const double mn = std::fmin(std::fmin(min_lam[0], min_lam[1]), min_lam[2]);
  const double mx = std::fmax(std::fmax(max_lam[0], max_lam[1]), max_lam[2]);
  if (mn < 0.0 || mx > 1.0) {  // :488-503
    // t = -C' * min_lam, parsed as (-C') * min_lam
    double t[3];
    for (int k = 0; k < 3; ++k)
      t[k] = ((-C[3 * k + 0]) * min_lam[0] + (-C[3 * k + 1]) * min_lam[1]) + (-C[3 * k + 2]) * min_lam[2];
    nl::launch_legacy_shift(d_X_fixed, int(nat), t, num_sms(), st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "launch cell fix shift");
    for (int k = 0; k < 3; ++k) {
      max_lam[k] = max_lam[k] - min_lam[k];
      min_lam[k] = 0.0;
    }
    for (int k = 0; k < 3; ++k)
      if (max_lam[k] > 1) max_lam[k] = max_lam[k] * 1.01;
    for (int r = 0; r < 3; ++r)  // row r of the new cell = max_lam[r] * row r
      for (int c = 0; c < 3; ++c) cell_fixed[r + 3 * c] = max_lam[r] * C[r + 3 * c];
  }
  return NL_OK;
}

int nl_legacy_count_pairs(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                          const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                          int index_bytes, void* d_first, int64_t* total_pairs, void* d_workspace,
                          size_t workspace_bytes, void* stream) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_first || (nat > 0 && !d_X))
    return fail(NL_ERR_ARG, "null argument");
  if (!(cutoff > 0)) return fail(NL_ERR_ARG, "cutoff must be positive");
  LegacyLayout Q;
  int s = legacy_check(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, Q);
  if (s) return s;
  const nl::Geometry g = make_geometry(cell, inv_cell, ncells, nullptr, pbc, cutoff, nat);
  const nl::LegacyGeo lg = legacy_geo(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    s = legacy_count_impl<int32_t>(d_X, nat, g, lg, static_cast<int32_t*>(d_first), d_workspace, Q, st);
  else
    s = legacy_count_impl<int64_t>(d_X, nat, g, lg, static_cast<int64_t*>(d_first), d_workspace, Q, st);
  if (s) return s;
  if (total_pairs) {
    if (nat == 0) {
      *total_pairs = 0;
      return sync_read(d_workspace, st, nullptr, nullptr);
    }
    return sync_read(d_workspace, st, at<long long>(d_workspace, Q.L.totals) + 1, total_pairs);
  }
  return NL_OK;
}

int nl_legacy_fill_pairs(int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                         const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes,
                         const void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, void* d_workspace,
                         size_t workspace_bytes, void* stream) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_first) return fail(NL_ERR_ARG, "null argument");
  if (capacity > 0 && (!d_i || !d_j || !d_S)) return fail(NL_ERR_ARG, "null argument");
  LegacyLayout Q;
  int s = legacy_check(nat, ncells, nxyz, index_bytes, d_workspace, workspace_bytes, Q);
  if (s) return s;
  const nl::LegacyGeo lg = legacy_geo(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (index_bytes == 4)
    return legacy_fill_impl<int32_t>(lg, static_cast<const int32_t*>(d_first), capacity, static_cast<int32_t*>(d_i),
                                     static_cast<int32_t*>(d_j), static_cast<int32_t*>(d_S), d_workspace, Q, st);
  return legacy_fill_impl<int64_t>(lg, static_cast<const int64_t*>(d_first), capacity, static_cast<int64_t*>(d_i),
                                   static_cast<int64_t*>(d_j), static_cast<int64_t*>(d_S), d_workspace, Q, st);
}

int nl_sync_status(void* d_workspace, void* stream) {
  if (!d_workspace) return fail(NL_ERR_ARG, "null workspace");
  return sync_read(d_workspace, static_cast<cudaStream_t>(stream), nullptr, nullptr);
}

int nl_last_recheck_count(void* d_workspace, void* stream, int64_t* rechecks) {
  if (!d_workspace || !rechecks) return fail(NL_ERR_ARG, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  long long* h = pinned_scratch();
  if (!h) return fail(NL_ERR_NOMEM, "cannot allocate pinned host scratch");
  cudaError_t e = cudaMemcpyAsync(h, static_cast<char*>(d_workspace) + 64, sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "read statistics");
  *rechecks = h[0];
  return NL_OK;
}

}  // extern "C"
