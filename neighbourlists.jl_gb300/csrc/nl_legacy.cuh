// Launchers of the legacy linked-list path (nl_legacy.cu).
//
// The reference keeps its original linked-list PairList constructor
// (PairList(X::Vector{SVec}, cutoff, cell, pbc; int_type, fixcell),
// cell_list.jl:11-20) as a second implementation: _fix_cell_ moves atoms into
// the cell (:459-505), _celllist_ bins them into linked lists (:185-230),
// _find_neighbours_! screens with cell-local coordinates (:301-366), and
// sort_neigs! orders each atom's neighbours by j (:427-446).  Its arithmetic
// differs from the sort-based path (the distance is formed from positions
// relative to the lower corner of each atom's bin, the shift by a truncating
// division), so near-cutoff membership and S can differ from the sort-based
// list; these kernels follow the legacy arithmetic exactly.
#pragma once
#include "nl_common.cuh"

namespace nl {

// Geometry of one legacy list, passed by value.
struct LegacyGeo {
  double inv[9];    // inv(cell), column-major
  double bins[9];   // bins[r + 3k] = cell[k, r] / ns[k]: column k is lattice vector k / ns[k]
  float binsf[9];   // bins rounded to FP32 (the screen's stencil offsets)
  double cutoff_sq; // cutoff^2 (cutoff * cutoff)
  double cutoff;
  double offmax;    // bound on |(bins * xyz)_r| over the stencil
  int ns[3];
  int nxyz[3];
  int pbc[3];
  int ncells;
  int nat;
};

template <typename TI>
struct LegacyArgs {
  LegacyGeo g;
  const double* Xs;        // sorted positions (nat x 3)
  const TI* perm;          // sorted slot -> 1-based original index
  const int* cell_start;   // 0-based CSR over cells (ncells + 1)
  double* D;               // per slot: position relative to the lower corner of its (clamped) bin, 3 doubles
  float4* Df;              // per slot: D rounded to FP32; w = 1 when c0 lies in the box on every periodic axis
  int4* c0;                // per slot: unwrapped cell index floor(frac * ns + 1)
  unsigned* dmax;          // max |D_r| over the atoms, FP32 bits rounded up
  int* counts;             // count: pairs per original atom (0-based)
  const TI* first;         // fill: 1-based pair offsets (nat + 1)
  TI* oi;
  TI* oj;
  TI* oS;
  long long capacity;
  int blocks_per_sm;
  unsigned long long* stats;  // [0] += FP64 rechecks
  unsigned* err;
};

// Largest and smallest fractional coordinate seen on the open axes, as
// order-preserving integer keys of the doubles (6 words: min0..2, max0..2).
__host__ __device__ inline unsigned long long legacy_key(double d) {
  unsigned long long u;
  memcpy(&u, &d, sizeof(u));
  return (u >> 63) ? ~u : (u | (1ull << 63));
}
inline double legacy_unkey(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & ~(1ull << 63)) : ~k;
  double d;
  memcpy(&d, &u, sizeof(d));
  return d;
}

// _fix_cell_ (cell_list.jl:459-505), per atom: wraps the periodic fractional
// coordinates outside [0, 1) with Julia's mod(x, 1.0) and rewrites the
// position as cell' * lambda, and records the open-axis extremes in minmax.
void launch_legacy_fix(const double* inv, const double* C, const int* pbc, const double* X, double* Xout, int nat,
                       unsigned long long* minmax, unsigned* err, int num_sms, cudaStream_t st);
// X += t for every atom (the open-axis shift of _fix_cell_)
void launch_legacy_shift(double* X, int nat, const double* t, int num_sms, cudaStream_t st);
// per sorted slot: D, Df, c0 and dmax
template <typename TI>
void launch_legacy_prepare(const LegacyArgs<TI>& a, int num_sms, cudaStream_t st);
// count (fill = false) or fill (fill = true) pass
template <typename TI>
void launch_legacy_pairs(bool fill, const LegacyArgs<TI>& a, int num_sms, cudaStream_t st);

}  // namespace nl
