// Launchers of the single-precision path (nl_f32.cu).
//
// The reference is generic in the float type T of the positions: with
// T = Float32 (its GPU tests run Float64 and Float32, test/test_gpu.jl:14,
// test/test_utils.jl:239) build_cell_list converts the cell and cutoff to
// Float32 (cell_list.jl:637-639) and every floating-point operation of
// analyze_cell, position_to_cell_index, R = xj - xi + C'S and the distance
// test runs in single precision.  These kernels do the same operations in
// FP32 with round-to-nearest and no contraction, so the cell list and the
// pairs (i, j, S, first and the bits of R) equal the reference's.
#pragma once
#include "nl_common.cuh"

namespace nl {

struct Geo32 {
  float C[9];        // cell, column-major, rows = lattice vectors
  float inv[9];      // inv(cell) in Float32 (StaticArrays operation order)
  float cutoff_sq;   // cutoff^2 in Float32
  int ns[3];
  int nxyz[3];
  int pbc[3];
  int ncells;
  int nat;
};

// A single-precision record is (x, y, z, meta): the caller's coordinates and
// the windings of the atom's cell, each biased by kW32Bias in a 10-bit field.
constexpr int kW32Bias = 512;

template <typename TI>
struct Pairs32Args {
  Geo32 g;
  const float4* rec;         // sorted records
  const int* scell;          // sorted slot -> 0-based cell
  const TI* cell_offsets;    // 1-based CSR over cells (ncells + 1)
  const TI* perm;            // sorted slot -> 1-based original index
  int* counts;               // count: pairs per original atom
  const TI* first;           // fill: 1-based pair offsets (nat + 1)
  TI* oi;
  TI* oj;
  TI* oS;
  float* oR;                 // may be null
  long long capacity;
  unsigned* err;
  // symmetric count (27-cell stencils of distinct cells): 27 neighbour-mask
  // words per atom, then 54 words of stencil table per cell, in `masks`
  int sym;
  unsigned* masks;
  int* sym_fail;             // a cell of more than 32 atoms: the per-cell passes run instead
  int half;                  // keep each unordered pair once: j > i, or j == i and S > 0 lexicographically
  // batches (nsys > 0): per-system geometry, slot and cell offsets of each
  // system in the launch, the system of every cell; cell_offsets, perm and
  // the pair outputs hold system-local values, counts and first are
  // launch-wide (index: the system's first slot + local index)
  const Geo32* geos;
  const int* sys_atom;       // nsys + 1
  const int* sys_cell;       // nsys + 1
  const int* cell_sys;       // ncells_total
  int* work;                 // cell counters of the count and fill passes (zeroed per call)
  // batches: a cell's home atoms are taken 32 at a time -- a first launch of
  // each pass takes every cell's first 32 (the count pass lists the other
  // rounds: cell, round), a second (round_pass) the listed rounds
  int2* rounds;
  int* n_rounds;
  int* round_work;           // counters of the second launches (count, fill)
  int round_pass;
  int nsys;
  int nat_total;
  int ncells_total;
};

// binning of the caller's positions (cell id, ticket, record, histogram)
void launch_bin32(const Geo32& g, const float* X, int nat, int* cid, int* ticket, float4* rec, int* cell_count,
                  unsigned* err, int num_sms, cudaStream_t st);
// the same for a batch: atom i of the launch belongs to the system s with
// atom0[s] <= i < atom0[s + 1] and is binned with geos[s]; its cell index is
// offset by cell0[s]
void launch_bin32_batch(const Geo32* geos, const int* atom0, const int* cell0, int nsys, const float* X, int nat,
                        int* cid, int* ticket, float4* rec, int* cell_count, unsigned* err, int num_sms,
                        cudaStream_t st);
// records of an existing sorted cell list (checks its cell ids)
template <typename TI>
void launch_prepare32(const Geo32& g, const float* Xs, const TI* cell_id, const TI* perm, int nat, float4* rec_sorted,
                      int* scell, unsigned* err, int num_sms, cudaStream_t st);
// count (fill = false) or fill (fill = true) pass
template <typename TI>
void launch_pairs32(bool fill, const Pairs32Args<TI>& a, int num_sms, cudaStream_t st);
// R of a whole list at new positions (Verlet reuse), and the largest squared
// displacement since a reference configuration (bits of a non-negative float)
template <typename TI>
void launch_pair_vectors32(const Geo32& g, const float* X, const TI* pi, const TI* pj, const TI* pS, long long npairs,
                           float* R, int num_sms, cudaStream_t st);
void launch_max_disp_sq32(const float* X, const float* Xref, long long nat, unsigned* out, int num_sms,
                          cudaStream_t st);

}  // namespace nl
