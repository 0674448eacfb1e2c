// Launchers of the pair-traversal kernels (nl_pairs.cu).
#pragma once
#include "nl_common.cuh"

namespace nl {

enum PairMode : int { kModeCount = 0, kModeFill = 1, kModeLazyR6 = 2 };

// The count pass records, per home atom, its accepted candidates in the
// reference's traversal order -- (sorted slot of j, candidate word) -- in a
// list of kListCap entries.  The write pass (k_emit) turns the lists into
// i, j, S, R without screening again; cells with an atom of more than
// kListCap pairs are listed for the screening write pass instead.
#ifndef NL_LIST_CAP
#define NL_LIST_CAP 192
#endif
constexpr int kListCap = NL_LIST_CAP;  // at most 255 * 32 (the write pass numbers passes in 8 bits)

// doubles in one C'S table (|S_k| <= 2)
constexpr int kCsTableDoubles = 3 * 125;

// A batch of independent systems is laid out as concatenated slots: system
// s owns sorted slots / original atoms [sys_atom[s], sys_atom[s+1]) and cells
// [sys_cell[s], sys_cell[s+1]) of the batch.  Its caller-facing arrays are
// the reference's per-system arrays placed one after another: perm and
// cell_id hold system-local 1-based values, and its cell_offsets (ncells+1
// entries) start at sys_cell[s] + s.
// Per sorted slot, what the original-order write pass gathers for a
// neighbour: its FP64 position, 1-based original index (perm) and record
// meta (windings, exact bit), in one 32-byte row (two 16-byte loads).
struct __align__(32) XPack {  // 32-byte aligned: read as one 256-bit load
  double x, y, z;
  int perm;
  unsigned meta;
};
static_assert(sizeof(XPack) == 32, "one 32-byte row per slot");
// An atom's row by its original index, for the original-order write pass
struct __align__(16) ORow {
  double x, y, z;
  int slot;  // sorted slot (0-based, the launch's)
  int cell;  // home cell (0-based, the launch's)
};
static_assert(sizeof(ORow) == 32, "one 32-byte row per original atom");

template <typename TI>
struct PairArgs {
  Geometry g;               // single system (nsys == 0)
  const Geometry* geo;      // batch: geometry of each system
  const int* sys_atom;      // batch: nsys+1 slot offsets
  const int* sys_cell;      // batch: nsys+1 cell offsets
  const int* cell_sys;      // batch: system of each cell
  const double* cs_sys;     // batch: C'S table of each system
  int nsys;                 // 0 for a single system
  int nat_total;            // slots of the whole launch
  int ncells_total;         // cells of the whole launch
  const TI* cell_offsets;   // 1-based CSR over cells (ncells+1 per system)
  const TI* perm;           // sorted slot -> 1-based original index within the system
  const double* Xs;         // sorted positions (nat x 3)
  const float4* rec;        // sorted FP32 records
  const int* scell;         // sorted slot -> 0-based cell index
  const TI* first;          // fill: 1-based pair offsets per original atom of the launch (nat_total+1)
  int* counts;              // count: pairs per original atom of the launch
  TI* oi;                   // fill outputs (1-based i, j; S as 3 x TI; R as 3 x double)
  TI* oj;
  TI* oS;
  double* oR;               // may be null (R not wanted)
  long long capacity;       // pairs the output buffers hold
  double* per_atom;         // lazy: per-atom reduction
  uint2* lists;             // per sorted slot: list_cap accepted (slot_j, candidate word)
  int* lcount;              // per sorted slot: pairs of the atom (count pass)
  int* sorig;               // per sorted slot: original atom index within the launch (0-based)
  ORow* orow;               // per original atom: position, sorted slot, home cell (symmetric count pass)
  XPack* xpk;               // per sorted slot: gather row of the original-order write pass (symmetric count pass)
  int list_cap;             // kListCap, or 0: no lists (every cell takes the screening write pass)
  int* cap_rec;             // list_cap of the count pass (the write pass checks it)
  double* cs_table;         // C'S for |S_k| <= 2 (built once per call by k_cs_table)
  int* screen_cells;            // count pass: home cells left to the screening write pass
  int* n_screen_cells;          // length of that list
  int* cell_flag;           // per cell (zeroed per count): already in that list
  int count_kernel;         // 1: one warp per home cell, 2: one thread per home atom (0 / 3: see sym)
  int sym;                  // count / write: each unordered cell pair screened once, neighbour masks
  int* sym_fail;            // set when a cell has more than 32 atoms: lists and the per-cell pass instead
  int sym_gate;             // a fused symmetric lazy pass already ran (launched by the caller, not by the
                            // count launcher): the per-cell passes run only if it set sym_fail
  int* sym_wound;           // bit 0: an atom has a winding or is exact (candidate words need its record);
                            // bit 1: a coordinate is -0 (R needs the signed-zero rule of C'S with S = 0)
  const int* sys_sym;       // batch: 1 for the systems the symmetric pass takes (27 distinct stencil cells)
  int* sys_fail;            // batch: per system, like sym_fail (zeroed per call)
  int half;                 // count / write: keep each unordered pair once (j > i, or j == i and S > 0)
  int pair_blocks_per_sm;   // launch tuning (0 = default): count / screening grids
  int emit_blocks_per_sm;   // launch tuning (0 = default): list write grid
  int vec_ok;               // S and R start on 16-byte boundaries: the write pass stores 16-byte vectors
  unsigned* stab;           // stencil table: 28 words per cell (symmetric pass -> mask write passes)
  int* work;                // batch: cell counters of the count and screening passes (zeroed per call)
  // batches with the symmetric pass: the cells and 32-slot chunks of the
  // systems it does not take (n_nonsym_* of them, uploaded), then those of
  // the systems that fail it, appended by the pass (extra_* counts them)
  int* nonsym_cells;
  int n_nonsym_cells;
  int* nonsym_chunks;
  int n_nonsym_chunks;
  int* extra_cells;
  int* extra_chunks;
  // the count pass over those cells takes 32 home atoms of a cell at a time:
  // a first launch takes each cell's first 32 and lists the rest in rounds
  // (cell, round; n_rounds of them), a second (round_pass) takes the rounds
  int2* rounds;
  int* n_rounds;
  int* round_work;
  int round_pass;
  unsigned long long* stats;  // [0] += FP64 rechecks
  unsigned* err;
};

// largest s in [0, nsys) with first[s] <= x (first nondecreasing)
__device__ __forceinline__ int batch_system(const int* __restrict__ first, int nsys, int x) {
  int lo = 0, hi = nsys - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <typename TI>
void launch_pairs(int mode, const PairArgs<TI>& a, int num_sms, cudaStream_t st);

// The fused symmetric lazy passes of single systems whose 27-cell stencil has
// distinct cells: per-atom counts (into a.counts, zeroed by the caller) or
// per-atom sums of 1/r^6 (into a.per_atom, zeroed by the caller).  A cell of
// more than 32 atoms sets a.sym_fail; the caller's per-cell passes (gated on
// it) then redo the whole reduction.
enum LazyWhat : int { kLazyCounts = 0, kLazyInvR6 = 1 };
template <typename TI>
void launch_sym_lazy(int what, const PairArgs<TI>& a, int num_sms, cudaStream_t st);

// R = (X[j] - X[i]) + C'S of an existing list; largest squared displacement
template <typename TI>
void launch_pair_vectors(const Geometry& g, const double* X, const TI* pi, const TI* pj, const TI* pS,
                         long long npairs, double* R, int num_sms, cudaStream_t st);
void launch_max_disp_sq(const double* X, const double* Xref, long long nat, unsigned long long* out, int num_sms,
                        cudaStream_t st);

// batches: the C'S table of every system, the system of every cell
void launch_cs_tables(const Geometry* geo, int nsys, double* out, cudaStream_t st);
void launch_cell_systems(const int* sys_cell, int nsys, int* out, cudaStream_t st);

}  // namespace nl
