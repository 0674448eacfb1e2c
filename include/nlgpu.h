/*
 * nlgpu.h -- C ABI of the GB300 (sm_103a) neighbour-list engine.
 *
 * Drop-in boundary for the sort-based path of NeighbourLists.jl v0.6.2:
 *   neighbour_list(X, cutoff, cell, pbc; lazy)  (src/cell_list.jl:897-916)
 *   -> build_cell_list                          (src/cell_list.jl:632-679)
 *   -> materialize_pairlist / for_each_neighbour (src/gpu_kernels.jl:299-364,
 *                                                 src/cell_list.jl:779-833)
 *
 * Conventions (identical to the reference's data layout):
 *   - positions: nat x 3 doubles, atom-major (Vector{SVector{3,Float64}});
 *   - cell / inv_cell: 9 doubles, column-major (SMatrix{3,3} memory order),
 *     ROWS of the cell are the lattice vectors;
 *   - every index array is 1-based in the caller's index type TI, selected by
 *     index_bytes = 4 (Int32) or 8 (Int64); S is nat_pairs x 3 TI (SVector{3,TI});
 *   - device pointers ("d_" prefix) are CUDA device memory; "stream" is a
 *     cudaStream_t passed as void* (NULL = legacy default stream);
 *   - every function returns an NL_* status; nl_last_error() gives details
 *     for the calling thread.
 *
 * Ownership: the caller owns every input/output buffer and the workspace
 * (sized by nl_workspace_bytes).  The library allocates no device memory at
 * run time; its device image holds the 32 MiB scratch array of
 * nl_neighbour_list_static.
 */
#ifndef NLGPU_H
#define NLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define NL_OK 0
#define NL_ERR_ARG 1              /* invalid argument */
#define NL_ERR_TOO_MANY_CELLS 2   /* cell_list.jl:655-659 "Ratio of simulation cell size to cutoff is very large" */
#define NL_ERR_NOMEM 3            /* workspace or host allocation too small */
#define NL_ERR_CUDA 4             /* CUDA runtime error */
#define NL_ERR_TIMEOUT 5          /* a bounded device-side wait gave up */
#define NL_ERR_BAD_POSITION 6     /* non-finite position or |frac*ncells| >= 2^30 */
#define NL_ERR_CAPACITY 7         /* pair buffers smaller than the pair count */
#define NL_ERR_INDEX_OVERFLOW 8   /* pair count does not fit the index type */
#define NL_ERR_INCONSISTENT 9     /* a cell list whose cell ids do not match its positions */

/* lazy reductions (nl_lazy_reduce) */
#define NL_REDUCE_COUNT 0         /* int32 per atom: count_neighbours (cell_list.jl:808-814) */
#define NL_REDUCE_INV_R6 1        /* double per atom: sum over neighbours of 1/r^6, in traversal order (bit-exact) */
#define NL_REDUCE_INV_R6_FAST 2   /* the same sum from the neighbour masks, each unordered pair once: relative
                                     error <= 1e-12, last bits vary with the order of the atomic additions */

/* Cell analysis: the reference's analyze_cell (cell_list.jl:152-170) plus the
 * stencil half-width nxyz of materialize_pairlist (gpu_kernels.jl:315-316),
 * and the FP32 screen band of this engine. */
typedef struct nl_cell_plan {
  double inv_cell[9];   /* inv(cell), column-major (StaticArrays operation order) */
  double lens[3];       /* abs.(lengths(cell)) */
  int64_t ncells[3];    /* max(floor(lens/cutoff), 1) */
  int64_t nxyz[3];      /* ceil(cutoff * ncells / lens) */
  int64_t ncells_total; /* prod(ncells) */
  double band;          /* half-width of the FP64 recheck band on r^2 (A^2) */
} nl_cell_plan;

/* Replaces analyze_cell (cell_list.jl:152-170) + nxyz (gpu_kernels.jl:315-316). */
int nl_analyze_cell(const double cell[9], double cutoff, int index_bytes, nl_cell_plan* plan);

/* Device workspace needed by every call below for a system of nat atoms and
 * ncells_total cells. */
size_t nl_workspace_bytes(int64_t nat, int64_t ncells_total);

/* Smallest workspace every call accepts: without room for the per-atom pair
 * lists of the count pass, every cell is written by the (slower) screening
 * write pass, with identical results.  Count and fill of one list must be
 * given the same workspace size (a mismatch is reported as
 * NL_ERR_INCONSISTENT). */
size_t nl_workspace_min_bytes(int64_t nat, int64_t ncells_total);

/* Replaces build_cell_list / _build_sorted_celllist (cell_list.jl:632-679),
 * i.e. _compute_cell_ids (gpu_kernels.jl:244-255,378-382), _get_sortperm
 * (cell_list.jl:711-718) and _compute_cell_offsets (gpu_kernels.jl:262-285,
 * 386-390).  Fills the SortedCellList arrays:
 *   d_perm[nat], d_X_sorted[nat*3], d_cell_id[nat], d_cell_offsets[ncells_total+1].
 * inv_cell / ncells are the caller's analyze_cell results.  Asynchronous. */
int nl_build_cell_list(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                       const int64_t ncells[3], const uint8_t pbc[3], double cutoff, int index_bytes,
                       void* d_perm, double* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                       void* d_workspace, size_t workspace_bytes, void* stream);

/* Replaces count_neighbours_kernel! + compute_pair_offsets + _scalar_getindex
 * (gpu_kernels.jl:132-152, 222-237, 320-333).  From a SortedCellList (any
 * producer) writes d_first[nat+1] (1-based CSR offsets per atom).  If
 * total_pairs is non-NULL the call synchronises the stream and stores the pair
 * count there (and reports any device-side error).  reuse_records = 1 skips the
 * per-atom record rebuild when the same workspace was just used by
 * nl_build_cell_list for this very cell list. */
int nl_count_pairs(const double* d_X_sorted, const void* d_perm, const void* d_cell_id, const void* d_cell_offsets,
                   int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                   const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes, int reuse_records,
                   void* d_first, int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream);

/* Replaces fill_pairs_kernel! (gpu_kernels.jl:159-180) and adds the pair
 * vectors R = X[j] - X[i] + cell' * S (_getR, cell_list.jl:525-531).
 * Requires the records of a preceding nl_count_pairs / nl_neighbour_list in
 * the same workspace.  Writes d_i, d_j [capacity], d_S [capacity*3] and, if
 * d_R is not NULL, d_R [capacity*3].  Asynchronous. */
int nl_fill_pairs(const double* d_X_sorted, const void* d_perm, const void* d_cell_offsets, int64_t nat,
                  const double cell[9], const double inv_cell[9], const int64_t ncells[3], const int64_t nxyz[3],
                  const uint8_t pbc[3], double cutoff, int index_bytes, const void* d_first, int64_t capacity,
                  void* d_i, void* d_j, void* d_S, double* d_R, void* d_workspace, size_t workspace_bytes,
                  void* stream);

/* Whole materialised path, neighbour_list(X, cutoff, cell, pbc) with
 * lazy = false (cell_list.jl:897-916): build + count + scan + fill in one
 * stream-ordered sequence with no host synchronisation in between.  Pairs
 * are written only if they fit in capacity.  If total_pairs is non-NULL the
 * call synchronises, stores the pair count and returns NL_ERR_CAPACITY when
 * it exceeds capacity (the cell list, first and the records stay valid:
 * re-run nl_fill_pairs with larger buffers). */
int nl_neighbour_list(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                      const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                      int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                      void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                      int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream);

/* nl_neighbour_list for a half list: of the two directions (i, j, S) and
 * (j, i, -S) of every pair only the one with j > i is kept, and for a
 * periodic image of an atom itself (j == i) the one with S > 0
 * lexicographically; each atom's pairs stay in the reference's order.  No
 * counterpart in the reference (force loops that visit every pair once). */
int nl_neighbour_list_half(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                           const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                           int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                           void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                           int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream);

/* R = (X[j] - X[i]) + C'S for every pair of an existing list, the
 * reference's _getR (cell_list.jl:525-531) over the whole list: d_X are the
 * original-order positions (nat x 3), d_i / d_j 1-based, d_S npairs x 3, all
 * in the index type.  Used for lists built without R and for Verlet reuse
 * (the pairs of an earlier list, the positions of now).  Asynchronous. */
int nl_pair_vectors(const double* d_X, int64_t nat, const double cell[9], int index_bytes, const void* d_i,
                    const void* d_j, const void* d_S, int64_t npairs, double* d_R, void* stream);

/* Largest |X[a] - X_ref[a]|^2 over the atoms (FP64; NaN if any position is
 * NaN) into *d_out; the Verlet skin test of a reused list.  No counterpart in
 * the reference.  Asynchronous; d_out is device memory. */
int nl_max_displacement_sq(const double* d_X, const double* d_Xref, int64_t nat, double* d_out, void* stream);

/* Lazy mode (for_each_neighbour over every atom, cell_list.jl:779-814) with a
 * built-in per-atom reduction: NL_REDUCE_COUNT -> int32 d_out[nat];
 * NL_REDUCE_INV_R6 -> double d_out[nat] = sum_j 1/((r2*r2)*r2), r2 = dot(R,R),
 * accumulated in the reference's traversal order (bit-identical to a
 * sequential for_each_neighbour sum); NL_REDUCE_INV_R6_FAST -> the same sum
 * screened and reduced in one pass that visits each unordered pair once (R
 * with the reference's FP64 operations, 1/r^6 in double-float, atomic
 * accumulation): relative error at most 1e-12.  Where the stencil is not 27
 * distinct cells, or a cell holds more than 32 atoms, the fast op computes
 * the traversal-order sum.  Asynchronous. */
int nl_lazy_reduce(const double* d_X_sorted, const void* d_perm, const void* d_cell_id, const void* d_cell_offsets,
                   int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                   const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes, int reuse_records,
                   int op, void* d_out, void* d_workspace, size_t workspace_bytes, void* stream);

/* Lazy per-atom traversal for a set of query atoms, without materialising
 * the system's list.  Replaces neighbours(clist, i) and
 * count_neighbours(clist, i) (cell_list.jl:808-833), i.e. for_each_neighbour
 * (cell_list.jl:779-801) / _for_each_neighbor_pair (gpu_kernels.jl:58-101)
 * for each atom of d_atoms[0 .. nq-1] (1-based original indices, TI).
 * d_X is the cell list's X_orig, d_X_sorted / d_perm / d_cell_offsets its
 * sorted arrays.  Count mode (d_j == NULL): d_counts[k] (int64) = the number
 * of neighbours of atom d_atoms[k].  Fill mode: the neighbours of d_atoms[k]
 * -- j (1-based), S (3 x TI) and, if d_R is not NULL, R (3 doubles) -- are
 * written from pair d_offsets[k] (int64, 0-based) in the reference's
 * traversal order; pairs at or beyond capacity are not written
 * (NL_ERR_CAPACITY).  Every decision is the reference's FP64 arithmetic.
 * The device-side error word is the first word of d_workspace (any
 * workspace of at least 128 bytes; read it with nl_sync_status).
 * Asynchronous. */
int nl_query_neighbours(const double* d_X, const double* d_X_sorted, const void* d_perm, const void* d_cell_offsets,
                        int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                        const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes,
                        const void* d_atoms, int64_t nq, int64_t* d_counts, const int64_t* d_offsets, int64_t capacity,
                        void* d_j, void* d_S, double* d_R, void* d_workspace, size_t workspace_bytes, void* stream);

/* nl_neighbour_list without a workspace, for callers that cannot allocate
 * device memory (a framework pool owns the device, a real-time loop forbids
 * allocation after start-up, or the host code may not call cudaMalloc).  No
 * counterpart in the reference: it exists only because this engine needs
 * scratch memory.  The scratch is a fixed 32 MiB array inside the library,
 * present on every GPU that loads it until the process exits; systems that
 * need more (about 500k atoms at liquid density) are rejected with
 * NL_ERR_NOMEM.  The first call on each device resolves the array's address
 * and should come before any stream capture.  Every call reuses the same
 * array: calls that overlap on the GPU race and must be serialised.  The call
 * allocates nothing; pass total_pairs to synchronise and get the pair count
 * and the status of the device-side checks. */
int nl_neighbour_list_static(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                             const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                             int index_bytes, void* d_perm, double* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                             void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                             int64_t* total_pairs, void* stream);

/* Status of the last nl_neighbour_list_static call on the current device,
 * for callers that made it asynchronously (total_pairs = NULL): synchronises
 * `stream`, then returns the result of that call's device-side checks
 * (NL_ERR_CAPACITY, NL_ERR_BAD_POSITION, NL_ERR_INDEX_OVERFLOW, ...) and, if
 * total_pairs is not NULL, its pair count.  Like the call it reports on, it
 * allocates nothing.  No counterpart in the reference. */
int nl_static_sync_status(int64_t* total_pairs, void* stream);

/* ---- batches of independent systems -------------------------------------
 * No counterpart in the reference, which handles one system per call: a
 * batch replaces a loop of neighbour_list(X_s, cutoff_s, cell_s, pbc_s)
 * calls (cell_list.jl:897-916) by one launch per stage over all systems.
 *
 * Layout: the atoms of system s are rows atom0[s] .. atom0[s]+nat_s-1 of the
 * batch's X (atom0 = running sum of nat).  Every per-system output is the
 * reference's array for that system, placed one after another in system
 * order, with system-local 1-based values:
 *   perm, cell_id, X_sorted : at atom0[s]            (nat_s entries)
 *   cell_offsets            : at cell0[s] + s        (ncells_s + 1 entries)
 *   first                   : at atom0[s] + s        (nat_s + 1 entries)
 *   i, j, S, R              : at pair_offsets[s]     (npairs_s entries)
 * where cell0 is the running sum of ncells_total and pair_offsets (nsys + 1
 * int64, written by the call) the running sum of the pair counts. */
typedef struct nl_system {
  int64_t nat;          /* atoms of this system */
  double cell[9];       /* column-major, rows = lattice vectors */
  double inv_cell[9];   /* the caller's analyze_cell results, as for nl_build_cell_list */
  int64_t ncells[3];
  int64_t nxyz[3];
  uint8_t pbc[3];
  double cutoff;
} nl_system;

typedef struct nl_batch nl_batch;   /* host-side plan of a batch (opaque) */

/* Validates the systems and builds the host plan.  index_bytes applies to
 * every system. */
int nl_batch_create(const nl_system* systems, int nsys, int index_bytes, nl_batch** batch);
/* Same, from raw systems: cells[9*s..] column-major, cutoffs[s], pbc[3*s..],
 * nat[s]; the cell analysis (analyze_cell + nxyz, as nl_analyze_cell) runs
 * inside.  For callers that assemble many small systems per batch (serving). */
int nl_batch_create_auto(const double* cells, const double* cutoffs, const uint8_t* pbc, const int64_t* nat, int nsys,
                         int index_bytes, nl_batch** batch);
void nl_batch_destroy(nl_batch* batch);
/* Workspace bytes for the batch, and its total atoms / cells. */
size_t nl_batch_workspace_bytes(const nl_batch* batch);
int nl_batch_sizes(const nl_batch* batch, int64_t* total_atoms, int64_t* total_cells);
/* Copies the batch's geometry tables into the workspace (returns after the
 * copy has completed).  Needed once per workspace before any run; runs do
 * not modify the tables, so many runs (and stream captures of runs) can
 * follow one upload. */
int nl_batch_upload(const nl_batch* batch, void* d_workspace, size_t workspace_bytes, void* stream);
/* Build + count + fill of every system of the batch, stream-ordered, with
 * no host synchronisation unless total_pairs is non-NULL (then as
 * nl_neighbour_list: the batch's total pair count, NL_ERR_CAPACITY when it
 * exceeds capacity). */
int nl_batch_neighbour_list(const nl_batch* batch, const double* d_X, void* d_perm, double* d_X_sorted,
                            void* d_cell_id, void* d_cell_offsets, void* d_first, int64_t* d_pair_offsets,
                            int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R, int64_t* total_pairs,
                            void* d_workspace, size_t workspace_bytes, void* stream);

/* ---- Float32 positions ----------------------------------------------------
 * The reference is generic in the position type T; with T = Float32 (its GPU
 * tests run Float64 and Float32, test/test_gpu.jl:14, test/test_utils.jl:239)
 * build_cell_list converts cell and cutoff to Float32 (cell_list.jl:637-639)
 * and every floating-point operation -- analyze_cell, position_to_cell_index,
 * R = xj - xi + C'S, dot(R, R) < cutoff^2 -- rounds to Float32.  These calls
 * are the Float64 calls above with that arithmetic: positions (nat x 3), the
 * cell and cutoff and R (npairs x 3) are float; the index arrays and the
 * workspace (nl_workspace_bytes) are unchanged.  Positions whose winding
 * exceeds 511 box lengths cannot be binned (NL_ERR_BAD_POSITION). */
typedef struct nl_cell_plan_f32 {
  float inv_cell[9];    /* inv(cell) in Float32, column-major */
  float lens[3];        /* abs.(lengths(cell)) in Float32 */
  int64_t ncells[3];
  int64_t nxyz[3];
  int64_t ncells_total;
} nl_cell_plan_f32;

/* analyze_cell (cell_list.jl:152-170) + nxyz (gpu_kernels.jl:315-316) in Float32. */
int nl_analyze_cell_f32(const float cell[9], float cutoff, int index_bytes, nl_cell_plan_f32* plan);
/* nl_build_cell_list for Float32 positions. */
int nl_build_cell_list_f32(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                           const int64_t ncells[3], const uint8_t pbc[3], float cutoff, int index_bytes, void* d_perm,
                           float* d_X_sorted, void* d_cell_id, void* d_cell_offsets, void* d_workspace,
                           size_t workspace_bytes, void* stream);
/* nl_count_pairs for Float32 positions. */
int nl_count_pairs_f32(const float* d_X_sorted, const void* d_perm, const void* d_cell_id, const void* d_cell_offsets,
                       int64_t nat, const float cell[9], const float inv_cell[9], const int64_t ncells[3],
                       const int64_t nxyz[3], const uint8_t pbc[3], float cutoff, int index_bytes, int reuse_records,
                       void* d_first, int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream);
/* nl_fill_pairs for Float32 positions (d_R: capacity x 3 floats, may be NULL). */
int nl_fill_pairs_f32(const float* d_X_sorted, const void* d_perm, const void* d_cell_offsets, int64_t nat,
                      const float cell[9], const float inv_cell[9], const int64_t ncells[3], const int64_t nxyz[3],
                      const uint8_t pbc[3], float cutoff, int index_bytes, const void* d_first, int64_t capacity,
                      void* d_i, void* d_j, void* d_S, float* d_R, void* d_workspace, size_t workspace_bytes,
                      void* stream);
/* nl_neighbour_list for Float32 positions. */
int nl_neighbour_list_f32(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                          const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], float cutoff,
                          int index_bytes, void* d_perm, float* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                          void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R,
                          int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream);

/* nl_pair_vectors and nl_max_displacement_sq for Float32 positions (R by
 * the reference's single-precision operations; the displacement in FP32). */
int nl_pair_vectors_f32(const float* d_X, int64_t nat, const float cell[9], int index_bytes, const void* d_i,
                        const void* d_j, const void* d_S, int64_t npairs, float* d_R, void* stream);
int nl_max_displacement_sq_f32(const float* d_X, const float* d_Xref, int64_t nat, float* d_out, void* stream);
/* nl_neighbour_list_half for Float32 positions: each unordered pair once
 * (j > i, or j == i and S > 0 lexicographically), in the reference's order. */
int nl_neighbour_list_half_f32(const float* d_X, int64_t nat, const float cell[9], const float inv_cell[9],
                               const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], float cutoff,
                               int index_bytes, void* d_perm, float* d_X_sorted, void* d_cell_id, void* d_cell_offsets,
                               void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R,
                               int64_t* total_pairs, void* d_workspace, size_t workspace_bytes, void* stream);

/* Float32 batches: as nl_batch_create / nl_batch_neighbour_list with
 * T = Float32 for every system (cell, cutoff and the nl_analyze_cell_f32
 * results in Float32; positions, sorted positions and R in Float32).
 * nl_batch_workspace_bytes, nl_batch_sizes, nl_batch_upload, nl_batch_destroy
 * and nl_batch_set_tuning take either kind of batch; each run entry takes
 * only its own kind (NL_ERR_ARG otherwise).  Every per-system output equals a
 * single-system nl_neighbour_list_f32 call. */
typedef struct nl_system_f32 {
  int64_t nat;
  float cell[9];        /* column-major, rows = lattice vectors */
  float inv_cell[9];    /* the nl_analyze_cell_f32 results */
  int64_t ncells[3];
  int64_t nxyz[3];
  uint8_t pbc[3];
  float cutoff;
} nl_system_f32;
int nl_batch_create_f32(const nl_system_f32* systems, int nsys, int index_bytes, nl_batch** batch);
/* Same from raw systems (cells[9*s..] column-major, cutoffs[s] in Float32):
 * the Float32 cell analysis runs inside, as nl_batch_create_auto. */
int nl_batch_create_auto_f32(const float* cells, const float* cutoffs, const uint8_t* pbc, const int64_t* nat,
                             int nsys, int index_bytes, nl_batch** batch);
int nl_batch_neighbour_list_f32(const nl_batch* batch, const float* d_X, void* d_perm, float* d_X_sorted,
                                void* d_cell_id, void* d_cell_offsets, void* d_first, int64_t* d_pair_offsets,
                                int64_t capacity, void* d_i, void* d_j, void* d_S, float* d_R, int64_t* total_pairs,
                                void* d_workspace, size_t workspace_bytes, void* stream);

/* ---- legacy linked-list PairList -----------------------------------------
 * The reference's legacy constructor PairList(X::Vector{SVec}, cutoff, cell,
 * pbc; int_type, fixcell) (cell_list.jl:11-20, _pairlist_ :369-385), kept
 * there as a second implementation.  Its arithmetic differs from the
 * sort-based path: the distance is formed from bin-relative positions
 * (_find_neighbours_!, :301-366), S = (ci0 - cj + xyz) .÷ ns with a
 * truncating division, and each atom's neighbours are sorted by j
 * (sort_neigs!, :427-446; ties keep the traversal order).  These calls
 * reproduce it exactly: i, j, S and first equal the reference's.
 *
 * Sequence: nl_legacy_fix_cell (fixcell = true) -> nl_analyze_cell on the
 * fixed cell -> nl_legacy_count_pairs -> allocate -> nl_legacy_fill_pairs. */

/* Workspace the cell fix needs (any larger workspace works). */
#define NL_LEGACY_FIX_WORKSPACE_BYTES 256

/* Replaces _fix_cell_ (cell_list.jl:459-505): d_X_fixed (nat x 3, may equal
 * d_X) receives the positions with periodic fractional coordinates outside
 * [0, 1) wrapped by mod(., 1) and, when an open axis has atoms outside the
 * cell, every position shifted by -cell' * min_lambda; cell_fixed (host)
 * receives the cell, with the rows of such open axes enlarged.
 * Synchronises the stream (the new cell depends on the positions). */
int nl_legacy_fix_cell(const double* d_X, int64_t nat, const double cell[9], const uint8_t pbc[3], double* d_X_fixed,
                       double cell_fixed[9], void* d_workspace, size_t workspace_bytes, void* stream);

/* Device workspace of the legacy count / fill calls (it holds the legacy
 * cell list: the reference's legacy PairList does not return one). */
size_t nl_legacy_workspace_bytes(int64_t nat, int64_t ncells_total, int index_bytes);

/* Replaces _celllist_ + _pairlist_(clist) + get_first (cell_list.jl:185-297,
 * 401-418): bins the atoms (d_X: the positions the list refers to, after
 * the cell fix if any), counts each atom's pairs with the legacy arithmetic
 * and writes d_first[nat+1].  cell / inv_cell / ncells / nxyz are
 * nl_analyze_cell's results for that cell.  If total_pairs is non-NULL the
 * call synchronises and stores the pair count. */
int nl_legacy_count_pairs(const double* d_X, int64_t nat, const double cell[9], const double inv_cell[9],
                          const int64_t ncells[3], const int64_t nxyz[3], const uint8_t pbc[3], double cutoff,
                          int index_bytes, void* d_first, int64_t* total_pairs, void* d_workspace,
                          size_t workspace_bytes, void* stream);

/* Writes d_i, d_j [capacity] and d_S [capacity*3]: every atom's pairs sorted
 * by j as sort_neigs! leaves them (cell_list.jl:427-446).  Requires the
 * preceding nl_legacy_count_pairs in the same workspace.  Asynchronous;
 * pairs beyond capacity are not written (NL_ERR_CAPACITY at the next
 * nl_sync_status). */
int nl_legacy_fill_pairs(int64_t nat, const double cell[9], const double inv_cell[9], const int64_t ncells[3],
                         const int64_t nxyz[3], const uint8_t pbc[3], double cutoff, int index_bytes,
                         const void* d_first, int64_t capacity, void* d_i, void* d_j, void* d_S, void* d_workspace,
                         size_t workspace_bytes, void* stream);

/* ---- launch tuning ------------------------------------------------------
 * Grid sizes of the pair kernels, as picked by an autotuner (the Python
 * package's autotune()).  0 keeps the default (every resident block slot of
 * every SM).  Results never depend on the tuning. */
typedef struct nl_tuning {
  int pair_blocks_per_sm;   /* count / screening write / lazy kernels, 1..256 */
  int emit_blocks_per_sm;   /* list write kernel, 1..256 */
  int count_kernel;         /* 0 default (3 where it applies, else 1);
                               1 one warp per home cell; 2 one thread per home atom; 3 each unordered
                               pair of cells screened once with neighbour masks (systems whose 27-cell
                               stencil has distinct cells, single or in a batch; a system with a cell
                               of more than 32 atoms falls back to 1) */
} nl_tuning;

/* Tuning of the single-system calls made by the calling thread (NULL: defaults). */
int nl_set_tuning(const nl_tuning* tuning);
/* Tuning of one batch (NULL: defaults). */
int nl_batch_set_tuning(nl_batch* batch, const nl_tuning* tuning);

/* Synchronises the stream, then reports (and clears) any device-side error
 * recorded in the workspace by earlier asynchronous calls. */
int nl_sync_status(void* d_workspace, void* stream);

/* Statistics of the last count pass in this workspace: number of candidate
 * pairs decided in FP64 (the FP32 screen's recheck band plus exact atoms).
 * Synchronises the stream. */
int nl_last_recheck_count(void* d_workspace, void* stream, int64_t* rechecks);

const char* nl_status_string(int status);
const char* nl_last_error(void);
int nl_version(void);

#ifdef __cplusplus
}
#endif
#endif /* NLGPU_H */
