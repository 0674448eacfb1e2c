// Launchers of the pair-traversal kernels (nl_pairs.cu).
#pragma once
#include "nl_common.cuh"

namespace nl {

enum PairMode : int { kModeCount = 0, kModeFill = 1, kModeLazyR6 = 2 };

// The count pass records, per home atom, the acceptance bitmask of its
// candidates (bit f = the f-th candidate in the reference's traversal order)
// when the home cell's stencil has at most 32 cells and 32*kMaskWords
// candidates.  The fill pass then writes those pairs without screening again.
constexpr int kMaskWords = 12;

template <typename TI>
struct PairArgs {
  Geometry g;
  const TI* cell_offsets;   // 1-based CSR over cells (ncells+1)
  const TI* perm;           // sorted slot -> 1-based original index
  const double* Xs;         // sorted positions (nat x 3)
  const float4* rec;        // sorted FP32 records
  const int* scell;         // sorted slot -> 0-based cell index
  const TI* first;          // fill: 1-based pair offsets per original atom (nat+1)
  int* counts;              // count: pairs per original atom
  TI* oi;                   // fill outputs (1-based i, j; S as 3 x TI; R as 3 x double)
  TI* oj;
  TI* oS;
  double* oR;               // may be null (R not wanted)
  long long capacity;       // pairs the output buffers hold
  double* per_atom;         // lazy: per-atom reduction
  unsigned* masks;          // per sorted slot: kMaskWords acceptance words
  double* cs_table;         // C'S for |S_k| <= 2 (built once per call by k_cs_table)
  int* unmasked;            // count pass: home cells left to the screening fill
  int* n_unmasked;          // length of that list
  unsigned long long* stats;  // [0] += FP64 rechecks
  unsigned* err;
};

template <typename TI>
void launch_pairs(int mode, const PairArgs<TI>& a, int num_sms, cudaStream_t st);

}  // namespace nl
