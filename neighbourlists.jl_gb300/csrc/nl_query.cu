// Per-atom lazy traversal on the device: neighbours(clist, i) and
// count_neighbours(clist, i) of the reference (cell_list.jl:779-833) for a set
// of query atoms, without materialising the system's pair list.
//
// One warp per query atom.  The atom is binned with the reference's FP64
// arithmetic (cell and winding, cell_list.jl:66-74,126-147); the stencil
// cells are visited in the reference's order (dz, dy, dx; cells outside an
// open axis skipped, gpu_kernels.jl:20-47); each stencil cell's atoms are
// taken 32 at a time in sorted order, lane k holding the k-th, and each
// candidate is binned, shifted (S = s_loop + wi - wj) and screened with
// R = (xj - xi) + C'S, dot(R, R) < cutoff^2 -- _for_each_neighbor_pair
// (gpu_kernels.jl:58-101) operation for operation, every operation rounded
// separately.  The self candidate (j == i with zero loop shift) is skipped.
// Accepted candidates are compacted with ballots that keep lane order, so an
// atom's pairs come out in the reference's traversal order, the order of its
// neighbours(clist, i).
//
// Two modes: counts only (count_neighbours), or j, S and R written from each
// query atom's offset (neighbours).  FP64 is the slow pipe on this GPU, so
// the traversal is meant for a few atoms per call; whole-system reductions
// run through nl_lazy_reduce.
#include <cuda_runtime.h>

#include <string>

#include "nl_api_internal.h"
#include "nl_common.cuh"
#include "nlgpu.h"

namespace nl {
namespace {

constexpr int kQueryWarps = 4;

template <typename TI>
__global__ void __launch_bounds__(kQueryWarps * 32) k_query(Geometry g, const double* __restrict__ X,
                                                           const double* __restrict__ Xs, const TI* __restrict__ perm,
                                                           const TI* __restrict__ cell_offsets,
                                                           const TI* __restrict__ atoms, long long nq,
                                                           long long* __restrict__ counts,
                                                           const long long* __restrict__ offsets, long long capacity,
                                                           TI* __restrict__ oj, TI* __restrict__ oS,
                                                           double* __restrict__ oR, unsigned* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long long nwarps = (long long)gridDim.x * kQueryWarps;
  unsigned bad = 0;
  for (long long k = (long long)blockIdx.x * kQueryWarps + (threadIdx.x >> 5); k < nq; k += nwarps) {
    const long long ia = (long long)atoms[k] - 1;  // 0-based original index
    if (ia < 0 || ia >= g.nat) {
      bad |= kFlagBadIndex;
      if (counts && lane == 0) counts[k] = 0;
      continue;
    }
    const double xi[3] = {X[3 * ia + 0], X[3 * ia + 1], X[3 * ia + 2]};
    Binned bi;
    if (!bin_position(g, xi[0], xi[1], xi[2], bi)) {
      bad |= kFlagBadPosition;
      if (counts && lane == 0) counts[k] = 0;
      continue;
    }
    const long long out0 = offsets ? offsets[k] : 0;
    long long cnt = 0;
    for (int dz = -g.nxyz[2]; dz <= g.nxyz[2]; ++dz)
      for (int dy = -g.nxyz[1]; dy <= g.nxyz[1]; ++dy)
        for (int dx = -g.nxyz[0]; dx <= g.nxyz[0]; ++dx) {
          const int d[3] = {dx, dy, dz};
          bool inb = true;
#pragma unroll
          for (int a = 0; a < 3; ++a)
            inb = inb && (g.pbc[a] || (bi.c[a] + d[a] >= 1 && bi.c[a] + d[a] <= g.ns[a]));
          if (!inb) continue;
          int s[3], c[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) c[a] = wrap_shift(bi.c[a] + d[a], g.ns[a], g.pbc[a], s[a]);
          const int lin = linear_cell(g, c[0], c[1], c[2]);
          const long long cs = (long long)cell_offsets[lin] - 1, ce = (long long)cell_offsets[lin + 1] - 1;
          for (long long base = max(cs, 0LL); base < min(ce, (long long)g.nat); base += 32) {
            const long long idx = base + lane;
            bool acc = false;
            long long jo = 0;
            int S[3] = {0, 0, 0};
            double R[3] = {0.0, 0.0, 0.0};
            if (idx < min(ce, (long long)g.nat)) {
              jo = (long long)perm[idx] - 1;
              const bool self = jo == ia && s[0] == 0 && s[1] == 0 && s[2] == 0;
              if (!self) {
                // X_sorted[idx] == X_orig[perm[idx]] bit for bit (the cell list's gather)
                const double xj[3] = {Xs[3 * idx + 0], Xs[3 * idx + 1], Xs[3 * idx + 2]};
                Binned bj;
                if (!bin_position(g, xj[0], xj[1], xj[2], bj)) bad |= kFlagBadPosition;
#pragma unroll
                for (int a = 0; a < 3; ++a) S[a] = s[a] + bi.w[a] - bj.w[a];
#pragma unroll
                for (int a = 0; a < 3; ++a) R[a] = dadd(dsub(xj[a], xi[a]), cts_k(g.C, S[0], S[1], S[2], a));
                acc = dadd(dadd(dmul(R[0], R[0]), dmul(R[1], R[1])), dmul(R[2], R[2])) < g.cutoff_sq;
              }
            }
            const unsigned m = __ballot_sync(0xffffffffu, acc);
            if (acc && oj) {
              const long long p = out0 + cnt + __popc(m & lt);
              if (p < capacity) {
                oj[p] = TI(jo + 1);
                oS[3 * p + 0] = TI(S[0]);
                oS[3 * p + 1] = TI(S[1]);
                oS[3 * p + 2] = TI(S[2]);
                if (oR) {
                  oR[3 * p + 0] = R[0];
                  oR[3 * p + 1] = R[1];
                  oR[3 * p + 2] = R[2];
                }
              } else {
                bad |= kFlagCapacity;
              }
            }
            cnt += __popc(m);
          }
        }
    if (counts && lane == 0) counts[k] = cnt;
  }
  if (bad) atomicOr(err, bad);
}

template <typename TI>
void launch_query(const Geometry& g, const double* X, const double* Xs, const TI* perm, const TI* cell_offsets,
                  const TI* atoms, long long nq, long long* counts, const long long* offsets, long long capacity,
                  TI* oj, TI* oS, double* oR, unsigned* err, cudaStream_t st) {
  long long blocks = (nq + kQueryWarps - 1) / kQueryWarps;
  if (blocks > 65535) blocks = 65535;
  k_query<TI><<<int(blocks), kQueryWarps * 32, 0, st>>>(g, X, Xs, perm, cell_offsets, atoms, nq, counts, offsets,
                                                        capacity, oj, oS, oR, err);
}

}  // namespace
}  // namespace nl

extern "C" int nl_query_neighbours(const double* d_X, const double* d_X_sorted, const void* d_perm,
                                   const void* d_cell_offsets, int64_t nat, const double cell[9],
                                   const double inv_cell[9], const int64_t ncells[3], const int64_t nxyz[3],
                                   const uint8_t pbc[3], double cutoff, int index_bytes, const void* d_atoms,
                                   int64_t nq, int64_t* d_counts, const int64_t* d_offsets, int64_t capacity,
                                   void* d_j, void* d_S, double* d_R, void* d_workspace, size_t workspace_bytes,
                                   void* stream) {
  if (!cell || !inv_cell || !ncells || !nxyz || !pbc || !d_cell_offsets || !d_workspace)
    return nl::report(NL_ERR_ARG, "null argument");
  if (index_bytes != 4 && index_bytes != 8) return nl::report(NL_ERR_ARG, "index_bytes must be 4 or 8");
  if (nat < 0 || nat > 2147483646LL || nq < 0) return nl::report(NL_ERR_ARG, "nat must be in [0, 2^31-2], nq >= 0");
  if (workspace_bytes < 128) return nl::report(NL_ERR_NOMEM, "workspace too small (at least 128 bytes)");
  if (!d_j && !d_counts) return nl::report(NL_ERR_ARG, "give d_counts (count mode) or d_j, d_S, d_offsets (fill mode)");
  if (d_j && (!d_S || !d_offsets)) return nl::report(NL_ERR_ARG, "fill mode needs d_S and d_offsets");
  if (nq == 0) return NL_OK;
  if (!d_atoms || (nat > 0 && (!d_X || !d_X_sorted || !d_perm))) return nl::report(NL_ERR_ARG, "null argument");
  for (int k = 0; k < 3; ++k) {
    if (ncells[k] < 1) return nl::report(NL_ERR_ARG, "ncells must be >= 1");
    if (nxyz[k] < 0 || nxyz[k] > 62) return nl::report(NL_ERR_ARG, "stencil half-width nxyz must be in [0, 62]");
  }
  if ((long double)ncells[0] * ncells[1] * ncells[2] > 2147483646.0L)
    return nl::report(NL_ERR_TOO_MANY_CELLS, "more than 2^31-2 cells");
  const nl::Geometry g = nl::geometry_for(cell, inv_cell, ncells, nxyz, pbc, cutoff, nat);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned* err = static_cast<unsigned*>(d_workspace);
  if (index_bytes == 4)
    nl::launch_query<int32_t>(g, d_X, d_X_sorted, static_cast<const int32_t*>(d_perm),
                              static_cast<const int32_t*>(d_cell_offsets), static_cast<const int32_t*>(d_atoms), nq,
                              reinterpret_cast<long long*>(d_counts), reinterpret_cast<const long long*>(d_offsets),
                              capacity, static_cast<int32_t*>(d_j), static_cast<int32_t*>(d_S), d_R, err, st);
  else
    nl::launch_query<int64_t>(g, d_X, d_X_sorted, static_cast<const int64_t*>(d_perm),
                              static_cast<const int64_t*>(d_cell_offsets), static_cast<const int64_t*>(d_atoms), nq,
                              reinterpret_cast<long long*>(d_counts), reinterpret_cast<const long long*>(d_offsets),
                              capacity, static_cast<int64_t*>(d_j), static_cast<int64_t*>(d_S), d_R, err, st);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NL_OK : nl::report(NL_ERR_CUDA, std::string("launch query: ") + cudaGetErrorString(e));
}
