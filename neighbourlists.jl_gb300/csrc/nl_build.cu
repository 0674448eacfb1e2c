// Stage (a) binning and stage (b) sorting of atoms by cell id.
//
// Replaces, on the GPU, the reference's
//   _compute_cell_ids / compute_cell_ids_kernel!   (cell_list.jl:684-701, gpu_kernels.jl:108-125)
//   _get_sortperm (stable Base.sortperm on CPU)     (cell_list.jl:705-718)
//   cell_ids[perm], X[perm]                          (cell_list.jl:669-670)
//   _compute_cell_offsets / _histogram_kernel!      (cell_list.jl:724-748, gpu_kernels.jl:191-197,262-285)
//
// The sort is a one-digit counting sort on the full cell id: a histogram with
// warp-aggregated atomics (the atomic return value is a per-atom ticket), the
// decoupled look-back scan of the histogram (nl_scan.cuh), a scatter by
// ticket, and a per-cell fix-up that orders each cell's atoms by original
// index.  The fix-up makes the permutation identical to the reference's
// stable sortperm, so perm, the sorted positions and the sorted cell ids are
// bit-identical to the reference's SortedCellList.
#include "nl_build.cuh"
#include "nl_pairs.cuh"

namespace nl {

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// --------------------------------------------------------------- binning --
// One thread per atom (original order).  Writes the 0-based cell id, the
// ticket (rank among the atoms of that cell that reached the histogram
// first) and the FP32 cell-local record.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_bin(Geometry g1, SysIndex si, const double* __restrict__ X, int nat,
                                             int* __restrict__ cid, int* __restrict__ ticket,
                                             float4* __restrict__ rec, int* __restrict__ cell_count,
                                             unsigned* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nat; base += stride) {
    const int i = int(base) + lane;
    const bool valid = i < nat;
    int c = 0;
    if (valid) {
      const double x0 = X[3LL * i + 0], x1 = X[3LL * i + 1], x2 = X[3LL * i + 2];
      const int sys = BATCH ? batch_system(si.atom0, si.nsys, i) : 0;
      const Geometry& g = BATCH ? si.geo[sys] : g1;
      Binned bn;
      if (!bin_fast(g, x0, x1, x2, bn) && !bin_position(g, x0, x1, x2, bn)) atomicOr(err, kFlagBadPosition);
      c = linear_cell(g, bn.c[0], bn.c[1], bn.c[2]) + (BATCH ? si.cell0[sys] : 0);
      rec[i] = make_record(g, bn);
      cid[i] = c;
    }
    // warp-aggregated histogram increment; invalid lanes get unique keys
    const int key = valid ? c : -1 - lane;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int b = 0;
    if (valid && lane == leader) b = atomicAdd(&cell_count[c], __popc(peers));
    b = __shfl_sync(0xffffffffu, b, leader);
    if (valid) ticket[i] = b + __popc(peers & lanemask_lt());
  }
}

// ---------------------------------------------------------------- scatter --
__global__ void __launch_bounds__(256) k_scatter(int nat, const int* __restrict__ cid, const int* __restrict__ ticket,
                                                 const int* __restrict__ cell_start, int* __restrict__ tmp) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nat; i += (long long)gridDim.x * blockDim.x)
    tmp[cell_start[cid[i]] + ticket[i]] = int(i);
}

template <typename TI, typename TX>
__device__ __forceinline__ void write_sorted(const SysIndex& si, long long dst, int i, int c,
                                             const TX* __restrict__ X, const float4* __restrict__ rec,
                                             TI* __restrict__ perm, TI* __restrict__ cell_id,
                                             TX* __restrict__ Xs, float4* __restrict__ rec_sorted,
                                             int* __restrict__ scell) {
  int li = i, lc = c;
  if (si.nsys > 0) {  // system-local indices
    const int sys = batch_system(si.atom0, si.nsys, i);
    li -= si.atom0[sys];
    lc -= si.cell0[sys];
  }
  perm[dst] = TI(li) + 1;
  cell_id[dst] = TI(lc) + 1;
  scell[dst] = c;
  Xs[3 * dst + 0] = X[3LL * i + 0];
  Xs[3 * dst + 1] = X[3LL * i + 1];
  Xs[3 * dst + 2] = X[3LL * i + 2];
  rec_sorted[dst] = rec[i];
}

// ------------------------------------------------------------ fix-up (small)
// One thread per sorted slot.  For cells of at most kFixMax atoms the stable
// position of atom i is (cell start) + #{atoms of the cell with index < i}.
// Larger cells are listed for k_fix_big.
template <typename TI, typename TX>
__global__ void __launch_bounds__(256) k_fix(SysIndex si, int nat, const int* __restrict__ tmp, const int* __restrict__ cid,
                                             const int* __restrict__ cell_start, const TX* __restrict__ X,
                                             const float4* __restrict__ rec, TI* __restrict__ perm,
                                             TI* __restrict__ cell_id, TX* __restrict__ Xs,
                                             float4* __restrict__ rec_sorted, int* __restrict__ scell,
                                             int* __restrict__ big_list, int* __restrict__ big_count) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nat; s += (long long)gridDim.x * blockDim.x) {
    const int i = tmp[s];
    const int c = cid[i];
    const int start = cell_start[c];
    const int k = cell_start[c + 1] - start;
    if (k > kFixMax) {
      if (s == start) big_list[atomicAdd(big_count, 1)] = c;
      continue;
    }
    int rank = 0;
    for (int t = start; t < start + k; ++t) rank += tmp[t] < i;
    write_sorted<TI, TX>(si, start + rank, i, c, X, rec, perm, cell_id, Xs, rec_sorted, scell);
  }
}

// ------------------------------------------------------------ fix-up (big)
// One block per listed cell.  Cells up to kBigSort atoms are sorted in shared
// memory (bitonic); larger ones are rebuilt by a block-wide ordered scan over
// all atoms (stable by construction).
template <typename TI, typename TX>
__global__ void __launch_bounds__(kFixBigThreads) k_fix_big(SysIndex si, int nat, const int* __restrict__ tmp,
                                                            const int* __restrict__ cid,
                                                            const int* __restrict__ cell_start,
                                                            const TX* __restrict__ X,
                                                            const float4* __restrict__ rec, TI* __restrict__ perm,
                                                            TI* __restrict__ cell_id, TX* __restrict__ Xs,
                                                            float4* __restrict__ rec_sorted,
                                                            int* __restrict__ scell,
                                                            const int* __restrict__ big_list,
                                                            const int* __restrict__ big_count) {
  __shared__ int s[kBigSort];
  __shared__ int s_warp[kFixBigThreads / 32];
  const int nbig = *big_count;
  for (int b = blockIdx.x; b < nbig; b += gridDim.x) {
    const int c = big_list[b];
    const int start = cell_start[c];
    const int k = cell_start[c + 1] - start;
    if (k <= kBigSort) {
      int P = 1;
      while (P < k) P <<= 1;
      for (int t = threadIdx.x; t < P; t += blockDim.x) s[t] = t < k ? tmp[start + t] : 0x7fffffff;
      __syncthreads();
      for (int size = 2; size <= P; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
          for (int t = threadIdx.x; t < P; t += blockDim.x) {
            int partner = t ^ stride;
            if (partner > t) {
              bool up = (t & size) == 0;
              int a = s[t], d = s[partner];
              if ((a > d) == up) {
                s[t] = d;
                s[partner] = a;
              }
            }
          }
          __syncthreads();
        }
      for (int t = threadIdx.x; t < k; t += blockDim.x)
        write_sorted<TI, TX>(si, start + t, s[t], c, X, rec, perm, cell_id, Xs, rec_sorted, scell);
      __syncthreads();
    } else {
      int run = 0;
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      for (int base = 0; base < nat; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const bool f = i < nat && cid[i] == c;
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_warp[warp] = __popc(m);
        __syncthreads();
        int before = 0, tot = 0;
        for (int w = 0; w < kFixBigThreads / 32; ++w) {
          if (w < warp) before += s_warp[w];
          tot += s_warp[w];
        }
        if (f)
          write_sorted<TI, TX>(si, start + run + before + __popc(m & lanemask_lt()), i, c, X, rec, perm, cell_id, Xs,
                           rec_sorted, scell);
        run += tot;
        __syncthreads();
      }
    }
  }
}

// ---------------------------------------------------------------- prepare --
// Rebuilds the FP32 records of an existing sorted cell list (e.g. one built
// by the reference's CPU path) from its sorted positions, and checks that
// each atom sits in the cell the list says.
template <typename TI>
__global__ void __launch_bounds__(256) k_prepare(Geometry g, const double* __restrict__ Xs,
                                                 const TI* __restrict__ cell_id, const TI* __restrict__ perm, int nat,
                                                 float4* __restrict__ rec_sorted, int* __restrict__ scell,
                                                 unsigned* __restrict__ err) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nat; s += (long long)gridDim.x * blockDim.x) {
    Binned bn;
    const double x0 = Xs[3 * s + 0], x1 = Xs[3 * s + 1], x2 = Xs[3 * s + 2];
    if (!bin_fast(g, x0, x1, x2, bn) && !bin_position(g, x0, x1, x2, bn)) atomicOr(err, kFlagBadPosition);
    rec_sorted[s] = make_record(g, bn);
    const int c = linear_cell(g, bn.c[0], bn.c[1], bn.c[2]);
    scell[s] = c;
    if ((long long)cell_id[s] != (long long)c + 1) atomicOr(err, kFlagInconsistent);
    if ((long long)perm[s] < 1 || (long long)perm[s] > nat) atomicOr(err, kFlagInconsistent);
  }
}

// ----------------------------------------------------------------- batches --
// largest s in [0, nsys) with first[s] + s <= e (first nondecreasing)
__device__ __forceinline__ int batch_entry_system(const int* __restrict__ first, int nsys, long long e) {
  int lo = 0, hi = nsys - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((long long)first[mid] + mid <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <typename TI>
__global__ void __launch_bounds__(256) k_batch_cell_offsets(SysIndex si, long long n_out,
                                                            const int* __restrict__ cell_start,
                                                            TI* __restrict__ cell_offsets) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n_out; e += (long long)gridDim.x * blockDim.x) {
    const int s = batch_entry_system(si.cell0, si.nsys, e);
    const long long k = e - si.cell0[s] - s;  // 0 .. ncells_s
    cell_offsets[e] = TI(cell_start[si.cell0[s] + k] - si.atom0[s] + 1);
  }
}

template <typename TI>
__global__ void __launch_bounds__(256) k_batch_first(SysIndex si, long long n_out, const TI* __restrict__ first_all,
                                                     TI* __restrict__ first, long long* __restrict__ pair_offsets) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n_out; e += (long long)gridDim.x * blockDim.x) {
    const int s = batch_entry_system(si.atom0, si.nsys, e);
    const long long k = e - si.atom0[s] - s;  // 0 .. nat_s
    const long long base = (long long)first_all[si.atom0[s]] - 1;
    first[e] = TI((long long)first_all[si.atom0[s] + k] - base);
    if (k == 0) pair_offsets[s] = base;
    if (e == n_out - 1) pair_offsets[si.nsys] = (long long)first_all[si.atom0[si.nsys]] - 1;
  }
}

// ------------------------------------------------------------- launchers --
static inline int grid_for(long long n, int block, int max_blocks) {
  long long g = (n + block - 1) / block;
  if (g > max_blocks) g = max_blocks;
  return g < 1 ? 1 : int(g);
}

void launch_bin(const Geometry& g, const SysIndex& si, const double* X, int nat, int* cid, int* ticket, float4* rec,
                int* cell_count, unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  if (si.nsys > 0)
    k_bin<true><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, si, X, nat, cid, ticket, rec, cell_count, err);
  else
    k_bin<false><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, si, X, nat, cid, ticket, rec, cell_count, err);
}

template <typename TI>
void launch_batch_cell_offsets(const SysIndex& si, int ncells_total, const int* cell_start, TI* cell_offsets,
                               int num_sms, cudaStream_t st) {
  const long long n = (long long)ncells_total + si.nsys;
  if (si.nsys <= 0 || n <= 0) return;
  k_batch_cell_offsets<TI><<<grid_for(n, 256, num_sms * 8), 256, 0, st>>>(si, n, cell_start, cell_offsets);
}

template <typename TI>
void launch_batch_first(const SysIndex& si, int nat_total, const TI* first_all, TI* first, long long* pair_offsets,
                        int num_sms, cudaStream_t st) {
  const long long n = (long long)nat_total + si.nsys;
  if (si.nsys <= 0) return;
  k_batch_first<TI><<<grid_for(n, 256, num_sms * 8), 256, 0, st>>>(si, n, first_all, first, pair_offsets);
}

void launch_scatter(int nat, const int* cid, const int* ticket, const int* cell_start, int* tmp, int num_sms,
                    cudaStream_t st) {
  if (nat <= 0) return;
  k_scatter<<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(nat, cid, ticket, cell_start, tmp);
}

template <typename TI, typename TX>
void launch_fix(const SysIndex& si, int nat, const int* tmp, const int* cid, const int* cell_start, const TX* X,
                const float4* rec, TI* perm, TI* cell_id, TX* Xs, float4* rec_sorted, int* scell, int* big_list,
                int* big_count, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  k_fix<TI, TX><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(si, nat, tmp, cid, cell_start, X, rec, perm, cell_id,
                                                                 Xs, rec_sorted, scell, big_list, big_count);
  k_fix_big<TI, TX><<<num_sms, kFixBigThreads, 0, st>>>(si, nat, tmp, cid, cell_start, X, rec, perm, cell_id, Xs,
                                                         rec_sorted, scell, big_list, big_count);
}

template <typename TI>
void launch_prepare(const Geometry& g, const double* Xs, const TI* cell_id, const TI* perm, int nat,
                    float4* rec_sorted, int* scell, unsigned* err, int num_sms, cudaStream_t st) {
  if (nat <= 0) return;
  k_prepare<TI><<<grid_for(nat, 256, num_sms * 8), 256, 0, st>>>(g, Xs, cell_id, perm, nat, rec_sorted, scell, err);
}

template <typename TI>
void launch_scan(const int* in, long long n, TI* out1, int* out0, unsigned long long* status, int* counter,
                 long long* total, unsigned* err, cudaStream_t st) {
  if (n <= 0) return;
  k_scan_offsets<TI><<<scan_tiles(n), kScanBlock, 0, st>>>(in, n, out1, out0, status, counter, total, err);
}

#define NL_INST(TI)                                                                                                  \
  template void launch_fix<TI, double>(const SysIndex&, int, const int*, const int*, const int*, const double*,    \
                                       const float4*, TI*, TI*, double*, float4*, int*, int*, int*, int,            \
                                       cudaStream_t);                                                               \
  template void launch_fix<TI, float>(const SysIndex&, int, const int*, const int*, const int*, const float*,      \
                                      const float4*, TI*, TI*, float*, float4*, int*, int*, int*, int,              \
                                      cudaStream_t);                                                                \
  template void launch_batch_cell_offsets<TI>(const SysIndex&, int, const int*, TI*, int, cudaStream_t);            \
  template void launch_batch_first<TI>(const SysIndex&, int, const TI*, TI*, long long*, int, cudaStream_t);        \
  template void launch_prepare<TI>(const Geometry&, const double*, const TI*, const TI*, int, float4*, int*,     \
                                   unsigned*, int, cudaStream_t);                                                   \
  template void launch_scan<TI>(const int*, long long, TI*, int*, unsigned long long*, int*, long long*, unsigned*, \
                                cudaStream_t);
NL_INST(int32_t)
NL_INST(int64_t)
#undef NL_INST

}  // namespace nl
