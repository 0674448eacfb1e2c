// Launchers of the binning / sorting kernels (nl_build.cu).
#pragma once
#include "nl_common.cuh"
#include "nl_scan.cuh"

namespace nl {

constexpr int kFixMax = 256;          // cells up to this size are fixed up per thread
constexpr int kBigSort = 8192;        // cells up to this size are sorted in shared memory
constexpr int kFixBigThreads = 1024;

// A batch of systems (nsys > 0): system s owns atoms [atom0[s], atom0[s+1])
// and cells [cell0[s], cell0[s+1]) of the launch; perm and cell_id are
// written system-local.  nsys == 0 means a single system.
struct SysIndex {
  const Geometry* geo;
  const int* atom0;
  const int* cell0;
  int nsys;
};

void launch_bin(const Geometry& g, const SysIndex& si, const double* X, int nat, int* cid, int* ticket, float4* rec,
                int* cell_count, unsigned* err, int num_sms, cudaStream_t st);
void launch_scatter(int nat, const int* cid, const int* ticket, const int* cell_start, int* tmp, int num_sms,
                    cudaStream_t st);
// TX: position type (double; float for the single-precision path)
template <typename TI, typename TX = double>
void launch_fix(const SysIndex& si, int nat, const int* tmp, const int* cid, const int* cell_start, const TX* X,
                const float4* rec, TI* perm, TI* cell_id, TX* Xs, float4* rec_sorted, int* scell, int* big_list,
                int* big_count, int num_sms, cudaStream_t st);
// batches: the per-system cell_offsets (ncells_s + 1 entries each, system s
// first at cell0[s] + s) from the launch's 0-based cell starts
template <typename TI>
void launch_batch_cell_offsets(const SysIndex& si, int ncells_total, const int* cell_start, TI* cell_offsets,
                               int num_sms, cudaStream_t st);
// batches: the per-system first (nat_s + 1 entries each, system s first at
// atom0[s] + s) and the 0-based start of each system's pairs (nsys + 1)
template <typename TI>
void launch_batch_first(const SysIndex& si, int nat_total, const TI* first_all, TI* first, long long* pair_offsets,
                        int num_sms, cudaStream_t st);
template <typename TI>
void launch_prepare(const Geometry& g, const double* Xs, const TI* cell_id, const TI* perm, int nat,
                    float4* rec_sorted, int* scell, unsigned* err, int num_sms, cudaStream_t st);
template <typename TI>
void launch_scan(const int* in, long long n, TI* out1, int* out0, unsigned long long* status, int* counter,
                 long long* total, unsigned* err, cudaStream_t st);

}  // namespace nl
