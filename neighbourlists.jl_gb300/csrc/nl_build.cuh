// Launchers of the binning / sorting kernels (nl_build.cu).
#pragma once
#include "nl_common.cuh"
#include "nl_scan.cuh"

namespace nl {

constexpr int kFixMax = 256;          // cells up to this size are fixed up per thread
constexpr int kBigSort = 8192;        // cells up to this size are sorted in shared memory
constexpr int kFixBigThreads = 1024;

void launch_bin(const Geometry& g, const double* X, int nat, int* cid, int* ticket, float4* rec, int* cell_count,
                unsigned* err, int num_sms, cudaStream_t st);
void launch_scatter(int nat, const int* cid, const int* ticket, const int* cell_start, int* tmp, int num_sms,
                    cudaStream_t st);
template <typename TI>
void launch_fix(int nat, const int* tmp, const int* cid, const int* cell_start, const double* X, const float4* rec,
                TI* perm, TI* cell_id, double* Xs, float4* rec_sorted, int* scell, int* big_list, int* big_count,
                int num_sms, cudaStream_t st);
template <typename TI>
void launch_prepare(const Geometry& g, const double* Xs, const TI* cell_id, const TI* perm, int nat,
                    float4* rec_sorted, int* scell, unsigned* err, int num_sms, cudaStream_t st);
template <typename TI>
void launch_scan(const int* in, long long n, TI* out1, int* out0, unsigned long long* status, int* counter,
                 long long* total, unsigned* err, cudaStream_t st);

}  // namespace nl
