// nl_neighbour_list_static: the materialised pipeline for callers that cannot
// allocate device memory.
//
// Every other entry point takes a caller-allocated workspace.  Some callers
// cannot provide one: code that runs while a framework's memory pool owns the
// whole device, real-time loops that forbid allocation after start-up, or
// host code that is not allowed to call cudaMalloc (or whose allocation would
// synchronise the device).  For them this entry point runs the same kernels
// with their scratch in a fixed array that lives in the library's own device
// image: kStaticScratchBytes (32 MiB) on every GPU that loads the library,
// held until the process exits.
//
// Set-up: the first call on each device (with that device current) resolves
// the array's device address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture.  The entry point itself calls
// no cudaMalloc, cudaFree or other allocating routine.
//
// All calls share the one array and each call overwrites it (it starts by
// clearing what must start at zero), so calls that overlap on the GPU -- on
// different streams, or from different host threads -- race and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "nl_api_internal.h"
#include "nlgpu.h"

namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Resolves (once per device, with that device current) the device address of
// the static scratch array.  Host code must never use the array's name as an
// address: on the host it is only a stand-in symbol.
int scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nl::report(NL_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return nl::report(NL_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return nl::report(NL_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return NL_OK;
}

// The status and pair total of the last call on the current device, read
// synchronously into host variables (no pinned staging, nothing allocated).
int read_back(void* scratch, int64_t nat, int64_t ncells_total, int64_t capacity, int64_t* total_pairs,
              cudaStream_t st) {
  cudaError_t e = cudaStreamSynchronize(st);
  unsigned flags = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&flags, scratch, sizeof(flags), cudaMemcpyDeviceToHost);
  long long total = 0;
  if (e == cudaSuccess && nat > 0)
    e = cudaMemcpy(&total, static_cast<char*>(scratch) + nl::workspace_total_offset(nat, ncells_total), sizeof(total),
                   cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return nl::report(NL_ERR_CUDA, std::string("read back: ") + cudaGetErrorString(e));
  if (total_pairs) *total_pairs = total;
  int s = nl::status_from_device_flags(flags);
  if (s == NL_OK && capacity >= 0 && total > capacity)
    return nl::report(NL_ERR_CAPACITY, "pair buffers are smaller than the pair count");
  return s;
}

// What the last call on each device was (for nl_static_sync_status).
struct LastCall {
  int64_t nat = -1, ncells_total = 0, capacity = -1;
};
LastCall g_last[kMaxDevices];

}  // namespace

extern "C" int nl_neighbour_list_static(const double* d_X, int64_t nat, const double cell[9],
                                        const double inv_cell[9], const int64_t ncells[3], const int64_t nxyz[3],
                                        const uint8_t pbc[3], double cutoff, int index_bytes, void* d_perm,
                                        double* d_X_sorted, void* d_cell_id, void* d_cell_offsets, void* d_first,
                                        int64_t capacity, void* d_i, void* d_j, void* d_S, double* d_R,
                                        int64_t* total_pairs, void* stream) {
  if (!ncells || !nxyz || !cell || !inv_cell || !pbc) return nl::report(NL_ERR_ARG, "null argument");
  if (nat < 0 || nat > 2147483646LL) return nl::report(NL_ERR_ARG, "nat must be in [0, 2^31-2]");
  if (ncells[0] < 1 || ncells[1] < 1 || ncells[2] < 1) return nl::report(NL_ERR_ARG, "ncells must be >= 1");
  const long double cells = (long double)ncells[0] * ncells[1] * ncells[2];
  if (cells > 2147483646.0L) return nl::report(NL_ERR_TOO_MANY_CELLS, "more than 2^31-2 cells");
  const int64_t nct = int64_t(cells);
  // the static scratch holds the pair lists only for small systems; larger
  // ones run with the screening write pass (same results)
  const size_t need = nl::workspace_min_bytes(nat, nct);
  if (need > kStaticScratchBytes)
    return nl::report(NL_ERR_NOMEM, "system needs " + std::to_string(need) +
                                        " bytes of scratch, more than the 32 MiB static scratch of "
                                        "nl_neighbour_list_static (about 500k atoms at liquid density); "
                                        "use nl_neighbour_list with a caller-allocated workspace");
  void* scratch = nullptr;
  int s = scratch_for_current_device(&scratch);
  if (s) return s;
  int dev = 0;
  cudaGetDevice(&dev);  // checked by scratch_for_current_device
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  s = nl_neighbour_list(d_X, nat, cell, inv_cell, ncells, nxyz, pbc, cutoff, index_bytes, d_perm, d_X_sorted,
                        d_cell_id, d_cell_offsets, d_first, capacity, d_i, d_j, d_S, d_R, nullptr, scratch,
                        kStaticScratchBytes, stream);
  if (s) return s;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    g_last[dev].nat = nat;
    g_last[dev].ncells_total = nct;
    g_last[dev].capacity = capacity;
  }
  if (!total_pairs) return NL_OK;
  return read_back(scratch, nat, nct, capacity, total_pairs, st);
}

extern "C" int nl_static_sync_status(int64_t* total_pairs, void* stream) {
  void* scratch = nullptr;
  int s = scratch_for_current_device(&scratch);
  if (s) return s;
  int dev = 0;
  cudaGetDevice(&dev);
  LastCall last;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    last = g_last[dev];
  }
  if (last.nat < 0) return nl::report(NL_ERR_ARG, "no nl_neighbour_list_static call on this device yet");
  return read_back(scratch, last.nat, last.ncells_total, last.capacity, total_pairs, static_cast<cudaStream_t>(stream));
}
