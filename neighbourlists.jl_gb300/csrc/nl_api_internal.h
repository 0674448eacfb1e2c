// Helpers shared by the C ABI translation units (not part of the C ABI).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include "nl_common.cuh"

namespace nl {
// Records msg as the calling thread's nl_last_error() text and returns status.
int report(int status, const std::string& msg);
// Maps the device-side error word of a workspace to an NL_* status.
int status_from_device_flags(unsigned flags);
// Smallest workspace the calls accept (without the pair lists, every cell is
// then written by the screening write pass); nl_workspace_bytes is the size
// with the lists.
size_t workspace_min_bytes(int64_t nat, int64_t ncells_total);
// Byte offset in a workspace of the int64 pair total the count pass writes
// (the last entry of its scan), for a system of nat atoms and ncells_total
// cells; the error word sits at offset 0.
size_t workspace_total_offset(int64_t nat, int64_t ncells_total);
// The kernels' view of one system (cell, inverse, grid, stencil, FP32 screen
// band, binning constants); nxyz may be null where no stencil is needed.
Geometry geometry_for(const double* cell, const double* inv, const int64_t* ns, const int64_t* nxyz,
                      const uint8_t* pbc, double cutoff, int64_t nat);
}  // namespace nl
