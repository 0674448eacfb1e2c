// Helpers shared by the C ABI translation units (not part of the C ABI).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

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
}  // namespace nl
