// Helpers shared by the C ABI translation units (not part of the C ABI).
#pragma once
#include <string>

namespace nl {
// Records msg as the calling thread's nl_last_error() text and returns status.
int report(int status, const std::string& msg);
// Maps the device-side error word of a workspace to an NL_* status.
int status_from_device_flags(unsigned flags);
}  // namespace nl
