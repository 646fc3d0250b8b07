// Shared helpers of the C ABI implementation.
#pragma once

#include <string>

namespace lfm {
// Records the calling thread's last error message and returns `code`.
int setError(int code, const std::string& msg);
}  // namespace lfm
