// error.hpp — per-thread last-error message behind rrsph_last_error().
#pragma once
#include <string>

namespace rrsph {
// Records msg as the calling thread's last error and returns code.
int set_error(int code, const std::string& msg);
}  // namespace rrsph
