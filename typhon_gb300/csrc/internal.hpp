// Internal declarations shared by the host translation units of libtyphon_gpu.
#pragma once
#include <string>

namespace tyi {
// Per-thread detail of the last error, returned by ty_last_error().
void set_error(const std::string& msg);
const char* last_error();
}  // namespace tyi
