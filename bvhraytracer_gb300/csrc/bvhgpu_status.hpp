// Status codes come from the public C header; helpers for the per-thread
// last-error message returned by bvhgpu_last_error().
#pragma once
#include <string>

#include "bvhgpu.h"

namespace bvhgpu {
// Records `msg` as this thread's last error and returns `code`.
int set_error(int code, const std::string& msg);
}  // namespace bvhgpu
