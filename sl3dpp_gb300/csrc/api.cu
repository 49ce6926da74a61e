// Error text and version of the sl3dgpu C ABI.
#include <string>

#include "common.cuh"

namespace sl3dgpu {

namespace {
thread_local std::string lastError;
}

void SetError(const std::string& text) { lastError = text; }

}  // namespace sl3dgpu

extern "C" const char* sl3dgpu_last_error(void) { return sl3dgpu::lastError.c_str(); }

extern "C" const char* sl3dgpu_version(void) { return "sl3dgpu 0.1 (sm_103a)"; }
