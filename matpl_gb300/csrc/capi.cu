// Library-wide C ABI pieces: error reporting and version.
#include <string>
#include "common.cuh"

namespace matpl {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace matpl

extern "C" const char *matpl_last_error(void) { return matpl::g_last_error.c_str(); }
extern "C" int matpl_version(void) { return 1; }
