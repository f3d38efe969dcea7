// The calling thread's last error message (fg_last_error): shared by the
// product library and the host-only problem library.
#include <string>

#include "../../include/fem_g_gb300.h"

namespace femg {

static thread_local std::string g_lastError;

void setLastError(const std::string &msg) { g_lastError = msg; }

}  // namespace femg

extern "C" const char *fg_last_error(void) { return femg::g_lastError.c_str(); }
