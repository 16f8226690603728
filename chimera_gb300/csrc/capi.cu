// Error reporting and version of the C ABI.
#include <stdarg.h>
#include <stdio.h>

#include "common.cuh"

namespace chm {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

}  // namespace chm

extern "C" const char *chm_last_error(void) { return chm::g_err; }

extern "C" const char *chm_version(void) { return "chimera_gb300 0.1 (sm_103a)"; }
