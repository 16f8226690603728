// Error reporting and version of the C ABI.
#include <stdarg.h>
#include <stdio.h>

#include <atomic>

#include "common.cuh"

namespace chm {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

static std::atomic<long long> g_launches{0};
static std::atomic<long long> g_gemm_flops{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_gemm_flops(double flops) {
  g_gemm_flops.fetch_add((long long)flops, std::memory_order_relaxed);
}

}  // namespace chm

extern "C" int64_t chm_launch_count(void) { return chm::g_launches.load(); }
extern "C" double chm_gemm_flops(void) { return (double)chm::g_gemm_flops.load(); }

extern "C" const char *chm_last_error(void) { return chm::g_err; }

extern "C" const char *chm_version(void) { return "chimera_gb300 0.1 (sm_103a)"; }
