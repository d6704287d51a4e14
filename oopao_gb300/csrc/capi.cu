// Error reporting and version entry points of the C ABI.
#include <stdio.h>
#include <string.h>

#include <atomic>

#include "common.cuh"

namespace {
thread_local char g_last_error[512] = "";
}

void oopao_set_last_error(const char* msg, const char* file, int line) {
  const char* base = strrchr(file, '/');
  snprintf(g_last_error, sizeof(g_last_error), "%s (%s:%d)", msg ? msg : "", base ? base + 1 : file, line);
}

namespace {
std::atomic<unsigned long long> g_launches{0};
}

void oopao_count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

extern "C" unsigned long long oopao_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" int oopao_abi_version(void) { return 2; }

extern "C" const char* oopao_last_error(void) { return g_last_error; }
