// gsdr_host.h -- internal helpers shared by the host-side translation units.
#pragma once
#include <cstdint>

namespace gsdr {
// Records `msg` as this thread's last error and returns `status`.
int fail(int status, const char* msg);
// Host wall clock in milliseconds.
double now_ms();
}  // namespace gsdr
