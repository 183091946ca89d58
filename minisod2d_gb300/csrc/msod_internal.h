// msod_internal.h -- shared host-side helpers of the msod library (not part of the ABI).
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "msod.h"

namespace msod {

// Records `code` with a printf-style message as the calling thread's last
// error and returns `code`.
int set_error(int code, const char *fmt, ...);
// Clears the calling thread's last error.
void clear_error();
// Whether checked mode is on (validation + synchronisation in every call).
bool checked_mode();

}  // namespace msod
