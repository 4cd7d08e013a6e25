// Shared host-side helpers of libcaustic_gb300: error state and status codes.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/caustic.h"

namespace ct {

// Records `msg` as the calling thread's last error and returns `status`.
ct_status fail(ct_status status, const char* fmt, ...);
void clear_error();
const char* last_error();

}  // namespace ct

#define CT_CHECK_ARG(cond, ...)                                        \
  do {                                                                 \
    if (!(cond)) return ::ct::fail(CT_ERR_INVALID_ARGUMENT, __VA_ARGS__); \
  } while (0)
