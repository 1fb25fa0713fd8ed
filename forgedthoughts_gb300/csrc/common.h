// Shared host helpers: the thread-local error message behind ft_last_error().
#pragma once

#include <string>

#include "forgedthoughts_gb300.h"

namespace ftcommon {

void set_last_error(const std::string& message);
void clear_last_error();
const char* last_error_cstr();

// Record `message` and return `status` (convenience for early returns).
inline ft_status fail(ft_status status, const std::string& message) {
  set_last_error(message);
  return status;
}

// Status and message for the exception being handled: host allocation and
// thread-creation failures give FT_ERR_OUT_OF_MEMORY, anything else
// FT_ERR_INTERNAL.  Call only inside a catch handler.
ft_status fail_current_exception() noexcept;

}  // namespace ftcommon

// Bodies of the C entry points run between FT_API_BEGIN and FT_API_END, so a
// C++ exception (a failed host allocation above all) becomes a status and
// never unwinds into the caller's frames.
#define FT_API_BEGIN try {
#define FT_API_END \
  }                \
  catch (...) {    \
    return ::ftcommon::fail_current_exception(); \
  }
