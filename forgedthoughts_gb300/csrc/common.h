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

}  // namespace ftcommon
