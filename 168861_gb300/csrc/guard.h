// Exception guard for the C entry points (host code only).
#pragma once
#include <exception>
#include <new>
#include <string>

#include "neurite_gb300.h"

namespace nrt {

void set_error(const std::string &msg);  // the calling thread's nrt_last_error() text

// Runs the body of a C entry point.  A C++ exception (a host allocation that failed)
// becomes a status, so none crosses the C boundary.
template <typename F>
int guarded(F &&body) {
  try {
    return body();
  } catch (const std::bad_alloc &) {
    try {
      set_error("host allocation failed");
    } catch (...) {
    }
    return NRT_ENOMEM;
  } catch (const std::exception &e) {
    try {
      set_error(e.what());
    } catch (...) {
    }
    return NRT_EINVAL;
  } catch (...) {
    return NRT_EINVAL;
  }
}

}  // namespace nrt
