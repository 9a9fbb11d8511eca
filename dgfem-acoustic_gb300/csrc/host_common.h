// Shared helpers of the host front end: error capture at the C boundary.
#pragma once
#include <exception>
#include <string>

#include "mshio.h"

// Opaque mesh handle of the C API (include/dgfem_host.h).
struct dgh_mesh {
  dgmsh::VolumeMesh m;
};

namespace dghost {
void set_error(const std::string& s);

// Runs f, converting any exception into a non-zero return code and an error
// message; nothing propagates across the C ABI.
template <class F>
int guard(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    set_error(e.what());
    return 1;
  } catch (...) {
    set_error("unknown error");
    return 1;
  }
}
}  // namespace dghost
