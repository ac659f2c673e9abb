// Implicit (backward Euler) path -- assembly and Krylov solve.
#include "nrt_solver.h"

namespace nrt {

struct ImplicitState {};

size_t Engine::implicit_bytes() const { return 0; }
int Engine::implicit_init() {
  set_error("implicit mode not available in this build");
  return NRT_EINVAL;
}
int Engine::implicit_step(int, int) { return NRT_EINVAL; }
void Engine::implicit_release() {}
int Engine::get_stats(nrt_stats *st) {
  memset(st, 0, sizeof(*st));
  st->steps = steps_done;
  st->device_bytes = (int64_t)arena.cap;
  return NRT_OK;
}

}  // namespace nrt

extern "C" int nrt_export_system(nrt_solver *, int, int32_t *, int32_t *, double *, double *,
                                 int32_t *) {
  nrt::set_error("implicit mode not available in this build");
  return NRT_EINVAL;
}
