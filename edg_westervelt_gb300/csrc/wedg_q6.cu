// Kernel instantiations for q_u = 6 (NU = 7), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q6(int nv, bool fast) {
  if (nv == 7) return make_launchers<7, 7>(fast);
  if (nv == 6) return make_launchers<7, 6>(fast);
  return Launchers();
}
}  // namespace wedg
