// Kernel instantiations for q_u = 2 (NU = 3), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q2(int nv, bool fast) {
  if (nv == 3) return make_launchers<3, 3>(fast);
  if (nv == 2) return make_launchers<3, 2>(fast);
  return Launchers();
}
}  // namespace wedg
