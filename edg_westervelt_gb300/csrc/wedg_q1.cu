// Kernel instantiations for q_u = 1 (NU = 2), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q1(int nv, bool fast) {
  if (nv == 2) return make_launchers<2, 2>(fast);
  if (nv == 1) return make_launchers<2, 1>(fast);
  return Launchers();
}
}  // namespace wedg
