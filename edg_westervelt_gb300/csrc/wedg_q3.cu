// Kernel instantiations for q_u = 3 (NU = 4), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q3(int nv, bool fast) {
  if (nv == 4) return make_launchers<4, 4>(fast);
  if (nv == 3) return make_launchers<4, 3>(fast);
  return Launchers();
}
}  // namespace wedg
