// Kernel instantiations for q_u = 5 (NU = 6), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q5(int nv, bool fast) {
  if (nv == 6) return make_launchers<6, 6>(fast);
  if (nv == 5) return make_launchers<6, 5>(fast);
  return Launchers();
}
}  // namespace wedg
