// Kernel instantiations for q_u = 7 (NU = 8), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q7(int nv, bool fast) {
  if (nv == 8) return make_launchers<8, 8>(fast);
  if (nv == 7) return make_launchers<8, 7>(fast);
  return Launchers();
}
}  // namespace wedg
