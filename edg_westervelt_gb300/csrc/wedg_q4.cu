// Kernel instantiations for q_u = 4 (NU = 5), both pairings q_v = q_u - 1, q_u.
#include "wedg_dispatch.h"

namespace wedg {
Launchers launchers_q4(int nv, bool fast) {
  if (nv == 5) return make_launchers<5, 5>(fast);
  if (nv == 4) return make_launchers<5, 4>(fast);
  return Launchers();
}
}  // namespace wedg
