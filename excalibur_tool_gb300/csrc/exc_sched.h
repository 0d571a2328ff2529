// exc_sched.h -- the launch-size rules shared by the host launchers and the C ABI.
#pragma once
#include <stdint.h>

namespace exc {

// Warps an SM for n similar trajectories, one a lane, at most `occ` warps an SM on `sms` SMs: the
// batch over the waves it needs at that limit, rounded up to whole warps an SM, so that the last
// wave is as full as the others (65,536 rays on 152 SMs with 9 warps an SM: 2 waves, 7 warps an
// SM, 1.92 rays a lane).
inline int balanced_warps_per_sm(int64_t n, int sms, int occ) {
  if (sms < 1) sms = 1;
  if (occ < 1) occ = 1;
  if (n < 1) return 1;
  const int64_t lanes_sm = (int64_t)sms * 32;
  const int64_t waves = (n + lanes_sm * occ - 1) / (lanes_sm * occ);
  const int64_t lanes = (n + waves - 1) / waves;
  const int64_t warps = (lanes + lanes_sm - 1) / lanes_sm;
  return (int)(warps < 1 ? 1 : (warps > occ ? occ : warps));
}

}  // namespace exc
