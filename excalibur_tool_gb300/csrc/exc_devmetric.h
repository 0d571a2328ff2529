// exc_devmetric.h -- kernel-side view of ExcMetric shared by every build.
#pragma once
#include "../../include/excalibur_gb300.h"

namespace exc {

// ExcMetric plus the reciprocals the fast path multiplies by (filled once on
// the host per launch; the parity path never reads them).
struct DevMetric {
  ExcMetric m;
  double ic2, ic4, i_eta_step;
  double finv[EXC_MAX_FIELDS][8];   // 1/s0, 1/s1, 1/s2, 1/s3, 1/(2 s0), 1/(2 s1), 1/(2 s2), 1/(2 s3)
  int retrace_only;                 // trace only photons whose status is EXC_PH_RETRACE
  int stage_table;                  // the a(eta) table is read from the block's shared-memory copy
  int retrace_sms;                  // SMs of the device (re-trace launches: sizes the active blocks)
};

}  // namespace exc
