// Host-side FP64 geometry tables with the reference's own arithmetic (used by
// the preps in runtime.cu and by the batched plan in batch.cu).
#pragma once

#include <vector>

namespace ctr {

// src/bp_fan_2d.cc:22-42: pixel centres by repeated addition
void pixel_positions(unsigned nx, unsigned ny, double dx, double dy, double ox, double oy,
                     std::vector<double>& xpos, std::vector<double>& ypos);
// src/bp_fan_2d.cc:28-34: (sin, cos) of orbit_start + ia*orbit by repeated addition
void fan_sincos(unsigned na, double orbit_start, double orbit, std::vector<double>& sc);
// src/filter.cc:18-65: taps n in [-ns, ns] at [n + ns]; false for an unknown type
bool ramp_taps(unsigned ns, double ds, double dsd, int type, std::vector<double>& taps);
// src/fan_weighting.cc:19-38: per-channel weight; false for an unknown type
bool fan_weights(unsigned ns, double ds, double offset, double dso, double dsd, int type,
                 std::vector<double>& w);

}  // namespace ctr
