// The optics table of the render-side passes (optics.cpp) and the passes themselves
// (optics.cu): one DevOptics row per material row, as material.rs's GpuOptics lays it out.
#pragma once

#include "device_types.h"

namespace sprout {

struct SimParams;
// material.rs's optics_table row r of the live material table
void optics_row(const SimParams& p, int r, DevOptics& o);
void optics_table(const SimParams& p, DevOptics* out);

}  // namespace sprout
