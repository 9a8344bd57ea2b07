// stats.cuh -- a solver's last-step statistics in the ABI's PpfStepStats.
#pragma once

#include "../../../include/ppf_gb300_ext.h"
#include "solver.cuh"

namespace ppf {
namespace gpu {
void fill_step_stats(const Solver &solver, PpfStepStats *out);
} // namespace gpu
} // namespace ppf
