// Device-side set-up of a scalar level (see pm_devsetup.cu).
#pragma once
#include "pm_disc.h"
#include "pm_linalg.cuh"

namespace pm {

// L.sys (the square CSR structure of L.space), the assembly gather plans
// gat_ptr / gat_idx and rgat_ptr / rgat_idx, and diag_pos, built on the
// context's GPU by sorting and copied into L: the same arrays as the host
// construction of build_disc.
void device_level_structure(pm_ctx* c, DiscLevel& L);

}  // namespace pm
