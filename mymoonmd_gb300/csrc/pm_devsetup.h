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

// build_hierarchy with the regular refinement on the context's GPU (the root
// mesh from the host; every level copied back into the host hierarchy)
pmsetup::Hierarchy device_hierarchy(pm_ctx* c, int geometry, int root_n, int n_refine);

// the combined CSR structure of a Stokes level (the 34 x 34 local coupling of
// the NSTYPE 4 blocks), its gather plans into the 220-entry element storage
// and the unit diagonals of the non-active rows, from L.cdof and the active
// flags: one stable radix sort as for a scalar level
void device_stokes_structure(pm_ctx* c, DiscLevel& L, const std::vector<char>& active);

// build_space with the first-touch numbering on the context's GPU: the same
// GlobalNumbers, node coordinates and class counts
pmsetup::Space device_space(pm_ctx* c, const pmsetup::Hierarchy& h, int level, int elem, int boundary,
                            int neumann_sides);

}  // namespace pm
