// wd_precision.h -- derived (lower-precision or double-float) copies of the
// resident links, built on first use and dropped when the links change.
#pragma once
#include "wd_internal.cuh"

void wd_lattice_invalidate_derived(wd_lattice *lat);
