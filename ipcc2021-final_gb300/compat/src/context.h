// context.h -- the process-wide GPU context behind the reference-API layer.
#pragma once
#include <stdexcept>
#include <string>
#include "wilson_gb300.h"

namespace wd_compat {
// The device is WD_DEVICE (default 0).  Created on first use; kept until exit.
wd_context *ctx();
// Throws std::runtime_error with the library's message unless s == WD_OK.
void check(wd_status s, const char *what);
// The reference passes the local block (subgs) and global extents
// (site_vec); one GPU holds the whole lattice, so they must agree.
void require_single_block(const int *subgs, const int *site_vec, const char *what);
}  // namespace wd_compat
