// load_gauge.h -- the reference's gauge loader (include/load_gauge.h:13).
#ifndef LOAD_GAUGE_H
#define LOAD_GAUGE_H

#include <complex>
#include <string>
#include "lattice_gauge.h"

// "UNIT": identity links.  "RANDOM": seeded SU(3) links exp(i 0.5 H) (the
// reference leaves this branch empty; seed from WD_GAUGE_SEED, default 1).
// Otherwise: a big-endian file of 72 doubles per site in lexicographic order
// (4 directions x 3x3 complex), optionally after a header (ILDG/LIME: the
// payload is taken as the last V*72 doubles, or V*72 floats for a
// single-precision file); reordered into the even-odd layout.
int load_gauge(std::complex<double> *gauge[4], std::string &filename, int *subgs, int *site_vec);

#endif
