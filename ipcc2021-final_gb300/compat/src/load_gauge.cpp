// load_gauge.cpp -- the reference's gauge loader (src/load_gauge.cpp:29-181) for one GPU;
// files are read by wd_read_gauge_file (the reference's format, NERSC, ILDG).
#include <cstdlib>
#include <stdexcept>
#include "context.h"
#include "load_gauge.h"

int load_gauge(std::complex<double> *gauge[4], std::string &filename, int *subgs, int *site_vec)
{
    wd_compat::require_single_block(subgs, site_vec, "load_gauge");
    const long V = (long)site_vec[0] * site_vec[1] * site_vec[2] * site_vec[3];
    if (filename == "UNIT") {
        for (int mu = 0; mu < 4; ++mu)
            for (long s = 0; s < V; ++s)
                for (int k = 0; k < 9; ++k) gauge[mu][s * 9 + k] = (k % 4 == 0) ? 1.0 : 0.0;
        return 0;
    }
    if (filename == "RANDOM") {
        const char *seed = std::getenv("WD_GAUGE_SEED");
        double *g[4];
        for (int mu = 0; mu < 4; ++mu) g[mu] = reinterpret_cast<double *>(gauge[mu]);
        wd_compat::check(wd_gen_gauge(site_vec, seed ? std::strtoull(seed, nullptr, 10) : 1, 0.5, g), "load_gauge");
        return 0;
    }
    // the reference's own format (whole file, or LIME-framed with its 280-byte
    // trailer), and beyond it NERSC and single-precision ILDG configurations
    double *g[4];
    for (int mu = 0; mu < 4; ++mu) g[mu] = reinterpret_cast<double *>(gauge[mu]);
    const wd_status st = wd_read_gauge_file(filename.c_str(), site_vec, WD_GAUGE_FILE_AUTO, g, nullptr);
    if (st == WD_ERR_BAD_ARG) throw std::runtime_error("load_gauge: can not open file: " + filename);
    if (st != WD_OK) throw std::runtime_error("load_gauge: file size does not match the lattice: " + filename);
    return 0;
}
