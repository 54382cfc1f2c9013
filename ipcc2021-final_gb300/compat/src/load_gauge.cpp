// load_gauge.cpp -- the reference's gauge loader (src/load_gauge.cpp:29-181) for one GPU.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>
#include "context.h"
#include "load_gauge.h"
#include "operator.h"

namespace {
uint64_t bswap64(uint64_t v)
{
    uint64_t r = 0;
    for (int i = 0; i < 8; ++i) r |= ((v >> (8 * i)) & 0xffu) << (8 * (7 - i));
    return r;
}
}  // namespace

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
    FILE *fh = std::fopen(filename.c_str(), "rb");
    if (!fh) throw std::runtime_error("load_gauge: can not open file: " + filename);
    std::fseek(fh, 0, SEEK_END);
    const long fsize = std::ftell(fh);
    const long payload = V * 72 * (long)sizeof(double);
    // plain file: the payload is the whole file; ILDG/LIME: the payload ends
    // 280 bytes before the end of the file (the reference's LIME convention)
    long offset;
    if (fsize == payload) offset = 0;
    else if (fsize >= payload + 280) offset = fsize - payload - 280;
    else {
        std::fclose(fh);
        throw std::runtime_error("load_gauge: file size does not match the lattice: " + filename);
    }
    std::vector<uint64_t> raw((size_t)V * 72);
    std::fseek(fh, offset, SEEK_SET);
    const size_t got = std::fread(raw.data(), sizeof(uint64_t), raw.size(), fh);
    std::fclose(fh);
    if (got != raw.size()) throw std::runtime_error("load_gauge: short read: " + filename);
    // big-endian doubles, [site lex][mu][row][col][re, im] -> even-odd per direction
    int x[4];
    for (long lex = 0; lex < V; ++lex) {
        index2site((int)lex, x, site_vec);
        const long eo = site2eoindex(x, site_vec);
        for (int mu = 0; mu < 4; ++mu)
            for (int k = 0; k < 9; ++k) {
                const uint64_t re = bswap64(raw[(size_t)lex * 72 + mu * 18 + 2 * k]);
                const uint64_t im = bswap64(raw[(size_t)lex * 72 + mu * 18 + 2 * k + 1]);
                double dr, di;
                std::memcpy(&dr, &re, 8);
                std::memcpy(&di, &im, 8);
                gauge[mu][eo * 9 + k] = std::complex<double>(dr, di);
            }
    }
    return 0;
}
