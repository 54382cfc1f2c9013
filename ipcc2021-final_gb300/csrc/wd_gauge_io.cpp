// wd_gauge_io.cpp -- gauge-configuration files into the reference layout
// (host only; no device work).
//
// Formats (all site-major with x fastest, then the four directions, each
// link a row-major 3x3 -- or its first two rows -- of (re, im) pairs):
//   REF   the reference's load_gauge input (src/load_gauge.cpp:58-161):
//         big-endian doubles, 72 per site, the payload either the whole file
//         or ending 280 bytes before its end (the LIME framing of the
//         contest's files);
//   NERSC an ASCII header BEGIN_HEADER ... END_HEADER (DATATYPE
//         4D_SU3_GAUGE = rows 0 and 1, 4D_SU3_GAUGE_3x3 = all three;
//         FLOATING_POINT IEEE64/IEEE32, BIG or LITTLE; DIMENSION_1..4), the
//         payload after it; row 2 of a two-row link is conj(row0 x row1), as
//         refs/utils_nersc_lat.cpp:56-63 rebuilds it;
//   ILDG  the binary record of a LIME file, big-endian, taken as the last
//         V*72 values of the file, in double precision when they fit the
//         file twice over and single precision otherwise
//         (refs/utils_nersc_lat.cpp:228-290).
// The reference layout is gauge[mu][eo*9 + row*3 + col] with
// eo = lex/2 + ((x+y+z+t) & 1) * V/2 (include/operator.h:56-67).
#include <cctype>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include "wilson_gb300.h"

namespace {

using cd = std::complex<double>;

struct File {
    FILE *f = nullptr;
    ~File()
    {
        if (f) std::fclose(f);
    }
};

template <int N>
void swap_bytes(unsigned char *p)
{
    for (int i = 0; i < N / 2; ++i) std::swap(p[i], p[N - 1 - i]);
}

// n values of `bytes` (8 or 4) each, optionally byte-swapped, as doubles
std::vector<double> decode(const std::vector<unsigned char> &raw, size_t n, int bytes, bool swap)
{
    std::vector<double> out(n);
    for (size_t i = 0; i < n; ++i) {
        unsigned char b[8];
        std::memcpy(b, raw.data() + i * bytes, bytes);
        if (bytes == 8) {
            if (swap) swap_bytes<8>(b);
            double d;
            std::memcpy(&d, b, 8);
            out[i] = d;
        } else {
            if (swap) swap_bytes<4>(b);
            float v;
            std::memcpy(&v, b, 4);
            out[i] = v;
        }
    }
    return out;
}

bool host_little_endian()
{
    const uint16_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

// values[site][mu][row < rows][col][re, im] in lexicographic site order -> reference layout
void scatter(const std::vector<double> &v, int rows, const int L[4], double *const gauge[4])
{
    const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
    const int per_link = rows * 6;
    for (int64_t lex = 0; lex < V; ++lex) {
        int64_t r = lex;
        const int x = (int)(r % L[0]);
        r /= L[0];
        const int y = (int)(r % L[1]);
        r /= L[1];
        const int z = (int)(r % L[2]);
        const int t = (int)(r / L[2]);
        const int64_t eo = lex / 2 + ((x + y + z + t) & 1) * (V / 2);
        for (int mu = 0; mu < 4; ++mu) {
            const double *src = v.data() + (lex * 4 + mu) * per_link;
            cd e[3][3];
            for (int a = 0; a < rows; ++a)
                for (int b = 0; b < 3; ++b) e[a][b] = cd(src[(a * 3 + b) * 2], src[(a * 3 + b) * 2 + 1]);
            if (rows == 2) {
                e[2][0] = std::conj(e[0][1] * e[1][2] - e[0][2] * e[1][1]);
                e[2][1] = std::conj(e[0][2] * e[1][0] - e[0][0] * e[1][2]);
                e[2][2] = std::conj(e[0][0] * e[1][1] - e[0][1] * e[1][0]);
            }
            double *dst = gauge[mu] + eo * 18;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    dst[(a * 3 + b) * 2] = e[a][b].real();
                    dst[(a * 3 + b) * 2 + 1] = e[a][b].imag();
                }
        }
    }
}

wd_status read_tail(FILE *f, long offset, size_t bytes, std::vector<unsigned char> &raw)
{
    raw.resize(bytes);
    if (std::fseek(f, offset, SEEK_SET) != 0) return WD_ERR_BAD_ARG;
    return std::fread(raw.data(), 1, bytes, f) == bytes ? WD_OK : WD_ERR_BAD_ARG;
}

std::string trim(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// NERSC header: key/value pairs and the payload offset; false if absent or malformed
bool nersc_header(FILE *f, std::map<std::string, std::string> &kv, long *payload)
{
    std::fseek(f, 0, SEEK_SET);
    char line[4096];
    if (!std::fgets(line, sizeof line, f) || trim(line) != "BEGIN_HEADER") return false;
    while (std::fgets(line, sizeof line, f)) {
        const std::string s = trim(line);
        if (s == "END_HEADER") {
            *payload = std::ftell(f);
            return true;
        }
        const size_t eq = s.find('=');
        if (eq != std::string::npos) kv[trim(s.substr(0, eq))] = trim(s.substr(eq + 1));
    }
    return false;
}

}  // namespace

extern "C" wd_status wd_read_gauge_file(const char *path, const int dims[4], int format, double *const gauge[4],
                                        int *format_found)
{
    if (!path || !dims || !gauge) return WD_ERR_BAD_ARG;
    for (int i = 0; i < 4; ++i)
        if (dims[i] <= 0 || !gauge[i]) return WD_ERR_BAD_ARG;
    if (dims[0] % 2) return WD_ERR_BAD_DIMS;
    const int64_t V = (int64_t)dims[0] * dims[1] * dims[2] * dims[3];
    const size_t nval = (size_t)V * 72;  // reals of the full links
    File fh;
    fh.f = std::fopen(path, "rb");
    if (!fh.f) return WD_ERR_BAD_ARG;
    std::fseek(fh.f, 0, SEEK_END);
    const long fsize = std::ftell(fh.f);
    const bool little = host_little_endian();

    std::map<std::string, std::string> kv;
    long payload = 0;
    const bool has_nersc = nersc_header(fh.f, kv, &payload);
    if (format == WD_GAUGE_FILE_AUTO) {
        if (has_nersc) format = WD_GAUGE_FILE_NERSC;
        else if (fsize == (long)(nval * 8) || fsize >= (long)(nval * 8) + 280) format = WD_GAUGE_FILE_REF;
        else if (fsize >= (long)(nval * 4)) format = WD_GAUGE_FILE_ILDG;
        else return WD_ERR_BAD_DIMS;
    }
    if (format_found) *format_found = format;
    std::vector<unsigned char> raw;
    wd_status st;
    switch (format) {
    case WD_GAUGE_FILE_REF: {
        const long bytes = (long)nval * 8;
        long offset;
        if (fsize == bytes) offset = 0;
        else if (fsize >= bytes + 280) offset = fsize - bytes - 280;
        else return WD_ERR_BAD_DIMS;
        if ((st = read_tail(fh.f, offset, (size_t)bytes, raw)) != WD_OK) return st;
        scatter(decode(raw, nval, 8, little), 3, dims, gauge);
        return WD_OK;
    }
    case WD_GAUGE_FILE_NERSC: {
        if (!has_nersc) return WD_ERR_BAD_ARG;
        for (int i = 0; i < 4; ++i) {
            auto it = kv.find("DIMENSION_" + std::to_string(i + 1));
            if (it != kv.end() && std::atoi(it->second.c_str()) != dims[i]) return WD_ERR_BAD_DIMS;
        }
        const std::string dt = kv.count("DATATYPE") ? kv["DATATYPE"] : "4D_SU3_GAUGE";
        const int rows = dt == "4D_SU3_GAUGE_3x3" ? 3 : 2;
        const std::string fp = kv.count("FLOATING_POINT") ? kv["FLOATING_POINT"] : "IEEE64BIG";
        const int bytes = fp.rfind("IEEE32", 0) == 0 ? 4 : 8;
        const bool big = fp.find("LITTLE") == std::string::npos;
        const size_t n = (size_t)V * 4 * rows * 6;
        if (fsize - payload < (long)(n * bytes)) return WD_ERR_BAD_DIMS;
        if ((st = read_tail(fh.f, payload, n * bytes, raw)) != WD_OK) return st;
        scatter(decode(raw, n, bytes, big == little), rows, dims, gauge);
        return WD_OK;
    }
    case WD_GAUGE_FILE_ILDG: {
        const int bytes = fsize >= (long)(nval * 8) ? 8 : 4;
        if (fsize < (long)(nval * bytes)) return WD_ERR_BAD_DIMS;
        if ((st = read_tail(fh.f, fsize - (long)(nval * bytes), nval * bytes, raw)) != WD_OK) return st;
        scatter(decode(raw, nval, bytes, little), 3, dims, gauge);
        return WD_OK;
    }
    default: return WD_ERR_BAD_ARG;
    }
}
