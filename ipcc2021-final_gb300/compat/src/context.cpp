// context.cpp -- process-wide context and error reporting of the reference-API layer.
#include "context.h"
#include <cstdlib>
#include <mutex>

namespace wd_compat {

wd_context *ctx()
{
    static std::once_flag once;
    static wd_context *c = nullptr;
    static wd_status st = WD_OK;
    std::call_once(once, [] {
        const char *dev = std::getenv("WD_DEVICE");
        st = wd_context_create(dev ? std::atoi(dev) : 0, &c);
    });
    if (st != WD_OK)
        throw std::runtime_error(std::string("wilson_gb300: no usable GB300 device: ") + wd_status_string(st));
    return c;
}

void check(wd_status s, const char *what)
{
    if (s == WD_OK) return;
    std::string msg = std::string("wilson_gb300: ") + what + ": " + wd_status_string(s);
    if (wd_context *c = ctx()) {
        const char *e = wd_last_error(c);
        if (e && *e) msg += std::string(" (") + e + ")";
    }
    throw std::runtime_error(msg);
}

void require_single_block(const int *subgs, const int *site_vec, const char *what)
{
    for (int i = 0; i < 4; ++i)
        if (subgs[i] != site_vec[i])
            throw std::runtime_error(std::string("wilson_gb300: ") + what +
                                     ": the lattice is not split across ranks on one GPU (subgs must equal site_vec)");
}

}  // namespace wd_compat
