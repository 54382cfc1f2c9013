// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points around the reference's own solver sources (compiled
// unmodified from the reference tree, single rank, against mpi_shim/mpi.h).
// Used to write the golden vectors under tests/golden/ and to pin the C
// restatement in wilson_oracle.c.  Built only where the reference tree and an
// x86 compiler are present (the reference uses AVX2 intrinsics).
#include <complex>
#include <cstdlib>
#include <sstream>
#include <string>
#include <iostream>
#include "invert.h"
#include "check.h"
#include "dslash.h"
#include "dslash_new.h"

typedef std::complex<double> cd;

namespace {
struct Dims {
    int v[4];
    explicit Dims(const int *d) { for (int i = 0; i < 4; ++i) v[i] = d[i]; }
};
// The reference's CG and check report through std::cout; capture it.
struct CoutCapture {
    std::ostringstream ss;
    std::streambuf *old;
    CoutCapture() : old(std::cout.rdbuf(ss.rdbuf())) {}
    ~CoutCapture() { std::cout.rdbuf(old); }
};
}  // namespace

extern "C" {

void ref_dslash_new(double *src, double *dest, double **gauge, const int *dims, double mass, int dag)
{
    Dims d(dims), s(dims);
    lattice_gauge U((cd **)gauge, s.v, d.v);
    lattice_fermion a((cd *)src, s.v, d.v), b((cd *)dest, s.v, d.v);
    DslashNew(a, b, U, mass, dag != 0);
}

void ref_dslash_old(double *src, double *dest, double **gauge, const int *dims, double mass, int dag)
{
    Dims d(dims), s(dims);
    lattice_gauge U((cd **)gauge, s.v, d.v);
    lattice_fermion a((cd *)src, s.v, d.v), b((cd *)dest, s.v, d.v);
    Dslash(a, b, U, mass, dag != 0);
}

void ref_dslashoffd_new(double *src, double *dest, double **gauge, const int *dims, int dag, int cb)
{
    Dims d(dims), s(dims);
    lattice_gauge U((cd **)gauge, s.v, d.v);
    lattice_fermion a((cd *)src, s.v, d.v), b((cd *)dest, s.v, d.v);
    DslashoffdNew(a, b, U, dag != 0, cb);
}

void ref_dslashoffd_old(double *src, double *dest, double **gauge, const int *dims, int dag, int cb)
{
    Dims d(dims), s(dims);
    lattice_gauge U((cd **)gauge, s.v, d.v);
    lattice_fermion a((cd *)src, s.v, d.v), b((cd *)dest, s.v, d.v);
    Dslashoffd(a, b, U, dag != 0, cb);
}

void ref_dslash_eeoo_new(double *src, double *dest, const int *dims, double mass)
{
    Dims d(dims), s(dims);
    lattice_fermion a((cd *)src, s.v, d.v), b((cd *)dest, s.v, d.v);
    DslashEEOONew(a, b, mass);
}

// srand(seed) then CGinvert exactly as the reference's main does; the
// iteration count and |r| come from the reference's own report line.
int ref_cginvert(double *src, double *dest, double **gauge, const int *dims, double mass, int max,
                 double accuracy, unsigned seed, double *rsd)
{
    Dims d(dims), s(dims);
    srand(seed);
    std::string text;
    {
        CoutCapture cap;
        CGinvert((cd *)src, (cd *)dest, (cd **)gauge, mass, max, accuracy, s.v, d.v);
        text = cap.ss.str();
    }
    int iters = -1;
    size_t pos = text.rfind("CG: ");
    if (pos != std::string::npos) {
        std::istringstream in(text.substr(pos + 4));
        in >> iters;
        size_t eq = text.find("= ", pos);
        if (rsd && eq != std::string::npos)
            *rsd = std::strtod(text.c_str() + eq + 2, nullptr);
    }
    return iters;
}

// check(): returns the text the reference prints.
int ref_check(double *src, double *x, double **gauge, const int *dims, double mass, char *buf, int len)
{
    Dims d(dims), s(dims);
    std::string text;
    {
        CoutCapture cap;
        std::cout.precision(17);
        check((cd *)src, (cd *)x, (cd **)gauge, mass, s.v, d.v);
        text = cap.ss.str();
    }
    int n = (int)text.size() < len - 1 ? (int)text.size() : len - 1;
    text.copy(buf, n);
    buf[n] = 0;
    return n;
}
}
