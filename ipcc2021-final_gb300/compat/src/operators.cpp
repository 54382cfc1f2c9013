// operators.cpp -- the reference's operator and solver entry points
// (include/dslash.h, dslash_new.h, invert.h, operator_mpi.h) on the GPU
// through the C ABI.  Host arrays in the reference layout go in and come out.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <iostream>
#include "context.h"
#include "invert.h"

using wd_compat::check;
using wd_compat::ctx;

namespace {
const double *const *links(lattice_gauge &U) { return reinterpret_cast<const double *const *>(U.A); }
const double *cd(const lattice_fermion &f) { return reinterpret_cast<const double *>(f.A); }
double *md(lattice_fermion &f) { return reinterpret_cast<double *>(f.A); }

void offd(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, bool dag, int cb, const char *who)
{
    wd_compat::require_single_block(src.subgs, src.site_vec, who);
    check(wd_host_dslash_offd(ctx(), src.site_vec, links(U), cd(src), md(dest), dag ? 1 : 0, cb), who);
}

void full(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, double mass, bool dag, const char *who)
{
    wd_compat::require_single_block(src.subgs, src.site_vec, who);
    check(wd_host_dslash_full(ctx(), src.site_vec, links(U), cd(src), md(dest), mass, dag ? 1 : 0), who);
}

// (4+m) src on the selected parity (-1: both); the other half of dest is zeroed
void diag(lattice_fermion &src, lattice_fermion &dest, double mass, int parity, const char *who)
{
    wd_compat::require_single_block(src.subgs, src.site_vec, who);
    check(wd_host_dslash_eeoo(ctx(), src.site_vec, cd(src), md(dest), mass, parity), who);
}
}  // namespace

namespace wd_compat {
double host_norm2(long n, const std::complex<double> *a)
{
    double r = 0.0;
    check(wd_host_norm2(ctx(), n, reinterpret_cast<const double *>(a), &r), "norm_2");
    return r;
}

std::complex<double> host_dot(long n, const std::complex<double> *a, const std::complex<double> *b)
{
    double r[2] = {0.0, 0.0};
    check(wd_host_dot(ctx(), n, reinterpret_cast<const double *>(a), reinterpret_cast<const double *>(b), r),
          "vector_p");
    return {r[0], r[1]};
}
}  // namespace wd_compat

// src/dslash.cpp:11-35
void DslashEE(lattice_fermion &src, lattice_fermion &dest, const double mass) { diag(src, dest, mass, 0, "DslashEE"); }
void DslashOO(lattice_fermion &src, lattice_fermion &dest, const double mass) { diag(src, dest, mass, 1, "DslashOO"); }
// src/dslash_new.cpp:1301-1338
void DslashEEOONew(lattice_fermion &src, lattice_fermion &dest, const double mass)
{
    diag(src, dest, mass, -1, "DslashEEOONew");
}

// src/dslash.cpp:38-1249 and src/dslash_new.cpp:1341-2677 (same operator)
void Dslashoffd(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag, int cb)
{
    offd(src, dest, U, dag, cb, "Dslashoffd");
}
void DslashoffdNew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag, int cb)
{
    offd(src, dest, U, dag, cb, "DslashoffdNew");
}
// declared but never defined by the reference (include/dslash.h:18-19, dslash_new.h:19-20):
// the even (cb 0) and odd (cb 1) halves of the hopping term
void DslashEO(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag)
{
    offd(src, dest, U, dag, 0, "DslashEO");
}
void DslashOE(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag)
{
    offd(src, dest, U, dag, 1, "DslashOE");
}
void DslashEONew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag)
{
    offd(src, dest, U, dag, 0, "DslashEONew");
}
void DslashOENew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag)
{
    offd(src, dest, U, dag, 1, "DslashOENew");
}

// src/invert.cpp:123-156
void Dslash(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const double mass, const bool dagger)
{
    full(src, dest, U, mass, dagger, "Dslash");
}
void DslashNew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const double mass, const bool dagger)
{
    full(src, dest, U, mass, dagger, "DslashNew");
}

// src/invert.cpp:25-121: random real initial guess from rand(), then CG on
// M^dag M x = M^dag b with the reference's recurrences and absolute stop.
// The reference prints every iteration unless built with VERBOSE_SIMPLE;
// here only its final report line is printed.
int CGinvert(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const double mass, const int max,
             const double accuracy)
{
    wd_compat::require_single_block(src.subgs, src.site_vec, "CGinvert");
    for (int i = 0; i < dest.size; ++i) dest.A[i] = 1.0 * rand() / RAND_MAX;
    wd_solver_params p;
    wd_solver_params_default(&p);
    p.kind = WD_SOLVER_CGNR_REF;
    p.mass = mass;
    p.tol = accuracy;
    p.max_iter = max;
    p.prec = WD_PREC_F64;
    if (const char *pr = std::getenv("WD_CG_PREC")) p.prec = std::atoi(pr) == 1 ? WD_PREC_DF64 : WD_PREC_F64;
    wd_solver_stats st;
    const wd_status s = wd_host_cg(ctx(), src.site_vec, links(U), cd(src), md(dest), &p, &st);
    if (s != WD_ERR_NOT_CONVERGED) check(s, "CGinvert");
    if (st.converged)
        std::cout << "CG: " << st.iterations << " iterations, convergence residual |r| = " << st.residual << std::endl;
    return 0;
}

// src/invert.cpp:15-23
int CGinvert(std::complex<double> *src_p, std::complex<double> *dest_p, std::complex<double> *gauge[4],
             const double mass, const int max, const double accuracy, int *subgs, int *site_vec)
{
    lattice_gauge U(gauge, subgs, site_vec);
    lattice_fermion src(src_p, subgs, site_vec);
    lattice_fermion dest(dest_p, subgs, site_vec);
    return CGinvert(src, dest, U, mass, max, accuracy);
}
