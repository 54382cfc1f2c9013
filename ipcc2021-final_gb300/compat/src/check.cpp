// check.cpp -- the reference's residual report (src/check.cpp:18-176).
// The six operator applications and all norms run on the GPU (wd_host_check);
// the report is printed in the reference's format.
#include <cmath>
#include <complex>
#include <iostream>
#include "check.h"
#include "context.h"
#include "operator.h"

int check(lattice_fermion &src, lattice_fermion &chi, lattice_gauge &U, double mass)
{
    wd_compat::require_single_block(src.subgs, src.site_vec, "check");
    double r[12];
    wd_compat::check(wd_host_check(wd_compat::ctx(), src.site_vec, reinterpret_cast<const double *const *>(U.A),
                                   reinterpret_cast<const double *>(src.A), reinterpret_cast<const double *>(chi.A),
                                   mass, r),
                     "check");
    const std::complex<double> MbMb(r[2], r[3]), bMMb(r[4], r[5]), MxMx(r[6], r[7]), xMMx(r[8], r[9]);
    std::cout << "===================================" << std::endl;
    std::cout << "|b| = " << r[0] << "    |x| = " << r[1] << std::endl;
    std::cout << "(Mb, Mb) = " << MbMb << "    (b, MMb) = " << bMMb << std::endl;
    std::cout << "(Mx, Mx) = " << MxMx << "    (x, MMx) = " << xMMx << std::endl;
    std::cout << "|M x -b| = " << r[10] << std::endl;
    std::cout << "|M^dagger M x - Mdb| = " << r[11] << std::endl;
    std::cout << "===================================" << std::endl;
    return 0;
}

int check(std::complex<double> *src_p, std::complex<double> *chi_p, std::complex<double> *gauge[4],
          const double mass, int *subgs, int *site_vec)
{
    lattice_fermion src(src_p, subgs, site_vec), chi(chi_p, subgs, site_vec);
    lattice_gauge U(gauge, subgs, site_vec);
    return check(src, chi, U, mass);
}

// prints every global site with the rank that owns it (one rank here: 0)
void check_lattice_site(int *subgs, int *site_vec)
{
    int nsub[4], site[4], coords[4];
    for (int i = 0; i < 4; ++i) nsub[i] = site_vec[i] / subgs[i];
    for (site[3] = 0; site[3] < site_vec[3]; ++site[3])
        for (site[2] = 0; site[2] < site_vec[2]; ++site[2])
            for (site[1] = 0; site[1] < site_vec[1]; ++site[1])
                for (site[0] = 0; site[0] < site_vec[0]; ++site[0]) {
                    for (int k = 0; k < 4; ++k) coords[k] = site[k] / subgs[k];
                    std::cout << "(" << site[0] << " " << site[1] << " " << site[2] << " " << site[3]
                              << ") ,    node_num= " << get_nodenum(coords, nsub, 4) << std::endl;
                }
}

// gamma5 = diag(1, 1, -1, -1) in the reference's chiral basis: flips the
// sign of spin components 2 and 3 of every site.  (The reference's version,
// unused there, negates every entry after the first six instead.)
void gamma5_lattcefermion(lattice_fermion &src, lattice_fermion &dest)
{
    for (int i = 0; i < src.size; ++i) dest.A[i] = (i % 12) < 6 ? src.A[i] : -src.A[i];
}

// prints U and U U^dag for one 3x3 link (src/check.cpp:112-134)
void check_gauge_unitary(std::complex<double> *U)
{
    std::cout << "U  = " << std::endl;
    for (int i = 0; i < 3; ++i) std::cout << U[i * 3] << "  " << U[i * 3 + 1] << "  " << U[i * 3 + 2] << std::endl;
    std::cout << "U U^dagger = " << std::endl;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            std::complex<double> s = 0;
            for (int k = 0; k < 3; ++k) s += U[i * 3 + k] * std::conj(U[j * 3 + k]);
            std::cout << s << (j < 2 ? "  " : "");
        }
        std::cout << std::endl;
    }
    std::cout << std::endl;
}

// empty in the reference (src/check.cpp:136-138)
void check_plaq(lattice_gauge &) {}
