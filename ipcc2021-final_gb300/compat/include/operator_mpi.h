// operator_mpi.h -- global reductions of the reference (include/operator_mpi.h:15-79).
// The reference sums with AVX and combines ranks with MPI; here both run as
// one deterministic FP64 reduction on the GPU.
#ifndef LATTICE_OPERATOR_MPI_H
#define LATTICE_OPERATOR_MPI_H

#include <complex>

namespace wd_compat {
double host_norm2(long n, const std::complex<double> *a);
std::complex<double> host_dot(long n, const std::complex<double> *a, const std::complex<double> *b);
}  // namespace wd_compat

// sum_i |s.A_i|^2
template <typename T>
double norm_2(const T &s)
{
    return wd_compat::host_norm2(s.size, s.A);
}

// sum_i conj(r1.A_i) r2.A_i
template <typename T>
std::complex<double> vector_p(const T &r1, const T &r2)
{
    return wd_compat::host_dot(r1.size, r1.A, r2.A);
}

#endif
