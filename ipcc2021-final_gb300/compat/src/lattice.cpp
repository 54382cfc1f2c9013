// lattice.cpp -- host containers of the reference API (src/lattice_fermion.cpp,
// src/lattice_gauge.cpp).  They own or borrow host arrays; element-wise
// container arithmetic (+=, Minus, Plus, clean) stays on the host memory the
// container lives in, as in the reference.  Operators run on the GPU.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include "lattice_fermion.h"
#include "lattice_gauge.h"
#include "operator.h"

namespace {
int volume(const int *d) { return d[0] * d[1] * d[2] * d[3]; }

std::complex<double> *alloc_zeroed(size_t n)
{
    void *p = nullptr;
    if (posix_memalign(&p, 64, n * sizeof(std::complex<double>)) != 0) throw std::bad_alloc();
    std::memset(p, 0, n * sizeof(std::complex<double>));
    return static_cast<std::complex<double> *>(p);
}
}  // namespace

lattice_fermion::lattice_fermion(std::complex<double> *data, int *subgs1, int *site_vec1)
    : site_vec(site_vec1), A(data), subgs(subgs1), size(volume(subgs1) * 12), mem_flag(false)
{
}

lattice_fermion::lattice_fermion(int *subgs1, int *site_vec1)
    : site_vec(site_vec1), A(nullptr), subgs(subgs1), size(volume(subgs1) * 12), mem_flag(true)
{
    A = alloc_zeroed(size);
}

lattice_fermion::~lattice_fermion()
{
    if (mem_flag) std::free(A);
    A = nullptr;
}

void lattice_fermion::clean() { std::fill(A, A + size, std::complex<double>(0.0, 0.0)); }

lattice_fermion &lattice_fermion::operator-(const lattice_fermion &a)
{
    for (int i = 0; i < size; ++i) A[i] -= a.A[i];
    return *this;
}

lattice_fermion &lattice_fermion::operator+(const lattice_fermion &a)
{
    for (int i = 0; i < size; ++i) A[i] += a.A[i];
    return *this;
}

void lattice_fermion::operator+=(const lattice_fermion &a)
{
    for (int i = 0; i < size; ++i) A[i] += a.A[i];
}

void Minus(lattice_fermion &src1, lattice_fermion &src2, lattice_fermion &a)
{
    for (int i = 0; i < src1.size; ++i) a.A[i] = src1.A[i] - src2.A[i];
}

void Plus(lattice_fermion &src1, lattice_fermion &src2, lattice_fermion &a)
{
    for (int i = 0; i < src1.size; ++i) a.A[i] = src1.A[i] + src2.A[i];
}

lattice_gauge::lattice_gauge(std::complex<double> *data[4], int *subgs1, int *site_vec1)
    : site_vec(site_vec1), subgs(subgs1), size(volume(subgs1) * 9), mem_flag(false)
{
    for (int i = 0; i < 4; ++i) A[i] = data[i];
}

lattice_gauge::lattice_gauge(int *subgs1, int *site_vec1)
    : site_vec(site_vec1), subgs(subgs1), size(volume(subgs1) * 9), mem_flag(true)
{
    for (int i = 0; i < 4; ++i) A[i] = alloc_zeroed(size);
}

lattice_gauge::~lattice_gauge()
{
    if (mem_flag)
        for (int i = 0; i < 4; ++i) std::free(A[i]);
}

std::complex<double> lattice_gauge::peeksite(const int *site, int ll, int mm, int dd)
{
    int x[4] = {site[0], site[1], site[2], site[3]};
    return A[dd][site2eoindex(x, subgs) * 9 + ll * 3 + mm];
}
