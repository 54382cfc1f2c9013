// operator.h -- index helpers of the reference (include/operator.h:11-75).
// Lexicographic order has x fastest; the even-odd index puts all even sites
// (x+y+z+t even) first, each parity in lexicographic order of x/2.
#ifndef OPERATOR_H
#define OPERATOR_H

#include <complex>

// lexicographic index of coord within a block of extents latt_size
static inline int local_site2(const int *coord, const int *latt_size)
{
    return coord[0] + latt_size[0] * (coord[1] + latt_size[1] * (coord[2] + latt_size[2] * coord[3]));
}

// rank number of grid coordinate x on a grid of extents l (first index fastest)
static inline int get_nodenum(const int *x, int *l, int nd)
{
    int n = 0;
    for (int i = nd - 1; i >= 0; --i) n = n * l[i] + x[i];
    return n;
}

// sum |A_i|^2 over the first / second half of a container.  Taken by
// reference: the reference passes the container by value, which compiles
// the same at every call site, but a copy of an owning container would free
// its array twice (the containers here are not copyable).
template <typename T>
double norm_2_E(const T &s)
{
    double r = 0.0;
    for (int i = 0; i < s.size / 2; ++i) r += std::norm(s.A[i]);
    return r;
}
template <typename T>
double norm_2_O(const T &s)
{
    double r = 0.0;
    for (int i = s.size / 2; i < s.size; ++i) r += std::norm(s.A[i]);
    return r;
}

// lexicographic index with periodic wrap
static inline int site2index(int *x, int *L)
{
    int w[4];
    for (int i = 0; i < 4; ++i) w[i] = x[i] % L[i];
    return local_site2(w, L);
}

// even-odd index: lex/2 within the parity block
static inline int site2eoindex(int *x, int *L)
{
    const int half_volume = L[0] * L[1] * L[2] * L[3] / 2;
    return site2index(x, L) / 2 + ((x[0] + x[1] + x[2] + x[3]) & 1) * half_volume;
}

// coordinates of lexicographic index idx
static inline void index2site(int idx, int x[4], int *L)
{
    for (int i = 0; i < 4; ++i) {
        x[i] = idx % L[i];
        idx /= L[i];
    }
}

#endif
