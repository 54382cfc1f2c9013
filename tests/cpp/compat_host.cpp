// compat_host.cpp -- the host-side parts of the reference-API layer
// (liblattice_gb300.so) that need no GPU: the containers (borrow / own,
// alignment, zeroing, element-wise arithmetic, clean), gamma5, the gauge
// container's peeksite, and the index helpers of operator.h.  Prints "ok" and
// returns 0, or names the first failed check and returns 1.
//   compat_host
#include <complex>
#include <cstdint>
#include <cstdio>
#include <vector>
#include "check.h"
#include "lattice_fermion.h"
#include "lattice_gauge.h"
#include "operator.h"

typedef std::complex<double> cd;

#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond);    \
            return 1;                                                \
        }                                                            \
    } while (0)

int main()
{
    int dims[4] = {4, 2, 6, 4};
    const int V = dims[0] * dims[1] * dims[2] * dims[3];

    // owning container: zeroed, 64-byte aligned, V*12 entries
    {
        lattice_fermion a(dims, dims);
        CHECK(a.size == V * 12);
        CHECK(((uintptr_t)a.A % 64) == 0);
        for (int i = 0; i < a.size; ++i) CHECK(a.A[i] == cd(0.0, 0.0));
    }

    // borrowing container: uses the caller's array and leaves it alive
    std::vector<cd> buf(V * 12), buf2(V * 12);
    for (int i = 0; i < V * 12; ++i) {
        buf[i] = cd(0.5 * i, -1.0 * i);
        buf2[i] = cd(1.0, 0.25 * i);
    }
    {
        lattice_fermion b(buf.data(), dims, dims);
        CHECK(b.A == buf.data());
        CHECK(b.size == V * 12);
    }
    CHECK(buf[7] == cd(3.5, -7.0));

    // element-wise arithmetic on host memory
    {
        lattice_fermion x(buf.data(), dims, dims), y(buf2.data(), dims, dims);
        lattice_fermion s(dims, dims), d(dims, dims);
        Plus(x, y, s);
        Minus(x, y, d);
        for (int i = 0; i < V * 12; ++i) {
            CHECK(s.A[i] == buf[i] + buf2[i]);
            CHECK(d.A[i] == buf[i] - buf2[i]);
        }
        s += y;  // s = x + 2y
        for (int i = 0; i < V * 12; ++i) CHECK(s.A[i] == buf[i] + buf2[i] + buf2[i]);
        s - y;   // in place: s = x + y
        for (int i = 0; i < V * 12; ++i) CHECK(s.A[i] == buf[i] + buf2[i]);
        d + y;   // in place: d = x
        for (int i = 0; i < V * 12; ++i) CHECK(d.A[i] == buf[i]);
        s.clean();
        for (int i = 0; i < V * 12; ++i) CHECK(s.A[i] == cd(0.0, 0.0));

        // gamma5 = diag(1, 1, -1, -1) in spin: the last six of each site's twelve entries negated
        lattice_fermion g(dims, dims);
        gamma5_lattcefermion(x, g);
        for (int i = 0; i < V * 12; ++i) CHECK(g.A[i] == ((i % 12) < 6 ? buf[i] : -buf[i]));
    }

    // index helpers: lexicographic order x fastest, even sites first, lex/2 within a parity
    {
        std::vector<int> seen(V, 0);
        for (int t = 0; t < dims[3]; ++t)
            for (int z = 0; z < dims[2]; ++z)
                for (int y = 0; y < dims[1]; ++y)
                    for (int x = 0; x < dims[0]; ++x) {
                        int c[4] = {x, y, z, t};
                        const int lex = x + dims[0] * (y + dims[1] * (z + dims[2] * t));
                        CHECK(local_site2(c, dims) == lex);
                        CHECK(site2index(c, dims) == lex);
                        const int eo = site2eoindex(c, dims);
                        CHECK(eo == lex / 2 + ((x + y + z + t) & 1) * (V / 2));
                        ++seen[eo];
                        int back[4];
                        index2site(lex, back, dims);
                        CHECK(back[0] == x && back[1] == y && back[2] == z && back[3] == t);
                        // periodic wrap
                        int w[4] = {x + dims[0], y + 2 * dims[1], z, t + dims[3]};
                        CHECK(site2index(w, dims) == lex);
                    }
        for (int i = 0; i < V; ++i) CHECK(seen[i] == 1);
    }

    // norms of the two halves (even and odd parity blocks)
    {
        lattice_fermion x(buf.data(), dims, dims);
        double e = 0, o = 0;
        for (int i = 0; i < V * 6; ++i) e += std::norm(buf[i]);
        for (int i = V * 6; i < V * 12; ++i) o += std::norm(buf[i]);
        CHECK(norm_2_E(x) == e);
        CHECK(norm_2_O(x) == o);
    }

    // gauge container: borrow, own (zeroed), peeksite = A[dir][eo*9 + row*3 + col]
    {
        std::vector<cd> gbuf[4];
        cd *gp[4];
        for (int mu = 0; mu < 4; ++mu) {
            gbuf[mu].resize(V * 9);
            for (int i = 0; i < V * 9; ++i) gbuf[mu][i] = cd(mu, i);
            gp[mu] = gbuf[mu].data();
        }
        lattice_gauge U(gp, dims, dims);
        CHECK(U.size == V * 9);
        for (int mu = 0; mu < 4; ++mu) CHECK(U.A[mu] == gp[mu]);
        int site[4] = {3, 1, 4, 2};
        const int lex = 3 + dims[0] * (1 + dims[1] * (4 + dims[2] * 2));
        const int eo = lex / 2 + ((3 + 1 + 4 + 2) & 1) * (V / 2);
        for (int mu = 0; mu < 4; ++mu)
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) CHECK(U.peeksite(site, r, c, mu) == gbuf[mu][eo * 9 + r * 3 + c]);
        lattice_gauge W(dims, dims);
        for (int mu = 0; mu < 4; ++mu)
            for (int i = 0; i < W.size; ++i) CHECK(W.A[mu][i] == cd(0.0, 0.0));
    }

    std::printf("ok\n");
    return 0;
}
