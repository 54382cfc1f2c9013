// compat_golden.cpp -- drives every entry point of the reference-API layer
// (liblattice_gb300.so) on inputs read from a binary file and writes the
// outputs, for tests/test_gpu_compat.py to compare with the golden vectors.
//   compat_golden in.bin out.bin
// in.bin:  int32 dims[4], float64 mass, int32 cg_seed, gauge 4*V*9 complex, src V*12 complex
// out.bin: for each named output, V*12 complex, in the order written below;
//          then float64 norm_2(src), complex vector_p(src, DslashNew(src)), the CGinvert
//          solution of the object overload, then that of the raw-pointer overload
//          (src/invert.cpp:15-23) on plain arrays, both after srand(cg_seed)
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "invert.h"

typedef std::complex<double> cd;

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    int dims[4], seed;
    double mass;
    if (!f || std::fread(dims, 4, 4, f) != 4 || std::fread(&mass, 8, 1, f) != 1 || std::fread(&seed, 4, 1, f) != 1)
        return 3;
    const long V = (long)dims[0] * dims[1] * dims[2] * dims[3];
    std::vector<cd> g[4], s(V * 12);
    cd *gp[4];
    for (int mu = 0; mu < 4; ++mu) {
        g[mu].resize(V * 9);
        gp[mu] = g[mu].data();
        if (std::fread(gp[mu], 16, V * 9, f) != (size_t)V * 9) return 4;
    }
    if (std::fread(s.data(), 16, V * 12, f) != (size_t)V * 12) return 5;
    std::fclose(f);
    int subgs[4] = {dims[0], dims[1], dims[2], dims[3]};
    lattice_gauge U(gp, subgs, dims);
    lattice_fermion src(s.data(), subgs, dims), out(subgs, dims);
    FILE *o = std::fopen(argv[2], "wb");
    auto put = [&](lattice_fermion &x) { std::fwrite(x.A, 16, x.size, o); };
    for (int dag = 0; dag < 2; ++dag)
        for (int cb = 0; cb < 2; ++cb) {
            DslashoffdNew(src, out, U, dag, cb);
            put(out);
        }
    DslashNew(src, out, U, mass, false);
    put(out);
    DslashNew(src, out, U, mass, true);
    put(out);
    Dslash(src, out, U, mass, false);
    put(out);
    DslashEEOONew(src, out, mass);
    put(out);
    DslashEO(src, out, U, false);
    put(out);
    DslashOE(src, out, U, true);
    put(out);
    DslashEE(src, out, mass);
    put(out);
    DslashOO(src, out, mass);
    put(out);
    lattice_fermion m(subgs, dims);
    DslashNew(src, m, U, mass, false);
    const double n2 = norm_2(src);
    const cd dp = vector_p(src, m);
    std::fwrite(&n2, 8, 1, o);
    std::fwrite(&dp, 16, 1, o);
    std::srand(seed);
    lattice_fermion x(subgs, dims);
    CGinvert(src, x, U, mass, 500, 1e-9);
    put(x);
    // the raw-pointer overload, as a caller holding plain arrays uses it
    std::vector<cd> raw_src(s), raw_x(V * 12);
    int subgs2[4] = {dims[0], dims[1], dims[2], dims[3]}, site_vec2[4] = {dims[0], dims[1], dims[2], dims[3]};
    std::srand(seed);
    CGinvert(raw_src.data(), raw_x.data(), gp, mass, 500, 1e-9, subgs2, site_vec2);
    std::fwrite(raw_x.data(), 16, raw_x.size(), o);
    std::fclose(o);
    return 0;
}
