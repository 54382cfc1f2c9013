// wilson_main.cpp -- command-line driver with the reference's interface
// (src/main.cpp:17-123):  wilson_main Mass gaugefile Lx Ly Lz Lt sx sy sz st [seed]
// Uniform [0,1) complex source from srand(seed) (one rank: rank 0), gauge from
// load_gauge ("UNIT", "RANDOM" or a file), CG on M^dag M x = M^dag b with
// at most 500 iterations to |r| < 1e-9, timing lines, then the check report.
// Everything after argument parsing runs on the GPU.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>
#include "check.h"
#include "invert.h"
#include "load_gauge.h"

int main(int argc, char **argv)
{
    int site_vec[4] = {8, 8, 8, 8}, subgs[4] = {8, 8, 8, 8};
    double mass = 0.05;
    std::string filename = "UNIT";
    int seed = 0;
    if (argc == 11 || argc == 12) {
        mass = std::stod(argv[1]);
        filename = argv[2];
        for (int i = 0; i < 4; ++i) {
            site_vec[i] = std::stoi(argv[3 + i]);
            subgs[i] = std::stoi(argv[7 + i]);
        }
        if (argc == 12) seed = std::atoi(argv[11]);
    } else if (argc != 1) {
        std::cerr << "wilson_main Mass gaugefile  lattice_size   subgrid_size [seed]" << std::endl;
        std::cerr << "Example: wilson_main 0.005 RANDOM  24 24 24 48  24 24 24 48" << std::endl;
        return 1;
    }
    const int max_cg = 500;
    const double accuracy = 1.0e-9;
    long vsub = 1;
    for (int i = 0; i < 4; ++i) {
        if (site_vec[i] != subgs[i]) {
            std::cerr << "Lattice partition size must be 1 on one GPU (subgrid == lattice)" << std::endl;
            return 1;
        }
        vsub *= subgs[i];
    }
    std::cout << "  Mass  " << mass << std::endl;
    std::cout << "  gauge file  " << filename << std::endl;
    std::printf("  lattice size  %d %d %d %d\n", site_vec[0], site_vec[1], site_vec[2], site_vec[3]);
    std::printf("  subgrid size  %d %d %d %d\n", subgs[0], subgs[1], subgs[2], subgs[3]);

    std::srand(seed);  // rank 0 of one
    std::vector<double> source((size_t)vsub * 24);
    for (double &v : source) v = (double)std::rand() / RAND_MAX;

    const auto t0 = std::chrono::steady_clock::now();
    lattice_fermion src(subgs, site_vec);
    for (long i = 0; i < vsub * 12; ++i) src.A[i] = std::complex<double>(source[2 * i], source[2 * i + 1]);
    lattice_gauge U(subgs, site_vec);
    load_gauge(U.A, filename, subgs, site_vec);
    const auto t1 = std::chrono::steady_clock::now();
    lattice_fermion dest(subgs, site_vec);
    CGinvert(src, dest, U, mass, max_cg, accuracy);
    const auto t2 = std::chrono::steady_clock::now();
    auto sec = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count(); };
    std::cout << "Source and Gauge, time: " << sec(t0, t1) << std::endl;
    std::cout << "CG invert, time: " << sec(t1, t2) << std::endl;
    std::cout << "Total time: " << sec(t0, t2) << std::endl;
    std::cout << "Result checking ..." << std::endl;
    std::cout << " [ Accuracy = " << accuracy << " ]" << std::endl;
    check(src, dest, U, mass);
    return 0;
}
