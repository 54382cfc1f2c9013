// lattice_gauge.h -- the reference's gauge container (include/lattice_gauge.h:11-26).
#ifndef LATTICE_LATTICE_GAUGE_H
#define LATTICE_LATTICE_GAUGE_H

#include <complex>

class lattice_gauge {
  public:
    int *site_vec;
    std::complex<double> *A[4];  // per direction: sites x 9 complex (row-major SU(3)), even-odd order
    int *subgs;
    int size;                    // complex entries per direction

    lattice_gauge(std::complex<double> *data[4], int *subgs1, int *site_vec1);  // borrow
    lattice_gauge(int *subgs1, int *site_vec1);                                 // own, zeroed
    ~lattice_gauge();
    lattice_gauge(const lattice_gauge &) = delete;
    lattice_gauge &operator=(const lattice_gauge &) = delete;
    // element (row ll, column mm) of U_dd at global coordinates site[4]
    std::complex<double> peeksite(const int *site, int ll = 0, int mm = 0, int dd = 0);

  private:
    bool mem_flag;
};

#endif
