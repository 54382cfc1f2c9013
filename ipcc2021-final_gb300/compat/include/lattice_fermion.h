// lattice_fermion.h -- the reference's fermion container (include/lattice_fermion.h:12-35),
// backed by host memory exactly as there; the operators that take it run on the GPU.
#ifndef LATTICE_LATTICE_FERMION_H
#define LATTICE_LATTICE_FERMION_H

#include <complex>

class lattice_fermion {
  public:
    int *site_vec;            // global extents {Lx, Ly, Lz, Lt} (not copied)
    std::complex<double> *A;  // subgs[0..3] sites x 12 complex, even-odd order
    int *subgs;               // local extents; this library runs one lattice per GPU: subgs == site_vec
    int size;                 // number of complex entries

    // borrow caller memory (not freed)
    lattice_fermion(std::complex<double> *data, int *subgs1, int *site_vec1);
    // own 64-byte aligned, zero-initialised memory
    lattice_fermion(int *subgs1, int *site_vec1);
    ~lattice_fermion();
    lattice_fermion(const lattice_fermion &) = delete;
    lattice_fermion &operator=(const lattice_fermion &) = delete;

    lattice_fermion &operator-(const lattice_fermion &a);  // in place: this -= a
    lattice_fermion &operator+(const lattice_fermion &a);  // in place: this += a
    void operator+=(const lattice_fermion &a);
    void clean();

  private:
    bool mem_flag;
};

void Minus(lattice_fermion &src1, lattice_fermion &src2, lattice_fermion &a);  // a = src1 - src2
void Plus(lattice_fermion &src1, lattice_fermion &src2, lattice_fermion &a);   // a = src1 + src2

#endif
