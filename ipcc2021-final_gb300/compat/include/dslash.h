// dslash.h -- the reference's scalar operator API (include/dslash.h:16-21), on the GPU.
#ifndef LATTICE_DSLASH_H
#define LATTICE_DSLASH_H

#include "lattice_fermion.h"
#include "lattice_gauge.h"
#include "operator.h"
#include "operator_mpi.h"

void DslashEE(lattice_fermion &src, lattice_fermion &dest, const double mass);  // even half: (4+m) src
void DslashOO(lattice_fermion &src, lattice_fermion &dest, const double mass);  // odd half:  (4+m) src
void DslashEO(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag);  // = Dslashoffd cb 0
void DslashOE(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag);  // = Dslashoffd cb 1
void Dslashoffd(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag, int cb);
#endif
