// dslash_new.h -- the reference's optimised operator API (include/dslash_new.h:18-22), on the GPU.
#ifndef LATTICE_DSLASH_NEW_H
#define LATTICE_DSLASH_NEW_H

#include "lattice_fermion.h"
#include "lattice_gauge.h"
#include "operator.h"
#include "operator_mpi.h"

void DslashEEOONew(lattice_fermion &src, lattice_fermion &dest, const double mass);
void DslashEONew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag);
void DslashOENew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag);
void DslashoffdNew(lattice_fermion &src, lattice_fermion &dest, lattice_gauge &U, const bool dag, int cb);
#endif
