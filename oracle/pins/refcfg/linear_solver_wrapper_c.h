// Prototype of the SWMF GMRES the reference calls (share/Library, absent from
// the reference tree); never called by the pinned functions.
#pragma once
#include "mpi.h"
extern "C" void linear_solver_wrapper(const char*, double*, int*, int*, int*, int*, int*, int*, int*, MPI_Fint*, double*, double*, double*, double*, int*);
extern void (*linear_solver_matvec_c)(double*, double*, int);
