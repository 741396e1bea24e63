/*
 * Single-process stand-in for the handful of MPI calls the TD-BEM reference
 * makes (main.cpp:28-29, SolverT.cpp:29-30, SolverT.cpp:698,731).
 *
 * Test infrastructure only: this lets the reference's own sources compile and
 * run as one rank so that their outputs can pin the oracle.  Nothing in the
 * product links it.
 */
#ifndef TDBEM_REF_SHIM_MPI_H
#define TDBEM_REF_SHIM_MPI_H

typedef int MPI_Comm;

#ifdef __cplusplus
extern "C" {
#endif

int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Barrier(MPI_Comm comm);

#ifdef __cplusplus
}
#endif

#endif
