// Test stand-in for <mpi.h>: the two names eQ's src/eQ.h uses (MPI_Comm in
// eQ::diffusionSolver::params, MPI_Wtime in simulationTiming).  Test infrastructure.
#pragma once
typedef int MPI_Comm;
inline double MPI_Wtime() { return 0.0; }
