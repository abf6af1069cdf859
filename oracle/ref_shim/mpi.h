// Stand-in for the MPI rank query used by exaDEM's color_log (single process).
#pragma once
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return 0; }
