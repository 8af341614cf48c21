/* Minimal single-process MPI surface for building the reference CSEM solver as a
 * CPU oracle. The reference uses MPI only for Init/rank/size/Wtime/Finalize
 * (main.c:54-56,103,119,142); this header maps those to a one-rank world. */
#ifndef CSEM_ORACLE_MPI_STUB_H
#define CSEM_ORACLE_MPI_STUB_H
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
int MPI_Init(int *argc, char ***argv);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
double MPI_Wtime(void);
int MPI_Finalize(void);
#endif
