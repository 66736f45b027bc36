/* TEST INFRASTRUCTURE (oracle).  Declarations used by the reference's
 * processor_grid.c (fields from processor_grid.c:7-12 and :49-58); the
 * reference ships no processor_grid.h. */
#ifndef ORACLE_SHIM_PROCESSOR_GRID_H
#define ORACLE_SHIM_PROCESSOR_GRID_H
#include <mpi.h>
struct grid_result {
  int ndim;
  int *length;
  int procs;
  int load;
  double asym;
};
typedef struct grid_result *GridResult;
int *makeProcessorGrid(MPI_Comm comm, int ndim, int tasks[]);
#endif
