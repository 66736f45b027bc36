/* TEST INFRASTRUCTURE (oracle).  Declarations the reference's logger.c
 * defines (logger.c:6-26); the reference ships no logger.h. */
#ifndef ORACLE_SHIM_LOGGER_H
#define ORACLE_SHIM_LOGGER_H
#include <mpi.h>
void logger(MPI_Comm comm, char *msg, ...);
void fragment_logger(char *msg, ...);
#endif
