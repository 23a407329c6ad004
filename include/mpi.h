#pragma once
/*
 * Single-rank stand-in for <mpi.h>.
 *
 * The LibRPA public header librpa_handler.h includes <mpi.h> because
 * librpa_create_handler takes an MPI communicator.  This GB300 build runs one
 * process per GPU and never calls MPI, so when no MPI implementation is on the
 * include path this header supplies the one type and constant the API names.
 * A caller that has a real MPI puts its own <mpi.h> first on the include path;
 * the communicator argument is then accepted and ignored (it travels in an
 * integer register either way, int- or pointer-typed).
 */
#ifndef LIBRPA_GB300_MPI_SHIM
#define LIBRPA_GB300_MPI_SHIM
typedef int MPI_Comm;
#ifndef MPI_COMM_WORLD
#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
#endif
#endif
