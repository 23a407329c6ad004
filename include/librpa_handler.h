#pragma once
/*
 * Handler management (replaces LibRPA include/librpa_handler.h:25-57).
 */
#include <mpi.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque handle; same layout as LibRPA (one const int instance id). */
typedef struct
{
    const int instance_id_;
} LibrpaHandler;

/* librpa_handler.h:45 -- create a handler bound to a communicator (single rank here). */
LibrpaHandler* librpa_create_handler(MPI_Comm comm);

/* librpa_handler.h:57 -- free the handler and every host/device buffer it owns. NULL is a no-op. */
void librpa_destroy_handler(LibrpaHandler *h);

#ifdef __cplusplus
}
#endif
