/* TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * The few MPI declarations the reference's layout/comms sources name, so that
 * their -DMPI branch compiles without an MPI library.  mpi_layout.c calls only
 * the layout functions that send no message (make_slices, sitemap,
 * set_parity, paritymap); the functions below exist for the linker and
 * report an error if anything calls them. */
#ifndef ORC_MPI_STUB_H
#define ORC_MPI_STUB_H

typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_REQUEST_NULL 0
#define MPI_UNDEFINED (-32766)
#define MPI_DOUBLE 1
#define MPI_LONG 2
#define MPI_INT 3
#define MPI_INTEGER 3
#define MPI_CHAR 4
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm c, int* r);
int MPI_Comm_size(MPI_Comm c, int* s);
int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out);
int MPI_Barrier(MPI_Comm c);
int MPI_Send(const void* b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c);
int MPI_Recv(void* b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* s);
int MPI_Isend(const void* b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request* r);
int MPI_Irecv(void* b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request* r);
int MPI_Wait(MPI_Request* r, MPI_Status* s);
int MPI_Waitall(int n, MPI_Request* r, MPI_Status* s);
int MPI_Probe(int src, int tag, MPI_Comm c, MPI_Status* s);
int MPI_Get_count(const MPI_Status* s, MPI_Datatype t, int* n);
int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c);
int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Abort(MPI_Comm c, int code);
double MPI_Wtime(void);

#endif
