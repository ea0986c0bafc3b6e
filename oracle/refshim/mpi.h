/*
 * Single-rank MPI stand-in used only to compile and run the LA3 reference
 * (np=1) as a CPU checker.  Test infrastructure: nothing in the product
 * links it.
 *
 * Semantics at one rank:
 *   - point-to-point messages are matched by tag, FIFO per tag; an Isend
 *     copies its buffer immediately, so the send request is complete at once;
 *   - a receive posted before its send completes when the send arrives;
 *   - a wait on a request that nothing can complete aborts (it would deadlock);
 *   - collectives over one rank are copies.
 * A mutex makes the calls safe under MPI_THREAD_MULTIPLE (the reference sends
 * from inside OpenMP regions).
 */
#ifndef LA3_REFSHIM_MPI_H
#define LA3_REFSHIM_MPI_H

#include <cstddef>

typedef int MPI_Comm;
typedef int MPI_Datatype; /* value = element size in bytes (0 = null type) */
typedef int MPI_Op;
typedef int MPI_Group;
struct la3shim_request;
typedef la3shim_request* MPI_Request;

struct MPI_Status
{
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  long la3shim_nbytes;
};

#define MPI_COMM_WORLD ((MPI_Comm) 0)
#define MPI_REQUEST_NULL ((MPI_Request) 0)
#define MPI_STATUS_IGNORE ((MPI_Status*) 0)
#define MPI_STATUSES_IGNORE ((MPI_Status*) 0)
#define MPI_IN_PLACE ((void*) 1)

#define MPI_DATATYPE_NULL ((MPI_Datatype) 0)
#define MPI_BYTE ((MPI_Datatype) 1)
#define MPI_CHAR ((MPI_Datatype) 1)
#define MPI_INT ((MPI_Datatype) 4)
#define MPI_UNSIGNED ((MPI_Datatype) 4)
#define MPI_UNSIGNED_LONG ((MPI_Datatype) 8)
#define MPI_DOUBLE ((MPI_Datatype) 8)

#define MPI_SUM ((MPI_Op) 1)
#define MPI_LAND ((MPI_Op) 2)

#define MPI_SUCCESS 0
#define MPI_ERR_IN_STATUS 17
#define MPI_UNDEFINED (-32766)
#define MPI_THREAD_MULTIPLE 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)

int MPI_Init_thread(int* argc, char*** argv, int required, int* provided);
int MPI_Finalize();
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_group(MPI_Comm comm, MPI_Group* group);
int MPI_Group_incl(MPI_Group group, int n, const int* ranks, MPI_Group* newgroup);
int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm);
int MPI_Barrier(MPI_Comm comm);

int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Type_free(MPI_Datatype* type);

int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
              MPI_Request* request);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm,
              MPI_Request* request);
int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status);
int MPI_Wait(MPI_Request* request, MPI_Status* status);
int MPI_Waitall(int count, MPI_Request* requests, MPI_Status* statuses);
int MPI_Waitsome(int incount, MPI_Request* requests, int* outcount, int* indices,
                 MPI_Status* statuses);
int MPI_Testsome(int incount, MPI_Request* requests, int* outcount, int* indices,
                 MPI_Status* statuses);
int MPI_Iprobe(int source, int tag, MPI_Comm comm, int* flag, MPI_Status* status);
int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Get_count(const MPI_Status* status, MPI_Datatype type, int* count);

int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
               int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Iallreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op,
                   MPI_Comm comm, MPI_Request* request);

#endif
