/*
 * Single-rank MPI stand-in (implementation).  Test infrastructure for the
 * reference CPU build only; see mpi.h for the semantics.
 */
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <vector>

struct la3shim_request
{
  bool complete = false;
  void* recv_buf = nullptr;  // pending receive target
  long recv_cap = 0;         // receive capacity in bytes
  int tag = 0;
  long nbytes = 0;           // bytes delivered
};

namespace
{
std::recursive_mutex mu;
std::map<int, std::deque<std::vector<char>>> queued;  // tag -> FIFO of unmatched sends
std::list<la3shim_request*> pending;                   // receives waiting for a send

[[noreturn]] void deadlock(const char* where)
{
  std::fprintf(stderr, "la3 refshim: %s would wait forever at one rank\n", where);
  std::abort();
}

void fill_status(MPI_Status* st, const la3shim_request* r)
{
  if (st == MPI_STATUS_IGNORE) return;
  st->MPI_SOURCE = 0;
  st->MPI_TAG = r->tag;
  st->MPI_ERROR = MPI_SUCCESS;
  st->la3shim_nbytes = r->nbytes;
}

void deliver(la3shim_request* r, const char* data, long nbytes)
{
  long n = nbytes < r->recv_cap ? nbytes : r->recv_cap;
  if (n > 0) std::memcpy(r->recv_buf, data, (size_t) n);
  r->nbytes = n;
  r->complete = true;
}
}  // namespace

int MPI_Init_thread(int*, char***, int, int* provided)
{
  *provided = MPI_THREAD_MULTIPLE;
  return MPI_SUCCESS;
}
int MPI_Finalize() { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_group(MPI_Comm, MPI_Group* g) { *g = 0; return MPI_SUCCESS; }
int MPI_Group_incl(MPI_Group, int, const int*, MPI_Group* g) { *g = 0; return MPI_SUCCESS; }
int MPI_Comm_create(MPI_Comm, MPI_Group, MPI_Comm* c) { *c = MPI_COMM_WORLD; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* t)
{
  *t = count * old;
  return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype* t) { *t = MPI_DATATYPE_NULL; return MPI_SUCCESS; }

int MPI_Isend(const void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request* request)
{
  std::lock_guard<std::recursive_mutex> lock(mu);
  long nbytes = (long) count * type;
  for (auto it = pending.begin(); it != pending.end(); ++it)
  {
    if ((*it)->tag == tag)
    {
      deliver(*it, (const char*) buf, nbytes);
      pending.erase(it);
      nbytes = -1;
      break;
    }
  }
  if (nbytes >= 0)
    queued[tag].emplace_back((const char*) buf, (const char*) buf + nbytes);
  auto* r = new la3shim_request;
  r->complete = true;
  r->tag = tag;
  *request = r;
  return MPI_SUCCESS;
}

int MPI_Irecv(void* buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request* request)
{
  std::lock_guard<std::recursive_mutex> lock(mu);
  auto* r = new la3shim_request;
  r->recv_buf = buf;
  r->recv_cap = (long) count * type;
  r->tag = tag;
  auto q = queued.find(tag);
  if (q != queued.end() && !q->second.empty())
  {
    deliver(r, q->second.front().data(), (long) q->second.front().size());
    q->second.pop_front();
  }
  else
  {
    pending.push_back(r);
  }
  *request = r;
  return MPI_SUCCESS;
}

int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int, int, void* recvbuf,
                 int recvcount, MPI_Datatype recvtype, int, int recvtag, MPI_Comm,
                 MPI_Status* status)
{
  long n = (long) sendcount * sendtype;
  long cap = (long) recvcount * recvtype;
  if (n > cap) n = cap;
  std::memmove(recvbuf, sendbuf, (size_t) n);
  if (status != MPI_STATUS_IGNORE)
  {
    status->MPI_SOURCE = 0;
    status->MPI_TAG = recvtag;
    status->MPI_ERROR = MPI_SUCCESS;
    status->la3shim_nbytes = n;
  }
  return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request* request, MPI_Status* status)
{
  std::lock_guard<std::recursive_mutex> lock(mu);
  if (*request == MPI_REQUEST_NULL) return MPI_SUCCESS;
  if (!(*request)->complete) deadlock("MPI_Wait");
  fill_status(status, *request);
  delete *request;
  *request = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

int MPI_Waitall(int count, MPI_Request* requests, MPI_Status* statuses)
{
  for (int i = 0; i < count; i++)
    MPI_Wait(&requests[i], statuses == MPI_STATUSES_IGNORE ? MPI_STATUS_IGNORE : &statuses[i]);
  return MPI_SUCCESS;
}

static int some(int incount, MPI_Request* requests, int* outcount, int* indices,
                MPI_Status* statuses, bool must_progress)
{
  std::lock_guard<std::recursive_mutex> lock(mu);
  int active = 0, done = 0;
  for (int i = 0; i < incount; i++)
  {
    if (requests[i] == MPI_REQUEST_NULL) continue;
    active++;
    if (requests[i]->complete)
    {
      if (statuses != MPI_STATUSES_IGNORE) fill_status(&statuses[done], requests[i]);
      indices[done++] = i;
      delete requests[i];
      requests[i] = MPI_REQUEST_NULL;
    }
  }
  if (active == 0)
  {
    *outcount = MPI_UNDEFINED;
    return MPI_SUCCESS;
  }
  if (done == 0 && must_progress) deadlock("MPI_Waitsome");
  *outcount = done;
  return MPI_SUCCESS;
}

int MPI_Waitsome(int incount, MPI_Request* requests, int* outcount, int* indices,
                 MPI_Status* statuses)
{
  return some(incount, requests, outcount, indices, statuses, true);
}

int MPI_Testsome(int incount, MPI_Request* requests, int* outcount, int* indices,
                 MPI_Status* statuses)
{
  return some(incount, requests, outcount, indices, statuses, false);
}

int MPI_Iprobe(int, int tag, MPI_Comm, int* flag, MPI_Status* status)
{
  std::lock_guard<std::recursive_mutex> lock(mu);
  auto q = queued.find(tag);
  *flag = (q != queued.end() && !q->second.empty()) ? 1 : 0;
  if (*flag && status != MPI_STATUS_IGNORE)
  {
    status->MPI_SOURCE = 0;
    status->MPI_TAG = tag;
    status->MPI_ERROR = MPI_SUCCESS;
    status->la3shim_nbytes = (long) q->second.front().size();
  }
  return MPI_SUCCESS;
}

int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* status)
{
  int flag = 0;
  MPI_Iprobe(source, tag, comm, &flag, status);
  if (!flag) deadlock("MPI_Probe");
  return MPI_SUCCESS;
}

int MPI_Get_count(const MPI_Status* status, MPI_Datatype type, int* count)
{
  *count = (int) (status->la3shim_nbytes / (type > 0 ? type : 1));
  return MPI_SUCCESS;
}

int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int,
               MPI_Datatype, int, MPI_Comm)
{
  if (sendbuf != MPI_IN_PLACE && sendbuf != recvbuf)
    std::memmove(recvbuf, sendbuf, (size_t) sendcount * sendtype);
  return MPI_SUCCESS;
}

int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op,
                  MPI_Comm)
{
  if (sendbuf != MPI_IN_PLACE && sendbuf != recvbuf)
    std::memmove(recvbuf, sendbuf, (size_t) count * type);
  return MPI_SUCCESS;
}

int MPI_Iallreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op,
                   MPI_Comm comm, MPI_Request* request)
{
  MPI_Allreduce(sendbuf, recvbuf, count, type, op, comm);
  auto* r = new la3shim_request;
  r->complete = true;
  *request = r;
  return MPI_SUCCESS;
}
