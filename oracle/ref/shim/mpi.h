/*
 * Test-only, single-rank stand-in for the MPI calls the KnightKing headers make.
 *
 * Oracle infrastructure: it lets the reference's own include/*.hpp and
 * src/apps/*.hpp compile and run as one process so that their paths can be
 * compared with this project's kernels.  It is never linked into the product.
 *
 * Semantics (rank 0 of a world of size 1):
 *   - MPI_Send / MPI_Isend copy the message into a per-tag FIFO mailbox and
 *     return at once (buffered send; the request completes immediately).
 *   - MPI_Probe / MPI_Recv / MPI_Irecv block until the tag's mailbox has a
 *     message.  The reference runs its send and receive threads concurrently
 *     (include/graph.hpp:733-855, include/path.hpp:282-325), so the mailbox is
 *     guarded by a mutex and a condition variable.
 *   - MPI_Allreduce with one rank is a copy; MPI_Barrier / MPI_Bcast are no-ops.
 * A datatype is its element size in bytes (see gemini/core/mpi.hpp).
 */
#pragma once

#include <stddef.h>
#include <string.h>

#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <vector>

typedef size_t MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Op;

struct MPI_Status
{
    size_t bytes;
    int MPI_SOURCE;
    int MPI_TAG;
};

struct MPI_Request
{
    int done;
};

#define MPI_COMM_WORLD 0
#define MPI_SUM 1
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

namespace kk_mpi_shim
{
struct Mailbox
{
    std::mutex lock;
    std::condition_variable cv;
    std::map<int, std::deque<std::vector<char> > > queues;
};

inline Mailbox &mailbox()
{
    static Mailbox box;
    return box;
}

inline void post(const void *buf, size_t bytes, int tag)
{
    Mailbox &box = mailbox();
    std::vector<char> msg(bytes);
    if (bytes != 0)
    {
        memcpy(msg.data(), buf, bytes);
    }
    {
        std::lock_guard<std::mutex> g(box.lock);
        box.queues[tag].push_back(std::move(msg));
    }
    box.cv.notify_all();
}

inline size_t peek(int tag)
{
    Mailbox &box = mailbox();
    std::unique_lock<std::mutex> g(box.lock);
    box.cv.wait(g, [&] { return !box.queues[tag].empty(); });
    return box.queues[tag].front().size();
}

inline size_t take(void *buf, size_t capacity, int tag)
{
    Mailbox &box = mailbox();
    std::unique_lock<std::mutex> g(box.lock);
    box.cv.wait(g, [&] { return !box.queues[tag].empty(); });
    std::vector<char> msg = std::move(box.queues[tag].front());
    box.queues[tag].pop_front();
    g.unlock();
    size_t n = msg.size() < capacity ? msg.size() : capacity;
    if (n != 0)
    {
        memcpy(buf, msg.data(), n);
    }
    return msg.size();
}
} // namespace kk_mpi_shim

inline int MPI_Comm_rank(MPI_Comm, int *rank)
{
    *rank = 0;
    return MPI_SUCCESS;
}

inline int MPI_Comm_size(MPI_Comm, int *size)
{
    *size = 1;
    return MPI_SUCCESS;
}

inline int MPI_Send(const void *buf, int count, MPI_Datatype type, int, int tag, MPI_Comm)
{
    kk_mpi_shim::post(buf, (size_t)count * type, tag);
    return MPI_SUCCESS;
}

inline int MPI_Isend(const void *buf, int count, MPI_Datatype type, int, int tag, MPI_Comm, MPI_Request *req)
{
    kk_mpi_shim::post(buf, (size_t)count * type, tag);
    req->done = 1;
    return MPI_SUCCESS;
}

inline int MPI_Probe(int src, int tag, MPI_Comm, MPI_Status *status)
{
    size_t bytes = kk_mpi_shim::peek(tag);
    if (status != MPI_STATUS_IGNORE)
    {
        status->bytes = bytes;
        status->MPI_SOURCE = src;
        status->MPI_TAG = tag;
    }
    return MPI_SUCCESS;
}

inline int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count)
{
    *count = (int)(status->bytes / type);
    return MPI_SUCCESS;
}

inline int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm, MPI_Status *status)
{
    size_t bytes = kk_mpi_shim::take(buf, (size_t)count * type, tag);
    if (status != MPI_STATUS_IGNORE)
    {
        status->bytes = bytes;
        status->MPI_SOURCE = src;
        status->MPI_TAG = tag;
    }
    return MPI_SUCCESS;
}

inline int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Request *req)
{
    MPI_Recv(buf, count, type, src, tag, comm, MPI_STATUS_IGNORE);
    req->done = 1;
    return MPI_SUCCESS;
}

inline int MPI_Wait(MPI_Request *, MPI_Status *)
{
    return MPI_SUCCESS;
}

inline int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op, MPI_Comm)
{
    if (send != recv)
    {
        memmove(recv, send, (size_t)count * type);
    }
    return MPI_SUCCESS;
}

inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm)
{
    return MPI_SUCCESS;
}

inline int MPI_Barrier(MPI_Comm)
{
    return MPI_SUCCESS;
}
