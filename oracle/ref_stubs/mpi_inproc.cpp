/*
 * Thread-based implementation of the MPI subset declared in mpi.h.
 * TEST INFRASTRUCTURE ONLY (used to run the reference's own code as an oracle).
 *
 * Semantics kept from MPI:
 *  - Send is buffered: it copies the payload and returns.
 *  - Recv takes the oldest queued message that matches (source, tag), with
 *    ANY_SOURCE / ANY_TAG wildcards, so messages from one source never
 *    overtake each other.
 *  - Bcast is collective: every rank calls it in the same order; the root's
 *    buffer is copied to all others, and the root waits until they have it.
 * Every wait is bounded (LEO2D_INPROC_TIMEOUT_S, default 600 s) and aborts the
 * process with a message instead of hanging.
 */
#include "mpi.h"

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <vector>

namespace MPI {
const Datatype INT = {4};
const Datatype DOUBLE = {8};
const Datatype CHAR = {1};
Intracomm COMM_WORLD;
}  // namespace MPI

namespace {

struct Message {
  int source;
  int tag;
  std::vector<char> bytes;
};

struct BcastSlot {
  std::vector<char> bytes;
  bool ready = false;
  int acks = 0;
};

std::mutex g_mu;
std::condition_variable g_cv;
int g_size = 1;
std::map<int, std::deque<Message>> g_queues;  // keyed by destination rank
std::map<int, BcastSlot> g_bcast;             // keyed by collective sequence
thread_local int t_rank = 0;
thread_local int t_bcast_seq = 0;

std::chrono::seconds wait_limit() {
  const char* env = std::getenv("LEO2D_INPROC_TIMEOUT_S");
  long s = env ? std::atol(env) : 600;
  return std::chrono::seconds(s > 0 ? s : 600);
}

template <class Pred>
void wait_or_die(std::unique_lock<std::mutex>& lk, Pred pred, const char* what) {
  if (!g_cv.wait_for(lk, wait_limit(), pred)) {
    std::fprintf(stderr, "mpi_inproc: rank %d timed out in %s\n", t_rank, what);
    std::abort();
  }
}

}  // namespace

void leo2d_inproc_set_rank(int rank, int size) {
  t_rank = rank;
  std::lock_guard<std::mutex> lk(g_mu);
  g_size = size;
}

int MPI_Init(int*, char***) { return 0; }
int MPI_Finalize() { return 0; }

namespace MPI {

int Intracomm::Get_rank() const { return t_rank; }

int Intracomm::Get_size() const {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_size;
}

void Intracomm::Bcast(void* buf, int count, const Datatype& type,
                      int root) const {
  const size_t n = static_cast<size_t>(count) * type.bytes;
  const int seq = t_bcast_seq++;
  std::unique_lock<std::mutex> lk(g_mu);
  if (g_size == 1) return;
  if (t_rank == root) {
    BcastSlot& slot = g_bcast[seq];
    slot.bytes.assign(static_cast<char*>(buf), static_cast<char*>(buf) + n);
    slot.ready = true;
    g_cv.notify_all();
    wait_or_die(lk, [&] { return g_bcast[seq].acks == g_size - 1; }, "Bcast(root)");
    g_bcast.erase(seq);
  } else {
    wait_or_die(lk, [&] { return g_bcast.count(seq) && g_bcast[seq].ready; },
                "Bcast");
    BcastSlot& slot = g_bcast[seq];
    std::memcpy(buf, slot.bytes.data(), n < slot.bytes.size() ? n : slot.bytes.size());
    slot.acks += 1;
    g_cv.notify_all();
  }
}

void Intracomm::Send(const void* buf, int count, const Datatype& type, int dest,
                     int tag) const {
  const size_t n = static_cast<size_t>(count) * type.bytes;
  Message m;
  m.source = t_rank;
  m.tag = tag;
  m.bytes.assign(static_cast<const char*>(buf), static_cast<const char*>(buf) + n);
  std::lock_guard<std::mutex> lk(g_mu);
  g_queues[dest].push_back(std::move(m));
  g_cv.notify_all();
}

void Intracomm::Recv(void* buf, int count, const Datatype& type, int source,
                     int tag, Status& status) const {
  const size_t cap = static_cast<size_t>(count) * type.bytes;
  std::unique_lock<std::mutex> lk(g_mu);
  std::deque<Message>& q = g_queues[t_rank];
  auto match = [&](const Message& m) {
    return (source == ANY_SOURCE || m.source == source) &&
           (tag == ANY_TAG || m.tag == tag);
  };
  std::deque<Message>::iterator it;
  wait_or_die(lk, [&] {
    for (it = q.begin(); it != q.end(); ++it)
      if (match(*it)) return true;
    return false;
  }, "Recv");
  const size_t n = it->bytes.size() < cap ? it->bytes.size() : cap;
  if (n) std::memcpy(buf, it->bytes.data(), n);
  status.source = it->source;
  status.tag = it->tag;
  q.erase(it);
}

void Intracomm::Recv(void* buf, int count, const Datatype& type, int source,
                     int tag) const {
  Status st;
  Recv(buf, count, type, source, tag, st);
}

}  // namespace MPI
