/*
 * In-process stand-in for the MPI C++ bindings used by LEO2D.
 *
 * TEST INFRASTRUCTURE ONLY. This header lets the reference's own sources
 * (src/locality.cpp, src/params/job_params.cpp, src/mpi/mat_comm.cpp) compile
 * in a container without an MPI installation. Ranks are threads of one
 * process (see mpi_inproc.cpp): every thread runs the reference's main(), and
 * Send/Recv/Bcast move bytes between them through mutex-protected queues with
 * MPI's ordering rules (non-overtaking per source, ANY_SOURCE/ANY_TAG
 * wildcards, buffered sends).
 *
 * Only the calls LEO2D makes are provided (grep of the reference tree:
 * COMM_WORLD.{Bcast,Send,Recv,Get_rank,Get_size}, Status.{Get_source,Get_tag},
 * the INT/DOUBLE/CHAR datatypes, MPI_Init, MPI_Finalize).
 */
#ifndef LEO2D_ORACLE_MPI_STUB_H
#define LEO2D_ORACLE_MPI_STUB_H

#include <cstddef>

namespace MPI {

struct Datatype {
  int bytes;
};

extern const Datatype INT;
extern const Datatype DOUBLE;
extern const Datatype CHAR;

const int ANY_SOURCE = -1;
const int ANY_TAG = -1;

class Status {
 public:
  int source = -1;
  int tag = -1;
  int Get_source() const { return source; }
  int Get_tag() const { return tag; }
};

class Intracomm {
 public:
  int Get_rank() const;
  int Get_size() const;
  void Bcast(void* buf, int count, const Datatype& type, int root) const;
  void Send(const void* buf, int count, const Datatype& type, int dest,
            int tag) const;
  void Recv(void* buf, int count, const Datatype& type, int source, int tag,
            Status& status) const;
  void Recv(void* buf, int count, const Datatype& type, int source,
            int tag) const;
};

extern Intracomm COMM_WORLD;

}  // namespace MPI

#define MPI_INT MPI::INT
#define MPI_DOUBLE MPI::DOUBLE
#define MPI_CHAR MPI::CHAR

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize();

/* Number of in-process ranks and the calling thread's rank. */
void leo2d_inproc_set_rank(int rank, int size);

#endif
