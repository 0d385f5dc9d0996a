// Implementation of the single-rank MPI shim (see mpi.h).  Test
// infrastructure: it lets the reference's unmodified src/WENOFD.cpp build and
// run as one rank, so its outputs can pin the oracle.
#include "mpi.h"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_CHAR: return 1;
    case MPI_OFFSET: return sizeof(MPI_Offset);
  }
  throw std::runtime_error("mpi shim: unknown datatype");
}

struct PendingRecv {
  void *buf;
  size_t bytes;
  int tag;
  bool open;
};

std::vector<PendingRecv> &pending() {
  static std::vector<PendingRecv> p;
  return p;
}

}  // namespace

struct wenofd_shim_file {
  FILE *f;
};

extern "C" {

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }

double MPI_Wtime(void) {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

int MPI_Abort(MPI_Comm, int code) {
  throw std::runtime_error("MPI_Abort called with code " + std::to_string(code));
}

int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int, MPI_Datatype,
                  MPI_Comm) {
  std::memmove(rbuf, sbuf, scount * type_size(stype));
  return MPI_SUCCESS;
}

int MPI_Reduce(const void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op, int, MPI_Comm) {
  std::memmove(rbuf, sbuf, count * type_size(type));
  return MPI_SUCCESS;
}

int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op, MPI_Comm) {
  std::memmove(rbuf, sbuf, count * type_size(type));
  return MPI_SUCCESS;
}

int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

// Rank 0's exclusive-scan result is undefined in MPI; the reference resets it
// (src/WENOFD.cpp:1206), so leaving the buffer untouched is faithful.
int MPI_Exscan(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int, int tag, MPI_Comm, MPI_Request *req) {
  pending().push_back({buf, count * type_size(type), tag, true});
  *req = static_cast<int>(pending().size()) - 1;
  return MPI_SUCCESS;
}

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int, int tag, MPI_Comm,
              MPI_Request *req) {
  const size_t bytes = count * type_size(type);
  for (auto &p : pending()) {
    if (p.open && p.tag == tag) {
      if (p.bytes < bytes) throw std::runtime_error("mpi shim: receive buffer too small");
      std::memcpy(p.buf, buf, bytes);
      p.open = false;
      *req = -1;
      return MPI_SUCCESS;
    }
  }
  throw std::runtime_error("mpi shim: self-send with no matching receive posted");
}

int MPI_Waitall(int, MPI_Request *, MPI_Status *) {
  for (const auto &p : pending())
    if (p.open) throw std::runtime_error("mpi shim: receive never matched");
  pending().clear();
  return MPI_SUCCESS;
}

int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  throw std::runtime_error("mpi shim: blocking receive on a single rank");
}

int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  throw std::runtime_error("mpi shim: blocking send on a single rank");
}

int MPI_File_open(MPI_Comm, const char *name, int, MPI_Info, MPI_File *fh) {
  FILE *f = std::fopen(name, "w+b");
  if (!f) throw std::runtime_error(std::string("mpi shim: cannot open ") + name);
  *fh = new wenofd_shim_file{f};
  return MPI_SUCCESS;
}

int MPI_File_set_size(MPI_File, MPI_Offset) { return MPI_SUCCESS; }

int MPI_File_write_at(MPI_File fh, MPI_Offset offset, const void *buf, int count, MPI_Datatype type,
                      MPI_Status *) {
  std::fseek(fh->f, static_cast<long>(offset), SEEK_SET);
  std::fwrite(buf, type_size(type), count, fh->f);
  return MPI_SUCCESS;
}

int MPI_File_close(MPI_File *fh) {
  std::fclose((*fh)->f);
  delete *fh;
  *fh = nullptr;
  return MPI_SUCCESS;
}

}  // extern "C"
