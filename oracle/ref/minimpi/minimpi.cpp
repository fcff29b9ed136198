// A minimal MPI over fork + socketpair, for running the reference prover's
// unmodified multi-rank code with N processes on one host.
//
// Test infrastructure only (the product never links it): it produces the
// N-party reference transcripts that pin the one-device party-shares path.
//
// World: MPI_Init in the launched process reads the world size from the
// environment variable MINIMPI_NP (default 1), opens one stream socketpair
// per pair of ranks and forks ranks 1..N-1; the launched process is rank 0
// and, in MPI_Finalize, waits for the others and exits non-zero if any of
// them failed.
//
// Point-to-point: sends are eager (the payload is copied into the peer's
// outgoing queue and the send completes at once), receives are matched in
// posting order against (source, tag) with MPI_ANY_SOURCE / MPI_ANY_TAG, and
// messages between two ranks are delivered in the order sent, as MPI
// requires.  Every blocking call drives one progress loop that writes the
// outgoing queues and reads every socket, so two ranks that both send large
// messages before receiving cannot deadlock.  Collectives run on their own
// context so they never match user messages.  A wait that makes no progress
// for MINIMPI_TIMEOUT seconds (default 600), or that waits on a rank that
// has exited, aborts the process with a message instead of hanging.
#include "mpi.h"

#include <cerrno>
#include <csignal>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <deque>
#include <fcntl.h>
#include <poll.h>
#include <sys/socket.h>
#include <sys/wait.h>
#include <unistd.h>
#include <vector>

namespace {

struct Header {
  int32_t tag;
  int32_t ctx;  // 0: user messages, 1: collectives
  uint64_t len;
};

struct Message {
  int src, tag, ctx;
  std::vector<char> data;
};

struct Peer {
  int fd = -1;
  bool closed = false;
  std::deque<std::vector<char>> out;  // framed messages not yet written
  size_t out_off = 0;                 // bytes of out.front() already written
  Header hdr{};
  size_t hdr_got = 0;
  std::vector<char> body;
  size_t body_got = 0;
};

struct Request {
  bool used = false;
  bool done = false;
  bool is_recv = false;
  void *buf = nullptr;
  size_t cap = 0;
  int src = 0, tag = 0, ctx = 0;
  MPI_Status st{};
  std::vector<int> parts;  // a composite request (Ialltoall) waits on these
};

int g_rank = 0, g_size = 1;
bool g_init = false;
std::vector<Peer> g_peers;
std::vector<pid_t> g_children;
std::deque<Message> g_unexpected;
std::vector<int> g_posted;  // receive requests not yet matched, in posting order
std::vector<Request> g_reqs;
double g_timeout = 600.0;

[[noreturn]] void die(const char *what) {
  std::fprintf(stderr, "minimpi rank %d: %s\n", g_rank, what);
  std::fflush(stderr);
  _exit(70);
}

double now() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_UINT64_T:
    case MPI_DOUBLE:
    case MPI_UNSIGNED_LONG_LONG:
      return 8;
    case MPI_INT:
    case MPI_UINT32_T:
      return 4;
    case MPI_UINT8_T:
    case MPI_BYTE:
    case MPI_CHAR:
      return 1;
    default:
      die("unknown datatype");
  }
}

int new_request() {
  for (size_t i = 0; i < g_reqs.size(); i++)
    if (!g_reqs[i].used) {
      g_reqs[i] = Request();
      g_reqs[i].used = true;
      return (int)i;
    }
  g_reqs.emplace_back();
  g_reqs.back().used = true;
  return (int)g_reqs.size() - 1;
}

bool matches(const Request &r, int src, int tag, int ctx) {
  return r.ctx == ctx && (r.src == MPI_ANY_SOURCE || r.src == src) && (r.tag == MPI_ANY_TAG || r.tag == tag);
}

void complete_recv(Request &r, int src, int tag, const std::vector<char> &data) {
  if (data.size() > r.cap) die("message longer than the receive buffer");
  if (!data.empty()) std::memcpy(r.buf, data.data(), data.size());
  r.done = true;
  r.st.MPI_SOURCE = src;
  r.st.MPI_TAG = tag;
  r.st.MPI_ERROR = MPI_SUCCESS;
  r.st.bytes_ = data.size();
}

// A whole message has arrived: hand it to the first posted receive that
// matches, or keep it for a later receive.
void deliver(int src, int tag, int ctx, std::vector<char> &&data) {
  for (size_t i = 0; i < g_posted.size(); i++) {
    Request &r = g_reqs[g_posted[i]];
    if (matches(r, src, tag, ctx)) {
      complete_recv(r, src, tag, data);
      g_posted.erase(g_posted.begin() + i);
      return;
    }
  }
  g_unexpected.push_back(Message{src, tag, ctx, std::move(data)});
}

// One round of progress: write what the sockets accept, read what they hold.
// Returns true if any byte moved.
bool progress(int wait_ms) {
  std::vector<pollfd> fds;
  std::vector<int> who;
  for (int p = 0; p < g_size; p++) {
    Peer &pe = g_peers[p];
    if (p == g_rank || pe.fd < 0) continue;
    short ev = 0;
    if (!pe.closed) ev |= POLLIN;
    if (!pe.out.empty()) ev |= POLLOUT;
    if (!ev) continue;
    fds.push_back(pollfd{pe.fd, ev, 0});
    who.push_back(p);
  }
  if (fds.empty()) return false;
  int n = poll(fds.data(), fds.size(), wait_ms);
  if (n < 0) {
    if (errno == EINTR) return false;
    die("poll failed");
  }
  bool moved = false;
  for (size_t i = 0; i < fds.size(); i++) {
    Peer &pe = g_peers[who[i]];
    if (fds[i].revents & POLLOUT) {
      while (!pe.out.empty()) {
        std::vector<char> &m = pe.out.front();
        ssize_t w = send(pe.fd, m.data() + pe.out_off, m.size() - pe.out_off, MSG_NOSIGNAL);
        if (w < 0) {
          if (errno == EAGAIN || errno == EWOULDBLOCK || errno == EINTR) break;
          die("send to a peer failed");
        }
        moved = moved || w > 0;
        pe.out_off += (size_t)w;
        if (pe.out_off == m.size()) {
          pe.out.pop_front();
          pe.out_off = 0;
        }
      }
    }
    if (fds[i].revents & (POLLIN | POLLHUP | POLLERR)) {
      for (;;) {
        char *dst;
        size_t want;
        if (pe.hdr_got < sizeof(Header)) {
          dst = (char *)&pe.hdr + pe.hdr_got;
          want = sizeof(Header) - pe.hdr_got;
        } else {
          dst = pe.body.data() + pe.body_got;
          want = pe.body.size() - pe.body_got;
        }
        ssize_t r = want ? recv(pe.fd, dst, want, 0) : 0;
        if (want && r < 0) {
          if (errno == EAGAIN || errno == EWOULDBLOCK || errno == EINTR) break;
          die("recv from a peer failed");
        }
        if (want && r == 0) {
          pe.closed = true;
          break;
        }
        moved = true;
        if (pe.hdr_got < sizeof(Header)) {
          pe.hdr_got += (size_t)r;
          if (pe.hdr_got == sizeof(Header)) {
            pe.body.assign(pe.hdr.len, 0);
            pe.body_got = 0;
          }
        } else {
          pe.body_got += (size_t)r;
        }
        if (pe.hdr_got == sizeof(Header) && pe.body_got == pe.body.size()) {
          deliver(who[i], pe.hdr.tag, pe.hdr.ctx, std::move(pe.body));
          pe.body = std::vector<char>();
          pe.hdr_got = 0;
          pe.body_got = 0;
        }
      }
    }
  }
  return moved;
}

int isend(const void *buf, size_t bytes, int dest, int tag, int ctx) {
  if (dest < 0 || dest >= g_size) die("send to a rank outside the world");
  int id = new_request();
  g_reqs[id].done = true;
  if (dest == g_rank) {
    std::vector<char> d((const char *)buf, (const char *)buf + bytes);
    deliver(g_rank, tag, ctx, std::move(d));
    return id;
  }
  std::vector<char> frame(sizeof(Header) + bytes);
  Header h{tag, ctx, (uint64_t)bytes};
  std::memcpy(frame.data(), &h, sizeof h);
  if (bytes) std::memcpy(frame.data() + sizeof h, buf, bytes);
  g_peers[dest].out.push_back(std::move(frame));
  progress(0);
  return id;
}

int irecv(void *buf, size_t cap, int src, int tag, int ctx) {
  int id = new_request();
  Request &r = g_reqs[id];
  r.is_recv = true;
  r.buf = buf;
  r.cap = cap;
  r.src = src;
  r.tag = tag;
  r.ctx = ctx;
  for (auto it = g_unexpected.begin(); it != g_unexpected.end(); ++it) {
    if (matches(r, it->src, it->tag, it->ctx)) {
      complete_recv(r, it->src, it->tag, it->data);
      g_unexpected.erase(it);
      return id;
    }
  }
  g_posted.push_back(id);
  return id;
}

bool req_done(int id) {
  Request &r = g_reqs[id];
  if (!r.parts.empty()) {
    for (int p : r.parts)
      if (!g_reqs[p].done) return false;
    return true;
  }
  return r.done;
}

void release(int id) {
  Request &r = g_reqs[id];
  for (int p : r.parts) g_reqs[p].used = false;
  r.used = false;
}

// Progress until `ready` holds; abort if a peer that could still satisfy the
// wait has exited, or nothing moves for the timeout.
template <class Ready>
void wait_until(Ready ready) {
  double last = now();
  while (!ready()) {
    if (progress(100)) {
      last = now();
      continue;
    }
    bool any_open = false;
    for (int p = 0; p < g_size; p++)
      if (p != g_rank && !g_peers[p].closed) any_open = true;
    if (!any_open && g_size > 1) die("waiting on a message, but every other rank has exited");
    if (now() - last > g_timeout) die("no progress within MINIMPI_TIMEOUT seconds");
  }
}

void flush_all() {
  wait_until([] {
    for (int p = 0; p < g_size; p++)
      if (p != g_rank && !g_peers[p].out.empty() && !g_peers[p].closed) return false;
    return true;
  });
}

}  // namespace

extern "C" {

int MPI_Init(int *, char ***) {
  if (g_init) return MPI_SUCCESS;
  g_init = true;
  const char *np = std::getenv("MINIMPI_NP");
  g_size = np ? std::atoi(np) : 1;
  if (g_size < 1 || g_size > 256) die("MINIMPI_NP must be 1..256");
  const char *to = std::getenv("MINIMPI_TIMEOUT");
  if (to) g_timeout = std::atof(to);
  g_peers.assign(g_size, Peer());
  // fds[a][b]: rank a's end of the (a, b) pair
  std::vector<std::vector<int>> fds(g_size, std::vector<int>(g_size, -1));
  for (int a = 0; a < g_size; a++)
    for (int b = a + 1; b < g_size; b++) {
      int sv[2];
      if (socketpair(AF_UNIX, SOCK_STREAM, 0, sv) != 0) die("socketpair failed (too many ranks for the fd limit?)");
      fds[a][b] = sv[0];
      fds[b][a] = sv[1];
    }
  std::fflush(stdout);
  std::fflush(stderr);
  int me = 0;
  for (int r = 1; r < g_size; r++) {
    pid_t pid = fork();
    if (pid < 0) die("fork failed");
    if (pid == 0) {
      me = r;
      g_children.clear();
      break;
    }
    g_children.push_back(pid);
  }
  g_rank = me;
  for (int a = 0; a < g_size; a++)
    for (int b = 0; b < g_size; b++) {
      if (fds[a][b] < 0) continue;
      if (a == g_rank) {
        g_peers[b].fd = fds[a][b];
        fcntl(fds[a][b], F_SETFL, fcntl(fds[a][b], F_GETFL) | O_NONBLOCK);
      } else {
        close(fds[a][b]);
      }
    }
  return MPI_SUCCESS;
}

int MPI_Finalize(void) {
  flush_all();
  for (int p = 0; p < g_size; p++)
    if (p != g_rank && g_peers[p].fd >= 0) shutdown(g_peers[p].fd, SHUT_WR);
  std::fflush(stdout);
  std::fflush(stderr);
  if (g_rank == 0) {
    int bad = 0;
    for (pid_t c : g_children) {
      int st = 0;
      if (waitpid(c, &st, 0) < 0 || !WIFEXITED(st) || WEXITSTATUS(st) != 0) bad++;
    }
    if (bad) {
      std::fprintf(stderr, "minimpi: %d rank(s) failed\n", bad);
      std::fflush(stderr);
      _exit(71);
    }
  }
  return MPI_SUCCESS;
}

int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = g_rank;
  return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm, int *size) {
  *size = g_size;
  return MPI_SUCCESS;
}

int MPI_Abort(MPI_Comm, int code) {
  std::fprintf(stderr, "minimpi rank %d: MPI_Abort(%d)\n", g_rank, code);
  std::fflush(stdout);
  std::fflush(stderr);
  _exit(code ? code : 72);
}

double MPI_Wtime(void) { return now(); }

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm, MPI_Request *req) {
  *req = isend(buf, (size_t)count * type_size(type), dest, tag, 0);
  return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm, MPI_Request *req) {
  *req = irecv(buf, (size_t)count * type_size(type), src, tag, 0);
  return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request *req, MPI_Status *st) {
  if (*req == MPI_REQUEST_NULL) return MPI_SUCCESS;
  int id = *req;
  if (id < 0 || id >= (int)g_reqs.size() || !g_reqs[id].used) die("MPI_Wait on an unknown request");
  wait_until([id] { return req_done(id); });
  if (st) *st = g_reqs[id].st;
  release(id);
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *sts) {
  for (int i = 0; i < n; i++) MPI_Wait(&reqs[i], sts ? &sts[i] : MPI_STATUS_IGNORE);
  return MPI_SUCCESS;
}

int MPI_Waitany(int n, MPI_Request *reqs, int *index, MPI_Status *st) {
  bool any = false;
  for (int i = 0; i < n; i++) any = any || reqs[i] != MPI_REQUEST_NULL;
  if (!any) {
    *index = -1;  // MPI_UNDEFINED
    return MPI_SUCCESS;
  }
  int found = -1;
  wait_until([&] {
    for (int i = 0; i < n; i++)
      if (reqs[i] != MPI_REQUEST_NULL && req_done(reqs[i])) {
        found = i;
        return true;
      }
    return false;
  });
  *index = found;
  return MPI_Wait(&reqs[found], st);
}

int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm) {
  MPI_Request r;
  MPI_Isend(buf, count, type, dest, tag, comm, &r);
  return MPI_Wait(&r, MPI_STATUS_IGNORE);
}

int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Status *st) {
  MPI_Request r;
  MPI_Irecv(buf, count, type, src, tag, comm, &r);
  return MPI_Wait(&r, st);
}

// Collectives use context 1, so no user receive can take their messages.
int MPI_Barrier(MPI_Comm) {
  char token = 0;
  if (g_rank == 0) {
    std::vector<int> rs;
    for (int p = 1; p < g_size; p++) rs.push_back(irecv(&token, 1, p, 0, 1));
    for (int r : rs) {
      wait_until([r] { return req_done(r); });
      release(r);
    }
    for (int p = 1; p < g_size; p++) release(isend(&token, 1, p, 0, 1));
  } else {
    release(isend(&token, 1, 0, 0, 1));
    int r = irecv(&token, 1, 0, 0, 1);
    wait_until([r] { return req_done(r); });
    release(r);
  }
  return MPI_SUCCESS;
}

int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm) {
  size_t bytes = (size_t)count * type_size(type);
  if (g_rank == root) {
    for (int p = 0; p < g_size; p++)
      if (p != root) release(isend(buf, bytes, p, 1, 1));
  } else {
    int r = irecv(buf, bytes, root, 1, 1);
    wait_until([r] { return req_done(r); });
    release(r);
  }
  return MPI_SUCCESS;
}

int MPI_Ialltoall(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount, MPI_Datatype rtype,
                  MPI_Comm, MPI_Request *req) {
  size_t sb = (size_t)scount * type_size(stype), rb = (size_t)rcount * type_size(rtype);
  int id = new_request();
  std::vector<int> parts;
  for (int p = 0; p < g_size; p++) parts.push_back(irecv((char *)rbuf + p * rb, rb, p, 2, 1));
  for (int p = 0; p < g_size; p++) parts.push_back(isend((const char *)sbuf + p * sb, sb, p, 2, 1));
  g_reqs[id].parts = parts;
  *req = id;
  return MPI_SUCCESS;
}

int MPI_Alltoall(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount, MPI_Datatype rtype,
                 MPI_Comm comm) {
  MPI_Request r;
  MPI_Ialltoall(sbuf, scount, stype, rbuf, rcount, rtype, comm, &r);
  return MPI_Wait(&r, MPI_STATUS_IGNORE);
}

}  // extern "C"
