// Multi-rank driver over the reference's distributed PCS commitments, for
// the oracle: runs the unmodified Batch_dCommit and dCommit
// (distributed_PCS.cpp:56-170, with distributed_batch_FFT /
// distributed_FFT, MPI_utils.cpp:2911-3298, and distributed_commit,
// coPCS.cpp:311-367) with N ranks (minimpi: MINIMPI_NP=N) on seeded
// per-rank inputs, and writes what every rank holds afterwards.
//
// Test infrastructure only (target pigeon_dpcs of oracle/ref/Makefile).
//
//   pigeon_dpcs batch  <logA> <batch> <rate> <seed> <out prefix>   Batch_dCommit(arr, arr2, ..., rate, N, batch)
//   pigeon_dpcs single <logA> <rate> <seed> <out prefix>           dCommit(arr, codeword, C, rate, N, 0)
//
// Rank p's inputs: arr (then arr2) of 2^logA extension-field elements from a
// SplitMix64 stream seeded with seed and p.  prepare_data(N, rate)
// (distributed_PCS.cpp:28-54) sets the fold degrees first, as coPIOP_prove
// does.  Output per rank into <out prefix>.<rank> (binary, little-endian):
//   batch:  u32 batch, u32 codeword length, commit_data rows, codeword rows,
//           32-byte local root, u32 count and every level of the local tree
//           (leaves first), then on rank 0 the 32-byte leader root
//   single: u32 codeword length, the codeword, then the same tree records
#include <mpi.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "coPCS.h"
#include "config_pc.hpp"
#include "distributed_PCS.h"
#include "utils.hpp"

using std::vector;

namespace {

const uint64_t P61 = (1ull << 61) - 1;

struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  uint64_t below_p() {
    for (;;) {
      uint64_t v = next() >> 3;
      if (v < P61) return v;
    }
  }
  F fe() {
    F x;
    x.real = below_p();
    x.img = below_p();
    return x;
  }
};

void put_u32(FILE *f, uint32_t v) { fwrite(&v, 4, 1, f); }
void put_fes(FILE *f, const vector<F> &v) {
  for (auto &x : v) {
    fwrite(&x.real, 8, 1, f);
    fwrite(&x.img, 8, 1, f);
  }
}
void put_root(FILE *f, const vector<vector<_hash>> &levels) { fwrite(levels.back()[0].arr, 1, 32, f); }
// every level of a tree, leaves first: u32 count, then the hashes
void put_levels(FILE *f, const vector<vector<_hash>> &levels) {
  uint32_t n = 0;
  for (auto &l : levels) n += (uint32_t)l.size();
  put_u32(f, n);
  for (auto &l : levels)
    for (auto &h : l) fwrite(h.arr, 1, 32, f);
}

}  // namespace

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  int rank = 0, N = 1;
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  MPI_Comm_size(MPI_COMM_WORLD, &N);
  const bool batch = argc >= 2 && std::string(argv[1]) == "batch";
  if ((batch && argc < 7) || (!batch && argc < 6)) {
    if (!rank) fprintf(stderr, "usage: pigeon_dpcs batch logA batch rate seed out | single logA rate seed out\n");
    MPI_Abort(MPI_COMM_WORLD, 2);
  }
  const int logA = atoi(argv[2]);
  const int nb = batch ? atoi(argv[3]) : 0;
  const int rate = atoi(argv[batch ? 4 : 3]);
  const uint64_t seed = strtoull(argv[batch ? 5 : 4], nullptr, 0);
  const char *out = argv[batch ? 6 : 5];
  const size_t A = 1ull << logA;
  prepare_data(N, rate);
  SplitMix g{seed * 0x10001ull + (uint64_t)rank * 0x9E3779B1ull + 11};
  vector<F> arr(A), arr2;
  for (auto &x : arr) x = g.fe();
  char path[4096];
  snprintf(path, sizeof path, "%s.%d", out, rank);
  FILE *f = fopen(path, "wb");
  if (!f) MPI_Abort(MPI_COMM_WORLD, 3);
  MT C;
  if (batch) {
    arr2.resize(A);
    for (auto &x : arr2) x = g.fe();
    vector<vector<F>> cd, cw;
    Batch_dCommit(arr, arr2, cd, cw, C, rate, N, nb);
    put_u32(f, (uint32_t)cd.size());
    put_u32(f, (uint32_t)cw[0].size());
    for (auto &r : cd) put_fes(f, r);
    for (auto &r : cw) put_fes(f, r);
  } else {
    vector<F> cw;
    dCommit(arr, cw, C, rate, N, 0);
    put_u32(f, (uint32_t)cw.size());
    put_fes(f, cw);
  }
  put_root(f, C.Base_MT);
  put_levels(f, C.Base_MT);
  if (rank == 0) put_root(f, C.Root_MT);
  fclose(f);
  MPI_Finalize();
  return 0;
}
