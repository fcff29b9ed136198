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
//   pigeon_dpcs pcs    <logM> <seed> <out prefix>
//       the coPCS test's dealing and PCS_commit (main.cpp:49-76), then
//       PCS_open_new with isPIOP = true (coPCS.cpp:1310-1700) as
//       coPIOP_prove calls it (coPIOP.cpp:1767-1773): input vectors b1 =
//       the Lagrange vector over 32 points, b2 = the tensor of two Lagrange
//       vectors (Lagrange_evals) over the row length, b3 = the one over N/4
//       points, at points from a SplitMix64 stream; K = 0.  Rank 0 then
//       writes the WHIR batch slots 2 and 3 the opening fills.
//   pigeon_dpcs open   <P> <logA> <batch> <rate> <seed> <out prefix>
//       P (2 or 3) Batch_dCommit calls as coPIOP_prove makes them
//       (coPIOP.cpp:868, 1708-1730), then PIOP_dOpen_batch_new
//       (distributed_PCS.cpp:1175-1534) with Verify = {true, false} on
//       points drawn from a stream all ranks share and claims y_l = the
//       committed data's evaluations; the data (arr2) of every polynomial
//       but the first is zero, as the dummy index's is, so that the first
//       round's check holds.  Rank 0 then writes the opening's final WHIR
//       inputs (whir_polys, whir_c, whir_betas, whir_claims, the tree root)
//       at slot 1 of the WHIR batch (sorted_indexes = identity).
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
#include <unordered_map>
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

extern vector<vector<F>> whir_polys, whir_c, whir_betas;  // coPIOP.cpp:47-55
extern vector<vector<vector<_hash>>> whir_MTs;
extern vector<F> whir_claims;
extern vector<int> whir_rates, sorted_indexes;
extern std::unordered_map<int, int> whir_kappas;
extern int randomness;          // coPCS.cpp:18
extern vector<int> _queries;    // New_PCS.cpp:5

namespace {

vector<F> beta_table(const vector<F> &r) {
  vector<F> b;
  precompute_beta(r, b);
  return b;
}

int open_mode(int argc, char **argv, int rank, int N) {
  double t_commit = 0;
  if (argc < 8) {
    if (!rank) fprintf(stderr, "usage: pigeon_dpcs open P logA batch rate seed out\n");
    MPI_Abort(MPI_COMM_WORLD, 2);
  }
  const int P = atoi(argv[2]), logA = atoi(argv[3]), nb = atoi(argv[4]), rate = atoi(argv[5]);
  const uint64_t seed = strtoull(argv[6], nullptr, 0);
  const char *out = argv[7];
  const size_t A = 1ull << logA, S = A / nb;
  prepare_data(N, rate);
  // the WHIR batch slots the opening writes into (get_whir_rates, Whir.cpp:18)
  whir_rates = {rate, rate, rate, rate};
  sorted_indexes = {0, 1, 2, 3};
  for (size_t sz = 1; sz <= (1u << 26); sz <<= 1) whir_kappas[(int)sz] = 4;
  whir_polys.resize(4);
  whir_c.resize(4);
  whir_betas.resize(4);
  whir_MTs.resize(4);
  whir_claims.resize(4);
  vector<vector<vector<F>>> cd(P), cw(P);
  vector<MT> C(P);
  vector<vector<F>> r(P);
  vector<F> y(P, F(0));
  int lrows = 0;
  while ((1 << lrows) < nb) lrows++;
  int lN = 0;
  while ((1 << lN) < N) lN++;
  int lS = 0;
  while (((size_t)1 << lS) < S) lS++;
  SplitMix gs{seed * 0x7F4A7C15ull + 3};  // shared by all ranks
  for (int l = 0; l < P; l++) {
    // every rank's arrays, so that each can form the claim
    vector<vector<F>> arr2_all(N);
    vector<F> arr_mine;
    for (int p = 0; p < N; p++) {
      SplitMix g{seed * 0x10001ull + (uint64_t)p * 0x9E3779B1ull + 11 + 0x1000ull * l};
      vector<F> a(A), a2(A);
      for (auto &x : a) x = g.fe();
      for (auto &x : a2) x = g.fe();
      if (l > 0)
        for (auto &x : a2) x = F(0);
      if (p == rank) arr_mine = a;
      arr2_all[p] = a2;
    }
    vector<F> arr2_mine = arr2_all[rank];
    const double t0 = MPI_Wtime();
    Batch_dCommit(arr_mine, arr2_mine, cd[l], cw[l], C[l], rate, N, nb);
    if (l == 0) t_commit = MPI_Wtime() - t0;
    for (int i = 0; i < lS + lrows + lN; i++) r[l].push_back(gs.fe());
    // y_l = sum_p b1[p] sum_k b2[k] sum_h b3[h] arr2_p[h S + k]
    // (r = (r2: log S, r3: log rows, r1: log N), distributed_PCS.cpp:1188-1203)
    vector<F> r2(r[l].begin(), r[l].begin() + lS), r3(r[l].begin() + lS, r[l].begin() + lS + lrows),
        r1(r[l].begin() + lS + lrows, r[l].end());
    vector<F> b1 = beta_table(r1), b2 = beta_table(r2), b3 = beta_table(r3);
    for (int p = 0; p < N; p++)
      for (int h = 0; h < nb; h++)
        for (size_t k = 0; k < S; k++) y[l] = y[l] + b1[p] * b2[k] * b3[h] * arr2_all[p][h * S + k];
  }
  vector<bool> verify = {true, false};
  const double t1 = MPI_Wtime();
  PIOP_dOpen_batch_new(cd, cw, C, r, y, verify, N);
  const double t_open = MPI_Wtime() - t1;
  // DPCS_TIMING=1: rank 0 reports the wall time of the first commitment and
  // of the opening (for the benchmark's reference figure)
  if (rank == 0 && getenv("DPCS_TIMING")) printf("seconds: commit %.6f open %.6f\n", t_commit, t_open);
  if (rank == 0) {
    char path[4096];
    snprintf(path, sizeof path, "%s.%d", out, rank);
    FILE *f = fopen(path, "wb");
    if (!f) MPI_Abort(MPI_COMM_WORLD, 3);
    vector<F> yv = y;
    put_u32(f, (uint32_t)yv.size());
    put_fes(f, yv);
    put_u32(f, (uint32_t)whir_polys[1].size());
    put_fes(f, whir_polys[1]);
    put_u32(f, (uint32_t)whir_c[1].size());
    put_fes(f, whir_c[1]);
    put_u32(f, (uint32_t)whir_betas[1].size());
    put_fes(f, whir_betas[1]);
    put_fes(f, vector<F>{whir_claims[1]});
    put_root(f, whir_MTs[1]);
    fclose(f);
  }
  MPI_Finalize();
  return 0;
}

int pcs_mode(int argc, char **argv, int rank, int N) {
  if (argc < 5) {
    if (!rank) fprintf(stderr, "usage: pigeon_dpcs pcs logM seed out\n");
    MPI_Abort(MPI_COMM_WORLD, 2);
  }
  const int logM = atoi(argv[2]);
  const uint64_t seed = strtoull(argv[3], nullptr, 0);
  const char *out = argv[4];
  const int M = 1 << logM, k = N / 4, _k = N / 2;
  vector<vector<int>> rate = {{4}, {4}, {4, 4}, {4, 4}};
  vector<vector<F>> codeword, Commit_data;
  vector<F> random_shares, shares;
  MT C;
  prepare_parameters(rate, rate.size(), N, M);
  secret_share_coefficients(shares, M, N, _k, k);
  secret_share_coefficients(random_shares, randomness * N / 4, N, _k, k);
  PCS_commit(C, codeword, Commit_data, shares, random_shares, rate, N);
  sorted_indexes = {0, 1, 2, 3};
  whir_polys.resize(4);
  whir_c.resize(4);
  whir_betas.resize(4);
  whir_MTs.resize(4);
  whir_claims.resize(4);
  // the input vectors (coPIOP.cpp:1741-1762)
  const int Bs = (int)Commit_data[0].size();
  int lB = 0;
  while ((1 << lB) < Bs) lB++;
  const int la = lB / 2, lb = lB - la;
  SplitMix gs{seed * 0x7F4A7C15ull + 3};
  const F p0 = gs.fe(), p1 = gs.fe(), p2 = gs.fe(), p3 = gs.fe();
  int lk = 0;
  while ((1 << lk) < N / 4) lk++;
  vector<vector<F>> inputs(3), Lagrange_evals;
  inputs[0] = compute_lagrange_coeff(getRootOfUnity(5), p0, 32);
  Lagrange_evals.push_back(compute_lagrange_coeff(getRootOfUnity(la), p1, 1 << la));
  Lagrange_evals.push_back(compute_lagrange_coeff(getRootOfUnity(lb), p2, 1 << lb));
  inputs[1] = Lagrange_evals[0];
  {
    vector<F> buff(inputs[1].size() * Lagrange_evals[1].size());
    for (size_t j = 0; j < Lagrange_evals[1].size(); j++)
      for (size_t kk = 0; kk < inputs[1].size(); kk++)
        buff[kk + j * inputs[1].size()] = Lagrange_evals[1][j] * inputs[1][kk];
    inputs[1] = buff;
  }
  inputs[2] = compute_lagrange_coeff(getRootOfUnity(lk), p3, N / 4);
  // the claim these vectors give the committed data: F_ip as the coPCS test
  // forms it (main.cpp:93-106), with the row weights b1 and, as
  // PCS_open_new uses them in this mode (coPCS.cpp:1328-1335), b2 zero on
  // the last _queries[0] entries of a row
  int batches = 0;
  for (auto &row : Commit_data) {
    if (row.empty()) break;
    batches++;
  }
  const size_t rows = Commit_data.size();
  vector<F> v(rows * Bs, F(0)), v1(rows * Bs, F(0));
  for (int i = 0; i < batches - 1; i++)
    for (int j = 0; j < Bs; j++) v[j * rows + i] = Commit_data[i][j];
  for (int j = 0; j < Bs - _queries[0]; j++)
    for (int i = 0; i < batches - 1; i++) v1[j * rows + i] = inputs[0][i] * inputs[1][j];
  F K = F_ip(v, v1, inputs[2], k, _k, N);
  const double t0 = MPI_Wtime();
  PCS_open_new(C, codeword, Commit_data, inputs, Lagrange_evals, K, rate, N, true);
  // DPCS_TIMING=1: rank 0 reports the opening's wall time
  if (rank == 0 && getenv("DPCS_TIMING")) printf("seconds: open_piop %.6f\n", MPI_Wtime() - t0);
  if (rank == 0) {
    char path[4096];
    snprintf(path, sizeof path, "%s.%d", out, rank);
    FILE *f = fopen(path, "wb");
    if (!f) MPI_Abort(MPI_COMM_WORLD, 3);
    for (int slot = 2; slot < 4; slot++) {
      put_u32(f, (uint32_t)whir_polys[slot].size());
      put_fes(f, whir_polys[slot]);
      put_u32(f, (uint32_t)whir_c[slot].size());
      put_fes(f, whir_c[slot]);
      put_u32(f, (uint32_t)whir_betas[slot].size());
      put_fes(f, whir_betas[slot]);
      put_fes(f, vector<F>{whir_claims[slot]});
      put_root(f, whir_MTs[slot]);
    }
    fclose(f);
  }
  MPI_Finalize();
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  int rank = 0, N = 1;
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  MPI_Comm_size(MPI_COMM_WORLD, &N);
  if (argc >= 2 && std::string(argv[1]) == "open") return open_mode(argc, argv, rank, N);
  if (argc >= 2 && std::string(argv[1]) == "pcs") return pcs_mode(argc, argv, rank, N);
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
