// Multi-rank driver over the reference's coSumcheck round functions, for the
// oracle: runs the unmodified quadratic_coSumcheck / cubic_coSumcheck
// (coSumcheck.cpp:233-448) with N ranks (minimpi: MINIMPI_NP=N) on seeded
// per-rank shares, and writes what the leader returns.
//
// Test infrastructure only (target pigeon_cosc of oracle/ref/Makefile; every
// rank's Fiat-Shamir and aggregation calls are captured by capture.cpp).
//
//   pigeon_cosc quad  <logn> <d0,d1,...> <seed> <out file>
//   pigeon_cosc cubic <logn> <d0,d1,...> <seed> <out file>
//
// Rank p's inputs (length 2^logn each): p1, p2 (and p3, r1, r2 for the cubic
// form) from SplitMix64 streams seeded with seed and p; in the cubic form
// every fifth block of p1 of prod_i d_i entries is zero, so that the
// zero-block skip of cubic_coSumcheck_phase1 is exercised in every round.  R[i] has 2 d_i
// (quadratic) or 4 d_i (cubic) entries per rank.  K and K_r are chosen so
// that every round check holds: the first round's aggregated message is
// A + c B for the challenge c, and K = A, K_r = B make K + c K_r match it;
// A and B come from two calls of the phase-1 function (which draws no
// challenge) with r = 0 and r = 1.
//
// Output on rank 0 into <out file> (binary, little-endian): F K, F K_r, u32
// count, then count claims of (F eval, u32 len, F r[len]).  Standard output keeps the
// reference's own messages (a failed check prints there).
#include <mpi.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "coSumcheck.h"
#include "config_pc.hpp"
#include "utils.hpp"

using std::vector;

vector<F> quadratic_coSumcheck_phase1(vector<F> &p1, vector<F> &p2, vector<vector<F>> R, F r, int d, int iter, int N);
vector<F> cubic_coSumcheck_phase1(vector<F> &p1, vector<F> &p2, vector<F> &p3, vector<F> &b1, vector<F> &b2,
                                  vector<vector<F>> R, F r, int d, int iter, int N);

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

vector<F> vec(SplitMix &g, size_t n) {
  vector<F> v(n);
  for (auto &x : v) x = g.fe();
  return v;
}

FILE *g_out = nullptr;
void put_u32(uint32_t v) { fwrite(&v, 4, 1, g_out); }
void put_fe(const F &x) {
  fwrite(&x.real, 8, 1, g_out);
  fwrite(&x.img, 8, 1, g_out);
}

}  // namespace

int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  int rank = 0, N = 1;
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  MPI_Comm_size(MPI_COMM_WORLD, &N);
  if (argc < 6) {
    if (!rank) fprintf(stderr, "usage: pigeon_cosc quad|cubic logn d0,d1,... seed out\n");
    MPI_Abort(MPI_COMM_WORLD, 2);
  }
  const bool cubic = std::string(argv[1]) == "cubic";
  const int logn = atoi(argv[2]);
  vector<int> degrees;
  for (char *t = strtok(argv[3], ","); t; t = strtok(nullptr, ",")) degrees.push_back(atoi(t));
  const uint64_t seed = strtoull(argv[4], nullptr, 0);
  const size_t n = 1ull << logn;

  SplitMix g{seed * 0x10001ull + (uint64_t)rank * 0x9E3779B1ull + 7};
  vector<F> p1 = vec(g, n), p2 = vec(g, n), p3;
  vector<vector<F>> R;
  for (int d : degrees) R.push_back(vec(g, (cubic ? 4 : 2) * d));
  vector<F> r1, r2, b1, b2;
  SplitMix gs{seed * 0x7F4A7C15ull + 3};  // shared by all ranks
  if (cubic) {
    p3 = vec(g, n);
    size_t zb = 1;
    for (int d : degrees) zb *= (size_t)d;
    for (size_t j = 0; j < n / zb; j += 5)
      for (size_t k = 0; k < zb; k++) p1[j * zb + k] = F(0);
    int nr1 = logn;
    for (int i = 0; i < nr1; i++) r1.push_back(gs.fe());
    int lk = 0;
    while ((1 << lk) < N / 4) lk++;
    for (int i = 0; i < lk; i++) r2.push_back(gs.fe());
    precompute_beta(r1, b1);
    precompute_beta(r2, b2);
  }
  // K = A, K_r = B with A + c B the first aggregated round value
  F A, B;
  {
    vector<F> q1 = p1, q2 = p2, q3 = p3, bb1 = b1, bb2 = b2;
    vector<F> H0 = cubic ? cubic_coSumcheck_phase1(q1, q2, q3, bb1, bb2, R, F(0), degrees[0], 0, N)
                         : quadratic_coSumcheck_phase1(q1, q2, R, F(0), degrees[0], 0, N);
    vector<F> H1 = cubic ? cubic_coSumcheck_phase1(q1, q2, q3, bb1, bb2, R, F(1), degrees[0], 0, N)
                         : quadratic_coSumcheck_phase1(q1, q2, R, F(1), degrees[0], 0, N);
    const int step = cubic ? 4 : 2;
    A = F(0);
    F AB = F(0);
    for (size_t j = 0; j < H0.size() / step; j++) {
      A = A + H0[step * j];
      AB = AB + H1[step * j];
    }
    B = AB - A;
  }
  double ps = 0;
  vector<pair<F, vector<F>>> claims =
      cubic ? cubic_coSumcheck(p1, p2, p3, r1, r2, R, A, B, degrees, N, ps)
            : quadratic_coSumcheck(p1, p2, R, A, B, degrees, N, ps);
  if (rank == 0) {
    g_out = fopen(argv[5], "wb");
    if (!g_out) MPI_Abort(MPI_COMM_WORLD, 3);
    put_fe(A);
    put_fe(B);
    put_u32((uint32_t)claims.size());
    for (auto &c : claims) {
      put_fe(c.first);
      put_u32((uint32_t)c.second.size());
      for (auto &x : c.second) put_fe(x);
    }
    fclose(g_out);
  }
  MPI_Finalize();
  return 0;
}
