// Reference-signature front end for libgbz.
//
// A maintainer of the reference prover adds this translation unit to its
// build and drops the bodies it replaces (listed below); no caller changes.
// It compiles against the reference's own headers and forwards to the C ABI
// of include/gbz.h.  Field elements are passed by pointer:
// virgo::fieldElement is {real, img} as two 64-bit words, which is the
// element layout gbz.h expects; _hash is 32 bytes.
//
// Replaced bodies (file of the reference, then function):
//   utils.cpp         fft, pfft, precompute_beta
//   Blake3_hash.cpp   blake3_hash
//   merkle_tree.cpp   MT_commit_Blake, create_tree_blake
//   Fiat_Shamir.cpp   hash_to_field (the chain value prev_challenge stays the
//                     reference's global)
//   Whir.cpp          Whir_Commit_initial, Whir_Commit, Whir_Open (one
//                     claim), Whir_Batch_Open, aggregate_claims,
//                     aggregate_commitments
//   coPCS.cpp         distributed_MT (one rank's part, MPI exchange kept)
//   fieldElement.cpp  fieldElement::_random
//   libc              random, rand, srandom, srand: one glibc-compatible
//                     generator (gbz_prng) shared by the reference's
//                     remaining code and the GPU calls, so that every draw
//                     lands in the same order as in an unmodified run
// open_tree_blake is not replaced: it is a lookup in the caller's host
// levels with no data-parallel work.
//
// The N-party calls of libgbz (gbz_pcs_commit / gbz_pcs_open /
// gbz_pcs_open_piop, gbz_cosumcheck, gbz_party_sumcheck, gbz_piop_phase1 /
// gbz_piop_phase2, gbz_dpcs_*)
// take every party's share at once, the one-device model of the
// collaborative prover; they replace the N-rank runs of PCS_commit /
// PCS_open_new, quadratic/cubic_coSumcheck, _quadratic/_cubic_sumcheck and
// prove_phase1 / prove_phase2, whose per-rank signatures hold one share, so
// they are called through the C ABI directly.
//
// Errors: the reference prints and exits; this shim does the same on a
// non-OK status so that callers see unchanged behaviour.
#include <mpi.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "Whir.h"
#include "coPCS.h"
#include "config_pc.hpp"
#include "gbz.h"
#include "merkle_tree.h"

extern F prev_challenge;           // Fiat_Shamir.cpp:5
extern double whir_ps;              // Whir.cpp
extern bool conjectured_security;   // main.cpp
extern int com_rounds;              // coPCS.cpp
extern double cm;                   // coPCS.cpp

namespace {

gbz_ctx *ctx() {
  static thread_local gbz_ctx *c = nullptr;
  if (!c) {
    gbz_status s = gbz_create(&c, 0);
    if (s != GBZ_OK) {
      std::fprintf(stderr, "gbz_create failed: %s\n", gbz_status_string(s));
      std::exit(-1);
    }
  }
  return c;
}

void check(gbz_status s, const char *what) {
  if (s != GBZ_OK) {
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, gbz_status_string(s), gbz_last_error(ctx()));
    std::exit(-1);
  }
}

uint64_t *words(F *p) { return reinterpret_cast<uint64_t *>(p); }
const uint64_t *words(const F *p) { return reinterpret_cast<const uint64_t *>(p); }
uint8_t *bytes(_hash *h) { return reinterpret_cast<uint8_t *>(h); }

static_assert(sizeof(F) == 16, "virgo::fieldElement must be two 64-bit words");
static_assert(sizeof(_hash) == 32, "_hash must be 32 bytes");

// The process's random() stream (glibc's default state until srandom).
gbz_prng &process_prng() {
  static gbz_prng g;
  static bool seeded = false;
  if (!seeded) {
    gbz_prng_seed(&g, 1);
    seeded = true;
  }
  return g;
}

// Levels back to back (leaves first) into the reference's vector of levels,
// the way MT_commit_Blake fills them: the vector is resized only when empty
// (merkle_tree.cpp:205-208), so levels above a shallower new tree keep what
// they held.
void assign_levels(vector<vector<_hash>> &hashes, const std::vector<_hash> &flat, uint64_t leaves) {
  int levels = 0;
  for (uint64_t c = leaves; c >= 1; c /= 2) levels++;
  if (hashes.empty()) hashes.resize(levels);
  if ((int)hashes.size() < levels) hashes.resize(levels);  // the reference writes past the end here
  size_t off = 0;
  int lv = 0;
  for (uint64_t c = leaves; c >= 1; c /= 2, lv++) {
    hashes[lv].assign(flat.begin() + off, flat.begin() + off + c);
    off += c;
  }
}

int log2i(uint64_t x) {
  int l = 0;
  while ((1ull << (l + 1)) <= x) l++;
  return l;
}

}  // namespace

// ------------------------------------------------------------- generator
extern "C" long random(void) noexcept { return gbz_prng_next(&process_prng()); }
extern "C" int rand(void) noexcept { return gbz_prng_next(&process_prng()); }
extern "C" void srandom(unsigned int seed) noexcept { gbz_prng_seed(&process_prng(), seed); }
extern "C" void srand(unsigned int seed) noexcept { gbz_prng_seed(&process_prng(), seed); }

// fieldElement::_random (fieldElement.cpp:119-125)
virgo::fieldElement virgo::fieldElement::_random() {
  uint64_t w[2];
  gbz_prng_field(&process_prng(), w);
  F r;
  r.real = w[0];
  r.img = w[1];
  return r;
}

// -------------------------------------------------------------- transforms
// fft (utils.cpp:904-964)
void fft(vector<F> &arr, int logn, bool flag) {
  check(gbz_fft(ctx(), words(arr.data()), logn, flag ? 1 : 0, GBZ_MEM_HOST), "fft");
}

// pfft (utils.cpp:1583-1673): the forward transform for lengths above 1024;
// below that it defers to fft with the caller's flag.
void pfft(vector<F> &arr, int logn, bool flag) {
  const bool inverse = ((1 << logn) / 256 <= 4) ? flag : false;
  check(gbz_fft(ctx(), words(arr.data()), logn, inverse ? 1 : 0, GBZ_MEM_HOST), "pfft");
}

// precompute_beta (utils.cpp:198-243)
void precompute_beta(vector<F> r, vector<F> &B) {
  B.resize(1u << r.size());
  check(gbz_precompute_beta(ctx(), words(r.data()), (int)r.size(), words(B.data()), GBZ_MEM_HOST),
        "precompute_beta");
}

// ------------------------------------------------------------ hashes
// blake3_hash (Blake3_hash.cpp:5-10)
void blake3_hash(uint8_t *src, uint8_t *dst) { check(gbz_blake3_64(ctx(), src, dst, 1, GBZ_MEM_HOST), "blake3_hash"); }

// hash_to_field (Fiat_Shamir.cpp:29-34) on the reference's chain value
F hash_to_field(vector<F> elements) {
  uint64_t st[2] = {prev_challenge.real, prev_challenge.img}, out[2];
  gbz_hash_to_field(st, words(elements.data()), (int)elements.size(), out);
  prev_challenge.real = out[0];
  prev_challenge.img = out[1];
  return prev_challenge;
}

// MT_commit_Blake (merkle_tree.cpp:195-233).  For N <= 2 the reference hashes
// the two elements followed by 32 bytes of uninitialised stack memory; the
// shim hashes zeros there (the reference's value is undefined).
void merkle_tree::merkle_tree_prover::MT_commit_Blake(F *leafs, vector<vector<_hash>> &hashes, int N) {
  if (N <= 2) {
    uint8_t data[64] = {0};
    std::memcpy(data, leafs, 2 * sizeof(F));
    hashes.resize(1);
    hashes[0].resize(1);
    check(gbz_blake3_64(ctx(), data, hashes[0][0].arr, 1, GBZ_MEM_HOST), "MT_commit_Blake");
    return;
  }
  std::vector<_hash> flat((size_t)N / 2 - 1);
  check(gbz_merkle_commit_blake(ctx(), words(leafs), (uint64_t)N, bytes(flat.data()), GBZ_MEM_HOST),
        "MT_commit_Blake");
  assign_levels(hashes, flat, (uint64_t)N / 4);
}

// create_tree_blake (merkle_tree.cpp:267-299): the levels above hashes[0]'s
// first ele_num hashes (ele_num a power of two).
void merkle_tree::merkle_tree_prover::create_tree_blake(int ele_num, vector<vector<_hash>> &hashes,
                                                        const int element_size, bool alloc_required) {
  (void)element_size;
  (void)alloc_required;
  if (ele_num < 2) return;
  if (ele_num & (ele_num - 1)) {
    std::fprintf(stderr, "create_tree_blake: %d leaves (the GPU path takes a power of two)\n", ele_num);
    std::exit(-1);
  }
  const int depth = log2i((uint64_t)ele_num);
  if ((int)hashes.size() < depth + 1) hashes.resize(depth + 1);  // the reference writes past the end here
  std::vector<_hash> up((size_t)ele_num - 1);
  check(gbz_merkle_tree_from_leaves(ctx(), bytes(hashes[0].data()), (uint64_t)ele_num, bytes(up.data()),
                                    GBZ_MEM_HOST),
        "create_tree_blake");
  size_t off = 0;
  for (int lv = 1, c = ele_num / 2; c >= 1; c /= 2, lv++) {
    hashes[lv].assign(up.begin() + off, up.begin() + off + c);
    off += c;
  }
}

// ------------------------------------------------------------------ WHIR
// Whir_Commit_initial (Whir.cpp:158-190): codeword = pfft of arr padded to
// rate * |arr|, MT = MT_commit_Blake of the codeword.
void Whir_Commit_initial(vector<F> &arr, vector<F> &codeword, vector<vector<_hash>> &MT, int rate, int kappa) {
  (void)kappa;  // the reference's strided leaf loop stores nothing
  codeword.resize(rate * arr.size());
  std::vector<_hash> flat(codeword.size() / 2 - 1);
  check(gbz_whir_commit(ctx(), words(arr.data()), arr.size(), rate, words(codeword.data()), bytes(flat.data()),
                        GBZ_MEM_HOST),
        "Whir_Commit_initial");
  assign_levels(MT, flat, codeword.size() / 4);
}

// Whir_Commit (Whir.cpp:192-213): the same codeword; the tree it keeps has
// codeword.size() / kappa zero leaf hashes (its leaf loop never stores a
// hash), built by create_tree_blake.
void Whir_Commit(vector<F> &arr, vector<F> &codeword, vector<vector<_hash>> &MT, int rate, int kappa) {
  codeword = arr;
  codeword.resize(rate * arr.size(), F(0));
  pfft(codeword, log2i(codeword.size()), false);
  MT.resize(log2i(codeword.size() / kappa) + 1);
  MT[0] = vector<_hash>(codeword.size() / kappa);
  for (auto &h : MT[0]) std::memset(h.arr, 0, 32);
  merkle_tree::merkle_tree_prover::create_tree_blake((int)MT[0].size(), MT, 32, true);
}

// Whir_Open (Whir.cpp:388-467) of one claim, whir_k = 4.  The reference's
// own verification steps after the last iteration are not repeated; the
// running claim is checked in every round on the device.
void Whir_Open(vector<F> &arr, vector<F> &codeword, vector<vector<_hash>> &MT, vector<pair<F, vector<F>>> claims,
               int rate) {
  (void)MT;
  if (claims.size() != 1) {
    std::fprintf(stderr, "Whir_Open: the GPU path opens one claim (got %zu)\n", claims.size());
    std::exit(-1);
  }
  const int logn = log2i(arr.size());
  std::vector<uint8_t> tr(gbz_whir_open_transcript_bytes(logn, rate));
  const uint64_t K[2] = {claims[0].first.real, claims[0].first.img};
  check(gbz_whir_open(ctx(), words(arr.data()), logn, rate, words(codeword.data()), words(claims[0].second.data()),
                      K, &process_prng(), tr.data(), tr.size(), GBZ_MEM_HOST),
        "Whir_Open");
  whir_ps += tr.size() / 1024.0;
}

// Whir_Batch_Open (Whir.cpp:706-898) with the reference's global whir_k.
void Whir_Batch_Open(vector<vector<F>> &arrays, vector<vector<F>> &codewords, vector<vector<vector<_hash>>> &MTs,
                     vector<F> evals, vector<vector<F>> &betas, int rate, bool Verify) {
  (void)Verify;  // the device checks every claim (GBZ_ECHECK otherwise)
  const int k = (int)arrays.size();
  std::vector<uint64_t> sizes(k);
  std::vector<const uint64_t *> a(k), c(k), b(k);
  for (int i = 0; i < k; i++) {
    sizes[i] = arrays[i].size();
    a[i] = words(arrays[i].data());
    c[i] = words(codewords[i].data());
    b[i] = words(betas[i].data());
  }
  uint64_t nbytes = 0;
  check(gbz_whir_batch_schedule(k, sizes.data(), rate, whir_k, nullptr, nullptr, nullptr, nullptr, &nbytes),
        "Whir_Batch_Open schedule");
  std::vector<uint8_t> levels0, tr(nbytes);
  for (auto &lv : MTs[0])
    levels0.insert(levels0.end(), reinterpret_cast<uint8_t *>(lv.data()),
                   reinterpret_cast<uint8_t *>(lv.data() + lv.size()));
  const uint64_t K0[2] = {evals[0].real, evals[0].img};
  check(gbz_whir_batch_open(ctx(), k, a.data(), sizes.data(), c.data(), levels0.data(), b.data(), K0, rate, whir_k,
                            &process_prng(), tr.data(), tr.size(), GBZ_MEM_HOST),
        "Whir_Batch_Open");
  whir_ps += tr.size() / 1024.0;
}

// aggregate_claims (Whir.cpp:608-668): the points of claims[i][j] in order.
vector<vector<F>> aggregate_claims(vector<vector<F>> &arrays, vector<F> &arr, vector<F> &b_arr,
                                   vector<vector<pair<F, vector<F>>>> claims, F &K) {
  const int k = (int)arrays.size();
  const uint64_t n = arrays[0].size();
  std::vector<const uint64_t *> a(k);
  for (int i = 0; i < k; i++) a[i] = words(arrays[i].data());
  std::vector<F> points;
  int c = 0;
  for (auto &ci : claims)
    for (auto &cl : ci) {
      points.insert(points.end(), cl.second.begin(), cl.second.end());
      c++;
    }
  std::vector<F> sum_arr(n), sum_b(n), ch(c + k);
  uint64_t Kw[2];
  check(gbz_whir_aggregate_claims(ctx(), k, a.data(), n, c, words(points.data()), &process_prng(),
                                  words(sum_arr.data()), words(sum_b.data()), Kw, words(ch.data()), nullptr,
                                  GBZ_MEM_HOST),
        "aggregate_claims");
  // the reference adds into arr and b_aggr as given (resized to n)
  arr.resize(n, F(0));
  b_arr.resize(n, F(0));
  check(gbz_field_ops(ctx(), words(arr.data()), words(sum_arr.data()), n, words(arr.data()), nullptr, nullptr,
                      GBZ_MEM_HOST),
        "aggregate_claims");
  check(gbz_field_ops(ctx(), words(b_arr.data()), words(sum_b.data()), n, words(b_arr.data()), nullptr, nullptr,
                      GBZ_MEM_HOST),
        "aggregate_claims");
  K.real = Kw[0];
  K.img = Kw[1];
  return {vector<F>(ch.begin(), ch.begin() + c), vector<F>(ch.begin() + c, ch.end())};
}

// aggregate_commitments (Whir.cpp:547-606)
void aggregate_commitments(vector<F> &codeword, vector<vector<_hash>> &MT, vector<vector<F>> &codewords_aggr,
                           vector<vector<vector<_hash>>> &MT_aggr, vector<F> r, int rate) {
  (void)MT_aggr;  // its openings are verifier-side (the queries still advance the generator)
  if (conjectured_security) {
    std::fprintf(stderr, "aggregate_commitments: the GPU path uses the proven query count\n");
    std::exit(-1);
  }
  const int k = (int)codewords_aggr.size();
  const uint64_t n = codewords_aggr[0].size();
  std::vector<const uint64_t *> cw(k);
  for (int i = 0; i < k; i++) {
    if (codewords_aggr[i].size() != n) {
      std::printf("Incorrect codeword size %zu,%zu\n", (size_t)n, codewords_aggr[i].size());
      std::exit(-1);
    }
    cw[i] = words(codewords_aggr[i].data());
  }
  codeword.assign(n, F(0));
  const uint64_t leaves = n / whir_k;
  std::vector<_hash> levels(2 * leaves - 1);
  check(gbz_whir_aggregate_commitments(ctx(), k, cw.data(), n, words(r.data()), rate, whir_k, &process_prng(),
                                       words(codeword.data()), bytes(levels.data()), GBZ_MEM_HOST),
        "aggregate_commitments");
  MT.clear();
  assign_levels(MT, levels, leaves);
}

// ----------------------------------------------------------------- coPCS
// distributed_MT (coPCS.cpp:152-230), one rank's part: the column roots of
// its batched codewords, the tree over them, the all-to-all of zero hashes
// the reference performs, and on rank 0 the root tree over {root, 0, ...}.
void distributed_MT(vector<vector<F>> &Codeword, MT &Com, int N) {
  int rank = 0;
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  int batches = 0;
  while (batches < (int)Codeword.size() && !Codeword[batches].empty()) batches++;
  const uint64_t L = Codeword[0].size();
  std::vector<F> rows((size_t)batches * L);
  for (int i = 0; i < batches; i++) std::memcpy(&rows[(size_t)i * L], Codeword[i].data(), 16 * L);
  std::vector<_hash> levels(2 * L - 1);
  _hash leader;
  check(gbz_column_merkle(ctx(), words(rows.data()), batches, log2i(L), N, bytes(levels.data()), leader.arr,
                          GBZ_MEM_HOST),
        "distributed_MT");
  Com.Base_MT.clear();
  assign_levels(Com.Base_MT, levels, L);
  std::vector<uint8_t> recv(32 * N), send(32 * N, 0);
  MPI_Request req;
  MPI_Ialltoall(send.data(), 32, MPI_UINT8_T, recv.data(), 32, MPI_UINT8_T, MPI_COMM_WORLD, &req);
  com_rounds++;
  cm += 32 * N / 1024.0;
  MPI_Wait(&req, MPI_STATUS_IGNORE);
  if (rank == 0) {
    Com.Root_MT.assign(log2i(N) + 1, vector<_hash>());
    Com.Root_MT[0].assign(N, _hash());
    for (auto &h : Com.Root_MT[0]) std::memset(h.arr, 0, 32);
    Com.Root_MT[0][0] = Com.Base_MT.back()[0];
    merkle_tree::merkle_tree_prover::create_tree_blake(N, Com.Root_MT, 32, true);
  }
}
