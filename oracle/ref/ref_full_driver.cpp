// Driver over the reference's coPCS-side functions (links every reference
// translation unit except main.cpp; see the ref_full target of the Makefile).
//
// Test infrastructure only: it writes golden vectors for the C restatement
// in oracle/gbz_oracle.c.  Each subcommand calls the reference function
// named in its comment; where a reference function ends in an MPI exchange
// that needs more than one rank (the coSumcheck phase 1 and sumcheck_aggr),
// the driver calls the reference's building blocks in the same order up to
// that exchange and writes the local result.
//
//   ref_full multifold5 <logn> <logd> <seed>            RS_multifold5 (coPCS_utils.cpp:386)
//   ref_full lagrange <logd> <seed>                      compute_lagrange_coeff (utils.cpp:169)
//   ref_full encode <rows> <logrow> <rate> <log_ro> <seed>  Encode (coPCS.cpp:131)
//   ref_full colmerkle <rows> <logL> <N> <seed>          distributed_MT (coPCS.cpp:152)
//   ref_full shares <logM> <N> <seed> <privacy> <prng>   compute_secret_shares (MPI_utils.cpp:2738)
//   ref_full aggr <N> <len> <seed>                       sumcheck_aggr leader path (MPI_utils.cpp:2629-2644)
//   ref_full cophase1 <logn> <logd> <seed>               local part of quadratic/cubic phase 1 (coSumcheck.cpp:9-64,150-198)
//   ref_full cophase2 <logn> <logd> <seed>               quadratic/cubic phase 2 (coSumcheck.cpp:66-148, 201-213)
//   ref_full zcround <logm> <iter> <seed>                _zero_check_sumcheck_phase1/2 (coSumcheck_MPI.cpp:12-44)
//   ref_full bround <logm> <iter> <seed>                 _quadratic_batch_sumcheck_phase1/2 (coSumcheck_MPI.cpp:156-187)
//   ref_full cubicsc <logM> <offset> <seed> <prng>       _cubic_sumcheck, one party (Distributed_Sumcheck.cpp:1122)
//   ref_full quadsc <logM> <offset> <seed> <prng>        _quadratic_sumcheck, one party (Distributed_Sumcheck.cpp:204)
//   ref_full aggclaims <logn> <k> <c> <seed> <prng>      aggregate_claims (Whir.cpp:608)
//   ref_full aggarrays <logn> <k> <seed>                 aggregate_arrays (Whir.cpp:670)
//   ref_full aggcommit <logn> <k> <rate> <whir_k> <seed> <prng>  aggregate_commitments (Whir.cpp:547)
//   ref_full tensor <logrows> <N> <rate> <my_id> <p0> <p1>         tensor_eval_vector (coPCS.cpp:602)
//   ref_full phase3 <logrows> <N> <l> <rate> <my_id> <seed>        pcs_sumcheck_phase3 (coPCS.cpp:634)
//   ref_full encconc <logn> <rate0> <rate1> <degree> <seed>       encode_concatenated (coPCS.cpp:653)
//   ref_full batchopen <rate> <whir_k> <seed> <prng> <logn0> [<logn1> ...]  Whir_Batch_Open (Whir.cpp:706)
#include "Distributed_Sumcheck.h"
#include "Whir.h"
#include "coPCS.h"
#include "coPCS_utils.h"
#include "coSumcheck.h"
#include "config_pc.hpp"
#include "utils.hpp"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>
#include <vector>

using std::vector;

extern unsigned int rate_offset;  // coPCS.cpp:22
void Encode(vector<vector<F>> &Codeword, int N, vector<int> rate);
void quadratic_coSumcheck_phase2(vector<F> &p1, vector<F> &p2, vector<F> L, int d);
void cubic_coSumcheck_phase2(vector<F> &p1, vector<F> &p2, vector<F> &p3, vector<F> &b1, vector<F> L, int d);
cubic_poly _zero_check_sumcheck_phase1(int iter, F b, vector<F> &v1, vector<F> &v2, vector<F> &v3, vector<F> &beta1,
                                       vector<F> &r1, vector<F> &r2);
void _zero_check_sumcheck_phase2(int iter, F r, vector<F> &v1, vector<F> &v2, vector<F> &v3, vector<F> &beta1,
                                 vector<F> &r1, vector<F> &r2);
quadratic_poly _quadratic_batch_sumcheck_phase1(int iter, F b, vector<F> &v1, vector<F> &v2, vector<F> &v3,
                                                vector<F> &v4, vector<F> &r1, vector<F> &r2);
void _quadratic_batch_sumcheck_phase2(int iter, F r, vector<F> &v1, vector<F> &v2, vector<F> &v3, vector<F> &v4,
                                      vector<F> &r1, vector<F> &r2);
extern int sumcheck_offset;  // main.cpp:36
extern int my_id;                        // coPCS.cpp:19
extern vector<vector<int>> _rates;       // New_PCS.cpp:6
vector<F> tensor_eval_vector(vector<u32> point, int cols, int rows, int rate);
void pcs_sumcheck_phase3(vector<F> &B, vector<vector<u32>> queries, F s, int iter, int N);
void encode_concatenated(vector<F> &Commit_Data, vector<F> &C_prime, vector<vector<F>> &C, vector<int> rate,
                         int degree);
F aggregate_arrays(vector<F> &arr, vector<F> &b, vector<vector<F>> &arrays, vector<vector<F>> &B, vector<F> r1,
                   vector<F> r2);
void compute_secret_shares(vector<F> &v, vector<vector<F>> &v_shares, int N, int k, int _k, bool privacy_preserving);
vector<F> unpack_secret_share(vector<F> &secret, int _k, int k);

// Reference functions defined in Whir.cpp without a header declaration.
quadratic_poly whir_sumcheck_step1(vector<F> &arr, vector<F> &b);
void whir_sumcheck_step2(vector<F> &arr, vector<F> &b, F c);
vector<F> whir_query(vector<F> &codeword, vector<vector<_hash>> &MT, vector<F> r, vector<int> &queries, int rate);
vector<F> update_betas(vector<F> &b, vector<int> queries, int n);

// rand() as glibc defines it (random()), logging the values while
// g_log_rand is set: the queries aggregate_commitments draws internally
// (Whir.cpp:574-576) are otherwise not observable.
static bool g_log_rand = false;
static vector<int> g_rand_log;
extern "C" int rand(void) noexcept {
  int v = (int)random();
  if (g_log_rand) g_rand_log.push_back(v);
  return v;
}

static const uint64_t P61 = 2305843009213693951ULL;
struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  uint64_t base() {
    for (;;) {
      uint64_t v = next() >> 3;
      if (v != P61) return v;
    }
  }
  F ext() { F x; x.real = base(); x.img = base(); return x; }
  vector<F> vec(size_t n) { vector<F> v(n); for (auto &x : v) x = ext(); return v; }
};

static void put(const void *p, size_t n) { fwrite(p, 1, n, stdout); }
static void putFs(const vector<F> &v) { for (auto &x : v) { put(&x.real, 8); put(&x.img, 8); } }

static void put_prefix(const vector<F> &v, size_t n) {
  for (size_t i = 0; i < n; i++) { put(&v[i].real, 8); put(&v[i].img, 8); }
}

// Transcript records (the tags of the prover's transcript format).
enum { T_WHIR_POLY = 7, T_WHIR_CHALLENGE = 8, T_WHIR_ROOT = 9, T_WHIR_QUERIES = 10, T_WHIR_REPLIES = 11,
       T_WHIR_ANSWERS = 12, T_WHIR_PATHS = 13, T_WHIR_COMBINE = 14, T_WHIR_K = 15, T_FINAL_POLY = 16,
       T_FINAL_POINT = 17, T_FINAL_EVAL = 18, T_SCHEDULE = 19, T_AGGR_CHALLENGES = 20, T_AGGR_K = 21,
       T_AGGR_QUERIES = 22, T_AGGR_PATHS = 23, T_AGGR_ROOT = 24 };
static void rec(uint32_t tag, uint32_t count, const void *p, size_t unit) {
  put(&tag, 4);
  put(&count, 4);
  put(p, unit * count);
}
static void recF(uint32_t tag, const vector<F> &v) {
  uint32_t count = (uint32_t)v.size();
  put(&tag, 4);
  put(&count, 4);
  putFs(v);
}
static void rec_paths(uint32_t tag, vector<vector<_hash>> &MT, const vector<int> &q) {
  vector<uint8_t> paths;
  for (int qi : q) {
    vector<_hash> p = merkle_tree::merkle_tree_prover::open_tree_blake(MT, qi);
    for (auto &h : p) paths.insert(paths.end(), h.arr, h.arr + 32);
  }
  rec(tag, (uint32_t)(paths.size() / 32), paths.data(), 32);
}

// Whir_Batch_Open on k polynomials of sizes 2^logs[i] (non-increasing):
// arrays from the seed, betas = precompute_beta of seeded points, K0 the
// true claim of array 0, codewords from Whir_Commit_initial at the rate
// each array is merged at.  The loop of Whir.cpp:706-898 is followed step
// by step with the reference's own functions (whir_sumcheck_step1/2,
// F::_random, Whir_Commit_initial, whir_query, open_tree_blake,
// update_betas, aggregate_arrays, aggregate_commitments, evaluate_vector)
// so that every intermediate value can be written; then the unmodified
// Whir_Batch_Open runs on the same inputs from the same generator state and
// the generator positions after both runs must agree (exit code 3
// otherwise).  Output: the records, then the next random() value.
static int cmd_batchopen(int rate, int wk, uint64_t seed, unsigned prng, const vector<int> &logs) {
  const int k = (int)logs.size();
  SplitMix g(seed);
  vector<vector<F>> arrays(k), betas(k);
  for (int i = 0; i < k; i++) arrays[i] = g.vec(1u << logs[i]);
  for (int i = 0; i < k; i++) precompute_beta(g.vec(logs[i]), betas[i]);
  F K = F(0);
  for (size_t j = 0; j < arrays[0].size(); j++) K += arrays[0][j] * betas[0][j];
  const F K0 = K;
  whir_k = wk;
  vector<vector<F>> cws(k);
  vector<vector<vector<_hash>>> MTs(k);
  Whir_Commit_initial(arrays[0], cws[0], MTs[0], rate, wk);
  // schedule (Whir.cpp:731-752)
  vector<int> kappas, aggr, sizes;
  for (int i = 1; i < k; i++) sizes.push_back((int)arrays[i].size());
  {
    int size = (int)arrays[0].size();
    while (true) {
      if (!sizes.size() || size / whir_k > sizes[0]) {
        kappas.push_back(whir_k);
        size /= whir_k;
        aggr.push_back(0);
      } else {
        kappas.push_back(size / sizes[0]);
        int s = sizes[0];
        while (sizes.size() && sizes[0] == s) sizes.erase(sizes.begin());
        size /= kappas.back();
        aggr.push_back(1);
      }
      if (size <= whir_k) break;
    }
  }
  {
    vector<uint32_t> sch;
    for (size_t i = 0; i < kappas.size(); i++) {
      sch.push_back((uint32_t)kappas[i]);
      sch.push_back((uint32_t)aggr[i]);
    }
    rec(T_SCHEDULE, (uint32_t)sch.size(), sch.data(), 4);
  }
  srandom(prng);
  vector<F> arr = arrays[0], b = betas[0], codeword = cws[0];
  vector<vector<_hash>> MT = MTs[0];
  int next = 1, iter = 0, cur = rate;
  while (true) {
    whir_k = kappas[iter];
    const bool ag = aggr[iter] != 0;
    if (!ag || whir_k != 1) {
      // Whir_Iteration (Whir.cpp:354-386)
      const int kap = whir_k;
      vector<F> r;
      for (int i = 0; i < (int)log2(kap); i++) {
        quadratic_poly h = whir_sumcheck_step1(arr, b);
        if (K != h.eval(F(0)) + h.eval(F(1))) { fprintf(stderr, "whir sumcheck inconsistent\n"); return 2; }
        recF(T_WHIR_POLY, {h.a, h.b, h.c});
        r.push_back(F::_random());
        recF(T_WHIR_CHALLENGE, {r[i]});
        K = h.eval(r[i]);
        whir_sumcheck_step2(arr, b, r[i]);
      }
      vector<F> new_cw;
      vector<vector<_hash>> new_MT;
      Whir_Commit_initial(arr, new_cw, new_MT, 2 * cur, kap);
      rec(T_WHIR_ROOT, 1, new_MT.back()[0].arr, 32);
      vector<int> queries;
      vector<F> ys = whir_query(codeword, MT, r, queries, cur);
      {
        vector<uint32_t> q(queries.begin(), queries.end());
        rec(T_WHIR_QUERIES, (uint32_t)q.size(), q.data(), 4);
        vector<F> replies;
        for (int qi : queries)
          for (int j = 0; j < kap; j++) replies.push_back(codeword[qi + j * codeword.size() / kap]);
        recF(T_WHIR_REPLIES, replies);
        recF(T_WHIR_ANSWERS, ys);
        rec_paths(T_WHIR_PATHS, MT, queries);
      }
      for (size_t i = 0; i < queries.size(); i++) queries[i] = queries[i] * (kap * new_cw.size() / codeword.size());
      codeword = new_cw;
      MT = new_MT;
      vector<F> ch = update_betas(b, queries, (int)new_cw.size());
      recF(T_WHIR_COMBINE, ch);
      for (size_t i = 0; i < ch.size(); i++) K += ch[i] * ys[i];
      recF(T_WHIR_K, {K});
      cur *= 2;
    }
    iter++;
    if (ag) {
      vector<vector<F>> B_aggr{b}, arr_aggr{arr}, cw_aggr{codeword};
      vector<vector<vector<_hash>>> MT_aggr{MT};
      int g_cnt = 1;
      for (int i = next; i < k; i++)
        if (arrays[i].size() == arr.size()) {
          Whir_Commit_initial(arrays[i], cws[i], MTs[i], (int)(codeword.size() / arr.size()), wk);
          B_aggr.push_back(betas[i]);
          arr_aggr.push_back(arrays[i]);
          cw_aggr.push_back(cws[i]);
          MT_aggr.push_back(MTs[i]);
          g_cnt++;
        }
      next += g_cnt - 1;
      vector<F> ch1, ch2;
      for (int i = 0; i < g_cnt; i++) ch1.push_back(F::_random());
      for (int i = 0; i < g_cnt; i++) ch2.push_back(F::_random());
      ch1[0] = 1;
      ch2[0] = 1;
      {
        vector<F> both = ch1;
        both.insert(both.end(), ch2.begin(), ch2.end());
        recF(T_AGGR_CHALLENGES, both);
      }
      K = aggregate_arrays(arr, b, arr_aggr, B_aggr, ch2, ch1);
      recF(T_AGGR_K, {K});
      if (iter + 1 >= (int)kappas.size()) { fprintf(stderr, "schedule read past its end\n"); return 4; }
      whir_k = kappas[iter + 1];
      if (next < k && arr.size() / whir_k <= arrays[next].size()) whir_k = arr.size() / arrays[next].size();
      MT.clear();
      g_rand_log.clear();
      g_log_rand = true;
      aggregate_commitments(codeword, MT, cw_aggr, MT_aggr, ch2, (int)(cw_aggr[0].size() / arr_aggr[0].size()));
      g_log_rand = false;
      vector<int> qa;
      for (int v : g_rand_log) qa.push_back(v % (int)(codeword.size() / 4));
      {
        vector<uint32_t> q(qa.begin(), qa.end());
        rec(T_AGGR_QUERIES, (uint32_t)q.size(), q.data(), 4);
      }
      rec_paths(T_AGGR_PATHS, MT_aggr[0], qa);
      rec(T_AGGR_ROOT, 1, MT.back()[0].arr, 32);
    }
    if ((int)arr.size() <= whir_k) break;
  }
  recF(T_FINAL_POLY, arr);
  {
    F Kc = K;
    for (size_t i = 0; i < arr.size(); i++) Kc -= arr[i] * b[i];
    if (Kc != F(0)) { fprintf(stderr, "final claim inconsistent\n"); return 2; }
  }
  vector<F> rf;
  for (int i = 0; i < (int)log2(arr.size()); i++) rf.push_back(F::_random());
  recF(T_FINAL_POINT, rf);
  recF(T_FINAL_EVAL, {evaluate_vector(b, rf)});
  const int32_t nxt1 = (int32_t)random();

  // The unmodified Whir_Batch_Open on the same inputs (its prints go to stderr).
  for (int i = 1; i < k; i++)
    if (cws[i].empty()) Whir_Commit_initial(arrays[i], cws[i], MTs[i], rate, wk);
  vector<F> evals(k, F(0));
  evals[0] = K0;
  vector<vector<F>> a2 = arrays, c2 = cws, b2 = betas;
  vector<vector<vector<_hash>>> m2 = MTs;
  whir_k = wk;
  srandom(prng);
  fflush(stdout);
  int saved = dup(1);
  dup2(2, 1);
  Whir_Batch_Open(a2, c2, m2, evals, b2, rate, true);
  fflush(stdout);
  dup2(saved, 1);
  close(saved);
  const int32_t nxt2 = (int32_t)random();
  if (nxt1 != nxt2) { fprintf(stderr, "generator position differs from Whir_Batch_Open's\n"); return 3; }
  put(&nxt1, 4);
  return 0;
}

// delegate_protocol.cpp defines it without a header
vector<std::pair<F, vector<F>>> quadruple_sumcheck(F y, vector<F> &v1, vector<F> &v2, vector<F> &v3, vector<F> &v4,
                                                   F previous_r, double &ps);

int main(int argc, char **argv) {
  if (argc < 2) return 1;
  std::string c = argv[1];
  auto I = [&](int k) { return atoi(argv[k]); };
  auto U = [&](int k) { return (uint64_t)strtoull(argv[k], nullptr, 0); };
  if (c == "zcround" || c == "bround") {
    // inputs: six vectors of 2^logm, then b and r; output: the round
    // polynomial at iteration iter and the first m / 2^(iter+1) entries of
    // every vector after the phase-2 fold by r.
    int logm = I(2), iter = I(3);
    SplitMix g(U(4));
    vector<vector<F>> v(6);
    for (auto &x : v) x = g.vec(1u << logm);
    F b = g.ext(), r = g.ext();
    size_t half = (1u << logm) >> (iter + 1);
    if (c == "zcround") {
      cubic_poly H = _zero_check_sumcheck_phase1(iter, b, v[0], v[1], v[2], v[3], v[4], v[5]);
      putFs({H.a, H.b, H.c, H.d});
      _zero_check_sumcheck_phase2(iter, r, v[0], v[1], v[2], v[3], v[4], v[5]);
    } else {
      quadratic_poly H = _quadratic_batch_sumcheck_phase1(iter, b, v[0], v[1], v[2], v[3], v[4], v[5]);
      putFs({H.a, H.b, H.c});
      _quadratic_batch_sumcheck_phase2(iter, r, v[0], v[1], v[2], v[3], v[4], v[5]);
    }
    for (auto &x : v) put_prefix(x, half);
    return 0;
  }
  if (c == "quadsc4") {
    // quadruple_sumcheck (delegate_protocol.cpp:57-115): inputs v1..v4 of
    // 2^logm from the seed, y the true sum, the glibc generator seeded with
    // prng (five F::_random() draws per round, the last one the challenge).
    // Output: y, the four final values, the number of challenges, the challenges.
    int logm = I(2);
    SplitMix g(U(3));
    srandom((unsigned)U(4));
    size_t m = 1u << logm;
    vector<F> v1 = g.vec(m), v2 = g.vec(m), v3 = g.vec(m), v4 = g.vec(m);
    F y = F(0);
    for (size_t i = 0; i < m; i++) y = y + v1[i] * v2[i] * v3[i] * v4[i];
    putFs({y});
    double ps = 0;
    vector<std::pair<F, vector<F>>> res = quadruple_sumcheck(y, v1, v2, v3, v4, F(0), ps);
    for (auto &pr : res) putFs({pr.first});
    uint32_t nr = (uint32_t)res[0].second.size();
    put(&nr, 4);
    putFs(res[0].second);
    return 0;
  }
  if (c == "cubicsc" || c == "quadsc") {
    // One party (N = 1, the MPI stub's single rank): inputs v1, v2 (, v3)
    // of 2^logM and the party weight w from the seed; y is the true sum.
    // Output: y, the reply values, the number of challenges, the challenges.
    int logM = I(2);
    sumcheck_offset = I(3);
    SplitMix g(U(4));
    srandom((unsigned)U(5));
    size_t M = 1u << logM;
    bool cubic = c == "cubicsc";
    vector<F> v1 = g.vec(M), v2 = g.vec(M), v3 = cubic ? g.vec(M) : vector<F>();
    vector<F> w = {g.ext()};
    F y = F(0);
    for (size_t i = 0; i < M; i++) y = y + (cubic ? v1[i] * v2[i] * v3[i] : v1[i] * v2[i]);
    if (cubic) y = y * w[0];
    putFs({y});
    vector<std::pair<F, vector<F>>> res = cubic ? _cubic_sumcheck(y, v1, v2, v3, w, 1) : _quadratic_sumcheck(y, v1, v2, 1);
    for (auto &pr : res) putFs({pr.first});
    uint32_t nr = (uint32_t)res[0].second.size();
    put(&nr, 4);
    putFs(res[0].second);
    return 0;
  }
  if (c == "aggclaims") {
    // inputs from the seed: k arrays of 2^logn, c points of logn; output:
    // arr, b_aggr, K, the beta challenges then the array challenges
    int logn = I(2), k = I(3), nc = I(4);
    SplitMix g(U(5));
    srandom((unsigned)U(6));
    vector<vector<F>> arrays(k);
    for (auto &a : arrays) a = g.vec(1u << logn);
    vector<vector<std::pair<F, vector<F>>>> claims(1);
    for (int j = 0; j < nc; j++) claims[0].push_back({F(0), g.vec(logn)});
    vector<F> arr, b_aggr;
    F K;
    vector<vector<F>> ch = aggregate_claims(arrays, arr, b_aggr, claims, K);
    putFs(arr); putFs(b_aggr); putFs({K}); putFs(ch[0]); putFs(ch[1]);
    return 0;
  }
  if (c == "aggarrays") {
    // k arrays and k B vectors of 2^logn, r1, r2 (k each); arr = arrays[0],
    // b = B[0] on entry.  Output: arr, b, K.
    int logn = I(2), k = I(3);
    SplitMix g(U(4));
    vector<vector<F>> arrays(k), B(k);
    for (auto &a : arrays) a = g.vec(1u << logn);
    for (auto &a : B) a = g.vec(1u << logn);
    vector<F> r1 = g.vec(k), r2 = g.vec(k);
    vector<F> arr = arrays[0], b = B[0];
    F K = aggregate_arrays(arr, b, arrays, B, r1, r2);
    putFs(arr); putFs(b); putFs({K});
    return 0;
  }
  if (c == "aggcommit") {
    // k codewords of 2^logn and r (k); the query openings use the Merkle
    // tree of codeword 0.  Output: codeword, the new tree (levels, leaves
    // first), then the next random() value (the generator's position).
    int logn = I(2), k = I(3), rate = I(4);
    whir_k = I(5);
    SplitMix g(U(6));
    srandom((unsigned)U(7));
    vector<vector<F>> cws(k);
    for (auto &a : cws) a = g.vec(1u << logn);
    vector<F> r = g.vec(k);
    vector<vector<vector<_hash>>> MT_aggr(1);
    merkle_tree::merkle_tree_prover::MT_commit_Blake(cws[0].data(), MT_aggr[0], 1 << logn);
    vector<F> codeword;
    vector<vector<_hash>> MT;
    aggregate_commitments(codeword, MT, cws, MT_aggr, r, rate);
    putFs(codeword);
    for (auto &lv : MT)
      for (auto &h : lv) put(h.arr, 32);
    int32_t nxt = (int32_t)random();
    put(&nxt, 4);
    return 0;
  }
  if (c == "batchopen") {
    vector<int> logs;
    for (int i = 6; i < argc; i++) logs.push_back(I(i));
    if (logs.empty()) return 1;
    return cmd_batchopen(I(2), I(3), U(4), (unsigned)U(5), logs);
  }
  if (c == "tensor") {
    int logrows = I(2), N = I(3), rate = I(4);
    my_id = I(5);
    vector<u32> point = {(u32)U(6), (u32)U(7)};
    putFs(tensor_eval_vector(point, N / 2, 1 << logrows, rate));
    return 0;
  }
  if (c == "phase3") {
    // B (2^logrows) and s from the seed, then l queries (u32 pairs, written
    // out); output: the queries and the updated B.
    int logrows = I(2), N = I(3), l = I(4), rate = I(5);
    my_id = I(6);
    SplitMix g(U(7));
    const uint32_t rows = 1u << logrows;
    vector<F> B = g.vec(rows);
    F s = g.ext();
    vector<vector<u32>> queries(l, vector<u32>(2));
    for (auto &q : queries) {
      q[0] = (u32)(g.next() % (uint64_t)(N / 2));
      q[1] = (u32)(g.next() % ((uint64_t)rate * rows));
      put(q.data(), 8);
    }
    _rates = {{rate}, {rate}};
    pcs_sumcheck_phase3(B, queries, s, 0, N);
    putFs(B);
    return 0;
  }
  if (c == "encconc") {
    int logn = I(2), rate0 = I(3), rate1 = I(4), degree = I(5);
    SplitMix g(U(6));
    vector<F> data = g.vec(1u << logn), Cp;
    vector<vector<F>> C;
    encode_concatenated(data, Cp, C, {rate0, rate1}, degree);
    putFs(Cp);
    for (auto &row : C) putFs(row);
    return 0;
  }
  if (c == "multifold5") {
    int logn = I(2), logd = I(3);
    SplitMix g(U(4));
    vector<F> cw = g.vec(1u << logn), a = g.vec(1u << logd);
    putFs(cw); putFs(a);
    RS_multifold5(cw, a, 1 << logd);
    putFs(cw);
    return 0;
  }
  if (c == "lagrange") {
    int logd = I(2);
    SplitMix g(U(3));
    F r = g.ext();
    putFs({r});
    putFs(compute_lagrange_coeff(F(0), r, 1 << logd));
    return 0;
  }
  if (c == "encode") {
    int rows = I(2), logrow = I(3), rate = I(4), log_ro = I(5);
    SplitMix g(U(6));
    rate_offset = 1u << log_ro;
    vector<vector<F>> cw(32);
    for (int i = 0; i < rows; i++) cw[i] = g.vec(1u << logrow);
    for (int i = 0; i < rows; i++) putFs(cw[i]);
    Encode(cw, 0, {rate});
    for (int i = 0; i < rows; i++) putFs(cw[i]);
    return 0;
  }
  if (c == "colmerkle") {
    int rows = I(2), logL = I(3), N = I(4);
    SplitMix g(U(5));
    vector<vector<F>> cw(32);
    for (int i = 0; i < rows; i++) cw[i] = g.vec(1u << logL);
    for (int i = 0; i < rows; i++) putFs(cw[i]);
    MT com;
    distributed_MT(cw, com, N);
    uint32_t lv = (uint32_t)com.Base_MT.size();
    put(&lv, 4);
    for (auto &level : com.Base_MT) {
      uint32_t cnt = (uint32_t)level.size();
      put(&cnt, 4);
      for (auto &h : level) put(h.arr, 32);
    }
    put(com.Root_MT.back()[0].arr, 32);
    return 0;
  }
  if (c == "shares") {
    int logM = I(2), N = I(3);
    SplitMix g(U(4));
    bool privacy = I(5) != 0;
    srandom((unsigned)U(6));
    vector<F> v = g.vec(1u << logM);
    putFs(v);
    vector<vector<F>> shares;
    compute_secret_shares(v, shares, N, N / 4, N / 2, privacy);
    for (auto &s : shares) putFs(s);
    return 0;
  }
  if (c == "aggr") {
    int N = I(2), len = I(3);
    SplitMix g(U(4));
    vector<vector<F>> P(N);
    for (auto &p : P) p = g.vec(len);
    vector<F> b = g.vec(N / 4);
    for (auto &p : P) putFs(p);
    putFs(b);
    // sumcheck_aggr, leader path (MPI_utils.cpp:2631-2644)
    P = transpose(P);
    for (size_t i = 0; i < P.size(); i++) P[i] = unpack_secret_share(P[i], N, N);
    vector<F> poly(len, F(0));
    for (size_t i = 0; i < P.size(); i++)
      for (size_t j = 0; j < P[i].size() / 4; j++) poly[i] += b[j] * P[i][2 * j];
    putFs(poly);
    return 0;
  }
  if (c == "cophase1") {
    int logn = I(2), logd = I(3);
    SplitMix g(U(4));
    int n = 1 << logn, d = 1 << logd;
    vector<F> p1 = g.vec(n), p2 = g.vec(n), p3 = g.vec(n), b1 = g.vec(n);
    for (int k = 0; k < d; k++) p1[k] = F(0);  // block 0 of p1 is zero: skipped
    putFs(p1); putFs(p2); putFs(p3); putFs(b1);
    // quadratic_coSumcheck_phase1 local sum (coSumcheck.cpp:153-179)
    vector<F> H(2 * d, F(0));
    for (int j = 0; j < n / d; j++) {
      vector<F> h1(d), h2(d);
      bool zero = true;
      for (int k = 0; k < d; k++) { h1[k] = p1[j * d + k]; h2[k] = p2[j * d + k]; if (h1[k] != 0) zero = false; }
      if (zero) continue;
      fft(h1, logd, true); fft(h2, logd, true);
      h1.resize(2 * d, F(0)); h2.resize(2 * d, F(0));
      fft(h1, logd + 1, false); fft(h2, logd + 1, false);
      for (int k = 0; k < 2 * d; k++) H[k] += h1[k] * h2[k];
    }
    putFs(H);
    // cubic_coSumcheck_phase1 local sum (coSumcheck.cpp:11-46)
    vector<F> H4(4 * d, F(0));
    for (int j = 0; j < n / d; j++) {
      vector<F> h1(d), h2(d), h3(d), h4(d);
      bool zero = true;
      for (int k = 0; k < d; k++) {
        h1[k] = p1[j * d + k]; h2[k] = p2[j * d + k]; h3[k] = b1[j * d + k]; h4[k] = p3[j * d + k];
        if (h1[k] != 0) zero = false;
      }
      if (zero) continue;
      fft(h1, logd, true); fft(h2, logd, true); fft(h3, logd, true); fft(h4, logd, true);
      h1.resize(4 * d, F(0)); h2.resize(4 * d, F(0)); h3.resize(4 * d, F(0)); h4.resize(4 * d, F(0));
      fft(h1, logd + 2, false); fft(h2, logd + 2, false); fft(h3, logd + 2, false); fft(h4, logd + 2, false);
      for (int k = 0; k < 4 * d; k++) H4[k] += (h1[k] * h2[k] - h4[k]) * h3[k];
    }
    putFs(H4);
    return 0;
  }
  if (c == "cophase2") {
    int logn = I(2), logd = I(3);
    SplitMix g(U(4));
    int n = 1 << logn, d = 1 << logd;
    vector<F> p1 = g.vec(n), p2 = g.vec(n), p3 = g.vec(n), b1 = g.vec(n), L = g.vec(d);
    for (int k = 0; k < d; k++) { p1[d + k] = F(0); p3[2 * d + k] = F(0); }  // zero blocks
    putFs(p1); putFs(p2); putFs(p3); putFs(b1); putFs(L);
    vector<F> q1 = p1, q2 = p2;
    quadratic_coSumcheck_phase2(q1, q2, L, d);
    putFs(q1); putFs(q2);
    vector<F> c1 = p1, c2 = p2, c3 = p3, c4 = b1;
    cubic_coSumcheck_phase2(c1, c2, c3, c4, L, d);
    putFs(c1); putFs(c2); putFs(c3); putFs(c4);
    return 0;
  }
  fprintf(stderr, "unknown command %s\n", argv[1]);
  return 1;
}
