// Link-time capture of the reference prover's transcript, one log per rank.
//
// Test infrastructure only.  The multi-rank reference binary (target
// `pigeon_mpi` of oracle/ref/Makefile) is linked with `-Wl,--wrap=<symbol>`
// for each function below, so every call made from another translation unit
// reaches the __wrap_ function here, which calls the real one (__real_) and
// appends what went in and came out to the file  $MINIMPI_CAPTURE.<rank>.
// Nothing in the reference is modified: the wrappers only observe.
//
// Record format (little-endian): u32 tag (four ASCII characters), u32 count,
// then `count` payload units: 16-byte field elements {real, img} for field
// vectors, 32-byte digests for hashes, u32 words for index lists.
#include "config_pc.hpp"
#include "merkle_tree.h"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mpi.h>
#include <vector>

using std::pair;
using std::vector;
typedef vector<vector<_hash>> Levels;

namespace {

FILE *g_log = nullptr;
bool g_tried = false;

FILE *log_file() {
  if (g_tried) return g_log;
  g_tried = true;
  const char *p = std::getenv("MINIMPI_CAPTURE");
  if (!p || !*p) return nullptr;
  int rank = 0;
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  char path[4096];
  std::snprintf(path, sizeof path, "%s.%d", p, rank);
  g_log = std::fopen(path, "wb");
  if (!g_log) {
    std::fprintf(stderr, "capture: cannot open %s\n", path);
    std::exit(3);
  }
  return g_log;
}

void put(const char tag[4], uint32_t count, const void *data, size_t bytes) {
  FILE *f = log_file();
  if (!f) return;
  std::fwrite(tag, 1, 4, f);
  std::fwrite(&count, 4, 1, f);
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fflush(f);
}

void put_field(const char tag[4], const vector<F> &v) {
  vector<uint64_t> w(2 * v.size());
  for (size_t i = 0; i < v.size(); i++) {
    w[2 * i] = v[i].real;
    w[2 * i + 1] = v[i].img;
  }
  put(tag, (uint32_t)v.size(), w.data(), w.size() * 8);
}

void put_words(const char tag[4], const vector<uint32_t> &v) { put(tag, (uint32_t)v.size(), v.data(), v.size() * 4); }

void put_root(const char tag[4], int n, const Levels &levels) {
  uint8_t rec[36] = {0};
  uint32_t nn = (uint32_t)n;
  std::memcpy(rec, &nn, 4);
  if (!levels.empty() && !levels.back().empty()) std::memcpy(rec + 4, levels.back()[0].arr, 32);
  put(tag, 1, rec, sizeof rec);
}

}  // namespace

extern "C" {

// Fiat_Shamir.cpp:29  F hash_to_field(vector<F>)
F __real__Z13hash_to_fieldSt6vectorIN5virgo12fieldElementESaIS1_EE(vector<F> elements);
F __wrap__Z13hash_to_fieldSt6vectorIN5virgo12fieldElementESaIS1_EE(vector<F> elements) {
  put_field("H2FI", elements);
  F r = __real__Z13hash_to_fieldSt6vectorIN5virgo12fieldElementESaIS1_EE(elements);
  put_field("H2FO", vector<F>{r});
  return r;
}

// Fiat_Shamir.cpp:37  vector<vector<u32>> get_indexes(int l, int N, int M, int pos)
vector<vector<u32>> __real__Z11get_indexesiiii(int l, int N, int M, int pos);
vector<vector<u32>> __wrap__Z11get_indexesiiii(int l, int N, int M, int pos) {
  vector<vector<u32>> r = __real__Z11get_indexesiiii(l, N, M, pos);
  vector<uint32_t> w = {(uint32_t)l, (uint32_t)N, (uint32_t)M, (uint32_t)pos};
  for (auto &q : r) w.insert(w.end(), q.begin(), q.end());
  put_words("GIDX", w);
  return r;
}

// fieldElement.cpp:119  F::_random()
F __real__ZN5virgo12fieldElement7_randomEv();
F __wrap__ZN5virgo12fieldElement7_randomEv() {
  F r = __real__ZN5virgo12fieldElement7_randomEv();
  put_field("FRND", vector<F>{r});
  return r;
}

// glibc rand(), as called by the reference (query draws)
int __real_rand(void);
int __wrap_rand(void) {
  int r = __real_rand();
  put_words("RAND", vector<uint32_t>{(uint32_t)r});
  return r;
}

// MPI_utils.cpp:2787  secret_share_coefficients(vector<F>& w, int M, int N, int _k, int k)
void __real__Z25secret_share_coefficientsRSt6vectorIN5virgo12fieldElementESaIS1_EEiiii(vector<F> &w, int M, int N,
                                                                                       int _k, int k);
void __wrap__Z25secret_share_coefficientsRSt6vectorIN5virgo12fieldElementESaIS1_EEiiii(vector<F> &w, int M, int N,
                                                                                       int _k, int k) {
  __real__Z25secret_share_coefficientsRSt6vectorIN5virgo12fieldElementESaIS1_EEiiii(w, M, N, _k, k);
  put_field("SHRS", w);
}

// MPI_utils.cpp:341  vector<F> pcs_sumcheck_aggr(vector<F>& poly, int N)
vector<F> __real__Z17pcs_sumcheck_aggrRSt6vectorIN5virgo12fieldElementESaIS1_EEi(vector<F> &poly, int N);
vector<F> __wrap__Z17pcs_sumcheck_aggrRSt6vectorIN5virgo12fieldElementESaIS1_EEi(vector<F> &poly, int N) {
  put_field("PAGI", poly);
  vector<F> r = __real__Z17pcs_sumcheck_aggrRSt6vectorIN5virgo12fieldElementESaIS1_EEi(poly, N);
  put_field("PAGO", r);
  return r;
}

// merkle_tree.cpp:195  MT_commit_Blake(F*, levels&, int N)
void __real__ZN11merkle_tree18merkle_tree_prover15MT_commit_BlakeEPN5virgo12fieldElementERSt6vectorIS4_I5_hashSaIS5_EESaIS7_EEi(
    F *p, Levels &levels, int n);
void __wrap__ZN11merkle_tree18merkle_tree_prover15MT_commit_BlakeEPN5virgo12fieldElementERSt6vectorIS4_I5_hashSaIS5_EESaIS7_EEi(
    F *p, Levels &levels, int n) {
  __real__ZN11merkle_tree18merkle_tree_prover15MT_commit_BlakeEPN5virgo12fieldElementERSt6vectorIS4_I5_hashSaIS5_EESaIS7_EEi(
      p, levels, n);
  put_root("MTCB", n, levels);
}

// merkle_tree.cpp:267  create_tree_blake(int size, levels&, int, bool)
void __real__ZN11merkle_tree18merkle_tree_prover17create_tree_blakeEiRSt6vectorIS1_I5_hashSaIS2_EESaIS4_EEib(
    int n, Levels &levels, int sz, bool alloc);
void __wrap__ZN11merkle_tree18merkle_tree_prover17create_tree_blakeEiRSt6vectorIS1_I5_hashSaIS2_EESaIS4_EEib(
    int n, Levels &levels, int sz, bool alloc) {
  __real__ZN11merkle_tree18merkle_tree_prover17create_tree_blakeEiRSt6vectorIS1_I5_hashSaIS2_EESaIS4_EEib(n, levels, sz,
                                                                                                        alloc);
  put_root("CTRB", n, levels);
}

// MPI_utils.cpp:58  send_pcs_data(arr, B, codeword, total_arr, total_B, C, N): the leader's final gather
void __real__Z13send_pcs_dataRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_RS_IS3_SaIS3_EES7_S7_i(
    vector<F> &arr, vector<F> &B, vector<F> &cw, vector<vector<F>> &ta, vector<vector<F>> &tb, vector<vector<F>> &C,
    int N);
void __wrap__Z13send_pcs_dataRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_RS_IS3_SaIS3_EES7_S7_i(
    vector<F> &arr, vector<F> &B, vector<F> &cw, vector<vector<F>> &ta, vector<vector<F>> &tb, vector<vector<F>> &C,
    int N) {
  put_field("SPDA", arr);
  put_field("SPDB", B);
  put_field("SPDC", cw);
  __real__Z13send_pcs_dataRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_RS_IS3_SaIS3_EES7_S7_i(arr, B, cw, ta, tb, C,
                                                                                                  N);
}

// Whir.cpp:158  Whir_Commit_initial(arr, codeword, MT, rate, k)
void __real__Z19Whir_Commit_initialRSt6vectorIN5virgo12fieldElementESaIS1_EES4_RS_IS_I5_hashSaIS5_EESaIS7_EEii(
    vector<F> &arr, vector<F> &cw, Levels &mt, int rate, int k);
void __wrap__Z19Whir_Commit_initialRSt6vectorIN5virgo12fieldElementESaIS1_EES4_RS_IS_I5_hashSaIS5_EESaIS7_EEii(
    vector<F> &arr, vector<F> &cw, Levels &mt, int rate, int k) {
  put_field("WCIA", arr);
  __real__Z19Whir_Commit_initialRSt6vectorIN5virgo12fieldElementESaIS1_EES4_RS_IS_I5_hashSaIS5_EESaIS7_EEii(arr, cw, mt,
                                                                                                            rate, k);
  put_root("WCIR", rate * 1000 + k, mt);
}

// MPI_utils.cpp:483  F F_ip(data, v1, v2, k, _k, N): the opening claim K
F __real__Z4F_ipRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_iii(vector<F> &d, vector<F> &v1, vector<F> &v2, int k,
                                                                   int _k, int N);
F __wrap__Z4F_ipRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_iii(vector<F> &d, vector<F> &v1, vector<F> &v2, int k,
                                                                   int _k, int N) {
  F r = __real__Z4F_ipRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_iii(d, v1, v2, k, _k, N);
  put_field("FIPK", vector<F>{r});
  return r;
}

// MPI_utils.cpp  get_segments(y, segments, queries, l, N, degree): the leader's gather of every
// party's folded values and segments in delegate_checks
void __real__Z12get_segmentsRSt6vectorIN5virgo12fieldElementESaIS1_EERS_IS3_SaIS3_EERS_IS_IjSaIjEESaIS9_EEiii(
    vector<F> &y, vector<vector<F>> &seg, vector<vector<u32>> &q, int l, int N, int d);
void __wrap__Z12get_segmentsRSt6vectorIN5virgo12fieldElementESaIS1_EERS_IS3_SaIS3_EERS_IS_IjSaIjEESaIS9_EEiii(
    vector<F> &y, vector<vector<F>> &seg, vector<vector<u32>> &q, int l, int N, int d) {
  put_field("GSYI", y);
  __real__Z12get_segmentsRSt6vectorIN5virgo12fieldElementESaIS1_EERS_IS3_SaIS3_EERS_IS_IjSaIjEESaIS9_EEiii(y, seg, q, l,
                                                                                                          N, d);
  vector<F> flat;
  for (auto &s : seg) flat.insert(flat.end(), s.begin(), s.end());
  vector<uint32_t> qs;
  for (auto &x : q) qs.insert(qs.end(), x.begin(), x.end());
  put_field("GSYO", y);
  put_field("GSSG", flat);
  put_words("GSQU", qs);
}

// MPI_utils.cpp:2604  vector<F> sumcheck_aggr(vector<F>& poly, vector<F>& b, int N)
vector<F> __real__Z13sumcheck_aggrRSt6vectorIN5virgo12fieldElementESaIS1_EES4_i(vector<F> &poly, vector<F> &b, int N);
vector<F> __wrap__Z13sumcheck_aggrRSt6vectorIN5virgo12fieldElementESaIS1_EES4_i(vector<F> &poly, vector<F> &b, int N) {
  put_field("SAGI", poly);
  vector<F> r = __real__Z13sumcheck_aggrRSt6vectorIN5virgo12fieldElementESaIS1_EES4_i(poly, b, N);
  put_field("SAGO", r);
  return r;
}

// MPI_utils.cpp:2672  vector<vector<F>> send_final_sumcheck_poly(vector<F> s, int N)
vector<vector<F>> __real__Z24send_final_sumcheck_polySt6vectorIN5virgo12fieldElementESaIS1_EEi(vector<F> s, int N);
vector<vector<F>> __wrap__Z24send_final_sumcheck_polySt6vectorIN5virgo12fieldElementESaIS1_EEi(vector<F> s, int N) {
  put_field("SFSI", s);
  vector<vector<F>> H = __real__Z24send_final_sumcheck_polySt6vectorIN5virgo12fieldElementESaIS1_EEi(s, N);
  vector<F> flat;
  for (auto &h : H) flat.insert(flat.end(), h.begin(), h.end());
  put_field("SFSO", flat);
  return H;
}

// The leader's side of PCS_open_new after the parties' rounds: the
// delegation proofs of delegate_checks and the final WHIR opening
// (coPCS.cpp:773-831, 1697-1754).  A claim is recorded as its value then its
// point.
void put_claim(const char tag[4], const pair<F, vector<F>> &c) {
  vector<F> v{c.first};
  v.insert(v.end(), c.second.begin(), c.second.end());
  put_field(tag, v);
}

// delegate_protocol.cpp:147  prove_multi_folding(segments, L, y, queries, n, ps)
pair<F, vector<F>> __real__Z19prove_multi_foldingRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES3_S3_S_IS_IjSaIjEESaIS8_EEiRd(
    vector<vector<F>> &seg, vector<F> L, vector<F> y, vector<vector<u32>> q, int n, double &ps);
pair<F, vector<F>> __wrap__Z19prove_multi_foldingRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES3_S3_S_IS_IjSaIjEESaIS8_EEiRd(
    vector<vector<F>> &seg, vector<F> L, vector<F> y, vector<vector<u32>> q, int n, double &ps) {
  pair<F, vector<F>> c =
      __real__Z19prove_multi_foldingRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES3_S3_S_IS_IjSaIjEESaIS8_EEiRd(
          seg, L, y, q, n, ps);
  put_claim("PMFC", c);
  return c;
}

// delegate_protocol.cpp:369  prove_extension(segments, extended, o, queries, rate, ps)
pair<F, vector<F>> __real__Z15prove_extensionRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES6_S3_S_IiSaIiEEiRd(
    vector<vector<F>> &seg, vector<vector<F>> &ext, vector<F> o, vector<int> q, int rate, double &ps);
pair<F, vector<F>> __wrap__Z15prove_extensionRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES6_S3_S_IiSaIiEEiRd(
    vector<vector<F>> &seg, vector<vector<F>> &ext, vector<F> o, vector<int> q, int rate, double &ps) {
  put_field("PEXO", o);
  pair<F, vector<F>> c =
      __real__Z15prove_extensionRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES6_S3_S_IiSaIiEEiRd(seg, ext, o, q,
                                                                                                         rate, ps);
  put_claim("PEXC", c);
  return c;
}

// delegate_protocol.cpp:431  delegate_beta_eval(r, L, y, offset, ps): the claim y it starts from
F __real__Z18delegate_beta_evalSt6vectorIN5virgo12fieldElementESaIS1_EES_IS3_SaIS3_EES1_iRd(vector<F> r,
                                                                                           vector<vector<F>> L, F y,
                                                                                           int offset, double &ps);
F __wrap__Z18delegate_beta_evalSt6vectorIN5virgo12fieldElementESaIS1_EES_IS3_SaIS3_EES1_iRd(vector<F> r,
                                                                                           vector<vector<F>> L, F y,
                                                                                           int offset, double &ps) {
  put_field("DBEY", vector<F>{y});
  F out = __real__Z18delegate_beta_evalSt6vectorIN5virgo12fieldElementESaIS1_EES_IS3_SaIS3_EES1_iRd(r, L, y, offset, ps);
  put("DBEE", 0, nullptr, 0);
  return out;
}

// Whir.cpp:608  aggregate_claims(arrays, arr, b_aggr, claims, K): the aggregated claim K and the
// challenges (beta weights, then array weights)
vector<vector<F>> __real__Z16aggregate_claimsRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EERS3_S7_S_IS_ISt4pairIS1_S3_ESaIS9_EESaISB_EERS1_(
    vector<vector<F>> &arrays, vector<F> &arr, vector<F> &b, vector<vector<pair<F, vector<F>>>> claims, F &K);
vector<vector<F>> __wrap__Z16aggregate_claimsRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EERS3_S7_S_IS_ISt4pairIS1_S3_ESaIS9_EESaISB_EERS1_(
    vector<vector<F>> &arrays, vector<F> &arr, vector<F> &b, vector<vector<pair<F, vector<F>>>> claims, F &K) {
  vector<vector<F>> ch =
      __real__Z16aggregate_claimsRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EERS3_S7_S_IS_ISt4pairIS1_S3_ESaIS9_EESaISB_EERS1_(
          arrays, arr, b, claims, K);
  put_field("AGCK", vector<F>{K});
  vector<F> flat;
  for (auto &c : ch) flat.insert(flat.end(), c.begin(), c.end());
  put_field("AGCC", flat);
  return ch;
}

// Whir.cpp:469  _Whir_Open(arr, codeword, MT, b, claims, challenges, K, rate, Verify): the final claim
pair<F, vector<F>> __real__Z10_Whir_OpenRSt6vectorIN5virgo12fieldElementESaIS1_EES4_RS_IS_I5_hashSaIS5_EESaIS7_EES4_S_IS_ISt4pairIS1_S3_ESaISC_EESaISE_EES3_S1_ib(
    vector<F> &arr, vector<F> &cw, Levels &mt, vector<F> &b, vector<vector<pair<F, vector<F>>>> claims,
    vector<F> challenges, F K, int rate, bool verify);
pair<F, vector<F>> __wrap__Z10_Whir_OpenRSt6vectorIN5virgo12fieldElementESaIS1_EES4_RS_IS_I5_hashSaIS5_EESaIS7_EES4_S_IS_ISt4pairIS1_S3_ESaISC_EESaISE_EES3_S1_ib(
    vector<F> &arr, vector<F> &cw, Levels &mt, vector<F> &b, vector<vector<pair<F, vector<F>>>> claims,
    vector<F> challenges, F K, int rate, bool verify) {
  put("WOPB", 0, nullptr, 0);
  pair<F, vector<F>> c =
      __real__Z10_Whir_OpenRSt6vectorIN5virgo12fieldElementESaIS1_EES4_RS_IS_I5_hashSaIS5_EESaIS7_EES4_S_IS_ISt4pairIS1_S3_ESaISC_EESaISE_EES3_S1_ib(
          arr, cw, mt, b, claims, challenges, K, rate, verify);
  put_claim("WOPC", c);
  return c;
}

// utils.cpp:1201  evaluate_vector(v, r): its length and value
F __real__Z15evaluate_vectorSt6vectorIN5virgo12fieldElementESaIS1_EES3_(vector<F> v, vector<F> r);
F __wrap__Z15evaluate_vectorSt6vectorIN5virgo12fieldElementESaIS1_EES3_(vector<F> v, vector<F> r) {
  const uint32_t n = (uint32_t)v.size();
  F out = __real__Z15evaluate_vectorSt6vectorIN5virgo12fieldElementESaIS1_EES3_(v, r);
  F len;
  len.real = n;
  len.img = 0;
  put_field("EVLV", vector<F>{len, out});
  return out;
}

}  // extern "C"
