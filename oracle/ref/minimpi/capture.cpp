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
#include "coPCS.h"
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
// glibc generator: the seed of the last srand/srandom (1 = never seeded) and
// the draws since then
uint32_t g_seed = 1;
uint64_t g_draws = 0;

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
  g_draws++;
  put_words("RAND", vector<uint32_t>{(uint32_t)r});
  return r;
}

// glibc random(), srand(), srandom(): counted, not logged (rand() and
// random() advance the same generator), so that a record can say how far
// the generator stood from its last seeding when a dealing step began.
long __real_random(void);
long __wrap_random(void) {
  g_draws++;
  return __real_random();
}
void __real_srand(unsigned s);
void __wrap_srand(unsigned s) {
  g_seed = s;
  g_draws = 0;
  __real_srand(s);
}
void __real_srandom(unsigned s);
void __wrap_srandom(unsigned s) {
  g_seed = s;
  g_draws = 0;
  __real_srandom(s);
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

// delegate_protocol.cpp:603  delegate_lagrange_eval(L1, L2, y, offset, queries, ps): the claim it starts from
F __real__Z22delegate_lagrange_evalSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES5_S1_iiRd(
    vector<vector<F>> L1, vector<vector<F>> L2, F y, int offset, int queries, double &ps);
F __wrap__Z22delegate_lagrange_evalSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES5_S1_iiRd(
    vector<vector<F>> L1, vector<vector<F>> L2, F y, int offset, int queries, double &ps) {
  put_field("DLEY", vector<F>{y});
  F out = __real__Z22delegate_lagrange_evalSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES5_S1_iiRd(
      L1, L2, y, offset, queries, ps);
  put("DLEE", 0, nullptr, 0);
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

// ---- the R1CS front end's first and second sumcheck phases (pigeon 1:
// coPIOP_prove, coPIOP.cpp:1382-1648).  Recorded only when
// MINIMPI_CAPTURE_PIOP is set, so the other captures keep their streams.
}  // extern "C"

extern vector<vector<F>> ip_vec;                         // coSumcheck.cpp:230
extern vector<F> sumcheck1_ip, sumcheck2_ip, sumcheck3_ip;  // coPIOP.cpp:57
extern F prev_challenge;                                 // Fiat_Shamir.cpp:5
extern int logm, logn, mask_l;                           // coPIOP.cpp:19,45

namespace {

bool piop_on() {
  static int on = -1;
  if (on < 0) on = std::getenv("MINIMPI_CAPTURE_PIOP") != nullptr;
  return on == 1;
}

// where the generator stood: {point, seed, draws since the seed (low, high)}
void put_draws(uint32_t point) {
  put_words("RNCT", vector<uint32_t>{point, g_seed, (uint32_t)g_draws, (uint32_t)(g_draws >> 32)});
}

vector<F> flat(const vector<vector<F>> &v) {
  vector<F> out;
  for (auto &x : v) out.insert(out.end(), x.begin(), x.end());
  return out;
}

// claims as their values then points, with the point lengths beside
void put_claims(const char tv[4], const char tn[4], const vector<pair<F, vector<F>>> &c) {
  vector<F> v;
  vector<uint32_t> n;
  for (auto &x : c) {
    v.push_back(x.first);
    v.insert(v.end(), x.second.begin(), x.second.end());
    n.push_back((uint32_t)x.second.size());
  }
  put_field(tv, v);
  put_words(tn, n);
}

void put_ints(const char tag[4], const vector<int> &v) {
  vector<uint32_t> w(v.begin(), v.end());
  put_words(tag, w);
}

}  // namespace

extern "C" {

// MPI_utils.cpp:2813  distribute_proving_data(vL, vR, vO, w, N, M, _k, k, cir_type)
void __real__Z23distribute_proving_dataRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_S4_iiiii(
    vector<F> &vL, vector<F> &vR, vector<F> &vO, vector<F> &w, int N, int M, int _k, int k, int t);
void __wrap__Z23distribute_proving_dataRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_S4_iiiii(
    vector<F> &vL, vector<F> &vR, vector<F> &vO, vector<F> &w, int N, int M, int _k, int k, int t) {
  if (piop_on()) {
    put_draws(1);
    put_words("PLMN", vector<uint32_t>{(uint32_t)logm, (uint32_t)logn, (uint32_t)mask_l});
  }
  __real__Z23distribute_proving_dataRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_S4_iiiii(vL, vR, vO, w, N, M, _k, k,
                                                                                           t);
  if (piop_on()) {
    put_field("DPDL", vL);
    put_field("DPDR", vR);
    put_field("DPDO", vO);
    put_field("DPDW", w);
  }
}

// MPI_utils.cpp:3633  generate_sumcheck_randomness(R, degrees1, degrees2, N)
F __real__Z28generate_sumcheck_randomnessRSt6vectorIS_IS_IN5virgo12fieldElementESaIS1_EESaIS3_EESaIS5_EES_IiSaIiEESA_i(
    vector<vector<vector<F>>> &R, vector<int> d1, vector<int> d2, int N);
F __wrap__Z28generate_sumcheck_randomnessRSt6vectorIS_IS_IN5virgo12fieldElementESaIS1_EESaIS3_EESaIS5_EES_IiSaIiEESA_i(
    vector<vector<vector<F>>> &R, vector<int> d1, vector<int> d2, int N) {
  if (piop_on()) put_draws(2);
  F K = __real__Z28generate_sumcheck_randomnessRSt6vectorIS_IS_IN5virgo12fieldElementESaIS1_EESaIS3_EESaIS5_EES_IiSaIiEESA_i(
      R, d1, d2, N);
  if (piop_on()) {
    put_field("GSR0", flat(R[0]));
    put_field("GSR1", flat(R[1]));
    put_field("GSRK", vector<F>{K});
  }
  return K;
}

// MPI_utils.cpp:2868  setup_randomness(R, N, _k, k, size)
void __real__Z16setup_randomnessRSt6vectorIN5virgo12fieldElementESaIS1_EEiiii(vector<F> &R, int N, int _k, int k,
                                                                              int size);
void __wrap__Z16setup_randomnessRSt6vectorIN5virgo12fieldElementESaIS1_EEiiii(vector<F> &R, int N, int _k, int k,
                                                                              int size) {
  if (piop_on()) {
    put_draws(3);
    put_words("SURN", vector<uint32_t>{(uint32_t)size});
  }
  __real__Z16setup_randomnessRSt6vectorIN5virgo12fieldElementESaIS1_EEiiii(R, N, _k, k, size);
  if (piop_on()) put_field("SURO", R);
}

// coPCS.cpp  PCS_commit(C, codeword, Commit_data, witness, randomness, rate, N)
void __real__Z10PCS_commitR2MTRSt6vectorIS1_IN5virgo12fieldElementESaIS3_EESaIS5_EES8_RS5_S9_S1_IS1_IiSaIiEESaISB_EEi(
    MT &C, vector<vector<F>> &cw, vector<vector<F>> &cd, vector<F> &w, vector<F> &rnd, vector<vector<int>> rate, int N);
void __wrap__Z10PCS_commitR2MTRSt6vectorIS1_IN5virgo12fieldElementESaIS3_EESaIS5_EES8_RS5_S9_S1_IS1_IiSaIiEESaISB_EEi(
    MT &C, vector<vector<F>> &cw, vector<vector<F>> &cd, vector<F> &w, vector<F> &rnd, vector<vector<int>> rate, int N) {
  if (piop_on()) {
    put_draws(4);
    put_field("PCWI", w);
    put_field("PCRI", rnd);
  }
  __real__Z10PCS_commitR2MTRSt6vectorIS1_IN5virgo12fieldElementESaIS3_EESaIS5_EES8_RS5_S9_S1_IS1_IiSaIiEESaISB_EEi(
      C, cw, cd, w, rnd, rate, N);
  if (piop_on()) {
    vector<uint32_t> rows;
    for (auto &r : cd) rows.push_back((uint32_t)r.size());
    put_words("PCCN", rows);
    put_field("PCCD", flat(cd));
    put_field("PCFS", vector<F>{prev_challenge});
  }
}

// MPI_utils.cpp:3620  compute_Kr(R, b, N)
F __real__Z10compute_KrRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES3_i(vector<vector<F>> &R, vector<F> b,
                                                                                int N);
F __wrap__Z10compute_KrRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES3_i(vector<vector<F>> &R, vector<F> b,
                                                                                int N) {
  F K = __real__Z10compute_KrRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES3_i(R, b, N);
  if (piop_on()) put_field("CKRO", vector<F>{K});
  return K;
}

// coSumcheck.cpp:335  cubic_coSumcheck(p1, p2, p3, r1, r2, R, K, K_r, degrees, N, ps)
vector<pair<F, vector<F>>> __real__Z16cubic_coSumcheckRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_S4_S4_S_IS3_SaIS3_EES1_S1_S_IiSaIiEEiRd(
    vector<F> &p1, vector<F> &p2, vector<F> &p3, vector<F> &r1, vector<F> &r2, vector<vector<F>> R, F K, F K_r,
    vector<int> degrees, int N, double &ps);
vector<pair<F, vector<F>>> __wrap__Z16cubic_coSumcheckRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_S4_S4_S_IS3_SaIS3_EES1_S1_S_IiSaIiEEiRd(
    vector<F> &p1, vector<F> &p2, vector<F> &p3, vector<F> &r1, vector<F> &r2, vector<vector<F>> R, F K, F K_r,
    vector<int> degrees, int N, double &ps) {
  if (piop_on()) {
    put_field("CBP1", p1);
    put_field("CBP2", p2);
    put_field("CBP3", p3);
    put_field("CBR1", r1);
    put_field("CBR2", r2);
    put_field("CBRR", flat(R));
    put_field("CBKK", vector<F>{K, K_r});
    put_ints("CBDG", degrees);
  }
  vector<pair<F, vector<F>>> c =
      __real__Z16cubic_coSumcheckRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S4_S4_S4_S_IS3_SaIS3_EES1_S1_S_IiSaIiEEiRd(
          p1, p2, p3, r1, r2, R, K, K_r, degrees, N, ps);
  if (piop_on()) {
    put_claims("CBCL", "CBCN", c);
    put_field("CBIP", flat(ip_vec));
  }
  return c;
}

// Distributed_Sumcheck.cpp:2283  _reduce_R1CS_matrixes_multivariate(size, r, RA, RB, RC, degrees, N)
void __real__Z34_reduce_R1CS_matrixes_multivariatemSt6vectorIN5virgo12fieldElementESaIS1_EERS3_S4_S4_S_IiSaIiEEi(
    size_t size, vector<F> r, vector<F> &RA, vector<F> &RB, vector<F> &RC, vector<int> degrees, int N);
void __wrap__Z34_reduce_R1CS_matrixes_multivariatemSt6vectorIN5virgo12fieldElementESaIS1_EERS3_S4_S4_S_IiSaIiEEi(
    size_t size, vector<F> r, vector<F> &RA, vector<F> &RB, vector<F> &RC, vector<int> degrees, int N) {
  if (piop_on()) {
    put_field("RDIR", r);
    put_ints("RDDG", degrees);
    // the first sumcheck's inner-product vector, final after prove_phase1
    put_field("SIP1", sumcheck1_ip);
  }
  __real__Z34_reduce_R1CS_matrixes_multivariatemSt6vectorIN5virgo12fieldElementESaIS1_EERS3_S4_S4_S_IiSaIiEEi(
      size, r, RA, RB, RC, degrees, N);
  if (piop_on()) {
    put_field("RDRA", RA);
    put_field("RDRB", RB);
    put_field("RDRC", RC);
  }
}

// Distributed_Sumcheck.cpp:2352  secret_share_vector(v, _k, k, N)
void __real__Z19secret_share_vectorRSt6vectorIN5virgo12fieldElementESaIS1_EEiii(vector<F> &v, int _k, int k, int N);
void __wrap__Z19secret_share_vectorRSt6vectorIN5virgo12fieldElementESaIS1_EEiii(vector<F> &v, int _k, int k, int N) {
  if (piop_on()) put_field("SSVI", v);
  __real__Z19secret_share_vectorRSt6vectorIN5virgo12fieldElementESaIS1_EEiii(v, _k, k, N);
  if (piop_on()) put_field("SSVO", v);
}

// coSumcheck.cpp:233  quadratic_coSumcheck(p1, p2, R, K, K_r, degrees, N, ps)
vector<pair<F, vector<F>>> __real__Z20quadratic_coSumcheckRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S_IS3_SaIS3_EES1_S1_S_IiSaIiEEiRd(
    vector<F> &p1, vector<F> &p2, vector<vector<F>> R, F K, F K_r, vector<int> degrees, int N, double &ps);
vector<pair<F, vector<F>>> __wrap__Z20quadratic_coSumcheckRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S_IS3_SaIS3_EES1_S1_S_IiSaIiEEiRd(
    vector<F> &p1, vector<F> &p2, vector<vector<F>> R, F K, F K_r, vector<int> degrees, int N, double &ps) {
  if (piop_on()) {
    put_field("QDP1", p1);
    put_field("QDP2", p2);
    put_field("QDRR", flat(R));
    put_field("QDKK", vector<F>{K, K_r});
    put_ints("QDDG", degrees);
  }
  vector<pair<F, vector<F>>> c =
      __real__Z20quadratic_coSumcheckRSt6vectorIN5virgo12fieldElementESaIS1_EES4_S_IS3_SaIS3_EES1_S1_S_IiSaIiEEiRd(
          p1, p2, R, K, K_r, degrees, N, ps);
  if (piop_on()) {
    put_claims("QDCL", "QDCN", c);
    put_field("QDIP", flat(ip_vec));
  }
  return c;
}

// MPI_utils.cpp  send_performance_data(v, N): called after every phase of
// coPIOP_prove; after the second sumcheck it sees prove_phase2's outputs
vector<double> __real__Z21send_performance_dataSt6vectorIdSaIdEEi(vector<double> v, int N);
vector<double> __wrap__Z21send_performance_dataSt6vectorIdSaIdEEi(vector<double> v, int N) {
  if (piop_on()) {
    put_field("SIP2", sumcheck2_ip);
    put_field("SIP3", sumcheck3_ip);
  }
  return __real__Z21send_performance_dataSt6vectorIdSaIdEEi(v, N);
}

// coPCS.cpp:369  distributed_commit_batch(Com, N): every commitment's local
// root, then the leader's (the distributed PCS opening's batched and FRI
// commitments, distributed_PCS.cpp:357, 632)
void __real__Z24distributed_commit_batchRSt6vectorI2MTSaIS0_EEi(vector<MT> &Com, int N);
void __wrap__Z24distributed_commit_batchRSt6vectorI2MTSaIS0_EEi(vector<MT> &Com, int N) {
  __real__Z24distributed_commit_batchRSt6vectorI2MTSaIS0_EEi(Com, N);
  if (piop_on())
    for (auto &c : Com) {
      put_root("DCBL", (int)c.Base_MT[0].size(), c.Base_MT);
      put_root("DCBR", N, c.Root_MT);
    }
}

// MPI_utils.cpp:3508  send_codeword_batch(arr, B, codeword, fold_depth, N):
// what the leader holds after gathering every party's data
void __real__Z19send_codeword_batchRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES6_S6_ii(
    vector<vector<F>> &arr, vector<vector<F>> &B, vector<vector<F>> &cw, int fold_depth, int N);
void __wrap__Z19send_codeword_batchRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES6_S6_ii(
    vector<vector<F>> &arr, vector<vector<F>> &B, vector<vector<F>> &cw, int fold_depth, int N) {
  __real__Z19send_codeword_batchRSt6vectorIS_IN5virgo12fieldElementESaIS1_EESaIS3_EES6_S6_ii(arr, B, cw, fold_depth,
                                                                                             N);
  if (piop_on()) {
    put_field("SCBA", arr[0]);
    put_field("SCBB", B[0]);
    put_field("SCBC", cw[0]);
  }
}

}  // extern "C"
