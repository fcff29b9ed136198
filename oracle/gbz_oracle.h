/*
 * gbz_oracle — CPU restatement of the reference prover's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the GPU path is
 * compared against (tests/, __graft_entry__.smoke()) and the CPU baseline
 * that bench.py times.  The product (libgbz) never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py compares every function
 * here with golden vectors written by the unmodified reference sources
 * (oracle/ref/ref_driver.cpp, generated by tests/golden/make_golden.py).
 *
 * Field elements are two uint64 words, `real` then `img`, exactly the
 * memory layout of virgo::fieldElement (fieldElement.hpp:96-97).
 */
#ifndef GBZ_ORACLE_H
#define GBZ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* glibc random()/rand() replica (TYPE_3 additive feedback generator). */
typedef struct {
  int32_t tbl[31];
  int f, r;
} orc_prng;

void orc_prng_seed(orc_prng *g, uint32_t seed);
int32_t orc_prng_next(orc_prng *g);
void orc_prng_skip(orc_prng *g, uint64_t count);
/* F::_random (fieldElement.cpp:119-125, 363-368). */
void orc_prng_field(orc_prng *g, uint64_t out[2]);

/* Field F_{p^2}, p = 2^61-1 (fieldElement.cpp:34-103, 337-361). */
void orc_field_ops(int64_t n, const uint64_t *a, const uint64_t *b, uint64_t *add,
                   uint64_t *sub, uint64_t *mul, uint64_t *neg, uint64_t *inv);
void orc_root_of_unity(int log_order, uint64_t out[2]);

/* BLAKE3 of exactly 64 bytes (Blake3_hash.cpp:5-10). */
void orc_blake3_64(int64_t count, const uint8_t *in, uint8_t *out);

/* fft (utils.cpp:904-964); pfft (utils.cpp:1583-1673) computes the same
 * forward transform.  threads <= 0 means "all online cores". */
void orc_fft(uint64_t *a, int logn, int inverse, int threads);

/* MT_commit_Blake (merkle_tree.cpp:195-233) + create_tree_blake (:267-299).
 * levels_out holds level 0 (N/4 leaf hashes) then each upper level, 32 B
 * per hash, (N/2 - 1) hashes in total.  Requires N >= 4. */
int orc_merkle_commit(const uint64_t *elems, int64_t N, uint8_t *levels_out, int threads);
/* open_tree_blake (merkle_tree.cpp:320-335): depth = log2(N/4) hashes. */
int orc_merkle_open(const uint8_t *levels, int64_t N, int64_t pos, uint8_t *path_out);

/* Fiat-Shamir (Fiat_Shamir.cpp:8-34).  state holds prev_challenge. */
void orc_hash_F(const uint64_t x[2], const uint64_t y[2], uint64_t out[2]);
void orc_hash_to_field(uint64_t state[2], const uint64_t *elems, int count, uint64_t out[2]);

/* precompute_beta (utils.cpp:198-243), evaluate_vector (:1201-1214),
 * beta_identity (:1337-1343). */
void orc_precompute_beta(const uint64_t *r, int nr, uint64_t *B, int threads);
void orc_evaluate_vector(const uint64_t *v, int64_t n, const uint64_t *r, uint64_t out[2]);
void orc_beta_identity(const uint64_t *r1, const uint64_t *r2, int nr, uint64_t out[2]);

/* One quadratic sumcheck round message over pairs (coSumcheck_MPI.cpp:199,
 * Whir.cpp:215-221): out = (a, b, c) of sum_j (v1-line)(v2-line). */
void orc_sumcheck_quadratic(const uint64_t *v1, const uint64_t *v2, int64_t m, uint64_t out[6],
                            int threads);
/* Fold v[j] = r*(v[2j+1]-v[2j]) + v[2j] for j < m/2, in place. */
void orc_sumcheck_fold(uint64_t *v, int64_t m, const uint64_t r[2], int threads);

/* get_RS_multifold_segment_tensor (coPCS_utils.cpp:333-383). */
void orc_rs_fold_tensor(const uint64_t *segment, int logk, const uint64_t *r, int64_t n,
                        int64_t idx, uint64_t out[2]);
/* RS_multifold5 (coPCS_utils.cpp:386-437): codeword len n -> n/d. */
void orc_rs_multifold5(const uint64_t *codeword, int64_t n, const uint64_t *a, int logd,
                       uint64_t *out, int threads);

/* update_betas (Whir.cpp:316-342) given the drawn r: b[j] += c_i * w_i^j,
 * c_i = r^(i+1), w_i = omega_N^{q_i}.  challenges_out gets the l c_i. */
void orc_update_betas(uint64_t *b, int64_t nb, const int32_t *queries, int l, int64_t N,
                      const uint64_t r[2], uint64_t *challenges_out, int threads);

/* WHIR query count (Whir.cpp:253-258, conjectured_security = false). */
int orc_whir_queries(int rate);

/* The plain single-party prover transcript (see oracle/ref/ref_driver.cpp
 * cmd_prove for the call sequence it restates).  Returns the number of
 * bytes written, or -1 when cap is too small / arguments are invalid. */
int64_t orc_transcript_bytes(int logn, int rate);
int64_t orc_prove(const uint64_t *witness, int logn, int rate, uint32_t prng_seed,
                  uint8_t *transcript, int64_t cap, int threads);

/* ---- coPCS side ------------------------------------------------------ */

/* compute_lagrange_coeff (utils.cpp:169-197): powers r^i, i < 2^logd, then
 * the inverse transform. */
void orc_lagrange_coeff(const uint64_t r[2], int logd, uint64_t *out);

/* Encode (coPCS.cpp:131-147) of nrows rows of 2^logrow elements: inverse
 * transform, scale by w^{-j} with w = getRootOfUnity(1 + log_ro + logrow),
 * zero-pad to rate * 2^logrow, forward transform.  out: nrows rows of
 * rate * 2^logrow. */
void orc_encode_rows(const uint64_t *rows, int nrows, int logrow, int rate, int log_rate_offset, uint64_t *out,
                     int threads);

/* distributed_MT (coPCS.cpp:152-202) for one party: column roots of the
 * 32-row batch (rows >= nrows are zero), the tree over them (levels: L + L/2
 * + ... + 1 hashes), and the leader's root over {root, 0, ..., 0} of N
 * parties (root_out). */
void orc_column_merkle(const uint64_t *rows, int nrows, int logL, int N, uint8_t *levels, uint8_t root_out[32]);

/* compute_secret_shares (MPI_utils.cpp:2738-2764), k = N/4, _k = N/2:
 * shares[j][i] for party j and group i; with privacy the slots k.._k-1 of
 * each group take random() from the glibc stream seeded with prng_seed. */
void orc_secret_shares(const uint64_t *v, int64_t M, int N, int privacy, uint32_t prng_seed, uint64_t *shares);
/* The same, drawing the random slots from a generator the caller holds. */
void orc_secret_shares_g(const uint64_t *v, int64_t M, int N, int privacy, orc_prng *g, uint64_t *shares);

/* generate_randomness (utils.cpp:1285-1295): x_i = c + F(rand()) with c =
 * F(random()) refreshed every 100 entries, from the caller's generator. */
void orc_generate_randomness(orc_prng *g, int64_t n, uint64_t *out);

/* The party shares of the reference's coPCS test (main.cpp:49-68): rank 0
 * draws, from glibc's default seed, secret_share_coefficients of M values
 * and then of R random values (MPI_utils.cpp:2787-2810), each as
 * generate_randomness + compute_secret_shares with privacy.  shares is
 * N x (M / (N/4)), random N x (R / (N/4)), party-major. */
void orc_copcs_party_shares(int N, int64_t M, int64_t R, uint64_t *shares, uint64_t *random);
void orc_copcs_party_shares_g(int N, int64_t M, int64_t R, uint64_t *shares, uint64_t *random, orc_prng *g_out);

/* sumcheck_aggr leader computation (MPI_utils.cpp:2631-2644): msgs is N
 * party messages of len elements; b has N/4 weights. */
void orc_party_aggregate(const uint64_t *msgs, int N, int64_t len, const uint64_t *b, uint64_t *out);

/* Local sums of quadratic_coSumcheck_phase1 (coSumcheck.cpp:153-179; H of
 * 2d) and cubic_coSumcheck_phase1 (:11-46; H4 of 4d) over blocks of d. */
void orc_cophase1(const uint64_t *p1, const uint64_t *p2, const uint64_t *p3, const uint64_t *b1, int64_t n,
                  int logd, uint64_t *H, uint64_t *H4);
/* quadratic/cubic_coSumcheck_phase2 fold of one vector by Lagrange weights
 * L (coSumcheck.cpp:66-148, 201-213): out[j] = sum_k L[k] v[j*d + k]. */
void orc_cophase2(const uint64_t *v, int64_t n, const uint64_t *L, int logd, uint64_t *out);

/* ---- sumcheck round forms ---------------------------------------------- */

/* Round message over the m/2 pairs of the vectors v (l = linear_poly(v[2j+1]
 * - v[2j], v[2j]), coefficients highest degree first):
 *   form 0 quadratic (v1, v2): sum l1 l2                   (coSumcheck_MPI.cpp:199)
 *   form 1 cubic (v1, v2, v3): sum l1 l2 l3                (Distributed_Sumcheck.cpp:1144-1151)
 *   form 2 batch (v1, v2, v3, v4, r1, r2; b):
 *          sum l1 l2 + l3 l4 + b sum lr1 lr2               (coSumcheck_MPI.cpp:156-176)
 *   form 3 zero-check (v1, v2, v3, beta, r1, r2; b):
 *          sum (l1 l2 + b lr1 lr2 - x l3) lbeta            (coSumcheck_MPI.cpp:12-32)
 *   form 4 quadruple (v1, v2, v3, v4): sum l1 l2 l3 l4     (delegate_protocol.cpp:66-76) */
int orc_sumcheck_form_vectors(int form);
int orc_sumcheck_form_degree(int form);
void orc_sumcheck_round(int form, const uint64_t *const *v, int64_t m, const uint64_t b[2], uint64_t *out);
/* v[j] = v[2j] + r (v[2j+1] - v[2j]) for j < m/2, every vector, in place. */
void orc_sumcheck_fold_many(int nvec, uint64_t *const *v, int64_t m, const uint64_t r[2]);
/* _quadratic_sumcheck (form 0) / _cubic_sumcheck (form 1) of
 * Distributed_Sumcheck.cpp for N parties in one process (see the .c file). */
void orc_party_sumcheck(int form, uint64_t *v1, uint64_t *v2, uint64_t *v3, int64_t M, int N, const uint64_t *w,
                        int offset, uint64_t fs[2], orc_prng *g, uint64_t y_io[2], uint64_t *polys,
                        uint64_t *chal, uint64_t *fin);

/* ---- WHIR aggregation ------------------------------------------------- */
/* aggregate_claims (Whir.cpp:608-668), every point with log2(n) coordinates. */
void orc_aggregate_claims(int k, const uint64_t *const *arrays, int64_t n, int c, const uint64_t *points,
                          orc_prng *g, uint64_t *arr, uint64_t *b_aggr, uint64_t K[2], uint64_t *chal,
                          uint64_t *sums);
/* aggregate_arrays (Whir.cpp:670-704); arr and b are updated in place. */
void orc_aggregate_arrays(uint64_t *arr, uint64_t *b, int k, const uint64_t *const *arrays, int nB,
                          const uint64_t *const *B, int64_t n, const uint64_t *r1, const uint64_t *r2, uint64_t K[2]);
/* aggregate_commitments (Whir.cpp:547-606). */
void orc_aggregate_commitments(int k, const uint64_t *const *cws, int64_t n, const uint64_t *r, int rate, int whir_k,
                               orc_prng *g, uint64_t *codeword, uint8_t *levels);

/* ---- coPCS open rounds ------------------------------------------------ */
/* tensor_eval_vector (coPCS.cpp:602-632) for party my_id: B has rows entries. */
void orc_tensor_eval_vector(uint32_t p0, uint32_t p1, int cols, int64_t rows, int rate, int my_id, uint64_t *B);
/* pcs_sumcheck_phase3 (coPCS.cpp:634-648) with _rates[iter+1][0] = rate. */
void orc_pcs_phase3(uint64_t *B, int64_t rows, const uint32_t *queries, int l, const uint64_t s[2], int N, int rate,
                    int my_id);

/* encode_concatenated (coPCS.cpp:653-677): Cprime (rate0 * n), C
 * (rate0 * n / degree rows of degree * rate1). */
void orc_encode_concatenated(const uint64_t *data, int64_t n, int rate0, int rate1, int degree, uint64_t *Cprime,
                             uint64_t *C);

/* ---- Whir_Batch_Open (Whir.cpp:706-898) ----------------------------- */
/* Schedule of the batch opening of k polynomials of non-increasing sizes:
 * returns the number of schedule steps (kappa[i], aggr[i]) or -1 for inputs
 * the reference cannot run; cw_len[i] receives the codeword length that
 * array i must come with (0: never merged), *bytes the transcript length. */
int orc_whir_batch_schedule(int k, const int64_t *sizes, int rate, int whir_k, int32_t *kappa, int32_t *aggr,
                            int64_t *cw_len, int64_t *bytes);
/* The batch opening's transcript (length or -1); *check_ok: whether the
 * final claim equals sum arr * b. */
int64_t orc_whir_batch_open(int k, const uint64_t *const *arrays, const int64_t *sizes,
                            const uint64_t *const *codewords, const uint8_t *levels0, const uint64_t *const *betas,
                            const uint64_t K0[2], int rate, int whir_k, orc_prng *g, uint8_t *transcript,
                            int64_t cap, int *check_ok, int threads);

/* SplitMix64 witness generator shared by tests and bench. */
void orc_witness(uint64_t seed, int64_t n, uint64_t *out);

#ifdef __cplusplus
}
#endif
#endif
