/*
 * gbz.h — C ABI of the GB300 prover hot path (libgbz.so).
 *
 * Each entry point replaces one function (or one fixed call sequence) of the
 * reference prover and names it as "replaces <file>:<line>" with paths
 * relative to the reference's src/ directory.  Signatures use plain
 * pointers and sizes only.
 *
 * Data layout
 *   A field element of F_{p^2}, p = 2^61 - 1, is two uint64 words, `real`
 *   then `img` (virgo::fieldElement, fieldElement.hpp:96-97).  Arrays of n
 *   elements are 2n words.  Inputs must be canonical (each word < p), which
 *   every value the reference produces on this path is.
 *   A hash is 32 bytes (_hash, Blake3_hash.h:3-5).  Merkle levels are stored
 *   back to back: N/4 leaf hashes, then N/8, ..., 1 (N/2 - 1 hashes).
 *
 * Memory
 *   `mem` = GBZ_MEM_HOST: pointers are host memory; the call copies inputs
 *   in and results out and returns when the results are in place.
 *   `mem` = GBZ_MEM_DEVICE: pointers are device memory of the context's
 *   device; the work is enqueued on the context's stream and the call may
 *   return before it finishes (gbz_synchronize waits).
 *
 * Errors
 *   Every call returns a gbz_status instead of the reference's printf+exit.
 *   gbz_last_error() gives a message for the last failing call of a context.
 *
 * Threading
 *   A context owns one CUDA stream and its scratch buffers; use one context
 *   per host thread.  Contexts on the same device run concurrently.
 */
#ifndef GBZ_H
#define GBZ_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbz_ctx gbz_ctx;
typedef int gbz_status;

#define GBZ_OK 0
#define GBZ_EINVAL 1      /* bad size, length not a power of two, null pointer */
#define GBZ_ENOMEM 2      /* device or pinned-host allocation failed */
#define GBZ_ECUDA 3       /* a CUDA call failed */
#define GBZ_ECHECK 4      /* a device-side protocol consistency check failed */
#define GBZ_ESMALL 5      /* output capacity too small */

#define GBZ_MEM_HOST 0
#define GBZ_MEM_DEVICE 1

/* ------------------------------------------------------------- context */
gbz_status gbz_create(gbz_ctx **ctx, int device);
void gbz_destroy(gbz_ctx *ctx);
/* Use an existing cudaStream_t (passed as void*) instead of the context's own. */
gbz_status gbz_set_stream(gbz_ctx *ctx, void *cuda_stream);
void *gbz_get_stream(gbz_ctx *ctx);
gbz_status gbz_synchronize(gbz_ctx *ctx);
const char *gbz_status_string(gbz_status s);
const char *gbz_last_error(const gbz_ctx *ctx);
/* Pinned host memory (for GBZ_MEM_HOST calls that should not stage). */
gbz_status gbz_host_alloc(void **ptr, uint64_t bytes);
void gbz_host_free(void *ptr);
gbz_status gbz_device_alloc(gbz_ctx *ctx, void **ptr, uint64_t bytes);
void gbz_device_free(gbz_ctx *ctx, void *ptr);

/* ---------------------------------------------------- field and hashes */

/* Elementwise a+b, a-b, a*b (any output may be null).
 * replaces fieldElement::operator+ / operator- / operator* (fieldElement.cpp:34-96). */
gbz_status gbz_field_ops(gbz_ctx *ctx, const uint64_t *a, const uint64_t *b, uint64_t n, uint64_t *sum,
                         uint64_t *diff, uint64_t *prod, int mem);

/* count independent BLAKE3 hashes of 64-byte blocks (in: 64*count bytes,
 * out: 32*count bytes).
 * replaces blake3_hash (Blake3_hash.cpp:5-10). */
gbz_status gbz_blake3_64(gbz_ctx *ctx, const uint8_t *in, uint8_t *out, uint64_t count, int mem);

/* In-place transform of 2^logn elements: forward, or inverse scaled by 2^-logn.
 * replaces fft (utils.cpp:904-964) and pfft (utils.cpp:1583-1673; forward only there). */
gbz_status gbz_fft(gbz_ctx *ctx, uint64_t *data, int logn, int inverse, int mem);

/* Reed-Solomon encoding as WHIR commits it: codeword (rate*m elements) =
 * forward transform of arr (m elements) zero-padded to rate*m.
 * replaces the padding + pfft of Whir_Commit_initial (Whir.cpp:160-163). */
gbz_status gbz_rs_encode(gbz_ctx *ctx, const uint64_t *arr, uint64_t m, int rate, uint64_t *codeword,
                         int mem);

/* Blake3 Merkle tree over N elements (N a power of two >= 4): leaves hash
 * four consecutive elements, each inner node hashes its left child twice.
 * levels: (N/2 - 1) * 32 bytes.
 * replaces MT_commit_Blake + create_tree_blake (merkle_tree.cpp:195-233, 267-299). */
gbz_status gbz_merkle_commit_blake(gbz_ctx *ctx, const uint64_t *elems, uint64_t N, uint8_t *levels,
                                   int mem);

/* Authentication path of leaf pos: log2(N/4) sibling hashes (host memory).
 * replaces open_tree_blake (merkle_tree.cpp:320-335). */
gbz_status gbz_merkle_open_blake(const uint8_t *levels, uint64_t N, uint64_t pos, uint8_t *path,
                                 uint32_t *depth);

/* codeword = encode(arr, rate); levels = Merkle tree of the codeword.
 * replaces Whir_Commit_initial (Whir.cpp:158-190). */
gbz_status gbz_whir_commit(gbz_ctx *ctx, const uint64_t *arr, uint64_t m, int rate, uint64_t *codeword,
                           uint8_t *levels, int mem);

/* The tree above L leaf hashes (L a power of two, 32 B each): levels gets
 * the upper levels back to back, L/2, L/4, ..., 1 hashes (L - 1 in total);
 * every inner node is blake3(left || left) as the reference builds it.
 * replaces create_tree_blake (merkle_tree.cpp:267-299). */
gbz_status gbz_merkle_tree_from_leaves(gbz_ctx *ctx, const uint8_t *leaves, uint64_t L, uint8_t *levels, int mem);

/* eq table B[x] = prod_i (bit_i(x) ? r_i : 1 - r_i), 2^nr elements.
 * replaces precompute_beta (utils.cpp:198-243). */
gbz_status gbz_precompute_beta(gbz_ctx *ctx, const uint64_t *r, int nr, uint64_t *B, int mem);

/* ------------------------------------------------------------ sumcheck */

/* Round message (a, b, c) of sum_j (v1 line_j)(v2 line_j) over m elements
 * (coeffs: 6 words, host memory).
 * replaces whir_sumcheck_step1 (Whir.cpp:215-221) and the round sums of
 * _quadratic_cosumcheck (coSumcheck_MPI.cpp:199) / _quadratic_sumcheck
 * (delegate_protocol.cpp:16-21). */
gbz_status gbz_sumcheck_quadratic(gbz_ctx *ctx, const uint64_t *v1, const uint64_t *v2, uint64_t m,
                                  uint64_t *coeffs, int mem);

/* v[j] = r*(v[2j+1]-v[2j]) + v[2j] for j < m/2, in place (r: host memory).
 * replaces the fold loops of whir_sumcheck_step2 (Whir.cpp:223-231) and
 * _quadratic_cosumcheck (coSumcheck_MPI.cpp:215-218). */
gbz_status gbz_sumcheck_fold(gbz_ctx *ctx, uint64_t *v, uint64_t m, const uint64_t *r, int mem);

/* b[j] += c_i * omega_N^(q_i * j) with c_i = r^(i+1); challenges (l
 * elements, host memory, may be null) receives the c_i.  r is the value the
 * reference draws with F::_random() at Whir.cpp:327.
 * replaces update_betas (Whir.cpp:325-342). */
gbz_status gbz_whir_update_betas(gbz_ctx *ctx, uint64_t *b, uint64_t nb, const int32_t *queries, int l,
                                 uint64_t N, const uint64_t *r, uint64_t *challenges, int mem);

/* ------------------------------------------- many proofs: batch, serving */

/* Options of the many-proof scheduler.  A slot is one CUDA stream with its
 * own per-shape plan (buffers, verifier state, transcript); proofs in
 * different slots overlap on the device and never share memory, so every
 * transcript is the one gbz_prove returns for the same inputs.  Plans (and
 * their captured graphs) stay cached in the context across calls. */
typedef struct gbz_sched_opts {
  int lanes;               /* concurrent slots (0: 8) */
  int depth;               /* serving: proofs in flight per slot before admission waits (0: 2) */
  int graphs;              /* 1: replay one captured CUDA graph per (slot, shape); 0: direct launches */
  uint64_t reserve_bytes;  /* device memory left free when a new shape is admitted (0: 1 GiB) */
} gbz_sched_opts;

/* Proves count independent statements of mixed shapes as one batch: the
 * proofs are assigned longest-first to the least-loaded slot and enqueued
 * round-robin over the slots.  witness[i] holds 2^logn[i] elements and
 * transcript[i] capacity[i] >= gbz_prove_transcript_bytes(logn[i], rate[i])
 * bytes, all host or all device per mem.  Host transcripts in pageable
 * memory are written through a pinned staging buffer the context keeps
 * (a device-to-pageable copy would wait for each slot's earlier work) and
 * copied out when the batch ends; pinned ones (gbz_host_alloc) directly.
 * latency_s[i] (optional) = completion of proof i after the
 * batch started; *makespan_s (optional) = completion of the last one.
 * opts may be NULL (defaults).  No counterpart in the reference, which
 * proves one statement per process (main.cpp). */
gbz_status gbz_prove_batch(gbz_ctx *ctx, int count, const uint64_t *const *witness, const int *logn, const int *rate,
                           const uint32_t *prng_seed, uint8_t *const *transcript, const uint64_t *capacity, int mem,
                           const gbz_sched_opts *opts, double *latency_s, double *makespan_s);

/* Serving loop over timed arrivals: proof i is admitted no earlier than
 * arrival_s[i] seconds after the call starts, to the least-loaded slot with
 * fewer than opts->depth proofs in flight, once its plan fits in free device
 * memory (idle cached plans are evicted least recently used first).
 * latency_s[i] = completion - arrival; other arguments as gbz_prove_batch. */
gbz_status gbz_serve(gbz_ctx *ctx, int count, const double *arrival_s, const uint64_t *const *witness,
                     const int *logn, const int *rate, const uint32_t *prng_seed, uint8_t *const *transcript,
                     const uint64_t *capacity, int mem, const gbz_sched_opts *opts, double *latency_s,
                     double *makespan_s);

/* gbz_prove_batch groups the proofs of one shape into one batched plan
 * (on by default): every kernel of the proof is launched once for the
 * whole group (grid.y or grid.x = proof, per-proof buffers at fixed
 * strides), so a batch of many small proofs is not bound by the device's
 * launch rate.  Off: one plan and one graph replay per proof.  Transcripts
 * are the same either way. */
gbz_status gbz_sched_set_grouping(gbz_ctx *ctx, int on);

/* Frees the scheduler's cached slot plans and the scratch the N-party
 * calls (gbz_pcs_claim, gbz_pcs_open, gbz_pcs_open_full, gbz_cosumcheck)
 * keep per shape between calls; *cached_bytes (optional) gets the device
 * bytes they held. */
gbz_status gbz_sched_release(gbz_ctx *ctx, uint64_t *cached_bytes);

/* ----------------------------------------------------- coPCS-side rows */

/* RS fold of a codeword of n elements by d = 2^logd (1 <= logd <= 4) with
 * fold weights a (d elements, host memory); out has n/d elements.
 * replaces RS_multifold5 (coPCS_utils.cpp:386-437). */
gbz_status gbz_rs_multifold5(gbz_ctx *ctx, const uint64_t *codeword, uint64_t n, const uint64_t *a, int logd,
                             uint64_t *out, int mem);

/* Lagrange basis at r (2 words, host) over the 2^logd-point subgroup: the
 * inverse transform of (1, r, r^2, ...); out has 2^logd elements.
 * replaces compute_lagrange_coeff (utils.cpp:169-197). */
gbz_status gbz_lagrange_coeff(gbz_ctx *ctx, const uint64_t *r, int logd, uint64_t *out, int mem);

/* coPCS encoding of nrows rows of 2^logrow elements: inverse transform,
 * scale by w^{-j} with w = getRootOfUnity(1 + log_rate_offset + logrow),
 * zero-pad to rate * 2^logrow, forward transform.  out: nrows rows of
 * rate * 2^logrow elements.
 * replaces Encode (coPCS.cpp:131-147), rate_offset = 2^log_rate_offset. */
gbz_status gbz_encode_rows(gbz_ctx *ctx, const uint64_t *rows, int nrows, int logrow, int rate, int log_rate_offset,
                           uint64_t *out, int mem);

/* encode_concatenated (coPCS.cpp:653-677): C' (optional, rate0 * n
 * entries) = forward transform of data zero-padded to rate0 * n; column
 * j < rate0 n / degree gathers C'[j + k rate0 n / degree] for k < degree,
 * is zero-padded to degree * rate1 (<= 2^13) and transformed into row j of
 * C (rate0 n / degree rows of degree * rate1 entries). */
gbz_status gbz_encode_concatenated(gbz_ctx *ctx, const uint64_t *data, uint64_t n, int rate0, int rate1, int degree,
                                   uint64_t *Cprime, uint64_t *C, int mem);

/* The leader's root over {root, 0, ..., 0} of nparties commitments (the
 * create_tree_blake of distributed_MT / commit_concatenated, coPCS.cpp:
 * 193-201, 701-709): log2(nparties) self-hashes of root.  Host only. */
void gbz_leader_root(const uint8_t *root, int nparties, uint8_t *out);

/* One party's commitment of a batch of nrows <= 32 codeword rows of 2^logL
 * elements: per-column Blake3 roots (MT_commit_Blake over the 32-entry
 * column, missing rows zero), the tree over them (levels: 2^(logL+1) - 1
 * hashes, column roots first) and the leader's root over nparties entries
 * {root, 0, ..., 0} (root: 32 bytes).
 * replaces distributed_MT (coPCS.cpp:152-202). */
gbz_status gbz_column_merkle(gbz_ctx *ctx, const uint64_t *rows, int nrows, int logL, int nparties, uint8_t *levels,
                             uint8_t *root, int mem);

/* Packed Shamir shares of M values for N parties (N a power of two, 4..64):
 * k = N/4 secrets per group padded to N/2 with zeros, or with the glibc
 * random() stream from srandom(prng_seed) when privacy is set; shares holds
 * N rows of 4M/N elements.
 * replaces compute_secret_shares (MPI_utils.cpp:2738-2764). */
gbz_status gbz_secret_shares(gbz_ctx *ctx, const uint64_t *v, uint64_t M, int N, int privacy, uint32_t prng_seed,
                             uint64_t *shares, int mem);

/* Leader aggregation of N party round messages (N rows of len elements)
 * with weights b (N/4 elements, host): unpack every coefficient's shares
 * and combine the secrets.  out: len elements.
 * replaces the leader computation of sumcheck_aggr (MPI_utils.cpp:2604-2670). */
gbz_status gbz_party_aggregate(gbz_ctx *ctx, const uint64_t *msgs, int N, uint64_t len, const uint64_t *b,
                               uint64_t *out, int mem);

/* Local round sums of the block-univariate sumcheck over blocks of d =
 * 2^logd (n elements per vector).  Quadratic (p3 = b1 = NULL): H (2d
 * elements, host) = sum over blocks of ext(p1) * ext(p2), ext = inverse
 * transform of the block, zero-padded, forward transform of twice the
 * length.  Cubic: H (4d elements) = sum over blocks whose p1 part is not
 * all zero of (ext(p1) ext(p2) - ext(p3)) ext(b1) at four times the length.
 * The extended length (2d or 4d) is at most 2^13.
 * replaces the local loops of quadratic_coSumcheck_phase1
 * (coSumcheck.cpp:150-179) and cubic_coSumcheck_phase1 (:9-46). */
gbz_status gbz_cosumcheck_phase1(gbz_ctx *ctx, const uint64_t *p1, const uint64_t *p2, const uint64_t *p3,
                                 const uint64_t *b1, uint64_t n, int logd, uint64_t *H, int mem);

/* Fold of n elements by blocks of d = 2^logd with Lagrange weights L (d
 * elements, host): out[j] = sum_k L[k] v[j d + k] (n/d elements).
 * replaces quadratic_coSumcheck_phase2 / cubic_coSumcheck_phase2
 * (coSumcheck.cpp:201-213, 66-148). */
gbz_status gbz_cosumcheck_phase2(gbz_ctx *ctx, const uint64_t *v, uint64_t n, const uint64_t *L, int logd,
                                 uint64_t *out, int mem);

/* With nb = 0 (or l = 0) b is left as it is and the l combination weights
 * are still written to challenges (both update_betas entry points). */

/* The same update as gbz_whir_update_betas, for callers that must not let
 * the library allocate device memory at call time (a service that has
 * already handed all device memory to request slots, or a host runtime with
 * a fixed device budget behind a foreign-function boundary).  No
 * counterpart in the reference.
 *   b, queries and challenges (l elements, may be null) are device memory of
 *   the current device; r (2 words) is host memory; the work is enqueued on
 *   cuda_stream (a cudaStream_t; null = the default stream).
 *   Working memory is one file-scope device array of about 1 MiB that
 *   every GPU loading the library keeps until exit; it holds at most 256
 *   queries, so l > 256 returns GBZ_EINVAL (as do a null b/r, a null queries
 *   with l > 0, and N not a power of two or above 2^28).
 *   A call looks up that array's device address (with the device current),
 *   so a context re-created after a device reset gets its own; a call made
 *   while its stream is being captured uses the address that the last
 *   uncaptured call on the device found, so make one call on each device
 *   before any stream capture.
 *   All calls share the array: calls that overlap on the GPU (other streams,
 *   other host threads) race and must be serialised by the caller.  Nothing
 *   in it needs to start at zero: each call writes every entry it reads.
 *   The call allocates nothing: no cudaMalloc, no cudaFree, no pool. */
gbz_status gbz_whir_update_betas_noalloc(uint64_t *b, uint64_t nb, const int32_t *queries, int l, uint64_t N,
                                         const uint64_t *r, uint64_t *challenges, void *cuda_stream);

/* ---------------------------------------------- host-side protocol state */

/* Fiat-Shamir: state[2] is the chain value (prev_challenge, initially 0);
 * absorbs count elements and returns the new challenge in out[2].
 * replaces hash_to_field / hash_F (Fiat_Shamir.cpp:8-34), with the chain
 * held by the caller instead of a process global. */
void gbz_hash_to_field(uint64_t *state, const uint64_t *elems, int count, uint64_t *out);

/* glibc random()/rand() stream, seeded like srandom(seed).
 * replaces the process-global generator behind F::_random
 * (fieldElement.cpp:119-125, 363-368) and rand() (Whir.cpp:262-268). */
typedef struct {
  int32_t tbl[31];
  int32_t f, r;
} gbz_prng;
void gbz_prng_seed(gbz_prng *g, uint32_t seed);
int32_t gbz_prng_next(gbz_prng *g);
/* F::_random(): out[2] = (randomNumber() % p, randomNumber() % p). */
void gbz_prng_field(gbz_prng *g, uint64_t *out);

/* Host twin of the device field arithmetic (same source), elementwise. */
void gbz_field_ops_host(const uint64_t *a, const uint64_t *b, uint64_t n, uint64_t *sum, uint64_t *diff,
                        uint64_t *prod);

/* ------------------------------------------------- sumcheck round forms */

/* Round forms of the multilinear sumcheck provers.  Over the pairs
 * (v[2j], v[2j+1]) with lines l(x) = (v[2j+1] - v[2j]) x + v[2j], the round
 * polynomial (coefficients highest degree first) is */
#define GBZ_SC_QUADRATIC 0 /* (v1, v2): sum l1 l2, 3 coefficients (coSumcheck_MPI.cpp:199) */
#define GBZ_SC_CUBIC 1     /* (v1, v2, v3): sum l1 l2 l3, 4 (Distributed_Sumcheck.cpp:1144-1151) */
#define GBZ_SC_BATCH 2     /* (v1, v2, v3, v4, r1, r2; b): sum l1 l2 + l3 l4 + b lr1 lr2, 3
                              (_quadratic_batch_sumcheck_phase1, coSumcheck_MPI.cpp:156-176) */
#define GBZ_SC_ZEROCHECK 3 /* (v1, v2, v3, beta1, r1, r2; b): sum (l1 l2 + b lr1 lr2 - x l3) lbeta1, 4
                              (_zero_check_sumcheck_phase1, coSumcheck_MPI.cpp:12-32) */
#define GBZ_SC_QUADRUPLE 4 /* (v1, v2, v3, v4): sum l1 l2 l3 l4, 5 coefficients (the round message of
                              quadruple_sumcheck, delegate_protocol.cpp:57-115, whose challenges are
                              the fifth of five F::_random() draws per round) */

/* One round of a form over vectors v[0..k) of m entries (m a power of two).
 * r == NULL: coeffs = the round polynomial of v (the reference's phase 1).
 * r != NULL (2 words, host): every vector is first folded in place by r,
 * v[j] = v[2j] + r (v[2j+1] - v[2j]) for j < m/2 (phase 2,
 * coSumcheck_MPI.cpp:34-44, 178-187), and coeffs is the round polynomial
 * of the folded vectors.  b (2 words, host) is required by the batch and
 * zero-check forms.  coeffs (host) receives 3, 4 or 5 elements. */
gbz_status gbz_sumcheck_round(gbz_ctx *ctx, int form, uint64_t *const *v, uint64_t m, const uint64_t *b,
                              const uint64_t *r, uint64_t *coeffs, int mem);

/* Rounds of gbz_party_sumcheck: max(log2 M - offset, 0) Fiat-Shamir rounds
 * plus log2(N 2^offset') leader rounds (offset' = log2 M when the first
 * count is not positive). */
int gbz_party_sumcheck_rounds(uint64_t M, int N, int offset);

/* The distributed sumcheck of N parties held on this device:
 * form GBZ_SC_QUADRATIC replaces _quadratic_sumcheck
 * (Distributed_Sumcheck.cpp:204-349), form GBZ_SC_CUBIC _cubic_sumcheck
 * (:1122-1269).  Party p owns entries [p M, (p+1) M) of v1, v2 (, v3), all
 * read only.  The parties' round polynomials are combined as aggregate_poly
 * does (a sum; for the cubic form weighted by w[p], N elements, host, NULL
 * for ones), the first rounds draw hash_to_field of the coefficients from
 * the chain fs_state (2 words, in/out: prev_challenge), and the leader's
 * rounds over the gathered N 2^offset entries (cubic: v3 scaled by w[p])
 * take the fourth F::_random() draw of each round from *prng (in/out).
 * y (2 words, in/out) is the claim; every round is checked against it and
 * GBZ_ECHECK is returned if one does not match (outputs are still written).
 * Outputs (host): polys (3 or 4 per round), challenges (one per round), fin
 * (the leader's final v1[0], v2[0] (, v3[0])).  For the quadratic form the
 * reference's leader reads zeros for the other parties' v2 entries when
 * N > 1 (its receive buffers are N times too long, :289-306) and its
 * consistency check then exits; here the parties' entries are gathered as
 * intended, so reference parity is defined for N = 1. */
gbz_status gbz_party_sumcheck(gbz_ctx *ctx, int form, const uint64_t *v1, const uint64_t *v2, const uint64_t *v3,
                              uint64_t M, int N, const uint64_t *w, int offset, uint64_t *fs_state, gbz_prng *prng,
                              uint64_t *y, uint64_t *polys, uint64_t *challenges, uint64_t *fin, int mem);

/* ------------------------------------------------------ WHIR aggregation */

/* aggregate_claims (Whir.cpp:608-668) for k arrays of n entries and c claim
 * points of log2(n) coordinates (points: c*log2(n) elements, host):
 * Sums[i][j] = <precompute_beta(point_j), array_i>; F::_random() draws c
 * beta weights then k array weights from *prng (in/out); K = sum_ij
 * bw_j aw_i Sums[i][j] (2 words, host); b_aggr = sum_j bw_j beta_j and
 * arr = sum_i aw_i array_i (n entries each, mem); challenges (host) gets
 * the c + k weights, sums (host, optional) the k x c inner products. */
gbz_status gbz_whir_aggregate_claims(gbz_ctx *ctx, int k, const uint64_t *const *arrays, uint64_t n, int c,
                                     const uint64_t *points, gbz_prng *prng, uint64_t *arr, uint64_t *b_aggr,
                                     uint64_t *K, uint64_t *challenges, uint64_t *sums, int mem);

/* aggregate_arrays (Whir.cpp:670-704): arr += sum_{i>=1} r1_i arrays_i and
 * b += sum_{i>=1} r2_i B_i in place (n entries, mem); K (host) = sum over
 * i < k, j < nB of r1_i r2_j <arrays_i, B_j>.  r1 (k) and r2 (nB) are host. */
gbz_status gbz_whir_aggregate_arrays(gbz_ctx *ctx, int k, const uint64_t *const *arrays, int nB,
                                     const uint64_t *const *B, uint64_t n, const uint64_t *r1, const uint64_t *r2,
                                     uint64_t *arr, uint64_t *b, uint64_t *K, int mem);

/* aggregate_commitments (Whir.cpp:547-606): codeword = sum_i r_i
 * codewords_i (n entries, mem; r host); the query openings advance *prng
 * by l rand() draws (l as the WHIR query count of `rate`); levels (mem)
 * receives the new Merkle tree over n / whir_k leaves, 2 n / whir_k - 1
 * hashes.  The reference's loop that hashes the strided leaf groups never
 * stores its result (:594-601), so every leaf of that tree is the zero hash;
 * the levels here are the same. */
gbz_status gbz_whir_aggregate_commitments(gbz_ctx *ctx, int k, const uint64_t *const *codewords, uint64_t n,
                                          const uint64_t *r, int rate, int whir_k, gbz_prng *prng,
                                          uint64_t *codeword, uint8_t *levels, int mem);

/* --------------------------------------------------- WHIR batch opening */

/* Schedule of Whir_Batch_Open (kappas and merge flags of Whir.cpp:731-752,
 * then the loop of :761-833) for k <= 64 polynomials of non-increasing
 * power-of-two sizes: *steps entries kappa[i], aggr[i] (room for 64),
 * cw_len[i] = the codeword length polynomial i must come with (0: the loop
 * ends before it is merged), *transcript_bytes.  Every output may be NULL.
 * Host only.  GBZ_EINVAL for inputs the reference cannot run: it reads its
 * schedule past the end when a merge is among the last two steps, and
 * exits in open_tree_blake when a query exceeds a merged tree. */
gbz_status gbz_whir_batch_schedule(int k, const uint64_t *sizes, int rate, int whir_k, int *steps, int32_t *kappa,
                                   int32_t *aggr, uint64_t *cw_len, uint64_t *transcript_bytes);

/* Whir_Batch_Open(arrays, codewords, MTs, evals, betas, rate, true)
 * (Whir.cpp:706-898) with the reference's global whir_k = whir_k (2, 4, 8
 * or 16): arrays[i] (sizes[i] elements) with their claim vectors betas[i],
 * K0 = evals[0] (the claim of array 0), codewords[i] (cw_len[i] elements,
 * the RS encoding at the rate array i is merged at), levels0 = MTs[0] (the
 * MT_commit_Blake levels of codewords[0]; the other trees are never read by
 * the reference).  prng: the glibc generator state, advanced past every
 * draw.  Transcript records:
 *  19 SCHEDULE u32 x 2 steps (kappa, merge flag)
 *  per executed step: a WHIR iteration with folding factor kappa
 *    (log2 kappa x (7 WHIR_POLY, 8 WHIR_CHALLENGE), 9 WHIR_ROOT,
 *    10 WHIR_QUERIES, 11 WHIR_REPLIES 16B x kappa l, 12 WHIR_ANSWERS,
 *    13 WHIR_PATHS, 14 WHIR_COMBINE, 15 WHIR_K), then for a merge
 *    20 AGGR_CHALLENGES 16B x 2g (ch1 then ch2, each starting with 1),
 *    21 AGGR_K 16B, 22 AGGR_QUERIES u32 x l (aggregate_commitments'
 *    openings), 23 AGGR_PATHS 32B x l depth, 24 AGGR_ROOT 32B (the tree over
 *    zero leaves the reference installs)
 *  16 FINAL_POLY 16B x m | 17 FINAL_POINT 16B x log2 m | 18 FINAL_EVAL 16B
 * Returns GBZ_ECHECK (outputs still written) when a sumcheck claim or the
 * final K == <arr, b> (verification step 2) fails on the device. */
gbz_status gbz_whir_batch_open(gbz_ctx *ctx, int k, const uint64_t *const *arrays, const uint64_t *sizes,
                               const uint64_t *const *codewords, const uint8_t *levels0,
                               const uint64_t *const *betas, const uint64_t *K0, int rate, int whir_k,
                               gbz_prng *prng, uint8_t *transcript, uint64_t capacity, int mem);

/* ------------------------------------------------------ coPCS open rounds */

/* tensor_eval_vector (coPCS.cpp:602-632) for party my_id (< 2 cols):
 * out[j] = c w1^j for j < rows, w1 = omega_{rate rows}^{point[1]}, c the
 * party's entry of the transformed powers of omega_{4 cols}^{2 point[0] + 1}. */
gbz_status gbz_tensor_eval_vector(gbz_ctx *ctx, const uint32_t *point, int cols, uint64_t rows, int rate, int my_id,
                                  uint64_t *out, int mem);

/* pcs_sumcheck_phase3 (coPCS.cpp:634-648): B += sum_i s^(i+1)
 * tensor_eval_vector(query_i, N/2, rows, rate) in place; queries holds l
 * (point[0], point[1]) pairs (host), s 2 words (host); rate is the
 * reference's _rates[iter+1][0] (the caller skips the call where the
 * reference returns early). */
gbz_status gbz_pcs_sumcheck_phase3(gbz_ctx *ctx, uint64_t *B, uint64_t rows, const uint32_t *queries, int l,
                                   const uint64_t *s, int N, int rate, int my_id, int mem);

/* ------------------------------------------- collaborative PCS, N parties */

/* The collaborative PCS of N parties on one device (N = 4..64, a power of
 * two): the reference runs it with one MPI rank per party; here every
 * party's share is a row of one party-major device array and the leader's
 * aggregation runs on the device.
 *
 * rate0[i] = rates[i][0] and rate1[i] = rates[i][1] (0 where absent) of the
 * reference's `rates` (e.g. {{4},{4},{4,4},{4,4}}, main.cpp:54), rounds =
 * rates.size(); M = the number of shared coefficients (a power of two).
 *
 * gbz_pcs_schedule: prepare_parameters (coPCS.cpp:38-72; get_degrees /
 * get_queries, New_PCS.cpp:23-77): the folding degrees and query counts of
 * every round, and the random shares each party holds (randomness of
 * coPCS.cpp:53-55; secret_share_coefficients deals randomness * N / 4
 * values, main.cpp:68).  No GPU.
 * replaces prepare_parameters (coPCS.cpp:38-72). */
gbz_status gbz_pcs_schedule(int N, uint64_t M, int rounds, const int *rate0, const int *rate1, int *degrees,
                            int *queries, uint64_t *random_per_party);

typedef struct gbz_pcs gbz_pcs;

/* PCS_commit of every party: prepare_data (coPCS.cpp:76-129), Encode
 * (:131-147) and distributed_MT (:152-230).  shares: N x (4M/N) elements,
 * random: N x random_per_party elements, party-major.  *out receives the
 * commitment (device memory held until gbz_pcs_free); party_roots (N x 32 B)
 * and leader_root (32 B; the leader's tree over {root_0, 0, ..., 0}) may be
 * NULL.
 * replaces PCS_commit (coPCS.cpp:236-250) on N ranks. */
gbz_status gbz_pcs_commit(gbz_ctx *ctx, int N, uint64_t M, int rounds, const int *rate0, const int *rate1,
                          const uint64_t *shares, const uint64_t *random, int mem, gbz_pcs **out,
                          uint8_t *party_roots, uint8_t *leader_root);
void gbz_pcs_free(gbz_pcs *pcs);
/* Shape of a commitment: Commit_data rows with entries (batches), their
 * length, the codeword length, and the transcript bytes of gbz_pcs_open. */
gbz_status gbz_pcs_info(const gbz_pcs *pcs, int *batches, uint64_t *row_len, uint64_t *codeword_len,
                        uint64_t *open_transcript_bytes);
/* One party's Commit_data rows (batches x row_len), codewords (batches x
 * codeword_len) and column-root tree (2 codeword_len - 1 hashes); any
 * output may be NULL. */
gbz_status gbz_pcs_commit_data(gbz_ctx *ctx, const gbz_pcs *pcs, int party, uint64_t *rows, uint64_t *codewords,
                               uint8_t *levels, int mem);

/* The claim the coPCS test opens (main.cpp:87-112): F_ip of the committed
 * data at the point r (the same r as gbz_pcs_open): every party's inner
 * product of its batched rows with precompute_beta(r[log2(N/4)..]), and the
 * leader's unpack of the N values weighted by precompute_beta(r[0 ..
 * log2(N/4))) into K (2 words).
 * replaces F_ip (MPI_utils.cpp:483-553) on N ranks. */
gbz_status gbz_pcs_claim(gbz_ctx *ctx, const gbz_pcs *pcs, const uint64_t *r, int nr, uint64_t *K, int mem);

/* The parties' side of PCS_open_new with the leader's aggregation
 * (coPCS.cpp:1310-1607, isPIOP = false): row batching and the batching
 * round, batch_commitments_new (:1242-1308), per round pcs_sumcheck_phase1
 * (aggregated as pcs_sumcheck_aggr does, MPI_utils.cpp:341-405), the
 * leader's check and Fiat-Shamir challenge, pcs_sumcheck_phase2,
 * encode_concatenated + commit_concatenated or RS_multifold5 +
 * commit_tensorcode, delegate_checks' queries, folded answers and segment
 * gather (:740-891), and pcs_sumcheck_phase3 (:634-648).
 * r: the opening point, log2(N/4) + 5 + log2(row_len) elements; K: the
 * claim (F_ip, MPI_utils.cpp:483); fs: the Fiat-Shamir chain value
 * (prev_challenge) before the opening, updated in place.  The leader's
 * delegation proofs and WHIR opening of the gathered segments follow in the
 * reference and are not part of this call.  The commitment's device state
 * is read, not changed: a commitment can be opened again.
 * Transcript records {u32 tag, u32 count, payload}:
 *   34 PARTY_POLYS 16B x 3N | 35 POLY 16B x3 | 36 CHALLENGE 16B | 41 K 16B |
 *   32 ROOTS 32B x N | 33 LEADER_ROOT 32B | 37 QUERIES u32 x 2 l0
 *   per round: 34 PARTY_POLYS 16B x 2dN, 35 POLY 16B x 2d, 36 CHALLENGE,
 *     32 ROOTS, 33 LEADER_ROOT, 37 QUERIES u32 x 2l ((party, position)
 *     pairs, party by party as the leader holds them), 38 Y 16B x l,
 *     39 SEGMENTS 16B x l d, 40 S 16B, 41 K 16B
 *   42 FINAL 16B x N (data, B, C') per party (send_pcs_data)
 * The reference's quirk that commit_tensorcode reports the previous
 * commitment's root (it reuses a deeper levels vector) is kept.
 * GBZ_ECHECK when a round message does not match the claim or a delegate
 * check fails.
 * replaces PCS_open_new (coPCS.cpp:1310-1607) on N ranks, up to the leader's
 * delegation. */
gbz_status gbz_pcs_open(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *r, int nr, const uint64_t *K, uint64_t *fs,
                        uint8_t *transcript, uint64_t capacity, int mem);

/* The whole of PCS_open_new: gbz_pcs_open's records, then the leader's tail,
 * which draws from the leader's glibc generator *prng (rank 0's random()
 * stream when the opening starts; updated in place) and never from the
 * Fiat-Shamir chain:
 *  per delegate check after the first (coPCS.cpp:770-831):
 *   46 D_ROOT 32B (Whir_Commit_initial(segments padded to the largest
 *   delegation size, rate 4): the root of MT_commit_Blake over its codeword)
 *   | 47 D_QUERIES u32 x l (rand() % C[0].size()) | prove_multi_folding
 *   (delegate_protocol.cpp:147-250): 48 D_POLYS 16B x 5R, 49 D_FINAL 16B x 4
 *   (quadruple_sumcheck), 48 16B x 3 log2 d, 49 16B x 2 (_quadratic_sumcheck),
 *   50 D_CLAIM 16B x (1 + log2 max_delegation) (value, point, zeros) |
 *   51 D_OPEN 16B x l (the extended segments at the queries) |
 *   prove_extension (:369-429): 48 16B x 4R', 49 16B x 3 (_cubic_sumcheck),
 *   48 16B x 3 log2 C0, 49 16B x 2 (prove_fft's _quadratic_sumcheck),
 *   52 D_EXT_CLAIM 16B x (1 + log2 d + log2 S)
 *  then (coPCS.cpp:1697-1753): 53 UNPACKED 16B x N (the parties' final data
 *   and B unpacked, N/2 each) | aggregate_claims and aggregate_commitments
 *   (Whir.cpp:547-668): 20 AGGR_CHALLENGES (beta weights, array weights),
 *   21 AGGR_K, 22 AGGR_QUERIES, 23 AGGR_PATHS, 24 AGGR_ROOT | _Whir_Open
 *   (Whir.cpp:469-545, whir_k = 8) as the records 19, 7-18 of
 *   gbz_whir_batch_open | 54 WHIR_CLAIM 16B x (1 + log2 max_delegation) |
 *   55 RC 16B x 2 (r_c, B_eval_claim) | delegate_beta_eval
 *   (delegate_protocol.cpp:431-504): 56 BETA_Y 16B, 48/49 (_cubic_sumcheck),
 *   57 L_EVALS 16B x rounds, 48/49 (_quadratic_sumcheck; the reference reads
 *   past the end of b there, here b is zero beyond its length)
 * *flags (may be NULL) receives the checks the reference prints (bit 0: a
 * quadruple/cubic round message, bit 3: final verification step 1, bit 5:
 * WHIR verification step 3) and those it stops at (bit 1: a delegation
 * check, bit 2: decoding, bit 4: the WHIR opening's checks, bit 6: the
 * final verification step, bit 7: delegating the betas); the latter return
 * GBZ_ECHECK.  Transcript bytes: gbz_pcs_open_full_bytes.
 * replaces PCS_open_new (coPCS.cpp:1310-1607, 1610-1755) on N ranks. */
gbz_status gbz_pcs_open_full(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *r, int nr, const uint64_t *K, uint64_t *fs,
                             gbz_prng *prng, uint32_t *flags, uint8_t *transcript, uint64_t capacity, int mem);
gbz_status gbz_pcs_open_full_bytes(const gbz_pcs *pcs, uint64_t *bytes);

/* One WHIR batch slot of the PIOP mode (whir_polys, whir_c, whir_betas,
 * whir_claims, whir_MTs of coPCS.cpp:1620-1629); any pointer may be NULL.
 * arr: slot_len field elements (the delegation round's gathered segments,
 * zero-padded), codeword: 4 slot_len (rate 4), betas: slot_len
 * (precompute_beta of the claim's point, zero beyond the reference's
 * 2^(point length) entries), claim: one value, root: the 32-byte root of
 * the codeword's tree. */
typedef struct {
  uint64_t *arr, *codeword, *betas, *claim;
  uint8_t *root;
} gbz_whir_slot;

/* PCS_open_new with isPIOP = true, as coPIOP_prove calls it: the row
 * weights b1 (nb1 entries; the first batches - 1 are used), the row vector
 * b2 (the row length's entries; its last _queries[0] entries are zeroed as
 * the reference does), the party weights b3 (N/4 entries) and the row
 * vector's Lagrange factors (_Lagrange_Evals_input: nlag <= 8 vectors of
 * 2^log_lengths[k] entries back to back, their tensor product factor 0 on
 * the lowest index digits; the log lengths sum to log2 of the row length).
 * The parties' records are gbz_pcs_open_full's; the leader's tail keeps the
 * delegation rounds, 53 UNPACKED and 55 RC, skips aggregate_claims and
 * _Whir_Open and fills the WHIR batch slots 2 and 3 (slots: 2 entries, may
 * be NULL) from the first two delegation rounds; then
 * delegate_lagrange_eval (delegate_protocol.cpp:603-710): 56 BETA_Y 16B
 * (y), 48/49 (_cubic_sumcheck of the rounds' Lagrange tensor, the
 * transform of the factors' tensor with its last _queries[0] entries
 * zeroed, omega^j), 57 L_EVALS 16B x rounds, 48/49 (_cubic_sumcheck of
 * phi / row length, the factors' tensor and the ones vector, unchecked), 69
 * LAG_EVALS 16B x nlag.  *flags as gbz_pcs_open_full's, plus bit 8: a
 * "delegating betas 2" check (returns GBZ_ECHECK) and bit 9: "delegating
 * betas 3" (printed).  Transcript bytes and slot_len:
 * gbz_pcs_open_piop_bytes.
 * replaces PCS_open_new (coPCS.cpp:1310-1690, isPIOP) on N ranks. */
gbz_status gbz_pcs_open_piop(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *b1, int nb1, const uint64_t *b2,
                             uint64_t nb2, const uint64_t *b3, int nb3, const uint64_t *lagrange,
                             const int *log_lengths, int nlag, const uint64_t *K, uint64_t *fs, gbz_prng *prng,
                             uint32_t *flags, gbz_whir_slot *slots, uint8_t *transcript, uint64_t capacity, int mem);
gbz_status gbz_pcs_open_piop_bytes(const gbz_pcs *pcs, const int *log_lengths, int nlag, uint64_t *bytes,
                                   uint64_t *slot_len);

/* F_ip of the committed data with input vectors (MPI_utils.cpp:483-553, as
 * coPIOP_prove forms the claim of its PCS opening): K = sum_p lambda_p
 * sum_{i < batches - 1} sum_j b1[i] b2[j] Commit_data_p[i][j], with
 * lambda the party weights of b3 (N/4 entries) and b2 (the row length's
 * entries) zero on its last _queries[0] entries as gbz_pcs_open_piop uses
 * it.  K: 2 words (mem). */
gbz_status gbz_pcs_claim_piop(gbz_ctx *ctx, const gbz_pcs *pcs, const uint64_t *b1, int nb1, const uint64_t *b2,
                              uint64_t nb2, const uint64_t *b3, int nb3, uint64_t *K, int mem);

/* quadratic_coSumcheck / cubic_coSumcheck of N parties on one device
 * (form GBZ_SC_QUADRATIC or GBZ_SC_CUBIC).  p1, p2 (and p3): N x n party
 * shares, party-major; R: the parties' sparse vectors, N x sum_i (2 or 4)
 * degrees[i], R[i] back to back; r1 (cubic: log2 n entries, b1 =
 * precompute_beta(r1)) and r2 (cubic: log2(N/4) entries, the aggregation
 * weights b2 = precompute_beta(r2)); K, K_r: the claim and the sparse claim;
 * fs: the Fiat-Shamir chain, updated.  Every round runs the parties' block
 * transforms (phase 1, the cubic form skipping blocks whose p1 part is zero
 * as the reference does), adds c R, aggregates the N messages as
 * sumcheck_aggr, checks, draws the challenge, folds R and every vector
 * (phase 2); then the parties' final values are unpacked and checked and the
 * claims formed.  claims: rows x (eval, r[0..ndeg]) with rows = 5
 * (quadratic) / 4 (cubic) and r = the final challenge then the round
 * challenges, 2 (ndeg + 2) words per row.  The reference prints and
 * continues when a check fails; *flags (may be NULL) gets the same
 * information: bit i = round i's message did not match K, bit 29 = the
 * final check, bit 30 = the cubic form's b1 check.  The inputs are not
 * modified.  Transcript (may be NULL; gbz_cosumcheck_transcript_bytes):
 *   36 CHALLENGE (c of {K, K_r}) | per round 34 PARTY_POLYS 16B x DN,
 *   35 POLY 16B x D, 36 CHALLENGE (D = 2d / 4d) | 43 FINAL_SHARES 16B x
 *   rows N (party-major) | 44 UNPACKED 16B x rows N/2 | 36 CHALLENGE |
 *   45 CLAIMS 16B x rows
 * replaces quadratic_coSumcheck (coSumcheck.cpp:233-331) and
 * cubic_coSumcheck (coSumcheck.cpp:335-448) on N ranks. */
gbz_status gbz_cosumcheck(gbz_ctx *ctx, int form, int N, uint64_t n, const uint64_t *p1, const uint64_t *p2,
                          const uint64_t *p3, const uint64_t *R, const uint64_t *r1, int nr1, const uint64_t *r2,
                          const uint64_t *K, const uint64_t *K_r, const int *degrees, int ndeg, uint64_t *fs,
                          uint64_t *claims, uint32_t *flags, uint8_t *transcript, uint64_t capacity, int mem);
uint64_t gbz_cosumcheck_transcript_bytes(int form, int N, const int *degrees, int ndeg);

/* ------------------------------------------------- R1CS front end (pigeon 1) */

/* The parties' rows of the R1CS matrices A, B, C (what pA, pB, pC hold on
 * every rank after distribute_index, MPI_utils.cpp:2205-2270, 2483-2597):
 * per matrix a CSR over N x rows rows, party p owning rows [p rows,
 * (p + 1) rows): ptr[t] (N rows + 1 entries, from 0 to nnz[t]) and cols[t]
 * (the constraint index of every nonzero, below 2^logm; all nonzeros are 1),
 * host arrays, uploaded once. */
typedef struct gbz_r1cs gbz_r1cs;
gbz_status gbz_r1cs_create(gbz_ctx *ctx, int N, uint64_t rows, int logm, const uint32_t *const *ptr,
                           const uint32_t *const *cols, const uint64_t *nnz, gbz_r1cs **out);
gbz_status gbz_r1cs_free(gbz_r1cs *m);

/* _reduce_R1CS_matrixes_multivariate (Distributed_Sumcheck.cpp:2283-2350) of
 * every party: with degrees' = (N/4, degrees1[0 .. ndeg1-2]), beta1 = the
 * tensor of compute_lagrange_coeff(degrees'[i], r[i]) for i < ndeg1 - 1 (the
 * first factor varying fastest) and beta2 = compute_lagrange_coeff(
 * degrees'[ndeg1-1], r[ndeg1-1]), row j of party p of RA is the sum over its
 * columns c of beta1[c mod S] beta2[c div S], S = |beta1| = 2^logm / |beta2|;
 * RB, RC likewise.  r: ndeg1 = nr entries; RA, RB, RC: N x rows. */
gbz_status gbz_r1cs_reduce(gbz_ctx *ctx, const gbz_r1cs *m, const uint64_t *r, int nr, const int *degrees1,
                           int ndeg1, uint64_t *RA, uint64_t *RB, uint64_t *RC, int mem);

/* prove_phase1 (coPIOP.cpp:241-346) of N parties: the first sumcheck of the
 * R1CS front end.  vL, vR, vO: N x n party shares; masks: N x 12 (rL, rR,
 * rO: the first 12 entries of each party's mask randomness R,
 * coPIOP.cpp:1585-1589); R1: N x sum_i 4 degrees[i] (the parties' shares of
 * the first sumcheck's randomness, rounds back to back); degrees: degrees1
 * (their product is 2n); fs: the Fiat-Shamir chain, updated.  Draws _r1
 * (log2 n) and _r2 (log2 N/4) by hash_to_field({0}), forms every party's
 * y = sum_{i<4} _beta(i, _r1) (rL rR - rO) and the leader's interpolation,
 * draws r1's last entry, doubles vL, vR, vO with the masks at the start of
 * the new half, computes K_r (compute_Kr) and runs cubic_coSumcheck.
 * Outputs: claims (4 rows x (ndeg + 2) field elements: eval, r_final, the
 * round challenges, as gbz_cosumcheck), ip (N x sum 4 degrees: every party's
 * sumcheck1_ip), ip_b1 (N/4: the Lagrange vector _sumcheck1_ip[1]; may be
 * NULL), vectors (3 x N x 2n: the doubled vL, vR, vO; may be NULL), flags
 * (gbz_cosumcheck's).  Transcript (gbz_piop_phase1_bytes; may be NULL):
 *   58 PIOP_DRAWS 16B x (log2 n + log2(N/4) + 1) | 59 PIOP_Y 16B x (N + 2):
 *   the parties' y, the leader's y, K_r | the cubic coSumcheck's records. */
gbz_status gbz_piop_phase1(gbz_ctx *ctx, int N, uint64_t n, const uint64_t *vL, const uint64_t *vR,
                           const uint64_t *vO, const uint64_t *masks, const uint64_t *R1, const int *degrees,
                           int ndeg, uint64_t *fs, uint64_t *claims, uint64_t *ip, uint64_t *ip_b1,
                           uint64_t *vectors, uint32_t *flags, uint8_t *transcript, uint64_t capacity, int mem);
uint64_t gbz_piop_phase1_bytes(int N, uint64_t n, const int *degrees, int ndeg);

/* prove_phase2 (coPIOP.cpp:406-627) of N parties: the second sumcheck.  w:
 * N x nw (each party's witness as coPIOP_prove hands it over after
 * PCS_commit); masks: as phase 1; m: the R1CS rows; mask_l: the PCS mask
 * length (the gap in each of the 32 segments); R2: N x sum_i 2 degrees2[i];
 * point1: phase 1's claim point (ndeg1 + 1 entries: r_final then the round
 * challenges); evals1: phase 1's first three claim values (yL, yR, yO); K:
 * the second sumcheck's randomness claim (generate_sumcheck_randomness).
 * Reduces the R1CS rows at point1 without its last entry, draws a, b, c,
 * forms L_last[0] (a RA + b RB + c RC), reshares it (secret_share_vector)
 * into 32 segments, appends the parties' beta shares (times L_last[1]),
 * pairs it with (w, a rL + b rR + c rO) and runs quadratic_coSumcheck on
 * a yL + b yR + c yO.  Outputs: claims (5 rows x (ndeg2 + 2); row 1's value
 * divided by L_last[0] as the reference returns it), abc (3), ip2 (N x sum
 * 2 degrees2: sumcheck2_ip), ip3 (N x 12: sumcheck3_ip), ip_b1 (N/4), vectors
 * (2 x N x 2nw: the coSumcheck's two vectors; may be NULL), flags.
 * Transcript (gbz_piop_phase2_bytes): 60 PIOP_ABC 16B x 3 | the quadratic
 * coSumcheck's records. */
gbz_status gbz_piop_phase2(gbz_ctx *ctx, int N, uint64_t nw, const uint64_t *w, const uint64_t *masks,
                           const gbz_r1cs *m, int mask_l, const uint64_t *R2, const uint64_t *point1,
                           const uint64_t *evals1, const int *degrees1, int ndeg1, const int *degrees2, int ndeg2,
                           const uint64_t *K, uint64_t *fs, uint64_t *claims, uint64_t *abc, uint64_t *ip2,
                           uint64_t *ip3, uint64_t *ip_b1, uint64_t *vectors, uint32_t *flags, uint8_t *transcript,
                           uint64_t capacity, int mem);
uint64_t gbz_piop_phase2_bytes(int N, const int *degrees2, int ndeg2);

/* ------------------------------------------------- distributed PCS (witness) */

/* Batch_dCommit (distributed_PCS.cpp:56-147) of N parties (8 <= N <= 64):
 * arr, arr2: N x A.  Row k < batch of party p is arr_p[k S, (k+1) S)
 * (S = A / batch) zero-padded to L = rate S; the reference's distributed
 * FFT over the N ranks (distributed_batch_FFT, MPI_utils.cpp:3133-3298) is
 * the transform of length N L of the rows interleaved across the parties
 * (party p's entry t is coefficient t N + p), party r keeping the L/N
 * outputs from r L/N + m L for every m < N.  Each party's tree hashes the
 * columns of its batch rows (MT_commit_Blake over the column) and builds
 * create_tree_blake over the L column hashes; the leader's root is taken
 * over {party 0's root, 0, ..., 0}.  Outputs (each may be NULL):
 * commit_data (N x A: arr2, as the reference keeps it), codewords (N x
 * batch x L), levels (N x (2L - 1) x 32, leaves first), roots (N x 32, host),
 * leader_root (32, host).  batch: a power of two in [4, 64]. */
gbz_status gbz_dpcs_batch_commit(gbz_ctx *ctx, int N, uint64_t A, const uint64_t *arr, const uint64_t *arr2, int rate,
                                 int batch, uint64_t *commit_data, uint64_t *codewords, uint8_t *levels, uint8_t *roots,
                                 uint8_t *leader_root, int mem);

/* dCommit (distributed_PCS.cpp:150-170): one row of A entries per party,
 * codeword N x (rate A) by the same distributed transform; the columns are
 * d = 2^(log2 N - log2 N / 2) entries spaced rate A / d apart (the fold
 * degree plaintext_degrees[1] of prepare_data, :28-54); levels: N x
 * (2 rate A / d - 1) x 32. */
gbz_status gbz_dpcs_commit(gbz_ctx *ctx, int N, uint64_t A, const uint64_t *arr, int rate, uint64_t *codeword,
                           uint8_t *levels, uint8_t *roots, uint8_t *leader_root, int mem);

/* PIOP_dOpen_batch_new (distributed_PCS.cpp:1175-1534) of N parties (8 <=
 * N <= 64), P = 2 or 3 committed polynomials (batches = 1): commit_data,
 * codewords: per polynomial what gbz_dpcs_batch_commit returns (P x N x rows
 * x S, P x N x rows x L, L = rate S); points: P x (log2 S + log2 rows +
 * log2 N) (r2, r3, r1 as the reference splits them); claims: P; verify: the
 * reference's Verify[0].  Row-batches every party's data and codeword,
 * forms the eval claims, draws a and b (b[0] set to zero), batches the data
 * with weights {1, b[0], b[1]} as PIOP_dBatch_batched_new receives them,
 * commits the batched codeword (every party's slice of the distributed
 * codeword, columns of plaintext_degrees[1] entries; the leader's root is
 * taken over N zero leaves, coPCS.cpp:398-408) and draws get_indexes; then
 * per fold degree (prepare_data's, :28-54) the parties' block products, the
 * leader's sum, check, challenge and claim, the folds of the data, the
 * betas and (RS_distributed_fold, coPCS_utils.cpp:440-504: the multifold of
 * the global codeword) the codeword, and a commitment of the folded
 * codeword but after the last; finally the leader's Whir_Commit_initial of
 * the gathered data at whir_rate.  Outputs (may be NULL): arr_out, betas_out
 * (N S / prod(degrees): the gathered data and betas, party by party), K_out
 * (the claim), whir_codeword (whir_rate times that), whir_root (32, host);
 * flags bit 0: the first check failed (the reference prints "Sumcheck
 * Error Round" and returns; so does this call, with GBZ_OK).  Transcript
 * (gbz_dpcs_open_bytes): 61 EVAL_CLAIMS 16B x P(P-1) | 62 DRAWS 16B x 4 (a0,
 * a1, b0 as drawn, b1) | per commitment 63 ROOTS 32B x (N + 1) (parties',
 * leader's), 64 QUERIES u32 x 2l ((party, position) per draw) | per round
 * 65 POLY 16B x 2d, 66 CHALLENGE, 67 K | 68 WHIR_ROOT 32B. */
gbz_status gbz_dpcs_open(gbz_ctx *ctx, int N, int P, int rows, uint64_t S, int rate, const uint64_t *commit_data,
                         const uint64_t *codewords, const uint64_t *points, const uint64_t *claims, int verify,
                         int whir_rate, uint64_t *fs, uint64_t *arr_out, uint64_t *betas_out, uint64_t *K_out,
                         uint64_t *whir_codeword, uint8_t *whir_root, uint32_t *flags, uint8_t *transcript,
                         uint64_t capacity, int mem);
uint64_t gbz_dpcs_open_bytes(int N, int P, int rate);

/* ------------------------------------------------------------- verifier */

/* Checks a gbz_prove transcript of a 2^logn witness at `rate` whose glibc
 * stream was seeded with prng_seed, from the transcript alone (host code, no
 * context): the evaluation point and every sumcheck challenge against the
 * Fiat-Shamir chain, every round message against the running claim, the
 * final values against the last claim and eq(z, challenges); per WHIR
 * iteration the round messages against K, the challenges, queries and
 * combination weights against the glibc stream, every folded answer against
 * its replies, and K; then Whir_Open's verification steps 2 and 3
 * (Whir.cpp:441-467) with the betas' final values formed from the closed
 * forms of their terms.  The commitment roots and paths are not checked
 * (with inner nodes hashing their left child twice, merkle_tree.cpp:267-299,
 * a path does not bind a query's replies).  The reference has no standalone
 * verifier; these are the checks its prover runs inline.  *failed (may be
 * NULL) gets one bit per failed check: 1 layout, 2 evaluation point, 4
 * sumcheck sum, 8 sumcheck challenge, 16 final values, 32 WHIR sum, 64 WHIR
 * challenge, 128 queries, 256 answers, 512 combination weights, 1024 K,
 * 2048 final point, 4096 step 2, 8192 step 3.  Returns GBZ_OK when every
 * check holds, GBZ_ECHECK otherwise. */
gbz_status gbz_verify_proof(const uint8_t *transcript, uint64_t bytes, int logn, int rate, uint32_t prng_seed,
                            uint32_t *failed);

/* --------------------------------------------------------------- prover */

/* Bytes of the transcript of one proof of a 2^logn witness at `rate`. */
uint64_t gbz_prove_transcript_bytes(int logn, int rate);

/* One single-party proof: Whir_Commit_initial of the witness (Whir.cpp:158),
 * evaluation point hash_to_field({0}) x logn (main.cpp:83-85), quadratic
 * sumcheck of sum_x w(x) eq(z, x) with Fiat-Shamir challenges
 * (_quadratic_cosumcheck round body, coSumcheck_MPI.cpp:195-219), and
 * Whir_Open of its claim with whir_k = 4 (Whir.cpp:388-467).  The glibc
 * random() stream that the reference draws WHIR challenges and queries from
 * starts from srandom(prng_seed) (1 = the unseeded reference process).
 *
 * The transcript is a sequence of records {u32 tag, u32 count, payload}:
 *  1 COMMIT_ROOT 32B | 2 EVAL_POINT 16B x logn | 3 CLAIM 16B
 *  per round: 4 SC_POLY 16B x3, 5 SC_CHALLENGE 16B | 6 SC_FINAL 16B x2
 *  per WHIR iteration: 2 x (7 WHIR_POLY 16B x3, 8 WHIR_CHALLENGE 16B),
 *    9 WHIR_ROOT 32B, 10 WHIR_QUERIES u32 x l, 11 WHIR_REPLIES 16B x 4l,
 *    12 WHIR_ANSWERS 16B x l, 13 WHIR_PATHS 32B x l*depth,
 *    14 WHIR_COMBINE 16B x l, 15 WHIR_K 16B
 *  16 FINAL_POLY 16B x m | 17 FINAL_POINT 16B x log2 m | 18 FINAL_EVAL 16B
 * witness: 2^logn elements (3 <= logn <= 25, rate a power of two in [2, 64],
 * codeword rate * 2^logn <= 2^26); transcript: gbz_prove_transcript_bytes bytes.
 * With GBZ_MEM_HOST the call also checks the device-side consistency flags
 * (every round's claim) and returns GBZ_ECHECK if one failed. */
gbz_status gbz_prove(gbz_ctx *ctx, const uint64_t *witness, int logn, int rate, uint32_t prng_seed,
                     uint8_t *transcript, uint64_t capacity, int mem);

/* Whir_Open of one claim (Whir.cpp:388-467) on caller arrays, whir_k = 4:
 * arr (2^logn elements), codeword = its rate-fold RS encoding (the codeword
 * Whir_Commit_initial made; rate * 2^logn elements), point (logn elements)
 * and K (2 words) the claim (K = sum_x arr(x) eq(point, x)).  prng is the
 * glibc random() state the reference's F::_random / rand() draws continue
 * from; it is advanced past every draw of the opening.  The commitment tree
 * is not an input: the paths are recomputed from the codeword (inner nodes
 * hash their left child twice, so every node is a chain from one leaf).
 * Transcript: 1 COMMIT_ROOT of the codeword, then the WHIR records of
 * gbz_prove (tags 7-18); gbz_whir_open_transcript_bytes bytes.
 * GBZ_ECHECK when a round message does not match the running claim.
 * replaces Whir_Open (Whir.cpp:388-467). */
gbz_status gbz_whir_open(gbz_ctx *ctx, const uint64_t *arr, int logn, int rate, const uint64_t *codeword,
                         const uint64_t *point, const uint64_t *K, gbz_prng *prng, uint8_t *transcript,
                         uint64_t capacity, int mem);
uint64_t gbz_whir_open_transcript_bytes(int logn, int rate);

/* Kernel launches of one proof (host-side count, no GPU needed); 0 for an
 * unsupported shape. */
int gbz_prove_launches(int logn, int rate);

/* ----------------------------------------------------------- calibration */

/* Measures, on the context's device, the throughput of the F_{p^2} multiply
 * (*fmul_per_s, independent multiply chains on every SM) and of the 64-byte
 * Blake3 compression (*blake3_per_s): the integer-pipe peaks that the NTT,
 * RS fold and Merkle kernels are bounded by.  Either output may be NULL.
 * Takes a few tens of milliseconds.  No counterpart in the reference. */
gbz_status gbz_calibrate(gbz_ctx *ctx, double *fmul_per_s, double *blake3_per_s);

/* ------------------------------------------------------------ autotuning */

/* The shape of the two-pass (four-step) transforms of length 2^logn,
 * 14 <= logn <= 28: k1 = log2 of the contiguous second pass (the first pass
 * has length 2^(logn - k1)), 2^log_cols_a columns staged per CTA in the first
 * pass and 2^log_rows_b rows per CTA in the second.  Every valid shape
 * computes the same values; only speed differs.  Shapes are process-wide:
 * change them while no transform is in flight. */
gbz_status gbz_ntt_set_shape(int logn, int k1, int log_cols_a, int log_rows_b);
gbz_status gbz_ntt_get_shape(int logn, int *shape);  /* shape: 3 ints */

/* Times every candidate shape for 2^logn on the context's device (best of
 * reps forward transforms each) and installs the fastest; shape (3 ints),
 * ms_default and ms_best (optional) report the choice.  No counterpart in
 * the reference, whose fft has a single radix-2 schedule. */
gbz_status gbz_ntt_autotune(gbz_ctx *ctx, int logn, int reps, int *shape, double *ms_default, double *ms_best);

/* The first pass of a two-pass transform multiplies by omega_L^(n1 k2) read
 * from a table of L elements per (length, split, direction), built with the
 * length's twiddles (2 L * 16 bytes of device memory, kept for the process);
 * disabled, it forms each factor from two small tables with one more
 * multiply.  Same values either way; process-wide. */
void gbz_ntt_full_twiddles(int enable);

/* Merkle level fusion: each launch computes 2^log_nodes_per_cta nodes of a
 * level per CTA and the levels above them inside its subtree (10 or 11;
 * process-wide; the hashes are the same either way). */
gbz_status gbz_merkle_set_fusion(int log_nodes_per_cta);
int gbz_merkle_get_fusion(void);
/* Times both fusion depths on a tree over 2^logN elements and installs the
 * faster. */
gbz_status gbz_merkle_autotune(gbz_ctx *ctx, int logN, int reps, int *log_nodes, double *ms_default,
                               double *ms_best);

/* gbz_prove replays the proof as a captured CUDA graph (captured on first
 * use of a witness address, at most four per shape; the seed is a graph
 * parameter) unless disabled here, profiling is on, or the context's stream
 * is a default stream (which cannot be captured).  Same transcript either way. */
gbz_status gbz_set_graphs(gbz_ctx *ctx, int enable);

/* ------------------------------------------------------------ profiling */

/* Per-category CUDA-event timing of the kernels gbz_prove enqueues, on the
 * context's stream.  Categories: 0 NTT, 1 Merkle, 2 sumcheck fold/reduce,
 * 3 eq table, 4 WHIR beta update, 5 WHIR queries, 6 protocol steps
 * (Fiat-Shamir, PRNG draws, round messages). */
#define GBZ_PROF_CATEGORIES 7
gbz_status gbz_profile_enable(gbz_ctx *ctx, int enable);
/* Milliseconds and event-bracketed launch groups per category summed over
 * the proofs of shape (logn, rate) since the last read; resets the sums.
 * Waits for those proofs to finish. */
gbz_status gbz_profile_read(gbz_ctx *ctx, int logn, int rate, double *ms, int *groups);

#ifdef __cplusplus
}
#endif

#endif /* GBZ_H */
