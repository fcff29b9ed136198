// Internal declarations shared by the libgbz translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "gbz_blake3.cuh"
#include "gbz_field.cuh"

namespace gbz {

constexpr int kMaxLogN = 28;        // largest vector, Merkle tree or eq table: 2^28 elements
constexpr int kMaxNttLogN = 26;     // largest transform: two passes of at most 2^13
constexpr int kMaxQueries = 256;    // WHIR queries per iteration (rate 2 needs 200)
constexpr int kWhirLogK = 2;        // folding factor 4 (whir_k = 4) of the plain prover
constexpr int kWhirK = 1 << kWhirLogK;
constexpr int kMaxWhirLogK = 4;     // batch opening: folding factors up to 16
constexpr int kFinalMax = 16;       // largest final polynomial of an opening
constexpr int kMaxWhirIter = 16;    // WHIR iterations of one proof (2^26 at rate 2 needs 12)

// Transcript record tags (one u32 tag, one u32 count, then count units).
enum : uint32_t {
  T_COMMIT_ROOT = 1, T_EVAL_POINT = 2, T_CLAIM = 3, T_SC_POLY = 4, T_SC_CHALLENGE = 5,
  T_SC_FINAL = 6, T_WHIR_POLY = 7, T_WHIR_CHALLENGE = 8, T_WHIR_ROOT = 9,
  T_WHIR_QUERIES = 10, T_WHIR_REPLIES = 11, T_WHIR_ANSWERS = 12, T_WHIR_PATHS = 13,
  T_WHIR_COMBINE = 14, T_WHIR_K = 15, T_FINAL_POLY = 16, T_FINAL_POINT = 17,
  T_FINAL_EVAL = 18, T_SCHEDULE = 19, T_AGGR_CHALLENGES = 20, T_AGGR_K = 21, T_AGGR_QUERIES = 22,
  T_AGGR_PATHS = 23, T_AGGR_ROOT = 24
};

// Batched launches: proof p of a batch of same-shape proofs works on its
// pointer arguments advanced by p times their per-proof byte strides (the
// proof index is grid.y for kernels of many CTAs per proof, grid.x for
// kernels of one CTA per proof).  A single proof passes zero strides.
struct BStr {
  uint64_t s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
};
template <typename T>
__device__ __forceinline__ T *badv(T *q, uint64_t stride, uint32_t p) {
  return reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(q) + stride * p);
}

// Transcript records start at 4-byte multiples (query records have 4-byte
// units), so every store into the transcript is a 32-bit store.
__device__ __forceinline__ void put_fe(uint8_t *tr, uint64_t off, fe v) {
  uint32_t *p = reinterpret_cast<uint32_t *>(tr + off);
  p[0] = (uint32_t)v.re;
  p[1] = (uint32_t)(v.re >> 32);
  p[2] = (uint32_t)v.im;
  p[3] = (uint32_t)(v.im >> 32);
}

// Verifier-side randomness and running claims of one proof, resident in
// device memory so that the whole proof is one stream of launches with no
// host round trip (and can be captured in a CUDA graph).  Replaces the
// reference's process-global prev_challenge (Fiat_Shamir.cpp:5) and glibc
// generator state with per-proof state.
struct ProofState {
  fe fs;                      // Fiat-Shamir chain value (prev_challenge)
  glibc_prng prng;            // glibc random() state
  fe y;                       // running sumcheck claim
  fe K;                       // WHIR running claim
  fe chal[64];                // sumcheck challenges (the claim point)
  fe z[64];                   // evaluation point
  fe rw[kMaxWhirLogK];        // WHIR round challenges of the current iteration
  fe hw[kMaxWhirLogK][3];     // WHIR round messages of the current iteration
  fe fin_r[8];                // final point
  int32_t q[kMaxQueries];     // queries scaled to the new codeword
  fe comb[kMaxQueries];       // update_betas combination weights c_i = r^(i+1)
  fe qw[kMaxQueries];         // c_i-weighted query roots, see whir kernels
  fe omega_q[kMaxQueries];    // omega_N^{q_i}
  uint32_t error;             // non-zero: a device-side consistency check failed
  uint32_t seed_in;           // PRNG seed of the next proof when it is replayed from a graph
  uint32_t nonreal;           // the witness has an imaginary word (general commit transform)
  fe epre;                    // prod_{k < i} eq1(z_k, chal_k): the folded eq prefix of the sumcheck
  // The prover's WHIR randomness, drawn up front (it depends on the seed
  // only): per iteration the two round challenges, the query positions and
  // update_betas' r; and the round messages, kept per iteration for the
  // query chain that checks and updates K.
  fe wr[kMaxWhirIter][kWhirLogK];
  fe wrb[kMaxWhirIter];
  int32_t wq[kMaxWhirIter][kMaxQueries];
  fe whw[kMaxWhirIter][kWhirLogK][3];
};

// Error capture for the C-ABI.
struct Err {
  int code = 0;
  std::string msg;
};

#define GBZ_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) throw ::gbz::CudaError(e_, #call, __FILE__, __LINE__);         \
  } while (0)

struct CudaError {
  cudaError_t err;
  std::string what;
  CudaError(cudaError_t e, const char *call, const char *file, int line) : err(e) {
    what = std::string(cudaGetErrorString(e)) + " in " + call + " at " + file + ":" + std::to_string(line);
  }
};

struct ArgError {
  std::string what;
  explicit ArgError(std::string w) : what(std::move(w)) {}
};

inline int ilog2(uint64_t x) {
  int l = 0;
  while ((1ull << (l + 1)) <= x) l++;
  return l;
}
inline bool is_pow2(uint64_t x) { return x && !(x & (x - 1)); }

// ------------------------------------------------------------------ NTT
// Twiddle tables for one transform length, resident in device memory.
struct NttTables {
  int logn = -1;
  fe *sub_fwd = nullptr;   // omega_S^t for every sub-length S = 2^s, s <= 13, packed
  fe *sub_inv = nullptr;
  fe *lo_fwd = nullptr, *hi_fwd = nullptr;  // omega_L^e = lo[e & 4095] * hi[e >> 12]
  fe *lo_inv = nullptr, *hi_inv = nullptr;
  fe inv_len;              // L^{-1}
};

// Forward (inverse = false) or inverse transform of length 2^logn with the
// reference's semantics (utils.cpp:904-964): out[k] = sum_j in[j] w^{jk},
// w = getRootOfUnity(logn) (inverted and scaled by 2^-logn for the inverse).
// `in` holds n_valid elements; the rest of the length is zero (RS padding).
// `tmp` must hold 2^logn elements when logn > 13.  in may equal out.
void ntt_launch(const NttTables &t, const fe *in, uint64_t n_valid, fe *out, fe *tmp, bool inverse,
                cudaStream_t s);
// The forward transform (length N = 2^t_full.logn) of an input whose
// entries are expected in the base field: pairs of them are packed into one
// extension element, transformed at length N/2 (t_half) and unpacked by the
// conjugate symmetry of a base-field input's spectrum.  The packed pass sets
// *nonreal (device, to be zeroed by the caller) when an imaginary word is
// non-zero, and then the general transform, which otherwise exits at once,
// overwrites out: the result is the plain transform for every input.  tmp
// holds N entries; n_valid is even.
void ntt_launch_real(const NttTables &t_half, const NttTables &t_full, const fe *in, uint64_t n_valid, fe *out,
                     fe *tmp, uint32_t *nonreal, cudaStream_t s);
int ntt_launch_real_count(int logn);
// `rows` transforms of the same length in the same launches: row r reads
// in + r in_stride (n_valid entries, zero beyond) and writes out + r
// out_stride, output k at out_elem_stride * k within the row; tmp holds
// rows * 2^logn elements when logn > 13.
void ntt_launch_rows(const NttTables &t, const fe *in, uint64_t n_valid, uint64_t in_stride, fe *out,
                     uint64_t out_stride, int rows, fe *tmp, bool inverse, cudaStream_t s,
                     uint64_t out_elem_stride = 1);
// acc[j] += sum_i c[i] * omega_L^{q[i] j} for j < nacc (L = 2^t.logn > 2^13,
// 1 <= l <= kMaxQueries): the forward transform of the sparse vector
// sum_i c_i e_{q_i} as one second-pass launch whose rows are formed directly
// from the entries (the first pass of a few nonzeros is skipped), only the
// first nacc outputs accumulated.  tmp holds 768 bytes of column chains.  With q_shift > 0
// the positions are q[i] >> q_shift (the caller guarantees the dropped bits
// are zero, so omega_L^{q j} = omega_{L'}^{(q >> shift) j} on t of length L').
void ntt_sparse_accumulate(const NttTables &t, const int32_t *q, const fe *c, int l, fe *acc, uint64_t nacc,
                           fe *tmp, cudaStream_t s, int q_shift = 0);
void ntt_tables_build(NttTables &t, int logn);
int ntt_launch_count(int logn);
// count independent transforms of length 2^t.logn (<= 2^13): transform g
// reads in[g * in_stride + j] for j < j_valid (zero beyond) and writes
// out[g * 2^logn + k].
void ntt_batched(const NttTables &t, const fe *in, uint64_t in_stride, uint32_t j_valid, fe *out, uint64_t count,
                 bool inverse, cudaStream_t s);
// count transforms of length 2^t.logn (<= 2^13) over columns: transform g
// reads in[g + j * col_stride] for j < j_valid (zero beyond) and writes
// out[g * 2^logn + k].
void ntt_batched_strided(const NttTables &t, const fe *in, uint64_t col_stride, uint32_t j_valid, fe *out,
                         uint64_t count, bool inverse, cudaStream_t s);
void ntt_tables_free(NttTables &t);
// Four-step shape of the two-pass transforms (lengths above 2^13): pass B
// length 2^k1 (contiguous rows), 2^logBA columns per CTA in pass A and
// 2^logBB rows per CTA in pass B.  Every shape computes the same values.
struct NttShape {
  int k1 = -1, logBA = -1, logBB = -1;
};
NttShape ntt_default_shape(int logn);
NttShape ntt_get_shape(int logn);
bool ntt_shape_valid(int logn, const NttShape &sh);
void ntt_set_shape(int logn, const NttShape &sh);  // process-wide
std::vector<NttShape> ntt_shape_candidates(int logn);
// Frees the first-pass twiddle tables of splits other than k1 (process-wide).
void outer_table_keep_only(int logn, int k1);
// Whether the first pass reads its twiddles from the full tables (default)
// or forms them from the two-level tables; the values are the same.
void ntt_use_full_twiddles(bool on);

// --------------------------------------------------------------- Merkle
// MT_commit_Blake (merkle_tree.cpp:195-233) over N elements: levels holds
// N/4 leaf hashes followed by every upper level (N/2 - 1 hashes, 32 B each).
void merkle_commit_launch(const fe *elems, uint64_t N, uint8_t *levels, cudaStream_t s);
void blake3_batch_launch(const uint8_t *in, uint8_t *out, uint64_t count, cudaStream_t s);
inline uint64_t merkle_hashes(uint64_t N) { return N / 2 - 1; }
int merkle_launch_count(uint64_t N);
// Level-fusion depth of the Merkle launches: each CTA computes 2^log nodes
// of a level and the log levels above them (log = 10 or 11; process-wide).
void merkle_set_fusion(int log_nodes_per_cta);
int merkle_get_fusion();
// create_tree_blake (merkle_tree.cpp:267-299) over L leaf hashes stored at
// levels[0 .. L): writes levels 1.. after them (2L - 1 hashes in total).
// trees > 1: that many trees of the same shape, 2L - 1 hashes apart, in the
// same launches.
void merkle_from_leaves_launch(uint8_t *levels, uint64_t L, cudaStream_t s, int trees = 1);

// ------------------------------------------------------------- sumcheck
// One fused sumcheck step over vectors (a, b) of length m:
//   chal == nullptr : round message of (a, b) itself;
//   chal != nullptr : fold a, b by *chal into (a2, b2) of length m/2 and,
//                     when reduce, the round message of the folded vectors.
// Per-block partial sums go to `partial` (3 fe per block).
int sc_blocks(uint64_t pairs);
void sc_step_launch(const fe *a, const fe *b, uint64_t m, const fe *chal, fe *a2, fe *b2, bool reduce,
                    fe *partial, int blocks, cudaStream_t s);
// Two rounds whose challenges are known in advance, in one pass: the
// messages of (a, b) and of its fold by *chal0 (partials of blocks CTAs in
// partial0 and partial1, blocks <= sc_blocks(m / 4)), and (a4, b4) of length
// m/4, the fold by *chal0 then *chal1.  m >= 4.
// batch > 1: grid.y = proof, bs the strides of (a, b, chal0, chal1, a4, b4,
// partial0, partial1) (sc_fold2) / (a, E2, c, chal0, chal1, a4, b4,
// partial0, partial1) (sc_fold2_eq) / (a, E, chal, a2, E2, partial)
// (sc_eq_step).
void sc_fold2_launch(const fe *a, const fe *b, uint64_t m, const fe *chal0, const fe *chal1, fe *a4, fe *b4,
                     fe *partial0, fe *partial1, int blocks, cudaStream_t s, int batch = 1, const BStr &bs = BStr());
// The same with b = precompute_beta(c) given by E2, the eq table of c[2..]
// (m/4 entries): b is not read, b4 = eq1(c0, r0) eq1(c1, r1) E2.
void sc_fold2_eq_launch(const fe *a, const fe *E2, uint64_t m, const fe *c, const fe *chal0, const fe *chal1, fe *a4,
                        fe *b4, fe *partial0, fe *partial1, int blocks, cudaStream_t s, int batch = 1,
                        const BStr &bs = BStr());
// The same steps for the sumcheck of sum_x w(x) eq(z, x) with the eq vector
// kept as the shrinking table E_i of z_{i+1..}: chal == nullptr gives the
// sums S(0), S(1) of (a, E); otherwise a is folded by *chal into a2 (m/2),
// E2 = pairwise sums of E (m/4) and, when reduce, the sums of (a2, E2).
// Partials are (S0, S1, 0) per block.
void sc_eq_step_launch(const fe *a, const fe *E, uint64_t m, const fe *chal, fe *a2, fe *E2, bool reduce,
                       fe *partial, int blocks, cudaStream_t s, int batch = 1, const BStr &bs = BStr());
// Round-message reduction of `blocks` partials into out[3].
void sc_sum_launch(const fe *partial, int blocks, fe *out3, cudaStream_t s);

// precompute_beta (utils.cpp:198-243) of r (nr values, device) into B.
// batch > 1: grid.y = proof, r and B advanced by their byte strides per proof.
void beta_launch(const fe *r, int nr, fe *B, cudaStream_t s, int batch = 1, uint64_t r_stride = 0,
                 uint64_t B_stride = 0);

// update_betas (Whir.cpp:325-342): b[j] += sum_i comb[i] * omega_q[i]^j.
// pw_scratch holds kUpdateBetasScratch elements.
constexpr uint64_t kUpdateBetasScratch = (uint64_t)kMaxQueries * 256;
// batch > 1: proof p updates b + p b_stride with st + p and its scratch at
// pw_scratch + p pw_stride (byte strides).
void update_betas_launch(fe *b, uint64_t nb, const ProofState *st, int l, fe *pw_scratch, cudaStream_t s,
                         int batch = 1, uint64_t b_stride = 0, uint64_t pw_stride = 0);

// ----------------------------------------------------------- calibration
// Measured throughput of the F_{p^2} multiply and of the 64-byte Blake3
// compression on the current device (scratch: calibrate_scratch_bytes).
void calibrate_int_pipes(cudaStream_t s, void *scratch, double *fmul_per_s, double *blake3_per_s);
uint64_t calibrate_scratch_bytes(int sms);

}  // namespace gbz
