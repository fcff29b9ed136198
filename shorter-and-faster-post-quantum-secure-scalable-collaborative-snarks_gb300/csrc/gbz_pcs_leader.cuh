// The leader's side of PCS_open_new after the parties' rounds
// (gbz_pcs_leader.cu): the delegation proofs of every delegate check after
// the first (coPCS.cpp:770-831 with prove_multi_folding and
// prove_extension, delegate_protocol.cpp:147-429), the final checks on the
// parties' data, the aggregation of the delegation claims and the WHIR
// opening of the gathered segments (coPCS.cpp:1697-1753 with
// aggregate_claims, aggregate_commitments and _Whir_Open, Whir.cpp:469-668)
// and delegate_beta_eval (delegate_protocol.cpp:431-504); in the PIOP mode
// (isPIOP, coPCS.cpp:1619-1690) the WHIR batch slots instead of the opening
// and delegate_lagrange_eval (delegate_protocol.cpp:603-710).
#pragma once
#include <functional>
#include <vector>

#include "gbz_prover.cuh"

namespace gbz {

// One round of the parties' opening as the tail reads it (device pointers).
struct LeaderRound {
  int d = 0, l = 0;        // fold degree _degrees[i+1], delegate-check queries _queries[i+1]
  uint64_t n = 0;          // C_prime.size() when the round starts
  uint64_t C0 = 0;         // C[0].size(): row length of the previous concatenated code (rounds >= 1)
  int rate_next = 0, rate_cur = 0;  // _rates[i+2][0], _rates[i+1][0]: the positions' rescale
  const fe *L = nullptr;   // d Lagrange weights of the round
  const fe *seg = nullptr; // l x d gathered segments (rounds >= 1)
  const fe *y = nullptr;   // l folded values (rounds >= 1)
  const int32_t *qp = nullptr, *qpos = nullptr;  // l (party, position), the leader's order
  const fe *s = nullptr;   // the round's phase-3 challenge (every round but the last)
};

// One WHIR batch slot the PIOP mode fills (whir_polys, whir_c, whir_betas,
// whir_claims, whir_MTs of coPCS.cpp:1620-1629): device buffers, each may be null.
struct WhirSlotDev {
  fe *arr = nullptr;      // max_delegation entries
  fe *cw = nullptr;       // 4 max_delegation entries
  fe *betas = nullptr;    // precompute_beta of the claim's point (max_delegation entries)
  fe *claim = nullptr;    // the claim's value
  uint8_t *root = nullptr;  // 32 bytes
};

struct LeaderInputs {
  int N = 0;
  uint64_t Bs = 0;               // row length (instance_size[0])
  int log_rate_offset = 0;
  std::vector<int> rate0;        // _rates[i][0]
  std::vector<LeaderRound> rounds;
  const fe *bcd = nullptr, *B = nullptr, *Cp = nullptr;  // every party's final data, B and C'
  uint64_t n_final = 0, cpl_final = 0;
  const fe *K = nullptr, *r_first = nullptr;  // running claim and batching challenge (device)
  const fe *b2 = nullptr;        // the transform of precompute_beta(r2) (Bs entries)
  const fe *b3 = nullptr;        // precompute_beta(r3) (N/4 entries)
  const fe *r2 = nullptr;        // r2 (log2 Bs entries)
  uint64_t max_delegation = 0;
  const fe *unpack = nullptr;    // (N/2) x N: share weights of unpack_secret_share(., N/2, N)
  // the PIOP mode: the Lagrange factors of the input row vector
  // (_Lagrange_Evals_input, back to back, 2^loglag[k] entries each), the
  // entries _queries[0] zeroed at the end of a row, the slots to fill
  bool piop = false;
  int nlag = 0;
  int loglag[8] = {};
  const fe *lag = nullptr;
  uint64_t q0 = 0;
  WhirSlotDev slot[2];
};

// Flag bits of the tail, after the reference's messages.
enum : uint32_t {
  LF_ROUND = 1u,         // "Error in sumcheck round": a quadruple / cubic round message (printed, continues)
  LF_DELEGATION = 2u,    // "Error V, Delegation 1..7" or a verified quadratic round (exits)
  LF_DECODING = 4u,      // "ERROR in decoding" of a party's final codeword (returns)
  LF_FINAL1 = 8u,        // "Error in final verification step 1" (printed)
  LF_WHIR = 16u,         // the WHIR opening's sumcheck, K or re-encoding check (exits)
  LF_WHIR_STEP3 = 32u,   // "Error in verification step 3" (printed)
  LF_FINAL = 64u,        // "Error in final verification step" (exits)
  LF_BETAS = 128u,       // "Error in delegating betas 1" (exits)
  LF_LAG2 = 256u,        // "Error in delegating betas 2" of delegate_lagrange_eval (exits)
  LF_LAG3 = 512u,        // "Error in delegating betas 3" of delegate_lagrange_eval (printed)
  LF_FATAL = LF_DELEGATION | LF_DECODING | LF_WHIR | LF_FINAL | LF_BETAS | LF_LAG2
};

struct LeaderResources {
  cudaStream_t s = nullptr;
  std::function<void *(uint64_t)> alloc;     // device scratch held until the call ends
  std::function<NttTables &(int)> tables;    // twiddle tables by log2 length
};

// The tail's draws from the leader's generator, in order: F::_random()
// values into the arena at off, rand() % mod values into the transcript at
// off, the state handed to the WHIR opening (which draws itself), the calls
// the opening makes.
enum { DRAW_FIELDS = 0, DRAW_INTS = 1, DRAW_STATE = 2, DRAW_SKIP = 3 };
struct DrawOp {
  int kind, count;
  uint32_t mod;
  uint64_t off;
};
struct LeaderDraws {
  fe *arena = nullptr;               // the F::_random() values
  glibc_prng *after_walk = nullptr;  // the state after the opening's calls (checked against the opening's)
  glibc_prng *final_state = nullptr; // the generator at the end of the tail
};

// Lays out (tr == nullptr: records appended to lay, the draws to *script,
// the arena length to *arena_len) or enqueues the tail (offsets relative
// to tr; the draws read from d, which the script kernel fills).  st: the
// generator the WHIR opening draws from and its flags; *flags receives the
// LF_* bits on the device.
void leader_tail(LeaderResources &R, const LeaderInputs &in, ProofState *st, uint32_t *flags, uint8_t *tr,
                 Layout &lay, std::vector<DrawOp> *script, uint64_t *arena_len, const LeaderDraws *d);
// st's generator from g, its flags and *flags cleared (enqueued on s).
void leader_tail_init(ProofState *st, const glibc_prng &g, uint32_t *flags, cudaStream_t s);
// The script of draws (ops: device memory) from state g0, one thread on s;
// it runs beside the parties' rounds: nothing it reads depends on them.
void leader_draws_launch(const glibc_prng &g0, const DrawOp *ops, int nops, const LeaderDraws &d, uint8_t *tr,
                         ProofState *st, cudaStream_t s);

}  // namespace gbz
