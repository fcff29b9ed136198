// Round forms of the multilinear sumcheck provers and the device-resident
// distributed sumcheck (gbz_rounds.cu).
#pragma once
#include "gbz_internal.cuh"

namespace gbz {

enum { SC_QUADRATIC = 0, SC_CUBIC = 1, SC_BATCH = 2, SC_ZEROCHECK = 3, SC_QUADRUPLE = 4 };
constexpr int kMaxFormCoeffs = 5;  // the quadruple form's degree-4 message

struct RoundArgs {
  const fe *in[6];      // vectors of the form, in order
  fe *out[6];           // folded vectors (modes 1 and 2)
  uint64_t pairs;       // pairs of the message (modes 0, 1) or outputs (mode 2)
  const fe *r;          // fold challenge (device)
  const fe *b;          // batching scalar of the batch / zero-check forms (device, optional)
  fe *partial;          // per-CTA message partials (coefficients per CTA)
  const fe *scale;      // optional: vector 2 entry e is multiplied by scale[e >> scale_log] when read
  int scale_log;
};

// Verifier-side state of a device-resident sumcheck.
struct RoundState {
  fe fs;            // Fiat-Shamir chain (prev_challenge)
  glibc_prng prng;  // F::_random() stream of the leader's rounds
  fe y;             // running claim
  uint32_t error;   // bit 0: a round message did not match the claim
};

int form_vectors(int form);
int form_coeffs(int form);
int round_blocks(uint64_t pairs);
// mode 0: message of in; 1: fold by *r into out and message of the result;
// 2: fold only.
void form_step_launch(int form, const RoundArgs &a, int mode, int blocks, cudaStream_t s);
// The rounds i0 (>= 1) .. rounds-1 and the final fold of a sumcheck of
// n-entry vectors whose challenges are drawn ahead, in one CTA (for n >> i0
// up to a few thousand entries): in holds the vectors entering round i0
// (n >> (i0 - 1) entries), buf two sets of n >> i0 entries; round i's
// challenge is draw[first + stride i] (ch[i0 - 1] the previous one); round
// messages go to the transcript at off_polys (coefficients of round i at
// i nc), the final values to fin and to off_fin; *y is the running claim.
struct DrawnTailArgs {
  const fe *in[4];
  fe *buf[2][4];
  uint64_t n;
  int i0, rounds;
  const fe *draw;
  int first, stride;
  fe *ch, *y, *fin;
  uint32_t *flags;
  uint32_t bit;
  uint8_t *tr;
  uint64_t off_polys, off_fin;
};
void form_tail_drawn_launch(int form, const DrawnTailArgs &a, cudaStream_t s);
// Sum of `blocks` partials of nc coefficients into out (device).
void form_sum_launch(const fe *partial, int blocks, int nc, fe *out, cudaStream_t s);

// Rounds of the N-party distributed sumcheck of M entries per party
// (_quadratic_sumcheck / _cubic_sumcheck, Distributed_Sumcheck.cpp:204, 1122):
// log2(M) - offset Fiat-Shamir rounds (none when not positive, and then
// offset = log2 M) plus log2(N 2^offset) leader rounds.
int party_sumcheck_rounds(uint64_t M, int N, int offset, int *fs_rounds);
// Enqueues the whole prover: v holds the form's vectors (N * M entries,
// party-major, read only), w the parties' weights (cubic form), st the
// chain / generator / claim, scratch 12 buffers of N*M/2 entries (two sets
// of six), partial round_blocks(N*M/2) * 4 entries; polys, chal and fin
// receive the round polynomials, challenges and the leader's final values.
// A second stream and two events (fork, join) for work that runs beside
// the rounds; a null stream runs it in line.
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
// Entries per vector from which the party sumcheck runs its remaining
// rounds in one CTA.
constexpr uint64_t kTailEntries = 1u << 14;
// drawn: room for one challenge per glibc round (rounds minus FS rounds).
void party_sumcheck_enqueue(int form, const fe *const *v, uint64_t M, int N, const fe *w, int offset, RoundState *st,
                            fe *const *scratch, fe *partial, fe *polys, fe *chal, fe *fin, fe *drawn,
                            const SideStream &side, cudaStream_t s);

}  // namespace gbz
