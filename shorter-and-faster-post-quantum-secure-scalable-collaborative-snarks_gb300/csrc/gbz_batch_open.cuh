// Batched WHIR opening of several polynomials (Whir_Batch_Open,
// Whir.cpp:706-898) on one device (gbz_batch_open.cu).
#pragma once
#include <functional>
#include <vector>

#include "gbz_internal.cuh"
#include "gbz_prover.cuh"

namespace gbz {

// One executed step of the opening loop (Whir.cpp:761-833).
struct BatchStep {
  bool iterate = false;   // a WHIR iteration folding by kappa
  int kappa = 0;
  bool aggregate = false; // merge arrays first .. first + group - 2 into the current one
  int group = 0, first = 0;
  uint64_t m = 0, L = 0;  // polynomial and codeword length when the step starts
  int rate = 0;
  int l = 0, depth = 0;   // iteration: queries, authentication path length
  int la = 0, depth_a = 0;  // aggregation: queries, path length
  uint64_t leaves_after = 0;  // leaf hashes of the tree the step leaves behind
};

struct BatchPlan {
  int k = 0, rate = 0, whir_k = 0;
  std::vector<uint64_t> sizes;
  std::vector<int> kappa, aggr;     // the schedule of Whir.cpp:731-752
  std::vector<BatchStep> steps;
  std::vector<uint64_t> cw_len;     // codeword length array i comes with (0: never merged)
  uint64_t m_final = 0, transcript_bytes = 0;
  bool zero_tree0 = false;          // the first queries open a tree over zero leaves
};

// The schedule and per-step sizes for k polynomials of non-increasing
// power-of-two sizes; throws ArgError for inputs the reference cannot run
// (it reads its schedule past the end, or opens a leaf beyond its tree).
// With zero_leaves0 > 0 the tree of the first codeword is the one
// aggregate_commitments installs (Whir.cpp:590-605): zero_leaves0 leaf
// hashes, all zero.
BatchPlan batch_plan(int k, const uint64_t *sizes, int rate, int whir_k, uint64_t zero_leaves0 = 0);

struct BatchResources {
  cudaStream_t s = nullptr;
  std::function<void *(int, uint64_t)> buf;  // device scratch by slot
  std::function<NttTables &(int)> tables;    // twiddle tables by log2 length
  ProofState *st = nullptr;
  fe *ub_scratch = nullptr;                  // kUpdateBetasScratch elements
};

// Where the walk put what a verifier of the opening reads again: per
// sumcheck round its challenge, per iteration its queries (raw draws), the
// update_betas weights, the query count and the new codeword length; the
// final point and evaluation.
struct WalkTrace {
  std::vector<uint64_t> chal, queries, comb, NL;
  std::vector<int> l, kappa;
  uint64_t final_point = 0, final_eval = 0, final_poly = 0;
  uint64_t m_final = 0, L_final = 0;  // final polynomial and codeword lengths
  const fe *last_codeword = nullptr;  // the codeword of the last iteration (device)
  const fe *final_arr = nullptr;      // the final polynomial (device)
};

// The opening loop itself: with dry set only the records are laid out in
// lay, otherwise the kernels are enqueued on R.s.  The generator, the
// running claim K and the flags are R.st's, which the caller initialises.
void batch_open_walk(BatchResources &R, const BatchPlan &P, const fe *const *arrays, const fe *const *betas,
                     const fe *const *codewords, const uint8_t *levels0, uint8_t *tr, Layout &lay, bool dry,
                     WalkTrace *trace = nullptr);

// Enqueues the whole opening on R.s (no host synchronisation): inputs are
// device pointers (arrays / betas / codewords of the merged polynomials,
// the Merkle levels of codeword 0), dtr receives P.transcript_bytes bytes.
// The generator state and the device-side consistency flags end in R.st.
void batch_open_enqueue(BatchResources &R, const BatchPlan &P, const fe *const *arrays, const fe *const *betas,
                        const fe *const *codewords, const uint8_t *levels0, fe K0, const glibc_prng &g0,
                        uint8_t *dtr);

}  // namespace gbz
