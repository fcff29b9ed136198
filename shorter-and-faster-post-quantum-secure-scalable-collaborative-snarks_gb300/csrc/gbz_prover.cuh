// Plan and enqueue interface of the single-party prover (gbz_prover.cu).
#pragma once
#include <map>
#include <memory>
#include <vector>

#include "gbz_internal.cuh"

namespace gbz {

// Transcript layout: record offsets are fixed by (logn, rate), so they are
// computed once; the constant record headers are written at plan creation
// and the kernels fill in the payloads.
struct Layout {
  struct Header {
    uint64_t off;
    uint32_t tag, count;
  };
  uint64_t len = 0;
  bool record_headers = false;
  std::vector<Header> headers;
  // Appends a record of `count` units of `unit` bytes; returns the payload offset.
  uint64_t rec(uint32_t tag, uint32_t count, uint32_t unit);
};

// Optional per-category CUDA-event timing of the kernels of a proof, on the
// stream the kernels are launched on.
enum ProfCat { PC_NTT = 0, PC_MERKLE, PC_SUMCHECK, PC_BETA, PC_UPDATE_BETAS, PC_QUERY, PC_PROTOCOL, PC_COUNT };
struct Profiler {
  bool enabled = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[PC_COUNT];
  size_t used[PC_COUNT] = {0};
  int open_cat = -1;
  void begin(int cat, cudaStream_t s);
  void end(cudaStream_t s);
  void reset() { for (int c = 0; c < PC_COUNT; c++) used[c] = 0; }
  // Total milliseconds per category since reset (synchronises on the events).
  void read(double ms[PC_COUNT], int counts[PC_COUNT]);
  ~Profiler();
};

// A proof captured as a CUDA graph for one witness address; the PRNG seed
// is a parameter of the captured k_init node, updated before each launch.
struct ProofGraph {
  const fe *w = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t init_node = nullptr;
  cudaKernelNodeParams init_params{};
  uint64_t last_use = 0;
};

// Device buffers and tables for proofs of one shape (n = 2^logn, rate).
// A plan for a batch holds B proofs of the shape: every buffer below is B
// copies back to back (bs_* their byte strides, the states B consecutive
// ProofStates, the transcripts B copies of transcript_bytes), and every
// launch of the proof covers the whole batch.
struct ProofPlan {
  int logn = 0, rate = 0;
  uint64_t n = 0, L = 0;
  int B = 1;
  uint64_t bs_w = 0, bs_cw0 = 0, bs_cw1 = 0, bs_tmp = 0, bs_tmp2 = 0, bs_v = 0, bs_arr = 0, bs_beta = 0,
           bs_part = 0, bs_ub = 0;
  fe *w = nullptr;                // witness staging (host-input proofs)
  fe *cw[2] = {nullptr, nullptr}; // codeword ping-pong (L, L/2)
  fe *tmp = nullptr;              // NTT intermediate of the commits (L)
  fe *tmp2 = nullptr;             // NTT intermediate of the sparse beta updates (L/2)
  // The opening runs as three chains joined by events: folds and beta
  // updates on the caller's stream, commits (NTT + Merkle) on s2, queries
  // (replies, answers, paths, the running claim K) on s3.  Each waits only
  // for the data it reads; the WHIR randomness is drawn up front on s3.
  cudaStream_t s2 = nullptr, s3 = nullptr;
  static constexpr int kMaxIter = kMaxWhirIter;
  cudaEvent_t ev_in = nullptr, ev_init = nullptr, ev_sched = nullptr, ev_fold[kMaxIter] = {}, ev_commit[kMaxIter + 1] = {},
              ev_query[kMaxIter] = {}, ev_root_tail = nullptr;
  fe *va[2] = {nullptr, nullptr}; // folded first vector ping-pong (n/2 each)
  fe *arr = nullptr;              // the folded polynomials arr_1, arr_2, ... back to back (read by the commits)
  fe *vb[2] = {nullptr, nullptr}; // folded second vector ping-pong
  fe *beta = nullptr;             // eq table (n)
  fe *partial = nullptr;          // per-CTA round-message partials
  fe *partial2 = nullptr;         // the second round's, when two rounds share a pass
  fe *ub_scratch = nullptr;       // update_betas power tables
  ProofState *st = nullptr;
  uint8_t *transcript = nullptr;
  uint64_t transcript_bytes = 0;
  uint8_t *open_transcript = nullptr;  // an opening alone (gbz_whir_open): its own records and headers
  uint64_t open_transcript_bytes = 0;
  Layout layout;
  int launches = 0;               // kernel launches per proof (counted by the dry run)
  int cat_launches[PC_COUNT] = {0};
  Profiler *prof = nullptr;
  std::map<int, NttTables> ntt;
  std::vector<void *> allocs;
  std::vector<ProofGraph> graphs;  // a few witness addresses, least recently used dropped
  uint64_t graph_tick = 0;

  ProofPlan() = default;
  ProofPlan(const ProofPlan &) = delete;
  ProofPlan &operator=(const ProofPlan &) = delete;
  ~ProofPlan();
  void *dalloc(uint64_t bytes);
  NttTables &tables(int lg);
};

// Protocol kernels shared by the prover and the batch opening
// (gbz_prover.cu): a WHIR sumcheck round from the reduction partials, the
// authentication paths of the queries in a tree of `leaves` leaf hashes,
// and the final round (its point drawn from the generator, or read from
// `point` when the randomness was drawn up front).
__global__ void k_whir_round(const fe *partial, int blocks, ProofState *st, int i, uint8_t *tr,
                             uint64_t off_poly, uint64_t off_chal);
__global__ void k_whir_paths(const uint8_t *tree, uint64_t leaves, int l, uint8_t *tr, uint64_t off_q,
                             uint64_t off_path);
// The same nodes without the tree (inner nodes hash their left child
// twice, so every node is a chain of compressions from one leaf): the root
// of the tree over a codeword, the paths of l queries into it, and the
// root and paths of a tree whose leaf hashes are all zero.
__global__ void k_merkle_root(const fe *cw, int depth, uint8_t *tr, uint64_t off);
// cws, trs: per-proof strides of a batch (grid.y = proof), 0 for one proof.
__global__ void k_whir_paths_chain(const fe *cw, uint64_t leaves, int l, uint8_t *tr, uint64_t off_q,
                                   uint64_t off_path, uint64_t cws, uint64_t trs);
__global__ void k_zero_tree_root(int depth, uint8_t *tr, uint64_t off);
__global__ void k_zero_tree_paths(int depth, int l, uint8_t *tr, uint64_t off_path);
__global__ void k_final(ProofState *st, const fe *arr, const fe *b, int m, uint8_t *tr, uint64_t off_poly,
                        uint64_t off_point, uint64_t off_eval, int check_K, const fe *point);

// An opening alone (Whir_Open, Whir.cpp:388-467): the caller's codeword of
// the polynomial (device, rate * n entries), the claim's point (device, logn
// entries) and value K, and the glibc generator state the draws start from.
struct OpenOnly {
  const fe *codeword = nullptr;
  const fe *point = nullptr;
  fe K;
  glibc_prng prng;
};

std::unique_ptr<ProofPlan> plan_create(int logn, int rate, int batch = 1);
// Allocates the plan's buffer for openings alone, with its record headers
// (once; the proof's layout and launch counts are left as they are).
void plan_prepare_open(ProofPlan &p);
// Enqueues one proof on stream s (dry: only computes the layout).  With
// seed_in_state the PRNG seed is read from the plan's state (written by
// set_seed_launch), so that the enqueued work can be captured once as a CUDA
// graph and replayed for any seed.
// With `open`, only the opening of (witness, open->codeword) at the given
// claim is enqueued: the commitment root of the codeword, then the WHIR
// records (no evaluation point, claim or sumcheck records).
void enqueue_proof(ProofPlan &p, const fe *witness, uint32_t prng_seed, cudaStream_t s, bool dry,
                   bool seed_in_state = false, const OpenOnly *open = nullptr);
void set_seed_launch(ProofPlan &p, uint32_t seed, cudaStream_t s);
// The seeds of the first count proofs of a batched plan (passed by value).
void set_seeds_launch(ProofPlan &p, const uint32_t *seeds, int count, cudaStream_t s);
// Enqueues one proof of the witness at w by replaying a captured graph
// (captured on first use of this address; s must be a capturable stream).
void launch_proof_graph(ProofPlan &p, const fe *w, uint32_t prng_seed, cudaStream_t s);
// Device bytes a plan of this shape allocates (an upper bound).
uint64_t plan_bytes(int logn, int rate, int batch = 1);
// Reads the device-side consistency flags (synchronises s).
uint32_t plan_error_flags(ProofPlan &p, cudaStream_t s);
int whir_query_count(int rate);
// Whether update_betas over nb entries with l queries of a length-N codeword
// runs as a sparse transform (else as direct geometric sums).
bool update_betas_by_transform(int l, uint64_t nb, uint64_t N);

}  // namespace gbz
