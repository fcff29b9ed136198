// Many-proof scheduler: batched proving of independent statements of mixed
// sizes and a serving loop over timed arrivals (gbz_sched.cu).
//
// The reference proves one statement per process (main.cpp); it has no
// batching or serving layer.  Here a proof is a fixed, data-independent
// sequence of launches on device-resident state (gbz_prover.cu), so proofs
// of any shape can run side by side: the scheduler keeps `lanes` slots,
// each a CUDA stream with its own plan (buffers, state, transcript) per
// proof shape, and replays one captured CUDA graph per (slot, shape).
// Proofs in different slots overlap on the device; their results do not
// depend on the mix because nothing is shared between slots.
#pragma once
#include <array>
#include <map>
#include <memory>
#include <vector>

#include "gbz_prover.cuh"

namespace gbz {

struct SchedOpts {
  int lanes = 8;                     // concurrent slots (streams)
  bool group = true;                 // batch: proofs of one shape share every launch (a batched plan)
  int depth = 2;                     // serving: proofs queued per slot before admission waits
  bool graphs = true;                // replay a captured graph per (slot, shape)
  uint64_t reserve = 1ull << 30;     // device bytes left free when a new shape is admitted
};

// Serving: the first kHighSlots slots run at the device's greatest stream
// priority and take proofs of 2^kBigLogn or more first, so that the long
// proofs (the latency tail) are not slowed by the many short ones, which
// fill the SMs they leave idle.  One such slot measured best: two long
// proofs side by side slow each other down.
constexpr int kHighSlots = 1;
constexpr int kBigLogn = 20;
// Batch grouping: the codeword elements one batched plan covers at most.
constexpr int64_t kGroupMaxElems = (int64_t)1 << 23;

struct ProofJob {
  const fe *witness = nullptr;       // host (pinned for overlap) or device, 2^logn elements
  int logn = 0, rate = 0;
  uint32_t seed = 1;
  uint8_t *transcript = nullptr;     // host (pinned for overlap) or device
};

// One (slot, shape) plan with its captured graph.
struct SlotPlan {
  std::unique_ptr<ProofPlan> plan;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t idle = nullptr;        // recorded after the last proof enqueued on this plan
  uint64_t last_use = 0;
  SlotPlan() = default;
  SlotPlan(const SlotPlan &) = delete;
  SlotPlan &operator=(const SlotPlan &) = delete;
  ~SlotPlan();
};

// A slot's plans by (log2 n, rate, proofs per launch).
using PlanKey = std::array<int, 3>;
struct Slot {
  cudaStream_t s = nullptr;
  bool high = false;                 // created with the device's greatest stream priority
  std::map<PlanKey, std::unique_ptr<SlotPlan>> plans;
};

class Scheduler {
 public:
  Scheduler() = default;
  Scheduler(const Scheduler &) = delete;
  Scheduler &operator=(const Scheduler &) = delete;
  ~Scheduler();

  // Proves every job; arrival == nullptr runs them as one batch (longest
  // first, balanced over the slots), else job i is admitted no earlier than
  // arrival[i] seconds after the call starts, to the least-loaded slot with
  // fewer than `depth` proofs in flight.  latency[i] (optional) = completion
  // time - arrival (0 for batches); makespan = completion of the last proof.
  // errors[i] = the device consistency flags of proof i.
  void run(const std::vector<ProofJob> &jobs, const double *arrival, int mem, const SchedOpts &o,
           double *latency, double *makespan, std::vector<uint32_t> &errors);
  // Device bytes currently held by cached plans.
  uint64_t cached_bytes() const;
  void clear();

 private:
  std::vector<Slot> slots_;
  uint64_t tick_ = 0;
  uint32_t *dev_errors_ = nullptr;
  uint64_t dev_errors_cap_ = 0;
  // Pinned staging for transcripts the caller passes in pageable host
  // memory: a copy from the device into pageable memory returns only when
  // the stream has finished all earlier work, which would serialise the
  // slots; such transcripts are copied into this buffer and from it to the
  // caller's buffers once every proof has completed.
  uint8_t *staging_ = nullptr;
  uint64_t staging_cap_ = 0;

  void ensure_slots(int n);
  SlotPlan &plan_for(int slot, int logn, int rate, const SchedOpts &o, int batch = 1);
  bool evict_one_idle(int keep_slot, PlanKey keep_key);
  void enqueue(int slot, SlotPlan &sp, const ProofJob &j, int mem, bool graphs, uint32_t *err_slot);
  // Proofs of one shape as one batched plan (its B = idx.size()): every
  // launch of the proof covers all of them.
  void enqueue_group(int slot, SlotPlan &sp, const std::vector<ProofJob> &jobs, const std::vector<int> &idx, int mem,
                     bool graphs, uint32_t *errors);
};

// Longest-processing-time assignment of jobs with the given costs to
// `lanes` slots; returns the slot of every job (host only).
std::vector<int> lpt_assign(const std::vector<double> &cost, int lanes);
// Relative device cost of one proof of this shape (for the assignment).
double proof_cost(int logn, int rate);

}  // namespace gbz
