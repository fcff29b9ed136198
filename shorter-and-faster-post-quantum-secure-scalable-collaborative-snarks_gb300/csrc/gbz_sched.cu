// Many-proof scheduler (see gbz_sched.cuh): slots of streams with cached
// per-shape plans, graph capture and replay, longest-first batch
// assignment, and a serving loop that admits timed arrivals by slot
// occupancy and free device memory.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstring>
#include <numeric>
#include <thread>

#include "../../include/gbz.h"
#include "gbz_sched.cuh"

namespace gbz {

namespace {

// Captures one proof of the plan's shape on stream s; the graph reads the
// witness from plan->w and the PRNG seed from the plan state.
void capture(SlotPlan &sp, cudaStream_t s) {
  GBZ_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    enqueue_proof(*sp.plan, sp.plan->w, 0, s, false, /*seed_in_state=*/true);
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  GBZ_CUDA(cudaStreamEndCapture(s, &sp.graph));
  GBZ_CUDA(cudaGraphInstantiate(&sp.exec, sp.graph, 0));
}

// Timing events of one run, destroyed on every exit path.
struct RunEvents {
  std::vector<cudaEvent_t> done;
  cudaEvent_t ev0 = nullptr;
  explicit RunEvents(size_t n) : done(n, nullptr) {
    GBZ_CUDA(cudaEventCreate(&ev0));
    for (auto &e : done) GBZ_CUDA(cudaEventCreate(&e));
  }
  ~RunEvents() {
    for (auto e : done)
      if (e) cudaEventDestroy(e);
    if (ev0) cudaEventDestroy(ev0);
  }
};

}  // namespace

SlotPlan::~SlotPlan() {
  if (idle) cudaEventSynchronize(idle);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (idle) cudaEventDestroy(idle);
  plan.reset();
}

double proof_cost(int logn, int rate) {
  // about one millisecond of dependent launches per proof plus a term
  // proportional to the codeword length (2^21 elements per millisecond)
  const double L = std::ldexp(1.0, logn) * rate;
  return 1.0 + L / 2097152.0;
}

std::vector<int> lpt_assign(const std::vector<double> &cost, int lanes) {
  const int n = (int)cost.size();
  lanes = std::max(1, lanes);
  std::vector<int> order(n), slot(n, 0);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(lanes, 0.0);
  for (int i : order) {
    const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    slot[i] = l;
    load[l] += cost[i];
  }
  return slot;
}

Scheduler::~Scheduler() {
  try {
    clear();
  } catch (...) {
  }
}

void Scheduler::clear() {
  for (auto &sl : slots_) {
    if (sl.s) cudaStreamSynchronize(sl.s);
    sl.plans.clear();
    if (sl.s) cudaStreamDestroy(sl.s);
    sl.s = nullptr;
  }
  slots_.clear();
  if (staging_) cudaFreeHost(staging_);
  staging_ = nullptr;
  staging_cap_ = 0;
  if (dev_errors_) cudaFree(dev_errors_);
  dev_errors_ = nullptr;
  dev_errors_cap_ = 0;
}

uint64_t Scheduler::cached_bytes() const {
  uint64_t b = 0;
  for (auto &sl : slots_)
    for (auto &kv : sl.plans) b += plan_bytes(kv.first[0], kv.first[1], kv.first[2]);
  return b;
}

void Scheduler::ensure_slots(int n) {
  int least = 0, greatest = 0;
  GBZ_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  while ((int)slots_.size() < n) {
    Slot s;
    s.high = (int)slots_.size() < kHighSlots;
    GBZ_CUDA(cudaStreamCreateWithPriority(&s.s, cudaStreamNonBlocking, s.high ? greatest : least));
    slots_.push_back(std::move(s));
  }
}

bool Scheduler::evict_one_idle(int keep_slot, PlanKey keep_key) {
  int best_slot = -1;
  PlanKey best_key{};
  uint64_t best_use = ~0ull;
  for (int l = 0; l < (int)slots_.size(); l++)
    for (auto &kv : slots_[l].plans) {
      if (l == keep_slot && kv.first == keep_key) continue;
      if (cudaEventQuery(kv.second->idle) != cudaSuccess) continue;  // still in flight
      if (kv.second->last_use < best_use) {
        best_use = kv.second->last_use;
        best_slot = l;
        best_key = kv.first;
      }
    }
  if (best_slot < 0) return false;
  slots_[best_slot].plans.erase(best_key);
  return true;
}

SlotPlan &Scheduler::plan_for(int slot, int logn, int rate, const SchedOpts &o, int batch) {
  const PlanKey key{logn, rate, batch};
  auto &m = slots_[slot].plans;
  auto it = m.find(key);
  if (it != m.end()) {
    it->second->last_use = ++tick_;
    return *it->second;
  }
  // Admission by free device memory: evict idle cached plans (least
  // recently used first), then wait for busy slots to drain.
  const uint64_t need = plan_bytes(logn, rate, batch) + o.reserve;
  for (;;) {
    size_t fr = 0, tot = 0;
    GBZ_CUDA(cudaMemGetInfo(&fr, &tot));
    if (fr >= need) break;
    if (evict_one_idle(slot, key)) continue;
    bool waited = false;
    for (auto &sl : slots_) {
      const cudaError_t q = cudaStreamQuery(sl.s);
      if (q == cudaErrorNotReady) {
        GBZ_CUDA(cudaStreamSynchronize(sl.s));
        waited = true;
        break;
      }
      if (q != cudaSuccess) GBZ_CUDA(q);
    }
    if (!waited) throw CudaError(cudaErrorMemoryAllocation, "admission: proof shape does not fit in free device memory",
                                 __FILE__, __LINE__);
  }
  std::unique_ptr<SlotPlan> sp(new SlotPlan());
  sp->plan = plan_create(logn, rate, batch);
  GBZ_CUDA(cudaEventCreateWithFlags(&sp->idle, cudaEventDisableTiming));
  sp->last_use = ++tick_;
  SlotPlan &ref = *sp;
  m.emplace(key, std::move(sp));
  return ref;
}

void Scheduler::enqueue(int slot, SlotPlan &sp, const ProofJob &j, int mem, bool graphs, uint32_t *err_slot) {
  ProofPlan &p = *sp.plan;
  const cudaStream_t s = slots_[slot].s;
  p.prof = nullptr;
  const bool host = mem == 0;
  const cudaMemcpyKind in_kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind out_kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (graphs) {
    if (!sp.exec) capture(sp, s);
    GBZ_CUDA(cudaMemcpyAsync(p.w, j.witness, sizeof(fe) * p.n, in_kind, s));
    set_seed_launch(p, j.seed, s);
    GBZ_CUDA(cudaGraphLaunch(sp.exec, s));
  } else {
    const fe *w = j.witness;
    if (host) {
      GBZ_CUDA(cudaMemcpyAsync(p.w, j.witness, sizeof(fe) * p.n, in_kind, s));
      w = p.w;
    }
    enqueue_proof(p, w, j.seed, s, false);
  }
  GBZ_CUDA(cudaMemcpyAsync(j.transcript, p.transcript, p.transcript_bytes, out_kind, s));
  GBZ_CUDA(cudaMemcpyAsync(err_slot, &p.st->error, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  GBZ_CUDA(cudaEventRecord(sp.idle, s));
}

void Scheduler::enqueue_group(int slot, SlotPlan &sp, const std::vector<ProofJob> &jobs, const std::vector<int> &idx,
                              int mem, bool graphs, uint32_t *errors) {
  ProofPlan &p = *sp.plan;
  const cudaStream_t s = slots_[slot].s;
  p.prof = nullptr;
  const bool host = mem == 0;
  const cudaMemcpyKind in_kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind out_kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (graphs && !sp.exec) capture(sp, s);
  std::vector<uint32_t> seeds(idx.size());
  for (size_t b = 0; b < idx.size(); b++) {
    const ProofJob &j = jobs[idx[b]];
    GBZ_CUDA(cudaMemcpyAsync(reinterpret_cast<char *>(p.w) + p.bs_w * b, j.witness, p.bs_w, in_kind, s));
    seeds[b] = j.seed;
  }
  // the seeds every proof's k_init reads, as kernel arguments (a copy from
  // pageable memory may wait for the stream)
  set_seeds_launch(p, seeds.data(), (int)seeds.size(), s);
  if (graphs) {
    GBZ_CUDA(cudaGraphLaunch(sp.exec, s));
  } else {
    enqueue_proof(p, p.w, 0, s, false, /*seed_in_state=*/true);
  }
  for (size_t b = 0; b < idx.size(); b++) {
    const ProofJob &j = jobs[idx[b]];
    GBZ_CUDA(cudaMemcpyAsync(j.transcript, p.transcript + p.transcript_bytes * b, p.transcript_bytes, out_kind, s));
    GBZ_CUDA(cudaMemcpyAsync(errors + idx[b], &p.st[b].error, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
  GBZ_CUDA(cudaEventRecord(sp.idle, s));
}

void Scheduler::run(const std::vector<ProofJob> &jobs_in, const double *arrival, int mem, const SchedOpts &o,
                    double *latency, double *makespan, std::vector<uint32_t> &errors) {
  const int nj = (int)jobs_in.size();
  errors.assign(nj, 0);
  if (makespan) *makespan = 0;
  if (!nj) return;
  // transcripts in pageable host memory go through the pinned staging buffer
  std::vector<ProofJob> jobs = jobs_in;
  std::vector<uint64_t> staged(nj, ~0ull);
  if (mem == 0) {
    uint64_t need = 0;
    for (int i = 0; i < nj; i++) {
      cudaPointerAttributes a{};
      const cudaError_t e = cudaPointerGetAttributes(&a, jobs[i].transcript);
      if (e != cudaSuccess) (void)cudaGetLastError();
      if (e != cudaSuccess || a.type == cudaMemoryTypeUnregistered) {
        staged[i] = need;
        need += (gbz_prove_transcript_bytes(jobs[i].logn, jobs[i].rate) + 255) & ~255ull;
      }
    }
    if (need > staging_cap_) {
      if (staging_) GBZ_CUDA(cudaFreeHost(staging_));
      staging_ = nullptr;
      staging_cap_ = 0;
      GBZ_CUDA(cudaHostAlloc((void **)&staging_, need, cudaHostAllocDefault));
      staging_cap_ = need;
    }
    for (int i = 0; i < nj; i++)
      if (staged[i] != ~0ull) jobs[i].transcript = staging_ + staged[i];
  }
  const int lanes = std::max(1, o.lanes);
  const int depth = std::max(1, o.depth);
  ensure_slots(lanes);
  if (dev_errors_cap_ < (uint64_t)nj) {
    if (dev_errors_) GBZ_CUDA(cudaFree(dev_errors_));
    dev_errors_ = nullptr;
    dev_errors_cap_ = 0;
    GBZ_CUDA(cudaMalloc(&dev_errors_, sizeof(uint32_t) * nj));
    dev_errors_cap_ = nj;
  }
  for (int l = 0; l < lanes; l++) GBZ_CUDA(cudaStreamSynchronize(slots_[l].s));

  RunEvents ev(nj);
  auto drain = [&]() {
    for (int l = 0; l < lanes; l++) cudaStreamSynchronize(slots_[l].s);
  };
  try {
    if (!arrival && o.group) {
      // Batch, grouped: the proofs of each shape are one batched plan (every
      // launch covers all of them), the groups longest first over the
      // slots; plans and graphs prepared before the clock starts.
      std::map<std::pair<int, int>, std::vector<int>> groups;
      for (int i = 0; i < nj; i++) groups[{jobs[i].logn, jobs[i].rate}].push_back(i);
      // a group costing more than an even share of the whole batch is cut
      // into that many equal sub-batches, so that one shape's chain does not
      // set the makespan while other slots idle
      double total = 0;
      for (auto &kv : groups) total += proof_cost(kv.first.first, kv.first.second) * (double)kv.second.size();
      const double share = total / lanes;
      std::vector<std::vector<int>> units;
      std::vector<double> cost;
      for (auto &kv : groups) {
        const double c1 = proof_cost(kv.first.first, kv.first.second);
        const int cnt = (int)kv.second.size();
        // and a batched plan holds at most kGroupMaxElems codeword elements:
        // a proof that long fills the device by itself, so batching it
        // saves no launches and only makes every witness upload of the
        // sub-batch wait ahead of its first kernel
        const int64_t L = ((int64_t)1 << kv.first.first) * kv.first.second;
        const int cap = (int)std::max<int64_t>(1, std::min<int64_t>(cnt, kGroupMaxElems / L));
        const int parts = std::max({1, (cnt + cap - 1) / cap, std::min(cnt, (int)std::ceil(c1 * cnt / share))});
        for (int k = 0; k < parts; k++) {
          const int a = (int)((int64_t)cnt * k / parts), b = (int)((int64_t)cnt * (k + 1) / parts);
          units.emplace_back(kv.second.begin() + a, kv.second.begin() + b);
          cost.push_back(c1 * (double)(b - a));
        }
      }
      const std::vector<int> asg = lpt_assign(cost, lanes);
      std::vector<int> order(units.size());
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
      std::vector<std::vector<int>> per(lanes);
      for (int u : order) per[asg[u]].push_back(u);
      for (int l = 0; l < lanes; l++)
        for (int u : per[l]) {
          const ProofJob &j0 = jobs[units[u][0]];
          SlotPlan &sp = plan_for(l, j0.logn, j0.rate, o, (int)units[u].size());
          if (o.graphs && !sp.exec) capture(sp, slots_[l].s);
        }
      GBZ_CUDA(cudaEventRecord(ev.ev0, slots_[0].s));
      for (int l = 1; l < lanes; l++) GBZ_CUDA(cudaStreamWaitEvent(slots_[l].s, ev.ev0, 0));
      size_t longest = 0;
      for (auto &v : per) longest = std::max(longest, v.size());
      for (size_t k = 0; k < longest; k++)
        for (int l = 0; l < lanes; l++) {
          if (k >= per[l].size()) continue;
          const std::vector<int> &idx = units[per[l][k]];
          const ProofJob &j0 = jobs[idx[0]];
          SlotPlan &sp = plan_for(l, j0.logn, j0.rate, o, (int)idx.size());
          enqueue_group(l, sp, jobs, idx, mem, o.graphs, dev_errors_);
          for (int i : idx) GBZ_CUDA(cudaEventRecord(ev.done[i], slots_[l].s));
        }
    } else if (!arrival) {
      // Batch: longest first over the slots, plans and graphs prepared
      // before the clock starts, then enqueued round-robin over the slots.
      std::vector<double> cost(nj);
      for (int i = 0; i < nj; i++) cost[i] = proof_cost(jobs[i].logn, jobs[i].rate);
      const std::vector<int> asg = lpt_assign(cost, lanes);
      std::vector<int> order(nj);
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
      std::vector<std::vector<int>> per(lanes);
      for (int i : order) per[asg[i]].push_back(i);
      for (int l = 0; l < lanes; l++)
        for (int i : per[l]) {
          SlotPlan &sp = plan_for(l, jobs[i].logn, jobs[i].rate, o);
          if (o.graphs && !sp.exec) capture(sp, slots_[l].s);
        }
      GBZ_CUDA(cudaEventRecord(ev.ev0, slots_[0].s));
      for (int l = 1; l < lanes; l++) GBZ_CUDA(cudaStreamWaitEvent(slots_[l].s, ev.ev0, 0));
      size_t longest = 0;
      for (auto &v : per) longest = std::max(longest, v.size());
      for (size_t k = 0; k < longest; k++)
        for (int l = 0; l < lanes; l++) {
          if (k >= per[l].size()) continue;
          const int i = per[l][k];
          SlotPlan &sp = plan_for(l, jobs[i].logn, jobs[i].rate, o);
          enqueue(l, sp, jobs[i], mem, o.graphs, dev_errors_ + i);
          GBZ_CUDA(cudaEventRecord(ev.done[i], slots_[l].s));
        }
    } else {
      // Serving: job i is admitted at its arrival time to the least-loaded
      // slot with fewer than `depth` proofs in flight.
      std::vector<int> order(nj);
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return arrival[a] < arrival[b]; });
      std::vector<std::vector<int>> inflight(lanes);
      using clock = std::chrono::steady_clock;
      GBZ_CUDA(cudaEventRecord(ev.ev0, slots_[0].s));
      for (int l = 1; l < lanes; l++) GBZ_CUDA(cudaStreamWaitEvent(slots_[l].s, ev.ev0, 0));
      const auto t0 = clock::now();
      for (int i : order) {
        const auto target = t0 + std::chrono::duration_cast<clock::duration>(std::chrono::duration<double>(arrival[i]));
        if (clock::now() < target) std::this_thread::sleep_until(target);
        // least-loaded slot with room, among the slots of the job's
        // priority class first (long proofs: high-priority slots)
        const bool big = jobs[i].logn >= kBigLogn && lanes > kHighSlots;
        int best = -1;
        for (;;) {
          for (int l = 0; l < lanes; l++) {
            auto &q = inflight[l];
            q.erase(std::remove_if(q.begin(), q.end(),
                                   [&](int k) { return cudaEventQuery(ev.done[k]) == cudaSuccess; }),
                    q.end());
          }
          for (int pass = 0; pass < 2 && best < 0; pass++) {
            size_t best_n = ~(size_t)0;
            double best_cost = 0;
            for (int l = 0; l < lanes; l++) {
              if (pass == 0 && lanes > kHighSlots && slots_[l].high != big) continue;
              const auto &q = inflight[l];
              if (q.size() >= (size_t)depth) continue;
              double c = 0;
              for (int k : q) c += proof_cost(jobs[k].logn, jobs[k].rate);
              if (q.size() < best_n || (q.size() == best_n && c < best_cost)) {
                best = l;
                best_n = q.size();
                best_cost = c;
              }
            }
          }
          if (best >= 0) break;
          std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
        SlotPlan &sp = plan_for(best, jobs[i].logn, jobs[i].rate, o);
        enqueue(best, sp, jobs[i], mem, o.graphs, dev_errors_ + i);
        GBZ_CUDA(cudaEventRecord(ev.done[i], slots_[best].s));
        inflight[best].push_back(i);
      }
    }
    for (int l = 0; l < lanes; l++) GBZ_CUDA(cudaStreamSynchronize(slots_[l].s));
  } catch (...) {
    drain();
    throw;
  }
  double last = 0;
  for (int i = 0; i < nj; i++) {
    float ms = 0;
    GBZ_CUDA(cudaEventElapsedTime(&ms, ev.ev0, ev.done[i]));
    const double t = ms * 1e-3;
    last = std::max(last, t);
    if (latency) latency[i] = t - (arrival ? arrival[i] : 0.0);
  }
  if (makespan) *makespan = last;
  GBZ_CUDA(cudaMemcpy(errors.data(), dev_errors_, sizeof(uint32_t) * nj, cudaMemcpyDeviceToHost));
  for (int i = 0; i < nj; i++)
    if (staged[i] != ~0ull)
      std::memcpy(jobs_in[i].transcript, staging_ + staged[i], gbz_prove_transcript_bytes(jobs[i].logn, jobs[i].rate));
}

}  // namespace gbz
