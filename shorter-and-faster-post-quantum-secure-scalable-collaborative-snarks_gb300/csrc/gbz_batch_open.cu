// Whir_Batch_Open (Whir.cpp:706-898) on one device.
//
// The largest polynomial is opened by WHIR iterations of folding factor
// kappa (log2 kappa sumcheck rounds, re-encoding at twice the rate, Merkle
// commitment, queries of the previous codeword, update_betas); whenever it
// has been folded to the size of the next polynomials they are merged into
// it: aggregate_arrays (Whir.cpp:670-704) with challenges drawn from the
// reference's generator, and aggregate_commitments (Whir.cpp:547-606),
// whose new tree is built over zero leaves as in the reference.  The
// schedule depends on the sizes alone, so the host lays out the transcript
// and enqueues every step up front; all randomness and running claims live
// in device memory (ProofState), as in the single-polynomial prover.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gbz_batch_open.cuh"
#include "gbz_prover.cuh"
#include "gbz_whir_aggr.cuh"

namespace gbz {

namespace {

__device__ __forceinline__ fe pow_tab(const fe *lo, const fe *hi, uint64_t e) {
  return fmul(lo[e & 4095u], hi[e >> 12]);
}

__global__ void bo_init_kernel(ProofState *st, glibc_prng g, fe K0) {
  if (threadIdx.x) return;
  st->prng = g;
  st->K = K0;
  st->fs = fe_zero();
  st->y = fe_zero();
  st->error = 0;
}

struct BoQueryArgs {
  ProofState *st;
  const fe *cw;       // the codeword the queries open
  uint64_t L, qmod;   // its length; queries are rand() % qmod
  int logk, l;
  uint8_t *tr;
  uint64_t off_q, off_rep, off_ans, off_comb, off_K;
  const fe *inv_lo, *inv_hi;  // omega_L^{-e}
  const fe *new_lo, *new_hi;  // omega_NL^{e}
  fe len_inv;                 // kappa^{-1}
};

// whir_query (Whir.cpp:251-314) for folding factor kappa = 2^logk <= 16,
// the rescaling of the queries to the new codeword (:371-372, factor
// kappa NL / L = 2) and update_betas' weights c_i = r^(i+1) with
// K += sum_i c_i y_i (:325-342, :383-384).  Thread i handles query i.
__global__ void __launch_bounds__(kMaxQueries) bo_query_kernel(BoQueryArgs a) {
  __shared__ int32_t q[kMaxQueries];
  __shared__ fe rb_s;
  __shared__ fe red[kMaxQueries / 32];
  __shared__ glibc_prng g;
  ProofState *st = a.st;
  if (threadIdx.x == 0) {
    g = st->prng;
    for (int i = 0; i < a.l; i++) q[i] = prng_next(g) % (int32_t)a.qmod;
    rb_s = prng_field(g);  // update_betas' F::_random(), drawn after the queries
    st->prng = g;
  }
  __syncthreads();
  const int i = threadIdx.x;
  fe contrib = fe_zero();
  if (i < a.l) {
    const uint64_t qi = (uint64_t)(uint32_t)q[i];
    reinterpret_cast<int32_t *>(a.tr + a.off_q)[i] = q[i];
    const int k = 1 << a.logk;
    const uint64_t stride = a.L / (uint64_t)k;
    fe part[1 << kMaxWhirLogK];
    for (int j = 0; j < k; j++) {
      part[j] = a.cw[qi + (uint64_t)j * stride];
      put_fe(a.tr, a.off_rep + 16 * ((uint64_t)k * i + j), part[j]);
    }
    // get_RS_multifold_segment_tensor (coPCS_utils.cpp:333-383): level t
    // pairs (j, j + k / 2^(t+1)) with omega_L^{-2^t (qi + j L / k)}.
    int half = k / 2;
    for (int t = 0; t < a.logk; t++) {
      const fe r = st->rw[t], omr = fsub(fe_one(), r);
      for (int j = 0; j < half; j++) {
        const uint64_t e = ((qi + (uint64_t)j * stride) << t) & (a.L - 1);
        const fe w = pow_tab(a.inv_lo, a.inv_hi, e);
        const fe s = fadd(part[j], part[j + half]), d = fsub(part[j], part[j + half]);
        part[j] = fadd(fmul(omr, s), fmul(r, fmul(w, d)));
      }
      half >>= 1;
    }
    const fe y = fmul(a.len_inv, part[0]);
    put_fe(a.tr, a.off_ans + 16 * i, y);
    const uint32_t scaled = 2u * (uint32_t)qi;
    st->q[i] = (int32_t)scaled;
    st->omega_q[i] = pow_tab(a.new_lo, a.new_hi, scaled);
    const fe c = fpow(rb_s, (uint64_t)i + 1);
    st->comb[i] = c;
    put_fe(a.tr, a.off_comb + 16 * i, c);
    contrib = fmul(c, y);
  }
  for (int dd = 16; dd > 0; dd >>= 1) {
    fe t;
    t.re = __shfl_down_sync(0xffffffffu, contrib.re, dd);
    t.im = __shfl_down_sync(0xffffffffu, contrib.im, dd);
    contrib = fadd(contrib, t);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = contrib;
  __syncthreads();
  if (threadIdx.x == 0) {
    fe K = st->K;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) K = fadd(K, red[w]);
    st->K = K;
    put_fe(a.tr, a.off_K, K);
  }
}

// The aggregation challenges (Whir.cpp:809-814): g draws for ch1, g for
// ch2, then ch1[0] = ch2[0] = 1.  coef = (ch1, ch2).
__global__ void bo_aggr_draw_kernel(ProofState *st, int g, fe *coef, uint8_t *tr, uint64_t off) {
  __shared__ glibc_prng gs;
  if (threadIdx.x) return;
  gs = st->prng;
  for (int i = 0; i < 2 * g; i++) {
    fe c = prng_field(gs);
    if (i == 0 || i == g) c = fe_one();
    coef[i] = c;
    put_fe(tr, off + 16 * (uint64_t)i, c);
  }
  st->prng = gs;
}

// aggregate_arrays' claim (Whir.cpp:695-702) with r1 = ch2, r2 = ch1:
// K = sum_{i,j} ch2[i] ch1[j] <A_i, B_j>.
__global__ void bo_aggr_k_kernel(ProofState *st, const fe *evals, const fe *coef, int g, uint8_t *tr,
                                 uint64_t off) {
  if (threadIdx.x) return;
  fe K = fe_zero();
  for (int i = 0; i < g; i++)
    for (int j = 0; j < g; j++) K = fadd(K, fmul(fmul(coef[g + i], coef[j]), evals[i * g + j]));
  st->K = K;
  put_fe(tr, off, K);
}

// The openings aggregate_commitments draws (Whir.cpp:574-576).
__global__ void bo_aggr_queries_kernel(ProofState *st, int la, int32_t qmod, uint8_t *tr, uint64_t off) {
  __shared__ glibc_prng gs;
  if (threadIdx.x) return;
  gs = st->prng;
  int32_t *q = reinterpret_cast<int32_t *>(tr + off);
  for (int i = 0; i < la; i++) q[i] = prng_next(gs) % qmod;
  st->prng = gs;
}

int ilog2i(uint64_t x) { return ilog2(x); }

}  // namespace

BatchPlan batch_plan(int k, const uint64_t *sizes, int rate, int whir_k, uint64_t zero_leaves0) {
  BatchPlan P;
  if (k < 1 || k > kMaxVecs) throw ArgError("batch open: 1..64 polynomials");
  if (!sizes) throw ArgError("null pointer: sizes");
  if (!(whir_k == 2 || whir_k == 4 || whir_k == 8 || whir_k == 16))
    throw ArgError("batch open: whir_k must be 2, 4, 8 or 16");
  if (rate < 2 || !is_pow2((uint64_t)rate) || rate > 64) throw ArgError("batch open: rate must be a power of two in [2, 64]");
  for (int i = 0; i < k; i++) {
    if (!is_pow2(sizes[i])) throw ArgError("batch open: sizes must be powers of two");
    if (i && sizes[i] > sizes[i - 1]) throw ArgError("batch open: sizes must not increase");
  }
  if (sizes[0] < 2 * (uint64_t)whir_k) throw ArgError("batch open: the largest polynomial needs 2 whir_k entries");
  if (ilog2(sizes[0] * (uint64_t)rate) > kMaxNttLogN) throw ArgError("batch open: codeword longer than 2^26");
  P.k = k;
  P.rate = rate;
  P.whir_k = whir_k;
  P.sizes.assign(sizes, sizes + k);
  // kappa schedule (Whir.cpp:731-752)
  {
    uint64_t size = sizes[0];
    int si = 1;
    for (;;) {
      if (P.kappa.size() >= 64) throw ArgError("batch open: schedule too long");
      if (si >= k || size / whir_k > sizes[si]) {
        P.kappa.push_back(whir_k);
        P.aggr.push_back(0);
        size /= whir_k;
      } else {
        const uint64_t kap = size / sizes[si], s = sizes[si];
        while (si < k && sizes[si] == s) si++;
        P.kappa.push_back((int)kap);
        P.aggr.push_back(1);
        size /= kap;
      }
      if (size <= (uint64_t)whir_k) break;
    }
  }
  // the loop of Whir.cpp:761-833 on sizes only
  uint64_t m = sizes[0], L = m * (uint64_t)rate, leaves = L / 4;
  if (zero_leaves0) {
    if (!is_pow2(zero_leaves0) || zero_leaves0 > leaves) throw ArgError("batch open: bad zero tree size");
    leaves = zero_leaves0;
    P.zero_tree0 = true;
  }
  int cur = rate, iter = 0, next = 1, wk = whir_k;
  uint64_t bytes = 8 + 8 * (uint64_t)P.kappa.size();
  P.cw_len.assign(k, 0);
  P.cw_len[0] = L;
  for (;;) {
    if (iter >= (int)P.kappa.size() || P.steps.size() >= 64) throw ArgError("batch open: schedule overrun");
    BatchStep e;
    wk = P.kappa[iter];
    const bool ag = P.aggr[iter] != 0;
    e.m = m;
    e.L = L;
    e.rate = cur;
    if (!ag || wk != 1) {
      const int kap = wk, logk = ilog2i((uint64_t)kap);
      if (kap < 2 || m < (uint64_t)kap || kap > (1 << kMaxWhirLogK)) throw ArgError("batch open: bad folding factor");
      const uint64_t qmod = kap > 4 ? L / kap : L / 4;
      if (qmod > leaves) throw ArgError("batch open: the reference would open a leaf beyond its tree");
      e.iterate = true;
      e.kappa = kap;
      e.l = whir_query_count(cur);
      e.depth = ilog2(leaves);
      const uint64_t nm = m / kap, NL = 2 * (uint64_t)cur * nm;
      if (NL < 8 || e.l > kMaxQueries || e.l < 1) throw ArgError("batch open: codeword too short");
      bytes += (uint64_t)logk * (8 + 48 + 8 + 16) + (8 + 32) + (8 + 4ull * e.l) + (8 + 16ull * kap * e.l) +
               (8 + 16ull * e.l) + (8 + 32ull * e.l * e.depth) + (8 + 16ull * e.l) + (8 + 16);
      m = nm;
      L = NL;
      leaves = L / 4;
      cur *= 2;
    }
    iter++;
    if (ag) {
      int g = 1;
      while (next + g - 1 < k && sizes[next + g - 1] == m) g++;
      e.aggregate = true;
      e.group = g;
      e.first = next;
      for (int i = 0; i < g - 1; i++) P.cw_len[next + i] = L;
      next += g - 1;
      if (iter + 1 >= (int)P.kappa.size())
        throw ArgError("batch open: the reference reads its schedule past the end for these sizes");
      uint64_t wk2 = (uint64_t)P.kappa[iter + 1];
      if (next < k && m / wk2 <= sizes[next]) wk2 = m / sizes[next];
      if (wk2 < 1 || L % wk2 || leaves != L / 4) throw ArgError("batch open: unsupported aggregation shape");
      e.la = whir_query_count((int)(L / m));
      e.depth_a = ilog2(leaves);
      if (e.la > kMaxQueries || e.la < 1) throw ArgError("batch open: too many queries");
      leaves = L / wk2;
      wk = (int)wk2;
      bytes += (8 + 32ull * g) + (8 + 16) + (8 + 4ull * e.la) + (8 + 32ull * e.la * e.depth_a) + (8 + 32);
    }
    e.leaves_after = leaves;
    P.steps.push_back(e);
    if (m <= (uint64_t)wk) break;
  }
  if (m > (uint64_t)kFinalMax) throw ArgError("batch open: final polynomial too long");
  P.m_final = m;
  bytes += (8 + 16 * m) + (8 + 16ull * ilog2(m)) + (8 + 16);
  P.transcript_bytes = bytes;
  return P;
}

// Walks the opening once: with dry set it only lays out the records
// (lay.headers), otherwise it enqueues the kernels that fill them.
void batch_open_walk(BatchResources &R, const BatchPlan &P, const fe *const *arrays, const fe *const *betas,
                     const fe *const *codewords, const uint8_t *levels0, uint8_t *tr, Layout &lay, bool dry,
                     WalkTrace *trace) {
  cudaStream_t s = R.s;
  ProofState *st = R.st;
  const uint64_t n0 = P.sizes[0], L0 = n0 * (uint64_t)P.rate;
  fe *A[2] = {nullptr, nullptr}, *B[2] = {nullptr, nullptr}, *C[2] = {nullptr, nullptr};
  fe *tmp = nullptr, *tmp2 = nullptr, *partial = nullptr, *coef = nullptr, *evals = nullptr, *mdp = nullptr;
  if (!dry) {
    A[0] = (fe *)R.buf(300, 16 * n0);
    A[1] = (fe *)R.buf(301, 16 * std::max<uint64_t>(n0 / 2, 1));
    B[0] = (fe *)R.buf(302, 16 * n0);
    B[1] = (fe *)R.buf(303, 16 * std::max<uint64_t>(n0 / 2, 1));
    C[0] = (fe *)R.buf(304, 16 * L0);
    C[1] = (fe *)R.buf(305, 16 * L0);
    tmp = (fe *)R.buf(308, 16 * L0);
    tmp2 = (fe *)R.buf(309, 16 * std::max<uint64_t>(L0 / 2, 1));
    partial = (fe *)R.buf(310, 16 * 3 * (uint64_t)sc_blocks(n0 / 2));
    coef = (fe *)R.buf(311, 16 * 2 * kMaxVecs);
    evals = (fe *)R.buf(312, 16 * kMaxVecs * kMaxVecs);
    mdp = (fe *)R.buf(313, 16 * multidot_scratch(n0));
    GBZ_CUDA(cudaMemcpyAsync(A[0], arrays[0], 16 * n0, cudaMemcpyDeviceToDevice, s));
    GBZ_CUDA(cudaMemcpyAsync(B[0], betas[0], 16 * n0, cudaMemcpyDeviceToDevice, s));
  }
  // schedule record
  {
    const uint64_t off = lay.rec(T_SCHEDULE, (uint32_t)(2 * P.kappa.size()), 4);
    if (!dry) {
      std::vector<uint32_t> sch;
      for (size_t i = 0; i < P.kappa.size(); i++) {
        sch.push_back((uint32_t)P.kappa[i]);
        sch.push_back((uint32_t)P.aggr[i]);
      }
      GBZ_CUDA(cudaMemcpyAsync(tr + off, sch.data(), 4 * sch.size(), cudaMemcpyHostToDevice, s));
    }
  }
  int ai = 0;                 // arr / b live in A[ai] / B[ai]
  const fe *cw = codewords[0];
  // The tree the next queries open: the caller's levels (first polynomial),
  // a commitment over the current codeword (its nodes are computed as
  // compression chains from the codeword, never stored), or the tree over
  // zero leaves that aggregate_commitments builds.
  enum { TREE_LEVELS, TREE_CODEWORD, TREE_ZERO } tree_kind = P.zero_tree0 ? TREE_ZERO : TREE_LEVELS;
  const uint8_t *tree = levels0;
  int ci = -1;                // which working buffer holds cw (-1: the caller's)
  // open_tree_blake for l queries into the current tree of lv leaves
  auto launch_paths = [&](int kind, const uint8_t *levels, const fe *codeword, uint64_t lv, int l, int depth,
                          uint64_t off_path, uint64_t off_q) {
    const uint64_t hashes = (uint64_t)l * depth;
    if (!hashes) return;
    if (depth != ilog2(lv)) throw ArgError("batch open: path length does not match the tree");
    const unsigned blocks = (unsigned)((hashes + 127) / 128);
    if (kind == TREE_LEVELS) k_whir_paths<<<blocks, 128, 0, s>>>(levels, lv, l, tr, off_q, off_path);
    else if (kind == TREE_CODEWORD) k_whir_paths_chain<<<blocks, 128, 0, s>>>(codeword, lv, l, tr, off_q, off_path, 0, 0);
    else k_zero_tree_paths<<<(unsigned)((depth + 31) / 32), 32, 0, s>>>(depth, l, tr, off_path);
    GBZ_CUDA(cudaGetLastError());
  };
  uint64_t m = n0, L = L0, leaves = P.zero_tree0 && !P.steps.empty() ? (1ull << P.steps[0].depth) : L0 / 4;
  int cur = P.rate;
  for (const BatchStep &e : P.steps) {
    if (e.iterate) {
      const int logk = ilog2((uint64_t)e.kappa);
      // whir_sumcheck (Whir.cpp:233-249): log2 kappa rounds, fold i fused with message i+1
      for (int i = 0; i < logk; i++) {
        const uint64_t op = lay.rec(T_WHIR_POLY, 3, 16), oc = lay.rec(T_WHIR_CHALLENGE, 1, 16);
        if (trace) trace->chal.push_back(oc);
        const int blocks = sc_blocks(i == 0 ? m / 2 : std::max<uint64_t>(m / 4, 1));
        if (!dry) {
          if (i == 0)
            sc_step_launch(A[ai], B[ai], m, nullptr, nullptr, nullptr, true, partial, blocks, s);
          else
            sc_step_launch(A[ai], B[ai], m, &st->rw[i - 1], A[ai ^ 1], B[ai ^ 1], true, partial, blocks, s);
          k_whir_round<<<1, 256, 0, s>>>(partial, blocks, st, i, tr, op, oc);
          GBZ_CUDA(cudaGetLastError());
        }
        if (i > 0) {
          ai ^= 1;
          m /= 2;
        }
      }
      if (!dry)
        sc_step_launch(A[ai], B[ai], m, &st->rw[logk - 1], A[ai ^ 1], B[ai ^ 1], false, partial,
                       sc_blocks(std::max<uint64_t>(m / 4, 1)), s);
      ai ^= 1;
      m /= 2;
      // Whir_Commit_initial(arr, 2 rate) (Whir.cpp:158-190)
      const uint64_t NL = 2 * (uint64_t)cur * m;
      const int nci = ci == 0 ? 1 : 0;
      const uint64_t off_root = lay.rec(T_WHIR_ROOT, 1, 32);
      if (!dry) {
        ntt_launch(R.tables(ilog2(NL)), A[ai], m, C[nci], tmp, false, s);
        k_merkle_root<<<1, 32, 0, s>>>(C[nci], ilog2(NL / 4), tr, off_root);
        GBZ_CUDA(cudaGetLastError());
      }
      // whir_query on the current codeword and tree
      BoQueryArgs qa{};
      qa.off_q = lay.rec(T_WHIR_QUERIES, e.l, 4);
      qa.off_rep = lay.rec(T_WHIR_REPLIES, e.l * e.kappa, 16);
      qa.off_ans = lay.rec(T_WHIR_ANSWERS, e.l, 16);
      const uint64_t off_path = lay.rec(T_WHIR_PATHS, e.l * e.depth, 32);
      qa.off_comb = lay.rec(T_WHIR_COMBINE, e.l, 16);
      qa.off_K = lay.rec(T_WHIR_K, 1, 16);
      if (trace) {
        trace->queries.push_back(qa.off_q);
        trace->comb.push_back(qa.off_comb);
        trace->l.push_back(e.l);
        trace->kappa.push_back(e.kappa);
        trace->NL.push_back(NL);
      }
      if (!dry) {
        const NttTables &told = R.tables(ilog2(L)), &tnew = R.tables(ilog2(NL));
        qa.st = st;
        qa.cw = cw;
        qa.L = L;
        qa.qmod = e.kappa > 4 ? L / e.kappa : L / 4;
        qa.logk = logk;
        qa.l = e.l;
        qa.tr = tr;
        qa.inv_lo = told.lo_inv;
        qa.inv_hi = told.hi_inv;
        qa.new_lo = tnew.lo_fwd;
        qa.new_hi = tnew.hi_fwd;
        qa.len_inv = finv(fe_make((uint64_t)e.kappa, 0));
        bo_query_kernel<<<1, kMaxQueries, 0, s>>>(qa);
        GBZ_CUDA(cudaGetLastError());
        launch_paths(tree_kind, tree, cw, leaves, e.l, e.depth, off_path, qa.off_q);
        // update_betas on the new codeword length: exponents 2 q_i of
        // omega_NL, i.e. q_i of omega_{NL/2}
        if (update_betas_by_transform(e.l, m, NL / 2)) {
          ntt_sparse_accumulate(R.tables(ilog2(NL) - 1), st->q, st->comb, e.l, B[ai], m, tmp2, s, 1);
        } else {
          update_betas_launch(B[ai], m, st, e.l, R.ub_scratch, s);
        }
      }
      cw = dry ? nullptr : C[nci];
      tree_kind = TREE_CODEWORD;
      ci = nci;
      L = NL;
      leaves = L / 4;
      cur *= 2;
    }
    if (e.aggregate) {
      const int g = e.group;
      const uint64_t off_ch = lay.rec(T_AGGR_CHALLENGES, 2 * g, 16), off_K = lay.rec(T_AGGR_K, 1, 16);
      const uint64_t off_q = lay.rec(T_AGGR_QUERIES, e.la, 4), off_p = lay.rec(T_AGGR_PATHS, e.la * e.depth_a, 32);
      const uint64_t off_root = lay.rec(T_AGGR_ROOT, 1, 32);
      const int nci = ci == 0 ? 1 : 0;
      if (!dry) {
        bo_aggr_draw_kernel<<<1, 32, 0, s>>>(st, g, coef, tr, off_ch);
        GBZ_CUDA(cudaGetLastError());
        VecList va{}, vb{}, vc{};
        va.p[0] = A[ai];
        vb.p[0] = B[ai];
        vc.p[0] = cw;
        for (int i = 1; i < g; i++) {
          va.p[i] = arrays[e.first + i - 1];
          vb.p[i] = betas[e.first + i - 1];
          vc.p[i] = codewords[e.first + i - 1];
        }
        // aggregate_arrays: the inner products first (they read arr and b
        // as they were), then arr += sum_{i>=1} ch2_i A_i, b += sum ch1_i B_i
        multidot_launch(va, g, vb, g, m, mdp, evals, s);
        bo_aggr_k_kernel<<<1, 32, 0, s>>>(st, evals, coef, g, tr, off_K);
        GBZ_CUDA(cudaGetLastError());
        if (g > 1) {
          VecList oa{}, ob{};
          for (int i = 1; i < g; i++) {
            oa.p[i - 1] = va.p[i];
            ob.p[i - 1] = vb.p[i];
          }
          lincomb_launch(oa, coef + g + 1, g - 1, m, A[ai], true, s);
          lincomb_launch(ob, coef + 1, g - 1, m, B[ai], true, s);
        }
        // aggregate_commitments: codeword = sum ch2_i C_i, openings in the
        // current tree, then the tree over zero leaves
        lincomb_launch(vc, coef + g, g, L, C[nci], false, s);
        bo_aggr_queries_kernel<<<1, 32, 0, s>>>(st, e.la, (int32_t)(L / 4), tr, off_q);
        GBZ_CUDA(cudaGetLastError());
        launch_paths(tree_kind, tree, cw, leaves, e.la, e.depth_a, off_p, off_q);
        k_zero_tree_root<<<1, 32, 0, s>>>(ilog2(e.leaves_after), tr, off_root);
        GBZ_CUDA(cudaGetLastError());
        cw = C[nci];
      }
      tree_kind = TREE_ZERO;
      ci = nci;
      leaves = e.leaves_after;
    }
  }
  const uint64_t off_poly = lay.rec(T_FINAL_POLY, (uint32_t)m, 16);
  const uint64_t off_point = lay.rec(T_FINAL_POINT, ilog2(m), 16);
  const uint64_t off_eval = lay.rec(T_FINAL_EVAL, 1, 16);
  if (trace) {
    trace->final_poly = off_poly;
    trace->final_point = off_point;
    trace->final_eval = off_eval;
    trace->m_final = m;
    trace->L_final = L;
    trace->last_codeword = cw;
    trace->final_arr = A[ai];
  }
  if (!dry) {
    k_final<<<1, 32, 0, s>>>(st, A[ai], B[ai], (int)m, tr, off_poly, off_point, off_eval, 1, nullptr);
    GBZ_CUDA(cudaGetLastError());
  }
}

void batch_open_enqueue(BatchResources &R, const BatchPlan &P, const fe *const *arrays, const fe *const *betas,
                        const fe *const *codewords, const uint8_t *levels0, fe K0, const glibc_prng &g0,
                        uint8_t *dtr) {
  Layout lay;
  lay.record_headers = true;
  batch_open_walk(R, P, arrays, betas, codewords, levels0, nullptr, lay, true);
  if (lay.len != P.transcript_bytes) throw ArgError("batch open: transcript layout mismatch");
  // record headers, payloads filled by the kernels
  std::vector<uint8_t> img(lay.len, 0);
  for (const auto &h : lay.headers) {
    std::memcpy(&img[h.off], &h.tag, 4);
    std::memcpy(&img[h.off + 4], &h.count, 4);
  }
  GBZ_CUDA(cudaMemcpyAsync(dtr, img.data(), lay.len, cudaMemcpyHostToDevice, R.s));
  GBZ_CUDA(cudaStreamSynchronize(R.s));  // img is host memory
  bo_init_kernel<<<1, 32, 0, R.s>>>(R.st, g0, K0);
  GBZ_CUDA(cudaGetLastError());
  Layout lay2;
  batch_open_walk(R, P, arrays, betas, codewords, levels0, dtr, lay2, false);
}

}  // namespace gbz
