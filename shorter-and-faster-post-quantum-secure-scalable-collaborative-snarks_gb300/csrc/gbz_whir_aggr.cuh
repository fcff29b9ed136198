// Streaming kernels of the WHIR claim / commitment aggregation
// (gbz_whir_aggr.cu).
#pragma once
#include <algorithm>

#include "gbz_internal.cuh"

namespace gbz {

constexpr int kMaxVecs = 64;
struct VecList {
  const fe *p[kMaxVecs];
};

// out[t] = (accumulate ? out[t] : 0) + sum_{i<k} coef[i] v.p[i][t], t < n
// (coef: k device elements).
void lincomb_launch(const VecList &v, const fe *coef, int k, uint64_t n, fe *out, bool accumulate, cudaStream_t s);
// out[i * kb + j] = <a_i, b_j> over n entries (device, row-major); partial
// holds multidot_scratch(n) elements.
uint64_t multidot_scratch(uint64_t n);
void multidot_launch(const VecList &a, int ka, const VecList &b, int kb, uint64_t n, fe *partial, fe *out,
                     cudaStream_t s);
// aggregate_claims for k <= 4 arrays and c <= 4 points in passes of two
// points over the arrays, no eq table written: elo /
// ehi hold the c eq tables of the points' first h and last lg - h
// coordinates (2^h and 2^(lg - h) entries each, table j at j times that);
// w: the c beta weights then the k array weights (device).  Writes arr,
// baggr (n entries) and sums[i * c + j] = <a_i, eq_j>; partial holds
// multidot_scratch(n) elements.  Returns false (nothing launched) outside
// those counts.
bool aggr_claims_fused(const VecList &a, int k, int c, const fe *elo, const fe *ehi, int h, int lg, uint64_t n,
                       const fe *w, fe *arr, fe *baggr, fe *partial, fe *sums, cudaStream_t s);

}  // namespace gbz
