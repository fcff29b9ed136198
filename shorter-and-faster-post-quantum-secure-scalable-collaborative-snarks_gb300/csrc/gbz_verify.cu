// A standalone verifier of the single-party proof transcript (gbz_prove):
// every check the reference's prover runs inline on its own data
// (main.cpp:83-112 for the sumcheck, Whir_Iteration and the verification
// steps of Whir_Open, Whir.cpp:254-386, 422-467), replayed from the
// transcript alone.  Host code: the work is a few thousand field operations
// and Blake3 compressions per proof.
//
// What a transcript cannot show is not checked: the commitment roots and
// authentication paths.  The reference's trees hash the left child twice
// at every inner node (merkle_tree.cpp:267-299), so a root depends on the
// first leaf only and a path does not bind the replies of a query; the
// paths' shape is checked, their content is not.
#include <cstring>
#include <vector>

#include "gbz_ctx.cuh"

using namespace gbz_api;

namespace gbz {
namespace {

enum : uint32_t {
  V_LAYOUT = 1u << 0,       // a record's tag or count is not the expected one
  V_POINT = 1u << 1,        // the evaluation point is not the Fiat-Shamir draws
  V_SC_SUM = 1u << 2,       // a sumcheck message does not sum to the claim
  V_SC_CHALLENGE = 1u << 3, // a sumcheck challenge is not hash_to_field(message)
  V_SC_FINAL = 1u << 4,     // the final values do not give the last claim, or eq is wrong
  V_WHIR_SUM = 1u << 5,     // a WHIR round message does not sum to K
  V_WHIR_CHALLENGE = 1u << 6,
  V_QUERIES = 1u << 7,
  V_ANSWERS = 1u << 8,      // a folded answer is not the fold of its replies
  V_COMBINE = 1u << 9,      // the combination weights are not powers of the draw
  V_WHIR_K = 1u << 10,
  V_FINAL_POINT = 1u << 11,
  V_STEP2 = 1u << 12,       // Whir_Open's verification step 2: K = sum arr b
  V_STEP3 = 1u << 13,       // step 3: the final evaluation of b
};

struct Reader {
  const uint8_t *p;
  uint64_t len, off = 0;
  uint32_t bad = 0;
  // the payload of the next record if it has this tag and count, else null
  const uint8_t *rec(uint32_t tag, uint32_t count, uint32_t unit) {
    if (bad || off + 8 > len) {
      bad = 1;
      return nullptr;
    }
    uint32_t t, c;
    std::memcpy(&t, p + off, 4);
    std::memcpy(&c, p + off + 4, 4);
    const uint64_t n = (uint64_t)unit * count;
    if (t != tag || c != count || off + 8 + n > len) {
      bad = 1;
      return nullptr;
    }
    const uint8_t *out = p + off + 8;
    off += 8 + n;
    return out;
  }
};

fe ld(const uint8_t *p, uint64_t i) {
  fe v;
  std::memcpy(&v, p + 16 * i, 16);
  return v;
}

fe sum01(const fe h[3]) {  // p(0) + p(1) of p(x) = h0 x^2 + h1 x + h2
  return fadd(quad_eval(h[0], h[1], h[2], fe_zero()), quad_eval(h[0], h[1], h[2], fe_one()));
}

// prod_k (1 - x_k + x_k w^(q 2^k)): the multilinear extension of the
// geometric vector j -> w^(q j) (omega_identity, utils.cpp) at x.
fe geometric_at(fe w, uint64_t q, const std::vector<fe> &x) {
  fe acc = fe_one(), wp = fpow(w, q);
  for (const fe &xk : x) {
    acc = fmul(acc, fadd(fsub(fe_one(), xk), fmul(xk, wp)));
    wp = fmul(wp, wp);
  }
  return acc;
}

// prod_k eq(a_k, x_k) (beta_identity, utils.cpp).
fe eq_at(const std::vector<fe> &a, const std::vector<fe> &x) {
  fe acc = fe_one();
  for (size_t k = 0; k < a.size(); k++) {
    const fe ak = a[k], xk = x[k];
    acc = fmul(acc, fadd(fmul(ak, xk), fmul(fsub(fe_one(), ak), fsub(fe_one(), xk))));
  }
  return acc;
}

struct Term {  // c w^(q j) added to the betas while `vars` variables remained
  fe c, w;
  uint64_t q;
  int round;  // WHIR rounds (challenges) taken before it was added
};

uint32_t verify(const uint8_t *tr, uint64_t bytes, int logn, int rate, uint32_t seed) {
  constexpr int kK = 4, kLogK = 2;  // whir_k = 4
  Reader R{tr, bytes};
  uint32_t f = 0;
  glibc_prng g;
  prng_seed(g, seed);
  const uint64_t n = 1ull << logn;
  uint64_t L = n * (uint64_t)rate;
  R.rec(T_COMMIT_ROOT, 1, 32);
  // the evaluation point
  const uint8_t *pz = R.rec(T_EVAL_POINT, logn, 16);
  if (!pz) return V_LAYOUT;
  fe fs = fe_zero();
  std::vector<fe> z(logn);
  for (int i = 0; i < logn; i++) {
    fs = hash_F(fs, fe_zero());
    z[i] = ld(pz, i);
    if (!fe_eq(z[i], fs)) f |= V_POINT;
  }
  const uint8_t *pc = R.rec(T_CLAIM, 1, 16);
  if (!pc) return V_LAYOUT;
  fe y = ld(pc, 0);
  // the sumcheck of sum_x w(x) eq(z, x)
  std::vector<fe> chal(logn);
  for (int i = 0; i < logn; i++) {
    const uint8_t *ph = R.rec(T_SC_POLY, 3, 16), *pr = R.rec(T_SC_CHALLENGE, 1, 16);
    if (!ph || !pr) return V_LAYOUT;
    const fe h[3] = {ld(ph, 0), ld(ph, 1), ld(ph, 2)};
    if (!fe_eq(sum01(h), y)) f |= V_SC_SUM;
    for (int k = 0; k < 3; k++) fs = hash_F(fs, h[k]);
    chal[i] = ld(pr, 0);
    if (!fe_eq(chal[i], fs)) f |= V_SC_CHALLENGE;
    y = quad_eval(h[0], h[1], h[2], chal[i]);
  }
  const uint8_t *pf = R.rec(T_SC_FINAL, 2, 16);
  if (!pf) return V_LAYOUT;
  const fe wfin = ld(pf, 0), efin = ld(pf, 1);
  if (!fe_eq(fmul(wfin, efin), y) || !fe_eq(efin, eq_at(z, chal))) f |= V_SC_FINAL;
  // WHIR opening of w at chal with claim wfin
  fe K = wfin;
  std::vector<fe> rounds;  // every WHIR round challenge in order
  std::vector<Term> terms;
  uint64_t m = n;
  int cur = rate;
  for (int it = 0; it < kMaxWhirIter; it++) {
    fe r[kLogK];
    for (int i = 0; i < kLogK; i++) {
      const uint8_t *ph = R.rec(T_WHIR_POLY, 3, 16), *pr = R.rec(T_WHIR_CHALLENGE, 1, 16);
      if (!ph || !pr) return V_LAYOUT;
      const fe h[3] = {ld(ph, 0), ld(ph, 1), ld(ph, 2)};
      if (!fe_eq(sum01(h), K)) f |= V_WHIR_SUM;
      r[i] = ld(pr, 0);
      if (!fe_eq(r[i], prng_field(g))) f |= V_WHIR_CHALLENGE;
      K = quad_eval(h[0], h[1], h[2], r[i]);
      rounds.push_back(r[i]);
      m /= 2;
    }
    const uint64_t NL = m * 2 * (uint64_t)cur;
    R.rec(T_WHIR_ROOT, 1, 32);
    const int l = whir_query_count(cur);
    const uint8_t *pq = R.rec(T_WHIR_QUERIES, l, 4), *prep = R.rec(T_WHIR_REPLIES, l * kK, 16),
                  *pa = R.rec(T_WHIR_ANSWERS, l, 16);
    const int depth = ilog2(L / 4);
    R.rec(T_WHIR_PATHS, (uint32_t)(l * depth), 32);
    const uint8_t *pw = R.rec(T_WHIR_COMBINE, l, 16), *pk = R.rec(T_WHIR_K, 1, 16);
    if (!pq || !prep || !pa || !pw || !pk) return V_LAYOUT;
    // the queries (Whir.cpp:262-268) and the fold of each query's replies
    // (get_RS_multifold_segment_tensor at the two round challenges)
    const fe winv = finv(root_of_unity(ilog2(L))), quarter = finv(fe_make(4, 0));
    std::vector<uint64_t> qs(l);
    for (int i = 0; i < l; i++) {
      int32_t q;
      std::memcpy(&q, pq + 4 * i, 4);
      const int32_t draw = prng_next(g) % (int32_t)(L / 4);
      if (q != draw || q < 0) f |= V_QUERIES;
      qs[i] = (uint64_t)(uint32_t)q % (L / 4);
      fe seg[kK];
      for (int j = 0; j < kK; j++) seg[j] = ld(prep, (uint64_t)kK * i + j);
      fe part[2];
      fe om = fpow(winv, qs[i]);
      const fe step = fpow(winv, L / 4);
      for (int j = 0; j < 2; j++) {
        const fe s = fadd(seg[j], seg[j + 2]), d = fsub(seg[j], seg[j + 2]);
        part[j] = fadd(fmul(fsub(fe_one(), r[0]), s), fmul(fmul(r[0], om), d));
        om = fmul(om, step);
      }
      const fe po = fpow(winv, (2 * qs[i]) & (L - 1));
      const fe s = fadd(part[0], part[1]), d = fsub(part[0], part[1]);
      const fe ans = fmul(quarter, fadd(fmul(fsub(fe_one(), r[1]), s), fmul(r[1], fmul(po, d))));
      if (!fe_eq(ans, ld(pa, i))) f |= V_ANSWERS;
    }
    // update_betas (Whir.cpp:325-342): weights r^(i+1), the queries scaled
    // to the new codeword, the running claim
    const fe rb = prng_field(g);
    fe c = fe_one();
    const fe wnew = root_of_unity(ilog2(NL));
    for (int i = 0; i < l; i++) {
      c = fmul(c, rb);
      if (!fe_eq(c, ld(pw, i))) f |= V_COMBINE;
      K = fadd(K, fmul(c, ld(pa, i)));
      terms.push_back({c, wnew, qs[i] * (uint64_t)(kK * NL / L), (int)rounds.size()});
    }
    if (!fe_eq(K, ld(pk, 0))) f |= V_WHIR_K;
    L = NL;
    cur *= 2;
    if (m <= (uint64_t)kK) break;
  }
  const uint8_t *pp = R.rec(T_FINAL_POLY, (uint32_t)m, 16);
  const int lgm = ilog2(m);
  const uint8_t *prf = R.rec(T_FINAL_POINT, lgm, 16), *pe = R.rec(T_FINAL_EVAL, 1, 16);
  if (!pp || !prf || !pe) return V_LAYOUT;
  std::vector<fe> rf(lgm);
  for (int i = 0; i < lgm; i++) {
    rf[i] = ld(prf, i);
    if (!fe_eq(rf[i], prng_field(g))) f |= V_FINAL_POINT;
  }
  // the betas after every fold and update, entry j: each term's multilinear
  // extension at (the rounds after it, the bits of j)
  std::vector<fe> bfin(m);
  for (uint64_t j = 0; j < m; j++) {
    std::vector<fe> bits(lgm);
    for (int k = 0; k < lgm; k++) bits[k] = ((j >> k) & 1) ? fe_one() : fe_zero();
    std::vector<fe> x(rounds);
    x.insert(x.end(), bits.begin(), bits.end());
    fe v = eq_at(chal, x);
    for (const Term &t : terms) {
      std::vector<fe> xt(rounds.begin() + t.round, rounds.end());
      xt.insert(xt.end(), bits.begin(), bits.end());
      v = fadd(v, fmul(t.c, geometric_at(t.w, t.q, xt)));
    }
    bfin[j] = v;
  }
  // verification step 2: K = sum_j arr[j] b[j]; step 3: y = b(rf)
  fe s = fe_zero();
  for (uint64_t j = 0; j < m; j++) s = fadd(s, fmul(ld(pp, j), bfin[j]));
  if (!fe_eq(s, K)) f |= V_STEP2;
  fe ev = fe_zero();
  for (uint64_t j = 0; j < m; j++) {
    fe e = fe_one();
    for (int k = 0; k < lgm; k++) e = fmul(e, ((j >> k) & 1) ? rf[k] : fsub(fe_one(), rf[k]));
    ev = fadd(ev, fmul(bfin[j], e));
  }
  if (!fe_eq(ev, ld(pe, 0))) f |= V_STEP3;
  if (R.bad || R.off != bytes) f |= V_LAYOUT;
  return f;
}

}  // namespace
}  // namespace gbz

using namespace gbz;

extern "C" {

gbz_status gbz_verify_proof(const uint8_t *transcript, uint64_t bytes, int logn, int rate, uint32_t prng_seed,
                            uint32_t *failed) {
  if (!transcript) return GBZ_EINVAL;
  if (logn < 3 || logn > 25 || rate < 2 || rate > 64 || !is_pow2((uint64_t)rate)) return GBZ_EINVAL;
  uint32_t f = 0;
  try {
    f = verify(transcript, bytes, logn, rate, prng_seed);
  } catch (...) {
    f = 1;
  }
  if (failed) *failed = f;
  return f ? GBZ_ECHECK : GBZ_OK;
}

}  // extern "C"
