// Reference-signature front end for libgbz.
//
// A maintainer of the reference prover adds this translation unit to its
// build (and removes the bodies it replaces from utils.cpp, merkle_tree.cpp
// and Blake3_hash.cpp) to run the hot path on the GPU without touching any
// caller.  It compiles against the reference's own headers (config_pc.hpp,
// merkle_tree.h, Blake3_hash.h) and forwards to the C ABI of include/gbz.h.
// Field elements are passed by pointer: virgo::fieldElement is {real, img}
// as two 64-bit words, which is exactly the element layout gbz.h expects.
//
// Errors: the reference prints and exits; this shim does the same on a
// non-OK status so that callers see unchanged behaviour.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "config_pc.hpp"
#include "merkle_tree.h"
#include "gbz.h"

namespace {

gbz_ctx *ctx() {
  static thread_local gbz_ctx *c = nullptr;
  if (!c) {
    gbz_status s = gbz_create(&c, 0);
    if (s != GBZ_OK) {
      std::fprintf(stderr, "gbz_create failed: %s\n", gbz_status_string(s));
      std::exit(-1);
    }
  }
  return c;
}

void check(gbz_status s, const char *what) {
  if (s != GBZ_OK) {
    std::fprintf(stderr, "%s failed: %s (%s)\n", what, gbz_status_string(s), gbz_last_error(ctx()));
    std::exit(-1);
  }
}

uint64_t *words(F *p) { return reinterpret_cast<uint64_t *>(p); }
const uint64_t *words(const F *p) { return reinterpret_cast<const uint64_t *>(p); }

static_assert(sizeof(F) == 16, "virgo::fieldElement must be two 64-bit words");
static_assert(sizeof(_hash) == 32, "_hash must be 32 bytes");

}  // namespace

// fft (utils.cpp:904-964)
void fft(vector<F> &arr, int logn, bool flag) {
  check(gbz_fft(ctx(), words(arr.data()), logn, flag ? 1 : 0, GBZ_MEM_HOST), "fft");
}

// pfft (utils.cpp:1583-1673): the forward transform for lengths above 1024;
// below that it defers to fft with the caller's flag.
void pfft(vector<F> &arr, int logn, bool flag) {
  const bool inverse = ((1 << logn) / 256 <= 4) ? flag : false;
  check(gbz_fft(ctx(), words(arr.data()), logn, inverse ? 1 : 0, GBZ_MEM_HOST), "pfft");
}

// blake3_hash (Blake3_hash.cpp:5-10)
void blake3_hash(uint8_t *src, uint8_t *dst) { check(gbz_blake3_64(ctx(), src, dst, 1, GBZ_MEM_HOST), "blake3_hash"); }

// precompute_beta (utils.cpp:198-243)
void precompute_beta(vector<F> r, vector<F> &B) {
  B.resize(1u << r.size());
  check(gbz_precompute_beta(ctx(), words(r.data()), (int)r.size(), words(B.data()), GBZ_MEM_HOST),
        "precompute_beta");
}

// MT_commit_Blake (merkle_tree.cpp:195-233) for N > 2; the reference's N <= 2
// branch hashes two elements plus 32 unset bytes and is not on the GPU path.
void merkle_tree::merkle_tree_prover::MT_commit_Blake(F *leafs, vector<vector<_hash>> &hashes, int N) {
  if (N <= 2) {
    std::fprintf(stderr, "MT_commit_Blake: N <= 2 is not supported by the GPU path\n");
    std::exit(-1);
  }
  std::vector<_hash> flat((size_t)N / 2 - 1);
  check(gbz_merkle_commit_blake(ctx(), words(leafs), (uint64_t)N, reinterpret_cast<uint8_t *>(flat.data()),
                                GBZ_MEM_HOST),
        "MT_commit_Blake");
  int levels = 0;
  for (int c = N / 4; c >= 1; c /= 2) levels++;
  if ((int)hashes.size() == 0) hashes.resize(levels);
  size_t off = 0, lv = 0;
  for (int c = N / 4; c >= 1; c /= 2, lv++) {
    hashes[lv].assign(flat.begin() + off, flat.begin() + off + c);
    off += c;
  }
}
