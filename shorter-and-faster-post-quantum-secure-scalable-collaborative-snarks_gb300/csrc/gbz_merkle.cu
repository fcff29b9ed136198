// Blake3 Merkle commitment.
//
// Replaces MT_commit_Blake (merkle_tree.cpp:195-233) and create_tree_blake
// (merkle_tree.cpp:267-299):
//   level 0, leaf i  = blake3(e[4i] || e[4i+1] || e[4i+2] || e[4i+3])
//                      (the 64 raw bytes of four field elements);
//   level k, node i  = blake3(node_{k-1}[2i] || node_{k-1}[2i])
//                      (the reference hashes the LEFT child twice and never
//                      reads the right one; reproduced as is).
// Every level is stored because opening paths (open_tree_blake,
// merkle_tree.cpp:320-335) read siblings from all of them.
//
// One thread compresses one node with the 64-byte message in registers.  A
// CTA computes kNodesPerCta nodes of its first level and then, in shared
// memory, every level above them that lies inside its subtree, so one
// launch covers log2(kNodesPerCta) + 1 levels.
#include "gbz_internal.cuh"

namespace gbz {

namespace {

constexpr int kThreads = 256;
// Nodes of a CTA's first level: 2^10 or 2^11 (the even halves of two levels
// in shared memory take 24 or 48 KiB).  Larger subtrees leave fewer threads
// idle in the upper levels of a CTA; set by merkle_set_fusion.
int g_log_nodes = 10;
// Small trees are latency bound (one dependent compression per level): the
// subtree per CTA shrinks, down to 2^8 nodes, until the first level spreads
// over at least two CTAs per SM of the 152 SMs, so that a thread hashes
// about one node per level instead of eight.
constexpr int kMinLogNodes = 8;
constexpr uint64_t kFillCtas = 2 * 152;
int fusion_for(uint64_t first_level_nodes) {
  int lg = g_log_nodes;
  while (lg > kMinLogNodes && (first_level_nodes >> lg) < kFillCtas) lg--;
  return lg;
}

struct Hash {
  uint32_t w[8];
};

__device__ __forceinline__ void load_hash(const uint8_t *p, uint32_t w[8]) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  uint4 a = q[0], b = q[1];
  w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
  w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
}
__device__ __forceinline__ void store_hash(uint8_t *p, const uint32_t w[8]) {
  uint4 *q = reinterpret_cast<uint4 *>(p);
  q[0] = make_uint4(w[0], w[1], w[2], w[3]);
  q[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// With elems != nullptr the first level is leaves over `elems`; otherwise
// the first level is parents of the level stored at `child`.
template <int LOGN>
__global__ void __launch_bounds__(kThreads)
merkle_levels_kernel(const fe *elems, const uint8_t *child, uint64_t cnt0, uint8_t *levels,
                     uint64_t level_off0, int nlevels, uint64_t tree_hashes) {
  // grid.y: independent trees of the same shape, tree_hashes apart (the
  // child levels live in the same tree)
  levels += 32 * tree_hashes * blockIdx.y;
  if (child) child += 32 * tree_hashes * blockIdx.y;
  constexpr int kNodesPerCta = 1 << LOGN;
  // Only even nodes feed the level above (the right child is never read),
  // so each ping-pong buffer keeps the even half of a level.
  __shared__ Hash buf0[kNodesPerCta / 2];
  __shared__ Hash buf1[kNodesPerCta / 4];
  const uint64_t base = (uint64_t)blockIdx.x * kNodesPerCta;
  const uint32_t T = (uint32_t)min((uint64_t)kNodesPerCta, cnt0 - base);
  uint8_t *out = levels + 32 * level_off0;
  for (uint32_t i = threadIdx.x; i < T; i += kThreads) {
    uint64_t gi = base + i;
    uint32_t m[16], h[8];
    if (elems) {
      const uint4 *src = reinterpret_cast<const uint4 *>(elems + 4 * gi);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        uint4 v = src[k];
        m[4 * k] = v.x; m[4 * k + 1] = v.y; m[4 * k + 2] = v.z; m[4 * k + 3] = v.w;
      }
    } else {
      load_hash(child + 32 * (2 * gi), m);
#pragma unroll
      for (int k = 0; k < 8; k++) m[8 + k] = m[k];
    }
    blake3_block64(m, h);
    store_hash(out + 32 * gi, h);
    if (!(i & 1)) {
#pragma unroll
      for (int k = 0; k < 8; k++) buf0[i >> 1].w[k] = h[k];
    }
  }
  __syncthreads();
  uint64_t lvl_off = level_off0, lvl_cnt = cnt0, cta_base = base;
  uint32_t cur = T;
  Hash *rd = buf0, *wr = buf1;
  for (int l = 1; l < nlevels && cur > 1; l++) {
    lvl_off += lvl_cnt;
    lvl_cnt >>= 1;
    cta_base >>= 1;
    cur >>= 1;
    uint8_t *o = levels + 32 * lvl_off;
    for (uint32_t i = threadIdx.x; i < cur; i += kThreads) {
      uint32_t m[16], h[8];
#pragma unroll
      for (int k = 0; k < 8; k++) { m[k] = rd[i].w[k]; m[8 + k] = m[k]; }
      blake3_block64(m, h);
      store_hash(o + 32 * (cta_base + i), h);
      if (!(i & 1)) {
#pragma unroll
        for (int k = 0; k < 8; k++) wr[i >> 1].w[k] = h[k];
      }
    }
    Hash *t = rd;
    rd = wr;
    wr = t;
    __syncthreads();
  }
}

__global__ void blake3_batch_kernel(const uint8_t *in, uint8_t *out, uint64_t count) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint32_t m[16], h[8];
  const uint8_t *p = in + 64 * i;
  for (int k = 0; k < 16; k++)
    m[k] = (uint32_t)p[4 * k] | ((uint32_t)p[4 * k + 1] << 8) | ((uint32_t)p[4 * k + 2] << 16) |
           ((uint32_t)p[4 * k + 3] << 24);
  blake3_block64(m, h);
  for (int k = 0; k < 8; k++)
    for (int b = 0; b < 4; b++) out[32 * i + 4 * k + b] = (uint8_t)(h[k] >> (8 * b));
}

void launch_levels(int logn_cta, const fe *elems, const uint8_t *child, uint64_t cnt, uint8_t *levels,
                   uint64_t off, int nlev, cudaStream_t s, int trees = 1, uint64_t tree_hashes = 0) {
  const dim3 g((unsigned)((cnt + (1ull << logn_cta) - 1) >> logn_cta), (unsigned)trees);
  switch (logn_cta) {
    case 11: merkle_levels_kernel<11><<<g, kThreads, 0, s>>>(elems, child, cnt, levels, off, nlev, tree_hashes); break;
    case 10: merkle_levels_kernel<10><<<g, kThreads, 0, s>>>(elems, child, cnt, levels, off, nlev, tree_hashes); break;
    case 9: merkle_levels_kernel<9><<<g, kThreads, 0, s>>>(elems, child, cnt, levels, off, nlev, tree_hashes); break;
    default: merkle_levels_kernel<8><<<g, kThreads, 0, s>>>(elems, child, cnt, levels, off, nlev, tree_hashes); break;
  }
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace

void merkle_set_fusion(int log_nodes_per_cta) {
  if (log_nodes_per_cta != 10 && log_nodes_per_cta != 11) throw ArgError("Merkle fusion: 10 or 11");
  g_log_nodes = log_nodes_per_cta;
}
int merkle_get_fusion() { return g_log_nodes; }

void merkle_commit_launch(const fe *elems, uint64_t N, uint8_t *levels, cudaStream_t s) {
  if (N < 4 || !is_pow2(N)) throw ArgError("Merkle commitment needs a power-of-two length >= 4");
  const int depth = ilog2(N / 4);  // levels 0..depth
  const int lg = fusion_for(N / 4);
  uint64_t cnt = N / 4, off = 0;
  int level = 0;
  uint64_t child_off = 0;
  while (level <= depth) {
    int nlev = min(lg + 1, depth - level + 1);
    launch_levels(lg, level == 0 ? elems : nullptr, level == 0 ? nullptr : levels + 32 * child_off, cnt, levels,
                  off, nlev, s);
    // advance past the nlev levels just written
    for (int k = 0; k < nlev; k++) {
      child_off = off;
      off += cnt;
      cnt >>= 1;
    }
    level += nlev;
  }
}

void merkle_from_leaves_launch(uint8_t *levels, uint64_t L, cudaStream_t s, int trees) {
  if (!is_pow2(L)) throw ArgError("Merkle tree over leaves needs a power-of-two count");
  if (trees < 1 || trees > 65535) throw ArgError("Merkle trees: 1..65535 per launch");
  const int depth = ilog2(L);  // levels 1..depth above the leaves
  const int lg = fusion_for(L / 2 * (uint64_t)trees);
  uint64_t cnt = L / 2, off = L, child_off = 0;
  int level = 1;
  while (level <= depth) {
    const int nlev = min(lg + 1, depth - level + 1);
    launch_levels(lg, nullptr, levels + 32 * child_off, cnt, levels, off, nlev, s, trees, 2 * L - 1);
    for (int k = 0; k < nlev; k++) {
      child_off = off;
      off += cnt;
      cnt >>= 1;
    }
    level += nlev;
  }
}

int merkle_launch_count(uint64_t N) {
  const int depth = ilog2(N / 4);
  const int lg = fusion_for(N / 4);
  int level = 0, k = 0;
  while (level <= depth) {
    level += min(lg + 1, depth - level + 1);
    k++;
  }
  return k;
}

void blake3_batch_launch(const uint8_t *in, uint8_t *out, uint64_t count, cudaStream_t s) {
  if (!count) return;
  blake3_batch_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(in, out, count);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace gbz
