// The three-axis binned-SAH tree of scene.cpp:build_sah3, built on the GPU.
//
// The host builder splits a node of more than 4 primitives at the cheapest
// of the 3 x 127 bin boundaries (128 bins per axis over the node's centroid
// bounds, cost = half-area x count on each side), or at the object median of
// the widest centroid axis below depth 36 or when no axis has a valid
// boundary. Every choice depends only on the SET of primitives in the node,
// so a builder that makes the same f32 computations on the same sets makes
// the same tree: the same node boxes, the same children, the same leaf ranges
// in the same preorder numbering. Only the order of the primitives inside a
// leaf may differ (the host partitions in place, unstably; this builder
// partitions stably), and no traversal result depends on it under the
// near-tie rule, which is the only rule that walks this tree.
//
// Two phases:
//   * large nodes (more than kSmall primitives), one level at a time: every
//     node's primitives are cut into chunks of kChunk, one block per chunk;
//     blocks reduce the node's bounds, then bin the centroids of the chunk on
//     all three axes in shared memory and add the bins to the node's bins
//     (ordered-integer atomics: min/max of floats is exact in any order),
//     then one block per node sweeps the bins (three warps, one per axis),
//     then the chunks partition stably into a scratch copy;
//   * small nodes: one block per node builds its whole subtree in shared
//     memory (depth first, an explicit stack of pending right children),
//     taking node ids from a global counter.
// The host reads back the node table and numbers it in the host builder's
// preorder (a node, then its left subtree, then its right subtree).
#include <cfloat>
#include <cstring>
#include <vector>

#include "omg_internal.h"

namespace omg {

namespace {

constexpr int kBins = 128;
constexpr uint32_t kLeafMax = 4;       // mesh.rs:16
constexpr uint32_t kMedianDepth = 36;  // scene.cpp: Sah3Builder::kMedianDepth
constexpr uint32_t kSmall = 2048;      // a node of at most this many primitives: one block builds its subtree
constexpr uint32_t kChunk = 2048;      // primitives per block in the large-node passes
constexpr int kThreads = 256;
constexpr int kPer = kChunk / kThreads;  // positions per thread in a chunk (consecutive: stable partition)
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kStack = 64;
constexpr int kBinWords = 7;            // lo[3], hi[3] (ordered integers), count

__device__ __forceinline__ uint32_t f2o(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

// BinBox::half_area (scene.cpp), operation for operation
__device__ __forceinline__ float half_area(const float lo[3], const float hi[3]) {
  float e[3];
#pragma unroll
  for (int k = 0; k < 3; k++) e[k] = fmaxf(__fsub_rn(hi[k], lo[k]), 0.0f);
  return __fadd_rn(__fadd_rn(__fmul_rn(e[0], e[1]), __fmul_rn(e[1], e[2])), __fmul_rn(e[2], e[0]));
}

// Per-primitive box and box centre: pd[3i] = (lo, c.x), pd[3i+1] = (hi, c.y),
// pd[3i+2].x = c.z (build_sah3: the box of a, a + e1, a + e2).
__global__ void prim_data_kernel(const float4* __restrict__ prims, uint32_t n, float4* __restrict__ pd,
                                 uint32_t* __restrict__ idx) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = prims[3 * i], e1 = prims[3 * i + 1], e2 = prims[3 * i + 2];
  const float av[3] = {a.x, a.y, a.z}, bv[3] = {e1.x, e1.y, e1.z}, cv[3] = {e2.x, e2.y, e2.z};
  float lo[3], hi[3], c[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float x0 = av[k], x1 = __fadd_rn(av[k], bv[k]), x2 = __fadd_rn(av[k], cv[k]);
    lo[k] = fminf(fminf(x0, x1), x2);
    hi[k] = fmaxf(fmaxf(x0, x1), x2);
    c[k] = __fmul_rn(__fadd_rn(lo[k], hi[k]), 0.5f);
  }
  pd[3 * i] = make_float4(lo[0], lo[1], lo[2], c[0]);
  pd[3 * i + 1] = make_float4(hi[0], hi[1], hi[2], c[1]);
  pd[3 * i + 2] = make_float4(c[2], 0.0f, 0.0f, 0.0f);
  idx[i] = i;
}

struct PrimBox {
  float lo[3], hi[3], c[3];
};
__device__ __forceinline__ PrimBox load_prim(const float4* __restrict__ pd, uint32_t id) {
  const float4 q0 = __ldg(pd + 3 * id), q1 = __ldg(pd + 3 * id + 1), q2 = __ldg(pd + 3 * id + 2);
  PrimBox b;
  b.lo[0] = q0.x; b.lo[1] = q0.y; b.lo[2] = q0.z;
  b.hi[0] = q1.x; b.hi[1] = q1.y; b.hi[2] = q1.z;
  b.c[0] = q0.w; b.c[1] = q1.w; b.c[2] = q2.x;
  return b;
}

// Node bounds: box lo (min), box hi (max), centroid min, centroid max.
struct Bounds {
  float v[12];
  __device__ void clear() {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      v[k] = FLT_MAX; v[3 + k] = -FLT_MAX; v[6 + k] = FLT_MAX; v[9 + k] = -FLT_MAX;
    }
  }
  __device__ void grow(const PrimBox& p) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      v[k] = fminf(v[k], p.lo[k]);
      v[3 + k] = fmaxf(v[3 + k], p.hi[k]);
      v[6 + k] = fminf(v[6 + k], p.c[k]);
      v[9 + k] = fmaxf(v[9 + k], p.c[k]);
    }
  }
  __device__ void warp_reduce() {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], d));
        v[3 + k] = fmaxf(v[3 + k], __shfl_xor_sync(0xffffffffu, v[3 + k], d));
        v[6 + k] = fminf(v[6 + k], __shfl_xor_sync(0xffffffffu, v[6 + k], d));
        v[9 + k] = fmaxf(v[9 + k], __shfl_xor_sync(0xffffffffu, v[9 + k], d));
      }
    }
  }
};
__device__ __forceinline__ bool is_min_word(int k) { return k < 3 || (k >= 6 && k < 9); }

// Block-wide bounds of a node (every thread of the block calls this; all get
// the result). red: 8 x 12 floats of shared memory.
__device__ Bounds block_bounds(Bounds b, float* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  b.warp_reduce();
  if (lane == 0)
    for (int k = 0; k < 12; k++) red[12 * warp + k] = b.v[k];
  __syncthreads();
  Bounds r;
  r.clear();
  for (int w = 0; w < nw; w++)
    for (int k = 0; k < 12; k++) r.v[k] = is_min_word(k) ? fminf(r.v[k], red[12 * w + k]) : fmaxf(r.v[k], red[12 * w + k]);
  __syncthreads();
  return r;
}

// The binning of one node: per axis, whether it takes part (centroid extent
// above 1e-6), its lower bound and scale (build_sah3: kBins / extent).
struct Axes {
  float lo[3], scale[3];
  bool valid[3];
};
__device__ __forceinline__ Axes axes_of(const float* cmin, const float* cmax) {
  Axes x;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float w = __fsub_rn(cmax[a], cmin[a]);
    x.valid[a] = w > 1e-6f;
    x.lo[a] = cmin[a];
    x.scale[a] = x.valid[a] ? __fdiv_rn((float)kBins, w) : 0.0f;
  }
  return x;
}
__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
  return min(kBins - 1, __float2int_rz(__fmul_rn(__fsub_rn(c, lo), scale)));
}

__device__ __forceinline__ void clear_bins(uint32_t* bins, int n_words_per_axis) {
  for (int t = threadIdx.x; t < 3 * n_words_per_axis; t += blockDim.x) {
    const int w = (t % (kBins * kBinWords)) % kBinWords;
    bins[t] = w < 3 ? f2o(FLT_MAX) : (w < 6 ? f2o(-FLT_MAX) : 0u);
  }
}

__device__ __forceinline__ void bin_prim(uint32_t* bins, const Axes& x, const PrimBox& p) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (!x.valid[a]) continue;
    uint32_t* b = bins + (a * kBins + bin_of(p.c[a], x.lo[a], x.scale[a])) * kBinWords;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      atomicMin(b + k, f2o(p.lo[k]));
      atomicMax(b + 3 + k, f2o(p.hi[k]));
    }
    atomicAdd(b + 6, 1u);
  }
}

struct Cut {
  float cost;
  int k;
  uint32_t nl;
};

// The sweep of one axis's 128 bins by one warp (lane l holds bins 4l..4l+3):
// the build_sah3 loops, whose result is the first boundary k in 0..126 with
// the least cost, among boundaries with 0 < left count < n and cost below
// FLT_MAX (cost = HA(left) * nl + (nr ? HA(right) * nr : 0)). Box unions
// are min/max, exact in any order; every cost is the f32 expression the host
// evaluates.
__device__ Cut sweep_axis(const uint32_t* __restrict__ bins, uint32_t n) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  float lo[4][3], hi[4][3];
  uint32_t cnt[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const uint32_t* b = bins + (4 * lane + j) * kBinWords;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      lo[j][k] = o2f(b[k]);
      hi[j][k] = o2f(b[3 + k]);
    }
    cnt[j] = b[6];
  }
  // inclusive prefixes inside the lane, then over the lanes below
  float plo[4][3], phi[4][3];
  uint32_t pc[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      plo[j][k] = j ? fminf(plo[j - 1][k], lo[j][k]) : lo[j][k];
      phi[j][k] = j ? fmaxf(phi[j - 1][k], hi[j][k]) : hi[j][k];
    }
    pc[j] = j ? pc[j - 1] + cnt[j] : cnt[j];
  }
  // suffixes inside the lane
  float slo[4][3], shi[4][3];
  uint32_t sc[4];
#pragma unroll
  for (int j = 3; j >= 0; j--) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      slo[j][k] = j < 3 ? fminf(slo[j + 1][k], lo[j][k]) : lo[j][k];
      shi[j][k] = j < 3 ? fmaxf(shi[j + 1][k], hi[j][k]) : hi[j][k];
    }
    sc[j] = j < 3 ? sc[j + 1] + cnt[j] : cnt[j];
  }
  // exclusive scans of the lane totals: below (prefix) and above (suffix)
  float elo[3], ehi[3], alo[3], ahi[3];
  uint32_t ec = 0, ac = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    elo[k] = FLT_MAX; ehi[k] = -FLT_MAX; alo[k] = FLT_MAX; ahi[k] = -FLT_MAX;
  }
  {
    float tlo[3], thi[3], ulo[3], uhi[3];
    uint32_t tc = pc[3], uc = sc[0];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      tlo[k] = plo[3][k]; thi[k] = phi[3][k]; ulo[k] = slo[0][k]; uhi[k] = shi[0][k];
    }
    // inclusive scans of the lane totals, then shifted by one lane
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      float ol[3], oh[3], pl[3], ph[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        ol[k] = __shfl_up_sync(FULL, tlo[k], d);
        oh[k] = __shfl_up_sync(FULL, thi[k], d);
        pl[k] = __shfl_down_sync(FULL, ulo[k], d);
        ph[k] = __shfl_down_sync(FULL, uhi[k], d);
      }
      const uint32_t oc = __shfl_up_sync(FULL, tc, d), qc = __shfl_down_sync(FULL, uc, d);
      if (lane >= d) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          tlo[k] = fminf(tlo[k], ol[k]);
          thi[k] = fmaxf(thi[k], oh[k]);
        }
        tc += oc;
      }
      if (lane + d < 32) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          ulo[k] = fminf(ulo[k], pl[k]);
          uhi[k] = fmaxf(uhi[k], ph[k]);
        }
        uc += qc;
      }
    }
    float ol[3], oh[3], pl[3], ph[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ol[k] = __shfl_up_sync(FULL, tlo[k], 1);
      oh[k] = __shfl_up_sync(FULL, thi[k], 1);
      pl[k] = __shfl_down_sync(FULL, ulo[k], 1);
      ph[k] = __shfl_down_sync(FULL, uhi[k], 1);
    }
    const uint32_t oc = __shfl_up_sync(FULL, tc, 1), qc = __shfl_down_sync(FULL, uc, 1);
    if (lane > 0) {
#pragma unroll
      for (int k = 0; k < 3; k++) { elo[k] = ol[k]; ehi[k] = oh[k]; }
      ec = oc;
    }
    if (lane < 31) {
#pragma unroll
      for (int k = 0; k < 3; k++) { alo[k] = pl[k]; ahi[k] = ph[k]; }
      ac = qc;
    }
  }
  Cut best{FLT_MAX, 0x7FFFFFFF, 0u};
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int k = 4 * lane + j;
    if (k >= kBins - 1) continue;
    float L[3], H[3], RL[3], RH[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      L[q] = fminf(elo[q], plo[j][q]);
      H[q] = fmaxf(ehi[q], phi[j][q]);
      RL[q] = j < 3 ? fminf(slo[j + 1][q], alo[q]) : alo[q];
      RH[q] = j < 3 ? fmaxf(shi[j + 1][q], ahi[q]) : ahi[q];
    }
    const uint32_t nl = ec + pc[j];
    const uint32_t nr = j < 3 ? sc[j + 1] + ac : ac;
    if (nl == 0u || nl == n) continue;
    const float rc = nr ? __fmul_rn(half_area(RL, RH), (float)nr) : 0.0f;
    const float cost = __fadd_rn(__fmul_rn(half_area(L, H), (float)nl), rc);
    if (cost < best.cost) {
      best.cost = cost;
      best.k = k;
      best.nl = nl;
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const float oc = __shfl_xor_sync(FULL, best.cost, d);
    const int ok = __shfl_xor_sync(FULL, best.k, d);
    const uint32_t onl = __shfl_xor_sync(FULL, best.nl, d);
    if (oc < best.cost || (oc == best.cost && ok < best.k)) {
      best.cost = oc;
      best.k = ok;
      best.nl = onl;
    }
  }
  return best;
}

// The split of one node: SAH (axis, bin boundary) or the object median of
// the widest centroid axis (build_sah3's fallback).
struct Decision {
  int32_t axis;
  int32_t cut;     // -1: median
  uint32_t nl;     // primitives on the left
  uint32_t pad;
};

__device__ Decision decide(const Cut* cuts, const Bounds& b, uint32_t n, uint32_t depth) {
  Decision d{-1, -1, 0u, 0u};
  if (depth < kMedianDepth) {
    float best = FLT_MAX;
    for (int a = 0; a < 3; a++)
      if (cuts[a].cost < best) {
        best = cuts[a].cost;
        d.axis = a;
        d.cut = cuts[a].k;
        d.nl = cuts[a].nl;
      }
  }
  if (d.axis < 0) {
    int a = 0;
    for (int k = 1; k < 3; k++)
      if (__fsub_rn(b.v[9 + k], b.v[6 + k]) > __fsub_rn(b.v[9 + a], b.v[6 + a])) a = k;
    d.axis = a;
    d.cut = -1;
    d.nl = n / 2;
  }
  return d;
}

// The median order: (centre on the axis, tessellation index), as the host's
// nth_element comparator (-0 and +0 compare equal there, so +0 is used).
__device__ __forceinline__ unsigned long long median_key(const float4* __restrict__ pd, uint32_t id, int axis) {
  const PrimBox p = load_prim(pd, id);
  return ((unsigned long long)f2o(__fadd_rn(p.c[axis], 0.0f)) << 32) | id;
}

// ---------------------------------------------------------------- large nodes
struct Chunk {
  uint32_t slot, b, e, node_s;
};
struct Slot {
  uint32_t id, s, e, depth;
};

__global__ void init_slots_kernel(uint32_t* __restrict__ sb, uint32_t* __restrict__ gbins, uint32_t n_slots) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_slots * 12) {
    const int k = t % 12;
    sb[t] = f2o(is_min_word(k) ? FLT_MAX : -FLT_MAX);
  }
  const uint32_t per = 3 * kBins * kBinWords;
  if (t < n_slots * per) {
    const int w = (t % (kBins * kBinWords)) % kBinWords;
    gbins[t] = w < 3 ? f2o(FLT_MAX) : (w < 6 ? f2o(-FLT_MAX) : 0u);
  }
}

__global__ void __launch_bounds__(kThreads) large_bounds_kernel(const Chunk* __restrict__ chunks,
                                                                const uint32_t* __restrict__ idx,
                                                                const float4* __restrict__ pd, uint32_t* __restrict__ sb) {
  __shared__ float red[8 * 12];
  const Chunk C = chunks[blockIdx.x];
  Bounds b;
  b.clear();
  for (uint32_t p = C.b + threadIdx.x; p < C.e; p += blockDim.x) b.grow(load_prim(pd, idx[p]));
  const Bounds r = block_bounds(b, red);
  if (threadIdx.x < 12) {
    const int k = threadIdx.x;
    if (is_min_word(k)) atomicMin(sb + 12 * C.slot + k, f2o(r.v[k]));
    else atomicMax(sb + 12 * C.slot + k, f2o(r.v[k]));
  }
}

__device__ __forceinline__ void slot_bounds(const uint32_t* sb, uint32_t slot, Bounds& b) {
  for (int k = 0; k < 12; k++) b.v[k] = o2f(sb[12 * slot + k]);
}

__global__ void __launch_bounds__(kThreads) large_bin_kernel(const Chunk* __restrict__ chunks,
                                                             const uint32_t* __restrict__ idx,
                                                             const float4* __restrict__ pd,
                                                             const uint32_t* __restrict__ sb,
                                                             uint32_t* __restrict__ gbins) {
  __shared__ uint32_t bins[3 * kBins * kBinWords];
  const Chunk C = chunks[blockIdx.x];
  Bounds nb;
  slot_bounds(sb, C.slot, nb);
  const Axes x = axes_of(nb.v + 6, nb.v + 9);
  clear_bins(bins, kBins * kBinWords);
  __syncthreads();
  for (uint32_t p = C.b + threadIdx.x; p < C.e; p += blockDim.x) bin_prim(bins, x, load_prim(pd, idx[p]));
  __syncthreads();
  uint32_t* g = gbins + (size_t)C.slot * 3 * kBins * kBinWords;
  for (int t = threadIdx.x; t < 3 * kBins; t += blockDim.x) {
    const uint32_t* b = bins + t * kBinWords;
    if (b[6] == 0u) continue;
    uint32_t* o = g + t * kBinWords;
    for (int k = 0; k < 3; k++) {
      atomicMin(o + k, b[k]);
      atomicMax(o + 3 + k, b[3 + k]);
    }
    atomicAdd(o + 6, b[6]);
  }
}

// one block of 96 threads per slot: warp a sweeps axis a
__global__ void large_sweep_kernel(const Slot* __restrict__ slots, const uint32_t* __restrict__ sb,
                                   const uint32_t* __restrict__ gbins, Decision* __restrict__ dec,
                                   float* __restrict__ nd_box) {
  __shared__ Cut cuts[3];
  const uint32_t si = blockIdx.x;
  const Slot S = slots[si];
  Bounds b;
  slot_bounds(sb, si, b);
  const Axes x = axes_of(b.v + 6, b.v + 9);
  const uint32_t n = S.e - S.s;
  const int warp = threadIdx.x >> 5;
  if (warp < 3) {
    Cut c{FLT_MAX, 0x7FFFFFFF, 0u};
    if (x.valid[warp] && S.depth < kMedianDepth)
      c = sweep_axis(gbins + ((size_t)si * 3 + warp) * kBins * kBinWords, n);
    if ((threadIdx.x & 31) == 0) cuts[warp] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    dec[si] = decide(cuts, b, n, S.depth);
    for (int k = 0; k < 6; k++) nd_box[6 * (size_t)S.id + k] = b.v[k];
  }
}

// left flags of a chunk's positions; returns this thread's kPer flags as bits
__device__ __forceinline__ uint32_t chunk_flags(const Chunk& C, const uint32_t* __restrict__ idx,
                                                const float4* __restrict__ pd, const Axes& x, const Decision& d,
                                                uint32_t& n_items) {
  const uint32_t p0 = C.b + threadIdx.x * kPer;
  uint32_t bits = 0;
  n_items = 0;
  for (int j = 0; j < kPer; j++) {
    const uint32_t p = p0 + j;
    if (p >= C.e) break;
    n_items++;
    const PrimBox q = load_prim(pd, idx[p]);
    if (bin_of(q.c[d.axis], x.lo[d.axis], x.scale[d.axis]) <= d.cut) bits |= 1u << j;
  }
  return bits;
}

// exclusive block scan of v (kThreads threads); returns the block total in tot
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* red, uint32_t& tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) red[warp] = inc;
  __syncthreads();
  uint32_t base = 0;
  tot = 0;
  for (int w = 0; w < nw; w++) {
    if (w < warp) base += red[w];
    tot += red[w];
  }
  __syncthreads();
  return base + inc - v;
}

__global__ void __launch_bounds__(kThreads) large_count_kernel(const Chunk* __restrict__ chunks,
                                                               const uint32_t* __restrict__ idx,
                                                               const float4* __restrict__ pd,
                                                               const uint32_t* __restrict__ sb,
                                                               const Decision* __restrict__ dec,
                                                               uint32_t* __restrict__ chunk_left) {
  __shared__ uint32_t red[32];
  const Chunk C = chunks[blockIdx.x];
  const Decision d = dec[C.slot];
  if (d.cut < 0) return;   // median nodes are ordered by the sort
  Bounds nb;
  slot_bounds(sb, C.slot, nb);
  const Axes x = axes_of(nb.v + 6, nb.v + 9);
  uint32_t ni;
  const uint32_t bits = chunk_flags(C, idx, pd, x, d, ni);
  uint32_t tot;
  block_exclusive_scan(__popc(bits), red, tot);
  if (threadIdx.x == 0) chunk_left[blockIdx.x] = tot;
}

// per slot: exclusive offsets of its chunks' left and right counts (one thread per slot)
__global__ void large_offsets_kernel(const uint32_t* __restrict__ first_chunk, uint32_t n_slots,
                                     const Chunk* __restrict__ chunks, const uint32_t* __restrict__ chunk_left,
                                     const Decision* __restrict__ dec, uint32_t* __restrict__ off_l,
                                     uint32_t* __restrict__ off_r, uint32_t* __restrict__ err) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_slots || dec[s].cut < 0) return;
  uint32_t l = 0, r = 0;
  for (uint32_t c = first_chunk[s]; c < first_chunk[s + 1]; c++) {
    off_l[c] = l;
    off_r[c] = r;
    l += chunk_left[c];
    r += (chunks[c].e - chunks[c].b) - chunk_left[c];
  }
  if (l != dec[s].nl) atomicOr(err, 1u);   // the partition must agree with the bins
}

__global__ void __launch_bounds__(kThreads) large_scatter_kernel(const Chunk* __restrict__ chunks,
                                                                 const uint32_t* __restrict__ idx,
                                                                 const float4* __restrict__ pd,
                                                                 const uint32_t* __restrict__ sb,
                                                                 const Decision* __restrict__ dec,
                                                                 const uint32_t* __restrict__ off_l,
                                                                 const uint32_t* __restrict__ off_r,
                                                                 uint32_t* __restrict__ tmp) {
  __shared__ uint32_t red[32];
  const Chunk C = chunks[blockIdx.x];
  const Decision d = dec[C.slot];
  if (d.cut < 0) return;
  Bounds nb;
  slot_bounds(sb, C.slot, nb);
  const Axes x = axes_of(nb.v + 6, nb.v + 9);
  uint32_t ni;
  const uint32_t bits = chunk_flags(C, idx, pd, x, d, ni);
  uint32_t tot;
  const uint32_t lbase = block_exclusive_scan(__popc(bits), red, tot);
  const uint32_t rbase = threadIdx.x * kPer - lbase;   // positions before this thread's, minus their lefts
  const uint32_t p0 = C.b + threadIdx.x * kPer;
  uint32_t nl = 0, nr = 0;
  for (uint32_t j = 0; j < ni; j++) {
    const uint32_t id = idx[p0 + j];
    if (bits >> j & 1u) tmp[C.node_s + off_l[blockIdx.x] + lbase + nl++] = id;
    else tmp[C.node_s + d.nl + off_r[blockIdx.x] + rbase + nr++] = id;
  }
}

__global__ void copy_range_kernel(const Chunk* __restrict__ chunks, const uint32_t* __restrict__ src,
                                  uint32_t* __restrict__ dst, const Decision* __restrict__ dec) {
  const Chunk C = chunks[blockIdx.x];
  if (dec[C.slot].cut < 0) return;
  for (uint32_t p = C.b + threadIdx.x; p < C.e; p += blockDim.x) dst[p] = src[p];
}

// median of a large node: keys over its range padded to a power of two, sorted bitonically
__global__ void median_keys_kernel(const uint32_t* __restrict__ idx, const float4* __restrict__ pd, uint32_t s,
                                   uint32_t n, uint32_t np, int axis, unsigned long long* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  keys[i] = i < n ? median_key(pd, idx[s + i], axis) : 0xFFFFFFFFFFFFFFFFull;
}
__global__ void bitonic_step_kernel(unsigned long long* __restrict__ keys, uint32_t np, uint32_t j, uint32_t k) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const uint32_t l = i ^ j;
  if (l <= i) return;
  const unsigned long long a = keys[i], b = keys[l];
  if ((a > b) == ((i & k) == 0)) {
    keys[i] = b;
    keys[l] = a;
  }
}
__global__ void median_write_kernel(const unsigned long long* __restrict__ keys, uint32_t s, uint32_t n,
                                    uint32_t* __restrict__ idx) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) idx[s + i] = (uint32_t)(keys[i] & 0xFFFFFFFFull);
}

// ---------------------------------------------------------------- small nodes
struct Task {
  uint32_t s, e, depth, id;
};

// One block builds the subtree of one node of at most kSmall primitives.
__global__ void __launch_bounds__(kThreads) small_kernel(const Task* __restrict__ tasks, uint32_t* __restrict__ idx_g,
                                                         const float4* __restrict__ pd, float* __restrict__ nd_box,
                                                         uint32_t* __restrict__ nd_ab, uint32_t* __restrict__ counter,
                                                         uint32_t cap, uint32_t* __restrict__ err) {
  __shared__ uint32_t ids[kSmall];
  __shared__ uint32_t tmp[kSmall];
  __shared__ uint32_t bins[3 * kBins * kBinWords];
  __shared__ float red[8 * 12];
  __shared__ uint32_t sred[32];
  __shared__ Task stack[kStack];
  __shared__ Task cur;
  __shared__ int top;
  __shared__ Cut cuts[3];
  __shared__ Decision dec;
  __shared__ int stop;

  const Task T0 = tasks[blockIdx.x];
  const uint32_t s0 = T0.s, n0 = T0.e - T0.s;
  for (uint32_t i = threadIdx.x; i < n0; i += blockDim.x) ids[i] = idx_g[s0 + i];
  if (threadIdx.x == 0) {
    cur = Task{0u, n0, T0.depth, T0.id};
    top = 0;
    stop = 0;
  }
  __syncthreads();
  while (true) {
    const Task N = cur;
    const uint32_t n = N.e - N.s;
    // bounds of the node's primitives
    Bounds b;
    b.clear();
    for (uint32_t p = N.s + threadIdx.x; p < N.e; p += blockDim.x) b.grow(load_prim(pd, ids[p]));
    const Bounds nb = block_bounds(b, red);
    if (threadIdx.x == 0)
      for (int k = 0; k < 6; k++) nd_box[6 * (size_t)N.id + k] = nb.v[k];
    bool leaf = n <= kLeafMax;
    if (leaf) {
      if (threadIdx.x == 0) {
        nd_ab[2 * (size_t)N.id] = kLeafBit | (s0 + N.s);
        nd_ab[2 * (size_t)N.id + 1] = n;
      }
    } else {
      const Axes x = axes_of(nb.v + 6, nb.v + 9);
      const bool sah = N.depth < kMedianDepth && (x.valid[0] || x.valid[1] || x.valid[2]);
      if (sah) {
        clear_bins(bins, kBins * kBinWords);
        __syncthreads();
        for (uint32_t p = N.s + threadIdx.x; p < N.e; p += blockDim.x) bin_prim(bins, x, load_prim(pd, ids[p]));
        __syncthreads();
      }
      const int warp = threadIdx.x >> 5;
      if (warp < 3) {
        Cut c{FLT_MAX, 0x7FFFFFFF, 0u};
        if (sah && x.valid[warp]) c = sweep_axis(bins + warp * kBins * kBinWords, n);
        if ((threadIdx.x & 31) == 0) cuts[warp] = c;
      }
      __syncthreads();
      if (threadIdx.x == 0) dec = decide(cuts, nb, n, N.depth);
      __syncthreads();
      const Decision d = dec;
      // new order of [N.s, N.e) into tmp: SAH flags stably, or the median sort
      const uint32_t per = (n + blockDim.x - 1) / blockDim.x;   // <= kSmall / kThreads = 8
      const uint32_t p0 = N.s + threadIdx.x * per;
      const uint32_t p1 = min(p0 + per, N.e);
      if (d.cut >= 0) {
        uint32_t bits = 0, cl = 0;
        for (uint32_t p = p0; p < p1; p++) {
          const PrimBox q = load_prim(pd, ids[p]);
          if (bin_of(q.c[d.axis], x.lo[d.axis], x.scale[d.axis]) <= d.cut) {
            bits |= 1u << (p - p0);
            cl++;
          }
        }
        uint32_t tot;
        const uint32_t lb = block_exclusive_scan(cl, sred, tot);
        if (threadIdx.x == 0 && tot != d.nl) atomicOr(err, 1u);
        const uint32_t rb = (p0 > N.e ? n : p0 - N.s) - lb;
        uint32_t nl = 0, nr = 0;
        for (uint32_t p = p0; p < p1; p++) {
          if (bits >> (p - p0) & 1u) tmp[N.s + lb + nl++] = ids[p];
          else tmp[N.s + tot + rb + nr++] = ids[p];
        }
      } else {
        // rank of each primitive under the median order (ranks are distinct:
        // tessellation indices are); the centres on the axis staged in the
        // bins' shared memory (2688 words >= kSmall)
        for (uint32_t p = N.s + threadIdx.x; p < N.e; p += blockDim.x)
          bins[p - N.s] = (uint32_t)(median_key(pd, ids[p], d.axis) >> 32);
        __syncthreads();
        for (uint32_t p = N.s + threadIdx.x; p < N.e; p += blockDim.x) {
          const unsigned long long kp = ((unsigned long long)bins[p - N.s] << 32) | ids[p];
          uint32_t rank = 0;
          for (uint32_t q = N.s; q < N.e; q++)
            rank += (((unsigned long long)bins[q - N.s] << 32) | ids[q]) < kp ? 1u : 0u;
          tmp[N.s + rank] = ids[p];
        }
      }
      __syncthreads();
      for (uint32_t p = N.s + threadIdx.x; p < N.e; p += blockDim.x) ids[p] = tmp[p];
      if (threadIdx.x == 0) {
        const uint32_t l = atomicAdd(counter, 2u);
        if (l + 2u > cap || top >= kStack) {
          atomicOr(err, 2u);
          stop = 1;
        } else {
          nd_ab[2 * (size_t)N.id] = l;
          nd_ab[2 * (size_t)N.id + 1] = l + 1u;
          stack[top++] = Task{N.s + d.nl, N.e, N.depth + 1u, l + 1u};
          cur = Task{N.s, N.s + d.nl, N.depth + 1u, l};
        }
      }
      __syncthreads();
      if (stop) break;
      continue;
    }
    // a leaf: the next pending right child
    __syncthreads();
    if (threadIdx.x == 0) {
      if (top > 0) cur = stack[--top];
      else stop = 1;
    }
    __syncthreads();
    if (stop) break;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n0; i += blockDim.x) idx_g[s0 + i] = ids[i];
}

template <class T>
struct Buf {
  T* p = nullptr;
  ~Buf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
  }
  cudaError_t alloc(size_t n) {
    release();
    return cudaMalloc(&p, (n ? n : 1) * sizeof(T));
  }
};

#define SAH3_CK(x)                    \
  do {                                \
    cudaError_t e_ = (x);             \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

uint32_t pow2_at_least(uint32_t v) {
  uint32_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

}  // namespace

cudaError_t sah3_build_device(const float4* prims, uint32_t n, std::vector<float>& ref_boxes,
                              std::vector<uint32_t>& ref_ab, std::vector<uint32_t>& perm, cudaStream_t st) {
  ref_boxes.clear();
  ref_ab.clear();
  perm.clear();
  if (n == 0) return cudaSuccess;
  const uint32_t cap = 2 * n;   // nodes of a binary tree with n non-empty leaves: at most 2n - 1
  Buf<float4> pd;
  Buf<uint32_t> idx, tmp, nd_ab, counter, err;
  Buf<float> nd_box;
  SAH3_CK(pd.alloc(3 * (size_t)n));
  SAH3_CK(idx.alloc(n));
  SAH3_CK(tmp.alloc(n));
  SAH3_CK(nd_ab.alloc(2 * (size_t)cap));
  SAH3_CK(nd_box.alloc(6 * (size_t)cap));
  SAH3_CK(counter.alloc(1));
  SAH3_CK(err.alloc(1));
  SAH3_CK(cudaMemsetAsync(err.p, 0, 4, st));
  prim_data_kernel<<<(n + 255) / 256, 256, 0, st>>>(prims, n, pd.p, idx.p);
  SAH3_CK(cudaGetLastError());

  // node 0 is the root; ids are handed out two at a time (left, right)
  uint32_t next_id = 1;
  std::vector<Slot> active;
  std::vector<Task> small;
  std::vector<uint32_t> ab_large;   // (id, left) pairs of the large phase
  if (n > kSmall) active.push_back(Slot{0u, 0u, n, 0u});
  else small.push_back(Task{0u, n, 0u, 0u});

  Buf<uint32_t> sb, gbins, first_chunk, chunk_left, off_l, off_r;
  Buf<Chunk> d_chunks;
  Buf<Slot> d_slots;
  Buf<Decision> d_dec;
  Buf<unsigned long long> keys;
  size_t slot_cap = 0, chunk_cap = 0, key_cap = 0;
  std::vector<Chunk> chunks;
  std::vector<uint32_t> fc;
  std::vector<Decision> dec;
  while (!active.empty()) {
    const uint32_t ns = (uint32_t)active.size();
    chunks.clear();
    fc.assign(1, 0u);
    for (uint32_t si = 0; si < ns; si++) {
      const Slot& S = active[si];
      for (uint32_t b = S.s; b < S.e; b += kChunk) chunks.push_back(Chunk{si, b, std::min(b + kChunk, S.e), S.s});
      fc.push_back((uint32_t)chunks.size());
    }
    const uint32_t nc = (uint32_t)chunks.size();
    if (ns > slot_cap) {
      slot_cap = std::max<size_t>(ns, 2 * slot_cap);
      SAH3_CK(cudaStreamSynchronize(st));
      SAH3_CK(d_slots.alloc(slot_cap));
      SAH3_CK(d_dec.alloc(slot_cap));
      SAH3_CK(sb.alloc(12 * slot_cap));
      SAH3_CK(gbins.alloc(slot_cap * 3 * kBins * kBinWords));
      SAH3_CK(first_chunk.alloc(slot_cap + 1));
    }
    if (nc > chunk_cap) {
      chunk_cap = std::max<size_t>(nc, 2 * chunk_cap);
      SAH3_CK(cudaStreamSynchronize(st));
      SAH3_CK(d_chunks.alloc(chunk_cap));
      SAH3_CK(chunk_left.alloc(chunk_cap));
      SAH3_CK(off_l.alloc(chunk_cap));
      SAH3_CK(off_r.alloc(chunk_cap));
    }
    SAH3_CK(cudaMemcpyAsync(d_slots.p, active.data(), ns * sizeof(Slot), cudaMemcpyHostToDevice, st));
    SAH3_CK(cudaMemcpyAsync(d_chunks.p, chunks.data(), nc * sizeof(Chunk), cudaMemcpyHostToDevice, st));
    SAH3_CK(cudaMemcpyAsync(first_chunk.p, fc.data(), fc.size() * 4, cudaMemcpyHostToDevice, st));
    const uint32_t init_n = ns * 3 * kBins * kBinWords;
    init_slots_kernel<<<(init_n + 255) / 256, 256, 0, st>>>(sb.p, gbins.p, ns);
    large_bounds_kernel<<<nc, kThreads, 0, st>>>(d_chunks.p, idx.p, pd.p, sb.p);
    large_bin_kernel<<<nc, kThreads, 0, st>>>(d_chunks.p, idx.p, pd.p, sb.p, gbins.p);
    large_sweep_kernel<<<ns, 96, 0, st>>>(d_slots.p, sb.p, gbins.p, d_dec.p, nd_box.p);
    large_count_kernel<<<nc, kThreads, 0, st>>>(d_chunks.p, idx.p, pd.p, sb.p, d_dec.p, chunk_left.p);
    large_offsets_kernel<<<(ns + 127) / 128, 128, 0, st>>>(first_chunk.p, ns, d_chunks.p, chunk_left.p, d_dec.p,
                                                           off_l.p, off_r.p, err.p);
    large_scatter_kernel<<<nc, kThreads, 0, st>>>(d_chunks.p, idx.p, pd.p, sb.p, d_dec.p, off_l.p, off_r.p, tmp.p);
    copy_range_kernel<<<nc, kThreads, 0, st>>>(d_chunks.p, tmp.p, idx.p, d_dec.p);
    SAH3_CK(cudaGetLastError());
    dec.resize(ns);
    SAH3_CK(cudaMemcpyAsync(dec.data(), d_dec.p, ns * sizeof(Decision), cudaMemcpyDeviceToHost, st));
    SAH3_CK(cudaStreamSynchronize(st));
    // median splits of large nodes (degenerate inputs only): sort the range
    for (uint32_t si = 0; si < ns; si++) {
      if (dec[si].cut >= 0) continue;
      const Slot& S = active[si];
      const uint32_t m = S.e - S.s, np = pow2_at_least(m);
      if (np > key_cap) {
        SAH3_CK(cudaStreamSynchronize(st));
        key_cap = np;
        SAH3_CK(keys.alloc(key_cap));
      }
      median_keys_kernel<<<(np + 255) / 256, 256, 0, st>>>(idx.p, pd.p, S.s, m, np, dec[si].axis, keys.p);
      for (uint32_t k = 2; k <= np; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) bitonic_step_kernel<<<(np + 255) / 256, 256, 0, st>>>(keys.p, np, j, k);
      median_write_kernel<<<(m + 255) / 256, 256, 0, st>>>(keys.p, S.s, m, idx.p);
      SAH3_CK(cudaGetLastError());
    }
    std::vector<Slot> next;
    for (uint32_t si = 0; si < ns; si++) {
      const Slot& S = active[si];
      const uint32_t mid = S.s + dec[si].nl;
      const uint32_t l = next_id, r = next_id + 1;
      next_id += 2;
      ab_large.push_back(S.id);
      ab_large.push_back(l);
      const Slot kids[2] = {Slot{l, S.s, mid, S.depth + 1}, Slot{r, mid, S.e, S.depth + 1}};
      for (const Slot& K : kids) {
        if (K.e - K.s > kSmall) next.push_back(K);
        else small.push_back(Task{K.s, K.e, K.depth, K.id});
      }
    }
    active.swap(next);
  }
  // links of the large nodes (ids below next_id; the entries of the ids
  // that went to the small phase are written again by small_kernel)
  std::vector<uint32_t> h(2 * (size_t)next_id, 0u);
  for (size_t k = 0; k < ab_large.size(); k += 2) {
    h[2 * ab_large[k]] = ab_large[k + 1];
    h[2 * ab_large[k] + 1] = ab_large[k + 1] + 1u;
  }
  SAH3_CK(cudaMemcpyAsync(nd_ab.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice, st));
  SAH3_CK(cudaMemcpyAsync(counter.p, &next_id, 4, cudaMemcpyHostToDevice, st));
  Buf<Task> d_tasks;
  SAH3_CK(d_tasks.alloc(small.size()));
  SAH3_CK(cudaMemcpyAsync(d_tasks.p, small.data(), small.size() * sizeof(Task), cudaMemcpyHostToDevice, st));
  small_kernel<<<(uint32_t)small.size(), kThreads, 0, st>>>(d_tasks.p, idx.p, pd.p, nd_box.p, nd_ab.p, counter.p,
                                                           cap, err.p);
  SAH3_CK(cudaGetLastError());
  uint32_t total = 0, herr = 0;
  SAH3_CK(cudaMemcpyAsync(&total, counter.p, 4, cudaMemcpyDeviceToHost, st));
  SAH3_CK(cudaMemcpyAsync(&herr, err.p, 4, cudaMemcpyDeviceToHost, st));
  SAH3_CK(cudaStreamSynchronize(st));
  if (herr || total > cap) return cudaErrorInvalidValue;
  std::vector<float> box(6 * (size_t)total);
  std::vector<uint32_t> ab(2 * (size_t)total);
  perm.resize(n);
  SAH3_CK(cudaMemcpyAsync(box.data(), nd_box.p, box.size() * 4, cudaMemcpyDeviceToHost, st));
  SAH3_CK(cudaMemcpyAsync(ab.data(), nd_ab.p, ab.size() * 4, cudaMemcpyDeviceToHost, st));
  SAH3_CK(cudaMemcpyAsync(perm.data(), idx.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  SAH3_CK(cudaStreamSynchronize(st));
  // the host builder's numbering: preorder, left subtree first
  std::vector<uint32_t> order;
  order.reserve(total);
  std::vector<uint32_t> newid(total, 0xFFFFFFFFu);
  std::vector<uint32_t> stk{0u};
  while (!stk.empty()) {
    const uint32_t i = stk.back();
    stk.pop_back();
    if (i >= total || newid[i] != 0xFFFFFFFFu) return cudaErrorInvalidValue;
    newid[i] = (uint32_t)order.size();
    order.push_back(i);
    if (!(ab[2 * (size_t)i] & kLeafBit)) {
      stk.push_back(ab[2 * (size_t)i + 1]);
      stk.push_back(ab[2 * (size_t)i]);
    }
  }
  if (order.size() != total) return cudaErrorInvalidValue;
  ref_boxes.resize(6 * (size_t)total);
  ref_ab.resize(2 * (size_t)total);
  for (uint32_t k = 0; k < total; k++) {
    const uint32_t i = order[k];
    std::memcpy(&ref_boxes[6 * (size_t)k], &box[6 * (size_t)i], 24);
    const uint32_t a = ab[2 * (size_t)i], b = ab[2 * (size_t)i + 1];
    if (a & kLeafBit) {
      ref_ab[2 * (size_t)k] = a;
      ref_ab[2 * (size_t)k + 1] = b;
    } else {
      ref_ab[2 * (size_t)k] = newid[a];
      ref_ab[2 * (size_t)k + 1] = newid[b];
    }
  }
  return cudaSuccess;
}

}  // namespace omg
