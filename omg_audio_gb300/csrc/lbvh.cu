// LBVH build on the GPU (Karras 2012, "Maximizing parallelism in the
// construction of BVHs, octrees, and k-d trees"):
//   1. centroid bounds (ordered-integer atomics),
//   2. 30-bit Morton code per primitive centroid, key = code << 32 | index
//      (unique keys, so the sort needs no stability),
//   3. bitonic sort of the padded key array,
//   4. hierarchy: internal node i covers a key range found by prefix lengths,
//   5. bottom-up refit with one atomic arrival counter per node,
//   6. write the child-box BVH2 records the tracer walks; subtrees of <= 4
//      primitives become leaves (ranges are contiguous in sorted order).
#include <cfloat>

#include "omg_internal.h"

namespace omg {

namespace {

constexpr uint32_t kCollapse = 4;  // leaf size, as the reference's LEAF_SIZE (mesh.rs:16)

__device__ __forceinline__ uint32_t f2o(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t o) {
  uint32_t b = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
  return __uint_as_float(b);
}

__device__ __forceinline__ void prim_bounds(const float4* prims, uint32_t i, float lo[3], float hi[3]) {
  const float4 p0 = prims[3 * i], p1 = prims[3 * i + 1], p2 = prims[3 * i + 2];
  const float a[3] = {p0.x, p0.y, p0.z};
  const float b[3] = {p0.x + p1.x, p0.y + p1.y, p0.z + p1.z};
  const float c[3] = {p0.x + p2.x, p0.y + p2.y, p0.z + p2.z};
  for (int k = 0; k < 3; k++) {
    lo[k] = fminf(fminf(a[k], b[k]), c[k]);
    hi[k] = fmaxf(fmaxf(a[k], b[k]), c[k]);
  }
}

__device__ __forceinline__ void centroid(const float4* prims, uint32_t i, float c[3]) {
  const float4 p0 = prims[3 * i], p1 = prims[3 * i + 1], p2 = prims[3 * i + 2];
  c[0] = p0.x + (p1.x + p2.x) * (1.0f / 3.0f);
  c[1] = p0.y + (p1.y + p2.y) * (1.0f / 3.0f);
  c[2] = p0.z + (p1.z + p2.z) * (1.0f / 3.0f);
}

__global__ void bounds_kernel(const float4* __restrict__ prims, uint32_t n, uint32_t* __restrict__ cb) {
  __shared__ uint32_t s[6];
  if (threadIdx.x < 6) s[threadIdx.x] = threadIdx.x < 3 ? 0xFFFFFFFFu : 0u;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float c[3];
    centroid(prims, i, c);
    for (int k = 0; k < 3; k++) {
      atomicMin(&s[k], f2o(c[k]));
      atomicMax(&s[3 + k], f2o(c[k]));
    }
  }
  __syncthreads();
  if (threadIdx.x < 3) atomicMin(&cb[threadIdx.x], s[threadIdx.x]);
  else if (threadIdx.x < 6) atomicMax(&cb[threadIdx.x], s[threadIdx.x]);
}

__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v &= 0x3FFu;
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void morton_kernel(const float4* __restrict__ prims, uint32_t n, uint32_t n_pad,
                              const uint32_t* __restrict__ cb, unsigned long long* __restrict__ keys) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  if (i >= n) {
    keys[i] = 0xFFFFFFFFFFFFFFFFull;
    return;
  }
  float c[3];
  centroid(prims, i, c);
  uint32_t q[3];
  for (int k = 0; k < 3; k++) {
    float lo = o2f(cb[k]), hi = o2f(cb[3 + k]);
    float ext = hi - lo;
    float u = ext > 0.0f ? (c[k] - lo) / ext : 0.0f;
    float s = fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
    q[k] = (uint32_t)s;
  }
  uint32_t code = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
  keys[i] = ((unsigned long long)code << 32) | i;
}

// one compare-exchange stage of the bitonic network
__global__ void bitonic_kernel(unsigned long long* __restrict__ keys, uint32_t n_pad, uint32_t j, uint32_t k) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  uint32_t l = i ^ j;
  if (l <= i) return;
  unsigned long long a = keys[i], b = keys[l];
  bool up = (i & k) == 0;
  if ((a > b) == up) {
    keys[i] = b;
    keys[l] = a;
  }
}

// sort a block-sized run entirely in shared memory (all stages with j < 1024)
__global__ void bitonic_local_kernel(unsigned long long* __restrict__ keys, uint32_t n_pad, uint32_t k_start,
                                     uint32_t k_end) {
  __shared__ unsigned long long s[2048];
  const uint32_t base = blockIdx.x * 2048;
  for (uint32_t t = threadIdx.x; t < 2048; t += blockDim.x) s[t] = keys[base + t];
  __syncthreads();
  for (uint32_t k = k_start; k <= k_end; k <<= 1) {
    for (uint32_t j = (k == k_start && k_start > 2048) ? 1024 : (k >> 1); j > 0; j >>= 1) {
      for (uint32_t t = threadIdx.x; t < 2048; t += blockDim.x) {
        uint32_t l = t ^ j;
        if (l > t) {
          unsigned long long a = s[t], b = s[l];
          bool up = ((base + t) & k) == 0;
          if ((a > b) == up) {
            s[t] = b;
            s[l] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t t = threadIdx.x; t < 2048; t += blockDim.x) keys[base + t] = s[t];
}

__device__ __forceinline__ int delta(const unsigned long long* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(keys[i] ^ keys[j]);
}

// Karras 2012, Algorithm 1 (keys are unique)
__global__ void hierarchy_kernel(const unsigned long long* __restrict__ keys, int n, int* __restrict__ left,
                                 int* __restrict__ right, int* __restrict__ parent_int, int* __restrict__ parent_leaf,
                                 int* __restrict__ range_lo, int* __restrict__ range_hi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(keys, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  int gamma = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  range_lo[i] = lo;
  range_hi[i] = hi;
  if (lo == gamma) {
    left[i] = ~gamma;  // leaf gamma
    parent_leaf[gamma] = i;
  } else {
    left[i] = gamma;
    parent_int[gamma] = i;
  }
  if (hi == gamma + 1) {
    right[i] = ~(gamma + 1);
    parent_leaf[gamma + 1] = i;
  } else {
    right[i] = gamma + 1;
    parent_int[gamma + 1] = i;
  }
  if (i == 0) parent_int[0] = -1;
}

__global__ void gather_kernel(const float4* __restrict__ in, const unsigned long long* __restrict__ keys,
                              uint32_t n, float4* __restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t src = (uint32_t)(keys[i] & 0xFFFFFFFFull);
  out[3 * i] = in[3 * src];
  out[3 * i + 1] = in[3 * src + 1];
  out[3 * i + 2] = in[3 * src + 2];
}

// bottom-up boxes: the second thread to arrive at a node computes its box
__global__ void refit_kernel(const float4* __restrict__ prims, int n, const int* __restrict__ left,
                             const int* __restrict__ right, const int* __restrict__ parent_int,
                             const int* __restrict__ parent_leaf, float* __restrict__ boxes,
                             unsigned int* __restrict__ flags, unsigned int* __restrict__ err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int p = parent_leaf[i];
  // keys are 62 bits wide, so no path to the root is longer than 64 nodes
  for (int guard = 0; p >= 0; guard++) {
    if (guard >= 128) {
      atomicOr(err, 1u);
      return;
    }
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0u) return;
    __threadfence();
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    const int ch[2] = {left[p], right[p]};
    for (int c = 0; c < 2; c++) {
      float cl[3], chh[3];
      if (ch[c] < 0) {
        prim_bounds(prims, (uint32_t)~ch[c], cl, chh);
      } else {
        const volatile float* b = boxes + 6 * ch[c];
        for (int k = 0; k < 3; k++) {
          cl[k] = b[k];
          chh[k] = b[3 + k];
        }
      }
      for (int k = 0; k < 3; k++) {
        lo[k] = fminf(lo[k], cl[k]);
        hi[k] = fmaxf(hi[k], chh[k]);
      }
    }
    volatile float* o = boxes + 6 * p;
    for (int k = 0; k < 3; k++) {
      o[k] = lo[k];
      o[3 + k] = hi[k];
    }
    p = parent_int[p];
  }
}

__device__ __forceinline__ int child_ref(int c, const int* range_lo, const int* range_hi) {
  if (c < 0) return ~(((~c) << 3) | 0);             // single-primitive leaf
  int cnt = range_hi[c] - range_lo[c] + 1;
  if (cnt <= (int)kCollapse) return ~((range_lo[c] << 3) | (cnt - 1));
  return c;
}

__global__ void write_nodes_kernel(const float4* __restrict__ prims, int n, const int* __restrict__ left,
                                   const int* __restrict__ right, const int* __restrict__ range_lo,
                                   const int* __restrict__ range_hi, const float* __restrict__ boxes,
                                   float4* __restrict__ nodes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  float b[2][6];
  const int ch[2] = {left[i], right[i]};
  for (int c = 0; c < 2; c++) {
    if (ch[c] < 0) {
      prim_bounds(prims, (uint32_t)~ch[c], &b[c][0], &b[c][3]);
    } else {
      for (int k = 0; k < 6; k++) b[c][k] = boxes[6 * ch[c] + k];
    }
  }
  int r0 = child_ref(ch[0], range_lo, range_hi), r1 = child_ref(ch[1], range_lo, range_hi);
  nodes[4 * i + 0] = make_float4(b[0][0], b[0][1], b[0][2], b[0][3]);
  nodes[4 * i + 1] = make_float4(b[0][4], b[0][5], b[1][0], b[1][1]);
  nodes[4 * i + 2] = make_float4(b[1][2], b[1][3], b[1][4], b[1][5]);
  nodes[4 * i + 3] = make_float4(__int_as_float(r0), __int_as_float(r1), 0.0f, 0.0f);
}

uint32_t next_pow2(uint32_t v) {
  uint32_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

}  // namespace

size_t lbvh_scratch_bytes(uint32_t n) {
  size_t np = next_pow2(n < 2048 ? 2048 : n);
  size_t b = 0;
  b += 64;                       // centroid bounds
  b += np * 8;                   // keys
  b += (size_t)n * 4 * 6;        // left, right, parent_int, parent_leaf, range_lo, range_hi
  b += (size_t)n * 24;           // boxes
  b += (size_t)n * 4;            // flags
  return b + 1024;
}

cudaError_t lbvh_build(const float4* prims_in, uint32_t n, float4* prims_out, float4* nodes_out, int32_t* root_ref,
                       void* scratch, size_t scratch_bytes, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (scratch_bytes < lbvh_scratch_bytes(n)) return cudaErrorInvalidValue;
  uint32_t np = next_pow2(n < 2048 ? 2048 : n);
  char* p = (char*)scratch;
  uint32_t* cb = (uint32_t*)p;
  p += 64;
  unsigned long long* keys = (unsigned long long*)p;
  p += (size_t)np * 8;
  int* left = (int*)p;
  p += (size_t)n * 4;
  int* right = (int*)p;
  p += (size_t)n * 4;
  int* parent_int = (int*)p;
  p += (size_t)n * 4;
  int* parent_leaf = (int*)p;
  p += (size_t)n * 4;
  int* range_lo = (int*)p;
  p += (size_t)n * 4;
  int* range_hi = (int*)p;
  p += (size_t)n * 4;
  float* boxes = (float*)p;
  p += (size_t)n * 24;
  unsigned int* flags = (unsigned int*)p;

  const uint32_t init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u};  // bounds + error word
  cudaError_t e = cudaMemcpyAsync(cb, init, sizeof(init), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  bounds_kernel<<<std::min<uint32_t>((n + 255) / 256, 1024), 256, 0, s>>>(prims_in, n, cb);
  morton_kernel<<<(np + 255) / 256, 256, 0, s>>>(prims_in, n, np, cb, keys);
  // bitonic: stages with j >= 1024 in global memory, the rest per 2048-key tile in shared memory
  bitonic_local_kernel<<<np / 2048, 1024, 0, s>>>(keys, np, 2, 2048);
  for (uint32_t k = 4096; k <= np; k <<= 1) {
    for (uint32_t j = k >> 1; j >= 2048; j >>= 1) bitonic_kernel<<<(np + 255) / 256, 256, 0, s>>>(keys, np, j, k);
    bitonic_local_kernel<<<np / 2048, 1024, 0, s>>>(keys, np, k, k);
  }
  gather_kernel<<<(n + 255) / 256, 256, 0, s>>>(prims_in, keys, n, prims_out);
  if (n == 1) {
    int32_t r = ~0;
    e = cudaMemcpyAsync(root_ref, &r, 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
  }
  hierarchy_kernel<<<(n - 1 + 255) / 256, 256, 0, s>>>(keys, (int)n, left, right, parent_int, parent_leaf, range_lo,
                                                         range_hi);
  e = cudaMemsetAsync(flags, 0, (size_t)n * 4, s);
  if (e != cudaSuccess) return e;
  refit_kernel<<<(n + 255) / 256, 256, 0, s>>>(prims_out, (int)n, left, right, parent_int, parent_leaf, boxes, flags,
                                                 cb + 6);
  write_nodes_kernel<<<(n - 1 + 255) / 256, 256, 0, s>>>(prims_out, (int)n, left, right, range_lo, range_hi, boxes,
                                                          nodes_out);
  // root: internal node 0, or a leaf when the whole tree fits one leaf
  int32_t root = n <= kCollapse ? (int32_t)~((0u << 3) | (n - 1)) : 0;
  e = cudaMemcpyAsync(root_ref, &root, 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return e;
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  uint32_t herr = 0;
  e = cudaMemcpyAsync(&herr, cb + 6, 4, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  return herr ? cudaErrorInvalidValue : cudaSuccess;
}


namespace {
// Child boxes of every binary node grown by 2^-19 m[a] on each side, rounded
// outward (DScene::nodes_f).
__global__ void grow_nodes_kernel(const float4* __restrict__ in, float4* __restrict__ out, uint32_t n, float mx,
                                  float my, float mz, float pad) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float g[3] = {__fadd_ru(ldexpf(mx, -19), pad), __fadd_ru(ldexpf(my, -19), pad), __fadd_ru(ldexpf(mz, -19), pad)};
  float v[16];
  for (int i = 0; i < 4; i++) {
    const float4 q = in[4 * k + i];
    v[4 * i] = q.x; v[4 * i + 1] = q.y; v[4 * i + 2] = q.z; v[4 * i + 3] = q.w;
  }
  for (int c = 0; c < 2; c++)
    for (int a = 0; a < 3; a++) {
      v[6 * c + a] = __fsub_rd(v[6 * c + a], g[a]);
      v[6 * c + 3 + a] = __fadd_ru(v[6 * c + 3 + a], g[a]);
    }
  for (int i = 0; i < 4; i++) out[4 * k + i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
}
}  // namespace

cudaError_t grow_nodes(const float4* nodes, float4* out, uint32_t n_nodes, const float m[3], float pad,
                       cudaStream_t s) {
  if (n_nodes == 0) return cudaSuccess;
  grow_nodes_kernel<<<(n_nodes + 255) / 256, 256, 0, s>>>(nodes, out, n_nodes, m[0], m[1], m[2], pad);
  return cudaGetLastError();
}

}  // namespace omg
