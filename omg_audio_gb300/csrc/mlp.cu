// The surrogate's dense layers on the tensor cores: a tcgen05 GEMM with the
// accumulator in TMEM, fused bias + GELU epilogues, and the elementwise and
// optimizer kernels of training (GELU backward, bias gradients, MSE loss,
// AdamW on FP32 master weights with BF16 copies).
//
// GEMM: D[M x N] = A[M x K] . B[N x K]^T with A, B in BF16 and FP32
// accumulation. Operands are read through strides, so transposed operands of
// the backward pass need no copies: element (m, k) of A is A[m a_rs + k a_ks].
// One CTA of 128 threads computes a 128 x n_tile tile (n_tile <= 256): each
// round stages a 64-wide K chunk of both operands into shared memory (K-major
// core matrices, tc_gemm.cuh), one thread issues four K = 16 MMAs and commits
// them to an mbarrier, and the CTA waits (bounded) before the next round. The
// epilogue reads the accumulator lanes of each warp with tcgen05.ld. A grid z
// dimension splits K; the split partials are added atomically.
#include <algorithm>

#include <cuda_bf16.h>

#include "omg_internal.h"
#include "tc_gemm.cuh"

namespace omg {

namespace {

constexpr uint32_t kTileM = 128;
constexpr uint32_t kMaxTileN = 256;
constexpr uint32_t kPolls = 1u << 24;   // mbarrier poll limit (error 16 in the error word)

__device__ __forceinline__ float gelu_f(float z) {
  // tanh form of GELU
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (z + k1 * z * z * z);
  return 0.5f * z * (1.0f + tanhf(u));
}

__device__ __forceinline__ float gelu_grad(float z) {
  const float k0 = 0.7978845608028654f, k1 = 0.044715f;
  const float u = k0 * (z + k1 * z * z * z);
  const float t = tanhf(u);
  const float du = k0 * (1.0f + 3.0f * k1 * z * z);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * du;
}

// Stage rows [r0, r0 + rows) x K [k0, k0 + 64) of an operand into a tile.
__device__ __forceinline__ void stage(uint8_t* tile, const __nv_bfloat16* __restrict__ X, int64_t rs, int64_t ks,
                                      uint32_t r0, uint32_t rows, uint32_t R, uint32_t k0, uint32_t K) {
  const uint32_t pieces = rows * 8u;  // 16-byte pieces: (row, k8)
  for (uint32_t p = threadIdx.x; p < pieces; p += blockDim.x) {
    // consecutive threads take consecutive rows of the same k8 (coalesced when ks != 1)
    const uint32_t r = p % rows, k8 = p / rows;
    const uint32_t gr = r0 + r, gk = k0 + 8u * k8;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (gr < R) {
      const __nv_bfloat16* src = X + (int64_t)gr * rs + (int64_t)gk * ks;
      if (ks == 1 && gk + 8u <= K && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0u)) {
        v = *reinterpret_cast<const uint4*>(src);
      } else {
        uint16_t h[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          h[j] = 0;
          if (gk + (uint32_t)j < K) h[j] = __bfloat16_as_ushort(src[(int64_t)j * ks]);
        }
        v.x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
        v.y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
        v.z = (uint32_t)h[4] | ((uint32_t)h[5] << 16);
        v.w = (uint32_t)h[6] | ((uint32_t)h[7] << 16);
      }
    }
    *reinterpret_cast<uint4*>(tile + tc::tile_offset(r, 8u * k8)) = v;
  }
}

// Asynchronous staging of rows [r0, r0 + rows) x K [k0, k0 + 64) of a K-major
// operand (element (r, k) at X[r rs + k], rs a multiple of 8, X 16-byte
// aligned, K a multiple of 8): one 16-byte cp.async per (row, k8) piece,
// zero-filled beyond R rows or K.
__device__ __forceinline__ void stage_async(uint8_t* tile, const __nv_bfloat16* __restrict__ X, int64_t rs,
                                            uint32_t r0, uint32_t rows, uint32_t R, uint32_t k0, uint32_t K) {
  const uint32_t pieces = rows * 8u;
  for (uint32_t p = threadIdx.x; p < pieces; p += blockDim.x) {
    // 8 consecutive threads take the same k8 of 8 consecutive rows (their 128
    // bytes of shared memory are contiguous: no bank conflict); a warp reads 64
    // contiguous bytes of each of its 8 rows
    const uint32_t r = ((p >> 6) << 3) | (p & 7u), k8 = (p >> 3) & 7u;
    const uint32_t gr = r0 + r, gk = k0 + 8u * k8;
    const bool in = gr < R && gk < K;
    const __nv_bfloat16* src = in ? X + (int64_t)gr * rs + gk : X;
    tc::cp_async16(tile + tc::tile_offset(r, 8u * k8), src, in ? 16u : 0u);
  }
}

constexpr uint32_t kStages = 3;   // cp.async pipeline depth

// The epilogue: TMEM -> bias, optional GELU, the requested outputs. The
// accumulator comes out of TMEM one row per thread (tcgen05.ld 32x32b); the
// transposed activation Yt is written from that layout (consecutive lanes,
// consecutive rows: coalesced). For the row-major outputs D, Z and Y each warp
// stages 32 x 32 blocks in shared memory (the operand stages, free once the
// last MMA has completed) and writes them row by row with consecutive lanes on
// consecutive columns: whole 128-byte lines instead of one sector per element.
__device__ __forceinline__ void gemm_epilogue(const GemmArgs& g, uint8_t* smem, uint32_t taddr, uint32_t m0,
                                              uint32_t n0, uint32_t nt, uint32_t nt16) {
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  __nv_bfloat16* gY = static_cast<__nv_bfloat16*>(g.Y);
  __nv_bfloat16* gYt = static_cast<__nv_bfloat16*>(g.Yt);
  const bool rowwise = g.D || g.Z || gY;
  float* st = reinterpret_cast<float*>(smem) + warp * (32u * 33u);
  const uint32_t trow = m0 + warp * 32u + lane;          // this thread's TMEM row
  const uint32_t lane_addr = taddr + ((warp * 32u) << 16);
  for (uint32_t c = 0; c < nt16; c += 32u) {
    const uint32_t w = min(32u, nt16 - c);               // 16 or 32 columns
    float v[32];
    {
      float a[16], b[16];
      tc::tmem_ld16(lane_addr + c, a);
      if (w == 32u) tc::tmem_ld16(lane_addr + c + 16u, b);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        v[j] = a[j];
        v[16 + j] = w == 32u ? b[j] : 0.0f;
      }
    }
#pragma unroll
    for (uint32_t j = 0; j < 32u; j++) {
      if (j >= w) break;
      const uint32_t col = n0 + c + j;
      const bool ok = c + j < nt;
      float z = v[j];
      if (g.bias && ok) z += g.bias[col];
      if (gYt && ok && trow < g.M) gYt[(int64_t)col * g.ldyt + trow] = __float2bfloat16_rn(g.act ? gelu_f(z) : z);
      st[lane * 33u + j] = z;
    }
    __syncwarp();
    if (rowwise) {
      const uint32_t col = n0 + c + lane;
      const bool ok = lane < w && c + lane < nt;
      for (uint32_t r = 0; r < 32u; r++) {
        const uint32_t row = m0 + warp * 32u + r;
        if (row >= g.M) break;
        if (!ok) continue;
        const float z = st[r * 33u + lane];
        if (g.D) {
          float* d = g.D + (int64_t)row * g.ldd + col;
          if (g.accumulate) atomicAdd(d, z);
          else *d = z;
        }
        if (g.Z) g.Z[(int64_t)row * g.ldz + col] = z;
        if (gY) gY[(int64_t)row * g.ldy + col] = __float2bfloat16_rn(g.act ? gelu_f(z) : z);
      }
    }
    __syncwarp();
  }
}

// D = A . B^T on a 128 x n_tile tile. ASYNC: both operands K-major and
// 16-byte aligned, staged by a kStages-deep cp.async pipeline (the copies of
// the next chunks run under the MMAs of the current one); otherwise each
// 64-wide K chunk is staged by plain loads, then multiplied.
template <bool ASYNC>
__global__ void __launch_bounds__(128, 1) gemm_kernel(GemmArgs g) {
  const __nv_bfloat16* __restrict__ gA = static_cast<const __nv_bfloat16*>(g.A);
  const __nv_bfloat16* __restrict__ gB = static_cast<const __nv_bfloat16*>(g.B);
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar[kStages];
  __shared__ uint32_t taddr_s;
  __shared__ uint32_t failed;
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t m0 = blockIdx.x * kTileM;
  const uint32_t n0 = blockIdx.y * g.n_tile;
  const uint32_t nt = min(g.n_tile, g.N - n0);          // columns of this tile
  const uint32_t nt16 = (nt + 15u) & ~15u;              // MMA N (multiple of 16)
  const uint32_t stage_bytes = (kTileM + g.n_tile) * tc::kChunkK * 2u;
  // this CTA's K range
  const uint32_t k_per = ((g.K + gridDim.z - 1) / gridDim.z + tc::kChunkK - 1) / tc::kChunkK * tc::kChunkK;
  const uint32_t kb = blockIdx.z * k_per;
  const uint32_t ke = min(g.K, kb + k_per);
  const uint32_t nk = ke > kb ? (ke - kb + tc::kChunkK - 1) / tc::kChunkK : 0u;
  if (threadIdx.x == 0) {
    for (uint32_t i = 0; i < kStages; i++) tc::mbar_init(&mbar[i], 1);
    failed = 0;
  }
  if (warp == 0) tc::tmem_alloc(&taddr_s, kMaxTileN);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = taddr_s;
  const uint32_t idesc = tc::idesc_bf16_f32(nt16, kTileM);
  uint32_t phase_bits = 0;   // bit b: the parity of buffer b's next completion
  uint32_t issued = 0;       // chunks whose MMAs have been issued (the same count in every thread)
  auto issue = [&](uint32_t buf, bool acc0) {
    uint8_t* sa = smem + buf * stage_bytes;
    uint8_t* sb = sa + kTileM * tc::kChunkK * 2u;
    tc::fence_after_sync();
    const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
    for (uint32_t s = 0; s < tc::kChunkK / 16u; s++)
      tc::mma_bf16(taddr, tc::smem_desc(a0 + 256u * s), tc::smem_desc(b0 + 256u * s), idesc, acc0 || s > 0);
    tc::mma_commit(&mbar[buf]);
  };
  auto wait_buf = [&](uint32_t buf) {
    if (!tc::mbar_wait(&mbar[buf], (phase_bits >> buf) & 1u, kPolls)) failed = 1;
    phase_bits ^= 1u << buf;
  };
  if (ASYNC) {
    auto load = [&](uint32_t chunk) {
      uint8_t* sa = smem + (chunk % kStages) * stage_bytes;
      uint8_t* sb = sa + kTileM * tc::kChunkK * 2u;
      const uint32_t k0 = kb + chunk * tc::kChunkK;
      stage_async(sa, gA, g.a_rs, m0, kTileM, g.M, k0, ke);
      stage_async(sb, gB, g.b_rs, n0, nt16, n0 + nt, k0, ke);
    };
    for (uint32_t c = 0; c + 1 < kStages; c++) {
      if (c < nk) load(c);
      tc::cp_async_commit();
    }
    for (uint32_t i = 0; i < nk; i++) {
      tc::cp_async_wait<kStages - 2>();     // chunk i has landed (this thread's copies)
      tc::fence_proxy_async();
      __syncthreads();                      // ... and every thread's
      if (threadIdx.x == 0) issue(i % kStages, i > 0);
      issued = i + 1;
      const uint32_t j = i + kStages - 1;   // refill the buffer chunk i - 1 used
      if (j < nk) {
        if (i >= 1) wait_buf((i - 1) % kStages);
        __syncthreads();
        if (failed) break;
        load(j);
      }
      tc::cp_async_commit();
    }
    tc::cp_async_wait_all();
  } else {
    uint8_t* sa = smem;
    uint8_t* sb = smem + kTileM * tc::kChunkK * 2u;
    for (uint32_t i = 0; i < nk; i++) {
      const uint32_t k0 = kb + i * tc::kChunkK;
      stage(sa, gA, g.a_rs, g.a_ks, m0, kTileM, g.M, k0, ke);
      stage(sb, gB, g.b_rs, g.b_ks, n0, nt16, n0 + nt, k0, ke);
      tc::fence_proxy_async();
      __syncthreads();
      if (threadIdx.x == 0) issue(0, i > 0);
      issued = i + 1;
      // the tiles are read asynchronously: wait before restaging them
      wait_buf(0);
      __syncthreads();
      if (failed) break;
    }
  }
  // the last chunk's MMAs (and with them, in order, every earlier one)
  if (ASYNC && !failed && nk > 0) wait_buf((nk - 1) % kStages);
  __syncthreads();
  tc::fence_after_sync();
  if (!failed && nk > 0) {
    gemm_epilogue(g, smem, taddr, m0, n0, nt, nt16);
  } else if (failed) {
    // give the last MMAs issued one more bounded wait before the TMEM is freed
    // (the slow path's only buffer was waited on already)
    if (ASYNC && issued > 0) {
      const uint32_t b = (issued - 1) % kStages;
      tc::mbar_wait(&mbar[b], (phase_bits >> b) & 1u, kPolls);
    }
    if (threadIdx.x == 0 && g.err) atomicOr(g.err, 16u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, kMaxTileN);
}

// dZ = dA * GELU'(Z) (f32 in, bf16 and f32 out)
__global__ void gelu_back_kernel(const float* __restrict__ dA, const float* __restrict__ Z, float* __restrict__ dZ,
                                 __nv_bfloat16* __restrict__ dZh, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float d = dA[i] * gelu_grad(Z[i]);
    dZ[i] = d;
    dZh[i] = __float2bfloat16_rn(d);
  }
}

// column sums of X [rows x cols] (bias gradients); one thread per column
__global__ void colsum_kernel(const float* __restrict__ X, uint32_t rows, uint32_t cols, float* __restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.0f;
  for (uint32_t r = 0; r < rows; r++) s += X[(uint64_t)r * cols + c];
  out[c] = s;
}

// MSE over [rows x cols] with a per-column weight: dY = 2 w (Y - T) / (rows cols),
// bf16 copy of dY for the GEMMs, per-block partial losses
__global__ void mse_kernel(const float* __restrict__ Y, const float* __restrict__ T, const float* __restrict__ w,
                           uint32_t rows, uint32_t cols, float* __restrict__ dY, __nv_bfloat16* __restrict__ dYh,
                           float* __restrict__ loss_parts) {
  __shared__ float red[256];
  const uint64_t n = (uint64_t)rows * cols;
  const float scale = 2.0f / (float)n;
  float acc = 0.0f;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float wc = w ? w[i % cols] : 1.0f;
    const float e = Y[i] - T[i];
    acc += wc * e * e;
    const float d = scale * wc * e;
    dY[i] = d;
    dYh[i] = __float2bfloat16_rn(d);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (uint32_t s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_parts[blockIdx.x] = red[0] / (float)n;
}

// AdamW on FP32 master weights; writes the BF16 copy used by the GEMMs.
__global__ void adamw_kernel(float* __restrict__ W, float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ g, __nv_bfloat16* __restrict__ Wh, uint64_t n, float lr,
                             float b1, float b2, float eps, float wd, float bc1, float bc2) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    float w = W[i];
    w = w - lr * (mh / (sqrtf(vh) + eps) + wd * w);
    W[i] = w;
    if (Wh) Wh[i] = __float2bfloat16_rn(w);
  }
}

__global__ void to_bf16_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

// out[r] = X[idx[r]] (row gather of a [n x cols] f32 matrix), optional bf16 copy
__global__ void gather_rows_kernel(const float* __restrict__ X, uint32_t cols, const uint32_t* __restrict__ idx,
                                   uint32_t rows, float* __restrict__ out, __nv_bfloat16* __restrict__ out_h) {
  const uint64_t n = (uint64_t)rows * cols;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(i / cols), c = (uint32_t)(i % cols);
    const float v = X[(uint64_t)idx[r] * cols + c];
    if (out) out[i] = v;
    if (out_h) out_h[i] = __float2bfloat16_rn(v);
  }
}

// (x - mean) / std per column, to bf16 (inference inputs)
__global__ void standardize_kernel(const float* __restrict__ x, const float* __restrict__ mean,
                                   const float* __restrict__ sd, uint32_t cols, uint64_t n,
                                   __nv_bfloat16* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)(i % cols);
    out[i] = __float2bfloat16_rn((x[i] - mean[c]) / sd[c]);
  }
}

// ensemble moments of the de-standardized outputs: acc (+)= y, acc2 (+)= y^2;
// final: mean = acc / E, spread = sqrt(max(acc2 / E - mean^2, 0))
__global__ void ensemble_kernel(const float* __restrict__ y, const float* __restrict__ mean,
                                const float* __restrict__ sd, uint32_t cols, uint64_t n, float* __restrict__ acc,
                                float* __restrict__ acc2, uint32_t first, uint32_t last, float inv_e) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)(i % cols);
    const float v = y[i] * sd[c] + mean[c];
    float a = first ? v : acc[i] + v;
    float a2 = first ? v * v : acc2[i] + v * v;
    if (last) {
      const float m = a * inv_e;
      a2 = sqrtf(fmaxf(a2 * inv_e - m * m, 0.0f));
      a = m;
    }
    acc[i] = a;
    acc2[i] = a2;
  }
}

// per row: the largest ensemble spread among outputs whose mean is >= level
// (one warp per row)
__global__ void row_spread_kernel(const float* __restrict__ mean, const float* __restrict__ sd, uint32_t cols,
                                  uint32_t rows, float level, float* __restrict__ out) {
  const uint32_t row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
  if (row >= rows) return;
  float m = 0.0f;
  for (uint32_t c = lane; c < cols; c += 32) {
    const uint64_t i = (uint64_t)row * cols + c;
    if (mean[i] >= level) m = fmaxf(m, sd[i]);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) out[row] = m;
}

// The elementwise kernels of the backward pass on 32 x 32 tiles (block 32 x 8,
// each thread 4 rows of one column): the f32 and bf16 gradient row-major, its
// bf16 transpose (the K-major operand of the next dW GEMM) through shared
// memory, and the column sums (the bias gradient) added atomically into gb,
// which the caller zeroes first.
//   mode 0 (the loss): d = 2 w (Y - T) / (rows cols), loss += w (Y - T)^2 / (rows cols)
//   mode 1 (GELU'):    d = dA * GELU'(Z)
__global__ void grad_tile_kernel(uint32_t mode, const float* __restrict__ P, const float* __restrict__ Q,
                                 const float* __restrict__ w, uint32_t rows, uint32_t cols, float* __restrict__ dZ,
                                 __nv_bfloat16* __restrict__ dZh, __nv_bfloat16* __restrict__ dZht,
                                 float* __restrict__ gb, float* __restrict__ loss) {
  __shared__ __nv_bfloat16 tile[32][34];
  __shared__ float part[8][33];
  __shared__ float lpart[8];
  const uint32_t tx = threadIdx.x, ty = threadIdx.y;
  const uint32_t c = blockIdx.x * 32u + tx, r0 = blockIdx.y * 32u;
  const float inv_n = 1.0f / ((float)rows * (float)cols);
  float csum = 0.0f, lsum = 0.0f;
#pragma unroll
  for (uint32_t k = 0; k < 4; k++) {
    const uint32_t rl = ty + 8u * k, r = r0 + rl;
    float d = 0.0f;
    if (r < rows && c < cols) {
      const uint64_t i = (uint64_t)r * cols + c;
      if (mode == 0) {
        const float wc = w ? w[c] : 1.0f;
        const float e = P[i] - Q[i];
        lsum += wc * e * e;
        d = 2.0f * wc * e * inv_n;
      } else {
        d = P[i] * gelu_grad(Q[i]);
      }
      dZ[i] = d;
      dZh[i] = __float2bfloat16_rn(d);
      csum += d;
    }
    tile[rl][tx] = __float2bfloat16_rn(d);
  }
  part[ty][tx] = csum;
  if (mode == 0) {
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (tx == 0) lpart[ty] = lsum;
  }
  __syncthreads();
  if (ty == 0) {
    float t = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) t += part[k][tx];
    if (c < cols && gb) atomicAdd(gb + c, t);
    if (mode == 0 && tx == 0 && loss) {
      float l = 0.0f;
#pragma unroll
      for (int k = 0; k < 8; k++) l += lpart[k];
      atomicAdd(loss, l * inv_n);
    }
  }
  // transposed: consecutive threads write consecutive rows of one column
#pragma unroll
  for (uint32_t k = 0; k < 4; k++) {
    const uint32_t cl = ty + 8u * k, cc = blockIdx.x * 32u + cl, r = r0 + tx;
    if (cc < cols && r < rows) dZht[(uint64_t)cc * rows + r] = tile[tx][cl];
  }
}

// AdamW on one layer's FP32 master weights W [out x in] and biases b [out]
// (no weight decay on biases), learning rate and bias corrections of step
// *step from sched (3 floats a step); writes the bf16 copy Wh and its
// transpose Wht [in x out].
__global__ void adamw_layer_kernel(float* __restrict__ W, float* __restrict__ mW, float* __restrict__ vW,
                                   const float* __restrict__ gW, __nv_bfloat16* __restrict__ Wh,
                                   __nv_bfloat16* __restrict__ Wht, uint32_t in, uint32_t out, float* __restrict__ b,
                                   float* __restrict__ mb, float* __restrict__ vb, const float* __restrict__ gb,
                                   const float* __restrict__ sched, const uint32_t* __restrict__ step, float b1,
                                   float b2, float eps, float wd) {
  const uint32_t t = *step;
  const float lr = sched[3u * t], bc1 = sched[3u * t + 1u], bc2 = sched[3u * t + 2u];
  const uint64_t nw = (uint64_t)in * out, n = nw + out;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const bool isw = i < nw;
    float* P = isw ? W + i : b + (i - nw);
    float* M1 = isw ? mW + i : mb + (i - nw);
    float* V1 = isw ? vW + i : vb + (i - nw);
    const float gi = isw ? gW[i] : gb[i - nw];
    const float mi = b1 * *M1 + (1.0f - b1) * gi;
    const float vi = b2 * *V1 + (1.0f - b2) * gi * gi;
    *M1 = mi;
    *V1 = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    float x = *P;
    x = x - lr * (mh / (sqrtf(vh) + eps) + (isw ? wd : 0.0f) * x);
    *P = x;
    if (isw) {
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      Wh[i] = h;
      const uint32_t o = (uint32_t)(i / in), k = (uint32_t)(i % in);
      Wht[(uint64_t)k * out + o] = h;
    }
  }
}

__global__ void step_kernel(uint32_t* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1u;
}

// Rows of this step's batch: out[r] = X[perm[((*step) mod spe) B + r]] (f32,
// optional), its bf16 copy (optional) and bf16 transpose [cols x rows] (optional).
__global__ void gather_step_kernel(const float* __restrict__ X, uint32_t cols, const uint32_t* __restrict__ perm,
                                   const uint32_t* __restrict__ step, uint32_t spe, uint32_t rows,
                                   float* __restrict__ out, __nv_bfloat16* __restrict__ out_h,
                                   __nv_bfloat16* __restrict__ out_ht) {
  const uint32_t* idx = perm + (uint64_t)((*step) % spe) * rows;
  const uint64_t n = (uint64_t)rows * cols;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(i / cols), c = (uint32_t)(i % cols);
    const float v = X[(uint64_t)idx[r] * cols + c];
    if (out) out[i] = v;
    if (out_h) out_h[i] = __float2bfloat16_rn(v);
    if (out_ht) out_ht[(uint64_t)c * rows + r] = __float2bfloat16_rn(v);
  }
}

// x [rows x cols] f32 -> bf16 copy and bf16 transpose [cols x rows]
__global__ void to_bf16_t_kernel(const float* __restrict__ x, uint32_t rows, uint32_t cols,
                                 __nv_bfloat16* __restrict__ xh, __nv_bfloat16* __restrict__ xht) {
  const uint64_t n = (uint64_t)rows * cols;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(i / cols), c = (uint32_t)(i % cols);
    const __nv_bfloat16 h = __float2bfloat16_rn(x[i]);
    if (xh) xh[i] = h;
    if (xht) xht[(uint64_t)c * rows + r] = h;
  }
}

}  // namespace

cudaError_t launch_row_spread(const float* mean, const float* sd, uint32_t cols, uint32_t rows, float level,
                              float* out, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  row_spread_kernel<<<(rows + 7) / 8, 256, 0, s>>>(mean, sd, cols, rows, level, out);
  return cudaGetLastError();
}

cudaError_t launch_standardize(const float* x, const float* mean, const float* sd, uint32_t cols, uint64_t n,
                               void* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  standardize_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      x, mean, sd, cols, n, static_cast<__nv_bfloat16*>(out));
  return cudaGetLastError();
}

cudaError_t launch_ensemble(const float* y, const float* mean, const float* sd, uint32_t cols, uint64_t n,
                            float* acc, float* acc2, bool first, bool last, float inv_e, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  ensemble_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      y, mean, sd, cols, n, acc, acc2, first ? 1u : 0u, last ? 1u : 0u, inv_e);
  return cudaGetLastError();
}

size_t gemm_smem_bytes() { return (size_t)(kTileM + kMaxTileN) * tc::kChunkK * 2; }

namespace {
bool k_major_ok(const void* p, int64_t rs, int64_t ks) {
  return ks == 1 && rs % 8 == 0 && (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}
}  // namespace

namespace {
constexpr int kMaxDev = 64;
bool g_attr_done[kMaxDev] = {};
}  // namespace

// The GEMM kernels' shared-memory limits, once per device (call it outside
// any stream capture, before the first launch_gemm on a device).
cudaError_t gemm_init() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  if (g_attr_done[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(kStages * gemm_smem_bytes()));
  if (e != cudaSuccess) return e;
  g_attr_done[dev] = true;
  return cudaSuccess;
}

cudaError_t launch_gemm(const GemmArgs& g, uint32_t k_split, cudaStream_t s) {
  if (g.M == 0 || g.N == 0 || g.K == 0) return cudaSuccess;
  if (g.n_tile == 0 || g.n_tile > kMaxTileN || (g.n_tile & 15u)) return cudaErrorInvalidValue;
  cudaError_t e = gemm_init();
  if (e != cudaSuccess) return e;
  dim3 grid((g.M + kTileM - 1) / kTileM, (g.N + g.n_tile - 1) / g.n_tile, k_split ? k_split : 1);
  const size_t stage = (size_t)(kTileM + g.n_tile) * tc::kChunkK * 2;
  if (k_major_ok(g.A, g.a_rs, g.a_ks) && k_major_ok(g.B, g.b_rs, g.b_ks) && g.K % 8 == 0)
    gemm_kernel<true><<<grid, 128, kStages * stage, s>>>(g);
  else
    gemm_kernel<false><<<grid, 128, stage, s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_gelu_back(const float* dA, const float* Z, float* dZ, void* dZh, uint64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  gelu_back_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      dA, Z, dZ, static_cast<__nv_bfloat16*>(dZh), n);
  return cudaGetLastError();
}

cudaError_t launch_colsum(const float* X, uint32_t rows, uint32_t cols, float* out, cudaStream_t s) {
  colsum_kernel<<<(cols + 127) / 128, 128, 0, s>>>(X, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t launch_mse(const float* Y, const float* T, const float* w, uint32_t rows, uint32_t cols, float* dY,
                       void* dYh, float* loss_parts, uint32_t n_parts, cudaStream_t s) {
  mse_kernel<<<n_parts, 256, 0, s>>>(Y, T, w, rows, cols, dY, static_cast<__nv_bfloat16*>(dYh), loss_parts);
  return cudaGetLastError();
}

cudaError_t launch_adamw(float* W, float* m, float* v, const float* g, void* Wh, uint64_t n, float lr, float b1,
                         float b2, float eps, float wd, float bc1, float bc2, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  adamw_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      W, m, v, g, static_cast<__nv_bfloat16*>(Wh), n, lr, b1, b2, eps, wd, bc1, bc2);
  return cudaGetLastError();
}

cudaError_t launch_grad_tile(uint32_t mode, const float* P, const float* Q, const float* w, uint32_t rows,
                             uint32_t cols, float* dZ, void* dZh, void* dZht, float* gb, float* loss,
                             cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  grad_tile_kernel<<<grid, block, 0, s>>>(mode, P, Q, w, rows, cols, dZ, static_cast<__nv_bfloat16*>(dZh),
                                          static_cast<__nv_bfloat16*>(dZht), gb, loss);
  return cudaGetLastError();
}

cudaError_t launch_adamw_layer(float* W, float* mW, float* vW, const float* gW, void* Wh, void* Wht, uint32_t in,
                               uint32_t out, float* b, float* mb, float* vb, const float* gb, const float* sched,
                               const uint32_t* step, float b1, float b2, float eps, float wd, cudaStream_t s) {
  const uint64_t n = (uint64_t)in * out + out;
  adamw_layer_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 1024), 256, 0, s>>>(
      W, mW, vW, gW, static_cast<__nv_bfloat16*>(Wh), static_cast<__nv_bfloat16*>(Wht), in, out, b, mb, vb, gb,
      sched, step, b1, b2, eps, wd);
  return cudaGetLastError();
}

cudaError_t launch_step(uint32_t* step, cudaStream_t s) {
  step_kernel<<<1, 32, 0, s>>>(step);
  return cudaGetLastError();
}

cudaError_t launch_gather_step(const float* X, uint32_t cols, const uint32_t* perm, const uint32_t* step,
                               uint32_t spe, uint32_t rows, float* out, void* out_h, void* out_ht, cudaStream_t s) {
  const uint64_t n = (uint64_t)rows * cols;
  gather_step_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 2048), 256, 0, s>>>(
      X, cols, perm, step, spe, rows, out, static_cast<__nv_bfloat16*>(out_h), static_cast<__nv_bfloat16*>(out_ht));
  return cudaGetLastError();
}

cudaError_t launch_to_bf16_t(const float* x, uint32_t rows, uint32_t cols, void* xh, void* xht, cudaStream_t s) {
  const uint64_t n = (uint64_t)rows * cols;
  if (n == 0) return cudaSuccess;
  to_bf16_t_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 2048), 256, 0, s>>>(
      x, rows, cols, static_cast<__nv_bfloat16*>(xh), static_cast<__nv_bfloat16*>(xht));
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* x, void* y, uint64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  to_bf16_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      x, static_cast<__nv_bfloat16*>(y), n);
  return cudaGetLastError();
}

cudaError_t launch_gather_rows(const float* X, uint32_t cols, const uint32_t* idx, uint32_t rows, float* out,
                               void* out_bf16, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  const uint64_t n = (uint64_t)rows * cols;
  gather_rows_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
      X, cols, idx, rows, out, static_cast<__nv_bfloat16*>(out_bf16));
  return cudaGetLastError();
}

}  // namespace omg
