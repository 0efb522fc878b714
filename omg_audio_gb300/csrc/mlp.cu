// The surrogate's dense layers on the tensor cores: a tcgen05 GEMM with the
// accumulator in TMEM and fused bias + GELU epilogues, and the elementwise and
// optimizer kernels of training (loss and GELU gradients with fused bias
// gradients, batch gathers, AdamW on FP32 master weights with BF16 copies).
//
// GEMM: D[M x N] = A[M x K] . B[N x K]^T with A, B in BF16 and FP32
// accumulation. Operands are read through strides: element (m, k) of A is
// A[m a_rs + k a_ks]. One CTA of 128 threads computes a 128 x n_tile tile
// (n_tile <= 256) in 64-wide K chunks staged into shared memory as K-major
// core matrices (tc_gemm.cuh); one thread issues four K = 16 MMAs per chunk
// and commits them to an mbarrier (bounded waits). When both operands are
// K-major and 16-byte aligned (every GEMM of training: the backward pass reads
// transposed copies that the producing kernels write), the chunks are staged
// by a three-deep cp.async pipeline, so the copies of the next chunks run
// under the current MMAs; otherwise each chunk is staged by plain loads. The
// epilogue reads the accumulator with tcgen05.ld and writes the row-major
// outputs through shared memory, whole lines at a time. A grid z dimension
// splits K; the split partials are added atomically.
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
  // TMEM columns: the tile's width rounded up to a power of two (>= 32)
  uint32_t tcols = 32u;
  while (tcols < ((g.n_tile + 15u) & ~15u)) tcols <<= 1;
  if (warp == 0) tc::tmem_alloc(&taddr_s, tcols);
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
  if (warp == 0) tc::tmem_dealloc(taddr, tcols);
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

__global__ void step_kernel(uint32_t* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1u;
}

// AdamW of every layer of one member in one launch (layer table by value);
// otherwise as adamw_layer_kernel.
__global__ void adamw_all_kernel(AdamwTable tab, const float* __restrict__ sched, const uint32_t* __restrict__ step,
                                 float b1, float b2, float eps, float wd) {
  const uint32_t t = *step;
  const float lr = sched[3u * t], bc1 = sched[3u * t + 1u], bc2 = sched[3u * t + 2u];
  for (uint64_t gi = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; gi < tab.total;
       gi += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t l = 0;
    while (l + 1 < tab.n && gi >= tab.L[l + 1].off) l++;
    const AdamwLayer& Y = tab.L[l];
    const uint64_t i = gi - Y.off, nw = (uint64_t)Y.in * Y.out;
    const bool isw = i < nw;
    float* P = isw ? Y.W + i : Y.b + (i - nw);
    float* M1 = isw ? Y.mW + i : Y.mb + (i - nw);
    float* V1 = isw ? Y.vW + i : Y.vb + (i - nw);
    const float g = isw ? Y.gW[i] : Y.gb[i - nw];
    const float mi = b1 * *M1 + (1.0f - b1) * g;
    const float vi = b2 * *V1 + (1.0f - b2) * g * g;
    *M1 = mi;
    *V1 = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    float x = *P;
    x = x - lr * (mh / (sqrtf(vh) + eps) + (isw ? wd : 0.0f) * x);
    *P = x;
    if (isw) {
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      static_cast<__nv_bfloat16*>(Y.Wh)[i] = h;
      const uint32_t o = (uint32_t)(i / Y.in), k = (uint32_t)(i % Y.in);
      static_cast<__nv_bfloat16*>(Y.Wht)[(uint64_t)k * Y.out + o] = h;
    }
  }
}

// This step's batch rows of the inputs (blockIdx.y 0: bf16 copy and
// transpose) and of the targets (blockIdx.y 1: f32), as gather_step_kernel.
__global__ void gather_pair_kernel(const float* __restrict__ X, uint32_t xcols, const float* __restrict__ Y,
                                   uint32_t ycols, const uint32_t* __restrict__ perm,
                                   const uint32_t* __restrict__ step, uint32_t spe, uint32_t rows,
                                   __nv_bfloat16* __restrict__ xh, __nv_bfloat16* __restrict__ xht,
                                   float* __restrict__ t) {
  const uint32_t* idx = perm + (uint64_t)((*step) % spe) * rows;
  const bool isx = blockIdx.y == 0;
  const uint32_t cols = isx ? xcols : ycols;
  const float* S = isx ? X : Y;
  const uint64_t n = (uint64_t)rows * cols;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(i / cols), c = (uint32_t)(i % cols);
    const float v = S[(uint64_t)idx[r] * cols + c];
    if (isx) {
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      xh[i] = h;
      xht[(uint64_t)c * rows + r] = h;
    } else {
      t[i] = v;
    }
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

cudaError_t launch_grad_tile(uint32_t mode, const float* P, const float* Q, const float* w, uint32_t rows,
                             uint32_t cols, float* dZ, void* dZh, void* dZht, float* gb, float* loss,
                             cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  grad_tile_kernel<<<grid, block, 0, s>>>(mode, P, Q, w, rows, cols, dZ, static_cast<__nv_bfloat16*>(dZh),
                                          static_cast<__nv_bfloat16*>(dZht), gb, loss);
  return cudaGetLastError();
}

cudaError_t launch_adamw_all(const AdamwTable& tab, const float* sched, const uint32_t* step, float b1, float b2,
                             float eps, float wd, cudaStream_t s) {
  if (tab.total == 0) return cudaSuccess;
  adamw_all_kernel<<<(uint32_t)std::min<uint64_t>((tab.total + 255) / 256, 1024), 256, 0, s>>>(tab, sched, step, b1,
                                                                                              b2, eps, wd);
  return cudaGetLastError();
}

cudaError_t launch_gather_pair(const float* X, uint32_t xcols, const float* Y, uint32_t ycols, const uint32_t* perm,
                               const uint32_t* step, uint32_t spe, uint32_t rows, void* xh, void* xht, float* t,
                               cudaStream_t s) {
  const uint64_t n = (uint64_t)rows * std::max(xcols, ycols);
  dim3 grid((uint32_t)std::min<uint64_t>((n + 255) / 256, 1024), 2);
  gather_pair_kernel<<<grid, 256, 0, s>>>(X, xcols, Y, ycols, perm, step, spe, rows,
                                          static_cast<__nv_bfloat16*>(xh), static_cast<__nv_bfloat16*>(xht), t);
  return cudaGetLastError();
}

cudaError_t launch_step(uint32_t* step, cudaStream_t s) {
  step_kernel<<<1, 32, 0, s>>>(step);
  return cudaGetLastError();
}

cudaError_t launch_to_bf16_t(const float* x, uint32_t rows, uint32_t cols, void* xh, void* xht, cudaStream_t s) {
  const uint64_t n = (uint64_t)rows * cols;
  if (n == 0) return cudaSuccess;
  to_bf16_t_kernel<<<(uint32_t)std::min<uint64_t>((n + 255) / 256, 2048), 256, 0, s>>>(
      x, rows, cols, static_cast<__nv_bfloat16*>(xh), static_cast<__nv_bfloat16*>(xht));
  return cudaGetLastError();
}

}  // namespace omg
