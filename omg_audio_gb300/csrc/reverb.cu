// estimate_reverb on the GPU (crates/omg-core/src/tracer.rs:204-257): one warp
// per (echogram, band). FP64 is used only here, for the Schroeder backward
// integral and the line fit. The late level is the reference's own f32 sum of
// the bins from 80 ms on, in its order (tracer.rs:246-254), by one lane. The
// warp first stages the band's bins in shared memory (coalesced loads), so the
// sequential sums read shared memory instead of waiting on one load each.
#include <cfloat>

#include "omg_internal.h"

namespace omg {

namespace {

__device__ __forceinline__ double db_of(double e, double total) {
  return 10.0 * log10(fmax(e / total, 1e-12));
}

__global__ void reverb_kernel(const DReverbJob* __restrict__ rj, uint32_t n_jobs, const float* __restrict__ bins,
                              omg_reverb* __restrict__ out, const uint32_t* __restrict__ job_segments,
                              uint32_t max_bins) {
  extern __shared__ double edc[];           // max_bins doubles, then the band's bins (max_bins floats)
  float* sb = reinterpret_cast<float*>(edc + max_bins);
  const uint32_t j = blockIdx.x, b = blockIdx.y;
  const DReverbJob R = rj[j];
  const uint32_t lane = threadIdx.x;
  if (j >= n_jobs) return;
  if (b >= R.nb) {
    if (b < OMG_MAX_BANDS && lane == 0) {
      out[j].rt60[b] = 0.0f;
      out[j].level[b] = 0.0f;
      out[j].rt60_fit[b] = 0.0f;
    }
    return;
  }
  const uint32_t n = R.n_bins, nb = R.nb;
  const float* B = bins + R.bins_off;
  for (uint32_t i = lane; i < n; i += 32) sb[i] = B[(uint64_t)i * nb + b];
  __syncwarp();
  // per-lane contiguous chunk, sequential backward sum, then a suffix scan of
  // the chunk totals across the warp
  const uint32_t chunk = (n + 31) / 32;
  const uint32_t lo = lane * chunk, hi = min(n, lo + chunk);
  double run = 0.0;
  for (int64_t i = (int64_t)hi - 1; i >= (int64_t)lo; i--) {
    run += (double)sb[i];
    edc[i] = run;
  }
  // exclusive suffix of chunk totals: sum over lanes > lane
  double incl = run;
  for (int off = 1; off < 32; off <<= 1) {
    double v = __shfl_down_sync(0xffffffffu, incl, off);
    if (lane + off < 32) incl += v;
  }
  const double after = incl - run;
  for (uint32_t i = lo; i < hi; i++) edc[i] += after;
  __syncwarp();
  const double total = __shfl_sync(0xffffffffu, incl, 0);

  float rt60 = 0.5f, fit = 0.5f;
  if (total > 0.0) {
    // first bins at <= -5 dB and <= -25 dB. The EDC is non-increasing, so each
    // lane stops at its first bin past both levels. The dB value is computed
    // only for a bin within 1e-9 (relative) of a level's energy: elsewhere the
    // energy ratio decides the same comparison, without a logarithm per bin.
    const double r5 = sqrt(0.1);            // 10^(-5/10)
    const double e5 = total * r5, e25 = total * (r5 * 0.01);
    auto below = [&](double e, double level, double thr) {
      if (e < thr * (1.0 - 1e-9)) return true;
      if (e > thr * (1.0 + 1e-9)) return false;
      return db_of(e, total) <= level;
    };
    uint32_t f5 = 0xFFFFFFFFu, f25 = 0xFFFFFFFFu;
    for (uint32_t i = lane; i < n && f25 == 0xFFFFFFFFu; i += 32) {
      const double e = edc[i];
      if (f5 == 0xFFFFFFFFu && below(e, -5.0, e5)) f5 = i;
      if (below(e, -25.0, e25)) f25 = i;
    }
    for (int off = 16; off > 0; off >>= 1) {
      f5 = min(f5, __shfl_xor_sync(0xffffffffu, f5, off));
      f25 = min(f25, __shfl_xor_sync(0xffffffffu, f25, off));
    }
    // the reference stops scanning at t25, so t5 is only set when found first
    if (f25 != 0xFFFFFFFFu && f5 != 0xFFFFFFFFu && f5 <= f25 && f25 > f5) {
      const double d5 = db_of(edc[f5], total), d25 = db_of(edc[f25], total);
      const float dt = (float)(f25 - f5) * R.bin_dt;
      const float ddb = (float)(d25 - d5);
      rt60 = fminf(fmaxf(-60.0f * dt / ddb, 0.1f), 5.0f);
      // least-squares T20 line of dB(EDC) over [t5, t25]
      double sx = 0, sy = 0, sxx = 0, sxy = 0;
      for (uint32_t i = f5 + lane; i <= f25; i += 32) {
        const double x = (double)i * (double)R.bin_dt, y = db_of(edc[i], total);
        sx += x; sy += y; sxx += x * x; sxy += x * y;
      }
      for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
        sxx += __shfl_xor_sync(0xffffffffu, sxx, off);
        sxy += __shfl_xor_sync(0xffffffffu, sxy, off);
      }
      const double cnt = (double)(f25 - f5 + 1);
      const double den = cnt * sxx - sx * sx;
      if (den > 0) {
        const double slope = (cnt * sxy - sx * sy) / den;
        if (slope < 0) fit = (float)fmin(fmax(-60.0 / slope, 0.1), 5.0);
      }
    }
  }
  if (lane == 0) {
    out[j].rt60[b] = rt60;
    out[j].rt60_fit[b] = fit;
    // tracer.rs:246: late_start = (0.080 / BIN_DT) as usize in f32
    const float q = 0.080f / R.bin_dt;
    const uint64_t ls = (q >= 0.0f) ? (uint64_t)q : 0;
    float late = 0.0f;
    for (uint64_t i = ls; i < n; i++) late += sb[i];
    out[j].level[b] = fminf(sqrtf(late), 0.7f);
    if (b == 0) out[j].segments = job_segments ? job_segments[j] : 0;
  }
}

}  // namespace

cudaError_t launch_reverb(const DReverbJob* rj, uint32_t n_jobs, uint32_t max_bins, const float* bins,
                          omg_reverb* out, const uint32_t* job_segments, cudaStream_t s) {
  if (n_jobs == 0) return cudaSuccess;
  size_t smem = (size_t)max_bins * (sizeof(double) + sizeof(float));
  if (smem > 227 * 1024) return cudaErrorInvalidValue;   // more than 19,370 bins: beyond a block's shared memory
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(reverb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  dim3 grid(n_jobs, OMG_MAX_BANDS);
  reverb_kernel<<<grid, 32, smem, s>>>(rj, n_jobs, bins, out, job_segments, max_bins);
  return cudaGetLastError();
}

}  // namespace omg
