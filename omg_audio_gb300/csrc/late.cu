// The late field of many sim instances on the GPU: each slot keeps its
// temporally averaged echogram in device memory (Sim::echo_avg, sim.rs:79-100).
// A tick traces the gated slots in one batch; then, per traced slot,
//   - late_ema_kernel blends the fresh echogram in (Echogram::ema,
//     tracer.rs:46-57: a += alpha (o - a), with the caller's alpha per
//     update: sim.rs:338-341, 372-375 take 1 when a result lands on a sim's
//     first call and 0.3 otherwise);
//   - the reverb of the averaged echogram (estimate_reverb) runs through
//     reverb.cu on the slot's echogram;
//   - late_state_kernel writes the slot's state: reverb, late direction and
//     anisotropy (Echogram::late_direction, tracer.rs:59-77).
// Only the per-slot states travel back to the host.
#include <cfloat>

#include "omg_internal.h"

namespace omg {

namespace {

__global__ void late_ema_kernel(const DLateUpdate* __restrict__ up, uint32_t n_up, const float* __restrict__ fresh,
                                float* __restrict__ avg, uint32_t n_bins, uint32_t nb) {
  const uint32_t u = blockIdx.y;
  if (u >= n_up) return;
  const DLateUpdate U = up[u];
  const float alpha = U.alpha;
  const uint64_t n = (uint64_t)n_bins * (nb + 3);   // bins then dirs, as the batch lays out one job
  const float* o = fresh + U.fresh_off;
  float* a = avg + (uint64_t)U.slot * n;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float ai = a[i];
    a[i] = ai + alpha * (o[i] - ai);
  }
}

// One warp per traced slot: the late direction from bin `from_bin` on (the
// sum of the direction vectors and of the energy of band `dir_band`, tracer.rs:
// 59-77), the slot's reverb from the reverb kernel's output, the new version.
__global__ void late_state_kernel(const DLateUpdate* __restrict__ up, uint32_t n_up, const float* __restrict__ avg,
                                  const omg_reverb* __restrict__ rev, uint32_t* __restrict__ version,
                                  omg_late_state* __restrict__ state, uint32_t n_bins, uint32_t nb,
                                  uint32_t from_bin, uint32_t dir_band) {
  const uint32_t u = blockIdx.x;
  if (u >= n_up) return;
  const uint32_t lane = threadIdx.x;
  const DLateUpdate U = up[u];
  const float* a = avg + (uint64_t)U.slot * n_bins * (nb + 3);
  const float* dirs = a + (uint64_t)n_bins * nb;
  float vx = 0.0f, vy = 0.0f, vz = 0.0f, e = 0.0f;
  for (uint32_t i = from_bin + lane; i < n_bins; i += 32u) {
    vx += dirs[3 * i + 0];
    vy += dirs[3 * i + 1];
    vz += dirs[3 * i + 2];
    e += a[(uint64_t)i * nb + dir_band];
  }
  for (int off = 16; off > 0; off >>= 1) {
    vx += __shfl_xor_sync(0xffffffffu, vx, off);
    vy += __shfl_xor_sync(0xffffffffu, vy, off);
    vz += __shfl_xor_sync(0xffffffffu, vz, off);
    e += __shfl_xor_sync(0xffffffffu, e, off);
  }
  if (lane != 0) return;
  omg_late_state& S = state[U.slot];
  const float len = sqrtf(vx * vx + vy * vy + vz * vz);
  if (len < 1e-12f || e < 1e-12f) {
    S.dir[0] = 1.0f;
    S.dir[1] = 0.0f;
    S.dir[2] = 0.0f;
    S.anisotropy = 0.0f;
  } else {
    S.dir[0] = vx / len;
    S.dir[1] = vy / len;
    S.dir[2] = vz / len;
    S.anisotropy = fminf(len / e, 1.0f);
  }
  const omg_reverb& R = rev[u];
  for (int b = 0; b < OMG_MAX_BANDS; b++) {
    S.rt60[b] = R.rt60[b];
    S.level[b] = R.level[b];
  }
  const uint32_t v = version[U.slot] + 1u;
  version[U.slot] = v;
  S.version = v;
  S.updated_tick = U.tick;
}

}  // namespace

cudaError_t launch_late_update(const DLateUpdate* up, uint32_t n_up, const float* fresh, float* avg,
                               uint32_t* version, const DReverbJob* rj, omg_reverb* rev, omg_late_state* state,
                               uint32_t n_bins, uint32_t nb, uint32_t from_bin, uint32_t dir_band, cudaStream_t s) {
  if (n_up == 0) return cudaSuccess;
  const uint64_t n = (uint64_t)n_bins * (nb + 3);
  const uint32_t bx = (uint32_t)((n + 255) / 256 < 64 ? (n + 255) / 256 : 64);
  late_ema_kernel<<<dim3(bx, n_up), 256, 0, s>>>(up, n_up, fresh, avg, n_bins, nb);
  cudaError_t e = launch_reverb(rj, n_up, n_bins, avg, rev, nullptr, s);
  if (e != cudaSuccess) return e;
  late_state_kernel<<<n_up, 32, 0, s>>>(up, n_up, avg, rev, version, state, n_bins, nb, from_bin, dir_band);
  return cudaGetLastError();
}

}  // namespace omg
